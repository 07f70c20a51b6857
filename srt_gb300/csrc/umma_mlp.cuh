// umma_mlp.cuh — fully fused MLP inference on the 5th-generation tensor
// cores: D = act(A W^T) layer after layer for 128-row tiles, BF16 operands,
// FP32 accumulation in tensor memory, activations kept on chip.
//
// One CTA = 4 warps = 128 threads; thread t owns row t of the tile (TMEM lane
// t).  Per tile and layer: one thread issues K/16 tcgen05.mma (M = 128,
// N = layer width, K = 16 each) from shared-memory descriptors and commits
// them to an mbarrier; every thread then reads its row's accumulator with
// tcgen05.ld, applies the activation, converts to BF16 and writes it back to
// shared memory in the canonical layout as the next layer's A operand (the
// last layer's values go to the task's output instead).
//
// Weights arrive by bulk copy (cp.async.bulk on the TMA engine) from a
// global buffer already in the canonical layout (pack_canonical_weights):
// either all layers once per CTA (Task::kResident, small networks, several
// CTAs per SM overlap one another's epilogues), or layer by layer, the next
// layer's copy issued as soon as the current layer's MMAs have completed so
// that it overlaps the epilogue.  The input tile is either built by the
// threads (Task::make_input) or bulk-copied from a global buffer written in
// the canonical tile layout (Task::kInputBulk).
//
// Every wait is bounded (mbar_wait); a timeout sets *err, ends the CTA's
// loop for all its threads at once and still frees the CTA's TMEM.
#pragma once

#include <cuda_bf16.h>

#include <algorithm>

#include "common.h"
#include "umma.cuh"

namespace srt {

constexpr int kUmmaRows = 128;     // M of every tcgen05.mma (one row per thread)
constexpr int kUmmaThreads = 128;

// Task interface (all static sizes):
//   kLayers, in(l), out(l): layer shapes (out(l) a multiple of 16 in
//     [16, 256], in(l) a multiple of 16); in(l + 1) == out(l)
//   kResident: every layer's weights stay in shared memory
//   kInputBulk: the input tile is copied from input_tile(tile) (128 x in(0)
//     BF16 in the canonical layout); else make_input(row, valid, a, r)
//     writes row r of the tile
//   relu(l): ReLU after layer l (not after the last)
//   weights(): the packed weights, layer l at byte w_off(l)
//   rows(): rows to process; store(row, float (&v)[out(last)])
template <class Task>
struct UmmaMlpLayout {
    __host__ __device__ static constexpr int imax(int a, int b) { return a > b ? a : b; }
    __host__ __device__ static constexpr int max_in()
    {
        int m = 0;
        for (int l = 0; l < Task::kLayers; ++l) m = Task::in(l) > m ? Task::in(l) : m;
        return m;
    }
    __host__ __device__ static constexpr int max_out()
    {
        int m = 0;
        for (int l = 0; l < Task::kLayers; ++l) m = Task::out(l) > m ? Task::out(l) : m;
        return m;
    }
    __host__ __device__ static constexpr uint32_t w_bytes(int l) { return (uint32_t)Task::in(l) * Task::out(l) * 2u; }
    __host__ __device__ static constexpr uint32_t w_total()
    {
        uint32_t s = 0;
        for (int l = 0; l < Task::kLayers; ++l) s += w_bytes(l);
        return s;
    }
    __host__ __device__ static constexpr uint32_t w_max()
    {
        uint32_t m = 0;
        for (int l = 0; l < Task::kLayers; ++l) m = w_bytes(l) > m ? w_bytes(l) : m;
        return m;
    }
    static constexpr uint32_t kWSmem = Task::kResident ? w_total() : w_max();
    static constexpr uint32_t kASmem = (uint32_t)kUmmaRows * imax(max_in(), max_out()) * 2u;
    static constexpr uint32_t kAOff = (kWSmem + 1023u) / 1024u * 1024u;
    static constexpr uint32_t kBarOff = kAOff + (kASmem + 127u) / 128u * 128u;
    static constexpr uint32_t kSmem = kBarOff + 64u;  // two mbarriers + the TMEM address
    __host__ __device__ static constexpr uint32_t tmem_cols()
    {
        uint32_t c = 32;
        while (c < (uint32_t)max_out()) c <<= 1;
        return c;
    }
};

template <class Task>
__global__ void __launch_bounds__(kUmmaThreads, 1) k_umma_mlp(Task task, int* err)
{
    using L = UmmaMlpLayout<Task>;
    extern __shared__ __align__(1024) uint8_t umma_smem[];
    uint8_t* wsm = umma_smem;
    uint8_t* asm_ = umma_smem + L::kAOff;
    uint64_t* bar_mma = reinterpret_cast<uint64_t*>(umma_smem + L::kBarOff);
    uint64_t* bar_ld = bar_mma + 1;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar_mma + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int64_t n = task.rows();
    const int64_t tiles = (n + kUmmaRows - 1) / kUmmaRows;
    if ((int64_t)blockIdx.x >= tiles) return;  // uniform over the CTA, before any TMEM or barrier use

    if (warp == 0) tmem_alloc(tslot, L::tmem_cols());
    if (tid == 0) {
        mbar_init(bar_mma, 1);
        mbar_init(bar_ld, 1);
        mbar_fence_init();
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;  // this warp's TMEM lanes
    // copies per tile: the bulk input tile and/or the first layer's weights
    constexpr bool kTileLoads = Task::kInputBulk || !Task::kResident;
    constexpr uint32_t kInBytes = (uint32_t)kUmmaRows * Task::in(0) * 2u;
    // Every thread tracks the same schedule: ld_pending / mma_pending say
    // that a copy / an MMA group is in flight on bar_ld / bar_mma with the
    // current parity; thread 0 alone issues them.
    uint32_t ph_mma = 0, ph_ld = 0;
    bool ld_pending = false, mma_pending = false;
    bool ok = true;

    auto issue_tile_loads = [&](int64_t tile) {
        mbar_arrive_expect_tx(bar_ld, (Task::kInputBulk ? kInBytes : 0u) + (Task::kResident ? 0u : L::w_bytes(0)));
        if (Task::kInputBulk) bulk_g2s(asm_, task.input_tile(tile), kInBytes, bar_ld);
        if (!Task::kResident) bulk_g2s(wsm, task.weights() + Task::w_off(0), L::w_bytes(0), bar_ld);
    };
    auto wait_ld = [&]() {
        if (mbar_wait(bar_ld, ph_ld)) {
            ph_ld ^= 1u;
            ld_pending = false;
            return true;
        }
        return false;
    };

    if (Task::kResident) {
        if (tid == 0) {
            mbar_arrive_expect_tx(bar_ld, L::w_total());
            for (int l = 0; l < Task::kLayers; ++l)  // one copy per layer
                bulk_g2s(wsm + Task::w_off(l), task.weights() + Task::w_off(l), L::w_bytes(l), bar_ld);
        }
        ld_pending = true;
        ok = __syncthreads_and(wait_ld());
    }
    if (ok && kTileLoads) {
        if (tid == 0) issue_tile_loads(blockIdx.x);
        ld_pending = true;
    }

    for (int64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int64_t row = tile * kUmmaRows + tid;
        const bool valid = row < n;
        if (!Task::kInputBulk) task.make_input(row, valid, asm_, tid);
        for (int l = 0; l < Task::kLayers; ++l) {
            const int K = Task::in(l), N = Task::out(l);
            // this layer's weights (streaming) and, for layer 0, the bulk input tile
            bool w_ok = true;
            if (ld_pending && (l == 0 || !Task::kResident)) w_ok = wait_ld();
            fence_async_smem();  // this thread's generic writes to the A tile -> async proxy
            ok = __syncthreads_and(w_ok);
            if (!ok) break;
            if (tid == 0) {
                tc_fence_after_sync();
                const uint32_t a0 = smem_u32(asm_);
                const uint32_t b0 = smem_u32(wsm + (Task::kResident ? Task::w_off(l) : 0u));
                const uint32_t sbo = (uint32_t)K * 16u;
                const uint32_t idesc = umma_idesc_bf16(kUmmaRows, N);
                for (int k = 0; k < K / 16; ++k)
                    umma_bf16(tmem, umma_desc(a0 + 256u * k, 128u, sbo), umma_desc(b0 + 256u * k, 128u, sbo), idesc,
                              k > 0 ? 1u : 0u);
                umma_commit(bar_mma);
            }
            mma_pending = true;
            bool m_ok = mbar_wait(bar_mma, ph_mma);
            if (m_ok) {
                ph_mma ^= 1u;
                mma_pending = false;
            }
            ok = __syncthreads_and(m_ok);
            if (!ok) break;
            tc_fence_after_sync();
            // the A tile (after the last layer) and the weight buffer are free:
            // start the next copies so that they overlap the epilogue
            if (!Task::kResident && l + 1 < Task::kLayers) {
                if (tid == 0) {
                    mbar_arrive_expect_tx(bar_ld, L::w_bytes(l + 1));
                    bulk_g2s(wsm, task.weights() + Task::w_off(l + 1), L::w_bytes(l + 1), bar_ld);
                }
                ld_pending = true;
            } else if (kTileLoads && l + 1 == Task::kLayers && tile + gridDim.x < tiles) {
                if (tid == 0) issue_tile_loads(tile + gridDim.x);
                ld_pending = true;
            }
            // epilogue: this thread's row of the accumulator
            const uint32_t trow = tmem + lane_base;
            if (l + 1 < Task::kLayers) {
                const int Kn = N;  // the next layer's K
                const bool relu = Task::relu(l);
#pragma unroll 1
                for (int c0 = 0; c0 < N; c0 += 32) {
                    uint32_t v[32];
                    tmem_ld32(trow + (uint32_t)c0, v);
                    tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; j += 8) {
                        float f[8];
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            f[e] = __uint_as_float(v[j + e]);
                            if (relu) f[e] = fmaxf(f[e], 0.0f);
                        }
                        uint4 q;
                        q.x = pack2_bf16(f[0], f[1]);
                        q.y = pack2_bf16(f[2], f[3]);
                        q.z = pack2_bf16(f[4], f[5]);
                        q.w = pack2_bf16(f[6], f[7]);
                        *reinterpret_cast<uint4*>(asm_ + canon_off(tid, c0 + j, Kn)) = q;
                    }
                }
            } else {
                constexpr int kOut = Task::out(Task::kLayers - 1);
                float o[kOut];
#pragma unroll
                for (int c0 = 0; c0 < kOut; c0 += 16) {
                    uint32_t v[16];
                    tmem_ld16(trow + (uint32_t)c0, v);
                    tmem_ld_wait();
#pragma unroll
                    for (int e = 0; e < 16; ++e) o[c0 + e] = __uint_as_float(v[e]);
                }
                if (valid) task.store(row, o);
            }
            tc_fence_before_sync();
        }
    }
    // nothing of this CTA may still be in flight when its TMEM is freed
    if (tid == 0 && ld_pending) mbar_wait(bar_ld, ph_ld);
    if (tid == 0 && mma_pending) mbar_wait(bar_mma, ph_mma);
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (warp == 0) tmem_dealloc(tmem, L::tmem_cols());
    if (!ok && tid == 0) atomicExch(err, 1);
}

// ---------------------------------------------------------------------------
// Streaming variant for wide networks whose weights do not fit in shared
// memory (k_umma_mlp_stream): two 128-row tiles per CTA share every weight
// chunk (both accumulators in TMEM: 2 x 256 columns), and the weights arrive
// as K-chunks of kChunkK columns (N x 32 BF16, 16 KB for N = 256) through a
// ring of kStreamStages slots that a producer warp keeps filled: chunk
// copies overlap the MMAs of earlier chunks and the epilogues, and each
// chunk is read from L2 once per 256 rows.  Warps 0-3 own tile 0's rows,
// warps 4-7 tile 1's; warp 8 is the producer; thread 0 issues the MMAs.
// Barriers: full[s] (chunk landed), empty[s] (its MMAs done), x_full (the two
// input tiles landed), a_free (the last layer's MMAs done: the A tiles may
// be overwritten), mma (a layer's MMAs done: epilogue).
constexpr int kChunkK = 32;
constexpr int kStreamStages = 6;
constexpr int kStreamConsumers = 2 * kUmmaRows;
constexpr int kStreamThreads = kStreamConsumers + 32;

template <class Task>
struct UmmaStreamLayout {
    using L = UmmaMlpLayout<Task>;
    __host__ __device__ static constexpr uint32_t chunk_bytes(int l) { return (uint32_t)Task::out(l) * kChunkK * 2u; }
    static constexpr uint32_t kChunkMax = (uint32_t)L::max_out() * kChunkK * 2u;
    static constexpr uint32_t kATile = (uint32_t)kUmmaRows * L::imax(L::max_in(), L::max_out()) * 2u;
    static constexpr uint32_t kRingOff = 2u * kATile;
    static constexpr uint32_t kBarOff = kRingOff + kStreamStages * kChunkMax;
    static constexpr uint32_t kSmem = kBarOff + (2 * kStreamStages + 3) * 8 + 16;
    static constexpr uint32_t kTmemCols = 2u * 256u;  // two accumulators of up to 256 columns
};

template <class Task>
__global__ void __launch_bounds__(kStreamThreads, 1) k_umma_mlp_stream(Task task, int* err)
{
    using L = UmmaMlpLayout<Task>;
    using SL = UmmaStreamLayout<Task>;
    static_assert(Task::kInputBulk && !Task::kResident, "the streaming kernel takes bulk input tiles");
    static_assert(L::max_out() <= 256, "one accumulator per tile holds at most 256 columns");
    extern __shared__ __align__(1024) uint8_t umma_smem[];
    uint8_t* ring = umma_smem + SL::kRingOff;
    uint64_t* full = reinterpret_cast<uint64_t*>(umma_smem + SL::kBarOff);
    uint64_t* empty = full + kStreamStages;
    uint64_t* x_full = empty + kStreamStages;
    uint64_t* a_free = x_full + 1;
    uint64_t* bar_mma = a_free + 1;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar_mma + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int64_t n = task.rows();
    const int64_t tiles = (n + kUmmaRows - 1) / kUmmaRows;
    const int64_t pairs = (tiles + 1) / 2;
    if ((int64_t)blockIdx.x >= pairs) return;  // uniform over the CTA, before any TMEM or barrier use

    if (warp == 0) tmem_alloc(tslot, SL::kTmemCols);
    if (tid == 0) {
        for (int s = 0; s < kStreamStages; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(x_full, 1);
        mbar_init(a_free, 1);
        mbar_init(bar_mma, 1);
        mbar_fence_init();
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = *tslot;
    constexpr uint32_t kInBytes = (uint32_t)kUmmaRows * Task::in(0) * 2u;
    bool ok = true;

    if (warp == kStreamConsumers / 32) {
        // ---- producer: the input tiles and the weight chunks, in the order
        // the MMAs consume them -------------------------------------------
        if ((tid & 31) == 0) {
            uint32_t it = 0, ph_af = 0;
            for (int64_t pair = blockIdx.x; pair < pairs && ok; pair += gridDim.x) {
                if (pair != (int64_t)blockIdx.x) {  // the A tiles are free once the last layer's MMAs are done
                    ok = mbar_wait(a_free, ph_af);
                    ph_af ^= 1u;
                    if (!ok) break;
                }
                const int64_t t0 = 2 * pair, t1 = t0 + 1;
                mbar_arrive_expect_tx(x_full, kInBytes * (t1 < tiles ? 2u : 1u));
                bulk_g2s(umma_smem, task.input_tile(t0), kInBytes, x_full);
                if (t1 < tiles) bulk_g2s(umma_smem + SL::kATile, task.input_tile(t1), kInBytes, x_full);
                for (int l = 0; l < Task::kLayers && ok; ++l) {
                    const uint32_t cb = SL::chunk_bytes(l);
                    for (int c = 0; c < Task::in(l) / kChunkK; ++c, ++it) {
                        const uint32_t s = it % kStreamStages, k = it / kStreamStages;
                        if (k > 0 && !(ok = mbar_wait(empty + s, (k - 1u) & 1u))) break;
                        mbar_arrive_expect_tx(full + s, cb);
                        bulk_g2s(ring + s * SL::kChunkMax, task.weights() + Task::w_off(l) + (size_t)c * cb, cb,
                                 full + s);
                    }
                }
            }
        }
    } else {
        // ---- consumers: thread = row of tile (warp / 4); thread 0 issues ----
        const int t = warp >> 2, r = tid & (kUmmaRows - 1);
        uint8_t* a_tile = umma_smem + t * SL::kATile;
        const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)t * 256u;
        uint32_t it = 0, ph_x = 0, ph_m = 0;
        for (int64_t pair = blockIdx.x; pair < pairs && ok; pair += gridDim.x) {
            const int64_t row = (2 * pair + t) * kUmmaRows + r;
            const bool valid = row < n;
            for (int l = 0; l < Task::kLayers; ++l) {
                const int K = Task::in(l), N = Task::out(l);
                bool w_ok = true;
                if (l == 0) {
                    w_ok = mbar_wait(x_full, ph_x);
                    if (w_ok) ph_x ^= 1u;
                }
                fence_async_smem();  // this thread's epilogue writes to its A tile -> async proxy
                ok = named_bar_and(1, kStreamConsumers, w_ok);
                if (!ok) break;
                bool issue_ok = true;
                if (tid == 0) {
                    tc_fence_after_sync();
                    const uint32_t a0 = smem_u32(umma_smem), a1 = smem_u32(umma_smem + SL::kATile);
                    const uint32_t sbo = (uint32_t)K * 16u;
                    const uint32_t idesc = umma_idesc_bf16(kUmmaRows, N);
                    for (int c = 0; c < K / kChunkK; ++c, ++it) {
                        const uint32_t s = it % kStreamStages, k = it / kStreamStages;
                        if (!mbar_wait(full + s, k & 1u)) {
                            issue_ok = false;
                            break;
                        }
                        tc_fence_after_sync();
                        const uint32_t b0 = smem_u32(ring + s * SL::kChunkMax);
#pragma unroll
                        for (int j = 0; j < kChunkK / 16; ++j) {
                            const uint32_t kk = (uint32_t)(c * (kChunkK / 16) + j);
                            const uint64_t bd = umma_desc(b0 + 256u * j, 128u, kChunkK * 16u);
                            umma_bf16(tmem, umma_desc(a0 + 256u * kk, 128u, sbo), bd, idesc, kk > 0 ? 1u : 0u);
                            umma_bf16(tmem + 256u, umma_desc(a1 + 256u * kk, 128u, sbo), bd, idesc, kk > 0 ? 1u : 0u);
                        }
                        umma_commit(empty + s);  // the slot is free once these MMAs are done
                    }
                    umma_commit(bar_mma);
                    if (l + 1 == Task::kLayers) umma_commit(a_free);
                }
                bool m_ok = mbar_wait(bar_mma, ph_m);
                if (m_ok) ph_m ^= 1u;
                ok = named_bar_and(1, kStreamConsumers, m_ok && issue_ok);
                if (!ok) break;
                tc_fence_after_sync();
                if (l + 1 < Task::kLayers) {
                    const bool relu = Task::relu(l);
#pragma unroll 1
                    for (int c0 = 0; c0 < N; c0 += 32) {
                        uint32_t v[32];
                        tmem_ld32(trow + (uint32_t)c0, v);
                        tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 32; j += 8) {
                            float f[8];
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                f[e] = __uint_as_float(v[j + e]);
                                if (relu) f[e] = fmaxf(f[e], 0.0f);
                            }
                            uint4 q;
                            q.x = pack2_bf16(f[0], f[1]);
                            q.y = pack2_bf16(f[2], f[3]);
                            q.z = pack2_bf16(f[4], f[5]);
                            q.w = pack2_bf16(f[6], f[7]);
                            *reinterpret_cast<uint4*>(a_tile + canon_off(r, c0 + j, N)) = q;
                        }
                    }
                } else {
                    constexpr int kOut = Task::out(Task::kLayers - 1);
                    float o[kOut];
#pragma unroll
                    for (int c0 = 0; c0 < kOut; c0 += 16) {
                        uint32_t v[16];
                        tmem_ld16(trow + (uint32_t)c0, v);
                        tmem_ld_wait();
#pragma unroll
                        for (int e = 0; e < 16; ++e) o[c0 + e] = __uint_as_float(v[e]);
                    }
                    if (valid) task.store(row, o);
                }
                tc_fence_before_sync();
            }
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (warp == 0) tmem_dealloc(tmem, SL::kTmemCols);
    if (!ok) atomicExch(err, 1);
}

// Packs one layer's FP32 weights W[out][in] (row-major) into the BF16
// canonical K-major layout at dst (out x in elements).
srt_status umma_pack_layer(const float* src, int in, int out, __nv_bfloat16* dst, cudaStream_t st);
// The same, as in / kChunkK consecutive K-chunks (out x kChunkK each, in the
// canonical layout with K = kChunkK): the streaming kernel's weight order.
srt_status umma_pack_layer_chunked(const float* src, int in, int out, __nv_bfloat16* dst, cudaStream_t st);

// Sets up the fused-MLP kernels on the current device (shared-memory limits,
// the device address of the timeout flag); call before any stream capture
// that launches them.
srt_status umma_prepare();
// The timeout flag's device address on the current device (after umma_prepare).
int* umma_error_word();
// SRT_ERR_TIMEOUT (and clears the flag) if a fused-MLP kernel gave up a wait
// since the last call; synchronous.
srt_status umma_take_error();

// Launches k_umma_mlp<Task> over at most max_rows rows (the task's rows()
// may be fewer, read on the device), grid_y CTAs in y for the task to tell
// apart (jobs), persistent CTAs in x: min(tiles, resident CTAs).
template <class Task>
srt_status umma_mlp_launch(const Task& task, int64_t max_rows, unsigned grid_y, cudaStream_t st)
{
    using L = UmmaMlpLayout<Task>;
    static const int resident = [] {
        cudaFuncSetAttribute(k_umma_mlp<Task>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kSmem);
        // the whole unified L1 / shared array as shared memory, so that several
        // CTAs fit on an SM (the default carveout leaves room for one)
        cudaFuncSetAttribute(k_umma_mlp<Task>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
        // resident CTAs per SM from the limits that bind here: shared memory
        // (with the 1 KB the driver reserves per CTA), the 512 TMEM columns,
        // threads
        int dev = 0, smem_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        int nb = smem_sm / (int)(L::kSmem + 1024u);
        nb = std::min(nb, (int)(512u / L::tmem_cols()));
        nb = std::min(nb, 2048 / kUmmaThreads);
        return std::max(nb, 1);
    }();
    int* err = umma_error_word();
    if (!err) return set_error(SRT_ERR_CUDA, "fused MLP kernels not prepared on this device (umma_prepare)");
    if (max_rows <= 0 || grid_y == 0) return SRT_OK;
    const int64_t tiles = (max_rows + kUmmaRows - 1) / kUmmaRows;
    const int64_t gx = std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)device_sm_count() * resident));
    k_umma_mlp<Task><<<dim3((unsigned)gx, grid_y), kUmmaThreads, L::kSmem, st>>>(task, err);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

// Launches k_umma_mlp_stream<Task> over n rows: one CTA per SM at most, each
// taking pairs of 128-row tiles.
template <class Task>
srt_status umma_mlp_stream_launch(const Task& task, int64_t n, cudaStream_t st)
{
    using SL = UmmaStreamLayout<Task>;
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_umma_mlp_stream<Task>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL::kSmem);
    SRT_CUDA_TRY(attr);
    int* err = umma_error_word();
    if (!err) return set_error(SRT_ERR_CUDA, "fused MLP kernels not prepared on this device (umma_prepare)");
    if (n <= 0) return SRT_OK;
    const int64_t pairs = ((n + kUmmaRows - 1) / kUmmaRows + 1) / 2;
    const int64_t gx = std::max<int64_t>(1, std::min<int64_t>(pairs, (int64_t)device_sm_count()));
    k_umma_mlp_stream<Task><<<(unsigned)gx, kStreamThreads, SL::kSmem, st>>>(task, err);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

}  // namespace srt

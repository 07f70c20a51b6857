"""In-tree build of the CUDA library (sm_103a) and of the test oracles.

`build()` compiles every translation unit under srt_gb300/csrc in parallel
(nvcc for .cu, g++ for .cpp) and links srt_gb300/libsrt_gb300.so.  Only
files newer than their object are rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "libsrt_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit multiply-add contraction, so the device evaluates
# the reference formulas with the same roundings as the FP32 oracle (explicit
# fmaf calls in the BVH slab tests stay fused)
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
# build-time switches of the kernels (e.g. "-DSRT_NODE_EVICT_LAST=1"); a change
# needs a clean rebuild (clean())
NVCC_FLAGS += os.environ.get("SRT_NVCC_DEFINES", "").split()
# host translation units: -ffp-contract=off keeps host float math identical
# on x86-64 and aarch64 (scene flattening, CDFs, camera set-up)
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", os.path.join(CUDA, "include")]


def _sources():
    out = []
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, name))
    return out


def _headers_mtime():
    m = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for name in os.listdir(d):
            if name.endswith((".h", ".cuh")):
                m = max(m, os.path.getmtime(os.path.join(d, name)))
    return m


def _compile(src, hdr_mtime, log):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_mtime):
        return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    if log is not None and r.stderr.strip():
        log.append(f"== {os.path.basename(src)}\n{r.stderr}")
    return obj, None


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183}


def drop_foreign(path: str) -> None:
    """Removes a shared object built for another CPU architecture."""
    want = _ELF_MACHINE.get(platform.machine())
    if want is None or not os.path.exists(path):
        return
    with open(path, "rb") as f:
        head = f.read(20)
    if len(head) == 20 and head[:4] == b"\x7fELF" and int.from_bytes(head[18:20], "little") != want:
        os.remove(path)


def build_library(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    drop_foreign(LIB)
    hdr = _headers_mtime()
    srcs = _sources()
    log: list[str] = []
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, hdr, log), srcs))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("srt_gb300 build failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        for entry in log:
            print(entry, file=sys.stderr)
    return LIB


CLI = os.path.join(HERE, "srt")


def build_cli() -> str:
    """The `srt -c config.json` command (srt_gb300/cli/srt_main.cpp), linked
    against the library through its C ABI only."""
    drop_foreign(CLI)
    src = os.path.join(HERE, "cli", "srt_main.cpp")
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(src), os.path.getmtime(LIB)):
        return CLI
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", CLI, "-L", HERE,
           "-lsrt_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cli build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return CLI


def build_oracle() -> str:
    """CPU oracle (test infrastructure): oracle/liboracle.so."""
    d = os.path.join(ROOT, "oracle")
    for name in ("liboracle.so", "srt_oracle.o", "curand_host.o", "scene_inputs.o"):
        drop_foreign(os.path.join(d, name))
    r = subprocess.run(["make", "-s", "-C", d], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return os.path.join(d, "liboracle.so")


def build_reference(ref_root: str | None = None) -> str | None:
    """Reference headers built for the host (oracle/_ref), from the reference
    tree at `ref_root` or $SRT_REFERENCE_ROOT; skipped (None) when neither
    names a reference tree."""
    ref_root = ref_root or os.environ.get("SRT_REFERENCE_ROOT")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src", "device_include")):
        return None
    d = os.path.join(ROOT, "oracle", "ref")
    r = subprocess.run(["make", "-s", "-C", d, f"REF={ref_root}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    return os.path.join(ROOT, "oracle", "_ref", "libsrtref.so")


def clean():
    shutil.rmtree(OBJ, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    print(build_library(verbose="-v" in sys.argv))
    print(build_cli())
    print(build_oracle())
    print(build_reference())

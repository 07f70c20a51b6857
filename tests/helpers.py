"""Shared test helpers: golden-vector loading and scene rebuilds."""
import ctypes as C
import os

import numpy as np

from srt_gb300 import SceneArrays, _capi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def scene_from_npz(z):
    """Rebuilds the SceneArrays stored by tests/golden/make_golden.py."""
    s = SceneArrays()
    for i in range(int(z["num_meshes"])):
        s.meshes.append({"vertices": z[f"mesh{i}_v"], "indices": z[f"mesh{i}_f"], "normals": None,
                         "material": int(z[f"mesh{i}_mat"])})
    for mid, xf in zip(z["inst_mesh"], z["inst_xf"]):
        s.instances.append((int(mid), xf))
    raw = z["materials"].tobytes()
    sz = C.sizeof(_capi.Material)
    for k in range(len(raw) // sz):
        s.materials.append(_capi.Material.from_buffer_copy(raw[k * sz:(k + 1) * sz]))
    s.camera = _capi.CameraDesc.from_buffer_copy(z["camera"].tobytes())
    s.env = tuple(float(x) for x in z["env"])
    return s


def rel_err(a, b, floor=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)

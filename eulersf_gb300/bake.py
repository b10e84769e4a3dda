"""Offline mass baking on the GPU (esf_rasterize_solid): a solid's rest-pose
mass grid from its closed triangle mesh, the job of the reference's
rasterizeSolid tool (projects/rasterizeSolid/main.cpp:20-80).

    res, dh, origin, mass, total = rasterize_solid(vertices, triangles, 0.001, 1000.0)

`mass` is a (res[2], res[1], res[0]) float64 array, x fastest, in the layout of
the reference's .mass files (scene.write_field_gz writes it as one).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def rasterize_solid(vertices, triangles, mass_dh: float, density: float, lib=None):
    from . import load
    lib = lib or load()
    v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
    res, origin, total = (C.c_int * 3)(), (C.c_double * 3)(), C.c_double()
    args = (v.ctypes.data_as(C.c_void_p), len(v), t.ctypes.data_as(C.c_void_p), len(t), mass_dh, density,
            res, origin)
    st = lib.esf_rasterize_solid(*args, None, 0, None)
    if st != 0:
        raise abi.EsfError(st, "esf_rasterize_solid", (lib.esf_last_error() or b"").decode())
    n = res[0] * res[1] * res[2]
    out = np.empty(n, dtype=np.float64)
    st = lib.esf_rasterize_solid(*args, out.ctypes.data_as(C.c_void_p), n, C.byref(total))
    if st != 0:
        raise abi.EsfError(st, "esf_rasterize_solid", (lib.esf_last_error() or b"").decode())
    return tuple(res), mass_dh, tuple(origin), out.reshape(res[2], res[1], res[0]), total.value

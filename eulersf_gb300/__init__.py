"""GB300 (sm_103a) implementation of EULERSF's coupled solid-fluid step.

The product is the C-ABI library eulersf_gb300/_lib/libeulersf_gb300.so
(include/eulersf.h). This package loads it with ctypes and mirrors the
reference's integrator call surface (``CoupledIntegrator3D``). There is no
CPU fallback: if the library is missing or no GPU is visible, the calls fail.
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi
from .integrator import CoupledIntegrator3D, build_from_scene, run_frames  # noqa: F401
from .scene import SceneDesc, SolidDesc  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libeulersf_gb300.so")
_lib = None

# every symbol include/eulersf.h declares
EXPORTS = [
    "esf_abi_version", "esf_last_error", "esf_params_default", "esf_parse_config", "esf_create",
    "esf_destroy", "esf_add_solid", "esf_set_fluid", "esf_init", "esf_set_max_dt", "esf_step",
    "esf_dt", "esf_field_info", "esf_get_field", "esf_set_field", "esf_pressure_apply",
    "esf_pressure_solve", "esf_pressure_solve_batch", "esf_pressure_solve_static", "esf_write_frame", "esf_read_frame", "esf_write_frame_async", "esf_frame_wait", "esf_kernel_launches",
    "esf_time_pressure_kernels", "esf_scene_footprint", "esf_server_create", "esf_server_submit",
    "esf_server_poll", "esf_server_wait", "esf_server_get_field", "esf_server_release",
    "esf_server_destroy", "esf_server_batch_stats", "esf_selftest_bounded_wait", "esf_rasterize_solid",
    "esf_solid_load_rest_sdf", "esf_rest_sdf_query", "esf_svol_read",
]


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load the CUDA library (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is not built; run eulersf_gb300/build.py")
        from .build import build
        build()
    lib = C.CDLL(LIB_PATH)
    abi.declare(lib, "esf_", device_pointer_ops=True)
    vp = C.c_void_p
    lib.esf_create.argtypes = [C.POINTER(abi.Grid), C.POINTER(abi.Params), vp, C.POINTER(vp)]
    lib.esf_create.restype = C.c_int
    lib.esf_last_error.restype = C.c_char_p
    lib.esf_abi_version.restype = C.c_int
    lib.esf_pressure_apply.argtypes = [C.POINTER(abi.Grid), vp, vp, vp, vp]
    lib.esf_pressure_solve.argtypes = [C.POINTER(abi.Grid), vp, vp, vp, vp, C.c_double, C.c_int,
                                       C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), vp]
    lib.esf_pressure_solve_batch.argtypes = [C.c_int, C.POINTER(abi.Grid), C.POINTER(vp), C.POINTER(vp),
                                             C.POINTER(vp), C.POINTER(vp), C.c_double, C.c_int, C.c_int,
                                             C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), vp, vp]
    lib.esf_pressure_solve_static.argtypes = [C.POINTER(abi.Grid), vp, vp, vp, vp, C.c_double,
                                              C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                              vp]
    lib.esf_parse_config.argtypes = [C.c_char_p, C.POINTER(abi.Grid), C.POINTER(abi.Params),
                                     C.POINTER(C.c_int), C.c_char_p, C.c_size_t,
                                     C.POINTER(abi.SolidDesc), C.c_int]
    lib.esf_kernel_launches.restype = C.c_uint64
    lib.esf_time_pressure_kernels.argtypes = [vp, C.c_int, C.POINTER(C.c_double),
                                              C.POINTER(C.c_double)]
    lib.esf_write_frame.argtypes = [vp, C.c_char_p, C.c_int, C.c_int]
    from . import serve as _serve
    _serve.declare(lib)
    lib.esf_read_frame.argtypes = [vp, C.c_char_p, C.c_int, C.c_int]
    lib.esf_write_frame_async.argtypes = [vp, C.c_char_p, C.c_int, C.c_int]
    lib.esf_frame_wait.argtypes = [vp]
    lib.esf_rasterize_solid.argtypes = [vp, C.c_int, vp, C.c_int, C.c_double, C.c_double,
                                        C.POINTER(C.c_int), C.POINTER(C.c_double), vp, C.c_size_t,
                                        C.POINTER(C.c_double)]
    lib.esf_selftest_bounded_wait.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.esf_solid_load_rest_sdf.argtypes = [vp, C.c_int, C.c_char_p]
    lib.esf_rest_sdf_query.argtypes = [vp, C.c_int, C.c_int, vp, C.c_double, vp, vp]
    lib.esf_svol_read.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double), vp, vp, C.c_size_t]
    _lib = lib
    return lib


def make_scene(desc: SceneDesc, precision: int = abi.ESF_FP64, noise: bool = True,
          stream: int | None = None, rest_sdf: bool = True) -> CoupledIntegrator3D:
    """GPU integrator for a synthetic scene, set up as the reference's driver
    does (with each solid's rest SDF when the scene has several solids)."""
    return build_from_scene(load(), "esf_", desc, precision=precision, noise=noise, stream=stream,
                            rest_sdf=rest_sdf)


def last_error() -> str:
    return (load().esf_last_error() or b"").decode()

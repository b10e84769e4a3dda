"""Python handle on the multi-scene server of include/eulersf.h
(esf_server_*): submit synthetic rubber-ball scenes, poll or wait for them,
read their fields, release them.

    with Server(max_active=4) as srv:
        t = srv.submit(SceneDesc(N=64, noise_seed=3), steps=10, precision=abi.ESF_MIXED)
        st = srv.wait(t)
        v = srv.get(t, "velocity", 65 ** 3 * 3)
        srv.release(t)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi

ESF_REQ_QUEUED, ESF_REQ_RUNNING, ESF_REQ_DONE, ESF_REQ_FAILED = 0, 1, 2, 3


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_active", C.c_int), ("no_batching", C.c_int),
                ("autotune", C.c_int)]


class BatchStats(C.Structure):
    _fields_ = [("launches", C.c_longlong), ("task_launches", C.c_longlong),
                ("max_tasks", C.c_longlong), ("inner_solves", C.c_longlong),
                ("timed_launches", C.c_longlong), ("timed_rows", C.c_longlong),
                ("timed_ms", C.c_double)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["mean_tasks"] = (self.task_launches / self.launches) if self.launches else 0.0
        # device time of one batched launch, and the one-pass iteration's 48
        # bytes a row it stands for, over the timed launches
        d["launch_ms"] = (self.timed_ms / self.timed_launches) if self.timed_launches else None
        d["launch_gbs"] = (48.0 * self.timed_rows / (self.timed_ms * 1e-3) / 1e9) if self.timed_ms else None
        return d


class Request(C.Structure):
    _fields_ = [("grid", abi.Grid), ("params", abi.Params), ("num_solids", C.c_int),
                ("solids", C.POINTER(abi.SolidDesc)), ("fluid_density", C.c_double),
                ("fluid_viscosity", C.c_double), ("smoke_carpet", C.c_double),
                ("noise_seed", C.c_ulonglong), ("noise_amplitude", C.c_double), ("steps", C.c_int),
                ("rest_sdf_paths", C.POINTER(C.c_char_p))]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int), ("steps_done", C.c_int), ("status", C.c_int),
                ("queued_ms", C.c_double), ("latency_ms", C.c_double), ("device_ms", C.c_double),
                ("footprint_bytes", C.c_size_t), ("last", abi.StepReport)]

    def as_dict(self) -> dict:
        return {"state": self.state, "steps_done": self.steps_done, "status": self.status,
                "queued_ms": self.queued_ms, "latency_ms": self.latency_ms,
                "device_ms": self.device_ms, "footprint_bytes": self.footprint_bytes,
                "last": self.last.as_dict()}


def declare(lib: C.CDLL) -> None:
    vp, u64 = C.c_void_p, C.c_uint64
    lib.esf_scene_footprint.argtypes = [C.POINTER(abi.Grid), C.POINTER(abi.Params), C.c_int,
                                        C.POINTER(abi.SolidDesc)]
    lib.esf_scene_footprint.restype = C.c_size_t
    lib.esf_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(vp)]
    lib.esf_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(u64)]
    lib.esf_server_poll.argtypes = [vp, u64, C.POINTER(RequestStatus)]
    lib.esf_server_wait.argtypes = [vp, u64, C.POINTER(RequestStatus)]
    lib.esf_server_get_field.argtypes = [vp, u64, C.c_int, C.c_int, vp, C.c_size_t]
    lib.esf_server_release.argtypes = [vp, u64]
    lib.esf_server_destroy.argtypes = [vp]
    lib.esf_server_batch_stats.argtypes = [vp, C.POINTER(BatchStats)]


def request_for(desc, steps: int, precision: int = abi.ESF_MIXED):
    """An esf_request for a synthetic scene (scene.py), set up like
    integrator.build_from_scene: the same params, solids, carpet and noise.
    Returns (request, keep-alive objects)."""
    from .integrator import make_solid_desc, params_from_desc
    from .scene import assets_of
    descs, keep = [], []
    for s in desc.solids:
        d, k = make_solid_desc(s.radius, s.center, s.density, s.E, s.nu, s.velocity,
                               s.plastic_yield, s.rotation, s.scaling, s.rotation_matrix,
                               assets=assets_of(s))
        descs.append(d)
        keep.extend(k)
    arr = (abi.SolidDesc * len(descs))(*descs)
    res = desc.res
    q = Request()
    q.grid = abi.Grid(res, res, res, desc.dh, (C.c_double * 3)(0, 0, 0))
    q.params = params_from_desc(desc, precision)
    q.num_solids = len(descs)
    q.solids = C.cast(arr, C.POINTER(abi.SolidDesc))
    q.fluid_density = desc.fluid_density
    q.fluid_viscosity = 0.0
    q.smoke_carpet = desc.fluid_height
    q.noise_seed = desc.noise_seed
    q.noise_amplitude = desc.noise_amplitude
    q.steps = steps
    if len(desc.solids) > 1:  # rest SDFs for solid-solid contact
        from .integrator import sphere_svol_path
        paths = (C.c_char_p * len(desc.solids))(*[sphere_svol_path(s.radius).encode() for s in desc.solids])
        q.rest_sdf_paths = C.cast(paths, C.POINTER(C.c_char_p))
        keep.append(paths)
    return q, (arr, keep)


class Server:
    def __init__(self, hbm_budget_bytes: int = 0, max_active: int = 0, lib=None, batching: bool = True,
                 autotune: bool = False):
        from . import load
        self._lib = lib or load()
        cfg = ServerConfig(hbm_budget_bytes, max_active, 0 if batching else 1, 1 if autotune else 0)
        h = C.c_void_p()
        st = self._lib.esf_server_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise abi.EsfError(st, "esf_server_create", self._err())
        self._h = h

    def _err(self):
        return (self._lib.esf_last_error() or b"").decode()

    def submit(self, desc, steps: int, precision: int = abi.ESF_MIXED) -> int:
        q, keep = request_for(desc, steps, precision)
        t = C.c_uint64()
        st = self._lib.esf_server_submit(self._h, C.byref(q), C.byref(t))
        if st != 0:
            raise abi.EsfError(st, "esf_server_submit", self._err())
        del keep  # the server copied everything it needs
        return t.value

    def poll(self, ticket: int) -> dict:
        s = RequestStatus()
        st = self._lib.esf_server_poll(self._h, ticket, C.byref(s))
        if st != 0:
            raise abi.EsfError(st, "esf_server_poll", self._err())
        return s.as_dict()

    def wait(self, ticket: int) -> dict:
        s = RequestStatus()
        st = self._lib.esf_server_wait(self._h, ticket, C.byref(s))
        if st != 0:
            raise abi.EsfError(st, "esf_server_wait", self._err())
        return s.as_dict()

    def get(self, ticket: int, name: str, count: int, solid: int = 0) -> np.ndarray:
        """Field `name` (abi.FIELDS) of a finished request; `count` elements
        (e.g. nodes x 3 for the velocity, cells for lambda1)."""
        fid, dtype, comp = abi.FIELDS[name]
        out = np.empty(count, dtype=dtype)
        st = self._lib.esf_server_get_field(self._h, ticket, fid, solid,
                                            out.ctypes.data_as(C.c_void_p), out.nbytes)
        if st != 0:
            raise abi.EsfError(st, "esf_server_get_field", self._err())
        return out.reshape(-1, comp) if comp > 1 else out

    def release(self, ticket: int) -> None:
        st = self._lib.esf_server_release(self._h, ticket)
        if st != 0:
            raise abi.EsfError(st, "esf_server_release", self._err())

    def batch_stats(self) -> dict:
        """Counters of the continuous batching of inner solves (esf_server_batch_stats)."""
        b = BatchStats()
        st = self._lib.esf_server_batch_stats(self._h, C.byref(b))
        if st != 0:
            raise abi.EsfError(st, "esf_server_batch_stats", self._err())
        return b.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.esf_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

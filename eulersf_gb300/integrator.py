"""Host-side mirror of the reference's driver -> integrator call surface.

``CoupledIntegrator3D`` keeps the method names of COUPLED_INTEGRATOR_3D
(include/integrator/COUPLED_INTEGRATOR_3D.h:29-78) over a C-ABI scene
(include/eulersf.h), and ``build_from_scene`` replays the set-up order of
projects/rubberBall/main.cpp:63-160 (integrator, solids, fluid, init, smoke
carpet). The backend is the CUDA library (eulersf_gb300.lib); the CPU
oracle's Python wrapper drives its own library through the same class.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .scene import SceneDesc, assets_of, lame, noise_field, solid_assets


class CoupledIntegrator3D:
    def __init__(self, lib, prefix, xRes, yRes, zRes, dh, origin=(0.0, 0.0, 0.0),
                 params: abi.Params | None = None, stream: int | None = None):
        self._lib, self._p = lib, prefix
        self.grid = abi.Grid(xRes, yRes, zRes, dh, (C.c_double * 3)(*origin))
        if params is None:
            params = abi.Params()
            self._call("params_default", C.byref(self.grid), C.byref(params))
        self.params = params
        fn = getattr(lib, prefix + "create")
        if prefix == "esf_":
            out = C.c_void_p()
            st = fn(C.byref(self.grid), C.byref(params), C.c_void_p(stream or 0), C.byref(out))
            if st != 0:
                raise abi.EsfError(st, "esf_create", self.last_error())
            self._h = out
        else:
            h = fn(C.byref(self.grid), C.byref(params))
            if not h:
                raise abi.EsfError(1, prefix + "create")
            self._h = C.c_void_p(h)
        self._keep = []

    # ------------------------------------------------------------ plumbing
    def last_error(self) -> str:
        f = getattr(self._lib, self._p + "last_error", None)
        if f is None:
            return ""
        f.restype = C.c_char_p
        return (f() or b"").decode()

    def _call(self, name, *args):
        st = getattr(self._lib, self._p + name)(*args)
        if st != 0:
            raise abi.EsfError(st, self._p + name, self.last_error())
        return st

    def close(self):
        if getattr(self, "_h", None):
            getattr(self._lib, self._p + "destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------- reference call surface
    def xRes(self):
        return self.grid.xRes

    def yRes(self):
        return self.grid.yRes

    def zRes(self):
        return self.grid.zRes

    def dh(self):
        return self.grid.dh

    def origin(self):
        return tuple(self.grid.origin)

    def addSolid(self, desc: abi.SolidDesc, keep=()):
        self._keep.extend(keep)
        self._call("add_solid", self._h, C.byref(desc))

    def loadRestSDF(self, solid: int, path: str):
        """DEFOR_SOLID_3D::loadRestSDF (DEFOR_SOLID_3D.cpp:210-214) of solid i."""
        self._call("solid_load_rest_sdf", self._h, int(solid), path.encode())

    def restSdfQuery(self, solid: int, points, safe_dist: float):
        """SPARSE_SDF::signedDistAndCurrentNormal of solid i at rest points
        (n x 3): (distances, normals n x 3)."""
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        n = len(pts)
        sd = np.zeros(n)
        nrm = np.zeros((n, 3))
        self._call("rest_sdf_query", self._h, int(solid), n, pts.ctypes.data, C.c_double(safe_dist),
                   sd.ctypes.data, nrm.ctypes.data)
        return sd, nrm

    def setFluidDensity(self, d):
        self._fluid = (d, getattr(self, "_fluid", (1.0, 0.0))[1])
        self._call("set_fluid", self._h, C.c_double(self._fluid[0]), C.c_double(self._fluid[1]))

    def setFluidViscocity(self, v):
        self._fluid = (getattr(self, "_fluid", (1.0, 0.0))[0], v)
        self._call("set_fluid", self._h, C.c_double(self._fluid[0]), C.c_double(self._fluid[1]))

    def init(self):
        self._call("init", self._h)

    def setMaxDt(self, dt):
        self._call("set_max_dt", self._h, C.c_double(dt))

    def stepImplicit(self) -> dict:
        rep = abi.StepReport()
        st = getattr(self._lib, self._p + "step")(self._h, C.byref(rep))
        if st not in (0, 6):  # ESF_ERR_NUMERIC still completes the step
            raise abi.EsfError(st, self._p + "step", self.last_error())
        return rep.as_dict()

    def dt(self) -> float:
        return getattr(self._lib, self._p + "dt")(self._h)

    def writeFrame(self, frame: int, debug: bool = False, data_path: str = ""):
        """COUPLED_INTEGRATOR_3D::writeFrame: files "<data_path>frame.NNNN.*"."""
        self._call("write_frame", self._h, data_path.encode(), int(frame), int(bool(debug)))

    def writeFrameAsync(self, frame: int, debug: bool = False, data_path: str = ""):
        """writeFrame through pinned memory and a writer thread; returns at once
        (esf_write_frame_async). frameWait() waits for it."""
        self._call("write_frame_async", self._h, data_path.encode(), int(frame), int(bool(debug)))

    def frameWait(self):
        self._call("frame_wait", self._h)

    def readFrame(self, frame: int, debug: bool = False, data_path: str = ""):
        """COUPLED_INTEGRATOR_3D::readFrame of files written by writeFrame (or the reference)."""
        self._call("read_frame", self._h, data_path.encode(), int(frame), int(bool(debug)))

    # ------------------------------------------------------------ fields
    def field_info(self, name, solid=0):
        fid, dtype, comp = abi.FIELDS[name]
        n, eb = C.c_size_t(), C.c_size_t()
        self._call("field_info", self._h, fid, solid, C.byref(n), C.byref(eb))
        return n.value, eb.value

    def get(self, name, solid=0) -> np.ndarray:
        fid, dtype, comp = abi.FIELDS[name]
        n, eb = self.field_info(name, solid)
        out = np.empty(n, dtype=dtype)
        assert out.itemsize == eb
        self._call("get_field", self._h, fid, solid, out.ctypes.data_as(C.c_void_p),
                   C.c_size_t(out.nbytes))
        if comp > 1:
            out = out.reshape(-1, comp)
        return out

    def set(self, name, values, solid=0):
        fid, dtype, comp = abi.FIELDS[name]
        arr = np.ascontiguousarray(values, dtype=dtype).reshape(-1)
        self._call("set_field", self._h, fid, solid, arr.ctypes.data_as(C.c_void_p),
                   C.c_size_t(arr.nbytes))

    def intensity(self):
        return self.get("intensity")


def make_solid_desc(radius, center, density, E, nu, velocity=(0, 0, 0), plastic_yield=-1.0,
                    rotation=(0.0, 0.0, 0.0), scaling=(1.0, 1.0, 1.0), rotation_matrix=None,
                    assets=None):
    """Solid descriptor for the synthetic sphere (rest assets from scene.py,
    or the given (mass field, vertices, triangles)); `rotation` in the cfg's
    units (angles / pi), or an exact `rotation_matrix`."""
    from .scene import rotation_matrix as _rot
    (res, mdh, morig, mdata), verts, faces = assets if assets is not None else solid_assets(radius)
    lam, mu = lame(E, nu)
    rest = np.ascontiguousarray(mdata.reshape(-1), dtype=np.float64)
    v = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1)
    t = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1)
    d = abi.SolidDesc()
    d.mass_res[:] = list(res)
    d.mass_dh = mdh
    d.mass_origin[:] = [float(x) for x in morig]
    d.rest_mass = rest.ctypes.data_as(C.POINTER(C.c_double))
    d.lambda_, d.mu, d.density = lam, mu, density
    rm = rotation_matrix if rotation_matrix is not None else _rot(rotation).reshape(-1)
    d.rotation[:] = [float(x) for x in np.asarray(rm).reshape(-1)]
    d.translation[:] = [float(x) for x in center]
    d.scaling[:] = [float(x) for x in scaling]
    d.initial_velocity[:] = [float(x) for x in velocity]
    d.num_vertices = len(verts)
    d.vertices = v.ctypes.data_as(C.POINTER(C.c_double))
    d.num_triangles = len(faces)
    d.triangles = t.ctypes.data_as(C.POINTER(C.c_int))
    d.plastic_yield = float(plastic_yield)
    return d, (rest, v, t)


_SVOL_DIR = None


def sphere_svol_path(radius: float) -> str:
    """A ".svol" rest SDF of the synthetic sphere of this radius, written
    once per process into a private temporary directory."""
    global _SVOL_DIR
    import tempfile
    from .svol import sphere_svol
    if _SVOL_DIR is None:
        _SVOL_DIR = tempfile.mkdtemp(prefix="esf_svol_")
    path = os.path.join(_SVOL_DIR, f"sphere_{float(radius)!r}.svol")
    if not os.path.exists(path):
        sphere_svol(path + ".tmp", radius)
        os.replace(path + ".tmp", path)
    return path


def params_from_desc(desc: SceneDesc, precision: int = abi.ESF_FP64) -> abi.Params:
    dh = desc.dh
    p = abi.Params()
    p.dt = desc.dt
    p.fluid_density = desc.fluid_density
    p.fluid_viscosity = 0.0
    p.vorticity_eps = desc.vorticity_eps
    p.buoyancy = desc.buoyancy
    p.gravity = desc.gravity
    p.rayleigh_alpha = p.rayleigh_beta = 0.0
    p.implicit_solver_eps = p.div_free_solver_eps = desc.eps
    p.cr_max_iterations = desc.max_iters
    p.mass_sample_dh = desc.mass_sample_dh
    p.tight_border = desc.tight_border
    p.extrapolation_cells = desc.extrapolation_cells
    p.particles_per_cell = desc.particles_per_cell
    p.flip_alpha = desc.flip_alpha
    p.contact_safe_distance = 0.5 * dh
    p.wall_thickness = 1.5 * dh
    p.contact_spring_stiffness = 10000.0
    p.friction = 0.5
    p.flip_cutoff = 3
    p.flow_rate = desc.flow_rate
    p.precision = precision
    p.inner_eps = desc.inner_eps
    p.max_refinements = 50
    return p


def build_from_scene(lib, prefix, desc: SceneDesc, precision=abi.ESF_FP64, noise=True,
                     stream=None, rest_sdf=True) -> CoupledIntegrator3D:
    """APPLICATION::init (main.cpp:63-97) for a synthetic scene: integrator,
    solids, fluid density, init(), smoke carpet, then the seeded fluid noise
    added at nodes without solid mass."""
    res = desc.res
    if len(desc.solids) > 1 and rest_sdf and not hasattr(lib, prefix + "solid_load_rest_sdf"):
        raise NotImplementedError(f"{prefix}: scenes with several solids need solid-solid contact, "
                                  "which this library does not provide")
    I = CoupledIntegrator3D(lib, prefix, res, res, res, desc.dh, (0.0, 0.0, 0.0),
                            params_from_desc(desc, precision), stream=stream)
    for i, s in enumerate(desc.solids):
        d, keep = make_solid_desc(s.radius, s.center, s.density, s.E, s.nu, s.velocity,
                                  s.plastic_yield, s.rotation, s.scaling, s.rotation_matrix,
                                  assets=assets_of(s))
        I.addSolid(d, keep)
        if len(desc.solids) > 1 and rest_sdf:
            I.loadRestSDF(i, sphere_svol_path(s.radius))
    I.setFluidDensity(desc.fluid_density)
    I.setFluidViscocity(0.0)
    I.init()
    carpet = int(desc.fluid_height / desc.dh)
    inten = I.get("intensity").reshape(res, res, res)
    inten[1:res - 1, 1:max(carpet, 1), 1:res - 1] = float(np.float32(0.8))  # "0.8f"
    I.set("intensity", inten)
    if noise and desc.noise_amplitude > 0:
        v = I.get("velocity")
        m = I.get("solidMass")
        nz = noise_field(res, desc.noise_seed, desc.noise_amplitude)
        v[m == 0] += nz[m == 0]
        I.set("velocity", v)
    return I


def run_frames(I: CoupledIntegrator3D, frames: int, frame_dt: float, on_step=None):
    """APPLICATION::step (main.cpp:174-204): each frame substeps until the
    frame time is covered; returns the per-substep reports."""
    reports = []
    for f in range(frames):
        sim = 0.0
        while sim < frame_dt:
            I.setMaxDt(frame_dt - sim)
            r = I.stepImplicit()
            sim += I.dt()
            r["frame"] = f
            reports.append(r)
            if on_step:
                on_step(len(reports), r)
    return reports

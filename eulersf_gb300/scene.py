"""Synthetic rubber-ball scenes in the reference's own input formats.

A scene is what projects/rubberBall/main.cpp:63-160 reads: a ``key = value``
config (SIMPLE_PARSER, src/util/SIMPLE_PARSER.cpp:64-117), a rest-pose mass
grid ``<solid>.mass`` in the gz layout of FIELD_3D::writeGz
(include/geometry/FIELD_3D.h:299-321) and a surface mesh ``<solid>.obj``.

The grid convention maps "N^3 cells in the unit cube" to ``xRes = N + 1``
nodes per axis, ``dh = 1/N``, ``origin = 0,0,0`` (node i sits at i*dh,
DEFOR_SOLID_3D.cpp:134-136), so there are exactly N^3 pressure rows.

Inputs that stand in for the reference's shipped assets (meshes/sphere/*):

* rest mass: an analytic rasterisation of a sphere of the scene's radius r
  that follows projects/rasterizeSolid/main.cpp:44-72 (bbox expanded by
  10*mass_dh, ``int`` resolution, density where the signed distance is
  <= mass_dh/2) with the exact sphere distance in place of the DT-Grid SDF,
  on a grid of mass_dh = r/100 (the shipped 0.1-radius sphere uses 0.001);
* surface mesh: a subdivided icosahedron of radius r (only its vertex
  AABB drives the step, via the CFL factor, COUPLED_INTEGRATOR_3D.cpp:386-410);
* ``solid scaling`` defaults to 1: the reference treats it as a deformation
  of the rest shape (X = R^T (x - T) / s, DEFOR_SOLID_3D.cpp:126-152), so a
  scaled ball starts stretched (F = s I);
* rest SDF (scenes with more than one solid, for solid-solid contact): the
  exact distance of the sphere on a DT-Grid narrow band (svol.py) in place of
  the shipped ``sphere.svol``;
* fluid noise: U(-a, a) per component at interior nodes from a counter-based
  splitmix64 stream keyed by (seed, node, component), so that C, CUDA and
  numpy produce the same values.
"""
from __future__ import annotations

import gzip
import os
import struct
from dataclasses import dataclass, field

import numpy as np

from .svol import sphere_svol

REST_RADIUS = 0.1
REST_MASS_DH = 0.001
REST_DENSITY = 1000.0


def lame(E: float, nu: float) -> tuple[float, float]:
    """Lame parameters from Young's modulus and Poisson ratio."""
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    return lam, mu


def _fmt(v) -> str:
    if isinstance(v, str):
        return v
    if isinstance(v, (tuple, list, np.ndarray)):
        return ",".join(_fmt(x) for x in v)
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return repr(float(v))


@dataclass
class SolidDesc:
    center: tuple = (0.5, 0.65, 0.5)
    radius: float = 0.15
    density: float = 1100.0
    E: float = 2e5
    nu: float = 0.45
    velocity: tuple = (0.0, 0.0, 0.0)
    plastic_yield: float = -1.0  # "solid plastic yield i"; <= 0: elastic
    rotation: tuple = (0.0, 0.0, 0.0)  # "solid rotation i": angles about x, y, z in units of pi
    scaling: tuple = (1.0, 1.0, 1.0)   # "solid scaling i" (deforms the rest shape)
    # the 3x3 rotation (row-major) the reference built from `rotation`, when
    # known exactly (golden fixtures); otherwise computed by rotation_matrix()
    rotation_matrix: tuple | None = None
    # registered rest assets (register_assets) in place of the synthetic
    # sphere of `radius`, e.g. the reference's shipped mesh and baked mass
    asset: str = ""


@dataclass
class SceneDesc:
    """One coupled scene (the rubber-ball family of the benchmark configurations)."""
    N: int = 64
    solids: list = field(default_factory=lambda: [SolidDesc()])
    fluid_height: float = 0.3
    fluid_density: float = 1000.0
    gravity: float = 9.8
    dt: float = 1.0 / 240.0
    eps: float = 1e-8
    max_iters: int = 200000
    vorticity_eps: float = 0.0
    buoyancy: float = 0.0
    mass_sample_dh: float = 0.00125
    particles_per_cell: int = 32
    flip_alpha: float = 0.99
    extrapolation_cells: int = 20
    tight_border: int = 5
    noise_amplitude: float = 1e-3
    noise_seed: int = 0
    inner_eps: float = 1e-4  # mixed precision: FP32 inner relative tolerance
    flow_rate: float = 0.5   # "flow rate" of the plastic update

    @property
    def res(self) -> int:
        return self.N + 1

    @property
    def dh(self) -> float:
        return 1.0 / self.N

    def config(self, solid_dir: str = "./", solid_name: str = "sphere") -> dict:
        """The reference's cfg keys for this scene (main.cpp:64-141 and the
        keys listed at each SIMPLE_PARSER read site on the step path)."""
        dh = self.dh
        c = {
            "xRes": self.res, "yRes": self.res, "zRes": self.res,
            "dh": dh, "origin": (0.0, 0.0, 0.0),
            "number of solids": len(self.solids),
            "fluid density": self.fluid_density, "fluid viscocity": 0.0,
            "vorticity eps": self.vorticity_eps, "buoyancy": self.buoyancy,
            "smoke carpet thickness": self.fluid_height,
            "wall thickness": 1.5 * dh, "contact safe distance": 0.5 * dh,
            "contact spring stiffness": 10000.0, "friction": 0.5,
            "flip alpha": self.flip_alpha, "dt": self.dt, "gravity": self.gravity,
            "extrapolation cells": self.extrapolation_cells,
            "tight border": self.tight_border,
            "rayleigh alpha": 0.0, "rayleigh beta": 0.0,
            "cr max iterations": self.max_iters,
            "implicit solver eps": self.eps, "div free solver eps": self.eps,
            "number of particles per material cell": self.particles_per_cell,
            "mass sample dh": self.mass_sample_dh, "flip cutoff": 3,
            "flow rate": self.flow_rate,
        }
        for i, s in enumerate(self.solids):
            lam, mu = lame(s.E, s.nu)
            c.update({
                f"solid path {i}": solid_dir, f"solid name {i}": f"{solid_name}{i}",
                f"solid mass density {i}": s.density,
                f"material lambda {i}": lam, f"material mu {i}": mu,
                f"solid plastic yield {i}": s.plastic_yield,
                f"solid initial velocity {i}": tuple(s.velocity),
                f"solid translation {i}": tuple(s.center),
                f"solid scaling {i}": tuple(s.scaling),
                f"solid rotation {i}": tuple(s.rotation),
            })
        return c


def write_cfg(path: str, cfg: dict) -> None:
    with open(path, "w") as f:
        for k, v in cfg.items():
            f.write(f"{k} = {_fmt(v)}\n")


def parse_cfg(path: str) -> dict:
    """SIMPLE_PARSER::parse semantics: '#' comment lines, 'lhs = rhs',
    both sides trimmed and lowercased (SIMPLE_PARSER.cpp:64-117)."""
    vals = {}
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line or line[0] == "#":
                continue
            if "=" in line:
                lhs, rhs = line.split("=", 1)
                vals[lhs.strip().lower()] = rhs.strip().lower()
            elif line.strip():
                raise ValueError(f"unable to parse line: {line!r}")
    return vals


# --------------------------------------------------------------- rest mass
def rest_mass_field(radius: float = REST_RADIUS, mass_dh: float | None = None,
                    density: float = REST_DENSITY):
    """Rest-pose mass grid of a sphere, laid out like rasterizeSolid's output.

    Returns (res[3], dh, origin[3], data[z, y, x] float64)."""
    if mass_dh is None:
        mass_dh = radius / 100.0
    boxmin = np.full(3, -radius) - 10 * mass_dh
    boxmax = np.full(3, radius) + 10 * mass_dh
    res = [int((boxmax[k] - boxmin[k]) / mass_dh) for k in range(3)]
    z = np.arange(res[2]) * mass_dh + boxmin[2]
    y = np.arange(res[1]) * mass_dh + boxmin[1]
    x = np.arange(res[0]) * mass_dh + boxmin[0]
    r = np.sqrt(z[:, None, None] ** 2 + y[None, :, None] ** 2 + x[None, None, :] ** 2)
    data = np.where(r - radius <= mass_dh / 2, density, 0.0).astype(np.float64)
    return res, mass_dh, boxmin.astype(np.float64), data


def write_field_gz(path: str, res, dh, origin, data) -> None:
    """FIELD_3D::writeGz layout: 3 int32 dims, 4 float64 (dh, origin), then
    float64 data in x-fastest order."""
    hdr = struct.pack("<3i4d", int(res[0]), int(res[1]), int(res[2]), float(dh),
                      float(origin[0]), float(origin[1]), float(origin[2]))
    with gzip.open(path, "wb", compresslevel=1) as f:
        f.write(hdr)
        f.write(np.ascontiguousarray(data, dtype="<f8").tobytes())


def read_field_gz(path: str):
    with gzip.open(path, "rb") as f:
        raw = f.read()
    xr, yr, zr, dh, ox, oy, oz = struct.unpack("<3i4d", raw[:44])
    data = np.frombuffer(raw[44:], dtype="<f8")
    ncomp = data.size // (xr * yr * zr)
    shape = (zr, yr, xr) if ncomp == 1 else (zr, yr, xr, ncomp)
    return (xr, yr, zr), dh, np.array([ox, oy, oz]), data.reshape(shape)


# ------------------------------------------------------------- surface mesh
def icosphere(level: int = 3, radius: float = REST_RADIUS):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
         (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, float) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9),
             (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2),
             (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts) * radius, np.array(faces, dtype=np.int32)


def write_obj(path: str, verts, faces) -> None:
    with open(path, "w") as f:
        for p in verts:
            f.write(f"v {float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
        for a, b, c in faces:
            f.write(f"f {a + 1} {b + 1} {c + 1}\n")


# -------------------------------------------------------------------- noise
_M64 = (1 << 64) - 1


def noise_field(res: int, seed: int, amplitude: float = 1e-3) -> np.ndarray:
    """U(-a, a) per component at interior nodes, zero on the boundary faces.

    value = a * (2 * u - 1) with u = (splitmix64(seed * 2^40 + 3 * node + comp)
    >> 11) * 2^-53.  Shape (res^3, 3), node index x + y*res + z*res^2."""
    n = res ** 3
    idx = (np.arange(n, dtype=np.uint64)[:, None] * np.uint64(3)
           + np.arange(3, dtype=np.uint64)[None, :])
    with np.errstate(over="ignore"):
        z = idx + np.uint64((seed << 40) & _M64)
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    v = amplitude * (2.0 * u - 1.0)
    k = np.arange(n)
    x, y, zz = k % res, (k // res) % res, k // (res * res)
    interior = (x > 0) & (x < res - 1) & (y > 0) & (y < res - 1) & (zz > 0) & (zz < res - 1)
    v[~interior] = 0.0
    return v


_CACHE = {}


def solid_assets(radius: float):
    """(rest mass field, mesh vertices, mesh triangles) of a sphere of radius r."""
    key = float(radius)
    if key not in _CACHE:
        _CACHE[key] = (rest_mass_field(radius), *icosphere(3, radius))
        if len(_CACHE) > 8:
            _CACHE.pop(next(iter(_CACHE)))
    return _CACHE[key]


_ASSETS = {}


def register_assets(name: str, mass_field, verts, faces) -> None:
    """Rest assets for solids whose ``asset`` names them: the rest mass grid
    (res, dh, origin, data[z, y, x]) and the closed surface mesh."""
    _ASSETS[name] = (mass_field, np.asarray(verts, dtype=np.float64),
                     np.asarray(faces, dtype=np.int32))


def assets_of(s: SolidDesc):
    """(rest mass field, mesh vertices, mesh triangles) of a solid."""
    if s.asset:
        if s.asset not in _ASSETS:
            raise KeyError(f"rest assets {s.asset!r} are not registered")
        return _ASSETS[s.asset]
    return solid_assets(s.radius)


def write_scene(desc: SceneDesc, directory: str, name: str = "sphere") -> str:
    """Write cfg + assets + noise into ``directory``; returns the cfg path.
    Solid i's assets are ``<name><i>.mass`` and ``<name><i>.obj``."""
    os.makedirs(directory, exist_ok=True)
    solid_dir = os.path.abspath(directory) + "/"
    cfg = desc.config(solid_dir=solid_dir, solid_name=name)
    cfg_path = os.path.join(directory, "scene.cfg")
    write_cfg(cfg_path, cfg)
    for i, s in enumerate(desc.solids):
        (res, mdh, morig, mdata), verts, faces = assets_of(s)
        write_field_gz(os.path.join(directory, f"{name}{i}.mass"), res, mdh, morig, mdata)
        write_obj(os.path.join(directory, f"{name}{i}.obj"), verts, faces)
        if len(desc.solids) > 1:  # rest SDF for solid-solid contact (main.cpp:146-148)
            sphere_svol(os.path.join(directory, f"{name}{i}.svol"), s.radius)
    noise = noise_field(desc.res, desc.noise_seed, desc.noise_amplitude)
    noise.astype("<f8").tofile(os.path.join(directory, "noise.f64"))
    return cfg_path


def pressure_problem(desc: SceneDesc, seed: int = 0):
    """A pressure system of the scene's size, for the solver seam alone:
    node m^-1 of the fluid (rho_f dh^3) with the sphere's nodes also carrying
    solid mass (boundary nodes carry no unknown), the Jacobi diagonal of
    J diag(m^-1) J^T (3 m^-1 summed over each cell's DOF corners) and a
    seeded standard-normal right-hand side. Returns (minv, diag, b) as
    float64 arrays of X^3, N^3 and N^3 entries. The cost of a PCR iteration
    depends only on the grid, not on these values."""
    res, N, dh = desc.res, desc.N, desc.dh
    s = desc.solids[0]
    z, y, x = np.meshgrid(*(np.arange(res) * dh,) * 3, indexing="ij")
    fluid = desc.fluid_density * dh ** 3
    inside = (x - s.center[0]) ** 2 + (y - s.center[1]) ** 2 + (z - s.center[2]) ** 2 <= s.radius ** 2
    mass = fluid + np.where(inside, s.density * dh ** 3, 0.0)
    minv = (1.0 / mass).reshape(-1)
    m = minv.reshape(res, res, res).copy()
    m[0], m[-1], m[:, 0], m[:, -1], m[:, :, 0], m[:, :, -1] = 0, 0, 0, 0, 0, 0
    diag = np.zeros((N, N, N))
    for i in range(8):
        dx, dy, dz = i & 1, (i >> 1) & 1, (i >> 2) & 1
        diag += 3 * m[dz:dz + N, dy:dy + N, dx:dx + N]
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(N ** 3)
    return minv, diag.reshape(-1), b


def rotation_matrix(angles) -> np.ndarray:
    """Rx(a pi) Ry(b pi) Rz(c pi) (main.cpp:131-136), row-major 3x3. The
    reference forms it through Eigen quaternions, so the last bits can
    differ; golden fixtures carry the reference's own matrix instead."""
    a, b, c = (float(x) * np.pi for x in angles)
    rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
    rz = np.array([[np.cos(c), -np.sin(c), 0], [np.sin(c), np.cos(c), 0], [0, 0, 1]])
    return rx @ ry @ rz

"""Headless stand-in for the reference's rubberBall application
(projects/rubberBall/main.cpp:30-270): reads a reference cfg with the same
keys, loads each solid's ``<path><name>.mass`` (FIELD_3D gz layout) and
``<path><name>.obj``, sets up the integrator in the order of
APPLICATION::init/addSolids, seeds the smoke carpet, and runs frames with
APPLICATION::step's substep loop on the GPU. Instead of GLUT windows it
prints one JSON line per substep. With "save data = true" it writes each
frame's files under "data path" (main.cpp:198-199); a "start frame" above 0
resumes from the previous frame's files (main.cpp:95).

    python -m eulersf_gb300.driver scene.cfg [frames] [--mixed | --mixed-x64]

--mixed: FP32 inner solves in FP64 iterative refinement; --mixed-x64: one
FP32 Krylov run per pressure solve with its iterate and direction in FP64
(ESF_MIXED_X64). Without either, the plain FP64 method.
"""
from __future__ import annotations

import ctypes as C
import json
import sys

import numpy as np

from . import abi, load
from .integrator import CoupledIntegrator3D, run_frames
from .scene import parse_cfg, read_field_gz, rotation_matrix


def read_obj(path):
    """Vertices and triangles of an OBJ (``v`` and ``f`` records; polygon
    faces fanned into triangles, ``a/b/c`` index forms accepted)."""
    verts, tris = [], []
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "v":
                verts.append([float(x) for x in p[1:4]])
            elif p[0] == "f":
                idx = [int(t.split("/")[0]) for t in p[1:]]
                idx = [i - 1 if i > 0 else len(verts) + i for i in idx]
                for k in range(1, len(idx) - 1):
                    tris.append([idx[0], idx[k], idx[k + 1]])
    return np.array(verts, dtype=np.float64), np.array(tris, dtype=np.int32)


def run(cfg_path, frames=None, precision=abi.ESF_FP64, out=sys.stdout):
    lib = load()
    cfg = parse_cfg(cfg_path)
    g, p, n = abi.Grid(), abi.Params(), C.c_int()
    st = lib.esf_parse_config(cfg_path.encode(), C.byref(g), C.byref(p), C.byref(n), None, 0, None, 0)
    if st != 0:
        raise abi.EsfError(st, "esf_parse_config", (lib.esf_last_error() or b"").decode())
    p.precision = precision
    I = CoupledIntegrator3D(lib, "esf_", g.xRes, g.yRes, g.zRes, g.dh, tuple(g.origin), p)

    def vec(key, default):
        return tuple(float(x) for x in cfg[key].split(",")) if key in cfg else default

    for i in range(n.value):
        base = cfg.get(f"solid path {i}", "") + cfg.get(f"solid name {i}", "")
        res, mdh, morig, mdata = read_field_gz(base + ".mass")
        verts, tris = read_obj(base + ".obj")
        d = abi.SolidDesc()
        rest = np.ascontiguousarray(mdata.reshape(-1))
        v = np.ascontiguousarray(verts.reshape(-1))
        t = np.ascontiguousarray(tris.reshape(-1))
        d.mass_res[:] = list(res)
        d.mass_dh = mdh
        d.mass_origin[:] = [float(x) for x in morig]
        d.rest_mass = rest.ctypes.data_as(C.POINTER(C.c_double))
        d.lambda_ = float(cfg.get(f"material lambda {i}", 100))
        d.mu = float(cfg.get(f"material mu {i}", 100))
        d.density = float(cfg.get(f"solid mass density {i}", 1))
        d.rotation[:] = list(rotation_matrix(vec(f"solid rotation {i}", (0, 0, 0))).reshape(-1))
        d.translation[:] = list(vec(f"solid translation {i}", (0, 0, 0)))
        d.scaling[:] = list(vec(f"solid scaling {i}", (1, 1, 1)))
        d.initial_velocity[:] = list(vec(f"solid initial velocity {i}", (0, 0, 0)))
        d.num_vertices, d.vertices = len(verts), v.ctypes.data_as(C.POINTER(C.c_double))
        d.num_triangles, d.triangles = len(tris), t.ctypes.data_as(C.POINTER(C.c_int))
        d.plastic_yield = float(cfg.get(f"solid plastic yield {i}", -1))
        I.addSolid(d, keep=(rest, v, t))
        # main.cpp:146-148; a rest SDF is only read by solid-solid contact
        if n.value > 1:
            I.loadRestSDF(i, base + ".svol")
    I.setFluidDensity(float(cfg.get("fluid density", 1)))
    I.setFluidViscocity(float(cfg.get("fluid viscocity", 0)))
    I.init()
    # smoke carpet (main.cpp:80-90): 0.8f in layers 1 .. carpet-1
    carpet = int(float(cfg.get("smoke carpet thickness", 0.06)) / g.dh)
    inten = I.get("intensity").reshape(g.zRes, g.yRes, g.xRes)
    inten[1:g.zRes - 1, 1:max(carpet, 1), 1:g.xRes - 1] = float(np.float32(0.8))
    I.set("intensity", inten)
    start = int(float(cfg.get("start frame", 0)))
    end = int(float(cfg.get("end frame", 100)))
    nframes = frames if frames is not None else end - start
    frame_dt = float(cfg.get("dt", 0.005))
    data_path = cfg.get("data path", "")
    save = cfg.get("save data", "false") in ("1", "true")
    debug = cfg.get("debug", "false") in ("1", "true")
    # main.cpp:95: resume from the previous frame's files
    if start > 0:
        I.readFrame(start - 1, debug, data_path)

    reports = []
    for f in range(start, start + nframes):
        def report(k, r, f=f):
            r["frame"] = f
            reports.append(r)
            out.write(json.dumps({"substep": len(reports), **r}) + "\n")
            out.flush()

        run_frames(I, 1, frame_dt, on_step=report)
        if save:  # main.cpp:198-199
            I.writeFrame(f, debug, data_path)
    I.close()
    return reports


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    prec = (abi.ESF_MIXED_X64 if "--mixed-x64" in argv else
            abi.ESF_MIXED if "--mixed" in argv else abi.ESF_FP64)
    argv = [a for a in argv if a not in ("--mixed", "--mixed-x64")]
    if not argv:
        print(__doc__)
        return 2
    frames = int(argv[1]) if len(argv) > 1 else None
    run(argv[0], frames, prec)
    return 0


if __name__ == "__main__":
    sys.exit(main())

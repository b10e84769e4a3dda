"""The C++ facade (include/eulersf.hpp) and the cfg driver
(eulersf_gb300/driver.py): the two ways a reference user drives the step
without Python glue of their own.

CPU: the facade compiles and links against the library, and reports a
missing device as esf::Error (exit 3). GPU: one facade step equals the same
step through the Python integrator bit for bit, and the cfg driver's first
substep equals a step of the same scene built in memory."""
import ctypes as C
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from common import ROOT

from eulersf_gb300 import abi
from eulersf_gb300.integrator import make_solid_desc, params_from_desc
from eulersf_gb300.scene import SceneDesc, lame, solid_assets, write_scene

DESC = SceneDesc(N=16, mass_sample_dh=(1.0 / 16) / 4)


def _build_facade(tmp_path):
    import eulersf_gb300 as E
    E.load(build_if_missing=True)
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "facade_step")
    libdir = os.path.dirname(E.LIB_PATH)
    cmd = [cxx, "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_step.cpp"), "-o", exe,
           "-L", libdir, "-leulersf_gb300", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _write_inputs(d, desc):
    os.makedirs(d, exist_ok=True)
    p = params_from_desc(desc)
    with open(os.path.join(d, "params.bin"), "wb") as f:
        f.write(bytes(p))
    res = desc.res
    with open(os.path.join(d, "grid.txt"), "w") as f:
        f.write(f"{res} {res} {res} {desc.dh!r} 0 0 0\n")
    s = desc.solids[0]
    (mres, mdh, morig, mdata), verts, faces = solid_assets(s.radius)
    lam, mu = lame(s.E, s.nu)
    fields = list(mres) + [mdh] + [float(x) for x in morig] + [lam, mu, s.density]
    fields += list(s.center) + list(s.velocity) + [len(verts), len(faces)]
    with open(os.path.join(d, "solid.txt"), "w") as f:
        f.write(" ".join(repr(float(x)) if isinstance(x, float) else str(x) for x in fields) + "\n")
    np.ascontiguousarray(mdata.reshape(-1), dtype="<f8").tofile(os.path.join(d, "rest.f64"))
    np.ascontiguousarray(verts, dtype="<f8").tofile(os.path.join(d, "verts.f64"))
    np.ascontiguousarray(faces, dtype="<i4").tofile(os.path.join(d, "tris.i32"))


def test_facade_compiles_and_reports_errors(tmp_path):
    """Without a device esf_create fails; the facade turns it into esf::Error."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible; the GPU test covers the facade")
    except ImportError:
        pass
    exe = _build_facade(tmp_path)
    _write_inputs(str(tmp_path / "in"), DESC)
    r = subprocess.run([exe, str(tmp_path / "in")], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
    assert "esf_create" in r.stderr


@pytest.mark.gpu
def test_facade_step_matches_python_integrator(tmp_path, gpu_lib):
    from eulersf_gb300.integrator import CoupledIntegrator3D
    exe = _build_facade(tmp_path)
    _write_inputs(str(tmp_path / "in"), DESC)
    r = subprocess.run([exe, str(tmp_path / "in"), repr(DESC.dt)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = json.loads(r.stdout)
    res = DESC.res
    I = CoupledIntegrator3D(gpu_lib, "esf_", res, res, res, DESC.dh, (0.0, 0.0, 0.0),
                            params_from_desc(DESC))
    s = DESC.solids[0]
    d, keep = make_solid_desc(s.radius, s.center, s.density, s.E, s.nu, s.velocity)
    I.addSolid(d, keep)
    I.setFluidDensity(DESC.fluid_density)
    I.setFluidViscocity(0.0)
    I.init()
    I.setMaxDt(DESC.dt)
    rep = I.stepImplicit()
    assert got["status"] == 0
    assert got["energy"] == rep["energy"] and got["dt"] == I.dt()
    assert got["iterations"] == list(rep["iterations"])
    assert got["velocity_l1"] == float(np.abs(I.get("velocity")).sum())
    I.close()


@pytest.mark.gpu
def test_cfg_driver_first_substep(tmp_path, gpu_lib):
    """driver.run reads the cfg + assets from disk (main.cpp's inputs) and
    substeps a frame; its first substep equals an in-memory build of the
    scene stepped with the same max dt."""
    import io
    import eulersf_gb300 as E
    from eulersf_gb300 import driver
    cfg = write_scene(DESC, str(tmp_path / "scene"))
    reports = driver.run(cfg, frames=1, out=io.StringIO())
    assert reports and all(r["status"] == 0 for r in reports)
    assert reports[0]["frame"] == 0
    G = E.make_scene(DESC, noise=False)
    G.setMaxDt(float(DESC.dt))
    r0 = G.stepImplicit()
    first = reports[0]
    assert abs(first["iterations"][1] - r0["iterations"][1]) <= 5, (first["iterations"], r0["iterations"])
    assert abs(first["energy"] - r0["energy"]) <= 1e-9 * abs(r0["energy"])
    assert first["dt"] == r0["dt"]
    G.close()


@pytest.mark.gpu
def test_cfg_driver_saves_and_resumes_frames(tmp_path, gpu_lib):
    """"save data" writes each frame's files under "data path"
    (main.cpp:198-199); "start frame = 1" resumes from frame 0's files
    (main.cpp:95) and keeps stepping."""
    import io
    from eulersf_gb300 import driver
    cfg = write_scene(DESC, str(tmp_path / "scene"))
    data = str(tmp_path / "out") + "/"
    os.makedirs(data)
    with open(cfg, "a") as f:
        f.write(f"save data = true\ndata path = {data}\n")
    driver.run(cfg, frames=1, out=io.StringIO())
    names = set(os.listdir(data))
    assert {"frame.0000.velocity", "frame.0000.intensity", "frame.0000.solid.0.obj",
            "frame.0000.solid.0.displacement"} <= names
    with open(cfg, "a") as f:
        f.write("start frame = 1\n")
    reports = driver.run(cfg, frames=1, out=io.StringIO())
    assert reports and reports[0]["frame"] == 1 and all(r["status"] == 0 for r in reports)
    assert "frame.0001.intensity" in set(os.listdir(data))

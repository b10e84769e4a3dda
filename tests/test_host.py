"""CPU-only checks: the C-ABI library loads and exports every declared
symbol, host-side argument checks, the cfg reader, and the scene generator.
No kernel is launched."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from common import ROOT

from eulersf_gb300 import abi, scene


def _declared():
    text = open(os.path.join(ROOT, "include", "eulersf.h")).read()
    return sorted(set(re.findall(r"\b(esf_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import eulersf_gb300 as E
    return E.load(build_if_missing=True)


def test_exports_every_declared_symbol(lib):
    import eulersf_gb300 as E
    names = _declared()
    assert set(names) == set(E.EXPORTS)
    for n in names:
        assert hasattr(lib, n), n
    assert lib.esf_abi_version() == 1


def test_oracle_exports():
    import oracle
    o = oracle.load()
    for n in ("esfo_create", "esfo_step", "esfo_pressure_apply", "esfo_pressure_solve"):
        assert hasattr(o, n)


def test_invalid_arguments_need_no_gpu(lib):
    g = abi.Grid(2, 10, 10, 0.1, (C.c_double * 3)(0, 0, 0))
    p = abi.Params()
    assert lib.esf_params_default(C.byref(g), C.byref(p)) == 0
    assert p.cr_max_iterations == 10 and p.particles_per_cell == 8 and p.flip_alpha == 0.95
    h = C.c_void_p()
    assert lib.esf_create(C.byref(g), C.byref(p), None, C.byref(h)) == 1
    assert b"grid" in lib.esf_last_error()
    assert lib.esf_create(None, C.byref(p), None, C.byref(h)) == 1
    assert lib.esf_step(None, None) == 1
    assert lib.esf_destroy(None) == 0


def test_parse_config_reads_reference_keys(lib, tmp_path):
    desc = scene.SceneDesc(N=48, vorticity_eps=1.5, buoyancy=0.2, eps=1e-6, max_iters=1234,
                           solids=[scene.SolidDesc(center=(0.4, 0.6, 0.5), radius=0.12, E=3e5)])
    cfg = scene.write_scene(desc, str(tmp_path / "s"))
    g, p, n = abi.Grid(), abi.Params(), C.c_int()
    paths = C.create_string_buffer(4 * 256)
    solids = (abi.SolidDesc * 4)()
    st = lib.esf_parse_config(cfg.encode(), C.byref(g), C.byref(p), C.byref(n), paths, 256, solids, 4)
    assert st == 0
    assert (g.xRes, g.yRes, g.zRes) == (49, 49, 49) and g.dh == 1.0 / 48
    assert p.dt == 1.0 / 240 and p.gravity == 9.8 and p.vorticity_eps == 1.5 and p.buoyancy == 0.2
    assert p.div_free_solver_eps == 1e-6 and p.cr_max_iterations == 1234
    assert p.particles_per_cell == 32 and p.mass_sample_dh == 0.00125 and p.tight_border == 5
    assert n.value == 1
    lam, mu = scene.lame(3e5, 0.45)
    assert solids[0].lambda_ == pytest.approx(lam, rel=1e-15) and solids[0].mu == pytest.approx(mu, rel=1e-15)
    assert tuple(solids[0].translation) == (0.4, 0.6, 0.5)
    assert paths.raw[:256].split(b"\0")[0].decode().endswith("sphere0")
    assert list(solids[0].rotation) == [1, 0, 0, 0, 1, 0, 0, 0, 1]
    # the Python reader agrees (SIMPLE_PARSER lowercases keys and values)
    vals = scene.parse_cfg(cfg)
    assert float(vals["dt"]) == p.dt and vals["xres"] == "49"
    assert lib.esf_parse_config(b"/nonexistent.cfg", C.byref(g), C.byref(p), None, None, 0,
                                None, 0) == 5


def test_noise_field():
    a = scene.noise_field(9, 0)
    b = scene.noise_field(9, 0)
    c = scene.noise_field(9, 1)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.abs(a).max() <= 1e-3
    v = a.reshape(9, 9, 9, 3)
    for face in (v[0], v[-1], v[:, 0], v[:, -1], v[:, :, 0], v[:, :, -1]):
        assert not face.any()
    assert abs(a[a != 0].mean()) < 2e-4


def test_rest_mass_and_mesh(tmp_path):
    res, mdh, orig, data = scene.rest_mass_field(0.15)
    assert mdh == 0.0015 and all(r >= 219 for r in res)
    # volume of the rasterised sphere ~ 4/3 pi r^3 (density 1000)
    vol = (data > 0).sum() * mdh ** 3
    assert abs(vol - 4 / 3 * np.pi * 0.15 ** 3) / vol < 0.02
    p = str(tmp_path / "m.mass")
    scene.write_field_gz(p, res, mdh, orig, data)
    r2, d2, o2, data2 = scene.read_field_gz(p)
    assert tuple(r2) == tuple(res) and d2 == mdh and np.array_equal(data2, data)
    v, f = scene.icosphere(3, 0.2)
    assert len(v) == 642 and len(f) == 1280
    assert np.allclose(np.linalg.norm(v, axis=1), 0.2)


def test_lame():
    lam, mu = scene.lame(2e5, 0.45)
    assert lam == pytest.approx(620689.6551724138) and mu == pytest.approx(68965.51724137931)


def test_server_without_gpu_and_footprint_model(lib):
    """The server needs a device (a clean status without one); the admission
    estimate is host arithmetic and grows with the grid."""
    import ctypes as C
    from eulersf_gb300.scene import SceneDesc
    from eulersf_gb300.serve import ServerConfig, request_for
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if not has_gpu:
        h = C.c_void_p()
        assert lib.esf_server_create(C.byref(ServerConfig(0, 2)), C.byref(h)) == 7
        assert b"device" in lib.esf_last_error()
    sizes = []
    for n in (32, 64):
        q, keep = request_for(SceneDesc(N=n), 1)
        sizes.append(lib.esf_scene_footprint(C.byref(q.grid), C.byref(q.params), q.num_solids, q.solids))
    assert 0 < sizes[0] < sizes[1] and sizes[1] > 2 * sizes[0]
    # ESF_MIXED_X64 adds its double-float correction and direction, 16 bytes a
    # pressure row (with the estimate's 10% margin)
    desc = SceneDesc(N=64)
    q1, k1 = request_for(desc, 1, abi.ESF_MIXED)
    q2, k2 = request_for(desc, 1, abi.ESF_MIXED_X64)
    f1 = lib.esf_scene_footprint(C.byref(q1.grid), C.byref(q1.params), q1.num_solids, q1.solids)
    f2 = lib.esf_scene_footprint(C.byref(q2.grid), C.byref(q2.params), q2.num_solids, q2.solids)
    assert abs((f2 - f1) - 16 * 64 ** 3 * 1.1) <= 2


def test_precision_values_and_config_key(lib, tmp_path):
    """abi.py's precision constants are the header's, and the cfg key
    "precision" selects each of them (a GB300 addition to the reference's
    keys)."""
    import re
    hdr = open(os.path.join(ROOT, "include", "eulersf.h")).read()
    vals = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(ESF_FP64|ESF_MIXED|ESF_MIXED_X64)\s*=\s*(\d+)", hdr)}
    assert vals == {"ESF_FP64": abi.ESF_FP64, "ESF_MIXED": abi.ESF_MIXED, "ESF_MIXED_X64": abi.ESF_MIXED_X64}
    cfg = scene.write_scene(scene.SceneDesc(N=16), str(tmp_path / "s"))
    base = open(cfg).read()
    for word, want in (("fp64", abi.ESF_FP64), ("mixed", abi.ESF_MIXED), ("mixed x64", abi.ESF_MIXED_X64)):
        with open(cfg, "w") as f:
            f.write(base + f"\nprecision = {word}\n")
        g, p = abi.Grid(), abi.Params()
        assert lib.esf_parse_config(cfg.encode(), C.byref(g), C.byref(p), None, None, 0, None, 0) == 0
        assert p.precision == want, word


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import os
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "ESF_BENCH_GLOO": "1"})
    import bench
    r, w, pg = bench.dist_setup(world)
    bench.barrier(pg)
    mx = bench.max_over_ranks(pg, 10.0 * (r + 1))
    sm = bench.sum_over_ranks(pg, float(r + 1))
    bench.barrier(pg)
    out.put((r, w, mx, sm))
    pg.destroy_process_group()


def test_bench_rank_reductions_two_ranks_gloo():
    """bench.py's replica bookkeeping on two gloo ranks: every rank sees the
    maximum time and the summed work of all ranks."""
    import multiprocessing as mp
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 20.0, 3.0), (1, 2, 20.0, 3.0)]


def test_reference_arm_two_ranks_prints_one_line(tmp_path):
    """`bench.py --impl reference` launched as two ranks (torchrun, gloo):
    rank 0 times the CPU port and prints the one JSON line, the other rank
    exits 0 without work."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, ESF_BENCH_GLOO="1", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--size", "24", "--steps", "1", "--warmup", "0",
           "--cpu-iters", "2"]
    p = subprocess.run(cmd, cwd=root, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_reads_the_reference_frame_layout(tmp_path):
    """scene.read_field_gz (the FIELD_3D gz layout of esf_io.cpp) reads a frame
    file the reference's writeFrame wrote: three int32 resolutions, dh and
    origin as float64, then the data; the velocity it holds is the state the
    reference's readFrame restored, away from the solid's nodes (which
    recoverVelocityField overwrites on reading)."""
    from common import load_golden
    desc, z, _ = load_golden("frame16")
    p = tmp_path / "frame.0000.velocity"
    p.write_bytes(z["file.frame.0000.velocity"].tobytes())
    res, dh, origin, data = scene.read_field_gz(str(p))
    assert tuple(res) == (desc.res,) * 3 and dh == desc.dh and list(origin) == [0.0, 0.0, 0.0]
    v = data.reshape(-1, 3)
    fluid = z["r0.gridIdxToSolidIdx"] < 0
    assert np.array_equal(v[fluid], z["r0.velocity"].reshape(-1, 3)[fluid])

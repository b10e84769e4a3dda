"""Frame files (esf_write_frame / esf_read_frame, the reference's
COUPLED_INTEGRATOR_3D::writeFrame/readFrame): the written gz fields are the
scene's fields bit for bit in the FIELD_3D layout the reference reads
(the same layout tests/golden's .mass inputs use), the OBJ holds the current
mesh to 6 significant digits, the every-10th-frame rule is kept, and a fresh
scene that reads a frame holds the same fields and keeps stepping. Against
the reference's own frame files (tests/golden/frame16.npz): reading them
restores the reference's read state and steps like the reference's restart,
and writing after the read gives the reference's bytes."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from eulersf_gb300.scene import SceneDesc, read_field_gz

pytestmark = pytest.mark.gpu

DESC = SceneDesc(N=16, mass_sample_dh=(1.0 / 16) / 4, noise_seed=3)


def _obj_vertices(path):
    with open(path) as f:
        return np.array([[float(t) for t in line.split()[1:4]] for line in f if line.startswith("v ")])


def test_write_frame_holds_the_scene_fields(tmp_path, gpu_lib):
    import eulersf_gb300 as E
    G = E.make_scene(DESC)
    G.stepImplicit()
    pre = str(tmp_path) + "/"
    G.writeFrame(0, data_path=pre)
    X = DESC.res
    for name, field in (("frame.0000.velocity", "velocity"), ("frame.0000.intensity", "intensity"),
                        ("frame.0000.solid.0.displacement", "solid.u"),
                        ("frame.0000.solid.0.velocity", "solid.velocity"),
                        ("frame.0000.solid.0.phi", "solid.phi")):
        res, dh, origin, data = read_field_gz(pre + name)
        assert res == (X, X, X) and dh == DESC.dh and list(origin) == [0.0, 0.0, 0.0], name
        assert np.array_equal(data.reshape(-1), G.get(field).reshape(-1)), name
    v = _obj_vertices(pre + "frame.0000.solid.0.obj")
    ref = G.get("solid.meshVertices").reshape(-1, 3)
    assert v.shape == ref.shape
    assert np.abs(v - ref).max() <= 1e-5 * np.abs(ref).max()
    # frame 3: only the mesh and the intensity (every-10th-frame rule) ...
    G.writeFrame(3, data_path=pre)
    names = set(os.listdir(tmp_path))
    assert {"frame.0003.intensity", "frame.0003.solid.0.obj"} <= names
    assert "frame.0003.velocity" not in names and "frame.0003.solid.0.phi" not in names
    # ... unless debug
    G.writeFrame(4, debug=True, data_path=pre)
    assert "frame.0004.velocity" in set(os.listdir(tmp_path))
    G.close()


def test_read_frame_restores_fields_and_steps(tmp_path, gpu_lib):
    import eulersf_gb300 as E
    pre = str(tmp_path) + "/"
    A = E.make_scene(DESC)
    for _ in range(2):
        A.stepImplicit()
    A.writeFrame(10, data_path=pre)
    B = E.make_scene(DESC)
    B.readFrame(10, data_path=pre)
    for name in ("velocity", "intensity", "solid.u", "solid.velocity", "solid.phi"):
        if name == "velocity":
            continue  # recoverVelocityField overwrites the solid's nodes after the read
        assert np.array_equal(B.get(name), A.get(name)), name
    # X = node position - u (origin 0)
    X = DESC.res
    z, y, x = np.meshgrid(*(np.arange(X) * DESC.dh,) * 3, indexing="ij")
    pos = np.stack([x.reshape(-1), y.reshape(-1), z.reshape(-1)], axis=1)
    assert np.array_equal(B.get("solid.X").reshape(-1, 3), pos - A.get("solid.u").reshape(-1, 3))
    fluid = A.get("solidMass") == 0
    assert np.array_equal(B.get("velocity")[fluid], A.get("velocity")[fluid])
    r = B.stepImplicit()
    assert r["status"] == 0 and all(r["converged"]), r
    # a frame of another grid size is refused with a message
    C_ = E.make_scene(SceneDesc(N=12, mass_sample_dh=(1.0 / 12) / 4))
    with pytest.raises(Exception):
        C_.readFrame(10, data_path=pre)
    assert "needs" in E.last_error() or "holds" in E.last_error()
    for s in (A, B, C_):
        s.close()


def _reference_frames(tmp_path):
    """The reference's own frame files (tests/golden/frame16.npz, written by
    COUPLED_INTEGRATOR_3D::writeFrame) into tmp_path; returns the fixture."""
    from common import load_golden
    desc, z, log = load_golden("frame16")
    for k in z.files:
        if k.startswith("file."):
            with open(os.path.join(tmp_path, k[5:]), "wb") as f:
                f.write(z[k].tobytes())
    return desc, z


def test_reads_reference_frame_and_steps_like_the_reference(tmp_path, gpu_lib):
    """esf_read_frame on the files the reference wrote restores the state the
    reference's readFrame restores (maps and flags bit-exact, fields to 1e-6),
    and one step from there matches the reference's step from its read (the
    warm start, which no frame carries, set to the reference's)."""
    import eulersf_gb300 as E
    desc, z = _reference_frames(tmp_path)
    G = E.make_scene(desc)
    G.readFrame(0, debug=True, data_path=str(tmp_path) + "/")
    # (the pressure warm start is not part of a frame: the reference's is the
    # static left by its last solve)
    fails = _compare(G.get, z, "r0.", skip=("lambda1",))
    assert not fails, fails
    G.set("lambda1", z["r0.lambda1"])
    r = G.stepImplicit()
    ref = json.loads(str(z["log_restart"]))[0]
    assert r["status"] == 0 and all(r["converged"]), r
    want = [ref["solid_iters"][0], ref["pressure_iters"][0], ref["solid_iters"][1]]
    assert all(abs(a - b) <= 5 for a, b in zip(r["iterations"], want)), (r["iterations"], want)
    assert r["dt"] == ref["dt"]
    assert abs(r["energy"] - ref["energy"]) <= 1e-8 * abs(ref["energy"])
    fails = _compare(G.get, z, "r1.")
    assert not fails, fails
    G.close()


def _compare(get, z, pre, tol=1e-6, skip=()):
    from common import EXACT, NAME, rel_err
    fails = []
    for k in z.files:
        if not k.startswith(pre) or k[len(pre):] in skip:
            continue
        f = k[len(pre):]
        mine, ref = np.asarray(get(NAME[f])), z[k]
        if f in EXACT:
            if not np.array_equal(mine.reshape(-1), ref.reshape(-1).astype(mine.dtype)):
                fails.append(f"{k}: not bit-exact")
        else:
            a, b = mine.reshape(-1), ref.reshape(-1)
            if f == "solid0.particles":
                a, b = mine.reshape(-1, 10)[:, :9], ref.reshape(-1, 10)[:, :9]
            if a.size != b.size or not rel_err(a, b) <= tol:
                fails.append(f"{k}: rel err {rel_err(a, b) if a.size == b.size else 'size'}")
    return fails


def test_written_frame_is_the_reference_frame(tmp_path, gpu_lib):
    """After reading the reference's frame 0, esf_write_frame writes frame 1
    with the same content as the reference's writeFrame after its read: the
    gz fields decompress to the same bytes (header and data), and the OBJ is
    the same text."""
    import gzip
    import eulersf_gb300 as E
    desc, z = _reference_frames(tmp_path)
    out = tmp_path / "ours"
    out.mkdir()
    G = E.make_scene(desc)
    G.readFrame(0, debug=True, data_path=str(tmp_path) + "/")
    G.writeFrame(1, debug=True, data_path=str(out) + "/")
    names = [k[5:] for k in z.files if k.startswith("file.frame.0001.")]
    assert names
    for n in names:
        ref = z["file." + n].tobytes()
        with open(out / n, "rb") as f:
            mine = f.read()
        if n.endswith(".obj"):
            assert mine == ref, n
        else:
            assert gzip.decompress(mine) == gzip.decompress(ref), n
    G.close()


def test_asynchronous_frame_is_the_synchronous_frame(tmp_path, gpu_lib):
    """esf_write_frame_async snapshots the state when it is called: stepping on
    at once does not change what it writes, which is what esf_write_frame
    writes (gz fields decompressing to the same bytes, the same OBJ)."""
    import gzip
    import eulersf_gb300 as E
    a, b = tmp_path / "sync", tmp_path / "async"
    a.mkdir()
    b.mkdir()
    G = E.make_scene(DESC)
    G.stepImplicit()
    G.writeFrame(0, data_path=str(a) + "/")
    G.writeFrameAsync(0, data_path=str(b) + "/")
    G.stepImplicit()  # the state moves on while the frame is written
    G.frameWait()
    names = sorted(os.listdir(a))
    assert names == sorted(os.listdir(b)) and len(names) >= 7
    for n in names:
        x, y = (a / n).read_bytes(), (b / n).read_bytes()
        if n.endswith(".obj"):
            assert x == y, n
        else:
            assert gzip.decompress(x) == gzip.decompress(y), n
    G.close()

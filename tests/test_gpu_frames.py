"""Frame files (esf_write_frame / esf_read_frame, the reference's
COUPLED_INTEGRATOR_3D::writeFrame/readFrame): the written gz fields are the
scene's fields bit for bit in the FIELD_3D layout the reference reads
(the same layout tests/golden's .mass inputs use), the OBJ holds the current
mesh to 6 significant digits, the every-10th-frame rule is kept, and a fresh
scene that reads a frame holds the same fields and keeps stepping."""
import ctypes as C
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

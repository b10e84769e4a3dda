"""Solid-solid contact on the GPU against the reference's own build.

The fixture (tests/golden/make_golden.py --contact) is two balls moving
towards each other one grid cell apart, run by the reference with the rest
SDFs the scene writer made (".svol", read through SPARSE_SDF). It holds the
contact query SPARSE_SDF::signedDistAndCurrentNormal alone at seeded rest
points, and the state of both solids after each of 3 steps.

Bars: the query's distances and normals within 1e-9 (the same lattice values,
the same walk, the same triangle); DOF maps, cell flags and boxes of both
solids bit-exact; the system matrix the two solids assemble together within
1e-9 and its sparsity exact; every other field within 1e-6 relative, as for
the one-solid fixtures.
"""
import re

import numpy as np
import pytest

from common import compare_to_golden, csr_to_blocks, load_golden, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-6


class _Solid:
    """The fixture seen through solid i's names (solid0.* -> solid<i>.*)."""

    def __init__(self, z, i):
        self.z, self.i = z, i
        self.files = [f.replace(f"solid{i}.", "solid0.") for f in z.files
                      if f"solid{i}." in f or not re.search(r"solid\d\.", f)]

    def __getitem__(self, k):
        return self.z[k.replace("solid0.", f"solid{self.i}.")]


def _getter(G, i):
    def get(name):
        if name.startswith("solid."):
            return G.get(name, solid=i)
        return G.get(name)
    return get


def test_rest_sdf_query_matches_reference(gpu_lib):
    import eulersf_gb300 as E
    desc, z, _ = load_golden("contact20")
    G = E.make_scene(desc)
    pts, safe = z["sdfq.points"], float(z["sdfq.safe"])
    for i in range(len(desc.solids)):
        sd, nrm = G.restSdfQuery(i, pts, safe)
        ref = z[f"sdfq.solid{i}"]
        far = ref[:, 0] == 1
        assert np.array_equal(sd == 1, far), (i, int(np.count_nonzero((sd == 1) != far)))
        assert np.abs(sd[~far] - ref[~far, 0]).max() <= 1e-9
        assert np.abs(nrm[~far] - ref[~far, 1:]).max() <= 1e-9
    G.close()


def test_contact_step_matches_reference(gpu_lib):
    import eulersf_gb300 as E
    desc, z, log = load_golden("contact20")
    G = E.make_scene(desc)
    for i in range(len(desc.solids)):
        fails = compare_to_golden(_getter(G, i), _Solid(z, i), 0, tol=0.0)
        assert not fails, (i, fails)
    contacts = 0
    for k, ref in enumerate(log, start=1):
        sdof = G.get("gridIdxToSolidIdx")
        r = G.stepImplicit()
        assert r["status"] == 0 and all(r["converged"]), r
        it = [ref["solid_iters"][0], ref["pressure_iters"][0], ref["solid_iters"][1]]
        assert all(abs(a - b) <= 5 for a, b in zip(r["iterations"], it)), (r["iterations"], it)
        assert r["dt"] == ref["dt"]
        assert abs(r["energy"] - ref["energy"]) <= 1e-8 * abs(ref["energy"]), (r["energy"], ref["energy"])
        contacts += r["solid_contacts"]
        for i in range(len(desc.solids)):
            fails = compare_to_golden(_getter(G, i), _Solid(z, i), k, tol=TOL)
            assert not fails, (k, i, fails)
        if f"s{k}.systemMatrix.indptr" in z.files:
            blocks, mask = csr_to_blocks(z[f"s{k}.systemMatrix.indptr"], z[f"s{k}.systemMatrix.indices"],
                                         z[f"s{k}.systemMatrix.data"], sdof, desc.res, desc.res)
            assert np.array_equal(G.get("systemMask"), mask)
            assert rel_err(G.get("systemBlocks").reshape(-1, 27, 3, 3), blocks) <= 1e-9
    assert contacts > 0, "no particle took a solid-solid impulse"
    G.close()


def test_several_solids_need_their_rest_sdf(gpu_lib):
    """A scene with two solids and no rest SDF refuses to step (the reference
    would dereference a null SPARSE_SDF); nothing ran, the scene stays usable."""
    import eulersf_gb300 as E
    from eulersf_gb300.abi import EsfError
    desc, _, _ = load_golden("contact20")
    G = E.make_scene(desc, rest_sdf=False)
    with pytest.raises(EsfError) as e:
        G.stepImplicit()
    assert e.value.status == 2 and "rest SDF" in str(e.value)
    from eulersf_gb300.integrator import sphere_svol_path
    for i, s in enumerate(desc.solids):
        G.loadRestSDF(i, sphere_svol_path(s.radius))
    r = G.stepImplicit()
    assert r["status"] == 0 and all(r["converged"])
    G.close()


def test_two_solids_mixed_precision(gpu_lib):
    """Two solids in mixed precision (the assembled FP32 blocks serve the
    inner solid solves when there is more than one solid): the refined
    solves reach the FP64 tolerance and the state stays within the mixed
    path's bar of the FP64 one."""
    import eulersf_gb300 as E
    desc, _, _ = load_golden("contact20")
    A, B = E.make_scene(desc, precision=0), E.make_scene(desc, precision=1)
    for _ in range(2):
        ra, rb = A.stepImplicit(), B.stepImplicit()
        assert all(rb["converged"]) and max(rb["rel_residual"]) < 1e-8, rb
    for i in range(2):
        assert rel_err(B.get("solid.velocity", solid=i), A.get("solid.velocity", solid=i)) <= 1e-3
    assert rel_err(B.get("velocity"), A.get("velocity")) <= 1e-3
    A.close()
    B.close()


def test_two_solid_frames_round_trip(gpu_lib, tmp_path):
    """Frames of a two-solid scene (frame.NNNN.solid.<i>.* per solid, as
    COUPLED_INTEGRATOR_3D::writeFrame names them): a fresh scene with the
    same solids and rest SDFs reads back both solids' fields and keeps
    stepping with contact."""
    import eulersf_gb300 as E
    desc, _, _ = load_golden("contact20")
    pre = str(tmp_path) + "/"
    A = E.make_scene(desc)
    A.stepImplicit()
    A.writeFrame(0, debug=True, data_path=pre)
    for i in range(2):
        for ext in ("displacement", "velocity", "phi", "obj"):
            assert (tmp_path / f"frame.0000.solid.{i}.{ext}").exists(), (i, ext)
    B = E.make_scene(desc)
    B.readFrame(0, debug=True, data_path=pre)
    for i in range(2):
        for name in ("solid.u", "solid.velocity", "solid.phi"):
            assert np.array_equal(B.get(name, solid=i), A.get(name, solid=i)), (i, name)
    assert np.array_equal(B.get("intensity"), A.get("intensity"))
    ra, rb = A.stepImplicit(), B.stepImplicit()
    assert rb["status"] == 0 and all(rb["converged"]), rb
    # the mesh went through 6-digit OBJ text (contact normals come from it),
    # the rest is exact: the two continue together to near the step's tolerance
    for i in range(2):
        assert rel_err(B.get("solid.u", solid=i), A.get("solid.u", solid=i)) <= 1e-5
    assert rel_err(B.get("velocity"), A.get("velocity")) <= 1e-5
    A.close()
    B.close()

"""The CPU oracle (oracle/esf_oracle.c) against golden vectors written by the
reference's own build (tests/golden/make_golden.py): this pins the checker
the GPU parity tests use."""
import json

import numpy as np
import pytest

from common import GOLDEN_SCENES, compare_to_golden, csr_to_blocks, load_golden

import oracle


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_oracle_matches_reference(name):
    desc, z, log = load_golden(name)
    I = oracle.scene(desc)
    # set-up (init + smoke carpet + noise) is bit-exact
    fails = compare_to_golden(I.get, z, 0, tol=0.0)
    assert not fails, fails
    for k, ref in enumerate(log, start=1):
        sdof = I.get("gridIdxToSolidIdx")  # the map the step assembles with
        r = I.stepImplicit()
        assert r["iterations"] == [ref["solid_iters"][0], ref["pressure_iters"][0],
                                   ref["solid_iters"][1]], (k, r, ref)
        assert r["dt"] == ref["dt"]
        assert abs(r["energy"] - ref["energy"]) <= 1e-9 * abs(ref["energy"])
        fails = compare_to_golden(I.get, z, k, tol=1e-7)
        assert not fails, fails
        # _systemMatrix: sparsity bit-exact, values to rounding
        blocks, mask = csr_to_blocks(z[f"s{k}.systemMatrix.indptr"], z[f"s{k}.systemMatrix.indices"],
                                     z[f"s{k}.systemMatrix.data"], sdof, desc.res, desc.res)
        assert np.array_equal(I.get("systemMask"), mask)
        mine = I.get("systemBlocks").reshape(-1, 27, 3, 3)
        assert np.abs(mine - blocks).max() <= 1e-9 * np.abs(blocks).max()


def test_mt19937_stream():
    """MERSENNETWISTER(123456) is the standard MT19937 stream; the particle
    seeding of the golden fixture consumes it as (z, y, x) per particle."""
    desc, z, _ = load_golden("ball16")
    p = z["s0.solid0.particles"]
    r = oracle.mt19937(123456, 3 * len(p)).astype(np.float64) * (1.0 / 4294967295.0) * desc.dh
    valid = z["s0.solid0.valid"].reshape(desc.N, desc.N, desc.N)
    box = z["s0.solid0.boxes"]
    cells = [(x, y, zz) for zz in range(box[8], box[11] - 1) for y in range(box[7], box[10] - 1)
             for x in range(box[6], box[9] - 1) if valid[zz, y, x] == 1]
    ppc = len(p) // len(cells)
    for i in (0, 1, len(p) - 1):
        x, y, zz = cells[i // ppc]
        assert p[i, 0] == x * desc.dh + r[3 * i + 2]
        assert p[i, 1] == y * desc.dh + r[3 * i + 1]
        assert p[i, 2] == zz * desc.dh + r[3 * i]


@pytest.mark.parametrize("name", ["ball16", "wall20"])
def test_pressure_residual_helper_on_reference_solutions(name):
    """oracle.pressure_residual (the independent residual check used by the
    smoke step and the benchmark) gives the reference's own pressure solutions
    a relative residual below its 1e-8 tolerance, step by step."""
    desc, z, log = load_golden(name)

    class Dump:
        def __init__(self, k):
            self.k = k

        def get(self, f):
            key = f"s0.{f}" if f == "gridIdxToSolutionIdx" else f"s{self.k}.{f}"
            return z[key]

        def xRes(self):
            return desc.res
        yRes = zRes = xRes

        def dh(self):
            return desc.dh

        def origin(self):
            return (0.0, 0.0, 0.0)

    for k in range(1, len(log) + 1):
        res = oracle.pressure_residual(Dump(k))
        assert res < 1.01e-8, (k, res)


def test_oracle_matches_reference_at_64():
    """The oracle against the reference's OpenMP build on the 64^3 benchmark
    scene (compact fixture), first step: maps and flags bit-exact, identical
    iteration counts and dt, fields within 1e-7."""
    from common import compare_big, load_big
    desc, z, log, _ = load_big("config1_64")
    I = oracle.scene(desc)
    fails, _ = compare_big(I.get, z, 0, tol=0.0)
    assert not fails, fails
    r = I.stepImplicit()
    ref = log[0]
    assert r["iterations"] == [ref["solid_iters"][0], ref["pressure_iters"][0], ref["solid_iters"][1]]
    assert r["dt"] == ref["dt"]
    assert abs(r["energy"] - ref["energy"]) <= 1e-9 * abs(ref["energy"])
    fails, _ = compare_big(I.get, z, 1, tol=1e-7)
    assert not fails, fails

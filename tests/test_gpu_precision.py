"""The mixed-precision path's FP32 stress evaluation (k_element_stiffness_f32)
and its FP64 fallback for near-degenerate deformation gradients.

The element stiffness, forces and energy of an elastic solid are evaluated in
FP32 in mixed precision, except in cells whose F has cond(F) > 1e3, which go
through the reference's FP64 arithmetic. Compared with the FP64 path on the
same state, before any solve: the assembled system blocks and the solid
forces agree to FP32 rounding. A state with a compressed lower half (F_zz =
1/c in those cells, c = 5e-4, so cond(F) = 2000) sends those cells to the FP64
fallback and keeps the others in FP32.
"""
import numpy as np
import pytest

from common import rel_err

pytestmark = pytest.mark.gpu


def _pair(desc):
    import eulersf_gb300 as E
    return E.make_scene(desc, precision=0), E.make_scene(desc, precision=1)


def _compress_lower_half(I, desc, c):
    """u_z += (1 - c)(z - zc) below the solid's centre plane zc: there the
    material coordinate X_z = z - u_z changes c times slower than z."""
    X = desc.res
    u = I.get("solid.u").copy()
    zc = desc.solids[0].center[2]
    z = (np.arange(X ** 3) // (X * X)) * desc.dh
    low = z < zc
    u[low, 2] += (1.0 - c) * (z[low] - zc)
    I.set("solid.u", u)


def test_fp32_stiffness_matches_fp64_on_a_normal_state(gpu_lib):
    from eulersf_gb300.scene import SceneDesc
    desc = SceneDesc(N=24, mass_sample_dh=(1 / 24) / 4, noise_seed=5)
    A, B = _pair(desc)
    ra, rb = A.stepImplicit(), B.stepImplicit()
    assert rb["fp64_stress_cells"] == 0 and rb["valid_cells"] > 0, rb
    assert ra["fp64_stress_cells"] == ra["valid_cells"]
    for n in ("systemBlocks", "systemDiag", "solidUnitForce"):
        assert rel_err(B.get(n), A.get(n)) <= 1e-6, n
    assert abs(rb["energy"] - ra["energy"]) <= 1e-6 * abs(ra["energy"])
    A.close()
    B.close()


def test_near_degenerate_cells_fall_back_to_fp64(gpu_lib):
    from eulersf_gb300.scene import SceneDesc
    desc = SceneDesc(N=16, mass_sample_dh=(1 / 16) / 4, noise_seed=8)
    A, B = _pair(desc)
    for I in (A, B):
        _compress_lower_half(I, desc, 5e-4)
    ra, rb = A.stepImplicit(), B.stepImplicit()
    # some cells, not all, went through the FP64 fallback
    assert 0 < rb["fp64_stress_cells"] < rb["valid_cells"], rb
    # the system blocks assembled from them agree with the FP64 path to FP32
    # rounding of the well-conditioned cells' share
    assert rel_err(B.get("systemBlocks"), A.get("systemBlocks")) <= 1e-5
    assert rel_err(B.get("solidUnitForce"), A.get("solidUnitForce")) <= 1e-5
    A.close()
    B.close()


def test_matrix_free_solid_operator_matches_assembled(gpu_lib, monkeypatch):
    """The mixed inner solid solves apply the stiffness matrix-free (cell
    shares gathered per node) by default, and the FP32 copy of the assembled
    blocks with ESF_SOLID_ASSEMBLED=1. Both refine to the same 1e-8 FP64
    residual of the same assembled FP64 system, so the solid solutions agree
    to that system's conditioning times the tolerance."""
    import eulersf_gb300 as E
    from eulersf_gb300.scene import SceneDesc
    desc = SceneDesc(N=24, mass_sample_dh=(1 / 24) / 4, noise_seed=6)
    out = {}
    for mode in ("matrix_free", "assembled"):
        if mode == "assembled":
            monkeypatch.setenv("ESF_SOLID_ASSEMBLED", "1")
        else:
            monkeypatch.delenv("ESF_SOLID_ASSEMBLED", raising=False)
        I = E.make_scene(desc, precision=1)
        r = I.stepImplicit()
        assert r["status"] == 0 and all(r["converged"]) and max(r["rel_residual"]) < 1e-8, r
        out[mode] = (r, I.get("solidVelocityAtDt0"), I.get("solidPressureCorrection"), I.get("velocity"))
        I.close()
    (ra, va, pa, ua), (rb, vb, pb, ub) = out["matrix_free"], out["assembled"]
    assert rel_err(va, vb) <= 1e-5 and rel_err(pa, pb) <= 1e-4
    assert rel_err(ua, ub) <= 1e-4
    # comparable inner iteration counts (the operators differ by FP32 rounding)
    for k in (0, 2):
        assert ra["iterations"][k] <= 2 * rb["iterations"][k] + 10, (ra["iterations"], rb["iterations"])

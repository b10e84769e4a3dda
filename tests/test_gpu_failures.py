"""Failure paths of the CUDA library, made to fire without faulting the GPU.

* The bounded waits: a one-block kernel waits, with the kernels' own wait
  function, on something that never happens (an mbarrier armed for a TMA copy
  that is never issued; a grid barrier that no other block reaches). The wait
  runs out, the kernel returns on its own with its error word set, and the
  context keeps working.
* NaN/Inf in a solve: a NaN placed on the host in the right-hand side of the
  pressure solve comes back as ESF_ERR_NUMERIC (FP64 and mixed), and the
  next solve is fine. In a step, a NaN in the fluid velocity stops the step
  after the solve that meets it (nothing downstream runs on non-finite
  values), further steps are refused, and reading a frame restores a state
  that steps again. The reference instead prints "didn't converge" and
  carries on (CONJUGATE_RESIDUAL.inl:186-189).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from common import rel_err

pytestmark = pytest.mark.gpu

ESF_ERR_STATE, ESF_ERR_NUMERIC = 2, 6


def _dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _apply_still_works(lib):
    import torch
    X = 13
    rng = np.random.default_rng(5)
    g = oracle.grid(X, 1.0 / (X - 1))
    minv = rng.uniform(0.5, 2.0, X ** 3)
    x = rng.standard_normal((X - 1) ** 3)
    dm, dx, do = _dev(minv), _dev(x), _dev(np.zeros_like(x))
    assert lib.esf_pressure_apply(C.byref(g), _ptr(dm), _ptr(dx), _ptr(do), None) == 0
    torch.cuda.synchronize()
    assert rel_err(do.cpu().numpy(), oracle.pressure_apply(g, minv, x)) <= 1e-13


@pytest.mark.parametrize("kind", [0, 1], ids=["mbarrier", "grid_barrier"])
def test_bounded_wait_runs_out_and_the_kernel_returns(kind, gpu_lib):
    gave_up, ms = C.c_int(-1), C.c_double(-1)
    assert gpu_lib.esf_selftest_bounded_wait(kind, C.byref(gave_up), C.byref(ms)) == 0
    assert gave_up.value == 1
    assert 0 < ms.value < 60_000, ms.value
    print(f"wait kind {kind}: gave up after {ms.value:.1f} ms")
    _apply_still_works(gpu_lib)


def _system(X, seed):
    rng = np.random.default_rng(seed)
    g = oracle.grid(X, 1.0 / (X - 1))
    minv = rng.uniform(50.0, 300.0, X ** 3)
    m = minv.reshape(X, X, X).copy()
    m[0], m[-1], m[:, 0], m[:, -1], m[:, :, 0], m[:, :, -1] = 0, 0, 0, 0, 0, 0
    diag = np.zeros((X - 1,) * 3)
    for i in range(8):
        dx, dy, dz = i & 1, (i >> 1) & 1, (i >> 2) & 1
        diag += 3 * m[dz:dz + X - 1, dy:dy + X - 1, dx:dx + X - 1]
    b = oracle.pressure_apply(g, minv, rng.standard_normal((X - 1) ** 3))
    return g, minv, diag.reshape(-1), b


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_nan_in_the_pressure_rhs_is_reported(precision, gpu_lib):
    import torch
    g, minv, diag, b = _system(25, 3)
    bad = b.copy()
    bad[len(b) // 3] = np.nan
    it, rr = C.c_int(), C.c_double()
    for rhs, want in ((bad, ESF_ERR_NUMERIC), (b, 0)):
        dm, dd, db, dx = _dev(minv), _dev(diag), _dev(rhs), _dev(np.zeros(len(b)))
        s = gpu_lib.esf_pressure_solve(C.byref(g), _ptr(dm), _ptr(dd), _ptr(db), _ptr(dx), 1e-8,
                                       20000, precision, C.byref(it), C.byref(rr), None)
        torch.cuda.synchronize()
        assert s == want, (s, gpu_lib.esf_last_error())
    assert rr.value < 1e-8


def test_nan_in_a_step_stops_it_and_a_frame_restores_the_scene(gpu_lib, tmp_path):
    import eulersf_gb300 as E
    from eulersf_gb300 import abi
    from eulersf_gb300.scene import SceneDesc
    desc = SceneDesc(N=16, mass_sample_dh=(1.0 / 16) / 4, noise_seed=2)
    G = E.make_scene(desc)
    G.stepImplicit()
    pre = str(tmp_path) + "/"
    G.writeFrame(0, data_path=pre)
    good = {n: G.get(n) for n in ("velocity", "lambda1", "solid.u")}
    # a NaN at a fluid node far from the ball (which sits at y = 0.65)
    X = desc.res
    v = G.get("velocity").copy()
    v[3 + 3 * X + 8 * X * X, 0] = np.nan
    G.set("velocity", v)
    r = G.stepImplicit()
    assert r["status"] == ESF_ERR_NUMERIC, r
    # the step stopped after the solve: the solid state was not advanced
    assert np.array_equal(G.get("solid.u"), good["solid.u"])
    with pytest.raises(abi.EsfError) as e:
        G.stepImplicit()
    assert e.value.status == ESF_ERR_STATE
    # the frame restores the fluid velocity, the solid state and the pressure
    # warm start (recoverVelocityField rewrites the solid's nodes on reading)
    G.readFrame(0, data_path=pre)
    fluid = G.get("solidMass") == 0
    assert np.array_equal(G.get("velocity")[fluid], good["velocity"][fluid])
    for n in ("lambda1", "solid.u"):
        assert np.array_equal(G.get(n), good[n]), n
    r = G.stepImplicit()
    assert r["status"] == 0 and all(r["converged"]), r
    assert np.all(np.isfinite(G.get("velocity")))
    G.close()

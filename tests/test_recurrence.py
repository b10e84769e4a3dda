"""The one-pass CR recurrence of the FP32 inner pressure solves
(pcr_iteration_fused) against the reference's PCR recurrence
(CONJUGATE_RESIDUAL::solvePCR, CONJUGATE_RESIDUAL.inl:139-160), both written
out in numpy over the oracle's pressure operator. In FP64 the two produce
the same iterates to rounding (the one-pass form only reorders the algebra:
t = s/diag and q = Ap/diag are stored, and (Ap, Ap/diag) is expanded as
mu + 2 beta nu + beta^2 omega); in FP32 they take the same iterations."""
import numpy as np
import pytest

import oracle


def _problem(N, seed):
    X = N + 1
    rng = np.random.default_rng(seed)
    g = oracle.grid(X, 1.0 / N)
    minv = rng.uniform(50.0, 300.0, X ** 3)
    m = minv.reshape(X, X, X).copy()
    m[0], m[-1], m[:, 0], m[:, -1], m[:, :, 0], m[:, :, -1] = 0, 0, 0, 0, 0, 0
    diag = np.zeros((N, N, N))
    for i in range(8):
        dx, dy, dz = i & 1, (i >> 1) & 1, (i >> 2) & 1
        diag += 3 * m[dz:dz + N, dy:dy + N, dx:dx + N]
    A = lambda v: oracle.pressure_apply(g, minv, v.astype(np.float64))
    b = A(rng.standard_normal(N ** 3))
    return A, diag.reshape(-1), b


def _reference(A, iv, b, iters, dt):
    x = np.zeros_like(b, dtype=dt)
    r = (b * iv).astype(dt)
    s = A(r).astype(dt)
    delta = float(r.astype(np.float64) @ s)
    d = np.zeros_like(x)
    Ap = np.zeros_like(x)
    beta = 0.0
    hist = []
    for _ in range(iters):
        d = (dt(beta) * d + r).astype(dt)
        Ap = (dt(beta) * Ap + s).astype(dt)
        alpha = delta / float(Ap.astype(np.float64) @ (Ap * iv))
        x = (x + dt(alpha) * d).astype(dt)
        r = (r - dt(alpha) * (Ap * iv)).astype(dt)
        s = A(r).astype(dt)
        dn = float(r.astype(np.float64) @ s)
        beta, delta = dn / delta, dn
        hist.append(dn)
    return x, np.array(hist)


def _one_pass(A, iv, b, iters, dt):
    diag = 1.0 / iv
    x = np.zeros_like(b, dtype=dt)
    r = (b * iv).astype(dt)
    d = np.zeros_like(x)
    q = np.zeros_like(x)
    s = A(r).astype(dt)
    t = (iv * s).astype(dt)
    delta = float(r.astype(np.float64) @ s)
    alpha, beta = delta / float(s.astype(np.float64) @ t), 0.0
    hist = []
    for _ in range(iters):
        q = (dt(beta) * q + t).astype(dt)
        d = (dt(beta) * d + r).astype(dt)
        x = (x + dt(alpha) * d).astype(dt)
        r = (r - dt(alpha) * q).astype(dt)
        om = float((q.astype(np.float64) ** 2) @ diag)
        s = A(r).astype(dt)
        t = (iv * s).astype(dt)
        dl = float(r.astype(np.float64) @ s)
        mu = float(s.astype(np.float64) @ t)
        nu = float(s.astype(np.float64) @ q)
        beta = dl / delta
        alpha = dl / (mu + 2 * beta * nu + beta * beta * om)
        delta = dl
        hist.append(dl)
    return x, np.array(hist)


def test_one_pass_recurrence_is_the_reference_recurrence_fp64():
    A, diag, b = _problem(12, 3)
    iv = 1.0 / diag
    xr, hr = _reference(A, iv, b, 40, np.float64)
    xo, ho = _one_pass(A, iv, b, 40, np.float64)
    assert np.allclose(ho, hr, rtol=1e-8, atol=0)
    assert np.linalg.norm(xo - xr) <= 1e-9 * np.linalg.norm(xr)


@pytest.mark.parametrize("N,eps", [(16, 1e-4), (20, 1e-5)])
def test_one_pass_recurrence_same_iterations_fp32(N, eps):
    A, diag, b = _problem(N, N)
    iv = (1.0 / diag).astype(np.float32)

    def its(fn):
        _, h = fn(A, iv, b, 600, np.float32)
        d0 = float((b * iv) @ A(b * iv))
        hit = h <= eps * eps * d0
        assert hit.any(), fn.__name__
        return int(np.argmax(hit)) + 1

    a, r = its(_one_pass), its(_reference)
    assert a == r and a > 10, (a, r)

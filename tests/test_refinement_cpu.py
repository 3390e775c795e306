"""The mixed-precision wide-band solve restated on the CPU: a no-pivot
blocked FP32 band LU (64-column panels: panel LU, triangular solves, FP32
trailing update, as the device's k_wb_diag / k_wb_trsm / k_wb_update32)
with FP64 iterative refinement against the FP64 K_AA, stopped by the rule
of k_ir_check (a correction below 2^-52 |x|, or one that shrinks by less
than half).  On the oracle's first tangent of square plates it reaches the
FP64 solve's own accuracy; the contraction per sweep grows with the plate
(measured with this restatement: 0.01 per sweep at 24x24, 0.04 at 44x44,
0.09 at 64x64, where refinement still converges in nine sweeps), which is
why the device path keeps an FP64 fallback for solves that stall."""
import numpy as np
import pytest
import scipy.linalg as sl

from giraffe_gb300 import configs
from oracle import oracle

NB = 64


def _dense(ab, kl):
    return oracle._gb_dense(ab, kl)


def _lu32(A, kl, dtype=np.float32):
    """No-pivot blocked LU in FP32 (or dtype) of a band matrix held dense."""
    L = A.astype(dtype)
    n = L.shape[0]
    for j0 in range(0, n, NB):
        j1 = min(n, j0 + NB)
        r1 = min(n, j1 + kl)
        for k in range(j0, j1):
            L[k + 1:r1, k] /= L[k, k]
            if k + 1 < j1:
                L[k + 1:r1, k + 1:j1] -= np.outer(L[k + 1:r1, k], L[k, k + 1:j1])
        if j1 < n:
            L[j0:j1, j1:r1] = sl.solve_triangular(L[j0:j1, j0:j1], L[j0:j1, j1:r1], lower=True,
                                                  unit_diagonal=True, check_finite=False)
            L[j1:r1, j1:r1] -= L[j1:r1, j0:j1] @ L[j0:j1, j1:r1]
    return L


def _solve32(L, r):
    y = sl.solve_triangular(L, r.astype(L.dtype), lower=True, unit_diagonal=True, check_finite=False)
    return sl.solve_triangular(L, y, lower=False, check_finite=False).astype(np.float64)


def refine(A, b, kl, max_sweeps=30):
    """Returns (x, sweeps, fell_back, corrections) under the device's rule."""
    L = _lu32(A, kl)
    x = _solve32(L, b)
    dprev = np.abs(x).max()
    ds = []
    for k in range(1, max_sweeps + 1):
        d = _solve32(L, b - A @ x)
        x = x + d
        dn, xn = np.abs(d).max(), np.abs(x).max()
        ds.append(dn / xn)
        if dn <= 2.0 ** -52 * xn:
            return x, k, False, ds
        if dn > 0.5 * dprev:
            return x, k, dn > 2.0 ** -30 * xn, ds
        dprev = dn
    return x, max_sweeps, True, ds


@pytest.mark.parametrize("n_side", [4, 8])
def test_fp32_factor_with_fp64_refinement_reaches_the_fp64_solve(n_side):
    s = configs.square_plate(n_side, steps=20)
    ab, P, kl = oracle.first_tangent(s)
    A = _dense(ab, kl)
    x64 = np.linalg.solve(A, P)
    x, sweeps, fell_back, ds = refine(A, P, kl)
    assert not fell_back
    assert sweeps <= 8
    # the FP64 floor: as close to LAPACK's FP64 solve as the device's own
    # FP64 path (the same blocked LU in FP64) is, far below the FP32
    # factor's error
    x0 = _solve32(_lu32(A, kl), P)
    xf = _solve32(_lu32(A, kl, np.float64), P)
    err0 = np.abs(x0 - x64).max() / np.abs(x64).max()
    err64 = np.abs(xf - x64).max() / np.abs(x64).max()
    err = np.abs(x - x64).max() / np.abs(x64).max()
    assert err0 > 1e-6
    assert err <= max(4 * err64, 1e-14)
    # linear convergence: every sweep that stays above the floor gains at
    # least a factor of ten
    pairs = [(ds[i], ds[i + 1]) for i in range(len(ds) - 1) if ds[i + 1] > 10 * err64]
    assert pairs and all(b < 0.1 * a for a, b in pairs)


def test_stalled_refinement_falls_back():
    """A factor too poor to refine (here: the FP32 LU of a perturbed matrix,
    contraction above one half) stalls at once, far above the FP64 level:
    the rule hands the solve to the FP64 fallback."""
    s = configs.square_plate(4, steps=20)
    ab, P, kl = oracle.first_tangent(s)
    A = _dense(ab, kl)
    rng = np.random.default_rng(5)
    Ap = A * (1.0 + 0.9 * rng.uniform(-1, 1, A.shape) * (A != 0))
    L = _lu32(Ap, kl)
    x = _solve32(L, P)
    dprev = np.abs(x).max()
    d = _solve32(L, P - A @ x)
    x = x + d
    dn, xn = np.abs(d).max(), np.abs(x).max()
    assert dn > 0.5 * dprev and dn > 2.0 ** -30 * xn

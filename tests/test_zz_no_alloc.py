"""gf_band_solve_noalloc (static device scratch, no per-call allocation)
against gf_band_solve through the C ABI and against a CPU FP64 band solve
(scipy's LAPACK gbsv, partial pivoting) of the same system: results agree
to the band-solve tolerance of the other tests (1e-12 relative), on
consecutive calls with different sizes and bandwidths, so stale scratch from
one call cannot leak into the next.  After warm-up calls, further calls
leave the device's free memory unchanged: nothing is allocated per call."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GF_NOALLOC_MAX_N = 16384  # include/giraffe_gpu.h
GF_NOALLOC_MAX_KB = 17


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _gb_system(rng, n, kl, ku, fill=0.0):
    """Diagonally dominant band matrix in LAPACK GB storage ([n][ldab], column
    j contiguous), unreferenced entries set to `fill`, and a right-hand side."""
    ldab = 2 * kl + ku + 1
    ab = np.full((n, ldab), fill)
    for j in range(n):
        i0, i1 = max(0, j - ku), min(n, j + kl + 1)
        ab[j, kl + ku + i0 - j: kl + ku + i1 - j] = rng.normal(size=i1 - i0)
        ab[j, kl + ku] += 4 * (kl + ku + 1)
    return ab, rng.normal(size=n)


def _cpu_solve(ab, kl, ku, b):
    """FP64 solve of the same GB system on the host (LAPACK gbsv through
    scipy), from the stored band rows kl .. 2kl+ku of every column."""
    from scipy.linalg import solve_banded

    n = ab.shape[0]
    bands = np.ascontiguousarray(ab[:, kl:2 * kl + ku + 1].T)  # (kl+ku+1) x n, LAPACK's banded form
    bands = np.where(np.isnan(bands), 0.0, bands)
    return solve_banded((kl, ku), bands, b)


def test_noalloc_matches_band_solve_on_consecutive_calls(gpu_ctx):
    rng = np.random.default_rng(7)
    cases = [(5000, 17, 17, 0.0), (5000, 17, 17, 0.0), (3001, 3, 9, np.nan), (GF_NOALLOC_MAX_N, 17, 5, 0.0),
             (64, 0, 2, np.nan)]
    for n, kl, ku, fill in cases:
        ab, b = _gb_system(rng, n, kl, ku, fill)
        x_ref, info_ref = gpu_ctx.band_solve(ab, kl, ku, b)
        x1, info1 = gpu_ctx.band_solve_noalloc(ab, kl, ku, b)
        x2, info2 = gpu_ctx.band_solve_noalloc(ab, kl, ku, b)
        assert info_ref == info1 == info2 == 0
        assert np.isfinite(x1).all() and np.isfinite(x2).all()
        assert rel(x1, x_ref) < 1e-12, (n, kl, ku)
        assert rel(x2, x_ref) < 1e-12, (n, kl, ku)
        x_cpu = _cpu_solve(ab, kl, ku, b)
        assert rel(x1, x_cpu) < 1e-12, (n, kl, ku)
        assert rel(x2, x_cpu) < 1e-12, (n, kl, ku)


def test_noalloc_calls_leave_free_device_memory_unchanged(gpu_ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    ab, b = _gb_system(rng, 8000, 17, 11)
    for _ in range(2):  # warm-up: loads the kernels, looks up the scratch address
        gpu_ctx.band_solve_noalloc(ab, 17, 11, b)
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(5):
        x, info = gpu_ctx.band_solve_noalloc(ab, 17, 11, b)
        assert info == 0
    free1 = torch.cuda.mem_get_info(0)[0]
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_bands_wider_than_17(gpu_ctx):
    n, kl, ku = 200, GF_NOALLOC_MAX_KB + 1, 3
    rng = np.random.default_rng(3)
    ab, b = _gb_system(rng, n, kl, ku)
    with pytest.raises(RuntimeError, match="kl, ku must be <= 17"):
        gpu_ctx.band_solve_noalloc(ab, kl, ku, b)
    # the same system through gf_band_solve (wide branch) still solves
    x, info = gpu_ctx.band_solve(ab, kl, ku, b)
    assert info == 0 and rel(x, _cpu_solve(ab, kl, ku, b)) < 1e-12


def test_noalloc_reports_zero_pivot(gpu_ctx):
    ab = np.zeros((4, 4))
    ab[:, 2] = [1.0, 0.0, 2.0, 3.0]  # kl = ku = 1: diagonal at row kl + ku
    _, info = gpu_ctx.band_solve_noalloc(ab, 1, 1, np.ones(4))
    assert info == 1


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu_ctx):
    n = GF_NOALLOC_MAX_N + 1
    ab = np.zeros((n, 3))
    ab[:, 1] = 1.0
    with pytest.raises(RuntimeError, match="GF_NOALLOC_MAX_N"):
        gpu_ctx.band_solve_noalloc(ab, 1, 0, np.ones(n))

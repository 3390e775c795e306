"""gf_sparse_solve (the sparsesystem drop-in on SparseMatrix's CSR) and the
wide branch of gf_band_solve (bandsystem with kl or ku above 17), through the
C ABI, against LAPACK's dense LU (numpy) on the same FP64 inputs.  Both GPU
paths factor without pivoting, so the matrices here are diagonally dominant
or near-SPD, as K_AA is; the tolerance is 1e-11 relative to max|x| (FP64
round-off of banded LU at these sizes), and 1e-10 for the plate K_AA."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu

pytestmark = pytest.mark.gpu


def banded(n, kl, ku, seed, sym=False):
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n))
    for d in range(-kl, ku + 1):
        k = np.arange(max(0, -d), min(n, n - d))
        A[k, k + d] = rng.uniform(-1.0, 1.0, len(k))
    if sym:
        A = 0.5 * (A + A.T)
    A[np.arange(n), np.arange(n)] = np.abs(A).sum(axis=1) + 1.0
    return A


def to_csr(A):
    rows, cols = np.nonzero(A)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    rp = np.zeros(A.shape[0] + 1, dtype=np.int32)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp).astype(np.int32), cols.astype(np.int32), A[rows, cols]


def to_gb(A, kl, ku):
    n = A.shape[0]
    ab = np.zeros((n, 2 * kl + ku + 1))
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[j, kl + ku + i - j] = A[i, j]
    return ab


def close(x, ref, tol=1e-11):
    return np.abs(x - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("n,kl,ku", [(300, 4, 6), (700, 40, 25), (130, 70, 70)])
def test_sparse_solve_matches_dense(gpu_ctx, n, kl, ku):
    A = banded(n, kl, ku, seed=n + kl)
    b = np.random.default_rng(1).normal(size=n)
    x, info = gpu_ctx.sparse_solve(*to_csr(A), b)
    assert info == 0
    assert close(x, np.linalg.solve(A, b))


def test_sparse_solve_reorders_a_scrambled_band(gpu_ctx):
    """A band matrix under a random symmetric permutation: the natural
    ordering is wide, reverse Cuthill-McKee recovers a narrow band."""
    n = 900
    A0 = banded(n, 3, 3, seed=5, sym=True)
    p = np.random.default_rng(2).permutation(n)
    A = A0[np.ix_(p, p)]
    b = np.random.default_rng(3).normal(size=n)
    x, info = gpu_ctx.sparse_solve(*to_csr(A), b)
    assert info == 0
    assert close(x, np.linalg.solve(A, b))


def test_sparse_solve_sums_repeated_entries(gpu_ctx):
    """Entries repeated within a row add up, as SparseMatrix's triplets do."""
    n = 200
    A = banded(n, 30, 30, seed=9)
    rp, ci, v = to_csr(A)
    # split every value into two entries of the same (row, column)
    rp2 = rp * 2
    ci2 = np.repeat(ci, 2)
    v2 = np.empty(2 * len(v))
    v2[0::2] = 0.25 * v
    v2[1::2] = 0.75 * v
    b = np.ones(n)
    x, info = gpu_ctx.sparse_solve(rp2, ci2, v2, b)
    assert info == 0
    assert close(x, np.linalg.solve(A, b), 1e-10)


def test_sparse_solve_reports_zero_pivot(gpu_ctx):
    n = 160
    A = banded(n, 20, 20, seed=4)
    A[0, :] = 0.0
    A[:, 0] = 0.0
    rp, ci, v = to_csr(A)  # row and column 0 hold no entries: the first pivot is zero
    _, info = gpu_ctx.sparse_solve(rp, ci, v, np.ones(n))
    assert info == 1


def test_sparse_solve_rejects_bad_csr(gpu_ctx):
    rp = np.array([0, 2, 1], dtype=np.int32)
    with pytest.raises(RuntimeError):
        gpu_ctx.sparse_solve(rp, np.array([0], dtype=np.int32), np.array([1.0]), np.ones(2))
    with pytest.raises(RuntimeError):
        gpu_ctx.sparse_solve(np.array([0, 1, 2], dtype=np.int32), np.array([0, 5], dtype=np.int32),
                             np.ones(2), np.ones(2))


@pytest.mark.parametrize("n,kl,ku", [(500, 30, 22), (257, 18, 40)])
def test_wide_band_solve_matches_dense(gpu_ctx, n, kl, ku):
    A = banded(n, kl, ku, seed=kl * ku)
    b = np.random.default_rng(6).normal(size=n)
    x, info = gpu_ctx.band_solve(to_gb(A, kl, ku), kl, ku, b)
    assert info == 0
    assert close(x, np.linalg.solve(A, b))


def backward_error(A, x, b):
    return np.abs(A @ x - b).max() / (np.abs(A).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())


@pytest.mark.parametrize("kind", ["plate", "chain"])
def test_first_pass_K_AA_solves_alike_in_csr_and_band(gpu_ctx, kind):
    """The first Newton pass's K_AA of a Shell_1 plate and of a pipe chain,
    read back in the CSR and the GB layouts and solved by gf_sparse_solve and
    gf_band_solve: backward error at FP64 round-off (1e-14) for both.  The
    plate's increment also matches a dense LU to 1e-10; the chain's K_AA is
    too ill-conditioned (condition ~ n_e^4) for a forward comparison, but
    there both calls reach the same 35-row band solver in the same
    numbering, so they agree bit for bit."""
    s = configs.square_plate(6, steps=10) if kind == "plate" else \
        configs.pipe_chain(60, 0.4, 0.03, [1e5, 2e4, -3e4])
    b = gpu.BatchSolver(gpu_ctx, [s])
    rp, ci, v, P = b.assemble_csr(0)
    ab, P2, kb = b.assemble(0)
    b.close()
    n = len(P)
    A = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(rp))
    A[rows, ci] = v
    assert np.array_equal(P, P2)
    x, info = gpu_ctx.sparse_solve(rp, ci, v, P)
    assert info == 0
    xb, info = gpu_ctx.band_solve(ab, kb, kb, P2)
    assert info == 0
    assert backward_error(A, x, P) < 1e-14
    assert backward_error(A, xb, P) < 1e-14
    if kind == "plate":
        ref = np.linalg.solve(A, P)
        assert close(x, ref, 1e-10)
        assert close(xb, ref, 1e-10)
    else:
        assert np.array_equal(x, xb)

"""Parity at the benchmarked sizes, through the C ABI.

The bench's workloads themselves, not smaller stand-ins:

* batched static chains (512 pipe chains, 50-2000 elements, seed 0): a
  size-stratified sample of 8 that holds the longest chains (n_e >= 1500,
  24k DOF, where the bending operator's condition number is near 1e13),
  against the oracle;
* batched dynamics (256 risers of 100-1000 elements, seed 0): a sample of 6
  with the longest risers, over the first 50 of the 1000 time steps;
* the plate family at a half-bandwidth of 506 (24x24x2, 11,667 free DOFs),
  whose trailing updates span eight 64-wide tiles per window row, all 20
  load steps against the reference build, with the tensor-core update and
  the FP64 one;
* the 64x64x2 plate's first K_AA (84,867 DOFs, half-bandwidth 1346) solved
  by gf_sparse_solve with the tensor-core and the FP64 update, by backward
  error and against a CPU FP64 band solve (LAPACK gbsv);
* a band whose rows span 1e8 in magnitude (a diagonal scaling of a
  well-conditioned band, as translational and rotational DOFs scale the
  shell's K_AA), where per-row slicing alone would lose about eight digits:
  the tensor-core solve agrees with the FP64 one to FP64 accuracy.

Relative error = ||u - u_oracle||_2 / ||u_oracle||_2 over the converged
nodal translations (u = position - reference position); the nodal rotation
tensors are compared entry by entry.  Tolerance: 1e-10 with identical
converged steps, Newton iterations and bisections.
"""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _solve(ctx, structs, **opts):
    b = gpu.BatchSolver(ctx, structs, ctx.opts(**opts))
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


def _rel_u(s, f, fo):
    u, uo = f[:, :3] - s.nodes, fo[:, :3] - s.nodes
    return float(np.linalg.norm(u - uo) / np.linalg.norm(uo))


def _stratified(structs, k):
    order = np.argsort([len(s.beams) for s in structs])
    return [structs[i] for i in order[np.linspace(0, len(order) - 1, k).astype(int)]]


def test_batched_static_sample_with_the_longest_chains_matches_oracle(gpu_ctx):
    sample = _stratified(configs.batched_static(512, seed=0), 8)
    assert max(len(s.beams) for s in sample) >= 1500
    finals, stats = _solve(gpu_ctx, sample)
    fo, so, fails = oracle.solve_batch(sample, threads=8)
    assert fails == 0
    for k, s in enumerate(sample):
        assert list(stats[k]) == list(so[k]), (len(s.beams), stats[k], so[k])
        assert _rel_u(s, finals[k], fo[k]) <= TOL, len(s.beams)
        assert np.abs(finals[k][:, 6:] - fo[k][:, 6:]).max() <= 1e-9, len(s.beams)


def test_batched_dynamics_sample_with_the_longest_risers_matches_oracle(gpu_ctx):
    structs = configs.batched_dynamic(256, seed=0)
    sample = _stratified(structs, 6)
    assert max(len(s.beams) for s in sample) >= 950
    for s in sample:
        s.solution.end_time = 50 * 0.01
    finals, stats = _solve(gpu_ctx, sample)
    fo, so, fails = oracle.solve_batch(sample, threads=8)
    assert fails == 0
    for k, s in enumerate(sample):
        assert stats[k][0] == 50 and stats[k][3] == 0
        assert list(stats[k]) == list(so[k]), (len(s.beams), stats[k], so[k])
        assert _rel_u(s, finals[k], fo[k]) <= TOL, len(s.beams)
        assert np.abs(finals[k][:, 6:] - fo[k][:, 6:]).max() <= 1e-9, len(s.beams)


@pytest.mark.parametrize("update", ["tensor", "fp64"])
def test_plate_24_with_many_update_tiles_matches_reference(gpu_ctx, golden, update):
    g = golden("ref_plate24.npz")
    s = configs.square_plate(24, steps=20)
    wide = gpu.GF_WIDE_TENSOR if update == "tensor" else gpu.GF_WIDE_FP64
    finals, stats = _solve(gpu_ctx, [s], wide_update=wide)
    ref = g["nodes"][-1]
    assert _rel_u(s, finals[0], ref) <= TOL
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9
    steps = g["steps"]
    conv = steps[steps[:, 2] == 0]
    assert stats[0][0] == len(conv) == 20
    assert stats[0][3] == 0
    # the reference's Newton solves over its converged steps, plus the
    # pass of each step that finds it converged
    assert stats[0][1] == int(conv[:, 1].sum() + len(conv))


def _csr_matvec(rp, ci, v, x):
    from scipy.sparse import csr_matrix

    n = len(rp) - 1
    return csr_matrix((v, ci, rp), shape=(n, n)) @ x


def _backward_error(rp, ci, v, x, b):
    """||b - K x||_inf / (||K||_inf ||x||_inf + ||b||_inf)."""
    from scipy.sparse import csr_matrix

    n = len(rp) - 1
    K = csr_matrix((v, ci, rp), shape=(n, n))
    r = b - K @ x
    normK = float(np.abs(K).sum(axis=1).max())
    return float(np.abs(r).max() / (normK * np.abs(x).max() + np.abs(b).max()))


def test_plate_64_first_solve_tensor_and_fp64_by_backward_error(gpu_ctx):
    from scipy.linalg import solve_banded
    from scipy.sparse import csr_matrix

    s = configs.square_plate(64, steps=20)
    b = gpu.BatchSolver(gpu_ctx, [s])
    rp, ci, v, P = b.assemble_csr(0)
    b.close()
    xs = {}
    try:
        for name, mode in (("tensor", gpu.GF_WIDE_TENSOR), ("fp64", gpu.GF_WIDE_FP64)):
            gpu_ctx.set_standalone_opts(wide_update=mode)
            x, info = gpu_ctx.sparse_solve(rp, ci, v, P)
            assert info == 0
            xs[name] = x
    finally:
        gpu_ctx.set_standalone_opts(wide_update=gpu.GF_WIDE_TENSOR)
    # CPU FP64 band solve (partial pivoting) in the reference's numbering
    n = len(P)
    K = csr_matrix((v, ci, rp), shape=(n, n)).tocoo()
    kl = int((K.row - K.col).max())
    ku = int((K.col - K.row).max())
    ab = np.zeros((kl + ku + 1, n))
    ab[ku + K.row - K.col, K.col] = K.data
    x_cpu = solve_banded((kl, ku), ab, P)
    be = {k: _backward_error(rp, ci, v, x, P) for k, x in xs.items()}
    be["cpu"] = _backward_error(rp, ci, v, x_cpu, P)
    assert be["tensor"] <= 1e-14 and be["fp64"] <= 1e-14, be
    # forward differences are bounded by the condition number times the
    # backward error (the plate's K_AA is near 1e9 conditioned): the two
    # GPU updates and the pivoting CPU solve agree to about 1e-9
    for k in ("tensor", "fp64"):
        assert np.linalg.norm(xs[k] - x_cpu) / np.linalg.norm(x_cpu) <= 1e-8, k
    assert np.linalg.norm(xs["tensor"] - xs["fp64"]) / np.linalg.norm(xs["fp64"]) <= 1e-8


def _scaled_band(rng, n, w, spread):
    """A = S B S in LAPACK GB storage ([n][ldab], column j contiguous): B a
    diagonally dominant band (half-bandwidths w), S = diag(s) with s = spread
    on every third DOF and 1 elsewhere, so each row of A holds entries about
    `spread` apart in magnitude.  Also returns s and B in LAPACK's banded
    form."""
    ldab = 3 * w + 1
    s = np.where(np.arange(n) % 3 == 0, spread, 1.0)
    ab = np.zeros((n, ldab))
    bb = np.zeros((2 * w + 1, n))
    for j in range(n):
        i0, i1 = max(0, j - w), min(n, j + w + 1)
        col = rng.normal(size=i1 - i0)
        col[j - i0] += 4.0 * (2 * w + 1)
        ab[j, 2 * w + i0 - j: 2 * w + i1 - j] = s[i0:i1] * col * s[j]
        bb[w + i0 - j: w + i1 - j, j] = col
    return ab, s, bb


def test_tensor_core_update_keeps_fp64_accuracy_on_rows_spanning_1e8(gpu_ctx):
    from scipy.linalg import solve_banded

    rng = np.random.default_rng(5)
    n, w, spread = 3000, 300, 1e4  # entries of a row span spread^2 = 1e8
    ab, s, bb = _scaled_band(rng, n, w, spread)
    b = s * rng.normal(size=n)
    xs = {}
    try:
        for name, mode in (("tensor", gpu.GF_WIDE_TENSOR), ("fp64", gpu.GF_WIDE_FP64)):
            gpu_ctx.set_standalone_opts(wide_update=mode)
            x, info = gpu_ctx.band_solve(ab, w, w, b)
            assert info == 0
            xs[name] = x
    finally:
        gpu_ctx.set_standalone_opts(wide_update=gpu.GF_WIDE_TENSOR)
    # the CPU FP64 reference solves the well-scaled system B (S x) = S^-1 b
    # (partial pivoting on A itself is not scale invariant and loses digits)
    x_cpu = solve_banded((w, w), bb, b / s) / s
    # errors in the scaled unknowns S x, where B is well conditioned
    def err(x, y):
        return np.linalg.norm(s * (x - y)) / np.linalg.norm(s * y)

    assert err(xs["fp64"], x_cpu) <= 1e-13
    assert err(xs["tensor"], x_cpu) <= 1e-13
    assert err(xs["tensor"], xs["fp64"]) <= 1e-13

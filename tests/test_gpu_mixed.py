"""Mixed-precision path (GF_PREC_MIXED, through the C ABI): the Beam_1
tangent operator in FP32-pair arithmetic, the internal force, residual,
rotations and solves in FP64.  Stated tolerance: every converged nodal
displacement within 1e-8 relative of the FP64 oracle; the Newton trajectory
is unchanged (same step and iteration counts)."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu


def _run(ctx, structs, precision):
    b = gpu.BatchSolver(ctx, structs, ctx.opts(precision))
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


def test_mixed_chains_within_1e8_of_the_oracle(gpu_ctx):
    structs = configs.batched_static(12, seed=7, n_max=800) + [configs.cantilever_rollup(), configs.tutorial01()]
    fm, sm = _run(gpu_ctx, structs, gpu.GF_PREC_MIXED)
    ff, sf = _run(gpu_ctx, structs, gpu.GF_PREC_FP64)
    for k, s in enumerate(structs):
        fo, so, _ = oracle.solve(s, 0)
        assert tuple(sm[k]) == tuple(so), k
        u_o = fo[:, :3] - s.nodes
        u_m = fm[k][:, :3] - s.nodes
        assert np.linalg.norm(u_m - u_o) <= 1e-8 * np.linalg.norm(u_o), k
        assert np.abs(fm[k][:, 6:] - fo[:, 6:]).max() <= 1e-8, k
    assert np.array_equal(sm, sf)


def test_mixed_dynamics_within_1e8_of_fp64(gpu_ctx):
    structs = configs.batched_dynamic(4, seed=3, n_min=60, n_max=120, steps=40)
    fm, sm = _run(gpu_ctx, structs, gpu.GF_PREC_MIXED)
    ff, sf = _run(gpu_ctx, structs, gpu.GF_PREC_FP64)
    assert np.array_equal(sm, sf)
    for k, s in enumerate(structs):
        u_f = ff[k][:, :3] - s.nodes
        u_m = fm[k][:, :3] - s.nodes
        assert np.linalg.norm(u_m - u_f) <= 1e-8 * np.linalg.norm(u_f), k

"""FP32 wide-band factor with FP64 iterative refinement (GF_PREC_MIXED on
Shell_1 structures, through the C ABI).  The refinement runs until the
corrections stop shrinking, i.e. to the FP64 floor, so a plate solves as the
reference does: the same step and iteration counts and 1e-10 relative to
the reference's golden states, the plain FP64 path's stated tolerance.  A
solve whose refinement stops early falls back to the FP64 LU, and that
solve is the FP64 path's, bit for bit."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu


def _run(ctx, structs, **kw):
    b = gpu.BatchSolver(ctx, structs, ctx.opts(**kw))
    b.reset()
    b.run()
    finals, stats = b.results()
    extra = b.solve_stats()
    b.close()
    return finals, stats, extra


@pytest.mark.parametrize("name,make", [
    ("ref_plate.npz", lambda: configs.square_plate(4, steps=20)),
    ("ref_plate_fixed_area.npz", lambda: configs.square_plate(3, steps=10, area_update=0)),
])
def test_mixed_plate_matches_reference(gpu_ctx, golden, name, make):
    g = golden(name)
    finals, stats, extra = _run(gpu_ctx, [make()], precision=gpu.GF_PREC_MIXED)
    ref = g["nodes"][-1]
    assert stats[0][3] == 0
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9
    steps = g["steps"]
    conv = steps[steps[:, 2] == 0]
    assert stats[0][0] == len(conv)
    assert stats[0][1] == int(conv[:, 1].sum() + len(conv))
    solves, sweeps, fallbacks = extra[0]
    assert fallbacks == 0
    # every solve refines at least once, and a small plate within a dozen sweeps
    assert solves <= sweeps <= 12 * solves


def test_mixed_fallback_is_the_fp64_solve(gpu_ctx):
    """max_refine = 1 stops every refinement after one sweep, short of the
    FP64 level: each solve is refactored in FP64 from the saved right-hand
    side, so the run is the FP64 run exactly."""
    fm, sm, em = _run(gpu_ctx, [configs.square_plate(4, steps=20)], precision=gpu.GF_PREC_MIXED, max_refine=1)
    ff, sf, ef = _run(gpu_ctx, [configs.square_plate(4, steps=20)], precision=gpu.GF_PREC_FP64)
    assert np.array_equal(sm, sf)
    assert np.array_equal(fm[0], ff[0])
    assert em[0][2] == em[0][0] > 0
    assert ef[0][1] == 0 and ef[0][2] == 0


def test_mixed_finer_plate_beside_chains(gpu_ctx):
    """A 16x16x2 plate (3,000 DOFs, several panels) and a smaller one beside
    a beam chain in one mixed batch: the plates as the FP64 path solves them
    (same counts, 1e-10 of the displacement scale), the chain within the
    mixed Beam_1 tangent's 1e-8 of the oracle; the launched (host-driven)
    refinement gives the captured one's results bit for bit."""
    make = lambda: [configs.square_plate(16, steps=6), configs.square_plate(5, steps=4, area_update=0),
                    configs.pipe_chain(40, 0.4, 0.03, [1e5, 2e4, -3e4])]
    fm, sm, em = _run(gpu_ctx, make(), precision=gpu.GF_PREC_MIXED)
    ff, sf, _ = _run(gpu_ctx, make(), precision=gpu.GF_PREC_FP64)
    fl, sl, el = _run(gpu_ctx, make(), precision=gpu.GF_PREC_MIXED, use_graph=False)
    structs = make()
    assert np.array_equal(sm, sf)
    for k in (0, 1):
        scale = np.abs(ff[k][:, :3] - structs[k].nodes).max()
        assert np.abs(fm[k][:, :3] - ff[k][:, :3]).max() <= 1e-10 * scale, k
        assert em[k][2] == 0 and em[k][1] >= em[k][0], k
    fo, so, _ = oracle.solve(structs[2], 0)
    assert tuple(sm[2]) == tuple(so)
    u_o = fo[:, :3] - structs[2].nodes
    assert np.linalg.norm(fm[2][:, :3] - structs[2].nodes - u_o) <= 1e-8 * np.linalg.norm(u_o)
    assert np.array_equal(sl, sm) and np.array_equal(el, em)
    for k in range(3):
        assert np.array_equal(fl[k], fm[k]), k

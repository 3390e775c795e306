"""Solution steps in sequence on the CUDA path (gf_model_desc.next_steps):
each step starts from the state the previous one ends in, with its own step
control, Newmark parameters, Rayleigh matrices and initial velocities, as the
reference's main loop runs them.  Against the reference's goldens (1e-10
relative on positions) and the oracle (same counts)."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu


def _solve(ctx, structs):
    b = gpu.BatchSolver(ctx, structs)
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


@pytest.mark.parametrize("name,make", [("ref_plate_release.npz", lambda: configs.plate_release(3)),
                                       ("ref_chain_sequence.npz", configs.chain_sequence)])
def test_sequences_match_reference(gpu_ctx, golden, name, make):
    s = make()
    g = golden(name)
    finals, stats = _solve(gpu_ctx, [s])
    ref = g["nodes"][-1]
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9
    assert stats[0][0] == len(g["steps"]) and stats[0][3] == 0
    _, so, _ = oracle.solve(s)
    assert list(stats[0]) == list(so)


def test_sequences_share_a_batch_with_single_steps(gpu_ctx):
    """Multi-step and single-step structures of both element families in one
    batch, each bit-identical to its run alone and equal to the oracle."""
    mix = [configs.chain_sequence(), configs.riser_chain(25, 0.4, 0.03, 1.0, 5.0, steps=30),
           configs.plate_release(3, static_steps=3, dynamic_steps=8), configs.chain_sequence(12),
           configs.cantilever_rollup()]
    finals, stats = _solve(gpu_ctx, mix)
    for k, s in enumerate(mix):
        fo, so, _ = oracle.solve(s)
        assert list(stats[k]) == list(so), k
        scale = np.abs(fo[:, :3]).max()
        assert np.abs(finals[k][:, :3] - fo[:, :3]).max() <= 1e-10 * scale, k
        alone, st1 = _solve(gpu_ctx, [s])
        assert np.array_equal(alone[0], finals[k]), k


def test_zero_ic_is_honoured(gpu_ctx):
    """Dropping ZeroIC from the third step changes the motion of that step."""
    a = configs.chain_sequence()
    b = configs.chain_sequence()
    b.next_steps = b.next_steps[:2]
    c = configs.chain_sequence()
    c.next_steps = c.next_steps[:2]
    c.next_steps[1].zero_ic = 0
    fa, _ = _solve(gpu_ctx, [b])
    fc, _ = _solve(gpu_ctx, [c])
    fo_b, _, _ = oracle.solve(b)
    fo_c, _, _ = oracle.solve(c)
    scale = np.abs(fo_b[:, :3]).max()
    assert np.abs(fa[0][:, :3] - fo_b[:, :3]).max() <= 1e-10 * scale
    assert np.abs(fc[0][:, :3] - fo_c[:, :3]).max() <= 1e-10 * scale
    assert np.abs(fo_b[:, :3] - fo_c[:, :3]).max() > 1e-3


def test_reference_tutorial05(gpu_ctx, golden):
    """The reference's own Shell_1 deck: a strip of 400 six-node triangles
    loaded at its tip in a Static step (with bisections), then released into
    a Dynamic step of 80 Newmark steps.  The final configuration and the
    step counts as the reference writes them."""
    from giraffe_gb300.deck import read_deck

    g = golden("ref_tutorial05.npz")
    s = read_deck(str(g["deck"]))
    assert len(s.shells) == 400 and len(s.next_steps) == 1
    finals, stats = _solve(gpu_ctx, [s])
    steps = g["steps"]
    assert stats[0][0] == int((steps[:, 2] == 0).sum())
    assert stats[0][2] == int((steps[:, 2] == 1).sum()) and stats[0][3] == 0
    ref = g["nodes"][-1]
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9

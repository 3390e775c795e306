"""Implicit dynamics on the CUDA path (Beam_1 inertia, Newmark, Dynamic
step control) against the reference's goldens and the oracle; FP64, stated
tolerance 1e-10 relative on positions (1e-12 on element matrices)."""
import numpy as np
import pytest

from giraffe_gb300 import configs
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_beam_inertia_matches_reference(gpu_ctx, golden):
    g = golden("ref_beam_inertia.npz")
    for i in range(len(g["M"])):
        nh = int(g["n_hist"][i])
        hist = g["hist"][i][None, :nh] if nh else None
        M, F = gpu_ctx.beam_inertia(g["xyz"][i:i + 1], g["mat"][i:i + 1], g["sec6"][i:i + 1], g["cs"][i:i + 1], hist,
                                    g["disp"][i:i + 1], g["vel"][i:i + 1], g["acc"][i:i + 1], float(g["dt"][i]),
                                    float(g["beta"][i]), float(g["gamma"][i]))
        assert rel(M[0], g["M"][i]) < 1e-12, i
        assert rel(F[0], g["F"][i]) < 1e-12, i


def _solve(ctx, structs):
    from giraffe_gb300 import gpu

    b = gpu.BatchSolver(ctx, structs)
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


def test_tutorial10_matches_reference(gpu_ctx, golden):
    s = configs.tutorial10()
    g = golden("ref_tutorial10.npz")
    finals, stats = _solve(gpu_ctx, [s])
    ref_final = g["nodes"][-1]
    scale = np.abs(ref_final[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref_final[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref_final[:, 6:]).max() <= 1e-9
    _, so, _ = oracle.solve(s)
    assert list(stats[0]) == list(so)


def test_riser_batch_matches_oracle(gpu_ctx):
    rng = np.random.default_rng(4)
    structs = [configs.riser_chain(int(n), 0.4, 0.03, float(a), float(p), steps=60)
               for n, a, p in zip(rng.integers(20, 80, 6), rng.uniform(0.5, 2, 6), rng.uniform(5, 15, 6))]
    finals, stats = _solve(gpu_ctx, structs)
    for s, f, st in zip(structs, finals, stats):
        fo, so, _ = oracle.solve(s)
        assert list(st) == list(so)
        scale = np.abs(fo[:, :3]).max()
        assert np.abs(f[:, :3] - fo[:, :3]).max() <= 1e-10 * scale


def test_static_and_dynamic_in_one_batch(gpu_ctx):
    """Structures of both solution types share a batch; each result equals the
    one it gets alone."""
    mix = [configs.riser_chain(30, 0.35, 0.025, 1.0, 6.0, steps=40), configs.cantilever_rollup(),
           configs.riser_chain(45, 0.45, 0.03, 0.7, 9.0, steps=40)]
    finals, stats = _solve(gpu_ctx, mix)
    for k, s in enumerate(mix):
        alone, st1 = _solve(gpu_ctx, [s])
        assert np.array_equal(alone[0], finals[k])
        assert list(st1[0]) == list(stats[k])


@pytest.mark.parametrize("name,update", [("ref_tutorial10_rayleigh.npz", 0), ("ref_tutorial10_rayleigh_update.npz", 1)])
def test_tutorial10_rayleigh_matches_reference(gpu_ctx, golden, name, update):
    """Rayleigh damping (MountDamping: C = alpha M_modal + beta K, formed at
    the step's first iteration or, with Update 1, at every iteration) against
    the reference's own run: same positions to 1e-10, same iteration counts
    as the oracle."""
    s = configs.tutorial10(0.2, 0.002, update)
    g = golden(name)
    finals, stats = _solve(gpu_ctx, [s])
    ref_final = g["nodes"][-1]
    scale = np.abs(ref_final[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref_final[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref_final[:, 6:]).max() <= 1e-9
    _, so, _ = oracle.solve(s)
    assert list(stats[0]) == list(so)


def test_riser_rayleigh_matches_reference(gpu_ctx, golden):
    s = configs.riser_chain(12, 0.4, 0.03, 1.0, 4.0, steps=120, element_length=2.0, rayleigh_alpha=0.3,
                            rayleigh_beta=0.004, update_rayleigh=1)
    g = golden("ref_riser_rayleigh.npz")
    finals, stats = _solve(gpu_ctx, [s])
    ref_final = g["nodes"][-1]
    scale = np.abs(ref_final[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref_final[:, :3]).max() <= 1e-10 * scale
    steps = g["steps"]
    conv = steps[steps[:, 2] == 0]
    assert stats[0][0] == len(conv)


def test_damped_and_undamped_risers_in_one_batch_match_the_oracle(gpu_ctx):
    """Damped (both Update modes) and undamped risers in one batch, each as
    the oracle solves it."""
    rng = np.random.default_rng(9)
    structs = []
    for k, (n, a, p) in enumerate(zip(rng.integers(20, 60, 6), rng.uniform(0.5, 2, 6), rng.uniform(5, 15, 6))):
        ray = (0.0, 0.0) if k % 3 == 0 else (0.25, 0.003)
        structs.append(configs.riser_chain(int(n), 0.4, 0.03, float(a), float(p), steps=50, rayleigh_alpha=ray[0],
                                           rayleigh_beta=ray[1], update_rayleigh=k % 2))
    finals, stats = _solve(gpu_ctx, structs)
    for s, f, st in zip(structs, finals, stats):
        fo, so, _ = oracle.solve(s)
        assert list(st) == list(so)
        scale = np.abs(fo[:, :3]).max()
        assert np.abs(f[:, :3] - fo[:, :3]).max() <= 1e-10 * scale

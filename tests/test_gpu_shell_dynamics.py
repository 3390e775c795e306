"""Shell_1 in Dynamic steps on the CUDA path (MountMass of the director
fibre, Rayleigh damping with the modal mass, Newmark) against the
reference's goldens and the oracle; FP64, stated tolerance 1e-12 relative on
element matrices and 1e-10 relative on positions."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_shell_inertia_matches_reference(gpu_ctx, golden):
    """gf_shell_inertia_elements against Shell_1::MountMass run by the
    reference: the whole matrix, and the rotational blocks on their own
    (four to six orders smaller)."""
    g = golden("ref_shell_inertia.npz")
    for i in range(len(g["M"])):
        nh = int(g["n_hist"][i])
        hist = g["hist"][i][None, :nh] if nh else None
        M, F = gpu_ctx.shell_inertia(g["xyz"][i:i + 1], g["mat"][i:i + 1], g["thick"][i:i + 1], hist,
                                     g["disp"][i:i + 1], g["vel"][i:i + 1], g["acc"][i:i + 1], float(g["dt"][i]),
                                     float(g["beta"][i]), float(g["gamma"][i]))
        assert rel(M[0], g["M"][i]) < 1e-12, i
        assert rel(M[0][18:, 18:], g["M"][i][18:, 18:]) < 1e-12, i
        assert rel(F[0], g["F"][i]) < 1e-12, i
        assert rel(F[0][18:], g["F"][i][18:]) < 1e-12, i


def _solve(ctx, structs):
    b = gpu.BatchSolver(ctx, structs)
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


DECKS = [
    ("ref_plate_dynamic.npz", {}),
    ("ref_plate_dynamic_rayleigh.npz", dict(area_update=0, rayleigh_alpha=8.0, rayleigh_beta=2e-5)),
    ("ref_plate_dynamic_rayleigh_update.npz", dict(rayleigh_alpha=8.0, rayleigh_beta=2e-5, update_rayleigh=1)),
]


@pytest.mark.parametrize("name,kw", DECKS)
def test_plate_dynamics_matches_reference(gpu_ctx, golden, name, kw):
    """A clamped plate set vibrating by a quickly applied follower pressure,
    undamped, damped with C formed once (AreaUpdate 0) and damped with C
    formed at every iteration: the final configuration as the reference
    writes it, and the oracle's step and iteration counts."""
    s = configs.plate_dynamics(3, steps=20, **kw)
    g = golden(name)
    finals, stats = _solve(gpu_ctx, [s])
    ref = g["nodes"][-1]
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9
    _, so, _ = oracle.solve(s)
    assert list(stats[0]) == list(so)


def test_plate_dynamics_batch_matches_oracle(gpu_ctx):
    """Larger plates, damped and undamped, with Beam_1 risers and a static
    plate in one batch: each against the oracle, and each equal bit for bit
    to its result alone."""
    mix = [configs.plate_dynamics(6, steps=8, rayleigh_alpha=5.0, rayleigh_beta=1e-5, update_rayleigh=1),
           configs.riser_chain(30, 0.35, 0.025, 1.0, 6.0, steps=30, rayleigh_alpha=0.2, rayleigh_beta=0.003),
           configs.plate_dynamics(5, steps=8, pressure=2e5),
           configs.square_plate(4, steps=5)]
    finals, stats = _solve(gpu_ctx, mix)
    for k, s in enumerate(mix):
        fo, so, _ = oracle.solve(s)
        assert list(stats[k]) == list(so), k
        scale = np.abs(fo[:, :3]).max()
        assert np.abs(finals[k][:, :3] - fo[:, :3]).max() <= 1e-10 * scale, k
        alone, st1 = _solve(gpu_ctx, [s])
        assert np.array_equal(alone[0], finals[k]), k
        assert list(st1[0]) == list(stats[k]), k

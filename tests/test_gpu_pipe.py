"""Pipe_1 on the CUDA path: PipeSection constants through the Beam_1
kernels, PipeLoad internal pressure in k_pipe_pressure (its load stiffness
in the element tangent), against the reference's goldens and the oracle.
FP64; stated tolerances: 1e-13 relative on assembled K_AA / P_A, 1e-10
relative on positions, and the oracle's step / iteration / bisection counts
exactly."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from giraffe_gb300.model import PipeLoad, Structure, Table
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _solve(ctx, structs):
    b = gpu.BatchSolver(ctx, structs)
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


def _static_pipes(n_el, pressure, steps=10):
    """A Static pipe chain clamped at one end under a tip force, its Pipe_1
    elements all under an internal pressure raised with the load factor."""
    s = configs.pipe_chain(n_el, 0.4, 0.03, [4e4, -1e4, 2e4], steps=steps)
    ps = s.add_pipe_section(2e9, 4e8, 3e8, 8e8, 300.0, 0.4, 0.34)
    for e in range(len(s.beams)):
        s.pipe_of[e] = ps
    s.loads.append(PipeLoad(list(range(n_el)), Table(np.array([0.0, 1.0]),
                                                    np.array([[0.0] * 4, [pressure, 0.0, 0.0, 0.0]]))))
    return s


def test_first_assembly_with_pressure_matches_oracle(gpu_ctx):
    """K_AA and P_A of the first Newton iteration of Static steps:
    pressurized pipes (the pressure is already nonzero at the first step's
    time), one under a negative pressure, and a Beam_1 chain in the same
    batch."""
    structs = [_static_pipes(12, 8e6), _static_pipes(7, -5e6), configs.pipe_chain(23, 0.35, 0.025, [1e5, 2e4, -3e4])]
    b = gpu.BatchSolver(gpu_ctx, structs)
    for s, st in enumerate(structs):
        ab, P, kb = b.assemble(s)
        ab_o, P_o, kl_o = oracle.first_tangent(st)
        assert kb == kl_o
        assert rel(ab, ab_o) < 1e-13, s
        assert rel(P, P_o) < 1e-13, s
    b.close()


def test_tutorial04_matches_reference(gpu_ctx, golden):
    """The reference's tutorial04 deck (from the fixture's deck text): a
    pinned pipe perturbed laterally, then internal pressure raised to
    1.2 MPa over 200 Static steps of a second solution step."""
    g = golden("ref_tutorial04.npz")
    s = Structure.from_inp(str(g["deck"]))
    finals, stats = _solve(gpu_ctx, [s])
    ref = g["nodes"][-1]
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9
    _, so, _ = oracle.solve(s)
    assert list(stats[0]) == list(so)


@pytest.mark.parametrize("name,kw", [("ref_pipe_riser.npz", {}),
                                     ("ref_pipe_riser_rayleigh.npz",
                                      dict(rayleigh_alpha=0.3, rayleigh_beta=0.004, update_rayleigh=1))])
def test_pipe_riser_dynamics_matches_reference(gpu_ctx, golden, name, kw):
    s = configs.pipe_riser(**kw)
    g = golden(name)
    finals, stats = _solve(gpu_ctx, [s])
    ref = g["nodes"][-1]
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9
    _, so, _ = oracle.solve(s)
    assert list(stats[0]) == list(so)


def test_pressurized_pipes_beside_beams_match_the_oracle(gpu_ctx):
    """A batch of pipe risers of different lengths and pressures (some with
    Rayleigh damping), a Static pipe under pressure and a tip force, and
    Beam_1 risers: each structure as the oracle solves it."""
    rng = np.random.default_rng(11)
    structs = []
    for k in range(6):
        structs.append(configs.pipe_riser(int(rng.integers(8, 40)), pressure=float(rng.uniform(-1e7, 3e7)),
                                          amp=float(rng.uniform(0.2, 1.0)), steps=40,
                                          rayleigh_alpha=0.2 if k % 3 == 2 else 0.0,
                                          rayleigh_beta=0.003 if k % 3 == 2 else 0.0))
    st = _static_pipes(16, 8e6, steps=8)
    st.loads[1].pipes = list(range(0, 16, 2))  # every other element pressurized
    structs.append(st)
    structs += [configs.riser_chain(int(n), 0.4, 0.03, 1.0, 6.0, steps=40) for n in (15, 31)]
    finals, stats = _solve(gpu_ctx, structs)
    for s, f, sg in zip(structs, finals, stats):
        fo, so, _ = oracle.solve(s)
        assert list(sg) == list(so)
        scale = np.abs(fo[:, :3]).max()
        assert np.abs(f[:, :3] - fo[:, :3]).max() <= 1e-10 * scale


def test_pipe_loads_are_checked(gpu_ctx):
    """A PipeLoad on an element that is not a Pipe_1, and two PipeLoads on
    one pipe, are refused with an error."""
    s = configs.pipe_riser(4, steps=4)
    s.beams[1] = (2, 3, 4, s.add_material(2.1e11, 0.3, 7850.0), s.add_tube(0.3, 0.26), 0)
    del s.pipe_of[1]
    with pytest.raises(RuntimeError, match="not a Pipe_1"):
        gpu.BatchSolver(gpu_ctx, [s])
    s = configs.pipe_riser(4, steps=4)
    s.loads.append(PipeLoad([2], s.loads[0].table))
    with pytest.raises(RuntimeError, match="more than one PipeLoad"):
        gpu.BatchSolver(gpu_ctx, [s])

"""The CPU oracle against the golden fixtures made by the reference itself
(tests/golden/make_golden.py) and against known answers."""
import numpy as np
import pytest

from giraffe_gb300 import configs
from oracle import oracle
from tests.monitor_check import monitor_close


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_beam_elements_match_reference(golden):
    g = golden("ref_beam_elements.npz")
    for i in range(len(g["K"])):
        nh = int(g["n_hist"][i])
        K, f = oracle.beam_element(g["xyz"][i], g["mat"][i], g["sec6"][i], g["cs"][i], g["hist"][i][:nh],
                                   g["disp"][i])
        assert rel(K, g["K"][i]) < 1e-12, i
        assert rel(f, g["P"][i]) < 1e-12, i


def test_beam_inertia_matches_reference(golden):
    g = golden("ref_beam_inertia.npz")
    for i in range(len(g["M"])):
        nh = int(g["n_hist"][i])
        M, F, ke = oracle.beam_inertia(g["xyz"][i], g["mat"][i], g["sec6"][i], g["cs"][i], g["hist"][i][:nh],
                                       g["disp"][i], g["vel"][i], g["acc"][i], float(g["dt"][i]),
                                       float(g["beta"][i]), float(g["gamma"][i]))
        assert rel(M, g["M"][i]) < 1e-12, i
        assert rel(F, g["F"][i]) < 1e-12, i
        assert abs(ke - g["ke"][i]) <= 1e-12 * abs(g["ke"][i]), i


def test_shell_elements_match_reference(golden):
    g = golden("ref_shell_elements.npz")
    for i in range(len(g["K"])):
        nh = int(g["n_hist"][i])
        p = float(g["pressure"][i])
        K, f = oracle.shell_element(g["xyz"][i], g["mat"][i], float(g["thick"][i]), g["hist"][i][:nh],
                                    g["disp"][i], None if np.isnan(p) else p, int(g["area_update"][i]))
        assert rel(K, g["K"][i]) < 1e-12, i
        assert rel(f, g["P"][i]) < 1e-12, i


def _check_run(g, s, tol=1e-11):
    final, stats, rec = oracle.solve(s, record_cap=4096)
    assert stats[3] == 0 and int(g["rc"]) == 0
    # every configuration the reference wrote, at the same time
    for k, t in enumerate(g["times"]):
        j = int(np.argmin(np.abs(rec["time"] - t)))
        assert abs(rec["time"][j] - t) < 1e-12
        ref_nodes = g["nodes"][k]
        scale = np.abs(ref_nodes[:, :3]).max()
        assert np.abs(rec["nodes"][j][:, :3] - ref_nodes[:, :3]).max() <= tol * scale, t
        assert np.abs(rec["nodes"][j][:, 6:] - ref_nodes[:, 6:]).max() <= tol * 10, t
        if g["gp_Q"][k].size:
            assert np.abs(rec["gp_Q"][j] - g["gp_Q"][k]).max() <= tol * 10, t
    # Newton solves per converged step
    steps = g["steps"]
    conv = steps[steps[:, 2] == 0]
    assert len(conv) == stats[0]
    its = rec["iterations"]
    assert np.array_equal(its[its > 0], conv[:, 1].astype(int) + 1)  # (records at step starts carry 0)
    return final, stats, rec


def test_tutorial01_matches_reference(golden):
    _check_run(golden("ref_tutorial01.npz"), configs.tutorial01())


def test_rollup_matches_reference(golden):
    _check_run(golden("ref_rollup.npz"), configs.cantilever_rollup())


def test_chain_matches_reference(golden):
    from tests.golden.make_golden import small_chain
    _check_run(golden("ref_chain.npz"), small_chain())


def test_plate_matches_reference(golden):
    _check_run(golden("ref_plate.npz"), configs.square_plate(4, steps=20))


def test_plate_fixed_area_matches_reference(golden):
    _check_run(golden("ref_plate_fixed_area.npz"), configs.square_plate(3, steps=10, area_update=0))


def test_tutorial10_dynamics_matches_reference(golden):
    _check_run(golden("ref_tutorial10.npz"), configs.tutorial10(), tol=1e-10)


@pytest.mark.parametrize("name,update", [("ref_tutorial10_rayleigh.npz", 0), ("ref_tutorial10_rayleigh_update.npz", 1)])
def test_tutorial10_rayleigh_matches_reference(golden, name, update):
    """Rayleigh damping C = alpha M_modal + beta K (MountDamping), formed at
    the first iteration (Update 0) or at every iteration (Update 1); the
    damped motion differs from the undamped one by far more than the
    tolerance."""
    final, _, _ = _check_run(golden(name), configs.tutorial10(0.2, 0.002, update), tol=1e-10)
    undamped = golden("ref_tutorial10.npz")["nodes"][-1]
    assert np.abs(final[:, :3] - undamped[:, :3]).max() > 1e-4 * np.abs(undamped[:, :3]).max()


def test_riser_rayleigh_matches_reference(golden):
    _check_run(golden("ref_riser_rayleigh.npz"),
               configs.riser_chain(12, 0.4, 0.03, 1.0, 4.0, steps=120, element_length=2.0, rayleigh_alpha=0.3,
                                   rayleigh_beta=0.004, update_rayleigh=1), tol=1e-10)


def test_rollup_known_answer():
    """An end moment 2 pi E I / L rolls the cantilever into a circle: at load
    factor t the tip is at (L sin(th)/th, L (1 - cos(th))/th) with th = 2 pi t."""
    L = 10.0
    final, stats, rec = oracle.solve(configs.cantilever_rollup(), record_cap=64)
    assert stats[0] == 20 and stats[2] == 0
    for t, nodes in zip(rec["time"][1:], rec["nodes"][1:]):
        th = 2 * np.pi * t
        ex = np.array([L * np.sin(th) / th, L * (1 - np.cos(th)) / th, 0.0])
        assert np.abs(nodes[-1][:3] - ex).max() < 1e-6 * L
    # full circle: tip back at the clamp, tip rotation tensor back to I
    assert np.abs(final[-1][:3]).max() < 1e-6 * L
    assert np.abs(final[-1][6:].reshape(3, 3) - np.eye(3)).max() < 1e-6


def test_tutorial01_known_small_load_limit():
    """Small tip force: the linear Timoshenko cantilever deflection
    F L^3 / (3 E I) + F L / (G A) is recovered."""
    s = configs.tutorial01()
    s.loads[0].table.values[1, 0] = 1e-3
    final, stats, _ = oracle.solve(s)
    E, nu = 1e7, 0.3
    A, I = 0.01, 0.1 ** 4 / 12
    G = E / (2 * (1 + nu))
    F, L = 1e-3, 1.0
    ex = F * L ** 3 / (3 * E * I) + F * L / (G * A)
    assert abs(final[-1][0] - ex) < 1e-9 * max(1, ex / 1e-6) + 1e-3 * ex


@pytest.mark.parametrize("name,angular", [("ref_rotating_base_angles.npz", "EulerAngles"),
                                          ("ref_rotating_base_vector.npz", "EulerVector")])
def test_prescribed_base_rotation_matches_reference(golden, name, angular):
    """NodalDisplacement rotations read as Euler angles and as an Euler
    rotation vector (AngularParameters); the two readings give different
    motions, each as the reference computes it."""
    final, _, _ = _check_run(golden(name), configs.rotating_base(angular), tol=1e-10)
    other = golden("ref_rotating_base_vector.npz" if angular == "EulerAngles" else "ref_rotating_base_angles.npz")
    assert np.abs(final[:, :3] - other["nodes"][-1][:, :3]).max() > 0.1


def test_pretensioned_chain_matches_reference(golden):
    """Beam_1 PreTension: reference length shortened by 1 + T0 / EA and the
    Gauss points starting stretched (Beam_1::PreCalc)."""
    _check_run(golden("ref_pretension.npz"), configs.pretensioned_chain(), tol=1e-10)


def test_shell_inertia_matches_reference(golden):
    """Shell_1 MountMass: the director-fibre inertia.  The rotational blocks
    are four to six orders below the translational ones, so they are checked
    on their own scale."""
    g = golden("ref_shell_inertia.npz")
    for i in range(len(g["M"])):
        nh = int(g["n_hist"][i])
        M, F, ke = oracle.shell_inertia(g["xyz"][i], g["mat"][i], float(g["thick"][i]), g["hist"][i][:nh],
                                        g["disp"][i], g["vel"][i], g["acc"][i], float(g["dt"][i]),
                                        float(g["beta"][i]), float(g["gamma"][i]))
        R = g["M"][i]
        assert rel(M, R) < 1e-12, i
        assert rel(M[18:, 18:], R[18:, 18:]) < 1e-12, i
        assert np.abs(R[:18, 18:]).max() == 0.0 and np.abs(M[:18, 18:]).max() == 0.0
        assert rel(F, g["F"][i]) < 1e-12, i
        assert rel(F[18:], g["F"][i][18:]) < 1e-12, i
        assert abs(ke - g["ke"][i]) <= 1e-12 * abs(g["ke"][i]), i


@pytest.mark.parametrize("name,kw", [
    ("ref_plate_dynamic.npz", {}),
    ("ref_plate_dynamic_rayleigh.npz", dict(area_update=0, rayleigh_alpha=8.0, rayleigh_beta=2e-5)),
    ("ref_plate_dynamic_rayleigh_update.npz", dict(rayleigh_alpha=8.0, rayleigh_beta=2e-5, update_rayleigh=1)),
])
def test_plate_dynamics_matches_reference(golden, name, kw):
    """Shell_1 in a Dynamic step (MountMass, MountDamping with the modal mass
    of EvaluateMassModal, MountDyn): a clamped plate set vibrating by a
    quickly applied follower pressure, with and without Rayleigh damping."""
    final, _, _ = _check_run(golden(name), configs.plate_dynamics(3, steps=20, **kw), tol=1e-10)
    if kw:
        undamped = golden("ref_plate_dynamic.npz")["nodes"][-1]
        assert np.abs(final[:, 2] - undamped[:, 2]).max() > 1e-2 * np.abs(undamped[:, 2]).max()


@pytest.mark.parametrize("name,make", [("ref_plate_release.npz", lambda: configs.plate_release(3)),
                                       ("ref_chain_sequence.npz", configs.chain_sequence)])
def test_solution_step_sequences_match_reference(golden, name, make):
    """Several solution steps run in sequence from the state the previous
    one ends in (the reference's main loop): Static then Dynamic for a
    released plate; Static, damped Dynamic, Dynamic from rest (ZeroIC) and
    Static for a pipe chain."""
    final, stats, _ = _check_run(golden(name), make(), tol=1e-10)
    assert stats[0] == len(golden(name)["steps"])


def test_pipe_elements_match_reference(golden):
    """Pipe_1: Beam_1 kinematics with a PipeSection's stiffness, and the
    internal-pressure load of MountPipeSpecialLoads with its load
    stiffness (half of the elements)."""
    g = golden("ref_pipe_elements.npz")
    pressed = 0
    for i in range(len(g["K"])):
        nh = int(g["n_hist"][i])
        p = float(g["pressure"][i])
        K, f = oracle.pipe_element(g["xyz"][i], g["ps"][i], g["cs"][i], g["hist"][i][:nh], g["disp"][i], p)
        assert rel(K, g["K"][i]) < 1e-12, i
        assert rel(f, g["P"][i]) < 1e-12, i
        if p != 0.0:
            pressed += 1
            K0, _ = oracle.pipe_element(g["xyz"][i], g["ps"][i], g["cs"][i], g["hist"][i][:nh], g["disp"][i])
            # the load stiffness itself, on its own scale
            assert rel(K - K0, g["K"][i] - K0) < 1e-9, i
    assert pressed == len(g["K"]) // 2


def test_tutorial04_pressurized_pipe_matches_reference(golden):
    """The reference's tutorial04 deck (read back from the fixture's deck
    text): 50 Pipe_1 elements, a lateral perturbation, then internal
    pressure raised to 1.2 MPa in 200 Static steps."""
    from giraffe_gb300.model import Structure
    g = golden("ref_tutorial04.npz")
    s = Structure.from_inp(str(g["deck"]))
    assert len(s.pipe_of) == 50 and len(s.next_steps) == 1
    _check_run(g, s, tol=1e-10)


@pytest.mark.parametrize("name,kw", [("ref_pipe_riser.npz", {}),
                                     ("ref_pipe_riser_rayleigh.npz",
                                      dict(rayleigh_alpha=0.3, rayleigh_beta=0.004, update_rayleigh=1))])
def test_pipe_riser_dynamics_matches_reference(golden, name, kw):
    """Pipe_1 in a Dynamic step (the pipe section's mass and rotary inertia)
    under a rising internal pressure, with and without Rayleigh damping."""
    final, _, _ = _check_run(golden(name), configs.pipe_riser(**kw), tol=1e-10)
    # the pressure changes the motion by far more than the tolerance
    s = configs.pipe_riser(pressure=0.0, **kw)
    f0, _, _ = oracle.solve(s)
    assert np.abs(final[:, :3] - f0[:, :3]).max() > 1e-6 * np.abs(final[:, :3]).max()


@pytest.mark.parametrize("name", ["ref_modal_cantilever.npz", "ref_modal_plate.npz", "ref_modal_riser.npz"])
def test_modal_matrices_match_reference(golden, name):
    """The two matrices of a Modal step (K_AA, and M_AA of MountMassModal)
    equal the reference's own to rounding, and the oracle's eigenvalues (LAPACK's
    symmetric-definite solver, standing in for the reference's ARPACK
    shift-invert) equal the golden ones to 1e-7 relative: the smallest
    eigenvalues of these stiff problems carry an error of about
    eps |lambda_max| / |lambda| from any dense solver."""
    from giraffe_gb300.model import Structure
    g = golden(name)
    s = Structure.from_inp(str(g["deck"]))
    assert s.modal is not None and s.modal.number_modes == len(g["eig"])
    K, M = oracle.modal_matrices(s)
    assert rel(K, g["K"]) < 1e-14
    assert rel(M, g["M"]) < 1e-14
    w, V = oracle.modal(s, len(g["eig"]))
    assert np.abs(w - g["eig"]).max() <= 1e-7 * np.abs(g["eig"]).max()
    assert np.allclose(V.T @ g["M"] @ V, np.eye(len(w)), atol=1e-9)


@pytest.mark.parametrize("name", ["ref_monitor_chain.npz", "ref_monitor_plate.npz", "ref_monitor_tutorial10.npz",
                                  "ref_monitor_sequence.npz", "ref_tutorial04.npz"])
def test_monitor_lines_match_reference(golden, name):
    """Node::WriteMonitor's lines of the monitored nodes (the reference's
    Monitor Sample / MonitorNodes): at the first step's start, after every
    sample-th converged step of each solution step and at each step's end;
    reactions at constrained DOFs, the internal force at free ones, moments
    from the pseudo-moments."""
    from giraffe_gb300.model import Structure
    g = golden(name)
    s = Structure.from_inp(str(g["deck"]))
    assert s.monitor is not None and list(s.monitor.nodes) == list(g["monitor_nodes"])
    _, _, rec = oracle.solve(s, record_cap=4096)
    monitor_close(rec["monitor"], g["monitor"])

"""Seeded synthetic structures of the benchmark shapes.

* :func:`cantilever_rollup` — 20 Beam_1 elements (41 nodes, 246 DOF), L = 10 m,
  E = 210 GPa, nu = 0.3, 0.1 x 0.1 m rectangle, clamped at x = 0, tip moment
  about z ramped to 2*pi*E*I/L over 20 load steps (the beam rolls into a full
  circle), residual tolerance 1e-8.
* :func:`pipe_chain` / :func:`batched_static` — pipe-section Beam_1 chains
  (Tube De ~ U(0.3, 0.5) m, wall ~ U(0.02, 0.04) m, E = 210 GPa), clamped at
  one end, tip force ~ N(0, 1e5) N per component, 10 load steps; element
  counts log-uniform in [50, 2000] from the seed.  The chain length is not
  fixed by the benchmark description; every chain here is 10 m long along +z
  (element length 10 m / n_e), so the batch is one physical problem meshed
  at different resolutions.  With 1 m elements the longer chains (hundreds of
  metres under 1e5 N) do not converge in 10 load steps in the reference's own
  Newton/bisection control either.
* :func:`tutorial01` — the reference's tutorial01 deck (5 Beam_1 cantilever,
  tip force), built programmatically.
* :func:`riser_chain` / :func:`batched_dynamic` — implicit dynamics: pipe
  chains of 100-1000 elements (uniform from the seed), rho = 7850 kg/m^3,
  Newmark beta = 0.25, gamma = 0.5, dt = 0.01 s, 1000 steps, the top node
  driven laterally by u(t) = A sin(2 pi t / T) with A ~ U(0.5, 2) m and
  T ~ U(5, 15) s (tabulated at every time step, so exact at step times), its
  rotations held; bottom free.  E = 210 GPa and 0.5 m elements (chains of
  50-500 m) are this generator's choices; the description fixes neither.
* :func:`pipe_riser` — Pipe_1 elements (PipeSection of a steel tube) pinned
  at the bottom, the top driven laterally as in :func:`riser_chain`, under
  an internal pressure (PipeLoad) raised over the first quarter of the run;
  Newmark dynamics.

Every generator is deterministic in its seed (numpy default_rng).
"""
from __future__ import annotations

import math

import numpy as np

from .model import (GF_DYNAMIC, GF_STATIC, NodalDisplacement, NodalLoad, PipeLoad, PressureLoad, Solution,
                    Structure, Table)

E_STEEL = 210e9
NU_STEEL = 0.3
RHO_STEEL = 7850.0


def straight_chain(n_el: int, length: float, direction=(1.0, 0.0, 0.0)) -> np.ndarray:
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    t = np.linspace(0.0, length, 2 * n_el + 1)
    return t[:, None] * d[None, :]


def _chain_beams(s: Structure, n_el: int, mat: int, sec: int, cs: int) -> None:
    """Beam_1 elements (2e, 2e+1, 2e+2) along a straight chain of 2 n_el + 1 nodes."""
    e = np.arange(n_el)
    s.beams.extend(np.stack([2 * e, 2 * e + 1, 2 * e + 2, np.full(n_el, mat), np.full(n_el, sec),
                             np.full(n_el, cs)], axis=1))


def cantilever_rollup(n_el: int = 20, steps: int = 20, tol: float = 1e-8) -> Structure:
    L = 10.0
    s = Structure(nodes=straight_chain(n_el, L))
    mat = s.add_material(E_STEEL, NU_STEEL, RHO_STEEL)
    sec = s.add_rectangle(0.1, 0.1)
    cs_beam = s.add_cs((0.0, 1.0, 0.0), (1.0, 0.0, 0.0))   # E3 along the axis
    cs_glob = s.add_cs((1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
    _chain_beams(s, n_el, mat, sec, cs_beam)
    s.clamp(0)
    I = s.sections[sec][2]  # bending about global z is about the section's E2 axis
    Mz = 2.0 * math.pi * E_STEEL * I / L
    s.loads.append(NodalLoad([2 * n_el], cs_glob,
                             Table(np.array([0.0, 1.0]),
                                   np.array([[0, 0, 0, 0, 0, 0], [0, 0, 0, 0, 0, Mz]], dtype=float))))
    dt = 1.0 / steps
    s.solution = Solution(GF_STATIC, 0.0, 1.0, dt, dt, dt / 1024, 20, 3, 4, 1.0)
    # No force is applied, so the force criterion falls back to
    # ForceMinimumReference * tol; 1e4 N puts it (1e-4 N) above the FP64
    # round-off floor of the axial force residual (~1e-6 N for EA = 2.1e9 N).
    s.criteria.update(force_tol=tol, moment_tol=tol, force_min=1e4)
    return s


def tutorial01() -> Structure:
    s = Structure(nodes=np.array([[0.0, 0.0, 0.1 * i] for i in range(11)]))
    s.nodes[:, 2] = [0.0, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0]
    mat = s.add_material(1e7, 0.3, 2000)
    sec = s.add_rectangle(0.1, 0.1)
    cs = s.add_cs((1, 0, 0), (0, 0, 1))
    for e in range(5):
        s.beams.append((2 * e, 2 * e + 1, 2 * e + 2, mat, sec, cs))
    s.clamp(0)
    s.loads.append(NodalLoad([10], cs, Table(np.array([0.0, 1.0]),
                                              np.array([[0, 0, 0, 0, 0, 0], [1000, 0, 0, 0, 0, 0]],
                                                       dtype=float))))
    s.solution = Solution(GF_STATIC, 0.0, 1.0, 0.1, 0.1, 0.01, 20, 3, 4, 1.0, sample=2)
    return s


def tutorial10(rayleigh_alpha: float = 0.0, rayleigh_beta: float = 0.0, update_rayleigh: int = 0) -> Structure:
    """The reference's tutorial10 deck: 5 Beam_1 elements, Dynamic step with a
    prescribed base motion (translations and an Euler-angle rotation about z),
    Newmark beta = 0.3, gamma = 0.5; optionally with Rayleigh damping
    C = alpha M + beta K (formed once, or at every iteration with
    update_rayleigh = 1)."""
    s = Structure(nodes=np.array([[0.0, 0.0, 0.1 * i] for i in range(11)]))
    s.nodes[:, 2] = [0.0, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0]
    mat = s.add_material(1e7, 0.3, 2000)
    sec = s.add_rectangle(0.1, 0.1)
    cs = s.add_cs((1, 0, 0), (0, 0, 1))
    for e in range(5):
        s.beams.append((2 * e, 2 * e + 1, 2 * e + 2, mat, sec, cs))
    s.clamp(0)
    s.displacements.append(NodalDisplacement([0], cs, Table(
        np.array([0.0, 2.5, 5.0, 7.5, 10.0]),
        np.array([[0, 0, 0, 0, 0, 0], [0, 0.5, 0.25, 0, 0, 0], [0, 0, 0, 0, 0, 3.14],
                  [0, -0.5, -0.25, 0, 0, 0], [0, 0, 0, 0, 0, 0]], dtype=float))))
    s.solution = Solution(GF_DYNAMIC, 0.0, 10.0, 0.005, 0.005, 0.001, 20, 3, 4, 1.0, sample=10,
                          beta=0.3, gamma=0.5, rayleigh_alpha=rayleigh_alpha, rayleigh_beta=rayleigh_beta,
                          update_rayleigh=update_rayleigh)
    return s


def pretensioned_chain(n_el: int = 20, T0: float = 2e5, steps: int = 10) -> Structure:
    """A pipe chain like the benchmark's (10 m, tube 0.4 x 0.03) whose
    elements carry a PreTension T0 (reference length shortened by
    1 + T0 / EA, Gauss points starting stretched), under a lateral tip
    force."""
    s = pipe_chain(n_el, 0.4, 0.03, [4e4, -2e4, 0.0], steps=steps, element_length=10.0 / n_el)
    s.pretension = {e: T0 for e in range(n_el)}
    return s


def rotating_base(angular: str = "EulerAngles", steps: int = 10) -> Structure:
    """tutorial01's cantilever (10 Beam_1 along z) whose clamped base is turned
    by a prescribed rotation with components (0.4, -0.3, 1.2) at t = 1, read
    as Euler angles or as an Euler rotation vector (NodalDisplacement
    AngularParameters), with a tip force, in `steps` load steps."""
    s = Structure(nodes=straight_chain(10, 1.0, (0.0, 0.0, 1.0)))
    mat = s.add_material(1e7, 0.3, 2000)
    sec = s.add_rectangle(0.1, 0.1)
    cs = s.add_cs((1, 0, 0), (0, 0, 1))
    _chain_beams(s, 10, mat, sec, cs)
    s.clamp(0)
    s.displacements.append(NodalDisplacement([0], cs, Table(
        np.array([0.0, 1.0]), np.array([[0.0] * 6, [0.0, 0.0, 0.0, 0.4, -0.3, 1.2]])), angular=angular))
    s.loads.append(NodalLoad([20], cs, Table(np.array([0.0, 1.0]), np.array([[0.0] * 6, [50.0, 0, 0, 0, 0, 0]]))))
    dt = 1.0 / steps
    s.solution = Solution(GF_STATIC, 0.0, 1.0, dt, dt, dt / 64, 20, 3, 4, 1.0)
    s.criteria.update(force_tol=1e-8, moment_tol=1e-8, force_min=1.0, moment_min=1.0)
    return s


def pipe_chain(n_el: int, De: float, wall: float, tip_force, steps: int = 10,
               element_length: float = 1.0, tol: float = 1e-8) -> Structure:
    s = Structure(nodes=straight_chain(n_el, n_el * element_length, (0.0, 0.0, 1.0)))
    mat = s.add_material(E_STEEL, NU_STEEL, RHO_STEEL)
    sec = s.add_tube(De, De - 2.0 * wall)
    cs = s.add_cs((1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
    _chain_beams(s, n_el, mat, sec, cs)
    s.clamp(0)
    f = np.asarray(tip_force, dtype=np.float64)
    s.loads.append(NodalLoad([2 * n_el], cs, Table(np.array([0.0, 1.0]),
                                                   np.array([[0.0] * 6, [*f, 0.0, 0.0, 0.0]]))))
    dt = 1.0 / steps
    s.solution = Solution(GF_STATIC, 0.0, 1.0, dt, dt, dt / 4096, 30, 3, 4, 1.0)
    # Only forces are applied, so the moment criterion falls back to
    # MomentMinimumReference * tol; 1e4 N m keeps it above the FP64 round-off
    # floor of the bending-moment residual.
    s.criteria.update(force_tol=tol, moment_tol=tol, disp_tol=tol, rot_tol=tol, moment_min=1e4)
    return s


def batched_static(n_chains: int = 512, seed: int = 0, n_min: int = 50, n_max: int = 2000,
                   steps: int = 10, tol: float = 1e-8, chain_length: float = 10.0) -> list:
    rng = np.random.default_rng(seed)
    n_el = np.rint(np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_chains))).astype(int)
    De = rng.uniform(0.3, 0.5, n_chains)
    wall = rng.uniform(0.02, 0.04, n_chains)
    F = rng.normal(0.0, 1e5, (n_chains, 3))
    return [pipe_chain(int(n), float(d), float(w), F[i], steps=steps, tol=tol,
                       element_length=chain_length / int(n))
            for i, (n, d, w) in enumerate(zip(n_el, De, wall))]


def served_chains(n_requests: int, seed: int = 0, dof_min: int = 1000, dof_max: int = 50000,
                  steps: int = 10, tol: float = 1e-8, chain_length: float = 10.0) -> list:
    """Static pipe-chain requests of the mixed served stream: free-DOF counts
    log-uniform in [dof_min, dof_max] (n_e = (DOF/6 - 1)/2 elements), section
    and tip force drawn as in batched_static."""
    rng = np.random.default_rng(seed)
    dof = np.exp(rng.uniform(math.log(dof_min), math.log(dof_max), n_requests))
    n_el = np.maximum(1, np.rint((dof / 6.0 - 1.0) / 2.0)).astype(int)
    De = rng.uniform(0.3, 0.5, n_requests)
    wall = rng.uniform(0.02, 0.04, n_requests)
    F = rng.normal(0.0, 1e5, (n_requests, 3))
    return [pipe_chain(int(n), float(d), float(w), F[i], steps=steps, tol=tol,
                       element_length=chain_length / int(n))
            for i, (n, d, w) in enumerate(zip(n_el, De, wall))]


def riser_chain(n_el: int, De: float, wall: float, amp: float, period: float, steps: int = 1000,
                dt: float = 0.01, element_length: float = 0.5, tol: float = 1e-8, rayleigh_alpha: float = 0.0,
                rayleigh_beta: float = 0.0, update_rayleigh: int = 0) -> Structure:
    L = n_el * element_length
    s = Structure(nodes=straight_chain(n_el, L, (0.0, 0.0, 1.0)))
    mat = s.add_material(E_STEEL, NU_STEEL, RHO_STEEL)
    sec = s.add_tube(De, De - 2.0 * wall)
    cs = s.add_cs((1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
    _chain_beams(s, n_el, mat, sec, cs)
    top = 2 * n_el
    s.clamp(top)
    t = np.arange(steps + 1) * dt
    vals = np.zeros((steps + 1, 6))
    vals[:, 0] = amp * np.sin(2.0 * math.pi * t / period)
    s.displacements.append(NodalDisplacement([top], cs, Table(t, vals)))
    s.solution = Solution(GF_DYNAMIC, 0.0, steps * dt, dt, dt, dt / 64, 20, 3, 4, 1.0, beta=0.25, gamma=0.5,
                          rayleigh_alpha=rayleigh_alpha, rayleigh_beta=rayleigh_beta, update_rayleigh=update_rayleigh)
    s.criteria.update(force_tol=tol, moment_tol=tol, disp_tol=tol, rot_tol=tol, force_min=1.0, moment_min=1.0)
    return s


def pipe_riser(n_el: int = 16, De: float = 0.3, wall: float = 0.02, amp: float = 0.5, period: float = 2.0,
               pressure: float = 2e7, steps: int = 100, dt: float = 0.01, element_length: float = 1.0,
               tol: float = 1e-8, rayleigh_alpha: float = 0.0, rayleigh_beta: float = 0.0,
               update_rayleigh: int = 0) -> Structure:
    L = n_el * element_length
    s = Structure(nodes=straight_chain(n_el, L, (0.0, 0.0, 1.0)))
    Di = De - 2.0 * wall
    A = math.pi / 4.0 * (De * De - Di * Di)
    I = math.pi / 64.0 * (De ** 4 - Di ** 4)
    G = E_STEEL / (2.0 * (1.0 + NU_STEEL))
    ps = s.add_pipe_section(E_STEEL * A, E_STEEL * I, G * 2.0 * I, G * A, RHO_STEEL * A, De, Di)
    cs = s.add_cs((1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
    for e in range(n_el):
        s.add_pipe(2 * e, 2 * e + 1, 2 * e + 2, ps, cs)
    s.clamp(0, (1, 1, 1, 0, 0, 0))
    top = 2 * n_el
    s.clamp(top)
    t = np.arange(steps + 1) * dt
    vals = np.zeros((steps + 1, 6))
    vals[:, 0] = amp * np.sin(2.0 * math.pi * t / period)
    s.displacements.append(NodalDisplacement([top], cs, Table(t, vals)))
    ramp = max(steps // 4, 1) * dt
    s.loads.append(PipeLoad(list(range(n_el)), Table(np.array([0.0, ramp, steps * dt]),
                                                     np.array([[0.0] * 4, [pressure, 0, 0, 0],
                                                               [pressure, 0, 0, 0]]))))
    s.solution = Solution(GF_DYNAMIC, 0.0, steps * dt, dt, dt, dt / 64, 20, 3, 4, 1.0, beta=0.25, gamma=0.5,
                          rayleigh_alpha=rayleigh_alpha, rayleigh_beta=rayleigh_beta, update_rayleigh=update_rayleigh)
    s.criteria.update(force_tol=tol, moment_tol=tol, disp_tol=tol, rot_tol=tol, force_min=1.0, moment_min=1.0)
    return s


def batched_dynamic(n_chains: int = 256, seed: int = 0, n_min: int = 100, n_max: int = 1000,
                    steps: int = 1000, tol: float = 1e-8) -> list:
    rng = np.random.default_rng(seed)
    n_el = rng.integers(n_min, n_max + 1, n_chains)
    De = rng.uniform(0.3, 0.5, n_chains)
    wall = rng.uniform(0.02, 0.04, n_chains)
    amp = rng.uniform(0.5, 2.0, n_chains)
    per = rng.uniform(5.0, 15.0, n_chains)
    return [riser_chain(int(n), float(d), float(w), float(a), float(p), steps=steps, tol=tol)
            for n, d, w, a, p in zip(n_el, De, wall, amp, per)]


def square_plate(n: int = 64, side: float = 1.0, thickness: float = 0.01, E: float = 70e9, nu: float = 0.33,
                 pressure: float = 1e5, steps: int = 20, area_update: int = 1, tol: float = 1e-8) -> Structure:
    """Square plate in the x-y plane meshed into n x n squares, each split
    into two six-node Shell_1 triangles ((2n+1)^2 grid nodes: corners at even
    grid indices, midside nodes elsewhere), all four edges clamped, uniform
    follower pressure ramped linearly to `pressure` over `steps` load steps."""
    m = 2 * n + 1
    h = side / (2 * n)
    gx, gy = np.meshgrid(np.arange(m) * h, np.arange(m) * h, indexing="xy")
    s = Structure(nodes=np.stack([gx.ravel(), gy.ravel(), np.zeros(m * m)], axis=1))
    mat = s.add_material(E, nu, 2700.0)
    sec = s.add_shell_section(thickness)
    cs = s.add_cs((1.0, 0.0, 0.0), (0.0, 0.0, 1.0))

    def node(i, j):
        return j * m + i

    for j in range(n):
        for i in range(n):
            a, b = node(2 * i, 2 * j), node(2 * i + 2, 2 * j)
            c, d = node(2 * i + 2, 2 * j + 2), node(2 * i, 2 * j + 2)
            ab, bc, cd, da = node(2 * i + 1, 2 * j), node(2 * i + 2, 2 * j + 1), node(2 * i + 1, 2 * j + 2), \
                node(2 * i, 2 * j + 1)
            ac = node(2 * i + 1, 2 * j + 1)
            s.shells.append((a, b, c, ab, bc, ac, mat, sec, cs))
            s.shells.append((a, c, d, ac, cd, da, mat, sec, cs))
    for j in range(m):
        for i in range(m):
            if i in (0, m - 1) or j in (0, m - 1):
                s.clamp(node(i, j))
    s.loads.append(PressureLoad(list(range(len(s.shells))), Table(np.array([0.0, 1.0]),
                                                                  np.array([[0.0], [pressure]])),
                                area_update=area_update))
    dt = 1.0 / steps
    s.solution = Solution(GF_STATIC, 0.0, 1.0, dt, dt, dt / 4096, 30, 3, 4, 1.0)
    # No moment is applied, so the moment criterion falls back to
    # MomentMinimumReference * tol; 1 N m keeps it above the FP64 round-off
    # floor of the rotational residual.
    s.criteria.update(force_tol=tol, moment_tol=tol, disp_tol=tol, rot_tol=tol, moment_min=1.0)
    return s


def plate_dynamics(n: int = 4, pressure: float = 1e5, rise: float = 0.002, dt: float = 0.001, steps: int = 30,
                   area_update: int = 1, rayleigh_alpha: float = 0.0, rayleigh_beta: float = 0.0,
                   update_rayleigh: int = 0, beta: float = 0.25, gamma: float = 0.5, tol: float = 1e-8,
                   **plate) -> Structure:
    """The clamped square plate of square_plate in a Dynamic step (Newmark
    beta, gamma, time step dt, `steps` steps): the follower pressure rises
    linearly to `pressure` over `rise` seconds and then stays, so the plate
    vibrates about its static deflection (the first mode of the 1 m, 10 mm
    aluminium plate has a period near 11 ms).  Optional Rayleigh damping
    C = alpha M + beta K, formed once or (update_rayleigh 1) every
    iteration."""
    s = square_plate(n, pressure=pressure, steps=steps, area_update=area_update, tol=tol, **plate)
    s.loads[0].table = Table(np.array([0.0, rise]), np.array([[0.0], [pressure]]))
    s.solution = Solution(GF_DYNAMIC, 0.0, steps * dt, dt, dt, dt / 4096, 30, 3, 4, 1.0, beta=beta, gamma=gamma,
                          rayleigh_alpha=rayleigh_alpha, rayleigh_beta=rayleigh_beta, update_rayleigh=update_rayleigh)
    return s


def plate_release(n: int = 3, pressure: float = 1e5, static_steps: int = 5, dt: float = 0.001,
                  dynamic_steps: int = 15, area_update: int = 1, tol: float = 1e-8) -> Structure:
    """Two solution steps, as the reference's Shell_1 tutorial: a Static step
    loads the clamped plate of square_plate with a follower pressure over
    [0, 1], the pressure is released at t = 1.0001, and a Dynamic step (beta
    0.3, gamma 0.5) follows the free vibration from the deformed state for
    `dynamic_steps` steps of dt."""
    s = square_plate(n, pressure=pressure, steps=static_steps, area_update=area_update, tol=tol)
    s.loads[0].table = Table(np.array([0.0, 1.0, 1.0001]), np.array([[0.0], [pressure], [0.0]]))
    s.next_steps = [Solution(GF_DYNAMIC, 1.0, 1.0 + dynamic_steps * dt, dt, dt, dt / 4096, 30, 3, 4, 1.0,
                             beta=0.3, gamma=0.5)]
    return s


def chain_sequence(n_el: int = 20, tip_force=(2e5, 0.0, 1e5), tol: float = 1e-8) -> Structure:
    """Four solution steps on a 10 m clamped pipe chain (first bending period
    near 0.26 s): Static [0, 1] raises a tip force; at t = 1.0001 it drops to
    half and a damped Dynamic step [1, 1.5] (Rayleigh alpha 0.5 1/s, beta
    0.002 s) follows the motion; a Dynamic step [1.5, 2] restarts from rest
    in the deformed shape (ZeroIC); a Static step [2, 2.5] raises the force
    back to its full value."""
    s = pipe_chain(n_el, 0.4, 0.03, list(tip_force), steps=5, element_length=10.0 / n_el, tol=tol)
    f = np.asarray(tip_force, dtype=np.float64)
    s.loads[0].table = Table(np.array([0.0, 1.0, 1.0001, 2.0, 2.5]),
                             np.array([[0.0] * 6, [*f, 0.0, 0.0, 0.0], [*(0.5 * f), 0.0, 0.0, 0.0],
                                       [*(0.5 * f), 0.0, 0.0, 0.0], [*f, 0.0, 0.0, 0.0]]))
    s.next_steps = [
        Solution(GF_DYNAMIC, 1.0, 1.5, 0.02, 0.02, 0.02 / 64, 30, 3, 4, 1.0, beta=0.25, gamma=0.5,
                 rayleigh_alpha=0.5, rayleigh_beta=0.002),
        Solution(GF_DYNAMIC, 1.5, 2.0, 0.025, 0.025, 0.025 / 64, 30, 3, 4, 1.0, beta=0.3, gamma=0.55, zero_ic=1),
        Solution(GF_STATIC, 2.0, 2.5, 0.1, 0.1, 0.1 / 64, 30, 3, 4, 1.0),
    ]
    return s


def served_mixed(n_requests: int, seed: int = 0, plate_share: float = 0.3, chain_dof=(1000, 50000),
                 plate_dof=(10000, 200000), steps: int = 10, tol: float = 1e-8) -> list:
    """The mixed served stream: each request is a pipe chain (free DOFs
    log-uniform in chain_dof, drawn as in served_chains) or, with probability
    plate_share, a clamped square Shell_1 plate (free DOFs log-uniform in
    plate_dof; an n x n x 2 mesh has about 20.7 n^2 free DOFs) under a
    follower pressure drawn from U(5e4, 1e5) Pa, ramped over `steps` load
    steps."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_requests):
        if rng.random() < plate_share:
            dof = math.exp(rng.uniform(math.log(plate_dof[0]), math.log(plate_dof[1])))
            n = max(2, int(round(math.sqrt(dof / 20.7))))
            out.append(square_plate(n, pressure=float(rng.uniform(5e4, 1e5)), steps=steps, tol=tol))
        else:
            dof = math.exp(rng.uniform(math.log(chain_dof[0]), math.log(chain_dof[1])))
            n_el = max(1, int(round((dof / 6.0 - 1.0) / 2.0)))
            De, wall = rng.uniform(0.3, 0.5), rng.uniform(0.02, 0.04)
            F = rng.normal(0.0, 1e5, 3)
            out.append(pipe_chain(n_el, float(De), float(wall), F, steps=steps, tol=tol,
                                  element_length=10.0 / n_el))
    return out

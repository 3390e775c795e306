"""Generates the golden fixtures in this folder from the reference itself.

Runs the reference's own Beam_1 / Static sources, compiled by
oracle/build_ref.py into oracle/_ref/libgiraffe_ref.so (this needs the
reference tree, so it runs only where that tree is present), on decks written
in the reference's .inp syntax by giraffe_gb300.model.Structure.to_inp, and
stores what the reference computes:

* ref_beam_elements.npz  Beam_1 tangent K (18x18) and unbalanced force P (18)
                         of single elements with random geometry, section,
                         coordinate system, committed history and increment
                         (Beam_1::PreCalc, SaveLagrange, Mount,
                         MountElementLoads).
* ref_tutorial01.npz     the reference's tutorial01 cantilever, every
                         converged configuration the reference writes
                         (Sample 2) and its Newton solve counts.
* ref_rollup.npz         20-element roll-up into a circle, every step.
* ref_chain.npz          a 30-element pipe chain under a tip force, 10 steps.
* ref_tutorial10.npz     the reference's tutorial10: Dynamic step (Newmark),
                         prescribed base translation and rotation, 2000 steps
                         (every 10th configuration, as the deck's Sample).
* ref_tutorial10_rayleigh.npz, ref_tutorial10_rayleigh_update.npz
                         tutorial10 with Rayleigh damping (alpha 0.2 1/s,
                         beta 0.002 s): C formed at the first iteration
                         (Update 0), and at every iteration (Update 1).
* ref_riser_rayleigh.npz a 12-element riser under a prescribed top motion
                         with Rayleigh damping (alpha 0.3, beta 0.004,
                         Update 1), 120 steps.
* ref_rotating_base_angles.npz, ref_rotating_base_vector.npz
                         a cantilever whose base turns by a prescribed rotation
                         read as Euler angles / as an Euler rotation vector
                         (NodalDisplacement AngularParameters), 10 steps.
* ref_pretension.npz     a 20-element pipe chain with PreTension 2e5 N in every
                         element under a lateral tip force, 10 steps.
* ref_beam_inertia.npz   Beam_1 inertial force and mass/gyroscopic tangent of
                         single elements (Beam_1::MountMass) with random
                         history, increments, nodal velocities/accelerations.
* ref_pipe_elements.npz  Pipe_1 tangent K (18x18) and unbalanced force P (18)
                         of single elements with random geometry, pipe
                         section, frame, history and increment, half of them
                         under an internal pressure (Pipe_1::PreCalc, Mount,
                         MountPipeSpecialLoads).
* ref_tutorial04.npz     the reference's tutorial04 deck itself (50 Pipe_1, a
                         lateral perturbation, then internal pressure raised
                         to 1.2 MPa over 200 Static steps), every step.
* ref_pipe_riser.npz     a 16-element Pipe_1 riser, pinned at the bottom, its
                         top driven laterally, under an internal pressure
                         raised to 20 MPa: Dynamic (Newmark), 100 steps.
* ref_pipe_riser_rayleigh.npz  the same with Rayleigh damping (alpha 0.3,
                         beta 0.004, Update 1).
* ref_monitor_tutorial10.npz, ref_monitor_chain.npz, ref_monitor_plate.npz,
  ref_monitor_sequence.npz
                         runs with a Monitor block: besides the configurations,
                         the reference's own monitor line of every monitored
                         node at every monitored time (Node::WriteMonitor).
* ref_modal_cantilever.npz, ref_modal_plate.npz, ref_modal_riser.npz
                         the two matrices of a Modal step (K_AA and the modal
                         mass M_AA, dense) from the reference build for
                         tutorial01's cantilever, a 3x3x2 plate and the
                         Pipe_1 riser, and their ten smallest eigenvalues.
* ref_shell_elements.npz Shell_1 tangent K (27x27) and unbalanced force P (27)
                         of single elements with random geometry, material,
                         thickness, committed history and increment, half of
                         them with a follower pressure (Shell_1::PreCalc,
                         SaveLagrange, Mount, MountElementLoads,
                         MountShellSpecialLoads; both AreaUpdate modes).
* ref_plate.npz          a clamped 4x4x2 Shell_1 plate under follower
                         pressure (AreaUpdate 1), 20 steps, every step.
* ref_plate_fixed_area.npz  a clamped 3x3x2 plate, AreaUpdate 0, 10 steps.
* ref_shell_inertia.npz  Shell_1 inertial force and mass/gyroscopic tangent of
                         single elements (Shell_1::MountMass) with random
                         history, increments, nodal velocities/accelerations.
* ref_plate_dynamic.npz  the clamped 3x3x2 plate in a Dynamic step: follower
                         pressure raised over 2 ms, Newmark, 20 steps of 1 ms.
* ref_plate_dynamic_rayleigh.npz, ref_plate_dynamic_rayleigh_update.npz
                         the same with Rayleigh damping (alpha 8 1/s, beta
                         2e-5 s), AreaUpdate 0 with C formed once, and
                         AreaUpdate 1 with C formed at every iteration.
* ref_plate_release.npz  two solution steps: the 3x3x2 plate loaded in a Static
                         step, then released into a Dynamic step (15 steps).
* ref_chain_sequence.npz four solution steps on a pipe chain: Static, damped
                         Dynamic after a load drop, Dynamic from rest (ZeroIC),
                         Static reloading.
* ref_plate24.npz        a clamped 24x24x2 Shell_1 plate (11,667 free DOFs,
                         half-bandwidth 506) under follower pressure ramped to
                         1e5 Pa over 20 steps: the Newton solve counts, every
                         5th configuration and the last (nodes only).
* ref_tutorial05.npz     the reference's tutorial05 deck itself (400 Shell_1,
                         a Static then a Dynamic step), every 10th
                         configuration; the reference needs tens of minutes.

Node records hold copy_coordinates (position and accumulated Rodrigues
vector) then the nodal Q (row-major); Gauss-point records hold Q_i
(row-major).

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py <fixture>  # one (elements | ref_*.npz)
"""
import ctypes as C
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from giraffe_gb300 import configs  # noqa: E402
from giraffe_gb300.model import NodalLoad, PipeLoad, PressureLoad, Solution, Structure, Table  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "libgiraffe_ref.so")


def ref_lib():
    if not os.path.exists(REF):
        subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "build_ref.py")], check=True)
    L = C.CDLL(REF)
    dp = C.POINTER(C.c_double)
    L.giraffe_ref_load.argtypes = [C.c_char_p]
    L.giraffe_ref_solve.argtypes = [C.c_char_p, C.c_char_p]
    L.giraffe_ref_set_increment.argtypes = [C.c_int, dp]
    L.giraffe_ref_element_mount.argtypes = [C.c_int, dp, dp]
    L.giraffe_ref_shell_pressure.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp]
    L.giraffe_ref_pipe_pressure.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp]
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def parse_monitor(path):
    """Monitor lines "M <node>" + Node::WriteMonitor's 31 columns (TIME, X..Z,
    ROTX..ROTZ, FX..MZ, FXloc..MZloc, dX..dROTZ, ddX..ddROTZ): (0-based node
    ids, [node][record][31])."""
    rows = {}
    for line in open(path):
        p = line.split()
        if p and p[0] == "M":
            rows.setdefault(int(p[1]), []).append([float(x) for x in p[2:]])
    ids = list(rows)
    return np.array([i - 1 for i in ids], dtype=np.int32), np.array([rows[i] for i in ids])


def parse_rec(path):
    recs = []
    cur = None
    for line in open(path):
        p = line.split()
        if p[0] == "M":
            continue
        if p[0] == "T":
            cur = {"t": float(p[2]), "N": [], "G": []}
            recs.append(cur)
        elif p[0] == "N":
            v = [float(x) for x in p[2:]]
            q = np.array(v[6:]).reshape(3, 3).T.ravel()  # column-major -> row-major
            cur["N"].append(v[:6] + list(q))
        elif p[0] == "G":
            v = [float(x) for x in p[3:]]
            cur["G"].append(list(np.array(v).reshape(3, 3).T.ravel()))
    times = np.array([r["t"] for r in recs])
    nodes = np.array([r["N"] for r in recs])
    gq = np.array([np.array(r["G"]).reshape(-1, 2, 9) for r in recs])
    return times, nodes, gq


def parse_log(path):
    """Per load step: (time, Newton solves, diverged)."""
    steps = []
    for line in open(path):
        m = re.match(r"Time: ([0-9.eE+-]+)", line)
        if m:
            steps.append([float(m.group(1)), 0, 0])
        elif line.startswith("It.:"):
            steps[-1][1] += 1
        elif "diverged" in line:
            steps[-1][2] = 1
    return np.array(steps)


def run_deck(L, s, tag, tmp):
    deck = os.path.join(tmp, tag + ".inp")
    with open(deck, "w") as f:
        f.write(s.to_inp())
    assert L.giraffe_ref_load(deck.encode()) == 0, tag
    rec = os.path.join(tmp, tag + ".rec")
    log = os.path.join(tmp, tag + ".log")
    rc = L.giraffe_ref_solve(rec.encode(), log.encode())
    times, nodes, gq = parse_rec(rec)
    steps = parse_log(log)
    out = dict(rc=np.array(rc), times=times, nodes=nodes, gp_Q=gq, steps=steps, deck=np.array(s.to_inp()))
    if s.monitor is not None and s.monitor.nodes:
        out["monitor_nodes"], out["monitor"] = parse_monitor(rec)
    return out


def element_cases(rng, n):
    cases = []
    for k in range(n):
        # random element geometry along a random axis, CS with E3 on the axis
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        L = rng.uniform(0.2, 2.0)
        x0 = rng.normal(size=3)
        xyz = np.array([x0, x0 + 0.5 * L * axis, x0 + L * axis])
        t = rng.normal(size=3)
        e1 = t - t.dot(axis) * axis
        e1 /= np.linalg.norm(e1)
        if k % 3 == 0:
            sec = ("rect", rng.uniform(0.05, 0.2), rng.uniform(0.05, 0.2))
        else:
            De = rng.uniform(0.2, 0.5)
            sec = ("tube", De, De - 2 * rng.uniform(0.01, 0.04))
        mat = (rng.uniform(5e9, 2.5e11), rng.uniform(0.2, 0.4), 7850.0)
        nh = int(rng.integers(0, 4))
        scale = np.array([0.02 * L] * 3 + [0.15] * 3)
        hist = rng.normal(size=(nh, 3, 6)) * scale
        disp = rng.normal(size=(3, 6)) * scale
        cases.append(dict(xyz=xyz, e1=e1, e3=axis, sec=sec, mat=mat, hist=hist, disp=disp))
    return cases


def run_elements(L, cases, tmp):
    out = {k: [] for k in ("xyz", "mat", "sec6", "cs", "hist", "disp", "K", "P")}
    for i, c in enumerate(cases):
        s = Structure(nodes=c["xyz"])
        mat = s.add_material(*c["mat"])
        sec = s.add_rectangle(c["sec"][1], c["sec"][2]) if c["sec"][0] == "rect" else s.add_tube(c["sec"][1], c["sec"][2])
        cs = s.add_cs(c["e1"], c["e3"])
        s.beams.append((0, 1, 2, mat, sec, cs))
        deck = os.path.join(tmp, f"el{i}.inp")
        with open(deck, "w") as f:
            f.write(s.to_inp())
        assert L.giraffe_ref_load(deck.encode()) == 0
        L.giraffe_ref_prepare()
        for h in c["hist"]:
            for n in range(3):
                v = np.ascontiguousarray(h[n])
                L.giraffe_ref_set_increment(n + 1, _dp(v))
            L.giraffe_ref_commit()
        for n in range(3):
            v = np.ascontiguousarray(c["disp"][n])
            L.giraffe_ref_set_increment(n + 1, _dp(v))
        K = np.zeros(324)
        P = np.zeros(18)
        assert L.giraffe_ref_element_mount(1, _dp(K), _dp(P)) == 18
        hist = np.zeros((3, 18))
        hist[: len(c["hist"])] = c["hist"].reshape(-1, 18)
        out["xyz"].append(c["xyz"].ravel())
        out["mat"].append(np.array(s.materials[0]))
        out["sec6"].append(np.array(s.sections[0]))
        out["cs"].append(np.array(s.cs[0]))
        out["hist"].append(hist)
        out["disp"].append(c["disp"].ravel())
        out["K"].append(K.reshape(18, 18).T)  # row-major [r][s]
        out["P"].append(P)
    res = {k: np.array(v) for k, v in out.items()}
    res["n_hist"] = np.array([len(c["hist"]) for c in cases])
    return res


def run_inertia(L, cases, tmp, rng):
    dp = C.POINTER(C.c_double)
    L.giraffe_ref_set_vel_accel.argtypes = [C.c_int, dp, dp]
    L.giraffe_ref_beam_inertia.argtypes = [C.c_int, C.c_double, dp, dp, dp]
    out = {k: [] for k in ("xyz", "mat", "sec6", "cs", "hist", "disp", "vel", "acc", "dt", "beta", "gamma",
                           "M", "F", "ke")}
    nh_list = []
    for i, c in enumerate(cases):
        s = Structure(nodes=c["xyz"])
        mat = s.add_material(*c["mat"])
        sec = s.add_rectangle(c["sec"][1], c["sec"][2]) if c["sec"][0] == "rect" else s.add_tube(c["sec"][1], c["sec"][2])
        cs = s.add_cs(c["e1"], c["e3"])
        s.beams.append((0, 1, 2, mat, sec, cs))
        beta, gamma, dt = rng.uniform(0.25, 0.35), rng.uniform(0.5, 0.6), rng.uniform(1e-3, 2e-2)
        s.solution = Solution(1, 0.0, 1.0, dt, dt, dt / 100, 20, 3, 4, 1.0, beta=beta, gamma=gamma)
        deck = os.path.join(tmp, f"in{i}.inp")
        with open(deck, "w") as f:
            f.write(s.to_inp())
        assert L.giraffe_ref_load(deck.encode()) == 0
        L.giraffe_ref_prepare()
        for h in c["hist"]:
            for n in range(3):
                L.giraffe_ref_set_increment(n + 1, _dp(np.ascontiguousarray(h[n])))
            L.giraffe_ref_commit()
        vel = rng.normal(size=(3, 6))
        acc = rng.normal(size=(3, 6)) * 5
        for n in range(3):
            L.giraffe_ref_set_vel_accel(n + 1, _dp(np.ascontiguousarray(vel[n])), _dp(np.ascontiguousarray(acc[n])))
            L.giraffe_ref_set_increment(n + 1, _dp(np.ascontiguousarray(c["disp"][n])))
        M = np.zeros(324)
        F = np.zeros(18)
        ke = np.zeros(1)
        assert L.giraffe_ref_beam_inertia(1, dt, _dp(M), _dp(F), _dp(ke)) == 18
        hist = np.zeros((3, 18))
        hist[: len(c["hist"])] = c["hist"].reshape(-1, 18)
        for k, v in (("xyz", c["xyz"].ravel()), ("mat", np.array(s.materials[0])), ("sec6", np.array(s.sections[0])),
                     ("cs", np.array(s.cs[0])), ("hist", hist), ("disp", c["disp"].ravel()), ("vel", vel.ravel()),
                     ("acc", acc.ravel()), ("dt", dt), ("beta", beta), ("gamma", gamma), ("M", M.reshape(18, 18).T),
                     ("F", F), ("ke", ke[0])):
            out[k].append(v)
        nh_list.append(len(c["hist"]))
    res = {k: np.array(v) for k, v in out.items()}
    res["n_hist"] = np.array(nh_list)
    return res


def run_pipe_elements(L, rng, n, tmp):
    """Single Pipe_1 elements: random geometry, pipe section, frame, history
    and increment; half of them under an internal pressure (PipeLoad)."""
    out = {k: [] for k in ("xyz", "ps", "cs", "hist", "disp", "pressure", "K", "P")}
    nh_list = []
    for i, c in enumerate(element_cases(rng, n)):
        s = Structure(nodes=c["xyz"])
        De = rng.uniform(0.2, 0.7)
        Di = De - 2 * rng.uniform(0.01, 0.04)
        E = rng.uniform(5e10, 2.1e11)
        A = np.pi / 4 * (De * De - Di * Di)
        I = np.pi / 64 * (De ** 4 - Di ** 4)
        ps = s.add_pipe_section(E * A, E * I, 0.8 * E * I, 0.4 * E * A, 7850.0 * A, De, Di)
        cs = s.add_cs(c["e1"], c["e3"])
        s.add_pipe(0, 1, 2, ps, cs)
        press = i % 2 == 1
        p = rng.uniform(-2e6, 2e6)
        if press:
            s.loads.append(PipeLoad([0], Table(np.array([0.0, 10.0]), np.array([[p, 0, 0, 0], [p, 0, 0, 0]]))))
        deck = os.path.join(tmp, f"pp{i}.inp")
        with open(deck, "w") as f:
            f.write(s.to_inp())
        assert L.giraffe_ref_load(deck.encode()) == 0
        L.giraffe_ref_prepare()
        for h in c["hist"]:
            for nd in range(3):
                L.giraffe_ref_set_increment(nd + 1, _dp(np.ascontiguousarray(h[nd])))
            L.giraffe_ref_commit()
        for nd in range(3):
            L.giraffe_ref_set_increment(nd + 1, _dp(np.ascontiguousarray(c["disp"][nd])))
        K = np.zeros(324)
        P = np.zeros(18)
        if press:
            assert L.giraffe_ref_pipe_pressure(1, 1, 1.0, _dp(K), _dp(P)) == 18
        else:
            assert L.giraffe_ref_element_mount(1, _dp(K), _dp(P)) == 18
        hist = np.zeros((3, 18))
        hist[: len(c["hist"])] = c["hist"].reshape(-1, 18)
        for k, v in (("xyz", c["xyz"].ravel()), ("ps", np.array(s.pipe_sections[0])), ("cs", np.array(s.cs[0])),
                     ("hist", hist), ("disp", c["disp"].ravel()), ("pressure", p if press else 0.0),
                     ("K", K.reshape(18, 18).T), ("P", P)):
            out[k].append(v)
        nh_list.append(len(c["hist"]))
    res = {k: np.array(v) for k, v in out.items()}
    res["n_hist"] = np.array(nh_list)
    return res


def run_shell_elements(L, rng, n, tmp):
    out = {k: [] for k in ("xyz", "mat", "thick", "hist", "disp", "pressure", "area_update", "K", "P")}
    nh_list = []
    for i in range(n):
        c = rng.normal(size=(3, 3))
        if i % 4 == 0:
            c[:, 2] = 0.0  # in the x-y plane
        xyz = np.vstack([c, 0.5 * (c[0] + c[1]), 0.5 * (c[1] + c[2]), 0.5 * (c[2] + c[0])])
        s = Structure(nodes=xyz)
        matv = (rng.uniform(5e10, 2.1e11), rng.uniform(0.2, 0.4), 7850.0)
        mat = s.add_material(*matv)
        t = rng.uniform(0.005, 0.05)
        sec = s.add_shell_section(t)
        cs = s.add_cs((1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
        s.shells.append((0, 1, 2, 3, 4, 5, mat, sec, cs))
        press = i % 2 == 1
        area_update = int(i % 4 == 3)
        p = rng.uniform(-1e5, 1e5)
        if press:
            s.loads.append(PressureLoad([0], Table(np.array([0.0, 10.0]), np.array([[p], [p]])),
                                        area_update=area_update))
        deck = os.path.join(tmp, f"sh{i}.inp")
        with open(deck, "w") as f:
            f.write(s.to_inp())
        assert L.giraffe_ref_load(deck.encode()) == 0
        L.giraffe_ref_prepare()
        nh = int(rng.integers(0, 4))
        scale = np.array([0.01] * 3 + [0.1] * 3)
        hist = np.zeros((3, 27))
        for q in range(nh + 1):
            dn = rng.normal(size=(6, 6)) * scale
            dn[:3, 3:] = 0.0  # corner nodes carry no rotation
            for nd in range(6):
                L.giraffe_ref_set_increment(nd + 1, _dp(np.ascontiguousarray(dn[nd])))
            d27 = np.concatenate([dn[:, :3].ravel(), dn[3:, 3:].ravel()])
            if q < nh:
                L.giraffe_ref_commit()
                hist[q] = d27
        K = np.zeros(729)
        P = np.zeros(27)
        if press:
            assert L.giraffe_ref_shell_pressure(1, 1, 1.0, _dp(K), _dp(P)) == 27
        else:
            assert L.giraffe_ref_element_mount(1, _dp(K), _dp(P)) == 27
        for k, v in (("xyz", xyz.ravel()), ("mat", np.array(matv)), ("thick", t), ("hist", hist), ("disp", d27),
                     ("pressure", p if press else np.nan), ("area_update", area_update),
                     ("K", K.reshape(27, 27).T), ("P", P)):
            out[k].append(v)
        nh_list.append(nh)
    res = {k: np.array(v) for k, v in out.items()}
    res["n_hist"] = np.array(nh_list)
    return res


def run_shell_inertia(L, rng, n, tmp):
    dp = C.POINTER(C.c_double)
    L.giraffe_ref_set_vel_accel.argtypes = [C.c_int, dp, dp]
    L.giraffe_ref_shell_inertia.argtypes = [C.c_int, C.c_double, dp, dp, dp]
    out = {k: [] for k in ("xyz", "mat", "thick", "hist", "disp", "vel", "acc", "dt", "beta", "gamma", "M", "F", "ke")}
    nh_list = []
    for i in range(n):
        c = rng.normal(size=(3, 3))
        if i % 4 == 0:
            c[:, 2] = 0.0  # in the x-y plane
        xyz = np.vstack([c, 0.5 * (c[0] + c[1]), 0.5 * (c[1] + c[2]), 0.5 * (c[2] + c[0])])
        s = Structure(nodes=xyz)
        matv = (rng.uniform(5e10, 2.1e11), rng.uniform(0.2, 0.4), rng.uniform(2000.0, 8000.0))
        mat = s.add_material(*matv)
        t = rng.uniform(0.005, 0.05)
        sec = s.add_shell_section(t)
        cs = s.add_cs((1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
        s.shells.append((0, 1, 2, 3, 4, 5, mat, sec, cs))
        beta, gamma, dt = rng.uniform(0.25, 0.35), rng.uniform(0.5, 0.6), rng.uniform(1e-3, 2e-2)
        s.solution = Solution(1, 0.0, 1.0, dt, dt, dt / 100, 20, 3, 4, 1.0, beta=beta, gamma=gamma)
        deck = os.path.join(tmp, f"si{i}.inp")
        with open(deck, "w") as f:
            f.write(s.to_inp())
        assert L.giraffe_ref_load(deck.encode()) == 0
        L.giraffe_ref_prepare()
        nh = int(rng.integers(0, 4))
        scale = np.array([0.01] * 3 + [0.1] * 3)
        hist = np.zeros((3, 27))
        vel = rng.normal(size=(6, 6))
        acc = rng.normal(size=(6, 6)) * 5
        vel[:3, 3:] = 0.0  # corner nodes carry no rotation
        acc[:3, 3:] = 0.0
        for q in range(nh + 1):
            dn = rng.normal(size=(6, 6)) * scale
            dn[:3, 3:] = 0.0
            for nd in range(6):
                L.giraffe_ref_set_increment(nd + 1, _dp(np.ascontiguousarray(dn[nd])))
            d27 = np.concatenate([dn[:, :3].ravel(), dn[3:, 3:].ravel()])
            if q < nh:
                L.giraffe_ref_commit()
                hist[q] = d27
        for nd in range(6):
            L.giraffe_ref_set_vel_accel(nd + 1, _dp(np.ascontiguousarray(vel[nd])), _dp(np.ascontiguousarray(acc[nd])))
        M = np.zeros(729)
        F = np.zeros(27)
        ke = np.zeros(1)
        assert L.giraffe_ref_shell_inertia(1, dt, _dp(M), _dp(F), _dp(ke)) == 27
        for k, v in (("xyz", xyz.ravel()), ("mat", np.array(matv)), ("thick", t), ("hist", hist), ("disp", d27),
                     ("vel", vel.ravel()), ("acc", acc.ravel()), ("dt", dt), ("beta", beta), ("gamma", gamma),
                     ("M", M.reshape(27, 27).T), ("F", F), ("ke", ke[0])):
            out[k].append(v)
        nh_list.append(nh)
    res = {k: np.array(v) for k, v in out.items()}
    res["n_hist"] = np.array(nh_list)
    return res


def small_chain():
    return configs.pipe_chain(30, 0.4, 0.03, [1.5e5, -1.0e5, 0.8e5], element_length=10.0 / 30)


DECKS = {
    "ref_tutorial01.npz": configs.tutorial01,
    "ref_rollup.npz": configs.cantilever_rollup,
    "ref_chain.npz": small_chain,
    "ref_tutorial10.npz": configs.tutorial10,
    "ref_plate.npz": lambda: configs.square_plate(4, steps=20),
    "ref_plate_fixed_area.npz": lambda: configs.square_plate(3, steps=10, area_update=0),
    "ref_pretension.npz": configs.pretensioned_chain,
    "ref_rotating_base_angles.npz": lambda: configs.rotating_base("EulerAngles"),
    "ref_rotating_base_vector.npz": lambda: configs.rotating_base("EulerVector"),
    "ref_tutorial10_rayleigh.npz": lambda: configs.tutorial10(0.2, 0.002, 0),
    "ref_tutorial10_rayleigh_update.npz": lambda: configs.tutorial10(0.2, 0.002, 1),
    "ref_plate_dynamic.npz": lambda: configs.plate_dynamics(3, steps=20),
    "ref_plate_dynamic_rayleigh.npz": lambda: configs.plate_dynamics(3, steps=20, area_update=0, rayleigh_alpha=8.0,
                                                                     rayleigh_beta=2e-5),
    "ref_plate_dynamic_rayleigh_update.npz": lambda: configs.plate_dynamics(3, steps=20, rayleigh_alpha=8.0,
                                                                            rayleigh_beta=2e-5, update_rayleigh=1),
    "ref_plate_release.npz": lambda: configs.plate_release(3),
    "ref_chain_sequence.npz": configs.chain_sequence,
    "ref_pipe_riser.npz": configs.pipe_riser,
    "ref_pipe_riser_rayleigh.npz": lambda: configs.pipe_riser(rayleigh_alpha=0.3, rayleigh_beta=0.004,
                                                              update_rayleigh=1),
    "ref_riser_rayleigh.npz": lambda: configs.riser_chain(12, 0.4, 0.03, 1.0, 4.0, steps=120, element_length=2.0,
                                                          rayleigh_alpha=0.3, rayleigh_beta=0.004,
                                                          update_rayleigh=1),
}


REF_INPUTS = os.path.join(os.environ.get("GIRAFFE_REFERENCE", "/root/reference"), "inputs")


def make_tutorial05(stride: int = 10):
    """The reference's own Shell_1 deck, tutorial05 (a strip loaded at its tip
    in a Static step, then released into a Dynamic step), run from its file.
    The deck writes every step; every `stride`-th configuration and the last
    are kept.  The stored deck is the same structure written by
    Structure.to_inp, which reads back identically."""
    from giraffe_gb300.deck import read_deck_file

    path = os.path.join(REF_INPUTS, "tutorial05", "tutorial05.inp")
    L = ref_lib()
    s = read_deck_file(path)
    with tempfile.TemporaryDirectory() as tmp:
        assert L.giraffe_ref_load(path.encode()) == 0
        rec = os.path.join(tmp, "t05.rec")
        log = os.path.join(tmp, "t05.log")
        rc = L.giraffe_ref_solve(rec.encode(), log.encode())
        times, nodes, gq = parse_rec(rec)
        steps = parse_log(log)
    keep = sorted(set(range(0, len(times), stride)) | {len(times) - 1})
    np.savez_compressed(os.path.join(HERE, "ref_tutorial05.npz"), rc=np.array(rc), times=times[keep],
                        nodes=nodes[keep], gp_Q=gq[keep], steps=steps, deck=np.array(s.to_inp()))


def make_plate24(stride: int = 5):
    """The benchmark's plate family at a size whose band (half-bandwidth
    506) spans many 64-wide tiles of the wide-band LU: every `stride`-th
    configuration and the last, without the Gauss-point records."""
    L = ref_lib()
    with tempfile.TemporaryDirectory() as tmp:
        r = run_deck(L, configs.square_plate(24, steps=20), "plate24", tmp)
    keep = sorted(set(range(0, len(r["times"]), stride)) | {len(r["times"]) - 1})
    np.savez_compressed(os.path.join(HERE, "ref_plate24.npz"), rc=r["rc"], times=r["times"][keep],
                        nodes=r["nodes"][keep], steps=r["steps"], deck=r["deck"])


def make_elements():
    L = ref_lib()
    rng = np.random.default_rng(20261203)
    with tempfile.TemporaryDirectory() as tmp:
        np.savez_compressed(os.path.join(HERE, "ref_beam_elements.npz"), **run_elements(L, element_cases(rng, 24), tmp))
        np.savez_compressed(os.path.join(HERE, "ref_beam_inertia.npz"),
                            **run_inertia(L, element_cases(rng, 16), tmp, rng))
        np.savez_compressed(os.path.join(HERE, "ref_shell_elements.npz"), **run_shell_elements(L, rng, 24, tmp))
        np.savez_compressed(os.path.join(HERE, "ref_shell_inertia.npz"), **run_shell_inertia(L, rng, 16, tmp))


def _monitored(make, nodes, sample=1, end_steps=None):
    """A configuration with a Monitor block on `nodes` (optionally cut to its
    first `end_steps` time steps)."""
    def build():
        from giraffe_gb300.model import MonitorSpec
        s = make()
        if end_steps is not None:
            s.solution.end_time = s.solution.start_time + end_steps * s.solution.time_step
        s.monitor = MonitorSpec(sample, list(nodes))
        return s
    return build


DECKS.update({
    # monitored nodes: Node::WriteMonitor's columns after each converged
    # step (positions, Euler rotation vectors, the internal-force / reaction
    # vector with pseudo-moments turned to moments, velocities, accelerations)
    "ref_monitor_tutorial10.npz": _monitored(configs.tutorial10, [0, 5, 10], sample=3, end_steps=150),
    "ref_monitor_chain.npz": _monitored(small_chain, [0, 1, 30, 60]),
    "ref_monitor_plate.npz": _monitored(lambda: configs.square_plate(3, steps=10), [0, 3, 24, 23]),
    "ref_monitor_sequence.npz": _monitored(configs.chain_sequence, [0, 20, 40], sample=2),
})

MODAL_DECKS = {
    "ref_modal_cantilever.npz": configs.tutorial01,
    "ref_modal_plate.npz": lambda: configs.square_plate(3, steps=10),
    "ref_modal_riser.npz": configs.pipe_riser,
}


def make_modal(name, n_modes: int = 10):
    """The two matrices of a Modal step from the reference build (K_AA and
    the modal mass M_AA, dense, the reference's numbering) and the n_modes
    smallest eigenvalues of K x = lambda M x from them.  The reference's own
    eigen solve is ARPACK's shift-invert Arnoldi (arpack-ng, a vcpkg
    dependency not in the reference tree); LAPACK's symmetric-definite
    solver stands in for it on these symmetric matrices."""
    import scipy.linalg
    from giraffe_gb300.model import ModalStep

    L = ref_lib()
    dp = C.POINTER(C.c_double)
    L.giraffe_ref_modal_matrices.argtypes = [dp, dp, C.c_int]
    s = MODAL_DECKS[name]()
    s.modal = ModalStep(number_modes=n_modes, tolerance=0.0)
    with tempfile.TemporaryDirectory() as tmp:
        deck = os.path.join(tmp, "modal.inp")
        with open(deck, "w") as f:
            f.write(s.to_inp())
        assert L.giraffe_ref_load(deck.encode()) == 0
        nmax = 4096
        K = np.zeros(nmax * nmax)
        M = np.zeros(nmax * nmax)
        n = L.giraffe_ref_modal_matrices(_dp(K), _dp(M), nmax)
        assert n > 0
    K = K[: n * n].reshape(n, n).T.copy()
    M = M[: n * n].reshape(n, n).T.copy()
    w = scipy.linalg.eigh(K, M, eigvals_only=True, subset_by_index=[0, n_modes - 1])
    np.savez_compressed(os.path.join(HERE, name), K=K, M=M, eig=w, deck=np.array(s.to_inp()))


def make_pipe_elements():
    L = ref_lib()
    rng = np.random.default_rng(20261204)
    with tempfile.TemporaryDirectory() as tmp:
        np.savez_compressed(os.path.join(HERE, "ref_pipe_elements.npz"), **run_pipe_elements(L, rng, 24, tmp))


def make_tutorial04():
    """The reference's own Pipe_1 deck, tutorial04 (a pinned pipe perturbed
    by a lateral load, then under internal pressure raised to 1.2 MPa in 200
    steps), run from its file; every converged configuration."""
    from giraffe_gb300.deck import read_deck_file

    path = os.path.join(REF_INPUTS, "tutorial04", "tutorial04.inp")
    L = ref_lib()
    s = read_deck_file(path)
    with tempfile.TemporaryDirectory() as tmp:
        assert L.giraffe_ref_load(path.encode()) == 0
        rec = os.path.join(tmp, "t04.rec")
        log = os.path.join(tmp, "t04.log")
        rc = L.giraffe_ref_solve(rec.encode(), log.encode())
        times, nodes, gq = parse_rec(rec)
        steps = parse_log(log)
        mon_ids, mon = parse_monitor(rec)
    np.savez_compressed(os.path.join(HERE, "ref_tutorial04.npz"), rc=np.array(rc), times=times, nodes=nodes,
                        gp_Q=gq, steps=steps, deck=np.array(s.to_inp()), monitor_nodes=mon_ids, monitor=mon)


def make_deck(name):
    L = ref_lib()
    with tempfile.TemporaryDirectory() as tmp:
        np.savez_compressed(os.path.join(HERE, name), **run_deck(L, DECKS[name](), name.split(".")[0], tmp))


def main():
    """Each deck runs in a process of its own: the reference keeps its
    database in one global object, which a second deck does not fully
    reset."""
    if len(sys.argv) > 1:
        if sys.argv[1] == "elements":
            make_elements()
        elif sys.argv[1] == "ref_tutorial05.npz":
            make_tutorial05()
        elif sys.argv[1] == "ref_tutorial04.npz":
            make_tutorial04()
        elif sys.argv[1] == "ref_pipe_elements.npz":
            make_pipe_elements()
        elif sys.argv[1] in MODAL_DECKS:
            make_modal(sys.argv[1])
        elif sys.argv[1] == "ref_plate24.npz":
            make_plate24()
        else:
            make_deck(sys.argv[1])
        return
    ref_lib()
    for job in (["elements", "ref_pipe_elements.npz"] + list(DECKS) + list(MODAL_DECKS) +
                ["ref_tutorial04.npz", "ref_tutorial05.npz", "ref_plate24.npz"]):
        subprocess.run([sys.executable, os.path.abspath(__file__), job], check=True)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()

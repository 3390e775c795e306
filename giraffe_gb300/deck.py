"""Reader of GIRAFFE input decks (.inp) for what this library solves.

The reference reads a deck token by token (fscanf "%s") in IO::ReadFile
(reference src/IO.cpp:193-657), each top-level keyword handing the stream to
the block's own reader.  This reader follows the same keywords and layouts
for the blocks of a sequence of Beam_1 / Shell_1 Static and Dynamic
solution steps:

  SolutionSteps   Static / Dynamic (src/Static.cpp:40-130,
                  src/Dynamic.cpp:60-215: EndTime ... Sample, RayleighDamping,
                  NewmarkCoefficients, optional ZeroIC); a deck's only step
                  may be Modal (src/Modal.cpp:42-108: ExportMatrices,
                  NumberModes, Tolerance, ComputeEigenvectors, NumberFrames)
  Nodes           Node id x y z
  Elements        Beam_1 id Mat Sec CS Nodes a b c [PreTension p]
                  (src/Beam_1.cpp:371-430); Pipe_1 id PipeSec CS Nodes a b c
                  (src/Pipe_1.cpp:535-572); Shell_1 id Mat Sec [CS] Nodes
                  six ids (src/Shell_1.cpp:538-590)
  Materials       Hooke id E Nu Rho
  Sections        Rectangle id B H; Tube id De Di
  PipeSections    PS id EA EI GJ GA Rho CDt CDn CAt CAn De Di
                  (src/PipeSection.cpp:19-131)
  ShellSections   Homogeneous id Thickness
  CoordinateSystems  CS id E1 x y z E3 x y z
  NodeSets / ElementSets  List ids | Sequence Initial i Increment d
                  (src/NodeSet.cpp:30-95)
  Loads           NodalLoad id NodeSet CS NTimes n + n rows (t, 6 values);
                  ShellLoad id ElementSet AreaUpdate NTimes n + n rows (t, p);
                  PipeLoad id ElementSet NTimes n + n rows (t, P0I, P0E,
                  RhoI, RhoE) (src/PipeLoad.cpp:45-88)
  Displacements   NodalDisplacement id NodeSet CS [AngularParameters
                  EulerAngles | EulerVector] [BoolTable ...] NTimes n + n rows
                  (src/NodalDisplacement.cpp:40-120)
  Constraints     NodalConstraint id NodeSet + UX..ROTZ BoolTable ...
  ConvergenceCriteria  the twelve tolerances and references
                  (src/ConvergenceCriteria.cpp:60-165)

Monitor blocks are read (Sample and MonitorNodes; the other monitor lists
are read past).  Output and run-control blocks (PostFiles, SolverOptions,
ExecutionData, ConfigurationSave) are skipped.  A block this library does not
solve (contact, particles, other elements, environment loads, special
constraints, ...) raises DeckError naming it, instead of being ignored.
Text from '//' to the end of a line is a comment.  Bool tables hold one
value per solution step and repeat their last value (src/BoolTable.cpp:23-80).
"""
from __future__ import annotations

import numpy as np

from .model import (DEFAULT_CRITERIA, GF_DYNAMIC, GF_STATIC, ModalStep, MonitorSpec, NodalDisplacement, NodalLoad,
                    PipeLoad, PressureLoad, Solution, Structure, Table)

# Every top-level keyword of IO::ReadFile: a block reader stops at the next one.
TOP = {
    "SolutionSteps", "Nodes", "SuperNodes", "Points", "Arcs", "Elements", "Particles", "InitialConditions",
    "Materials", "Sections", "PipeSections", "ShellSections", "CoordinateSystems", "RigidBodyData", "Environment",
    "Monitor", "SolverOptions", "AnalyticalSurfaces", "Surfaces", "Splines", "LineRegions", "SurfaceRegions",
    "Contacts", "NodeSets", "SuperNodeSets", "SurfaceSets", "ElementSets", "Loads", "Displacements", "Constraints",
    "SpecialConstraints", "SectionDetails", "AerodynamicData", "BEM", "GeneralContactSearch", "ConfigurationSave",
    "ConcomitantSolution", "ConvergenceCriteria", "PostFiles", "ExecutionData", "PSYCoupling", "CADData",
    "ContactInterfaces", "Boundaries", "Geometries", "BodyGeometries", "EOF",
}
SKIPPED = {"PostFiles", "SolverOptions", "ExecutionData", "ConfigurationSave", "ConcomitantSolution"}
CRITERIA_KEYS = {
    "ForceTolerance": "force_tol", "MomentTolerance": "moment_tol", "ForceMinimumReference": "force_min",
    "MomentMinimumReference": "moment_min", "ConstraintMinimumReference": "constraint_min",
    "DisplacementTolerance": "disp_tol", "RotationTolerance": "rot_tol", "LagrangeTolerance": "lag_tol",
    "DisplacementMinimumReference": "disp_min", "RotationMinimumReference": "rot_min",
    "LagrangeMinimumReference": "lag_min", "DivergenceReference": "divergence_ref",
}
DOF_NAMES = ("UX", "UY", "UZ", "ROTX", "ROTY", "ROTZ")


class DeckError(ValueError):
    """A deck this reader cannot turn into a solvable structure."""


class _Tokens:
    def __init__(self, text: str):
        toks = []
        for line in text.splitlines():
            k = line.find("//")
            toks.extend((line if k < 0 else line[:k]).split())
        self.t = toks
        self.i = 0

    def more(self) -> bool:
        return self.i < len(self.t)

    def peek(self) -> str | None:
        return self.t[self.i] if self.i < len(self.t) else None

    def next(self) -> str:
        if self.i >= len(self.t):
            raise DeckError("unexpected end of deck")
        self.i += 1
        return self.t[self.i - 1]

    def expect(self, word: str) -> None:
        w = self.next()
        if w != word:
            raise DeckError(f"expected '{word}', found '{w}' (token {self.i})")

    def int(self) -> int:
        w = self.next()
        try:
            return int(w)
        except ValueError:
            raise DeckError(f"expected an integer, found '{w}' (token {self.i})") from None

    def float(self) -> float:
        w = self.next()
        try:
            return float(w)
        except ValueError:
            raise DeckError(f"expected a number, found '{w}' (token {self.i})") from None

    def bool_table(self) -> list:
        # values while the next token starts with a digit
        vals = [self.int() == 1]
        while self.more() and self.peek()[0].isdigit():
            vals.append(self.int() == 1)
        return vals


def _step_value(table: list, step: int) -> bool:
    return table[step - 1] if step - 1 < len(table) else table[-1]


def _ids(tk: _Tokens, n: int) -> list:
    kind = tk.next()
    if kind == "List":
        return [tk.int() for _ in range(n)]
    if kind == "Sequence":
        tk.expect("Initial")
        first = tk.int()
        tk.expect("Increment")
        inc = tk.int()
        return [first + k * inc for k in range(n)]
    raise DeckError(f"a set needs 'List' or 'Sequence', found '{kind}'")


def _table(tk: _Tokens, n_times: int, n_cols: int) -> Table:
    rows = np.array([[tk.float() for _ in range(n_cols + 1)] for _ in range(n_times)], dtype=np.float64)
    return Table(rows[:, 0].copy(), rows[:, 1:].copy())


def _solution(tk: _Tokens, kind: str) -> Solution:
    tk.int()  # solution number
    keys = ("EndTime", "TimeStep", "MaxTimeStep", "MinTimeStep", "MaxIt", "MinIt", "ConvIncrease", "IncFactor",
            "Sample")
    v = {}
    for k in keys:
        tk.expect(k)
        v[k] = tk.float() if k in ("EndTime", "TimeStep", "MaxTimeStep", "MinTimeStep", "IncFactor") else tk.int()
    s = Solution(GF_STATIC if kind == "Static" else GF_DYNAMIC, 0.0, v["EndTime"], v["TimeStep"], v["MaxTimeStep"],
                 v["MinTimeStep"], v["MaxIt"], v["MinIt"], v["ConvIncrease"], v["IncFactor"], sample=v["Sample"])
    if kind == "Dynamic":
        tk.expect("RayleighDamping")
        tk.expect("Alpha")
        s.rayleigh_alpha = tk.float()
        tk.expect("Beta")
        s.rayleigh_beta = tk.float()
        tk.expect("Update")
        s.update_rayleigh = tk.int()
        tk.expect("NewmarkCoefficients")
        tk.expect("Beta")
        s.beta = tk.float()
        tk.expect("Gamma")
        s.gamma = tk.float()
        if tk.peek() == "ZeroIC":  # a bare keyword (src/Dynamic.cpp:209-216)
            tk.next()
            s.zero_ic = 1
    return s


def read_deck(text: str, step: int = None) -> Structure:
    """The structure of a deck with its solution steps: the first as
    `solution`, the others in `next_steps`, run in sequence as the
    reference's main loop does.  `step` = 1 keeps the first step alone;
    later steps on their own raise DeckError (only the first starts from the
    undeformed configuration)."""
    tk = _Tokens(text)
    steps, nodes, elems, mats, secs, shell_secs, css, pipe_secs = [], {}, [], {}, {}, {}, {}, {}
    node_sets, elem_sets, loads, disps, cons = {}, {}, [], [], []
    criteria = dict(DEFAULT_CRITERIA)
    mon_sample, mon_nodes = None, []
    while tk.more():
        kw = tk.next()
        if kw == "EOF":
            break
        if kw in SKIPPED:
            while tk.more() and tk.peek() not in TOP:
                tk.next()
            continue
        if kw == "Monitor":
            # Sample n, then MonitorNodes / MonitorElements / ... id lists;
            # the nodes are kept (their monitor files are what this library
            # writes), the other lists are read past
            tk.expect("Sample")
            mon_sample = tk.int()
            while tk.more() and (tk.peek() or "").startswith("Monitor") and tk.peek() not in TOP:
                which = tk.next()
                ids = []
                while tk.more() and (tk.peek() or "").isdigit():
                    ids.append(tk.int())
                if which == "MonitorNodes":
                    mon_nodes += ids
            continue
        if kw == "SolutionSteps":
            for _ in range(tk.int()):
                kind = tk.next()
                if kind == "Modal":
                    tk.int()
                    md = ModalStep()
                    tk.expect("ExportMatrices")
                    md.export_matrices = tk.int()
                    tk.expect("NumberModes")
                    md.number_modes = tk.int()
                    tk.expect("Tolerance")
                    md.tolerance = tk.float()
                    tk.expect("ComputeEigenvectors")
                    md.compute_eigenvectors = tk.int()
                    tk.expect("NumberFrames")
                    md.number_frames = tk.int()
                    steps.append(md)
                    continue
                if kind not in ("Static", "Dynamic"):
                    raise DeckError(f"solution type '{kind}' is not solved by this library")
                steps.append(_solution(tk, kind))
        elif kw == "Nodes":
            for _ in range(tk.int()):
                tk.expect("Node")
                i = tk.int()
                nodes[i] = (tk.float(), tk.float(), tk.float())
        elif kw == "Elements":
            for _ in range(tk.int()):
                kind = tk.next()
                eid = tk.int()
                if kind == "Beam_1":
                    tk.expect("Mat")
                    m = tk.int()
                    tk.expect("Sec")
                    sc = tk.int()
                    tk.expect("CS")
                    c = tk.int()
                    tk.expect("Nodes")
                    nd = [tk.int() for _ in range(3)]
                    t0 = 0.0
                    if tk.peek() == "PreTension":
                        tk.next()
                        t0 = tk.float()
                    elems.append(("Beam_1", eid, m, sc, c, nd, t0))
                elif kind == "Pipe_1":
                    tk.expect("PipeSec")
                    ps = tk.int()
                    tk.expect("CS")
                    c = tk.int()
                    tk.expect("Nodes")
                    nd = [tk.int() for _ in range(3)]
                    elems.append(("Pipe_1", eid, None, ps, c, nd, 0.0))
                elif kind == "Shell_1":
                    tk.expect("Mat")
                    m = tk.int()
                    tk.expect("Sec")
                    sc = tk.int()
                    c = 1
                    if tk.peek() == "CS":
                        tk.next()
                        c = tk.int()
                    tk.expect("Nodes")
                    nd = [tk.int() for _ in range(6)]
                    elems.append(("Shell_1", eid, m, sc, c, nd, 0.0))
                else:
                    raise DeckError(f"element type '{kind}' is not solved by this library")
        elif kw == "Materials":
            for _ in range(tk.int()):
                kind = tk.next()
                if kind != "Hooke":
                    raise DeckError(f"material '{kind}' is not supported")
                i = tk.int()
                tk.expect("E")
                E = tk.float()
                tk.expect("Nu")
                nu = tk.float()
                tk.expect("Rho")
                mats[i] = (E, nu, tk.float())
        elif kw == "Sections":
            for _ in range(tk.int()):
                kind = tk.next()
                i = tk.int()
                if kind == "Rectangle":
                    tk.expect("B")
                    b = tk.float()
                    tk.expect("H")
                    secs[i] = ("rect", b, tk.float())
                elif kind == "Tube":
                    tk.expect("De")
                    de = tk.float()
                    tk.expect("Di")
                    secs[i] = ("tube", de, tk.float())
                else:
                    raise DeckError(f"section '{kind}' is not supported")
        elif kw == "PipeSections":
            for _ in range(tk.int()):
                tk.expect("PS")
                i = tk.int()
                row = {}
                for name in ("EA", "EI", "GJ", "GA", "Rho", "CDt", "CDn", "CAt", "CAn", "De", "Di"):
                    tk.expect(name)
                    row[name] = tk.float()
                pipe_secs[i] = row
        elif kw == "ShellSections":
            for _ in range(tk.int()):
                kind = tk.next()
                if kind != "Homogeneous":
                    raise DeckError(f"shell section '{kind}' is not supported")
                i = tk.int()
                tk.expect("Thickness")
                shell_secs[i] = tk.float()
        elif kw == "CoordinateSystems":
            for _ in range(tk.int()):
                tk.expect("CS")
                i = tk.int()
                tk.expect("E1")
                e1 = (tk.float(), tk.float(), tk.float())
                tk.expect("E3")
                css[i] = (e1, (tk.float(), tk.float(), tk.float()))
        elif kw in ("NodeSets", "ElementSets"):
            word, item = ("NodeSet", "Nodes") if kw == "NodeSets" else ("ElementSet", "Elements")
            target = node_sets if kw == "NodeSets" else elem_sets
            for _ in range(tk.int()):
                tk.expect(word)
                i = tk.int()
                tk.expect(item)
                target[i] = _ids(tk, tk.int())
        elif kw == "Loads":
            for _ in range(tk.int()):
                kind = tk.next()
                tk.int()
                if kind == "NodalLoad":
                    tk.expect("NodeSet")
                    ns = tk.int()
                    tk.expect("CS")
                    c = tk.int()
                    if tk.next() != "NTimes":
                        raise DeckError("NodalLoad: only tabulated loads (NTimes) are supported")
                    loads.append(("nodal", ns, c, _table(tk, tk.int(), 6)))
                elif kind == "ShellLoad":
                    tk.expect("ElementSet")
                    es = tk.int()
                    tk.expect("AreaUpdate")
                    au = tk.int()
                    if tk.next() != "NTimes":
                        raise DeckError("ShellLoad: only tabulated pressures (NTimes) are supported")
                    loads.append(("shell", es, au, _table(tk, tk.int(), 1)))
                elif kind == "PipeLoad":
                    tk.expect("ElementSet")
                    es = tk.int()
                    if tk.next() != "NTimes":
                        raise DeckError("PipeLoad: only tabulated pressures (NTimes) are supported")
                    loads.append(("pipe", es, 0, _table(tk, tk.int(), 4)))
                else:
                    raise DeckError(f"load '{kind}' is not supported")
        elif kw == "Displacements":
            for _ in range(tk.int()):
                kind = tk.next()
                if kind != "NodalDisplacement":
                    raise DeckError(f"displacement '{kind}' is not supported")
                tk.int()
                tk.expect("NodeSet")
                ns = tk.int()
                tk.expect("CS")
                c = tk.int()
                ap = "EulerAngles"
                if tk.peek() == "AngularParameters":
                    tk.next()
                    ap = tk.next()
                    if ap not in ("EulerAngles", "EulerVector"):
                        raise DeckError(f"NodalDisplacement: AngularParameters '{ap}' is not supported")
                active = [True]
                if tk.peek() == "BoolTable":
                    tk.next()
                    active = tk.bool_table()
                if tk.next() != "NTimes":
                    raise DeckError("NodalDisplacement: only tabulated displacements (NTimes) are supported")
                disps.append((ns, c, active, _table(tk, tk.int(), 6), ap))
        elif kw == "Constraints":
            for _ in range(tk.int()):
                kind = tk.next()
                if kind != "NodalConstraint":
                    raise DeckError(f"constraint '{kind}' is not supported")
                tk.int()
                tk.expect("NodeSet")
                ns = tk.int()
                tables = []
                for name in DOF_NAMES:
                    tk.expect(name)
                    tk.expect("BoolTable")
                    tables.append(tk.bool_table())
                cons.append((ns, tables))
        elif kw == "ConvergenceCriteria":
            while tk.more() and tk.peek() in CRITERIA_KEYS:
                key = CRITERIA_KEYS[tk.next()]
                criteria[key] = tk.float()
        elif kw in TOP:
            # a block of another feature: an empty one is harmless
            nxt = tk.peek()
            if nxt is not None and nxt.isdigit() and int(nxt) == 0:
                tk.next()
                continue
            raise DeckError(f"block '{kw}' is not solved by this library")
        else:
            raise DeckError(f"unknown keyword '{kw}' (token {tk.i})")
    s = _build(steps, step, nodes, elems, mats, secs, shell_secs, css, node_sets, elem_sets, loads, disps, cons,
               criteria, pipe_secs)
    if mon_sample is not None:
        if any(n not in nodes for n in mon_nodes):
            raise DeckError("Monitor: a monitored node is not defined")
        s.monitor = MonitorSpec(mon_sample, [n - 1 for n in mon_nodes])
    return s


def _build(steps, step, nodes, elems, mats, secs, shell_secs, css, node_sets, elem_sets, loads, disps, cons,
           criteria, pipe_secs=None) -> Structure:
    if not steps:
        raise DeckError("the deck has no solution step")
    modal = None
    if any(isinstance(x, ModalStep) for x in steps):
        if len(steps) != 1:
            raise DeckError("a Modal step is solved only as a deck's only solution step")
        modal = steps[0]
        steps = [Solution()]
    if step is not None:
        if not 1 <= step <= len(steps):
            raise DeckError(f"the deck has {len(steps)} solution step(s), not {step}")
        if step != 1:
            raise DeckError("only the first solution step starts from the undeformed configuration")
    n_steps = len(steps) if step is None else 1
    if not nodes:
        raise DeckError("the deck has no nodes")
    ids = sorted(nodes)
    if ids != list(range(1, len(ids) + 1)):
        raise DeckError("nodes must be numbered 1..n")
    s = Structure(nodes=np.array([nodes[i] for i in ids], dtype=np.float64))
    mat_ix = {}
    for i in sorted(mats):
        mat_ix[i] = s.add_material(*mats[i])
    sec_ix = {}
    for i in sorted(secs):
        kind, x, y = secs[i]
        sec_ix[i] = s.add_rectangle(x, y) if kind == "rect" else s.add_tube(x, y)
    ssec_ix = {i: s.add_shell_section(shell_secs[i]) for i in sorted(shell_secs)}
    cs_ix = {i: s.add_cs(*css[i]) for i in sorted(css)}
    pipe_secs = pipe_secs or {}
    psec_ix = {}
    for i in sorted(pipe_secs):
        r = pipe_secs[i]
        psec_ix[i] = s.add_pipe_section(r["EA"], r["EI"], r["GJ"], r["GA"], r["Rho"], r["De"], r["Di"],
                                        r["CDt"], r["CDn"], r["CAt"], r["CAn"])

    def lookup(table, i, what):
        if i not in table:
            raise DeckError(f"{what} {i} is not defined")
        return table[i]

    shell_of, pipe_of = {}, {}
    for kind, eid, m, sc, c, nd, t0 in sorted(elems, key=lambda e: e[1]):
        if any(n not in nodes for n in nd):
            raise DeckError(f"element {eid} refers to a missing node")
        if kind == "Pipe_1":
            pipe_of[eid] = s.add_pipe(nd[0] - 1, nd[1] - 1, nd[2] - 1, lookup(psec_ix, sc, "pipe section"),
                                      lookup(cs_ix, c, "coordinate system"))
        elif kind == "Beam_1":
            if t0 != 0.0:
                s.pretension[len(s.beams)] = t0
            s.beams.append((nd[0] - 1, nd[1] - 1, nd[2] - 1, lookup(mat_ix, m, "material"),
                            lookup(sec_ix, sc, "section"), lookup(cs_ix, c, "coordinate system")))
        else:
            shell_of[eid] = len(s.shells)
            s.shells.append((*[n - 1 for n in nd], lookup(mat_ix, m, "material"),
                             lookup(ssec_ix, sc, "shell section"), cs_ix.get(c, 0)))
    for ns, tables in cons:
        mask = [1 if _step_value(t, 1) else 0 for t in tables]
        if any([1 if _step_value(t, k) else 0 for t in tables] != mask for k in range(2, n_steps + 1)):
            raise DeckError(f"NodalConstraint on node set {ns}: constraints that change between solution steps "
                            "are not supported")
        for n in lookup(node_sets, ns, "node set"):
            s.clamp(n - 1, mask)
    for ld in loads:
        if ld[0] == "nodal":
            _, ns, c, table = ld
            s.loads.append(NodalLoad([n - 1 for n in lookup(node_sets, ns, "node set")],
                                     lookup(cs_ix, c, "coordinate system"), table))
        elif ld[0] == "pipe":
            _, es, _, table = ld
            members = lookup(elem_sets, es, "element set")
            if any(e not in pipe_of for e in members):
                raise DeckError(f"PipeLoad on element set {es}: every element must be a Pipe_1")
            s.loads.append(PipeLoad([pipe_of[e] for e in members], table))
        else:
            _, es, au, table = ld
            members = lookup(elem_sets, es, "element set")
            if any(e not in shell_of for e in members):
                raise DeckError(f"ShellLoad on element set {es}: every element must be a Shell_1")
            s.loads.append(PressureLoad([shell_of[e] for e in members], table, area_update=au))
    for ns, c, active, table, ap in disps:
        on = [_step_value(active, k) for k in range(1, n_steps + 1)]
        if any(x != on[0] for x in on):
            raise DeckError(f"NodalDisplacement on node set {ns}: displacements active in some solution steps "
                            "only are not supported")
        if on[0]:
            s.displacements.append(NodalDisplacement([n - 1 for n in lookup(node_sets, ns, "node set")],
                                                     lookup(cs_ix, c, "coordinate system"), table, ap))
    start = 0.0  # each step starts where the previous one ends (src/Database.cpp:759-768)
    for so in steps[:n_steps]:
        so.start_time = start
        start = so.end_time
    s.solution = steps[0]
    s.next_steps = list(steps[1:n_steps])
    s.criteria = dict(criteria)
    s.modal = modal
    return s


def read_deck_file(path: str, step: int = None) -> Structure:
    with open(path, encoding="latin-1") as f:
        return read_deck(f.read(), step)

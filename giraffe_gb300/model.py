"""Structures for the implicit Beam_1 / Shell_1 path.

A :class:`Structure` holds what a GIRAFFE input deck holds for this path
(nodes, Hooke materials, sections, coordinate systems, Beam_1 / Shell_1
elements, nodal constraints, nodal loads, shell pressure loads, prescribed
nodal displacements, a sequence of Static and Dynamic solution steps and the
convergence criteria; reference src/IO.cpp:288-657).  It can

* produce the flat C description ``gf_model_desc`` (include/giraffe_model.h)
  that both the CUDA library and the CPU oracle take, and
* write itself as a deck in the reference's .inp syntax, which is how the
  golden fixtures are generated from the reference build.

Indices are 0-based here and 1-based in decks.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

PI = 3.1415926535897932384626433832795

GF_STATIC, GF_DYNAMIC = 0, 1
GF_LOAD_NODAL, GF_LOAD_SHELL_PRESSURE, GF_LOAD_PIPE_PRESSURE = 0, 1, 2


# --------------------------------------------------------------------------
# sections (reference src/SecRectangle.cpp:82-107, src/SecTube.cpp:86-106)
# --------------------------------------------------------------------------
def section_rectangle(b: float, h: float) -> tuple:
    A = b * h
    I11 = b * h * h * h / 12.0
    I22 = h * b * b * b / 12.0
    temp = 0.0
    for n in range(1, 22, 2):
        temp += (1.0 / (float(n) ** 5)) * math.tanh(n * PI * h / (2 * b))
    It = (1.0 / 3.0) * b * b * b * h * (1.0 - 192.0 * b * temp / (PI ** 5 * h))
    return (A, I11, I22, 0.0, It, I11 + I22)


def section_tube(De: float, Di: float) -> tuple:
    A = (PI / 4.0) * (De * De - Di * Di)
    I11 = (PI / 64.0) * (De ** 4 - Di ** 4)
    I33 = (PI / 32.0) * (De ** 4 - Di ** 4)
    return (A, I11, I11, 0.0, I33, I33)


# --------------------------------------------------------------------------
# ctypes mirror of include/giraffe_model.h
# --------------------------------------------------------------------------
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


# Pointer members are declared as void* here (same size and alignment as the
# typed pointers of the C header) so that numpy buffer addresses are stored
# without a ctypes pointer object per array.
_vp = C.c_void_p


class gf_table(C.Structure):
    _fields_ = [("n_times", C.c_int), ("n_cols", C.c_int), ("times", _vp), ("values", _vp)]


class gf_load(C.Structure):
    _fields_ = [("type", C.c_int), ("n_items", C.c_int), ("items", _vp), ("cs", C.c_int),
                ("area_update", C.c_int), ("table", gf_table)]


class gf_displacement(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("nodes", _vp), ("cs", C.c_int), ("table", gf_table), ("angular", C.c_int)]


class gf_solution(C.Structure):
    _fields_ = [("type", C.c_int), ("start_time", C.c_double), ("end_time", C.c_double),
                ("time_step", C.c_double), ("max_time_step", C.c_double),
                ("min_time_step", C.c_double), ("max_it", C.c_int), ("min_it", C.c_int),
                ("conv_increase", C.c_int), ("inc_factor", C.c_double), ("beta", C.c_double),
                ("gamma", C.c_double), ("rayleigh_alpha", C.c_double),
                ("rayleigh_beta", C.c_double), ("update_rayleigh", C.c_int), ("zero_ic", C.c_int)]


class gf_criteria(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "force_tol", "moment_tol", "force_min", "moment_min", "constraint_min", "disp_tol",
        "rot_tol", "lag_tol", "disp_min", "rot_min", "lag_min", "divergence_ref")]


class gf_model_desc(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("node_xyz", _vp),
                ("n_materials", C.c_int), ("materials", _vp),
                ("n_sections", C.c_int), ("sections", _vp),
                ("n_shell_sections", C.c_int), ("shell_sections", _vp),
                ("n_cs", C.c_int), ("cs", _vp),
                ("n_beams", C.c_int), ("beams", _vp),
                ("n_shells", C.c_int), ("shells", _vp),
                ("constraints", _vp),
                ("n_loads", C.c_int), ("loads", _vp),
                ("n_displacements", C.c_int), ("displacements", _vp),
                ("solution", gf_solution), ("criteria", gf_criteria), ("beam_pretension", _vp),
                ("n_next_steps", C.c_int), ("next_steps", _vp),
                ("n_pipe_sections", C.c_int), ("pipe_sections", _vp), ("beam_pipe_section", _vp),
                ("n_monitor_nodes", C.c_int), ("monitor_nodes", _vp), ("monitor_sample", C.c_int)]


def _r(v):
    return repr(float(v))


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a, t=None):
    """Address of a numpy buffer for a void* member (None when empty)."""
    return a.__array_interface__["data"][0] if a is not None and a.size else None


class ElementTable:
    """Element rows (node indices, then material, section and frame indices)
    kept in one growing int32 array, so that handing a structure to the C ABI
    passes that array as it is.  Behaves as a list of tuples: append, extend,
    indexing, assignment of a row, iteration, len."""

    def __init__(self, width: int, rows=()):
        self.width = width
        self._a = np.zeros((16, width), dtype=np.int32)
        self._n = 0
        self.extend(rows)

    def _reserve(self, n):
        if n > len(self._a):
            a = np.zeros((max(n, 2 * len(self._a)), self.width), dtype=np.int32)
            a[:self._n] = self._a[:self._n]
            self._a = a

    def append(self, row):
        self._reserve(self._n + 1)
        self._a[self._n] = row
        self._n += 1

    def extend(self, rows):
        rows = np.asarray(rows if not isinstance(rows, ElementTable) else rows.array(), dtype=np.int32)
        if rows.size == 0:
            return
        rows = rows.reshape(-1, self.width)
        self._reserve(self._n + len(rows))
        self._a[self._n:self._n + len(rows)] = rows
        self._n += len(rows)

    def array(self) -> np.ndarray:
        """The rows as an [n][width] int32 view (no copy)."""
        return self._a[:self._n]

    def __len__(self):
        return self._n

    def __bool__(self):
        return self._n > 0

    def __iter__(self):
        return iter([tuple(r) for r in self.array().tolist()])

    def __getitem__(self, k):
        if isinstance(k, slice):
            return [tuple(r) for r in self.array()[k].tolist()]
        return tuple(self.array()[k].tolist())

    def __setitem__(self, k, row):
        self.array()[k] = row

    def __eq__(self, other):
        return list(self) == list(other)

    def __repr__(self):
        return f"ElementTable({list(self)!r})"


# --------------------------------------------------------------------------
@dataclass
class Table:
    times: np.ndarray
    values: np.ndarray  # [n_times][n_cols]


@dataclass
class NodalLoad:
    nodes: list
    cs: int
    table: Table


@dataclass
class PressureLoad:
    shells: list
    table: Table
    area_update: int = 1


@dataclass
class PipeLoad:
    """PipeLoad (reference src/PipeLoad.cpp): pressure on Pipe_1 elements
    (beam indices); table columns P0I P0E RhoI RhoE, of which the internal
    pressure P0I acts on the section's internal area."""
    pipes: list
    table: Table


@dataclass
class NodalDisplacement:
    nodes: list
    cs: int
    table: Table
    angular: str = "EulerAngles"  # or "EulerVector": how the rotation columns are read


@dataclass
class MonitorSpec:
    """A deck's Monitor block (reference src/Monitor.cpp:112-195): the nodes
    whose state is written after every `sample`-th converged step (and at a
    solution step's end)."""
    sample: int = 1
    nodes: list = field(default_factory=list)  # 0-based node indices


@dataclass
class ModalStep:
    """A Modal solution step (reference src/Modal.cpp:42-108): the
    number_modes smallest eigenvalues of K x = lambda M x at the structure's
    start, by shift-invert with shift 0 (src/SparseMatrix.cpp:270-)."""
    number_modes: int = 10
    tolerance: float = 1e-6
    export_matrices: int = 0
    compute_eigenvectors: int = 0
    number_frames: int = 0


@dataclass
class Solution:
    type: int = GF_STATIC
    start_time: float = 0.0
    end_time: float = 1.0
    time_step: float = 0.1
    max_time_step: float = 0.1
    min_time_step: float = 1e-4
    max_it: int = 20
    min_it: int = 3
    conv_increase: int = 4
    inc_factor: float = 1.0
    sample: int = 1
    beta: float = 0.3
    gamma: float = 0.5
    rayleigh_alpha: float = 0.0
    rayleigh_beta: float = 0.0
    update_rayleigh: int = 0
    zero_ic: int = 0          # Dynamic: ZeroIC


# reference src/ConvergenceCriteria.cpp:15-60
DEFAULT_CRITERIA = dict(force_tol=1e-4, moment_tol=1e-4, force_min=1e-5, moment_min=1e-5,
                        constraint_min=1e-7, disp_tol=1e-4, rot_tol=1e-4, lag_tol=1e-4,
                        disp_min=1e-6, rot_min=1e-6, lag_min=1e-6, divergence_ref=1e15)


@dataclass
class Structure:
    nodes: np.ndarray                        # [n][3]
    materials: list = field(default_factory=list)      # (E, nu, rho)
    sections: list = field(default_factory=list)       # (A, I11, I22, I12, It, I33)
    section_decks: list = field(default_factory=list)  # deck text of each section
    shell_sections: list = field(default_factory=list)  # thickness
    cs: list = field(default_factory=list)             # (E1 xyz, E3 xyz)
    beams: ElementTable = field(default_factory=lambda: ElementTable(6))   # (n0, n1, n2, mat, sec, cs)
    shells: ElementTable = field(default_factory=lambda: ElementTable(9))  # (6 nodes, mat, shell sec, cs)
    constraints: np.ndarray | None = None              # [n][6] 0/1
    loads: list = field(default_factory=list)
    displacements: list = field(default_factory=list)
    solution: Solution = field(default_factory=Solution)
    next_steps: list = field(default_factory=list)     # Solution steps run after `solution`
    criteria: dict = field(default_factory=lambda: dict(DEFAULT_CRITERIA))
    pretension: dict = field(default_factory=dict)     # beam index -> Beam_1 PreTension T0
    # Pipe_1: PipeSection rows (EA, EI, GJ, GA, Rho, CDt, CDn, CAt, CAn, De, Di)
    # and the pipe section of each beam that is a Pipe_1 element
    pipe_sections: list = field(default_factory=list)
    pipe_of: dict = field(default_factory=dict)        # beam index -> pipe section
    modal: ModalStep | None = None                     # a deck whose step is Modal
    monitor: MonitorSpec | None = None                 # the deck's monitored nodes

    def __setattr__(self, name, value):
        # element rows assigned as lists become ElementTables
        if name in ("beams", "shells") and not isinstance(value, ElementTable):
            value = ElementTable(6 if name == "beams" else 9, value)
        object.__setattr__(self, name, value)

    # ---- building helpers ----
    def add_material(self, E, nu, rho):
        self.materials.append((float(E), float(nu), float(rho)))
        return len(self.materials) - 1

    def add_rectangle(self, b, h):
        self.sections.append(section_rectangle(b, h))
        self.section_decks.append(f"Rectangle\t{len(self.sections)}\tB\t{_r(b)}\tH\t{_r(h)}")
        return len(self.sections) - 1

    def add_tube(self, De, Di):
        self.sections.append(section_tube(De, Di))
        self.section_decks.append(f"Tube\t{len(self.sections)}\tDe\t{_r(De)}\tDi\t{_r(Di)}")
        return len(self.sections) - 1

    def add_pipe_section(self, EA, EI, GJ, GA, Rho, De, Di, CDt=0.0, CDn=0.0, CAt=0.0, CAn=0.0):
        self.pipe_sections.append(tuple(float(v) for v in (EA, EI, GJ, GA, Rho, CDt, CDn, CAt, CAn, De, Di)))
        return len(self.pipe_sections) - 1

    def add_pipe(self, n0, n1, n2, pipe_section, cs):
        """A Pipe_1 element: Beam_1 kinematics with the pipe section's
        stiffness and mass; its material and section columns are -1."""
        self.pipe_of[len(self.beams)] = int(pipe_section)
        self.beams.append((n0, n1, n2, -1, -1, cs))
        return len(self.beams) - 1

    def add_shell_section(self, thickness):
        self.shell_sections.append(float(thickness))
        return len(self.shell_sections) - 1

    def add_cs(self, e1, e3):
        self.cs.append(tuple(float(v) for v in (*e1, *e3)))
        return len(self.cs) - 1

    def clamp(self, node, mask=(1, 1, 1, 1, 1, 1)):
        if self.constraints is None:
            self.constraints = np.zeros((len(self.nodes), 6), dtype=np.int32)
        self.constraints[node] = np.maximum(self.constraints[node], mask)

    @property
    def n_nodes(self):
        return len(self.nodes)

    @property
    def n_free(self):
        active = np.zeros((self.n_nodes, 6), dtype=bool)
        active[self.beams.array()[:, :3].ravel()] = True
        active[self.shells.array()[:, :3].ravel(), :3] = True
        active[self.shells.array()[:, 3:6].ravel()] = True
        cons = self.constraints if self.constraints is not None else 0
        return int((active & (cons == 0)).sum())

    # ---- C description ----
    def desc(self) -> "DescHandle":
        return DescHandle(self)

    # ---- deck in the reference's syntax ----
    @staticmethod
    def from_inp(text: str, step: int = None) -> "Structure":
        """The structure and solution steps of a deck in the reference's .inp
        syntax (giraffe_gb300.deck.read_deck)."""
        from .deck import read_deck
        return read_deck(text, step)

    def to_inp(self) -> str:
        o = []
        steps = [self.solution] + list(self.next_steps)
        if self.modal is not None:
            md = self.modal
            o.append(f"SolutionSteps\t1\nModal\t1\nExportMatrices\t{int(md.export_matrices)}\n"
                     f"NumberModes\t{int(md.number_modes)}\nTolerance\t{_r(md.tolerance)}\n"
                     f"ComputeEigenvectors\t{int(md.compute_eigenvectors)}\nNumberFrames\t{int(md.number_frames)}")
            steps = []
        else:
            o.append(f"SolutionSteps\t{len(steps)}")
        for k, s in enumerate(steps, 1):
            if s.type == GF_STATIC:
                o.append(f"Static\t{k}\nEndTime\t{_r(s.end_time)}\nTimeStep\t{_r(s.time_step)}\n"
                         f"MaxTimeStep\t{_r(s.max_time_step)}\nMinTimeStep\t{_r(s.min_time_step)}\n"
                         f"MaxIt\t{s.max_it}\nMinIt\t{s.min_it}\nConvIncrease\t{s.conv_increase}\n"
                         f"IncFactor\t{_r(s.inc_factor)}\nSample\t{s.sample}")
            else:
                o.append(f"Dynamic\t{k}\nEndTime\t{_r(s.end_time)}\nTimeStep\t{_r(s.time_step)}\n"
                         f"MaxTimeStep\t{_r(s.max_time_step)}\nMinTimeStep\t{_r(s.min_time_step)}\n"
                         f"MaxIt\t{s.max_it}\nMinIt\t{s.min_it}\nConvIncrease\t{s.conv_increase}\n"
                         f"IncFactor\t{_r(s.inc_factor)}\nSample\t{s.sample}\n"
                         f"RayleighDamping\tAlpha\t{_r(s.rayleigh_alpha)}\tBeta\t{_r(s.rayleigh_beta)}"
                         f"\tUpdate\t{s.update_rayleigh}\n"
                         f"NewmarkCoefficients\tBeta\t{_r(s.beta)}\tGamma\t{_r(s.gamma)}"
                         + ("\nZeroIC" if s.zero_ic else ""))
        o.append(f"Nodes\t{self.n_nodes}")
        for i, x in enumerate(np.asarray(self.nodes, dtype=np.float64)):
            o.append(f"Node\t{i + 1}\t{_r(x[0])}\t{_r(x[1])}\t{_r(x[2])}")
        o.append(f"Elements\t{len(self.beams) + len(self.shells)}")
        k = 0
        for e, b in enumerate(self.beams):
            k += 1
            if e in self.pipe_of:
                o.append(f"Pipe_1\t{k}\tPipeSec\t{self.pipe_of[e] + 1}\tCS\t{b[5] + 1}\tNodes\t"
                         f"{b[0] + 1}\t{b[1] + 1}\t{b[2] + 1}")
                continue
            t0 = float(self.pretension.get(e, 0.0))
            o.append(f"Beam_1\t{k}\tMat\t{b[3] + 1}\tSec\t{b[4] + 1}\tCS\t{b[5] + 1}\tNodes\t"
                     f"{b[0] + 1}\t{b[1] + 1}\t{b[2] + 1}" + (f"\tPreTension\t{_r(t0)}" if t0 != 0.0 else ""))
        for sh in self.shells:
            k += 1
            nodes = "\t".join(str(v + 1) for v in sh[:6])
            o.append(f"Shell_1\t{k}\tMat\t{sh[6] + 1}\tSec\t{sh[7] + 1}\tCS\t{sh[8] + 1}\tNodes\t{nodes}")
        if self.materials:
            o.append(f"Materials\t{len(self.materials)}")
        for i, (E, nu, rho) in enumerate(self.materials):
            o.append(f"Hooke\t{i + 1}\tE\t{_r(E)}\tNu\t{_r(nu)}\tRho\t{_r(rho)}")
        if self.sections:
            o.append(f"Sections\t{len(self.section_decks)}")
            o.extend(self.section_decks)
        if self.pipe_sections:
            o.append(f"PipeSections\t{len(self.pipe_sections)}")
            names = ("EA", "EI", "GJ", "GA", "Rho", "CDt", "CDn", "CAt", "CAn", "De", "Di")
            for i, row in enumerate(self.pipe_sections):
                o.append(f"PS\t{i + 1}\t" + "\t".join(f"{n}\t{_r(v)}" for n, v in zip(names, row)))
        if self.shell_sections:
            o.append(f"ShellSections\t{len(self.shell_sections)}")
            for i, t in enumerate(self.shell_sections):
                o.append(f"Homogeneous\t{i + 1}\tThickness\t{_r(t)}")
        o.append(f"CoordinateSystems\t{len(self.cs)}")
        for i, c in enumerate(self.cs):
            o.append(f"CS\t{i + 1}\tE1\t{_r(c[0])}\t{_r(c[1])}\t{_r(c[2])}\tE3\t{_r(c[3])}\t{_r(c[4])}\t{_r(c[5])}")
        # node sets: one per constrained node group, load and displacement
        sets, elem_sets, cons_lines, load_lines, disp_lines = [], [], [], [], []

        def new_set(nodes):
            sets.append(list(nodes))
            return len(sets)

        if self.constraints is not None:
            groups = {}
            for i, row in enumerate(self.constraints):
                if row.any():
                    groups.setdefault(tuple(int(v) for v in row), []).append(i)
            for mask, nodes in groups.items():
                ns = new_set(nodes)
                names = ("UX", "UY", "UZ", "ROTX", "ROTY", "ROTZ")
                body = "\n".join(f"\t{n}\tBoolTable\t{v}" for n, v in zip(names, mask))
                cons_lines.append(f"NodalConstraint\t{len(cons_lines) + 1}\tNodeSet\t{ns}\n{body}")
        for L in self.loads:
            if isinstance(L, NodalLoad):
                ns = new_set(L.nodes)
                rows = "\n".join("\t".join(repr(float(v)) for v in (t, *vals))
                                 for t, vals in zip(L.table.times, L.table.values))
                load_lines.append(f"NodalLoad\t{len(load_lines) + 1}\tNodeSet\t{ns}\tCS\t{L.cs + 1}"
                                  f"\tNTimes\t{len(L.table.times)}\n{rows}")
            elif isinstance(L, PipeLoad):
                rows = "\n".join("\t".join(repr(float(v)) for v in (t, *vals))
                                  for t, vals in zip(L.table.times, L.table.values))
                elem_sets.append(list(L.pipes))
                load_lines.append(f"PipeLoad\t{len(load_lines) + 1}\tElementSet\t{len(elem_sets)}"
                                  f"\tNTimes\t{len(L.table.times)}\n{rows}")
            else:
                rows = "\n".join(f"{_r(float(t))}\t{_r(float(v[0]))}"
                                 for t, v in zip(L.table.times, L.table.values))
                elem_sets.append([len(self.beams) + e for e in L.shells])
                load_lines.append(f"ShellLoad\t{len(load_lines) + 1}\tElementSet\t{len(elem_sets)}"
                                  f"\tAreaUpdate\t{int(L.area_update)}\tNTimes\t{len(L.table.times)}\n{rows}")
        for D in self.displacements:
            ns = new_set(D.nodes)
            rows = "\n".join("\t".join(repr(float(v)) for v in (t, *vals))
                             for t, vals in zip(D.table.times, D.table.values))
            disp_lines.append(f"NodalDisplacement\t{len(disp_lines) + 1}\tNodeSet\t{ns}\tCS\t{D.cs + 1}"
                              f"\tAngularParameters\t{D.angular}\tNTimes\t{len(D.table.times)}\n{rows}")
        if sets:
            o.append(f"NodeSets\t{len(sets)}")
            for i, nodes in enumerate(sets):
                o.append(f"NodeSet\t{i + 1}\tNodes\t{len(nodes)}\tList\t" +
                         "\t".join(str(n + 1) for n in nodes))
        if elem_sets:
            o.append(f"ElementSets\t{len(elem_sets)}")
            for i, els in enumerate(elem_sets):
                o.append(f"ElementSet\t{i + 1}\tElements\t{len(els)}\tList\t" +
                         "\t".join(str(e + 1) for e in els))
        if load_lines:
            o.append(f"Loads\t{len(load_lines)}")
            o.extend(load_lines)
        if disp_lines:
            o.append(f"Displacements\t{len(disp_lines)}")
            o.extend(disp_lines)
        if cons_lines:
            o.append(f"Constraints\t{len(cons_lines)}")
            o.extend(cons_lines)
        if self.monitor is not None:
            o.append(f"Monitor\tSample\t{int(self.monitor.sample)}" +
                     ("\nMonitorNodes\t" + "\t".join(str(int(n) + 1) for n in self.monitor.nodes)
                      if self.monitor.nodes else ""))
        c = self.criteria
        o.append("ConvergenceCriteria\n"
                 f"ForceTolerance\t{_r(c['force_tol'])}\nMomentTolerance\t{_r(c['moment_tol'])}\n"
                 f"ForceMinimumReference\t{_r(c['force_min'])}\nMomentMinimumReference\t{_r(c['moment_min'])}\n"
                 f"ConstraintMinimumReference\t{_r(c['constraint_min'])}\n"
                 f"DisplacementTolerance\t{_r(c['disp_tol'])}\nRotationTolerance\t{_r(c['rot_tol'])}\n"
                 f"LagrangeTolerance\t{_r(c['lag_tol'])}\n"
                 f"DisplacementMinimumReference\t{_r(c['disp_min'])}\n"
                 f"RotationMinimumReference\t{_r(c['rot_min'])}\n"
                 f"LagrangeMinimumReference\t{_r(c['lag_min'])}\n"
                 f"DivergenceReference\t{_r(c['divergence_ref'])}")
        o.append("SolverOptions\nProcessors\t1\tLinSys\tDirect")
        return "\n".join(o) + "\n"


class DescHandle:
    """Owns the numpy buffers behind one ``gf_model_desc``."""

    def __init__(self, s: Structure):
        self.keep = []

        def d(a):
            a = _d(a)
            self.keep.append(a)
            return a

        def i(a):
            a = _i(a)
            self.keep.append(a)
            return a

        nodes = d(np.asarray(s.nodes, dtype=np.float64).reshape(-1, 3))
        mats = d(np.asarray(s.materials, dtype=np.float64).reshape(-1, 3))
        secs = d(np.asarray(s.sections, dtype=np.float64).reshape(-1, 6))
        ssec = d(np.asarray(s.shell_sections, dtype=np.float64).reshape(-1, 1))
        cs = d(np.asarray(s.cs, dtype=np.float64).reshape(-1, 6))
        beams = i(s.beams.array())
        shells = i(s.shells.array())
        cons = i(s.constraints) if s.constraints is not None else None
        loads = (gf_load * max(1, len(s.loads)))()
        for k, L in enumerate(s.loads):
            kind = (GF_LOAD_NODAL if isinstance(L, NodalLoad) else
                    GF_LOAD_PIPE_PRESSURE if isinstance(L, PipeLoad) else GF_LOAD_SHELL_PRESSURE)
            items = i(np.asarray(L.nodes if kind == GF_LOAD_NODAL else
                                 L.pipes if kind == GF_LOAD_PIPE_PRESSURE else L.shells))
            tt = d(L.table.times)
            tv = d(np.asarray(L.table.values, dtype=np.float64).reshape(len(tt), -1))
            loads[k].type = kind
            loads[k].n_items = len(items)
            loads[k].items = _ptr(items, _ip)
            loads[k].cs = L.cs if isinstance(L, NodalLoad) else 0
            loads[k].area_update = getattr(L, "area_update", 0)
            loads[k].table = gf_table(len(tt), tv.shape[1], _ptr(tt, _dp), _ptr(tv, _dp))
        disps = (gf_displacement * max(1, len(s.displacements)))()
        for k, D in enumerate(s.displacements):
            nd = i(np.asarray(D.nodes))
            tt = d(D.table.times)
            tv = d(np.asarray(D.table.values, dtype=np.float64).reshape(len(tt), -1))
            disps[k].n_nodes = len(nd)
            disps[k].nodes = _ptr(nd, _ip)
            disps[k].cs = D.cs
            disps[k].angular = 1 if D.angular == "EulerVector" else 0
            disps[k].table = gf_table(len(tt), tv.shape[1], _ptr(tt, _dp), _ptr(tv, _dp))
        self.keep += [loads, disps]
        def csol(so):
            return gf_solution(so.type, so.start_time, so.end_time, so.time_step, so.max_time_step,
                               so.min_time_step, so.max_it, so.min_it, so.conv_increase, so.inc_factor,
                               so.beta, so.gamma, so.rayleigh_alpha, so.rayleigh_beta, so.update_rayleigh,
                               int(so.zero_ic))

        sol = csol(s.solution)
        nxt = (gf_solution * max(1, len(s.next_steps)))(*[csol(so) for so in s.next_steps])
        self.keep.append(nxt)
        crit = gf_criteria(**{k: float(v) for k, v in s.criteria.items()})
        pre = None
        if s.pretension:
            pre = np.zeros(max(1, len(s.beams)))
            for e, t0 in s.pretension.items():
                pre[int(e)] = float(t0)
            self.keep.append(pre)
        psec, bps = None, None
        if s.pipe_of:
            psec = d(np.asarray(s.pipe_sections, dtype=np.float64).reshape(-1, 11))
            bps = np.full(max(1, len(s.beams)), -1, dtype=np.int32)
            for e, p in s.pipe_of.items():
                bps[int(e)] = int(p)
            self.keep.append(bps)
        mon_nodes = i(np.asarray(s.monitor.nodes)) if s.monitor is not None and s.monitor.nodes else None
        self.desc = gf_model_desc(
            len(nodes), _ptr(nodes, _dp), len(mats), _ptr(mats, _dp), len(secs), _ptr(secs, _dp),
            len(ssec), _ptr(ssec, _dp), len(cs), _ptr(cs, _dp), len(beams), _ptr(beams, _ip),
            len(shells), _ptr(shells, _ip), _ptr(cons, _ip), len(s.loads), C.addressof(loads),
            len(s.displacements), C.addressof(disps), sol, crit, _ptr(pre), len(s.next_steps),
            C.addressof(nxt) if s.next_steps else None,
            len(psec) if psec is not None else 0, _ptr(psec, _dp), _ptr(bps, _ip),
            len(mon_nodes) if mon_nodes is not None else 0, _ptr(mon_nodes, _ip),
            int(s.monitor.sample) if s.monitor is not None else 1)

    @property
    def ref(self):
        return C.byref(self.desc)

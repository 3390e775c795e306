"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE: the values the CUDA path is tested against and the
timed CPU baseline; never used by
the product path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle.build())
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        _lib.oracle_solve.argtypes = [C.c_void_p, C.c_void_p, dp, ip]
        _lib.oracle_solve_batch.argtypes = [C.c_int, C.c_void_p, C.POINTER(dp), ip, C.c_int]
        _lib.oracle_beam_element.argtypes = [dp, dp, dp, dp, C.c_int, dp, dp, dp, dp]
        _lib.oracle_first_tangent.argtypes = [C.c_void_p, dp, dp, ip]
        _lib.oracle_modal_matrices.argtypes = [C.c_void_p, dp, dp, ip]
        _lib.oracle_pipe_element.argtypes = [dp, dp, dp, C.c_int, dp, dp, C.c_double, dp, dp]
        _lib.oracle_shell_element.argtypes = [dp, dp, C.c_double, C.c_int, dp, dp, C.c_int, C.c_double, C.c_int,
                                              dp, dp]
        _lib.oracle_beam_inertia_element.argtypes = [dp, dp, dp, dp, C.c_int, dp, dp, dp, dp, C.c_double, C.c_double,
                                                     C.c_double, dp, dp, dp]
        _lib.oracle_shell_inertia_element.argtypes = [dp, dp, C.c_double, C.c_int, dp, dp, dp, dp, C.c_double,
                                                      C.c_double, C.c_double, dp, dp, dp]
    return _lib


class Record(C.Structure):
    _fields_ = [("cap", C.c_int), ("n", C.c_int), ("time", C.POINTER(C.c_double)),
                ("iterations", C.POINTER(C.c_int)), ("nodes", C.POINTER(C.c_double)),
                ("gp_Q", C.POINTER(C.c_double)), ("mon_n", C.c_int), ("mon_nodes", C.POINTER(C.c_int)),
                ("mon_sample", C.c_int), ("mon_cap", C.c_int), ("mon_rows", C.c_int),
                ("monitor", C.POINTER(C.c_double))]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def solve(structure, record_cap: int = 0):
    """Runs one structure.  Returns (final nodes [n_nodes x 15], stats
    [converged steps, Newton iterations, bisections, aborted], record dict)."""
    h = structure.desc()
    final = np.zeros((structure.n_nodes, 15))
    stats = (C.c_int * 4)()
    rec = None
    rd = None
    mon = structure.monitor if getattr(structure, "monitor", None) is not None else None
    if record_cap:
        t = np.zeros(record_cap)
        it = np.zeros(record_cap, np.int32)
        nodes = np.zeros((record_cap, structure.n_nodes, 15))
        gq = np.zeros((record_cap, max(1, len(structure.beams)), 2, 9))
        mon_nodes = np.asarray(mon.nodes if mon else [0], dtype=np.int32)
        mon_rows = np.zeros((record_cap + 1, max(1, len(mon_nodes)), 31))
        rec = Record(record_cap, 0, _dp(t), it.ctypes.data_as(C.POINTER(C.c_int)), _dp(nodes), _dp(gq),
                     len(mon.nodes) if mon else 0, mon_nodes.ctypes.data_as(C.POINTER(C.c_int)),
                     int(mon.sample) if mon else 1, record_cap + 1, 0, _dp(mon_rows))
    if lib().oracle_solve(C.cast(h.ref, C.c_void_p), C.byref(rec) if rec else None, _dp(final), stats) < 0:
        raise ValueError("oracle: invalid structure description")
    if rec:
        n = rec.n
        rd = dict(time=t[:n], iterations=it[:n], nodes=nodes[:n], gp_Q=gq[:n])
        if mon and mon.nodes:
            # [node][row][31], as the reference writes one file per node
            rd["monitor"] = np.transpose(mon_rows[:rec.mon_rows], (1, 0, 2)).copy()
    return final, np.array(list(stats)), rd


def solve_batch(structures, threads: int = 1):
    hs = [s.desc() for s in structures]
    from giraffe_gb300.model import gf_model_desc
    arr = (gf_model_desc * len(hs))(*[h.desc for h in hs])
    finals = [np.zeros((s.n_nodes, 15)) for s in structures]
    ptrs = (C.POINTER(C.c_double) * len(finals))(*[_dp(f) for f in finals])
    stats = np.zeros((len(hs), 4), np.int32)
    fails = lib().oracle_solve_batch(len(hs), C.cast(arr, C.c_void_p), ptrs,
                                     stats.ctypes.data_as(C.POINTER(C.c_int)), threads)
    return finals, stats, fails


def beam_element(xyz9, mat3, sec6, cs6, hist_disp, disp18):
    K = np.zeros(324)
    f = np.zeros(18)
    hd = np.ascontiguousarray(hist_disp if hist_disp is not None and len(hist_disp) else np.zeros((1, 18)),
                              dtype=np.float64)
    nh = 0 if hist_disp is None else len(hist_disp)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz9, mat3, sec6, cs6, disp18)]
    lib().oracle_beam_element(_dp(args[0]), _dp(args[1]), _dp(args[2]), _dp(args[3]), nh, _dp(hd),
                              _dp(args[4]), _dp(K), _dp(f))
    return K.reshape(18, 18).T, f  # row-major [r][s]


def _gb_dense(ab, kl):
    """Dense n x n of GB storage [n][3 kl + 1] (entry (i, j) at ab[j][2 kl + i - j])."""
    n = ab.shape[0]
    A = np.zeros((n, n))
    for j in range(n):
        i0, i1 = max(0, j - kl), min(n, j + kl + 1)
        A[i0:i1, j] = ab[j, 2 * kl + np.arange(i0, i1) - j]
    return A


def modal_matrices(structure):
    """K_AA and M_AA of a Modal step at the structure's start (dense, the
    reference's numbering): oracle_modal_matrices."""
    h = structure.desc()
    dims = (C.c_int * 2)()
    if lib().oracle_modal_matrices(C.cast(h.ref, C.c_void_p), None, None, dims) < 0:
        raise ValueError("oracle: invalid structure description")
    n, kl = dims[0], dims[1]
    K = np.zeros((n, 3 * kl + 1))
    M = np.zeros((n, 3 * kl + 1))
    lib().oracle_modal_matrices(C.cast(h.ref, C.c_void_p), _dp(K), _dp(M), dims)
    return _gb_dense(K, kl), _gb_dense(M, kl)


def modal(structure, n_modes: int):
    """The n_modes smallest eigenvalues of K x = lambda M x (Modal::Solve's
    shift-invert problem with sigma 0), by LAPACK's symmetric-definite
    generalized solver on the assembled matrices, and the M-normalized
    modes (columns, the reference's numbering)."""
    import scipy.linalg
    K, M = modal_matrices(structure)
    w, V = scipy.linalg.eigh(K, M, subset_by_index=[0, n_modes - 1])
    return w, V


def pipe_element(xyz9, ps11, cs6, hist_disp, disp18, p0i=0.0):
    """One Pipe_1 element with an internal pressure p0i
    (oracle_pipe_element): K row-major [r][s], f."""
    K = np.zeros(324)
    f = np.zeros(18)
    nh = 0 if hist_disp is None else len(hist_disp)
    hd = np.ascontiguousarray(hist_disp if nh else np.zeros((1, 18)), dtype=np.float64)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz9, ps11, cs6, disp18)]
    lib().oracle_pipe_element(_dp(args[0]), _dp(args[1]), _dp(args[2]), nh, _dp(hd), _dp(args[3]), float(p0i),
                              _dp(K), _dp(f))
    return K.reshape(18, 18).T, f  # row-major [r][s]


def shell_element(xyz18, mat3, thickness, hist_disp, disp27, pressure=None, area_update=1):
    """One Shell_1 element (oracle_shell_element): K row-major [r][s], f."""
    K = np.zeros(729)
    f = np.zeros(27)
    nh = 0 if hist_disp is None else len(hist_disp)
    hd = np.ascontiguousarray(hist_disp if nh else np.zeros((1, 27)), dtype=np.float64)
    x = np.ascontiguousarray(xyz18, dtype=np.float64)
    m = np.ascontiguousarray(mat3, dtype=np.float64)
    d = np.ascontiguousarray(disp27, dtype=np.float64)
    lib().oracle_shell_element(_dp(x), _dp(m), float(thickness), nh, _dp(hd), _dp(d), int(pressure is not None),
                               float(pressure or 0.0), int(area_update), _dp(K), _dp(f))
    return K.reshape(27, 27).T, f


def first_tangent(structure):
    h = structure.desc()
    dims = (C.c_int * 2)()
    lib().oracle_first_tangent(C.cast(h.ref, C.c_void_p), None, None, dims)
    n, kl = dims[0], dims[1]
    ab = np.zeros((n, 3 * kl + 1))
    P = np.zeros(n)
    lib().oracle_first_tangent(C.cast(h.ref, C.c_void_p), _dp(ab), _dp(P), dims)
    return ab, P, kl


def beam_inertia(xyz9, mat3, sec6, cs6, hist_disp, disp18, vel18, acc18, dt, beta, gamma):
    M = np.zeros(324)
    F = np.zeros(18)
    ke = np.zeros(1)
    nh = 0 if hist_disp is None else len(hist_disp)
    hd = np.ascontiguousarray(hist_disp if nh else np.zeros((1, 18)), dtype=np.float64)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz9, mat3, sec6, cs6, disp18, vel18, acc18)]
    lib().oracle_beam_inertia_element(_dp(args[0]), _dp(args[1]), _dp(args[2]), _dp(args[3]), nh, _dp(hd),
                                      _dp(args[4]), _dp(args[5]), _dp(args[6]), dt, beta, gamma, _dp(M), _dp(F),
                                      _dp(ke))
    return M.reshape(18, 18).T, F, ke[0]


def shell_inertia(xyz18, mat3, thickness, hist_disp, disp27, vel36, acc36, dt, beta, gamma):
    """Shell_1 MountMass of one element (oracle_shell_inertia_element): the
    mass/gyroscopic tangent row-major [r][s], the inertial force, the kinetic
    energy."""
    M = np.zeros(729)
    F = np.zeros(27)
    ke = np.zeros(1)
    nh = 0 if hist_disp is None else len(hist_disp)
    hd = np.ascontiguousarray(hist_disp if nh else np.zeros((1, 27)), dtype=np.float64)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz18, mat3, disp27, vel36, acc36)]
    lib().oracle_shell_inertia_element(_dp(args[0]), _dp(args[1]), float(thickness), nh, _dp(hd), _dp(args[2]),
                                       _dp(args[3]), _dp(args[4]), dt, beta, gamma, _dp(M), _dp(F), _dp(ke))
    return M.reshape(27, 27).T, F, ke[0]

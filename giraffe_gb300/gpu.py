"""ctypes binding of libgiraffe_gpu.so (include/giraffe_gpu.h).

The CUDA library is the only implementation: importing this module loads it
and raises if it is missing; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .model import Structure, gf_model_desc

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libgiraffe_gpu.so")

GF_PREC_FP64, GF_PREC_MIXED = 0, 1
GF_N_KERNELS = 18  # kernel classes of gf_batch_profile
GF_WIDE_FP64, GF_WIDE_TENSOR, GF_WIDE_TENSOR_SYNC = 0, 1, 2

EXPORTS = ["gf_create", "gf_destroy", "gf_last_error", "gf_default_opts", "gf_batch_create",
           "gf_batch_destroy", "gf_batch_reset", "gf_batch_run", "gf_batch_results",
           "gf_batch_last_ms", "gf_batch_last_launches", "gf_batch_assemble", "gf_solve",
           "gf_beam_elements", "gf_band_solve", "gf_batch_solve_timed", "gf_batch_profile",
           "gf_kernel_name", "gf_batch_bytes", "gf_batch_host_ms", "gf_batch_step", "gf_batch_snapshot_bytes",
           "gf_batch_snapshot", "gf_batch_restore", "gf_batch_work", "gf_device_fp_peaks",
           "gf_beam_inertia_elements", "gf_band_solve_noalloc", "gf_sparse_solve", "gf_batch_device_bytes",
           "gf_server_default_opts", "gf_server_create", "gf_server_destroy", "gf_server_submit",
           "gf_server_poll", "gf_server_get_status", "gf_shell_elements", "gf_batch_assemble_csr",
           "gf_shell_inertia_elements", "gf_ctx_set_opts", "gf_upload_structure", "gf_structure_destroy",
           "gf_structure_dims", "gf_structure_dofs", "gf_structure_pattern", "gf_structure_set_step", "gf_begin_step",
           "gf_assemble", "gf_set_increment", "gf_commit", "gf_rollback", "gf_structure_nodes", "gf_beam_mount",
           "gf_beam_save_lagrange", "gf_shell_mount", "gf_shell_save_lagrange", "gf_structure_modal", "gf_modal", "gf_batch_monitor",
           "gf_batch_wide_tiles"]

GF_LAYOUT_CSR, GF_LAYOUT_GB = 0, 1
GF_BEAM_LAG, GF_SHELL_LAG = 21, 27


class gf_solve_opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("poll_every", C.c_int),
                ("use_graph", C.c_int), ("wide_update", C.c_int), ("max_passes", C.c_int),
                ("monitor_rows", C.c_int), ("max_refine", C.c_int), ("wide_tiles", C.c_int * 4)]


class gf_stats(C.Structure):
    _fields_ = [("converged_steps", C.c_int), ("newton_iterations", C.c_int), ("bisections", C.c_int),
                ("aborted", C.c_int), ("linear_solves", C.c_int),
                ("refine_sweeps", C.c_int), ("fp64_fallbacks", C.c_int)]


class gf_server_opts(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_waves", C.c_int), ("max_wave_structs", C.c_int),
                ("passes_per_chunk", C.c_int), ("max_wave_passes", C.c_int), ("precision", C.c_int)]


class gf_server_result(C.Structure):
    _fields_ = [("tag", C.c_longlong), ("status", C.c_int), ("pad", C.c_int), ("stats", gf_stats),
                ("queued_ms", C.c_double), ("total_ms", C.c_double)]


class gf_server_status(C.Structure):
    _fields_ = [("queued", C.c_int), ("waves", C.c_int), ("structures", C.c_int), ("pad", C.c_int),
                ("budget_in_use", C.c_size_t), ("passes", C.c_longlong), ("launches", C.c_longlong),
                ("reported", C.c_longlong)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library {LIB_PATH} is not built; run giraffe_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.gf_create.restype = vp
        L.gf_create.argtypes = [C.c_int]
        L.gf_destroy.argtypes = [vp]
        L.gf_last_error.restype = C.c_char_p
        L.gf_last_error.argtypes = [vp]
        L.gf_default_opts.argtypes = [C.POINTER(gf_solve_opts)]
        L.gf_ctx_set_opts.argtypes = [vp, C.POINTER(gf_solve_opts)]
        L.gf_batch_create.restype = vp
        L.gf_batch_create.argtypes = [vp, C.c_int, C.POINTER(gf_model_desc), C.POINTER(gf_solve_opts)]
        L.gf_batch_destroy.argtypes = [vp]
        L.gf_batch_reset.argtypes = [vp]
        L.gf_batch_run.argtypes = [vp]
        L.gf_batch_results.argtypes = [vp, C.POINTER(dp), C.POINTER(gf_stats)]
        L.gf_batch_last_ms.restype = C.c_double
        L.gf_batch_last_ms.argtypes = [vp]
        L.gf_batch_last_launches.restype = C.c_longlong
        L.gf_batch_last_launches.argtypes = [vp]
        L.gf_batch_host_ms.argtypes = [vp, dp, C.c_int]
        L.gf_batch_step.argtypes = [vp, C.c_int, ip]
        L.gf_batch_snapshot_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
        L.gf_batch_snapshot.argtypes = [vp, vp]
        L.gf_batch_restore.argtypes = [vp, vp]
        L.gf_batch_assemble.argtypes = [vp, C.c_int, dp, dp, ip]
        L.gf_solve.argtypes = [vp, C.c_int, C.POINTER(gf_model_desc), C.POINTER(gf_solve_opts),
                               C.POINTER(dp), C.POINTER(gf_stats)]
        L.gf_beam_elements.argtypes = [vp, C.c_int, dp, dp, dp, dp, C.c_int, dp, dp, dp, dp]
        L.gf_band_solve.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, C.c_int, dp, ip]
        L.gf_band_solve_noalloc.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, C.c_int, dp, ip]
        L.gf_sparse_solve.argtypes = [vp, C.c_int, ip, ip, dp, dp, ip]
        L.gf_beam_inertia_elements.argtypes = [vp, C.c_int, dp, dp, dp, dp, C.c_int, dp, dp, dp, dp, C.c_double,
                                               C.c_double, C.c_double, dp, dp]
        L.gf_batch_assemble_csr.argtypes = [vp, C.c_int, ip, ip, dp, dp, ip]
        L.gf_shell_elements.argtypes = [vp, C.c_int, dp, dp, dp, C.c_int, dp, dp, dp, C.c_int, dp, dp]
        L.gf_shell_inertia_elements.argtypes = [vp, C.c_int, dp, dp, dp, C.c_int, dp, dp, dp, dp, C.c_double,
                                                C.c_double, C.c_double, dp, dp]
        L.gf_batch_device_bytes.argtypes = [vp, C.c_int, C.POINTER(gf_model_desc), C.POINTER(C.c_size_t)]
        L.gf_upload_structure.restype = vp
        L.gf_upload_structure.argtypes = [vp, C.POINTER(gf_model_desc), C.POINTER(gf_solve_opts)]
        L.gf_structure_destroy.argtypes = [vp]
        L.gf_structure_dims.argtypes = [vp, ip]
        L.gf_structure_dofs.argtypes = [vp, ip]
        L.gf_structure_pattern.argtypes = [vp, ip, ip]
        L.gf_structure_set_step.argtypes = [vp, C.c_int]
        L.gf_begin_step.argtypes = [vp, C.c_double, C.c_double]
        L.gf_assemble.argtypes = [vp, C.c_int, dp, dp]
        L.gf_set_increment.argtypes = [vp, dp]
        L.gf_commit.argtypes = [vp]
        L.gf_rollback.argtypes = [vp]
        L.gf_structure_nodes.argtypes = [vp, dp, dp]
        L.gf_structure_modal.argtypes = [vp, C.c_double, C.c_int, C.c_double, dp, dp, ip]
        L.gf_modal.argtypes = [vp, C.POINTER(gf_model_desc), C.c_int, C.c_double, dp, dp, ip]
        L.gf_batch_monitor.argtypes = [vp, C.c_int, dp, ip]
        L.gf_batch_wide_tiles.argtypes = [vp, ip]
        L.gf_beam_mount.argtypes = [vp, C.c_int, dp, dp, dp, dp, dp, dp, dp, dp]
        L.gf_beam_save_lagrange.argtypes = [vp, C.c_int, dp, dp, dp, dp, dp, dp]
        L.gf_shell_mount.argtypes = [vp, C.c_int, dp, dp, dp, dp, dp, dp, dp, C.c_int, dp, dp]
        L.gf_shell_save_lagrange.argtypes = [vp, C.c_int, dp, dp, dp, dp, dp]
        L.gf_server_default_opts.argtypes = [C.POINTER(gf_server_opts)]
        L.gf_server_create.restype = vp
        L.gf_server_create.argtypes = [vp, C.POINTER(gf_server_opts)]
        L.gf_server_destroy.argtypes = [vp]
        L.gf_server_submit.argtypes = [vp, C.POINTER(gf_model_desc), dp, C.c_longlong]
        L.gf_server_poll.argtypes = [vp, C.POINTER(gf_server_result), C.c_int, ip]
        L.gf_server_get_status.argtypes = [vp, C.POINTER(gf_server_status)]
        _lib = L
    return _lib


def device_bytes(structures) -> int:
    """Device bytes one batch of these structures holds (gf_batch_device_bytes;
    needs no GPU)."""
    L = lib()
    handles = [s.desc() for s in structures]
    descs = (gf_model_desc * len(handles))(*[h.desc for h in handles])
    n = C.c_size_t(0)
    rc = L.gf_batch_device_bytes(None, len(handles), descs, C.byref(n))
    if rc != 0:
        raise RuntimeError(f"gf_batch_device_bytes failed ({rc})")
    return n.value


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Context:
    def __init__(self, device: int = 0):
        self.L = lib()
        self.h = self.L.gf_create(device)
        if not self.h:
            raise RuntimeError("gf_create failed (no CUDA device?)")

    def close(self):
        if self.h:
            self.L.gf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self) -> str:
        return self.L.gf_last_error(self.h).decode()

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed ({rc}): {self.error()}")

    def opts(self, precision=GF_PREC_FP64, use_graph=True, poll_every=8, wide_update=None,
             max_passes=0, monitor_rows=0, max_refine=0, wide_tiles=None):
        o = gf_solve_opts()
        self.L.gf_default_opts(C.byref(o))
        o.precision, o.use_graph, o.poll_every, o.max_passes = precision, int(use_graph), poll_every, max_passes
        o.monitor_rows, o.max_refine = monitor_rows, max_refine
        if wide_tiles is not None:
            for k, v in enumerate(wide_tiles):
                o.wide_tiles[k] = v
        if wide_update is not None:
            o.wide_update = wide_update
        return o

    def beam_elements(self, xyz, mat, sec, cs, hist_disp, disp):
        n = xyz.shape[0]
        nh = 0 if hist_disp is None else hist_disp.shape[1]
        K = np.zeros((n, 324))
        f = np.zeros((n, 18))
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz, mat, sec, cs, disp)]
        hd = np.ascontiguousarray(hist_disp if nh else np.zeros((n, 1, 18)), dtype=np.float64)
        self.check(self.L.gf_beam_elements(self.h, n, _dp(arrs[0]), _dp(arrs[1]), _dp(arrs[2]), _dp(arrs[3]), nh,
                                           _dp(hd), _dp(arrs[4]), _dp(K), _dp(f)), "gf_beam_elements")
        return K.reshape(n, 18, 18).transpose(0, 2, 1), f

    def beam_inertia(self, xyz, mat, sec, cs, hist_disp, disp, vel, acc, dt, beta, gamma):
        n = xyz.shape[0]
        nh = 0 if hist_disp is None else hist_disp.shape[1]
        M = np.zeros((n, 324))
        F = np.zeros((n, 18))
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz, mat, sec, cs, disp, vel, acc)]
        hd = np.ascontiguousarray(hist_disp if nh else np.zeros((n, 1, 18)), dtype=np.float64)
        self.check(self.L.gf_beam_inertia_elements(self.h, n, *[_dp(a) for a in arrs[:4]], nh, _dp(hd), _dp(arrs[4]),
                                                   _dp(arrs[5]), _dp(arrs[6]), dt, beta, gamma, _dp(M), _dp(F)),
                   "gf_beam_inertia_elements")
        return M.reshape(n, 18, 18).transpose(0, 2, 1), F

    def shell_elements(self, xyz, mat, thick, hist_disp, disp, pressure=None, area_update=1):
        """gf_shell_elements: K [n][27][27] (row-major [r][s]) and f [n][27]."""
        n = len(disp)
        nh = 0 if hist_disp is None else hist_disp.shape[1]
        K = np.zeros((n, 729))
        f = np.zeros((n, 27))
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz, mat, thick, disp)]
        hd = np.ascontiguousarray(hist_disp if nh else np.zeros((n, 1, 27)), dtype=np.float64)
        pr = None if pressure is None else np.ascontiguousarray(pressure, dtype=np.float64)
        self.check(self.L.gf_shell_elements(self.h, n, _dp(arrs[0]), _dp(arrs[1]), _dp(arrs[2]), nh, _dp(hd),
                                            _dp(arrs[3]), None if pr is None else _dp(pr), int(area_update), _dp(K),
                                            _dp(f)), "gf_shell_elements")
        return K.reshape(n, 27, 27).transpose(0, 2, 1), f

    def shell_inertia(self, xyz, mat, thick, hist_disp, disp, vel, acc, dt, beta, gamma):
        """gf_shell_inertia_elements: M [n][27][27] (row-major [r][s]) and F [n][27]."""
        n = len(disp)
        nh = 0 if hist_disp is None else hist_disp.shape[1]
        M = np.zeros((n, 729))
        F = np.zeros((n, 27))
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (xyz, mat, thick, disp, vel, acc)]
        hd = np.ascontiguousarray(hist_disp if nh else np.zeros((n, 1, 27)), dtype=np.float64)
        self.check(self.L.gf_shell_inertia_elements(self.h, n, _dp(arrs[0]), _dp(arrs[1]), _dp(arrs[2]), nh, _dp(hd),
                                                    _dp(arrs[3]), _dp(arrs[4]), _dp(arrs[5]), dt, beta, gamma,
                                                    _dp(M), _dp(F)), "gf_shell_inertia_elements")
        return M.reshape(n, 27, 27).transpose(0, 2, 1), F

    def band_solve(self, ab, kl, ku, b):
        ab = np.ascontiguousarray(ab, dtype=np.float64)  # [n][ldab] (column j contiguous)
        n, ldab = ab.shape
        x = np.ascontiguousarray(b, dtype=np.float64).copy()
        info = C.c_int(0)
        self.check(self.L.gf_band_solve(self.h, n, kl, ku, _dp(ab), ldab, _dp(x), C.byref(info)), "gf_band_solve")
        return x, info.value

    def sparse_solve(self, row_ptr, col_idx, val, b):
        """gf_sparse_solve: K x = b for K in 0-based row-major CSR; returns
        (x, info)."""
        n = len(b)
        rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
        ci = np.ascontiguousarray(col_idx, dtype=np.int32)
        v = np.ascontiguousarray(val, dtype=np.float64)
        if len(rp) != n + 1 or len(ci) != rp[-1] or len(v) != rp[-1]:
            raise ValueError("CSR arrays do not match n and nnz")
        x = np.ascontiguousarray(b, dtype=np.float64).copy()
        info = C.c_int(0)
        ip = C.POINTER(C.c_int)
        self.check(self.L.gf_sparse_solve(self.h, n, rp.ctypes.data_as(ip), ci.ctypes.data_as(ip), _dp(v), _dp(x),
                                          C.byref(info)), "gf_sparse_solve")
        return x, info.value

    def set_standalone_opts(self, wide_update=GF_WIDE_TENSOR):
        """gf_ctx_set_opts: the wide-band trailing update of this context's
        standalone solves (band_solve, sparse_solve)."""
        o = self.opts(wide_update=wide_update)
        self.check(self.L.gf_ctx_set_opts(self.h, C.byref(o)), "gf_ctx_set_opts")

    def beam_mount(self, xyz, mat, sec, cs, lag, disp):
        """gf_beam_mount: K [n][18][18] (row r, column s) and P_loading on the
        reference's LagrangeSave state lag [n][2][21]."""
        n = xyz.shape[0]
        K = np.zeros((n, 324))
        f = np.zeros((n, 18))
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (xyz, mat, sec, cs, lag, disp)]
        self.check(self.L.gf_beam_mount(self.h, n, *[_dp(v) for v in a], _dp(K), _dp(f)), "gf_beam_mount")
        return K.reshape(n, 18, 18).transpose(0, 2, 1), f

    def beam_save_lagrange(self, xyz, mat, sec, cs, lag, disp):
        """gf_beam_save_lagrange: the state after committing disp (a new array)."""
        n = xyz.shape[0]
        out = np.ascontiguousarray(lag, dtype=np.float64).copy()
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (xyz, mat, sec, cs)]
        d = np.ascontiguousarray(disp, dtype=np.float64)
        self.check(self.L.gf_beam_save_lagrange(self.h, n, *[_dp(v) for v in a], _dp(out), _dp(d)),
                   "gf_beam_save_lagrange")
        return out

    def shell_mount(self, xyz, mat, thick, lag, disp, cur_xyz=None, pressure=None, area_update=1):
        n = xyz.shape[0]
        K = np.zeros((n, 729))
        f = np.zeros((n, 27))
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (xyz, mat, thick, lag, disp)]
        cur = None if cur_xyz is None else np.ascontiguousarray(cur_xyz, dtype=np.float64)
        p = None if pressure is None else np.ascontiguousarray(pressure, dtype=np.float64)
        self.check(self.L.gf_shell_mount(self.h, n, *[_dp(v) for v in a], _dp(cur) if cur is not None else None,
                                         _dp(p) if p is not None else None, area_update, _dp(K), _dp(f)),
                   "gf_shell_mount")
        return K.reshape(n, 27, 27).transpose(0, 2, 1), f

    def shell_save_lagrange(self, xyz, mat, thick, lag, disp):
        n = xyz.shape[0]
        out = np.ascontiguousarray(lag, dtype=np.float64).copy()
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (xyz, mat, thick)]
        d = np.ascontiguousarray(disp, dtype=np.float64)
        self.check(self.L.gf_shell_save_lagrange(self.h, n, *[_dp(v) for v in a], _dp(out), _dp(d)),
                   "gf_shell_save_lagrange")
        return out

    def modal(self, structure: Structure, n_modes: int, tol: float = 0.0, modes: bool = True):
        """A Modal step of the structure at its start (gf_modal): (eigenvalues
        ascending, modes [n_modes x n free DOFs] or None, iterations)."""
        h = structure.desc()
        eig = np.zeros(n_modes)
        V = np.zeros((n_modes, structure.n_free)) if modes else None
        it = C.c_int(0)
        self.check(self.L.gf_modal(self.h, C.byref(h.desc), n_modes, tol, _dp(eig), _dp(V) if modes else None,
                                   C.byref(it)), "gf_modal")
        return eig, V, it.value

    def band_solve_noalloc(self, ab, kl, ku, b):
        """gf_band_solve_noalloc: band_solve through the static device scratch."""
        ab = np.ascontiguousarray(ab, dtype=np.float64)
        n, ldab = ab.shape
        x = np.ascontiguousarray(b, dtype=np.float64).copy()
        info = C.c_int(0)
        self.check(self.L.gf_band_solve_noalloc(self.h, n, kl, ku, _dp(ab), ldab, _dp(x), C.byref(info)),
                   "gf_band_solve_noalloc")
        return x, info.value


class DeviceStructure:
    """One device-resident structure driven one Newton stage at a time
    (gf_upload_structure ... gf_rollback): the calls a caller's own
    Static::Solve / Dynamic::Solve loop makes.  Vectors are in the
    reference's free-DOF numbering."""

    def __init__(self, ctx: Context, structure: Structure, opts=None):
        self.ctx = ctx
        self.L = ctx.L
        self.structure = structure
        self.handle = structure.desc()
        o = opts or ctx.opts()
        self.h = self.L.gf_upload_structure(ctx.h, C.byref(self.handle.desc), C.byref(o))
        if not self.h:
            raise RuntimeError("gf_upload_structure failed: " + ctx.error())
        dims = (C.c_int * 4)()
        self.L.gf_structure_dims(self.h, dims)
        self.n, self.nnz, self.kb, self.n_nodes = list(dims)
        ip = C.POINTER(C.c_int)
        self.dof = np.zeros(self.n, dtype=np.int32)
        self.L.gf_structure_dofs(self.h, self.dof.ctypes.data_as(ip))
        self.row_ptr = np.zeros(self.n + 1, dtype=np.int32)
        self.col_idx = np.zeros(max(self.nnz, 1), dtype=np.int32)
        self.L.gf_structure_pattern(self.h, self.row_ptr.ctypes.data_as(ip), self.col_idx.ctypes.data_as(ip))
        self.col_idx = self.col_idx[:self.nnz]

    def close(self):
        if self.h:
            self.L.gf_structure_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_step(self, k: int):
        self.ctx.check(self.L.gf_structure_set_step(self.h, k), "gf_structure_set_step")

    def begin_step(self, last_converged_time: float, time_step: float):
        self.ctx.check(self.L.gf_begin_step(self.h, last_converged_time, time_step), "gf_begin_step")

    def assemble(self, layout=GF_LAYOUT_CSR):
        """(K, P_A): CSR values in the pattern's order, or GB storage
        [n][3 kb + 1] (column j contiguous), and the residual f_ext - f_int."""
        K = np.zeros(self.nnz if layout == GF_LAYOUT_CSR else (self.n, 3 * self.kb + 1))
        P = np.zeros(self.n)
        self.ctx.check(self.L.gf_assemble(self.h, layout, _dp(K), _dp(P)), "gf_assemble")
        return K, P

    def set_increment(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self.ctx.check(self.L.gf_set_increment(self.h, _dp(x)), "gf_set_increment")

    def commit(self):
        self.ctx.check(self.L.gf_commit(self.h), "gf_commit")

    def rollback(self):
        self.ctx.check(self.L.gf_rollback(self.h), "gf_rollback")

    def modal(self, time: float, n_modes: int, tol: float = 0.0):
        """Modal analysis at the structure's current configuration with the
        loads at `time` (gf_structure_modal): (eigenvalues, modes
        [n_modes x n] in the reference's free-DOF numbering, iterations)."""
        eig = np.zeros(n_modes)
        modes = np.zeros((n_modes, self.n))
        it = C.c_int(0)
        self.ctx.check(self.L.gf_structure_modal(self.h, time, n_modes, tol, _dp(eig), _dp(modes), C.byref(it)),
                       "gf_structure_modal")
        return eig, modes, it.value

    def nodes(self):
        """(nodes [n_nodes x 15], increments [n_nodes x 6])."""
        nodes = np.zeros((self.n_nodes, 15))
        inc = np.zeros((self.n_nodes, 6))
        self.ctx.check(self.L.gf_structure_nodes(self.h, _dp(nodes), _dp(inc)), "gf_structure_nodes")
        return nodes, inc


class BatchSolver:
    """A device-resident batch of structures (gf_batch_*)."""

    def __init__(self, ctx: Context, structures, opts=None):
        self.ctx = ctx
        self.structures = list(structures)
        self.handles = [s.desc() for s in self.structures]
        self.descs = (gf_model_desc * len(self.handles))(*[h.desc for h in self.handles])
        o = opts or ctx.opts()
        self.h = ctx.L.gf_batch_create(ctx.h, len(self.handles), self.descs, C.byref(o))
        if not self.h:
            raise RuntimeError("gf_batch_create failed: " + ctx.error())

    def close(self):
        if self.h:
            self.ctx.L.gf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        self.ctx.check(self.ctx.L.gf_batch_reset(self.h), "gf_batch_reset")

    def run(self):
        self.ctx.check(self.ctx.L.gf_batch_run(self.h), "gf_batch_run")
        return self.ctx.L.gf_batch_last_ms(self.h)

    def host_ms(self):
        """Host wall time (ms) of the batch: model work, device allocation and
        uploads of gf_batch_create, graph capture, the last results read."""
        ms = (C.c_double * 5)()
        self.ctx.check(self.ctx.L.gf_batch_host_ms(self.h, ms, 5), "gf_batch_host_ms")
        return dict(zip(("build", "alloc", "upload", "graph", "results"), list(ms)))

    def step(self, passes: int) -> int:
        """Runs up to `passes` Newton passes; returns the structures still running."""
        r = C.c_int(0)
        self.ctx.check(self.ctx.L.gf_batch_step(self.h, passes, C.byref(r)), "gf_batch_step")
        return r.value

    def snapshot(self) -> np.ndarray:
        """The batch's device state between passes, as host bytes."""
        n = C.c_size_t(0)
        self.ctx.check(self.ctx.L.gf_batch_snapshot_bytes(self.h, C.byref(n)), "gf_batch_snapshot_bytes")
        buf = np.empty(n.value, dtype=np.uint8)
        self.ctx.check(self.ctx.L.gf_batch_snapshot(self.h, buf.ctypes.data), "gf_batch_snapshot")
        return buf

    def restore(self, buf: np.ndarray) -> None:
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        self.ctx.check(self.ctx.L.gf_batch_restore(self.h, buf.ctypes.data), "gf_batch_restore")

    def launches(self):
        return self.ctx.L.gf_batch_last_launches(self.h)

    def results(self):
        outs = [np.empty((s.n_nodes, 15)) for s in self.structures]
        ptrs = (C.POINTER(C.c_double) * len(outs))(*[_dp(o) for o in outs])
        stats = (gf_stats * len(outs))()
        self.ctx.check(self.ctx.L.gf_batch_results(self.h, ptrs, stats), "gf_batch_results")
        st = np.array([[x.converged_steps, x.newton_iterations, x.bisections, x.aborted] for x in stats])
        self.last_stats = stats
        return outs, st

    def wide_tiles(self):
        """The wide-band LU tile shapes this batch runs with
        (gf_batch_wide_tiles): [bulk trsm rows, first trsm rows, corner tile,
        solve rows]."""
        t = (C.c_int * 4)()
        self.ctx.check(self.ctx.L.gf_batch_wide_tiles(self.h, t), "gf_batch_wide_tiles")
        return list(t)

    def solve_stats(self):
        """Per structure, after results(): linear solves, FP64 refinement
        sweeps of the FP32 wide-band factor and solves refactored in FP64
        (GF_PREC_MIXED), as rows [linear_solves, refine_sweeps,
        fp64_fallbacks]."""
        return np.array([[x.linear_solves, x.refine_sweeps, x.fp64_fallbacks] for x in self.last_stats])

    def monitor(self, s: int):
        """Structure s's monitor lines (gf_batch_monitor): [node][line][31]
        in Node::WriteMonitor's columns, and the number of lines the run
        produced (more than returned when monitor_rows ran out)."""
        dims = (C.c_int * 3)()
        self.ctx.check(self.ctx.L.gf_batch_monitor(self.h, s, None, dims), "gf_batch_monitor")
        out = np.zeros((dims[0], dims[1], 31))
        if dims[0]:
            self.ctx.check(self.ctx.L.gf_batch_monitor(self.h, s, _dp(out), dims), "gf_batch_monitor")
        return out, dims[2]

    def assemble(self, s: int):
        dims = (C.c_int * 2)()
        self.ctx.check(self.ctx.L.gf_batch_assemble(self.h, s, None, None, dims), "gf_batch_assemble")
        n, kb = dims[0], dims[1]
        ab = np.zeros((n, 3 * kb + 1))
        P = np.zeros(n)
        self.ctx.check(self.ctx.L.gf_batch_assemble(self.h, s, _dp(ab), _dp(P), dims), "gf_batch_assemble")
        return ab, P, kb

    def assemble_csr(self, s: int):
        """First-pass K_AA of structure s in CSR (row_ptr, col_idx, val) and P_A."""
        L = self.ctx.L
        dims = (C.c_int * 2)()
        self.ctx.check(L.gf_batch_assemble_csr(self.h, s, None, None, None, None, dims), "gf_batch_assemble_csr")
        n, nnz = dims[0], dims[1]
        rp = np.zeros(n + 1, dtype=np.int32)
        ci = np.zeros(nnz, dtype=np.int32)
        v = np.zeros(nnz)
        P = np.zeros(n)
        ip = C.POINTER(C.c_int)
        self.ctx.check(L.gf_batch_assemble_csr(self.h, s, rp.ctypes.data_as(ip), ci.ctypes.data_as(ip), _dp(v),
                                               _dp(P), dims), "gf_batch_assemble_csr")
        return rp, ci, v, P


def solve(structures, precision=GF_PREC_FP64, device=0, timings=None):
    """Solves every structure's solution step on the GPU; returns final nodal
    states (n_nodes x 15 each) and stats rows (converged steps, Newton
    iterations, bisections, aborted).  A dict passed as `timings` receives
    the device time of the run and the host-time split of gf_batch_host_ms
    (ms)."""
    ctx = Context(device)
    b = BatchSolver(ctx, structures, ctx.opts(precision))
    b.reset()
    dev_ms = b.run()
    out = b.results()
    if timings is not None:
        timings.update(b.host_ms(), device_run=dev_ms)
    b.close()
    ctx.close()
    return out

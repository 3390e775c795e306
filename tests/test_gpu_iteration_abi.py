"""The Newton-iteration boundary and the element entries on the reference's
stored Gauss-point state, through the C ABI.

* tests/iteration_abi/static_loop.cpp is the reference's Static::Solve loop
  with its convergence criteria, calling gf_begin_step / gf_assemble /
  gf_sparse_solve / gf_set_increment / gf_commit / gf_rollback where the
  reference calls Zeros + MountDisplacements / Mount* + MountGlobal +
  MountSparse / sparsesystem / UpdateDisps / SaveConfiguration /
  RestoreConfiguration.  It is compiled here with g++ against include/ and
  libgiraffe_gpu.so and driven through ctypes; its results match the
  reference's goldens (tutorial01, the 2 pi roll-up with its bisections, a
  pipe chain, a 4x4x2 plate under follower pressure) to 1e-10 with the
  oracle's step, iteration and bisection counts.
* gf_beam_mount / gf_beam_save_lagrange and gf_shell_mount /
  gf_shell_save_lagrange: the reference's element goldens, their history
  built by committing the recorded increments onto the state of a new
  element, match to 1e-12.
* a Newmark step sequence driven through the same calls (tutorial10's
  first steps, Python loop) matches the batch path.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from giraffe_gb300 import build, configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = build.build()
    out = str(tmp_path_factory.mktemp("iter") / "libstatic_loop.so")
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "iteration_abi", "static_loop.cpp"), "-o", out,
           "-L", os.path.dirname(lib), "-lgiraffe_gpu", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True)
    d = C.CDLL(out)
    d.drive_static.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)]
    return d


def _drive(driver, ctx, s):
    h = s.desc()
    final = np.zeros((s.n_nodes, 15))
    stats = (C.c_int * 4)()
    rc = driver.drive_static(ctx.h, C.cast(C.byref(h.desc), C.c_void_p), final.ctypes.data_as(C.POINTER(C.c_double)),
                             stats)
    assert rc == 0, ctx.error()
    return final, list(stats)


def _small_chain():
    return configs.pipe_chain(30, 0.4, 0.03, [1.5e5, -1.0e5, 0.8e5], element_length=10.0 / 30)


@pytest.mark.parametrize("name,make", [
    ("ref_tutorial01.npz", configs.tutorial01),
    ("ref_rollup.npz", configs.cantilever_rollup),
    ("ref_chain.npz", _small_chain),
    ("ref_plate.npz", lambda: configs.square_plate(4, steps=20)),
])
def test_reference_static_loop_through_the_iteration_boundary(gpu_ctx, golden, driver, name, make):
    g = golden(name)
    s = make()
    final, stats = _drive(driver, gpu_ctx, s)
    ref = g["nodes"][-1]
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(final[:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(final[:, 6:] - ref[:, 6:]).max() <= 1e-9
    _, so, _ = oracle.solve(s)
    assert stats == list(so)


def _lag0_beam(n):
    """LagrangeSave of new Beam_1 elements: Q_i = I, dz_i = (0, 0, 1)."""
    lag = np.zeros((n, 2, 21))
    lag[:, :, [0, 4, 8]] = 1.0
    lag[:, :, 20] = 1.0
    return lag


def test_beam_mount_on_lagrange_state_matches_reference(gpu_ctx, golden):
    g = golden("ref_beam_elements.npz")
    n = len(g["K"])
    xyz, mat, sec, cs = g["xyz"], g["mat"], g["sec6"], g["cs"]
    lag = _lag0_beam(n)
    # SaveLagrange of each committed increment (elements with fewer get zero
    # increments, which leave the state as it is)
    for q in range(g["hist"].shape[1]):
        d = np.array([g["hist"][i][q] if q < int(g["n_hist"][i]) else np.zeros(18) for i in range(n)])
        lag = gpu_ctx.beam_save_lagrange(xyz, mat, sec, cs, lag, d)
    K, f = gpu_ctx.beam_mount(xyz, mat, sec, cs, lag, g["disp"])
    for i in range(n):
        assert rel(K[i], g["K"][i]) < 1e-12, i
        assert rel(f[i], g["P"][i]) < 1e-12, i
    # the state of an element that has committed nothing is the new state
    K0, f0 = gpu_ctx.beam_mount(xyz, mat, sec, cs, _lag0_beam(n), g["disp"])
    Ke, fe = gpu_ctx.beam_elements(xyz, mat, sec, cs, None, g["disp"])
    assert np.array_equal(K0, Ke) and np.array_equal(f0, fe)


def test_shell_mount_on_stored_state_matches_reference(gpu_ctx, golden):
    g = golden("ref_shell_elements.npz")
    n = len(g["K"])
    xyz, mat, thick = g["xyz"], g["mat"], g["thick"]
    lag = np.zeros((n, 3, 27))
    lag[:, :, [0, 4, 8]] = 1.0
    lag[:, :, 21] = 1.0  # z_x1_i = (1, 0, 0)
    lag[:, :, 25] = 1.0  # z_x2_i = (0, 1, 0)
    cur = np.array(xyz, dtype=float)
    for q in range(g["hist"].shape[1]):
        d = np.array([g["hist"][i][q] if q < int(g["n_hist"][i]) else np.zeros(27) for i in range(n)])
        lag = gpu_ctx.shell_save_lagrange(xyz, mat, thick, lag, d)
        cur += d[:, :18]
    press = ~np.isnan(g["pressure"])
    for au in (0, 1):
        idx = [i for i in range(n) if (not press[i]) or int(g["area_update"][i]) == au]
        p = np.where(press[idx], g["pressure"][idx], np.nan)
        K, f = gpu_ctx.shell_mount(xyz[idx], mat[idx], thick[idx], lag[idx], g["disp"][idx], cur[idx], p, au)
        for k, i in enumerate(idx):
            assert rel(K[k], g["K"][i]) < 1e-12, i
            assert rel(f[k], g["P"][i]) < 1e-12, i


def test_newmark_steps_through_the_iteration_boundary_match_the_batch_path(gpu_ctx):
    """tutorial10's Dynamic step (prescribed base motion, Newmark) for 40
    time steps, driven by a Python restatement of the Newton loop through
    the iteration boundary with the linear solve on gf_band_solve: every
    step converges with the batch path's iteration count, and the final
    state equals the batch path's to 1e-12."""
    s = configs.tutorial10()
    s.solution.end_time = 40 * s.solution.time_step
    ds = gpu.DeviceStructure(gpu_ctx, s)
    crit = s.criteria
    so = s.solution
    t, dt = so.start_time, so.time_step
    total_it = 0
    fc = mc = 0.0
    n_ev = 0
    for _ in range(40):
        ds.begin_step(t, dt)
        inc = np.zeros(ds.n_nodes * 6)
        it, res_conv, gl_conv = 1, False, False
        while not (res_conv and gl_conv):
            K, P = ds.assemble(gpu.GF_LAYOUT_GB)
            trans = ds.dof % 6 < 3
            mf, mm = np.abs(P[trans]).max(), np.abs(P[~trans]).max()
            if it == 1:
                f1 = max(mf * crit["force_tol"], crit["force_min"] * crit["force_tol"])
                m1 = max(mm * crit["moment_tol"], crit["moment_min"] * crit["moment_tol"])
                fc, mc = (n_ev * fc + f1) / (n_ev + 1), (n_ev * mc + m1) / (n_ev + 1)
                n_ev += 1
            res_conv = mf <= fc and mm <= mc
            if not (res_conv and gl_conv):
                x, info = gpu_ctx.band_solve(K, ds.kb, ds.kb, P)
                assert info == 0
                res_conv = False
                ds.set_increment(x)
                inc[ds.dof] += x
                mdv, mrv = np.abs(inc[ds.dof][trans]).max(), np.abs(inc[ds.dof][~trans]).max()
                dc = max(crit["disp_tol"] * mdv, crit["disp_min"] * crit["disp_tol"])
                rc = max(crit["rot_tol"] * mrv, crit["rot_min"] * crit["rot_tol"])
                gl_conv = np.abs(x[trans]).max() <= dc and np.abs(x[~trans]).max() <= rc
            it += 1
            total_it += 1
            assert it <= so.max_it + 1
        ds.commit()
        t += dt
    final, _ = ds.nodes()
    ds.close()
    b = gpu.BatchSolver(gpu_ctx, [s])
    b.reset()
    b.run()
    fb, sb = b.results()
    b.close()
    assert sb[0][0] == 40 and sb[0][1] == total_it
    scale = np.abs(fb[0][:, :3]).max()
    assert np.abs(final[:, :3] - fb[0][:, :3]).max() <= 1e-12 * scale

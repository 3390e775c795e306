"""Shell_1 on the CUDA path (through the C ABI) against the reference's
golden fixtures and the oracle: element tangent and force with follower
pressure (1e-12 relative), the first assembled K_AA in the reference's
BandMatrix layout and numbering (1e-13), and complete plate solves on the
wide-band LU (reverse Cuthill-McKee numbering, no pivoting) against the
reference (1e-10 relative, the plain path's stated tolerance, with the same
step and iteration counts)."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_shell_elements_match_reference(gpu_ctx, golden):
    g = golden("ref_shell_elements.npz")
    n = len(g["K"])
    press = ~np.isnan(g["pressure"])
    groups = {}
    for i in range(n):
        groups.setdefault((int(g["n_hist"][i]), bool(press[i]), int(g["area_update"][i])), []).append(i)
    for (nh, has_p, au), idx in groups.items():
        hist = np.stack([g["hist"][i][:nh] for i in idx]) if nh else None
        K, f = gpu_ctx.shell_elements(g["xyz"][idx], g["mat"][idx], g["thick"][idx], hist, g["disp"][idx],
                                      g["pressure"][idx] if has_p else None, au)
        for k, i in enumerate(idx):
            assert rel(K[k], g["K"][i]) < 1e-12, i
            assert rel(f[k], g["P"][i]) < 1e-12, i


def test_plate_first_assembly_matches_oracle(gpu_ctx):
    for s in (configs.square_plate(4, steps=20), configs.square_plate(3, steps=10, area_update=0)):
        b = gpu.BatchSolver(gpu_ctx, [s])
        ab, P, kb = b.assemble(0)
        ab_o, P_o, kl_o = oracle.first_tangent(s)
        b.close()
        assert kb == kl_o
        assert rel(ab, ab_o) < 1e-13
        assert rel(P, P_o) < 1e-13


def _solve(ctx, structs):
    b = gpu.BatchSolver(ctx, structs)
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


@pytest.mark.parametrize("name,make", [
    ("ref_plate.npz", lambda: configs.square_plate(4, steps=20)),
    ("ref_plate_fixed_area.npz", lambda: configs.square_plate(3, steps=10, area_update=0)),
])
def test_plate_solve_matches_reference(gpu_ctx, golden, name, make):
    g = golden(name)
    s = make()
    finals, stats = _solve(gpu_ctx, [s])
    ref = g["nodes"][-1]
    assert stats[0][3] == 0
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    assert np.abs(finals[0][:, 6:] - ref[:, 6:]).max() <= 1e-9
    steps = g["steps"]
    conv = steps[steps[:, 2] == 0]
    assert stats[0][0] == len(conv)
    assert stats[0][1] == int(conv[:, 1].sum() + len(conv))


def test_plate_and_beams_in_one_batch_match_the_oracle(gpu_ctx):
    """A finer plate (8x8x2, 10 steps) next to beam chains: wide-band and
    chain solvers in the same pass; every structure as the oracle solves it."""
    structs = [configs.square_plate(8, steps=10), configs.pipe_chain(40, 0.4, 0.03, [1e5, 2e4, -3e4]),
               configs.square_plate(2, steps=5, area_update=0)]
    finals, stats = _solve(gpu_ctx, structs)
    for k, s in enumerate(structs):
        fo, so, _ = oracle.solve(s, 0)
        assert tuple(stats[k]) == tuple(so), k
        scale = np.abs(fo[:, :3]).max()
        assert np.abs(finals[k][:, :3] - fo[:, :3]).max() <= 1e-10 * scale, k


@pytest.mark.parametrize("name,make", [
    ("ref_plate.npz", lambda: configs.square_plate(4, steps=20)),
    ("ref_plate_fixed_area.npz", lambda: configs.square_plate(3, steps=10, area_update=0)),
])
def test_plate_tensor_core_and_fp64_updates_match_reference(gpu_ctx, golden, name, make):
    """The wide-band LU's trailing update on the tensor cores (FP64 products
    from exact bf16 slices, GF_WIDE_TENSOR, the default) and in FP64 FMA
    (GF_WIDE_FP64): both solve the plate as the reference does (1e-10, same
    step and iteration counts) and agree to 1e-13."""
    g = golden(name)
    s = make()
    b = gpu.BatchSolver(gpu_ctx, [s], gpu_ctx.opts(wide_update=gpu.GF_WIDE_TENSOR))
    b.reset()
    b.run()
    finals, stats = b.results()
    b.close()
    ref = g["nodes"][-1]
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(finals[0][:, :3] - ref[:, :3]).max() <= 1e-10 * scale
    steps = g["steps"]
    conv = steps[steps[:, 2] == 0]
    assert stats[0][0] == len(conv)
    assert stats[0][1] == int(conv[:, 1].sum() + len(conv))
    b = gpu.BatchSolver(gpu_ctx, [make()], gpu_ctx.opts(wide_update=gpu.GF_WIDE_FP64))
    b.reset()
    b.run()
    f64, st64 = b.results()
    b.close()
    assert tuple(st64[0]) == tuple(stats[0])
    assert np.abs(finals[0][:, :3] - f64[0][:, :3]).max() <= 1e-13 * scale

"""Benchmark: Newton solves per second of the batched static Beam_1 step.

Workload (one "step" = one complete solve of the batch from its initial
configuration): 512 independent pipe-section Beam_1 chains, element counts
log-uniform in [50, 2000] from seed 0, Tube De ~ U(0.3, 0.5) m, wall
~ U(0.02, 0.04) m, E = 210 GPa, clamped at one end, tip force ~ N(0, 1e5) N
per component, 10 load steps, each chain 10 m long.  A Newton solve is one
load step of one structure iterated to convergence (reference
src/Static.cpp:200-250); the metric counts converged load steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours (default) runs the CUDA library; --impl reference times the
reference's CPU algorithm for the path (the oracle restatement, on all host
threads, on a bounded sample of the same chains).  Under torchrun with N
ranks the workload is N x 512 chains of the same family (seed 0), split
across the ranks by greedy LPT on each chain's estimated Newton-pass cost
(giraffe_gb300.partition): about 512 chains of work per GPU (weak
scaling), no collective on the data path; rank 0 prints one JSON line.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Newton solves/sec (batched static Beam_1 chains, FP64, converged load steps)"
UNIT = "Newton solves/s"
# DRAM bytes per element mount of k_beam_tangent, from one ncu capture on 128
# chains: (54.9 MB read + 173.1 MB written) / 79,322 elements
TANGENT_DRAM_BYTES_PER_ELEMENT = (55.088384e6 + 202.853120e6) / 79322


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chains", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=512, help="chains in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-sample", type=int, default=32,
                    help="chains solved one at a time for the plain single-structure leg")
    ap.add_argument("--serve-requests", type=int, default=400,
                    help="requests in the served-stream leg (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="Poisson arrival rate of the served stream (1/s)")
    ap.add_argument("--serve-budget-gb", type=int, default=16, help="device-memory budget of the server")
    ap.add_argument("--serve-mixed-requests", type=int, default=60,
                    help="requests in the mixed chain/plate served leg (0 = skip)")
    ap.add_argument("--serve-plate-max-dof", type=int, default=20000,
                    help="largest plate (free DOFs) in the mixed served leg")
    ap.add_argument("--mixed-steps", type=int, default=3,
                    help="timed solves of the mixed-precision leg (0 = skip)")
    ap.add_argument("--shell-n", type=int, default=64,
                    help="squares per side of the plate of the shell leg (64: the 64x64x2 benchmark plate)")
    ap.add_argument("--shell-steps", type=int, default=20,
                    help="load steps (of 20) of the 64x64x2 Shell_1 plate leg (0 = skip); its FP64-FMA and "
                         "mma.sync comparisons run the first two")
    ap.add_argument("--dyn-steps", type=int, default=1000,
                    help="time steps (of 1000) of the batched-dynamics leg (0 = skip)")
    ap.add_argument("--rollup", type=int, default=1, help="time the 20-element cantilever roll-up (0 = skip)")
    ap.add_argument("--serve-saturated", type=int, default=1,
                    help="the 512-chain workload submitted at once through the server (0 = skip)")
    ap.add_argument("--serve-full-requests", type=int, default=12,
                    help="requests of the mixed served stream with the full 10k-200k plate range (0 = skip)")
    return ap.parse_args()


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl"
        try:
            import torch

            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend, init_method="env://")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p:
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "of measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "of fallback"


def cpu_baseline(structs, sample_n, rank):
    """Oracle restatement on all host threads over a bounded, size-stratified
    sample of the workload's chains."""
    from oracle import oracle

    order = np.argsort([len(s.beams) for s in structs])
    idx = order[np.linspace(0, len(order) - 1, min(sample_n, len(order))).astype(int)]
    sample = [structs[i] for i in idx]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    finals, stats, fails = oracle.solve_batch(sample, threads=threads)
    dt = time.perf_counter() - t0
    solves = int(stats[:, 0].sum())
    return {"value": solves / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(sample)} of the {len(structs)} chains (every size stratum), "
                      f"{solves} Newton solves in {dt:.2f} s on {threads} host threads"}, (idx, finals, stats)


def oracle_parity(structs, idx, finals, stats, o_finals, o_stats):
    """The headline's own results against the oracle's, chain by chain, on
    the chains the CPU baseline solved: relative error of the converged
    nodal translations (2-norm), largest deviation of the nodal rotation
    tensors, and whether converged steps, Newton iterations and bisections
    are the same."""
    rel, dq, same = [], 0.0, 0
    for k, i in enumerate(idx):
        s = structs[i]
        u, uo = finals[i][:, :3] - s.nodes, o_finals[k][:, :3] - s.nodes
        rel.append(float(np.linalg.norm(u - uo) / np.linalg.norm(uo)))
        dq = max(dq, float(np.abs(finals[i][:, 6:] - o_finals[k][:, 6:]).max()))
        same += int(np.array_equal(np.asarray(stats[i]), np.asarray(o_stats[k])))
    worst = int(np.argmax(rel))
    return {"chains": len(idx), "max_rel_err_displacement": max(rel), "median_rel_err_displacement":
            float(np.median(rel)), "worst_chain_elements": len(structs[idx[worst]].beams),
            "max_abs_err_rotation": dq, "counts_match": same,
            "tolerance": 1e-10, "within_tolerance": int(sum(r <= 1e-10 for r in rel))}


def run_reference(args, rank, world):
    from giraffe_gb300 import configs

    if rank != 0:
        return
    # the same workload as this repository's arm at this N (N x chains), of
    # which each step solves a bounded size-stratified sample
    structs = configs.batched_static(args.chains * world, seed=args.seed)
    vals, step_ms = [], []
    info = None
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        info, _ = cpu_baseline(structs, args.cpu_sample, rank)
        if k >= args.warmup:
            vals.append(info["value"])
            step_ms.append((time.perf_counter() - t0) * 1e3)
    value = statistics.median(vals)
    info["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(step_ms),
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"batched static: {args.chains} Beam_1 pipe chains per GPU, "
                                   f"50-2000 elements log-uniform, 10 load steps, seed {args.seed}",
                       "chains": args.chains * world, "chains_per_gpu": args.chains, "load_steps": 10,
                       "precision": "plain FP64 (element tangent and force, chain/band solver, residual)"},
            "cpu_baseline": info,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def plain_leg(ctx, structs, sample_n):
    """The plain FP64 path one structure at a time (a batch of one per
    gf_batch_run, as a caller replacing Static::Solve per structure would run
    it) over a size-stratified sample of the same chains; device time of each
    run after one warm-up run of the same structure."""
    from giraffe_gb300 import gpu

    order = np.argsort([len(s.beams) for s in structs])
    idx = order[np.linspace(0, len(order) - 1, min(sample_n, len(order))).astype(int)]
    ms, solves = 0.0, 0
    for i in idx:
        b = gpu.BatchSolver(ctx, [structs[i]])
        b.reset()
        b.run()
        b.reset()
        ms += b.run()
        solves += int(b.results()[1][0, 0])
        b.close()
    return {"value": solves / (ms / 1e3), "unit": UNIT,
            "sample": f"{len(idx)} of the {len(structs)} chains (every size stratum), one structure per solve, "
                      f"{solves} Newton solves in {ms:.1f} ms of device time"}


def mixed_leg(ctx, structs, args, f64_finals, f64_stats):
    """The same batched workload with GF_PREC_MIXED (the Beam_1 tangent
    operator in FP32-pair arithmetic; force, residual, rotations and solves
    FP64), device-timed like the headline, with its deviation from the FP64
    path: max over chains of |u_mixed - u_fp64| / |u_fp64| (translations,
    2-norm) and of the nodal rotation tensors."""
    import ctypes as C

    from giraffe_gb300 import gpu

    L = ctx.L
    b = gpu.BatchSolver(ctx, structs, ctx.opts(gpu.GF_PREC_MIXED))
    b.reset()
    b.run()
    fm, sm = b.results()
    ms = C.c_double(0.0)
    ctx.check(L.gf_batch_solve_timed(b.h, args.mixed_steps, C.byref(ms)), "gf_batch_solve_timed")
    b.close()
    solves = int(sm[:, 0].sum()) * args.mixed_steps
    rel_u, dq = 0.0, 0.0
    for k, s in enumerate(structs):
        u_f = f64_finals[k][:, :3] - s.nodes
        u_m = fm[k][:, :3] - s.nodes
        rel_u = max(rel_u, float(np.linalg.norm(u_m - u_f) / np.linalg.norm(u_f)))
        dq = max(dq, float(np.abs(fm[k][:, 6:] - f64_finals[k][:, 6:]).max()))
    return {"value": solves / (ms.value / 1e3), "unit": UNIT, "ms_per_step": ms.value / args.mixed_steps,
            "precision": "Beam_1 tangent: rotation to the global frame and K_e expansion in FP32-pair (~48-bit) "
                         "arithmetic on the FP32 pipe; Gauss-point operator, internal force, residual, rotation "
                         "updates, chain/band solves and convergence checks FP64",
            "max_rel_err_displacement_vs_fp64": rel_u, "max_abs_err_rotation_vs_fp64": dq,
            "same_step_and_iteration_counts": bool(np.array_equal(sm, f64_stats)),
            "structures_with_other_counts": int((sm != f64_stats).any(axis=1).sum())}


def shell_leg(ctx, args, fp64_peak):
    """The Shell_1 plate (64x64 squares x 2 six-node triangles, 84,867 free
    DOFs, clamped edges, follower pressure ramped to 1e5 Pa over 20 load
    steps): the first `shell_steps` load steps, device-timed, with the
    wide-band LU's FP64 rate; and an 8x8 plate solved completely by the GPU
    and by the oracle on the host cores, like for like."""
    import ctypes as C

    from giraffe_gb300 import configs, gpu
    from oracle import oracle

    L = ctx.L
    s = configs.square_plate(args.shell_n, steps=20)
    s.solution.end_time = args.shell_steps / 20.0
    # the first two steps with the trailing update in FP64 FMA and in the
    # mma.sync form, for comparison
    s2 = configs.square_plate(args.shell_n, steps=20)
    s2.solution.end_time = min(args.shell_steps, 2) / 20.0
    b2 = gpu.BatchSolver(ctx, [s2])
    b2.reset()
    ms_tc2 = b2.run()
    f_tc2, st_tc2 = b2.results()
    b2.close()
    bf = gpu.BatchSolver(ctx, [s2], ctx.opts(wide_update=gpu.GF_WIDE_FP64))
    bf.reset()
    ms_fp64 = bf.run()
    st_fp64 = bf.results()[1]
    bf.close()
    # and with the warp-level mma.sync form of the tensor-core update
    bsy = gpu.BatchSolver(ctx, [s2], ctx.opts(wide_update=gpu.GF_WIDE_TENSOR_SYNC))
    bsy.reset()
    ms_sync = bsy.run()
    f_sync, st_sync = bsy.results()
    bsy.close()
    b = gpu.BatchSolver(ctx, [s])
    b.reset()
    ms = b.run()
    fin, st = b.results()
    lu, ab, mf = C.c_double(), C.c_double(), C.c_double()
    L.gf_batch_work(b.h, C.byref(lu), C.byref(ab), C.byref(mf))
    dims = (C.c_int * 2)()
    L.gf_batch_assemble(b.h, 0, None, None, dims)
    launches = b.launches()
    tiles = b.wide_tiles()
    # per-kernel-class device time of a pass over the first load step (events
    # around every launch, no graph; classes on the lookahead's helper
    # streams overlap the main stream, so the classes sum to more than a pass)
    L.gf_batch_profile.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    L.gf_kernel_name.restype = C.c_char_p
    s1 = configs.square_plate(args.shell_n, steps=20)
    s1.solution.end_time = 1.0 / 20.0
    bp = gpu.BatchSolver(ctx, [s1])
    kms, kl = (C.c_double * gpu.GF_N_KERNELS)(), (C.c_longlong * gpu.GF_N_KERNELS)()
    ctx.check(L.gf_batch_profile(bp.h, kms, kl), "gf_batch_profile")
    passes = max(1, int(bp.results()[1][0][1]))
    bp.close()
    split = {L.gf_kernel_name(i).decode(): round(kms[i] / passes, 3) for i in range(gpu.GF_N_KERNELS) if kl[i]}
    # the sparsesystem drop-in on the same plate: the first pass's K_AA as a
    # host CSR, solved through gf_sparse_solve (ordering, upload, wide-band
    # LU, solution back to the host)
    rp, ci, v, P = b.assemble_csr(0)
    b.close()
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        x, info = ctx.sparse_solve(rp, ci, v, P)
        times.append(time.perf_counter() - t0)
    t_sp = statistics.median(times)
    n_sp, kl_sp = len(P), dims[1]
    sparse = {"workload": f"first-pass K_AA of the {args.shell_n}x{args.shell_n}x2 plate as host CSR: n {n_sp}, "
                          f"nnz {len(v)}, "
                          f"half-bandwidth {kl_sp}", "ms": t_sp * 1e3, "linear_solves_per_s": 1.0 / t_sp,
              "info": int(info), "lu_tflops_end_to_end": 2.0 * n_sp * kl_sp * kl_sp / t_sp / 1e12,
              "note": "host CSR in, x out; includes the RCM trial, CSR upload, scatter, factor and "
                      "substitutions (2 n kl^2 flops counted)"}
    # FP32 band factor with FP64 iterative refinement (GF_PREC_MIXED), the
    # same plate and load steps
    sm_ = configs.square_plate(args.shell_n, steps=20)
    sm_.solution.end_time = args.shell_steps / 20.0
    bm = gpu.BatchSolver(ctx, [sm_], ctx.opts(gpu.GF_PREC_MIXED))
    bm.reset()
    ms_mx = bm.run()
    fin_mx, st_mx = bm.results()
    ex_mx = bm.solve_stats()[0]
    launches_mx = bm.launches()
    bm.close()
    s1m = configs.square_plate(args.shell_n, steps=20)
    s1m.solution.end_time = 1.0 / 20.0
    bpm = gpu.BatchSolver(ctx, [s1m], ctx.opts(gpu.GF_PREC_MIXED))
    ctx.check(L.gf_batch_profile(bpm.h, kms, kl), "gf_batch_profile")
    passes_m = max(1, int(bpm.results()[1][0][1]))
    bpm.close()
    split_mx = {L.gf_kernel_name(i).decode(): round(kms[i] / passes_m, 3) for i in range(gpu.GF_N_KERNELS) if kl[i]}
    u64 = fin[0][:, :3] - s.nodes
    mixed = {"precision": "FP32 wide-band LU (FP32 FMA panel kernels and trailing update) beside the FP64 K_AA; "
                          "FP64 residual b - K x and x += K32^-1 r until a correction is below 2^-52 |x| or "
                          "shrinks by less than half; FP64 refactor when refinement stalls above 2^-30 |x| or "
                          "exceeds 30 sweeps",
             "ms": ms_mx, "ms_per_pass": ms_mx / max(1, st_mx[0][1]),
             "solves_per_s": st_mx[0][0] / (ms_mx / 1e3),
             "speedup_vs_fp64_per_pass": (ms / max(1, st[0][1])) / (ms_mx / max(1, st_mx[0][1])),
             "linear_solves": int(ex_mx[0]), "refine_sweeps": int(ex_mx[1]),
             "sweeps_per_solve": float(ex_mx[1]) / max(1, int(ex_mx[0])), "fp64_fallbacks": int(ex_mx[2]),
             "same_step_and_iteration_counts_as_fp64": bool(tuple(st_mx[0]) == tuple(st[0])),
             "max_rel_err_displacement_vs_fp64":
                 float(np.abs(fin_mx[0][:, :3] - fin[0][:, :3]).max() / max(np.abs(u64).max(), 1e-300)),
             "gpu_launches": launches_mx, "pass_split_ms_first_step": split_mx}
    small = configs.square_plate(8, steps=20)
    bs = gpu.BatchSolver(ctx, [small])
    bs.reset()
    bs.run()
    bs.reset()
    ms_small = bs.run()
    st_small = bs.results()[1][0]
    bs.close()
    t0 = time.perf_counter()
    _, so, _ = oracle.solve(small, 0)
    cpu_s = time.perf_counter() - t0
    return {"workload": f"Shell_1 plate {args.shell_n}x{args.shell_n}x2, {dims[0]} free DOFs, natural numbering "
                        f"half-bandwidth "
                        f"{dims[1]}, first {args.shell_steps} of 20 load steps",
            "newton_solves": int(st[0][0]), "newton_passes": int(st[0][1]), "ms": ms,
            "solves_per_s": st[0][0] / (ms / 1e3), "ms_per_pass": ms / max(1, st[0][1]),
            "wide_update": "tensor cores: FP64 products from exact bf16 slices (Ozaki), tcgen05.mma 128x64x16 with "
                           "TMEM accumulators, bulk-copy (TMA) staged slices",
            "wide_lu_tflops": lu.value / (ms / 1e3) / 1e12, "fp64_peak_tflops": fp64_peak,
            "wide_lu_frac_of_measured_fp64": lu.value / (ms / 1e3) / 1e12 / fp64_peak,
            "first_two_steps": {"tcgen05_ms_per_pass": ms_tc2 / max(1, st_tc2[0][1]),
                                "fp64_fma_update_ms_per_pass": ms_fp64 / max(1, st_fp64[0][1]),
                                "mma_sync_update_ms_per_pass": ms_sync / max(1, st_sync[0][1]),
                                "same_counts": bool(tuple(st_fp64[0]) == tuple(st_tc2[0]) == tuple(st_sync[0])),
                                "counts_steps_iterations_bisections":
                                    {"tcgen05": [int(v) for v in st_tc2[0][:3]],
                                     "fp64_fma": [int(v) for v in st_fp64[0][:3]],
                                     "mma_sync": [int(v) for v in st_sync[0][:3]]},
                                "max_abs_diff_m_sync_vs_tcgen05":
                                    float(np.abs(f_sync[0][:, :3] - f_tc2[0][:, :3]).max())},
            "gpu_launches": launches, "center_deflection_m": float(fin[0][:, 2].min()),
            "wide_tiles": {"trsm_rows": tiles[0], "first_trsm_rows": tiles[1], "corner_tile": tiles[2],
                           "solve_rows": tiles[3], "how": "picked by the library's autotuner (timed on a "
                                                         "synthetic band of the plate's half-bandwidth)"},
            "pass_split_ms": split,
            "sparse_solve": sparse,
            "mixed_precision": mixed,
            "plate8": {"workload": "Shell_1 plate 8x8x2 (1,203 free DOFs), all 20 load steps",
                        "gpu_solves_per_s": st_small[0] / (ms_small / 1e3), "gpu_ms": ms_small,
                        "cpu_oracle_solves_per_s": so[0] / cpu_s, "cpu_cores": 1,
                        "same_counts": bool(tuple(st_small) == tuple(so))}}


def dynamics_leg(ctx, args):
    """Batched implicit dynamics (256 pipe Beam_1 chains of 100-1000
    elements, Newmark beta 0.25 gamma 0.5, dt 0.01 s, sinusoidal top
    displacement): the first `dyn_steps` of the 1000 time steps,
    device-timed after one warm-up run."""
    from giraffe_gb300 import configs, gpu

    structs = configs.batched_dynamic(256, seed=args.seed)
    for s in structs:
        s.solution.end_time = args.dyn_steps * 0.01
    b = gpu.BatchSolver(ctx, structs)
    b.reset()
    ms = b.run()  # device time after the pass graph's capture
    _, st = b.results()
    launches = b.launches()
    b.close()
    solves = int(st[:, 0].sum())
    return {"workload": f"256 pipe chains, 100-1000 elements uniform (seed {args.seed}), Newmark, "
                        f"{args.dyn_steps} of 1000 time steps", "newton_solves": solves, "ms": ms,
            "solves_per_s": solves / (ms / 1e3), "aborted": int(st[:, 3].sum()), "gpu_launches": launches}


def rollup_leg(ctx):
    """The 20-element cantilever rolled into a circle by a tip
    moment over 20 load steps (plain FP64 path, one structure), device time
    after a warm-up run, beside the oracle on one host core."""
    from giraffe_gb300 import configs, gpu
    from oracle import oracle

    s = configs.cantilever_rollup(n_el=20, steps=20)
    b = gpu.BatchSolver(ctx, [s])
    b.reset()
    b.run()
    b.reset()
    ms = b.run()
    fin, st = b.results()
    b.close()
    t0 = time.perf_counter()
    fo, so, _ = oracle.solve(s)
    cpu_s = time.perf_counter() - t0
    u, uo = fin[0][:, :3] - s.nodes, fo[:, :3] - s.nodes
    return {"workload": "20 Beam_1 cantilever (246 DOF), tip moment 2 pi EI/L over 20 load steps, FP64",
            "newton_solves": int(st[0][0]), "newton_passes": int(st[0][1]), "gpu_ms": ms,
            "gpu_solves_per_s": st[0][0] / (ms / 1e3), "cpu_oracle_ms": cpu_s * 1e3,
            "cpu_oracle_solves_per_s": so[0] / cpu_s, "cpu_cores": 1,
            "same_counts": bool(tuple(st[0]) == tuple(so)),
            "rel_err_vs_oracle": float(np.linalg.norm(u - uo) / np.linalg.norm(uo)),
            "tip_x_m": float(fin[0][-1, 0])}


def served_saturated_leg(ctx, args, structs, plain_value):
    """The 512-chain batched-static workload through the server: all chains
    submitted at once, the server admitting them in waves under its budget;
    sustained Newton solves per second from the first submission to the last
    result, against the plain single-structure path."""
    from giraffe_gb300 import serve

    srv = serve.Server(ctx, hbm_budget=args.serve_budget_gb << 30)
    out = serve.run_stream(srv, structs, np.zeros(len(structs)))
    srv.close()
    res = out["results"]
    r = {"workload": f"the {len(structs)}-chain batched-static workload submitted at t = 0 through gf_server_*",
         "solves_per_s": out["solves"] / out["wall_s"], "wall_s": out["wall_s"],
         "p50_latency_ms": out["p50_ms"], "p99_latency_ms": out["p99_ms"],
         "aborted": int(sum(x.stats[3] for x in res))}
    if plain_value:
        r["over_plain_single_structure"] = r["solves_per_s"] / plain_value
    # the batched mixed-precision served path: the same submission with
    # every wave built with GF_PREC_MIXED
    from giraffe_gb300 import gpu
    srv = serve.Server(ctx, hbm_budget=args.serve_budget_gb << 30, precision=gpu.GF_PREC_MIXED)
    outm = serve.run_stream(srv, structs, np.zeros(len(structs)))
    srv.close()
    m = {"solves_per_s": outm["solves"] / outm["wall_s"], "wall_s": outm["wall_s"],
         "p50_latency_ms": outm["p50_ms"], "p99_latency_ms": outm["p99_ms"],
         "aborted": int(sum(x.stats[3] for x in outm["results"]))}
    if plain_value:
        m["over_plain_single_structure"] = m["solves_per_s"] / plain_value
    r["mixed_precision"] = m
    return r


def served_full_leg(ctx, args, rank):
    """The mixed served stream with plates over the full DOF range: 70 % pipe
    chains (1k-50k DOF), 30 % Shell_1 plates of 10k-200k DOF (log-uniform),
    Poisson arrivals at 200/s.  One GPU cannot sustain the plates' share of the
    offered load; the leg reports what it sustains and the queueing."""
    from giraffe_gb300 import configs, serve

    seed = args.seed + 4000 + rank
    reqs = configs.served_mixed(args.serve_full_requests, seed=seed, plate_dof=(10000, 200000))
    arrivals = serve.poisson_arrivals(len(reqs), args.serve_rate, seed=seed)
    srv = serve.Server(ctx, hbm_budget=args.serve_budget_gb << 30)
    out = serve.run_stream(srv, reqs, arrivals, timeout_s=1200.0)
    srv.close()
    res = out["results"]
    is_plate = np.array([bool(s.shells) for s in reqs])
    lat = out["latency_ms"]
    dofs = [int(s.n_free) for s in reqs]
    return {"workload": f"{len(reqs)} requests: {int((~is_plate).sum())} pipe chains 1k-50k DOF and "
                        f"{int(is_plate.sum())} Shell_1 plates of 10k-200k DOF (largest "
                        f"{max([d for d, p in zip(dofs, is_plate) if p], default=0)}), 10 load steps each, "
                        f"Poisson arrivals at {args.serve_rate:g}/s",
            "p50_latency_ms": out["p50_ms"], "p99_latency_ms": out["p99_ms"],
            "chain_p50_ms": float(np.percentile(lat[~is_plate], 50)) if (~is_plate).any() else None,
            "plate_p50_ms": float(np.percentile(lat[is_plate], 50)) if is_plate.any() else None,
            "plate_max_ms": float(lat[is_plate].max()) if is_plate.any() else None,
            "solves_per_s": out["solves_per_s"], "requests_per_s": out["requests_per_s"], "wall_s": out["wall_s"],
            "offered_requests_per_s": args.serve_rate,
            "mean_queued_ms": float(np.mean([r.queued_ms for r in res])),
            "aborted": int(sum(r.stats[3] for r in res))}


def served_leg(ctx, args, rank):
    """Continuous batching of a Poisson stream of static pipe-chain requests
    (1k-50k DOF log-uniform) through gf_server_*: admitted by the device
    budget as they arrive; latency = result returned - scheduled arrival."""
    from giraffe_gb300 import configs, serve

    reqs = configs.served_chains(args.serve_requests, seed=args.seed + 1000 + rank)
    arrivals = serve.poisson_arrivals(len(reqs), args.serve_rate, seed=args.seed + 1000 + rank)
    srv = serve.Server(ctx, hbm_budget=args.serve_budget_gb << 30)
    warm = configs.served_chains(8, seed=args.seed + 2000 + rank)  # first-use costs out of the stream
    serve.run_stream(srv, warm, np.zeros(len(warm)))
    st0 = srv.status()
    out = serve.run_stream(srv, reqs, arrivals)
    st1 = srv.status()
    srv.close()
    res = out["results"]
    return {"workload": f"{len(reqs)} static Beam_1 pipe chains, 1k-50k free DOF log-uniform, 10 load steps, "
                        f"Poisson arrivals at {args.serve_rate:g}/s (seeded); Shell_1 plates not included",
            "requests": len(reqs), "p50_latency_ms": out["p50_ms"], "p99_latency_ms": out["p99_ms"],
            "solves_per_s": out["solves_per_s"], "requests_per_s": out["requests_per_s"], "wall_s": out["wall_s"],
            "aborted": int(sum(r.stats[3] for r in res)), "budget_gb": args.serve_budget_gb,
            "gpu_launches": st1["launches"] - st0["launches"],
            "mean_queued_ms": float(np.mean([r.queued_ms for r in res]))}


def served_mixed_leg(ctx, args, rank):
    """The mixed served stream: 70 % pipe chains (1k-50k DOF), 30 % Shell_1
    plates (10k DOF up to --serve-plate-max-dof), Poisson arrivals."""
    from giraffe_gb300 import configs, serve

    seed = args.seed + 3000 + rank
    reqs = configs.served_mixed(args.serve_mixed_requests, seed=seed,
                                plate_dof=(10000, max(10001, args.serve_plate_max_dof)))
    arrivals = serve.poisson_arrivals(len(reqs), args.serve_rate, seed=seed)
    srv = serve.Server(ctx, hbm_budget=args.serve_budget_gb << 30)
    out = serve.run_stream(srv, reqs, arrivals)
    st = srv.status()
    srv.close()
    res = out["results"]
    is_plate = np.array([bool(s.shells) for s in reqs])
    lat = out["latency_ms"]
    return {"workload": f"{len(reqs)} requests: {int((~is_plate).sum())} pipe chains 1k-50k DOF and "
                        f"{int(is_plate.sum())} Shell_1 plates 10k-{args.serve_plate_max_dof} DOF (of the 10k-200k "
                        f"range), 10 load steps each, Poisson arrivals at {args.serve_rate:g}/s; plates run in "
                        f"waves of their own",
            "p50_latency_ms": out["p50_ms"], "p99_latency_ms": out["p99_ms"],
            "chain_p50_ms": float(np.percentile(lat[~is_plate], 50)) if (~is_plate).any() else None,
            "plate_p50_ms": float(np.percentile(lat[is_plate], 50)) if is_plate.any() else None,
            "solves_per_s": out["solves_per_s"], "requests_per_s": out["requests_per_s"], "wall_s": out["wall_s"],
            "aborted": int(sum(r.stats[3] for r in res)), "gpu_launches": st["launches"]}


def rank_structures(args, rank, world):
    """This rank's chains: the N x --chains workload of seed --seed split by
    LPT on estimated Newton-pass cost (all of it at N = 1), and the
    estimated load of every rank (None at N = 1)."""
    from giraffe_gb300 import configs, partition

    allc = configs.batched_static(args.chains * world, seed=args.seed)
    if world == 1:
        return allc, None
    mine, loads = partition.shard(allc, rank, world)
    return [allc[i] for i in mine], loads


def run_ours(args, rank, world):
    import ctypes as C

    from giraffe_gb300 import build, gpu

    build.build()
    structs, rank_loads = rank_structures(args, rank, world)
    device = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = gpu.Context(device)
    L = ctx.L
    b = gpu.BatchSolver(ctx, structs, ctx.opts())
    # warm-up
    for _ in range(args.warmup):
        b.reset()
        b.run()
    f64_finals, stats = b.results()
    solves_per_step = int(stats[:, 0].sum())
    assert stats[:, 3].sum() == 0, "a structure aborted"
    L.gf_batch_solve_timed.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    ms = C.c_double(0.0)
    barrier(world)
    with Clocks(device) as clk:
        ctx.check(L.gf_batch_solve_timed(b.h, args.steps, C.byref(ms)), "gf_batch_solve_timed")
    barrier(world)
    launches = b.launches()
    total_ms = max_over_ranks(ms.value, world)
    total_solves = sum_over_ranks(solves_per_step * args.steps, world)
    value = total_solves / (total_ms / 1e3)
    # per-kernel device times (one profiled solve, events around every launch)
    L.gf_batch_profile.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    L.gf_kernel_name.restype = C.c_char_p
    kms = (C.c_double * gpu.GF_N_KERNELS)()
    kl = (C.c_longlong * gpu.GF_N_KERNELS)()
    ctx.check(L.gf_batch_profile(b.h, kms, kl), "gf_batch_profile")
    kernels = {L.gf_kernel_name(i).decode(): {"ms": kms[i], "launches": kl[i]} for i in range(gpu.GF_N_KERNELS) if kl[i]}
    L.gf_batch_work.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 3
    lu_f, asm_b, mnt_f = C.c_double(), C.c_double(), C.c_double()
    ctx.check(L.gf_batch_work(b.h, C.byref(lu_f), C.byref(asm_b), C.byref(mnt_f)), "gf_batch_work")
    L.gf_device_fp_peaks.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    fp64, fp32 = C.c_double(), C.c_double()
    ctx.check(L.gf_device_fp_peaks(ctx.h, C.byref(fp64), C.byref(fp32)), "gf_device_fp_peaks")
    L.gf_batch_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    h2d, d2h = C.c_longlong(), C.c_longlong()
    L.gf_batch_bytes(b.h, C.byref(h2d), C.byref(d2h))
    b.close()
    # e2e through the C ABI's whole-step call gf_solve (the drop-in for
    # Static::Solve, on the caller's context): from the caller's model
    # descriptors and output buffers, as the reference's db holds its model,
    # each call creates the batch (host numbering and PreCalc, the H2D copy of
    # the inputs), runs it and reads the final states and stats back (D2H)
    from giraffe_gb300.model import gf_model_desc
    handles = [s.desc() for s in structs]
    descs = (gf_model_desc * len(handles))(*[h.desc for h in handles])
    outs = [np.empty((s.n_nodes, 15)) for s in structs]
    optrs = (C.POINTER(C.c_double) * len(outs))(*[o.ctypes.data_as(C.POINTER(C.c_double)) for o in outs])
    ostats = (gpu.gf_stats * len(outs))()
    eo = ctx.opts()
    e2e_times = []
    for k in range(max(1, min(args.steps, 3))):
        barrier(world)
        t0 = time.perf_counter()
        ctx.check(L.gf_solve(ctx.h, len(handles), descs, C.byref(eo), optrs, ostats), "gf_solve")
        e2e_times.append(time.perf_counter() - t0)
    st = np.array([[x.converged_steps, x.newton_iterations, x.bisections, x.aborted] for x in ostats])
    assert np.array_equal(st, stats), "gf_solve counts differ from the timed batch"
    e2e_t = max_over_ranks(statistics.median(e2e_times), world)
    e2e_value = sum_over_ranks(int(st[:, 0].sum()), world) / e2e_t
    # the host-time split of the same call's phases (one more run, untimed)
    e2e_split = [{}]
    gpu.solve(structs, device=device, timings=e2e_split[0])
    # roofline of the dominant kernel
    peaks, tag = measured_peaks()
    # The dominant single kernel is k_beam_tangent (the chain solver is a
    # class of nine kernels, none as large); its roofline is the headline one,
    # the chain solver's is reported beside it.
    def tangent_roof(name):
        t = kernels[name]["ms"] / 1e3
        achieved = mnt_f.value / t / 1e12
        mounts_per_launch = mnt_f.value / 9000.0 / max(kernels[name]["launches"], 1)
        return {"kernel": name, "bound": "fp64", "achieved": achieved, "peak": fp64.value, "unit": "TFLOP/s",
                "frac": achieved / fp64.value,
                "traffic": TANGENT_DRAM_BYTES_PER_ELEMENT * mounts_per_launch,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_beam_tangent "
                                  "launch on 128 chains (profiles/k_beam_tangent_128chains.md): "
                                  f"{TANGENT_DRAM_BYTES_PER_ELEMENT:.0f} B per element, scaled by the "
                                  f"{mounts_per_launch:.0f} element mounts of an average launch here",
                "note": "FP64 CUDA-core bound (no HBM or tensor-core bound applies: per-element 18x18 algebra); "
                        "achieved counts 9000 FP64 flops per Beam_1 Mount (both Gauss points); peak = FP64 FMA "
                        "throughput measured live by gf_device_fp_peaks (of measured); HBM view: "
                        f"{TANGENT_DRAM_BYTES_PER_ELEMENT * mnt_f.value / 9000.0 / t / 1e9:.1f} GB/s of "
                        f"{peaks.get('hbm_gbs')} GB/s {tag}"}

    def solver_roof(name):
        t = kernels[name]["ms"] / 1e3
        achieved = lu_f.value / t / 1e12
        return {"kernel": name, "bound": "fp64", "achieved": achieved, "peak": fp64.value, "unit": "TFLOP/s",
                "frac": achieved / fp64.value, "traffic": None,
                "note": "FP64 CUDA-core bound; achieved counts the banded-LU-equivalent flops 2 n kl ku + "
                        "2 n (kl+ku) per Newton solve of each structure (the chain solver's own count, "
                        "condensation + cyclic reduction, is about 0.8 of it); peak = FP64 FMA throughput "
                        "measured live (of measured)"}

    if "beam_tangent" in kernels:
        roof = tangent_roof("beam_tangent")
    else:
        dom = max(kernels.items(), key=lambda kv: kv[1]["ms"])[0]
        roof = solver_roof(dom)
    roof_solver = None
    for name in ("chain_solve", "band_solve"):
        if name in kernels and kernels[name]["ms"] > 1.0:
            roof_solver = solver_roof(name)
            break
    plain = None
    if args.plain_sample > 0:
        plain = plain_leg(ctx, structs, args.plain_sample)
        plain["batched_over_plain"] = value / plain["value"]
    mixed = mixed_leg(ctx, structs, args, f64_finals, stats) if args.mixed_steps > 0 else None
    if mixed:
        mixed["over_plain_fp64_batched"] = mixed["value"] / value
        if plain:
            mixed["over_plain_single_structure"] = mixed["value"] / plain["value"]
    shell = shell_leg(ctx, args, fp64.value) if args.shell_steps > 0 else None
    dyn = dynamics_leg(ctx, args) if args.dyn_steps > 0 else None
    serving = None
    if args.serve_requests > 0:
        serving = served_leg(ctx, args, rank)
    serving_mixed = served_mixed_leg(ctx, args, rank) if args.serve_mixed_requests > 0 else None
    serving_full = served_full_leg(ctx, args, rank) if args.serve_full_requests > 0 else None
    saturated = (served_saturated_leg(ctx, args, structs, plain["value"] if plain else None)
                 if args.serve_saturated else None)
    rollup = rollup_leg(ctx) if args.rollup else None
    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, (idx, o_finals, o_stats) = cpu_baseline(structs, args.cpu_sample, rank)
        parity = oracle_parity(structs, idx, f64_finals, stats, o_finals, o_stats)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": f"batched static: {args.chains} Beam_1 pipe chains per GPU, "
                                       f"50-2000 elements log-uniform, 10 load steps, seed {args.seed}",
                           "chains": args.chains * world, "chains_per_gpu": args.chains, "load_steps": 10,
                           "sharding": "one workload of N x chains split by greedy LPT on estimated Newton-pass "
                                       "cost (giraffe_gb300.partition)" if world > 1 else "single GPU",
                           "estimated_rank_loads": rank_loads,
                           "newton_solves_per_step": solves_per_step,
                           "precision": "plain FP64 (element tangent and force, chain/band solver, residual)",
                           "l2": "working set larger than L2: element tangent scratch 0.62 GB and chain-solver "
                                 "scratch written and read every Newton pass",
                           "parallelism": f"{world} independent batch(es)"},
                "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_t * 1e3,
                        "timed": "one gf_solve call per step on the caller's context: batch creation (host "
                                 "numbering and PreCalc, H2D of the inputs), the run, D2H of final states "
                                 "and stats",
                        "split_ms": {k: round(statistics.median(x[k] for x in e2e_split), 2)
                                     for k in e2e_split[0]},
                        "h2d_bytes_per_step": h2d.value,
                        "d2h_bytes_per_step": d2h.value},
                "gpu_launches": launches,
                "roofline": roof,
                "roofline_linear_solve": roof_solver,
                "kernels_ms_per_solve": {k: round(v["ms"], 3) for k, v in kernels.items()},
                "peaks_measured": {"fp64_tflops": fp64.value, "fp32_tflops": fp32.value},
                "clocks": clk.summary(),
                "plain_single_structure": plain,
                "mixed_precision": mixed,
                "shell_plate": shell,
                "dynamics": dyn,
                "serving": serving,
                "serving_mixed": serving_mixed,
                "serving_full_plate_range": serving_full,
                "serving_saturated_512_chains": saturated,
                "rollup_20_elements": rollup,
                "cpu_baseline": cpu,
                "parity_vs_oracle": parity}
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse()
    rank, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Served path (gf_server_* through the C ABI): structures admitted while
others run, several waves on the device at once, a device-memory budget.
Each result in the mix must equal the structure's result solved alone
(gf_batch of that one structure): stated tolerance 1e-8 relative on the
converged nodal states, and the same step / iteration / bisection counts;
the batch path is deterministic, so the comparison is also bit-exact."""
import time

import numpy as np
import pytest

from giraffe_gb300 import configs, gpu, serve

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def _alone(ctx, s):
    b = gpu.BatchSolver(ctx, [s])
    b.reset()
    b.run()
    outs, st = b.results()
    b.close()
    return outs[0], tuple(int(v) for v in st[0])


def _check_same_as_alone(ctx, structs, results):
    for i, s in enumerate(structs):
        r = results[i]
        fa, sa = _alone(ctx, s)
        assert r.status == 0, i
        assert tuple(int(v) for v in r.stats) == sa, i
        assert rel(r.final, fa) <= 1e-8, i
        assert np.array_equal(r.final, fa), i


def test_results_in_the_mix_equal_results_alone(gpu_ctx):
    structs = configs.served_chains(13, seed=5, dof_min=600, dof_max=8000)
    structs += [configs.cantilever_rollup(), configs.tutorial01()]
    srv = serve.Server(gpu_ctx, hbm_budget=1 << 30, max_waves=3, max_wave_structs=4, passes_per_chunk=2)
    results, max_waves = {}, 0
    for i, s in enumerate(structs):
        srv.submit(s, tag=i)
        for r in srv.poll():
            results[r.tag] = r
        max_waves = max(max_waves, srv.status()["waves"])
        if i % 3 == 2:
            time.sleep(0.003)
    t0 = time.perf_counter()
    while len(results) < len(structs):
        for r in srv.poll():
            results[r.tag] = r
        max_waves = max(max_waves, srv.status()["waves"])
        assert time.perf_counter() - t0 < 300
    # the last wave retires once its trailing chunk has drained
    while srv.status()["waves"]:
        assert not srv.poll()
        assert time.perf_counter() - t0 < 300
    st = srv.status()
    srv.close()
    assert st["reported"] == len(structs) and st["queued"] == 0 and st["waves"] == 0
    assert st["budget_in_use"] == 0
    assert max_waves >= 2  # later arrivals ran beside earlier waves
    _check_same_as_alone(gpu_ctx, structs, results)


def test_admission_respects_the_budget(gpu_ctx):
    structs = configs.served_chains(8, seed=9, dof_min=3000, dof_max=12000)
    need = [gpu.device_bytes([s]) for s in structs]
    budget = int(2.2 * max(need)) + (1 << 17)
    srv = serve.Server(gpu_ctx, hbm_budget=budget, max_waves=4, max_wave_structs=8, passes_per_chunk=4)
    for i, s in enumerate(structs):
        srv.submit(s, tag=i)
    results, peak, saw_queue = {}, 0, False
    t0 = time.perf_counter()
    while len(results) < len(structs):
        for r in srv.poll():
            results[r.tag] = r
        st = srv.status()
        peak = max(peak, st["budget_in_use"])
        saw_queue |= st["queued"] > 0 and st["waves"] > 0
        assert time.perf_counter() - t0 < 300
    srv.close()
    assert peak <= budget
    assert saw_queue  # not everything fitted at once: some structures waited for memory
    _check_same_as_alone(gpu_ctx, structs, results)


def test_structure_larger_than_the_budget_is_refused(gpu_ctx):
    s = configs.pipe_chain(400, 0.4, 0.03, [1e5, 0.0, 0.0])
    srv = serve.Server(gpu_ctx, hbm_budget=gpu.device_bytes([s]) // 2)
    with pytest.raises(RuntimeError, match="budget"):
        srv.submit(s)
    srv.close()


def test_poisson_stream_latency(gpu_ctx):
    structs = configs.served_chains(40, seed=11, dof_min=1000, dof_max=20000)
    arrivals = serve.poisson_arrivals(len(structs), 200.0, seed=11)
    srv = serve.Server(gpu_ctx, hbm_budget=4 << 30)
    out = serve.run_stream(srv, structs, arrivals)
    srv.close()
    assert all(r.status == 0 and r.stats[3] == 0 for r in out["results"])
    assert np.all(out["latency_ms"] > 0)
    assert out["p99_ms"] >= out["p50_ms"] > 0


def test_mixed_chains_and_plates_equal_alone(gpu_ctx):
    """Shell_1 plates and beam chains in one stream: plates go to their own
    waves (the wide-band pass is long), every result equals its structure
    solved alone."""
    structs = configs.served_mixed(12, seed=21, plate_share=0.4, chain_dof=(600, 6000), plate_dof=(200, 1500))
    assert any(s.shells for s in structs) and any(s.beams for s in structs)
    srv = serve.Server(gpu_ctx, hbm_budget=1 << 30, max_waves=4, max_wave_structs=3, passes_per_chunk=2)
    results = {}
    t0 = time.perf_counter()
    for i, s in enumerate(structs):
        srv.submit(s, tag=i)
        for r in srv.poll():
            results[r.tag] = r
        if i % 4 == 3:
            time.sleep(0.002)
    while len(results) < len(structs):
        for r in srv.poll():
            results[r.tag] = r
        assert time.perf_counter() - t0 < 300
    srv.close()
    _check_same_as_alone(gpu_ctx, structs, results)


def test_mixed_precision_served_wave_equals_the_mixed_batch(gpu_ctx):
    """gf_server_opts.precision = GF_PREC_MIXED: each wave is built with the
    mixed options (FP32-pair Beam_1 tangents; an FP32 wide-band factor with
    FP64 refinement for Shell_1, its panel loops as graph loops in the served
    pass), and each served result is the mixed batch's result for that
    structure, bit for bit and with the same counts."""
    structs = configs.served_chains(5, seed=11, dof_min=600, dof_max=4000) + [configs.square_plate(6, steps=4)]
    srv = serve.Server(gpu_ctx, hbm_budget=1 << 30, max_waves=2, max_wave_structs=3, passes_per_chunk=2,
                       precision=gpu.GF_PREC_MIXED)
    for i, s in enumerate(structs):
        srv.submit(s, tag=i)
    results = {}
    t0 = time.perf_counter()
    while len(results) < len(structs):
        for r in srv.poll():
            results[r.tag] = r
        assert time.perf_counter() - t0 < 300
    while srv.status()["waves"]:
        assert not srv.poll()
    srv.close()
    for i, s in enumerate(structs):
        b = gpu.BatchSolver(gpu_ctx, [s], gpu_ctx.opts(gpu.GF_PREC_MIXED))
        b.reset()
        b.run()
        outs, st = b.results()
        b.close()
        r = results[i]
        assert r.status == 0, i
        assert tuple(int(v) for v in r.stats) == tuple(int(v) for v in st[0]), i
        assert np.array_equal(r.final, outs[0]), i

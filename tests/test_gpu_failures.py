"""Failure detection and recovery on the CUDA path, injected on the host (no
GPU fault, trap or hang): a structure with a NaN in its input, a singular
structure (a chain with no support), and one whose Newton loop may take
only one iteration (MaxIt 1).  Each is detected on the device (NaN / huge
detector, divergence reference, MaxIt), rolled back and bisected down to
MinTimeStep, and reported as aborted -- as the reference's
ConvergenceCriteria::NaNDetector and Static::Solve control do -- while the
healthy structures of the same batch finish bit for bit as they do alone."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu
from oracle import oracle

pytestmark = pytest.mark.gpu


def _solve(ctx, structs):
    b = gpu.BatchSolver(ctx, structs)
    b.reset()
    b.run()
    out = b.results()
    b.close()
    return out


def _healthy():
    return [configs.pipe_chain(30, 0.4, 0.03, [1e5, -5e4, 2e4], element_length=10.0 / 30),
            configs.pipe_chain(55, 0.35, 0.025, [-8e4, 3e4, 6e4], element_length=10.0 / 55)]


def _nan_input():
    s = configs.pipe_chain(20, 0.4, 0.03, [1e5, 0.0, 0.0], element_length=0.5)
    s.nodes = np.array(s.nodes)
    s.nodes[8, 0] = np.nan  # a corner node: the element geometry (PreCalc) takes it
    return s


def _singular():
    s = configs.pipe_chain(20, 0.4, 0.03, [1e5, 2e4, 0.0], element_length=0.5)
    s.constraints[:] = 0  # no support: rigid-body modes, K_AA singular
    return s


def _max_it_one():
    s = configs.pipe_chain(20, 0.4, 0.03, [3e5, -2e5, 1e5], element_length=0.5)
    s.solution.max_it = 1
    return s


def test_failing_structures_abort_and_leave_the_others_untouched(gpu_ctx):
    healthy = _healthy()
    bad = [_nan_input(), _singular(), _max_it_one()]
    structs = [healthy[0], bad[0], bad[1], healthy[1], bad[2]]
    finals, stats = _solve(gpu_ctx, structs)
    # the failing structures: rolled back and bisected until the step is
    # below MinTimeStep, then aborted, without an error from the library
    for k in (1, 2, 4):
        assert stats[k][3] == 1, k
        assert stats[k][2] > 0, k
    # the healthy ones: as alone, and as the oracle solves them
    for k, s in ((0, healthy[0]), (3, healthy[1])):
        alone, st1 = _solve(gpu_ctx, [s])
        assert np.array_equal(alone[0], finals[k])
        assert list(st1[0]) == list(stats[k])
        fo, so, _ = oracle.solve(s)
        assert list(stats[k]) == list(so)


@pytest.mark.parametrize("make", [_nan_input, _max_it_one])
def test_failure_path_follows_the_step_control_of_the_oracle(gpu_ctx, make):
    """NaN detection and MaxIt exhaustion take the same roll-back / bisection
    / abort path as the oracle's restatement of Static::Solve: the same
    converged steps, Newton iterations and bisections."""
    s = make()
    _, stats = _solve(gpu_ctx, [s])
    _, so, _ = oracle.solve(s)
    assert list(stats[0]) == list(so)
    assert so[3] == 1


def test_pass_cap_ends_the_run_with_timeout(gpu_ctx):
    """The host cap on Newton passes (gf_solve_opts.max_passes) stops a run
    that has not finished with GF_ERR_TIMEOUT; a fresh run with the default
    cap then finishes as the oracle does."""
    s = configs.pipe_chain(30, 0.4, 0.03, [1e5, -5e4, 2e4], element_length=10.0 / 30)
    b = gpu.BatchSolver(gpu_ctx, [s], gpu_ctx.opts(poll_every=4, max_passes=8))
    b.reset()
    with pytest.raises(RuntimeError, match=r"gf_batch_run failed \(4\)"):
        b.run()
    b.close()
    _, st = _solve(gpu_ctx, [s])
    _, so, _ = oracle.solve(s)
    assert list(st[0]) == list(so)


def test_server_wave_pass_cap_reports_timeout(gpu_ctx):
    """A served wave that runs past gf_server_opts.max_wave_passes reports its
    unfinished structures with GF_ERR_TIMEOUT instead of running on; the
    server stays usable and solves the next structure normally."""
    from giraffe_gb300 import serve

    s = configs.pipe_chain(30, 0.4, 0.03, [1e5, -5e4, 2e4], element_length=10.0 / 30)
    srv = serve.Server(gpu_ctx, hbm_budget=1 << 30, passes_per_chunk=2, max_wave_passes=4)
    srv.submit(s, tag=1)
    res = srv.drain(timeout_s=120)
    srv.close()
    assert len(res) == 1 and res[0].status == 4  # GF_ERR_TIMEOUT
    srv = serve.Server(gpu_ctx, hbm_budget=1 << 30)
    srv.submit(s, tag=2)
    res = srv.drain(timeout_s=120)
    srv.close()
    _, so, _ = oracle.solve(s)
    assert res[0].status == 0 and list(res[0].stats) == list(so)

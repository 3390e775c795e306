"""Checkpoint / resume of a device batch (gf_batch_step, gf_batch_snapshot,
gf_batch_restore) through the C ABI: a batch of static chains, a damped
dynamic riser, a static and a damped vibrating Shell_1 plate and a chain
running four solution steps in sequence is stopped between Newton passes,
snapshotted, run to the end, restored and run to the end again; both ends
and a run without a stop are bit-identical."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu

pytestmark = pytest.mark.gpu


def _mixed():
    return configs.batched_static(4, seed=5, n_min=20, n_max=90) + [
        configs.riser_chain(25, 0.4, 0.03, 1.0, 5.0, steps=30, rayleigh_alpha=0.2, rayleigh_beta=0.003),
        configs.square_plate(3, steps=10, area_update=0),
        configs.plate_dynamics(3, steps=10, rayleigh_alpha=8.0, rayleigh_beta=2e-5),
        configs.chain_sequence(10),
    ]


def test_snapshot_restore_resumes_bit_for_bit(gpu_ctx):
    structs = _mixed()
    b = gpu.BatchSolver(gpu_ctx, structs)
    b.reset()
    b.run()
    ref, st_ref = b.results()
    b.reset()
    running = b.step(17)
    assert running > 0
    snap = b.snapshot()
    b.run()
    r1, st1 = b.results()
    b.restore(snap)
    b.run()
    r2, st2 = b.results()
    # restoring into a batch that has moved on in between
    b.reset()
    b.step(40)
    b.restore(snap)
    b.run()
    r3, st3 = b.results()
    b.close()
    for k in range(len(structs)):
        assert np.array_equal(r1[k], ref[k]), k
        assert np.array_equal(r2[k], ref[k]), k
        assert np.array_equal(r3[k], ref[k]), k
    assert np.array_equal(st1, st_ref) and np.array_equal(st2, st_ref) and np.array_equal(st3, st_ref)


def test_step_counts_down_to_zero(gpu_ctx):
    b = gpu.BatchSolver(gpu_ctx, configs.batched_static(3, seed=1, n_min=20, n_max=60))
    b.reset()
    seen = [b.step(8) for _ in range(40)]
    b.close()
    assert seen[0] > 0 and seen[-1] == 0
    assert all(x >= y for x, y in zip(seen, seen[1:]))


def test_restore_refuses_a_snapshot_of_another_batch(gpu_ctx):
    """A snapshot carries a header (counts, damping flags, size): restoring it
    into a batch of other structures, or restoring bytes that are not a
    snapshot, fails with GF_ERR_ARG and leaves the batch as it was."""
    a = gpu.BatchSolver(gpu_ctx, configs.batched_static(3, seed=1, n_min=20, n_max=60))
    other = gpu.BatchSolver(gpu_ctx, configs.batched_static(4, seed=2, n_min=20, n_max=60))
    a.reset()
    a.step(5)
    snap = a.snapshot()
    other.reset()
    other.run()
    before, st_before = other.results()
    with pytest.raises(RuntimeError, match=r"gf_batch_restore failed \(1\).*different batch"):
        other.restore(snap)
    junk = np.zeros_like(snap)
    with pytest.raises(RuntimeError, match=r"gf_batch_restore failed \(1\).*not a batch snapshot"):
        a.restore(junk)
    after, st_after = other.results()
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    assert np.array_equal(st_before, st_after)
    # the snapshot still restores into its own batch
    a.restore(snap)
    a.run()
    a.close()
    other.close()

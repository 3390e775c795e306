"""Comparison of monitor lines (shared by the oracle and GPU tests)."""
import numpy as np


def monitor_close(mine, ref, tol=2e-6):
    """Monitor lines (31 columns: time, position, Euler rotation vector,
    load F and M, the same again, velocities, accelerations) against the
    reference's printed ones (%.6e): each block of columns within tol of its
    largest magnitude over the whole record, so that equilibrium residues of
    order 1e-8 N in a record of 1e4 N compare as the zeros they are."""
    mine, ref = np.asarray(mine), np.asarray(ref)
    assert mine.shape == ref.shape, (mine.shape, ref.shape)
    assert np.abs(mine[..., 0] - ref[..., 0]).max() <= 1e-9 * max(1.0, np.abs(ref[..., 0]).max())
    load = max(np.abs(ref[..., 7:19]).max(), 1e-300)
    for a, b in ((1, 4), (4, 7), (7, 10), (10, 13), (13, 16), (16, 19), (19, 25), (25, 31)):
        scale = np.abs(ref[..., a:b]).max()
        if 7 <= a < 19:
            # forces and moments in equilibrium can be pure round-off of the
            # other: below 1e-5 of the record's largest load they are noise
            scale = max(scale, 1e-5 * load)
        assert np.abs(mine[..., a:b] - ref[..., a:b]).max() <= tol * scale + 1e-12, (a, b)

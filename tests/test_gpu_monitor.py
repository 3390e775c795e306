"""Monitor lines from the device run (gf_batch_monitor: the monitored nodes'
state after every Sample-th converged step, recorded on the device inside
the captured Newton pass) against the reference's own monitor lines
(Node::WriteMonitor, recorded from the reference build) and the oracle's.
Stated tolerance, against both: each block of columns within 2e-6 of its
largest magnitude (the reference prints %.6e; forces and moments in
equilibrium compare against 1e-5 of the record's largest load, below which
they are round-off of the residual)."""
import numpy as np
import pytest

from giraffe_gb300 import gpu
from giraffe_gb300.model import Structure
from giraffe_gb300.monitor import node_lines
from oracle import oracle
from tests.monitor_check import monitor_close

pytestmark = pytest.mark.gpu

CASES = ["ref_monitor_chain.npz", "ref_monitor_plate.npz", "ref_monitor_tutorial10.npz",
         "ref_monitor_sequence.npz", "ref_tutorial04.npz"]


def _run(ctx, structs, rows=4096):
    b = gpu.BatchSolver(ctx, structs, ctx.opts(monitor_rows=rows))
    b.reset()
    b.run()
    out = [b.monitor(k) for k in range(len(structs))]
    finals, stats = b.results()
    b.close()
    return out, finals, stats


@pytest.mark.parametrize("name", CASES)
def test_monitor_lines_match_reference(gpu_ctx, golden, name):
    g = golden(name)
    s = Structure.from_inp(str(g["deck"]))
    [(lines, produced)], _, _ = _run(gpu_ctx, [s])
    assert produced == lines.shape[1]
    monitor_close(lines, g["monitor"])
    _, _, rec = oracle.solve(s, record_cap=4096)
    monitor_close(lines, rec["monitor"])


def test_monitored_structures_in_one_batch(gpu_ctx, golden):
    """Structures with and without a Monitor block in one batch: each keeps
    its own lines; the final states equal those of the same batch without
    monitoring (recording reads, never writes, the solver's state)."""
    structs = [Structure.from_inp(str(golden(n)["deck"])) for n in ("ref_monitor_chain.npz", "ref_monitor_plate.npz")]
    plain = Structure.from_inp(str(golden("ref_monitor_chain.npz")["deck"]))
    plain.monitor = None
    out, finals, stats = _run(gpu_ctx, structs + [plain])
    for k, n in enumerate(("ref_monitor_chain.npz", "ref_monitor_plate.npz")):
        monitor_close(out[k][0], golden(n)["monitor"])
    assert out[2][0].shape[0] == 0
    b = gpu.BatchSolver(gpu_ctx, structs + [plain])
    b.reset()
    b.run()
    f2, s2 = b.results()
    b.close()
    for a, c in zip(finals, f2):
        assert np.array_equal(a, c)
    assert np.array_equal(stats, s2)


def test_monitor_capacity(gpu_ctx, golden):
    """With room for fewer lines than the run produces, the first ones are
    kept and the count of all is reported."""
    g = golden("ref_monitor_tutorial10.npz")
    s = Structure.from_inp(str(g["deck"]))
    [(lines, produced)], _, _ = _run(gpu_ctx, [s], rows=10)
    assert lines.shape[1] == 11 and produced == g["monitor"].shape[1]
    monitor_close(lines, g["monitor"][:, :11])

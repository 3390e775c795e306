"""The multi-GPU path of bench.py on CPU ranks (gloo, world size 2, no GPU
work): both ranks build the same 2 x 512-chain workload, the LPT split
gives each a disjoint part, together they cover every chain once, the
estimated loads are within 1 % of each other, and the barrier and the
max / sum reductions bench.py uses for its timing agree across ranks.
Also the LPT split itself on a known case."""
import os
import socket
import sys

import pytest

from giraffe_gb300 import partition

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def test_lpt_split_balances_and_covers():
    costs = [7.0, 5.0, 4.0, 4.0, 3.0, 3.0, 2.0, 1.0, 1.0]
    parts = partition.lpt_partition(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = sorted(sum(costs[i] for i in p) for p in parts)
    assert loads == [10.0, 10.0, 10.0]
    # deterministic: ties go to the lower part
    assert parts == partition.lpt_partition(costs, 3)


def test_shape_estimate_matches_the_oracle_numbering():
    from giraffe_gb300 import configs
    from oracle import oracle

    for s in (configs.pipe_chain(30, 0.4, 0.03, [1.0, 0.0, 0.0]), configs.square_plate(8)):
        _, P, kl = oracle.first_tangent(s)
        n, kb, _, _, _ = partition.structure_shape(s)
        assert (n, kb) == (len(P), kl)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import argparse

    import torch.distributed as dist

    import bench

    r, w = bench.dist_init()
    assert (r, w) == (rank, world) and dist.get_backend() == "gloo"
    args = argparse.Namespace(chains=512, seed=0)
    structs, loads = bench.rank_structures(args, r, w)
    from giraffe_gb300 import configs

    allc = configs.batched_static(512 * w, seed=0)
    key = {(len(s.beams), float(s.sections[0][0]), tuple(s.loads[0].table.values[1][:3])): i
           for i, s in enumerate(allc)}
    mine = sorted(key[(len(s.beams), float(s.sections[0][0]), tuple(s.loads[0].table.values[1][:3]))]
                  for s in structs)
    gathered = [None] * w
    dist.all_gather_object(gathered, mine)
    bench.barrier(w)
    mx = bench.max_over_ranks(float(r + 1), w)
    sm = bench.sum_over_ranks(float(len(structs)), w)
    if r == 0:
        out.put((gathered, loads, mx, sm, len(allc)))
    dist.destroy_process_group()


def test_bench_ranks_split_one_workload_over_gloo():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered, loads, mx, sm, total = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    flat = sorted(i for part in gathered for i in part)
    assert flat == list(range(total)) and total == 1024
    assert not set(gathered[0]) & set(gathered[1])
    assert abs(loads[0] - loads[1]) <= 0.01 * max(loads)
    assert mx == 2.0 and sm == 1024.0

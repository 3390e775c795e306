"""Sharding a batch of independent structures across GPUs (one process per
GPU): greedy longest-processing-time (LPT) bin packing on an estimate of
each structure's work per Newton pass.

Structures share nothing, so no collective is needed on the data path:
every rank builds the same list, takes its own part and solves it as one
device batch; results are gathered on the host.  The reference has no
multi-process layer (it solves one model per process, src/main.cpp:55-62).

Work per Newton pass of a structure with n free DOFs, half-bandwidth kb,
N_e Beam_1 or Shell_1 elements and N nodes (FP64):

* factor and solve: 2 n kb^2 + 4 n kb flops (no-pivot band LU);
* element tangents: 9,000 flops per Beam_1 element, ~100,000 per Shell_1;
* assembly traffic: 8 [6 N + h N_e + c N_e + (2 kb + 1) n + n] bytes, with
  h + c = 80 doubles per Beam_1 element and 183 per Shell_1 element.

The estimate is flops / FP64 rate + bytes / HBM rate, with the rates of
one GB300 (1.25 TFLOP/s FP64, 6.8 TB/s); only ratios matter for the split.
"""
from __future__ import annotations

import heapq

import numpy as np

FP64_FLOPS = 1.25e12
HBM_BYTES = 6.8e12
BEAM_MOUNT_FLOPS = 9000.0
SHELL_MOUNT_FLOPS = 1.0e5


def structure_shape(s) -> tuple:
    """(free DOFs, half-bandwidth, Beam_1 elements, Shell_1 elements, nodes)
    of a Structure without numbering it on the device: free DOFs counted
    from the constraints and the element masks (6 per Beam_1 node, 3 on a
    Shell_1 corner and 6 on a midside node), the half-bandwidth of the
    node-major numbering from the element connectivity."""
    nn = s.n_nodes
    beams, shells = s.beams.array(), s.shells.array()
    active = np.zeros((nn, 6), dtype=bool)
    active[beams[:, :3].ravel()] = True
    active[shells[:, :3].ravel(), :3] = True
    active[shells[:, 3:6].ravel()] = True
    cons = np.asarray(s.constraints, dtype=bool) if s.constraints is not None else np.zeros((nn, 6), bool)
    free = active & ~cons
    cnt = free.sum(axis=1)
    first = np.cumsum(cnt) - cnt
    last = first + cnt - 1
    has = cnt > 0
    lo = np.where(has, first, np.iinfo(np.int64).max)
    hi = np.where(has, last, -1)
    kb = 0
    for conn in (beams[:, :3], shells[:, :6]):
        if len(conn):
            span = hi[conn].max(axis=1) - lo[conn].min(axis=1)
            span = span[has[conn].any(axis=1)]
            if len(span):
                kb = max(kb, int(span.max()))
    return int(free.sum()), kb, len(beams), len(shells), nn


def pass_cost(s) -> float:
    """Estimated seconds of one Newton pass of structure s on one GB300."""
    n, kb, nb, ns, nn = structure_shape(s)
    flops = 2.0 * n * kb * kb + 4.0 * n * kb + BEAM_MOUNT_FLOPS * nb + SHELL_MOUNT_FLOPS * ns
    bytes_ = 8.0 * (6.0 * nn + 80.0 * nb + 183.0 * ns + (2 * kb + 1) * n + n)
    return flops / FP64_FLOPS + bytes_ / HBM_BYTES


def lpt_partition(costs, n_parts: int) -> list:
    """Greedy LPT: items in decreasing cost, each to the part with the least
    load so far (ties to the lower part index, so every rank computes the
    same split).  Returns n_parts lists of item indices, each in increasing
    order."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, p) for p in range(n_parts)]
    parts = [[] for _ in range(n_parts)]
    for i in order:
        load, p = heapq.heappop(heap)
        parts[p].append(i)
        heapq.heappush(heap, (load + costs[i], p))
    return [sorted(x) for x in parts]


def shard(structures, rank: int, world: int):
    """This rank's structures (indices into `structures`) under the LPT split
    of their estimated Newton-pass costs, and the estimated load of every
    rank."""
    costs = [pass_cost(s) for s in structures]
    parts = lpt_partition(costs, world)
    loads = [sum(costs[i] for i in p) for p in parts]
    return parts[rank], loads

"""Served path: continuous batching of independent structures under a device
memory budget, through the gf_server_* C ABI (include/giraffe_gpu.h).

`Server` wraps one gf_server: `submit` queues a structure, `poll` advances the
device work and returns finished structures.  `run_stream` replays a timed
arrival stream against a server (submitting each structure at its arrival
time, polling in between) and reports per-request latency.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from .gpu import Context, _dp, gf_server_opts, gf_server_result, gf_server_status, lib
from .model import Structure


@dataclass
class Result:
    tag: int
    status: int
    final: np.ndarray  # n_nodes x 15 (position + rotation vector, Q row-major)
    stats: tuple       # converged steps, Newton iterations, bisections, aborted
    queued_ms: float
    total_ms: float


class Server:
    def __init__(self, ctx: Context, hbm_budget: int = 8 << 30, max_waves: int = 4, max_wave_structs: int = 128,
                 passes_per_chunk: int = 4, max_wave_passes: int = 0, precision: int = 0):
        self.ctx = ctx
        self.L = lib()
        o = gf_server_opts()
        self.L.gf_server_default_opts(C.byref(o))
        o.hbm_budget, o.max_waves, o.max_wave_structs, o.passes_per_chunk = (hbm_budget, max_waves,
                                                                             max_wave_structs, passes_per_chunk)
        o.max_wave_passes = max_wave_passes
        o.precision = precision  # GF_PREC_FP64 or GF_PREC_MIXED for every wave
        self.h = self.L.gf_server_create(ctx.h, C.byref(o))
        if not self.h:
            raise RuntimeError("gf_server_create failed: " + ctx.error())
        self.max_results = 256
        self._buf = (gf_server_result * self.max_results)()
        self._live = {}  # tag -> (descriptor handle, output array)
        self._next = 0

    def submit(self, structure: Structure, tag: int | None = None) -> int:
        if tag is None:
            tag = self._next
        self._next = max(self._next, tag + 1)
        h = structure.desc()  # holds the arrays the descriptor points to
        out = np.zeros((structure.n_nodes, 15))
        rc = self.L.gf_server_submit(self.h, C.byref(h.desc), _dp(out), tag)
        if rc != 0:
            raise RuntimeError(f"gf_server_submit failed ({rc}): {self.ctx.error()}")
        self._live[tag] = (h, out)
        return tag

    def poll(self) -> list:
        n = C.c_int(0)
        out = []
        while True:
            rc = self.L.gf_server_poll(self.h, self._buf, self.max_results, C.byref(n))
            if rc != 0:
                raise RuntimeError(f"gf_server_poll failed ({rc}): {self.ctx.error()}")
            for i in range(n.value):
                r = self._buf[i]
                _, arr = self._live.pop(r.tag)
                st = r.stats
                out.append(Result(r.tag, r.status, arr, (st.converged_steps, st.newton_iterations, st.bisections,
                                                         st.aborted), r.queued_ms, r.total_ms))
            if n.value < self.max_results:
                return out

    def status(self) -> dict:
        s = gf_server_status()
        self.L.gf_server_get_status(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in gf_server_status._fields_ if k != "pad"}

    def drain(self, timeout_s: float = 600.0) -> list:
        """Polls until every submitted structure is reported."""
        out = []
        t0 = time.perf_counter()
        while self._live:
            out += self.poll()
            if time.perf_counter() - t0 > timeout_s:
                raise TimeoutError(f"{len(self._live)} structures still in flight after {timeout_s} s")
        return out

    def close(self):
        if self.h:
            self.L.gf_server_destroy(self.h)
            self.h = None
        self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_arrivals(n: int, rate_hz: float, seed: int) -> np.ndarray:
    """Arrival times (s) of n requests of a Poisson process of rate rate_hz."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_hz, n))


def run_stream(server: Server, structures, arrivals, timeout_s: float = 600.0) -> dict:
    """Submits structures[i] at arrivals[i] seconds after the start (as soon as
    the host clock passes it), polling the server in between, until every
    result is back.  Latency of a request = the time its result was returned
    minus its scheduled arrival time."""
    n = len(structures)
    arrivals = np.asarray(arrivals, dtype=np.float64)
    done_at = np.full(n, np.nan)
    results = [None] * n
    t0 = time.perf_counter()
    i = 0
    remaining = n
    while remaining:
        now = time.perf_counter() - t0
        while i < n and arrivals[i] <= now:
            server.submit(structures[i], tag=i)
            i += 1
        for r in server.poll():
            done_at[r.tag] = time.perf_counter() - t0
            results[r.tag] = r
            remaining -= 1
        if now > arrivals[-1] + timeout_s:
            raise TimeoutError(f"{remaining} requests unfinished")
        if i < n and remaining == n - i and arrivals[i] > now:
            time.sleep(min(arrivals[i] - now, 1e-3))
    wall = time.perf_counter() - t0
    lat = (done_at - arrivals) * 1e3
    solves = sum(r.stats[0] for r in results)
    return {"results": results, "latency_ms": lat, "wall_s": wall, "solves": solves,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "solves_per_s": solves / wall, "requests_per_s": n / wall}

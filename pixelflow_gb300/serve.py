"""The serving form: a request loop with continuous batching on one GPU.

Requests (a geometry, grid, physics and a step count) arrive over time.  The
loop keeps every admitted case's fields resident in HBM inside one `Batch`;
a request is admitted as soon as its memory fits the HBM budget (and a slot
is free), in arrival order.  Each round advances every active case by up to
`chunk` steps: cases of up to `large_cells` cells in one persistent launch per
dimension, larger ones as full-GPU step graphs on their own streams at the
same time.  Requests that arrive while others are running join at the next
round and their work overlaps on the device with the cases already there.  A finished case's result (its
fields and norms) is read back, its slot and memory freed, and its latency
(completion minus arrival) recorded.

Each case's arithmetic is independent of what else is in the batch, so a
result is the same alone and in any mix (bit for bit; tests/test_gpu_serve.py).

Round policy: "rr" advances every active case each round; "srpt" advances
the cases with the least remaining work (cells x steps left) first, adding
cases in that order until a round holds at least `round_cells` cells, so the
GPU stays full while short requests finish early (a lower p50 at the same
throughput; the longest requests still finish last).  Both give every case
of a round the same `chunk` steps, so a round lasts as long as its slowest
case's chunk, and a cheap request with many steps needs many rounds.
"srpt_fill" keeps the shortest-remaining-work order but gives each case the
steps it runs alone in `round_ms` (a per-step cost model: a fixed launch
latency plus a per-cell time, one rate for cases in the persistent kernel,
one for full-GPU step graphs), and adds cases until the round's cell-steps
reach `round_rate` x `round_ms`; the case that does not fit whole gets the
steps that fill the rest.  The default rate, twice the ~1.3-1.6 G
cell-steps/s the GPU sustains on a mixed stream, keeps every round's GPU full
(measured on 32 Poisson requests: 1.3e9 gave p50 2.5 s at 1423
Mcell-steps/s, 2.6e9 2.1 s at 1558, 5.2e9 2.5 s at 1605).  Cheap requests then
finish in a round or two while the large ones fill the rest of the GPU.
"""
from __future__ import annotations

import dataclasses
import time
from collections import deque
from typing import Dict, List, Optional, Tuple

import numpy as np

from ._lib import PfError
from .batch import GIB, Batch, case_bytes
from .geometry import Request, to_pf_shapes


@dataclasses.dataclass
class Result:
    rid: int
    arrival_s: float
    admitted_s: float
    done_s: float
    cells: int
    steps: int
    max_div: float
    sor_error: float
    state: Optional[Dict[str, np.ndarray]] = None

    @property
    def latency_s(self) -> float:
        return self.done_s - self.arrival_s


class Server:
    # per-step device time of a case running alone, in ms: launch latency plus
    # cells x (ms per cell); measured on GB300 with clusters of 8 x 512 threads
    # (persistent kernel: 0.4-1.2 ms per step for 2D cases whose rows fit in
    # shared memory, up to ~125k cells; ~50 Mcell-steps/s for the others, which
    # sweep from global memory; step graphs: 0.4-0.6 ms per 2D step, ~1.5 G
    # cell-steps/s for large 3D cases)
    STEP_MS = 0.35
    ON_CHIP_CELLS = 125_000
    ON_CHIP_MS_PER_CELL = 7.0e-6
    CLUSTER_MS_PER_CELL = 2.0e-5
    GRAPH_MS_PER_CELL = 0.67e-6

    def __init__(self, hbm_budget_bytes: int = 150 * GIB, chunk: int = 25, cluster: int = 4, threads: int = 512,
                 max_cases: int = 1024, keep_state: bool = True, edge: float = 1.0, large_cells: int = 100000,
                 policy: str = "rr", round_cells: int = 24_000_000, batch=None, round_ms: float = 200.0,
                 round_rate: float = 2.6e9):
        # precision-form schedule (outer, inner) per (dim, shape), set by
        # tune_schedules; requests of other sizes keep their own settings
        self.schedules: Dict[Tuple[int, Tuple[int, ...]], Tuple[int, int]] = {}
        if policy not in ("rr", "srpt", "srpt_fill"):
            raise ValueError(f"unknown policy {policy!r}")
        self.large_cells = large_cells
        self.round_ms = round_ms
        self.round_work = round_rate * round_ms / 1e3  # cell-steps the GPU does in round_ms
        self.batch = batch if batch is not None else Batch(cluster=cluster, threads=threads, max_cases=max_cases,
                                                           hbm_budget_bytes=hbm_budget_bytes,
                                                           large_cells=large_cells)
        self.policy = policy
        self.round_cells = round_cells
        self.chunk = chunk
        self.keep_state = keep_state
        self.edge = edge
        self.peak_bytes = 0
        self.max_waiting = 0  # longest queue of arrived requests not yet admitted
        self.rounds = 0
        self.device_ms = 0.0

    def close(self):
        self.batch.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def tune_schedules(self, requests: List[Request], bound: float, steps: int = 5,
                       schedules=((1, 100), (2, 50), (4, 25)), use_cache: bool = True) -> Dict[str, list]:
        """The autotuner's outer x inner schedule for every grid size among
        `requests`: the fastest candidate whose error against the plain FP64
        step after `steps` steps stays within `bound` (else the fastest of
        the most accurate class), tuned as a single-case step on the first
        request of that size.  Later admissions of that size use it."""
        from .autotune import tune_schedule
        out = {}
        for r in requests:
            key = (r.dim, tuple(r.shape))
            if key in self.schedules:
                continue
            best, trials = tune_schedule(r.settings, r.shape, None, bound=bound, steps=steps, schedules=schedules,
                                         use_cache=use_cache, shapes=to_pf_shapes(r.shapes, r.dim))
            self.schedules[key] = tuple(best)
            out[f"{r.dim}D {r.shape[0]}"] = [list(best), [[t["outer"], t["inner"], round(t["ms"], 3),
                                                     max(t["rel_l2"].values())] for t in trials]]
        return out

    def _settings(self, r: Request):
        sch = self.schedules.get((r.dim, tuple(r.shape)))
        return r.settings if sch is None else r.settings.replace(outer_max=sch[0], inner_sweeps=sch[1])

    def run(self, requests: List[Request], realtime: bool = True) -> List[Result]:
        """Serve `requests` (sorted by arrival).  With realtime=True arrivals
        follow the wall clock from the start of the call; otherwise every
        request is available at once (a closed batch)."""
        reqs = sorted(requests, key=lambda r: r.arrival_s)
        for r in reqs:
            need = case_bytes(r.settings, r.shape, self.large_cells)
            if need > self.batch.memory()[1]:
                raise ValueError(f"request {r.rid} needs {need} bytes, more than the whole budget")
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        incoming = deque(reqs)
        waiting: deque = deque()
        active: Dict[int, dict] = {}
        results: List[Result] = []
        while incoming or waiting or active:
            t = now()
            while incoming and (not realtime or incoming[0].arrival_s <= t):
                waiting.append(incoming.popleft())
            self.max_waiting = max(self.max_waiting, len(waiting))
            # admission in arrival order while memory and slots allow
            while waiting:
                r = waiting[0]
                try:
                    slot = self.batch.add_shapes(self._settings(r), r.shape, to_pf_shapes(r.shapes, r.dim),
                                                 self.edge)
                except PfError as e:
                    if e.code in (-3, -7):  # over budget / no slot: wait for a case to finish
                        break
                    raise
                waiting.popleft()
                active[slot] = {"req": r, "left": r.steps, "admitted": now()}
                self.peak_bytes = max(self.peak_bytes, self.batch.memory()[0])
            if not active:
                if incoming and realtime:
                    time.sleep(max(0.0, min(0.005, incoming[0].arrival_s - now())))
                continue
            slots, steps = self._plan(active)
            self.batch.step_slots(slots, steps)
            self.rounds += 1
            self.device_ms += self.batch.last_ms()
            for s, k in zip(slots, steps):
                a = active[s]
                a["left"] -= k
                if a["left"] == 0:
                    md, se = self.batch.norms(s)
                    st = self.batch.get_state(s) if self.keep_state else None
                    r = a["req"]
                    results.append(Result(r.rid, r.arrival_s, a["admitted"], now(), r.cells, r.steps, md, se, st))
                    self.batch.remove(s)
                    del active[s]
        return sorted(results, key=lambda x: x.rid)

    def _step_ms(self, cells: int, dim: int = 2) -> float:
        """Modelled device time of one step of a case running alone."""
        if cells > self.large_cells:
            per_cell = self.GRAPH_MS_PER_CELL
        elif dim == 2 and cells <= self.ON_CHIP_CELLS:
            per_cell = self.ON_CHIP_MS_PER_CELL
        else:
            per_cell = self.CLUSTER_MS_PER_CELL
        return self.STEP_MS + cells * per_cell

    def _plan(self, active: Dict[int, dict]) -> Tuple[List[int], List[int]]:
        """The slots advanced this round and their step counts (see the module
        docstring)."""
        if self.policy == "rr":
            slots = list(active)
            return slots, [min(self.chunk, active[s]["left"]) for s in slots]
        order = sorted(active, key=lambda s: (active[s]["req"].cells * active[s]["left"], active[s]["req"].rid))
        chosen, steps, cells, work = [], [], 0, 0
        for s in order:
            a = active[s]
            c = a["req"].cells
            if self.policy == "srpt":
                chosen.append(s)
                steps.append(min(self.chunk, a["left"]))
                cells += c
                if cells >= self.round_cells:
                    break
                continue
            k = min(a["left"], max(1, int(self.round_ms / self._step_ms(c, a["req"].dim))))
            room = self.round_work - work
            if chosen and room < c:  # the round is full
                break
            k = min(k, max(1, int(room // c)))  # a case that does not fit whole fills the rest
            chosen.append(s)
            steps.append(k)
            work += c * k
        return chosen, steps


def summarize(results: List[Result], wall_s: float) -> dict:
    lat = np.array([r.latency_s for r in results])
    cell_steps = sum(r.cells * r.steps for r in results)
    return {"requests": len(results), "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
            "wall_s": wall_s, "cell_steps": cell_steps, "mcell_steps_per_s": cell_steps / wall_s / 1e6,
            "nonfinite_results": int(sum(1 for r in results if not np.isfinite(r.max_div)))}

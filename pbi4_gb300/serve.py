"""Continuous-batching request loop for estimator boxes on one GPU.

Requests (a box configuration + host positions) arrive at any time.  The loop
keeps one resident plan per (configuration, slot) -- grids, cuFFT plans, bin and
shell tables, triangle counts -- and runs admitted boxes on `slots` CUDA streams
so several boxes are on the device at once.  Admission is by device footprint:
a box starts when a slot is free and the plans it needs fit under the HBM
budget; idle plans are evicted least-recently-used to make room.  Requests of
the same configuration reuse the same plans back to back.

Each box is issued asynchronously on its slot's stream: pinned host -> device
copy of the positions, the plan's kernels, device -> pinned host copy of the
outputs, then an event; the loop thread polls events, so new requests are
admitted while others are still running (no per-box synchronisation of the
device).  Latency = completion time - arrival time; p50/p99 are reported by
``stats()``.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from .estimator import Estimator, EstimatorConfig, footprint


@dataclass
class Request:
    cfg: EstimatorConfig
    pos: np.ndarray                   # (3, npart) float64 in [0, 1)
    rid: int = 0
    t_arrival: float = field(default_factory=time.perf_counter)


@dataclass
class Result:
    rid: int
    pout: np.ndarray
    bout: np.ndarray | None
    t_arrival: float
    t_start: float
    t_done: float

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival


class _Slot:
    def __init__(self, torch, idx):
        self.idx = idx
        self.stream = torch.cuda.Stream()
        self.busy = None   # (request, future, plan, event, host outputs, t_start)


class Server:
    def __init__(self, hbm_budget_bytes: int, slots: int = 4, device: int = 0, max_npart: int = 10_000_000):
        import torch
        self.torch = torch
        torch.cuda.set_device(device)
        self.budget = int(hbm_budget_bytes)
        self.max_npart = int(max_npart)
        self.slots = [_Slot(torch, k) for k in range(slots)]
        self.plans: "collections.OrderedDict[tuple, Estimator]" = collections.OrderedDict()  # (cfg key, slot) -> plan
        self.plan_bytes: dict[tuple, int] = {}
        self.queue: "collections.deque[tuple[Request, Future]]" = collections.deque()
        self.lock = threading.Condition()
        self.results: list[Result] = []
        self.rejected = 0
        self.evictions = 0
        self._stop = False
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()

    # ---------------------------------------------------------------- API ---
    def submit(self, req: Request) -> Future:
        fut: Future = Future()
        if req.pos.shape[1] > self.max_npart:
            self.rejected += 1
            fut.set_exception(ValueError("npart above the server's max_npart"))
            return fut
        with self.lock:
            self.queue.append((req, fut))
            self.lock.notify()
        return fut

    def close(self, wait: bool = True):
        with self.lock:
            self._stop = True
            self.lock.notify()
        if wait:
            self._thread.join()
        for p in self.plans.values():
            p.close()
        self.plans.clear()

    def resident_bytes(self) -> int:
        return sum(self.plan_bytes.values())

    def stats(self) -> dict:
        lat = np.array([r.latency for r in self.results]) if self.results else np.zeros(1)
        if not self.results:
            return {"n": 0}
        t0 = min(r.t_arrival for r in self.results)
        t1 = max(r.t_done for r in self.results)
        return {"n": len(self.results), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
                "boxes_per_s": len(self.results) / max(t1 - t0, 1e-9), "evictions": self.evictions,
                "rejected": self.rejected, "resident_gb": self.resident_bytes() / 1e9}

    # --------------------------------------------------------------- loop ---
    def _plan_for(self, cfg: EstimatorConfig, slot: _Slot, npart: int):
        key = (cfg.key(), slot.idx)
        if key in self.plans:
            self.plans.move_to_end(key)
            return self.plans[key]
        need = footprint(cfg, self.max_npart)
        if need > self.budget:
            raise MemoryError(f"plan footprint {need / 1e9:.2f} GB exceeds the HBM budget {self.budget / 1e9:.2f} GB")
        # evict idle plans (least recently used first) until the new one fits
        while self.resident_bytes() + need > self.budget:
            victim = None
            for k in self.plans:
                if not any(s.busy is not None and s.busy[2] is self.plans[k] for s in self.slots):
                    victim = k
                    break
            if victim is None:
                return None  # everything resident is busy: wait for a completion
            self.plans.pop(victim).close()
            self.plan_bytes.pop(victim)
            self.evictions += 1
            self.torch.cuda.empty_cache()
        plan = Estimator(cfg)
        self.plans[key] = plan
        self.plan_bytes[key] = need
        return plan

    def _start(self, slot: _Slot, req: Request, fut: Future, plan: Estimator):
        torch = self.torch
        npart = req.pos.shape[1]
        plan.set_stream(slot.stream)
        with torch.cuda.stream(slot.stream):
            hpos = torch.from_numpy(np.ascontiguousarray(req.pos, dtype=np.float64))
            if not hpos.is_pinned():
                hpos = hpos.pin_memory()
            dpos = torch.empty((3, npart), dtype=torch.float64, device="cuda")
            dpos.copy_(hpos, non_blocking=True)
            pout_d, bout_d = plan.alloc_outputs()
            plan.run_device(npart, dpos, pout_d, bout_d)
            pout_h = torch.empty(pout_d.shape[::-1], dtype=torch.float64, pin_memory=True)
            pout_h.copy_(pout_d.t(), non_blocking=True)
            bout_h = None
            if bout_d is not None:
                bout_h = torch.empty(bout_d.shape[::-1], dtype=torch.float64, pin_memory=True)
                bout_h.copy_(bout_d.t(), non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(slot.stream)
        # keep every buffer of the in-flight box alive until its event completes
        slot.busy = (req, fut, plan, ev, (pout_h, bout_h, hpos, dpos, pout_d, bout_d), time.perf_counter())

    def _finish(self, slot: _Slot):
        req, fut, plan, ev, (pout_h, bout_h, *_), t_start = slot.busy
        pout = pout_h.numpy().T
        bout = None if bout_h is None else bout_h.numpy().T
        res = Result(req.rid, pout, bout, req.t_arrival, t_start, time.perf_counter())
        self.results.append(res)
        slot.busy = None
        fut.set_result(res)

    def _loop(self):
        while True:
            progressed = False
            for s in self.slots:
                if s.busy is not None and s.busy[3].query():
                    self._finish(s)
                    progressed = True
            with self.lock:
                if self._stop and not self.queue and all(s.busy is None for s in self.slots):
                    return
                free = [s for s in self.slots if s.busy is None]
                while free and self.queue:
                    req, fut = self.queue[0]
                    # prefer a free slot that already holds a plan for this configuration
                    key = req.cfg.key()
                    free.sort(key=lambda s: (key, s.idx) not in self.plans)
                    slot = free[0]
                    try:
                        plan = self._plan_for(req.cfg, slot, req.pos.shape[1])
                    except MemoryError as e:  # can never fit: reject this request
                        self.queue.popleft()
                        self.rejected += 1
                        fut.set_exception(e)
                        continue
                    if plan is None:
                        break
                    self.queue.popleft()
                    try:
                        self._start(slot, req, fut, plan)
                    except Exception as e:  # report per request; keep serving
                        slot.busy = None
                        fut.set_exception(e)
                        continue
                    free.remove(slot)
                    progressed = True
                if not progressed:
                    if not self.queue and all(s.busy is None for s in self.slots) and not self._stop:
                        self.lock.wait(timeout=0.05)
            if not progressed:
                time.sleep(0.0002)

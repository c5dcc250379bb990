"""Continuous-batching request loop for estimator boxes on one GPU.

Requests (a box configuration + host positions) arrive at any time.  The loop
keeps resident plans per configuration -- grids, cuFFT plans, bin and shell
tables, triangle counts, shell-map buffers, captured graphs -- and runs admitted
work on `slots` CUDA streams so several boxes are on the device at once; an idle
plan runs on whichever slot is free, and a second instance of a configuration
is built only when the first is busy.

Batching: when a slot frees up, the request at the head of the queue and up to
`batch - 1` further queued requests of the same configuration (the same grid,
binning and precision: same-size boxes) form one batch, and the whole batch is
one launch of a CUDA graph the plan captured for that batch size
(pbi4g_plan_graph_run_host): per-box particle counts and their normalisation
factors are read from device memory, so one captured graph serves any counts
up to the server's max_npart.  Configurations the captured form does not cover
(FP64 plans, grids that are not a multiple of 16 or below 32, weighted boxes) run box by
box through the direct path on the same slots.

Admission is by device footprint: a batch starts when a slot is free and the
plan it needs fits under the HBM budget; idle plans are evicted least recently
used to make room, and a request whose plan can never fit is rejected.  The
plans that run on one slot share its assignment record buffers (AssignScratch,
3.2 GB at 10^7 particles), so a resident plan holds only its grids, tables and
maps.  Each
batch is issued asynchronously on its slot's stream (pageable positions are
staged by the driver, outputs land in pinned buffers) followed by an event; the
loop thread polls events, so new requests are admitted while others run.
Latency = completion time - arrival time; p50/p99 are reported by ``stats()``.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from .estimator import AssignScratch, Estimator, EstimatorConfig, footprint, scratch_footprint, uses_owner_work


@dataclass
class Request:
    cfg: EstimatorConfig
    pos: np.ndarray                   # (3, npart) float64 in [0, 1)
    rid: int = 0
    weight: np.ndarray | None = None
    t_arrival: float = field(default_factory=time.perf_counter)


@dataclass
class Result:
    rid: int
    pout: np.ndarray
    bout: np.ndarray | None
    t_arrival: float
    t_start: float
    t_done: float
    batch: int = 1
    plan_s: float = 0.0     # seconds the loop spent building the batch's plan (0: resident)
    evictions: int = 0      # plans evicted to make room for it

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival

    @property
    def queue_s(self) -> float:
        """Arrival to the batch's start on a slot (includes the plan build)."""
        return self.t_start - self.t_arrival

    @property
    def service_s(self) -> float:
        """The batch's start on its slot to its completion being seen by the loop."""
        return self.t_done - self.t_start


def graph_capable(cfg: EstimatorConfig) -> bool:
    """Configurations the captured (graph) form covers: FP32-family plans on the
    grids the owner-computes assignment takes (multiples of 16 from 32 to 2048)."""
    g = int(cfg.grid)
    return cfg.precision != "fp64" and g % 16 == 0 and 32 <= g <= 2048


class _Slot:
    def __init__(self, torch, idx, scratch=None):
        self.idx = idx
        self.stream = torch.cuda.Stream()
        self.scratch = scratch  # assignment buffers of the plans that run on this slot
        self.busy = None   # (requests, futures, plan, event, keep-alive objects, t_start)


class Server:
    def __init__(self, hbm_budget_bytes: int, slots: int = 4, device: int = 0, max_npart: int = 10_000_000,
                 batch: int = 4, lookahead: int = 64, shared_scratch: bool = True, scratch_grid_max: int = 1024):
        import torch
        self.torch = torch
        torch.cuda.set_device(device)
        self.budget = int(hbm_budget_bytes)
        self.max_npart = int(max_npart)
        self.batch = int(batch)
        self.lookahead = int(lookahead)
        # one set of assignment record buffers per slot, shared by every plan up to
        # scratch_grid_max that runs there (a plan's own would be 3.2 GB at 10^7
        # particles), counted as resident; larger grids keep their own
        self.shared_scratch = bool(shared_scratch)
        self.scratch_grid_max = int(scratch_grid_max)
        self.slots = [_Slot(torch, k, AssignScratch(self.scratch_grid_max, self.max_npart, self.batch)
                            if self.shared_scratch else None) for k in range(slots)]
        self.fixed_bytes = sum(sl.scratch.bytes for sl in self.slots if sl.scratch is not None)
        # (cfg key, instance) -> plan, least recently used first
        self.plans: "collections.OrderedDict[tuple, Estimator]" = collections.OrderedDict()
        self.plan_bytes: dict[tuple, int] = {}
        self.queue: "collections.deque[tuple[Request, Future]]" = collections.deque()
        self.lock = threading.Condition()
        self.results: list[Result] = []
        self.rejected = 0
        self.failed = 0       # requests that ended in an error other than a rejection
        self.cancelled = 0    # requests cancelled while queued
        self.evictions = 0
        self.plans_built = 0
        self.batches = 0
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

    def warm(self, cfgs):
        """Build the resident plans of these configurations on every slot ahead of
        the traffic (plan creation, tables, triangle counts, graph buffers)."""
        with self.lock:
            for cfg in cfgs:
                if self._plan_for(cfg, self.slots[0]) is None:
                    break
            self.plans_built = 0  # counts the plans built while serving
        self.torch.cuda.synchronize()

    def close(self, wait: bool = True):
        with self.lock:
            self._stop = True
            self.lock.notify()
        if wait:
            self._thread.join()
        for p in self.plans.values():
            p.close()
        self.plans.clear()
        for sl in self.slots:
            if sl.scratch is not None:
                sl.scratch.close()
                sl.scratch = None

    def resident_bytes(self) -> int:
        return self.fixed_bytes + sum(self.plan_bytes.values())

    def stats(self) -> dict:
        """Latency percentiles and throughput of the completed requests, with the
        latency split into queue wait (arrival to the batch's start, plan build
        included) and service (start to completion), and what the slowest 1% of
        requests waited on."""
        if not self.results:
            return {"n": 0}
        lat = np.array([r.latency for r in self.results])
        q = np.array([r.queue_s for r in self.results])
        sv = np.array([r.service_s for r in self.results])
        t0 = min(r.t_arrival for r in self.results)
        t1 = max(r.t_done for r in self.results)
        p99 = float(np.percentile(lat, 99))
        tail = [r for r in self.results if r.latency >= p99]
        return {"n": len(self.results), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": p99 * 1e3, "mean_ms": float(lat.mean() * 1e3),
                "queue_p50_ms": float(np.percentile(q, 50) * 1e3), "queue_p99_ms": float(np.percentile(q, 99) * 1e3),
                "service_p50_ms": float(np.percentile(sv, 50) * 1e3),
                "service_p99_ms": float(np.percentile(sv, 99) * 1e3),
                "tail": {"requests": len(tail), "queue_ms": float(np.mean([r.queue_s for r in tail]) * 1e3),
                         "service_ms": float(np.mean([r.service_s for r in tail]) * 1e3),
                         "with_plan_build": sum(1 for r in tail if r.plan_s > 0),
                         "plan_build_ms": float(np.mean([r.plan_s for r in tail]) * 1e3),
                         "evictions": sum(r.evictions for r in tail),
                         "mean_batch": float(np.mean([r.batch for r in tail]))},
                "boxes_per_s": len(self.results) / max(t1 - t0, 1e-9), "evictions": self.evictions,
                "rejected": self.rejected, "failed": self.failed, "cancelled": self.cancelled,
                "batches": self.batches, "plans_built": self.plans_built,
                "mean_batch": len(self.results) / max(1, self.batches), "resident_gb": self.resident_bytes() / 1e9}

    # --------------------------------------------------------------- loop ---
    def _footprint(self, cfg: EstimatorConfig) -> int:
        need = footprint(cfg, self.max_npart)
        if self._shares(cfg):
            need -= scratch_footprint(cfg.grid, self.max_npart)  # held by the slots' scratch
        elif graph_capable(cfg):
            need += self.batch * 3 * self.max_npart * 8  # its own graph position slots
        return need

    def _shares(self, cfg: EstimatorConfig) -> bool:
        return self.shared_scratch and uses_owner_work(cfg) and int(cfg.grid) <= self.scratch_grid_max

    def _scratch_for(self, cfg: EstimatorConfig, slot: _Slot):
        return slot.scratch if self._shares(cfg) else None

    def _busy(self, plan) -> bool:
        return any(s.busy is not None and s.busy[2] is plan for s in self.slots)

    def _plan_for(self, cfg: EstimatorConfig, slot: _Slot):
        ck = cfg.key()
        insts = [k for k in self.plans if k[0] == ck]
        for k in insts:
            plan = self.plans[k]
            if not self._busy(plan):
                self.plans.move_to_end(k)
                if plan.stream is not slot.stream:
                    plan.set_stream(slot.stream)
                    plan.stream = slot.stream
                plan.use_scratch(self._scratch_for(cfg, slot))
                return plan
        key = (ck, max((k[1] for k in insts), default=-1) + 1)
        need = self._footprint(cfg)
        if need + self.fixed_bytes > self.budget:
            raise MemoryError(f"plan footprint {need / 1e9:.2f} GB (beside {self.fixed_bytes / 1e9:.2f} GB of slot "
                              f"scratch) exceeds the HBM budget {self.budget / 1e9:.2f} GB")
        # evict idle plans (least recently used first) until the new one fits
        while self.resident_bytes() + need > self.budget:
            victim = None
            for k in self.plans:
                if not self._busy(self.plans[k]):
                    victim = k
                    break
            if victim is None:
                return None  # everything resident is busy: wait for a completion
            self.plans.pop(victim).close()
            self.plan_bytes.pop(victim)
            self.evictions += 1
            self.torch.cuda.empty_cache()
        plan = Estimator(cfg, stream=slot.stream)
        plan.stream = slot.stream
        plan.use_scratch(self._scratch_for(cfg, slot))
        if graph_capable(cfg):
            plan.graph_build(self.batch, self.max_npart)
        self.plans[key] = plan
        self.plan_bytes[key] = need
        self.plans_built += 1
        return plan

    def _take_batch(self):
        """The head request and up to batch-1 queued requests of the same
        configuration, each moved to the running state (a request cancelled
        while queued is dropped here, and cannot be cancelled once it runs)."""
        req, fut = self.queue[0]
        if not graph_capable(req.cfg) or req.weight is not None:
            self.queue.popleft()
            return [(req, fut)] if fut.set_running_or_notify_cancel() else []
        key = req.cfg.key()
        picked = [0]
        for k in range(1, min(len(self.queue), self.lookahead)):
            if len(picked) == self.batch:
                break
            r, _ = self.queue[k]
            if r.weight is None and r.cfg.key() == key:
                picked.append(k)
        items = [self.queue[k] for k in picked]
        for k in reversed(picked):
            del self.queue[k]
        return [(r, f) for r, f in items if f.set_running_or_notify_cancel()]

    def _drop_cancelled_head(self):
        while self.queue and self.queue[0][1].cancelled():
            self.queue.popleft()
            self.cancelled += 1

    def _start(self, slot: _Slot, items, plan: Estimator, plan_s: float = 0.0, evicted: int = 0):
        torch = self.torch
        reqs = [r for r, _ in items]
        futs = [f for _, f in items]
        t_start = time.perf_counter()
        keep = []
        if plan.graph_ready and all(r.weight is None for r in reqs):
            pos = [np.ascontiguousarray(r.pos, dtype=np.float64) for r in reqs]
            pouts = [torch.empty((plan.nbins_ps, 5), dtype=torch.float64, pin_memory=True) for _ in reqs]
            bouts = ([torch.empty((plan.itot, plan.brows), dtype=torch.float64, pin_memory=True) for _ in reqs]
                     if plan.itot else None)
            plan.graph_run_host(pos, [p.numpy() for p in pouts], [b.numpy() for b in bouts] if bouts else None)
            outs = [(pouts[b].numpy().T, bouts[b].numpy().T if bouts else None) for b in range(len(reqs))]
            keep = [pos, pouts, bouts]
        else:
            # direct path, one box: device copies on the slot stream, outputs to pinned buffers
            r = reqs[0]
            npart = r.pos.shape[1]
            with torch.cuda.stream(slot.stream):
                hpos = torch.from_numpy(np.ascontiguousarray(r.pos, dtype=np.float64))
                dpos = torch.empty((3, npart), dtype=torch.float64, device="cuda")
                dpos.copy_(hpos, non_blocking=True)
                dw = None
                if r.weight is not None:
                    dw = torch.from_numpy(np.ascontiguousarray(r.weight, dtype=np.float64)).cuda(non_blocking=True)
                pout_d, bout_d = plan.alloc_outputs()
                plan.run_device(npart, dpos, pout_d, bout_d, weight=dw)
                pout_h = torch.empty(pout_d.shape[::-1], dtype=torch.float64, pin_memory=True)
                pout_h.copy_(pout_d.t(), non_blocking=True)
                bout_h = None
                if bout_d is not None:
                    bout_h = torch.empty(bout_d.shape[::-1], dtype=torch.float64, pin_memory=True)
                    bout_h.copy_(bout_d.t(), non_blocking=True)
            outs = [(pout_h.numpy().T, None if bout_h is None else bout_h.numpy().T)]
            keep = [hpos, dpos, dw, pout_d, bout_d, pout_h, bout_h]
        ev = torch.cuda.Event()
        ev.record(slot.stream)
        self.batches += 1
        # every buffer of the batch in flight stays alive until its event completes
        slot.busy = (reqs, futs, plan, ev, (outs, keep), t_start, plan_s, evicted)

    def _finish(self, slot: _Slot):
        reqs, futs, plan, ev, (outs, _), t_start, plan_s, evicted = slot.busy
        slot.busy = None
        t_done = time.perf_counter()
        err = None
        try:
            plan.check()  # the slot's work is complete: this only reads the launch error flags
        except Exception as e:  # a bounded wait in a tensor-core launch gave up
            err = e
        for r, f, (po, bo) in zip(reqs, futs, outs):
            if err is not None:
                self.failed += 1
                f.set_exception(err)
                continue
            res = Result(r.rid, po.copy(), None if bo is None else bo.copy(), r.t_arrival, t_start, t_done, len(reqs),
                         plan_s, evicted)
            self.results.append(res)
            f.set_result(res)

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
                self._drop_cancelled_head()
                while free and self.queue:
                    req, fut = self.queue[0]
                    slot = free[0]
                    t_plan, ev0, built0 = time.perf_counter(), self.evictions, self.plans_built
                    try:
                        plan = self._plan_for(req.cfg, slot)
                    except MemoryError as e:  # can never fit: reject this request
                        self.queue.popleft()
                        self.rejected += 1
                        if fut.set_running_or_notify_cancel():
                            fut.set_exception(e)
                        self._drop_cancelled_head()
                        continue
                    except Exception as e:  # plan creation failed (e.g. out of memory): report, keep serving
                        self.queue.popleft()
                        self.failed += 1
                        if fut.set_running_or_notify_cancel():
                            fut.set_exception(e)
                        self._drop_cancelled_head()
                        continue
                    if plan is None:
                        break
                    items = self._take_batch()
                    if not items:   # the batch's requests were all cancelled
                        self._drop_cancelled_head()
                        continue
                    plan_s = time.perf_counter() - t_plan if self.plans_built > built0 else 0.0
                    try:
                        self._start(slot, items, plan, plan_s, self.evictions - ev0)
                    except Exception as e:  # report per request; keep serving
                        slot.busy = None
                        self.failed += len(items)
                        for _, f in items:
                            f.set_exception(e)
                        self._drop_cancelled_head()
                        continue
                    free.remove(slot)
                    progressed = True
                if not progressed:
                    if not self.queue and all(s.busy is None for s in self.slots) and not self._stop:
                        self.lock.wait(timeout=0.05)
            if not progressed:
                time.sleep(0.0002)

"""Reconstruction serving loop over libnufft3d (continuous batching).

Requests are iNUFT reconstructions: (trajectory om, image size N, kernel
options, raw data [M, nc], iterations, damp).  The server

* keeps trajectory state resident on the device: one base plan (sorted
  samples, tiles, deapodization, density) per trajectory key, in an LRU
  cache;
* admits work by HBM footprint: a batch starts only when the plan tables (if
  the trajectory is new) plus the batch's work buffers fit in the budget, with
  idle cached plans evicted first;
* runs `slots` batches at once, each on its own CUDA stream through a shared
  plan handle (nufft3d_plan_share), so requests that arrive while others are
  on the GPU start as soon as a slot and memory are free and their kernels
  overlap on the device;
* merges queued requests with the same trajectory and settings into one
  multi-coil solve (coils are independent systems, so each request's result is
  the same alone and merged, up to floating-point rounding).

`run_plain` is the reference-style baseline: one request at a time, each
building its own plan (constructor + density) and solving, as
`obj = nufft_3d(om, N, ...); im = obj.iNUFT(raw, maxit, damp)` does.
"""
from __future__ import annotations

import ctypes
import hashlib
import threading
import time
from collections import OrderedDict
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .nufft_3d import nufft_3d


@dataclass(eq=False)
class Request:
    om: np.ndarray                 # [3, M] cycles/FOV
    N: int
    raw: np.ndarray                # [M, nc] complex
    maxit: int = 20
    damp: float = 0.0
    opts: dict = field(default_factory=lambda: {"J": 6, "u": 2})
    solver: str = "cg"
    tol: float = 0.0
    arrival: float = 0.0           # seconds from the start of the run
    key: str = ""
    # filled by the server
    t_start: float = 0.0
    t_done: float = 0.0
    plan_s: float = 0.0            # time spent building this request's plan (0 if resident)
    result: np.ndarray = None

    def __post_init__(self):
        if not self.key:
            h = hashlib.sha1()
            h.update(np.ascontiguousarray(self.om, dtype=np.float64).tobytes())
            h.update(repr((int(self.N), sorted(self.opts.items()))).encode())
            self.key = h.hexdigest()

    @property
    def nc(self):
        return 1 if self.raw.ndim == 1 else self.raw.shape[1]

    @property
    def latency(self):
        return self.t_done - self.arrival


def _gib(x):
    return x / 2 ** 30


class ReconServer:
    """Continuous-batching reconstruction server on one GPU."""

    def __init__(self, slots=4, hbm_budget=None, device=0, max_batch_coils=16, cache_size=8):
        import torch
        self.torch = torch
        self.device = device
        torch.cuda.set_device(device)
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(device)
            hbm_budget = int(free * 0.8)
        self.budget = int(hbm_budget)
        self.slots = slots
        self.max_batch_coils = max_batch_coils
        self.cache_size = cache_size
        self.cache = OrderedDict()      # key -> {"plan": nufft_3d, "bytes": int, "users": int}
        self.used = 0                   # bytes reserved (cached tables + running batches)
        self.queue = []                 # pending (Request, Future)
        self.cv = threading.Condition()
        self.stop = False
        self.errors = []
        self.handle = [None] * slots      # per slot: (key, shared handle) kept between batches
        self.busy = [False] * slots       # per slot: a batch is between admission and finish
        self.slot_res = [(None, 0)] * slots  # per slot: (key, bytes reserved for its handle)
        self.workers = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(slots)]
        for w in self.workers:
            w.start()

    # ------------------------------------------------------------ public
    def submit(self, req: Request) -> Future:
        fut = Future()
        with self.cv:
            self.queue.append((req, fut))
            self.cv.notify_all()
        return fut

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for w in self.workers:
            w.join()
        for h in self.handle:
            if h is not None:
                h[1].close()
        for e in self.cache.values():
            e["plan"].close()
        self.cache.clear()

    # ---------------------------------------------------------- internals
    @staticmethod
    def _plan_bytes_estimate(req):
        N = int(req.N)
        K = 2 * int(np.ceil(N * req.opts.get("u", 2) / 2))
        M = req.om.shape[1] if req.om.ndim == 2 else req.om.size // 3
        # sorted records, perm, inv, d, d_orig, U, tiles
        b = M * (16 + 4 + 4 + 4 + 4) + N ** 3 * 4 + (K // 8 + 1) ** 3 * 20
        # the stored H (8-byte entries, rows padded to chunks of 8) and its
        # transpose H' (the same entries per grid point, plus row headers and
        # bundle padding: about 12 entries per sample more) that plans with
        # ceil(J/2) <= 3 build when they fit
        J = float(req.opts.get("J", 4))
        if int(np.ceil(J / 2)) <= 3:
            taps = 4.0 / 3.0 * np.pi * (J / 2) ** 3 if req.opts.get("radial", 1) else J ** 3
            b += int(M * ((taps + 4) * 8 + 4))
            b += int(M * (taps + 12) * 8)
        return b

    @staticmethod
    def _work_bytes(req, nc):
        N = int(req.N)
        K = 2 * int(np.ceil(N * req.opts.get("u", 2) / 2))
        M = req.om.shape[1] if req.om.ndim == 2 else req.om.size // 3
        c8 = 8 * nc
        fft = (K * N * N + K * K * N + K ** 3) * c8
        solver = 7 * N ** 3 * c8
        stage = M * c8 + M * 4 + N ** 3 * c8
        return fft + M * c8 + solver + stage

    def _take_batch(self):
        """First queued request plus later ones with the same key and settings."""
        req0, fut0 = self.queue[0]
        batch = [(req0, fut0)]
        coils = req0.nc
        for item in self.queue[1:]:
            r = item[0]
            if (r.key == req0.key and r.maxit == req0.maxit and r.damp == req0.damp and r.solver == req0.solver
                    and r.tol == req0.tol and coils + r.nc <= self.max_batch_coils):
                batch.append(item)
                coils += r.nc
        return batch, coils

    def _release_slot(self, slot):
        """Under the lock: close the slot's idle handle and credit back the
        work-buffer bytes reserved for it.  Its trajectory's tables stay with
        the cached base plan (if any), whose bytes are counted separately."""
        cur = self.handle[slot]
        if cur is not None:
            cur[1].close()
            self.handle[slot] = None
        self.used -= self.slot_res[slot][1]
        self.slot_res[slot] = (None, 0)

    def _evict_for(self, need, slot, keep):
        """Under the lock: free memory for `need` more bytes.  First cached
        trajectories that nothing uses (tables that no handle holds are freed
        with their base plan); then the handles of idle slots, which pin their
        trajectory and hold work buffers, and the trajectories they released.
        The requesting slot has already closed a handle on another key; the
        key the request needs stays."""
        def evict_idle_plans():
            for key in list(self.cache):
                if self.used + need <= self.budget:
                    return
                e = self.cache[key]
                if (key != keep and e["users"] == 0 and e["plan"] is not None
                        and all(r[0] != key for i, r in enumerate(self.slot_res) if i != slot)):
                    e["plan"].close()
                    self.used -= e["bytes"]
                    del self.cache[key]

        evict_idle_plans()
        if self.used + need <= self.budget:
            return
        for i in range(len(self.slot_res)):
            # an idle slot is waiting in _admit under this lock: its handle is unused
            if i != slot and not self.busy[i] and self.slot_res[i][0] is not None:
                self._release_slot(i)
        evict_idle_plans()

    def _admit(self, slot):
        """Under the lock: pick a batch whose memory fits, reserve it for `slot`."""
        if not self.queue:
            return None
        batch, coils = self._take_batch()
        req0 = batch[0][0]
        work = self._work_bytes(req0, coils)
        if self.slot_res[slot][0] not in (None, req0.key):
            # the slot changes trajectory: close its old handle now, so the
            # bytes credited back are free before anything new is allocated
            self._release_slot(slot)
        rkey, rbytes = self.slot_res[slot]
        if rkey == req0.key:
            extra = max(0, work - rbytes)
            new_res = max(work, rbytes)
        else:
            extra = work
            new_res = work
        new_plan = req0.key not in self.cache
        pbytes = self._plan_bytes_estimate(req0) if new_plan else 0
        need = extra + pbytes
        if self.used + need > self.budget:
            self._evict_for(need, slot, req0.key)
        if self.used + need > self.budget:
            if any(self.busy):
                return None           # wait for memory to be released by running work
            raise MemoryError("reconstruction needs %.2f GiB of device memory beyond the %.2f GiB held; "
                              "budget %.2f GiB" % (_gib(need), _gib(self.used), _gib(self.budget)))
        for item in batch:
            self.queue.remove(item)
        if new_plan:
            self.cache[req0.key] = {"plan": None, "bytes": pbytes, "users": 0, "ready": threading.Event()}
        entry = self.cache[req0.key]
        self.cache.move_to_end(req0.key)
        entry["users"] += 1
        self.used += need
        self.slot_res[slot] = (req0.key, new_res)
        self.busy[slot] = True
        return batch, coils, entry, new_plan

    def _worker(self, slot):
        torch = self.torch
        torch.cuda.set_device(self.device)
        while True:
            with self.cv:
                job = None
                while not self.stop:
                    try:
                        job = self._admit(slot)
                    except Exception as e:  # fail the head request, keep serving the rest
                        self.errors.append(e)
                        if self.queue:
                            _, fut = self.queue.pop(0)
                            fut.set_exception(e)
                        job = None
                    if job is not None:
                        break
                    self.cv.wait(0.01)
                if job is None:
                    return
            batch, coils, entry, new_plan = job
            req0 = batch[0][0]
            t0 = time.perf_counter()
            try:
                h = self._acquire_handle(slot, req0, entry, new_plan)
                t_plan = time.perf_counter() - t0 if new_plan else 0.0
                raws = [r.raw.reshape(r.raw.shape[0], -1) for r, _ in batch]
                raw = np.concatenate(raws, axis=1) if len(raws) > 1 else raws[0]
                im = h.iNUFT(raw, req0.maxit, req0.damp, solver=req0.solver, tol=req0.tol)
                t1 = time.perf_counter()
                c = 0
                for r, fut in batch:
                    r.result = im[..., c:c + r.nc]
                    c += r.nc
                    r.t_start = t0
                    r.t_done = t1
                    r.plan_s = t_plan
                    fut.set_result(r)
            except Exception as e:  # report to every waiting request
                if new_plan:
                    entry["ready"].set()
                self.errors.append(e)
                for r, fut in batch:
                    if not fut.done():
                        fut.set_exception(e)
            finally:
                self._finish(slot, req0.key, entry)

    def _make_plan(self, req):
        return nufft_3d(req.om, req.N, device=self.device, **req.opts)

    def _acquire_handle(self, slot, req0, entry, new_plan):
        """The slot's handle on req0's trajectory, building the base plan if
        this batch admitted a new one.  A handle on another trajectory was
        closed by _admit, so old and new tables are never both held here."""
        if new_plan:
            entry["plan"] = self._make_plan(req0)
            entry["ready"].set()
        else:
            entry["ready"].wait()
            if entry["plan"] is None:
                raise RuntimeError("plan construction failed in another slot")
        cur = self.handle[slot]
        if cur is None or cur[0] != req0.key:
            if cur is not None:  # not reached: _admit releases a handle on another key
                cur[1].close()
            self.handle[slot] = (req0.key, entry["plan"].share())
        return self.handle[slot][1]

    def _finish(self, slot, key, entry):
        with self.cv:
            self.busy[slot] = False
            entry["users"] -= 1
            if entry["plan"] is None and entry["users"] == 0:
                self.used -= entry["bytes"]
                self.cache.pop(key, None)
            while len(self.cache) > self.cache_size:
                k, e = next(iter(self.cache.items()))
                if e["users"] or any(r[0] == k for r in self.slot_res):
                    break
                e["plan"].close()
                self.used -= e["bytes"]
                del self.cache[k]
            self.cv.notify_all()


def run_served(requests, slots=4, hbm_budget=None, device=0, max_batch_coils=16, t0=None):
    """Feed requests at their arrival times; returns (requests, wall seconds)."""
    srv = ReconServer(slots=slots, hbm_budget=hbm_budget, device=device, max_batch_coils=max_batch_coils)
    try:
        futs = []
        start = time.perf_counter() if t0 is None else t0
        for r in sorted(requests, key=lambda r: r.arrival):
            delay = start + r.arrival - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(srv.submit(r))
        done = [f.result() for f in futs]
        wall = time.perf_counter() - start
    finally:
        srv.close()
    for r in done:
        r.t_done -= start
        r.t_start -= start
    return done, wall


def run_plain(requests, device=0):
    """Reference-style sequential path: build the plan, solve, destroy -- per request."""
    start = time.perf_counter()
    for r in sorted(requests, key=lambda r: r.arrival):
        delay = start + r.arrival - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        r.t_start = time.perf_counter() - start
        obj = nufft_3d(r.om, r.N, device=device, **r.opts)
        r.plan_s = time.perf_counter() - start - r.t_start
        r.result = obj.iNUFT(r.raw.reshape(r.raw.shape[0], -1), r.maxit, r.damp, solver=r.solver, tol=r.tol)
        obj.close()
        r.t_done = time.perf_counter() - start
    return requests, time.perf_counter() - start


def summarize(requests, wall):
    lat = np.array([r.latency for r in requests]) * 1e3
    built = [r.plan_s for r in requests if r.plan_s > 0]
    return {"requests": len(requests), "wall_s": round(wall, 3),
            "volumes_per_s": round(len(requests) / wall, 3),
            "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
            "mean_ms": round(float(lat.mean()), 2), "plans_built": len(built),
            "plan_build_ms_mean": round(1e3 * float(np.mean(built)), 2) if built else 0.0}

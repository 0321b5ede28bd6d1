"""CPU tests of the serving loop's HBM admission bookkeeping (no GPU).

The server reserves a plan estimate plus the batch's work buffers before it
runs a batch, and evicts idle cached trajectories to make room.  These tests
drive `_admit` / `_evict_for` with stand-in plans.
"""
import collections
import threading

import numpy as np

from nufft_3d_gb300.serving import ReconServer, Request


class _Plan:
    def __init__(self):
        self.closed = False

    def close(self):
        self.closed = True


def _server(budget, slots=2):
    srv = object.__new__(ReconServer)  # bookkeeping only: no workers, no device
    srv.cv = threading.Condition()
    srv.queue = []
    srv.cache = collections.OrderedDict()
    srv.slot_res = [(None, 0)] * slots
    srv.handle = [None] * slots
    srv.busy = [False] * slots
    srv.cache_size = 8
    srv.used = 0
    srv.budget = budget
    srv.max_batch_coils = 8
    return srv


def _req(key, N=32, M=5000, nc=2, J=6):
    return Request(om=np.zeros((3, M)), N=N, raw=np.zeros((M, nc), np.complex64), key=key,
                   opts={"J": J, "u": 2})


def _cache(srv, key, nbytes, users=0):
    srv.cache[key] = {"plan": _Plan(), "bytes": nbytes, "users": users, "ready": threading.Event()}
    srv.used += nbytes


def test_plan_estimate_counts_the_stored_h():
    r6, r8 = _req("a", J=6), _req("b", J=8)
    per_sample6 = (ReconServer._plan_bytes_estimate(r6) - ReconServer._plan_bytes_estimate(_req("c", M=0))) / 5000
    # J=6 radial: ~113 taps of 8 bytes plus padding and the row offset (H),
    # the same taps again with row headers and padding (H')
    assert 1900 < per_sample6 < 2200
    # ceil(J/2) = 4 builds no stored H
    per_sample8 = (ReconServer._plan_bytes_estimate(r8) - ReconServer._plan_bytes_estimate(_req("d", M=0, J=8))) / 5000
    assert per_sample8 < 64


def test_requested_trajectory_is_never_evicted():
    srv = _server(budget=10 ** 12)
    _cache(srv, "A", 100)
    srv._evict_for(10 ** 13, 0, "A")
    assert "A" in srv.cache and not srv.cache["A"]["plan"].closed


def test_own_slot_does_not_pin_its_old_trajectory():
    srv = _server(budget=1000)
    _cache(srv, "A", 600)
    srv.slot_res[0] = ("A", 100)
    srv.used += 100
    # another slot running a batch on A pins it
    srv.slot_res[1] = ("A", 0)
    srv.busy[1] = True
    srv._evict_for(500, 0, "B")
    assert "A" in srv.cache
    # once that slot is idle its handle is closed and A is released for B
    srv.busy[1] = False
    srv.handle[1] = ("A", _Plan())
    h1 = srv.handle[1][1]
    srv._evict_for(500, 0, "B")
    assert "A" not in srv.cache and srv.used == 100 and h1.closed and srv.handle[1] is None


def test_busy_trajectory_is_kept():
    srv = _server(budget=1000)
    _cache(srv, "A", 900, users=1)
    srv._evict_for(500, 0, "B")
    assert "A" in srv.cache


def test_admit_stays_within_budget_and_waits_for_running_work():
    r = _req("A")
    one = ReconServer._work_bytes(r, 2) + ReconServer._plan_bytes_estimate(r)
    assert ReconServer._plan_bytes_estimate(r) > 0.2 * one  # so B cannot join A without an eviction
    srv = _server(budget=int(one * 1.2))
    srv.queue = [(r, None), (_req("B"), None)]
    job = srv._admit(0)
    assert job is not None and srv.used <= srv.budget
    # slot 1 wants B while A is still running: it must wait, not overcommit
    assert srv._admit(1) is None and srv.used <= srv.budget
    # A finishes on slot 0; slot 0 then takes B, releasing A (its own old trajectory)
    srv.cache["A"]["users"] -= 1
    srv.busy[0] = False
    srv.cache["A"]["plan"] = _Plan()
    job = srv._admit(0)
    assert job is not None and "A" not in srv.cache and srv.used <= srv.budget


class _Ledger:
    """Device bytes actually held: plan tables (while a base plan or a handle
    refers to them) plus every live handle's work buffers."""

    def __init__(self):
        self.live = 0
        self.peak = 0

    def add(self, n):
        self.live += n
        self.peak = max(self.peak, self.live)


class _Tables:
    def __init__(self, ledger, nbytes):
        self.ledger, self.nbytes, self.refs = ledger, nbytes, 1
        ledger.add(nbytes)

    def decref(self):
        self.refs -= 1
        if self.refs == 0:
            self.ledger.add(-self.nbytes)


class _Handle:
    def __init__(self, tables):
        self.t, self.work, self.closed = tables, 0, False
        tables.refs += 1

    def run(self, nbytes):  # work buffers grow on first use (freed before regrown)
        if nbytes > self.work:
            self.t.ledger.add(nbytes - self.work)
            self.work = nbytes

    def close(self):
        if not self.closed:
            self.closed = True
            self.t.ledger.add(-self.work)
            self.t.decref()


class _BasePlan:
    def __init__(self, ledger, nbytes):
        self.t = _Tables(ledger, nbytes)
        self.closed = False

    def share(self):
        return _Handle(self.t)

    def close(self):
        if not self.closed:
            self.closed = True
            self.t.decref()


def test_switching_trajectory_never_holds_old_and_new_tables():
    """A slot that moves to a new trajectory closes its old handle before the
    new plan is built, so the bytes held (tables + live handles' buffers)
    never exceed the budget, and the reservation always covers them."""
    reqs = {k: _req(k, M=20000) for k in "ABCD"}
    one = ReconServer._work_bytes(reqs["A"], 2) + ReconServer._plan_bytes_estimate(reqs["A"])
    ledger = _Ledger()
    srv = _server(budget=int(one * 1.6), slots=2)
    srv._make_plan = lambda req: _BasePlan(ledger, ReconServer._plan_bytes_estimate(req))

    def run_on(slot, key):
        srv.queue = [(reqs[key], None)]
        job = srv._admit(slot)
        assert job is not None, (slot, key)
        batch, coils, entry, new_plan = job
        h = srv._acquire_handle(slot, batch[0][0], entry, new_plan)
        h.run(ReconServer._work_bytes(batch[0][0], coils))
        assert ledger.live <= srv.used <= srv.budget, (key, ledger.live, srv.used, srv.budget)
        srv._finish(slot, key, entry)

    for slot, key in [(0, "A"), (0, "B"), (0, "A"), (1, "A"), (0, "C"), (0, "D"), (1, "D")]:
        run_on(slot, key)
    assert ledger.peak <= srv.budget


def test_batch_larger_than_budget_is_refused_not_overcommitted():
    import pytest
    r = _req("A", M=20000)
    srv = _server(budget=ReconServer._work_bytes(r, 2) // 2)
    srv.queue = [(r, None)]
    with pytest.raises(MemoryError):
        srv._admit(0)
    assert srv.used == 0

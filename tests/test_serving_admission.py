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
    # J=6 radial: ~113 taps of 8 bytes plus padding and the row offset
    assert 900 < per_sample6 < 1100
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
    # another slot holding A pins it
    srv.slot_res[1] = ("A", 0)
    srv._evict_for(500, 0, "B")
    assert "A" in srv.cache
    # only the requesting slot holds A: it is released for B
    srv.slot_res[1] = (None, 0)
    srv._evict_for(500, 0, "B")
    assert "A" not in srv.cache and srv.used == 100


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
    srv.cache["A"]["plan"] = _Plan()
    job = srv._admit(0)
    assert job is not None and "A" not in srv.cache and srv.used <= srv.budget

"""Served solves (include/ts_fvm.h, ts_server_*): continuous batching over
one batch, gated by a memory budget.

The bar: every served result equals the same problem run alone in a batch,
bit for bit (the stated tolerance is zero), while requests overlap on the
device; the budget and the cap on running solves are never exceeded.
"""
import threading
import time

import numpy as np
import pytest

from test_batch import BUDGET, mixed_problems, run_batch

pytestmark = pytest.mark.gpu


def overlapping(times):
    """Pairs of requests that were on the device at the same time."""
    n = 0
    for a in range(len(times)):
        for b in range(a + 1, len(times)):
            ta, tb = times[a], times[b]
            if ta["admit_s"] < tb["finish_s"] and tb["admit_s"] < ta["finish_s"]:
                n += 1
    return n


def max_concurrent(times):
    ev = sorted([(t["admit_s"], 1) for t in times] + [(t["finish_s"], -1) for t in times])
    cur = best = 0
    for _, d in ev:
        cur += d
        best = max(best, cur)
    return best


def submit_stream(srv, probs, gaps_s):
    """Submits probs from a client thread with the given gaps; returns ids."""
    ids = [None] * len(probs)

    def client():
        for k, (case, ic) in enumerate(probs):
            time.sleep(gaps_s[k])
            ids[k] = srv.submit(case, ic)

    th = threading.Thread(target=client)
    th.start()
    th.join()
    return ids


def test_served_results_equal_alone_while_overlapping(tslib):
    from turbostructred_gb300 import capi
    probs = mixed_problems() * 2
    rng = np.random.default_rng(5)
    gaps = rng.exponential(0.004, len(probs))
    alone = {k: run_batch([p])[0] for k, p in enumerate(probs[:9])}
    with capi.Server(BUDGET) as srv:
        ids = submit_stream(srv, probs, gaps)
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(probs) and st["rejected"] == 0 and st["worker_status"] == 0
    for k, (got, info, t) in enumerate(res):
        ref = alone[k % 9]
        assert info["iteration"] == ref[1]["iteration"]
        assert info["time"] == ref[1]["time"]
        assert np.array_equal(got, ref[0]), k
        assert t["submit_s"] <= t["admit_s"] <= t["finish_s"]
    assert overlapping([r[2] for r in res]) > 0
    assert st["latency_p50_ms"] <= st["latency_p99_ms"] <= st["latency_max_ms"]


def test_served_budget_and_cap(tslib):
    from turbostructred_gb300 import capi
    case = capi.make_case(ndims=2, nx=96, ny=64, periodic=(1, 1, 1), recon=3, solver=3, cfl=0.4, max_time=0.03)
    ics = [capi.fill_scenario(case, 1, s, [2.0, 1.0, 0.5, 2.5, 0.01]) for s in range(6)]
    per = capi.batch_problem_bytes(case)
    alone = [run_batch([(case, ic)])[0] for ic in ics]
    # memory for two solves at a time
    with capi.Server(2 * per + 1024) as srv:
        ids = [srv.submit(case, ic) for ic in ics]
        res = [srv.wait(i) for i in ids]
    times = [r[2] for r in res]
    assert max_concurrent(times) <= 2
    for (got, info, _), ref in zip(res, alone):
        assert np.array_equal(got, ref[0])
    # a cap of one running solve: strictly one after another, in arrival order
    with capi.Server(BUDGET, max_active=1) as srv:
        ids = [srv.submit(case, ic) for ic in ics[:3]]
        res = [srv.wait(i) for i in ids]
    times = [r[2] for r in res]
    assert max_concurrent(times) == 1
    assert times[0]["finish_s"] <= times[1]["admit_s"] and times[1]["finish_s"] <= times[2]["admit_s"]


def test_served_errors(tslib):
    from turbostructred_gb300 import capi
    small = capi.make_case(ndims=2, nx=128, ny=128, periodic=(1, 1, 1), max_iter=5000, max_time=1e30)
    ic = capi.fill_scenario(small, 1, 1, [2.0, 1.0, 0.5, 2.5, 0.01])
    with capi.Server(capi.batch_problem_bytes(small) + 1024) as srv:
        with pytest.raises(capi.TsError) as e:
            srv.submit(capi.make_case(ndims=3, nx=8, ny=8, nz=8), np.ones((8, 8, 8, 5)))
        assert e.value.status == 2
        big = capi.make_case(ndims=2, nx=256, ny=256, periodic=(1, 1, 1))
        with pytest.raises(capi.TsError) as e:
            srv.submit(big, np.ones((256, 256, 5)))
        assert e.value.status == 4
        with pytest.raises(capi.TsError) as e:
            srv.wait(777)
        assert e.value.status == 8
        rid = srv.submit(small, ic, keep_state=False)
        with pytest.raises(capi.TsError) as e:
            srv.wait(rid, timeout_ms=0)
        assert e.value.status == 6
        got, info, _ = srv.wait(rid)
        assert got is None and info["iteration"] == 5000
        srv.drain(10000)
        st = srv.stats()
        assert st["queued"] == 0 and st["active"] == 0 and st["bytes_in_use"] == 0


def test_served_shortest_first_and_cell_cap(tslib):
    """Least-work-first admission: with one solve admitted at a time, queued
    small solves overtake large ones; a cap on admitted cells holds."""
    from turbostructred_gb300 import capi
    big = capi.make_case(ndims=2, nx=128, ny=128, periodic=(1, 1, 1), max_iter=60, max_time=1e30)
    small = capi.make_case(ndims=2, nx=32, ny=32, periodic=(1, 1, 1), max_iter=60, max_time=1e30)
    shear = [2.0, 1.0, 0.5, 2.5, 0.01]
    reqs = [(big, capi.fill_scenario(big, 1, k, shear)) for k in range(3)] + \
           [(small, capi.fill_scenario(small, 1, k, shear)) for k in range(3)]
    alone = [run_batch([r])[0] for r in reqs]
    with capi.Server(BUDGET, max_active=1, order=capi.SERVE_SHORTEST_FIRST) as srv:
        ids = [srv.submit(c, v) for c, v in reqs]
        res = [srv.wait(i) for i in ids]
    times = [r[2] for r in res]
    first = min(range(6), key=lambda k: times[k]["admit_s"])
    later_big = [times[k]["finish_s"] for k in range(3) if k != first]
    assert max(times[k]["finish_s"] for k in range(3, 6) if k != first) <= min(later_big)
    for (got, info, _), ref in zip(res, alone):
        assert np.array_equal(got, ref[0])
    with capi.Server(BUDGET, max_cells=2 * 128 * 128) as srv:
        ids = [srv.submit(c, v) for c, v in reqs[:3]]
        res = [srv.wait(i) for i in ids]
    assert max_concurrent([r[2] for r in res]) <= 2

"""Host logic of the served RVE stream: the seeded trace and the admission
loop (lanes, batch limits, memory budget, failure reporting) with a fake
batch solver, no GPU."""
import threading
import time

import numpy as np

from tahoe_gb300 import serve


def test_trace_seeded_and_in_range():
    a1, n1, F1 = serve.sample_requests(2000, 5000.0, seed=3)
    a2, n2, F2 = serve.sample_requests(2000, 5000.0, seed=3)
    assert np.array_equal(a1, a2) and np.array_equal(n1, n2) and np.array_equal(F1, F2)
    assert np.all(np.diff(a1) > 0)
    assert n1.min() >= 4 and n1.max() <= 24
    assert set(np.unique(n1)) == set(range(4, 25))
    # log-uniform: small sides more frequent than large ones
    assert (n1 <= 8).sum() > (n1 >= 17).sum()
    # mean inter-arrival time near 1/rate
    assert abs(np.mean(np.diff(a1)) * 5000.0 - 1.0) < 0.1
    S = F1 - np.eye(3)
    assert np.allclose(S, np.swapaxes(S, 1, 2)) and np.abs(S).max() <= 0.05


def fake_solver(log, delay=0.002, fail_sizes=()):
    lock = threading.Lock()

    def solve(ns, Fs, lane_state):
        with lock:
            log.append(list(ns))
        time.sleep(delay)
        if any(int(n) in fail_sizes for n in ns):
            raise RuntimeError("planted batch failure")
        return np.zeros(len(ns), dtype=np.int64), Fs * ns[:, None, None]

    return solve


def test_every_request_served_once_with_its_own_result():
    arr, ns, Fs = serve.sample_requests(300, 20000.0, seed=1)
    log = []
    srv = serve.Server(fake_solver(log), lanes=3, max_batch=16)
    res = srv.run(arr, ns, Fs)
    served = np.concatenate([np.asarray(b) for b in log])
    assert len(served) == len(ns)
    assert res["completed"] == 300 and np.all(res["status"] == 0)
    assert np.allclose(res["P"], Fs * ns[:, None, None])
    assert max(len(b) for b in log) <= 16
    assert np.all(res["latency"] >= 0) and np.all(res["start"] >= arr - 1e-9)
    assert res["p99_ms"] >= res["p50_ms"] > 0
    assert res["max_concurrent_lanes"] >= 2


def test_batches_respect_memory_budget():
    arr, ns, Fs = serve.sample_requests(200, 50000.0, seed=2)
    log = []
    budget = 5 * serve.rve_bytes(24)
    srv = serve.Server(fake_solver(log), lanes=4, max_batch=1000, hbm_budget=budget)
    res = srv.run(arr, ns, Fs)
    assert res["completed"] == 200
    for b in log:
        assert len(b) == 1 or sum(serve.rve_bytes(int(n)) for n in b) <= budget
    # the in-flight total across lanes never exceeded the budget
    assert 0 < res["peak_inflight_bytes"] <= budget
    assert len(res["batches"]) == len(log)


def test_failed_batch_reported_retried_and_lane_continues():
    arr, ns, Fs = serve.sample_requests(120, 10000.0, seed=4)
    log = []
    srv = serve.Server(fake_solver(log, fail_sizes=(24,)), lanes=2, max_batch=4)
    res = srv.run(arr, ns, Fs)
    bad = res["status"] != 0
    # only the size-24 requests fail: their batch-mates succeed when retried alone
    assert np.array_equal(bad, ns == 24) and bad.any()
    assert np.all(res["status"][bad] == -2)
    assert res["completed"] == int((~bad).sum())
    assert res["retried"] >= int(bad.sum()) and len(res["errors"]) >= 1
    assert np.allclose(res["P"][~bad], (Fs * ns[:, None, None])[~bad])
    assert np.all(np.isnan(res["P"][bad]))


def test_one_at_a_time_mode():
    arr, ns, Fs = serve.sample_requests(40, 1000.0, seed=5)
    log = []
    srv = serve.Server(fake_solver(log, delay=0.0), lanes=1, max_batch=1)
    res = srv.run(arr, ns, Fs)
    assert all(len(b) == 1 for b in log) and res["completed"] == 40
    assert [b[0] for b in log] == list(ns)  # arrival order

"""Served RVE stream on the GPU: a Poisson trace through two lanes with
continuous batching, mixed precision; every request's averaged first Piola
stress is bitwise the same request solved alone through the same mixed path
(one Krylov solve per RVE), equals (1e-6) the same RVE solved one at a time
in FP64, a
sample of the served requests equals (1e-6) the oracle's solve of the same
RVE, and the lanes actually batched and overlapped."""
import numpy as np
import pytest

from tahoe_gb300 import lib, rve, serve
from tests.helpers import oracle_rve, rel_err

pytestmark = pytest.mark.gpu


def test_served_stream_equals_one_at_a_time_fp64():
    arr, ns, Fs = serve.sample_requests(24, 20000.0, seed=7, nmin=4, nmax=9)
    srv = serve.Server(serve.gpu_batch_solver(lib.MIXED), lanes=2, max_batch=8)
    try:
        res = srv.run(arr, ns, Fs)
    finally:
        srv.close()
    assert np.all(res["status"] == 0), res["status"]
    assert max(b[1] for b in res["batches"]) > 1
    plain = serve.Server(serve.gpu_batch_solver(lib.FP64), lanes=1, max_batch=1)
    try:
        ref = plain.run(arr, ns, Fs, time_scale=0.0)
    finally:
        plain.close()
    assert np.all(ref["status"] == 0)
    assert all(b[1] == 1 for b in ref["batches"])
    for r in range(len(ns)):
        assert rel_err(res["P"][r], ref["P"][r]) < 1e-6, (r, int(ns[r]))
    # the same requests one at a time through the same mixed path: every
    # served result (solved inside a batch of other requests) is bitwise the
    # result of the request alone
    alone = serve.Server(serve.gpu_batch_solver(lib.MIXED), lanes=1, max_batch=1)
    try:
        one = alone.run(arr, ns, Fs, time_scale=0.0)
    finally:
        alone.close()
    assert np.all(one["status"] == 0)
    assert np.array_equal(one["P"], res["P"])
    # served results against the oracle (independent of both GPU paths): the
    # first requests of each side length in the trace
    picked = [int(np.nonzero(ns == n)[0][0]) for n in np.unique(ns)][:4]
    for r in picked:
        _, Po = oracle_rve(int(ns[r]), Fs[r])
        assert rel_err(res["P"][r], Po) < 1e-6, (r, int(ns[r]))


def test_lane_context_reused_across_batches():
    """A lane's context takes a new mesh per batch; a batch solved after a
    larger one (pool memory reused) gives the same result as a fresh context."""
    rng = np.random.default_rng(3)
    big = (np.array([7, 8, 6]), np.stack([rve.sample_F(rng) for _ in range(3)]))
    small = (np.array([5, 4]), np.stack([rve.sample_F(rng) for _ in range(2)]))
    solve = serve.gpu_batch_solver(lib.MIXED)
    lane = {"device": 0}
    st, _ = solve(*big, lane)
    assert np.all(st == 0)
    st, P_reused = solve(*small, lane)
    assert np.all(st == 0)
    st, P_fresh = solve(*small, {"device": 0})
    assert np.all(st == 0)
    assert rel_err(P_reused, P_fresh) < 1e-12


def test_native_request_loop_equals_one_at_a_time():
    """The request loop in the library (tg_serve_*: lanes as C++ threads,
    admission by size, memory and latency target): every request completes,
    batches form, and each result is bitwise the same request solved alone
    (the C++ RVE templates are the Python ones, node for node)."""
    arr, ns, Fs = serve.sample_requests(24, 20000.0, seed=3, nmin=4, nmax=8)
    srv = serve.NativeServer(lanes=2, max_batch=8, hbm_budget=8e9, precision=lib.MIXED, target_batch_ms=50.0)
    try:
        res = srv.run(arr, ns, Fs)
    finally:
        srv.close()
    assert np.all(res["status"] == 0), res["status"]
    assert res["mean_batch"] > 1.0
    alone = serve.Server(serve.gpu_batch_solver(lib.MIXED), lanes=1, max_batch=1)
    try:
        one = alone.run(arr, ns, Fs, time_scale=0.0)
    finally:
        alone.close()
    assert np.array_equal(one["P"], res["P"])

"""Served RVE stream (configuration 5): continuous batching over device lanes.

Requests (one RVE each: side n, macroscopic F) arrive as a Poisson process.
A pool of lanes serves them; each lane owns a context (its own CUDA stream)
and loops: take every request that has arrived and is not yet started, in
arrival order, as long as the batch fits the lane's share of the free-HBM
budget; solve that batch (predictor + Newton to the per-RVE tolerance,
mixed precision by default); report each RVE's averaged first Piola stress
and release its memory.  Requests that arrive while other lanes are busy on
the GPU are admitted by the next free lane, so work from several batches
overlaps on the device (one stream per lane); no request waits for an
unrelated batch to finish unless every lane or the memory budget is taken.

The batch solver is pluggable so the admission logic can be exercised on the
host without a GPU.
"""
import ctypes
import threading
import time

import numpy as np

from . import lib, rve


def sample_requests(count, rate, seed=0, nmin=4, nmax=24):
    """Poisson arrivals at `rate` per second; n log-uniform in {nmin..nmax};
    F as in the batched configuration."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count))
    ns = np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1), size=count))).astype(np.int64)
    ns = np.clip(ns, nmin, nmax)
    Fs = np.stack([rve.sample_F(rng) for _ in range(count)])
    return arrivals, ns, Fs


def rve_bytes(n, precision=lib.MIXED):
    """Device bytes one RVE of side n holds while it is solved (element
    staging, contribution map, point geometry, tile storage, vectors,
    history), estimated."""
    s = 4 if precision == lib.MIXED else 8
    nel, nnd = n ** 3, (n + 1) ** 3
    return nel * (432 * s + 256 + 8 * 32 + 128 + 8 * 25 * 8) + nnd * (27 * (9 * s + 8) + 10 * 16 + 6 * 4 * s + 64)


def gpu_batch_solver(precision=lib.MIXED, rel_tol=1e-8, lin_rel_tol=1e-4):
    """Solve a batch on the lane's context, composed on the device from the
    lane's resident RVE templates: returns (statuses, P (k,3,3))."""

    def solve(ns, Fs, lane_state):
        res = lane_state.get("rves")
        if res is None:
            ctx = lib.Context(lane_state.get("device", 0))
            res = rve.ResidentRVEs(ctx)
            lane_state["ctx"] = ctx
            lane_state["rves"] = res
        rc, rep, rel, P = res.solve(ns, Fs, precision=precision, rel_tol=rel_tol, lin_rel_tol=lin_rel_tol)
        # status per RVE: an RVE that failed fails alone, the others are valid
        st = np.asarray(getattr(res, "status", np.full(len(ns), rc)), dtype=np.int64)
        if rc not in (0, -4, -5, -6, -7):
            st = np.full(len(ns), rc)  # a CUDA, memory or argument error ends the batch
        if (st != 0).any():
            lane_state.setdefault("failures", []).append(
                (rc, lane_state["ctx"].L.tg_last_error(lane_state["ctx"].h).decode(), list(map(int, ns)),
                 float(np.max(rel)) if len(rel) else None))
        return st, P

    return solve


class Server:
    def __init__(self, solve_batch, lanes=4, max_batch=512, hbm_budget=None, precision=lib.MIXED, device=0,
                 bytes_fn=None):
        self.solve_batch = solve_batch
        self.lanes = lanes
        self.max_batch = max_batch
        self.hbm_budget = hbm_budget if hbm_budget is not None else 64e9
        self.device = device
        self.bytes_fn = bytes_fn or (lambda n: rve_bytes(int(n), precision))
        # per-lane state (the lane's context) persists across runs, so a
        # warm-up trace leaves the lanes' contexts and memory pools primed
        self.lane_states = [{"device": device} for _ in range(lanes)]

    def run(self, arrivals, ns, Fs, time_scale=1.0):
        """Replays the trace in real time (arrival times scaled by
        time_scale); returns a dict of per-request results and statistics."""
        count = len(arrivals)
        lock = threading.Lock()
        state = {"next": 0, "ready": [], "inflight": 0.0, "done": 0, "peak": 0.0, "retried": 0}
        start = np.full(count, np.nan)
        finish = np.full(count, np.nan)
        status = np.zeros(count, dtype=np.int64)
        P = np.full((count, 3, 3), np.nan)
        batches = []
        errors = []
        need = np.array([self.bytes_fn(n) for n in ns])
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        def lane(lid):
            lane_state = self.lane_states[lid]
            while True:
                with lock:
                    tnow = now()
                    while state["next"] < count and arrivals[state["next"]] * time_scale <= tnow:
                        state["ready"].append(state["next"])
                        state["next"] += 1
                    if state["done"] >= count:
                        return
                    take, used = [], 0.0
                    room = self.hbm_budget - state["inflight"]
                    for rid in state["ready"]:
                        if len(take) >= self.max_batch:
                            break
                        if used + need[rid] > room and take:
                            break
                        if used + need[rid] > room and state["inflight"] > 0:
                            break  # wait for memory to free up
                        take.append(rid)
                        used += need[rid]
                    if take:
                        state["ready"] = state["ready"][len(take):]
                        state["inflight"] += used
                        state["peak"] = max(state["peak"], state["inflight"])
                    nxt = arrivals[state["next"]] * time_scale if state["next"] < count else None
                if not take:
                    wait = 0.0005 if nxt is None else max(0.0, min(0.005, nxt - now()))
                    time.sleep(wait)
                    continue
                ts = now()
                start[take] = ts
                try:
                    st, Pb = self.solve_batch(ns[take], Fs[take], lane_state)
                except Exception as e:  # a failed batch reports its requests and the lane carries on
                    st, Pb = np.full(len(take), -2), np.full((len(take), 3, 3), np.nan)
                    with lock:
                        errors.append((lid, len(take), str(e)))
                st = np.asarray(st)
                bad = np.nonzero(st != 0)[0]
                if len(take) > 1 and len(bad):
                    # requests of a failed batch are retried alone
                    for j in bad:
                        rid = take[j]
                        try:
                            s1, P1 = self.solve_batch(ns[[rid]], Fs[[rid]], lane_state)
                            st[j], Pb[j] = s1[0], P1[0]
                        except Exception as e:
                            with lock:
                                errors.append((lid, 1, str(e)))
                    with lock:
                        state["retried"] += len(bad)
                te = now()
                with lock:
                    finish[take] = te
                    status[take] = st
                    P[take] = Pb
                    state["inflight"] -= used
                    state["done"] += len(take)
                    batches.append((lid, len(take), ts, te))

        threads = [threading.Thread(target=lane, args=(i,), daemon=True) for i in range(self.lanes)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        lat = finish - arrivals * time_scale
        okm = status == 0
        elapsed = np.nanmax(finish) - arrivals[0] * time_scale if count else 0.0
        return {
            "P": P, "status": status, "latency": lat, "start": start, "finish": finish, "batches": batches,
            "completed": int(okm.sum()), "elapsed_s": float(elapsed),
            "solves_per_s": float(okm.sum() / elapsed) if elapsed > 0 else 0.0,
            "p50_ms": float(np.percentile(lat[okm], 50) * 1e3) if okm.any() else None,
            "p99_ms": float(np.percentile(lat[okm], 99) * 1e3) if okm.any() else None,
            "mean_batch": float(np.mean([b[1] for b in batches])) if batches else 0.0,
            "max_concurrent_lanes": _max_overlap(batches),
            "peak_inflight_bytes": state["peak"],
            "errors": errors,
            "retried": state["retried"],
            "failures": [f for st in self.lane_states for f in st.get("failures", [])],
        }


    def close(self):
        for st in self.lane_states:
            st.pop("rves", None)
            ctx = st.pop("ctx", None)
            if ctx is not None:
                ctx.close()


class NativeServer:
    """The request loop in the library (tg_serve_*): lanes are C++ threads,
    each with its own context and resident RVE templates; admission by size,
    device-memory budget and a latency target (predicted batch time).  This
    class only replays a trace: it submits each request at its arrival time
    and collects the results."""

    def __init__(self, lanes=4, max_batch=1024, hbm_budget=64e9, precision=lib.MIXED,
                 precond=lib.PRECOND_BLOCK_JACOBI, rel_tol=1e-8, lin_rel_tol=1e-4, target_batch_ms=0.0, device=0):
        self.L = lib.load()
        h = ctypes.c_void_p()
        rc = self.L.tg_serve_create(ctypes.byref(h), int(device), int(lanes), int(max_batch), float(hbm_budget),
                                    int(precision), int(precond), float(rel_tol), float(lin_rel_tol),
                                    float(target_batch_ms))
        if rc != lib.TG_OK:
            raise lib.TahoeError(rc, "tg_serve_create", "bad arguments")
        self.h = h

    def submit(self, n, F):
        F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
        rid = ctypes.c_longlong(0)
        rc = self.L.tg_serve_submit(self.h, int(n), F.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    ctypes.byref(rid))
        if rc != lib.TG_OK:
            raise lib.TahoeError(rc, "tg_serve_submit", "bad arguments")
        return rid.value

    def result(self, rid):
        """(status, P (3,3), latency ms) or None while pending"""
        P = np.zeros(9)
        st = ctypes.c_int(0)
        lat = ctypes.c_double(0)
        rc = self.L.tg_serve_poll(self.h, ctypes.c_longlong(rid), P.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  ctypes.byref(st), ctypes.byref(lat))
        if rc == 1:
            return None
        if rc != lib.TG_OK:
            raise lib.TahoeError(rc, "tg_serve_poll", "unknown request")
        return st.value, P.reshape(3, 3), lat.value

    def stats(self):
        out = np.zeros(6)
        self.L.tg_serve_stats(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 6)
        return dict(batches=int(out[0]), mean_batch=float(out[1]), max_concurrent_lanes=int(out[2]),
                    retried=int(out[3]), model_ms_per_1000_elements=float(out[4]), completed=int(out[5]))

    def run(self, arrivals, ns, Fs, time_scale=1.0):
        """Replays the trace in real time; same result dict as Server.run."""
        count = len(arrivals)
        ids = np.zeros(count, dtype=np.int64)
        s0 = self.stats()
        t0 = time.perf_counter()
        for i in range(count):
            wait = arrivals[i] * time_scale - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            ids[i] = self.submit(ns[i], Fs[i])
        self.L.tg_serve_wait(self.h)
        status = np.zeros(count, dtype=np.int64)
        P = np.zeros((count, 3, 3))
        lat = np.zeros(count)
        for i in range(count):
            st, Pi, li = self.result(ids[i])
            status[i], P[i], lat[i] = st, Pi, li * 1e-3
        s1 = self.stats()
        okm = status == 0
        # elapsed: first arrival to last completion (latency of the last finisher)
        finish = arrivals * time_scale + lat
        elapsed = float(np.max(finish) - arrivals[0] * time_scale) if count else 0.0
        nb = s1["batches"] - s0["batches"]
        return {
            "P": P, "status": status, "latency": lat, "completed": int(okm.sum()), "elapsed_s": elapsed,
            "solves_per_s": float(okm.sum() / elapsed) if elapsed > 0 else 0.0,
            "p50_ms": float(np.percentile(lat[okm], 50) * 1e3) if okm.any() else None,
            "p99_ms": float(np.percentile(lat[okm], 99) * 1e3) if okm.any() else None,
            "mean_batch": float(count / nb) if nb else 0.0, "batches": [None] * nb,
            "max_concurrent_lanes": s1["max_concurrent_lanes"], "retried": s1["retried"] - s0["retried"],
            "errors": [], "failures": [], "model_ms_per_1000_elements": s1["model_ms_per_1000_elements"],
        }

    def error(self):
        return self.L.tg_serve_error(self.h).decode()

    def close(self):
        if getattr(self, "h", None):
            self.L.tg_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _max_overlap(batches):
    ev = sorted([(b[2], 1) for b in batches] + [(b[3], -1) for b in batches])
    cur = best = 0
    for _, d in ev:
        cur += d
        best = max(best, cur)
    return best

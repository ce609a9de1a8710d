"""Benchmark of the GB300 hex8 implicit path.

Headline workload (configuration 2 of the benchmark set): total-Lagrangian
compressible neo-Hookean block, 64^3 hex8 (274,625 nodes, 823,875 dofs),
mu=1, kappa=10, interior nodes jittered +-0.2h (seed 0), bottom fixed, top
compressed 1% in the first of 10 load steps.  Synthetic, seeded input (no
dataset exists).

A timed step is one Newton iteration of that load step from its start state
(the prescribed-increment predictor's): FP32 element tangent + deterministic
block-CSR assembly + Jacobi PCG (the reference's diagonal_matrix; FP32
vectors, compensated dot products, FP64 scalars) to the inner tolerance 1e-4
+ update + element residual (double-float element forces, FP64 gather) and
norm.  Every step starts from the same device snapshot, so the K
steps do identical work.  The metric is the Newton-step time (ms per
iteration, lower is better).  Inputs stay resident in HBM; the block-CSR
matrix (about 290 MB) is larger than the 129 MB L2, so no flush is needed
between steps.

`e2e` repeats the step through the C ABI with host buffers: displacement
uploaded from pinned host memory, residual at the step start, the iteration,
and the displacement read back into pinned host memory, all inside the timed
region.

The same line carries the other halves of the metric, each measured in this
run: C1 (16^3 small-strain elastic cube, one static step), the full 10-step
C2 load history in both precision forms, the C4 batch of 4,096 RVEs (RVE
solves/s, mixed vs FP64, with the SpMV roofline on the batch mesh) and a short
C5 served stream (p50/p99 beside the plain FP64 one-at-a-time solve).

--impl reference runs the reference algorithm on the host cores: the CPU
oracle restatement of the path (the reference's own build needs its CMake
system over the whole library, so it is not compiled here), one complete
Newton iteration of the same workload per step -- tangent + MSR assembly
(serial, as the reference's AssembleLHS), Jacobi CG to the same 1e-4 on all
host threads, update, residual -- from the same predictor start state.

Multi-GPU: independent replicas (the single-mesh path has a real halo
exchange that is not built); --gpus N under torchrun runs N replicas.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LIN_TOL = 1e-4          # inner PCG relative tolerance (inexact Newton)
NEWTON_TOL = 1e-8       # outer relative tolerance on the residual
C2_T = 1.0              # load step 1 of 10 (schedule 0 -> 1 over t = 0..10)


def c2_config(nel, nnd, neq, precond, ws):
    """The workload description both arms print (identical dicts)."""
    return {"workload": "C2: 64^3 hex8 total-Lagrangian Simo neo-Hookean (mu=1, kappa=10), jitter 0.2h seed 0, "
                        "load step 1/10 from the predictor state, one Newton iteration (inner %s-PCG rel tol %g)"
                        % ("block-Jacobi" if precond == "block" else "Jacobi", LIN_TOL),
            "nel": int(nel), "nodes": int(nnd), "dofs": int(3 * nnd), "equations": int(neq),
            "precond": precond, "parallelism": "replicas x%d" % ws,
            "l2": "inputs larger than L2 (assembled matrix about 290 MB FP32 block CSR on the GPU)"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def spmv_roofline(ctx, precision):
    """Event-timed streamed SpMV on the context's current tangent against the
    measured copy bandwidth (algorithmic bytes as for configuration 2)."""
    from tahoe_gb300 import lib, workloads
    ms = ctx.time_kernel(0, 20)
    s_val = 4 if precision == lib.MIXED else 8
    product = ctx.product_kernel()
    push = product in ("pcg_cg_push_kernel", "pcg_seg_push_kernel")
    sym = product == "pcg_spmv_sym_kernel"
    b = (workloads.spmv_bytes_push if push else workloads.spmv_bytes_sym if sym else
         workloads.spmv_bytes)(ctx.block_nnz, ctx.nnd, s_val)
    peak, kind = peaks()
    ach = b / (ms * 1e-3) / 1e9
    return {"kernel": product, "storage": "symmetric push" if push else "symmetric" if sym else "full",
            "bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
            "frac": round(ach / peak, 4), "peak_kind": kind, "algorithmic_bytes": int(b),
            "l2_intermediate_bytes": int(workloads.push_l2_bytes(ctx.block_nnz, ctx.nnd, s_val)) if push else 0,
            "ms_per_launch": round(ms, 4),
            "note": "algorithmic bytes are the DRAM bytes of the push storage's stream; its pushed products "
                    "(l2_intermediate_bytes) stay in L2 where they fit and also cross DRAM where they do not, "
                    "so the fraction is a lower bound on a mesh that large" if push else ""}


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for ln in f:
                parts = [p.strip() for p in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def pinned_pair(n):
    """Two float64 host arrays of n values in page-locked memory (through
    torch), or pageable numpy arrays where pinning is unavailable."""
    try:
        import torch
        a = torch.empty(n, dtype=torch.float64, pin_memory=True)
        b = torch.empty(n, dtype=torch.float64, pin_memory=True)
        return a.numpy(), b.numpy(), "pinned"
    except Exception:
        return np.empty(n), np.empty(n), "pageable"


def profiled_traffic(name):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    from the committed ncu summary profiles/<name>, or None.  The figure is
    the capture's, not a measurement of this run."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_launch:"):
                    return int(ln.split(":")[1])
    except OSError:
        pass
    return None


def setup_c2(device, precision, precond):
    from tahoe_gb300 import workloads
    mesh, model, run = workloads.c2(add=None)
    model.device = device
    model.setup()
    # load step 1: prescribed increment through the linearised predictor
    pred_its = model.apply_step(C2_T, (precision, precond, LIN_TOL))
    ctx = model.ctx
    ctx.set_iteration(-1)
    ctx.residual(want_vector=False, precision=precision)
    ctx.checkpoint()
    return mesh, model, ctx, pred_its


def one_iteration(ctx, precision, lin_tol, precond=0):
    ctx.rollback()
    ctx.set_iteration(-1)
    return ctx.newton_iteration(precision=precision, precond=precond, lin_rel_tol=lin_tol, lin_max_it=20000)


def cpu_newton_port(threads, steps, warmup, n=64):
    """The oracle port of the C2 Newton iteration on the host cores: mesh,
    equations and MSR structure, the predictor to the step-1 start state (not
    timed), then per step one complete Newton iteration from that state --
    tangent + MSR assembly, Jacobi CG to LIN_TOL on `threads` threads, update,
    residual -- timed with the wall clock."""
    from oracle.pyoracle import OracleModel
    from tahoe_gb300 import workloads
    t0 = time.perf_counter()
    mesh, om, _ = workloads.c2(n=n, add=lambda X, conn, form, mat: OracleModel(X, conn, form, mat, threads=threads))
    _, neq = om.equations()
    pred_its = om.predict(C2_T, LIN_TOL)
    u0 = om.get_u()
    setup_s = time.perf_counter() - t0
    times, parts, its = [], [], []
    for k in range(warmup + steps):
        om.set_u(u0)
        om.residual(C2_T, -1)
        t0 = time.perf_counter()
        n_its, nrm, tm = om.newton_iteration(C2_T, -1, LIN_TOL)
        dt = time.perf_counter() - t0
        if k >= warmup:
            times.append(dt)
            parts.append(tm)
            its.append(n_its)
    parts = np.mean(np.array(parts), axis=0)
    return {"ms": 1e3 * float(np.mean(times)), "ms_steps": [round(1e3 * t, 1) for t in times],
            "pcg_iterations": its, "predictor_pcg_iterations": pred_its, "setup_s": round(setup_s, 2),
            "phase_s": {"tangent_and_assembly": round(float(parts[0]), 3), "pcg": round(float(parts[1]), 3),
                        "residual": round(float(parts[2]), 3)},
            "nel": mesh.nel, "nnd": mesh.nnd, "neq": neq}


def cpu_sample_text(r, threads):
    return ("oracle port, one complete C2 Newton iteration per step from the step-1 predictor state: tangent + "
            "serial MSR assembly (%.2f s, element formation on %d threads), Jacobi CG to %g on %d threads "
            "(%s iterations, %.2f s), update, residual (%.2f s); mean of %d timed steps"
            % (r["phase_s"]["tangent_and_assembly"], threads, LIN_TOL, threads,
               "/".join(str(i) for i in sorted(set(r["pcg_iterations"]))), r["phase_s"]["pcg"],
               r["phase_s"]["residual"], len(r["ms_steps"])))


def c2_history(model, precond):
    """The full 10-step C2 load history from the undeformed state in both
    forms: Newton / PCG iterations per step, device time, and the mixed form's
    displacement error against the FP64 form at every step end."""
    from tahoe_gb300 import lib
    ctx = model.ctx
    out, hist = {}, {}
    for name, p in (("mixed", lib.MIXED), ("fp64", lib.FP64)):
        ctx.set_u(np.zeros((model.X.shape[0], 3)))
        ctx.timer_start()
        h, reps = model.run(10, 1.0, rel_tol=NEWTON_TOL, abs_tol=0.0, max_iterations=20, div_tol=10.0, precision=p,
                            precond=precond, lin_rel_tol=LIN_TOL, lin_max_it=20000, predictor=True)
        ms = ctx.timer_stop()
        hist[name] = h
        newton = [r.iterations for r in reps]
        out[name] = {"ms": round(ms, 1), "newton_per_step": newton, "pcg_per_step": [r.pcg_iterations for r in reps],
                     "ms_per_newton_iteration": round(ms / max(sum(newton), 1), 3)}
    err = [float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(hist["mixed"], hist["fp64"])]
    out["u_rel_err_mixed_vs_fp64_per_step"] = [float("%.3g" % e) for e in err]
    out["note"] = "pcg_per_step excludes the predictor's iterations; ms covers predictors and Newton"
    return out


def c1_step():
    """C1: 16^3 small-strain Hookean cube, 1 MPa traction, one static step
    from setup on a fresh context (after one untimed step), PCG-Jacobi to
    1e-10, both forms; the oracle port's time for the same step on the host
    (single thread, as the reference's implicit path)."""
    from oracle.pyoracle import OracleModel
    from tahoe_gb300 import lib, workloads
    res, u = {}, {}
    for name, p in (("mixed", lib.MIXED), ("fp64", lib.FP64)):
        # one untimed step on its own context first: the first launch of a
        # kernel in a process loads its code, which is not the step's work
        for timed in (False, True):
            mesh, m, run = workloads.c1()
            m.setup()
            m.ctx.timer_start()
            # FP64: one Newton iteration with PCG to 1e-10 (the configuration's
            # solver); mixed: inexact Newton (FP32 PCG to 1e-4) to the same
            # 1e-10 on the residual
            h, reps = m.run(1, 1.0, rel_tol=1e-10, abs_tol=0.0, max_iterations=10, precision=p,
                            precond=lib.PRECOND_JACOBI, lin_rel_tol=1e-10 if p == lib.FP64 else LIN_TOL,
                            lin_max_it=20000)
            ms = m.ctx.timer_stop()
            if not timed:
                m.ctx.close()
        u[name] = h[-1]
        res[name] = {"ms": round(ms, 3), "newton_iterations": reps[0].iterations,
                     "pcg_iterations": reps[0].pcg_iterations}
        m.ctx.close()
    _, om, _ = workloads.c1(add=lambda X, conn, form, mat: OracleModel(X, conn, form, mat, threads=1))
    t0 = time.perf_counter()
    st, uh, its = om.run(1, 1.0, 1e-10, 0.0, 10, 10.0, 1, 1e-10)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    res["u_rel_err_mixed_vs_fp64"] = float(np.abs(u["mixed"] - u["fp64"]).max() / np.abs(u["fp64"]).max())
    res["cpu_baseline"] = {"value": round(cpu_ms, 1), "unit": "ms/static step", "cores": 1, "kind": "port",
                           "sample": "oracle port, the whole static step (Newton + serial Jacobi CG to 1e-10)"}
    res["config"] = "C1: 16^3 hex8 small-strain Hookean (E 200e3, nu 0.3), z=0 fixed, 1 MPa traction on z=1"
    return res


def run_ours(args):
    ws, rank, local = dist_init()
    from tahoe_gb300 import lib, workloads
    prec = lib.MIXED if args.precision == "mixed" else lib.FP64
    precond = lib.PRECOND_BLOCK_JACOBI if args.precond == "block" else lib.PRECOND_JACOBI
    mesh, model, ctx, pred_its = setup_c2(local, prec, precond)
    if args.form is not None:
        ctx.pcg_form(args.form)
    tuning = None
    if not args.no_tune:
        # launch shapes picked by the autotuner on this mesh and state
        from tahoe_gb300 import autotune
        t = autotune.Tuner(reps=20)
        tuning = t.tune(ctx, prec, lib.TOTAL_LAGRANGIAN)
        tuning = {k: tuning.get(k) for k in ("tile_blocks", "stages", "release", "sym", "sym_tile", "tangent_epb",
                                             "spmv_ms", "tangent_ms", "cached", "spmv_sweep", "push")}

    # warm-up (also captures the PCG graph)
    for _ in range(max(args.warmup, 1)):
        one_iteration(ctx, prec, LIN_TOL, precond)

    sampler = ClockSampler(local)
    barrier(ws)
    sampler.start()
    launches0 = ctx.launches
    ctx.timer_start()
    pcg_its = []
    for _ in range(args.steps):
        nrm, its = one_iteration(ctx, prec, LIN_TOL, precond)
        pcg_its.append(its)
    ms_total = ctx.timer_stop()
    launches = ctx.launches - launches0
    clocks = sampler.stop()
    barrier(ws)
    ms_total = max_over_ranks(ws, ms_total)
    ms_step = ms_total / args.steps

    # e2e through the C ABI with host buffers (pinned, as a host that streams
    # steps would hold them; pageable if pinning is unavailable)
    ctx.rollback()
    nnd = mesh.nnd
    u_in, u_out, host_mem = pinned_pair(nnd * 3)
    u_in[:] = ctx.get_u().reshape(-1)
    u0 = u_in.copy().reshape(-1, 3)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.set_u(u_in)
        ctx.set_iteration(-1)
        ctx.residual(want_vector=False, precision=prec)
        ctx.newton_iteration(precision=prec, precond=precond, lin_rel_tol=LIN_TOL)
        ctx.get_u(out=u_out)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_ms = max_over_ranks(ws, e2e_ms)
    # back to the step-start snapshot for the kernel timings below
    ctx.set_u(u0)
    ctx.set_iteration(-1)
    ctx.residual(want_vector=False, precision=prec)
    ctx.checkpoint()

    # per-kernel device times (CUDA events on the context stream)
    ctx.tangent(prec)
    t_spmv = ctx.time_kernel(0, 20)
    t_upd = ctx.time_kernel(1, 20)
    t_tan = ctx.time_kernel(2, 5)
    t_asm = ctx.time_kernel(3, 5)
    # the residual of the form's Newton driver (double-float for the mixed
    # form), and the FP64 one beside it
    t_res = ctx.time_kernel(5 if prec == lib.MIXED else 4, 5)
    t_res64 = ctx.time_kernel(4, 5) if prec == lib.MIXED else t_res
    s_val = 4 if prec == lib.MIXED else 8
    nnzb = ctx.block_nnz
    sym = bool(getattr(ctx, "sym_mode", 0))
    product = ctx.product_kernel()
    push = product == "pcg_cg_push_kernel"
    cg = product == "pcg_cg_spmv_kernel" or push
    prof = {"pcg_spmv_sym_kernel": "pcg_spmv_sym_c2_64cubed.md", "pcg_cg_spmv_kernel": "pcg_cg_spmv_c2_64cubed.md",
            "pcg_cg_push_kernel": "pcg_cg_push_c2_64cubed.md"}.get(product, "pcg_spmv_c2_64cubed.md")
    bytes_spmv = (workloads.spmv_bytes_push if push else workloads.spmv_bytes_sym if sym else
                  workloads.spmv_bytes)(nnzb, nnd, s_val)
    peak, peak_kind = peaks()
    achieved = bytes_spmv / (t_spmv * 1e-3) / 1e9
    elements_per_s = mesh.nel / ((t_tan + t_asm) * 1e-3)
    # the other HBM-bound kernels of the step, same peak and byte model
    other_rooflines = {}
    vec = ("pcg_cg_vector_kernel", workloads.cg_vector_bytes_push(nnzb, nnd, s_val) if push else
           workloads.cg_vector_bytes(nnd, s_val), t_upd) if cg else \
        ("pcg_update_kernel", workloads.update_bytes(nnd, s_val), t_upd)
    asm = ("assemble_upper_kernel", workloads.assembly_bytes_upper(mesh.nel, nnzb, nnd, s_val), t_asm) if push else \
        ("assemble_kernel", workloads.assembly_bytes(mesh.nel, nnzb, nnd, s_val), t_asm)
    for name, b, t in (asm, vec):
        a = b / (t * 1e-3) / 1e9
        other_rooflines[name] = {"bound": "hbm", "achieved": round(a, 1), "peak": peak, "unit": "GB/s",
                                 "frac": round(a / peak, 4), "algorithmic_bytes": int(b), "ms_per_launch": round(t, 5)}
    other_rooflines[vec[0]]["timed"] = "each launch right after an untimed product launch, as in the solve"

    line = {
        "metric": "Newton-step time",
        "value": round(ms_step, 4),
        "unit": "ms/Newton iteration",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 tangent+PCG, double-float residual, fp64 norms/scalars" if prec == lib.MIXED else "fp64",
        "data": "synthetic (seeded 64^3 jittered hex8 block)",
        "config": c2_config(mesh.nel, nnd, ctx.neq, args.precond, ws),
        "block_nnz": int(nnzb), "scalar_nnz": int(nnzb * 9),
        "pcg_iterations_per_step": float(np.mean(pcg_its)),
        "predictor_pcg_iterations": pred_its,
        "elements_assembled_per_s": round(elements_per_s, 1),
        "pcg_form": {0: "textbook", 1: "single-reduction (Chronopoulos-Gear), programmatic launch",
                     2: "single-reduction (Chronopoulos-Gear)",
                     3: "single-reduction (Chronopoulos-Gear), programmatic launch, symmetric push storage"}.get(
                         ctx.effective_form(), "textbook"),
        "kernel_ms": {"pcg_product": round(t_spmv, 5), "pcg_vector": round(t_upd, 5), "tangent": round(t_tan, 4),
                      "assembly": round(t_asm, 4), "residual": round(t_res, 4),
                      "residual_fp64": round(t_res64, 4)},
        "roofline": {"kernel": product,
                     "storage": "symmetric push" if push else "symmetric" if sym else "full", "bound": "hbm", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "algorithmic_bytes": int(bytes_spmv),
                     "l2_intermediate_bytes": int(workloads.push_l2_bytes(nnzb, nnd, s_val)) if push else 0,
                     "traffic": profiled_traffic(prof) if prec == lib.MIXED else None,
                     "traffic_source": "committed ncu capture of this kernel on this workload (profiles/%s), not "
                                       "measured in this run" % prof},
        "other_rooflines": other_rooflines,
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms/Newton iteration", "h2d_bytes_per_step": nnd * 24,
                "d2h_bytes_per_step": nnd * 24, "host_memory": host_mem},
        "gpu_launches": int(launches),
        "tuning": tuning,
        "clocks": clocks,
    }
    if not args.quick and ws == 1:
        # the metric's other halves, measured in this run (device timers)
        t_extra = time.perf_counter()
        line["c2_load_history"] = c2_history(model, precond)
        model.ctx.close()
        line["c1"] = c1_step()
        line["c4"] = c4_batch(args.rves, args.c4_precond, with_cpu=False, macro=True)
        line["c5"] = c5_trace(args, rates=[args.c5_rate], requests=args.c5_requests,
                              plain_requests=args.c5_plain_requests)
        line["c3"] = c3_run(args.c3_extra_steps, tune=False)
        line["extras_wall_s"] = round(time.perf_counter() - t_extra, 1)
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        r = cpu_newton_port(threads, steps=2, warmup=1)
        line["cpu_baseline"] = {"value": round(r["ms"], 1), "unit": "ms/Newton iteration", "cores": threads,
                                "kind": "port", "sample": cpu_sample_text(r, threads)}
    if rank == 0:
        print(json.dumps(line))


def run_reference(args):
    """The reference arm: the oracle port of the same Newton iteration on all
    host threads, one complete iteration per step (nothing extrapolated)."""
    ws, rank, local = dist_init()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t_run = time.perf_counter()
    r = cpu_newton_port(threads, steps=args.steps, warmup=args.warmup)
    v = r["ms"]
    line = {
        "impl": "reference", "metric": "Newton-step time", "value": round(v, 1), "unit": "ms/Newton iteration",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(v, 1),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded 64^3 jittered hex8 block)",
        "config": c2_config(r["nel"], r["nnd"], r["neq"], args.precond, ws),
        "pcg_iterations_per_step": float(np.mean(r["pcg_iterations"])),
        "ms_steps": r["ms_steps"],
        "cpu_baseline": {"value": round(v, 1), "unit": "ms/Newton iteration", "cores": threads, "kind": "port",
                         "sample": cpu_sample_text(r, threads)},
        "e2e": {"value": round(v, 1), "unit": "ms/Newton iteration", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": r["setup_s"], "wall_s": round(time.perf_counter() - t_run, 1),
    }
    if args.precond != "jacobi":
        line["note"] = "the port's CG is Jacobi (the reference's diagonal_matrix) whatever --precond says"
    print(json.dumps(line))


KERNELS = {"spmv": 0, "update": 1, "tangent": 2, "assembly": 3, "residual": 4, "residual_ff": 5}


def rve_cpu_sample(sizes_all, threads, seed=0):
    """Oracle port on one RVE per size (Jacobi-PCG inner solves, as the GPU
    path), timed single-threaded; the batch time for a pool of `threads`
    independent processes is the size-weighted mean divided by the pool."""
    from oracle.pyoracle import OracleModel
    from tahoe_gb300 import rve
    rng = np.random.default_rng(seed + 1)
    per_n = {}
    for n in sorted(set(int(x) for x in sizes_all)):
        t = rve.template(n)
        F = rve.sample_F(rng)
        o = OracleModel(t.X, t.conn, "total_lagrangian", [rve.MATRIX, rve.INCLUSION], blocks=t.blocks)
        o.set_schedule([(0.0, 1.0)])
        U = t.X @ (F - np.eye(3)).T
        for a in t.boundary:
            for d in range(3):
                o.add_kbc(int(a), d, float(U[a, d]), True)
        t0 = time.perf_counter()
        st, uh, its = o.run(1, 1.0, 1e-8, 0.0, 20, 1e3, 1, 1e-4)
        per_n[n] = time.perf_counter() - t0
    mean = float(np.mean([per_n[int(x)] for x in sizes_all]))
    return mean, per_n


def c4_batch(count, precond_name, with_cpu=False, macro=True):
    """Configuration 4: a batch of independent RVEs solved together.  The
    timed batch covers composing the batch mesh from the resident templates,
    the affine predictor, Newton to 1e-8 per RVE and the averaged stresses;
    the consistent macro tangent is timed separately."""
    from tahoe_gb300 import lib, rve
    ns, Fs = rve.sample_batch(count, seed=0)
    t0 = time.perf_counter()
    c = lib.Context(0)
    res = rve.ResidentRVEs(c)
    for n in np.unique(ns):
        res.template_id(n)
    t_setup = time.perf_counter() - t0
    precond = lib.PRECOND_BLOCK_JACOBI if precond_name == "block" else lib.PRECOND_JACOBI
    out = {}
    wn, wF = ns[:64], Fs[:64]
    for name, prec in (("mixed", lib.MIXED), ("fp64", lib.FP64)):
        res.solve(wn, wF, precision=prec, precond=precond)  # warm-up: pools
        c.timer_start()
        rc, rep, rel, P = res.solve(ns, Fs, precision=prec, precond=precond)
        ms = c.timer_stop()
        out[name] = dict(ms=ms, rc=rc, newton=rep.iterations, pcg=rep.pcg_iterations, worst_rel=float(rel.max()),
                         P=P, ms_tangent=rep.ms_tangent, ms_solve=rep.ms_solve, ms_residual=rep.ms_residual)
        if macro:
            # consistent macro tangent of every RVE at the converged state
            c.timer_start()
            Cm, cits = c.macro_tangent(np.ones(len(ns)), precision=prec, precond=precond, lin_rel_tol=1e-7)
            out[name].update(C=Cm, ms_macro=c.timer_stop(), macro_pcg=cits)
        if name == "mixed":
            c.tangent(lib.MIXED)
            roof = spmv_roofline(c, lib.MIXED)
            roof["on"] = "the composed batch mesh (%d nodes, %d block nonzeros)" % (c.nnd, c.block_nnz)
            geo = dict(elements=int(c.nel), nodes=int(c.nnd), dofs=int(3 * c.nnd), equations=int(c.neq),
                       block_nnz=int(c.block_nnz))
    c.close()
    Pm, Pf = out["mixed"]["P"], out["fp64"]["P"]
    err = float(np.abs(Pm - Pf).max() / np.abs(Pf).max())
    per_rve = np.abs(Pm - Pf).reshape(len(ns), -1).max(axis=1) / np.abs(Pf).reshape(len(ns), -1).max(axis=1)
    line = {
        "metric": "RVE solves/s", "value": round(len(ns) / (out["mixed"]["ms"] * 1e-3), 1), "unit": "RVE/s",
        "higher_is_better": True, "n_gpus": 1,
        "config": dict(workload="C4: %d independent RVEs, n x n x n hex8 unit cubes, n ~ U{4..16} (seed 0), two-phase "
                                "Simo neo-Hookean (mu 1/10, kappa 10/100, inclusion r=0.3 by centroid), affine BC "
                                "from F = I + 0.05 S, linear predictor then Newton to 1e-8 per RVE, %s-PCG 1e-4"
                                % (len(ns), "block-Jacobi" if precond_name == "block" else "Jacobi"), **geo),
        "batch_ms": {k: round(v["ms"], 2) for k, v in out.items()},
        "solves_per_s": {k: round(len(ns) / (v["ms"] * 1e-3), 1) for k, v in out.items()},
        "newton_iterations": {k: v["newton"] for k, v in out.items()},
        "pcg_iterations": {k: v["pcg"] for k, v in out.items()},
        "phase_ms": {k: {"tangent": round(v["ms_tangent"], 2), "solve": round(v["ms_solve"], 2),
                         "residual": round(v["ms_residual"], 2)} for k, v in out.items()},
        "worst_rve_rel_residual": {k: v["worst_rel"] for k, v in out.items()},
        "status": {k: v["rc"] for k, v in out.items()},
        "P_rel_err_mixed_vs_fp64": err,
        "P_rel_err_mixed_vs_fp64_worst_rve": float(per_rve.max()),
        "template_setup_s": round(t_setup, 3),
        "roofline": roof,
        "precond": precond_name,
    }
    if macro:
        line["macro_tangent_ms"] = {k: round(v["ms_macro"], 2) for k, v in out.items()}
        line["macro_tangent_pcg_iterations"] = {k: v["macro_pcg"] for k, v in out.items()}
        line["macro_tangent_rel_err_mixed_vs_fp64"] = float(np.abs(out["mixed"]["C"] - out["fp64"]["C"]).max() /
                                                            np.abs(out["fp64"]["C"]).max())
        line["solves_per_s_with_macro_tangent"] = {
            k: round(len(ns) / ((v["ms"] + v["ms_macro"]) * 1e-3), 1) for k, v in out.items()}
    if with_cpu:
        threads = os.cpu_count() or 1
        mean, per_n = rve_cpu_sample(ns, threads)
        line["cpu_baseline"] = {"value": round(threads / mean, 2), "unit": "RVE/s", "cores": threads, "kind": "port",
                                "sample": "oracle (Newton + Jacobi-PCG 1e-4, FP64) on one RVE per size n=4..16, "
                                          "single-threaded; batch rate = pool of %d independent processes at the "
                                          "size-weighted mean %.3f s per RVE" % (threads, mean)}
    return line


def run_c4(args):
    print(json.dumps(c4_batch(args.rves, args.c4_precond, with_cpu=not args.no_cpu, macro=True)))


def c5_trace(args, rates, requests, plain_requests):
    """Configuration 5: a Poisson stream of RVE requests served by the
    library's request loop (tg_serve_*: lanes as C++ threads, continuous
    batching with admission by size, memory and a latency target; mixed
    precision), beside the plain one-at-a-time FP64 GPU solve of the same
    requests through the same loop (one lane, batches of one)."""
    from tahoe_gb300 import lib, rve, serve
    import torch
    free, _ = torch.cuda.mem_get_info(0)
    budget = 0.5 * free
    srv = serve.NativeServer(lanes=args.lanes, max_batch=args.max_batch, hbm_budget=budget, precision=lib.MIXED,
                             target_batch_ms=args.c5_target_ms)
    plain = serve.NativeServer(lanes=1, max_batch=1, hbm_budget=budget, precision=lib.FP64)
    # warm-up: contexts, memory pools, templates, graph captures, the batch-time model
    wa, wn, wF = serve.sample_requests(16 * args.lanes, 1e5, seed=99, nmin=4, nmax=24)
    srv.run(wa, wn, wF)
    plain.run(wa[:2], wn[:2], wF[:2])
    sweep = []
    for i, rate in enumerate(rates):
        arr, ns, Fs = serve.sample_requests(requests, rate, seed=i)
        res = srv.run(arr, ns, Fs)
        k = min(plain_requests, len(ns))
        ref = plain.run(arr[:k], ns[:k], Fs[:k])
        both = (res["status"][:k] == 0) & (ref["status"] == 0)
        d = np.abs(res["P"][:k] - ref["P"]).reshape(k, -1).max(axis=1) / \
            np.abs(ref["P"]).reshape(k, -1).max(axis=1)
        sweep.append({
            "rate_per_s": rate, "requests": len(ns), "completed": res["completed"],
            "solves_per_s": round(res["solves_per_s"], 1), "p50_ms": round(res["p50_ms"], 2),
            "p99_ms": round(res["p99_ms"], 2), "mean_batch": round(res["mean_batch"], 1),
            "batches": len(res["batches"]), "max_concurrent_lanes": res["max_concurrent_lanes"],
            "retried_alone": res["retried"],
            "plain_fp64": {"requests": k, "completed": ref["completed"], "solves_per_s": round(ref["solves_per_s"], 1),
                           "p50_ms": round(ref["p50_ms"], 2), "p99_ms": round(ref["p99_ms"], 2)},
            "P_rel_err_vs_plain_fp64_worst": float(d[both].max()) if both.any() else None,
        })
        if res["completed"] < len(ns):
            codes, counts = np.unique(res["status"][res["status"] != 0], return_counts=True)
            sweep[-1]["failed"] = {int(k): int(v) for k, v in zip(codes, counts)}
            sweep[-1]["error"] = srv.error()[:200]
    model = srv.stats()["model_ms_per_1000_elements"]
    srv.close()
    plain.close()
    # SpMV roofline on a batch mesh of the stream's size mix (first 64 requests)
    c = lib.Context(0)
    res_t = rve.ResidentRVEs(c)
    res_t.compose(ns[:64])
    c.set_iteration(-1)
    c.residual(want_vector=False)
    c.tangent(lib.MIXED)
    roof = spmv_roofline(c, lib.MIXED)
    roof["on"] = "a batch mesh of the first 64 requests (%d nodes)" % c.nnd
    c.close()
    top = max(sweep, key=lambda r: r["solves_per_s"])
    return {
        "metric": "served RVE solves/s", "value": top["solves_per_s"], "unit": "RVE/s", "higher_is_better": True,
        "n_gpus": 1,
        "config": {"workload": "C5: Poisson stream of RVE requests, n log-uniform in {4..24}, two-phase Simo "
                               "neo-Hookean RVE as in C4, F = I + 0.05 S; request loop in the library "
                               "(tg_serve_*): %d lanes (C++ threads, one CUDA stream each), continuous batching up "
                               "to %d RVEs per batch, admission by half of free HBM and a %g ms batch-time target, "
                               "mixed precision, one PCG per RVE, Newton to 1e-8 per RVE"
                               % (args.lanes, args.max_batch, args.c5_target_ms),
                   "hbm_budget_bytes": int(budget)},
        "sweep": sweep,
        "batch_time_model_ms_per_1000_elements": round(model, 3),
        "roofline": roof,
    }


def run_c5(args):
    rates = [float(r) for r in args.rates.split(",")]
    print(json.dumps(c5_trace(args, rates, args.requests, args.plain_requests)))


def run_c3(args):
    print(json.dumps(c3_run(args.c3_steps, args.max_step_cuts, args.quick_solve_iter, tune=not args.no_tune)))


def c3_run(nsteps, max_step_cuts=6, quick_solve_iter=0, tune=True):
    """Configuration 3: small-strain J2 plate 96 x 96 x 48 under cyclic
    uniaxial displacement (+-0.5 % strain over 40 steps).  Both forms run the
    same load history through the reference's step sequence (Newton to 1e-8
    per step, Jacobi-PCG, load-step cuts where Newton fails); the final active
    (yielding) set of the mixed form is compared bitwise with the plain FP64
    form's, and the displacements at every original step end are compared."""
    from tahoe_gb300 import autotune, lib, workloads
    args = argparse.Namespace(no_tune=not tune, max_step_cuts=max_step_cuts, quick_solve_iter=quick_solve_iter)
    out, flags_ref, u_last = {}, {}, {}
    for name, prec in (("mixed", lib.MIXED), ("fp64", lib.FP64)):
        mesh, model, run = workloads.c3(nsteps=40)
        model.setup()
        c = model.ctx
        if not args.no_tune:
            # shapes tuned on the undeformed state (tangents only: no residual
            # is formed, so no history is touched)
            c.set_iteration(-1)
            autotune.Tuner(reps=10).tune(c, prec, lib.SMALL_STRAIN)
        rec = dict(newton=[], pcg=[], mismatch=[])
        c.timer_start()
        hist, reps = model.run(nsteps, 1.0, rel_tol=1e-8, abs_tol=1e-10, max_iterations=12, div_tol=1e3,
                               precision=prec, precond=lib.PRECOND_JACOBI, lin_rel_tol=1e-4, lin_max_it=50000,
                               max_step_cuts=args.max_step_cuts, quick_solve_iter=args.quick_solve_iter)
        total_ms = c.timer_stop()
        rec["total_ms"] = total_ms
        c.tangent(prec)
        rec["roofline"] = spmv_roofline(c, prec)
        rec["cuts"] = model.step_cuts
        for r in reps:
            rs = r if isinstance(r, list) else [r]
            rec["newton"].append(sum(x.iterations for x in rs))
            rec["pcg"].append(sum(x.pcg_iterations for x in rs))
        fl = c.active_set()
        rec["flags_final"] = {str(k): int((fl == k).sum()) for k in (0, 1, 3, 7)}
        # yielding set: points that yielded in the last step (kReset after
        # CloseStep) or are plastic; allocation: elements that ever voted to
        # allocate (also in intermediate Newton iterations)
        yielding, alloc = (fl == 0) | (fl == 3), fl != lib.J2_UNALLOCATED
        if name == "mixed":
            flags_ref["final"] = (yielding, alloc, fl)
        else:
            rec["mismatch"].append(int((yielding != flags_ref["final"][0]).sum()))
            rec["alloc_mismatch"] = int((alloc != flags_ref["final"][1]).sum())
            rec["raw_mismatch"] = int((fl != flags_ref["final"][2]).sum())
        u_last[name] = hist
        out[name] = rec
        c.close()
    m, f = out["mixed"], out["fp64"]
    tot = {k: v["total_ms"] for k, v in out.items()}
    its = {k: sum(v["newton"]) for k, v in out.items()}
    line = {
        "metric": "Newton-step time", "value": round(tot["mixed"] / max(its["mixed"], 1), 3),
        "unit": "ms/Newton iteration", "higher_is_better": False, "n_gpus": 1,
        "config": {"workload": "C3: small-strain J2 (E 200e3, nu 0.3, yield 250, H 1000) plate 96x96x48 hex8, "
                               "x=0 clamped, x=L gripped with u_x cycling to +-0.5%% strain, %d of 40 steps, "
                               "Newton to 1e-8 (at most 12 iterations), Jacobi-PCG 1e-4, load-step cuts as "
                               "TimeManagerT (max %d, quick_solve_iter %d)"
                               % (nsteps, args.max_step_cuts, args.quick_solve_iter),
                   "elements": int(mesh.nel), "nodes": int(mesh.nnd), "gauss_points": int(mesh.nel * 8)},
        "load_steps": nsteps,
        "total_ms": {k: round(v, 1) for k, v in tot.items()},
        "ms_per_load_step": {k: round(v / nsteps, 1) for k, v in tot.items()},
        "newton_iterations": its,
        "pcg_iterations": {k: int(sum(v["pcg"])) for k, v in out.items()},
        "ms_per_newton_iteration": {k: round(tot[k] / max(its[k], 1), 3) for k in out},
        "step_cuts": {k: v["cuts"] for k, v in out.items()},
        "newton_per_step": {k: v["newton"] for k, v in out.items()},
        "flags_final": {k: v["flags_final"] for k, v in out.items()},
        "roofline": out["mixed"]["roofline"],
        "yielding_set_mismatch_final": f["mismatch"][0],
        "yielding_set_bit_exact": f["mismatch"][0] == 0,
        "raw_flag_array_mismatch_final": f["raw_mismatch"],
        "raw_flag_array_bit_exact": f["raw_mismatch"] == 0,
        "allocated_points_mismatch_final": f["alloc_mismatch"],
        "flags_note": "yielding set = points flagged plastic or reset at the last converged step; the raw flag "
                      "array also records element allocation, which follows transient yields of intermediate "
                      "Newton iterates and so the precision form's iterate path",
        "u_rel_err_mixed_vs_fp64_worst_step": float(max(
            np.abs(a - b).max() / max(np.abs(b).max(), 1e-300) for a, b in zip(u_last["mixed"], u_last["fp64"]))),
    }
    return line


def run_kernel_only(args):
    """Standalone launches of one hot kernel on the C2 state (for ncu): the
    step's prescribed values applied directly, residual, tangent, then
    --launches launches of the chosen kernel timed with CUDA events."""
    from tahoe_gb300 import lib, workloads
    prec = lib.MIXED if args.precision == "mixed" else lib.FP64
    mesh, model, _ = workloads.c2(n=args.n)
    model.setup()
    model.apply_step(1.0)
    ctx = model.ctx
    ctx.set_iteration(-1)
    ctx.residual(want_vector=False)
    ctx.tangent(prec)
    if args.form is not None:
        ctx.pcg_form(args.form)
    ctx.time_kernel(KERNELS[args.kernel], 1)  # warm-up: forms what the kernel's first use forms
    ms = ctx.time_kernel(KERNELS[args.kernel], args.launches)
    print(json.dumps({"kernel": args.kernel, "n": args.n, "precision": args.precision, "launches": args.launches,
                      "ms_per_launch": ms, "block_nnz": ctx.block_nnz, "nodes": mesh.nnd, "elements": mesh.nel}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--quick", action="store_true", help="skip the full load-step comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-tune", action="store_true", help="default launch shapes, no autotuning")
    ap.add_argument("--kernel", choices=sorted(KERNELS), help="time standalone launches of one kernel only")
    ap.add_argument("--form", type=int, default=None, choices=[0, 1, 2, 3],
                    help="single-vector PCG form (tg_pcg_form); default the library's")
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--n", type=int, default=64, help="mesh size per side for --kernel")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--c3-steps", type=int, default=40, help="C3 load steps to run (of 40)")
    ap.add_argument("--c3-extra-steps", type=int, default=2, help="C3 load steps in the default run's line")
    ap.add_argument("--max-step-cuts", type=int, default=6, help="C3 load-step cuts allowed (TimeManagerT)")
    ap.add_argument("--quick-solve-iter", type=int, default=0,
                    help="C3 NLSolver quick_solve_iter (<= 1: a cut step is never doubled back)")
    ap.add_argument("--rves", type=int, default=4096)
    ap.add_argument("--rates", default="1000,5000,20000,50000", help="C5 arrival rates per second")
    ap.add_argument("--requests", type=int, default=2000, help="C5 requests per rate")
    ap.add_argument("--plain-requests", type=int, default=200, help="C5 requests for the one-at-a-time arm")
    ap.add_argument("--lanes", type=int, default=4)
    ap.add_argument("--max-batch", type=int, default=1024)
    ap.add_argument("--precond", default="jacobi", choices=["jacobi", "block"],
                    help="PCG preconditioner: Jacobi (the reference's diagonal_matrix) or block-Jacobi (3x3 node "
                         "blocks)")
    ap.add_argument("--c4-precond", default="block", choices=["jacobi", "block"], help="C4 batch preconditioner")
    ap.add_argument("--c5-rate", type=float, default=5000.0, help="C5 arrival rate of the default run's trace")
    ap.add_argument("--c5-target-ms", type=float, default=200.0,
                    help="C5 latency target: predicted batch time a lane admits up to (0: none)")
    ap.add_argument("--c5-requests", type=int, default=1000, help="C5 requests of the default run's trace")
    ap.add_argument("--c5-plain-requests", type=int, default=100, help="C5 one-at-a-time FP64 requests (default run)")
    args = ap.parse_args()
    if args.workload == "c1" and args.impl == "ours":
        print(json.dumps(c1_step()))
    elif args.workload == "c4" and args.impl == "ours":
        run_c4(args)
    elif args.workload == "c5" and args.impl == "ours":
        run_c5(args)
    elif args.workload == "c3" and args.impl == "ours":
        run_c3(args)
    elif args.kernel:
        run_kernel_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

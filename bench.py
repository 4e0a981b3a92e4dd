"""Benchmark: 12-source Wilson-clover propagator solve on one GB300, to FP64 true residual 1e-10.

Workload (the spec volume): 32^3 x 64, periodic space / antiperiodic time, hot-start links
U = reunit(exp(i 0.3 H)) (seeded), kappa = 0.1250, c_sw = 1.6, the 12 spin-colour point sources
at the origin solved together as one multi-RHS batch through the full even-odd system
(Schur prep, odd solve, even reconstruction: Chroma's PrecFermActQprop + quarkProp4_a).

The solve is the FP64 defect correction around a reliable BiCGStab on the even-odd operator M~
with the FP16 stencil (SolverType BICGSTAB); the same solve with the inner CGNE and an FP64
BiCGStab are reported beside it.

A step is one such propagator solve.  value = seconds per propagator (device-resident inputs,
CUDA events on the library stream, max over ranks / N for N replicas); e2e = the same through
gbc_solve with pinned host buffers (H2D of the sources and D2H of the solution inside the clock).
The baseline on the same GPU is plain FP64 CG (CGNE, InvCG2) solving the 12 sources one by one;
the CPU baseline is the oracle's FP64 CG on the host cores (bounded sample, extrapolated).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbc|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Solve time at rel. residual 1e-10: learned+mixed vs plain CG; Dslash HBM GB/s"
DIMS = (32, 32, 32, 64)
KAPPA, CSW, EPS, SEED = 0.1250, 1.6, 0.3, 20251203
RSD = 1e-10
DELTA = 0.01  # reliable-update threshold of the inner BiCGStab (the XML's Delta)
INNER_TOL = 1e-5  # inner relative tolerance of each outer step (the XML's InnerTol)
# InvCG2 iterations sampled per timed step of the CPU legs (bounded samples of the full solve)
CPU_SAMPLE_ITERS = 20
# ncu DRAM bytes (read + write) of one 12-RHS FP16 M~ (its two stencil launches) at 24^3x48
M12_TRAFFIC_24 = 1228.1e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbc", choices=["gbc", "reference"])
    ap.add_argument("--dims", default=None, help="override lattice, e.g. 16,16,16,32 (testing only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--op-only", default=None,
                    choices=["dslash16", "dslash32", "dslash64", "meo16", "meo64", "meodf", "dslashdf", "precond"],
                    help="profiling mode: set up the workload and time one operator only")
    ap.add_argument("--nrhs", type=int, default=12)
    ap.add_argument("--recon", type=int, default=12, choices=[12, 18])
    ap.add_argument("--no-extras", action="store_true", help="skip the smaller side workloads")
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--profile-timed", action="store_true",
                    help="bracket the timed solves with cudaProfilerStart/Stop (ncu --profile-from-start off)")
    ap.add_argument("--no-oracle-check", action="store_true",
                    help="skip the oracle's FP64 check of the solutions (residuals and one oracle solve)")
    return ap.parse_args()


def op_only(args):
    """Profiling mode (for ncu): the workload's operator alone, a few launches."""
    from chroma_gb300 import gbclover as G
    dims = tuple(int(x) for x in args.dims.split(",")) if args.dims else DIMS
    links, _ = workload(dims)
    ctx = G.Context(dims, 1 / (2 * KAPPA) - 4, CSW, t_boundary=-1, max_rhs=max(12, args.nrhs),
                    sloppy_reconstruct=args.recon)
    ctx.load_gauge(links)
    if args.op_only == "precond":
        ctx.load_precond(WEIGHTS32 if dims == DIMS else WEIGHTS)
    op, prec = {"precond": (G.TIME_PRECOND, G.PREC_SINGLE),
                "dslash16": (G.OP_DSLASH, G.PREC_HALF), "dslash32": (G.OP_DSLASH, G.PREC_SINGLE),
                "dslash64": (G.OP_DSLASH, G.PREC_DOUBLE), "meo16": (G.OP_MEO, G.PREC_HALF),
                "meo64": (G.OP_MEO, G.PREC_DOUBLE), "meodf": (G.OP_MEO, G.PREC_DF64),
                "dslashdf": (G.OP_DSLASH, G.PREC_DF64)}[args.op_only]
    sec, byts = ctx.time_operator(op, prec, nrhs=args.nrhs, iters=args.iters, flush_l2=True)
    if args.profile_timed:
        # a second, tuned run inside cudaProfilerStart/Stop (ncu --profile-from-start off)
        import torch
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        sec, byts = ctx.time_operator(op, prec, nrhs=args.nrhs, iters=args.iters, flush_l2=True)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    print(json.dumps({"op": args.op_only, "dims": dims, "nrhs": args.nrhs, "seconds": sec, "bytes": byts,
                      "GBps": byts / sec / 1e9, "tuned": ctx.tune_report().strip().splitlines()}), flush=True)
    ctx.close()


def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() and args.impl == "gbc" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.flush()
        rows = []
        try:
            for line in open(self.f.name):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        finally:
            os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows]
        smax = max(float(r[2]) for r in rows)
        load = [s for s in sm if s > 0.5 * smax] or sm
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def workload(dims):
    from chroma_gb300 import gbclover as G
    from chroma_gb300 import sources as S
    links = G.gauge_synthetic(dims, EPS, SEED, t_boundary=-1)
    src = S.point_sources(dims).reshape(12, -1, 12)
    return links, src


def workload_desc(dims):
    """The workload string of the JSON line's config (the same for both arms)."""
    return (f"{'x'.join(map(str, dims))} Wilson-clover propagator, 12 point sources, kappa={KAPPA}, c_sw={CSW}, "
            f"hot start eps={EPS}, antiperiodic t, full system, FP64 true residual {RSD}")


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cg_iteration_seconds(op, chi, k):
    """Seconds per oracle InvCG2 iteration: a k-iteration and a 2-iteration solve, so that the
    per-solve work (M~^dag chi, the initial and final residuals) cancels."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    op.solve(chi, solver=O.SOLVER_CG, rsd=1e-30, maxit=2)
    t2 = time.perf_counter() - t0
    t0 = time.perf_counter()
    op.solve(chi, solver=O.SOLVER_CG, rsd=1e-30, maxit=k)
    tk = time.perf_counter() - t0
    return (tk - t2) / (k - 2), tk


def cpu_baseline(dims, links, chi_one, iters_full, nsrc, budget_s=20.0):
    """Oracle FP64 InvCG2 on the host cores: a bounded number of iterations on one source,
    extrapolated to the full 12-source solve by the measured FP64 iteration count."""
    from oracle import OracleOp
    from oracle import oracle as O
    t0 = time.perf_counter()
    op = OracleOp(dims, links, 1 / (2 * KAPPA) - 4, CSW)
    setup = time.perf_counter() - t0
    # calibrate, then run as many iterations as fit in the budget
    per, _ = cg_iteration_seconds(op, chi_one, 4)
    k = max(4, min(200, int(budget_s / max(per, 1e-6))))
    per_iter, dt = cg_iteration_seconds(op, chi_one, k)
    threads = O.load().orc_num_threads()
    return {"value": per_iter * iters_full * nsrc, "unit": "s", "cores": threads, "kind": "port",
            "sample": f"{k} InvCG2 iterations of 1 of {nsrc} sources ({dt:.1f} s, oracle FP64, OpenMP), per "
                      f"iteration from the difference to a 2-iteration solve; extrapolated x {iters_full} "
                      f"iterations x {nsrc} sources; operator setup {setup:.1f} s",
            "seconds_per_cg_iteration": per_iter}


def oracle_check(dims, links, src, psi):
    """The oracle's FP64 view of the benchmark's solutions (outside the timed region): the true
    relative residual |chi - M psi| / |chi| of every source with the oracle's unpreconditioned
    operator, and the error of source 0 against the oracle's own FP64 solve (Chroma's InvCG2 on the
    Schur system, target 1e-12)."""
    from oracle import OracleOp
    t0 = time.perf_counter()
    op = OracleOp(dims, links, 1 / (2 * KAPPA) - 4, CSW)
    rr = op.full_residuals(psi, src)
    ref, info = op.qprop(src[0], rsd=1e-12)
    err = float(np.linalg.norm(psi[0] - ref) / np.linalg.norm(ref))
    return {"oracle_true_rel_resid_max": float(rr.max()), "oracle_true_rel_resid_min": float(rr.min()),
            "rel_error_vs_oracle_src0": err, "oracle_solve": {"iterations": info["n_count"],
                                                              "rel_resid": info["rel_resid"]},
            "seconds": time.perf_counter() - t0}, op


def chroma_factory_path(ctx, G, op, src, solve_kw):
    """What a factory-only Chroma input gets: quarkProp4_a calls the solver once per source, and
    PrecFermActQprop (eoprec_fermact_qprop.cc:41-80) prepares each source and reconstructs the even
    sites on the host around a LinOp solve of M~ psi_o = chi_o, which the adapter hands to gbc_solve
    with nrhs = 1.  The host steps are timed with the oracle's OpenMP operator standing in for
    QDP++ (the adapter's own gather/scatter loops are not included); the device solves are timed
    through gbc_solve with host buffers."""
    import ctypes as C
    from oracle import oracle as O
    nsrc = src.shape[0]
    host = 0.0
    dev = 0.0
    p = G.SolveParams(solve_kw["solver"], G.SYS_MEO, RSD, 10000, DELTA, 10.0, G.PREC_HALF, INNER_TOL, 0, 16, 0, 1)
    iters = []
    for k in range(nsrc):
        chi = src[k]
        t0 = time.perf_counter()
        t1 = op.apply(O.OP_CLOVER_INV, chi, +1, 0)
        t2 = op.apply(O.OP_DSLASH, t1, +1, 1)
        chi_tmp = np.ascontiguousarray(chi + 0.5 * t2)  # chi_o - D_oe A_ee^-1 chi_e, D_oe = -1/2 D'
        host += time.perf_counter() - t0
        psi = np.zeros_like(chi_tmp)
        res = (G.Result * 1)()
        t0 = time.perf_counter()
        rc = ctx.lib.gbc_solve(ctx.h, C.byref(p), 1, psi.ctypes.data_as(C.POINTER(C.c_double)),
                               chi_tmp.ctypes.data_as(C.POINTER(C.c_double)), res)
        dev += time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(f"factory-path solve failed: {rc}")
        iters.append(res[0].n_count)
        t0 = time.perf_counter()
        t1 = op.apply(O.OP_DSLASH, psi, +1, 0)
        t2 = op.apply(O.OP_CLOVER_INV, chi + 0.5 * t1, +1, 0)  # psi_e = A_ee^-1 (chi_e - D_eo psi_o)
        r = op.apply(O.OP_UNPREC, psi + t2) - chi  # the residual PrecFermActQprop reports
        float(np.vdot(r, r).real)
        host += time.perf_counter() - t0
    return {"device_solves_s": dev, "host_schur_s": host, "total_s": dev + host,
            "inner_iterations_per_source": iters,
            "what": f"{nsrc} x gbc_solve(nrhs=1, GBC_SYS_MEO, host buffers) as the LinOp factory entry "
                    "runs under quarkProp4_a; the host Schur preparation, even reconstruction and residual "
                    "of PrecFermActQprop timed with the oracle's OpenMP operator in QDP++'s place"}


WEIGHTS = os.path.join(ROOT, "chroma_gb300", "weights", "cnn_16x16x16x32_k0.115_csw1.0.gbcw")
# the network retrained on this workload's volume and action (32^3 x 64, kappa 0.125, c_sw 1.6) from
# low-mode and full-inverse pairs on two configurations other than the benchmark's
WEIGHTS32 = os.path.join(ROOT, "chroma_gb300", "weights", "cnn_32x32x32x64_k0.125_csw1.6.gbcw")


def learned_headline(ctx, G, chi_d, nsrc, plain_s):
    """The benchmark spec's full form on the headline workload: the learned preconditioner inside
    FGMRES(16) (flexible, right-preconditioned), mixed precision (FP64 defect correction, FP16
    operator), the 12 sources as one batch; against plain FP64 CG on the same GPU.  Also one
    application of the network to the 12 sources and the same FGMRES without it."""
    import torch
    if not os.path.exists(WEIGHTS32):
        return None
    ctx.load_precond(WEIGHTS32)
    out = {"weights": os.path.basename(WEIGHTS32)}
    psi = torch.zeros_like(chi_d)
    for name, use in (("fgmres_with_net", 1), ("fgmres_without_net", 0)):
        res, rc = ctx.solve_device(psi.data_ptr(), chi_d.data_ptr(), nsrc, solver=G.SOLVER_FGMRES, system=G.SYS_FULL,
                                   rsd_target=RSD, sloppy_precision=G.PREC_HALF, nkrylov=16, use_precond=use)
        out[name] = {"seconds": res[0]["device_seconds"], "inner_iterations_max": max(r["n_count"] for r in res),
                     "true_rel_resid_max": max(r["rel_resid"] for r in res), "rc": rc}
    out["speedup_vs_plain_cg"] = plain_s / out["fgmres_with_net"]["seconds"] if plain_s else None
    sec, _ = ctx.time_operator(G.TIME_PRECOND, G.PREC_SINGLE, nrhs=nsrc, iters=3, flush_l2=True)
    out["network_application_12rhs_s"] = sec
    return out


def side_workloads(G):
    """The smaller configurations, each reported beside the headline (not part of `value`):
    - stout16: 16^3x32, eps 0.2 + 4 stout steps rho 0.1, kappa 0.12, c_sw 1.2, one Gaussian source:
      mixed FP16/FP64 (inner CGNE and inner BiCGStab) vs plain FP64 CG on the same GPU;
    - uneven_batch: 8^3x16, 12^3x24, 16^3x32, 20^3x40 (kappa 0.124, c_sw 1.5, one Z2 source each)
      solved as one batch vs one by one; the batch runs its inner iterations as one launch per
      step replayed from graphs (batched_*, the default) and as the persistent kernel
      (batched_persistent_*);
    - learned16: 16^3x32, kappa 0.115, c_sw 1.0, FGMRES(16) with and without the trained network on
      a gauge configuration outside its training set."""
    from chroma_gb300 import sources as S
    out = {}
    # stout-smeared 16^3 x 32
    dims = (16, 16, 16, 32)
    u = G.gauge_synthetic(dims, 0.2, 4242, n_stout=4, rho=0.1, t_boundary=-1)
    ctx = G.Context(dims, 1 / (2 * 0.12) - 4, 1.2, t_boundary=-1, max_rhs=1)
    ctx.load_gauge(u)
    chi = S.gaussian(dims, 17, cb=1).reshape(1, -1, 12)
    rec = {}
    for name, kw in (("mixed_fp16", dict(solver=G.SOLVER_MIXED)), ("mixed_fp16_bicgstab", dict(solver=G.SOLVER_BICGSTAB)),
                     ("plain_fp64_cg", dict(solver=G.SOLVER_CG))):
        ctx.solve(chi, rsd_target=RSD, **kw)  # warm-up (tuning, workspaces)
        ts = []
        for _ in range(3):
            _, res, rc = ctx.solve(chi, rsd_target=RSD, **kw)
            ts.append(res[0]["device_seconds"])
        rec[name] = {"seconds": statistics.median(ts), "iterations": res[0]["n_count"],
                     "true_rel_resid": res[0]["rel_resid"]}
    rec["speedup"] = rec["plain_fp64_cg"]["seconds"] / rec["mixed_fp16"]["seconds"]
    rec["speedup_bicgstab"] = rec["plain_fp64_cg"]["seconds"] / rec["mixed_fp16_bicgstab"]["seconds"]
    out["stout16"] = rec
    ctx.close()
    # uneven lattices
    lats = [(8, 8, 8, 16), (12, 12, 12, 24), (16, 16, 16, 32), (20, 20, 20, 40)]
    mass = 1 / (2 * 0.124) - 4
    ctxs, chis = [], []
    for k, d in enumerate(lats):
        c = G.Context(d, mass, 1.5, t_boundary=-1, max_rhs=1)
        c.load_gauge(G.gauge_synthetic(d, 0.3, 7000 + k, t_boundary=-1))
        ctxs.append(c)
        chis.append(S.z2_noise(d, 8000 + k, cb=1).reshape(-1, 12))
    batch = G.Batch(ctxs)
    paths = {}
    for mode in ("0", "1"):  # per-launch (graph-replayed) path, the default, then the persistent kernel
        os.environ["GBC_PERSISTENT"] = mode
        batch.solve(chis, rsd_target=RSD)
        tb = []
        for _ in range(3):
            _, res = batch.solve(chis, rsd_target=RSD)
            tb.append(res[0]["device_seconds"])
        paths[mode] = (statistics.median(tb), res[0]["launches"])
    os.environ.pop("GBC_PERSISTENT", None)
    for c, x in zip(ctxs, chis):
        c.solve(x.reshape(1, -1, 12), solver=G.SOLVER_MIXED, rsd_target=RSD)
    ts = []
    for _ in range(3):
        tot = 0.0
        for c, x in zip(ctxs, chis):
            _, r1, _ = c.solve(x.reshape(1, -1, 12), solver=G.SOLVER_MIXED, rsd_target=RSD)
            tot += r1[0]["device_seconds"]
        ts.append(tot)
    out["uneven_batch"] = {"lattices": ["x".join(map(str, d)) for d in lats],
                           "batched_seconds": paths["0"][0], "batched_launches": paths["0"][1],
                           "batched_persistent_seconds": paths["1"][0], "batched_persistent_launches": paths["1"][1],
                           "one_by_one_seconds": statistics.median(ts),
                           "true_rel_resid_max": max(r["rel_resid"] for r in res),
                           "iterations": [r["n_count"] for r in res]}
    batch.close()
    for c in ctxs:
        c.close()
    # learned preconditioner
    if os.path.exists(WEIGHTS):
        from chroma_gb300 import learn
        dims = (16, 16, 16, 32)
        ctx = G.Context(dims, 1 / (2 * 0.115) - 4, 1.0, t_boundary=-1, max_rhs=1)
        ctx.load_gauge(G.gauge_synthetic(dims, 0.3, 999_999, t_boundary=-1))
        ctx.load_precond(WEIGHTS)
        learn.ablation(ctx, dims)  # warm-up
        out["learned16"] = learn.ablation(ctx, dims)
        ctx.close()
    return out


def run_reference(args, rank, world):
    """--impl reference: Chroma's FP64 CG restated (the oracle) on all host cores.  One point source
    is solved to the target first (untimed by the steps) for the iteration count and the measured
    time of a whole single-source solve; each timed step is a bounded sample of CPU_SAMPLE_ITERS
    InvCG2 iterations; value = seconds per iteration x iterations x 12 sources."""
    if rank != 0:
        return
    dims = tuple(int(x) for x in args.dims.split(",")) if args.dims else DIMS
    from chroma_gb300 import sources as S
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    o = Oracle()
    links = o.apply_bc(dims, o.gauge_hot(dims, EPS, SEED), (1, 1, 1, -1))
    op = OracleOp(dims, links, 1 / (2 * KAPPA) - 4, CSW)
    src = S.point_sources(dims).reshape(12, -1, 12)
    t0 = time.perf_counter()
    _, info = op.qprop(src[0], rsd=RSD)
    one_source = time.perf_counter() - t0
    iters_full = info["n_count"]
    # an InvCG2 iteration costs the same for any source: time it on odd-site noise
    chi = S.gaussian(dims, 1, cb=1).reshape(-1, 12)
    k = CPU_SAMPLE_ITERS
    per_step = []
    for i in range(args.warmup + args.steps):
        per, _ = cg_iteration_seconds(op, chi, k)
        if i >= args.warmup:
            per_step.append(per)
    per_iter = statistics.median(per_step)
    value = per_iter * iters_full * 12
    line = {"metric": METRIC, "value": value, "unit": "s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_iter * k * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_desc(dims),
                       "solver": "Chroma's FP64 CGNE (InvCG2, CG_INVERTER) restated by the oracle, OpenMP on "
                                 "the host cores; sources one by one"},
            "cpu_baseline": {"value": value, "unit": "s", "cores": O.load().orc_num_threads(), "kind": "port",
                             "sample": f"{k} InvCG2 iterations per step on 1 source (per iteration from the "
                                       f"difference to a 2-iteration solve), x {iters_full} iterations (measured: "
                                       f"one point source solved to {RSD} in {one_source:.1f} s) x 12 sources",
                             "one_source_solve_s": one_source, "iterations_per_source": iters_full},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.op_only:
        op_only(args)
        return
    rank, world = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    from chroma_gb300 import gbclover as G
    dims = tuple(int(x) for x in args.dims.split(",")) if args.dims else DIMS
    V = int(np.prod(dims))
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    links, src = workload(dims)
    mass = 1 / (2 * KAPPA) - 4
    ctx = G.Context(dims, mass, CSW, t_boundary=-1, sloppy_precision=G.PREC_HALF, max_rhs=12)
    ctx.load_gauge(links)
    nsrc = src.shape[0]
    # device-resident sources / solutions in the canonical layout
    chi_d = torch.from_numpy(src.view(np.float64)).cuda()
    psi_d = torch.zeros_like(chi_d)
    # Delta 0.01: a reliable update (FP32 operator) each time the iterated residual fell by 100x
    solve_kw = dict(solver=G.SOLVER_BICGSTAB, system=G.SYS_FULL, rsd_target=RSD, sloppy_precision=G.PREC_HALF,
                    delta=DELTA, inner_tol=INNER_TOL)

    def step():
        res, rc = ctx.solve_device(psi_d.data_ptr(), chi_d.data_ptr(), nsrc, **solve_kw)
        if rc != 0:
            raise RuntimeError(f"solve failed: {rc} {res}")
        return res

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        step()
    clocks = Clocks()
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    times, results = [], []
    for _ in range(args.steps):
        flush.random_()  # L2 flush between timed steps (outside the events)
        torch.cuda.synchronize()
        if args.profile_timed:
            torch.cuda.profiler.start()
        res = step()
        if args.profile_timed:
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()
        times.append(res[0]["device_seconds"])
        results.append(res)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    t_step = max_over_ranks(sum(times) / len(times), world)
    value = t_step / world  # seconds per propagator over the whole job (N replicas)
    last = results[-1]
    psi_host = psi_d.cpu().numpy().view(np.complex128).reshape(nsrc, V, 12)

    # e2e through the public API with pinned host buffers, right after the device-timed steps
    chi_h = torch.from_numpy(src.view(np.float64).copy()).pin_memory()
    psi_h = torch.zeros_like(chi_h).pin_memory()
    e2e_t, e2e_dev, e2e_its = [], [], []
    import ctypes as C
    p = G.SolveParams(G.SOLVER_BICGSTAB, G.SYS_FULL, RSD, 10000, DELTA, 10.0, G.PREC_HALF, INNER_TOL, 0, 16, 0, 1)
    # the same K steps as the device-timed loop, each through gbc_solve with pinned host buffers
    e2e_clocks = Clocks()
    e2e_clocks.start()
    for i in range(args.steps):
        flush.random_()
        torch.cuda.synchronize()
        res_arr = (G.Result * nsrc)()
        t0 = time.perf_counter()
        rc = ctx.lib.gbc_solve(ctx.h, C.byref(p), nsrc, C.cast(psi_h.data_ptr(), C.POINTER(C.c_double)),
                               C.cast(chi_h.data_ptr(), C.POINTER(C.c_double)), res_arr)
        e2e_t.append(time.perf_counter() - t0)
        e2e_dev.append(res_arr[0].device_seconds)
        e2e_its.append(max(res_arr[r].n_count for r in range(nsrc)))
        if rc != 0:
            raise RuntimeError("e2e solve failed")
    e2e_clk = e2e_clocks.stop()
    e2e = max_over_ranks(sum(e2e_t) / len(e2e_t), world) / world
    nbytes = src.nbytes

    # plain FP64 CG on the same GPU, sources one at a time (quarkProp4_a's loop)
    plain, plain_iters, plain_res, err_vs_fp64 = None, [], [None], None
    if args.plain_steps > 0:
        plain_t, plain_res = [], []
        for _ in range(args.plain_steps):
            tot = 0.0
            its = []
            for k in range(nsrc):
                psi1 = torch.zeros_like(chi_d[k:k + 1])
                res, rc = ctx.solve_device(psi1.data_ptr(), chi_d[k:k + 1].data_ptr(), 1, solver=G.SOLVER_CG,
                                           system=G.SYS_FULL, rsd_target=RSD)
                if rc != 0:
                    raise RuntimeError(f"plain CG failed {res}")
                tot += res[0]["device_seconds"]
                its.append(res[0]["n_count"])
                plain_res.append(res[0]["rel_resid"])
            plain_t.append(tot)
            plain_iters = its
        plain = statistics.median(plain_t)
        # error of the accelerated solution against the FP64 CG solution of source 0
        psi_cg = torch.zeros_like(chi_d[0:1])
        ctx.solve_device(psi_cg.data_ptr(), chi_d[0:1].data_ptr(), 1, solver=G.SOLVER_CG, system=G.SYS_FULL,
                         rsd_target=1e-12)
        ref0 = psi_cg.cpu().numpy().view(np.complex128).reshape(V, 12)
        err_vs_fp64 = float(np.linalg.norm(psi_host[0] - ref0) / np.linalg.norm(ref0))

    # the same solve with the inner CGNE, and FP64 BiCGStab (12-RHS batch, FP64 defect correction
    # around an FP64 inner BiCGStab): context for the choice of the inner solver
    inner_cgne, plain_bicg, fp64_outer = None, None, None
    if args.plain_steps > 0:
        psi1 = torch.zeros_like(chi_d)
        for _ in range(2):  # the first one tunes the stencil variants that only CGNE uses
            res, rc = ctx.solve_device(psi1.data_ptr(), chi_d.data_ptr(), nsrc,
                                       **dict(solve_kw, solver=G.SOLVER_MIXED, delta=0.1, inner_tol=0.0))
        inner_cgne = {"seconds": res[0]["device_seconds"], "inner_iterations_per_rhs": res[0]["n_count"],
                      "true_rel_resid_max": max(r["rel_resid"] for r in res), "rc": rc}
        res, rc = ctx.solve_device(psi1.data_ptr(), chi_d.data_ptr(), nsrc,
                                   **dict(solve_kw, sloppy_precision=G.PREC_DOUBLE))
        plain_bicg = {"seconds": res[0]["device_seconds"], "iterations_per_rhs": res[0]["n_count"],
                      "true_rel_resid_max": max(r["rel_resid"] for r in res), "rc": rc}
        # the same headline solve with its Schur prep and intermediate outer residual in FP64
        # arithmetic instead of double-float (GBC_OUTER_DF=0)
        os.environ["GBC_OUTER_DF"] = "0"
        for _ in range(2):
            res, rc = ctx.solve_device(psi1.data_ptr(), chi_d.data_ptr(), nsrc, **solve_kw)
        os.environ.pop("GBC_OUTER_DF", None)
        fp64_outer = {"seconds": res[0]["device_seconds"], "inner_iterations_per_rhs": res[0]["n_count"],
                      "true_rel_resid_max": max(r["rel_resid"] for r in res), "rc": rc}

    # Roofline of the dominant kernel pair: the FP16 M~ on 12 RHS (the A_ee^-1 D_eo and the
    # A_oo x - 1/4 D_oe t launches the solve runs twice per iteration, 40 % of its time), cold L2
    # per application, autotuned shapes as in the solve; algorithmic bytes Vh (16L + 2C + 5*12 S)
    pk, pk_kind = peaks()
    sec, byts = ctx.time_operator(G.OP_MEO, G.PREC_HALF, nrhs=12, iters=20, flush_l2=True)
    secd, bytd = ctx.time_operator(G.OP_DSLASH, G.PREC_HALF, nrhs=12, iters=20, flush_l2=True)
    sec1, byts1 = ctx.time_operator(G.OP_DSLASH, G.PREC_HALF, nrhs=1, iters=20, flush_l2=True)
    secm, bytm = ctx.time_operator(G.OP_MEO, G.PREC_HALF, nrhs=1, iters=20, flush_l2=True)
    sec64, byts64 = ctx.time_operator(G.OP_DSLASH, G.PREC_DOUBLE, nrhs=1, iters=10, flush_l2=True)
    # the outer loop's operator on 12 right-hand sides: FP64 arithmetic and double-float
    m64, _ = ctx.time_operator(G.OP_MEO, G.PREC_DOUBLE, nrhs=12, iters=3, flush_l2=True)
    mdf, _ = ctx.time_operator(G.OP_MEO, G.PREC_DF64, nrhs=12, iters=3, flush_l2=True)
    achieved = byts / sec / 1e9
    # DRAM traffic of one such M~: a constant, not measured in this run (ncu cannot run inside the
    # benchmark) -- dram__bytes_read.sum + dram__bytes_write.sum of the M~'s two launches captured
    # once by ncu on 24^3x48 (Vh = 331776 sites, 12 RHS), scaled to this lattice by the number of
    # sites (the traffic of a launch grows with the sites it covers)
    traffic = M12_TRAFFIC_24 / 331776 * (V // 2)
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
            "traffic_source": "constant from one ncu capture of the 12-RHS M~ at 24^3x48, scaled by sites; "
                              "not measured in this run",
            "peak_kind": pk_kind,
            "kernel": "M~ on 12 RHS, FP16 storage, 12-real links: hop_kernel_rp (A_ee^-1 D_eo) + hop_kernel_async "
                      "(A_oo x - 1/4 D_oe t), autotuned",
            "unit_of_work": "one M~ application (its two stencil launches)",
            "bytes_per_launch": byts, "seconds_per_launch": sec,
            "dslash_12rhs_fp16_gbs": bytd / secd / 1e9, "dslash_12rhs_fp16_frac": bytd / secd / 1e9 / pk["hbm_gbs"],
            "single_rhs_fp16_gbs": byts1 / sec1 / 1e9, "single_rhs_fp16_frac": byts1 / sec1 / 1e9 / pk["hbm_gbs"],
            "single_rhs_meo_fp16_gbs": bytm / secm / 1e9, "single_rhs_meo_fp16_frac": bytm / secm / 1e9 / pk["hbm_gbs"],
            "single_rhs_fp64_gbs": byts64 / sec64 / 1e9,
            "meo_12rhs_fp64_s": m64, "meo_12rhs_double_float_s": mdf}


    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and plain_iters:
        from chroma_gb300 import sources as S
        # the cost of an InvCG2 iteration does not depend on the source: time it on odd-site noise
        cpu = cpu_baseline(dims, links, S.gaussian(dims, 1, cb=1).reshape(-1, 12), int(np.median(plain_iters)), nsrc)

    # the oracle's FP64 check of the solutions, and the path a factory-only Chroma input takes
    check, factory = None, None
    if rank == 0 and not args.no_oracle_check:
        check, op = oracle_check(dims, links, src, psi_host)
        if not args.no_extras:
            factory = chroma_factory_path(ctx, G, op, src, solve_kw)
            factory["batched_hook_e2e_s"] = e2e
        del op

    extras = {} if args.no_extras else side_workloads(G)
    if not args.no_extras:
        extras["learned32"] = learned_headline(ctx, G, chi_d, nsrc, plain)
    iters = [r["n_count"] for r in last]
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f16-storage/f32-arith inner, f64 outer", "data": "synthetic",
        "config": {"workload": workload_desc(dims),
                   "solver": "FP64 defect correction + reliable-update BiCGStab on M~ (FP16 stencil, "
                             f"12-real links, Delta {DELTA}, InnerTol {INNER_TOL}), 12-RHS batch",
                   "l2": "256 MiB L2 flush between timed steps; the fields exceed L2",
                   "parallelism": f"replicas x{world}"},
        "plain_cg_fp64_s": plain, "speedup_vs_plain_cg": plain / value if (value and plain) else None,
        "iterations": {"mixed_inner_per_rhs_median": int(np.median(iters)), "plain_cg_per_rhs": plain_iters},
        "same_solve_inner_cgne": inner_cgne, "same_solve_fp64_outer_steps": fp64_outer,
        "plain_bicgstab_fp64_batched": plain_bicg,
        "true_rel_resid_max": max(r["rel_resid"] for r in last),
        "plain_cg_true_rel_resid_max": max(plain_res) if plain else None,
        "rel_error_vs_fp64_cg_src0": err_vs_fp64,
        "oracle_check": check,
        "chroma_factory_path": factory,
        "roofline": roof,
        "cpu_baseline": cpu,
        # a zero-guess full-system solve uploads only the sources (gbc_solve skips the psi upload)
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "device_seconds_median": statistics.median(e2e_dev), "steps_seconds": e2e_t,
                "steps_device_seconds": e2e_dev, "steps_inner_iterations_max": e2e_its, "clocks": e2e_clk},
        "gpu_launches": int(sum(r[0]["launches"] for r in results)),
        "clocks": clk,
        "side_workloads": extras,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()

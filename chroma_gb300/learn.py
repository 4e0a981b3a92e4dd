"""Training of the learned preconditioner (runs on the GPU through the library's own kernels).

Recipe: on each of `configs` seeded gauge configurations, `samples` seeded Gaussian vectors b
on the odd sites are solved approximately by `cg_iters` iterations of plain FP64 CGNE; the
residual r = b - M~ x_k and the error e = x* - x_k that those iterations leave (dominated by the
low modes the Krylov method resolves last) form the training pairs, x* the FP64 solution to
1e-10.  The network K is trained with Adam on |K(r) - e|^2 / |e|^2, cycling through the
configurations, and saved in the versioned weights format of gbc_precond_save.

    python -m chroma_gb300.learn --dims 16,16,16,32 --kappa 0.115 --csw 1.0 --out weights.gbcw
    python -m chroma_gb300.learn --config5 weights/cnn_32x32x32x64 --configs 2 --samples 8 --rounds 3
"""
import argparse
import json
import time

import numpy as np

from . import gbclover as G
from . import sources as S


def training_pairs(ctx, dims, nsamples, seed, cg_iters=50, rsd=1e-10, batch=12):
    """(r, e) pairs: r = b - M~ x_k and e = x* - x_k after cg_iters CGNE iterations from zero
    (cg_iters = 0 gives the full-inverse pairs (b, M~^-1 b))."""
    V = int(np.prod(dims))
    rs, es = [], []
    for k0 in range(0, nsamples, batch):
        nb = min(batch, nsamples - k0)
        b = np.stack([S.gaussian(dims, seed * 100003 + k0 + k, cb=1).reshape(V, 12) for k in range(nb)])
        xs, res, rc = ctx.solve(b, solver=G.SOLVER_MIXED, rsd_target=rsd)
        if cg_iters > 0:
            xk, _, _ = ctx.solve(b, solver=G.SOLVER_CG, max_iter=cg_iters, rsd_target=1e-30, raise_on_error=False)
        else:
            xk = np.zeros_like(b)
        r = b - ctx.apply(G.OP_MEO, xk, +1, 1, G.PREC_DOUBLE)
        e = xs - xk
        par = S.parity(dims)
        r[:, par == 0] = 0
        e[:, par == 0] = 0
        rs.append(r)
        es.append(e)
    return np.concatenate(rs), np.concatenate(es)


def train(dims, kappa, csw, eps=0.3, configs=8, samples=32, cg_iters=50, seed=1000, rounds=4, epochs=5, batch=8,
          lr=2e-3, hidden=12, layers=4, out=None, log=print, full_pairs=0):
    mass = 1 / (2 * kappa) - 4
    ctx = G.Context(dims, mass, csw, t_boundary=-1, max_rhs=12)
    ctx.precond_init(hidden=hidden, layers=layers, seed=seed)
    data = []
    t0 = time.time()
    for cfg in range(configs):
        links = G.gauge_synthetic(dims, eps, seed + cfg, t_boundary=-1)
        ctx.load_gauge(links)
        r, e = training_pairs(ctx, dims, samples, seed + cfg, cg_iters)
        if full_pairs:
            # as many full-inverse pairs: the network must also act sensibly on every mode that
            # FGMRES feeds it, not only on the low modes
            rf, ef = training_pairs(ctx, dims, full_pairs, seed + cfg + 7919, 0)
            r, e = np.concatenate([r, rf]), np.concatenate([e, ef])
        data.append((links, r, e))
        log(f"config {cfg}: {len(r)} pairs, |e|/|r| = {np.linalg.norm(e) / np.linalg.norm(r):.3f}")
    history = []
    for rnd in range(rounds):
        for cfg, (links, r, e) in enumerate(data):
            ctx.load_gauge(links)
            losses = ctx.precond_train(r, e, epochs=epochs, batch=batch, lr=lr, seed=rnd * 1000 + cfg)
            history.append(float(losses[-1] / batch))
        log(f"round {rnd}: mean relative loss {np.mean(history[-configs:]):.4f} ({time.time() - t0:.1f} s)")
    if out:
        ctx.precond_save(out)
    return ctx, history


def ablation(ctx, dims, seed=77, rsd=1e-10, sloppy=G.PREC_SINGLE, kappa=None):
    """FGMRES(16) on a configuration outside the training set, with and without the network."""
    V = int(np.prod(dims))
    chi = S.z2_noise(dims, seed, cb=1).reshape(1, V, 12)
    out = {}
    for use in (0, 1):
        _, res, rc = ctx.solve(chi, solver=G.SOLVER_FGMRES, use_precond=use, rsd_target=rsd, sloppy_precision=sloppy,
                               raise_on_error=False)
        out["with_net" if use else "without_net"] = {"iterations": res[0]["n_count"], "seconds": res[0]["seconds"],
                                                     "rel_resid": res[0]["rel_resid"], "status": res[0]["status"]}
    return out


def network_seconds(ctx, nrhs, prec=G.PREC_SINGLE, iters=5):
    """Device time of one application of the loaded network to nrhs odd-site fields (CUDA events)."""
    sec, _ = ctx.time_operator(G.TIME_PRECOND, prec, nrhs=nrhs, iters=iters, flush_l2=True)
    return sec


def propagator_study(ctx, dims, seed=999_999, eps=0.3, rsd=1e-10, sloppy=G.PREC_HALF, nkrylov=16):
    """The 12 point sources of one held-out configuration solved as one batch of the full system
    (FP64 defect correction, mixed precision): FGMRES(nkrylov) with and without the loaded
    network, and the reliable BiCGStab without it, on the same context."""
    ctx.load_gauge(G.gauge_synthetic(dims, eps, seed, t_boundary=-1))
    src = S.point_sources(dims).reshape(12, -1, 12)
    out = {}
    runs = (("fgmres_with_net", dict(solver=G.SOLVER_FGMRES, use_precond=1, nkrylov=nkrylov)),
            ("fgmres_without_net", dict(solver=G.SOLVER_FGMRES, use_precond=0, nkrylov=nkrylov)),
            ("bicgstab_without_net", dict(solver=G.SOLVER_BICGSTAB, delta=0.01, inner_tol=1e-5)))
    for name, kw in runs:
        _, res, rc = ctx.solve(src, system=G.SYS_FULL, rsd_target=rsd, sloppy_precision=sloppy, raise_on_error=False,
                               **kw)
        out[name] = {"inner_iterations_max": max(r["n_count"] for r in res), "device_seconds": res[0]["device_seconds"],
                     "true_rel_resid_max": max(r["rel_resid"] for r in res), "status": rc}
    out["network_seconds_12rhs"] = network_seconds(ctx, 12)
    return out


def config5(out_prefix, configs=2, samples=8, full_pairs=8, rounds=3, epochs=4, log=print):
    """The learned preconditioner at the 32^3 x 64 propagator workload (kappa 0.125, c_sw 1.6):
    trained on this volume with the low-mode pairs of 50 CG iterations alone, and with as many
    full-inverse pairs added; each network studied on a held-out configuration's 12-source solve."""
    dims, kappa, csw = (32, 32, 32, 64), 0.125, 1.6
    result = {}
    for variant, fp in (("low_mode", 0), ("low_mode_and_full_inverse", full_pairs)):
        t0 = time.time()
        ctx, hist = train(dims, kappa, csw, configs=configs, samples=samples, cg_iters=50, rounds=rounds,
                          epochs=epochs, out=f"{out_prefix}_{variant}.gbcw", log=log, full_pairs=fp)
        train_s = time.time() - t0
        study = propagator_study(ctx, dims)
        result[variant] = {"training_seconds": train_s, "loss_history": hist, "pairs_per_config": samples + fp,
                           "configs": configs, **study}
        log(json.dumps({variant: result[variant]}))
        ctx.close()
    return result


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", default="16,16,16,32")
    ap.add_argument("--kappa", type=float, default=0.115)
    ap.add_argument("--csw", type=float, default=1.0)
    ap.add_argument("--configs", type=int, default=8)
    ap.add_argument("--samples", type=int, default=32)
    ap.add_argument("--rounds", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=5)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--cg-iters", type=int, default=50)
    ap.add_argument("--full-pairs", type=int, default=0)
    ap.add_argument("--out", default=None)
    ap.add_argument("--config5", default=None, metavar="PREFIX",
                    help="train and study the network at 32^3x64 (kappa 0.125, c_sw 1.6); weights to PREFIX_*.gbcw")
    a = ap.parse_args()
    if a.config5:
        print(json.dumps(config5(a.config5, configs=a.configs, samples=a.samples, full_pairs=a.full_pairs or a.samples,
                                 rounds=a.rounds, epochs=a.epochs)))
        return
    dims = tuple(int(x) for x in a.dims.split(","))
    ctx, hist = train(dims, a.kappa, a.csw, configs=a.configs, samples=a.samples, rounds=a.rounds, epochs=a.epochs,
                      lr=a.lr, out=a.out, cg_iters=a.cg_iters, full_pairs=a.full_pairs)
    links = G.gauge_synthetic(dims, 0.3, 999_999, t_boundary=-1)
    ctx.load_gauge(links)
    print(json.dumps({"loss_history": hist, "ablation": ablation(ctx, dims)}))


if __name__ == "__main__":
    main()

"""Parameter sweeps with the batched ensemble and the learned surrogate.

    python -m main_gb300.sweep [--train 4096] [--held-out 256] [--sweep 4096] [--periods 500] ...

prints one JSON line with the surrogate's held-out errors and the timing of a
surrogate-screened sweep against plain simulation.

* ``simulate`` runs replicas in batched ensembles (``main_gb300.ensemble``)
  and returns their labels: the propulsion speed averaged over the run after
  its first fifth, the rotational diffusion from the axis autocorrelation
  over the whole run, and the B concentration around the dimer on 64 x 32
  (z, r) bins averaged over the second half.
* ``fit`` trains the surrogate (``main_gb300.surrogate``) on simulated
  replicas only.
* ``sweep`` predicts every point of a parameter sweep, sends the points it
  selects (the fastest predicted, and those where two independently trained
  networks disagree) back to the plain simulation, and reports the time of
  both routes.  The plain route runs every point through the simulator; its
  one-run-at-a-time form (single-context runs, as the reference runs a job
  array) is timed on a sample and scaled to the sweep.
"""
import argparse
import json
import math
import time

import numpy as np

from . import ensemble as E
from . import surrogate as S

FIELD_ZMAX, FIELD_RMAX = 8.0, 8.0


def simulate(reps, periods, batch=1024, field_every=10, precision=32, verbose=False):
    """Labels of every replica (speed, rotational diffusion, field [n, 64 * 32])
    and the simulated particle-steps and seconds."""
    n = len(reps)
    speed = np.zeros(n)
    drot = np.zeros(n)
    field = np.zeros((n, S.FIELD_Z * S.FIELD_R))
    ps, secs = 0, 0.0
    half = periods // 2
    warm = periods // 5
    for lo in range(0, n, batch):
        sub = reps[lo:lo + batch]
        ens = E.Ensemble(sub, precision=precision)
        P = ens.mpc_every
        t0 = time.perf_counter()
        ens.initial()
        ens.prepare()
        ens.reset_samples(history=periods)
        ens.run(warm * P)
        mean_a, cnt_a, _ = ens.samples()
        sum_a = mean_a * cnt_a
        ens.run((half - warm) * P)
        done = half
        while done < periods:
            k = min(field_every, periods - done)
            ens.run(k * P)
            done += k
            ens.field_accumulate(S.FIELD_Z, S.FIELD_R, FIELD_ZMAX, FIELD_RMAX)
        mean_b, cnt_b, axes = ens.samples()
        ens.synchronize()
        secs += time.perf_counter() - t0
        ps += int(sum(r["n_solvent"] for r in sub)) * P * periods
        second = (mean_b * cnt_b - sum_a) / np.maximum(cnt_b - cnt_a, 1)
        speed[lo:lo + len(sub)] = second
        drot[lo:lo + len(sub)] = E.rotational_diffusion(axes, dt=ens.cfg.mpc_dt, max_lag=max(2, periods // 5))
        field[lo:lo + len(sub)] = ens.concentration_field().reshape(len(sub), -1)
        ens.close()
        if verbose:
            print("simulated %d / %d replicas (%.1f s)" % (lo + len(sub), n, secs), flush=True)
    return speed, drot, field, ps, secs


def fit(X, Y, epochs=60, seed=1, lr=1e-3, batch=256, verbose=False):
    """A trained surrogate and its scaler."""
    sc = S.Scaler(X, Y)
    net = S.Mlp(batch=batch, max_rows=65536, seed=seed, lr=lr)
    w = S.output_weights()
    losses = S.train(net, sc.x(X), sc.y(Y), w, epochs, seed=seed, log_every=10 if verbose else 0)
    return net, sc, losses


def predict(net, sc, X, cols=None):
    """Denormalised predictions [n, outputs] (the first `cols` outputs only
    when given: the screen reads the speed without copying the fields)."""
    out = []
    for lo in range(0, len(X), 65536):
        y = net.forward(sc.x(X[lo:lo + 65536]))
        if cols is not None:
            y = y[:, :cols]
        out.append(y.cpu().numpy().astype(np.float64))
    Y = np.concatenate(out)
    k = Y.shape[1]
    return Y * sc.ys[:k] + sc.ym[:k]


def forward_device_ms(net, sc, X, repeats=5):
    """Device time of one forward pass over X (CUDA events around the call)."""
    import torch
    x = torch.as_tensor(sc.x(X), device="cuda")
    net.forward(x)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(repeats):
        net.forward(x)
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / repeats


def single_context_seconds(reps, periods):
    """Seconds of plain single-context runs (one box per context, one after
    the other), each from initial placement to the end of the run."""
    from . import Engine
    t = 0.0
    for rep in reps:
        cfg = E.config_of_replica(rep, precision=32)
        t0 = time.perf_counter()
        e = Engine(cfg)
        e.initial()
        e.prepare()
        e.run(periods * cfg["mpc_every"])
        e.synchronize()
        t += time.perf_counter() - t0
        e.close()
    return t


def r2(pred, true):
    return 1.0 - float(((pred - true) ** 2).sum() / max(((true - true.mean()) ** 2).sum(), 1e-300))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=4096)
    ap.add_argument("--held-out", type=int, default=256)
    ap.add_argument("--sweep", type=int, default=4096)
    ap.add_argument("--infer", type=int, default=65536)
    ap.add_argument("--periods", type=int, default=500)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--keep", type=float, default=0.02, help="fraction of the sweep sent back to the simulator")
    ap.add_argument("--single-sample", type=int, default=8, help="single-context runs timed for the plain route")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args(argv)
    out = {"config": {"train": a.train, "held_out": a.held_out, "sweep": a.sweep, "periods": a.periods,
                      "epochs": a.epochs, "keep": a.keep}}

    # training data: replicas of the wide sampler, simulated in batched ensembles
    reps_tr = E.sample_replicas(a.train, seed=11, base_seed=10_000, wide=True)
    sp, dr, fd, ps_tr, t_gen = simulate(reps_tr, a.periods, verbose=a.verbose)
    X_tr = E.surrogate_inputs(reps_tr)
    Y_tr = S.targets(sp, dr, fd)
    t0 = time.perf_counter()
    net, sc, losses = fit(X_tr, Y_tr, epochs=a.epochs, seed=1, verbose=a.verbose)
    net2, sc2, _ = fit(X_tr, Y_tr, epochs=a.epochs, seed=2)
    t_train = time.perf_counter() - t0
    out["training"] = {"generate_s": t_gen, "particle_steps": ps_tr, "train_s": t_train,
                       "loss_first": losses[0], "loss_last": losses[-1], "steps": len(losses)}

    # held-out plain runs: new parameter points, new seeds
    reps_ho = E.sample_replicas(a.held_out, seed=12, base_seed=20_000, wide=True)
    sp_ho, dr_ho, fd_ho, _, _ = simulate(reps_ho, a.periods)
    X_ho = E.surrogate_inputs(reps_ho)
    P_ho = predict(net, sc, X_ho)
    pred_sp = P_ho[:, 0]
    rel = np.abs(pred_sp - sp_ho) / np.maximum(np.abs(sp_ho), 1e-12)
    # the plain runs' own noise: the same held-out points again with other seeds
    reps_rep = [dict(r, seed=r["seed"] + 5_000_000) for r in reps_ho]
    sp_rep, _, fd_rep, _, _ = simulate(reps_rep, a.periods)
    plain_mean = 0.5 * (sp_ho + sp_rep)
    out["held_out"] = {
        "speed_rel_err_median": float(np.median(rel)),
        "speed_within_5pct": float((rel <= 0.05).mean()),
        "speed_rmse": float(np.sqrt(((pred_sp - sp_ho) ** 2).mean())),
        "speed_rmse_plain_vs_plain": float(np.sqrt(((sp_rep - sp_ho) ** 2).mean())),
        "speed_rmse_vs_two_seed_mean": float(np.sqrt(((pred_sp - plain_mean) ** 2).mean())),
        "mean_speed_rel_err": float(abs(pred_sp.mean() - sp_ho.mean()) / max(abs(sp_ho.mean()), 1e-12)),
        "speed_r2": r2(pred_sp, sp_ho), "speed_r2_plain_vs_plain": r2(sp_rep, sp_ho),
        "log_drot_r2": r2(P_ho[:, 1], np.log10(np.clip(dr_ho, 1e-6, None))),
        "field_r2": r2(P_ho[:, 2:].ravel(), fd_ho.ravel()),
        "field_r2_plain_vs_plain": r2(fd_rep.ravel(), fd_ho.ravel()),
    }

    # inference throughput at 65,536 points
    X_inf = E.surrogate_inputs(E.sample_replicas(min(a.infer, 65536), seed=13, wide=True))
    predict(net, sc, X_inf[:1024], cols=2)
    t0 = time.perf_counter()
    predict(net, sc, X_inf, cols=2)
    t_host = time.perf_counter() - t0
    ms = forward_device_ms(net, sc, X_inf)
    rows = len(X_inf)
    shapes = net.shapes()
    flops = 2.0 * rows * sum(n * k for n, k in shapes)
    # the bytes a forward pass cannot avoid: the FP32 inputs (and their BF16
    # 64-column copy written and read), every BF16 activation written once and
    # read once, the BF16 weights, and the FP32 outputs
    hidden = [n for n, _ in shapes[:-1]]
    nbytes = (rows * shapes[0][1] * 4 + 2 * rows * 64 * 2 + sum(2 * rows * h * 2 for h in hidden)
              + sum(n * k * 2 for n, k in shapes) + rows * shapes[-1][0] * 4)
    out["inference"] = {"points": rows, "seconds_with_host": t_host, "device_ms": ms,
                        "tflops": flops / (ms * 1e-3) / 1e12, "flops": flops,
                        "bytes": nbytes, "gbs": nbytes / (ms * 1e-3) / 1e9}

    # the sweep: surrogate screen + plain fallback, against plain simulation of every point
    reps_sw = E.sample_replicas(a.sweep, seed=14, base_seed=30_000, wide=True)
    X_sw = E.surrogate_inputs(reps_sw)
    t0 = time.perf_counter()
    p1 = predict(net, sc, X_sw, cols=1)[:, 0]
    p2 = predict(net2, sc2, X_sw, cols=1)[:, 0]
    unc = np.abs(p1 - p2)
    sel = S.screen(p1, unc, keep_fraction=a.keep, trust=np.quantile(unc, 1.0 - a.keep / 2))
    sp_sel, _, _, _, t_fb = simulate([reps_sw[i] for i in sel], a.periods)
    t_screened = time.perf_counter() - t0
    t_single = single_context_seconds(reps_sw[:a.single_sample], a.periods)
    t_plain_single = t_single / a.single_sample * a.sweep
    # batched plain route on a sample of the sweep, scaled
    nb = min(a.sweep, 512)
    _, _, _, _, t_b = simulate(reps_sw[:nb], a.periods)
    t_plain_batched = t_b / nb * a.sweep
    out["sweep"] = {
        "points": a.sweep, "fallback_points": int(len(sel)), "screened_s": t_screened, "fallback_s": t_fb,
        "plain_single_context_s": t_plain_single, "plain_single_context_sample": a.single_sample,
        "plain_batched_s": t_plain_batched, "plain_batched_sample": nb,
        "speedup_vs_single_context": t_plain_single / t_screened,
        "speedup_vs_batched_plain": t_plain_batched / t_screened,
        "speedup_vs_single_context_with_training": t_plain_single / (t_screened + t_gen + t_train),
        "fallback_rel_err_median": float(np.median(np.abs(p1[sel] - sp_sel) / np.maximum(np.abs(sp_sel), 1e-12))),
    }
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()

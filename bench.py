#!/usr/bin/env python
"""Throughput benchmark: MPC+MD particle-steps/s on GB300.

A step is one collision period: mpc_every (= 50) MD steps of the solvent and
sphere dimers plus one reactive multiparticle collision (main_pattern.f95:
203-225 iterated 50 times).  Particle-steps = solvent particles x MD steps, all
50 MD steps counted for every particle.  The default workload is the 256^3-cell
Selkov-kinetics run (167,772,160 solvent particles, 512 dimers), synthetic and
seeded; its resident state (24 GB) is far larger than L2, so no flush is needed
between timed steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c2] [--scale 1.0]
    python bench.py --impl reference ...   (times the FP64 CPU restatement)

Under torchrun each rank runs an independent replica (seed + rank); the line
reports the aggregate over ranks with the max time over ranks.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MPC+MD particle-steps/s, 1 GB300; param-sweep time surrogate vs plain @≤5% err"
UNIT = "particle-steps/s"
WORKLOAD_TEXT = {
    "c0": "plain single dimer: 30^3 periodic cells, 270,000 solvent, 1 dimer, reaction_simple",
    "c1": "collective quasi-2D: 128x128x16 cells with z walls and reactive floor, 2,621,440 solvent, 64 dimers",
    "c2": "Selkov kinetics: 256^3 periodic cells, 167,772,160 solvent (FP32 cell-relative SoA, uint8 species), "
          "512 sphere dimers, six-channel RKMPC",
    "rot": "rotor grid (rotational_code/2d_array): 64x64x32 cells with z walls, 1,310,720 solvent, "
           "6x6 anchored dimers with a harmonic z tether",
    "rot_line": "rotor line (rotational_code/linear_periodic_ci): 256x64x32 cells with z walls, 5,242,880 solvent, "
                "13 anchored dimers",
    "rot_owner": "rotor line with owner tags (rotational_code/linear_periodic_no_ci): 256x64x32 cells with z walls, "
                 "5,242,880 solvent, 13 anchored dimers",
}
FALLBACK_HBM = 6800.0

# algorithmic bytes per unit of each kernel kind (FP32 build): the bytes each
# unit's state must move through DRAM once, whatever the kernel does
BYTES_PER_PARTICLE_REBUILD = 46      # read flag+cell+offset+velocity (29 B), write cell+offset+flag (17 B)
BYTES_PER_SHELL_ENTRY = 84           # shell entry written (55 B) and the previous shell entry read (29 B)
BYTES_PER_SHELL_FORCE = 87           # shell particle read (54 B) and written back (33 B) per MD step
BYTES_PER_PARTICLE_ROTATE = 33       # flag + shifted key + cell + velocity read, velocity written
BYTES_PER_CELL = 56                  # collision accumulator read + reset (32 B), rotation table written (24 B)
BYTES_PER_CELL_REACTION = 74         # packed counts + first keys + affected, read and reset


def rank_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rk = int(os.environ.get("RANK", "0"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rk, lr


def max_over_ranks(x, dist, device="cuda"):
    """The largest of each rank's x (every rank gets it); x itself without a
    process group.  `device`: where the reduction tensor lives (cuda for
    NCCL, cpu for gloo)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(ws, n_per_rank, md_steps, periods, seconds):
    """Whole-job particle-steps/s of ws replicas that each advanced n_per_rank
    particles by md_steps x periods MD steps, timed by the slowest rank."""
    return ws * n_per_rank * md_steps * periods / seconds


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.path = tempfile.mktemp(prefix="mpcmd_clocks_", suffix=".csv")
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        # the timed region starts after the first sample: nvidia-smi's own
        # start-up can hold the NVIDIA kernel driver for a good part of a second, which
        # would land inside a short timed region
        t0 = time.time()
        while self.proc is not None and time.time() - t0 < 10.0:
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.05)
        time.sleep(0.1)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        return json.load(open(p))
    except Exception:
        return {}


def cpu_sample_config(name, threads):
    from main_gb300 import config
    # same density, dimer density and physics; a box small enough for a bounded CPU sample
    scale = {"c0": 1.0, "c1": 0.5, "c2": 0.25, "rot": 0.5, "rot_line": 0.25, "rot_owner": 0.25}[name]
    return config.workload(name, scale=scale, precision=64), scale


def cpu_baseline(name, cycles_max=5, seconds=12.0, cell_lists=False, full=False):
    """FP64 oracle (OpenMP, all host cores) on a bounded sample of the workload.
    cell_lists: the pair search through cell bins instead of the reference's
    all-pairs loop (same lists, same results; a faster CPU for comparison).
    full: the workload at its full size instead of the sample (one timed
    collision period after the untimed initial placement and prepare)."""
    from oracle.oracle import Oracle
    import oracle.oracle as O
    from main_gb300 import config
    threads = os.cpu_count() or 1
    if full:
        cfg, scale = config.workload(name, precision=64), 1.0
    else:
        cfg, scale = cpu_sample_config(name, threads)
    o = Oracle(cfg, threads=threads)
    if cell_lists:
        o.set_list_mode(O.LISTS_CELLS)
    o.initial()
    o.prepare()
    S = cfg["mpc_every"]
    t0 = time.perf_counter()
    cycles = 0
    while cycles < cycles_max:
        o.run(S)
        cycles += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    value = cfg["n_solvent"] * S * cycles / dt
    box = "%dx%dx%d cells, %d solvent, %d dimers" % (cfg["lx"], cfg["ly"], cfg["lz"], cfg["n_solvent"],
                                                      cfg["n_dimers"])
    sample = ("%s scaled by %.2f per edge: %s; %d collision period(s) of %d MD steps after prepare"
              % (name, scale, box, cycles, S))
    return {"value": value, "unit": UNIT, "cores": O.lib().orc_set_threads(0), "kind": "port",
            "sample": sample, "seconds": dt, "box": box}


def pinned_state(n, ns):
    import numpy as np
    try:
        import torch
        mk = lambda shape, dt: torch.empty(shape, dtype=dt).pin_memory().numpy()
        st = {k: mk((n,), torch.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
        st["flag"] = mk((n,), torch.int32)
        for k in ("dpos", "dvel", "dforce"):
            st[k] = mk((max(ns, 1), 3), torch.float64)
        return st, True
    except Exception:
        st = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz")}
        st["flag"] = np.zeros(n, dtype=np.int32)
        for k in ("dpos", "dvel", "dforce"):
            st[k] = np.zeros((max(ns, 1), 3))
        return st, False


def gpu_arm(args, ws, rk, lr, dist):
    import numpy as np
    import main_gb300
    from main_gb300 import Engine, config

    main_gb300.set_device(lr)
    extra = {"n_dimers": args.dimers} if args.dimers else {}
    cfg = config.workload(args.workload, scale=args.scale, precision=32, seed=1 + rk, **extra)
    S = cfg["mpc_every"]
    N = cfg["n_solvent"]
    e = Engine(cfg)
    if args.resort is not None:
        e.set_resort(args.resort * S)
    e.initial()
    e.prepare()
    e.run(args.warmup * S)

    def barrier():
        if dist is not None:
            dist.barrier()

    # pass A: headline timing (CUDA events on the engine stream)
    barrier()
    e.synchronize()
    with Clocks(lr) as ck:
        l0 = main_gb300.kernel_launches()
        e.event_record(0)
        e.run(args.steps * S)
        e.event_record(1)
        ms = e.event_elapsed(0, 1)
        launches = main_gb300.kernel_launches() - l0
    barrier()
    clocks = ck.summary()
    ms = max_over_ranks(ms, dist)
    value = aggregate_rate(ws, N, S, args.steps, ms * 1e-3)

    # pass B: per-launch timing of each kernel kind over the same kind of region
    e.profile(True)
    e.run(args.steps * S)
    prof = e.profile_read()
    e.profile(False)
    work = e.counters()   # device work totals of pass B
    ncs = e.n_cells_shifted()
    nc = e.ncell

    def per_launch(total, kind):
        return total / max(prof[kind][1], 1)

    def bytes_per_launch(kind):
        # the work each kernel did, averaged over its launches: the rebuilds
        # between collisions visit only the watch list, the force kernel only
        # the active shell entries
        if kind == "rebuild":
            vis = per_launch(work["work_rebuild_particles"], "rebuild")
            placed = per_launch(work["work_rebuild_placed"], "rebuild")
            return vis * BYTES_PER_PARTICLE_REBUILD + placed * BYTES_PER_SHELL_ENTRY, vis, "particles visited"
        if kind == "force":
            ent = per_launch(work["work_force_entries"], "force")
            return ent * BYTES_PER_SHELL_FORCE, ent, "active shell entries"
        if kind == "rotate_main":
            return N * BYTES_PER_PARTICLE_ROTATE, N, "particles"
        if kind == "cells":
            return ncs * BYTES_PER_CELL + nc * BYTES_PER_CELL_REACTION, ncs, "cells"
        return None, None, None

    kinds = sorted(prof, key=lambda k: -prof[k][0])
    dom = next(k for k in kinds if bytes_per_launch(k)[0] is not None)
    tot_ms, cnt = prof[dom]
    avg_ms = tot_ms / max(cnt, 1)
    b, units, unit_name = bytes_per_launch(dom)
    peak, peak_kind = measured_hbm()
    achieved = b / (avg_ms * 1e-3) / 1e9
    traffic = ncu_traffic().get(args.workload, {}).get(dom)
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_kind,
        "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
        "algorithmic_bytes_per_launch": int(b), "units_per_launch": int(units), "unit_kind": unit_name,
        "avg_launch_ms": round(avg_ms, 4), "launches": cnt,
        "share_of_timed": {k: round(prof[k][0] / sum(v[0] for v in prof.values()), 4) for k in kinds if prof[k][1]},
    }

    # mean period over one whole sort cycle of the workload (its sort_every MD
    # steps, the sort included): the cell order of the particles decays
    # between sorts, which the periods right after the warm-up do not show
    whole = None
    if not args.no_whole_run and cfg["sort_every"] > 0:
        periods = max(1, cfg["sort_every"] // S)
        r0 = e.counters()["resorts"]
        barrier()
        e.synchronize()
        e.event_record(2)
        e.run(periods * S)
        e.event_record(3)
        wms = max_over_ranks(e.event_elapsed(2, 3), dist)
        whole = {"periods": periods, "ms_per_step": wms / periods,
                 "value": aggregate_rate(ws, N, S, periods, wms * 1e-3),
                 "order_only_resorts": e.counters()["resorts"] - r0,
                 "what": "mean over %d consecutive collision periods (one sort every %d MD steps and the "
                         "order-only re-sorts included)" % (periods, cfg["sort_every"])}

    # e2e: the reference-facing C ABI with host buffers, host<->device copies inside
    e2e = None
    if not args.no_e2e:
        ns = 2 * cfg["n_dimers"]
        host, pinned = pinned_state(N, ns)
        cur = e.download_state()
        for k in host:
            host[k][...] = cur[k] if k != "flag" else cur[k].astype(np.int32)
        barrier()
        t0 = time.perf_counter()
        e.upload_state(host)
        tu = time.perf_counter()
        e.prepare()
        e.synchronize()
        tp = time.perf_counter()
        for _ in range(args.steps):
            e.run(S)
            e.observables()
        tl = time.perf_counter()
        e.download_state(out=host)   # into the same page-locked buffers
        t1 = time.perf_counter()
        phases = {"upload": round(tu - t0, 4), "prepare": round(tp - tu, 4), "periods": round(tl - tp, 4),
                  "download": round(t1 - tl, 4)}
        state_bytes = N * (6 * 8 + 4) + ns * 3 * 8 * 3
        obs_bytes = 8 * 16 + ns * 3 * 8 + cfg["n_dimers"] * 8
        e2e_s = t1 - t0
        e2e_s = max_over_ranks(e2e_s, dist)
        e2e = {"value": aggregate_rate(ws, N, S, args.steps, e2e_s), "unit": UNIT,
               "h2d_bytes_per_step": int(state_bytes / args.steps),
               "d2h_bytes_per_step": int((state_bytes + args.steps * obs_bytes) / args.steps),
               "pinned_host": pinned, "phases_s": phases,
               "what": "upload of the full host state, prepare, %d x (collision period + observables), download "
                       "of the full host state" % args.steps}
    return dict(value=value, ms=ms, launches=launches, clocks=clocks, roofline=roofline, e2e=e2e, cfg=cfg,
                dev_bytes=e.device_bytes(), whole=whole)


ENSEMBLE_TEXT = ("batched ensemble: %d independent single-dimer periodic replicas, box edge U{16..48}, density "
                 "U[5,20], sigma_C U[2,5], sigma_N U[1,3], bond sigma_C+sigma_N+U[0.5,1.5], k2 log-U[1e-3,1e-1], "
                 "own seed each; one launch per stage, one CUDA graph per collision period, autotuned schedule")


def ensemble_replicas(n, rank=0):
    from main_gb300 import ensemble as E
    return E.sample_replicas(n, seed=1 + rank, base_seed=1000 + 100000 * rank)


def cpu_baseline_ensemble(reps, seconds=12.0):
    """The FP64 oracle (all host cores) running replicas of the ensemble one
    after the other, as the reference runs its job array, one collision
    period each, until `seconds` have passed."""
    from main_gb300 import ensemble as E
    from oracle.oracle import Oracle
    import oracle.oracle as O
    threads = os.cpu_count() or 1
    done_ps, dt, used = 0, 0.0, 0
    for rep in reps:
        cfg = E.config_of_replica(rep, precision=64)
        o = Oracle(cfg, threads=threads)
        o.initial()
        o.prepare()
        t0 = time.perf_counter()
        o.run(cfg["mpc_every"])
        dt += time.perf_counter() - t0
        done_ps += rep["n_solvent"] * cfg["mpc_every"]
        used += 1
        if dt > seconds:
            break
    return {"value": done_ps / dt, "unit": UNIT, "cores": O.lib().orc_set_threads(0), "kind": "port",
            "sample": "the first %d replicas of the ensemble, one after the other, one collision period each "
                      "after prepare (%d solvent in all)" % (used, sum(r["n_solvent"] for r in reps[:used])),
            "seconds": dt}


def ensemble_arm(args, ws, rk, lr, dist):
    """Batched ensemble workload: aggregate particle-steps/s over all replicas."""
    import numpy as np
    import main_gb300
    from main_gb300 import ensemble as E
    main_gb300.set_device(lr)
    reps = ensemble_replicas(args.replicas, rk)
    ens = E.Ensemble(reps, precision=32)
    ens.initial()
    ens.prepare()
    cache = os.path.join(ROOT, "main_gb300", "_build", "ensemble_schedules.txt")
    if args.schedule:
        ens.set_schedule(*[int(v) for v in args.schedule.split(",")])
        sched = ens.schedule()
    else:
        sched = ens.autotune(cache, periods=2)
    P = ens.mpc_every
    N = int(sum(r["n_solvent"] for r in reps))
    ens.run(args.warmup * P)

    def barrier():
        if dist is not None:
            dist.barrier()

    ens.reset_samples(0)
    barrier()
    ens.synchronize()
    with Clocks(lr) as ck:
        c0 = ens.counters()
        ens.event_record(0)
        ens.run(args.steps * P)
        ens.event_record(1)
        ms = ens.event_elapsed(0, 1)
        c1 = ens.counters()
    barrier()
    ms = max_over_ranks(ms, dist)
    value = aggregate_rate(ws, N, P, args.steps, ms * 1e-3)
    speeds, cnt, _ = ens.samples()
    obs = ens.observables()
    shell = sum(o["n_inside"] for o in obs)
    cells = sum(r["lx"] * r["ly"] * r["lz"] for r in reps)
    # whole collision period, algorithmic bytes: each particle's 25 B state
    # read and written once, each shell particle's state every MD step, the
    # cell table once
    b = 50.0 * N + 54.0 * shell * P + 8.0 * cells
    peak, peak_kind = measured_hbm()
    achieved = b / (ms / args.steps * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": "whole collision period (one graph replay)", "achieved": round(achieved, 1),
                "peak": peak, "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": None, "algorithmic_bytes_per_launch": int(b),
                "what": "B = 50 N + 54 N_shell S + 8 C per period over all replicas, N_shell at the end"}
    e2e = None
    if not args.no_e2e:
        # the public API with host buffers: upload every replica's FP64 state,
        # prepare, the timed periods with observables, download every replica
        states = [ens.download(r) for r in range(len(reps))]
        barrier()
        t0 = time.perf_counter()
        for r, stt in enumerate(states):
            ens.upload(r, stt)
        ens.prepare()
        for _ in range(args.steps):
            ens.run(P)
            ens.observables()
        for r in range(len(reps)):
            ens.download(r)
        e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
        sb = N * (6 * 8 + 4) + len(reps) * 3 * 3 * 8 * 2
        e2e = {"value": aggregate_rate(ws, N, P, args.steps, e2e_s), "unit": UNIT,
               "h2d_bytes_per_step": int(sb / args.steps),
               "d2h_bytes_per_step": int((sb + args.steps * len(reps) * 200) / args.steps),
               "what": "upload of every replica's host state, prepare, %d x (collision period + observables), "
                       "download of every replica" % args.steps}
    return dict(value=value, ms=ms, launches=c1["launches"] - c0["launches"], clocks=ck.summary(), roofline=roofline,
                e2e=e2e, reps=reps, N=N, speeds=speeds, samples=cnt, schedule=sched, dev_bytes=ens.device_bytes(),
                replays=c1["graph_replays"] - c0["graph_replays"], rebuilds=c1["rebuilds"] - c0["rebuilds"])


def main_ensemble(args, ws, rk, lr):
    import numpy as np
    conf = {"workload": ENSEMBLE_TEXT % args.replicas, "name": "c3", "replicas_per_rank": args.replicas,
            "md_steps_per_step": 50, "collisions_per_step": 1,
            "l2": "inputs larger than L2 (resident state >> 129 MB), no flush",
            "parallelism": "replicas" if ws > 1 else "single"}
    if args.impl == "reference":
        if rk != 0:
            return 0
        reps = ensemble_replicas(args.replicas, 0)
        cb = cpu_baseline_ensemble(reps, seconds=max(5.0, args.cpu_seconds))
        conf["measured_on"] = cb["sample"]
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": conf,
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(lr)
        tdist.init_process_group("nccl")
        dist = tdist
    r = ensemble_arm(args, ws, rk, lr, dist)
    cb = None
    if rk == 0 and ws == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline_ensemble(r["reps"], seconds=args.cpu_seconds)
        cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    if rk == 0:
        sp = np.asarray(r["speeds"])
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": conf,
                "roofline": r["roofline"], "cpu_baseline": cb, "e2e": r["e2e"], "gpu_launches": r["launches"],
                "clocks": r["clocks"], "device_bytes": r["dev_bytes"],
                "ensemble": {"replicas": len(r["reps"]), "solvent_total": r["N"], "schedule": list(r["schedule"]),
                             "graph_replays": r["replays"], "rebuilds": r["rebuilds"],
                             "speed_mean": float(sp.mean()), "speed_min": float(sp.min()),
                             "speed_max": float(sp.max()), "samples_per_replica": int(np.min(r["samples"])),
                             "speed_per_replica": [round(float(v), 6) for v in sp]}}
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main_surrogate(args, ws, rk, lr):
    """Learned surrogate workload: a 4096-point parameter sweep screened by the
    surrogate with plain-simulation fallback against plain simulation of every
    point (main_gb300.sweep); the value is the speed-up of the sweep."""
    if rk != 0:
        return 0
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the surrogate workload has no reference "
                          "counterpart; its plain route is timed inside the line of --impl gb300"}))
        return 0
    import main_gb300
    from main_gb300 import sweep
    main_gb300.set_device(lr)
    argv = ["--train", str(args.train), "--held-out", str(args.held_out), "--sweep", str(args.sweep),
            "--periods", str(args.periods), "--epochs", str(args.epochs)]
    out = sweep.main(argv)
    try:
        pk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, hbm, peak_kind = float(pk["bf16_tflops"]), float(pk["hbm_gbs"]), "measured"
    except Exception:
        peak, hbm, peak_kind = 1900.0, 6800.0, "fallback"
    inf = out["inference"]
    sw = out["sweep"]
    line = {"metric": METRIC, "value": sw["speedup_vs_single_context"], "unit": "x (sweep time plain / surrogate)",
            "n_gpus": ws, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * sw["screened_s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (network), f32 (simulation)",
            "data": "synthetic (seeded replicas simulated by the engine)",
            "config": {"workload": "learned surrogate: MLP 8 -> 4 x 256 SiLU -> 2 + 64 x 32, BF16 weights with FP32 "
                                   "accumulation, trained on %d batched-ensemble replicas (Adam, lr 1e-3, batch 256); "
                                   "%d-point sweep screened with plain-simulation fallback; %d collision periods per "
                                   "run" % (args.train, args.sweep, args.periods), "name": "c4"},
            # at K = 256 the forward pass moves more bytes than the tensor
            # cores need time for (the FP32 output alone is 537 MB at 65,536
            # points): its binding roofline is HBM; the tensor fraction is
            # given beside it
            "roofline": {"bound": "hbm", "kernel": "k_gemm (forward of %d points, five launches)" % inf["points"],
                         "achieved": round(inf["gbs"], 1), "peak": hbm, "peak_source": peak_kind,
                         "unit": "GB/s", "frac": round(inf["gbs"] / hbm, 4), "traffic": None,
                         "algorithmic_bytes_per_launch": int(inf["bytes"]),
                         "what": "inputs, BF16 activations written and read once, weights, FP32 outputs",
                         "tensor": {"achieved": round(inf["tflops"], 2), "peak": peak, "unit": "TFLOP/s",
                                    "frac": round(inf["tflops"] / peak, 4)}},
            "surrogate": out}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="c2", choices=["c0", "c1", "c2", "c3", "c4", "rot", "rot_line", "rot_owner"])
    ap.add_argument("--train", type=int, default=4096, help="c4: training replicas")
    ap.add_argument("--held-out", type=int, default=256, help="c4: held-out plain runs")
    ap.add_argument("--sweep", type=int, default=4096, help="c4: sweep points")
    ap.add_argument("--periods", type=int, default=500, help="c4: collision periods per run")
    ap.add_argument("--epochs", type=int, default=60, help="c4: training epochs")
    ap.add_argument("--replicas", type=int, default=256, help="replicas of the c3 ensemble workload")
    ap.add_argument("--schedule", default="", help="c3: tile,block,shell_block instead of the autotuner")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--dimers", type=int, default=0, help="override the dimer count (profiling cases)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-full", action="store_true", help="skip the full-size CPU period")
    ap.add_argument("--no-whole-run", action="store_true", help="skip the whole-run mean period time")
    ap.add_argument("--resort", type=int, default=None,
                    help="collision periods between order-only re-sorts (0: none; default: the engine's)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rk, lr = rank_info()

    if args.workload == "c3":
        return main_ensemble(args, ws, rk, lr)
    if args.workload == "c4":
        return main_surrogate(args, ws, rk, lr)

    from main_gb300 import config
    cfg0 = config.workload(args.workload, scale=args.scale, **({"n_dimers": args.dimers} if args.dimers else {}))
    conf = {
        "workload": WORKLOAD_TEXT[args.workload] if args.scale == 1.0 and not args.dimers else
        "%s scaled by %.3g per edge (%dx%dx%d cells, %d solvent, %d dimers)" % (
            args.workload, args.scale, cfg0["lx"], cfg0["ly"], cfg0["lz"], cfg0["n_solvent"], cfg0["n_dimers"]),
        "name": args.workload, "solvent_per_rank": cfg0["n_solvent"], "dimers_per_rank": cfg0["n_dimers"],
        "md_steps_per_step": cfg0["mpc_every"], "collisions_per_step": 1,
        "l2": "inputs larger than L2 (resident state >> 129 MB), no flush" if cfg0["n_solvent"] > 5_000_000 else
              "state fits in L2: every timed step streams the whole state once per collision period",
        "parallelism": "replicas" if ws > 1 else "single",
    }

    if args.impl == "reference":
        if rk != 0:
            return 0
        cb = cpu_baseline(args.workload, cycles_max=args.steps + args.warmup, seconds=1e9)
        # the CPU port runs a bounded sample of the workload: the line names
        # the box it measured, and the rate is per particle-step
        conf = dict(conf, workload="%s (bounded CPU sample of: %s)" % (cb["box"], conf["workload"]),
                    sample_box=cb["box"], measured_on="the sample box; particle-steps/s per particle-step")
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * cb["seconds"] / (args.steps + args.warmup), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": conf,
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    dist = None
    if ws > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(lr)
        tdist.init_process_group("nccl")
        dist = tdist
    r = gpu_arm(args, ws, rk, lr, dist)
    cb = None
    if rk == 0 and ws == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(args.workload, seconds=args.cpu_seconds)
        cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        # the same sample with the pair search through cell bins (same lists,
        # same trajectory), the faster of the two CPU loop structures
        cc = cpu_baseline(args.workload, seconds=args.cpu_seconds, cell_lists=True)
        cb["cell_list_value"] = cc["value"]
        if not args.no_cpu_full:
            # one period of the cell-list port at the workload's full size, to
            # show that the per-particle-step rate of the sample carries over
            cf = cpu_baseline(args.workload, cycles_max=1, seconds=1e9, cell_lists=True, full=True)
            cb["full_config_value"] = cf["value"]
            cb["full_config_sample"] = cf["sample"] + " (cell-binned pair search)"
    if rk == 0:
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": conf, "roofline": r["roofline"], "cpu_baseline": cb, "e2e": r["e2e"],
                "gpu_launches": r["launches"], "clocks": r["clocks"], "device_bytes": r["dev_bytes"],
                "whole_run": r["whole"]}
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

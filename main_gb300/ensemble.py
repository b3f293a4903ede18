"""Batched ensemble of single-dimer replicas (mpcmd_ens_* in include/mpcmd.h).

Hundreds of independent plain periodic runs (the collective_code step of
main_pattern.f95:203-225 with a periodic box and one sphere dimer), each with
its own box, density, sphere sizes, bond, interaction, rate and seed, advance
together on one GPU: one launch per stage covers every replica, each replica
decides its own list rebuilds on the device, and every collision period
replays as one CUDA graph.  The reference runs such replicas as the separate
jobs of a job array (rotational_code/linear_periodic_langevin/setup/
5_make_subjobs.sh with per-job inputs from 4_random_numbers_to_runs.sh).

``sample_replicas`` draws the replica parameters of the ensemble workload
(box edge U{16..48}, density U[5, 20], sigma_C U[2, 5], sigma_N U[1, 3],
bond sigma_C + sigma_N + U[0.5, 1.5], k2 log-uniform in [1e-3, 1e-1], seed per
replica); with ``wide=True`` also eps_B on N U[0.05, 1] and kT U[0.1, 0.25]
(the eight inputs of the learned surrogate).

The per-replica labels the surrogate learns come from here: the propulsion
speed (Output_SelkovDimer.f90:168-172), the rotational diffusion from the
axis autocorrelation (collective_code/1D_Orientation_Correlation.py:40-53)
and the axisymmetric B concentration around the dimer.
"""
import ctypes as C
import math

import numpy as np

from . import MpcmdEnsembleConfig, MpcmdError, MpcmdObs, MpcmdReplica, config, lib

CUT = 2.0 ** (1.0 / 6.0)


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def replica(lx, ly=None, lz=None, density=10.0, n_solvent=None, seed=1, rc=4.0, rn=2.0, dcn=6.5,
            eps_c=(1.0, 1.0, 1.0, 1.0), eps_n=(1.0, 0.1, 1.0, 1.0), kT=1.0 / 6.0, k1=0.01,
            mass=(1.0, 1.0, 1.0, 1.0), mc=0.0, mn=0.0):
    """Parameters of one replica (by default the plain single-dimer run: sigma_C 4, sigma_N 2, bond 6.5,
    density 10, kT 1/6, k1 0.01)."""
    ly = lx if ly is None else ly
    lz = lx if lz is None else lz
    n = int(round(density * lx * ly * lz)) if n_solvent is None else int(n_solvent)
    return dict(lx=int(lx), ly=int(ly), lz=int(lz), n_solvent=n, seed=int(seed), rc=float(rc), rn=float(rn),
                dcn=float(dcn), eps_c=list(eps_c), eps_n=list(eps_n), kT=float(kT), k1=float(k1),
                mass=list(mass), mc=float(mc), mn=float(mn))


def replica_of_config(cfg):
    """The replica of a single-context configuration (periodic, one dimer)."""
    return replica(cfg["lx"], cfg["ly"], cfg["lz"], n_solvent=cfg["n_solvent"], seed=cfg["seed"], rc=cfg["rc"],
                   rn=cfg["rn"], dcn=cfg["dcn"], eps_c=cfg["eps_c"], eps_n=cfg["eps_n"], kT=cfg["kT"],
                   k1=cfg["k"][0], mass=cfg["mass"], mc=cfg["mc"], mn=cfg["mn"])


def config_of_replica(rep, precision=64, md_dt=0.01, mpc_dt=0.5, rot_angle=2.0 * math.pi / 3.0, skin=1.5,
                      sort_every=10000, cell_capacity=100):
    """The single-context configuration (main_gb300.Engine) that runs the
    same replica on its own: the parity reference of the ensemble."""
    return config.base_config(
        lx=rep["lx"], ly=rep["ly"], lz=rep["lz"], geometry=config.GEOM_PERIODIC, n_dimers=1,
        kinetics=config.KIN_SIMPLE, exclusion=config.EXCL_PARTICLE, catalysis=config.CAT_DETERMINISTIC,
        rotation_sense=1, n_solvent=rep["n_solvent"], seed=rep["seed"], init_count=[rep["n_solvent"], 0, 0, 0],
        mass=list(rep["mass"]), eps_c=list(rep["eps_c"]), eps_n=list(rep["eps_n"]), rc=rep["rc"], rn=rep["rn"],
        dcn=rep["dcn"], mc=rep["mc"], mn=rep["mn"], kT=rep["kT"], k=[rep["k1"], 0, 0, 0, 0, 0], md_dt=md_dt,
        mpc_dt=mpc_dt, rot_angle=rot_angle, skin=skin, sort_every=sort_every, cell_capacity=cell_capacity,
        precision=precision)


def sample_replicas(n, seed=0, base_seed=1000, wide=False, skin=1.5, edge=(16, 48)):
    """Replica parameters of the ensemble workload (see the module docstring).
    The box edge is redrawn from the edges that keep the bond and the list
    radii below half the box (unique minimum images)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        rc = rng.uniform(2.0, 5.0)
        rn = rng.uniform(1.0, 3.0)
        dcn = rc + rn + rng.uniform(0.5, 1.5)
        rho = rng.uniform(5.0, 20.0)
        k1 = 10.0 ** rng.uniform(-3.0, -1.0)
        eps_bn = rng.uniform(0.05, 1.0) if wide else 0.1
        kT = rng.uniform(0.1, 0.25) if wide else 1.0 / 6.0
        need = 2.0 * max(dcn, rc * CUT + skin) + 1e-9
        lo = max(edge[0], int(math.floor(need)) + 1)
        L = int(rng.integers(lo, max(lo, edge[1]) + 1))
        out.append(replica(L, density=rho, seed=base_seed + i, rc=rc, rn=rn, dcn=dcn,
                           eps_n=(1.0, eps_bn, 1.0, 1.0), kT=kT, k1=k1))
    return out


def surrogate_inputs(reps):
    """The eight surrogate inputs of each replica: sigma_C, sigma_N, bond,
    eps_B on N, k2, density, kT, box edge."""
    return np.array([[r["rc"], r["rn"], r["dcn"], r["eps_n"][1], r["k1"], r["n_solvent"] / (r["lx"] * r["ly"] * r["lz"]),
                      r["kT"], r["lx"]] for r in reps], dtype=np.float64)


class Ensemble:
    """One batched ensemble on the current CUDA device."""

    def __init__(self, replicas, precision=32, md_dt=0.01, mpc_dt=0.5, rot_angle=2.0 * math.pi / 3.0, skin=1.5,
                 sort_every=10000, cell_capacity=100, rattle_max_iter=100000, schedule=(0, 0, 0)):
        self.reps = [dict(r) for r in replicas]
        R = len(self.reps)
        arr = (MpcmdReplica * R)()
        for i, r in enumerate(self.reps):
            a = arr[i]
            a.lx, a.ly, a.lz = r["lx"], r["ly"], r["lz"]
            a.n_solvent, a.seed = r["n_solvent"], r["seed"]
            for k in range(4):
                a.mass[k] = r["mass"][k]; a.eps_c[k] = r["eps_c"][k]; a.eps_n[k] = r["eps_n"][k]
            a.rc, a.rn, a.dcn, a.mc, a.mn, a.kT, a.k1 = r["rc"], r["rn"], r["dcn"], r["mc"], r["mn"], r["kT"], r["k1"]
        cfg = MpcmdEnsembleConfig(R, precision, sort_every, cell_capacity, rattle_max_iter, schedule[0], schedule[1],
                                  schedule[2], md_dt, mpc_dt, rot_angle, skin)
        self.cfg = cfg
        self.mpc_every = int(round(mpc_dt / md_dt))
        h = C.c_void_p()
        st = lib().mpcmd_ens_create(C.byref(cfg), arr, C.byref(h))
        if st != 0:
            raise MpcmdError(st, "ens_create")
        self.h = h
        self.R = R
        self.n = np.array([r["n_solvent"] for r in self.reps], dtype=np.int64)

    def close(self):
        if getattr(self, "h", None):
            lib().mpcmd_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, st, what):
        if st != 0:
            raise MpcmdError(st, what)

    def initial(self):
        self._c(lib().mpcmd_ens_initial(self.h), "ens_initial")

    def prepare(self):
        self._c(lib().mpcmd_ens_prepare(self.h), "ens_prepare")

    def run(self, nsteps):
        self._c(lib().mpcmd_ens_run(self.h, int(nsteps)), "ens_run")

    def upload(self, r, st):
        f = lambda k: np.ascontiguousarray(st[k], dtype=np.float64)
        arrs = [f(k) for k in ("x", "y", "z", "vx", "vy", "vz")]
        flag = np.ascontiguousarray(st["flag"], dtype=np.int32)
        dpos = f("dpos").reshape(-1)
        dvel = np.ascontiguousarray(st.get("dvel", np.zeros((2, 3))), dtype=np.float64).reshape(-1)
        dfrc = np.ascontiguousarray(st.get("dforce", np.zeros((2, 3))), dtype=np.float64).reshape(-1)
        if arrs[0].size != self.n[r]:
            raise ValueError("upload: replica %d holds %d particles" % (r, self.n[r]))
        dp = C.c_double
        self._c(lib().mpcmd_ens_upload(self.h, r, *[_ptr(a, dp) for a in arrs], _ptr(flag, C.c_int32),
                                       _ptr(dpos, dp), _ptr(dvel, dp), _ptr(dfrc, dp)), "ens_upload")

    def download(self, r):
        n = int(self.n[r])
        out = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz")}
        out["flag"] = np.zeros(n, dtype=np.int32)
        for k in ("dpos", "dvel", "dforce"):
            out[k] = np.zeros((2, 3))
        dp = C.c_double
        self._c(lib().mpcmd_ens_download(self.h, r, *[_ptr(out[k], dp) for k in ("x", "y", "z", "vx", "vy", "vz")],
                                         _ptr(out["flag"], C.c_int32), _ptr(out["dpos"], dp),
                                         _ptr(out["dvel"], dp), _ptr(out["dforce"], dp)), "ens_download")
        return out

    def observables(self):
        o = (MpcmdObs * self.R)()
        self._c(lib().mpcmd_ens_observables(self.h, o), "ens_observables")
        return [{"momentum": np.array(x.momentum[:]), "solvent_momentum": np.array(x.solvent_momentum[:]),
                 "kinetic_solvent": x.kinetic_solvent, "kinetic_dimer": x.kinetic_dimer, "potential": x.potential,
                 "species_count": np.array(x.species_count[:]), "n_inside": x.n_inside, "time_count": x.time_count,
                 "time_penetrate": x.time_penetrate, "cstep": x.cstep} for x in o]

    def reset_samples(self, history=0):
        self.history = int(history)
        self._c(lib().mpcmd_ens_reset_samples(self.h, self.history), "ens_reset_samples")

    def samples(self):
        """(mean propulsion speed [R], samples [R], unit axes [R, history, 3])."""
        mean = np.zeros(self.R)
        cnt = np.zeros(self.R, dtype=np.int64)
        h = getattr(self, "history", 0)
        axes = np.zeros((self.R, max(h, 1), 3), dtype=np.float32)
        self._c(lib().mpcmd_ens_samples(self.h, _ptr(mean, C.c_double), _ptr(cnt, C.c_int64),
                                        _ptr(axes, C.c_float) if h > 0 else None), "ens_samples")
        return mean, cnt, axes[:, :h]

    def field_accumulate(self, nz=64, nr=32, zmax=8.0, rmax=8.0):
        self.field_shape = (nz, nr, zmax, rmax)
        self._c(lib().mpcmd_ens_field_accumulate(self.h, nz, nr, zmax, rmax), "ens_field_accumulate")

    def field_read(self):
        """B counts per replica on (z, r) bins [R, nz, nr] and the number of accumulated samples."""
        nz, nr = self.field_shape[:2]
        c = np.zeros((self.R, nz, nr), dtype=np.uint32)
        s = C.c_int64(0)
        self._c(lib().mpcmd_ens_field_read(self.h, _ptr(c, C.c_uint32), C.byref(s)), "ens_field_read")
        return c, s.value

    def concentration_field(self):
        """B number density over the mean solvent density on the (z, r) bins,
        averaged over the accumulated samples [R, nz, nr]."""
        counts, samples = self.field_read()
        nz, nr, zmax, rmax = self.field_shape
        dz, dr = 2.0 * zmax / nz, rmax / nr
        r_lo = np.arange(nr) * dr
        vol = math.pi * ((r_lo + dr) ** 2 - r_lo ** 2) * dz
        rho = np.array([r["n_solvent"] / (r["lx"] * r["ly"] * r["lz"]) for r in self.reps])
        return counts / (max(samples, 1) * vol[None, None, :] * rho[:, None, None])

    def set_schedule(self, particle_tile, block, shell_block):
        self._c(lib().mpcmd_ens_set_schedule(self.h, particle_tile, block, shell_block), "ens_set_schedule")

    def schedule(self):
        s = np.zeros(3, dtype=np.int32)
        self._c(lib().mpcmd_ens_get_schedule(self.h, _ptr(s, C.c_int32)), "ens_get_schedule")
        return tuple(int(v) for v in s)

    def autotune(self, cache_path=None, periods=2):
        self._c(lib().mpcmd_ens_autotune(self.h, cache_path.encode() if cache_path else None, periods),
                "ens_autotune")
        return self.schedule()

    def counters(self):
        c = np.zeros(6, dtype=np.int64)
        self._c(lib().mpcmd_ens_counters(self.h, _ptr(c, C.c_int64), 6), "ens_counters")
        return dict(zip(("launches", "graph_replays", "status", "rattle_iters", "rebuilds", "cstep"),
                        (int(v) for v in c)))

    def event_record(self, slot):
        self._c(lib().mpcmd_ens_event_record(self.h, slot), "ens_event_record")

    def event_elapsed(self, a, b):
        ms = C.c_double(0)
        self._c(lib().mpcmd_ens_event_elapsed(self.h, a, b, C.byref(ms)), "ens_event_elapsed")
        return ms.value

    def synchronize(self):
        self._c(lib().mpcmd_ens_synchronize(self.h), "ens_synchronize")

    def device_bytes(self):
        b = C.c_int64(0)
        lib().mpcmd_ens_device_bytes(self.h, C.byref(b))
        return b.value


def rotational_diffusion(axes, dt, max_lag=None):
    """Rotational diffusion of each replica from its unit-axis samples
    [R, K, 3] taken every dt: C(t) = <u(s) . u(s + t)> over s
    (collective_code/1D_Orientation_Correlation.py:40-53, first Legendre
    order) decays as exp(-2 D_r t); D_r is the least-squares slope of
    -ln C(t) / 2 through the origin over the lags where C(t) > 0.2."""
    axes = np.asarray(axes, dtype=np.float64)
    R, K, _ = axes.shape
    max_lag = max_lag or max(1, K // 3)
    out = np.zeros(R)
    for r in range(R):
        t, y = [], []
        for lag in range(1, max_lag + 1):
            c = float(np.mean(np.sum(axes[r, :-lag] * axes[r, lag:], axis=1)))
            if c <= 0.2:
                break
            t.append(lag * dt)
            y.append(-math.log(c) / 2.0)
        t, y = np.array(t), np.array(y)
        out[r] = float((t * y).sum() / (t * t).sum()) if len(t) else float("nan")
    return out

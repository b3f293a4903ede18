"""GB300-native hybrid MD / reactive multiparticle-collision engine.

Python front end of the C ABI in include/mpcmd.h (libmpcmd.so, built in-tree
by main_gb300/build.py).  ``Engine`` mirrors the reference module call
surface of rober468/main (collective_code/main_pattern.f95 and the modules it
calls): ``initial``, ``prepare``, ``evolve``, ``distribute``, ``mpc_rotation``,
``reaction``, ``sort``, ``rebuild_lists``, plus ``step``/``run`` for whole
main-loop iterations.  There is no CPU fallback: every call runs the CUDA
library, and a missing library raises.
"""
import ctypes as C
import os

import numpy as np

from . import config
from .config import MpcmdConfig, to_struct, workload  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("MPCMD_LIB") or os.path.join(HERE, "_build", "libmpcmd.so")

STATUS = {
    0: "ok", 1: "invalid configuration", 2: "allocation failed", 3: "cell capacity exceeded",
    4: "shell or neighbour capacity exceeded", 5: "RATTLE did not converge", 6: "initial placement failed",
    7: "call out of order", 8: "CUDA error", 9: "checkpoint i/o failed", 10: "checkpoint corrupt or mismatched",
}


class MpcmdError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__("mpcmd %s failed: %s (%d)" % (what, STATUS.get(status, "?"), status))


class MpcmdConcParams(C.Structure):
    _fields_ = [("x_slab", C.c_double), ("y_slab", C.c_double), ("z_slab", C.c_double),
                ("half_width", C.c_double), ("x_width", C.c_double), ("y_width", C.c_double),
                ("z_width", C.c_double)]


class MpcmdObs(C.Structure):
    _fields_ = [
        ("momentum", C.c_double * 3), ("solvent_momentum", C.c_double * 3), ("kinetic_solvent", C.c_double),
        ("kinetic_dimer", C.c_double), ("potential", C.c_double), ("species_count", C.c_int64 * 4),
        ("n_inside", C.c_int64), ("n_pairs", C.c_int64), ("time_count", C.c_int32),
        ("time_penetrate", C.c_int32), ("cstep", C.c_int64),
    ]


class MpcmdReplica(C.Structure):
    """mpcmd_replica (include/mpcmd.h): one replica of a batched ensemble."""
    _fields_ = [("lx", C.c_int32), ("ly", C.c_int32), ("lz", C.c_int32), ("reserved", C.c_int32),
                ("n_solvent", C.c_int64), ("seed", C.c_uint64), ("mass", C.c_double * 4),
                ("eps_c", C.c_double * 4), ("eps_n", C.c_double * 4), ("rc", C.c_double), ("rn", C.c_double),
                ("dcn", C.c_double), ("mc", C.c_double), ("mn", C.c_double), ("kT", C.c_double),
                ("k1", C.c_double)]


class MpcmdEnsembleConfig(C.Structure):
    """mpcmd_ensemble_config (include/mpcmd.h)."""
    _fields_ = [("n_replicas", C.c_int32), ("precision", C.c_int32), ("sort_every", C.c_int32),
                ("cell_capacity", C.c_int32), ("rattle_max_iter", C.c_int32), ("particle_tile", C.c_int32),
                ("block", C.c_int32), ("shell_block", C.c_int32), ("md_dt", C.c_double), ("mpc_dt", C.c_double),
                ("rot_angle", C.c_double), ("skin", C.c_double)]


class MpcmdMlpConfig(C.Structure):
    """mpcmd_mlp_config (include/mpcmd.h)."""
    _fields_ = [("n_in", C.c_int32), ("n_hidden", C.c_int32), ("n_layers", C.c_int32), ("n_out", C.c_int32),
                ("batch", C.c_int32), ("max_rows", C.c_int32), ("seed", C.c_uint64), ("lr", C.c_double),
                ("beta1", C.c_double), ("beta2", C.c_double), ("eps", C.c_double)]


_lib = None

# Every entry point declared in include/mpcmd.h with its ctypes signature.
_P = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
SIGNATURES = {
    "mpcmd_create": (C.c_int, [C.POINTER(MpcmdConfig), C.POINTER(_P)]),
    "mpcmd_destroy": (C.c_int, [_P]),
    "mpcmd_error_string": (C.c_char_p, [C.c_int]),
    "mpcmd_device_bytes": (C.c_int, [_P, _lp]),
    "mpcmd_upload_state": (C.c_int, [_P, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp]),
    "mpcmd_download_state": (C.c_int, [_P, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp]),
    "mpcmd_set_cell_order": (C.c_int, [_P, _ip, C.c_int64]),
    "mpcmd_set_owner_tags": (C.c_int, [_P, _ip]),
    "mpcmd_get_owner_tags": (C.c_int, [_P, _ip]),
    "mpcmd_set_anchors": (C.c_int, [_P, _dp]),
    "mpcmd_get_anchors": (C.c_int, [_P, _dp]),
    "mpcmd_set_step": (C.c_int, [_P, C.c_int64, C.c_int32]),
    "mpcmd_set_collision": (C.c_int, [_P, C.c_double, C.c_double, _dp]),
    "mpcmd_set_resort": (C.c_int, [_P, C.c_int64]),
    "mpcmd_set_reactive_grid": (C.c_int, [_P, _ip]),
    "mpcmd_initial": (C.c_int, [_P]),
    "mpcmd_prepare": (C.c_int, [_P]),
    "mpcmd_prepare_restart": (C.c_int, [_P]),
    "mpcmd_step": (C.c_int, [_P]),
    "mpcmd_evolve": (C.c_int, [_P]),
    "mpcmd_run": (C.c_int, [_P, C.c_int64]),
    "mpcmd_sort": (C.c_int, [_P]),
    "mpcmd_rebuild_lists": (C.c_int, [_P]),
    "mpcmd_distribute": (C.c_int, [_P]),
    "mpcmd_mpc_rotation": (C.c_int, [_P]),
    "mpcmd_reaction": (C.c_int, [_P]),
    "mpcmd_observables": (C.c_int, [_P, C.POINTER(MpcmdObs)]),
    "mpcmd_concentration": (C.c_int, [_P, C.POINTER(MpcmdConcParams)] + [_dp] * 9),
    "mpcmd_dimer_axes": (C.c_int, [_P, C.c_int, _dp, _dp]),
    "mpcmd_checkpoint": (C.c_int, [_P, C.c_char_p]),
    "mpcmd_restore": (C.c_int, [_P, C.c_char_p]),
    "mpcmd_get_new_cell": (C.c_int, [_P, _lp]),
    "mpcmd_get_cell_rotation": (C.c_int, [_P, _dp, _dp, _ip]),
    "mpcmd_get_distribute": (C.c_int, [_P, _ip, _lp]),
    "mpcmd_get_affected": (C.c_int, [_P, _ip]),
    "mpcmd_get_shift": (C.c_int, [_P, _dp]),
    "mpcmd_get_pairs": (C.c_int, [_P, _lp, _lp, _ip]),
    "mpcmd_get_inside": (C.c_int, [_P, _lp, _lp]),
    "mpcmd_get_counters": (C.c_int, [_P, _lp, C.c_int32]),
    "mpcmd_reactive_grid_table": (C.c_int, [_P, _ip]),
    "mpcmd_cell_order": (C.c_int, [_P, _ip]),
    "mpcmd_kernel_launches": (C.c_int64, [_P]),
    "mpcmd_set_device": (C.c_int, [C.c_int]),
    "mpcmd_event_record": (C.c_int, [_P, C.c_int]),
    "mpcmd_event_elapsed": (C.c_int, [_P, C.c_int, C.c_int, _dp]),
    "mpcmd_synchronize": (C.c_int, [_P]),
    "mpcmd_profile": (C.c_int, [_P, C.c_int]),
    "mpcmd_profile_read": (C.c_int, [_P, _dp, _lp, C.c_int]),
    "mpcmd_contract_u01": (C.c_double, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]),
    # batched ensemble
    "mpcmd_ens_create": (C.c_int, [C.POINTER(MpcmdEnsembleConfig), C.POINTER(MpcmdReplica), C.POINTER(_P)]),
    "mpcmd_ens_destroy": (C.c_int, [_P]),
    "mpcmd_ens_device_bytes": (C.c_int, [_P, _lp]),
    "mpcmd_ens_initial": (C.c_int, [_P]),
    "mpcmd_ens_upload": (C.c_int, [_P, C.c_int32, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp]),
    "mpcmd_ens_download": (C.c_int, [_P, C.c_int32, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp]),
    "mpcmd_ens_prepare": (C.c_int, [_P]),
    "mpcmd_ens_run": (C.c_int, [_P, C.c_int64]),
    "mpcmd_ens_observables": (C.c_int, [_P, C.POINTER(MpcmdObs)]),
    "mpcmd_ens_reset_samples": (C.c_int, [_P, C.c_int32]),
    "mpcmd_ens_samples": (C.c_int, [_P, _dp, _lp, C.POINTER(C.c_float)]),
    "mpcmd_ens_field_accumulate": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_double, C.c_double]),
    "mpcmd_ens_field_read": (C.c_int, [_P, C.POINTER(C.c_uint32), _lp]),
    "mpcmd_ens_set_schedule": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "mpcmd_ens_get_schedule": (C.c_int, [_P, _ip]),
    "mpcmd_ens_autotune": (C.c_int, [_P, C.c_char_p, C.c_int32]),
    "mpcmd_ens_counters": (C.c_int, [_P, _lp, C.c_int32]),
    "mpcmd_ens_event_record": (C.c_int, [_P, C.c_int]),
    "mpcmd_ens_event_elapsed": (C.c_int, [_P, C.c_int, C.c_int, _dp]),
    "mpcmd_ens_synchronize": (C.c_int, [_P]),
    # learned surrogate (device pointers as integers)
    "mpcmd_mlp_create": (C.c_int, [C.POINTER(MpcmdMlpConfig), C.POINTER(_P)]),
    "mpcmd_mlp_destroy": (C.c_int, [_P]),
    "mpcmd_mlp_param_count": (C.c_int, [_P, _lp]),
    "mpcmd_mlp_get_params": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "mpcmd_mlp_set_params": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "mpcmd_mlp_forward": (C.c_int, [_P, C.c_void_p, C.c_int64, C.c_void_p]),
    "mpcmd_mlp_gradients": (C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_float), _dp]),
    "mpcmd_mlp_train_step": (C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_void_p, _dp]),
    "mpcmd_mlp_synchronize": (C.c_int, [_P]),
    # allocation-free collision on caller-owned device arrays (pointers as integers)
    "mpcmd_collide_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_double, C.c_int32, C.c_uint64, C.c_int64, C.c_void_p]),
}


def lib(build_if_missing=True):
    """Load libmpcmd.so (building it if absent).  Raises if it cannot be loaded."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) and build_if_missing:
            from . import build as _b
            _b.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libmpcmd.so is missing; run main_gb300/build.py (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def contract_u01(seed, tag, index, extra, step, which):
    return lib().mpcmd_contract_u01(seed, tag, index, extra, step, which)


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Engine:
    """One device-resident run (one mpcmd context on the current CUDA device)."""

    def __init__(self, cfg):
        self.cfg = dict(cfg)
        self.struct = to_struct(self.cfg)
        h = C.c_void_p()
        st = lib().mpcmd_create(C.byref(self.struct), C.byref(h))
        if st != 0:
            raise MpcmdError(st, "create")
        self.h = h
        self.n = int(self.cfg["n_solvent"])
        self.ns = 2 * int(self.cfg["n_dimers"])
        self.ncell = int(self.cfg["lx"]) * int(self.cfg["ly"]) * int(self.cfg["lz"])

    def close(self):
        if getattr(self, "h", None):
            lib().mpcmd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, st, what):
        if st != 0:
            raise MpcmdError(st, what)

    # -- state -----------------------------------------------------------
    def upload_state(self, st):
        f = lambda k: np.ascontiguousarray(st[k], dtype=np.float64)
        arrs = [f(k) for k in ("x", "y", "z", "vx", "vy", "vz")]
        flag = np.ascontiguousarray(st["flag"], dtype=np.int32)
        ns = max(self.ns, 1)
        dpos = np.ascontiguousarray(st.get("dpos", np.zeros((ns, 3))), dtype=np.float64)
        dvel = np.ascontiguousarray(st.get("dvel", np.zeros((ns, 3))), dtype=np.float64)
        dfrc = np.ascontiguousarray(st.get("dforce", np.zeros((ns, 3))), dtype=np.float64)
        self._keep = (arrs, flag, dpos, dvel, dfrc)
        self._c(lib().mpcmd_upload_state(self.h, *[_ptr(a, C.c_double) for a in arrs], _ptr(flag, C.c_int32),
                                         _ptr(dpos, C.c_double), _ptr(dvel, C.c_double), _ptr(dfrc, C.c_double)),
                "upload_state")

    def download_state(self, out=None):
        """The host state in the reference layout.  `out`: arrays to fill (for
        example page-locked ones, which the copies reach at full link speed):
        x..vz float64 [n], flag int32 [n], dpos/dvel/dforce float64 [n_spheres, 3],
        all C-contiguous; new arrays are allocated when it is None."""
        n, ns = self.n, max(self.ns, 1)
        if out is None:
            out = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz")}
            out["flag"] = np.zeros(n, dtype=np.int32)
            out["dpos"] = np.zeros((ns, 3)); out["dvel"] = np.zeros((ns, 3)); out["dforce"] = np.zeros((ns, 3))
        else:
            want = {k: (np.float64, (n,)) for k in ("x", "y", "z", "vx", "vy", "vz")}
            want["flag"] = (np.int32, (n,))
            for k in ("dpos", "dvel", "dforce"):
                want[k] = (np.float64, (ns, 3))
            for k, (dt, shape) in want.items():
                a = out[k]
                if a.dtype != dt or a.shape != shape or not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]:
                    raise ValueError("download_state: out[%r] must be a writeable C-contiguous %s array of shape %s"
                                     % (k, np.dtype(dt).name, shape))
        self._c(lib().mpcmd_download_state(self.h, *[_ptr(out[k], C.c_double) for k in ("x", "y", "z", "vx", "vy", "vz")],
                                           _ptr(out["flag"], C.c_int32), _ptr(out["dpos"], C.c_double),
                                           _ptr(out["dvel"], C.c_double), _ptr(out["dforce"], C.c_double)),
                "download_state")
        if self.ns == 0:
            for k in ("dpos", "dvel", "dforce"):
                out[k] = out[k][:0]
        return out

    def set_cell_order(self, order):
        a = np.ascontiguousarray(order, dtype=np.int32)
        self._c(lib().mpcmd_set_cell_order(self.h, _ptr(a, C.c_int32), a.size), "set_cell_order")

    def set_anchors(self, anchors):
        """Rotor anchors (motorCM), one row of three per dimer."""
        a = np.ascontiguousarray(anchors, dtype=np.float64).reshape(-1, 3)
        if a.shape[0] != self.ns // 2:
            raise ValueError("anchors: one row per dimer")
        self._c(lib().mpcmd_set_anchors(self.h, _ptr(a, C.c_double)), "set_anchors")

    def get_anchors(self):
        a = np.zeros((max(self.ns // 2, 1), 3))
        self._c(lib().mpcmd_get_anchors(self.h, _ptr(a, C.c_double)), "get_anchors")
        return a[: self.ns // 2]

    def set_owner_tags(self, tags):
        """type_B owner tags (1-based motor numbers, 0 for none), one per particle."""
        a = np.ascontiguousarray(tags, dtype=np.int32)
        if a.size != self.n:
            raise ValueError("owner tags: one per solvent particle")
        self._c(lib().mpcmd_set_owner_tags(self.h, _ptr(a, C.c_int32)), "set_owner_tags")

    def get_owner_tags(self):
        a = np.zeros(self.n, dtype=np.int32)
        self._c(lib().mpcmd_get_owner_tags(self.h, _ptr(a, C.c_int32)), "get_owner_tags")
        return a

    def cell_order(self):
        a = np.zeros(self.ncell, dtype=np.int32)
        lib().mpcmd_cell_order(self.h, _ptr(a, C.c_int32))
        return a

    def set_step(self, cstep, time_count=0):
        self._c(lib().mpcmd_set_step(self.h, cstep, time_count), "set_step")

    def set_resort(self, every):
        """Order-only re-sort every `every` MD steps (a multiple of the
        collision interval; 0 = never).  Results do not depend on it."""
        self._c(lib().mpcmd_set_resort(self.h, int(every)), "set_resort")

    # -- reference call surface ------------------------------------------
    def initial(self):
        self._c(lib().mpcmd_initial(self.h), "initial")

    def prepare(self):
        self._c(lib().mpcmd_prepare(self.h), "prepare")

    def prepare_restart(self):
        self._c(lib().mpcmd_prepare_restart(self.h), "prepare_restart")

    def step(self):
        self._c(lib().mpcmd_step(self.h), "step")

    def evolve(self):
        self._c(lib().mpcmd_evolve(self.h), "evolve")

    def run(self, nsteps):
        self._c(lib().mpcmd_run(self.h, nsteps), "run")

    def sort(self):
        self._c(lib().mpcmd_sort(self.h), "sort")

    def rebuild_lists(self):
        self._c(lib().mpcmd_rebuild_lists(self.h), "rebuild_lists")

    def distribute(self):
        self._c(lib().mpcmd_distribute(self.h), "distribute")

    def mpc_rotation(self):
        self._c(lib().mpcmd_mpc_rotation(self.h), "mpc_rotation")

    def reaction(self):
        self._c(lib().mpcmd_reaction(self.h), "reaction")

    def checkpoint(self, path):
        self._c(lib().mpcmd_checkpoint(self.h, path.encode()), "checkpoint")

    def restore(self, path):
        self._c(lib().mpcmd_restore(self.h, path.encode()), "restore")

    def observables(self):
        o = MpcmdObs()
        self._c(lib().mpcmd_observables(self.h, C.byref(o)), "observables")
        return {
            "momentum": np.array(o.momentum[:]), "solvent_momentum": np.array(o.solvent_momentum[:]),
            "kinetic_solvent": o.kinetic_solvent, "kinetic_dimer": o.kinetic_dimer, "potential": o.potential,
            "species_count": np.array(o.species_count[:]), "n_inside": o.n_inside,
            "time_count": o.time_count, "time_penetrate": o.time_penetrate, "cstep": o.cstep,
        }

    def concentration(self, x_slab, y_slab, z_slab, half_width, x_width=0.5, y_width=0.5, z_width=0.5):
        """Concentration fields of species A (0) and B (1), output_mod.f95:482-575:
        totals (TotA, TotB, ConcA, ConcB) and the 1D / 2D slab fields (2D arrays
        shaped (n_first, n_second) with the first index the reference's first)."""
        prm = MpcmdConcParams(x_slab, y_slab, z_slab, half_width, x_width, y_width, z_width)
        L = (self.cfg["lx"], self.cfg["ly"], self.cfg["lz"])
        nx, ny, nz = (int(L[c] / w) if w > 0 else 0 for c, w in enumerate((x_width, y_width, z_width)))
        out = {"totals": np.zeros(4), "c1d_a": np.zeros(nx), "c1d_b": np.zeros(nx),
               "xy_a": np.zeros(nx * ny), "xy_b": np.zeros(nx * ny), "xz_a": np.zeros(nx * nz),
               "xz_b": np.zeros(nx * nz), "yz_a": np.zeros(ny * nz), "yz_b": np.zeros(ny * nz)}
        keys = ("totals", "c1d_a", "c1d_b", "xy_a", "xy_b", "xz_a", "xz_b", "yz_a", "yz_b")
        self._c(lib().mpcmd_concentration(self.h, C.byref(prm), *[_ptr(out[k], C.c_double) for k in keys]),
                "concentration")
        return out

    def dimer_axes(self, normalize=0):
        """(nucvec [n_dimers, 3], propulsion speed [n_dimers]); normalize 0 divides
        by Dcn (output_mod.f95:826-846), 1 by |d| (Output_SelkovDimer.f90:146-172)."""
        nd = self.cfg["n_dimers"]
        nuc = np.zeros((max(nd, 1), 3))
        vd = np.zeros(max(nd, 1))
        self._c(lib().mpcmd_dimer_axes(self.h, normalize, _ptr(nuc, C.c_double), _ptr(vd, C.c_double)),
                "dimer_axes")
        return nuc[:nd], vd[:nd]

    # -- inspection ------------------------------------------------------
    def new_cell(self):
        a = np.zeros(self.n, dtype=np.int64)
        self._c(lib().mpcmd_get_new_cell(self.h, _ptr(a, C.c_int64)), "get_new_cell")
        return a

    def n_cells_shifted(self):
        c = self.cfg
        return c["lx"] * c["ly"] * (c["lz"] + 1 if c["geometry"] == config.GEOM_WALLS else c["lz"])

    def cell_rotation(self):
        nc = self.n_cells_shifted()
        cm = np.zeros((nc, 3)); ax = np.zeros((nc, 3)); cnt = np.zeros(nc, dtype=np.int32)
        self._c(lib().mpcmd_get_cell_rotation(self.h, _ptr(cm, C.c_double), _ptr(ax, C.c_double),
                                              _ptr(cnt, C.c_int32)), "get_cell_rotation")
        return cm, ax, cnt

    def distribute_result(self):
        cnt = np.zeros((self.ncell, 4), dtype=np.int32)
        first = np.zeros((self.ncell, 4), dtype=np.int64)
        self._c(lib().mpcmd_get_distribute(self.h, _ptr(cnt, C.c_int32), _ptr(first, C.c_int64)), "get_distribute")
        return cnt, first

    def affected(self):
        a = np.zeros(self.ncell, dtype=np.int32)
        self._c(lib().mpcmd_get_affected(self.h, _ptr(a, C.c_int32)), "get_affected")
        return a

    def shift(self):
        s = np.zeros(3)
        lib().mpcmd_get_shift(self.h, _ptr(s, C.c_double))
        return s

    def inside(self):
        n = C.c_int64(0)
        a = np.zeros(self.n, dtype=np.int64)
        self._c(lib().mpcmd_get_inside(self.h, C.byref(n), _ptr(a, C.c_int64)), "get_inside")
        return np.sort(a[: n.value])

    def pairs(self):
        """(particle, sphere) pairs of the shell lists, sorted by sphere then particle."""
        n = C.c_int64(0)
        cap = 8 * self.n
        part = np.zeros(cap, dtype=np.int64)
        sph = np.zeros(cap, dtype=np.int32)
        self._c(lib().mpcmd_get_pairs(self.h, C.byref(n), _ptr(part, C.c_int64), _ptr(sph, C.c_int32)), "get_pairs")
        part, sph = part[: n.value], sph[: n.value]
        o = np.lexsort((part, sph))
        return part[o], sph[o]

    def neighbours(self, sphere):
        part, sph = self.pairs()
        return part[sph == sphere]

    def counters(self):
        c = np.zeros(15, dtype=np.int64)
        self._c(lib().mpcmd_get_counters(self.h, _ptr(c, C.c_int64), 15), "get_counters")
        keys = ("n_inside", "status", "time_penetrate", "rattle_iters", "cstep", "time_count", "abort_step",
                "last_rebuild", "dbg_code", "dbg_val", "n_watch", "work_force_entries", "work_rebuild_particles",
                "work_rebuild_placed", "resorts")
        return dict(zip(keys, (int(v) for v in c)))

    def reactive_grid(self):
        t = np.zeros(int(self.cfg["lx"]) * int(self.cfg["ly"]), dtype=np.int32)
        lib().mpcmd_reactive_grid_table(self.h, _ptr(t, C.c_int32))
        return t

    # -- measurement -----------------------------------------------------
    PROFILE_KINDS = ("rebuild", "force", "dimer", "cells", "rotate_main", "shell_advance", "bins",
                     "finalize", "sort", "affected")

    def event_record(self, slot):
        self._c(lib().mpcmd_event_record(self.h, slot), "event_record")

    def event_elapsed(self, a, b):
        ms = C.c_double(0)
        self._c(lib().mpcmd_event_elapsed(self.h, a, b, C.byref(ms)), "event_elapsed")
        return ms.value

    def synchronize(self):
        self._c(lib().mpcmd_synchronize(self.h), "synchronize")

    def profile(self, enable):
        self._c(lib().mpcmd_profile(self.h, 1 if enable else 0), "profile")

    def profile_read(self):
        n = len(self.PROFILE_KINDS)
        ms = np.zeros(n)
        cnt = np.zeros(n, dtype=np.int64)
        self._c(lib().mpcmd_profile_read(self.h, _ptr(ms, C.c_double), _ptr(cnt, C.c_int64), n), "profile_read")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.PROFILE_KINDS)}

    def device_bytes(self):
        b = C.c_int64(0)
        lib().mpcmd_device_bytes(self.h, C.byref(b))
        return b.value


def kernel_launches():
    return int(lib().mpcmd_kernel_launches(None))


def set_device(device):
    st = lib().mpcmd_set_device(int(device))
    if st != 0:
        raise MpcmdError(st, "set_device")

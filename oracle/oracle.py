"""ctypes front end of the CPU oracle (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker.  The oracle restates the reference Fortran in
FP64 C (see oracle.h for what pins it).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_I32, _I64, _U64, _D = C.c_int32, C.c_int64, C.c_uint64, C.c_double

PARAM_FIELDS = [
    ("lx", _I32), ("ly", _I32), ("lz", _I32), ("geometry", _I32), ("n_dimers", _I32),
    ("kinetics", _I32), ("exclusion", _I32), ("catalysis", _I32), ("rotation_sense", _I32),
    ("mpc_every", _I32), ("sort_every", _I32), ("react_box_type", _I32), ("react_dir", _I32),
    ("cell_capacity", _I32), ("max_neighbour", _I32), ("rattle_max_iter", _I32),
    ("init_plane", _I32), ("pad0", _I32),
    ("n_solvent", _I64), ("seed", _U64), ("init_count", _I64 * 4),
    ("mass", _D * 4), ("eps_c", _D * 4), ("eps_n", _D * 4),
    ("rc", _D), ("rn", _D), ("dcn", _D), ("mc", _D), ("mn", _D), ("rw", _D), ("ew", _D),
    ("rm_delta", _D), ("em", _D), ("rp_ab", _D), ("rp_ba", _D), ("kT", _D), ("skin", _D),
    ("rot_angle", _D), ("md_dt", _D), ("mpc_dt", _D), ("k", _D * 6),
    ("engine_only", _I32 * 2),
    ("variant", _I32), ("layout", _I32), ("layout_rows", _I32), ("layout_cols", _I32),
    ("owner_tags", _I32), ("reserved", _I32), ("tether_k", _D), ("tether_z", _D), ("layout_sep", _D),
]


class OrcParams(C.Structure):
    _fields_ = PARAM_FIELDS


class OrcObs(C.Structure):
    _fields_ = [
        ("momentum", _D * 3), ("solvent_momentum", _D * 3), ("kinetic_solvent", _D),
        ("kinetic_dimer", _D), ("potential", _D), ("species_count", _I64 * 4),
        ("n_inside", _I64), ("n_pairs", _I64), ("time_count", _I32), ("time_penetrate", _I32),
        ("cstep", _I64),
    ]


RNG_CONTRACT, RNG_MT = 0, 1
LISTS_ALL_PAIRS, LISTS_CELLS = 0, 1
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        lp = C.POINTER(C.c_int64)
        up = C.POINTER(C.c_uint32)
        sig = {
            "orc_create": (P, [C.POINTER(OrcParams)]),
            "orc_destroy": (None, [P]),
            "orc_status": (C.c_int, [P]),
            "orc_set_threads": (C.c_int, [C.c_int]),
            "orc_set_rng": (C.c_int, [P, C.c_int, C.c_uint32]),
            "orc_set_list_mode": (C.c_int, [P, C.c_int]),
            "orc_set_state": (C.c_int, [P, dp, dp, dp, dp, dp, dp, ip, dp, dp, dp]),
            "orc_get_state": (C.c_int, [P, dp, dp, dp, dp, dp, dp, ip, dp, dp, dp]),
            "orc_restart_forces": (C.c_int, [P]),
            "orc_set_owner": (C.c_int, [P, ip]),
            "orc_get_owner": (C.c_int, [P, ip]),
            "orc_set_anchors": (C.c_int, [P, dp]),
            "orc_get_anchors": (C.c_int, [P, dp]),
            "orc_set_cell_order": (C.c_int, [P, ip, C.c_int64]),
            "orc_set_cstep": (C.c_int, [P, C.c_int64, C.c_int32]),
            "orc_initial": (C.c_int, [P]), "orc_prepare": (C.c_int, [P]),
            "orc_step": (C.c_int, [P]), "orc_run": (C.c_int, [P, C.c_int64]),
            "orc_sort": (C.c_int, [P]), "orc_rebuild_lists": (C.c_int, [P]),
            "orc_distribute": (C.c_int, [P]), "orc_mpc_rotation": (C.c_int, [P]),
            "orc_reaction": (C.c_int, [P]),
            "orc_selkov_prepare": (C.c_int, [P]), "orc_selkov_step": (C.c_int, [P]),
            "orc_observables": (C.c_int, [P, C.POINTER(OrcObs)]),
            "orc_concentration": (C.c_int, [C.c_int64, dp, dp, dp, ip, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]),
            "orc_n_cells_shifted": (C.c_int64, [P]),
            "orc_get_new_cell": (C.c_int, [P, lp]),
            "orc_get_cell_rotation": (C.c_int, [P, dp, dp, ip]),
            "orc_get_distribute": (C.c_int, [P, ip, lp]),
            "orc_get_affected": (C.c_int, [P, ip]),
            "orc_get_shift": (C.c_int, [P, dp]),
            "orc_neighbour_count": (C.c_int64, [P, C.c_int]),
            "orc_get_neighbours": (C.c_int, [P, C.c_int, lp]),
            "orc_get_inside": (C.c_int, [P, lp, lp]),
            "orc_get_pair_forces": (C.c_int, [P, C.c_int, dp, dp]),
            "orc_reactive_grid_table": (C.c_int, [P, ip]),
            "orc_philox4x32_10": (None, [up, up, up]),
            "orc_contract_u01": (C.c_double, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]),
            "orc_mt1998_sgrnd": (None, [C.c_uint32, up]),
            "orc_mt2002_init": (None, [C.c_uint32, up]),
            "orc_mt_next_u32": (None, [up, ip, up, C.c_int64]),
            "orc_mt_grnd": (C.c_double, [up, ip]),
            "orc_mt_real1": (C.c_double, [up, ip]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def make_params(cfg):
    """Fill an OrcParams from a dict of field values (missing fields are 0)."""
    p = OrcParams()
    for name, typ in PARAM_FIELDS:
        if name not in cfg:
            continue
        v = cfg[name]
        if hasattr(typ, "_length_"):
            arr = getattr(p, name)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, name, v)
    return p


# ------------------------------------------------------------ RNG KATs ----
def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32).copy()
    k = np.asarray(key, dtype=np.uint32).copy()
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_ptr(c, C.c_uint32), _ptr(k, C.c_uint32), _ptr(out, C.c_uint32))
    return out


def contract_u01(seed, tag, index, extra, step, which):
    return lib().orc_contract_u01(seed, tag, index, extra, step, which)


class MT:
    """MT19937 stream with the 1998 (mtmod.f90) or 2002 (mt95.f90) seeding."""

    def __init__(self, seed, kind):
        self.state = np.zeros(624, dtype=np.uint32)
        self.mti = C.c_int32(624)
        if kind == 1998:
            lib().orc_mt1998_sgrnd(seed & 0xFFFFFFFF, _ptr(self.state, C.c_uint32))
        else:
            lib().orc_mt2002_init(seed & 0xFFFFFFFF, _ptr(self.state, C.c_uint32))

    def u32(self, n):
        out = np.zeros(n, dtype=np.uint32)
        lib().orc_mt_next_u32(_ptr(self.state, C.c_uint32), C.byref(self.mti), _ptr(out, C.c_uint32), n)
        return out

    def grnd(self):
        return lib().orc_mt_grnd(_ptr(self.state, C.c_uint32), C.byref(self.mti))

    def real1(self):
        return lib().orc_mt_real1(_ptr(self.state, C.c_uint32), C.byref(self.mti))


# -------------------------------------------------------------- engine ----
class Oracle:
    """One FP64 oracle instance (collective driver with the selkov options)."""

    def __init__(self, cfg, threads=1):
        self.cfg = dict(cfg)
        L = lib()
        L.orc_set_threads(threads)
        self.p = make_params(cfg)
        self.h = L.orc_create(C.byref(self.p))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        self.n = int(cfg["n_solvent"])
        self.ns = 2 * int(cfg["n_dimers"])
        self.ncell = int(cfg["lx"]) * int(cfg["ly"]) * int(cfg["lz"])

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_destroy(h)
            self.h = None

    def _check(self, st, what):
        if st != 0:
            raise RuntimeError("oracle %s failed with status %d" % (what, st))
        return st

    def status(self):
        return lib().orc_status(self.h)

    def set_rng(self, mode, mt_seed=0):
        lib().orc_set_rng(self.h, mode, mt_seed)

    def set_list_mode(self, mode):
        self._check(lib().orc_set_list_mode(self.h, mode), "set_list_mode")

    def set_state(self, st):
        f = lambda k: np.ascontiguousarray(st[k], dtype=np.float64)
        x, y, z, vx, vy, vz = (f(k) for k in ("x", "y", "z", "vx", "vy", "vz"))
        flag = np.ascontiguousarray(st["flag"], dtype=np.int32)
        ns = max(self.ns, 1)
        dpos = np.ascontiguousarray(st.get("dpos", np.zeros((ns, 3))), dtype=np.float64)
        dvel = np.ascontiguousarray(st.get("dvel", np.zeros((ns, 3))), dtype=np.float64)
        dfrc = np.ascontiguousarray(st.get("dforce", np.zeros((ns, 3))), dtype=np.float64)
        dp = C.POINTER(C.c_double)
        self._check(lib().orc_set_state(self.h, _ptr(x, C.c_double), _ptr(y, C.c_double), _ptr(z, C.c_double),
                                        _ptr(vx, C.c_double), _ptr(vy, C.c_double), _ptr(vz, C.c_double),
                                        _ptr(flag, C.c_int32), _ptr(dpos, C.c_double),
                                        _ptr(dvel, C.c_double), _ptr(dfrc, C.c_double)), "set_state")

    def get_state(self):
        n, ns = self.n, max(self.ns, 1)
        out = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz")}
        out["flag"] = np.zeros(n, dtype=np.int32)
        out["dpos"] = np.zeros((ns, 3))
        out["dvel"] = np.zeros((ns, 3))
        out["dforce"] = np.zeros((ns, 3))
        lib().orc_get_state(self.h, *[_ptr(out[k], C.c_double) for k in ("x", "y", "z", "vx", "vy", "vz")],
                            _ptr(out["flag"], C.c_int32), _ptr(out["dpos"], C.c_double),
                            _ptr(out["dvel"], C.c_double), _ptr(out["dforce"], C.c_double))
        if self.ns == 0:
            for k in ("dpos", "dvel", "dforce"):
                out[k] = out[k][:0]
        return out

    def set_anchors(self, anchors):
        a = np.ascontiguousarray(anchors, dtype=np.float64).reshape(-1, 3)
        if a.shape[0] != self.ns // 2:
            raise ValueError("anchors: one row per dimer")
        self._check(lib().orc_set_anchors(self.h, _ptr(a, C.c_double)), "set_anchors")

    def get_anchors(self):
        a = np.zeros((max(self.ns // 2, 1), 3))
        lib().orc_get_anchors(self.h, _ptr(a, C.c_double))
        return a[: self.ns // 2]

    def set_owner(self, owner):
        a = np.ascontiguousarray(owner, dtype=np.int32)
        if a.size != self.n:
            raise ValueError("owner tags: one per solvent particle")
        self._check(lib().orc_set_owner(self.h, _ptr(a, C.c_int32)), "set_owner")

    def get_owner(self):
        a = np.zeros(self.n, dtype=np.int32)
        lib().orc_get_owner(self.h, _ptr(a, C.c_int32))
        return a

    def set_cell_order(self, order):
        a = np.ascontiguousarray(order, dtype=np.int32)
        self._check(lib().orc_set_cell_order(self.h, _ptr(a, C.c_int32), a.size), "set_cell_order")

    def set_cstep(self, cstep, time_count=0):
        lib().orc_set_cstep(self.h, cstep, time_count)

    def initial(self):
        return self._check(lib().orc_initial(self.h), "initial")

    def prepare(self):
        return self._check(lib().orc_prepare(self.h), "prepare")

    def restart_forces(self):
        return self._check(lib().orc_restart_forces(self.h), "restart_forces")

    def step(self):
        return self._check(lib().orc_step(self.h), "step")

    def run(self, n):
        return self._check(lib().orc_run(self.h, n), "run")

    def sort(self):
        return self._check(lib().orc_sort(self.h), "sort")

    def rebuild_lists(self):
        return self._check(lib().orc_rebuild_lists(self.h), "rebuild_lists")

    def distribute(self):
        return self._check(lib().orc_distribute(self.h), "distribute")

    def mpc_rotation(self):
        return self._check(lib().orc_mpc_rotation(self.h), "mpc_rotation")

    def reaction(self):
        return self._check(lib().orc_reaction(self.h), "reaction")

    def selkov_prepare(self):
        return self._check(lib().orc_selkov_prepare(self.h), "selkov_prepare")

    def selkov_step(self):
        return self._check(lib().orc_selkov_step(self.h), "selkov_step")

    def observables(self):
        o = OrcObs()
        lib().orc_observables(self.h, C.byref(o))
        return {
            "momentum": np.array(o.momentum[:]), "solvent_momentum": np.array(o.solvent_momentum[:]),
            "kinetic_solvent": o.kinetic_solvent, "kinetic_dimer": o.kinetic_dimer,
            "potential": o.potential, "species_count": np.array(o.species_count[:]),
            "n_inside": o.n_inside, "n_pairs": o.n_pairs, "time_count": o.time_count,
            "time_penetrate": o.time_penetrate, "cstep": o.cstep,
        }

    def new_cell(self):
        a = np.zeros(self.n, dtype=np.int64)
        lib().orc_get_new_cell(self.h, _ptr(a, C.c_int64))
        return a

    def cell_rotation(self):
        nc = lib().orc_n_cells_shifted(self.h)
        cm = np.zeros((nc, 3)); ax = np.zeros((nc, 3)); cnt = np.zeros(nc, dtype=np.int32)
        lib().orc_get_cell_rotation(self.h, _ptr(cm, C.c_double), _ptr(ax, C.c_double), _ptr(cnt, C.c_int32))
        return cm, ax, cnt

    def distribute_result(self):
        cnt = np.zeros((self.ncell, 4), dtype=np.int32)
        first = np.zeros((self.ncell, 4), dtype=np.int64)
        lib().orc_get_distribute(self.h, _ptr(cnt, C.c_int32), _ptr(first, C.c_int64))
        return cnt, first

    def affected(self):
        a = np.zeros(self.ncell, dtype=np.int32)
        lib().orc_get_affected(self.h, _ptr(a, C.c_int32))
        return a

    def shift(self):
        s = np.zeros(3)
        lib().orc_get_shift(self.h, _ptr(s, C.c_double))
        return s

    def neighbours(self, sphere):
        n = lib().orc_neighbour_count(self.h, sphere)
        a = np.zeros(max(n, 0), dtype=np.int64)
        if n > 0:
            lib().orc_get_neighbours(self.h, sphere, _ptr(a, C.c_int64))
        return a

    def pair_forces(self, sphere):
        n = lib().orc_neighbour_count(self.h, sphere)
        f = np.zeros((max(n, 0), 3)); pot = np.zeros(max(n, 0))
        if n > 0:
            lib().orc_get_pair_forces(self.h, sphere, _ptr(f, C.c_double), _ptr(pot, C.c_double))
        return f, pot

    def inside(self):
        n = C.c_int64(0)
        a = np.zeros(self.n, dtype=np.int64)
        lib().orc_get_inside(self.h, C.byref(n), _ptr(a, C.c_int64))
        return a[: n.value].copy()

    def reactive_grid(self):
        t = np.zeros(int(self.cfg["lx"]) * int(self.cfg["ly"]), dtype=np.int32)
        lib().orc_reactive_grid_table(self.h, _ptr(t, C.c_int32))
        return t


def concentration(x, y, z, flag, box, prm):
    """Concentration fields (output_mod.f95:482-575) of host arrays: box
    (Lx, Ly, Lz), prm = (x_slab, y_slab, z_slab, half_width, x_width, y_width,
    z_width).  Returns totals[4] and the 1D / 2D fields (2D in Fortran order,
    first index fastest)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    z = np.ascontiguousarray(z, dtype=np.float64)
    flag = np.ascontiguousarray(flag, dtype=np.int32)
    box = np.ascontiguousarray(box, dtype=np.float64)
    prm = np.ascontiguousarray(prm, dtype=np.float64)
    nx, ny, nz = (int(box[c] / prm[4 + c]) if prm[4 + c] > 0 else 0 for c in range(3))
    out = {"totals": np.zeros(4), "c1d_a": np.zeros(nx), "c1d_b": np.zeros(nx),
           "xy_a": np.zeros(nx * ny), "xy_b": np.zeros(nx * ny), "xz_a": np.zeros(nx * nz),
           "xz_b": np.zeros(nx * nz), "yz_a": np.zeros(ny * nz), "yz_b": np.zeros(ny * nz)}
    dp = C.c_double
    st = lib().orc_concentration(len(x), _ptr(x, dp), _ptr(y, dp), _ptr(z, dp), _ptr(flag, C.c_int32),
                                 _ptr(box, dp), _ptr(prm, dp),
                                 *[_ptr(out[k], dp) for k in ("totals", "c1d_a", "c1d_b", "xy_a", "xy_b",
                                                              "xz_a", "xz_b", "yz_a", "yz_b")])
    if st != 0:
        raise RuntimeError("orc_concentration failed (%d)" % st)
    return out

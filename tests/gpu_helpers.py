"""Shared helpers of the GPU parity tests: build an oracle/engine pair on the
same seeded input and compare their states."""
import numpy as np

from main_gb300 import Engine, config
from oracle.oracle import Oracle


def pair(cfg, init_on="oracle"):
    o = Oracle(cfg)
    o.initial()
    st = o.get_state()
    e = Engine(cfg)
    e.upload_state(st)
    o.set_cell_order(e.cell_order())
    return o, e


def min_image(d, L):
    return d - L * np.round(d / L)


def state_diff(se, so, cfg):
    """Max abs differences (positions with the minimum image)."""
    L = np.array([cfg["lx"], cfg["ly"], cfg["lz"]], float)
    out = {}
    for i, k in enumerate("xyz"):
        d = se[k] - so[k]
        if i < 2 or cfg["geometry"] == config.GEOM_PERIODIC:
            d = min_image(d, L[i])
        out[k] = np.abs(d)
    for k in ("vx", "vy", "vz"):
        out[k] = np.abs(se[k] - so[k])
    out["flag_equal"] = float((se["flag"] == so["flag"]).mean())
    if len(so["dpos"]):
        dd = se["dpos"] - so["dpos"]
        for c in range(2 if cfg["geometry"] == config.GEOM_WALLS else 3):
            dd[:, c] = min_image(dd[:, c], L[c])
        out["dpos"] = np.abs(dd)
        out["dvel"] = np.abs(se["dvel"] - so["dvel"])
    return out


def assert_close(se, so, cfg, pos, vel, flags=1.0, dimer=None):
    d = state_diff(se, so, cfg)
    for k in "xyz":
        assert d[k].max() <= pos, (k, d[k].max())
    for k in ("vx", "vy", "vz"):
        assert d[k].max() <= vel, (k, d[k].max())
    assert d["flag_equal"] >= flags, d["flag_equal"]
    if dimer is not None and "dpos" in d:
        assert d["dpos"].max() <= dimer, d["dpos"].max()
        assert d["dvel"].max() <= dimer, d["dvel"].max()
    return d


CASES = {
    # plain single dimer, fully periodic (c0 scaled to 16^3)
    "c0": lambda prec, **kw: config.workload("c0", scale=0.55, precision=prec, **kw),
    # collective quasi-2D: z walls, reactive floor, dimers in the mid-plane
    "c1": lambda prec, **kw: config.workload("c1", scale=0.25, precision=prec, **kw),
    # Selkov kinetics, affected cells, probabilistic catalysis, projection rotation
    "c2": lambda prec, **kw: config.workload("c2", scale=0.07, precision=prec, **kw),
}

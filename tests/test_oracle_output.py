"""The oracle's concentration fields (output_mod.f95:482-575) against an
independent numpy restatement, on random states with particles planted on
the edges the binning has to get right: a coordinate of exactly 0 (bin 0 in
the reference, counted in bin 1), coordinates on bin boundaries (ceiling puts
them in the lower bin), slab faces at exactly |u - slab| = half_width
(inside), species 2 and 3 (not counted)."""
import math

import numpy as np

from oracle import oracle as O


def numpy_fields(x, y, z, flag, box, prm):
    xs, ys, zs, hw, xw, yw, zw = prm
    nx, ny, nz = int(box[0] / xw), int(box[1] / yw), int(box[2] / zw)

    def b(u, w, nb):
        j = np.ceil(u / w).astype(np.int64)
        return np.clip(j, 1, nb) - 1

    out = {}
    a, bb = flag == 0, flag == 1
    vol = float(int(box[0] * box[1] * box[2]))
    out["totals"] = np.array([a.sum(), bb.sum(), a.sum() / vol, bb.sum() / vol], float)
    zin = (z <= zs + hw) & (z >= zs - hw)
    yin = (y <= ys + hw) & (y >= ys - hw)
    xin = (x <= xs + hw) & (x >= xs - hw)
    for sp, m in (("a", a), ("b", bb)):
        s = m & zin
        out["c1d_" + sp] = np.bincount(b(x[s], xw, nx), minlength=nx) / (xw * box[1] * 2 * hw)
        out["xy_" + sp] = np.bincount(b(x[s], xw, nx) + nx * b(y[s], yw, ny), minlength=nx * ny) / (xw * yw * 2 * hw)
        s = m & yin
        out["xz_" + sp] = np.bincount(b(x[s], xw, nx) + nx * b(z[s], zw, nz), minlength=nx * nz) / (xw * zw * 2 * hw)
        s = m & xin
        out["yz_" + sp] = np.bincount(b(y[s], yw, ny) + ny * b(z[s], zw, nz), minlength=ny * nz) / (yw * zw * 2 * hw)
    return out


def test_concentration_matches_numpy_restatement():
    rng = np.random.default_rng(7)
    box = (12.0, 10.0, 8.0)
    n = 20000
    x = rng.uniform(0, box[0], n)
    y = rng.uniform(0, box[1], n)
    z = rng.uniform(0, box[2], n)
    flag = rng.integers(0, 4, n).astype(np.int32)
    prm = (6.0, 5.0, 4.0, 1.25, 0.5, 0.5, 0.5)
    # planted edge cases
    x[:10] = 0.0
    y[10:20] = 2.5                      # a bin boundary
    z[20:30] = 4.0 + 1.25               # on the z slab's upper face
    z[30:40] = 4.0 - 1.25               # on its lower face
    x[40:50] = 6.0 + 1.25
    flag[:40] = np.arange(40) % 2
    ref = numpy_fields(x, y, z, flag, box, prm)
    got = O.concentration(x, y, z, flag, box, prm)
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    # the planted particles are counted where the reference's ceiling puts them
    assert got["totals"][0] + got["totals"][1] == np.isin(flag, (0, 1)).sum()
    assert math.isclose(got["c1d_a"].sum() * 0.5 * box[1] * 2.5 + got["c1d_b"].sum() * 0.5 * box[1] * 2.5,
                        (np.isin(flag, (0, 1)) & (np.abs(z - 4.0) <= 1.25)).sum())


def test_concentration_rejects_bad_widths():
    x = np.zeros(3)
    try:
        O.concentration(x, x, x, np.zeros(3, np.int32), (4.0, 4.0, 4.0), (2, 2, 2, 1, 0.0, 0.5, 0.5))
    except RuntimeError:
        return
    raise AssertionError("zero bin width accepted")

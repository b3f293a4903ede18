"""mpcmd_collide_static (the allocation-free collision on caller-owned device
arrays) agrees with the context entry point mpcmd_mpc_rotation on the same
FP64 state, over two calls in a row (the second call reuses the static scratch
array that the first one left behind)."""
import numpy as np
import pytest

import main_gb300
from main_gb300 import Engine

from gpu_helpers import CASES

torch = pytest.importorskip("torch")

# the FP64 collision-stage tolerance of the parity tests
VEL_TOL = 1e-13


def _collide_static(dev, cfg, step, stream):
    lib = main_gb300.lib()
    return lib.mpcmd_collide_static(
        dev["x"].data_ptr(), dev["y"].data_ptr(), dev["z"].data_ptr(),
        dev["vx"].data_ptr(), dev["vy"].data_ptr(), dev["vz"].data_ptr(),
        dev["x"].numel(), cfg["lx"], cfg["ly"], cfg["lz"], cfg["geometry"],
        cfg["rot_angle"], cfg["rotation_sense"], cfg["seed"], step, stream)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c0", "c1", "c2"])
def test_static_collision_matches_context_entry_point(case):
    cfg = CASES[case](64)
    e = Engine(cfg)
    e.initial()
    st = e.download_state()
    dev = {k: torch.from_numpy(np.ascontiguousarray(st[k])).to("cuda") for k in ("x", "y", "z", "vx", "vy", "vz")}
    stream = torch.cuda.current_stream().cuda_stream
    for step in (50, 100):
        e.set_step(step)
        e.mpc_rotation()
        ref = e.download_state()
        assert _collide_static(dev, cfg, step, stream) == 0
        torch.cuda.synchronize()
        for k in ("vx", "vy", "vz"):
            got = dev[k].cpu().numpy()
            err = np.abs(got - ref[k]).max()
            assert err <= VEL_TOL, (case, step, k, err)
        # the collision moved the velocities (the comparison is not vacuous)
        assert np.abs(ref["vx"] - st["vx"]).max() > 1e-3


@pytest.mark.gpu
def test_static_collision_rejects_boxes_beyond_the_scratch_array():
    cfg = CASES["c0"](64)
    dev = {k: torch.zeros(8, dtype=torch.float64, device="cuda") for k in ("x", "y", "z", "vx", "vy", "vz")}
    big = dict(cfg, lx=128, ly=128, lz=64)   # 1,048,576 cells > MPCMD_STATIC_MAX_CELLS
    assert main_gb300.STATUS[_collide_static(dev, big, 50, 0)] == "invalid configuration"
    torch.cuda.synchronize()
    assert torch.count_nonzero(dev["vx"]).item() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c0", "c1"])
def test_static_collision_places_edge_positions_as_the_upload_does(case):
    """Positions on a wall (z = lz, z just below 0) and outside the periodic
    box (x = lx + 0.3, y = -0.2) take the same cells in the static entry point
    as in the context upload, which converts them once."""
    cfg = CASES[case](64)
    e = Engine(cfg)
    e.initial()
    st = e.download_state()
    lx, ly, lz = cfg["lx"], cfg["ly"], cfg["lz"]
    m = 64
    st["x"][:m] = lx + 0.3
    st["y"][m:2 * m] = -0.2
    if cfg["geometry"] == 0:   # walls: the clamp of the z coordinate
        st["z"][2 * m:3 * m] = float(lz)
        st["z"][3 * m:4 * m] = -1e-12
    else:
        st["z"][2 * m:3 * m] = lz + 0.45
    e2 = Engine(cfg)
    e2.upload_state(st)
    dev = {k: torch.from_numpy(np.ascontiguousarray(st[k])).to("cuda") for k in ("x", "y", "z", "vx", "vy", "vz")}
    stream = torch.cuda.current_stream().cuda_stream
    for step in (50, 100):
        e2.set_step(step)
        e2.mpc_rotation()
        ref = e2.download_state()
        assert _collide_static(dev, cfg, step, stream) == 0
        torch.cuda.synchronize()
        for k in ("vx", "vy", "vz"):
            err = np.abs(dev[k].cpu().numpy() - ref[k]).max()
            assert err <= VEL_TOL, (case, step, k, err)

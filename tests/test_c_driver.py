"""The plain-C driver of the C ABI (fortran/mpcmd_driver.c): it compiles with
gcc against include/mpcmd.h and links to libmpcmd.so (CPU); run on the GPU,
the main-loop call sequence of main_pattern.f95:203-225 it issues gives the
oracle's trajectory (GPU)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
import main_gb300

SRC = os.path.join(ROOT, "fortran", "mpcmd_driver.c")


def build_driver(out_dir):
    lib = main_gb300.LIB_PATH
    main_gb300.lib()   # builds the library when it is missing
    exe = os.path.join(out_dir, "mpcmd_driver")
    subprocess.run(["gcc", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-L", os.path.dirname(lib),
                    "-lmpcmd", "-Wl,-rpath," + os.path.dirname(lib), "-lm", "-o", exe], check=True)
    return exe


def test_driver_compiles_and_links(tmp_path):
    exe = build_driver(str(tmp_path))
    assert os.access(exe, os.X_OK)


def read_run(path):
    with open(path, "rb") as f:
        n, ns, nc = np.fromfile(f, dtype=np.int64, count=3)
        order = np.fromfile(f, dtype=np.int32, count=nc)

        def state():
            st = {k: np.fromfile(f, dtype=np.float64, count=n) for k in ("x", "y", "z", "vx", "vy", "vz")}
            st["flag"] = np.fromfile(f, dtype=np.int32, count=n)
            st["dpos"] = np.fromfile(f, dtype=np.float64, count=3 * ns).reshape(ns, 3)
            st["dvel"] = np.fromfile(f, dtype=np.float64, count=3 * ns).reshape(ns, 3)
            return st

        first, last = state(), state()
        counts = np.fromfile(f, dtype=np.int64, count=4)
    return order, first, last, counts


@pytest.mark.gpu
@pytest.mark.parametrize("geometry", [0, 1])
def test_driver_run_matches_the_oracle(tmp_path, geometry):
    from gpu_helpers import assert_close
    from main_gb300 import config
    from oracle.oracle import Oracle
    exe = build_driver(str(tmp_path))
    out = str(tmp_path / "run.bin")
    edge, steps, seed = 16, 120, 7
    subprocess.run([exe, out, str(geometry), str(edge), str(steps), str(seed)], check=True)
    order, first, last, counts = read_run(out)
    cfg = config.base_config(lx=edge, ly=edge, lz=8 if geometry == 0 else edge, geometry=geometry, n_dimers=1,
                             seed=seed, k=[0.05, 0, 0, 0, 0, 0], init_plane=1 if geometry == 0 else 0,
                             react_box_type=6, precision=64)
    o = Oracle(cfg)
    o.set_state(first)
    o.set_cell_order(order)
    o.prepare()
    o.run(steps)
    assert_close(last, o.get_state(), cfg, pos=1e-9, vel=1e-9, flags=1.0, dimer=1e-9)
    assert np.array_equal(counts, o.observables()["species_count"])

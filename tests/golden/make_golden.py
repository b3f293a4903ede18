"""Regenerate the committed golden fixtures from the reference tree.

Run from the repository root with the reference checkout as the argument
(or in MPCMD_REFERENCE_ROOT):
    python tests/golden/make_golden.py <reference root>

hilbert_64x64x32.npz: the cell visiting order of collective_code/hilbert.txt
(read by sort_hilbert_mod.f95:57-62) as 0-based row-major cell ids (int32,
compressed), with a SHA-256 of the ids for an integrity check.
"""
import hashlib
import os
import sys

import numpy as np


def main(ref_root):
    src = os.path.join(ref_root, "collective_code", "hilbert.txt")
    xyz = np.loadtxt(src, dtype=np.int64)
    L = (64, 64, 32)
    ids = (xyz[:, 0] + L[0] * (xyz[:, 1] + L[1] * xyz[:, 2])).astype(np.int32)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hilbert_64x64x32.npz")
    np.savez_compressed(out, order=ids, box=np.array(L, dtype=np.int32),
                        sha256=np.frombuffer(hashlib.sha256(ids.tobytes()).digest(), dtype=np.uint8))
    print(out, ids.size)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MPCMD_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <reference root> (or set MPCMD_REFERENCE_ROOT)")
    main(root)

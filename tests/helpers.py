"""Shared helpers of the test suite."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_golden.npz")
REF_ROOT_RECORD = os.path.join(ROOT, "oracle", "_ref", "ref_root.txt")


def reference_root():
    """The reference source tree, or None: TSR_REFERENCE_ROOT, else the tree
    `make -C oracle ref` compiled oracle/_ref from.  Tests that read the
    reference's own files skip where it is absent (the GPU machine has none)."""
    d = os.environ.get("TSR_REFERENCE_ROOT")
    if not d and os.path.exists(REF_ROOT_RECORD):
        with open(REF_ROOT_RECORD) as f:
            d = f.read().strip()
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


def golden():
    return np.load(GOLDEN)


def hessenberg_from_golden(g, idx):
    """(m, alpha, H with ld = m + 1 column major, phi m x m) of golden case idx."""
    ms = g["phipade/m"]
    offH = int(sum(m * (m + 1) for m in ms[:idx]))
    offP = int(sum(m * m for m in ms[:idx]))
    m = int(ms[idx])
    H = g["phipade/H"][offH:offH + m * (m + 1)].reshape(m, m + 1)   # [col][row]
    phi = g["phipade/phi"][offP:offP + m * m].reshape(m, m)
    return m, float(g["phipade/alpha"][idx]), H, phi

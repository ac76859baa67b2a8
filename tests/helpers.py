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


FIXTURE = os.path.join(ROOT, "tests", "golden", "ref_fixture.npz")


def write_reference_fixture(directory):
    """Write the reference's own test scenario (tests/golden/ref_fixture.npz,
    made by tests/golden/make_fixture.py from the reference tree) back into
    its file formats under `directory`: problem_options.txt with the
    reference's 15 values (boundary_flux missing, as in the original),
    the two mesh files and Keff.txt.  Returns the options file path."""
    from twoscalerich_gb300 import meshgen
    g = np.load(FIXTURE)
    names = ("macro_structured_10by10.msh", "microB_unstructured_10by10.msh")
    for name, f in zip(("macro", "micro"), names):
        cell = g["mesh/micro/cell"] if name == "micro" else None
        meshgen.Mesh(int(g["mesh/%s/nv" % name][0]), g["mesh/%s/xy" % name],
                     g["mesh/%s/elems" % name], g["mesh/%s/bedges" % name],
                     cell=cell).write(os.path.join(directory, f))
    hdr = g["keff/header"]
    n = int(hdr[1])
    logh, kv = g["keff/logh"], g["keff/values"].reshape(4, n)
    with open(os.path.join(directory, "Keff.txt"), "w") as f:
        f.write("%.20e\n%d\n%.20e\n%.20e\n" % (hdr[0], n, hdr[2], hdr[3]))
        for i in range(n):
            f.write(" ".join("%.20e" % v for v in (logh[i], kv[0, i], kv[1, i], kv[2, i], kv[3, i])) + "\n")
    vals = [g["options/h0"][0], g["options/tend"][0], len(g["options/tspan"])]
    vals += list(g["options/tspan"]) + list(g["options/soilA"]) + list(g["options/soilB"])
    assert len(vals) == int(g["options/tokens"][0])
    opt = os.path.join(directory, "problem_options.txt")
    with open(opt, "w") as f:
        f.write("%s\n%s\nsolution.txt\n" % names)
        for v in vals:
            f.write(("%d\n" % v) if isinstance(v, int) else ("%.20e\n" % v))
    return opt

"""Van Genuchten-Mualem relations and the Keff table of the oracle against
independent evaluations: the textbook VG formulas in 50-digit arithmetic,
and numpy interpolation of the table."""
import ctypes as C

import numpy as np

import oracle
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P


def vg_reference(s, Ss, h):
    """The textbook formulas in 50-digit arithmetic (mpmath)."""
    import mpmath
    mpmath.mp.dps = 50
    n = mpmath.mpf(s["n"])
    m = 1 - 1 / n
    if h >= 0:
        return s["Ksat"], Ss, s["thetas"]
    a = mpmath.mpf(s["alpha"]) * mpmath.mpf(-h)
    t = a ** n
    Se = (1 + t) ** (-m)
    K = s["Ksat"] * mpmath.sqrt(Se) * (1 - (1 - Se ** (1 / m)) ** m) ** 2
    C_ = (mpmath.mpf(s["thetas"]) - s["thetar"]) * m * n * s["alpha"] * a ** (n - 1) * (1 + t) ** (-m - 1)
    th = s["thetar"] + (mpmath.mpf(s["thetas"]) - s["thetar"]) * Se
    return float(K), float(C_ + Ss), float(th)


def test_vg_relations():
    o = oracle.load()
    for soil in (P.SOIL_A, P.SOIL_B):
        sc = P.make_soil(**soil)
        for h in [-1e-6, -1e-3, -0.05, -0.1, -0.5, -1.0, -2.0, -5.0, -20.0, -100.0, -1e3, 0.0, 0.3]:
            out = np.zeros(3)
            o.oracle_vg(C.byref(sc), 1e-6, h, capi.ptr(out))
            ref = vg_reference(soil, 1e-6, h)
            for a, b in zip(out, ref):
                assert abs(a - b) <= 1e-13 * abs(b), (soil, h, a, b)


def test_keff_interpolation_and_clamping():
    o = oracle.load()
    logh = 1.3 - 0.0333 * np.arange(50)
    vals = np.stack([np.linspace(1, 2, 50), np.linspace(-0.1, 0.1, 50),
                     np.linspace(-0.1, 0.1, 50), np.linspace(3, 4, 50)])
    K = capi.Keff()
    kv = np.ascontiguousarray(vals.ravel())
    K.no_hvalues, K.logr, K.logh_first, K.epsilonA = 50, -0.0333, 1.3, 0.6
    K.Keff_values = capi.ptr(kv)
    out = np.zeros(4)
    for h in [-30.0, -20.0, -10.0, -1.0, -0.1, -0.02, -0.01, -1e-5, 0.0, 2.0]:
        o.oracle_keff(C.byref(K), h, capi.ptr(out))
        x = np.log10(abs(h)) if h != 0 else -np.inf
        for c in range(4):
            ref = np.interp(-x, -logh, vals[c])    # increasing abscissa for np.interp
            assert abs(out[c] - ref) <= 1e-13 * abs(ref) + 1e-15, (h, c, out[c], ref)

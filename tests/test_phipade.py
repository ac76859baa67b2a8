"""phi_1 by the (6,6) Pade approximant: this library's host phipade against
the reference's own src/phipade.cpp (golden vectors, OpenBLAS underneath),
against the oracle's restatement (bit for bit) and against an independent
evaluation (scipy expm of the augmented matrix [[A, I], [0, 0]])."""
import ctypes as C

import numpy as np
import pytest
import scipy.linalg

import oracle
from tests.helpers import golden, hessenberg_from_golden
from twoscalerich_gb300 import capi

MAXK = 40


def full_H(m, Hc):
    H = np.zeros((MAXK, MAXK + 1))
    H[:m, :m + 1] = Hc
    return np.ascontiguousarray(H)


def ours(m, alpha, H):
    phi = np.zeros((MAXK, MAXK))
    rc = capi.load().tsr_phipade(capi.ptr(phi.ravel()), capi.ptr(H.ravel()), alpha, m, MAXK)
    return rc, phi


def phi1_expm(A):
    m = A.shape[0]
    Z = np.zeros((2 * m, 2 * m))
    Z[:m, :m] = A
    Z[:m, m:] = np.eye(m)
    return scipy.linalg.expm(Z)[:m, m:]


def test_against_reference_golden_and_oracle():
    g = golden()
    o = oracle.load()
    for idx in range(len(g["phipade/m"])):
        m, alpha, Hc, ref = hessenberg_from_golden(g, idx)
        H = full_H(m, Hc)
        rc, phi = ours(m, alpha, H)
        assert rc == 0
        got = phi[:m, :m]
        scale = np.max(np.abs(ref))
        if m == 1 and alpha * H[0, 0] == 0.0:
            continue
        assert np.max(np.abs(got - ref)) <= 1e-13 * scale + 1e-300, (m, alpha)
        phio = np.zeros((MAXK, MAXK))
        assert o.oracle_phipade(capi.ptr(phio.ravel()), capi.ptr(H.ravel()), alpha, m, MAXK + 1, MAXK) == 0
        assert np.array_equal(phio, phi)


def test_against_expm():
    g = golden()
    for idx in range(len(g["phipade/m"])):
        m, alpha, Hc, _ = hessenberg_from_golden(g, idx)
        H = full_H(m, Hc)
        _, phi = ours(m, alpha, H)
        A = alpha * H[:m, :m].T            # row-major view of the column-major block
        ref = phi1_expm(A).T
        assert np.max(np.abs(phi[:m, :m] - ref)) <= 1e-11 * np.max(np.abs(ref)), (m, alpha)


def test_scalar_case_limits():
    """m = 1: phi_1(0) = 1 (the reference returns NaN at A = 0 and 0 for
    |A| < ~1e-16, src/phipade.cpp:32-40 -- a recorded deviation)."""
    for a, expect in [(0.0, 1.0), (1e-18, 1.0), (-1.4, (np.exp(-1.4) - 1) / -1.4),
                      (-800.0, 1.0 / 800.0), (2.0, (np.exp(2.0) - 1) / 2.0)]:
        H = full_H(1, np.array([[a, 0.0]]))
        rc, phi = ours(1, 1.0, H)
        assert rc == 0
        assert abs(phi[0, 0] - expect) <= 1e-15 * abs(expect)


def test_singular_denominator_returns_error_instead_of_exit():
    H = full_H(3, np.full((3, 4), np.nan))
    rc, _ = ours(3, 1.0, H)
    assert rc == 7          # TSR_ERR_SINGULAR; the reference calls exit() (src/phipade.cpp:160-166)


def test_random_hessenberg_bitwise_against_oracle():
    """The library's phi_1 (matrix products as interleaved FMA chains, work
    matrices kept per thread) equals the oracle's plain loops bit for bit
    on random upper Hessenberg matrices of every Krylov size up to 40 and
    step sizes from 1e-4 to 1e3 (0 to about 20 squarings)."""
    o = oracle.load()
    rng = np.random.default_rng(17)
    for m in range(1, MAXK + 1):
        for alpha in (1e-4, 0.3, 7.0, 1e3):
            Hc = np.zeros((m, m + 1))
            for j in range(m):
                Hc[j, :j + 2] = rng.normal(size=j + 2)
                Hc[j, j + 1] = abs(Hc[j, j + 1]) + 0.1
            H = full_H(m, Hc)
            rc, phi = ours(m, alpha, H)
            phio = np.zeros((MAXK, MAXK))
            rco = o.oracle_phipade(capi.ptr(phio.ravel()), capi.ptr(H.ravel()), alpha, m, MAXK + 1, MAXK)
            assert rc == rco
            if rc == 0:
                # the largest steps overflow where H has eigenvalues with a
                # positive real part: the same NaNs on both sides
                assert np.array_equal(phio, phi, equal_nan=True), (m, alpha)

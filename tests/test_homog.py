"""The unit-cell homogenisation that generates Keff(h) (tsr_keff_homogenize
on the GPU; its CPU restatement oracle/homog.py), checked against the
reference's own table (tests/Richards_Equation/Keff.txt, kept in
tests/golden/ref_fixture.npz):

  * the table's structure: each of its 100 rows is K_A(10^log10|h|) times one
    constant tensor -- K_A the van Genuchten-Mualem conductivity of the
    scenario's material A -- and its epsA is the area fraction of material A
    in the reference's own inclusion mesh, to the 15 digits its file holds;
  * the tensor itself: the reference's generating script is not in its tree
    and its discretisation is unknown; the cell problem here, solved on
    successively finer grids, agrees with the reference's tensor to 2.5 %
    on the diagonal and 5 % off it (3600 s/h converts the reference's
    conductivity unit).
CPU tests check the oracle (no inclusion gives the identity; the Voigt bound
K <= epsA; symmetry); the GPU tests check the GPU solver against it."""
import numpy as np
import pytest

from oracle import homog
from tests.helpers import FIXTURE

REF_FACTOR = 3600.0            # the reference table's K per the soil's Ks: m/h per m/s


def fixture_triangles():
    g = np.load(FIXTURE)
    xy = g["mesh/micro/xy"]
    n = xy.size // 2
    el = g["mesh/micro/elems"].reshape(-1, 3)
    return np.stack([np.stack([xy[el[:, v]], xy[n + el[:, v]]], 1) for v in range(3)], 1)


def reference_tensor():
    """The reference table's constant tensor (Keff / K_A), and its rows."""
    g = np.load(FIXTURE)
    logh, K = g["keff/logh"], g["keff/values"].reshape(4, -1)
    Ks, thr, ths, al, n = g["options/soilA"]
    m = 1.0 - 1.0 / n
    h = 10.0 ** logh
    t = (al * h) ** n
    Se = (1.0 + t) ** (-m)
    B = -np.expm1(m * np.log(t / (1.0 + t)))            # 1 - (1 - Se^(1/m))^m without cancellation
    KA = Ks * np.sqrt(Se) * B * B
    return K / KA, g


def test_reference_table_is_KA_times_a_constant_tensor():
    ratio, g = reference_tensor()
    for c in range(4):
        assert np.max(np.abs(ratio[c] - ratio[c, 0])) <= 1e-11 * abs(ratio[c, 0])
    assert ratio[1, 0] == pytest.approx(ratio[2, 0], rel=1e-14)       # symmetric


def test_oracle_homogenisation():
    tri = fixture_triangles()
    K, eps = homog.homogenize(tri, 0.1, 0.1, 48, 48)
    g = np.load(FIXTURE)
    # the reference's epsA (a 15-digit decimal in its file)
    assert abs(eps - g["keff/header"][0]) <= 1e-15
    assert abs(K[0, 1] - K[1, 0]) <= 1e-10
    assert K[0, 0] < eps and K[1, 1] < eps            # Voigt bound for holes
    ratio, _ = reference_tensor()
    ref = ratio[:, 0].reshape(2, 2) / REF_FACTOR
    assert np.max(np.abs(np.diag(K) - np.diag(ref)) / np.diag(ref)) <= 0.025
    assert abs(K[0, 1] - ref[0, 1]) <= 0.05 * abs(ref[0, 1])
    # no inclusion: the identity
    K0, eps0 = homog.homogenize(np.zeros((0, 3, 2)), 1.0, 1.0, 16, 16)
    assert np.allclose(K0, np.eye(2), atol=1e-12) and eps0 == 1.0

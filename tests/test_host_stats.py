"""CPU: the tail probabilities of the ANOVA statistics (eig_gb300/host/gp_stats.c) against
scipy's distributions."""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "eig_gb300", "_lib", "libgpsynth.so")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        pytest.skip("host library not built")
    L = C.CDLL(LIB)
    L.gp_ftail.restype = C.c_double
    L.gp_ftail.argtypes = [C.c_int, C.c_int, C.c_double]
    L.gp_chitail.restype = C.c_double
    L.gp_chitail.argtypes = [C.c_int, C.c_double]
    return L


def test_f_tail_matches_scipy(lib):
    stats = pytest.importorskip("scipy.stats")
    for d1 in [1, 2, 3, 4, 5, 10, 29]:
        for d2 in [1, 2, 3, 7, 50, 150, 500]:
            for F in [0.01, 0.3, 1.0, 2.5, 10.0, 50.0, 300.0]:
                want = stats.f.sf(F, d1, d2)
                got = lib.gp_ftail(d1, d2, F)
                # the reference's 1 - P form: absolute error at the double spacing of 1
                assert abs(got - want) <= 1e-9 * want + 4e-16, (d1, d2, F)
    assert lib.gp_ftail(3, 10, 1e-7) == 1.0
    assert lib.gp_ftail(3, 100, 1e6) == 0.0


def test_chi_square_tail_matches_scipy(lib):
    stats = pytest.importorskip("scipy.stats")
    for df in [1, 2, 3, 4, 6, 10, 20]:
        for z in [0.0, 0.01, 0.5, 2.0, 10.0, 50.0, 200.0, 900.0]:
            want = stats.chi2.sf(z, df)
            got = lib.gp_chitail(df, z)
            assert abs(got - want) <= 1e-12 * want, (df, z, got, want)

"""Tracy-Widom statistics of the log through the C ABI (gp_twstats, gp_tw_tail, gp_mpstats:
host code, no device): against the reference's logs, against the oracle's independent
restatement (scipy's Airy function, numpy determinants), TW1's known mean and variance, and
the reference's behaviour at the ends of its table.

Tolerances: statistics and effective n text-exact at the log's 3 decimals; p-values within
1e-5 relative of the log and 1e-8 of the oracle; moments 1e-6.
"""
import os

import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O
from tests.goldens import GOLDEN, tw_section
from tests.test_oracle_golden import TW_LOGS, compare_tw, log_cut


@pytest.mark.parametrize("case,name", TW_LOGS)
def test_twstats_match_reference_logs(case, name):
    d = os.path.join(GOLDEN, case)
    lam = np.loadtxt(os.path.join(d, name[:-4] + ".eval"))
    want_mp, shape, want_rows = tw_section(open(os.path.join(d, name)).read())
    if len(lam) != shape[0]:
        pytest.skip("the stored spectrum is truncated")
    compare_tw(native.mpstats(lam), native.twstats(lam, shape[0]), want_mp, want_rows,
               prefix=log_cut(d, name))


def test_tw_tail_matches_oracle_and_moments():
    xs = np.linspace(-9.0, 9.0, 721)
    mine = np.array([native.tw_tail(x) for x in xs])
    ref = np.array([O.tw_tail(x) for x in xs])
    assert np.max(np.abs(mine - ref) / np.maximum(ref, 1e-300)) <= 1e-8
    inside = (xs >= -8.0) & (xs < 8.0)
    assert np.all(mine[inside] <= 1.0 + 1e-12) and np.all(mine[inside] >= 0.0)
    assert np.all(np.diff(mine[inside]) <= 1e-15)  # a right tail decreases
    # TW1: mean -1.2065335746, variance 1.6077810346 (E X = a + int T, E X^2 = a^2 + int 2x T)
    g = np.linspace(-8.0, 7.999, 16000)
    t = np.array([native.tw_tail(x) for x in g])
    m1 = -8.0 + np.trapezoid(t, g)
    m2 = 64.0 + np.trapezoid(2.0 * g * t, g)
    assert abs(m1 - -1.2065335746) <= 1e-6 and abs(m2 - m1 * m1 - 1.6077810346) <= 1e-6


def test_tw_table_ends():
    """below the table the tail is 1; from its last point on the reference reports the
    Margetis-Edelman density (the outputs of its two asymptotic formulas are swapped there)"""
    assert native.tw_tail(-8.5) == 1.0
    for x in (8.0, 9.5, 20.0):
        me = np.exp(-0.25 * np.log(x) - 2.0 * x ** 1.5 / 3.0 - np.log(4.0 * np.sqrt(np.pi)))
        assert abs(native.tw_tail(x) - me) <= 1e-14 * me


def test_twstats_na_rows_and_mpstats_floor():
    lam = np.sort(np.random.default_rng(5).gamma(3.0, 0.4, size=40))[::-1]
    st = native.twstats(lam, 40)
    assert all(s is None for s in st[-9:]) and st[-10] is not None  # nostatslim 10
    assert native.twstats(lam, 40, nostatslim=5)[-5] is not None
    assert native.mpstats(lam[:9]) is None and native.mpstats(lam[:10]) is not None
    ref = O.twstats(lam)
    for a, b in zip(st, ref):
        assert (a is None) == (b is None)
        if a is not None:
            assert abs(a[0] - b[0]) <= 1e-12 * abs(b[0]) + 1e-12 and abs(a[2] - b[2]) <= 1e-9 * b[2]


def test_tw_table_first_use_from_many_threads():
    """the table is built once even when the first calls come from several threads at once
    (ctypes releases the GIL): every thread reads the finished table"""
    import subprocess
    import sys
    code = (
        "import threading, numpy as np\n"
        "from eig_gb300 import native\n"
        "xs = np.linspace(-7.9, 7.9, 41)\n"
        "out = [None] * 8\n"
        "def run(i):\n"
        "    out[i] = [native.tw_tail(x) for x in xs]\n"
        "ts = [threading.Thread(target=run, args=(i,)) for i in range(8)]\n"
        "[t.start() for t in ts]; [t.join() for t in ts]\n"
        "assert all(o == out[0] for o in out), 'threads disagree'\n"
        "print(repr(out[0][20]))\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert abs(float(r.stdout.strip()) - native.tw_tail(0.0)) == 0.0

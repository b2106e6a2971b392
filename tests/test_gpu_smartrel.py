"""smartrel on the GPU (gp_keep_gram + gp_relate, gpusmartrel) against the reference's output.

The golden case holds planted relatives (one sample copies another's genotype at a share of
the SNPs) and one outlier; the reference's pair list, order and full-precision scores are in
tests/golden/bn_rel.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O
from tests.goldens import REL_CASES, Case, compare_rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", REL_CASES)
def test_smartrel_run_matches_reference(gpu, case):
    c = Case(case)
    pairs, r = native.smartrel_run(gpu, c.records, c.nind, code=c.code, **c.rel_opts())
    assert [c.ids[k] for k, *_ in r["outliers"]] == c.ref_outliers
    assert len(pairs) == len(c.ref_rel)
    compare_rel(pairs, c.ids, c, tol=1e-9)


@pytest.mark.parametrize("prec", [native.GP_PREC_SPLIT_FP16, native.GP_PREC_SPLIT_BF16X4])
def test_smartrel_split_gram_scores(gpu, prec):
    """with the split tensor-core Gram the scores move by <= 1e-5; the pairs away from the
    threshold and their order (away from near-ties) are the reference's"""
    c = Case("bn_rel")
    pairs, r = native.smartrel_run(gpu, c.records, c.nind, code=c.code, precision=prec,
                                   **c.rel_opts())
    assert [c.ids[k] for k, *_ in r["outliers"]] == c.ref_outliers
    thr = c.rel_opts().get("relthresh", 0.05)
    ref = {(a, b): y for a, b, y in c.ref_rel}
    got = {(c.ids[a], c.ids[b]): y for a, b, y in pairs}
    for k in set(ref) ^ set(got):
        assert abs(ref.get(k, got.get(k)) - thr) <= 1e-5
    common = set(ref) & set(got)
    assert max(abs(ref[k] - got[k]) for k in common) <= 1e-5


def test_relate_grows_output_and_needs_kept_gram(gpu):
    """gp_relate reports the full count when the output is short (the binding then grows it),
    and fails with a state error when no Gram was kept"""
    c = Case("bn_rel")
    full, _ = native.smartrel_run(gpu, c.records, c.nind, code=c.code, **c.rel_opts())
    K = c.rel_opts()["numeigs"]
    small = gpu.relate(K, max_pairs=4)
    # the handle still holds the last pass's Gram and eigenvectors
    assert [(r_[2]) for r_ in small] == [p[2] for p in full]
    opts = native.default_opts(numeigs=K, numoutliter=0)
    native.smartpca_run(gpu, c.records, c.nind, opts, code=c.code)
    with pytest.raises(native.GpuError):
        gpu.relate(K)


def test_smartrel_random_panel_vs_oracle(gpu):
    """a larger synthetic panel with admixture and no outlier removal (which would take the
    relatives out): the oracle's pairs and scores (1e-9), the planted pairs found"""
    rec, pop = native.synth_records(6000, [150, 150, 100], [0.01, 0.02, 0.04], miss=0.03,
                                    seed=61, nthreads=4, n_admixed=30)
    nind = len(pop)
    g = O.unpack(rec, nind)
    rng = np.random.default_rng(62)
    for a, b, f in [(1, 2, 0.5), (200, 201, 0.5), (300, 420, 0.3), (10, 11, 0.25)]:
        m = rng.random(g.shape[0]) < f
        g[m, b] = g[m, a]
    rec = O.pack(g)
    want, wr = O.smartrel(rec, nind, numeigs=2, relthresh=0.08, numoutliter=0)
    got, r = native.smartrel_run(gpu, rec, nind, numeigs=2, relthresh=0.08, numoutliter=0)
    gk = {(a, b): y for a, b, y in got}
    wk = {(a, b): y for a, b, y in want}
    assert set(gk) == set(wk)
    assert max(abs(gk[k] - wk[k]) for k in wk) <= 1e-9
    assert set(gk) == {(1, 2), (200, 201), (300, 420), (10, 11)}


def test_cli_smartrel_matches_reference_text(tmp_path):
    """gpusmartrel -p par prints the reference's "rel:" lines and writes its outlier lines
    (z-score sign aside)"""
    c = Case("bn_rel")
    d = tmp_path / "bn_rel"
    shutil.copytree(c.dir, d)
    cli = os.path.join(native.LIB_DIR, "gpusmartrel")
    out = subprocess.run([cli, "-p", "par"], cwd=d, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr + out.stdout
    lines = [l for l in out.stdout.splitlines() if l.startswith("rel:")]
    assert len(lines) == len(c.ref_rel_text)
    diff = [i for i, (a, b) in enumerate(zip(lines, c.ref_rel_text)) if a != b]
    for i in diff:
        a, b = lines[i].split(), c.ref_rel_text[i].split()
        assert a[:3] == b[:3] and abs(float(a[3]) - float(b[3])) <= 1.0000001e-3
    assert len(diff) <= 1
    got = [l.split() for l in open(d / "out.outliers").read().splitlines()]
    exp = [l.split() for l in c.ref_outlier_lines]
    assert len(got) == len(exp)
    for g, x in zip(got, exp):
        assert g[:8] == x[:8] and g[8].lstrip("-") == x[8].lstrip("-")
    # an option that changes the matrix is refused, not ignored
    with open(d / "par_ld", "w") as f:
        f.write(open(d / "par").read() + "ldregress: 2\n")
    out = subprocess.run([cli, "-p", "par_ld"], cwd=d, capture_output=True, text=True)
    assert out.returncode != 0 and "ldregress" in out.stderr

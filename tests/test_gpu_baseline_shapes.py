"""Parity at the benchmark shapes, against the reference smartpca's own output.

Three panels whose reference outputs were made by tests/golden/make_golden.py (BIG_CASES):

  cfg1_plain     N=1,000 x M=50,000, 3 populations, F=0.01, 1% missing, seed 1, K=10, no
                 outlier removal
  cfg1_outliers  the same shape with 8 planted divergent samples, 5 outlier iterations
  cfg2_full      N=5,000 x M=600,000, 6 populations, 2% missing, K=20, 5 outlier iterations at
                 sigma 6, lsqproject (the benchmark's workload)

The genotypes are regenerated from their seed with the library's generator and checked
against the records' SHA-256 recorded when the reference ran on them.

Tolerances: FP64 path eigenvalues within 1e-10 of the largest, coordinates within 1e-8; split
fp16 path top-K eigenvalues within 1e-6 relative each; both: the same SNPs used, the same
outliers.  The outlier test reports the margin |z| - sigma of every sample (the reference's
ridoutlier z-score, src/eigensrc/smartsubs.c:18-91) for both paths and requires the split
path's z-scores to stay far closer to the FP64 ones than the nearest sample is to sigma.
"""
import functools
import hashlib
import json
import os

import numpy as np
import pytest

from eig_gb300 import native
from tests.goldens import GOLDEN, compare_coords

pytestmark = pytest.mark.gpu

BIG = ["cfg1_plain", "cfg1_outliers", "cfg2_full"]
SIGMA = 6.0


class BigCase:
    def __init__(self, name):
        d = os.path.join(GOLDEN, name)
        self.name = name
        self.spec = json.load(open(os.path.join(d, "spec.json")))
        self.nind = self.spec["nind"]
        self.ids = ["S%07d" % k for k in range(self.nind)]
        self.K = int(self.spec["par"]["numoutevec"])
        self.iters = int(self.spec["par"]["numoutlieriter"])
        self.ref_evals = np.loadtxt(os.path.join(d, "ref.eval"))
        lines = open(os.path.join(d, "ref.evec")).read().splitlines()
        self.ref_coords = {}
        for ln in lines[1:]:
            t = ln.split()
            self.ref_coords[t[0]] = np.array([float(x) for x in t[1:-1]])
        self.ref_outliers = [ln.split()[2] for ln in open(os.path.join(d, "ref.outliers"))
                             if ln.startswith("REMOVED")]

    def opts(self, precision, **kw):
        o = dict(numeigs=self.K, numoutliter=self.iters, outlthresh=SIGMA, precision=precision)
        o.update(kw)
        return native.default_opts(**o)


@functools.lru_cache(maxsize=1)
def _records(name):
    c = BigCase(name)
    s = c.spec
    rec, pop = native.synth_records(s["nsnp"], s["pops"], s["fst"], miss=s["miss"],
                                    seed=s["seed"])
    digest = hashlib.sha256(np.ascontiguousarray(rec).tobytes()).hexdigest()
    assert digest == s["records_sha256"], \
        "%s: the regenerated genotypes differ from those the reference ran on" % name
    return rec


def _check_run(c, r, eval_tol, coord_tol, top_only):
    """same SNP count, sample count and outliers as the reference; eigenvalues and coordinates
    within the tolerances"""
    assert r["nused"] == c.spec["kept_snps_per_pass"][-1]
    assert r["nrows"] == c.spec["eval_count"]
    assert [c.ids[k] for k, *_ in r["outliers"]] == c.ref_outliers
    ev = r["evals"]
    if top_only:
        e = np.abs(ev[:c.K] - c.ref_evals[:c.K]) / np.abs(c.ref_evals[:c.K])
    else:
        m = len(c.ref_evals)
        e = np.abs(ev[:m] - c.ref_evals) / abs(c.ref_evals[0])
        assert abs(np.sum(ev) - c.spec["eval_sum"]) <= eval_tol * c.spec["eval_sum"]
    assert np.max(e) <= eval_tol, "eigenvalue error %g" % np.max(e)
    mine = {c.ids[k]: r["coords"][:, k] for k in range(c.nind)
            if r["ind_out"][k] and c.ids[k] in c.ref_coords}
    ref = {i: v for i, v in c.ref_coords.items() if i in mine}
    assert len(ref) == len(c.ref_coords)
    scale = max(np.max(np.abs(v[:c.K])) for v in ref.values())
    err = compare_coords(ref, mine, c.K, coord_tol * scale)
    return float(np.max(e)), err / scale


@pytest.mark.parametrize("name", BIG)
def test_fp64_path_matches_reference(gpu, name):
    c = BigCase(name)
    rec = _records(name)
    r = native.smartpca_run(gpu, rec, c.nind, c.opts(native.GP_PREC_FP64))
    e, ce = _check_run(c, r, 1e-10, 1e-8, top_only=False)
    print("%s FP64: eigenvalue error %.2e (of the largest), coordinate error %.2e" % (name, e, ce))


@pytest.mark.parametrize("name", BIG)
def test_split_fp16_path_matches_reference(gpu, name):
    c = BigCase(name)
    rec = _records(name)
    r = native.smartpca_run(gpu, rec, c.nind, c.opts(native.GP_PREC_SPLIT_FP16))
    e, ce = _check_run(c, r, 1e-6, 1e-4, top_only=True)
    print("%s split fp16: top-%d eigenvalue error %.2e (relative), coordinate error %.2e"
          % (name, c.K, e, ce))


def zscores(evecs):
    """ridoutlier's z-scores (mode 0) of each eigenvector over the pass's samples"""
    E = np.asarray(evecs, np.float64)
    W = E - E.mean(axis=1, keepdims=True)
    return W / np.sqrt(np.mean(W * W, axis=1, keepdims=True))


@pytest.mark.parametrize("name", ["cfg1_outliers", "cfg2_full"])
def test_outlier_margins_split_vs_fp64(gpu, name):
    """Every outlier pass of the reference, redone as a single pass on its samples on both
    paths: the flagged sets agree with each other and with the reference, and the split
    path's z-scores differ from the FP64 ones by far less than the smallest margin
    ||z| - sigma| over all samples and eigenvectors."""
    c = BigCase(name)
    rec = _records(name)
    d = os.path.join(GOLDEN, name)
    by_iter = {}
    for ln in open(os.path.join(d, "ref.outliers")):
        t = ln.split()
        if t and t[0] == "REMOVED":
            by_iter.setdefault(int(t[4]), set()).add(t[2])
    removed = set()
    for it in range(1, c.iters + 2):
        ignore = np.zeros(c.nind, np.uint8)
        for sid in removed:
            ignore[c.ids.index(sid)] = 1
        z = {}
        for prec in (native.GP_PREC_FP64, native.GP_PREC_SPLIT_FP16):
            r = native.smartpca_run(gpu, rec, c.nind, c.opts(prec, numoutliter=0, lsqproject=0),
                                    ind_ignore=ignore)
            z[prec] = (zscores(r["evecs"][:10]), r["xindex"])
        z64, rows = z[native.GP_PREC_FP64]
        z16, rows16 = z[native.GP_PREC_SPLIT_FP16]
        assert np.array_equal(rows, rows16)
        sgn = np.sign(np.sum(z64 * z16, axis=1, keepdims=True))
        dz = float(np.max(np.abs(z16 * sgn - z64)))
        margin = np.abs(np.abs(z64) - SIGMA)
        flag64 = {c.ids[k] for k in rows[np.any(np.abs(z64) > SIGMA, axis=0)]}
        flag16 = {c.ids[k] for k in rows[np.any(np.abs(z16) > SIGMA, axis=0)]}
        near = np.argsort(margin.min(axis=0))[:5]
        print("%s pass %d: %d flagged; smallest margins %s; max |z_split - z_fp64| %.2e"
              % (name, it, len(flag64),
                 ", ".join("%s %.4f" % (c.ids[rows[k]], margin[:, k].min()) for k in near), dz))
        assert flag64 == flag16 == by_iter.get(it, set())
        assert dz < 0.01 * float(margin.min())
        if not flag64:
            break
        removed |= flag64
    assert removed == set().union(*by_iter.values()) if by_iter else not removed

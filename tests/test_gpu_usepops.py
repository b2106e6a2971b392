"""usepopsformissing through the C ABI against the oracle (reference goldens: the
bn_usepops cases of test_gpu_parity.py and the CLI text test).

Per pass the observed counts, the count still missing after the fill, the kill flags, xmean
and xfancy are bit-exact against the oracle's restatement of getcolxz + fvadjust; the filled
Gram within 1e-12 of the oracle's (summation order differs); lsqproj's nobs and status
identical and its coefficients within 1e-11.
"""
import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def panel(seed=31):
    # per-sample missing rates up to 0.6 and two 3-sample populations, so that some columns
    # have a population with every genotype missing (left missing by the fill)
    rec, pop = native.synth_records(2500, [90, 80, 70, 3, 3], [0.01, 0.02, 0.04, 0.2, 0.2],
                                    miss=0.0, miss_hi=0.6, seed=seed, nthreads=4, n_admixed=12)
    return rec, np.asarray(pop, np.int32)


@pytest.mark.parametrize("alt", [1, 0])
def test_pass_tables_bit_exact_and_gram(gpu, alt):
    rec, pop = panel()
    nind = len(pop)
    rng = np.random.default_rng(4)
    rows = np.sort(rng.choice(nind, 230, replace=False)).astype(np.int32)
    cols = np.sort(rng.choice(2500, 2100, replace=False)).astype(np.int32)
    # populations of the rows, with a few rows outside the list (-1: no fill)
    rowpop = np.where(pop[rows] >= 5, -1, pop[rows]).astype(np.int32)
    npop = 5
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    gpu.set_row_pops(rowpop, npop)
    r = gpu.xtx(altnormstyle=alt, minallelecnt=3, maxmissing=2)
    s = O.pass_columns(rec, cols, rows, altnormstyle=alt, minallelecnt=3, maxmissing=0x7FFFFFFF)
    O.popfill_columns(s, rowpop, npop, altnormstyle=alt, minallelecnt=3, maxmissing=2)
    assert np.array_equal(r["n0"], s.n0)
    assert np.array_equal(r["n1"], s.n1)
    assert np.array_equal(r["nmiss"], s.nmiss)
    assert np.array_equal(r["killed"], s.killed)
    assert np.array_equal(r["xmean"], s.xmean)  # bit-exact, not approx
    assert np.array_equal(r["xfancy"], s.xfancy)
    # the rule on the count after the fill keeps columns the raw count would kill
    raw = O.pass_columns(rec, cols, rows, altnormstyle=alt, minallelecnt=3, maxmissing=2)
    assert (raw.killed == 1).sum() > (s.killed == 1).sum() > 0
    X = O.gram(s)
    assert np.max(np.abs(r["XTX"] - X)) <= 1e-12 * np.max(np.abs(X))
    assert r["nused"] == int((s.killed == 0).sum())
    # the rows' populations belong to the rows: a new sample list turns the fill off
    gpu.set_samples(rows)
    r2 = gpu.xtx(altnormstyle=alt, minallelecnt=3, maxmissing=2)
    assert np.array_equal(r2["killed"], raw.killed)


def set_missing(rec, snps, k):
    for snp in snps:
        rec[snp, k >> 2] |= np.uint8(3 << ((3 - (k & 3)) * 2))


def test_weights_and_lsqproj_fill_vs_oracle(gpu):
    rec, pop = panel(seed=32)
    nind = len(pop)
    # sample 5 (a listed population) keeps 3 genotypes: dropped by the coverage check before
    # the population sums, although the fill would give it data
    set_missing(rec, range(3, 2500), 5)
    rows = np.nonzero(pop < 3)[0].astype(np.int32)  # the three large populations
    cols = np.arange(2500, dtype=np.int32)
    npop = 5
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    gpu.set_row_pops(pop[rows], npop)
    gpu.xtx(minallelecnt=2)
    ev, V = gpu.eigvecs(8)
    K = 5
    ff, fx, sc = gpu.snp_weights(K)
    s = O.pass_columns(rec, cols, rows, minallelecnt=2, maxmissing=0x7FFFFFFF)
    O.popfill_columns(s, pop[rows], npop, minallelecnt=2)
    off, ofx, osc = O.weights(s, V, K)
    assert np.max(np.abs(ff - off)) <= 1e-10 * np.max(np.abs(off))
    assert np.max(np.abs(fx - ofx)) <= 1e-10 * np.max(np.abs(ofx))
    # every sample projected; populations as lsqproj reads them, some without one; a few
    # samples with almost no data fall to the coverage check
    proj = np.arange(nind, dtype=np.int32)
    sampop = np.where(np.arange(nind) % 7 == 3, -2, np.where(pop >= 5, -1, pop)).astype(np.int32)
    a, b, nobs, st = gpu.lsqproj(K, proj, sampop, npop)
    oa, ob, onobs, ost = O.lsqproj_fill(s, off, osc, K, proj, sampop, npop)
    assert np.array_equal(st, ost)
    assert np.array_equal(nobs, onobs)
    assert st[5] == 1 and nobs[5] <= 3
    ok = st == 0
    assert np.max(np.abs(a[:, ok] - oa[:, ok])) <= 1e-11 * max(1.0, np.max(np.abs(oa)))
    assert np.max(np.abs(b[:, ok] - ob[:, ok])) <= 1e-11 * max(1.0, np.max(np.abs(ob)))
    # the fill counts as observed: more observations than the plain projection
    _, _, nobs0, _ = gpu.lsqproj(K, proj)
    filled = ok & (sampop >= 0)
    assert np.all(nobs[filled] >= nobs0[filled]) and np.any(nobs[filled] > nobs0[filled])


def test_split_precision_refused(gpu):
    rec, pop = panel(seed=33)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(np.arange(nind, dtype=np.int32))
    gpu.set_snps(np.arange(2500, dtype=np.int32))
    gpu.set_row_pops(np.where(pop >= 5, -1, pop), 5)
    with pytest.raises(native.GpuError, match="FP64 precision only"):
        gpu.xtx(precision=native.GP_PREC_SPLIT_FP16)
    with pytest.raises(native.GpuError, match="npop"):
        gpu.set_row_pops(np.full(nind, 7, np.int32), 5)

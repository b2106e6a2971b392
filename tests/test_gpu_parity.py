"""GPU parity: the CUDA path through the C ABI against the oracle and the reference goldens.

Tolerances: integer counts, kill flags and the normalisation table are bit-exact; the FP64
Gram is within 1e-12 of the oracle's (summation order differs); eigenvalues within 1e-10
relative (of the largest) of the reference; .evec coordinates within 1e-8 (sign per vector
is arbitrary, as with LAPACK); outlier sets identical.
"""
import os
import subprocess

import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O
from tests.goldens import CASES, Case, compare_coords, coords_by_id

pytestmark = pytest.mark.gpu


# split precisions: (elementwise tolerance of the Gram relative to its largest entry,
# relative tolerance of the top-20 eigenvalues)
SPLIT_TOL = {native.GP_PREC_SPLIT_BF16: (2e-5, 1e-5), native.GP_PREC_SPLIT_BF16X4: (2e-6, 1e-6),
             native.GP_PREC_SPLIT_FP16: (2e-6, 1e-6)}


def synth(nsnp, pops, fst, miss=0.02, seed=5, **kw):
    rec, pop = native.synth_records(nsnp, pops, fst, miss=miss, seed=seed, nthreads=4, **kw)
    return rec, pop


@pytest.mark.parametrize("code", [native.GP_CODE_PACKED, native.GP_CODE_BED])
def test_counts_and_table_bit_exact(gpu, code):
    rec, pop = synth(3000, [150, 150, 101], [0.01, 0.03, 0.05], miss=0.03, seed=21)
    nind = len(pop)
    rng = np.random.default_rng(0)
    rows = np.sort(rng.choice(nind, 333, replace=False)).astype(np.int32)
    cols = np.sort(rng.choice(3000, 2500, replace=False)).astype(np.int32)
    if code == native.GP_CODE_BED:
        g = O.unpack(rec, nind)
        bedcode = np.where(g < 0, 1, np.where(g == 2, 0, np.where(g == 1, 2, 3))).astype(np.uint8)
        blen = (nind + 3) // 4
        c = np.concatenate([bedcode, np.zeros((3000, blen * 4 - nind), np.uint8)], 1)
        c = c.reshape(3000, blen, 4)
        dev_rec = (c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)).astype(np.uint8)
    else:
        dev_rec = rec
    gpu.load_genotypes(dev_rec, nind, code)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    for alt in (1, 0):
        r = gpu.xtx(altnormstyle=alt, minallelecnt=5, maxmissing=12)
        s = O.pass_columns(rec, cols, rows, altnormstyle=alt, minallelecnt=5, maxmissing=12)
        assert np.array_equal(r["n0"], s.n0)
        assert np.array_equal(r["n1"], s.n1)
        assert np.array_equal(r["nmiss"], s.nmiss)
        assert np.array_equal(r["killed"], s.killed)
        assert np.array_equal(r["xmean"], s.xmean)  # bit-exact, not approx
        assert np.array_equal(r["xfancy"], s.xfancy)
        X = O.gram(s)
        scale = np.max(np.abs(X))
        assert np.max(np.abs(r["XTX"] - X)) <= 1e-12 * scale
        assert abs(r["trace"] - np.trace(X)) <= 1e-12 * abs(np.trace(X))
        assert r["nused"] == int((s.killed == 0).sum())


def test_valid_counts(gpu):
    rec, pop = synth(1000, [90, 90], [0.02, 0.02], miss=0.2, seed=22)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    g = O.unpack(rec, nind)
    rng = np.random.default_rng(1)
    su = (rng.random(nind) < 0.7).astype(np.uint8)
    pu = (rng.random(1000) < 0.6).astype(np.uint8)
    sv, iv = gpu.valid_counts(su, pu)
    assert np.array_equal(sv, ((g >= 0) & (su[None, :] == 1)).sum(1))
    assert np.array_equal(iv, ((g >= 0) & (pu[:, None] == 1)).sum(0))


def test_set_missing(gpu):
    rec, pop = synth(200, [40, 41], [0.02, 0.02], miss=0.0, seed=23)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    pairs = np.array([[3, 0], [3, 80], [150, 17]], np.int64)
    gpu.set_missing(pairs)
    sv, _ = gpu.valid_counts()
    g = O.unpack(rec, nind)
    for s, k in pairs:
        g[s, k] = -1
    assert np.array_equal(sv, (g >= 0).sum(1))


def test_eigvecs_fp64(gpu):
    rec, pop = synth(4000, [100, 100, 100], [0.01, 0.02, 0.04], seed=24)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(4000, dtype=np.int32)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    gpu.xtx()
    ev, V = gpu.eigvecs(10)
    s = O.pass_columns(rec, cols, rows)
    w, U = O.eig_scaled(O.gram(s))
    assert np.max(np.abs(ev - w)) <= 1e-10 * w[0]
    cosang = np.abs(np.sum(V * U[:10], axis=1))
    assert np.all(cosang > 1 - 1e-9)


def test_ridoutlier_host_matches_oracle():
    rng = np.random.default_rng(3)
    E = rng.standard_normal((6, 200)) / np.sqrt(200)
    E[2, 17] = 0.9
    E[4, 33] = -0.8
    for mode in (0, 1):
        b1, v1, s1 = native.ridoutlier(E, 6, 6.0, mode)
        b2, v2, s2 = O.ridoutlier(E, 6, 6.0, mode)
        assert list(b1) == list(b2) and len(b1) >= 2
        assert np.array_equal(v1, v2)
        assert np.array_equal(s1, s2)


@pytest.mark.parametrize("prec", [native.GP_PREC_FP64, native.GP_PREC_SPLIT_FP16])
def test_weights_and_lsqproj_vs_oracle(gpu, prec):
    """SNP weights, sample scores and lsqproject against the oracle on the same eigenvectors:
    FP64 SIMT kernels (FP64 path) or the exact sliced tensor-core products (split paths)."""
    rec, pop = synth(3000, [80, 80, 60], [0.01, 0.03, 0.05], miss=0.05, seed=25, n_admixed=10)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    rows = np.arange(0, nind, dtype=np.int32)[:200]
    cols = np.arange(3000, dtype=np.int32)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    gpu.xtx(minallelecnt=3, precision=prec)
    ev, V = gpu.eigvecs(8)
    K = 6
    ff, fx, sc = gpu.snp_weights(K)
    s = O.pass_columns(rec, cols, rows, minallelecnt=3)
    off, ofx, osc = O.weights(s, V, K)
    assert np.max(np.abs(ff - off)) <= 1e-10 * np.max(np.abs(off))
    assert np.max(np.abs(fx - ofx)) <= 1e-10 * np.max(np.abs(ofx))
    assert np.max(np.abs(sc - osc) / osc) <= 1e-10
    proj = np.arange(nind, dtype=np.int32)
    a, b, nobs, st = gpu.lsqproj(K, proj)
    oa, ob, onobs, ost = O.lsqproj(s, off, osc, K, proj)
    assert np.array_equal(nobs, onobs)
    assert np.array_equal(st, ost)
    ok = st == 0
    # lsqproject coefficients (before eigscale, magnitudes up to ~1e4): 1e-11 relative
    assert np.max(np.abs(a[:, ok] - oa[:, ok])) <= 1e-11 * max(1.0, np.max(np.abs(oa)))
    assert np.max(np.abs(b[:, ok] - ob[:, ok])) <= 1e-11 * max(1.0, np.max(np.abs(ob)))


@pytest.mark.parametrize("case", CASES)
def test_smartpca_run_matches_reference(gpu, case):
    c = Case(case)
    opts = native.default_opts(**c.opts())
    r = native.smartpca_run(gpu, c.records, c.nind, opts, code=c.code,
                            ind_affstatus=c.affstatus, ind_pop=c.ind_pop)
    assert r["nrows"] == len(c.ref_evals)
    scale = abs(c.ref_evals[0])
    assert np.max(np.abs(r["evals"] - c.ref_evals)) <= 1e-10 * scale
    assert [c.ids[k] for k, *_ in r["outliers"]] == c.ref_outliers
    mine = coords_by_id(c.ids, r["coords"], r["ind_out"])
    compare_coords(c.ref_coords, mine, r["numeigs"], 1e-8)


@pytest.mark.parametrize("case", CASES)
def test_cli_dropin_matches_reference_text(case, tmp_path):
    """gpusmartpca -p par writes the reference's .eval/.evec text (up to evec signs)."""
    c = Case(case)
    import shutil
    d = tmp_path / case
    shutil.copytree(c.dir, d)
    cli = os.path.join(native.LIB_DIR, "gpusmartpca")
    out = subprocess.run([cli, "-p", "par"], cwd=d, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr + out.stdout
    ev = [float(x) for x in open(d / "out.eval").read().split()]
    ref = [float(x) for x in open(d / "ref.eval.txt").read().split()]
    assert len(ev) == len(ref)
    assert np.max(np.abs(np.array(ev) - np.array(ref))) <= 1.0e-6
    mine = open(d / "out.evec").read().splitlines()
    want = open(d / "ref.evec.txt").read().splitlines()
    assert mine[0] == want[0]
    assert len(mine) == len(want)
    A = np.array([[float(x) for x in l.split()[1:-1]] for l in want[1:]])
    B = np.array([[float(x) for x in l.split()[1:-1]] for l in mine[1:]])
    assert [l.split()[0] for l in mine[1:]] == [l.split()[0] for l in want[1:]]
    s = np.sign(np.sum(A * B, axis=0))
    assert np.max(np.abs(A - B * s)) <= 1.01e-4
    # outlier lines: identical except the sign of the z-score, which follows the (arbitrary)
    # sign of the eigenvector, as the reference's does with its LAPACK build
    got = [l.split() for l in open(d / "out.outliers").read().splitlines()]
    exp = [l.split() for l in open(d / "ref.outliers").read().splitlines()]
    assert len(got) == len(exp)
    for g, x in zip(got, exp):
        assert g[:8] == x[:8] and g[9:] == x[9:]
        assert g[8].lstrip("-") == x[8].lstrip("-")
    # writesnpeigs: the eigbestsnp log lines, and the snpweightoutname file when the parfile
    # names one (weights up to each vector's sign, at the printed precision)
    from tests.goldens import eigbestsnp_lines, kurtosis_lines
    mine_k = kurtosis_lines(out.stdout)
    want_k = kurtosis_lines(open(d / "ref.log").read())
    assert [k[0] for k in mine_k] == [k[0] for k in want_k] and len(want_k) > 0
    assert all(abs(a[1] - b[1]) <= 1.01e-3 and abs(a[2] - b[2]) <= 1.01e-3
               for a, b in zip(mine_k, want_k))
    # the run-progress lines (preamble, per-pass kills and outlier removals, lsqproj's
    # marker): the reference's text
    from tests.goldens import progress_lines
    assert progress_lines(out.stdout) == progress_lines(open(d / "ref.log").read())
    # the mpstats line and the Tracy-Widom section: eigenvalues at the printed 6 decimals,
    # statistics and effective n at 3 decimals (1.01e-3: the GPU eigenvalues differ from the
    # reference's in the 13th digit, which can move a printed last digit), p-values 1e-4
    from tests.goldens import tw_section
    mine_mp, mine_shape, mine_tw = tw_section(out.stdout)
    want_mp, want_shape, want_tw = tw_section(open(d / "ref.log").read())
    assert mine_shape == want_shape and len(mine_tw) == len(want_tw) > 0
    assert all(abs(a - b) <= 1.01e-3 for a, b in zip(mine_mp, want_mp))
    for a, b in zip(mine_tw, want_tw):
        assert a[0] == b[0] and abs(a[1] - b[1]) <= 1.01e-6
        assert (a[3] is None) == (b[3] is None) and (a[5] is None) == (b[5] is None)
        if b[3] is not None:
            assert abs(a[3] - b[3]) <= 1.01e-3 and abs(a[5] - b[5]) <= 1.01e-3 * max(1.0, b[5] * 1e-6)
            assert abs(a[4] - b[4]) <= 1e-4 * max(b[4], 1e-6)
    mine_b = eigbestsnp_lines(out.stdout)
    want_b = eigbestsnp_lines(open(d / "ref.log").read())
    assert [m[:4] for m in mine_b] == [w[:4] for w in want_b]
    assert all(abs(m[4] - w[4]) <= 1.01e-3 for m, w in zip(mine_b, want_b))
    if "snpweightoutname" in c.par:
        mw = [l.split() for l in open(d / "out.snpwt").read().splitlines()]
        ww = [l.split() for l in open(d / "ref.snpwt.txt").read().splitlines()]
        assert [l[:3] for l in mw] == [l[:3] for l in ww]
        A = np.array([[float(x) for x in l[3:]] for l in ww])
        B = np.array([[float(x) for x in l[3:]] for l in mw])
        sg = np.sign(np.sum(A * B, axis=0))
        assert np.max(np.abs(A - B * sg)) <= 1.01e-6


@pytest.mark.parametrize("binary", [False, True])
def test_cli_grm_dump_matches_reference(binary, tmp_path):
    """grmoutname (and grmbinary): the last pass's GRM after outlier removal, as text
    (values within 1e-10 at full precision, printed lines identical up to %0.6f rounding
    boundaries) or float binary (within 1 ulp), with the reference's id and count files."""
    import shutil

    from tests.goldens import Grm, compare_grm_text, float_ulps
    c = Case("bn_grm")
    d = tmp_path / "bn_grm"
    shutil.copytree(c.dir, d)
    cli = os.path.join(native.LIB_DIR, "gpusmartpca")
    out = subprocess.run([cli, "-p", "par_bin" if binary else "par"], cwd=d, capture_output=True,
                         text=True)
    assert out.returncode == 0, out.stderr + out.stdout
    g = Grm("bn_grm")
    assert open(d / "out.grm.id").read().splitlines() == g.ids
    if binary:
        assert np.array_equal(np.fromfile(d / "out.grm.N.bin", np.int32), g.nbin)
        assert np.max(float_ulps(np.fromfile(d / "out.grm.bin", np.float32), g.bin)) <= 1
    else:
        lines = open(d / "out.grm").read().splitlines()
        vals = [float(l.split()[3]) for l in lines]
        # the printed values carry 6 decimals; the full-precision check is the run's XTX below
        compare_grm_text(lines, g.text, g.values, g.values)
        assert np.max(np.abs(np.array(vals) - g.values)) <= 5.0000001e-7


def test_smartpca_run_grm_values_full_precision(gpu):
    """the last pass's XTX returned by gp_smartpca_run gives the reference's GRM values
    within 1e-10 (relative to the largest)"""
    from tests.goldens import Grm
    c = Case("bn_grm")
    opts = native.default_opts(**c.opts())
    r = native.smartpca_run(gpu, c.records, c.nind, opts, code=c.code, want_xtx=True)
    g = Grm("bn_grm")
    txt, binv = O.grm(r["xtx"])
    assert r["nused"] == g.numsnps[0]
    assert np.max(np.abs(txt - g.values)) <= 1e-10 * np.max(np.abs(g.values))


def _gram_pair(gpu, rec, nind, rows, cols, precision):
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    return gpu.xtx(precision=precision)


@pytest.mark.parametrize("prec", list(SPLIT_TOL))
@pytest.mark.parametrize("shape", [(333, 3000), (128, 64), (1000, 5000)])
def test_split_gram_vs_oracle(gpu, shape, prec):
    """split-BF16 Gram (tcgen05) against the FP64 oracle Gram: the hi+lo split keeps about
    17 significant bits per value, so elementwise error <= 2e-5 of the largest entry."""
    nind, nsnp = shape
    rec, pop = synth(nsnp, [nind // 3, nind // 3, nind - 2 * (nind // 3)], [0.01, 0.03, 0.05],
                     miss=0.02, seed=31)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(nsnp, dtype=np.int32)
    r = _gram_pair(gpu, rec, nind, rows, cols, prec)
    s = O.pass_columns(rec, cols, rows)
    X = O.gram(s)
    scale = np.max(np.abs(X))
    err = np.max(np.abs(r["XTX"] - X)) / scale
    assert err <= SPLIT_TOL[prec][0], err
    assert np.array_equal(r["killed"], s.killed)


@pytest.mark.parametrize("prec", list(SPLIT_TOL))
def test_split_multi_tile_chunks_and_superchunks(gpu, monkeypatch, prec):
    """2600 samples (21 tile rows, 231 tiles: several per CTA), 6000 SNPs in super-chunks of
    2048 SNPs (the sum carried through the Gram between launches), against the FP64 GPU
    Gram."""
    nind, nsnp = 2600, 6000
    rec, pop = synth(nsnp, [900, 900, 800], [0.01, 0.02, 0.04], miss=0.02, seed=32)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(nsnp, dtype=np.int32)
    ref = _gram_pair(gpu, rec, nind, rows, cols, native.GP_PREC_FP64)["XTX"]
    monkeypatch.setenv("GP_BF16_BUDGET_BYTES", str(2688 * 4 * 2048))
    r = _gram_pair(gpu, rec, nind, rows, cols, prec)
    etol, vtol = SPLIT_TOL[prec]
    err = np.max(np.abs(r["XTX"] - ref)) / np.max(np.abs(ref))
    assert err <= etol, err
    w1 = np.linalg.eigvalsh(r["XTX"])[::-1][:20]
    w0 = np.linalg.eigvalsh(ref)[::-1][:20]
    assert np.max(np.abs(w1 - w0) / w0) <= vtol


@pytest.mark.parametrize("prec", list(SPLIT_TOL))
@pytest.mark.parametrize("density", ["dense", "sparse"])
def test_split_subset_rows(gpu, prec, density):
    """row subsets (outlier removal) and killed columns through the split path; the sparse
    subset (every 6th sample) spans more record bytes per 256-row tile than the shared-memory
    transpose stages, so it takes the per-thread path"""
    if density == "dense":
        rec, pop = synth(4000, [200, 200, 150], [0.01, 0.02, 0.05], miss=0.05, seed=33)
        nind = len(pop)
        rng = np.random.default_rng(4)
        rows = np.sort(rng.choice(nind, 401, replace=False)).astype(np.int32)
    else:
        rec, pop = synth(4000, [1200, 1000, 800], [0.01, 0.02, 0.05], miss=0.05, seed=33)
        nind = len(pop)
        rng = np.random.default_rng(4)
        rows = np.arange(1, nind, 6, dtype=np.int32)
    cols = np.sort(rng.choice(4000, 3333, replace=False)).astype(np.int32)
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    r = gpu.xtx(precision=prec, minallelecnt=20)
    s = O.pass_columns(rec, cols, rows, minallelecnt=20)
    X = O.gram(s)
    assert (s.killed == 1).sum() > 0
    assert np.max(np.abs(r["XTX"] - X)) / np.max(np.abs(X)) <= SPLIT_TOL[prec][0]


def test_tc_products_large_k_and_projection_subset(gpu):
    """exact tensor-core products over 20,000 SNPs (several 8,192-SNP chunks, k-splits) and a
    projection set of samples outside the PCA rows, against the oracle"""
    rec, pop = synth(20000, [150, 150, 100], [0.01, 0.02, 0.05], miss=0.1, seed=26, n_admixed=30)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    rows = np.arange(0, 300, dtype=np.int32)
    cols = np.arange(20000, dtype=np.int32)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    gpu.xtx(precision=native.GP_PREC_SPLIT_FP16)
    ev, V = gpu.eigvecs(10)
    K = 10
    ff, fx, sc = gpu.snp_weights(K)
    s = O.pass_columns(rec, cols, rows)
    off, ofx, osc = O.weights(s, V, K)
    assert np.max(np.abs(ff - off)) <= 1e-10 * np.max(np.abs(off))
    assert np.max(np.abs(fx - ofx)) <= 1e-10 * np.max(np.abs(ofx))
    proj = np.arange(250, nind, dtype=np.int32)
    a, b, nobs, st = gpu.lsqproj(K, proj)
    oa, ob, onobs, ost = O.lsqproj(s, off, osc, K, proj)
    assert np.array_equal(nobs, onobs) and np.array_equal(st, ost)
    ok = st == 0
    # lsqproject coefficients (before eigscale, magnitudes up to ~1e4): 1e-11 relative
    assert np.max(np.abs(a[:, ok] - oa[:, ok])) <= 1e-11 * max(1.0, np.max(np.abs(oa)))
    assert np.max(np.abs(b[:, ok] - ob[:, ok])) <= 1e-11 * max(1.0, np.max(np.abs(ob)))


@pytest.mark.parametrize("case", CASES)
def test_smartpca_run_split_fp16_vs_reference(gpu, case):
    """split-fp16 Gram + tensor-core weights/lsqproject against the reference goldens:
    eigenvalues within 1e-6 relative (of the largest), identical outliers and printed sets,
    the top two coordinates (population structure) within 1e-4."""
    c = Case(case)
    opts = native.default_opts(precision=native.GP_PREC_SPLIT_FP16, **c.opts())
    if opts.usepopsformissing:
        # the population fill runs in the FP64 drop-in precision only, and says so
        with pytest.raises(native.GpuError, match="FP64 precision only"):
            native.smartpca_run(gpu, c.records, c.nind, opts, code=c.code,
                                ind_affstatus=c.affstatus, ind_pop=c.ind_pop)
        return
    r = native.smartpca_run(gpu, c.records, c.nind, opts, code=c.code,
                            ind_affstatus=c.affstatus)
    assert r["nrows"] == len(c.ref_evals)
    assert np.max(np.abs(r["evals"] - c.ref_evals)) <= 1e-6 * abs(c.ref_evals[0])
    assert [c.ids[k] for k, *_ in r["outliers"]] == c.ref_outliers
    mine = coords_by_id(c.ids, r["coords"], r["ind_out"])
    compare_coords(c.ref_coords, mine, 2, 1e-4)


@pytest.mark.parametrize("path", ["default", "GP_EIG_NO_FF=1", "GP_EIG_II_GLOBAL=1",
                                  "GP_TRIDIAG_SWITCH=300", "GP_TRIDIAG_SWITCH=1"])
def test_eig_tridiag_all_values_top_vectors(gpu, monkeypatch, path):
    """sytrd + bisection + inverse iteration + ormtr: every eigenvalue within 1e-12 of the
    largest against LAPACK (numpy eigh), 24 top eigenvectors with small residuals, orthonormal,
    and equal (up to sign) to LAPACK's where the eigenvalues are separated; also through the
    multisection without its float-float phase, the inverse iteration with its factors in
    global memory (the paths of larger N), and the lower-triangle tiled reduction switching to
    whole columns at trailing order 300 or only for the last step (at N = 1,200 the default
    runs whole columns throughout)"""
    if path != "default":
        key, val = path.split("=")
        monkeypatch.setenv(key, val)
    rec, pop = synth(6000, [500, 400, 300], [0.01, 0.02, 0.04], miss=0.02, seed=27)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(6000, dtype=np.int32)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    X = gpu.xtx()["XTX"]
    ev, V = gpu.eigvecs(24)
    Xs = X * ((nind - 1) / np.trace(X))
    w, U = np.linalg.eigh(Xs)
    w = w[::-1]
    U = U[:, ::-1].T
    assert np.max(np.abs(ev - w)) <= 1e-12 * w[0]
    R = V @ Xs - ev[:24, None] * V
    assert np.max(np.linalg.norm(R, axis=1)) <= 1e-9 * w[0]
    assert np.max(np.abs(V @ V.T - np.eye(24))) <= 1e-10
    gaps = np.minimum(np.abs(np.diff(w[:25]))[:-1], np.abs(np.diff(w[:25]))[1:])
    sep = np.concatenate([[w[0] - w[1]], gaps])[:24] > 1e-3 * w[0]
    cos = np.abs(np.sum(V * U[:24], axis=1))
    assert np.all(cos[sep] > 1 - 1e-9)


@pytest.mark.parametrize("prec", [native.GP_PREC_FP64, native.GP_PREC_SPLIT_FP16])
def test_fastpca_vs_oracle(gpu, prec):
    """fastmode with the same Omega as the numpy restatement of kjg_fpca: eigenvalues within
    1e-9 relative, eigenvectors equal up to sign (|cos| > 1 - 1e-8) for the separated ones;
    row subset (every other sample) and all-sample paths"""
    rec, pop = synth(5000, [120, 120, 80], [0.01, 0.03, 0.05], miss=0.02, seed=28, n_admixed=20)
    nind = len(pop)
    cols = np.arange(5000, dtype=np.int32)
    K, L, I = 4, 8, 4
    for rows in (np.arange(nind, dtype=np.int32), np.arange(0, nind, 2, dtype=np.int32)):
        gpu.load_genotypes(rec, nind)
        gpu.set_samples(rows)
        gpu.set_snps(cols)
        om = np.random.default_rng(5).standard_normal((len(rows), L))
        ev, V = gpu.fastpca(K, L, I, omega=om, precision=prec)
        oev, oV = O.fastpca(rec, cols, rows, K, L, I, om)
        assert np.max(np.abs(ev - oev) / oev) <= 1e-9
        cos = np.abs(np.sum(V * oV, axis=1))
        sep = np.r_[oev[:-1] / oev[1:] > 1.01, True][:K]
        assert np.all(cos[sep] > 1 - 1e-8), cos
        assert np.allclose(np.linalg.norm(V, axis=1), 1.0)


def test_fastpca_top_eigenvalues_match_exact(gpu):
    """fastmode's top eigenvalues against the exact FP64 eigenvalues of X^T X / M (the
    randomized method converges on the separated population-structure eigenvalues)"""
    rec, pop = synth(8000, [150, 150, 100], [0.02, 0.04, 0.08], miss=0.01, seed=29)
    nind = len(pop)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(8000, dtype=np.int32)
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    ev, V = gpu.fastpca(2, 8, 4, seed=3, precision=native.GP_PREC_SPLIT_FP16)
    s = O.pass_columns(rec, cols, rows, minallelecnt=0, maxmissing=2 ** 31 - 1)
    w = np.linalg.eigvalsh(O.gram(s))[::-1] / (2.0 * 8000)
    assert np.max(np.abs(ev - w[:2]) / w[:2]) <= 1e-6


@pytest.mark.parametrize("nind", [1000, 1700])
def test_split_gram_clusters_equal_single_ctas(gpu, monkeypatch, nind):
    """the cluster kernels (four CTAs on a 2 x 2 block of tiles, two CTAs on two tiles of a
    row, boxes multicast) give the Gram of the one-CTA kernel bit for bit, odd tile counts
    (stand-in tiles) included"""
    rec, pop = synth(3000, [nind // 2, nind - nind // 2], [0.01, 0.03], miss=0.02, seed=37)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(3000, dtype=np.int32)
    grams = {}
    for cl in ("4", "2", "1"):
        monkeypatch.setenv("GP_GRAM_CLUSTER", cl)
        grams[cl] = _gram_pair(gpu, rec, nind, rows, cols, native.GP_PREC_SPLIT_FP16)["XTX"]
    assert np.array_equal(grams["4"], grams["1"])
    assert np.array_equal(grams["2"], grams["1"])



@pytest.mark.parametrize("prec,etol,vtol", [(native.GP_PREC_SPLIT_FP16, 2e-6, 1e-6),
                                            (native.GP_PREC_SPLIT_BF16X4, 4e-6, 2e-6)])
def test_split_gram_rare_variants(gpu, prec, etol, vtol):
    """ancestral allele frequencies down to 1/(2N) (hundreds of kept SNPs with a single minor
    allele copy): the common genotype's value -2 sqrt(p) is small, so its fp16 lo part can be
    subnormal (an absolute error of at most 3e-8, below the 2^-22 relative error of values near
    1), and the rare genotype's value is large (up to ~2 sqrt(2N)), so single SNPs dominate some
    entries.  fp16 hi+lo (22 bits) holds the usual 2e-6 elementwise and 1e-6 top-20 eigenvalue
    bounds against the FP64 GPU Gram; bf16 hi+lo (16 bits, 2^-17 per value) is within 4e-6
    elementwise (measured 2.1e-6) and 2e-6 on the eigenvalues (measured 1.1e-6, a uniform
    downward bias of the FP32 chunk sums)"""
    nind, nsnp = 2000, 20000
    rec, pop = synth(nsnp, [700, 700, 600], [0.01, 0.02, 0.03], miss=0.02, seed=41,
                     p_lo=1.0 / (2 * nind), p_hi=0.02)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(nsnp, dtype=np.int32)
    r64 = _gram_pair(gpu, rec, nind, rows, cols, native.GP_PREC_FP64)
    mac = np.minimum(r64["n0"], r64["n1"])
    assert np.sum((mac == 1) & (r64["killed"] == 0)) > 100
    ref = r64["XTX"]
    r = _gram_pair(gpu, rec, nind, rows, cols, prec)
    err = np.max(np.abs(r["XTX"] - ref)) / np.max(np.abs(ref))
    assert err <= etol, err
    w1 = np.linalg.eigvalsh(r["XTX"])[::-1][:20]
    w0 = np.linalg.eigvalsh(ref)[::-1][:20]
    assert np.max(np.abs(w1 - w0) / w0) <= vtol


@pytest.mark.parametrize("rounds", ["one", "three"])
def test_eig_n5000_vs_lapack(gpu, monkeypatch, rounds):
    """the eigensolver at the benchmark's order, N=5,000, where the float-float
    tridiagonalisation first streams a trailing matrix larger than L2: every eigenvalue within
    1e-12 of the largest against LAPACK (numpy eigh on the host), the top 20 eigenvectors with
    small residuals, orthonormal and equal (up to sign) to LAPACK's where separated; also with
    the tiled steps' parts cut into rounds of 32 per CTA (the path of orders above ~6,000,
    where a CTA's parts do not fit shared memory at once)"""
    if rounds == "three":
        monkeypatch.setenv("GP_TT_ROUND", "32")
    rec, pop = synth(7000, [1800, 1700, 1500], [0.01, 0.02, 0.04], miss=0.02, seed=43)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(np.arange(nind, dtype=np.int32))
    gpu.set_snps(np.arange(7000, dtype=np.int32))
    X = gpu.xtx()["XTX"]
    ev, V = gpu.eigvecs(20)
    Xs = X * ((nind - 1) / np.trace(X))
    w, U = np.linalg.eigh(Xs)
    w = w[::-1]
    U = U[:, ::-1].T
    assert np.max(np.abs(ev - w)) <= 1e-12 * w[0]
    R = V @ Xs - ev[:20, None] * V
    assert np.max(np.linalg.norm(R, axis=1)) <= 1e-9 * w[0]
    assert np.max(np.abs(V @ V.T - np.eye(20))) <= 1e-10
    gaps = np.minimum(np.abs(np.diff(w[:21]))[:-1], np.abs(np.diff(w[:21]))[1:])
    sep = np.concatenate([[w[0] - w[1]], gaps])[:20] > 1e-3 * w[0]
    cos = np.abs(np.sum(V * U[:20], axis=1))
    assert np.all(cos[sep] > 1 - 1e-9)

"""Edge cases of the CUDA path through the C ABI: tiny and ragged panels (a sample count that
is not a multiple of 4, a single SNP), the eigensolver above the float-float path's order
limit (the library's sytrd fallback at N > 8,533), and the error statuses the entry points
return instead of exiting (the reference's fatalx).

Tolerances: counts, kill flags and tables bit-exact; the FP64 Gram within 1e-12 of the
oracle's; eigenvalues within 1e-10 relative to the largest.
"""
import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nind,nsnp", [(2, 40), (3, 1), (5, 65), (131, 7), (257, 300)])
def test_tiny_and_ragged_panels(gpu, nind, nsnp):
    rng = np.random.default_rng(nind * 1000 + nsnp)
    g = rng.integers(0, 3, size=(nsnp, nind)).astype(np.int8)
    g[rng.random((nsnp, nind)) < 0.1] = -1
    if nsnp > 1:
        g[0, :] = 1  # heterozygous everywhere: kept (min(n0, n1) = nind)
    rec = O.pack(g)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(nsnp, dtype=np.int32)
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    r = gpu.xtx()
    s = O.pass_columns(rec, cols, rows)
    for key in ("n0", "n1", "nmiss", "killed", "xmean", "xfancy"):
        assert np.array_equal(r[key], getattr(s, key)), key
    X = O.gram(s)
    scale = max(np.max(np.abs(X)), 1e-300)
    assert np.max(np.abs(r["XTX"] - X)) <= 1e-12 * scale
    if np.trace(X) > 0:
        ev, V = gpu.eigvecs(min(2, nind))
        w, U = O.eig_scaled(X)
        assert np.max(np.abs(ev - w)) <= 1e-10 * max(abs(w[0]), 1.0)


def test_smartpca_run_tiny_panel_vs_oracle(gpu):
    """the whole flow on 9 samples x 60 SNPs (ragged last byte, missing data)"""
    rng = np.random.default_rng(3)
    g = rng.integers(0, 3, size=(60, 9)).astype(np.int8)
    g[rng.random(g.shape) < 0.05] = -1
    rec = O.pack(g)
    opts = native.default_opts(numeigs=3, numoutliter=0)
    r = native.smartpca_run(gpu, rec, 9, opts)
    ref = O.smartpca(rec, 9, numeigs=3, numoutliter=0)
    assert np.array_equal(r["xindex"], ref["xindex"])
    assert np.max(np.abs(r["evals"] - ref["evals"])) <= 1e-10 * ref["evals"][0]
    s = np.sign(np.sum(r["coords"] * ref["coords"], axis=1))
    assert np.max(np.abs(r["coords"] - ref["coords"] * s[:, None])) <= 1e-8


def test_eigensolve_above_float_float_limit(gpu):
    """N = 8,600 > 8,533: the tridiagonalisation falls back to the library's sytrd.  The
    Gram has rank <= M = 300, so its nonzero eigenvalues are those of the 300 x 300 matrix
    X^T X, which the host computes exactly enough to check 1e-10."""
    nind, nsnp = 8600, 300
    rec, pop = native.synth_records(nsnp, [3000, 3000, 2600], [0.02, 0.03, 0.05], miss=0.02,
                                    seed=77, nthreads=4)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(nsnp, dtype=np.int32)
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    r = gpu.xtx()
    ev, V = gpu.eigvecs(5)
    s = O.pass_columns(rec, cols, rows)
    tab = s.tab.reshape(-1, 4)
    geno = O.unpack(rec, nind)
    Xs = np.zeros((nind, nsnp))
    for c in range(nsnp):
        if s.killed[c]:
            continue
        code = np.where(geno[c] < 0, 3, geno[c])
        Xs[:, c] = tab[c][code]
    small = Xs.T @ Xs
    scale = (nind - 1) / np.trace(small)
    w = np.sort(np.linalg.eigvalsh(small * scale))[::-1]
    assert np.max(np.abs(ev[:nsnp] - w)) <= 1e-10 * w[0]
    assert np.all(np.abs(ev[nsnp:]) <= 1e-10 * w[0])  # the Gram's null space
    # the top vectors: residual of the scaled Gram's eigen-equation
    G = (Xs @ Xs.T) * scale
    for j in range(5):
        res = G @ V[j] - ev[j] * V[j]
        assert np.linalg.norm(res) <= 1e-9 * w[0]


def test_error_statuses(gpu):
    """entry points return an error status with a message instead of exiting"""
    with native.Handle(0) as h:
        with pytest.raises(native.GpuError, match="GP_ERR_STATE"):
            h.set_samples(np.arange(4, dtype=np.int32))  # no genotypes loaded
        rec = O.pack(np.ones((10, 8), np.int8))
        h.load_genotypes(rec, 8)
        with pytest.raises(native.GpuError, match="GP_ERR_ARG"):
            h.set_samples(np.array([3, 1], np.int32))  # not ascending
        with pytest.raises(native.GpuError, match="GP_ERR_ARG"):
            h.set_snps(np.array([0, 10], np.int32))  # out of range
        h.set_samples(np.arange(8, dtype=np.int32))
        h.set_snps(np.arange(10, dtype=np.int32))
        with pytest.raises(native.GpuError, match="GP_ERR_STATE"):
            h.snp_weights(2)  # no eigenvectors yet
        with pytest.raises(native.GpuError, match="GP_ERR_STATE"):
            h.lsqproj(2, np.arange(8, dtype=np.int32))
    # every SNP monomorphic: the flow reports no data (the reference's "no data" fatalx)
    mono = O.pack(np.zeros((20, 6), np.int8))
    with native.Handle(0) as h:
        with pytest.raises(native.GpuError):
            native.smartpca_run(h, mono, 6, native.default_opts(numeigs=2, numoutliter=0))


def test_lsqproj_non_pd_and_unobserved_samples(gpu):
    """host-planted failures of lsqproject: sample 7 is observed only at SNPs whose PCA rows
    are all heterozygous, so their values and weights are exactly 0 and its normal matrix is
    0 (not positive definite: status 2, the reference's regressit -1000, coefficients left
    as they were); sample 8 has no genotype (status 1, dropped).  Both as the oracle, and
    through the whole flow (which keeps the previous sample's coefficients for status 2)."""
    rec, pop = native.synth_records(2000, [90, 90], [0.02, 0.04], miss=0.02, seed=81,
                                    nthreads=4)
    nind = len(pop)
    g = O.unpack(rec, nind)
    g[:30, :] = 1
    g[30:, 7] = -1
    g[:, 8] = -1
    rec2 = O.pack(g)
    rows = np.array([k for k in range(nind) if k not in (7, 8)], np.int32)
    cols = np.arange(2000, dtype=np.int32)
    gpu.load_genotypes(rec2, nind)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    gpu.xtx()
    ev, V = gpu.eigvecs(5)
    K = 5
    ff, fx, sc = gpu.snp_weights(K)
    proj = np.arange(nind, dtype=np.int32)
    a, b, nobs, st = gpu.lsqproj(K, proj)
    s = O.pass_columns(rec2, cols, rows)
    off, ofx, osc = O.weights(s, V, K)
    oa, ob, onobs, ost = O.lsqproj(s, off, osc, K, proj)
    assert st[7] == 2 and nobs[7] == 30 and st[8] == 1 and nobs[8] == 0
    assert np.array_equal(st, ost) and np.array_equal(nobs, onobs)
    ok = st == 0
    assert np.max(np.abs(a[:, ok] - oa[:, ok])) <= 1e-11 * max(1.0, np.max(np.abs(oa)))
    # the flow: 7 and 8 outside the PCA (affstatus 0); 8 has no data at all and is ignored
    aff = np.ones(nind, np.uint8)
    aff[[7, 8]] = 0
    opts = native.default_opts(numeigs=K, numoutliter=0)
    r = native.smartpca_run(gpu, rec2, nind, opts, ind_affstatus=aff)
    ref = O.smartpca(rec2, nind, numeigs=K, numoutliter=0, ind_affstatus=aff)
    assert np.array_equal(r["ind_out"], ref["ind_out"]) and not r["ind_out"][8]
    sgn = np.sign(np.sum(r["coords"] * ref["coords"], axis=1))
    assert np.max(np.abs(r["coords"] - ref["coords"] * sgn[:, None])) <= 1e-8
    assert np.array_equal(r["coords"][:, 7], r["coords"][:, 6])  # the previous sample's

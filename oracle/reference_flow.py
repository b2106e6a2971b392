"""ORACLE — test infrastructure only: the reference smartpca flow timed on the host cores.

Used by bench.py's reference arm and its cpu_baseline leg; never imported by the product.
It times the reference's own algorithm for every phase of one smartpca pass on a bounded
SNP sample of a workload:

  filters + normalisation   getcolxz_binary1 / fvadjust_binary (smartpca.c:3219-3301,
                            2282-2313), restated in oracle/smartpca_oracle.c
  Gram                      the partial-sum lookup of domult_increment_lookup
                            (smartpca.c:3361-3495), restated, all host threads
  eigensolve                eigvecs -> eigxv_ -> LAPACK dspev (eigsubs.c:39-55,
                            eigx.c:97-117): the very LAPACK routine the reference calls, from
                            the OpenBLAS that scipy bundles, on the packed lower triangle
  SNP weights, scores       smartpca.c:1485-1525, restated (one thread, as the reference)
  lsqproject                lsqproj / regressit / choldc / cholsl (smartpca.c:4606-4757,
                            regsubs.c:8-72, linsubs.c:296-380), restated (one thread)

The per-SNP phases scale linearly with the number of SNPs; the eigensolve depends on the order
only.  The whole-workload time is therefore (per-SNP phases of the sample) x M / m + the
eigensolve at the workload's order.

The genotypes come from `bn_records`, a numpy Balding-Nichols generator of this module (the
same model and parameters as the workload, not the library's generator, so that nothing of the
product is loaded).
"""
import ctypes as C
import glob
import os
import time

import numpy as np

from oracle import oracle as O


def bn_records(nsnp, pop_sizes, fst, miss, seed, n_admixed=0, p_lo=0.05, p_hi=0.95):
    """packedancestrymap records (nsnp x max(ceil(N/4), 48)) of a Balding-Nichols panel:
    ancestral p ~ U(p_lo, p_hi); population frequency ~ Beta(p(1-F)/F, (1-p)(1-F)/F);
    genotype ~ Binomial(2, frequency); admixed samples draw each allele from one of two
    populations with a U(0,1) mixing fraction; each genotype missing with probability miss"""
    rng = np.random.default_rng(seed)
    npop = len(pop_sizes)
    p = rng.uniform(p_lo, p_hi, size=nsnp)
    f = np.asarray(fst, np.float64)[:, None]
    a = p[None, :] * (1 - f) / f
    b = (1 - p[None, :]) * (1 - f) / f
    pk = rng.beta(a, b)                                    # npop x nsnp
    freq = np.repeat(pk, pop_sizes, axis=0)                # N x nsnp
    if n_admixed:
        ab = rng.integers(0, npop, size=(n_admixed, 2))
        w = rng.uniform(size=(n_admixed, 1))
        mix = w * pk[ab[:, 0]] + (1 - w) * pk[ab[:, 1]]
        freq = np.concatenate([freq, mix])
    g = rng.binomial(2, freq.T).astype(np.int8)            # nsnp x N
    g[rng.random(g.shape) < miss] = -1
    return O.pack(g)


def _openblas():
    import scipy
    d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    libs = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    if not libs:
        raise RuntimeError("scipy's bundled OpenBLAS was not found")
    return C.CDLL(libs[0])


def dspev(X):
    """all eigenpairs of the symmetric X through LAPACK dspev (jobz V, uplo L, packed), as
    eigxv_ calls it: eigenvalues ascending, vector j as row j"""
    n = X.shape[0]
    lib = _openblas()
    f = lib.scipy_dspev_
    ap = np.ascontiguousarray(X.T[np.triu_indices(n)])    # column-major packed lower triangle
    w = np.zeros(n)
    z = np.zeros((n, n))
    work = np.zeros(3 * n)
    info = C.c_int(0)
    f(C.byref(C.c_char(b"V")), C.byref(C.c_char(b"L")), C.byref(C.c_int(n)),
      ap.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p), z.ctypes.data_as(C.c_void_p),
      C.byref(C.c_int(n)), work.ctypes.data_as(C.c_void_p), C.byref(info), C.c_size_t(1),
      C.c_size_t(1))
    if info.value != 0:
        raise RuntimeError("dspev info %d" % info.value)
    return w, z    # Fortran column j of z = row j here


def gram_phases(rec, nind, nthreads):
    """counts, filters and normalisation, then the lookup Gram, over all samples and SNPs of
    the records: (seconds per phase, pass state, Gram)"""
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(rec.shape[0], dtype=np.int32)
    t = {}
    t0 = time.perf_counter()
    s = O.pass_columns(rec, cols, rows)
    t["filter"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    X = O.gram(s, lookup=True, nthreads=nthreads)
    t["gram"] = time.perf_counter() - t0
    return t, s, X


def eig_phase(X):
    """trace scaling (smartpca.c:1230-1236) and dspev of -XTX (eigvecs passes the negated
    matrix so that LAPACK's ascending order is smartpca's descending one): (seconds, top
    eigenvectors as rows)"""
    n = X.shape[0]
    t0 = time.perf_counter()
    Xs = X * ((n - 1) / np.trace(X))
    w, V = dspev(-Xs)
    return time.perf_counter() - t0, V


def projection_phases(s, V, K):
    """SNP weights and scores, then lsqproject of every sample: seconds per phase"""
    t = {}
    t0 = time.perf_counter()
    ff, fx, sc = O.weights(s, V, K)
    t["weights"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.lsqproj(s, ff, sc, K, s.xindex)
    t["lsqproj"] = time.perf_counter() - t0
    return t


def whole_flow_seconds(per_snp_s, nsnp_full, eig_s):
    """the reference's time for one smartpca pass of the whole workload"""
    return per_snp_s * nsnp_full + eig_s

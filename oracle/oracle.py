"""ORACLE — test infrastructure only.

CPU restatement of the reference smartpca hot path (EIGENSOFT 8.0.0), used as the checker
by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg; never imported by the
product.  The O(N*M) loops are in oracle/smartpca_oracle.c (liboracle.so, built by
eig_gb300/build.py); this module composes them the way main() in src/eigensrc/smartpca.c
does, with numpy/LAPACK (dsyevd) standing in for the reference's LAPACK dspev call.

Pinned against the reference binary (oracle/build_ref.sh) through the golden fixtures in
tests/golden/ (generated by tests/golden/make_golden.py) and the reference's own example
outputs (EIGENSTRAT/example.eval, CONVERTF/example.*).
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_bin", "liboracle.so")
_lib = None

i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)
f64p = C.POINTER(C.c_double)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle/_bin/liboracle.so is not built; run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        L.orc_pass_columns.argtypes = [u8p, C.c_int64, i32p, C.c_int32, i32p, C.c_int32, C.c_int,
                                       C.c_int, C.c_int, C.c_int, i32p, i32p, i32p, u8p, f64p,
                                       f64p, f64p]
        L.orc_pass_columns.restype = None
        L.orc_gram_plain.argtypes = [u8p, C.c_int64, i32p, C.c_int32, u8p, f64p, i32p, C.c_int32,
                                     f64p]
        L.orc_gram_plain.restype = None
        L.orc_gram_lookup.argtypes = [u8p, C.c_int64, i32p, C.c_int32, u8p, f64p, i32p, C.c_int32,
                                      C.c_int, f64p]
        L.orc_gram_lookup.restype = None
        L.orc_ridoutlier.argtypes = [f64p, C.c_int32, C.c_int32, C.c_double, C.c_int, i32p, i32p,
                                     f64p]
        L.orc_ridoutlier.restype = C.c_int
        L.orc_weights.argtypes = [u8p, C.c_int64, i32p, C.c_int32, u8p, f64p, f64p, f64p, i32p,
                                  C.c_int32, f64p, C.c_int32, f64p, f64p, f64p]
        L.orc_weights.restype = None
        L.orc_lsqproj.argtypes = [u8p, C.c_int64, i32p, C.c_int32, u8p, f64p, f64p, f64p, f64p,
                                  C.c_int32, i32p, C.c_int32, f64p, f64p, i32p, i32p]
        L.orc_lsqproj.restype = None
        L.orc_popfill_columns.argtypes = [u8p, C.c_int64, i32p, C.c_int32, i32p, C.c_int32, i32p,
                                          C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, i32p,
                                          i32p, i32p, u8p, f64p, f64p, f64p, f64p]
        L.orc_popfill_columns.restype = None
        L.orc_gram_fill.argtypes = [u8p, C.c_int64, i32p, C.c_int32, u8p, f64p, f64p, C.c_int32,
                                    i32p, i32p, C.c_int32, f64p]
        L.orc_gram_fill.restype = None
        L.orc_lsqproj_fill.argtypes = [u8p, C.c_int64, i32p, C.c_int32, u8p, f64p, f64p, f64p,
                                       f64p, C.c_int32, i32p, i32p, C.c_int32, C.c_int32, f64p,
                                       f64p, i32p, i32p]
        L.orc_lsqproj_fill.restype = None
        _lib = L
    return _lib


def unpack(records, nind):
    """Genotype matrix (nsnp x nind) int8 with -1 for missing, from packed records."""
    rec = np.asarray(records, dtype=np.uint8)
    shifts = np.array([6, 4, 2, 0], dtype=np.uint8)
    g = ((rec[:, :, None] >> shifts[None, None, :]) & 3).reshape(rec.shape[0], -1)[:, :nind]
    g = g.astype(np.int8)
    g[g == 3] = -1
    return g


def bed_to_packed(bed_records, nind):
    """PLINK .bed records -> packedancestrymap records (ancval src/mcio.c:3995-4009)."""
    bed = np.asarray(bed_records, dtype=np.uint8)
    x = ((bed[:, :, None] >> np.array([0, 2, 4, 6], np.uint8)[None, None, :]) & 3).reshape(
        bed.shape[0], -1)[:, :nind]
    code = np.array([2, 3, 1, 0], np.uint8)[x]
    return pack(np.where(code == 3, -1, code.astype(np.int8)).astype(np.int8))


def pack(g):
    """Genotype matrix (nsnp x nind, -1 missing) -> packed records (rlen = max(ceil(N/4),48))."""
    g = np.asarray(g)
    nsnp, nind = g.shape
    rlen = max((nind + 3) // 4, 48)
    codes = np.where(g < 0, 3, g).astype(np.uint8)
    pad = np.zeros((nsnp, rlen * 4 - nind), np.uint8)  # the reference writer pads with 0
    c = np.concatenate([codes, pad], axis=1).reshape(nsnp, rlen, 4)
    out = (c[:, :, 0] << 6) | (c[:, :, 1] << 4) | (c[:, :, 2] << 2) | c[:, :, 3]
    return np.ascontiguousarray(out.astype(np.uint8))


class PassState:
    pass


def pass_columns(records, cols, xindex, fancynorm=1, altnormstyle=1, minallelecnt=1,
                 maxmissing=9999999):
    rec = np.ascontiguousarray(records, dtype=np.uint8)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    xi = np.ascontiguousarray(xindex, dtype=np.int32)
    nc = len(cols)
    s = PassState()
    s.n0 = np.zeros(nc, np.int32)
    s.n1 = np.zeros(nc, np.int32)
    s.nmiss = np.zeros(nc, np.int32)
    s.killed = np.zeros(nc, np.uint8)
    s.tab = np.zeros(4 * nc)
    s.xmean = np.zeros(nc)
    s.xfancy = np.zeros(nc)
    lib().orc_pass_columns(_p(rec, C.c_uint8), rec.shape[1], _p(cols, C.c_int32), nc,
                           _p(xi, C.c_int32), len(xi), fancynorm, altnormstyle, minallelecnt,
                           maxmissing, _p(s.n0, C.c_int32), _p(s.n1, C.c_int32),
                           _p(s.nmiss, C.c_int32), _p(s.killed, C.c_uint8), _p(s.tab, C.c_double),
                           _p(s.xmean, C.c_double), _p(s.xfancy, C.c_double))
    s.rec, s.cols, s.xindex = rec, cols, xi
    return s


def popfill_columns(s, rowpop, npop, fancynorm=1, altnormstyle=1, minallelecnt=1,
                    maxmissing=9999999):
    """usepopsformissing on a pass: replaces s's counts, kill flags, xmean and xfancy by
    the filled ones and adds the Gram table s.gtab [4 per column] and the population fill
    values s.gfill [ncols x npop]; s.tab stays the observed-only table the SNP weights use
    (getcolxf)."""
    nc, n = len(s.cols), len(s.xindex)
    s.rowpop = np.ascontiguousarray(rowpop, dtype=np.int32)
    s.npop = int(npop)
    s.gtab = np.zeros(4 * nc)
    s.gfill = np.zeros(nc * max(npop, 1))
    lib().orc_popfill_columns(_p(s.rec, C.c_uint8), s.rec.shape[1], _p(s.cols, C.c_int32), nc,
                              _p(s.xindex, C.c_int32), n, _p(s.rowpop, C.c_int32), npop,
                              fancynorm, altnormstyle, minallelecnt, maxmissing,
                              _p(s.n0, C.c_int32), _p(s.n1, C.c_int32), _p(s.nmiss, C.c_int32),
                              _p(s.killed, C.c_uint8), _p(s.gtab, C.c_double),
                              _p(s.gfill, C.c_double), _p(s.xmean, C.c_double),
                              _p(s.xfancy, C.c_double))
    dead = s.killed == 1
    s.tab.reshape(-1, 4)[dead] = 0.0
    return s


def gram(s, lookup=False, nthreads=1):
    n = len(s.xindex)
    X = np.zeros((n, n))
    if getattr(s, "gfill", None) is not None:
        lib().orc_gram_fill(_p(s.rec, C.c_uint8), s.rec.shape[1], _p(s.cols, C.c_int32),
                            len(s.cols), _p(s.killed, C.c_uint8), _p(s.gtab, C.c_double),
                            _p(s.gfill, C.c_double), s.npop, _p(s.rowpop, C.c_int32),
                            _p(s.xindex, C.c_int32), n, _p(X, C.c_double))
        return X
    args = (_p(s.rec, C.c_uint8), s.rec.shape[1], _p(s.cols, C.c_int32), len(s.cols),
            _p(s.killed, C.c_uint8), _p(s.tab, C.c_double), _p(s.xindex, C.c_int32), n)
    if lookup:
        lib().orc_gram_lookup(*args, nthreads, _p(X, C.c_double))
    else:
        lib().orc_gram_plain(*args, _p(X, C.c_double))
    return X


def eig_scaled(X):
    """trace scale (smartpca.c:1230-1236) + all eigenpairs, descending (eigvecs -> dspev)."""
    n = X.shape[0]
    y = np.trace(X) / (n - 1)
    if np.isnan(y) or y <= 0:
        raise ValueError("XTX has zero trace (perhaps no data)")
    Xs = X * (1.0 / y)
    w, V = np.linalg.eigh(Xs)
    return w[::-1].copy(), np.ascontiguousarray(V[:, ::-1].T)


def ridoutlier(evecs, neigs, thresh=6.0, mode=0):
    E = np.ascontiguousarray(evecs, dtype=np.float64)
    n = E.shape[1]
    bad = np.zeros(n, np.int32)
    vec = np.zeros(n, np.int32)
    sc = np.zeros(n)
    nb = lib().orc_ridoutlier(_p(E, C.c_double), n, neigs, thresh, mode, _p(bad, C.c_int32),
                              _p(vec, C.c_int32), _p(sc, C.c_double))
    return bad[:nb], vec, sc


def weights(s, evecs, K):
    n, nc = len(s.xindex), len(s.cols)
    E = np.ascontiguousarray(evecs[:K], dtype=np.float64)
    ff = np.zeros((K, nc))
    fx = np.zeros((K, n))
    sc = np.zeros(K)
    lib().orc_weights(_p(s.rec, C.c_uint8), s.rec.shape[1], _p(s.cols, C.c_int32), nc,
                      _p(s.killed, C.c_uint8), _p(s.tab, C.c_double), _p(s.xmean, C.c_double),
                      _p(s.xfancy, C.c_double), _p(s.xindex, C.c_int32), n, _p(E, C.c_double), K,
                      _p(ff, C.c_double), _p(fx, C.c_double), _p(sc, C.c_double))
    return ff, fx, sc


def lsqproj(s, ffvecs, fxscal, K, samples):
    smp = np.ascontiguousarray(samples, dtype=np.int32)
    q = len(smp)
    ff = np.ascontiguousarray(ffvecs[:K])
    a = np.zeros((K, q))
    b = np.zeros((K, q))
    nobs = np.zeros(q, np.int32)
    st = np.zeros(q, np.int32)
    lib().orc_lsqproj(_p(s.rec, C.c_uint8), s.rec.shape[1], _p(s.cols, C.c_int32), len(s.cols),
                      _p(s.killed, C.c_uint8), _p(s.xmean, C.c_double), _p(s.xfancy, C.c_double),
                      _p(ff, C.c_double), _p(np.ascontiguousarray(fxscal), C.c_double), K,
                      _p(smp, C.c_int32), q, _p(a, C.c_double), _p(b, C.c_double),
                      _p(nobs, C.c_int32), _p(st, C.c_int32))
    return a, b, nobs, st


def lsqproj_fill(s, ffvecs, fxscal, K, samples, sampop, npop):
    smp = np.ascontiguousarray(samples, dtype=np.int32)
    sp = np.ascontiguousarray(sampop, dtype=np.int32)
    q = len(smp)
    ff = np.ascontiguousarray(ffvecs[:K])
    a = np.zeros((K, q))
    b = np.zeros((K, q))
    nobs = np.zeros(q, np.int32)
    st = np.zeros(q, np.int32)
    lib().orc_lsqproj_fill(_p(s.rec, C.c_uint8), s.rec.shape[1], _p(s.cols, C.c_int32),
                           len(s.cols), _p(s.killed, C.c_uint8), _p(s.xmean, C.c_double),
                           _p(s.xfancy, C.c_double), _p(ff, C.c_double),
                           _p(np.ascontiguousarray(fxscal), C.c_double), K, _p(smp, C.c_int32),
                           _p(sp, C.c_int32), q, npop, _p(a, C.c_double), _p(b, C.c_double),
                           _p(nobs, C.c_int32), _p(st, C.c_int32))
    return a, b, nobs, st


def smartpca(records, nind, numeigs=10, numoutliter=5, numoutleigs=10, outlthresh=6.0,
             outliermode=0, fancynorm=1, altnormstyle=1, minallelecnt=1, maxmissing=9999999,
             lsqproject=1, snp_chrom=None, noxdata=1, numchrom=22, ind_ignore=None,
             ind_affstatus=None, gram_lookup=False, nthreads=1, missingmode=0,
             usepopsformissing=0, ind_pop=None):
    """The hot path of smartpca main() on packed records (sorted SNP order).

    Returns evals (all, descending), evecs (top K over the rows), xindex, the per-sample
    .evec coordinates, the set of printed samples and the outliers (sample, pass, evec, z).
    """
    rec = np.ascontiguousarray(records, dtype=np.uint8)
    nsnp = rec.shape[0]
    g = unpack(rec, nind)
    ind_ign = np.zeros(nind, bool) if ind_ignore is None else np.asarray(ind_ignore, bool).copy()
    aff = np.ones(nind, bool) if ind_affstatus is None else np.asarray(ind_affstatus, bool)
    aff = aff & ~ind_ign
    chrom = np.ones(nsnp, np.int32) if snp_chrom is None else np.asarray(snp_chrom)
    snp_ign = np.zeros(nsnp, np.uint8)
    snp_ign[(bool(noxdata) & (chrom == numchrom + 1)) | (chrom == 0) | (chrom > numchrom + 1)] = 1
    valid = g >= 0
    nodata = valid[:, ~ind_ign & aff].sum(axis=1) <= 1
    snp_ign[(snp_ign == 0) & nodata] = 1
    per_ind = valid[snp_ign == 0].sum(axis=0)
    ind_ign |= per_ind == 0

    if missingmode:
        # setmiss (src/qpsubs.c:462-483) after the pre-filters, then no fancynorm
        # (src/eigensrc/smartpca.c:901-904): genotypes become 1 = observed, 0 = missing
        g = valid.astype(np.int8)
        rec = pack(g)
        valid = np.ones_like(valid)
        fancynorm = 0

    def rows():
        return np.nonzero(~ind_ign & aff)[0].astype(np.int32)

    def columns():
        ok = (snp_ign == 0) & (valid[:, ~ind_ign].sum(axis=1) > 0)
        return np.nonzero(ok)[0].astype(np.int32)

    xindex = rows()
    cols = columns()
    # xtypes (smartpca.c:928-943, :1095-1099, :1505-1508): the population index of row i,
    # written for the current rows of every pass and never cleared (-2 before the first)
    xtypes = np.full(nind, -2, np.int32)
    npop = 0
    if usepopsformissing:
        ind_pop = np.asarray(ind_pop, np.int32)
        npop = int(ind_pop.max()) + 1 if len(ind_pop) else 0
    numoutiter = numoutliter + 1 if numoutliter >= 1 else 1
    mode = outliermode if numoutliter >= 1 else 2
    outliers = []
    for it in range(1, numoutiter + 1):
        if it > 1:
            cols = columns()
        if usepopsformissing:
            xtypes[:len(xindex)] = ind_pop[xindex]
            s = pass_columns(rec, cols, xindex, fancynorm, altnormstyle, minallelecnt,
                             0x7FFFFFFF)
            popfill_columns(s, xtypes[:len(xindex)], npop, fancynorm, altnormstyle,
                            minallelecnt, maxmissing)
        else:
            s = pass_columns(rec, cols, xindex, fancynorm, altnormstyle, minallelecnt,
                             maxmissing)
        snp_ign[cols[s.killed == 1]] = 2
        X = gram(s, lookup=gram_lookup, nthreads=nthreads)
        evals, evecs = eig_scaled(X)
        if it > numoutliter:
            break
        numoutleigs = min(numoutleigs, len(xindex) - 1)
        bad, vec, sc = ridoutlier(evecs, numoutleigs, outlthresh, mode)
        if len(bad) == 0:
            break
        for r in bad:
            outliers.append((int(xindex[r]), it, int(vec[r]), float(sc[r])))
            ind_ign[xindex[r]] = True
        xindex = rows()
    n = len(xindex)
    K = min(numeigs, n, len(cols))
    coords = np.zeros((K, nind))
    out = ~ind_ign
    ff = np.zeros((0, len(cols)))
    if K > 0:
        ff, fx, fxscal = weights(s, evecs, K)
        if lsqproject:
            proj = np.nonzero(~ind_ign)[0].astype(np.int32)
            if usepopsformissing:
                # lsqproj reads xtypes at the sample's index in the .ind file (idnum)
                a, b, nobs, st = lsqproj_fill(s, ff, fxscal, K, proj, xtypes[proj], npop)
            else:
                a, b, nobs, st = lsqproj(s, ff, fxscal, K, proj)
            prev = np.zeros(K)
            for q, k in enumerate(proj):
                if st[q] == 1:
                    ind_ign[k] = True
                    a[:, q] = 0.0
                    b[:, q] = 0.0
                    continue
                if st[q] == 2:
                    a[:, q] = prev
                prev = a[:, q].copy()
            pos = {int(k): q for q, k in enumerate(proj)}
            for j in range(K):
                av = np.array([a[j, pos[k]] if k in pos else 0.0 for k in xindex])
                bv = np.array([b[j, pos[k]] if k in pos else 0.0 for k in xindex])
                scale = np.dot(av, bv) / np.dot(av, av)
                coords[j, proj] = scale * a[j]
        out = ~ind_ign
    return dict(evals=evals, evecs=evecs[:K], xindex=xindex, coords=coords, ind_out=out,
                outliers=outliers, ncols=len(cols), nrows=n, numeigs=K, snp_state=snp_ign,
                xtx=X, nused=int((s.killed == 0).sum()), ffvecs=ff, cols=cols,
                killed=s.killed.copy())


def snpeigs(ffvecs, killed):
    """writesnpeigs (src/eigensrc/smartpca.c:3038-3081): each weight vector scaled to mean
    square 1 over the last pass's columns (sequential sum of squares), and per vector the 10
    columns of largest |weight| among the kept ones (first of equal values first; none when
    there are at most 10 columns).  Returns (scaled weights, [(vector, column, |w|)])."""
    ff = np.array(ffvecs, dtype=np.float64, copy=True)
    K, nc = ff.shape
    for j in range(K):
        y = 0.0
        for v in ff[j]:
            y += v * v
        ff[j] = ff[j] * np.sqrt(nc / y)
    best = []
    for j in range(K):
        sc = np.where(np.asarray(killed) == 1, -99999.0, np.abs(ff[j]))
        for _ in range(10):
            if nc <= 10:
                break
            k = int(np.argmax(sc))  # first index of the maximum
            if sc[k] < 0:
                break
            best.append((j, k, float(sc[k])))
            sc[k] = -1.0
    return ff, best


def grm(X):
    """The GRM dump of the last pass (dumpgrm / dumpgrmbin, src/eigensrc/smartpca.c:3770-3808,
    :3705-3767) from the unscaled Gram X: the PCA scaling XTX *= 1/(trace/(n-1)) (:1230-1236),
    then text values XTX * n/sum(diag) and binary float values XTX / (trace/n), lower
    triangle row by row, with the reference's sequential sums.  Returns (text, binary)."""
    n = X.shape[0]
    tr = 0.0
    for a in range(n):
        tr += X[a, a]
    ys = 1.0 / (tr / (n - 1))
    Xs = X * ys
    ds = 0.0
    for a in range(n):
        ds += Xs[a, a]
    recip = n / ds
    ynorm = ds / n
    il = np.tril_indices(n)
    return Xs[il] * recip, (Xs[il] / ynorm).astype(np.float32)


def grm_text_lines(X, numsnps):
    """dumpgrm text lines "a b numsnps %0.6f" (smartpca.c:3797-3804)"""
    n = X.shape[0]
    txt, _ = grm(X)
    il = np.tril_indices(n)
    return ["%d %d %d %0.6f" % (a + 1, b + 1, numsnps, v) for a, b, v in zip(il[0], il[1], txt)]


def relate(X, evals, evecs, numeigs, relthresh=0.05):
    """The relatedness scan of smartrel (src/eigensrc/smartrel.c:578-618) on the unscaled Gram
    X of the last pass: XTX scaled by 1/(trace/(n-1)) (:547-554), the top numeigs components
    removed one by one (subouter of sqrt(lambda_i) v_i, :581-585, src/nicksrc/vsubs.c:2135),
    then y = R_ab / sqrt(R_aa R_bb) + 1/(n-1) for a < b (:589-600).  Returns the pairs with
    y >= relthresh as (a, b, y), rows of the pass, highest y first (the sort of -y, :606)."""
    n = X.shape[0]
    tr = 0.0
    for a in range(n):
        tr += X[a, a]
    R = X * (1.0 / (tr / (n - 1)))
    for i in range(numeigs):
        w = evecs[i] * np.sqrt(evals[i])
        R -= np.outer(w, w)
    d = np.diag(R).copy()
    ia, ib = np.triu_indices(n, 1)
    y = R[ia, ib] / np.sqrt(d[ia] * d[ib]) + 1.0 / (n - 1)
    keep = y >= relthresh
    ia, ib, y = ia[keep], ib[keep], y[keep]
    order = np.lexsort((ib, ia, -y))
    return [(int(ia[k]), int(ib[k]), float(y[k])) for k in order]


def smartrel(records, nind, numeigs=10, relthresh=0.05, numoutliter=5, numoutleigs=10,
             outlthresh=6.0, minallelecnt=1, fancynorm=1, altnormstyle=1, snp_chrom=None,
             noxdata=1, numchrom=22, ind_ignore=None, ind_affstatus=None):
    """smartrel main() (src/eigensrc/smartrel.c:230-624): the smartpca outlier loop with a SNP
    dropped when min(n0, n1) <= minallelecnt (:477-480) and no missingness limit, then
    relate() on the last pass.  Returns (pairs with sample indices, the smartpca result)."""
    r = smartpca(records, nind, numeigs=numeigs, numoutliter=numoutliter,
                 numoutleigs=numoutleigs, outlthresh=outlthresh, fancynorm=fancynorm,
                 altnormstyle=altnormstyle, minallelecnt=minallelecnt + 1,
                 maxmissing=2 ** 31 - 1, lsqproject=0, snp_chrom=snp_chrom, noxdata=noxdata,
                 numchrom=numchrom, ind_ignore=ind_ignore, ind_affstatus=ind_affstatus)
    K = min(numeigs, r["numeigs"])
    pairs = relate(r["xtx"], r["evals"], r["evecs"], K, relthresh)
    xi = r["xindex"]
    return [(int(xi[a]), int(xi[b]), y) for a, b, y in pairs], r


def set_blocks(chrom, gpos, ignore, blocklen=0.05):
    """setblocks (src/qpsubs.c:1578-1627): (number of blocks, tag per SNP, -1 if ignored)"""
    n, lchrom, xsize, fpos = 0, -1, 0, -1.0e20
    tag = np.full(len(chrom), -1, np.int32)
    for i in range(len(chrom)):
        if ignore[i]:
            continue
        if chrom[i] != lchrom or gpos[i] - fpos >= blocklen:
            if xsize > 0:
                n += 1
            lchrom, fpos, xsize = chrom[i], gpos[i], 0
        tag[i] = n
        xsize += 1
    return n + (1 if xsize > 0 else 0), tag


def _wjack(mean, jmean, jwt):
    """wjackest / wjackestx (src/qpsubs.c:2793-2858), sequential sums"""
    keep = [k for k in range(len(jwt)) if jwt[k] >= 1.0e-6]
    jm = [jmean[k] for k in keep]
    jw = [jwt[k] for k in keep]
    g = len(jw)
    if g <= 1:
        return mean, 0.0
    yn = 0.0
    for w in jw:
        yn += w
    sd = 0.0
    for m in jm:
        sd += -(m + -mean)
    dot = 0.0
    for w, m in zip(jw, jm):
        dot += w * m
    jack = sd + dot / yn
    var = 0.0
    for w, m in zip(jw, jm):
        hh = yn / w
        w1 = hh + -1.0
        xt = (hh * mean - w1 * m) + -jack
        var += (xt * xt) / w1
    return jack, float(np.sqrt(var / g))


def fst(records, nind, xindex, xtypes, numeg, cols, tags, nblocks):
    """dofstnumx (src/qpsubs.c:2488-2720) with fstcolyy (:1205-1345) over the columns cols
    (SNP indices, none killed) and rows xindex with populations xtypes: (fstmean, fstans,
    fstsd, fstnum), each numeg x numeg"""
    g = unpack(np.ascontiguousarray(records)[np.asarray(cols)], nind)[:, np.asarray(xindex)]
    xt = np.asarray(xtypes)
    E = numeg
    cnt = np.zeros((len(cols), E, 2), np.int64)
    obs = g >= 0
    for p in range(E):
        m = (xt == p)[None, :] & obs
        c0 = np.where(m, g, 0).sum(axis=1)
        cnt[:, p, 0] = c0
        cnt[:, p, 1] = 2 * m.sum(axis=1) - c0
    top = np.zeros((nblocks, E, E))
    bot = np.zeros((nblocks, E, E))
    wj = np.zeros(nblocks)
    num = np.zeros((E, E), np.int64)
    for c, s in enumerate(cols):
        b = tags[s]
        if b < 0:
            continue
        wj[b] += 1.0
        for a in range(E):
            ya, yb = float(cnt[c, a, 0]), float(cnt[c, a, 1])
            for bb in range(a + 1, E):
                yaa, ybb = float(cnt[c, bb, 0]), float(cnt[c, bb, 1])
                zz, z = yaa + ybb, ya + yb
                if z < 1.5 or zz < 1.5:
                    continue
                yt = ya + yb
                p1 = ya / yt
                h1 = ya * yb / (yt * (yt - 1.0))
                yt = yaa + ybb
                p2 = yaa / yt
                h2 = yaa * ybb / (yt * (yt - 1.0))
                en = (p1 - p2) * (p1 - p2)
                en -= h1 / z
                en -= h2 / zz
                ed = en + h1
                ed += h2
                num[a, bb] += 1
                top[b, a, bb] += en
                bot[b, a, bb] += ed
    gtop = np.zeros((E, E))
    gbot = np.zeros((E, E))
    for k in range(nblocks):
        gtop += top[k]
        gbot += bot[k]
    djk = (gtop[None] - top) / ((gbot[None] - bot) + 1.0e-10)
    fmean = gtop / (gbot + 1.0e-10)
    fans = np.zeros((E, E))
    fsd = np.zeros((E, E))
    fnum = np.zeros((E, E), np.int64)
    for i in range(E):
        for j in range(i + 1, E):
            est, sig = fmean[i, j], 0.0
            if nblocks > 1:
                est, sig = _wjack(fmean[i, j], djk[:, i, j], wj)
            fans[i, j] = fans[j, i] = est
            fsd[i, j] = fsd[j, i] = sig
            fnum[i, j] = fnum[j, i] = num[i, j]
    return fmean, fans, fsd, fnum


def fastpca(records, cols, xindex, K, L, I, omega, fancynorm=1, altnormstyle=1):
    """kjg_fpca (src/ksrc/kjg_fpca.c:24-102) on the setgval table (src/gval.c:31-87), in numpy
    FP64 with the caller's Omega (nrows x L): returns evals [K] = S^2/M and evecs [K][nrows]."""
    rec = np.ascontiguousarray(records, dtype=np.uint8)
    s = pass_columns(rec, cols, xindex, fancynorm, altnormstyle, 0, 2 ** 31 - 1)
    g = unpack(rec[np.asarray(cols)], rec.shape[1] * 4)[:, np.asarray(xindex)]
    code = np.where(g < 0, 3, g)
    tab = s.tab.reshape(-1, 4)
    X = np.take_along_axis(tab, code, axis=1) / np.sqrt(2.0)  # m x n
    m = X.shape[0]
    G = np.asarray(omega, dtype=np.float64)
    blocks = []
    for _ in range(I):
        Qi = X @ G
        blocks.append(Qi)
        G = X.T @ Qi / m
    blocks.append(X @ G)
    U, _, _ = np.linalg.svd(np.hstack(blocks), full_matrices=False)
    B = X.T @ U
    Ub, Sb, _ = np.linalg.svd(B, full_matrices=False)
    return Sb[:K] ** 2 / m, np.ascontiguousarray(Ub[:, :K].T)


class GslMt19937:
    """GSL's default generator as kjg_gsl_rng_init sets it up (src/ksrc/kjg_gsl.c:100-110):
    MT19937 (Matsumoto & Nishimura 1998) with its 2002 initialisation, the seed 0 mapped to
    GSL's default 4357; uniform_pos = the next 32-bit output / 2^32, zero skipped."""

    def __init__(self, seed):
        s = int(seed) & 0xFFFFFFFFFFFFFFFF
        if s == 0:
            s = 4357
        mt = [s & 0xFFFFFFFF]
        for i in range(1, 624):
            mt.append((1812433253 * (mt[-1] ^ (mt[-1] >> 30)) + i) & 0xFFFFFFFF)
        self.mt, self.i = mt, 624

    def _twist(self):
        mt = self.mt
        for k in range(624):
            y = (mt[k] & 0x80000000) | (mt[(k + 1) % 624] & 0x7FFFFFFF)
            mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
        self.i = 0

    def next32(self):
        if self.i >= 624:
            self._twist()
        y = self.mt[self.i]
        self.i += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF

    def uniform_pos(self):
        while True:
            x = self.next32() / 4294967296.0
            if x != 0.0:
                return x


def gsl_omega(seed, nrows, L):
    """kjg_gsl_ran_ugaussian_matrix (src/ksrc/kjg_gsl.c:144-190) on a fresh generator: polar
    Box-Muller pairs along each row, the last column of an odd L holding one uniform draw"""
    r = GslMt19937(seed)
    om = np.zeros((nrows, L))
    for i in range(nrows):
        j = 0
        while j + 1 < L:
            while True:
                x = -1.0 + 2.0 * r.uniform_pos()
                y = -1.0 + 2.0 * r.uniform_pos()
                r2 = x * x + y * y
                if not (r2 > 1.0 or r2 == 0.0):
                    break
            f = np.sqrt(-2.0 * np.log(r2) / r2)
            om[i, j], om[i, j + 1] = x * f, y * f
            j += 2
        if L % 2:
            om[i, L - 1] = r.uniform_pos()
    return om


def kurtosis(a):
    """kurtosis (src/admutils.c:995-1017): mean fourth power of the standardised values,
    sums in index order"""
    a = np.asarray(a, dtype=np.float64)
    n = len(a)
    y1 = 0.0
    for v in a:
        y1 += v
    y1 = y1 / n
    w = a + (-y1)
    y2 = 0.0
    for v in w:
        y2 += v * v
    y2 = y2 / n
    w = w * (1.0 / np.sqrt(y2))
    w = w * w
    y4 = 0.0
    for v in w:
        y4 += v * v
    return y4 / n



# ---------------------------------------------------------------------------------------
# Tracy-Widom statistics of the log (src/eigensrc/smartpca.c:1306-1367): the statistic and
# effective number of markers of dotwcalc (src/nicksrc/statsubs.c:1680-1725) with twnorm
# (:1658-1677), and the TW1 right tail read as gettw does (:1811-1905: cubic Hermite between
# the points -8.0, -7.9, ..., 8.0 of a tail/density table; 1 below it; from 8 on the
# Margetis-Edelman density, which the reference returns there).  The table is computed here
# with scipy's Airy function and numpy determinants: F1(s) = det(I - K_s) on L2(0, inf),
# K_s(x, y) = Ai(x + y + s) (Ferrari & Spohn 2005), Gauss-Legendre Nystrom discretisation
# (Bornemann 2010), density F1 * d/ds log det from Jacobi's formula.

_TW = None


def tw1(s, m=80):
    """(right tail, density) of TW1 at s"""
    from scipy.special import airy
    L = 16.0 - s if s < 16.0 else 4.0
    z, w = np.polynomial.legendre.leggauss(m)
    x = 0.5 * L * (z + 1.0)
    w = 0.5 * L * w
    sw = np.sqrt(w)
    arg = x[:, None] + x[None, :] + s
    ai, aip, _, _ = airy(arg)
    K = sw[:, None] * ai * sw[None, :]
    Kp = sw[:, None] * aip * sw[None, :]
    if s >= 3.0:
        # log det(I - K) = -sum tr(K^n)/n where K is small (keeps a small tail's accuracy)
        ev = np.linalg.eigvalsh((K + K.T) * 0.5)
        logdet = float(np.sum(np.log1p(-ev)))
    else:
        sign, logdet = np.linalg.slogdet(np.eye(m) - K)
    dlog = -float(np.trace(np.linalg.solve(np.eye(m) - K, Kp)))
    F = np.exp(logdet)
    return float(-np.expm1(logdet)), float(F * dlog)


def _tw_table():
    global _TW
    if _TW is None:
        xs = np.round(np.arange(161) * 0.1 - 8.0, 1)
        vals = np.array([tw1(float(x)) for x in xs])
        _TW = (xs, vals[:, 0], vals[:, 1])
    return _TW


def _first_above(tab, lo, hi, val):
    """statsubs.c fgtx: the bisection for the first table entry above val"""
    if val >= tab[hi]:
        return hi + 1
    if val < tab[lo]:
        return lo
    k = (lo + hi) // 2
    if val <= tab[k]:
        return _first_above(tab, lo + 1, k, val)
    return _first_above(tab, k, hi - 1, val)


def tw_tail(x):
    xs, tail, dens = _tw_table()
    n = len(xs)
    k = _first_above(xs, 0, n - 1, x)
    if k <= 0:
        return 1.0
    if k >= n:
        if x <= 0.0:
            return 0.0
        return float(np.exp(-0.25 * np.log(x) - 2.0 * x ** 1.5 / 3.0 - np.log(4.0 * np.sqrt(np.pi))))
    x0, x1 = xs[k - 1], xs[k]
    inc = x1 - x0
    y = (x - x0) / inc
    a0, a1 = tail[k - 1], -dens[k - 1] * inc
    cc0, cc1 = tail[k] - (a0 + a1), -dens[k] * inc - a1
    a2, a3 = 3 * cc0 - cc1, cc1 - 2 * cc0
    return float(((a3 * y + a2) * y + a1) * y + a0)


def _twnorm(lam, p, n):
    if n < 0 or p < 0:
        return -10.0
    if n < p:
        return _twnorm(lam, n, p)
    y1 = np.sqrt(n - 1.0) + np.sqrt(p)
    mu = y1 * y1
    phi = y1 * (1.0 / np.sqrt(n - 1.0) + 1.0 / np.sqrt(p)) ** (1.0 / 3.0)
    return (lam - mu) / phi


def twstats(lam, nostatslim=10):
    """per positive eigenvalue (descending, > 1e-6): (twstat, p-value, effective n), None
    where the reference prints NA"""
    lam = np.asarray(lam, dtype=np.float64)
    m = int(np.sum(lam > 1e-6))
    out = []
    for i in range(m):
        t = lam[i:m]
        if len(t) < nostatslim or t.sum() <= 0.0:
            out.append(None)
            continue
        y = len(t) / float(sum(t))
        e = t * y
        zn = len(t) * (len(t) + 2) / (float(sum(e * e)) - len(t))
        tw = _twnorm(e[0] * zn, float(len(t)), zn)
        out.append((tw, tw_tail(tw), zn))
    return out


def mpstats(lam):
    """the mpstats line (mpestimate smartpca.c:4532-4560): quartiles 0.25, 0.5, 0.75 of the
    positive eigenvalues and (q3 - q1) / q2, or None for fewer than 10"""
    lam = np.asarray(lam, dtype=np.float64)
    t = np.sort(lam[lam > 1e-6])
    n = len(t)
    if n < 10:
        return None
    q = [float(np.interp(f * (n - 1), np.arange(n), t)) for f in (0.25, 0.5, 0.75)]
    return q + [(q[2] - q[0]) / q[1]]


def tw_lines(lam, nrows, ncols, nostatslim=10):
    """the log's mpstats line and Tracy-Widom section as text"""
    lam = np.asarray(lam, dtype=np.float64)
    m = int(np.sum(lam > 1e-6))
    lines = []
    mp = mpstats(lam)
    if mp is not None:
        lines.append("mpstats: %9.3f%9.3f%9.3f%12.6f" % tuple(mp))
    lines.append("")
    lines.append("## Tracy-Widom statistics: rows: %d  cols: %d" % (nrows, ncols))
    lines.append("%4s  %12s%12s %9s %12s %9s" % ("#N", "eigenvalue", "difference", "twstat",
                                                 "p-value", "effect. n"))
    st = twstats(lam, nostatslim)
    for i in range(m):
        s = "%4d  %12.6f" % (i + 1, lam[i])
        s += "%12s" % "NA" if i == 0 else "%12.6f" % (lam[i] - lam[i - 1])
        if st[i] is None:
            s += " %9s %12s %9s" % ("NA", "NA", "NA")
        else:
            s += " %9.3f %12.6g %9.3f" % st[i]
        lines.append(s)
    return lines

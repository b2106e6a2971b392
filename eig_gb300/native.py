"""ctypes binding of the gpupca C ABI (include/gpupca.h, include/gpupca_run.h).

This is the Python-side caller of the same entry points the drop-in CLI uses.  Loading
fails loudly when the CUDA library has not been built: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libgpupca.so")
SYNTH_PATH = os.path.join(LIB_DIR, "libgpsynth.so")

GP_OK = 0
GP_ERR = {-1: "GP_ERR_ARG", -2: "GP_ERR_CUDA", -3: "GP_ERR_NOMEM", -4: "GP_ERR_STATE",
          -5: "GP_ERR_SOLVER", -6: "GP_ERR_NODATA", -7: "GP_ERR_TIMEOUT", -8: "GP_ERR_FULL",
          -9: "GP_ERR_NOTBUILT"}
GP_ERR_TIMEOUT = -7
GP_CODE_PACKED, GP_CODE_BED = 0, 1
GP_OUT_PACKEDANCESTRYMAP, GP_OUT_PACKEDPED, GP_OUT_EIGENSTRAT = 0, 1, 2
GP_PREC_FP64, GP_PREC_SPLIT_BF16, GP_PREC_SPLIT_BF16X4, GP_PREC_SPLIT_FP16 = 0, 1, 2, 3
PRECISIONS = {"fp64": 0, "bf16": 1, "bf16x4": 2, "fp16": 3}
PHASES = ["load", "filter", "gram", "eig", "outlier", "weights", "lsqproj", "total"]

# every symbol the headers declare (checked by the CPU test suite)
EXPORTED = ["gp_version", "gp_last_error", "gp_open", "gp_close", "gp_device_bytes",
            "gp_load_genotypes", "gp_set_missing", "gp_set_missingmode", "gp_valid_counts",
            "gp_set_samples",
            "gp_set_snps", "gp_xtx", "gp_eigvecs", "gp_ridoutlier", "gp_snp_weights",
            "gp_lsqproj", "gp_fastpca", "gp_smartpca_defaults", "gp_smartpca_run",
            "gp_fail_msg", "gp_genotype_shape", "gp_timer_start", "gp_timer_stop",
            "gp_last_gram_time", "gp_last_tridiag_time", "gp_last_counts_time",
            "gp_host_register",
            "gp_host_unregister",
            "gp_transfer_bytes", "gp_launch_count", "gp_gram_fp64_noalloc",
            "gp_noalloc_last_error", "gp_serve_open", "gp_serve_layout",
            "gp_serve_panel_snps", "gp_serve_submit", "gp_serve_test", "gp_serve_wait",
            "gp_serve_stats", "gp_serve_last_error", "gp_serve_close", "gp_serve_pause",
            "gp_serve_submit_pca", "gp_serve_pca_stats", "gp_smartpca_footprint", "gp_release",
            "gp_keep_gram", "gp_relate", "gp_record_bytes", "gp_encode_records",
            "gp_last_encode_time", "gp_fst", "gp_set_blocks", "gp_set_row_pops",
            "gp_lsqproj_pops", "gp_serve_loop_stats", "gp_twstats", "gp_tw_tail",
            "gp_mpstats"]

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
u8p = C.POINTER(C.c_uint8)
f64p = C.POINTER(C.c_double)
vp = C.c_void_p


class XtxOpts(C.Structure):
    _fields_ = [("fancynorm", C.c_int32), ("altnormstyle", C.c_int32),
                ("minallelecnt", C.c_int32), ("maxmissing", C.c_int32),
                ("precision", C.c_int32)]


class SmartpcaOpts(C.Structure):
    _fields_ = [("numeigs", C.c_int32), ("numoutliter", C.c_int32), ("numoutleigs", C.c_int32),
                ("outlthresh", C.c_double), ("outliermode", C.c_int32),
                ("fancynorm", C.c_int32), ("altnormstyle", C.c_int32),
                ("minallelecnt", C.c_int32), ("maxmissing", C.c_int32),
                ("lsqproject", C.c_int32), ("noxdata", C.c_int32), ("numchrom", C.c_int32),
                ("precision", C.c_int32), ("fastmode", C.c_int32), ("fastdim", C.c_int32),
                ("fastiter", C.c_int32), ("seed", C.c_int64), ("missingmode", C.c_int32),
                ("usepopsformissing", C.c_int32)]


class Panel(C.Structure):
    _fields_ = [("records", u8p), ("record_bytes", C.c_int64), ("nsnp", C.c_int64),
                ("nind", C.c_int32), ("code", C.c_int32), ("snp_chrom", i32p),
                ("snp_ignore", u8p), ("ind_ignore", u8p), ("ind_affstatus", u8p),
                ("ind_male", u8p), ("ind_pop", i32p)]


class ServeOpts(C.Structure):
    _fields_ = [("numeigs", C.c_int32), ("max_batch", C.c_int32), ("pool_samples", C.c_int64),
                ("fp64_serial", C.c_int32), ("eigscale", f64p), ("pca_workers", C.c_int32),
                ("pca_budget_bytes", C.c_int64), ("host_loop", C.c_int32)]


class RunResult(C.Structure):
    _fields_ = [("xindex", i32p), ("evals", f64p), ("evecs", f64p), ("coords", f64p),
                ("ind_out", u8p), ("snp_state", u8p), ("outlier_idx", i32p),
                ("outlier_iter", i32p), ("outlier_vec", i32p), ("outlier_score", f64p),
                ("nrows", C.c_int32), ("ncols", C.c_int32), ("numeigs", C.c_int32),
                ("noutliers", C.c_int32), ("npasses", C.c_int32),
                ("t_phase", C.c_double * 8), ("gram_flops", C.c_double),
                ("gram_ms", C.c_double), ("xtx", f64p), ("nused", C.c_int32),
                ("ffvecs", f64p), ("snp_lastpass", u8p), ("pass_stats", i32p),
                ("pass_kills", i32p), ("nodata", C.c_int32), ("nrows0", C.c_int32),
                ("ncols0", C.c_int32)]


_lib = None
_synth = None


def load_library():
    """Load libgpupca.so (raises if it is missing: the CUDA path is mandatory)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libgpupca.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    sig = {
        "gp_version": (C.c_int, []),
        "gp_last_error": (C.c_char_p, [vp]),
        "gp_open": (C.c_int, [C.c_int, C.POINTER(vp)]),
        "gp_close": (None, [vp]),
        "gp_device_bytes": (C.c_int, [vp, i64p]),
        "gp_load_genotypes": (C.c_int, [vp, u8p, C.c_int64, C.c_int64, C.c_int32, C.c_int32]),
        "gp_set_missing": (C.c_int, [vp, i64p, C.c_int64]),
        "gp_set_missingmode": (C.c_int, [vp]),
        "gp_valid_counts": (C.c_int, [vp, u8p, u8p, i32p, i32p]),
        "gp_set_samples": (C.c_int, [vp, i32p, C.c_int32]),
        "gp_set_snps": (C.c_int, [vp, i32p, C.c_int32]),
        "gp_xtx": (C.c_int, [vp, C.POINTER(XtxOpts), i32p, i32p, i32p, u8p, f64p, f64p, f64p,
                             f64p, i32p]),
        "gp_eigvecs": (C.c_int, [vp, C.c_int32, f64p, f64p]),
        "gp_ridoutlier": (C.c_int, [f64p, C.c_int32, C.c_int32, C.c_double, C.c_int32, i32p,
                                    i32p, f64p]),
        "gp_snp_weights": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p]),
        "gp_lsqproj": (C.c_int, [vp, C.c_int32, i32p, C.c_int32, f64p, f64p, i32p, i32p]),
        "gp_set_row_pops": (C.c_int, [vp, i32p, C.c_int32]),
        "gp_lsqproj_pops": (C.c_int, [vp, C.c_int32, i32p, i32p, C.c_int32, C.c_int32, f64p,
                                      f64p, i32p, i32p]),
        "gp_fastpca": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, f64p,
                                 C.POINTER(XtxOpts), f64p, f64p]),
        "gp_smartpca_defaults": (None, [C.POINTER(SmartpcaOpts)]),
        "gp_genotype_shape": (C.c_int, [vp, i64p, i32p]),
        "gp_timer_start": (C.c_int, [vp]),
        "gp_timer_stop": (C.c_int, [vp, f64p]),
        "gp_last_gram_time": (C.c_int, [vp, f64p, i32p, f64p]),
        "gp_last_tridiag_time": (C.c_int, [vp, f64p, i32p]),
        "gp_last_counts_time": (C.c_int, [vp, f64p, i64p]),
        "gp_host_register": (C.c_int, [vp, C.c_size_t]),
        "gp_host_unregister": (C.c_int, [vp]),
        "gp_transfer_bytes": (C.c_int, [vp, i64p, i64p, C.c_int32]),
        "gp_launch_count": (C.c_int, [vp, i64p, C.c_int32]),
        "gp_gram_fp64_noalloc": (C.c_int, [vp, C.c_int64, C.c_int32, C.c_int32, vp, vp, vp]),
        "gp_noalloc_last_error": (C.c_char_p, []),
        "gp_serve_open": (C.c_int, [vp, C.POINTER(ServeOpts), C.POINTER(vp)]),
        "gp_serve_layout": (C.c_int, [vp, i64p, i64p]),
        "gp_serve_panel_snps": (C.c_int, [vp, i32p]),
        "gp_serve_submit": (C.c_int, [vp, u8p, C.c_int32, f64p, i32p, i64p]),
        "gp_serve_test": (C.c_int, [vp, C.c_int64]),
        "gp_serve_wait": (C.c_int, [vp, C.c_int64, C.c_double]),
        "gp_serve_stats": (C.c_int, [vp, i64p, i64p, i64p]),
        "gp_serve_pause": (C.c_int, [vp, C.c_int32]),
        "gp_serve_submit_pca": (C.c_int, [vp, C.POINTER(Panel), C.POINTER(SmartpcaOpts),
                                          C.POINTER(RunResult), i64p]),
        "gp_serve_pca_stats": (C.c_int, [vp, i64p, i32p, i64p]),
        "gp_serve_loop_stats": (C.c_int, [vp, i32p, i64p, i64p, i64p]),
        "gp_twstats": (C.c_int, [f64p, C.c_int32, C.c_int32, C.c_double, C.c_int32, f64p, f64p,
                                 f64p]),
        "gp_tw_tail": (C.c_double, [C.c_double]),
        "gp_mpstats": (C.c_int, [f64p, C.c_int32, f64p]),
        "gp_smartpca_footprint": (C.c_int64, [C.c_int32, C.c_int64, C.c_int32, C.c_int32]),
        "gp_release": (C.c_int, [vp]),
        "gp_keep_gram": (C.c_int, [vp, C.c_int32]),
        "gp_relate": (C.c_int, [vp, C.c_int32, C.c_double, C.c_int64, i32p, i32p, f64p, i64p]),
        "gp_record_bytes": (C.c_int64, [C.c_int32, C.c_int32]),
        "gp_last_encode_time": (C.c_int, [vp, f64p]),
        "gp_fst": (C.c_int, [vp, i32p, C.c_int32, i32p, C.c_int32, f64p, f64p, f64p, i32p]),
        "gp_set_blocks": (C.c_int32, [i32p, f64p, u8p, C.c_int64, C.c_double, i32p]),
        "gp_encode_records": (C.c_int, [vp, C.c_int32, i32p, C.c_int32, i64p, u8p, C.c_int64,
                                        vp, C.c_int32]),
        "gp_serve_last_error": (C.c_char_p, [vp]),
        "gp_serve_close": (None, [vp]),
        "gp_smartpca_run": (C.c_int, [vp, C.POINTER(SmartpcaOpts), C.POINTER(Panel),
                                      C.POINTER(RunResult)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def load_synth():
    global _synth
    if _synth is not None:
        return _synth
    if not os.path.exists(SYNTH_PATH):
        raise RuntimeError("libgpsynth.so is not built; run __graft_entry__.build()")
    s = C.CDLL(SYNTH_PATH)
    s.gp_packed_rlen.restype = C.c_int64
    s.gp_packed_rlen.argtypes = [C.c_int32]
    s.gp_synth_records.restype = C.c_int
    s.gp_synth_records.argtypes = [vp, u8p, C.c_int64, i32p, C.c_int]
    s.gp_synth_write_dataset.restype = C.c_int
    s.gp_synth_write_dataset.argtypes = [vp, C.c_char_p, C.c_int]
    s.gp_synth_sample_rows.restype = C.c_int
    s.gp_synth_sample_rows.argtypes = [vp, C.c_uint64, i64p, C.c_int64, C.c_int64, u8p, i32p,
                                       C.c_int]
    s.gp_hash_string.restype = C.c_int32
    s.gp_hash_string.argtypes = [C.c_char_p]
    _synth = s
    return s


def ptr(a, ctype):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


class GpuError(RuntimeError):
    pass


class Handle:
    """One gpupca handle (its own CUDA stream) on device `device`."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = vp()
        rc = self.lib.gp_open(device, C.byref(h))
        if rc != GP_OK:
            raise GpuError("gp_open: %s (%s)" % (GP_ERR.get(rc, rc),
                                                 self.lib.gp_last_error(None).decode()))
        self.h = h

    def check(self, rc, what):
        if rc < 0:
            msg = self.lib.gp_last_error(self.h).decode(errors="replace")
            raise GpuError("%s: %s: %s" % (what, GP_ERR.get(rc, rc), msg))
        return rc

    def close(self):
        if self.h:
            self.lib.gp_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- entry points -----------------------------------------------------------------
    def load_genotypes(self, records, nind, code=GP_CODE_PACKED):
        records = np.ascontiguousarray(records, dtype=np.uint8)
        nsnp, rb = records.shape
        self.check(self.lib.gp_load_genotypes(self.h, ptr(records, C.c_uint8), rb, nsnp, nind,
                                              code), "gp_load_genotypes")
        self.nind, self.nsnp = nind, nsnp

    def set_missing(self, pairs):
        pairs = np.ascontiguousarray(pairs, dtype=np.int64).reshape(-1, 2)
        self.check(self.lib.gp_set_missing(self.h, ptr(pairs, C.c_int64), len(pairs)),
                   "gp_set_missing")

    def set_missingmode(self):
        """missingmode: genotypes become observed (1) / missing (0) indicators (setmiss)"""
        self.check(self.lib.gp_set_missingmode(self.h), "gp_set_missingmode")

    def valid_counts(self, sample_use=None, snp_use=None):
        su = None if sample_use is None else np.ascontiguousarray(sample_use, dtype=np.uint8)
        pu = None if snp_use is None else np.ascontiguousarray(snp_use, dtype=np.uint8)
        sv = np.zeros(self.nsnp, np.int32)
        iv = np.zeros(self.nind, np.int32)
        self.check(self.lib.gp_valid_counts(self.h, ptr(su, C.c_uint8), ptr(pu, C.c_uint8),
                                            ptr(sv, C.c_int32), ptr(iv, C.c_int32)),
                   "gp_valid_counts")
        return sv, iv

    def set_samples(self, xindex):
        x = np.ascontiguousarray(xindex, dtype=np.int32)
        self.check(self.lib.gp_set_samples(self.h, ptr(x, C.c_int32), len(x)), "gp_set_samples")
        self.nrows = len(x)

    def set_snps(self, cols):
        c = np.ascontiguousarray(cols, dtype=np.int32)
        self.check(self.lib.gp_set_snps(self.h, ptr(c, C.c_int32), len(c)), "gp_set_snps")
        self.ncols = len(c)

    def xtx(self, precision=GP_PREC_FP64, fancynorm=1, altnormstyle=1, minallelecnt=1,
            maxmissing=9999999, want_xtx=True):
        o = XtxOpts(fancynorm, altnormstyle, minallelecnt, maxmissing, precision)
        nc, n = self.ncols, self.nrows
        n0 = np.zeros(nc, np.int32)
        n1 = np.zeros(nc, np.int32)
        nm = np.zeros(nc, np.int32)
        kl = np.zeros(nc, np.uint8)
        xm = np.zeros(nc)
        xf = np.zeros(nc)
        X = np.zeros((n, n)) if want_xtx else None
        tr = C.c_double()
        nu = C.c_int32()
        self.check(self.lib.gp_xtx(self.h, C.byref(o), ptr(n0, C.c_int32), ptr(n1, C.c_int32),
                                   ptr(nm, C.c_int32), ptr(kl, C.c_uint8), ptr(xm, C.c_double),
                                   ptr(xf, C.c_double), ptr(X, C.c_double), C.byref(tr),
                                   C.byref(nu)), "gp_xtx")
        return dict(n0=n0, n1=n1, nmiss=nm, killed=kl, xmean=xm, xfancy=xf, XTX=X,
                    trace=tr.value, nused=nu.value)

    def eigvecs(self, nvec):
        n = self.nrows
        ev = np.zeros(n)
        V = np.zeros((nvec, n))
        self.check(self.lib.gp_eigvecs(self.h, nvec, ptr(ev, C.c_double), ptr(V, C.c_double)),
                   "gp_eigvecs")
        return ev, V

    def snp_weights(self, numeigs):
        ff = np.zeros((numeigs, self.ncols))
        fx = np.zeros((numeigs, self.nrows))
        sc = np.zeros(numeigs)
        self.check(self.lib.gp_snp_weights(self.h, numeigs, ptr(ff, C.c_double),
                                           ptr(fx, C.c_double), ptr(sc, C.c_double)),
                   "gp_snp_weights")
        return ff, fx, sc

    def set_row_pops(self, row_pop, npop):
        """usepopsformissing: the current rows' population indices (< 0: none)"""
        rp = None if row_pop is None else np.ascontiguousarray(row_pop, dtype=np.int32)
        self.check(self.lib.gp_set_row_pops(self.h, ptr(rp, C.c_int32), int(npop)),
                   "gp_set_row_pops")

    def lsqproj(self, numeigs, samples, sample_pop=None, npop=0):
        """lsqproject; with sample_pop (and npop) the usepopsformissing fill"""
        s = np.ascontiguousarray(samples, dtype=np.int32)
        q = len(s)
        a = np.zeros((numeigs, q))
        b = np.zeros((numeigs, q))
        nobs = np.zeros(q, np.int32)
        st = np.zeros(q, np.int32)
        if sample_pop is None:
            self.check(self.lib.gp_lsqproj(self.h, numeigs, ptr(s, C.c_int32), q,
                                           ptr(a, C.c_double), ptr(b, C.c_double),
                                           ptr(nobs, C.c_int32), ptr(st, C.c_int32)),
                       "gp_lsqproj")
        else:
            sp = np.ascontiguousarray(sample_pop, dtype=np.int32)
            self.check(self.lib.gp_lsqproj_pops(self.h, numeigs, ptr(s, C.c_int32),
                                                ptr(sp, C.c_int32), int(npop), q,
                                                ptr(a, C.c_double), ptr(b, C.c_double),
                                                ptr(nobs, C.c_int32), ptr(st, C.c_int32)),
                       "gp_lsqproj_pops")
        return a, b, nobs, st

    def timer_start(self):
        self.check(self.lib.gp_timer_start(self.h), "gp_timer_start")

    def timer_stop(self):
        ms = C.c_double()
        self.check(self.lib.gp_timer_stop(self.h, C.byref(ms)), "gp_timer_stop")
        return ms.value

    def transfer_bytes(self, reset=False):
        a, b = C.c_int64(), C.c_int64()
        self.check(self.lib.gp_transfer_bytes(self.h, C.byref(a), C.byref(b), int(reset)),
                   "gp_transfer_bytes")
        return a.value, b.value

    def launch_count(self, reset=False):
        a = C.c_int64()
        self.check(self.lib.gp_launch_count(self.h, C.byref(a), int(reset)), "gp_launch_count")
        return a.value

    def last_gram_time(self):
        ms, n, fl = C.c_double(), C.c_int32(), C.c_double()
        self.check(self.lib.gp_last_gram_time(self.h, C.byref(ms), C.byref(n), C.byref(fl)),
                   "gp_last_gram_time")
        return ms.value, n.value, fl.value

    def last_tridiag_time(self):
        """(ms, n) of the last eigensolve's tridiagonalisation kernel (0 ms: cuSOLVER ran)"""
        ms, n = C.c_double(), C.c_int32()
        self.check(self.lib.gp_last_tridiag_time(self.h, C.byref(ms), C.byref(n)),
                   "gp_last_tridiag_time")
        return ms.value, n.value

    def last_counts_time(self):
        """(ms, algorithmic bytes) of the last pass's per-SNP counts kernel"""
        ms, b = C.c_double(), C.c_int64()
        self.check(self.lib.gp_last_counts_time(self.h, C.byref(ms), C.byref(b)),
                   "gp_last_counts_time")
        return ms.value, b.value

    def encode_records(self, fmt, snps, samples=None, flip=None, nsamples=None, out=None):
        """convertf's genotype records (gp_encode_records) of the resident panel: SNP list,
        ordered sample list (None: the first nsamples samples), per-SNP flips.  Returns a
        uint8 array [len(snps)][record bytes]; out may be a device pointer (int) instead."""
        snp = np.ascontiguousarray(snps, dtype=np.int64)
        smp = None if samples is None else np.ascontiguousarray(samples, dtype=np.int32)
        n = len(smp) if smp is not None else int(nsamples)
        fl = None if flip is None else np.ascontiguousarray(flip, dtype=np.uint8)
        rb = self.lib.gp_record_bytes(fmt, n)
        if out is None:
            buf = np.zeros((len(snp), max(rb, 0)), np.uint8)
            self.check(self.lib.gp_encode_records(self.h, fmt, ptr(smp, C.c_int32), n,
                                                  ptr(snp, C.c_int64), ptr(fl, C.c_uint8),
                                                  len(snp), buf.ctypes.data, 0),
                       "gp_encode_records")
            return buf
        self.check(self.lib.gp_encode_records(self.h, fmt, ptr(smp, C.c_int32), n,
                                              ptr(snp, C.c_int64), ptr(fl, C.c_uint8), len(snp),
                                              out, 1), "gp_encode_records")
        return None

    def last_encode_time(self):
        ms = C.c_double()
        self.check(self.lib.gp_last_encode_time(self.h, C.byref(ms)), "gp_last_encode_time")
        return ms.value

    def fst(self, xtypes, numeg, snp_block, nblocks):
        """Fst of the last pass (gp_fst): (fstmean, fstans, fstsd, fstnum) [numeg, numeg]"""
        xt = np.ascontiguousarray(xtypes, dtype=np.int32)
        sb = np.ascontiguousarray(snp_block, dtype=np.int32)
        out = [np.zeros((numeg, numeg)) for _ in range(3)] + [np.zeros((numeg, numeg), np.int32)]
        self.check(self.lib.gp_fst(self.h, ptr(xt, C.c_int32), numeg, ptr(sb, C.c_int32),
                                   nblocks, *[ptr(a, C.c_double) for a in out[:3]],
                                   ptr(out[3], C.c_int32)), "gp_fst")
        return tuple(out)

    def keep_gram(self, keep=True):
        """keep a copy of the next eigensolve's scaled Gram for relate()"""
        self.check(self.lib.gp_keep_gram(self.h, 1 if keep else 0), "gp_keep_gram")

    def relate(self, numeigs, relthresh=0.05, max_pairs=1 << 16):
        """smartrel's pair scan on the kept Gram: [(a, b, y)] in rows of the pass, highest y
        first (ties by a, then b)"""
        while True:
            a = np.zeros(max_pairs, np.int32)
            b = np.zeros(max_pairs, np.int32)
            y = np.zeros(max_pairs)
            n = C.c_int64()
            self.check(self.lib.gp_relate(self.h, numeigs, relthresh, max_pairs,
                                          ptr(a, C.c_int32), ptr(b, C.c_int32),
                                          ptr(y, C.c_double), C.byref(n)), "gp_relate")
            if n.value <= max_pairs:
                break
            max_pairs = n.value
        a, b, y = a[:n.value], b[:n.value], y[:n.value]
        order = np.lexsort((b, a, -y))
        return [(int(a[k]), int(b[k]), float(y[k])) for k in order]

    def fastpca(self, K, L, I, seed=0, omega=None, precision=GP_PREC_FP64, fancynorm=1,
                altnormstyle=1):
        n = self.nrows
        ev = np.zeros(K)
        V = np.zeros((K, n))
        om = None if omega is None else np.ascontiguousarray(omega, dtype=np.float64)
        o = XtxOpts(fancynorm, altnormstyle, 0, 0x7fffffff, precision)
        self.check(self.lib.gp_fastpca(self.h, K, L, I, seed, ptr(om, C.c_double), C.byref(o),
                                       ptr(ev, C.c_double), ptr(V, C.c_double)), "gp_fastpca")
        return ev, V


class ServeRequest:
    """One submitted request: keeps its code rows and output buffers alive until done."""

    def __init__(self, server, ticket, codes, coords, status):
        self.server, self.ticket = server, ticket
        self.codes, self.coords, self.status = codes, coords, status
        self.done = False

    def test(self):
        if self.done:
            return True
        rc = self.server.lib.gp_serve_test(self.server.s, self.ticket)
        if rc == 0:
            return False
        self.done = True
        self.server.check(rc, "gp_serve_test")
        return True

    def wait(self, timeout=60.0):
        """Block until done; returns (coords [nsamp, K], status [nsamp])."""
        if not self.done:
            rc = self.server.lib.gp_serve_wait(self.server.s, self.ticket, timeout)
            if rc != GP_ERR_TIMEOUT:
                self.done = True
            self.server.check(rc, "gp_serve_wait")
        return self.coords, self.status


class PcaJob(ServeRequest):
    """A full-PCA job queued on a Server; wait() returns the smartpca_run result dict."""

    def __init__(self, server, ticket, args):
        super().__init__(server, ticket, None, None, None)
        self.args = args

    def wait(self, timeout=600.0):
        super().wait(timeout)
        return self.args.collect()


class Server:
    """Projection server on the panel (SNP weights) resident in `handle` (gpupca_serve.h)."""

    def __init__(self, handle, numeigs, max_batch=0, pool_samples=0, fp64_serial=False,
                 eigscale=None, pca_workers=0, pca_budget_bytes=0, host_loop=False):
        self.lib = load_library()
        self.K = numeigs
        self._scale = None if eigscale is None else np.ascontiguousarray(eigscale, np.float64)
        o = ServeOpts(numeigs, max_batch, pool_samples, int(fp64_serial),
                      ptr(self._scale, C.c_double), pca_workers, pca_budget_bytes,
                      int(host_loop))
        s = vp()
        handle.check(self.lib.gp_serve_open(handle.h, C.byref(o), C.byref(s)), "gp_serve_open")
        self.s = s
        n, rb = C.c_int64(), C.c_int64()
        self.check(self.lib.gp_serve_layout(self.s, C.byref(n), C.byref(rb)), "gp_serve_layout")
        self.nsnp, self.row_bytes = n.value, rb.value
        self.snp_index = np.zeros(self.nsnp, np.int32)
        self.check(self.lib.gp_serve_panel_snps(self.s, ptr(self.snp_index, C.c_int32)),
                   "gp_serve_panel_snps")

    def check(self, rc, what):
        if rc < 0:
            msg = self.lib.gp_serve_last_error(self.s).decode(errors="replace")
            raise GpuError("%s: %s: %s" % (what, GP_ERR.get(rc, rc), msg))
        return rc

    def submit(self, codes, coords=None, status=None):
        """codes: uint8 [nsamp, row_bytes] request rows (see request_rows)."""
        codes = np.ascontiguousarray(codes, dtype=np.uint8)
        q = codes.shape[0]
        assert codes.shape[1] == self.row_bytes
        if coords is None:
            coords = np.zeros((q, self.K))
        if status is None:
            status = np.zeros(q, np.int32)
        t = C.c_int64()
        self.check(self.lib.gp_serve_submit(self.s, ptr(codes, C.c_uint8), q,
                                            ptr(coords, C.c_double), ptr(status, C.c_int32),
                                            C.byref(t)), "gp_serve_submit")
        return ServeRequest(self, t.value, codes, coords, status)

    def submit_pca(self, records, nind, opts, **panel):
        """queue a full-PCA job (gp_serve_submit_pca); returns a request whose wait() gives
        the smartpca_run result dict"""
        a = _RunArgs(records, nind, opts, **panel)
        t = C.c_int64()
        self.check(self.lib.gp_serve_submit_pca(self.s, C.byref(a.panel), C.byref(opts),
                                                C.byref(a.result), C.byref(t)),
                   "gp_serve_submit_pca")
        return PcaJob(self, t.value, a)

    def loop_stats(self):
        """(device loop running, graph launches, batches it ran, polls that ran out idle)"""
        a, b, c, d = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64()
        self.check(self.lib.gp_serve_loop_stats(self.s, C.byref(a), C.byref(b), C.byref(c),
                                                C.byref(d)), "gp_serve_loop_stats")
        return a.value, b.value, c.value, d.value

    def pca_stats(self):
        a, b, c = C.c_int64(), C.c_int32(), C.c_int64()
        self.check(self.lib.gp_serve_pca_stats(self.s, C.byref(a), C.byref(b), C.byref(c)),
                   "gp_serve_pca_stats")
        return a.value, b.value, c.value

    def pause(self, paused=True):
        self.check(self.lib.gp_serve_pause(self.s, int(paused)), "gp_serve_pause")

    def stats(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self.check(self.lib.gp_serve_stats(self.s, C.byref(a), C.byref(b), C.byref(c)),
                   "gp_serve_stats")
        return a.value, b.value, c.value

    def close(self):
        if self.s:
            self.lib.gp_serve_close(self.s)
            self.s = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def request_rows(records, nind, samples, snp_index, row_bytes):
    """Request rows for `samples` from SNP-major packed records (packedancestrymap layout:
    sample i of a record at byte i>>2, bits (3-(i&3))*2): one row per sample over the panel
    SNPs snp_index, MSB first, padded with code 3."""
    rec = np.asarray(records, dtype=np.uint8)[np.asarray(snp_index)]
    samples = np.asarray(samples, dtype=np.int64)
    g = (rec[:, samples >> 2] >> ((3 - (samples & 3)) * 2).astype(np.uint8)) & 3  # [nk, q]
    q, nk = len(samples), len(snp_index)
    codes = np.full((q, row_bytes * 4), 3, np.uint8)
    codes[:, :nk] = g.T
    c4 = codes.reshape(q, row_bytes, 4)
    return ((c4[:, :, 0] << 6) | (c4[:, :, 1] << 4) | (c4[:, :, 2] << 2) | c4[:, :, 3]).astype(
        np.uint8)


def ridoutlier(evecs, neigs, thresh=6.0, mode=0):
    lib = load_library()
    E = np.ascontiguousarray(evecs, dtype=np.float64)
    n = E.shape[1]
    bad = np.zeros(n, np.int32)
    vec = np.zeros(n, np.int32)
    sc = np.zeros(n)
    nb = lib.gp_ridoutlier(ptr(E, C.c_double), n, neigs, thresh, mode, ptr(bad, C.c_int32),
                           ptr(vec, C.c_int32), ptr(sc, C.c_double))
    if nb < 0:
        raise GpuError("gp_ridoutlier: %s" % GP_ERR.get(nb, nb))
    return bad[:nb], vec, sc


def default_opts(**kw):
    lib = load_library()
    o = SmartpcaOpts()
    lib.gp_smartpca_defaults(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


class _RunArgs:
    """ctypes panel + result of one gp_smartpca_run, with the arrays they point into"""

    def __init__(self, records, nind, opts, code=GP_CODE_PACKED, snp_chrom=None,
                 snp_ignore=None, ind_ignore=None, ind_affstatus=None, ind_male=None,
                 want_xtx=False, ind_pop=None, want_ffvecs=False):
        self.keep = []
        if isinstance(records, tuple):  # (nsnp, record_bytes): the panel resident on the handle
            rec = None
            nsnp, rb = records
        else:
            rec = np.ascontiguousarray(records, dtype=np.uint8)
            nsnp, rb = rec.shape
            self.keep.append(rec)

        def arr(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            self.keep.append(a)
            return a

        self.nind, self.opts, self.want_xtx = nind, opts, want_xtx
        chrom = arr(snp_chrom, np.int32)
        self.panel = Panel(ptr(rec, C.c_uint8), rb, nsnp, nind, code, ptr(chrom, C.c_int32),
                           ptr(arr(snp_ignore, np.uint8), C.c_uint8),
                           ptr(arr(ind_ignore, np.uint8), C.c_uint8),
                           ptr(arr(ind_affstatus, np.uint8), C.c_uint8),
                           ptr(arr(ind_male, np.uint8), C.c_uint8),
                           ptr(arr(ind_pop, np.int32), C.c_int32))
        K = max(opts.numeigs, 1)
        out = dict(xindex=np.zeros(nind, np.int32), evals=np.zeros(nind),
                   evecs=np.zeros(K * nind), coords=np.zeros(K * nind),
                   ind_out=np.zeros(nind, np.uint8), snp_state=np.zeros(nsnp, np.uint8),
                   outlier_idx=np.zeros(nind, np.int32), outlier_iter=np.zeros(nind, np.int32),
                   outlier_vec=np.zeros(nind, np.int32), outlier_score=np.zeros(nind))
        r = RunResult(ptr(out["xindex"], C.c_int32), ptr(out["evals"], C.c_double),
                      ptr(out["evecs"], C.c_double), ptr(out["coords"], C.c_double),
                      ptr(out["ind_out"], C.c_uint8), ptr(out["snp_state"], C.c_uint8),
                      ptr(out["outlier_idx"], C.c_int32), ptr(out["outlier_iter"], C.c_int32),
                      ptr(out["outlier_vec"], C.c_int32), ptr(out["outlier_score"], C.c_double))
        if want_xtx:
            out["xtx"] = np.zeros(nind * nind)
            r.xtx = ptr(out["xtx"], C.c_double)
        if want_ffvecs:
            out["ffvecs"] = np.zeros(K * nsnp)
            r.ffvecs = ptr(out["ffvecs"], C.c_double)
        self.nsnp = nsnp
        self.out, self.result = out, r

    def collect(self):
        r, out, nind, opts = self.result, self.out, self.nind, self.opts
        n, k = r.nrows, r.numeigs
        res = dict(nrows=n, ncols=r.ncols, numeigs=k, npasses=r.npasses,
                   xindex=out["xindex"][:n].copy(),
                   evals=out["evals"][: (k if opts.fastmode else n)].copy(),
                   evecs=out["evecs"][: k * n].reshape(k, n).copy(),
                   coords=out["coords"][: k * nind].reshape(k, nind).copy(),
                   ind_out=out["ind_out"].astype(bool), snp_state=out["snp_state"],
                   outliers=[(int(out["outlier_idx"][i]), int(out["outlier_iter"][i]),
                              int(out["outlier_vec"][i]), float(out["outlier_score"][i]))
                             for i in range(min(r.noutliers, nind))],
                   t_phase={PHASES[i]: r.t_phase[i] for i in range(8)},
                   gram_flops=r.gram_flops, gram_ms=r.gram_ms, nused=r.nused)
        if self.want_xtx:
            res["xtx"] = out["xtx"][: n * n].reshape(n, n).copy()
        if "ffvecs" in out:
            res["ffvecs"] = out["ffvecs"][: k * self.nsnp].reshape(k, self.nsnp).copy()
        return res


def smartpca_run(handle, records, nind, opts, code=GP_CODE_PACKED, snp_chrom=None,
                 snp_ignore=None, ind_ignore=None, ind_affstatus=None, ind_male=None,
                 want_xtx=False, ind_pop=None, want_ffvecs=False):
    """Run the whole smartpca hot path (gp_smartpca_run) on in-memory records.  ind_pop
    (the samples' population indices) is read with opts.usepopsformissing; want_ffvecs
    returns the last pass's SNP weights (K x nsnp, 0 for SNPs it did not use)."""
    a = _RunArgs(records, nind, opts, code, snp_chrom, snp_ignore, ind_ignore, ind_affstatus,
                 ind_male, want_xtx, ind_pop, want_ffvecs)
    handle.check(handle.lib.gp_smartpca_run(handle.h, C.byref(opts), C.byref(a.panel),
                                            C.byref(a.result)), "gp_smartpca_run")
    return a.collect()


def smartrel_run(handle, records, nind, numeigs=10, relthresh=0.05, minallelecnt=1,
                 code=GP_CODE_PACKED, **kw):
    """smartrel on in-memory records: the smartpca outlier loop with smartrel's SNP rule
    (dropped when min(n0, n1) <= minallelecnt, no missingness limit, no projection), then the
    relatedness scan.  Returns (pairs [(sample a, sample b, y)] highest first, run result)."""
    panel_keys = ("snp_chrom", "snp_ignore", "ind_ignore", "ind_affstatus", "ind_male",
                  "ind_pop")
    panel = {k: kw.pop(k) for k in panel_keys if k in kw}
    opts = default_opts(numeigs=numeigs, minallelecnt=minallelecnt + 1, maxmissing=0x7fffffff,
                        lsqproject=0, fastmode=0, **kw)
    handle.keep_gram(True)
    try:
        r = smartpca_run(handle, records, nind, opts, code=code, **panel)
        pairs = handle.relate(r["numeigs"], relthresh)
    finally:
        handle.keep_gram(False)
    xi = r["xindex"]
    return [(int(xi[a]), int(xi[b]), y) for a, b, y in pairs], r


def set_blocks(chrom, gpos, ignore, blocklen=0.05):
    """setblocks: (number of blocks, tag per SNP)"""
    ch = np.ascontiguousarray(chrom, dtype=np.int32)
    gp = np.ascontiguousarray(gpos, dtype=np.float64)
    ig = None if ignore is None else np.ascontiguousarray(ignore, dtype=np.uint8)
    tag = np.zeros(len(ch), np.int32)
    nb = load_library().gp_set_blocks(ptr(ch, C.c_int32), ptr(gp, C.c_double),
                                      ptr(ig, C.c_uint8), len(ch), blocklen,
                                      ptr(tag, C.c_int32))
    return nb, tag


def smartpca_footprint(nind, nsnp, precision, numeigs):
    return load_library().gp_smartpca_footprint(nind, nsnp, precision, numeigs)


class SynthSpec(C.Structure):
    _fields_ = [("nsnp", C.c_int64), ("nind", C.c_int32), ("npops", C.c_int32),
                ("pop_sizes", i32p), ("fst", f64p), ("p_lo", C.c_double), ("p_hi", C.c_double),
                ("miss_lo", C.c_double), ("miss_hi", C.c_double), ("seed", C.c_uint64)]


def synth_records(nsnp, pop_sizes, fst, miss=0.01, miss_hi=None, n_admixed=0, seed=1,
                  p_lo=0.05, p_hi=0.95, nthreads=None):
    """Seeded Balding-Nichols packed records (nsnp x rlen uint8) and per-sample labels."""
    s = load_synth()
    ps = np.ascontiguousarray(pop_sizes, dtype=np.int32)
    fs = np.ascontiguousarray(fst, dtype=np.float64)
    nind = int(ps.sum()) + int(n_admixed)
    spec = SynthSpec(nsnp, nind, len(ps), ptr(ps, C.c_int32), ptr(fs, C.c_double), p_lo, p_hi,
                     miss, miss if miss_hi is None else miss_hi, seed)
    rlen = s.gp_packed_rlen(nind)
    rec = np.zeros((nsnp, rlen), np.uint8)
    pop = np.zeros(nind, np.int32)
    rc = s.gp_synth_records(C.byref(spec), ptr(rec, C.c_uint8), rlen, ptr(pop, C.c_int32),
                            nthreads or os.cpu_count() or 1)
    if rc != 0:
        raise RuntimeError("gp_synth_records failed: %d" % rc)
    return rec, pop


def synth_sample_rows(nsnp, pop_sizes, fst, snp_index, row_bytes, sample_seed, miss=0.01,
                      miss_hi=None, n_admixed=0, seed=1, p_lo=0.05, p_hi=0.95, nthreads=None):
    """New samples of the populations of synth_records(nsnp, pop_sizes, fst, seed=seed) as
    request rows over the panel SNPs snp_index (uint8 [nind, row_bytes]) and their labels."""
    s = load_synth()
    ps = np.ascontiguousarray(pop_sizes, dtype=np.int32)
    fs = np.ascontiguousarray(fst, dtype=np.float64)
    nind = int(ps.sum()) + int(n_admixed)
    spec = SynthSpec(nsnp, nind, len(ps), ptr(ps, C.c_int32), ptr(fs, C.c_double), p_lo, p_hi,
                     miss, miss if miss_hi is None else miss_hi, seed)
    idx = np.ascontiguousarray(snp_index, dtype=np.int64)
    rows = np.empty((nind, row_bytes), np.uint8)
    pop = np.zeros(nind, np.int32)
    rc = s.gp_synth_sample_rows(C.byref(spec), sample_seed, ptr(idx, C.c_int64), len(idx),
                                row_bytes, ptr(rows, C.c_uint8), ptr(pop, C.c_int32),
                                nthreads or os.cpu_count() or 1)
    if rc != 0:
        raise RuntimeError("gp_synth_sample_rows failed: %d" % rc)
    return rows, pop


def synth_write_dataset(prefix, nsnp, pop_sizes, fst, miss=0.01, miss_hi=None, n_admixed=0,
                        seed=1, p_lo=0.05, p_hi=0.95, nthreads=None):
    s = load_synth()
    ps = np.ascontiguousarray(pop_sizes, dtype=np.int32)
    fs = np.ascontiguousarray(fst, dtype=np.float64)
    nind = int(ps.sum()) + int(n_admixed)
    spec = SynthSpec(nsnp, nind, len(ps), ptr(ps, C.c_int32), ptr(fs, C.c_double), p_lo, p_hi,
                     miss, miss if miss_hi is None else miss_hi, seed)
    rc = s.gp_synth_write_dataset(C.byref(spec), prefix.encode(), nthreads or os.cpu_count() or 1)
    if rc != 0:
        raise RuntimeError("gp_synth_write_dataset failed: %d" % rc)


def host_register(a):
    """page-lock a numpy buffer (cudaHostRegister) for fast uploads"""
    lib = load_library()
    rc = lib.gp_host_register(a.ctypes.data_as(vp), a.nbytes)
    if rc != GP_OK:
        raise GpuError("gp_host_register failed: %s" % lib.gp_last_error(None).decode())


def host_unregister(a):
    load_library().gp_host_unregister(a.ctypes.data_as(vp))


def twstats(evals, nrows, nostatslim=10, znval=-1.0):
    """smartpca's Tracy-Widom statistics of a spectrum (gp_twstats, host only): for each of the
    eigenvalues above 1e-6 (descending) a (twstat, p-value, effective n) tuple, None where the
    reference prints NA"""
    lam = np.ascontiguousarray(evals, dtype=np.float64)
    m = int(np.sum(lam > 1e-6))
    tw, pv, zn = np.zeros(m), np.zeros(m), np.zeros(m)
    lib = load_library()
    rc = lib.gp_twstats(ptr(lam, C.c_double), m, int(nrows), float(znval), int(nostatslim),
                        ptr(tw, C.c_double), ptr(pv, C.c_double), ptr(zn, C.c_double))
    if rc != GP_OK:
        raise GpuError("gp_twstats failed (%d)" % rc)
    return [None if pv[i] < 0.0 else (float(tw[i]), float(pv[i]), float(zn[i]))
            for i in range(m)]


def tw_tail(x):
    """the right tail of TW1 at x as smartpca reads it (gp_tw_tail, host only)"""
    return float(load_library().gp_tw_tail(float(x)))


def mpstats(evals):
    """the mpstats quartiles of the eigenvalues above 1e-6 (gp_mpstats), None below 10"""
    lam = np.ascontiguousarray(evals, dtype=np.float64)
    m = int(np.sum(lam > 1e-6))
    q = np.zeros(4)
    rc = load_library().gp_mpstats(ptr(lam, C.c_double), m, ptr(q, C.c_double))
    return None if rc != GP_OK else [float(v) for v in q]

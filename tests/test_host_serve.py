"""Host-side logic of the projection server (no GPU): request row layout and the bindings."""
import numpy as np

from eig_gb300 import native
from oracle import oracle as O


def test_request_rows_layout():
    rng = np.random.default_rng(3)
    nsnp, nind = 37, 23
    g = rng.integers(-1, 3, size=(nsnp, nind)).astype(np.int8)
    rec = O.pack(g)
    snp_index = rng.permutation(nsnp)[:29]
    samples = np.array([0, 5, 22, 7, 7])
    row_bytes = 16
    rows = native.request_rows(rec, nind, samples, snp_index, row_bytes)
    assert rows.shape == (len(samples), row_bytes) and rows.dtype == np.uint8
    back = O.unpack(rows, row_bytes * 4)  # rows read as records over "SNPs"
    want = np.full((len(samples), row_bytes * 4), -1, np.int8)
    want[:, :len(snp_index)] = g[snp_index][:, samples].T
    assert np.array_equal(back, want)


def test_serve_symbols_exported():
    lib = native.load_library()
    for name in ["gp_serve_open", "gp_serve_layout", "gp_serve_panel_snps", "gp_serve_submit",
                 "gp_serve_test", "gp_serve_wait", "gp_serve_stats", "gp_serve_last_error",
                 "gp_serve_close"]:
        assert hasattr(lib, name) and name in native.EXPORTED
    assert native.ServeOpts.numeigs.offset == 0 and native.ServeOpts.eigscale.offset == 24


def test_library_exports_every_declared_symbol():
    """every function declared in include/*.h is exported by libgpupca.so and bound"""
    import os
    import re
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    names = set()
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^[a-z_][a-z0-9_ ]*[ *]+(gp_[a-z0-9_]+)\(", txt, re.M))
    assert len(names) >= 38
    lib = native.load_library()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    unbound = [n for n in sorted(names) if n not in native.EXPORTED]
    assert not unbound, unbound


def test_synth_sample_rows_consistent_with_records():
    """with the panel's own seed the new-sample generator reproduces the panel genotypes in
    request-row layout; another sample seed gives other samples of the same populations"""
    pops, fst = [30, 20], [0.02, 0.05]
    rec, pop = native.synth_records(500, pops, fst, miss=0.1, miss_hi=0.3, n_admixed=7, seed=9)
    nind = len(pop)
    rng = np.random.default_rng(1)
    snp_index = rng.permutation(500)[:333]
    rows, p2 = native.synth_sample_rows(500, pops, fst, snp_index, 96, sample_seed=9, miss=0.1,
                                        miss_hi=0.3, n_admixed=7, seed=9)
    assert np.array_equal(p2, pop)
    want = native.request_rows(rec, nind, np.arange(nind), snp_index, 96)
    assert np.array_equal(rows, want)
    other, _ = native.synth_sample_rows(500, pops, fst, snp_index, 96, sample_seed=10, miss=0.1,
                                        miss_hi=0.3, n_admixed=7, seed=9)
    assert not np.array_equal(other, rows)

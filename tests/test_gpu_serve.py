"""Projection serving (gpupca_serve.h) against gp_lsqproj and the oracle.

The server's products are exact integer sums on the tensor cores followed by the same FP64
Cholesky as lsqproject, so its coordinates equal gp_lsqproj's (split path) bit for bit, and a
sample's coordinates do not depend on the requests batched with it.  The FP64 serial
baseline sums in another order: 1e-11 relative to the oracle.
"""
import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O

pytestmark = pytest.mark.gpu

K = 10


@pytest.fixture(scope="module")
def panel(gpu):
    rec, pop = native.synth_records(20000, [150, 150, 100], [0.01, 0.02, 0.05], miss=0.1,
                                    seed=31, nthreads=4, n_admixed=40)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    rows = np.arange(0, 300, dtype=np.int32)
    cols = np.arange(20000, dtype=np.int32)
    gpu.set_samples(rows)
    gpu.set_snps(cols)
    gpu.xtx(precision=native.GP_PREC_SPLIT_FP16)
    ev, V = gpu.eigvecs(K)
    ff, fx, sc = gpu.snp_weights(K)
    proj = np.arange(nind, dtype=np.int32)
    a, b, nobs, st = gpu.lsqproj(K, proj)
    s = O.pass_columns(rec, cols, rows)
    off, ofx, osc = O.weights(s, V, K)
    oa, ob, onobs, ost = O.lsqproj(s, off, osc, K, proj)
    return dict(rec=rec, nind=nind, a=a, st=st, oa=oa, ost=ost, ev=ev)


def _rows(srv, panel, samples):
    return native.request_rows(panel["rec"], panel["nind"], samples, srv.snp_index, srv.row_bytes)


def _check_vs_lsqproj(panel, samples, coords, status, scale=None):
    a, st = panel["a"][:, samples].T, panel["st"][samples]
    assert np.array_equal(status, st)
    ok = st == 0
    want = a[ok] if scale is None else a[ok] * scale[None, :]
    assert np.array_equal(coords[ok], want)
    assert np.all(coords[~ok] == 0.0)


def test_serve_matches_lsqproj_bit_exact(gpu, panel):
    nind = panel["nind"]
    with native.Server(gpu, K) as srv:
        assert srv.nsnp == 20000 and srv.row_bytes % 16 == 0
        assert np.array_equal(np.sort(srv.snp_index), np.arange(20000))
        sizes = [1, 7, 33, 100, 64, nind - 205]
        reqs, start = [], 0
        for n in sizes:
            samp = np.arange(start, start + n)
            reqs.append((samp, srv.submit(_rows(srv, panel, samp))))
            start += n
        assert start == nind
        for samp, r in reqs:
            coords, status = r.wait(60.0)
            _check_vs_lsqproj(panel, samp, coords, status)
        b, n, q = srv.stats()
        assert n == nind and q == len(sizes) and 1 <= b <= len(sizes)
    # and against the oracle
    ok = panel["ost"] == 0
    assert np.array_equal(panel["st"], panel["ost"])
    assert np.max(np.abs(panel["a"][:, ok] - panel["oa"][:, ok])) <= 1e-11 * np.max(
        np.abs(panel["oa"]))


def test_serve_alone_equals_mixed(gpu, panel):
    """a request's coordinates are the same alone and inside a stream of other requests"""
    rng = np.random.default_rng(7)
    nind = panel["nind"]
    target = rng.choice(nind, 57, replace=False)
    with native.Server(gpu, K, max_batch=512) as srv:
        alone, st_alone = srv.submit(_rows(srv, panel, target)).wait(60.0)
        others = [_rows(srv, panel, rng.choice(nind, int(rng.integers(1, 90)), replace=False))
                  for _ in range(40)]
        srv.pause(True)  # everything below is admitted before the first batch forms
        reqs = []
        for i, rows in enumerate(others):
            reqs.append(srv.submit(rows))
            if i == 17:
                mixed = srv.submit(_rows(srv, panel, target))
        srv.pause(False)
        cm, sm = mixed.wait(60.0)
        for r in reqs:
            r.wait(60.0)
        b, n, q = srv.stats()
        # ~1,900 samples in batches of <= 512 rows: a handful of batches for 42 requests
        assert q == 42 and b <= 16
    assert np.array_equal(st_alone, sm)
    assert np.array_equal(alone, cm)


def test_serve_device_loop_one_launch_bounded_polls(gpu, panel):
    """the batches run in one persistent launch (the device-resident loop); with no request
    its bounded poll runs out and the loop iterates instead of waiting for ever"""
    import time
    nind = panel["nind"]
    with native.Server(gpu, K) as srv:
        on, launches, b0, idle0 = srv.loop_stats()
        assert on == 1 and launches == 1 and b0 == 0
        time.sleep(0.05)
        _, _, _, idle1 = srv.loop_stats()
        assert idle1 > idle0
        reqs = [(samp, srv.submit(_rows(srv, panel, samp)))
                for samp in np.array_split(np.arange(nind), 5)]
        for samp, r in reqs:
            coords, status = r.wait(60.0)
            _check_vs_lsqproj(panel, samp, coords, status)
        on, launches, b1, _ = srv.loop_stats()
        assert on == 1 and launches == 1 and 1 <= b1 <= 5


def test_serve_host_loop_schedule(gpu, panel):
    """the host-launched schedule (host_loop) gives the same coordinates"""
    nind = panel["nind"]
    with native.Server(gpu, K, host_loop=True) as srv:
        assert srv.loop_stats()[0] == 0
        samp = np.arange(nind)
        coords, status = srv.submit(_rows(srv, panel, samp)).wait(60.0)
        _check_vs_lsqproj(panel, samp, coords, status)


def test_serve_small_pool_admission_and_eigscale(gpu, panel):
    """a pool of 64 rows forces admission to wait for memory; eigscale multiplies coords"""
    rng = np.random.default_rng(8)
    nind = panel["nind"]
    scale = np.sqrt(np.maximum(panel["ev"][:K], 0.0))
    with native.Server(gpu, K, max_batch=64, pool_samples=64, eigscale=scale) as srv:
        with pytest.raises(native.GpuError):
            srv.submit(_rows(srv, panel, np.arange(65)))
        reqs = []
        for _ in range(30):
            samp = rng.choice(nind, int(rng.integers(1, 41)), replace=False)
            reqs.append((samp, srv.submit(_rows(srv, panel, samp))))
        for samp, r in reqs:
            coords, status = r.wait(60.0)
            _check_vs_lsqproj(panel, samp, coords, status, scale)
        b, n, q = srv.stats()
        assert q == 30 and n == sum(len(s) for s, _ in reqs)


def test_serve_fp64_serial_baseline(gpu, panel):
    nind = panel["nind"]
    with native.Server(gpu, K, fp64_serial=True) as srv:
        samp = np.arange(nind)
        r1 = srv.submit(_rows(srv, panel, samp[:150]))
        r2 = srv.submit(_rows(srv, panel, samp[150:]))
        c1, s1 = r1.wait(60.0)
        c2, s2 = r2.wait(60.0)
        b, n, q = srv.stats()
        assert b == 2 and q == 2
    coords, status = np.vstack([c1, c2]), np.concatenate([s1, s2])
    assert np.array_equal(status, panel["ost"])
    ok = status == 0
    oa = panel["oa"]
    assert np.max(np.abs(coords[ok] - oa[:, ok].T)) <= 1e-11 * np.max(np.abs(oa))


def test_serve_ticket_released_after_wait(gpu, panel):
    with native.Server(gpu, K) as srv:
        r = srv.submit(_rows(srv, panel, np.arange(5)))
        r.wait(60.0)
        # the ticket was released by the completed wait
        assert srv.lib.gp_serve_wait(srv.s, r.ticket, 0.1) == -1
        assert srv.lib.gp_serve_test(srv.s, 10 ** 9) == -1


def _pca_data(nsnp, pops, seed):
    rec, pop = native.synth_records(nsnp, pops, [0.01, 0.03, 0.05][:len(pops)], miss=0.02,
                                    seed=seed, nthreads=4)
    return rec, len(pop)


@pytest.mark.parametrize("prec", [native.GP_PREC_FP64, native.GP_PREC_SPLIT_FP16])
def test_serve_pca_job_same_alone_and_in_the_mix(gpu, panel, prec):
    """a full-PCA job run by the server beside projection batches gives exactly the result
    of gp_smartpca_run on its own handle"""
    rec, nind = _pca_data(6000, [120, 100, 80], 41)
    opts = native.default_opts(numeigs=6, numoutliter=2, precision=prec)
    with native.Handle(0) as h2:
        alone = native.smartpca_run(h2, rec, nind, opts)
    rng = np.random.default_rng(9)
    with native.Server(gpu, K, max_batch=256, pca_workers=2) as srv:
        reqs = [srv.submit(_rows(srv, panel, rng.choice(panel["nind"], 50, replace=False)))
                for _ in range(10)]
        job = srv.submit_pca(rec, nind, opts)
        reqs += [srv.submit(_rows(srv, panel, rng.choice(panel["nind"], 50, replace=False)))
                 for _ in range(10)]
        mixed = job.wait(300.0)
        for r in reqs:
            r.wait(60.0)
        done, peak, used = srv.pca_stats()
        assert done == 1 and used == 0
    for key in ("xindex", "evals", "evecs", "coords", "ind_out"):
        assert np.array_equal(alone[key], mixed[key]), key
    assert alone["outliers"] == mixed["outliers"]


def test_serve_pca_admission_by_footprint(gpu, panel):
    """with a budget below one job's footprint the jobs run one at a time (a job is admitted
    alone when nothing else runs); all complete with their own results"""
    data = [_pca_data(3000, [60, 60], s) for s in (51, 52, 53)]
    opts = native.default_opts(numeigs=4, numoutliter=0, precision=native.GP_PREC_SPLIT_FP16)
    fp = native.smartpca_footprint(data[0][1], 3000, native.GP_PREC_SPLIT_FP16, 4)
    assert fp > 3000 * 32
    with native.Server(gpu, K, pca_workers=3, pca_budget_bytes=fp // 2) as srv:
        jobs = [srv.submit_pca(rec, n, opts) for rec, n in data]
        res = [j.wait(300.0) for j in jobs]
        done, peak, used = srv.pca_stats()
    assert done == 3 and peak == 1
    with native.Handle(0) as h2:
        for (rec, n), r in zip(data, res):
            want = native.smartpca_run(h2, rec, n, opts)
            assert np.array_equal(want["evals"], r["evals"])

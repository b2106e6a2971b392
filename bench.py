"""Benchmark of the smartpca hot path on GB300 (one JSON line on rank 0).

Workload (default): full smartpca at N=5,000 samples x M=600,000 SNPs, Balding-Nichols with
6 populations of sizes 500..1,100 and F in {0.005, 0.01, 0.02, 0.03, 0.04, 0.05}, 2% missing,
K=20, numoutlieriter 5, outlier sigma 6, lsqproject on.  Seeded synthetic genotypes stand in
for real panels (no dataset is read).

A step = one whole gp_smartpca_run (counts, normalisation, Gram, eigensolve, outlier passes,
SNP weights, lsqproject) on the panel resident in HBM.  `value` = whole-job XTX throughput:
the algorithmic Gram flops of every pass, sum of N_p (N_p+1) M_p, divided by the step time
(so eigensolve, weights and projection time count against it).  `e2e` is the same metric
through the C ABI with the packed records in pinned HOST memory: the upload and the result
read-back are inside the timed region.

--impl reference times the reference's own Gram algorithm (the partial-sum lookup of
smartpca, restated in oracle/smartpca_oracle.c) on the host cores with all threads over a
bounded SNP sample of the same workload, in the same unit.

One GPU only: the path does not shard (one PCA per panel) and the split Gram's cluster
schedule multicasts its TMA loads within this GPU's own memory, so the GPU arm refuses
--gpus N > 1 and a torchrun launch with WORLD_SIZE > 1: rank 0 prints one JSON line with an
"unavailable" reason and every rank exits 0 without touching a GPU.  The reference arm (CPU)
runs on rank 0 alone; the other ranks exit 0 without work.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

CONFIGS = {
    "full": dict(nsnp=600_000, pops=[500, 700, 800, 900, 1000, 1100],
                 fst=[0.005, 0.01, 0.02, 0.03, 0.04, 0.05], miss=0.02, K=20, seed=2,
                 name="smartpca N=5000 x M=600000 BN 6 pops, 2% missing, K=20, "
                      "numoutlieriter 5, sigma 6, lsqproject"),
    "fastmode": dict(nsnp=500_000, pops=[5000] * 10, n_admixed=5000, miss=0.01, K=10, L=20,
                     I=10, seed=3, fst_seed=3,
                     name="fastmode N=55000 (10 BN pops of 5000 + 5000 two-way admixed) x "
                          "M=500000, F~U(0.005,0.05), 1% missing, K=10, L=20, I=10, omega seed 3"),
    "mixed": dict(nsnp=600_000, pops=[500, 700, 800, 900, 1000, 1100],
                  fst=[0.005, 0.01, 0.02, 0.03, 0.04, 0.05], miss=0.02, K=20, seed=2,
                  jobs=6, nproj=200, rate=40.0, pca_every=21, pca_K=10, pca_burst=3,
                  name="mixed stream: projection requests on the N=5000 x M=600000 K=20 panel "
                       "+ full-PCA jobs at 1:20 (N log-U 200-8000, M U 50k-600k, 2-8 pops, "
                       "F~U(0.005,0.05), 1-5% missing, K=10), Poisson arrivals 40/s after a "
                       "burst of 3 PCA jobs"),
    "convertf": dict(nsnp=600_000, pops=[500, 700, 800, 900, 1000, 1100],
                     fst=[0.005, 0.01, 0.02, 0.03, 0.04, 0.05], miss=0.02, K=0, seed=2,
                     name="convertf packedancestrymap -> PLINK bed of the N=5000 x M=600000 "
                          "panel (all samples, all SNPs)"),
    "eig": dict(nsnp=4000, pops=[2500, 2500], fst=[0.02, 0.03], miss=0.01, K=20, seed=5,
                name="dense FP64 eigensolve of the N=5000 Gram (all eigenvalues, top 20 "
                     "vectors): tridiagonalisation, multisection, inverse iteration, WY "
                     "back-transformation"),
    "mid": dict(nsnp=200_000, pops=[500, 700, 800, 900, 1000, 1100],
                fst=[0.005, 0.01, 0.02, 0.03, 0.04, 0.05], miss=0.02, K=20, seed=2,
                name="smartpca N=5000 x M=200000 BN 6 pops, 2% missing, K=20 (profiling case: "
                     "250 MB of packed records, larger than L2)"),
    "small": dict(nsnp=60_000, pops=[100, 150, 200, 250, 150, 150],
                  fst=[0.005, 0.01, 0.02, 0.03, 0.04, 0.05], miss=0.02, K=20, seed=2,
                  name="smartpca N=1000 x M=60000 BN 6 pops (profiling case)"),
}

METRIC = "PCA wall-s & XTX TFLOP/s, split-BF16 vs FP64 @1e-6 eval err; proj p99 ms"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region"""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = []
        mx = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for p in self.samples:
            try:
                sm.append(float(p[0]))
                mx = float(p[1])
            except ValueError:
                continue
            for i, n in enumerate(names):
                if p[3 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def launch_shape(args):
    """(world, rank, local) of this process: torchrun's WORLD_SIZE/RANK/LOCAL_RANK, else the
    --gpus request on rank 0"""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return max(world, args.gpus), rank, local


def _subspace_angle_deg(A, B):
    """largest principal angle between the row spaces of A and B (k x n)"""
    qa, _ = np.linalg.qr(A.T)
    qb, _ = np.linalg.qr(B.T)
    sv = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return float(np.degrees(np.arccos(np.clip(sv.min(), -1.0, 1.0))))


def accuracy_vs_fp64(h, resident, nind, cfg, r_split, step_ms):
    """one plain FP64 GPU run of the same workload: wall time, eigenvalue error, subspace
    angle and outlier decisions of the split run against it"""
    from eig_gb300 import native
    opts = native.default_opts(numeigs=cfg["K"], numoutliter=5, outlthresh=6.0,
                               precision=native.GP_PREC_FP64)
    h.timer_start()
    r64 = native.smartpca_run(h, resident, nind, opts)
    ms = h.timer_stop()
    K = cfg["K"]
    e64, e16 = r64["evals"][:K], r_split["evals"][:K]
    same_rows = np.array_equal(r64["xindex"], r_split["xindex"])
    out = {"fp64_pca_wall_s": ms / 1e3, "split_speedup": ms / step_ms,
           "eval_max_rel_err": float(np.max(np.abs(e16 - e64) / np.abs(e64))),
           "outliers_identical": [o[:3] for o in r64["outliers"]] ==
                                 [o[:3] for o in r_split["outliers"]],
           "kept_samples_identical": bool(same_rows)}
    if same_rows:
        out["subspace_angle_deg"] = _subspace_angle_deg(r64["evecs"][:K], r_split["evecs"][:K])
        # ridoutlier's z-scores (src/eigensrc/smartsubs.c:18-91) of the last pass's top 10
        # vectors on both paths: the smallest margin ||z| - sigma| and the largest split-vs-FP64
        # z difference (a decision could flip only where the latter reaches the former)
        def z(E):
            W = E - E.mean(axis=1, keepdims=True)
            return W / np.sqrt(np.mean(W * W, axis=1, keepdims=True))
        z64, z16 = z(r64["evecs"][:10]), z(r_split["evecs"][:10])
        z16 = z16 * np.sign(np.sum(z64 * z16, axis=1, keepdims=True))
        margin = np.abs(np.abs(z64) - 6.0)
        out["outlier_margin"] = {"sigma": 6.0, "min_margin": float(margin.min()),
                                 "max_abs_z": float(np.abs(z64).max()),
                                 "max_z_diff_split_vs_fp64": float(np.abs(z16 - z64).max())}
    return out


def _serve_load(srv, rows, sizes, offsets, arrivals):
    """submit request i at arrivals[i] seconds; returns per-request latency (ms, from the
    scheduled arrival to completion), the span (s) and the completed requests"""
    n = len(sizes)
    done_t = [0.0] * n
    reqs = [None] * n
    ready = threading.Semaphore(0)
    errors = []

    def waiter():
        for i in range(n):
            ready.acquire()
            try:
                reqs[i].wait(300.0)
            except Exception as e:  # noqa: BLE001 - reported after the run
                errors.append(str(e))
            done_t[i] = time.perf_counter()

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    for i in range(n):
        while True:
            dt = t0 + arrivals[i] - time.perf_counter()
            if dt <= 0:
                break
            time.sleep(min(dt, 0.001))
        reqs[i] = srv.submit(rows[offsets[i]:offsets[i] + sizes[i]])
        ready.release()
    th.join()
    if errors:
        raise RuntimeError("serving request failed: %s" % errors[0])
    lat = np.array([(done_t[i] - (t0 + arrivals[i])) * 1e3 for i in range(n)])
    return lat, max(done_t) - t0, reqs


def run_serving(h, cfg, nreq=400, seed=11, n64=100):
    """Projection serving on the panel left resident by the PCA run: capacity, Poisson
    arrivals at 50% and 80% of it, the FP64 one-request-at-a-time baseline, and the
    coordinate error of the tensor-core path against the FP64 one."""
    from eig_gb300 import native
    K = cfg["K"]
    srv = native.Server(h, K, max_batch=4096, pool_samples=32768)
    npool = 4096
    npops = len(cfg["pops"])
    per = (3 * npool // 4) // npops
    t = time.time()
    rows, _ = native.synth_sample_rows(cfg["nsnp"], [per] * npops, cfg["fst"], srv.snp_index,
                                       srv.row_bytes, sample_seed=cfg["seed"] + 1000, miss=0.0,
                                       miss_hi=0.95, n_admixed=npool - per * npops,
                                       seed=cfg["seed"])
    gen_s = time.time() - t
    # pinning host memory synchronises the device: done with the device-resident loop
    # stopped (a paused server stops it)
    srv.pause(True)
    native.host_register(rows)
    srv.pause(False)
    rng = np.random.default_rng(seed)

    def draw(n):
        sz = rng.integers(1, 2001, size=n)
        off = np.array([rng.integers(0, npool - z + 1) for z in sz])
        return sz, off

    # warm-up and capacity: every request offered at t = 0
    sz, off = draw(20)
    _serve_load(srv, rows, sz, off, np.zeros(len(sz)))
    sz, off = draw(nreq)
    b0, s0, q0 = srv.stats()
    lat, span, reqs = _serve_load(srv, rows, sz, off, np.zeros(nreq))
    b1, s1, q1 = srv.stats()
    cap_sps = float(sz.sum()) / span
    cap_rps = nreq / span
    out = {"panel": "K=%d over %d kept SNPs (%d bytes per sample row)" % (K, srv.nsnp,
                                                                           srv.row_bytes),
           "requests": "1-2000 new samples each (3/4 from the %d panel populations, 1/4 "
                       "two-way admixed), per-sample missing ~U(0,0.95), rows in pinned host "
                       "memory, H2D inside the latency" % npops,
           "capacity": {"samples_per_s": cap_sps, "req_per_s": cap_rps, "n": nreq,
                        "batches": b1 - b0, "packed_gbs": cap_sps * srv.row_bytes / 1e9},
           "poisson": [], "request_gen_s": gen_s}
    for frac in (0.5, 0.8):
        rate = frac * cap_rps
        sz, off = draw(nreq)
        arr = np.cumsum(rng.exponential(1.0 / rate, size=nreq))
        lat, span, reqs = _serve_load(srv, rows, sz, off, arr)
        out["poisson"].append({"offered_req_per_s": rate, "load": frac, "n": nreq,
                               "samples_per_s": float(sz.sum()) / span,
                               "p50_ms": float(np.percentile(lat, 50)),
                               "p99_ms": float(np.percentile(lat, 99))})
    # the FP64 one-request-at-a-time baseline over n64 requests of the same distribution, and
    # the tensor-core server's coordinates for the same requests
    sz_c, off_c = draw(n64)
    _, _, creqs = _serve_load(srv, rows, sz_c, off_c, np.zeros(n64))
    on, launches, lbatches, idle = srv.loop_stats()
    out["device_loop"] = {"running": bool(on), "graph_launches": launches, "batches": lbatches,
                          "idle_polls": idle}
    srv.close()
    # the same capacity run with the host-launched schedule (one set of launches per batch)
    sh = native.Server(h, K, max_batch=4096, pool_samples=32768, host_loop=True)
    sz_h, off_h = draw(nreq)
    _, span_h, _ = _serve_load(sh, rows, sz_h, off_h, np.zeros(nreq))
    sh.close()
    out["capacity_host_loop"] = {"samples_per_s": float(sz_h.sum()) / span_h,
                                 "req_per_s": nreq / span_h, "n": nreq}
    s64 = native.Server(h, K, max_batch=2048, pool_samples=4096, fp64_serial=True)
    lat64, span64, r64 = _serve_load(s64, rows, sz_c, off_c, np.zeros(n64))
    s64.close()
    err_abs, err_rel = 0.0, 0.0
    for a, b in zip(creqs, r64):
        ok = (a.status == 0) & (b.status == 0)
        assert np.array_equal(a.status, b.status)
        d = np.abs(a.coords[ok] - b.coords[ok])
        if d.size:
            err_abs = max(err_abs, float(d.max()))
            err_rel = max(err_rel, float(d.max() / np.abs(b.coords[ok]).max()))
    sps64 = float(sz_c.sum()) / span64
    out["fp64_serial"] = {"samples_per_s": sps64, "n": n64, "samples": int(sz_c.sum()),
                          "ms_per_request": span64 / n64 * 1e3}
    out["speedup_vs_fp64_serial"] = cap_sps / sps64
    out["coord_max_abs_err_vs_fp64"] = err_abs
    out["coord_max_rel_err_vs_fp64"] = err_rel
    native.host_unregister(rows)
    return out


def _serial_queue(arrivals, service):
    """FIFO single-server queue: completion latency of each item given arrival times and
    service times (s)"""
    t, lat = 0.0, []
    for a, d in zip(arrivals, service):
        t = max(t, a) + d
        lat.append(t - a)
    return np.array(lat)


def run_mixed(args, cfg, local):
    """Config 5: projection requests and full-PCA jobs in one Poisson stream through the
    server (jobs admitted by device footprint on worker handles), against the plain FP64
    path run one item at a time (measured service times, FIFO queue on the same arrivals)."""
    import torch

    from eig_gb300 import native
    torch.cuda.set_device(local)
    prec = native.PRECISIONS[args.precision]
    rng = np.random.default_rng(cfg["seed"] + 7)
    t0 = time.time()
    rec, pop = native.synth_records(cfg["nsnp"], cfg["pops"], cfg["fst"], miss=cfg["miss"],
                                    seed=cfg["seed"])
    nind = len(pop)
    h = native.Handle(local)
    opts = native.default_opts(numeigs=cfg["K"], numoutliter=5, outlthresh=6.0, precision=prec)
    native.smartpca_run(h, rec, nind, opts)        # leaves the K=20 panel resident
    # the full-PCA job datasets
    jobs = []
    for j in range(cfg["jobs"]):
        n = int(round(np.exp(rng.uniform(np.log(200), np.log(8000)))))
        m = int(rng.uniform(50_000, 600_000))
        npop = int(rng.integers(2, 9))
        sizes = [n // npop] * npop
        sizes[0] += n - sum(sizes)
        fst = list(rng.uniform(0.005, 0.05, size=npop))
        miss = float(rng.uniform(0.01, 0.05))
        jr, _ = native.synth_records(m, sizes, fst, miss=miss, seed=cfg["seed"] + 100 + j)
        native.host_register(jr)
        jobs.append(dict(rec=jr, n=n, m=m, npop=npop, miss=miss))
    gen_s = time.time() - t0
    K2 = cfg["pca_K"]
    jopts = native.default_opts(numeigs=K2, numoutliter=5, outlthresh=6.0, precision=prec)
    srv = native.Server(h, cfg["K"], max_batch=4096, pool_samples=32768, pca_workers=2,
                        pca_budget_bytes=96 << 30)
    npool = 4096
    npops = len(cfg["pops"])
    per = (3 * npool // 4) // npops
    rows, _ = native.synth_sample_rows(cfg["nsnp"], [per] * npops, cfg["fst"], srv.snp_index,
                                       srv.row_bytes, sample_seed=cfg["seed"] + 1000, miss=0.0,
                                       miss_hi=0.95, n_admixed=npool - per * npops,
                                       seed=cfg["seed"])
    srv.pause(True)  # pinning host memory synchronises the device: loop stopped
    native.host_register(rows)
    srv.pause(False)
    # warm-up: every dataset once through the server, a few projections
    for jb in jobs:
        srv.submit_pca(jb["rec"], jb["n"], jopts).wait(600.0)
    for _ in range(5):
        srv.submit(rows[:1000]).wait(60.0)
    # the stream
    nitems = cfg["nproj"] + cfg["nproj"] // (cfg["pca_every"] - 1)
    arrivals = np.cumsum(rng.exponential(1.0 / cfg["rate"], size=nitems))
    kinds, sizes, offs, jidx = [], [], [], []
    for i in range(nitems):
        if i % cfg["pca_every"] == cfg["pca_every"] - 1:
            kinds.append(1)
            jidx.append(i // cfg["pca_every"] % len(jobs))
            sizes.append(0)
            offs.append(0)
        else:
            kinds.append(0)
            z = int(rng.integers(1, 2001))
            sizes.append(z)
            offs.append(int(rng.integers(0, npool - z + 1)))
            jidx.append(-1)
    # a burst: the stream opens with pca_burst full-PCA jobs offered at once, so that jobs
    # run side by side on the server's PCA workers while projections keep arriving
    nb = cfg.get("pca_burst", 0)
    if nb:
        arrivals = np.concatenate([np.zeros(nb), arrivals])
        kinds = [1] * nb + kinds
        jidx = [j % len(jobs) for j in range(nb)] + jidx
        sizes = [0] * nb + sizes
        offs = [0] * nb + offs
        nitems += nb
    done_t = [0.0] * nitems
    reqs = [None] * nitems
    ready = threading.Semaphore(0)
    errors = []

    def waiter():
        for i in range(nitems):
            ready.acquire()
            try:
                reqs[i].wait(900.0)
            except Exception as e:  # noqa: BLE001 - reported after the run
                errors.append(str(e))
            done_t[i] = time.perf_counter()

    th = threading.Thread(target=waiter)
    th.start()
    clocks = ClockSampler(local)
    clocks.start()
    ts = time.perf_counter()
    for i in range(nitems):
        while True:
            dt = ts + arrivals[i] - time.perf_counter()
            if dt <= 0:
                break
            time.sleep(min(dt, 0.001))
        if kinds[i]:
            jb = jobs[jidx[i]]
            reqs[i] = srv.submit_pca(jb["rec"], jb["n"], jopts)
        else:
            reqs[i] = srv.submit(rows[offs[i]:offs[i] + sizes[i]])
        ready.release()
    th.join()
    clk = clocks.stop()
    if errors:
        raise RuntimeError("mixed stream item failed: %s" % errors[0])
    span = max(done_t) - ts
    lat = np.array([(done_t[i] - (ts + arrivals[i])) * 1e3 for i in range(nitems)])
    kinds = np.array(kinds)
    split_evals = {}
    for i in range(nitems):
        if kinds[i] and jidx[i] not in split_evals:
            split_evals[jidx[i]] = reqs[i].args.collect()["evals"][:K2]
    done, peak, _ = srv.pca_stats()
    srv.close()
    # plain FP64 one item at a time: service times measured on the same GPU
    s64 = native.Server(h, cfg["K"], max_batch=2048, pool_samples=4096, fp64_serial=True)
    tt = time.perf_counter()
    z64 = 0
    for z in (500, 1000, 2000):
        s64.submit(rows[:z]).wait(600.0)
        z64 += z
    sps64 = z64 / (time.perf_counter() - tt)
    s64.close()
    o64 = native.default_opts(numeigs=K2, numoutliter=5, outlthresh=6.0,
                              precision=native.GP_PREC_FP64)
    t64, err = {}, {}
    for j, jb in enumerate(jobs):
        if j not in split_evals:
            continue
        h.timer_start()
        r64 = native.smartpca_run(h, jb["rec"], jb["n"], o64)
        t64[j] = h.timer_stop() / 1e3
        e64 = r64["evals"][:K2]
        err[j] = float(np.max(np.abs(split_evals[j] - e64) / np.abs(e64)))
    service = [sizes[i] / sps64 if not kinds[i] else t64[jidx[i]] for i in range(nitems)]
    lat64 = _serial_queue(arrivals, service) * 1e3
    span64 = max(float(np.sum(service)), float(arrivals[-1]))
    for jb in jobs:
        native.host_unregister(jb["rec"])
    native.host_unregister(rows)
    h.close()
    proj, pca = kinds == 0, kinds == 1
    nsamp = int(np.sum(np.array(sizes)[proj]))
    return {
        "items": nitems, "projection_requests": int(proj.sum()), "pca_jobs": int(pca.sum()),
        "span_s": span, "items_per_s": nitems / span, "samples_per_s": nsamp / span,
        "pca_jobs_per_s": int(pca.sum()) / span,
        "proj_p50_ms": float(np.percentile(lat[proj], 50)),
        "proj_p99_ms": float(np.percentile(lat[proj], 99)),
        "pca_p50_ms": float(np.percentile(lat[pca], 50)),
        "pca_p99_ms": float(np.percentile(lat[pca], 99)),
        "pca_peak_concurrent": peak,
        "jobs": [{"n": jb["n"], "m": jb["m"], "pops": jb["npop"], "miss": round(jb["miss"], 4),
                  "fp64_s": t64.get(j), "eval_max_rel_err_vs_fp64": err.get(j)}
                 for j, jb in enumerate(jobs)],
        "serial_fp64": {"span_s": span64, "items_per_s": nitems / span64,
                        "proj_p50_ms": float(np.percentile(lat64[proj], 50)),
                        "proj_p99_ms": float(np.percentile(lat64[proj], 99)),
                        "pca_p50_ms": float(np.percentile(lat64[pca], 50)),
                        "pca_p99_ms": float(np.percentile(lat64[pca], 99)),
                        "proj_samples_per_s": sps64,
                        "note": "measured FP64 service times, FIFO queue on the same arrivals"},
        "clocks": clk, "gen_s": gen_s}


def run_gpu(args, cfg, local):
    import torch

    from eig_gb300 import native
    torch.cuda.set_device(local)
    prec = native.PRECISIONS[args.precision]
    t0 = time.time()
    rec, pop = native.synth_records(cfg["nsnp"], cfg["pops"], cfg["fst"], miss=cfg["miss"],
                                    seed=cfg["seed"])
    nind = len(pop)
    gen_s = time.time() - t0
    h = native.Handle(local)
    h.load_genotypes(rec, nind)
    opts = native.default_opts(numeigs=cfg["K"], numoutliter=5, outlthresh=6.0,
                               precision=prec)
    resident = (rec.shape[0], rec.shape[1])

    def step(host):
        r = native.smartpca_run(h, rec if host else resident, nind, opts)
        return r

    # the Gram flops of a step: sum over passes of N_p (N_p + 1) M_p (recorded per gp_xtx)
    flops_holder = {}

    def one(host=False):
        h.timer_start()
        r = step(host)
        ms = h.timer_stop()
        return r, ms

    for _ in range(args.warmup):
        r, _ = one()
    # per-pass Gram flops from the final run's pass structure: re-derive from npasses
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    gram_ms = []
    tri_ms = []
    tri_n = 0
    total_flops = 0.0
    h.launch_count(reset=True)
    for _ in range(args.steps):
        torch.cuda.synchronize()
        r, ms = one()
        torch.cuda.synchronize()
        times.append(ms)
        g_ms, g_launch, g_flops = h.last_gram_time()
        gram_ms.append(g_ms)
        t_ms, tri_n = h.last_tridiag_time()
        tri_ms.append(t_ms)
        total_flops = r["gram_flops"]
    clk = clocks.stop()
    launches = h.launch_count(reset=True) / max(1, args.steps)
    step_ms = float(np.mean(times))
    # kernel (a): the per-SNP counts of the last pass
    c_ms, c_bytes = h.last_counts_time()
    # dominant kernel: the Gram of the last pass
    g_ms, g_launch, g_flops = h.last_gram_time()
    # e2e through the C ABI from pinned host memory (one untimed warm-up run first: it sizes
    # the upload's staging buffer, which the resident-panel steps do not use)
    native.host_register(rec)
    e2e_times = []
    step(True)
    torch.cuda.synchronize()
    h.transfer_bytes(reset=True)
    e2e_phases = []
    for _ in range(max(1, min(args.steps, args.e2e_steps))):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r2 = step(True)
        torch.cuda.synchronize()
        e2e_times.append((time.perf_counter() - t) * 1e3)
        e2e_phases.append({k: round(v * 1e3, 2) for k, v in r2["t_phase"].items()})
    h2d, d2h = h.transfer_bytes(reset=True)
    n_e2e = len(e2e_times)
    native.host_unregister(rec)
    e2e_ms = float(np.mean(e2e_times))
    # the split run's results and timing against one plain FP64 GPU run
    acc = None
    if not args.no_fp64_check and args.precision != "fp64":
        r_split = native.smartpca_run(h, resident, nind, opts)
        acc = accuracy_vs_fp64(h, resident, nind, cfg, r_split, step_ms)
    serving = None
    if not args.no_serving:
        r_split = native.smartpca_run(h, resident, nind, opts)  # leaves the K=20 panel resident
        serving = run_serving(h, cfg)
    h.close()
    peaks, peak_kind = load_peaks()
    res = dict(step_ms=step_ms, gram_flops=total_flops, gram_ms=g_ms, gram_launches=g_launch,
               tridiag_ms=float(np.mean(tri_ms)) if tri_ms else 0.0, tridiag_n=tri_n,
               gram_kernel_flops=g_flops, clocks=clk, e2e_ms=e2e_ms, e2e_runs_ms=e2e_times,
               e2e_phases=e2e_phases,
               h2d=h2d / n_e2e,
               d2h=d2h / n_e2e, run=r, gen_s=gen_s, peaks=peaks, peak_kind=peak_kind,
               nind=nind, launches=launches, acc=acc, serving=serving, counts=(c_ms, c_bytes))
    return res


def _fast_fst(cfg):
    rng = np.random.default_rng(cfg["fst_seed"])
    return list(rng.uniform(0.005, 0.05, size=len(cfg["pops"])))


def fast_flops(nind, nsnp, L, I):
    """algorithmic flops of kjg_fpca's products: N M L (6 I + 4)"""
    return float(nind) * nsnp * L * (6 * I + 4)


def run_fastmode(args, cfg, local):
    """fastmode at N=55,000 x M=500,000: split-fp16 exact tensor-core products with FP64
    orthogonalisation, against the FP64 path and a converged run (I=40)"""
    import torch

    from eig_gb300 import native
    torch.cuda.set_device(local)
    prec = native.PRECISIONS[args.precision]
    fst = _fast_fst(cfg)
    t0 = time.time()
    rec, pop = native.synth_records(cfg["nsnp"], cfg["pops"], fst, miss=cfg["miss"],
                                    n_admixed=cfg["n_admixed"], seed=cfg["seed"])
    nind = len(pop)
    gen_s = time.time() - t0
    K, L, I = cfg["K"], cfg["L"], cfg["I"]
    h = native.Handle(local)

    def load(host_pinned=False):
        h.load_genotypes(rec, nind)
        h.set_samples(np.arange(nind, dtype=np.int32))
        h.set_snps(np.arange(cfg["nsnp"], dtype=np.int32))

    load()
    for _ in range(args.warmup):
        h.fastpca(K, L, I, seed=cfg["seed"], precision=prec)
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    h.launch_count(reset=True)
    for _ in range(args.steps):
        torch.cuda.synchronize()
        h.timer_start()
        ev, V = h.fastpca(K, L, I, seed=cfg["seed"], precision=prec)
        times.append(h.timer_stop())
    clk = clocks.stop()
    launches = h.launch_count(reset=True) / max(1, args.steps)
    step_ms = float(np.mean(times))
    # e2e: upload of the packed records from pinned host memory + fastpca + read-back
    native.host_register(rec)
    h.transfer_bytes(reset=True)
    e2e, e2e_load = [], []
    for _ in range(max(1, min(args.steps, args.e2e_steps))):
        torch.cuda.synchronize()
        t = time.perf_counter()
        load()
        torch.cuda.synchronize()
        e2e_load.append((time.perf_counter() - t) * 1e3)
        h.fastpca(K, L, I, seed=cfg["seed"], precision=prec)
        torch.cuda.synchronize()
        e2e.append((time.perf_counter() - t) * 1e3)
    h2d, d2h = h.transfer_bytes(reset=True)
    native.host_unregister(rec)
    e2e_ms = float(np.mean(e2e))
    e2e_load_ms = float(np.mean(e2e_load))
    acc = {}
    if not args.no_fp64_check:
        h.timer_start()
        ev64, V64 = h.fastpca(K, L, I, seed=cfg["seed"], precision=native.GP_PREC_FP64)
        ms64 = h.timer_stop()
        # a converged Rayleigh-Ritz reference: FP64 products in block Krylov spaces of 41 and
        # 50 blocks (820 and 1,000 columns); the two agree to the figures reported
        evc, Vc = h.fastpca(K, L, 49, seed=cfg["seed"], precision=native.GP_PREC_FP64)
        evc40, Vc40 = h.fastpca(K, L, 40, seed=cfg["seed"], precision=native.GP_PREC_FP64)

        def per_vec(A, B):
            c = np.abs(np.sum(A * B, axis=1)) / np.sqrt(np.sum(A * A, axis=1) *
                                                          np.sum(B * B, axis=1))
            return [float(x) for x in np.degrees(np.arccos(np.clip(c, -1.0, 1.0)))]

        acc = {"fp64_fastmode_s": ms64 / 1e3, "split_speedup": ms64 / step_ms,
               "eval_rel_err_vs_fp64_fastmode": [float(x) for x in np.abs(ev - ev64) / ev64],
               "vec_angle_deg_vs_fp64_fastmode": per_vec(V, V64),
               "subspace_angle_deg_vs_fp64_fastmode": _subspace_angle_deg(V, V64),
               "converged_reference": "FP64 products, Rayleigh-Ritz on a block Krylov space "
                                      "of 50 blocks of L=20 (I=49, 1,000 columns)",
               "converged_check_I40_vs_I49": {
                   "eval_rel_diff": [float(x) for x in np.abs(evc40 - evc) / evc],
                   "vec_angle_deg": per_vec(Vc40, Vc)},
               "eval_rel_err_vs_converged": [float(x) for x in np.abs(ev - evc) / evc],
               "vec_angle_deg_vs_converged": per_vec(V, Vc),
               "subspace_angle_deg_vs_converged": _subspace_angle_deg(V, Vc)}
    h.close()
    flops = fast_flops(nind, cfg["nsnp"], L, I)
    n_e2e = len(e2e)
    return dict(step_ms=step_ms, flops=flops, clocks=clk, e2e_ms=e2e_ms, h2d=h2d / n_e2e,
                d2h=d2h / n_e2e, acc=acc, gen_s=gen_s, nind=nind, launches=launches, evals=ev,
                e2e_load_ms=e2e_load_ms)


def run_eig(args, cfg, local):
    """gp_eigvecs on the N=5,000 FP64 Gram of a small seeded panel (the Gram is rebuilt before
    every timed eigensolve, outside the timed region: the solver consumes it)"""
    import torch

    from eig_gb300 import native
    torch.cuda.set_device(local)
    rec, pop = native.synth_records(cfg["nsnp"], cfg["pops"], cfg["fst"], miss=cfg["miss"],
                                    seed=cfg["seed"])
    nind = len(pop)
    h = native.Handle(local)
    h.load_genotypes(rec, nind)
    h.set_samples(np.arange(nind, dtype=np.int32))
    h.set_snps(np.arange(cfg["nsnp"], dtype=np.int32))
    for _ in range(args.warmup):
        h.xtx(precision=native.GP_PREC_FP64)
        h.eigvecs(cfg["K"])
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    h.launch_count(reset=True)
    for _ in range(args.steps):
        h.xtx(precision=native.GP_PREC_FP64)
        torch.cuda.synchronize()
        h.launch_count(reset=True)
        h.timer_start()
        ev, V = h.eigvecs(cfg["K"])
        times.append(h.timer_stop())
    launches = h.launch_count(reset=True)
    clk = clocks.stop()
    h.close()
    return dict(ms=float(np.mean(times)), clocks=clk, launches=launches, nind=nind,
                top=[float(x) for x in ev[:5]])


def run_convertf(args, cfg, local):
    """convertf's record writer (gp_encode_records, packed -> bed) on the resident panel:
    device output timed by the kernel's CUDA events; e2e = pinned host records in, upload,
    encode, bed records back in pinned host memory"""
    import torch

    from eig_gb300 import native
    from oracle import convertf as CV
    from oracle import oracle as O
    torch.cuda.set_device(local)
    rec, pop = native.synth_records(cfg["nsnp"], cfg["pops"], cfg["fst"], miss=cfg["miss"],
                                    seed=cfg["seed"])
    nind = len(pop)
    M = cfg["nsnp"]
    fmt = native.GP_OUT_PACKEDPED
    rb = native.load_library().gp_record_bytes(fmt, nind)
    h = native.Handle(local)
    h.load_genotypes(rec, nind)
    snps = np.arange(M, dtype=np.int64)
    dev = torch.empty(M * rb, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        h.encode_records(fmt, snps, None, None, nsamples=nind, out=dev.data_ptr())
    clocks = ClockSampler(local)
    clocks.start()
    kern, wall = [], []
    h.launch_count(reset=True)
    for _ in range(args.steps):
        torch.cuda.synchronize()
        h.timer_start()
        h.encode_records(fmt, snps, None, None, nsamples=nind, out=dev.data_ptr())
        wall.append(h.timer_stop())
        kern.append(h.last_encode_time())
    clk = clocks.stop()
    launches = h.launch_count(reset=True) / max(1, args.steps)
    alg = float(M) * (rec.shape[1] + rb)  # one read of each input record, one write of each output
    # e2e through the C ABI: pinned host records -> device -> bed records in pinned host memory
    out = np.empty((M, rb), np.uint8)
    native.host_register(rec)
    native.host_register(out)
    h.transfer_bytes(reset=True)
    e2e = []
    for _ in range(max(1, min(args.steps, args.e2e_steps))):
        torch.cuda.synchronize()
        t = time.perf_counter()
        h.load_genotypes(rec, nind)
        native.load_library().gp_encode_records(h.h, fmt, None, nind,
                                                snps.ctypes.data_as(native.i64p), None, M,
                                                out.ctypes.data, 0)
        e2e.append(time.perf_counter() - t)
    h2d, d2h = h.transfer_bytes(reset=True)
    native.host_unregister(out)
    native.host_unregister(rec)
    ok = bool(np.array_equal(out.reshape(-1), dev.cpu().numpy()))
    # CPU: the oracle's writer (unpack + outpackped restated in numpy, 1 thread) on a sample
    ms = 20000
    t = time.perf_counter()
    CV.encode(O.unpack(rec[:ms], nind), "PACKEDPED", header=False)
    cpu_dt = time.perf_counter() - t
    cpu_val = ms * (rec.shape[1] + rb) / cpu_dt / 1e9
    h.close()
    n_e2e = len(e2e)
    return dict(kern_ms=float(np.mean(kern)), wall_ms=float(np.mean(wall)), alg=alg,
                e2e_s=float(np.mean(e2e)), h2d=h2d / n_e2e, d2h=d2h / n_e2e, clocks=clk,
                launches=launches, nind=nind, ok=ok, cpu=(cpu_val, ms, cpu_dt))


def reference_flow(cfg, msnp, steps=1, warmup=0, eig_order=None, nthreads=None):
    """The reference smartpca flow on the host cores (oracle/reference_flow.py): counts and
    filters, the partial-sum lookup Gram (all threads), LAPACK dspev, SNP weights and
    lsqproject of every sample, over an msnp-SNP sample of the workload's panel (generated by
    the oracle's own numpy Balding-Nichols generator, so nothing of this library is loaded).
    The eigensolve runs once, at the workload's order (or at eig_order and scaled by the cube
    of the order ratio); each step times the per-SNP phases of the sample.  Returns the
    per-step records and the whole-workload figures."""
    from oracle import reference_flow as RF
    nthreads = nthreads or os.cpu_count() or 1
    pops = list(cfg["pops"])
    nind = sum(pops) + cfg.get("n_admixed", 0)
    fst = cfg.get("fst") or _fast_fst(cfg)
    K, M = cfg["K"], cfg["nsnp"]
    rec = RF.bn_records(msnp, pops, fst, cfg["miss"], cfg["seed"] + 5000,
                        n_admixed=cfg.get("n_admixed", 0))
    t, s, X = RF.gram_phases(rec, nind, nthreads)
    n_e = nind if eig_order is None else min(eig_order, nind)
    eig_meas, V = RF.eig_phase(X[:n_e, :n_e])
    eig_s = eig_meas * (nind / n_e) ** 3
    if n_e < nind:
        V = np.linalg.eigh(X)[1][:, ::-1].T    # vectors for the weights (not timed)
    kept_frac = float((s.killed == 0).sum()) / msnp
    recs = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        tg, s, X = RF.gram_phases(rec, nind, nthreads)
        tp = RF.projection_phases(s, V, K)
        wall = time.perf_counter() - t0
        if i >= warmup:
            ph = dict(tg, **tp)
            per_snp = sum(ph.values()) / msnp
            whole = RF.whole_flow_seconds(per_snp, M, eig_s)
            recs.append(dict(wall=wall, phases=ph, whole_s=whole,
                             value=nind * (nind + 1.0) * M * kept_frac / whole / 1e12))
    ph_mean = {k: float(np.mean([r["phases"][k] for r in recs])) for k in recs[0]["phases"]}
    whole = float(np.mean([r["whole_s"] for r in recs]))
    return dict(recs=recs, value=float(np.mean([r["value"] for r in recs])), nthreads=nthreads,
                nind=nind, msnp=msnp, eig_s=eig_s, eig_meas_s=eig_meas, eig_order=n_e,
                whole_s=whole, phases_sample_s=ph_mean,
                phases_full_s=dict({k: v / msnp * M for k, v in ph_mean.items()}, eig=eig_s),
                step_s=float(np.mean([r["wall"] for r in recs])))


def reference_sample_text(rf, M):
    eig = ("LAPACK dspev at order %d (%.1f s)" % (rf["eig_order"], rf["eig_meas_s"])
           if rf["eig_order"] == rf["nind"] else
           "LAPACK dspev at order %d (%.1f s) scaled by (%d/%d)^3" % (
               rf["eig_order"], rf["eig_meas_s"], rf["nind"], rf["eig_order"]))
    return ("reference smartpca flow restated (counts/filters, partial-sum lookup Gram on %d "
            "threads, weights, lsqproject of all samples; one thread where the reference has "
            "one) over an N=%d x M=%d SNP sample (%.1f s per step), scaled to M=%d, plus %s; "
            "one pass: %.0f s" % (rf["nthreads"], rf["nind"], rf["msnp"], rf["step_s"], M, eig,
                                  rf["whole_s"]))


def tridiag_traffic(n):
    """DRAM bytes of one k_tridiag_tiled launch of order n from the committed ncu summary
    (profiles/tridiag_tiled_5000_dram.md), or None for other orders"""
    path = os.path.join(ROOT, "profiles", "tridiag_tiled_5000_dram.md")
    if n != 5000 or not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            return int(line.split(":")[1])
    return None


def tridiag_roofline(res, peaks, peak_kind):
    """roofline of the step's dominant kernel, the float-float tridiagonalisation: HBM-bound;
    algorithmic bytes = LAPACK dsytd2's fused symv + syr2 pass, which reads and writes the
    trailing lower triangle once per column step (8-byte elements):
    sum over m = 1 .. n-1 of 8 m (m + 1) = 8 (n-1) n (n+1) / 3 bytes per launch"""
    n, ms = res.get("tridiag_n", 0), res.get("tridiag_ms", 0.0)
    if not n or ms <= 0.0:
        return None
    alg = 8.0 * (n - 1) * n * (n + 1) / 3.0
    achieved = alg / (ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs", 6800.0)
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": tridiag_traffic(n),
            "kernel": "k_tridiag_tiled (float-float Householder tridiagonalisation, order %d, "
                      "one cooperative launch: lower-triangle tiles while the trailing order "
                      "exceeds 2,500, then whole columns; %.1f ms by CUDA events)" % (n, ms),
            "algorithmic_bytes": alg,
            "note": "DRAM traffic is below the algorithmic bytes: the tiled lower triangle "
                    "(103 MB at N=5,000) mostly stays in L2; the tiled steps are bound by "
                    "the per-step chain of phase A, part sums and the grid barrier, and FP32-pipe "
                    "issue (~62 instructions per lower-triangle element and step)",
            "peak_kind": "HBM copy, %s" % peak_kind}


def unpack_roofline(res, peaks):
    """kernel (a), the per-SNP counts / kill rule / value table of the last pass (k_snp_stats):
    HBM-bound; algorithmic bytes = one read of each selected record and the row mask plus the
    61 bytes of counts and tables written per SNP, over its CUDA-event time"""
    ms, nbytes = res.get("counts", (0.0, 0))
    if ms <= 0.0 or nbytes <= 0:
        return None
    achieved = nbytes / (ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs", 6800.0)
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": None,
            "kernel": "k_snp_stats (per-SNP counts and normalisation, %.3f ms by CUDA events)" % ms,
            "algorithmic_bytes": nbytes,
            "traffic_note": "DRAM bytes of an ncu capture at 200,000 SNPs: "
                            "profiles/snp_stats_5000x200000.md"}


def gram_traffic(args):
    """DRAM bytes per launch of the split Gram kernel from the committed ncu summary of the
    full workload (profiles/gram_split_fp16_full_dram.md, one-CTA schedule), or None for other
    workloads and for the cluster schedule (not captured: profiler replay of the cluster launch
    is not used)"""
    if args.config != "full" or args.precision != "fp16":
        return None
    if os.environ.get("GP_GRAM_CLUSTER", "4") != "1":
        return None
    p = os.path.join(ROOT, "profiles", "gram_split_fp16_full_dram.md")
    try:
        for line in open(p):
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--precision", default="fp16", choices=["fp64", "bf16", "bf16x4", "fp16"])
    ap.add_argument("--config", default="full", choices=list(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    args = ap.parse_args()
    cfg = CONFIGS[args.config]
    world, rank, local = launch_shape(args)
    nind = sum(cfg["pops"]) + cfg.get("n_admixed", 0)
    config = {"workload": cfg["name"], "nsamples": nind, "nsnps": cfg["nsnp"],
              "numeigs": cfg["K"], "parallelism": "one GPU",
              "l2": "inputs larger than L2 (packed panel %.0f MB)" % (
                  cfg["nsnp"] * max((nind + 3) // 4, 48) / 1e6)}
    if args.impl == "gpu" and world > 1:
        # one GPU only: no multi-GPU path exists (and the split Gram's cluster schedule must not
        # run in a multi-GPU process group); nothing touches a GPU here
        if rank == 0:
            print(json.dumps({"metric": METRIC, "n_gpus": world, "impl": "gpu",
                              "unavailable": "one GPU only: smartpca's path runs one PCA per "
                                             "panel on one GPU; no multi-GPU mode is built",
                              "config": config}))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        cfg_ref = CONFIGS["full"] if args.config not in ("full", "small") else cfg
        rf = reference_flow(cfg_ref, msnp=2000, steps=args.steps, warmup=args.warmup)
        value = rf["value"]
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "impl": "reference",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": rf["step_s"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic (seeded Balding-Nichols)", "config": config,
                "pca_wall_s": rf["whole_s"],
                "phases_s": {k: round(v, 3) for k, v in rf["phases_full_s"].items()},
                "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": rf["nthreads"],
                                 "kind": "port",
                                 "sample": reference_sample_text(rf, cfg_ref["nsnp"])},
                "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "note": "value = whole-job XTX throughput of one reference smartpca pass over "
                        "the full workload (per-SNP phases measured on the sample each step and "
                        "scaled to all SNPs, plus the eigensolve measured at the full order); "
                        "ms_per_step is the measured sample step"}
        print(json.dumps(line))
        return

    if args.config == "mixed":
        res = run_mixed(args, cfg, local)
        line = {"metric": "mixed serving: items/s and p50/p99 latency vs serial plain FP64",
                "value": res["items_per_s"], "unit": "items/s", "n_gpus": 1,
                "steps": 1, "warmup": 1, "ms_per_step": res["span_s"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "split fp16 Gram + exact tensor-core products, FP64 eigensolve",
                "data": "synthetic (seeded Balding-Nichols)", "config": config,
                "mixed": res, "clocks": res["clocks"]}
        if rank == 0:
            print(json.dumps(line))
        return
    if args.config == "eig":
        res = run_eig(args, cfg, local)
        line = {"metric": "dense FP64 eigensolve wall ms (all eigenvalues + top 20 vectors)",
                "value": res["ms"], "unit": "ms", "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64 (float-float reduction)",
                "data": "synthetic (seeded Balding-Nichols)",
                "config": dict(config, nsamples=res["nind"],
                               l2="the N x N FP64 Gram (200 MB at N=5000) is larger than L2 "
                                  "and is rebuilt before each timed solve"),
                "top_evals": res["top"],
                "clocks": res["clocks"], "gpu_launches": res["launches"]}
        if rank == 0:
            print(json.dumps(line))
        return
    if args.config == "convertf":
        res = run_convertf(args, cfg, local)
        peaks, kind = load_peaks()
        achieved = res["alg"] / (res["kern_ms"] * 1e-3) / 1e9
        line = {"metric": "convertf record conversion GB/s (input + output records)",
                "value": achieved, "unit": "GB/s", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["kern_ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u8", "data": "synthetic (seeded Balding-Nichols)",
                "config": dict(config, numeigs=None, output="PACKEDPED"),
                "call_ms": res["wall_ms"], "matches_host_path": res["ok"],
                "roofline": {"bound": "hbm", "achieved": achieved,
                             "peak": peaks.get("hbm_gbs", 6800.0), "unit": "GB/s",
                             "frac": achieved / peaks.get("hbm_gbs", 6800.0), "traffic": None,
                             "peak_kind": "HBM copy, %s" % kind,
                             "kernels": "k_encode<PACKEDPED> (algorithmic M x (rlen_in + "
                                        "rlen_out) bytes)"},
                "clocks": res["clocks"],
                "e2e": {"value": res["alg"] / res["e2e_s"] / 1e9, "unit": "GB/s",
                        "h2d_bytes_per_step": int(res["h2d"]),
                        "d2h_bytes_per_step": int(res["d2h"]), "wall_s": res["e2e_s"]},
                "cpu_baseline": {"value": res["cpu"][0], "unit": "GB/s", "cores": 1,
                                 "kind": "port",
                                 "sample": "numpy restatement of outpackped (unpack + encode), "
                                           "%d SNPs x %d samples, %.2f s" % (
                                               res["cpu"][1], res["nind"], res["cpu"][2])},
                "gpu_launches": res["launches"]}
        if rank == 0:
            print(json.dumps(line))
        return
    if args.config == "fastmode":
        res = run_fastmode(args, cfg, local)
        value = res["flops"] / (res["step_ms"] * 1e-3) / 1e12
        config["nsamples"] = res["nind"]
        line = {"metric": "fastmode wall-s & algorithmic TFLOP/s N*M*L*(6I+4)", "value": value,
                "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["step_ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "exact fp16-sliced tensor-core products, FP64 block Gram-Schmidt / "
                         "Rayleigh-Ritz",
                "data": "synthetic (seeded Balding-Nichols)", "config": config,
                "fastmode_wall_s": res["step_ms"] / 1e3, "accuracy": res["acc"],
                "top_evals": [float(x) for x in res["evals"]], "clocks": res["clocks"],
                "e2e": {"value": res["flops"] / (res["e2e_ms"] * 1e-3) / 1e12,
                        "unit": "TFLOP/s", "h2d_bytes_per_step": int(res["h2d"]),
                        "d2h_bytes_per_step": int(res["d2h"]), "wall_s": res["e2e_ms"] / 1e3,
                        "upload_and_setup_s": res["e2e_load_ms"] / 1e3},
                "gpu_launches": res["launches"]}
        if rank == 0:
            print(json.dumps(line))
        return
    res = run_gpu(args, cfg, local)
    r = res["run"]
    value = res["gram_flops"] / (res["step_ms"] * 1e-3) / 1e12
    e2e = res["gram_flops"] / (res["e2e_ms"] * 1e-3) / 1e12
    peaks = res["peaks"]
    if args.precision != "fp64":
        achieved = res["gram_kernel_flops"] / (res["gram_ms"] * 1e-3) / 1e12
        peak = peaks.get("bf16_tflops", 1900.0)
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": gram_traffic(args),
                "peak_kind": "bf16 burst, %s" % res["peak_kind"],
                "kernels": "k_split_transpose + k_gram_split (algorithmic N(N+1)M flop; the "
                           "split scheme issues 3 MMAs per algorithmic FMA)",
                "traffic_note": "DRAM bytes of the one-CTA schedule from "
                                "profiles/gram_split_fp16_full_dram.md when GP_GRAM_CLUSTER=1; "
                                "not captured for the cluster schedule"}
    else:
        achieved = res["gram_kernel_flops"] / (res["gram_ms"] * 1e-3) / 1e12
        roof = {"bound": "fp64", "achieved": achieved, "peak": 1.25, "unit": "TFLOP/s",
                "frac": achieved / 1.25, "traffic": None,
                "peak_kind": "nominal GB300 FP64 1.25 TFLOP/s (not in the measured peaks)"}
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["step_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "bf16": "bf16 hi+lo x3 MMA (fp32 in chunk, fp64 across)",
                      "bf16x4": "bf16 hi+lo x4 MMA (fp32 in chunk, fp64 across)",
                      "fp16": "fp16 hi+lo x3 MMA (fp32 in chunk, fp64 across)"}[args.precision],
            "data": "synthetic (seeded Balding-Nichols)", "config": config,
            "pca_wall_s": res["step_ms"] / 1e3,
            "phases_s": {k: round(v, 4) for k, v in r["t_phase"].items()},
            "passes": r["npasses"], "outliers": len(r["outliers"]),
            "gram_kernel_ms": res["gram_ms"],
            "roofline": tridiag_roofline(res, peaks, res["peak_kind"]) or roof,
            "roofline_gram": roof, "roofline_unpack": unpack_roofline(res, peaks),
            "clocks": res["clocks"],
            "e2e": {"value": e2e, "unit": "TFLOP/s", "h2d_bytes_per_step": int(res["h2d"]),
                    "d2h_bytes_per_step": int(res["d2h"]), "wall_s": res["e2e_ms"] / 1e3,
                    "runs_ms": [round(x, 2) for x in res["e2e_runs_ms"]],
                    "runs_phases_ms": res["e2e_phases"]},
            "accuracy_vs_fp64": res["acc"], "serving": res["serving"],
            "gpu_launches": res["launches"],
            "gpu_launches_note": "own kernels per timed step (all kernels of the step are this "
                                 "library's; cuSOLVER sytrd/ormtr only serve N > 8,533)"}
    if rank == 0 and not args.no_cpu_baseline:
        rf = reference_flow(cfg, msnp=1000, eig_order=2000)
        line["cpu_baseline"] = {"value": rf["value"], "unit": "TFLOP/s",
                                "cores": rf["nthreads"], "kind": "port",
                                "sample": reference_sample_text(rf, cfg["nsnp"]),
                                "pass_s": rf["whole_s"],
                                "phases_s": {k: round(v, 3) for k, v in
                                             rf["phases_full_s"].items()}}
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()

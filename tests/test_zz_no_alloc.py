"""The no-allocation Gram entry point (gp_gram_fp64_noalloc).

Some callers cannot allocate device memory: a serving process whose memory manager already
reserved the whole GPU for its own pool, or a latency-critical loop that must not call
cudaMalloc/cudaFree because they can synchronise the device.  This entry point takes only
caller-owned device buffers and keeps its split-K scratch in a fixed 16 MiB array inside the
library.  The test calls it twice in a row through the C ABI on the same inputs and compares
each result with the Gram of the regular entry point gp_xtx (same tolerance as the other FP64
Gram tests: 1e-12 of the largest entry).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_gram_matches_gp_xtx_on_two_calls():
    torch = pytest.importorskip("torch")
    from eig_gb300 import native
    from oracle import oracle as O

    nsnp = 2500
    rec, pop = native.synth_records(nsnp, [200, 200, 170], [0.01, 0.03, 0.05], miss=0.02,
                                    seed=41, nthreads=4)
    nind = len(pop)
    rows = np.arange(nind, dtype=np.int32)
    cols = np.arange(nsnp, dtype=np.int32)
    with native.Handle(0) as h:
        h.load_genotypes(rec, nind)
        h.set_samples(rows)
        h.set_snps(cols)
        ref = h.xtx()["XTX"]
    vtab = O.pass_columns(rec, cols, rows).tab  # the table gp_xtx builds (bit-identical)
    lib = native.load_library()
    dev = torch.device("cuda", 0)
    d_rec = torch.from_numpy(rec).to(dev)
    d_vtab = torch.from_numpy(vtab).to(dev)
    d_x = torch.empty((nind, nind), dtype=torch.float64, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    scale = np.max(np.abs(ref))
    for _ in range(2):
        d_x.fill_(float("nan"))
        rc = lib.gp_gram_fp64_noalloc(C.c_void_p(d_rec.data_ptr()), rec.shape[1], nind, nsnp,
                                      C.c_void_p(d_vtab.data_ptr()), C.c_void_p(d_x.data_ptr()),
                                      stream)
        torch.cuda.synchronize(dev)
        assert rc == 0, lib.gp_noalloc_last_error().decode()
        X = d_x.cpu().numpy()
        assert np.all(np.isfinite(X))
        assert np.max(np.abs(X - ref)) <= 1e-12 * scale


def test_noalloc_rejects_panels_over_the_limit():
    torch = pytest.importorskip("torch")
    from eig_gb300 import native
    lib = native.load_library()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(1024, dtype=torch.float64, device=dev)
    p = C.c_void_p(buf.data_ptr())
    rc = lib.gp_gram_fp64_noalloc(p, 300, 1025, 10, p, p, None)
    assert rc == -1  # GP_ERR_ARG
    assert b"1024" in lib.gp_noalloc_last_error()

"""fastmode on the GPU against the reference's own fastmode (kjg_fpca built against the GSL
shim, tests/golden/bn_fastmode): Omega drawn from GSL's mt19937 with the parfile's seed inside
the library, the Krylov products on the GPU (FP64 SIMT or exact tensor-core products), the
block Gram-Schmidt basis and Rayleigh-Ritz step on the library's own FP64 kernels.
Eigenvalues within 1e-9 relative, eigenvectors equal up to sign (|cos| > 1 - 1e-9); the
gpusmartpca CLI prints the reference's .evec text (up to eigenvector signs).  A block Krylov
space of 41 blocks stays orthonormal and reaches the exact eigenpairs."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O
from tests.goldens import FastCase

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [native.GP_PREC_FP64, native.GP_PREC_SPLIT_FP16])
@pytest.mark.parametrize("par", ["par", "par_odd"])
def test_fastpca_matches_reference_fastmode(gpu, prec, par):
    fc = FastCase()
    r = fc.run(par)
    gpu.load_genotypes(fc.records, fc.nind)
    gpu.set_samples(np.arange(fc.nind, dtype=np.int32))
    gpu.set_snps(np.arange(fc.nsnp, dtype=np.int32))
    ev, V = gpu.fastpca(r["K"], r["L"], r["I"], seed=r["seed"], precision=prec)
    assert np.max(np.abs(ev - r["evals"]) / r["evals"]) <= 1e-9, (ev, r["evals"])
    Vn = V / np.linalg.norm(V, axis=1, keepdims=True)
    cos = np.abs(np.sum(Vn * r["evecs"], axis=1)) / np.linalg.norm(r["evecs"], axis=1)
    assert np.all(cos > 1 - 1e-9), cos


@pytest.mark.parametrize("par", ["par", "par_odd"])
def test_cli_fastmode_matches_reference_text(tmp_path, par):
    fc = FastCase()
    r = fc.run(par)
    d = tmp_path / "bn_fastmode"
    shutil.copytree(fc.dir, d)
    cli = os.path.join(native.LIB_DIR, "gpusmartpca")
    out = subprocess.run([cli, "-p", par], cwd=d, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr + out.stdout
    from tests.goldens import progress_lines
    ref_log = "ref.log" if par == "par" else "ref_odd.log"
    assert progress_lines(out.stdout) == progress_lines(open(d / ref_log).read())
    mine = open(d / "out.evec").read().splitlines()
    want = r["text"]
    assert len(mine) == len(want)
    assert mine[0] == want[0]
    A = np.array([[float(x) for x in l.split()[1:-1]] for l in want[1:]])
    B = np.array([[float(x) for x in l.split()[1:-1]] for l in mine[1:]])
    assert [l.split()[0] for l in mine[1:]] == [l.split()[0] for l in want[1:]]
    assert [l.split()[-1] for l in mine[1:]] == [l.split()[-1] for l in want[1:]]
    s = np.sign(np.sum(A * B, axis=0))
    assert np.max(np.abs(A - B * s)) <= 1.01e-4


@pytest.mark.parametrize("prec", [native.GP_PREC_FP64, native.GP_PREC_SPLIT_FP16])
def test_fastpca_long_krylov_reaches_exact_eigenpairs(gpu, prec):
    """10 populations of 60 plus 60 admixed samples, K=10, L=20 and I=40 (820 columns, far
    more than the space has independent directions): the basis stays orthonormal through the
    dependent blocks, and all ten Ritz pairs, the bulk tenth included, match the exact
    eigenpairs of X^T X / M from LAPACK on the host (1e-9 relative, |cos| > 1 - 1e-9)"""
    rng = np.random.default_rng(3)
    rec, pop = native.synth_records(6000, [60] * 10, list(rng.uniform(0.005, 0.05, size=10)),
                                    miss=0.01, n_admixed=60, seed=9, nthreads=4)
    nind, nsnp = len(pop), 6000
    gpu.load_genotypes(rec, nind)
    gpu.set_samples(np.arange(nind, dtype=np.int32))
    gpu.set_snps(np.arange(nsnp, dtype=np.int32))
    ev, V = gpu.fastpca(10, 20, 40, seed=7, precision=prec)
    s = O.pass_columns(rec, np.arange(nsnp, dtype=np.int32), np.arange(nind, dtype=np.int32),
                       minallelecnt=0, maxmissing=2 ** 31 - 1)
    w, U = np.linalg.eigh(O.gram(s) / (2.0 * nsnp))
    w, U = w[::-1][:10], U[:, ::-1][:, :10].T
    assert np.max(np.abs(ev - w) / w) <= 1e-9, (ev, w)
    cos = np.abs(np.sum(V * U, axis=1)) / np.linalg.norm(V, axis=1)
    assert np.all(cos > 1 - 1e-9), cos

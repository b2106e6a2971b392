"""convertf's genotype writers on the GPU (gp_encode_records, gpuconvertf) against the
reference convertf's files and the oracle restatement (oracle/convertf.py)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from eig_gb300 import native
from oracle import convertf as CV
from oracle import oracle as O
from tests.goldens import GOLDEN

pytestmark = pytest.mark.gpu

FMTS = {"PACKEDANCESTRYMAP": native.GP_OUT_PACKEDANCESTRYMAP,
        "PACKEDPED": native.GP_OUT_PACKEDPED, "EIGENSTRAT": native.GP_OUT_EIGENSTRAT}


@pytest.mark.parametrize("run", ["pk2pk", "pk2bed", "pk2es", "bed2pk", "bed2es"])
def test_cli_convertf_byte_identical_to_reference(run, tmp_path):
    d = tmp_path / "cv"
    shutil.copytree(os.path.join(GOLDEN, "cv_edge"), d)
    for ext in ("geno", "snp", "ind"):
        os.rename(d / ("out_%s.%s" % (run, ext)), d / ("ref_%s.%s" % (run, ext)))
    cli = os.path.join(native.LIB_DIR, "gpuconvertf")
    out = subprocess.run([cli, "-p", "par_" + run], cwd=d, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr + out.stdout
    for ext in ("geno", "snp", "ind"):
        mine = open(d / ("out_%s.%s" % (run, ext)), "rb").read()
        ref = open(d / ("ref_%s.%s" % (run, ext)), "rb").read()
        assert mine == ref, ext


@pytest.mark.parametrize("fmt", list(FMTS))
@pytest.mark.parametrize("nind", [1001, 150, 7])
def test_encode_records_vs_oracle(gpu, fmt, nind):
    """shuffled sample subsets, flips, odd sample counts (partial last byte, 48-byte packed
    minimum): the records equal the oracle's encoder"""
    rng = np.random.default_rng(nind)
    nsnp = 3000
    g = rng.integers(0, 3, (nsnp, nind)).astype(np.int16)
    g[rng.random((nsnp, nind)) < 0.1] = -1
    rec = O.pack(g)
    gpu.load_genotypes(rec, nind)
    snps = rng.choice(nsnp, 2000, replace=False)
    flip = (rng.random(2000) < 0.3).astype(np.uint8)
    samples = rng.permutation(nind)[: max(1, nind - 3)]
    got = gpu.encode_records(FMTS[fmt], snps, samples, flip)
    sub = g[snps][:, samples].copy()
    f = flip.astype(bool)
    sub[f] = np.where(sub[f] < 0, -1, 2 - sub[f])
    want = CV.encode(sub, fmt, header=False)
    assert got.tobytes() == want
    # identity sample list (the per-byte path) without flips
    got = gpu.encode_records(FMTS[fmt], snps, None, None, nsamples=nind)
    assert got.tobytes() == CV.encode(g[snps], fmt, header=False)


def test_encode_full_size_round_trip(gpu):
    """N=5,000 x M=60,000 packed -> bed -> packed through the device: the panel comes back
    bit for bit (bed loaded with GP_CODE_BED), on the device-output path too"""
    import torch
    rec, pop = native.synth_records(60000, [2000, 2000, 1000], [0.01, 0.02, 0.03], miss=0.02,
                                    seed=71, nthreads=8)
    nind = len(pop)
    gpu.load_genotypes(rec, nind)
    snps = np.arange(60000)
    bed = gpu.encode_records(native.GP_OUT_PACKEDPED, snps, None, None, nsamples=nind)
    dev = torch.empty(bed.size, dtype=torch.uint8, device="cuda")
    gpu.encode_records(native.GP_OUT_PACKEDPED, snps, None, None, nsamples=nind,
                       out=dev.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), bed.reshape(-1))
    gpu.load_genotypes(bed, nind, code=native.GP_CODE_BED)
    back = gpu.encode_records(native.GP_OUT_PACKEDANCESTRYMAP, snps, None, None, nsamples=nind)
    rlen = back.shape[1]
    assert np.array_equal(O.unpack(back, nind), O.unpack(rec[:, :rlen], nind))


def test_encode_rejects_out_of_range(gpu):
    rec = O.pack(np.zeros((10, 20), np.int16))
    gpu.load_genotypes(rec, 20)
    with pytest.raises(native.GpuError):
        gpu.encode_records(native.GP_OUT_PACKEDPED, [0, 10], None, None, nsamples=20)
    with pytest.raises(native.GpuError):
        gpu.encode_records(native.GP_OUT_PACKEDPED, [0], [0, 20])
    with pytest.raises(native.GpuError):
        gpu.encode_records(7, [0], None, None, nsamples=20)


def test_encode_wide_records_direct_kernel(gpu):
    """EIGENSTRAT records wider than shared memory (210,001 bytes) take the per-warp kernel"""
    rng = np.random.default_rng(5)
    nind, nsnp = 210_000, 6
    g = rng.integers(0, 3, (nsnp, nind)).astype(np.int16)
    g[rng.random((nsnp, nind)) < 0.2] = -1
    gpu.load_genotypes(O.pack(g), nind)
    flip = np.array([0, 1, 0, 1, 1, 0], np.uint8)
    got = gpu.encode_records(native.GP_OUT_EIGENSTRAT, np.arange(nsnp), None, flip,
                             nsamples=nind)
    sub = g.copy()
    f = flip.astype(bool)
    sub[f] = np.where(sub[f] < 0, -1, 2 - sub[f])
    assert got.tobytes() == CV.encode(sub, "EIGENSTRAT", header=False)

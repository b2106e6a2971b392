"""Host-side failure handling of the drop-in CLI, injected on the host (no GPU involved): the
reference's fatalx cases for the input files (packed header, the header's hashes of the
sample and SNP files, a short genotype file, a missing file) and the options this path
refuses.  Each must end with a non-zero status and the message, before any device is opened.
"""
import os
import shutil
import subprocess

import pytest

from tests.goldens import GOLDEN

CASE = "bn_outliers"


def _cli():
    from eig_gb300 import native
    path = os.path.join(native.LIB_DIR, "gpusmartpca")
    if not os.path.exists(path):
        pytest.skip("gpusmartpca is not built")
    return path


def _case(tmp_path):
    d = tmp_path / CASE
    shutil.copytree(os.path.join(GOLDEN, CASE), d)
    return d


def _run(d, par="par"):
    return subprocess.run([_cli(), "-p", par], cwd=d, capture_output=True, text=True, timeout=120)


def test_bad_packed_header(tmp_path):
    d = _case(tmp_path)
    raw = bytearray(open(d / "data.geno", "rb").read())
    raw[5:12] = b"garbage"  # "GENO %7d ..." no longer parses
    open(d / "data.geno", "wb").write(bytes(raw))
    out = _run(d)
    assert out.returncode != 0
    assert "bad packed header" in out.stderr


def test_sample_file_changed_since_genotypes(tmp_path):
    """hashcheck: the header's hash of the sample IDs no longer matches"""
    d = _case(tmp_path)
    lines = open(d / "data.ind").read().splitlines()
    first = lines[0].split()
    first[0] = first[0] + "x"
    lines[0] = " ".join(first)
    open(d / "data.ind", "w").write("\n".join(lines) + "\n")
    out = _run(d)
    assert out.returncode != 0
    assert "sample file has changed" in out.stderr
    # hashcheck: NO skips the check (and the run then needs a GPU, so stop at the check)
    par = open(d / "par").read() + "hashcheck: NO\n"
    open(d / "par_nohash", "w").write(par)
    out2 = _run(d, "par_nohash")
    assert "sample file has changed" not in out2.stderr


def test_short_genotype_file(tmp_path):
    d = _case(tmp_path)
    raw = open(d / "data.geno", "rb").read()
    open(d / "data.geno", "wb").write(raw[: len(raw) - 1000])
    out = _run(d)
    assert out.returncode != 0
    assert "is short" in out.stderr


def test_missing_genotype_file(tmp_path):
    d = _case(tmp_path)
    os.remove(d / "data.geno")
    out = _run(d)
    assert out.returncode != 0
    assert "cannot open genotype file" in out.stderr


def test_refused_options(tmp_path):
    d = _case(tmp_path)
    for extra, msg in (("ldregress: 2\n", "ldregress is not supported"),
                       ("gpuprecision: FP32\n", "is not FP64"),
                       ("usepopsformissing: YES\nfastmode: YES\n",
                        "usepopsformissing with fastmode")):
        open(d / "par_x", "w").write(open(d / "par").read() + extra)
        out = _run(d, "par_x")
        assert out.returncode != 0, extra
        assert msg in out.stderr, (extra, out.stderr)


def test_missing_parfile(tmp_path):
    d = _case(tmp_path)
    out = _run(d, "no_such_par")
    assert out.returncode != 0
    assert "can't open" in out.stderr

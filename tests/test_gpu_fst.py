"""The Fst tail on the GPU (per-population counts on the device, gp_fst) and the log section
of gpusmartpca against the reference's logs and Fst files (tests/golden)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from eig_gb300 import native
from oracle import oracle as O
from tests.goldens import CASES, Case, eglist, log_section, read_fstdetails, snp_table

pytestmark = pytest.mark.gpu


def _run_cli(case, par_name, tmp_path):
    d = tmp_path / case
    shutil.copytree(Case(case).dir, d)
    cli = os.path.join(native.LIB_DIR, "gpusmartpca")
    out = subprocess.run([cli, "-p", par_name], cwd=d, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr + out.stdout
    return d, out.stdout


@pytest.mark.parametrize("case,par_name,ref_log", [(c, "par", "ref.log") for c in CASES] +
                         [("bn_fst", "par", "ref.log"), ("bn_fst", "par_pl", "ref_par_pl.log")])
def test_cli_fst_log_section_matches_reference(case, par_name, ref_log, tmp_path):
    """population sizes, block count, Fst lines / matrices and standard errors: the same text
    as the reference's log"""
    d, stdout = _run_cli(case, par_name, tmp_path)
    want = log_section(open(os.path.join(Case(case).dir, ref_log)).read())
    assert log_section(stdout) == want


def test_cli_fst_files_match_reference(tmp_path):
    d, _ = _run_cli("bn_fst", "par", tmp_path)
    ref = Case("bn_fst").dir
    assert open(d / "out.fstdetails").read() == open(os.path.join(ref, "ref.fstdetails.txt")).read()
    assert open(d / "out.mega").read() == open(os.path.join(ref, "ref.mega")).read()
    d2, _ = _run_cli("bn_fst", "par_pl", tmp_path / "pl")
    assert open(d2 / "out.phylip").read() == open(os.path.join(ref, "ref.phylip")).read()
    assert open(d2 / "out_pl.fstdetails").read() == open(os.path.join(ref, "ref_pl.fstdetails")).read()


def test_gp_fst_equals_oracle(gpu):
    """the device counts and host jackknife give the oracle's values bit for bit, and the
    reference's full-precision fstdetails within 1e-12"""
    c = Case("bn_fst")
    chrom, gpos = snp_table("bn_fst")
    eg = eglist("bn_fst")
    opts = native.default_opts(numeigs=4)
    r = native.smartpca_run(gpu, c.records, c.nind, opts, code=c.code, snp_chrom=chrom)
    xt = np.array([eg.index(c.pops[k]) for k in r["xindex"]], np.int32)
    nb, tag = native.set_blocks(chrom, gpos, r["snp_state"] != 0)
    onb, otag = O.set_blocks(chrom, gpos, r["snp_state"] != 0)
    assert nb == onb == 24 and np.array_equal(tag, otag)
    fmean, fans, fsd, fnum = gpu.fst(xt, len(eg), tag, nb)
    cols = np.nonzero(r["snp_state"] == 0)[0]
    om, oa, osd, on = O.fst(c.packed_records(), c.nind, r["xindex"], xt, len(eg), cols, tag, nb)
    iu = np.triu_indices(len(eg), 1)
    assert np.array_equal(fmean[iu], om[iu])
    assert np.array_equal(fans, oa) and np.array_equal(fsd, osd)
    assert np.array_equal(fnum, on)
    ref = read_fstdetails(os.path.join(c.dir, "ref.fstdetails"))
    for (p1, p2), (fm, fj, sd, z, n) in ref.items():
        a, b = eg.index(p1), eg.index(p2)
        assert abs(fans[a, b] - fj) <= 1e-12 and abs(fsd[a, b] - sd) <= 1e-12


@pytest.mark.parametrize("case,par_name,ref_log", [(c, "par", "ref.log") for c in CASES] +
                         [("bn_fst", "par", "ref.log"), ("bn_fst", "par_pl", "ref_par_pl.log")])
def test_cli_anova_section_matches_reference(case, par_name, ref_log, tmp_path):
    """per-eigenvector population means (up to the eigenvector's sign), ANOVA p-values and
    the popdifference chi-squares against the reference's log"""
    from tests.goldens import anova_section, compare_anova
    d, stdout = _run_cli(case, par_name, tmp_path)
    ref = anova_section(open(os.path.join(Case(case).dir, ref_log)).read())
    compare_anova(anova_section(stdout), ref)


def test_gp_fst_column_chunks_give_the_same_result(gpu, monkeypatch):
    """the counts taken in chunks of 999 columns give the one-chunk result bit for bit"""
    c = Case("bn_fst")
    chrom, gpos = snp_table("bn_fst")
    eg = eglist("bn_fst")
    r = native.smartpca_run(gpu, c.records, c.nind, native.default_opts(numeigs=4), code=c.code,
                            snp_chrom=chrom)
    xt = np.array([eg.index(c.pops[k]) for k in r["xindex"]], np.int32)
    nb, tag = native.set_blocks(chrom, gpos, r["snp_state"] != 0)
    whole = gpu.fst(xt, len(eg), tag, nb)
    monkeypatch.setenv("GP_FST_CHUNK_COLS", "999")
    parts = gpu.fst(xt, len(eg), tag, nb)
    for a, b in zip(whole, parts):
        assert np.array_equal(a, b)

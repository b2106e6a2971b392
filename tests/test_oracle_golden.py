"""CPU: the oracle restatement against the reference's own outputs (golden fixtures)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.goldens import (CASES, GOLDEN, REL_CASES, Case, compare_coords, coords_by_id,
                           eigbestsnp_lines, kurtosis_lines, snp_rows)

EX = os.path.join(GOLDEN, "ref_examples")


def test_convertf_formats_decode_identically():
    """CONVERTF/example.{packedancestrymapgeno,bed,eigenstratgeno}: one genotype matrix."""
    text = [l.strip() for l in open(os.path.join(EX, "CONVERTF_example.eigenstratgeno"))]
    G = np.array([[int(c) if c != "9" else -1 for c in l] for l in text])
    nsnp, nind = G.shape
    rlen = max((nind + 3) // 4, 48)
    raw = open(os.path.join(EX, "CONVERTF_example.packedancestrymapgeno"), "rb").read()
    packed = np.frombuffer(raw[rlen:], np.uint8).reshape(nsnp, rlen)
    assert raw[48:50] == bytes([0x54, 0x00])  # first record decodes to 1,1,1,0,0
    assert np.array_equal(O.unpack(packed, nind), G)
    bed = np.frombuffer(open(os.path.join(EX, "CONVERTF_example.bed"), "rb").read()[3:],
                        np.uint8).reshape(nsnp, (nind + 3) // 4)
    assert np.array_equal(O.unpack(O.bed_to_packed(bed, nind), nind), G)
    assert np.array_equal(O.pack(G)[:, : (nind + 3) // 4], packed[:, : (nind + 3) // 4])


def test_eigenstrat_example_eval():
    """EIGENSTRAT/example.eval (altnormstyle NO, 2 eigenvectors) from the oracle."""
    text = [l.strip() for l in open(os.path.join(EX, "EIGENSTRAT_example.geno"))]
    G = np.array([[int(c) if c != "9" else -1 for c in l] for l in text])
    r = O.smartpca(O.pack(G), G.shape[1], numeigs=2, numoutleigs=2, altnormstyle=0,
                   snp_chrom=np.full(G.shape[0], 11))
    golden = np.loadtxt(os.path.join(EX, "EIGENSTRAT_example.eval"))
    assert np.allclose(r["evals"], golden, atol=5e-7)
    lines = open(os.path.join(EX, "EIGENSTRAT_example.pca.evec")).read().splitlines()[1:]
    ref = np.array([[float(x) for x in l.split()[1:3]] for l in lines])
    mine = r["coords"].T
    s = np.sign(np.sum(ref * mine, axis=0))
    assert np.max(np.abs(ref - mine * s)) < 6e-5  # printed at %10.4f


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case):
    c = Case(case)
    kw = c.opts()
    r = O.smartpca(c.packed_records(), c.nind, ind_affstatus=c.affstatus, ind_pop=c.ind_pop,
                   **kw)
    n = r["nrows"]
    assert len(c.ref_evals) == n
    scale = max(abs(c.ref_evals[0]), 1.0)
    assert np.max(np.abs(r["evals"] - c.ref_evals)) / scale < 1e-12
    assert [c.ids[k] for k, *_ in r["outliers"]] == c.ref_outliers
    mine = coords_by_id(c.ids, r["coords"], r["ind_out"])
    compare_coords(c.ref_coords, mine, r["numeigs"], 1e-9)


@pytest.mark.parametrize("case", CASES)
def test_lookup_gram_equals_plain(case):
    """the reference's partial-sum lookup Gram (threaded) equals the plain FP64 sum"""
    c = Case(case)
    rec = c.packed_records()
    rows = np.arange(c.nind, dtype=np.int32)
    cols = np.arange(c.nsnp, dtype=np.int32)
    s = O.pass_columns(rec, cols, rows)
    a = O.gram(s)
    b = O.gram(s, lookup=True, nthreads=3)
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(a))


def test_oracle_grm_matches_reference():
    """GRM dump (dumpgrm/dumpgrmbin) of the oracle's last-pass Gram against the reference's
    text, binary and id files"""
    from tests.goldens import Grm, compare_grm_text, float_ulps
    c = Case("bn_grm")
    r = O.smartpca(c.packed_records(), c.nind, ind_affstatus=c.affstatus, **c.opts())
    g = Grm("bn_grm")
    txt, binv = O.grm(r["xtx"])
    lines = O.grm_text_lines(r["xtx"], r["nused"])
    assert np.all(g.numsnps == r["nused"]) and np.all(g.nbin == r["nused"])
    assert len(g.nbin) == len(binv)
    compare_grm_text(lines, g.text, txt, g.values)
    assert np.max(float_ulps(binv, g.bin)) <= 1
    assert g.ids == ["NA\t" + c.ids[k] for k in r["xindex"]]


@pytest.mark.parametrize("case", REL_CASES)
def test_oracle_smartrel_matches_reference(case):
    """smartrel: the oracle's outliers, pair list, order and scores against the reference"""
    from tests.goldens import compare_rel, rel_lines
    c = Case(case)
    pairs, r = O.smartrel(c.packed_records(), c.nind, **c.rel_opts())
    assert [c.ids[k] for k, *_ in r["outliers"]] == c.ref_outliers
    # the sign of an eigenvector (and so of its z score) is the eigensolver's choice
    assert ["REMOVED outlier %s iter %d evec %d sigmage %.3f" % (c.ids[k], it, v, abs(z))
            for k, it, v, z in r["outliers"]] == [l.replace("sigmage -", "sigmage ")
                                                   for l in c.ref_outlier_lines]
    assert len(pairs) == len(c.ref_rel) > 20
    compare_rel(pairs, c.ids, c, tol=1e-10)
    assert rel_lines(c.ids, pairs)[0] == c.ref_rel_text[0]


CV_RUNS = ["pk2pk", "pk2bed", "pk2es", "bed2pk", "bed2es"]


@pytest.mark.parametrize("run", CV_RUNS)
def test_oracle_convertf_matches_reference(run):
    """convertf's default path and packed writers restated (oracle/convertf.py): the three
    output files byte-identical to the reference convertf's on a panel with chromosome 0,
    duplicate positions, unknown alleles (flips), an Ignore sample and a sample without data"""
    from oracle import convertf as CV
    d = os.path.join(GOLDEN, "cv_edge")
    par = {}
    for line in open(os.path.join(d, "par_" + run)):
        k, v = line.split(None, 1)
        par[k.rstrip(":")] = v.strip()
    o = CV.run_par(d, par)
    assert o["geno"] == open(os.path.join(d, "out_%s.geno" % run), "rb").read()
    assert o["snp"] == open(os.path.join(d, "out_%s.snp" % run)).read()
    assert o["ind"] == open(os.path.join(d, "out_%s.ind" % run)).read()


def test_convertf_edge_case_is_exercised():
    """the fixture holds what it claims: dropped chromosome-0 and duplicate SNPs, flipped
    SNPs (alleles swapped, genotypes 2-g), the Ignore sample and the sample without data"""
    from oracle import convertf as CV
    d = os.path.join(GOLDEN, "cv_edge")
    snps, order = CV.read_snps(os.path.join(d, "data.snp"))
    out = [l.split() for l in open(os.path.join(d, "out_pk2pk.snp"))]
    assert len(out) < len(snps) - 3
    ids = {s[0]: s for s in snps}
    flipped = [o for o in out if ids[o[0]][4][0] in "X0" and ids[o[0]][4][1] not in "X0"]
    assert len(flipped) >= 10 and all(o[4] == ids[o[0]][4][1] for o in flipped)
    inds = [l.split()[0] for l in open(os.path.join(d, "out_pk2pk.ind"))]
    assert "S0000011" not in inds and "S0000007" not in inds and len(inds) == 148


@pytest.mark.parametrize("par_name,details,tol", [("par", "ref.fstdetails", 1e-12),
                                                   ("par_pl", "ref_pl.fstdetails", 6e-10)])
def test_oracle_fst_matches_reference(par_name, details, tol):
    """Fst tail (fstcolyy + block jackknife) of the oracle on the last pass against the
    reference's fstdetails file: 24 blocks over two chromosomes, 12 or 6 populations"""
    from tests.goldens import eglist, read_fstdetails, snp_table
    c = Case("bn_fst")
    par = {}
    for line in open(os.path.join(c.dir, par_name)):
        k, v = line.split(None, 1)
        par[k.rstrip(":")] = v.strip()
    chrom, gpos = snp_table("bn_fst")
    eg = eglist("bn_fst", par)
    aff = None
    if "poplistname" in par:
        aff = np.array([p in eg for p in c.pops], np.uint8)
    r = O.smartpca(c.packed_records(), c.nind, numeigs=int(par["numoutevec"]), snp_chrom=chrom,
                   ind_affstatus=aff)
    xt = [eg.index(c.pops[k]) if c.pops[k] in eg else -1 for k in r["xindex"]]
    nb, tag = O.set_blocks(chrom, gpos, r["snp_state"] != 0)
    assert nb == 24
    cols = np.nonzero(r["snp_state"] == 0)[0]
    fmean, fans, fsd, fnum = O.fst(c.packed_records(), c.nind, r["xindex"], xt, len(eg), cols,
                                   tag, nb)
    ref = read_fstdetails(os.path.join(c.dir, details))
    assert len(ref) == len(eg) * (len(eg) - 1) // 2
    for (p1, p2), (fm, fj, sd, z, n) in ref.items():
        a, b = eg.index(p1), eg.index(p2)
        assert abs(fmean[a, b] - fm) <= tol * max(1.0, abs(fm))
        assert abs(fans[a, b] - fj) <= tol * max(1.0, abs(fj))
        assert abs(fsd[a, b] - sd) <= tol * max(1.0, abs(sd))
        assert fnum[a, b] == n


@pytest.mark.parametrize("seed", [0, 3, 5489, 2 ** 32 + 7])
def test_gsl_mt19937_stream(seed):
    """the oracle's GSL mt19937 is the published generator: its 32-bit outputs equal numpy's
    legacy RandomState (MT19937 with the same 2002 initialisation) for the seed GSL uses
    (0 -> 4357, then the low 32 bits); seed 5489 starts with the published 3499211612"""
    g = O.GslMt19937(seed)
    mine = np.array([g.next32() for _ in range(3000)], np.uint64)
    s = 4357 if seed == 0 else seed & 0xFFFFFFFF
    ref = np.random.RandomState(s).randint(0, 2 ** 32, size=3000, dtype=np.uint64)
    assert np.array_equal(mine, ref)
    if seed == 5489:
        assert mine[0] == 3499211612


@pytest.mark.parametrize("par", ["par", "par_odd"])
def test_oracle_fastmode_matches_reference(par):
    """the reference's fastmode (kjg_fpca, built against the GSL shim) against the oracle's
    numpy kjg_fpca with the same GSL Omega: eigenvalues and unit eigenvectors to 1e-12 (an
    odd L puts uniform draws in Omega's last column)"""
    from tests.goldens import FastCase
    fc = FastCase()
    r = fc.run(par)
    om = O.gsl_omega(r["seed"], fc.nind, r["L"])
    ev, V = O.fastpca(fc.records, np.arange(fc.nsnp, dtype=np.int32),
                      np.arange(fc.nind, dtype=np.int32), r["K"], r["L"], r["I"], om)
    assert np.max(np.abs(ev - r["evals"]) / r["evals"]) < 1e-12
    Vn = V / np.linalg.norm(V, axis=1, keepdims=True)
    cos = np.abs(np.sum(Vn * r["evecs"], axis=1)) / np.linalg.norm(r["evecs"], axis=1)
    assert np.all(cos > 1 - 1e-12)


@pytest.mark.parametrize("case", CASES)
def test_oracle_snp_weights_match_reference(case):
    """writesnpeigs: the scaled weights' best SNPs of every case (the log's eigbestsnp lines)
    and, for bn_snpwt, the snpweightoutname file at full precision"""
    c = Case(case)
    r = O.smartpca(c.packed_records(), c.nind, ind_affstatus=c.affstatus, ind_pop=c.ind_pop,
                   **c.opts())
    ff, best = O.snpeigs(r["ffvecs"], r["killed"])
    rows = snp_rows(case)
    want = eigbestsnp_lines(open(os.path.join(c.dir, "ref.log")).read())
    got = [(j + 1,) + rows[r["cols"][k]] + (v,) for j, k, v in best]
    assert [g[:4] for g in got] == [w[:4] for w in want]
    assert max(abs(g[4] - w[4]) for g, w in zip(got, want)) <= 5.0001e-4
    if "snpweightoutname" in c.par:
        lines = [l.split() for l in open(os.path.join(c.dir, "ref.snpwt")) if l.strip()]
        kept = [k for k in range(len(r["cols"])) if not r["killed"][k]]
        assert [l[0] for l in lines] == [rows[r["cols"][k]][0] for k in kept]
        ref = np.array([[float(x) for x in l[3:]] for l in lines])
        mine = ff[:, kept].T
        sgn = np.sign(np.sum(ref * mine, axis=0))  # the eigenvectors' signs are arbitrary
        assert np.max(np.abs(ref - mine * sgn)) <= 1e-9 * np.max(np.abs(ref))


@pytest.mark.parametrize("case", CASES)
def test_oracle_kurtosis_lines_match_reference(case):
    """the log's kurtosis of each eigenvector's SNP weights and of its sample entries"""
    c = Case(case)
    r = O.smartpca(c.packed_records(), c.nind, ind_affstatus=c.affstatus, ind_pop=c.ind_pop,
                   **c.opts())
    want = kurtosis_lines(open(os.path.join(c.dir, "ref.log")).read())
    assert len(want) == r["numeigs"]
    for j, ks, ki in want:
        assert abs(O.kurtosis(r["ffvecs"][j - 1]) - ks) <= 5.0001e-4
        assert abs(O.kurtosis(10.0 * r["evecs"][j - 1]) - ki) <= 5.0001e-4



def _tw_logs():
    """golden logs with a Tracy-Widom section whose spectrum is stored in full"""
    out = []
    for case in sorted(os.listdir(GOLDEN)):
        d = os.path.join(GOLDEN, case)
        for name in sorted(os.listdir(d)) if os.path.isdir(d) else []:
            if not (name.startswith("ref") and name.endswith(".log")):
                continue
            ev = os.path.join(d, name[:-4] + ".eval")
            if os.path.exists(ev) and "Tracy-Widom" in open(os.path.join(d, name)).read():
                out.append((case, name))
    return out


TW_LOGS = _tw_logs()


def log_cut(d, name):
    """the stored log ends inside its Tracy-Widom section (the full-size cases keep only the
    head of the reference's log)"""
    last = open(os.path.join(d, name)).read().splitlines()[-1].split()
    return len(last) == 6 and last[0].isdigit()


def compare_tw(mine_mp, mine_rows, want_mp, want_rows, prefix=False):
    """text-exact statistics (3 decimals) and effective n; p-values within 1e-5 relative (the
    6th significant digit of a value on a rounding boundary); prefix: the stored log was cut
    short inside the section, so only its first rows are compared"""
    assert (mine_mp is None) == (want_mp is None)
    if want_mp is not None:
        assert ["%.3f" % v for v in mine_mp[:3]] == ["%.3f" % v for v in want_mp[:3]]
        assert "%.6f" % mine_mp[3] == "%.6f" % want_mp[3]
    if prefix:
        assert len(want_rows) > 10
        mine_rows = mine_rows[:len(want_rows)]
    assert len(mine_rows) == len(want_rows)
    for got, want in zip(mine_rows, want_rows):
        if want[3] is None:
            assert got is None, want
            continue
        tw, p, zn = got
        assert "%.3f" % tw == "%.3f" % want[3] and "%.3f" % zn == "%.3f" % want[5], (got, want)
        assert abs(p - want[4]) <= 1e-5 * max(want[4], 1e-300) or "%.6g" % p == "%.6g" % want[4]


@pytest.mark.parametrize("case,name", TW_LOGS)
def test_oracle_tw_section_matches_reference(case, name):
    """the log's mpstats line and Tracy-Widom section (smartpca.c:1306-1367): the oracle's
    statistics from the reference's own eigenvalues (full precision) against its log"""
    from tests.goldens import tw_section
    d = os.path.join(GOLDEN, case)
    lam = np.loadtxt(os.path.join(d, name[:-4] + ".eval"))
    want_mp, shape, want_rows = tw_section(open(os.path.join(d, name)).read())
    if len(lam) != shape[0]:
        pytest.skip("the stored spectrum is truncated")
    compare_tw(O.mpstats(lam), O.twstats(lam), want_mp, want_rows, prefix=log_cut(d, name))


def test_tw_logs_are_exercised():
    assert len(TW_LOGS) >= 10

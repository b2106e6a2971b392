"""Generate the golden fixtures under tests/golden/ by running the REFERENCE smartpca.

Run in a container where the reference sources are present (the binary is built by
oracle/build_ref.sh into oracle/_ref/smartpca, with fprintf wrapped so that
EIG_REF_FULLPREC=1 prints .eval/.evec numbers as %.17g).  Writes, per case:

  <case>/data.{geno|bed,snp|bim,ind|fam}  the inputs (small, seeded Balding-Nichols)
  <case>/par                              the parfile template (paths relative to the case)
  <case>/ref.eval, ref.evec               reference outputs at full precision
  <case>/ref.eval.txt, ref.evec.txt       reference outputs in the shipped text formats
  <case>/ref.outliers                     the reference's outlier-removal lines
  <case>/ref.log                          the reference's log
  <case>/ref.grm[.txt], ref.grm.id, ref.grm.bin, ref.grm.N.bin   GRM dumps (grm cases)
  <case>/ref.fstdetails[.txt], ref.mega   Fst files (bn_fst; ref_par_pl.log, ref.phylip and
                                          ref_pl.fstdetails from its second parfile par_pl)
  <case>/ref.snpwt[.txt]                  the snpweightoutname file (cases that set it)
  <case>/ref.rel, ref.rel.txt             smartrel "rel:" lines (tool == "smartrel": the case
                                          runs oracle/_ref/smartrel; relatives are planted by
                                          copying a share of one sample's genotypes to another)

and copies the reference's own example fixtures (CONVERTF/example.*,
EIGENSTRAT/example.*) into ref_examples/.  Usage:
  python tests/golden/make_golden.py REFERENCE_ROOT [--scratch DIR] [case ...]
(the benchmark-shaped cases of BIG_CASES run only when named, with --scratch for their
genotype files)
"""
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from eig_gb300 import native  # noqa: E402  (the synthetic generator)
from oracle import oracle as O  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "smartpca")
REF_REL = os.path.join(ROOT, "oracle", "_ref", "smartrel")

CASES = {
    # default options, 3 populations + 4 planted divergent samples -> outlier removal
    "bn_outliers": dict(nsnp=4000, pops=[80, 80, 76, 2, 2], fst=[0.01, 0.01, 0.02, 0.25, 0.25],
                        miss=0.01, seed=11, fmt="packed",
                        par={"numoutevec": "6", "numoutlieriter": "5"}),
    # PLINK bed input, altnormstyle NO, 5% missing, a maxmissing filter, 4 eigenvectors
    "bn_bed_altnorm": dict(nsnp=3000, pops=[60, 60, 60], fst=[0.02, 0.03, 0.05], miss=0.05,
                           seed=12, fmt="bed",
                           par={"numoutevec": "4", "altnormstyle": "NO", "maxmissing": "16",
                                "familynames": "NO"}),
    # projection: PCA on POP0/POP1 only (poplistname), POP2 + admixed projected by lsqproj;
    # per-sample missing up to 95% so that a few samples have too little data
    "bn_project": dict(nsnp=3000, pops=[70, 70, 40], fst=[0.02, 0.02, 0.04], miss=0.0,
                       miss_hi=0.97, n_admixed=20, seed=13, fmt="packed",
                       par={"numoutevec": "5", "numoutlieriter": "0",
                            "poplistname": "poplist"}, poplist=["POP0", "POP1"]),
    # GRM dump (grmoutname) of the last pass after outlier removal, text and binary
    "bn_grm": dict(nsnp=2500, pops=[24, 24, 20, 1, 1], fst=[0.01, 0.02, 0.03, 0.3, 0.3],
                   miss=0.02, seed=14, fmt="packed",
                   par={"numoutevec": "4", "numoutlieriter": "3", "grmoutname": "out.grm"},
                   grm=True),
    # Fst tail: 12 populations on two chromosomes spanning ~24 jackknife blocks (numeg > 10:
    # the per-pair Fst lines), fstdetails and mega files; a second run on 6 listed populations
    # with phylip output, fsthiprecision and fstz
    "bn_fst": dict(nsnp=3000, pops=[16, 18, 20, 15, 17, 19, 16, 18, 20, 15, 17, 19],
                   fst=[0.005, 0.01, 0.02, 0.03, 0.04, 0.05, 0.005, 0.01, 0.02, 0.03, 0.04, 0.05],
                   miss=0.02, seed=16, fmt="packed", relocate=(2, 4e-4),
                   par={"numoutevec": "4", "fstdetailsname": "out.fstdetails",
                        "megaoutname": "out.mega"},
                   runs2={"par_pl": {"poplistname": "poplist", "phylipname": "out.phylip",
                                     "fsthiprecision": "YES", "fstz": "YES",
                                     "fstdetailsname": "out_pl.fstdetails"}},
                   poplist=["POP5", "POP1", "POP3", "POP0", "POP9", "POP11"]),
    # smartrel: planted relatives (b copies a's genotype at a share of the SNPs), default
    # relthresh 0.05 / outlier removal (numoutlierevec 10), 3 components removed, minallelecnt 2
    "bn_rel": dict(nsnp=3000, pops=[40, 40, 30], fst=[0.01, 0.02, 0.03], miss=0.02, seed=15,
                   fmt="packed", tool="smartrel",
                   relatives=[(3, 4, 0.5), (10, 60, 0.5), (20, 21, 0.25), (45, 46, 0.9),
                              (90, 91, 0.5), (100, 101, 0.125)],
                   par={"minallelecnt": "2", "numoutevec": "3"}),
    # missingmode: the PCA of the missingness indicators (setmiss, fancynorm off); per-sample
    # missing rates ~U(0, 0.4) so that missingness has structure
    "bn_missingmode": dict(nsnp=3000, pops=[70, 70, 60], fst=[0.01, 0.02, 0.03], miss=0.0,
                           miss_hi=0.4, seed=18, fmt="packed",
                           par={"numoutevec": "4", "missingmode": "YES"}),
    # usepopsformissing: missing genotypes take their population's mean in the Gram and in
    # lsqproj; per-sample missing rates ~U(0, 0.5), two planted 2-sample populations removed
    # as outliers, maxmissing 1 applied to the count still missing after the fill (a SNP
    # where a whole population is missing)
    "bn_usepops": dict(nsnp=3000, pops=[60, 60, 50, 2, 2], fst=[0.01, 0.02, 0.03, 0.25, 0.25],
                       miss=0.0, miss_hi=0.5, seed=19, fmt="packed",
                       par={"numoutevec": "4", "usepopsformissing": "YES", "maxmissing": "1"}),
    # snpweightoutname: the SNP weights file (writesnpeigs) of a run on two chromosomes with
    # outlier removal and a maxmissing filter, hiprecision (weights at 6 decimals)
    "bn_snpwt": dict(nsnp=2500, pops=[60, 60, 50, 2], fst=[0.01, 0.02, 0.03, 0.3], miss=0.02,
                     seed=21, fmt="packed", relocate=(2, 4e-4),
                     par={"numoutevec": "3", "snpweightoutname": "out.snpwt",
                          "hiprecision": "YES", "maxmissing": "6"}),
    # the same option with a poplist (POP1, POP2): the other samples are projected, and
    # lsqproj reads each sample's population at its .ind index among the row-indexed xtypes
    "bn_usepops_pl": dict(nsnp=3000, pops=[60, 60, 50, 2, 2], fst=[0.01, 0.02, 0.03, 0.25, 0.25],
                          miss=0.0, miss_hi=0.5, n_admixed=10, seed=20, fmt="packed",
                          par={"numoutevec": "4", "usepopsformissing": "YES",
                               "poplistname": "poplist"}, poplist=["POP1", "POP2"]),
}

# fastmode (kjg_fpca) through the reference built with oracle/gsl_shim: default L = 2K, I = K
# with Omega from GSL's mt19937 seeded 3, and a second parfile with an odd L (fastdim 7, whose
# last Omega column holds uniform draws) and fastiter 3
FAST_CASES = {
    "bn_fastmode": dict(nsnp=5000, pops=[100, 100, 80], fst=[0.01, 0.03, 0.05], miss=0.01,
                        n_admixed=20, seed=17,
                        par={"fastmode": "YES", "numoutevec": "4", "seed": "3"},
                        runs2={"par_odd": {"fastdim": "7", "fastiter": "3", "numoutevec": "3",
                                           "seed": "5"}}),
}


def make_fast_case(name, spec):
    """fastmode writes only the .evec (smartpca.c:955-977): full precision and as shipped"""
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    prefix = os.path.join(d, "data")
    native.synth_write_dataset(prefix, spec["nsnp"], spec["pops"], spec["fst"],
                               miss=spec["miss"], n_admixed=spec.get("n_admixed", 0),
                               seed=spec["seed"], nthreads=4)
    base = {"genotypename": "data.geno", "snpname": "data.snp", "indivname": "data.ind",
            "evecoutname": "out.evec", "evaloutname": "out.eval"}
    runs = {"par": dict(base, **spec["par"])}
    for rname, extra in spec.get("runs2", {}).items():
        runs[rname] = dict(base, **dict(spec["par"], **extra))
    for rname, par in runs.items():
        with open(os.path.join(d, rname), "w") as f:
            for k, v in par.items():
                f.write("%s: %s\n" % (k, v))
        tag = "" if rname == "par" else "_" + rname.split("_", 1)[1]
        for prec, suffix in ((False, ".txt"), (True, "")):
            env = dict(os.environ, EIG_REF_FULLPREC="1" if prec else "0")
            with open(os.path.join(d, "ref%s.log" % tag), "w") as log:
                subprocess.run([REF_BIN, "-p", rname], cwd=d, env=env, stdout=log,
                               stderr=subprocess.STDOUT, check=True)
            shutil.move(os.path.join(d, "out.evec"), os.path.join(d, "ref%s.evec%s" % (tag, suffix)))


def relocate_snps(prefix, nchrom, step):
    """spread the SNPs over nchrom chromosomes in equal runs, genetic positions step morgans
    apart (physical 1e8 x genetic); the IDs, and so the GENO header hash, stay"""
    lines = [l.split() for l in open(prefix + ".snp") if l.strip()]
    per = (len(lines) + nchrom - 1) // nchrom
    with open(prefix + ".snp", "w") as f:
        for i, t in enumerate(lines):
            c, j = 1 + i // per, i % per
            f.write("%20s %4d %12.6f %12d %s %s\n" % (t[0], c, (j + 1) * step,
                                                     int(round((j + 1) * step * 1e8)), t[4], t[5]))


def plant_relatives(prefix, nsnp, nind, pairs, seed):
    """copy sample a's genotype to sample b at a seeded share of the SNPs (GENO records)"""
    raw = bytearray(open(prefix + ".geno", "rb").read())
    rlen = max((nind + 3) // 4, 48)
    rec = np.frombuffer(bytes(raw[rlen:]), np.uint8).reshape(nsnp, rlen)
    g = O.unpack(rec, nind)
    rng = np.random.default_rng(seed)
    for a, b, frac in pairs:
        m = rng.random(nsnp) < frac
        g[m, b] = g[m, a]
    out = O.pack(g)
    raw[rlen:] = np.ascontiguousarray(out[:, :rlen]).tobytes()
    with open(prefix + ".geno", "wb") as f:
        f.write(bytes(raw))


def write_bed_case(d, rec, nind, nsnp, pops):
    """PLINK .bed/.bim/.fam from packed records (packed code -> bed code)."""
    g = O.unpack(rec, nind)  # nsnp x nind, -1 missing
    bedcode = np.where(g < 0, 1, np.where(g == 2, 0, np.where(g == 1, 2, 3))).astype(np.uint8)
    blen = (nind + 3) // 4
    pad = np.zeros((nsnp, blen * 4 - nind), np.uint8)
    c = np.concatenate([bedcode, pad], axis=1).reshape(nsnp, blen, 4)
    by = c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)
    with open(os.path.join(d, "data.bed"), "wb") as f:
        f.write(bytes([0x6C, 0x1B, 0x01]))
        f.write(by.astype(np.uint8).tobytes())
    with open(os.path.join(d, "data.bim"), "w") as f:
        for s in range(nsnp):
            f.write("1\trs%09d\t%.8f\t%d\tA\tG\n" % (s, (s + 1) * 1e-6, (s + 1) * 1000))
    with open(os.path.join(d, "data.fam"), "w") as f:
        for k in range(nind):
            f.write("FAM%d S%07d 0 0 %d POP%d\n" % (k, k, 1 + (k & 1), pops[k]))


def make_case(name, spec):
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    prefix = os.path.join(d, "data")
    native.synth_write_dataset(prefix, spec["nsnp"], spec["pops"], spec["fst"],
                               miss=spec["miss"], miss_hi=spec.get("miss_hi"),
                               n_admixed=spec.get("n_admixed", 0), seed=spec["seed"], nthreads=4)
    par = {}
    if "relocate" in spec:
        relocate_snps(prefix, *spec["relocate"])
    if "relatives" in spec:
        plant_relatives(prefix, spec["nsnp"], sum(spec["pops"]), spec["relatives"],
                        spec["seed"] + 1000)
    if spec["fmt"] == "bed":
        nind = sum(spec["pops"])
        raw = open(prefix + ".geno", "rb").read()
        rlen = max((nind + 3) // 4, 48)
        rec = np.frombuffer(raw[rlen:], np.uint8).reshape(spec["nsnp"], rlen)
        pops = [k for k, n in enumerate(spec["pops"]) for _ in range(n)]
        write_bed_case(d, rec, nind, spec["nsnp"], pops)
        for ext in ("geno", "snp", "ind"):
            os.remove(prefix + "." + ext)
        par.update(genotypename="data.bed", snpname="data.bim", indivname="data.fam")
    else:
        par.update(genotypename="data.geno", snpname="data.snp", indivname="data.ind")
    if spec.get("tool") == "smartrel":
        par.update(outliername="out.outliers")
    else:
        par.update(evecoutname="out.evec", evaloutname="out.eval",
                   outlieroutname="out.outliers")
    par.update(spec["par"])
    if "poplist" in spec:
        with open(os.path.join(d, "poplist"), "w") as f:
            f.write("\n".join(spec["poplist"]) + "\n")
    with open(os.path.join(d, "par"), "w") as f:
        for k, v in par.items():
            f.write("%s: %s\n" % (k, v))
    if spec.get("tool") == "smartrel":
        run_smartrel(d)
        return
    extra = (("fstdetails",) if "fstdetailsname" in par else ()) + \
        (("snpwt",) if "snpweightoutname" in par else ())
    run_reference(d, spec.get("grm", False), extra=extra)
    for rname, extra_par in spec.get("runs2", {}).items():
        with open(os.path.join(d, rname), "w") as f:
            for k, v in par.items():
                if k not in extra_par and k not in ("fstdetailsname", "megaoutname"):
                    f.write("%s: %s\n" % (k, v))
            for k, v in extra_par.items():
                f.write("%s: %s\n" % (k, v))
        env = dict(os.environ, EIG_REF_FULLPREC="0")
        with open(os.path.join(d, "ref_%s.log" % rname), "w") as log:
            subprocess.run([REF_BIN, "-p", rname], cwd=d, env=env, stdout=log,
                           stderr=subprocess.STDOUT, check=True)
        for n in ("out.eval", "out.evec", "out.outliers"):
            os.remove(os.path.join(d, n))
        shutil.move(os.path.join(d, "out.phylip"), os.path.join(d, "ref.phylip"))
        shutil.move(os.path.join(d, "out_pl.fstdetails"), os.path.join(d, "ref_pl.fstdetails"))
    if spec.get("grm"):
        # the binary GRM from a second run of the same parfile with grmbinary: YES
        with open(os.path.join(d, "par_bin"), "w") as f:
            for k, v in par.items():
                f.write("%s: %s\n" % (k, v))
            f.write("grmbinary: YES\n")
        with open(os.path.join(d, "ref_bin.log"), "w") as log:
            subprocess.run([REF_BIN, "-p", "par_bin"], cwd=d, stdout=log,
                           stderr=subprocess.STDOUT, check=True)
        for ext in (".bin", ".N.bin"):
            shutil.move(os.path.join(d, "out.grm" + ext), os.path.join(d, "ref.grm" + ext))
        for n in ("out.eval", "out.evec", "out.outliers", "out.grm.id"):
            os.remove(os.path.join(d, n))


def run_reference(d, grm=False, extra=()):
    env = dict(os.environ)
    for prec, suffix in ((False, ".txt"), (True, "")):
        env["EIG_REF_FULLPREC"] = "1" if prec else "0"
        with open(os.path.join(d, "ref.log"), "w") as log:
            subprocess.run([REF_BIN, "-p", "par"], cwd=d, env=env, stdout=log,
                           stderr=subprocess.STDOUT, check=True)
        shutil.move(os.path.join(d, "out.eval"), os.path.join(d, "ref.eval" + suffix))
        shutil.move(os.path.join(d, "out.evec"), os.path.join(d, "ref.evec" + suffix))
        shutil.move(os.path.join(d, "out.outliers"), os.path.join(d, "ref.outliers"))
        if grm:
            shutil.move(os.path.join(d, "out.grm"), os.path.join(d, "ref.grm" + suffix))
            shutil.move(os.path.join(d, "out.grm.id"), os.path.join(d, "ref.grm.id"))
        for ext in extra:
            shutil.move(os.path.join(d, "out." + ext), os.path.join(d, "ref.%s%s" % (ext, suffix)))
        if os.path.exists(os.path.join(d, "out.mega")):
            shutil.move(os.path.join(d, "out.mega"), os.path.join(d, "ref.mega"))


def run_smartrel(d):
    env = dict(os.environ)
    for prec, suffix in ((False, ".txt"), (True, "")):
        env["EIG_REF_FULLPREC"] = "1" if prec else "0"
        with open(os.path.join(d, "ref.log"), "w") as log:
            subprocess.run([REF_REL, "-p", "par"], cwd=d, env=env, stdout=log,
                           stderr=subprocess.STDOUT, check=True)
        lines = [ln for ln in open(os.path.join(d, "ref.log")) if ln.startswith("rel:")]
        with open(os.path.join(d, "ref.rel" + suffix), "w") as f:
            f.writelines(lines)
        shutil.move(os.path.join(d, "out.outliers"), os.path.join(d, "ref.outliers"))


REF_CONVERTF = os.path.join(ROOT, "oracle", "_ref", "convertf")

# convertf: input panels with the reference's edge cases, and the runs made on them
CONVERT_CASES = {
    "cv_edge": dict(nsnp=400, pops=[60, 50, 40], fst=[0.01, 0.02, 0.04], miss=0.03, seed=21,
                    runs={"pk2pk": ("packed", "PACKEDANCESTRYMAP", False),
                          "pk2bed": ("packed", "PACKEDPED", False),
                          "pk2es": ("packed", "EIGENSTRAT", True),
                          "bed2pk": ("bed", "PACKEDANCESTRYMAP", True),
                          "bed2es": ("bed", "EIGENSTRAT", False)}),
}


def make_convert_case(name, spec):
    """A seeded panel written as packedancestrymap (.geno/.snp/.ind) and PLINK (.bed/.bim/
    .fam) with: chromosome 0 SNPs (dropped), chromosome X SNPs, duplicate positions (IDs of
    equal and of different lengths), unknown first alleles (X, 0: flipped) and unknown
    second ones, all-zero genetic positions (.snp: set from the physical position) and
    centimorgans (.bim), an "Ignore" sample, a sample without data and samples of unknown
    sex.  The reference convertf runs each entry of spec["runs"]:
    (input, outputformat, with poplistname) -> out_<run>.{geno,snp,ind}."""
    from oracle import convertf as CV
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(spec["seed"])
    rec, pop = native.synth_records(spec["nsnp"], spec["pops"], spec["fst"], miss=spec["miss"],
                                    seed=spec["seed"], nthreads=4)
    nind = len(pop)
    M = spec["nsnp"]
    g = O.unpack(rec, nind)
    g[:, 7] = -1                                  # a sample without data
    ids = ["S%07d" % k for k in range(nind)]
    pops = ["POP%d" % p for p in pop]
    pops[11] = "Ignore"
    sexes = ["M" if k % 3 == 0 else "F" if k % 3 == 1 else "U" for k in range(nind)]
    # SNP table in sorted order: 3 on chromosome 0, then 1, 2 and 23 (X)
    chrom = np.concatenate([np.zeros(3, int), np.ones(197, int), np.full(180, 2),
                            np.full(M - 380, 23)])
    ppos = np.zeros(M, int)
    for c in np.unique(chrom):
        k = np.nonzero(chrom == c)[0]
        ppos[k] = 1000 + np.cumsum(rng.integers(50, 5000, len(k)))
    snp_id = ["rs%d" % (1000000 + i) for i in range(M)]
    for i in range(20, M - 1, 37):                # duplicate positions
        ppos[i + 1] = ppos[i]
        if (i // 37) % 2:
            snp_id[i + 1] = "AFFX-%07d" % i       # longer ID: the rs ID stays
        else:
            snp_id[i + 1] = "rs%d" % (2000000 + i)  # equal lengths: the larger ID stays
    a0 = np.array(list("ACGT"))[rng.integers(0, 4, M)]
    a1 = np.array(list("ACGT"))[rng.integers(0, 4, M)]
    a0[5::23] = "X"                               # flipped
    a0[9::31] = "0"                               # flipped ('0' in .snp and .bim)
    a1[13::29] = "X"                              # not flipped
    gen = np.zeros(M)                             # .snp: all zero -> 1e-8 * ppos
    # packedancestrymap input
    with open(os.path.join(d, "data.snp"), "w") as f:
        for i in range(M):
            f.write("%20s %4d %12.6f %12d %s %s\n" % (snp_id[i], chrom[i], gen[i], ppos[i],
                                                     a0[i], a1[i]))
    with open(os.path.join(d, "data.ind"), "w") as f:
        for k in range(nind):
            f.write("%20s %s %12s\n" % (ids[k], sexes[k], pops[k]))
    with open(os.path.join(d, "data.geno"), "wb") as f:
        f.write(CV.encode(g, "PACKEDANCESTRYMAP", ids=ids, snp_ids=snp_id))
    # PLINK input: genetic positions in cM (> 100 somewhere -> converted)
    cm = np.round(ppos * 1e-3, 6)
    with open(os.path.join(d, "data.bim"), "w") as f:
        for i in range(M):
            f.write("%d\t%s\t%.6f\t%d\t%s\t%s\n" % (chrom[i], snp_id[i], cm[i], ppos[i], a0[i],
                                                   a1[i]))
    with open(os.path.join(d, "data.fam"), "w") as f:
        for k in range(nind):
            sx = {"M": 1, "F": 2, "U": 0}[sexes[k]]
            f.write("F%d %s 0 0 %d %s\n" % (k, ids[k], sx, "-9" if k == 11 else pops[k]))
    with open(os.path.join(d, "data.bed"), "wb") as f:
        f.write(_bed_bytes(g))
    with open(os.path.join(d, "poplist"), "w") as f:
        f.write("POP2\nPOP0\n")
    for run, (src, fmt, use_pl) in spec["runs"].items():
        par = {"genotypename": "data.geno" if src == "packed" else "data.bed",
               "snpname": "data.snp" if src == "packed" else "data.bim",
               "indivname": "data.ind" if src == "packed" else "data.fam",
               "outputformat": fmt, "genotypeoutname": "out_%s.geno" % run,
               "snpoutname": "out_%s.snp" % run, "indivoutname": "out_%s.ind" % run}
        if src == "bed":
            par["familynames"] = "NO"
        if use_pl:
            par["poplistname"] = "poplist"
        with open(os.path.join(d, "par_" + run), "w") as f:
            for k, v in par.items():
                f.write("%s: %s\n" % (k, v))
        with open(os.path.join(d, "log_" + run), "w") as log:
            subprocess.run([REF_CONVERTF, "-p", "par_" + run], cwd=d, stdout=log,
                           stderr=subprocess.STDOUT, check=True)


def _bed_bytes(g):
    """PLINK .bed of a genotype matrix (count of the first allele, -1 missing)"""
    nsnp, nind = g.shape
    bedcode = np.where(g < 0, 1, np.where(g == 2, 0, np.where(g == 1, 2, 3))).astype(np.uint8)
    blen = (nind + 3) // 4
    pad = np.zeros((nsnp, blen * 4 - nind), np.uint8)
    c = np.concatenate([bedcode, pad], axis=1).reshape(nsnp, blen, 4)
    by = c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)
    return bytes([0x6C, 0x1B, 0x01]) + by.astype(np.uint8).tobytes()


def copy_examples(ref_root):
    out = os.path.join(HERE, "ref_examples")
    os.makedirs(out, exist_ok=True)
    files = {
        "CONVERTF": ["example.eigenstratgeno", "example.packedancestrymapgeno", "example.bed",
                     "example.snp", "example.ind", "example.pedsnp", "example.pedind"],
        "EIGENSTRAT": ["example.geno", "example.snp", "example.ind", "example.eval",
                       "example.pca.evec"],
    }
    for sub, names in files.items():
        for n in names:
            shutil.copy(os.path.join(ref_root, sub, n), os.path.join(out, sub + "_" + n))


# Panels at the benchmark shapes.  Their genotypes are NOT committed: the tests regenerate them
# from the seed with the same generator and check the records' SHA-256 first.  Committed per
# case: spec.json (generator arguments, records hash, kept-SNP count, parfile), ref.eval (the
# first `keep_evals` eigenvalues at %.17g, plus their total), ref.evec (header + every
# `evec_stride`-th sample at %.17g), ref.outliers and the head of ref.log.
BIG_CASES = {
    # N=1,000 x M=50,000, 3 populations of ~333, F=0.01, 1% missing, seed 1, K=10, no outlier
    # removal: plain smartpca
    "cfg1_plain": dict(nsnp=50_000, pops=[334, 333, 333], fst=[0.01, 0.01, 0.01], miss=0.01,
                       seed=1, keep_evals=1000, evec_stride=1,
                       par={"numoutevec": "10", "numoutlieriter": "0"}),
    # the same shape with 8 planted divergent samples (two populations of 4 at F=0.25) and the
    # default outlier removal (5 iterations, 10 eigenvectors, sigma 6): real outlier decisions at
    # N > 1,000
    "cfg1_outliers": dict(nsnp=50_000, pops=[330, 330, 332, 4, 4],
                          fst=[0.01, 0.01, 0.01, 0.25, 0.25], miss=0.01, seed=4,
                          keep_evals=200, evec_stride=1,
                          par={"numoutevec": "10", "numoutlieriter": "5"}),
    # N=5,000 x M=600,000, 6 populations 500..1,100, F 0.005..0.05, 2% missing, K=20, 5 outlier
    # iterations at sigma 6, lsqproject (the benchmark's full workload, generator seed 2)
    "cfg2_full": dict(nsnp=600_000, pops=[500, 700, 800, 900, 1000, 1100],
                      fst=[0.005, 0.01, 0.02, 0.03, 0.04, 0.05], miss=0.02, seed=2,
                      keep_evals=200, evec_stride=25,
                      par={"numoutevec": "20", "numoutlieriter": "5",
                           "outliersigmathresh": "6.0"}),
}


def records_sha256(rec):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(rec).tobytes()).hexdigest()


def make_big_case(name, spec, scratch):
    """Run the reference on a benchmark-shaped panel written to `scratch` (not committed) and
    keep the outputs named above under tests/golden/<name>/."""
    import json
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    w = os.path.join(scratch, name)
    os.makedirs(w, exist_ok=True)
    prefix = os.path.join(w, "data")
    native.synth_write_dataset(prefix, spec["nsnp"], spec["pops"], spec["fst"],
                               miss=spec["miss"], seed=spec["seed"])
    nind = sum(spec["pops"])
    rlen = max((nind + 3) // 4, 48)
    raw = np.fromfile(prefix + ".geno", np.uint8)[rlen:].reshape(spec["nsnp"], rlen)
    par = {"genotypename": "data.geno", "snpname": "data.snp", "indivname": "data.ind",
           "evecoutname": "out.evec", "evaloutname": "out.eval",
           "outlieroutname": "out.outliers", "numthreads": str(os.cpu_count() or 8)}
    par.update(spec["par"])
    with open(os.path.join(w, "par"), "w") as f:
        for k, v in par.items():
            f.write("%s: %s\n" % (k, v))
    env = dict(os.environ, EIG_REF_FULLPREC="1")
    with open(os.path.join(w, "ref.log"), "w") as log:
        subprocess.run([REF_BIN, "-p", "par"], cwd=w, env=env, stdout=log,
                       stderr=subprocess.STDOUT, check=True)
    ev = [float(x) for x in open(os.path.join(w, "out.eval")).read().split()]
    with open(os.path.join(d, "ref.eval"), "w") as f:
        for x in ev[:spec["keep_evals"]]:
            f.write("%.17g\n" % x)
    lines = open(os.path.join(w, "out.evec")).read().splitlines()
    with open(os.path.join(d, "ref.evec"), "w") as f:
        f.write(lines[0] + "\n")
        for i, ln in enumerate(lines[1:]):
            if i % spec["evec_stride"] == 0:
                f.write(ln + "\n")
    shutil.copy(os.path.join(w, "out.outliers"), os.path.join(d, "ref.outliers"))
    log = open(os.path.join(w, "ref.log")).read().splitlines()
    used = [ln for ln in log if "number of snps killed in pass" in ln or
            "number of samples used" in ln or "samples after outlier removal" in ln]
    with open(os.path.join(d, "ref.log"), "w") as f:
        f.write("\n".join(log[:80]) + "\n")
    kept = [int(ln.split("used:")[1]) for ln in used if "killed in pass" in ln]
    meta = {"nsnp": spec["nsnp"], "pops": spec["pops"], "fst": spec["fst"],
            "miss": spec["miss"], "seed": spec["seed"], "nind": nind,
            "records_sha256": records_sha256(raw), "par": spec["par"],
            "eval_count": len(ev), "eval_sum": float(np.sum(ev)),
            "kept_snps_per_pass": kept, "evec_stride": spec["evec_stride"],
            "log_counts": used}
    with open(os.path.join(d, "spec.json"), "w") as f:
        json.dump(meta, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    # usage: make_golden.py REFERENCE_ROOT [--scratch DIR] [case ...]
    args = sys.argv[1:]
    scratch = None
    if "--scratch" in args:
        i = args.index("--scratch")
        scratch = args[i + 1]
        del args[i:i + 2]
    if not args:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT [--scratch DIR] [case ...]")
    ref_root = args[0]
    if not os.path.exists(REF_BIN):
        raise SystemExit("build the reference first: sh oracle/build_ref.sh REFERENCE_ROOT")
    only = args[1:]  # optional case names
    if not only:
        copy_examples(ref_root)
    for name, spec in CASES.items():
        if only and name not in only:
            continue
        make_case(name, spec)
        print("made", name)
    for name, spec in CONVERT_CASES.items():
        if only and name not in only:
            continue
        make_convert_case(name, spec)
        print("made", name)
    for name, spec in FAST_CASES.items():
        if only and name not in only:
            continue
        make_fast_case(name, spec)
        print("made", name)
    for name, spec in BIG_CASES.items():
        if not only or name not in only:
            continue  # benchmark-shaped cases only on request (minutes to hours of CPU)
        if scratch is None:
            raise SystemExit("%s needs --scratch DIR for its (uncommitted) genotype files" % name)
        make_big_case(name, spec, scratch)
        print("made", name)

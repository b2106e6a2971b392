"""Loaders for the golden fixtures made by tests/golden/make_golden.py (reference outputs)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["bn_outliers", "bn_bed_altnorm", "bn_project", "bn_grm", "bn_missingmode",
         "bn_usepops", "bn_usepops_pl", "bn_snpwt"]
REL_CASES = ["bn_rel"]


def read_par(case):
    par = {}
    for line in open(os.path.join(GOLDEN, case, "par")):
        line = line.split("#")[0].strip()
        if not line:
            continue
        k, v = line.split(None, 1)
        par[k.rstrip(":")] = v.strip()
    return par


def yesno(v):
    return 1 if v == "YES" else 0 if v == "NO" else int(v)


class Case:
    def __init__(self, case):
        self.name = case
        d = os.path.join(GOLDEN, case)
        self.dir = d
        self.par = p = read_par(case)
        gname = os.path.join(d, p["genotypename"])
        ind_lines = [l.split() for l in open(os.path.join(d, p["indivname"])) if l.strip()]
        snp_lines = [l.split() for l in open(os.path.join(d, p["snpname"])) if l.strip()]
        self.nsnp = len(snp_lines)
        if gname.endswith(".bed"):
            self.code = 1
            self.ids = [l[1] for l in ind_lines]
            self.pops = [l[5] for l in ind_lines]
            self.nind = len(self.ids)
            blen = (self.nind + 3) // 4
            raw = open(gname, "rb").read()[3:]
            self.records = np.frombuffer(raw, np.uint8).reshape(self.nsnp, blen).copy()
        else:
            self.code = 0
            self.ids = [l[0] for l in ind_lines]
            self.pops = [l[2] for l in ind_lines]
            self.nind = len(self.ids)
            rlen = max((self.nind + 3) // 4, 48)
            raw = open(gname, "rb").read()[rlen:]
            self.records = np.frombuffer(raw, np.uint8).reshape(self.nsnp, rlen).copy()
        self.affstatus = None
        if "poplistname" in p:
            names = [l.split()[0] for l in open(os.path.join(d, p["poplistname"])) if l.strip()]
            keep = set(names)
            self.affstatus = np.array([pp in keep for pp in self.pops], np.uint8)
            eglist = names
        else:
            # makeeglist: populations in order of first appearance, "Ignore" left out
            eglist = []
            for pp in self.pops:
                if pp != "Ignore" and pp not in eglist:
                    eglist.append(pp)
        # the sample's index in the population list (xtypes), -1 when not listed
        self.ind_pop = np.array([eglist.index(pp) if pp in eglist else -1 for pp in self.pops],
                                np.int32)
        if os.path.exists(os.path.join(d, "ref.eval")):
            self.ref_evals = np.loadtxt(os.path.join(d, "ref.eval"))
            lines = open(os.path.join(d, "ref.evec")).read().splitlines()
            self.ref_header = [float(x) for x in lines[0].split()[1:]]
            self.ref_coords = {}
            for l in lines[1:]:
                t = l.split()
                if t:
                    self.ref_coords[t[0]] = np.array([float(x) for x in t[1:-1]])
        if os.path.exists(os.path.join(d, "ref.rel")):
            # smartrel "rel: ID ID y" lines, highest y first: full precision and as shipped
            self.ref_rel = [(t[1], t[2], float(t[3])) for t in
                            (l.split() for l in open(os.path.join(d, "ref.rel")))]
            self.ref_rel_text = open(os.path.join(d, "ref.rel.txt")).read().splitlines()
        self.ref_outlier_lines = [l.rstrip("\n") for l in open(os.path.join(d, "ref.outliers"))
                                  if l.startswith("REMOVED")]
        self.ref_outliers = [l.split()[2] for l in open(os.path.join(d, "ref.outliers"))
                             if l.startswith("REMOVED")]

    def opts(self):
        p = self.par
        kw = {}
        if "numoutevec" in p:
            kw["numeigs"] = int(p["numoutevec"])
        if "numoutlieriter" in p:
            kw["numoutliter"] = int(p["numoutlieriter"])
        if "altnormstyle" in p:
            kw["altnormstyle"] = yesno(p["altnormstyle"])
        if "maxmissing" in p:
            kw["maxmissing"] = int(p["maxmissing"])
        if "missingmode" in p:
            kw["missingmode"] = yesno(p["missingmode"])
        if "usepopsformissing" in p:
            kw["usepopsformissing"] = yesno(p["usepopsformissing"])
        return kw

    def rel_opts(self):
        """smartrel keyword arguments of this case's parfile"""
        p = self.par
        kw = {}
        if "numoutevec" in p:
            kw["numeigs"] = int(p["numoutevec"])
        if "relthresh" in p:
            kw["relthresh"] = float(p["relthresh"])
        if "minallelecnt" in p:
            kw["minallelecnt"] = int(p["minallelecnt"])
        if "numoutlieriter" in p:
            kw["numoutliter"] = int(p["numoutlieriter"])
        return kw

    def packed_records(self):
        """records in packedancestrymap code (bed recoded on the host, for the oracle)."""
        if self.code == 0:
            return self.records
        from oracle import oracle as O
        return O.bed_to_packed(self.records, self.nind)


def coords_by_id(ids, coords, ind_out):
    return {ids[k]: coords[:, k] for k in range(len(ids)) if ind_out[k]}


def compare_coords(ref, mine, K, tol):
    """sign-invariant (per eigenvector) max abs difference of .evec coordinates"""
    assert set(ref) == set(mine), "printed sample sets differ"
    ids = sorted(ref)
    A = np.array([ref[i][:K] for i in ids])
    B = np.array([mine[i][:K] for i in ids])
    s = np.sign(np.sum(A * B, axis=0))
    s[s == 0] = 1
    err = np.max(np.abs(A - B * s))
    assert err < tol, "coordinate error %g" % err
    return err


class Grm:
    """The reference's GRM dump of a grm case: full-precision text values, the shipped text
    lines, the binary floats and counts, the id lines."""

    def __init__(self, case):
        d = os.path.join(GOLDEN, case)
        full = np.loadtxt(os.path.join(d, "ref.grm"))
        self.ij = full[:, :2].astype(np.int64)
        self.numsnps = full[:, 2].astype(np.int64)
        self.values = full[:, 3]
        self.text = open(os.path.join(d, "ref.grm.txt")).read().splitlines()
        self.bin = np.fromfile(os.path.join(d, "ref.grm.bin"), np.float32)
        self.nbin = np.fromfile(os.path.join(d, "ref.grm.N.bin"), np.int32)
        self.ids = open(os.path.join(d, "ref.grm.id")).read().splitlines()


def float_ulps(a, b):
    """distance in float32 units in the last place"""
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(ia - ib)


def compare_grm_text(lines, ref_lines, values, ref_values):
    """same pairs and counts; values within 1e-10 of the reference; printed lines identical
    except where a value sits on a rounding boundary of %0.6f"""
    assert len(lines) == len(ref_lines)
    diff = [i for i, (a, b) in enumerate(zip(lines, ref_lines)) if a != b]
    for i in diff:
        a, b = lines[i].split(), ref_lines[i].split()
        assert a[:3] == b[:3]
        assert abs(float(a[3]) - float(b[3])) <= 1.0000001e-6
    assert len(diff) <= max(1, len(lines) // 10000)
    assert np.max(np.abs(np.asarray(values) - ref_values)) <= 1e-10 * np.max(np.abs(ref_values))


def rel_lines(ids, pairs):
    """the "rel:" lines smartrel prints (src/eigensrc/smartrel.c:611-615)"""
    return ["rel: %20s %20s  %9.3f" % (ids[a], ids[b], y) for a, b, y in pairs]


def compare_rel(pairs, ids, case, tol=1e-10):
    """same pairs in the same order as the reference, scores within tol; printed lines equal
    except where a score sits on a rounding boundary of %9.3f"""
    got = [(ids[a], ids[b]) for a, b, _ in pairs]
    want = [(a, b) for a, b, _ in case.ref_rel]
    assert got == want
    err = max([abs(y - r[2]) for (_, _, y), r in zip(pairs, case.ref_rel)] + [0.0])
    assert err <= tol, "relatedness score error %g" % err
    lines = rel_lines(ids, pairs)
    diff = [i for i, (a, b) in enumerate(zip(lines, case.ref_rel_text)) if a != b]
    for i in diff:
        assert abs(float(lines[i].split()[3]) - float(case.ref_rel_text[i].split()[3])) <= 1.0000001e-3
    assert len(diff) <= 1
    return err


def snp_table(case):
    """(chrom, gpos in morgans) per SNP of a case's .snp file, in file order (sorted)"""
    c = Case(case)
    rows = [l.split() for l in open(os.path.join(c.dir, c.par["snpname"])) if l.strip()]
    chrom = np.array([int(r[1]) for r in rows], np.int32)
    gpos = np.array([float(r[2]) for r in rows])
    if gpos.max() <= 0.00001:
        gpos = 1e-8 * np.array([float(r[3]) for r in rows])
    elif gpos.max() > 100:
        gpos = gpos / 100.0
    return chrom, gpos


def eglist(case, par=None):
    """populations in the reference's order: the poplist, else first appearance"""
    c = Case(case)
    p = par or c.par
    if "poplistname" in p:
        return [l.split()[0] for l in open(os.path.join(c.dir, p["poplistname"])) if l.strip()]
    out = []
    for pop in c.pops:
        if pop != "Ignore" and pop not in out:
            out.append(pop)
    return out


def read_fstdetails(path):
    """{(pop1, pop2): (fst, fstjack, stderr, z, snpnumber)}"""
    out = {}
    for line in open(path):
        t = line.split()
        if t and t[0] == "F_st":
            out[(t[1], t[2])] = tuple(float(x) for x in t[3:7]) + (int(t[7]),)
    return out


def log_section(text):
    """the population summary and Fst section of a smartpca log: from the first
    "population:" line through the "std. err." matrix"""
    lines = text.splitlines()
    i0 = next(i for i, l in enumerate(lines) if l.startswith("population:"))
    i1 = next(i for i, l in enumerate(lines) if l.startswith("std. err."))
    j = i1 + 1
    while j < len(lines) and lines[j].strip():
        j += 1
    return lines[i0:j]


def anova_section(text):
    """the ANOVA tail of a smartpca log: {"means": {j: [(pop, mean)]}, "p": {name: p},
    "minmax": {j: (minpop, minv, maxpop, maxv)}, "popdiff": [(p1, p2, chisq, p, n1, n2)]}"""
    out = {"means": {}, "p": {}, "minmax": {}, "popdiff": []}
    lines = text.splitlines()
    j = None
    mode = None
    for line in lines:
        t = line.split()
        if line.startswith("eigenvector ") and line.endswith(":means"):
            j = int(t[1].split(":")[0])
            out["means"][j] = []
            mode = "means"
            continue
        if mode == "means" and len(t) == 2 and not t[0].startswith("eigenvector_"):
            out["means"][j].append((t[0], float(t[1])))
            continue
        mode = None
        if t and t[0].startswith("eigenvector_") and len(t) >= 2:
            out["p"][t[0]] = float(t[1])
        elif len(t) == 6 and t[1] == "minv:" and t[4] == "maxv:":
            out["minmax"][j] = (t[0], float(t[2]), t[3], float(t[5]))
        elif t and t[0] == "popdifference:":
            out["popdiff"].append((t[1], t[2], float(t[3]), float(t[4]), int(t[5]), int(t[6])))
    return out


def compare_anova(mine, ref):
    """means and min/max up to each eigenvector's sign; p-values and chi-squares numerically"""
    assert set(mine["means"]) == set(ref["means"]) and mine["means"]
    for j, want in ref["means"].items():
        got = mine["means"][j]
        same = sorted(got) == sorted(want)
        flip = sorted((p, -m if m != 0 else 0.0) for p, m in got) == \
            sorted((p, m if m != 0 else 0.0) for p, m in want)
        assert same or flip, (j, got, want)
    assert set(mine["p"]) == set(ref["p"])
    for k, b in ref["p"].items():
        a = mine["p"][k]
        assert abs(a - b) <= 2e-5 * abs(b) + 1e-15, (k, a, b)
    assert len(mine["popdiff"]) == len(ref["popdiff"])
    for a, b in zip(mine["popdiff"], ref["popdiff"]):
        assert a[:2] == b[:2] and a[4:] == b[4:]
        assert abs(a[2] - b[2]) <= 1.5e-3 * max(1.0, abs(b[2]) * 1e-6)
        assert abs(a[3] - b[3]) <= 2e-5 * abs(b[3]) + 1e-15, (a, b)


class FastCase:
    """The reference's fastmode runs on bn_fastmode (make_golden.py FAST_CASES): the panel,
    and per parfile its (K, L, I, seed) and the printed .evec (eigenvalues of the header,
    unit-norm vectors as rows), at full precision and as shipped."""

    RUNS = {"par": ("", 4, 8, 4, 3), "par_odd": ("_odd", 3, 7, 3, 5)}

    def __init__(self):
        d = os.path.join(GOLDEN, "bn_fastmode")
        self.dir = d
        ind = [l.split() for l in open(os.path.join(d, "data.ind")) if l.strip()]
        self.ids = [t[0] for t in ind]
        self.nind = len(ind)
        self.nsnp = sum(1 for l in open(os.path.join(d, "data.snp")) if l.strip())
        rlen = max((self.nind + 3) // 4, 48)
        raw = np.fromfile(os.path.join(d, "data.geno"), np.uint8)[rlen:]
        self.records = raw.reshape(self.nsnp, rlen).copy()

    def run(self, par):
        tag, K, L, I, seed = self.RUNS[par]
        lines = open(os.path.join(self.dir, "ref%s.evec" % tag)).read().splitlines()
        ev = np.array([float(x) for x in lines[0].split()[1:]])
        V = np.array([[float(x) for x in l.split()[1:-1]] for l in lines[1:]]).T
        return dict(K=K, L=L, I=I, seed=seed, evals=ev, evecs=V,
                    text=open(os.path.join(self.dir, "ref%s.evec.txt" % tag)).read().splitlines())


def snp_rows(case):
    """(ID, chrom, physpos) of each SNP of a case, in file order (the records' order)"""
    c = Case(case)
    path = os.path.join(c.dir, c.par["snpname"])
    rows = []
    for l in open(path):
        t = l.split()
        if not t:
            continue
        if path.endswith(".bim"):
            rows.append((t[1], int(t[0]), int(round(float(t[3])))))
        else:
            rows.append((t[0], int(t[1]), int(round(float(t[3])))))
    return rows


def eigbestsnp_lines(text):
    """the "eigbestsnp" log lines as (vector, ID, chrom, physpos, value)"""
    out = []
    for l in text.splitlines():
        if l.startswith("eigbestsnp"):
            t = l.split()
            out.append((int(t[1]), t[2], int(t[3]), int(t[4]), float(t[5])))
    return out


def kurtosis_lines(text):
    """the log's "eigenvector j kurt_snps kurt_indivs" lines after its kurtosis header"""
    out, on = [], False
    for l in text.splitlines():
        t = l.split()
        if t[:3] == ["kurtosis", "snps", "indivs"]:
            on = True
            continue
        if on:
            if len(t) == 4 and t[0] == "eigenvector":
                out.append((int(t[1]), float(t[2]), float(t[3])))
            else:
                break
    return out



def tw_section(text):
    """the log's mpstats quartiles (or None) and Tracy-Widom rows: per row (index, eigenvalue,
    difference or None, twstat or None, p-value or None, effective n or None), plus the
    section's (rows, cols); a section that runs to the end of a stored log that was cut short
    returns only the rows it holds"""
    lines = text.splitlines()
    mp, rows, shape = None, [], None
    for k, l in enumerate(lines):
        if l.startswith("mpstats:"):
            mp = [float(v) for v in l.split()[1:]]
        if l.startswith("## Tracy-Widom statistics:"):
            t = l.split()
            shape = (int(t[4]), int(t[6]))
            for r in lines[k + 2:]:
                f = r.split()
                if len(f) != 6 or not f[0].isdigit():
                    break
                val = [None if v == "NA" else float(v) for v in f[2:]]
                rows.append((int(f[0]), float(f[1])) + tuple(val))
            break
    return mp, shape, rows


PROGRESS_PREFIXES = ("norm used", "no norm used", "lsqproject used", "packed geno read OK",
                     "end of inpack", "genotype file processed", "snps deleted (nodata):",
                     "number of pops for axes:", " snp ", "total number of snps killed in pass:",
                     "number of samples after outlier removal:", "lsqproj called!",
                     "writing eigenvecotrs for", "end of smartpca(fastmode)")


def progress_lines(text):
    """the log's run-progress lines (the preamble after the parameters, the per-pass kill and
    outlier-removal lines, lsqproj's and fastmode's markers), in order"""
    return [l for l in text.splitlines() if l.startswith(PROGRESS_PREFIXES)]

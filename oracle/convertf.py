"""ORACLE — test infrastructure only.

CPU restatement of convertf's default path (src/convertf.c main, EIGENSOFT 8.0.0) and of its
packed writers, in numpy: the checker for the GPU record encoder (gp_encode_records) and the
gpuconvertf CLI.  Pinned against the reference convertf binary (oracle/build_ref.sh) through
the fixtures of tests/golden/cv_* (made by tests/golden/make_golden.py).
"""
import os

import numpy as np

from oracle import oracle as O


def hashit(s):
    """hashit (src/admutils.c:668-682): h = h*23 + c over the (signed) bytes, int32 wrap"""
    h = 0
    for c in s.encode():
        c = c - 256 if c > 127 else c
        h = (h * 23 + c) & 0xFFFFFFFF
    return h


def hasharr(ids):
    """hasharr (src/admutils.c:651-665): h = (h*17) ^ hashit(id), in list order"""
    h = 0
    for s in ids:
        h = ((h * 17) & 0xFFFFFFFF) ^ hashit(s)
    return h


def pedval_mod5(c):
    """pedval (src/mcio.c:3848-3887) % 5 of an allele character"""
    if c in "ACGT1234":
        return "ACGT1234".index(c) % 4 + 1
    if c in "XNDI0":
        return 0
    return 4


def read_snps(path):
    """SNP list as the reference reads it (readsnpdata src/mcio.c:420-535 / readsnpmapdata
    :538-660): ids, chrom, gpos (morgans; all zero -> 1e-8 * ppos; cM if any > 100), ppos,
    alleles; sorted by (chrom, gpos, ppos) as the records are."""
    plink = path.endswith((".bim", ".map", ".pedsnp"))
    rows = []
    for line in open(path):
        t = line.split()
        if not t or t[0].startswith("#"):
            continue
        sid, ch = (t[1], t[0]) if plink else (t[0], t[1])
        al = ["", ""]
        if len(t) >= 6:
            for a in range(2):
                c = t[4 + a][0]
                al[a] = ("X" if c == "0" else c) if plink else c.upper()
        rows.append([sid, chrom_of(ch), float(t[2]), float(t[3]), al])
    g = [r[2] for r in rows]
    if rows and max(g) <= 0.00001:
        for r in rows:
            r[2] = 1e-8 * r[3]
    elif any(x > 100 for x in g):
        for r in rows:
            r[2] /= 100.0
    order = sorted(range(len(rows)), key=lambda i: (rows[i][1], round(rows[i][2] * 1e6),
                                                    round(rows[i][3]), i))
    return [rows[i] for i in order], order


def chrom_of(s, numchrom=22):
    s = s[3:] if s.startswith("chr") else s
    s = s.upper()
    if s == "X":
        return numchrom + 1
    if s == "Y":
        return numchrom + 2
    if s == "MT":
        return 90
    if s == "XY":
        return 91
    return int(s) if s.isdigit() else -1


def read_inds(path, familynames=True):
    """(ids, gender, pop, ignore) as getindivs reads .ind / .fam (src/mcio.c:958-1100)"""
    ped = path.endswith((".fam", ".ped", ".pedind"))
    out = []
    for line in open(path):
        t = line.split()
        if not t or t[0].startswith("#"):
            continue
        if not ped:
            out.append((t[0], t[1][0], t[2], t[2] == "Ignore"))
        else:
            sid = "%s:%s" % (t[0], t[1]) if familynames else t[1]
            sx = int(t[4])
            g = "M" if sx == 1 else "F" if sx == 2 else "U"
            ph = t[5]
            pop = {"-9": "Ignore", "9": "Ignore", "0": "Ignore", "1": "Control",
                   "2": "Case"}.get(ph, ph)
            out.append((sid, g, pop, pop == "Ignore"))
    return out


def read_genotypes(path, nsnp, nind, order):
    """genotype matrix (sorted SNP order x samples, -1 missing) from packed, bed or text"""
    raw = open(path, "rb").read()
    if raw[:3] == bytes([0x6C, 0x1B, 0x01]):
        blen = (nind + 3) // 4
        rec = np.frombuffer(raw[3:], np.uint8).reshape(nsnp, blen)
        g = O.unpack(O.bed_to_packed(rec, nind), nind)
    elif raw[:4] == b"GENO":
        rlen = max((nind + 3) // 4, 48)
        rec = np.frombuffer(raw[rlen:], np.uint8).reshape(nsnp, rlen)
        g = O.unpack(rec, nind)
    else:
        lines = raw.decode().split("\n")[:nsnp]
        a = np.array([[int(c) for c in l[:nind]] for l in lines], np.int16)
        g = np.where(a == 9, -1, a)
    return np.asarray(g)[np.asarray(order)]


def convertf(geno, snps, inds, fmt, poplist=None, deletedup=True, minchrom=1, maxchrom=97):
    """convertf main() (src/convertf.c:206-540) on the default path, then outfiles
    (src/mcio.c:3206-3258): returns {"geno": bytes, "snp": str, "ind": str} of the output
    format fmt ("PACKEDANCESTRYMAP", "PACKEDPED" or "EIGENSTRAT")."""
    M, N = geno.shape
    ign = np.array([not (minchrom <= s[1] <= maxchrom) or s[1] <= 0 for s in snps])
    if deletedup:  # dedupit / pickx (:881-943)
        prev = -1
        for i in range(M):
            if ign[i]:
                continue
            if prev < 0 or snps[prev][1] != snps[i][1] or snps[prev][3] != snps[i][3]:
                prev = i
                continue
            a, b = snps[prev][0], snps[i][0]
            keep_prev = len(a) < len(b) if len(a) != len(b) else a >= b
            if keep_prev:
                ign[i] = True
            else:
                ign[prev] = True
                prev = i
    g = geno.copy()
    alleles = [list(s[4]) for s in snps]
    for i in range(M):  # flip1 (:356-368, :1017-1026)
        a0 = alleles[i][0] or "\x00"
        a1 = alleles[i][1] or "\x00"
        if pedval_mod5(a0) == 0 and pedval_mod5(a1) > 0:
            obs = g[i] >= 0
            g[i, obs] = 2 - g[i, obs]
            alleles[i] = [alleles[i][1], alleles[i][0]]
    keep = np.array([not x[3] for x in inds])
    aff = np.zeros(N, bool)
    if poplist is not None:
        aff = np.array([x[2] in poplist for x in inds])
        keep &= aff
    else:
        aff = np.array([x[2] == "Case" for x in inds])
    kept_snps = np.nonzero(~ign)[0]
    nodata = (g[kept_snps] >= 0).sum(axis=0) == 0
    keep &= ~nodata
    ks = np.nonzero(keep)[0]
    sub = g[np.ix_(kept_snps, ks)]
    n = len(ks)
    out = {}
    snp_lines, ind_lines = [], []
    for i in kept_snps:
        sid, ch, gp, pp, _ = snps[i]
        al = "".join(" %s" % c for c in alleles[i] if c)
        if fmt == "PACKEDPED":
            snp_lines.append("%-2s %12s %12.6f %12.0f%s\n" % (str(ch), sid, gp, pp, al))
        elif gp == 0.0:
            snp_lines.append("%20s %5s %15.0f %15.0f%s\n" % (sid, str(ch), gp, pp, al))
        else:
            snp_lines.append("%20s %5s %15.6f %15.0f%s\n" % (sid, str(ch), gp, pp, al))
    for j, k in enumerate(ks):
        sid, sex, pop, _ = inds[k]
        if fmt == "PACKEDPED":
            pg = 1 if sex == "M" else 2 if sex == "F" else 0
            ind_lines.append("%6d   %12s %d %d %d %d\n" % (j + 1, sid, 0, 0, pg, int(aff[k]) + 1))
        else:
            ind_lines.append("%20s %s %10s\n" % (sid, sex, pop))
    out["snp"] = "".join(snp_lines)
    out["ind"] = "".join(ind_lines)
    out["geno"] = encode(sub, fmt, ids=[inds[k][0] for k in ks],
                         snp_ids=[snps[i][0] for i in kept_snps])
    return out


def encode(sub, fmt, ids=None, snp_ids=None, header=True):
    """genotype file bytes of the records (SNPs x samples, -1 missing): outpack with its GENO
    header (src/mcio.c:2343-2457), outpackped with the bed magic (:3619-3741) or
    outeigenstrat text (:3262-3320)"""
    M, n = sub.shape
    if fmt == "EIGENSTRAT":
        ch = np.where(sub < 0, ord("9"), sub + ord("0")).astype(np.uint8)
        return np.concatenate([ch, np.full((M, 1), ord("\n"), np.uint8)], axis=1).tobytes()
    if fmt == "PACKEDANCESTRYMAP":
        rlen = max((n + 3) // 4, 48)
        codes = np.where(sub < 0, 3, sub).astype(np.uint8)
        pad = np.zeros((M, rlen * 4 - n), np.uint8)
        c = np.concatenate([codes, pad], axis=1).reshape(M, rlen, 4)
        rec = (c[:, :, 0] << 6) | (c[:, :, 1] << 4) | (c[:, :, 2] << 2) | c[:, :, 3]
        body = rec.astype(np.uint8).tobytes()
        if not header:
            return body
        h = ("GENO %7d %7d %x %x" % (n, M, hasharr(ids), hasharr(snp_ids))).encode()
        return h + bytes(rlen - len(h)) + body
    # PACKEDPED: g -> 2-g, bedval 0->00 1->10 2->11 missing->01, LSB first, pad 10
    blen = (n + 3) // 4
    gg = np.where(sub < 0, -1, 2 - sub)
    code = np.where(gg < 0, 1, np.where(gg == 2, 3, np.where(gg == 1, 2, 0))).astype(np.uint8)
    pad = np.full((M, blen * 4 - n), 2, np.uint8)
    c = np.concatenate([code, pad], axis=1).reshape(M, blen, 4)
    rec = c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)
    body = rec.astype(np.uint8).tobytes()
    return (bytes([0x6C, 0x1B, 0x01]) + body) if header else body


def run_par(d, par):
    """the oracle on a parfile dict with paths relative to directory d"""
    snps, order = read_snps(os.path.join(d, par["snpname"]))
    inds = read_inds(os.path.join(d, par["indivname"]), par.get("familynames", "YES") != "NO")
    geno = read_genotypes(os.path.join(d, par["genotypename"]), len(snps), len(inds), order)
    pl = None
    if "poplistname" in par:
        pl = {l.split()[0] for l in open(os.path.join(d, par["poplistname"])) if l.strip()}
    return convertf(geno, snps, inds, par.get("outputformat", "PACKEDANCESTRYMAP"), poplist=pl)

"""Build the native parts in-tree: the CUDA library (sm_103a), the host CLI, the synthetic
generator and the C oracle.  Plain nvcc/gcc invocations, compiled in parallel, no cmake.

Outputs (git-ignored):
  eig_gb300/_lib/libgpupca.so   C ABI of the hot path (include/gpupca.h, gpupca_run.h)
  eig_gb300/_lib/libgpsynth.so  host helpers: seeded Balding-Nichols generator (gp_synth.h) and
                                the ANOVA tail probabilities (gp_stats.h)
  eig_gb300/_lib/gpusmartpca    drop-in CLI: smartpca -p parfile
  eig_gb300/_lib/gpusmartrel    drop-in CLI: smartrel -p parfile
  eig_gb300/_lib/gpuconvertf    drop-in CLI: convertf -p parfile (packed/bed/EIGENSTRAT writers)
  oracle/_bin/liboracle.so      the CPU oracle (test infrastructure)
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "eig_gb300")
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIB = os.path.join(PKG, "_lib")
OBJ = os.path.join(LIB, "obj")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BIN = os.path.join(ORACLE, "_bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + os.path.join(ROOT, "include")]
CUDA_SOURCES = ["gp_api.cu", "gp_geno.cu", "gp_gram_f64.cu", "gp_geno_gemm_f64.cu",
                "gp_gram_bf16.cu", "gp_fast.cu",
                "gp_noalloc.cu", "gp_geno_tc.cu", "gp_eig.cu", "gp_serve.cu", "gp_convert.cu",
                "gp_fst.cu", "gp_popfill.cu"]
HOST_LIB_SOURCES = ["gp_smartpca.c", "gp_tw.c"]
# no FMA contraction in host code: the reference's host arithmetic is plain multiply-add
# (aarch64 would otherwise fuse it)
CFLAGS = ["-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wno-unused-result", "-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _headers(d):
    return [os.path.join(d, f) for f in os.listdir(d) if f.endswith(".h")] + [
        os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(ORACLE_BIN, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers(CSRC) + _headers(HOST)
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in HOST_LIB_SOURCES:
        s = os.path.join(HOST, src)
        o = os.path.join(OBJ, src.replace(".c", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append(["gcc"] + CFLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(LIB, "libgpupca.so")
    if force or _newer(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs +
             ["-lcusolver", "-lcublas", "-lcudart", "-lpthread", "-lm"])
    synth = os.path.join(LIB, "libgpsynth.so")
    ss = [os.path.join(HOST, "gp_synth.c"), os.path.join(HOST, "gp_stats.c")]
    if force or _newer(synth, ss + hdrs):
        _run(["gcc"] + CFLAGS + ["-shared", "-o", synth] + ss + ["-lm", "-lpthread"])
    cli = os.path.join(LIB, "gpusmartpca")
    cli_src = [os.path.join(HOST, "gpusmartpca_main.c"), os.path.join(HOST, "gp_io.c"),
               os.path.join(HOST, "gp_synth.c"), os.path.join(HOST, "gp_stats.c")]
    if all(os.path.exists(s) for s in cli_src) and (force or _newer(cli, cli_src + hdrs + [lib])):
        _run(["gcc"] + CFLAGS + ["-o", cli] + cli_src +
             ["-L" + LIB, "-lgpupca", "-Wl,-rpath,$ORIGIN", "-lm", "-lpthread"])
    rel = os.path.join(LIB, "gpusmartrel")
    rel_src = [os.path.join(HOST, "gpusmartrel_main.c"), os.path.join(HOST, "gp_io.c"),
               os.path.join(HOST, "gp_synth.c")]
    if all(os.path.exists(s) for s in rel_src) and (force or _newer(rel, rel_src + hdrs + [lib])):
        _run(["gcc"] + CFLAGS + ["-o", rel] + rel_src +
             ["-L" + LIB, "-lgpupca", "-Wl,-rpath,$ORIGIN", "-lm", "-lpthread"])
    cvt = os.path.join(LIB, "gpuconvertf")
    cvt_src = [os.path.join(HOST, "gpuconvertf_main.c"), os.path.join(HOST, "gp_io.c"),
               os.path.join(HOST, "gp_synth.c")]
    if all(os.path.exists(s) for s in cvt_src) and (force or _newer(cvt, cvt_src + hdrs + [lib])):
        _run(["gcc"] + CFLAGS + ["-o", cvt] + cvt_src +
             ["-L" + LIB, "-lgpupca", "-Wl,-rpath,$ORIGIN", "-lm", "-lpthread"])
    orc = os.path.join(ORACLE_BIN, "liboracle.so")
    osrc = os.path.join(ORACLE, "smartpca_oracle.c")
    if force or _newer(orc, [osrc]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-o", orc, osrc, "-lm", "-lpthread"])
    ref_sh = os.path.join(ORACLE, "build_ref.sh")
    ref_bin = os.path.join(ORACLE, "_ref", "smartpca")
    if force or not os.path.exists(ref_bin):
        # builds the reference smartpca only where its sources are present; else a no-op
        _run(["sh", ref_sh])
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print("ok")

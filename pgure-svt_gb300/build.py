"""Build recipe of libpgsvt.so (the CUDA library behind include/pgsvt.h).

Every translation unit under csrc/ is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
``pgure-svt_gb300/libpgsvt.so`` next to this file; the command-line tool
``cli/pgsvt_cli.cpp`` (host C++ on the C ABI) becomes ``pgure-svt_gb300/pgsvt_cli``.  nvcc cross-compiles without
a GPU, so the same recipe runs on a build host and on the GPU machine.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpgsvt.so")
SOURCES = ["prep.cu", "arps.cu", "svd.cu", "svd_i0.cu", "svd_i1.cu", "svd_i2.cu", "svd_i3.cu",
           "svd_i4.cu", "svd_i5.cu", "svd_i6.cu", "svd_i7.cu", "svd_i8.cu", "svd_split.cu", "svd_s0.cu", "svd_s1.cu",
           "svd_s2.cu", "svd_s3.cu", "svd_s4.cu", "eval.cu", "lambda.cu", "noise.cu", "hotpixel.cu",
           "capi.cu", "noalloc.cu"]
CLI_SRC = os.path.join(HERE, "cli", "pgsvt_cli.cpp")
CLI = os.path.join(HERE, "pgsvt_cli")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _flags(ptxas_verbose=False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    # developer knob for kernel experiments, e.g. PGSVT_NVCC_FLAGS="-DPGSVT_SVD_PRED"
    f += os.environ.get("PGSVT_NVCC_FLAGS", "").split()
    if ptxas_verbose:
        f += ["-Xptxas", "-v"]
    return f


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile (if out of date) and return the path of libpgsvt.so."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "pgsvt.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src[:-3] + ".o")
        objs.append(o)
        if force or ptxas_verbose or _stale(o, [s, __file__] + headers):
            jobs.append([nvcc()] + _flags(ptxas_verbose) + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(os.cpu_count() or 4, len(jobs))) as ex:
            for err in ex.map(run, jobs):
                if verbose and err:
                    print(err)
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        run([nvcc()] + ARCH + ["-shared", "-cudart=static", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    # the command-line tool: host C++ on the C ABI, next to the library
    if force or _stale(CLI, [CLI_SRC, LIB, os.path.join(ROOT, "include", "pgsvt.h")]):
        tmp = CLI + ".tmp%d" % os.getpid()
        run(["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), CLI_SRC,
             "-L", HERE, "-lpgsvt", "-Wl,-rpath,$ORIGIN", "-o", tmp])
        os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                ptxas_verbose="--ptxas" in sys.argv))

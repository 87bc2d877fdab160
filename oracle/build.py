"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/pgsvt_oracle.cpp`` and ``oracle/noise_oracle.cpp`` with g++ into
``oracle/_build/libpgsvt_oracle.so``.  ``-ffp-contract=off`` keeps the FP64
arithmetic identical on x86_64 and aarch64 (no fused multiply-adds), so the
oracle's ARPS costs and argmins are the same bits on both machines.

When the reference tree is present (``--ref`` or ``build_ref()``), it also
builds ``oracle/_ref/ref_probes``: a probe dump program compiled against the
reference's own vendored PCG header (src/pcg/pcg_random.hpp), used only to
generate the golden probe fixtures in tests/golden/, and
``oracle/_ref/libref_medfilter.so``: the reference's constant-time median
filter (src/medfilter.hpp) compiled from its header, used to generate the
golden median fixtures and to check the oracle's median restatement.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpgsvt_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_PROBES = os.path.join(REF_DIR, "ref_probes")
REF_MEDIAN = os.path.join(REF_DIR, "libref_medfilter.so")
# The reference tree: PGSVT_REFERENCE names its root; the default is where this
# recipe expects the read-only checkout.
REFERENCE_ROOT = os.environ.get("PGSVT_REFERENCE", "/root/reference")
REFERENCE_SRC = os.path.join(REFERENCE_ROOT, "src")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(force=False, verbose=False):
    """Compile the oracle shared library if it is missing or out of date."""
    src = os.path.join(HERE, "pgsvt_oracle.cpp")
    src2 = os.path.join(HERE, "noise_oracle.cpp")
    hdr = os.path.join(HERE, "pgsvt_oracle.h")
    if not force and not _stale(LIB, [src, src2, hdr, __file__]):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-pthread",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
           "-o", tmp, src, src2]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_ref(force=False):
    """Compile the probe dump program against the reference's PCG header.

    Returns the binary path, or None when the reference tree is absent.
    """
    pcg = os.path.join(REFERENCE_SRC, "pcg", "pcg_random.hpp")
    if not os.path.exists(pcg):
        return None
    src = os.path.join(HERE, "ref_probes.cpp")
    if not force and not _stale(REF_PROBES, [src]):
        return REF_PROBES
    os.makedirs(REF_DIR, exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(REFERENCE_SRC, "pcg"),
                    "-o", REF_PROBES, src], check=True)
    return REF_PROBES


def build_ref_median(force=False):
    """Compile the reference's median filter (src/medfilter.hpp, plain C)
    behind oracle/ref_medfilter.c.  Returns the library path, or None when
    the reference tree is absent."""
    hdr = os.path.join(REFERENCE_SRC, "medfilter.hpp")
    if not os.path.exists(hdr):
        return None
    src = os.path.join(HERE, "ref_medfilter.c")
    if not force and not _stale(REF_MEDIAN, [src]):
        return REF_MEDIAN
    os.makedirs(REF_DIR, exist_ok=True)
    subprocess.run(["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-I", REFERENCE_SRC,
                    "-o", REF_MEDIAN, src, "-lm"], check=True)
    return REF_MEDIAN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    if "--ref" in sys.argv:
        print(build_ref(force=True))
        print(build_ref_median(force=True))

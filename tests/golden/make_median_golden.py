"""Generate tests/golden/median.npz from the reference's own median filter.

Runs ConstantTimeMedianFilter (src/medfilter.hpp of the reference tree,
compiled by oracle/build.py into oracle/_ref/libref_medfilter.so) on seeded
uint16 frames, called as pguresvt.hpp:69-80 calls it, and stores inputs and
outputs.  Needs the reference tree; the fixture is committed.

    python tests/golden/make_median_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build  # noqa: E402

# (side, radius, value range): the default radius 5, small and large radii,
# full 16-bit range and a narrow one (many ties)
CASES = [(32, 5, 65536), (48, 5, 300), (33, 1, 12), (40, 7, 4096), (11, 5, 100),
         (64, 3, 65536), (24, 11, 1000)]


def main():
    lib = build.build_ref_median(force=True)
    if lib is None:
        raise SystemExit("reference tree not found")
    L = ctypes.CDLL(lib)
    L.ref_median_filter.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int]
    rng = np.random.default_rng(2024)
    out = {}
    for k, (S, r, hi) in enumerate(CASES):
        a = np.asfortranarray(rng.integers(0, hi, (S, S)).astype(np.uint16))
        ref = np.zeros_like(a, order="F")
        L.ref_median_filter(a.ctypes.data, ref.ctypes.data, S, S, r)
        out["in_%d" % k] = a
        out["out_%d" % k] = ref
        out["r_%d" % k] = np.array(r)
    out["n"] = np.array(len(CASES))
    np.savez_compressed(os.path.join(HERE, "median.npz"), **out)
    print("wrote", os.path.join(HERE, "median.npz"))


if __name__ == "__main__":
    main()

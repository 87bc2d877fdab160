"""Generate tests/golden/noise.npz: seeded normalised windows and the noise
estimator restatement's outputs on them (methods 1-4), frozen so that later
changes to the oracle and the GPU estimator are checked against them.

    python tests/golden/make_noise_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

# (workload, side, frames, seed): power-of-two frames as the estimator needs
CASES = [("arps_256", 32, 15, 1), ("lattice_512", 64, 9, 2), ("plain_64", 16, 5, 3),
         ("arps_256", 128, 3, 4)]


def main():
    pkg = entry.load_package()
    O = entry.load_oracle()
    out = {}
    for k, (wl, side, nt, seed) in enumerate(CASES):
        noisy, _, _ = pkg.synth.workload(wl, seed=seed, side=side, nt=nt)
        u = noisy.astype(np.float64)
        u /= u.max()
        out["u_%d" % k] = np.asfortranarray(u)
        out["est_%d" % k] = np.array([O.noise_estimate(u, method=m) for m in (1, 2, 3, 4)])
    out["n"] = np.array(len(CASES))
    np.savez_compressed(os.path.join(HERE, "noise.npz"), **out)
    print({k: v for k, v in out.items() if k.startswith("est")})


if __name__ == "__main__":
    main()

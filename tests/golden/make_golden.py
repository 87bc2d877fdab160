"""Generate the golden fixtures in tests/golden/.

* probes.npz / probes_sha256.json: the PGURE probe stream (delta1, delta2) of
  the reference's own vendored PCG engine and libstdc++'s bernoulli
  distribution, dumped by oracle/_ref/ref_probes (compiled from
  src/pcg/pcg_random.hpp of the reference tree, see oracle/build.py).  This
  pins the probe restatement of both the oracle and the CUDA library.
* oracle_small.npz: frozen FP64 oracle outputs (ARPS trajectory tables,
  singular values, a reconstruction, risks and a full denoise) on a seeded
  32x32x16 synthetic sequence, so GPU parity can also be checked against
  vectors that do not move if the oracle is edited.

Run from the repository root where the reference tree is mounted:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

SEEDS = [0, 1, 101, 7 + (1 << 40)]
N_SMALL = 4096
N_HASH = 1_000_000


def ref_probes(binary, seed, n):
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "p.bin")
        subprocess.run([binary, str(seed), str(n), out], check=True)
        raw = open(out, "rb").read()
    d1 = np.frombuffer(raw[:n], np.int8).copy()
    d2 = np.frombuffer(raw[n:], np.float64).copy()
    return d1, d2, hashlib.sha256(raw).hexdigest()


def main():
    ob = entry._load_builder(os.path.join(ROOT, "oracle", "build.py"), "_ob")
    binary = ob.build_ref(force=True)
    if binary is None:
        raise SystemExit("reference tree not mounted: cannot regenerate probe goldens")
    arrays, digests = {}, {}
    for s in SEEDS:
        d1, d2, _ = ref_probes(binary, s, N_SMALL)
        arrays["d1_%d" % s] = d1
        arrays["d2_%d" % s] = d2
        digests[str(s)] = ref_probes(binary, s, N_HASH)[2]
    np.savez_compressed(os.path.join(HERE, "probes.npz"), **arrays)
    with open(os.path.join(HERE, "probes_sha256.json"), "w") as f:
        json.dump({"n": N_HASH, "layout": "n int8 delta1 then n float64 delta2",
                   "sha256": digests}, f, indent=1)

    # frozen oracle vectors on a small synthetic sequence
    pkg = entry.load_package()
    O = entry.load_oracle()
    noisy, clean, (a, m, s) = pkg.synth.workload("arps_256", seed=5, side=32, nt=16)
    X = noisy.astype(np.float64)
    bs, mw, T = 4, 7, 15
    ntc, fw, nwin = O.window_geometry(T, bs)
    out = {"X": noisy, "alpha": a, "mu": m, "sigma": s}
    for t in (0, 3, 8, 15):
        s0 = 0 if t < fw else (len(X[0, 0]) - 2 * fw - 1 if t >= X.shape[2] - fw else t - fw)
        u = X[:, :, s0:s0 + nwin] / X[:, :, s0:s0 + nwin].max()
        rows, cols = O.arps_window(u, bs, mw, t, fw, X.shape[2])
        out["rows_%d" % t] = rows.astype(np.int16)
        out["cols_%d" % t] = cols.astype(np.int16)
        if t == 8:
            out["u_8"] = u
            out["S_8"] = O.svd_window(u, bs, 1, rows, cols)
            out["v_8_l1"] = O.reconstruct_window(u, bs, 1, rows, cols, 1.0)
            lams = np.array([0.05, 0.5, 2.0, 10.0, 60.0])
            out["risk_lams"] = lams
            out["risk_8_compat"] = O.risk_window(u, bs, 1, rows, cols, lams, a, m, s, 11,
                                                 compat=O.COMPAT_ALL)
            out["risk_8_fixed"] = O.risk_window(u, bs, 1, rows, cols, lams, a, m, s, 11, compat=0)
    kw = dict(traj_length=T, block_size=bs, block_overlap=1, motion_window=mw, median_size=-1,
              random_seed=11, optimize_pgure=1, alpha=a, mu=m, sigma=s, search_points=8,
              search_rounds=2)
    Y, est, _ = O.denoise(noisy, n_jobs=4, **kw)
    out["Y_pgure"] = Y
    out["est_pgure"] = est
    Y1, est1, _ = O.denoise(noisy, n_jobs=4, traj_length=T, block_size=bs, motion_window=mw,
                            median_size=-1, optimize_pgure=0, lambda_=0.1)
    out["Y_fixed"] = Y1
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **out)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()

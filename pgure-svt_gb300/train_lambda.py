"""Train the learned lambda proposal and write the shipped model.

    python pgure-svt_gb300/train_lambda.py --sequences 2000 --estimated 1000 \\
        --held-out 20 --out pgure-svt_gb300/lambda_mlp.npz --report lambda_report.json

Steps (all compute on the GPU through libpgsvt.so):
1. label: for each seeded random sequence (learned.random_sequence), the plain
   PGURE search of windows 7..10 gives (features, log10(lambda*/100)); the
   `--sequences` ones with their noise parameters given, the `--estimated`
   ones on the reference's default path (median pre-filter 5, noise
   parameters estimated per window);
2. train: pgsvt_lambda_train (bf16 weights, FP32 accumulation, AdamW,
   one CUDA graph per epoch) from learned.init_model;
3. evaluate on held-out sequences: prediction error, and plain vs learned
   search (risk evaluations and risk gap per window).
Sequences are generated by a spawn process pool started before the first
GPU call.
"""
import argparse
import importlib.util
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _package():
    if "pguresvt_gb300" in sys.modules:
        return sys.modules["pguresvt_gb300"]
    spec = importlib.util.spec_from_file_location(
        "pguresvt_gb300", os.path.join(HERE, "__init__.py"), submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["pguresvt_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def _gen(seed):  # pool worker: the package is imported per process
    return _package().learned.random_sequence(seed)


def _gen_est(seed):
    return _package().learned.random_sequence(seed, estimated=True)


def _gen_heldout(seed):
    return _package().learned.heldout_windows(seed)


def _gen_heldout_est(seed):
    return _package().learned.heldout_windows(seed, estimated=True)


GRID = np.concatenate([[0.0], np.geomspace(1e-4, 100.0, 255)])  # 256 values over [0, upper]


def grid_risks(pkg, X, noise):
    """The PGURE risk of the window centre (frame 7 of X) at every GRID
    value: 16 copies of the window, 16 fixed lambda values each, in one
    pgsvt_denoise_batch call."""
    L, C = pkg.learned, pkg._capi
    seqs = [dict(X=X, params=L.search_params(noise, (7, 8)), lambdas=GRID[16 * i:16 * (i + 1)])
            for i in range(16)]
    res, _ = C.denoise_batch(seqs)
    return np.concatenate([r["risks"][7] for r in res])


def evaluate_512(pkg, model, seeds, pool, estimated=False):
    """Held-out 512x512x200 sequences (config 5's evaluation set): for each
    sampled window, the plain search and the learned proposal + narrow
    search, their risk against the minimum over a 256-value lambda grid (the
    arbiter), risk evaluations and the PSNR of the denoised centre frame.
    Risk gaps are relative to the grid minimum's magnitude (gap_grid) and,
    since a risk minimum can sit near zero, to the risk's range over the grid
    (gap_span)."""
    L = pkg.learned
    rows = []
    mdl = np.ascontiguousarray(model, np.float32)
    t0 = time.time()
    for wins, noise in pool.imap(_gen_heldout_est if estimated else _gen_heldout, seeds):
        for X, clean in wins:
            res = L.compare(X, noise, mdl, frames=(7, 8))
            g = grid_risks(pkg, X, noise)
            gmin = float(g.min())
            span = float(g.max() - g.min())  # the risk's range over the grid
            c = clean[:, :, 7]
            peak = float(clean.max())
            row = dict(grid_min=gmin, grid_argmin=float(GRID[int(np.argmin(g))]),
                       proposal=float(res["learned"]["proposals"][7])
                       if res["learned"]["proposals"] is not None else None)
            for name in ("plain", "learned"):
                r = res[name]
                y = r["Y"][:, :, 7]
                row[name] = dict(lam=float(r["lambdas"][7]), risk=float(r["risk"][7]),
                                 evals=int(r["evals"][7]),
                                 gap_grid=float((r["risk"][7] - gmin) / abs(gmin)),
                                 gap_span=float((r["risk"][7] - gmin) / span) if span > 0 else 0.0,
                                 psnr=float(10 * np.log10(peak ** 2 / np.mean((c - y) ** 2))))
            rp, rl = row["plain"]["risk"], row["learned"]["risk"]
            row["gap_learned_vs_plain"] = float((rl - rp) / abs(rp))
            rows.append(row)
    def col(a, b):
        return np.array([r[a][b] for r in rows])
    gap = np.array([r["gap_learned_vs_plain"] for r in rows])
    out = dict(sequences=len(seeds), windows=len(rows), seconds=time.time() - t0,
               outputs=list(L.HELDOUT_OUTPUTS), grid="0 and 255 log-spaced values in [1e-4, 100]",
               gap_learned_vs_plain_max=float(gap.max()), gap_learned_vs_plain_mean=float(gap.mean()),
               frac_learned_vs_plain_le_1pct=float(np.mean(gap <= 0.01)))
    for name in ("plain", "learned"):
        gg = col(name, "gap_grid")
        gs = col(name, "gap_span")
        out[name] = dict(evals_mean=float(col(name, "evals").mean()),
                         gap_grid_max=float(gg.max()), gap_grid_mean=float(gg.mean()),
                         frac_gap_grid_le_1pct=float(np.mean(gg <= 0.01)),
                         gap_span_max=float(gs.max()),
                         frac_gap_span_le_1pct=float(np.mean(gs <= 0.01)),
                         psnr_mean=float(col(name, "psnr").mean()))
    out["worst_windows"] = sorted(rows, key=lambda r: -r["gap_learned_vs_plain"])[:8]
    out["psnr_delta_learned_minus_plain_db"] = dict(
        mean=float((col("learned", "psnr") - col("plain", "psnr")).mean()),
        min=float((col("learned", "psnr") - col("plain", "psnr")).min()),
        max=float((col("learned", "psnr") - col("plain", "psnr")).max()))
    return out


def evaluate(pkg, model, seeds, pool, estimated=False):
    """Held-out windows: prediction error, plain vs learned search."""
    L = pkg.learned
    rows = []
    for noisy, noise in pool.imap(_gen_est if estimated else _gen, seeds):
        lab = L.label(noisy, noise)
        res = L.compare(noisy, noise, model, frames=L.LABEL_FRAMES)
        f0, f1 = L.LABEL_FRAMES
        pl, le = res["plain"], res["learned"]
        for t in range(f0, f1):
            rp, rl = pl["risk"][t], le["risk"][t]
            rows.append(dict(side=int(noisy.shape[0]), y=float(lab["targets"][t - f0]),
                             y_hat=float(le["proposals"][t]), evals_plain=int(pl["evals"][t]),
                             evals_learned=int(le["evals"][t]),
                             risk_gap=float((rl - rp) / abs(rp)) if rp != 0 else 0.0))
    y = np.array([r["y"] for r in rows])
    yh = np.array([r["y_hat"] for r in rows])
    ep = np.array([r["evals_plain"] for r in rows])
    el = np.array([r["evals_learned"] for r in rows])
    gap = np.array([r["risk_gap"] for r in rows])
    return dict(windows=len(rows), rmse_log10=float(np.sqrt(np.mean((y - yh) ** 2))),
                evals_plain=float(ep.mean()), evals_learned=float(el.mean()),
                # beyond the narrow search's own evaluations (grid, two
                # sentinels, two refinement rounds of 4): the plain search ran
                fallbacks=int(np.sum(el > 4 + 2 + 2 * 4)),
                risk_gap_max=float(gap.max()),
                risk_gap_mean=float(gap.mean()), frac_gap_le_1pct=float(np.mean(gap <= 0.01)))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--sequences", type=int, default=2000)
    ap.add_argument("--estimated", type=int, default=1000,
                    help="sequences labelled on the default path (noise estimated)")
    ap.add_argument("--held-out", type=int, default=20)
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--workers", type=int, default=max(1, min(12, (os.cpu_count() or 2) - 2)))
    ap.add_argument("--out", default=os.path.join(HERE, "lambda_mlp.npz"))
    ap.add_argument("--data", default=None, help="also save the labelled set (.npz)")
    ap.add_argument("--report", default=None)
    ap.add_argument("--evaluate", default=None,
                    help="only evaluate this model on the held-out sequences")
    ap.add_argument("--held-out-512", type=int, default=0,
                    help="with --evaluate: also this many held-out 512x512x200 sequences "
                         "(4 sampled windows each), given and estimated noise")
    a = ap.parse_args()

    pool = mp.get_context("spawn").Pool(a.workers)  # before any GPU call
    pkg = _package()
    L = pkg.learned
    held = [10 ** 6 + a.seed * 1000003 + i for i in range(a.held_out)]
    held_est = [2 * 10 ** 6 + a.seed * 1000003 + i for i in range(a.held_out)]

    def evaluate_both(model):
        ev = evaluate(pkg, model, held, pool) if a.held_out else {}
        if a.held_out and a.estimated:
            ev["estimated"] = evaluate(pkg, model, held_est, pool, estimated=True)
        return ev

    if a.evaluate:
        ev = evaluate_both(L.load_model(a.evaluate))
        if a.held_out_512:
            mdl = L.load_model(a.evaluate)
            s512 = [3 * 10 ** 6 + a.seed * 1000003 + i for i in range(a.held_out_512)]
            ev["held_out_512"] = evaluate_512(pkg, mdl, s512, pool)
            s512 = [4 * 10 ** 6 + a.seed * 1000003 + i for i in range(a.held_out_512)]
            ev["held_out_512_estimated"] = evaluate_512(pkg, mdl, s512, pool, estimated=True)
        pool.close()
        pool.join()
        print(json.dumps(ev))
        if a.report:
            with open(a.report, "w") as f:
                json.dump(ev, f, indent=1)
        return
    t0 = time.time()
    seeds = [a.seed * 1000003 + i for i in range(a.sequences)]
    parts = [L.label(noisy, noise) for noisy, noise in pool.imap(_gen, seeds, chunksize=2)]
    n_given = sum(len(q["targets"]) for q in parts)
    seeds = [5 * 10 ** 6 + a.seed * 1000003 + i for i in range(a.estimated)]
    parts += [L.label(noisy, noise) for noisy, noise in pool.imap(_gen_est, seeds, chunksize=2)]
    data = {k: np.concatenate([q[k] for q in parts]) for k in parts[0]}
    t_label = time.time() - t0
    if a.data:
        np.savez_compressed(a.data, **data)
    t1 = time.time()
    model, curve = L.train(data["features"], data["targets"], epochs=a.epochs, batch=a.batch,
                           seed=a.seed, lr=a.lr)
    t_train = time.time() - t1
    ev = evaluate_both(model)
    pool.close()
    pool.join()
    L.save_model(model, a.out, n_train=len(data["targets"]), n_estimated=len(data["targets"]) - n_given,
                 epochs=a.epochs,
                 final_loss=float(curve[-1]), seed=a.seed)
    est = slice(n_given, None)
    rep = dict(train_windows=int(len(data["targets"])), estimated_windows=int(len(data["targets"]) - n_given),
               plain_evals_estimated=float(data["evals"][est].mean()) if a.estimated else None,
               label_seconds=t_label,
               train_seconds=t_train, epochs=a.epochs, loss_first=float(curve[0]),
               loss_last=float(curve[-1]), target_mean=float(data["targets"].mean()),
               target_std=float(data["targets"].std()),
               plain_evals_mean=float(data["evals"].mean()), held_out=ev)
    print(json.dumps(rep))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()

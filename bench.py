#!/usr/bin/env python
"""Benchmark: PGURE-optimal denoising throughput (output frames per second).

Workload (default): the 512x512x200 float32 lattice+blob sequence, 4x4
patches, trajectory 15, ARPS on (neighbourhood 7), PGURE lambda optimisation
on, Poisson-Gaussian noise alpha=0.5, mu=1, sigma=3, seeded probes.  One step
is one denoise of the whole sequence (200 output windows).

value: frames/s with the sequence already resident in HBM (pgsvt_denoise_device
on torch's current stream, CUDA events around the timed steps).
e2e:   frames/s through pgsvt_denoise with pinned host buffers (host->device
copy of the input and device->host copy of the result inside every step).
cpu_baseline: the FP64 oracle port on the host cores: 16 full windows of the
              sequence, one per thread (the reference's std::thread fan-out
              over output frames), measured, no extrapolation.  The same run
              gives the `parity` object: the oracle's frames against the GPU's.

Run with torchrun for N > 1: every rank denoises its own sequence (weak
scaling, no collective on the data path); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

METRIC = "frames/s at PGURE-optimal lambda (512^2, 4x4, T=15)"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--side", type=int, default=512)
    ap.add_argument("--frames", type=int, default=200)
    ap.add_argument("--patch", type=int, default=4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--hint", type=float, default=-1.0, help="fixed lambda proposal")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-lambda arm")
    ap.add_argument("--no-default-path", action="store_true",
                    help="skip timing the reference's default path (median 5 + noise estimation)")
    ap.add_argument("--batch", type=int, default=64,
                    help="also time pgsvt_denoise_batch on this many uneven sequences (0: skip)")
    ap.add_argument("--batch-full", action="store_true",
                    help="batch sequences of the full configuration (sides to 1024, 30-300 "
                         "frames) instead of the bench-time scaled ones")
    ap.add_argument("--autotune", type=int, default=1,
                    help="SVD kernel form: 1 tuned (default), 0 registers, 2 more lanes, "
                    "3 shared memory, 4 eight rows per lane, 5 QR-preconditioned, "
                    "6 TMA-staged factors")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the oracle leg (CPU baseline and parity)")
    ap.add_argument("--cpu-windows", type=int, default=16,
                    help="full windows of the oracle leg (one per host thread)")
    return ap.parse_args()


# The parameters of the benchmark workload, shared by the GPU arms and the
# oracle: PGURESVT's arguments (pguresvt.hpp:17-38) with the lambda search of
# the library (8 points, 4 rounds) on both sides.
def workload_kw(bs, a, m, s):
    return dict(traj_length=15, block_size=bs, block_overlap=1, motion_window=7,
                median_size=-1, random_seed=7, optimize_pgure=1, alpha=a, mu=m, sigma=s)


def params(capi, a, m, s, bs, hint, autotune=1):
    return capi.default_params(lambda_hint=hint, autotune=autotune, **workload_kw(bs, a, m, s))


def workload_config(S, nimg, bs, a, m, s, hint=-1.0):
    """The `config` object of both arms' lines."""
    return {"workload": "lattice_512: %dx%dx%d f32, patch %d (m=%d), T=15, ARPS mw=7, "
                        "PGURE on, alpha=%g mu=%g sigma=%g, median off"
                        % (S, S, nimg, bs, bs * bs, a, m, s),
            "lambda_search": "plain" if hint <= 0 else "hinted %g" % hint,
            "l2": "input larger than L2 (no flush needed)"}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=20).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.samples = []
        self.proc = None
        self.device = device

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for smp in self.samples:
            try:
                sm.append(float(smp[0]))
                smax.append(float(smp[1]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, smp[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(side, frames, seed, with_clean=False):
    pkg = entry.load_package()
    noisy, clean, (a, m, s) = pkg.synth.workload("lattice_512", seed=seed, side=side, nt=frames)
    if with_clean:
        return noisy, (a, m, s), clean
    return noisy, (a, m, s)


def psnr(clean, y):
    """PSNR (dB) of y against the clean sequence, peak = max(clean)."""
    return float(10 * np.log10(clean.max() ** 2 / np.mean((clean - y) ** 2)))


def svd_flops(m, n):
    """Golub-Van Loan thin-SVD operation count 14mn^2 + 8n^3 per matrix."""
    return 14 * m * n * n + 8 * n ** 3


def _batch_sequence(spec):
    """One sequence of the uneven-batch workload (a spawn-pool worker)."""
    i, seed, full = spec
    pkg = entry.load_package()
    rng = np.random.default_rng([seed, i])
    side = int(rng.choice([128, 256, 384, 512, 1024] if full else [128, 256, 384, 512]))
    nt = int(rng.integers(30, 301)) if full else int(rng.integers(30, 46))
    bs = int(rng.choice([4, 6, 8]))
    T = int(rng.choice([9, 15, 21]))
    a, sg = float(rng.uniform(0.05, 1.0)), float(rng.uniform(0.5, 5.0))
    nb = max(1, int(round(80 * (side / 256.0) ** 2)))
    clean = pkg.synth.blobs(side, nt, nb, seed * 1000 + i, 2.0, False, False)
    noisy = pkg.synth.poisson_gaussian(clean, a, 0.5, sg, seed * 1000 + i + 1)
    lam = np.geomspace(1e-3, 100.0, 16) * float(rng.uniform(0.5, 2.0))
    return dict(X=np.asfortranarray(noisy.astype(np.float32)), bs=bs, T=T,
                noise=(a, 0.5, sg), lambdas=lam)


def batch_workload(n, seed, full=False):
    """Sequences of the uneven-batch configuration: sides {128, 256, 384,
    512, 1024}, 30-300 frames (full=True), or scaled to bench time: sides up
    to 512, 30-45 frames; patch {4, 6, 8}, trajectory {9, 15, 21}, alpha
    U[0.05, 1], sigma U[0.5, 5], the blob generator with sub-pixel drift; 16
    fixed lambda values per sequence.  Generated in a spawn process pool."""
    import multiprocessing as mp
    specs = [(i, seed, full) for i in range(n)]
    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
    os.environ.update(OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")  # one core per worker
    try:
        with mp.get_context("spawn").Pool(max(1, min(16, (os.cpu_count() or 2) - 1))) as pool:
            return pool.map(_batch_sequence, specs, chunksize=1)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def run_batch(capi, n, seed, slots=2, full=False):
    seqs = batch_workload(n, seed, full)
    inp = []
    for q in seqs:
        a, m, s = q["noise"]
        p = capi.default_params(traj_length=q["T"], block_size=q["bs"], motion_window=7,
                                median_size=0, random_seed=7, alpha=a, mu=m, sigma=s,
                                autotune=1)
        inp.append(dict(X=q["X"], params=p, lambdas=q["lambdas"]))
    # warm-up: one sequence of every (patch, trajectory) shape, which also runs
    # the autotuner once per shape outside the timed call
    first = {}
    for q, x in zip(seqs, inp):
        first.setdefault((q["bs"], q["T"]), x)
    capi.denoise_batch(list(first.values()), slots=slots)
    t0 = time.perf_counter()
    res, st = capi.denoise_batch(inp, slots=slots)
    dt = time.perf_counter() - t0
    frames = sum(q["X"].shape[2] for q in seqs)
    vox = sum(q["X"].size for q in seqs)
    return {"sequences": n, "frames": frames, "voxels": int(vox), "seconds": dt,
            "value": frames / dt, "unit": "frames/s (e2e, host buffers)", "slots": slots,
            "risk_evals_per_window": st.risk_evals / max(1, st.windows),
            "gpu_launches": int(st.kernel_launches),
            "config": ("sides {128,256,384,512,1024}, 30-300 frames, patch {4,6,8}, T {9,15,21}, "
                       "16 fixed lambda per sequence (uneven-batch configuration, %d sequences)" % n)
                      if full else
                      ("sides {128,256,384,512}, 30-45 frames, patch {4,6,8}, T {9,15,21}, "
                       "16 fixed lambda per sequence (uneven-batch configuration scaled to "
                       "%d sequences)" % n)}


def window_of(X, t, fw):
    """The normalised window of output frame t (pguresvt.hpp:100-120)."""
    nt = X.shape[2]
    s0 = 0 if t < fw else (nt - 2 * fw - 1 if t >= nt - fw else t - fw)
    u = np.asarray(X[:, :, s0:s0 + 2 * fw + 1], np.float64)
    return np.asfortranarray(u / u.max())


def oracle_leg(capi, noisy, clean, nm, bs, Y, est, risk, nev, nwin, threads):
    """CPU baseline and parity on `nwin` full windows around the middle of the
    sequence: the oracle denoises them on `nwin` threads, one window each
    (the reference's fan-out over output frames, utils.hpp:108-168), with the
    same lambda search schedule as the GPU; its wall time is the baseline and
    its frames are compared with the GPU's (Y, est: the GPU run's outputs)."""
    O = entry.load_oracle()
    a, m, s = nm
    nimg = noisy.shape[2]
    nwin = max(1, min(nwin, nimg))
    fb = nimg // 2 - nwin // 2
    f = slice(fb, fb + nwin)
    X64 = np.asfortranarray(noisy, dtype=np.float64)
    t0 = time.perf_counter()
    Y0, est0, rep = O.denoise(X64, frame_begin=fb, frame_end=fb + nwin, n_jobs=nwin,
                              **workload_kw(bs, a, m, s))
    wall = time.perf_counter() - t0
    model = cpu_model()
    cpu = {"value": nwin / wall, "unit": "frames/s", "cores": nwin, "kind": "port",
           "cpu_model": model, "seconds": wall,
           "risk_evals_per_window": rep.risk_evals / max(1, rep.windows),
           "sample": "%d full windows (output frames %d-%d of the sequence), one per thread "
                     "(the reference's std::thread fan-out over output frames), every patch, "
                     "the lambda search schedule of the GPU plain search; measured wall time, "
                     "no extrapolation" % (nwin, fb, fb + nwin - 1)}
    # parity: the denoised frames against the clean sequence, GPU and oracle
    cl = clean[:, :, f]
    pg, po = psnr(cl, Y[:, :, f]), psnr(cl, Y0[:, :, f])
    par = {"frames": "%d-%d" % (fb, fb + nwin - 1), "windows": nwin,
           "psnr_gpu_db": pg, "psnr_ref_db": po, "psnr_delta_db": pg - po,
           "psnr_gpu_vs_ref_db": psnr(Y0[:, :, f], Y[:, :, f]),
           "max_abs_diff_rel": float(np.abs(Y[:, :, f] - Y0[:, :, f]).max()
                                     / np.abs(Y0[:, :, f]).max()),
           "lambda_gpu": [float(v) for v in est[f, 0]],
           "lambda_ref": [float(v) for v in est0[f, 0]],
           "risk_evals_gpu": float(np.mean(nev[f])),
           "risk_evals_ref": rep.risk_evals / max(1, rep.windows)}
    # trajectories, singular values and the risk gap on the first and last
    # windows of the sample (oracle stages on all host threads)
    O.set_threads(threads)
    try:
        ntc, fw, nw = O.window_geometry(15, bs)
        mv_equal, sv_max, sv_mean, sv_abs, gaps = True, 0.0, [], 0.0, []
        for t in (fb, fb + nwin - 1):
            u = window_of(noisy, t, fw)
            r0, c0 = O.arps_window(u, bs, 7, t, fw, nimg)
            r1, c1 = capi.arps_window(u, bs, 7, t, fw, nimg)
            mv_equal = mv_equal and np.array_equal(r0, r1) and np.array_equal(c0, c1)
            S0 = O.svd_window(u, bs, 1, r0, c0)
            S1 = capi.svd_window(u, bs, 1, r0, c0).astype(np.float64)
            smax = S0[:, :1]
            big = S0 > 1e-3 * smax
            rel = np.abs(S1 - S0) / np.maximum(S0, 1e-300)
            sv_max = max(sv_max, float(rel[big].max()))
            sv_mean.append(float(rel[big].mean()))
            sv_abs = max(sv_abs, float((np.abs(S1 - S0) / smax).max()))
            rr = O.risk_window(u, bs, 1, r0, c0, [est[t, 0], est0[t, 0]], a, m, s, 7)
            gaps.append(float((rr[0] - rr[1]) / abs(rr[1])))
    finally:
        O.set_threads(1)
    par.update({"motion_vectors_identical": bool(mv_equal), "sv_rel_err_max": sv_max,
                "sv_rel_err_mean": float(np.mean(sv_mean)), "sv_abs_err_max_over_smax": sv_abs,
                "sv_note": "FP32 Jacobi vs FP64 LAPACK dgesdd on windows %d and %d (every "
                           "patch); relative errors over s > 1e-3 s_max" % (fb, fb + nwin - 1),
                "risk_gap_max": max(gaps),
                "risk_gap_note": "oracle risk at the GPU's lambda over its own minimum, "
                                 "windows %d and %d" % (fb, fb + nwin - 1)})
    return cpu, par


def run_reference(args, rank):
    """Reference arm: the FP64 oracle port on all host threads (the reference
    itself does not build here: Armadillo and NLopt are absent).  One step is
    one complete output frame of the benchmark sequence: its window's noise
    estimate, ARPS, the four decompositions and the lambda search (the same
    schedule as the GPU plain search), every patch, the window's work spread
    over all host threads; consecutive steps take consecutive frames."""
    if rank != 0:
        return
    noisy, nm = make_workload(args.side, args.frames, args.seed)
    a, m, s = nm
    O = entry.load_oracle()
    threads = os.cpu_count() or 1
    X64 = np.asfortranarray(noisy, dtype=np.float64)
    nimg = args.frames
    kw = workload_kw(args.patch, a, m, s)
    times, evals = [], []
    for i in range(args.warmup + args.steps):
        t = (nimg // 2 - args.warmup + i) % nimg
        t0 = time.perf_counter()
        _, _, rep = O.denoise(X64, frame_begin=t, frame_end=t + 1, n_jobs=1,
                              window_threads=threads, **kw)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            evals.append(rep.risk_evals)
    ms = 1e3 * sum(times) / len(times)
    v = len(times) / sum(times)
    line = {"metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded blob+lattice sequence, Poisson-Gaussian noise)",
            "config": workload_config(args.side, nimg, args.patch, a, m, s),
            "impl": "reference",
            "cpu_baseline": {"kind": "port", "cores": threads, "cpu_model": cpu_model(),
                             "value": v,
                             "sample": "one complete output frame per step (frames %d-%d): "
                                       "noise estimate, ARPS, 4 decompositions, %.1f risk "
                                       "evaluations (the GPU plain search's schedule), every "
                                       "patch, on %d threads inside the window; measured, no "
                                       "extrapolation" % ((nimg // 2) % nimg,
                                                          (nimg // 2 + args.steps - 1) % nimg,
                                                          float(np.mean(evals)), threads)},
            "risk_evals_per_window": float(np.mean(evals)),
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        return run_reference(args, rank)
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg = entry.load_package()
    capi = pkg._capi
    capi.load()
    noisy, (a, m, s), clean = make_workload(args.side, args.frames, args.seed + rank, True)
    S, nimg = args.side, args.frames
    n = S * S * nimg
    p = params(capi, a, m, s, args.patch, args.hint, args.autotune)

    # ---- device-resident timing
    x = torch.from_numpy(np.ascontiguousarray(noisy.ravel(order="F"))).cuda()
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    est = torch.empty(nimg * 4, dtype=torch.float64, device="cuda")
    risk = torch.zeros(nimg, dtype=torch.float64, device="cuda")
    nev = torch.zeros(nimg, dtype=torch.int32, device="cuda")
    outs = capi.Outputs(risk=risk.data_ptr(), risk_evals=nev.data_ptr())
    stream = torch.cuda.current_stream()

    def step(prm=p):
        return capi.denoise_device_ex(x.data_ptr(), capi.PGSVT_F32, S, S, nimg, y.data_ptr(),
                                      est.data_ptr(), prm, outs, stream.cuda_stream)

    for _ in range(args.warmup):
        st = step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = []
    for _ in range(args.steps):
        stats.append(step())
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * nimg / (ms / 1e3)
    Y_plain = y.cpu().numpy().reshape(noisy.shape, order="F")
    plain = {"risk": risk.cpu().numpy().copy(), "evals": nev.cpu().numpy().copy(),
             "est": est.cpu().numpy().reshape(4, nimg).T.copy(),
             "psnr": psnr(clean, Y_plain)}

    # ---- learned-lambda form: the shipped MLP's proposal + narrow search
    learned = None
    if not args.no_learned and args.patch != 4:
        learned = {"skipped": "the shipped lambda model covers 4x4 patches and 15-frame windows"}
    elif not args.no_learned:
        model = pkg.learned.load_model()
        pl = params(capi, a, m, s, args.patch, -1.0, args.autotune)
        pl.lambda_model = model.ctypes.data
        step(pl)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        lst = [step(pl) for _ in range(args.steps)]
        f1.record(stream)
        torch.cuda.synchronize()
        lms = f0.elapsed_time(f1) / args.steps
        if dist:
            t = torch.tensor([lms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            lms = float(t.item())
        lr = risk.cpu().numpy()
        gap = (lr - plain["risk"]) / np.abs(plain["risk"])
        lpsnr = psnr(clean, y.cpu().numpy().reshape(noisy.shape, order="F"))
        learned = {"value": world * nimg / (lms / 1e3), "unit": "frames/s", "ms_per_step": lms,
                   "speedup_vs_plain": ms / lms,
                   "risk_evals_per_window": float(nev.cpu().numpy().mean()),
                   "plain_risk_evals_per_window": float(plain["evals"].mean()),
                   "risk_gap_max": float(gap.max()), "risk_gap_mean": float(gap.mean()),
                   "windows_gap_le_1pct": float(np.mean(gap <= 0.01)),
                   "psnr_db": lpsnr, "plain_psnr_db": plain["psnr"],
                   "psnr_delta_db": lpsnr - plain["psnr"],
                   "gpu_launches": int(sum(q.kernel_launches for q in lst)),
                   "model": "pgure-svt_gb300/lambda_mlp.npz (67-128-128-128-1 GELU, bf16 "
                            "weights, trained on the GPU by pgsvt_lambda_train)"}

    # ---- end to end through pgsvt_denoise with pinned host buffers
    xh = torch.from_numpy(np.ascontiguousarray(noisy.ravel(order="F"))).pin_memory()
    yh = torch.empty(n, dtype=torch.float64).pin_memory()
    eh = torch.empty(nimg * 4, dtype=torch.float64).pin_memory()
    import ctypes
    L = capi.load()

    def e2e_step():
        stt = capi.Status()
        rc = L.pgsvt_denoise(ctypes.c_void_p(xh.data_ptr()), capi.PGSVT_F32, S, S, nimg,
                             ctypes.c_void_p(yh.data_ptr()), ctypes.c_void_p(eh.data_ptr()),
                             ctypes.byref(p), ctypes.byref(stt))
        if rc != 0:
            raise capi.PgsvtError(rc, stt.message.decode())
        return stt

    e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ste = e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * nimg / e2e_s, "unit": "frames/s",
           "h2d_bytes_per_step": int(xh.numel() * 4), "d2h_bytes_per_step": int((n + nimg * 4) * 8)}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel (from the library's stage clocks)
    st = stats[-1]
    stage = {nm_: st.stage_seconds[i] for i, nm_ in enumerate(capi.STAGES)}
    M, N = args.patch ** 2, 15
    svd_t = st.stage_seconds[4] / max(1, st.svd_launches)
    svd_flop = svd_flops(M, N) * st.svd_matrices / max(1, st.svd_launches)
    peaks = json.load(open(PEAKS_PATH)) if os.path.exists(PEAKS_PATH) else {}
    sm_mhz = peaks.get("sm_max_mhz", 2070.0)
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * sm_mhz * 1e6 / 1e12
    svd_kernels = {0: "k_bsweep + k_bout" if M <= 16 and N <= 15 else "k_svd",
                   4: "k_qr + k_xsweep + k_qr_out"}.get(int(st.svd_variant), "k_svd")
    roof = {"kernel": "SVD stage: %s (batched one-sided Jacobi, FP32 CUDA cores)" % svd_kernels,
            "bound": "fp32",
            "achieved": svd_flop / svd_t / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": svd_flop / svd_t / 1e12 / fp32_peak,
            "peak_source": "nominal FP32 FMA rate: %d SMs (the device's multiprocessor "
                           "count) x 128 lanes x 2 flop x %.0f MHz (sm_max_mhz of "
                           "MEASURED_PEAKS.json); MEASURED_PEAKS has no non-tensor FP32 figure"
                           % (sm_count, sm_mhz),
            "sm_count": sm_count,
            "algorithmic_flops_per_launch": svd_flop, "avg_launch_ms": svd_t * 1e3,
            "traffic": None}
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        roof["traffic"] = json.load(open(prof)).get("svd_stage")
    # In the timed region the SVD of one window batch shares the GPU with the
    # other streams' lambda searches, so its event time overstates the
    # kernels' own.  The same launches alone: one batch of windows (the
    # library's batch size for this frame), hence one stream, after the
    # timed region.
    npatch = (S - args.patch + 1) ** 2
    wb = max(1, min(nimg, (500000 + npatch - 1) // npatch))
    pi = params(capi, a, m, s, args.patch, args.hint, args.autotune)
    pi.frame_begin, pi.frame_end = nimg // 2 - wb // 2, nimg // 2 - wb // 2 + wb
    iso = []
    for _ in range(4):
        sti = step(pi)
        iso.append(sti.stage_seconds[4] / max(1, sti.svd_launches))
    torch.cuda.synchronize()
    iso_t = min(iso[1:])
    iso_flop = svd_flops(M, N) * sti.svd_matrices / max(1, sti.svd_launches)
    roof.update({"isolated_launch_ms": iso_t * 1e3,
                 "achieved_isolated": iso_flop / iso_t / 1e12,
                 "frac_isolated": iso_flop / iso_t / 1e12 / fp32_peak,
                 "isolated_note": "the same SVD launch (%d windows x %d copies) with no other "
                                  "stream running, after the timed region" % (wb, sti.svd_matrices
                                  // max(1, sti.svd_launches) // npatch // wb or 1)})

    evals_per_window = max(1, round(st.risk_evals / max(1, st.windows)))
    line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded blob+lattice sequence, Poisson-Gaussian noise); input "
                    "%.0f MB > L2 per step" % (noisy.nbytes / 1e6),
            "config": workload_config(S, nimg, args.patch, a, m, s, args.hint),
            "e2e": e2e, "roofline": roof, "clocks": clk, "learned": learned,
            "psnr_db_vs_clean": plain["psnr"],
            "gpu_launches": int(sum(x.kernel_launches for x in stats)),
            "stage_seconds_per_step": stage,
            "risk_evals_per_window": evals_per_window,
            "arps_exact_steps": int(st.arps_exact_steps),
            "svd_fp64_tests": int(st.svd_fp64_tests),
            "svd_sweeps_per_warp": st.svd_warp_sweeps / max(1, st.svd_matrices / 8),
            "svd_variant": {0: "registers", 1: "more lanes per patch",
                            2: "shared memory", 3: "eight rows per lane",
                            4: "QR-preconditioned",
                            5: "registers, TMA-staged factors"}.get(int(st.svd_variant), "?")}
    if not args.no_default_path:
        # the reference's default configuration (SVT() / PGURE-SVT defaults):
        # median pre-filter 5, noise parameters estimated per window, PGURE on
        pd = capi.default_params(traj_length=15, block_size=args.patch, motion_window=7,
                                 median_size=5, random_seed=7, autotune=args.autotune)

        def timed(pp, steps):
            """Device time per step of `steps` steps after one untimed step."""
            step(pp)
            torch.cuda.synchronize()
            g0 = torch.cuda.Event(enable_timing=True)
            g1 = torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            for _ in range(steps):
                step(pp)
            g1.record(stream)
            torch.cuda.synchronize()
            return g0.elapsed_time(g1) / steps

        dms = timed(pd, args.steps)
        dp_risk = risk.cpu().numpy().copy()
        dp_evals = float(nev.cpu().numpy().mean())
        dp_psnr = psnr(clean, y.cpu().numpy().reshape(noisy.shape, order="F"))
        line["default_path"] = {"value": nimg / (dms / 1e3), "unit": "frames/s",
                                "ms_per_step": dms, "steps": args.steps, "psnr_db": dp_psnr,
                                "risk_evals_per_window": dp_evals,
                                "noise_estimates_frame0": [float(v) for v in
                                                           est.cpu().numpy().reshape(4, nimg)[1:, 0]],
                                "config": "median filter 5, alpha/mu/sigma estimated "
                                          "(noise method 4), PGURE on, same sequence"
                                          + ("; rank 0 alone" if world > 1 else "")}
        if not args.no_learned and args.patch == 4:  # the learned proposal on the default path
            model = pkg.learned.load_model()
            pd.lambda_model = model.ctypes.data
            lms = timed(pd, args.steps)
            gap = (risk.cpu().numpy() - dp_risk) / np.abs(dp_risk)
            line["default_path"]["learned"] = {
                "value": nimg / (lms / 1e3), "unit": "frames/s", "ms_per_step": lms,
                "steps": args.steps, "speedup_vs_plain": dms / lms,
                "risk_evals_per_window": float(nev.cpu().numpy().mean()),
                "risk_gap_max": float(gap.max()), "risk_gap_mean": float(gap.mean()),
                "windows_gap_le_1pct": float(np.mean(gap <= 0.01)),
                "psnr_db": psnr(clean, y.cpu().numpy().reshape(noisy.shape, order="F"))}
    if args.batch:
        line["batch"] = run_batch(capi, args.batch, args.seed, full=args.batch_full)
    if not args.no_cpu_baseline and world == 1:  # CPU baseline and parity: rank 0 at N = 1
        threads = os.cpu_count() or 1
        line["cpu_baseline"], line["parity"] = oracle_leg(
            capi, noisy, clean, (a, m, s), args.patch, Y_plain, plain["est"], plain["risk"],
            plain["evals"], min(args.cpu_windows, threads), threads)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

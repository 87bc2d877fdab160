"""The command-line tool (pgure-svt_gb300/pgsvt_cli), the counterpart of the
reference's src/PGURE-SVT.cpp: parameter file, TIFF in/out, hot-pixel filter.

CPU tests exercise the paths that end before the first device call (usage,
parameter errors, TIFF checks); GPU tests run the tool end to end and compare
its output with the library called directly on the same frames, and the
hot-pixel filter with the oracle.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "pgure-svt_gb300", "pgsvt_cli")


def write_tiff(path, frames, bits=16, big_endian=False, rows_per_strip=None):
    """Baseline multi-page TIFF of (pages, height, width) frames."""
    e = ">" if big_endian else "<"
    n, h, w = frames.shape
    rps = rows_per_strip or h
    nstrip = (h + rps - 1) // rps
    out = bytearray((b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, 8))
    dt = np.dtype(e + ("u2" if bits == 16 else "u1"))
    for p in range(n):
        ifd = len(out)
        tags = 10
        soff = ifd + 2 + 12 * tags + 4
        data_off = soff + 8 * nstrip
        strips = []
        for s in range(nstrip):
            rows = frames[p, s * rps:(s + 1) * rps].astype(dt).tobytes()
            strips.append(rows)
        offs, o = [], data_off
        for st in strips:
            offs.append(o)
            o += len(st)
        nxt = o if p + 1 < n else 0
        ent = [(256, 4, 1, w), (257, 4, 1, h), (258, 3, 1, bits), (259, 3, 1, 1), (262, 3, 1, 1),
               (273, 4, nstrip, offs[0] if nstrip == 1 else soff), (277, 3, 1, 1),
               (278, 4, 1, rps), (279, 4, nstrip, len(strips[0]) if nstrip == 1 else soff + 4 * nstrip),
               (284, 3, 1, 1)]
        out += struct.pack(e + "H", tags)
        for t, ty, c, v in ent:
            if ty == 3 and c == 1:
                out += struct.pack(e + "HHIHH", t, ty, c, v, 0)
            else:
                out += struct.pack(e + "HHII", t, ty, c, v)
        out += struct.pack(e + "I", nxt)
        out += b"".join(struct.pack(e + "I", x) for x in offs)
        out += b"".join(struct.pack(e + "I", len(st)) for st in strips)
        for st in strips:
            out += st
    with open(path, "wb") as f:
        f.write(bytes(out))


def read_tiff16(path):
    """Pages of a little-endian single-strip 16-bit TIFF (the tool's output)."""
    b = open(path, "rb").read()
    assert b[:2] == b"II"
    off = struct.unpack("<I", b[4:8])[0]
    pages = []
    while off:
        n = struct.unpack("<H", b[off:off + 2])[0]
        tags = {}
        for k in range(n):
            t, ty, c, v = struct.unpack("<HHII", b[off + 2 + 12 * k:off + 14 + 12 * k])
            tags[t] = v & 0xFFFF if ty == 3 else v
        w, h, so = tags[256], tags[257], tags[273]
        assert tags[258] == 16 and tags[259] == 1
        pages.append(np.frombuffer(b[so:so + 2 * w * h], "<u2").reshape(h, w))
        off = struct.unpack("<I", b[off + 2 + 12 * n:off + 6 + 12 * n])[0]
    return np.array(pages)


def run(paramfile, cwd):
    return subprocess.run([CLI, str(paramfile)], cwd=cwd, capture_output=True, text=True)


def test_usage_and_required_parameters(capi, tmp_path):
    assert os.path.exists(CLI), "pgsvt_cli not built"
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 255 and "Usage" in r.stdout
    pf = tmp_path / "p.svt"
    pf.write_text("filename : ./x.tif\nstart_frame : 1  # no end frame\n")
    r = run(pf, tmp_path)
    assert r.returncode == 255 and "Required parameters not specified" in r.stderr


def test_parameter_and_file_errors(capi, tmp_path):
    pf = tmp_path / "p.svt"
    pf.write_text("# comment line\nfilename : ./missing.tif # inline\nstart_frame : 1\n"
                  "end_frame : 4\noptimize_pgure : false\n")
    r = run(pf, tmp_path)
    assert r.returncode == 255 and "no lambda specified" in r.stderr
    pf.write_text("filename : ./missing.tif\nstart_frame : 1\nend_frame : 4\n")
    r = run(pf, tmp_path)
    assert r.returncode == 255 and "missing.tif not found" in r.stderr
    write_tiff(tmp_path / "rect.tif", np.zeros((4, 16, 24), np.uint16))
    pf.write_text("filename : ./rect.tif\nstart_frame : 1\nend_frame : 4\n")
    r = run(pf, tmp_path)
    assert r.returncode == 255 and "not square" in r.stderr
    write_tiff(tmp_path / "short.tif", np.zeros((3, 16, 16), np.uint16))
    pf.write_text("filename : ./short.tif\nstart_frame : 1\nend_frame : 5\n")
    r = run(pf, tmp_path)
    assert r.returncode == 255 and "only has 3 frames" in r.stderr


def test_hot_pixel_oracle_replaces_outliers(oracle):
    rng = np.random.default_rng(0)
    a = rng.integers(1000, 1010, (24, 24, 2)).astype(np.uint16)
    a[5, 5, 0] = 60000
    a[0, 7, 1] = 60000
    b = oracle.hot_pixel_filter(a, 10)
    assert b[5, 5, 0] < 1010 and b[0, 7, 1] < 1010
    # the reference subtracts the median in uint16: values below it wrap
    # around and count as outliers too (hotpixel.hpp:31-33)
    below = a[:, :, 0] < np.median(a[:, :, 0])
    assert (b[:, :, 0] != a[:, :, 0])[below].mean() > 0.5


@pytest.mark.gpu
def test_hot_pixel_filter_matches_oracle(capi, oracle):
    rng = np.random.default_rng(1)
    a = rng.integers(200, 400, (40, 40, 3)).astype(np.uint16)
    a[rng.integers(0, 40, 30), rng.integers(0, 40, 30), rng.integers(0, 3, 30)] = 30000
    for thr in (0, 3, 10):
        np.testing.assert_array_equal(capi.hot_pixel_filter(a, thr), oracle.hot_pixel_filter(a, thr))


@pytest.mark.gpu
@pytest.mark.parametrize("hot", [None, 10])
def test_cli_end_to_end_matches_library(capi, pkg, tmp_path, hot):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=5, side=48, nt=20)
    frames = np.clip(np.round(noisy), 0, 65535).astype(np.uint16)  # (rows, cols, t)
    pages = np.transpose(frames, (2, 0, 1))                          # (t, rows, cols)
    write_tiff(tmp_path / "seq.tif", pages, rows_per_strip=7, big_endian=True)
    txt = ("filename : ./seq.tif\nstart_frame : 3\nend_frame : 18\n"
           "patch_size : 4\noptimize_pgure : false\nlambda : 0.15  # fixed\n"
           "noise_alpha : 0.1\nnoise_mu : 0.1\nnoise_sigma : 0.1\nrandom_seed : 1\n")
    if hot is not None:
        txt += "hot_pixel : %d\n" % hot
    (tmp_path / "p.svt").write_text(txt)
    r = run(tmp_path / "p.svt", tmp_path)
    assert r.returncode == 0, r.stderr
    out = read_tiff16(tmp_path / "seq-CLEANED.tif")
    X = np.asfortranarray(frames[:, :, 2:18])
    if hot is not None:
        X = capi.hot_pixel_filter(X, hot)
    p = capi.default_params(median_size=5, optimize_pgure=0, lambda_=0.15, alpha=0.1, mu=0.1,
                            sigma=0.1, random_seed=1, max_iter=1000)
    Y, _, _ = capi.denoise(X, p)
    ref = np.clip(Y, 0, 65535).astype(np.uint16)  # truncation, as the tool converts
    np.testing.assert_array_equal(out, np.transpose(ref, (2, 0, 1)))


@pytest.mark.gpu
def test_cli_reference_example_parameters(capi, pkg, tmp_path):
    """The settings of the reference's examples/param_example.svt (16 x 16
    patches, overlap 2, trajectory 15, fixed lambda 0.15, given noise, motion
    estimation with the default median filter, seed 1) on a synthetic
    sequence of the example's shape."""
    noisy, _, _ = pkg.synth.workload("arps_256", seed=6, side=64, nt=25)
    frames = np.clip(np.round(noisy * 50), 0, 65535).astype(np.uint16)
    write_tiff(tmp_path / "example.tif", np.transpose(frames, (2, 0, 1)), rows_per_strip=16)
    (tmp_path / "p.svt").write_text(
        "filename    : ./example.tif  # TIFF file to be denoised\n"
        "start_frame : 1              # Start frame\n"
        "end_frame   : 25             # End frame\n"
        "patch_size            : 16    # Patch size in pixels (default = 4)\n"
        "patch_overlap         : 2     # Patch overlap in pixels (default = 1)\n"
        "trajectory_length     : 15    # must be odd\n"
        "normalize             : false # no normalisation\n"
        "noise_alpha           : 0.1\nnoise_mu              : 0.1\nnoise_sigma           : 0.1\n"
        "optimize_pgure        : false # fixed lambda\nlambda                : 0.15\n"
        "motion_estimation     : true  # ARPS\n#median_filter        : 5\n"
        "exponential_weighting : true  # weighting\nrandom_seed           : 1\n")
    r = run(tmp_path / "p.svt", tmp_path)
    assert r.returncode == 0, r.stderr
    out = read_tiff16(tmp_path / "example-CLEANED.tif")
    p = capi.default_params(block_size=16, block_overlap=2, traj_length=15, median_size=5,
                            optimize_pgure=0, lambda_=0.15, alpha=0.1, mu=0.1, sigma=0.1,
                            random_seed=1, max_iter=1000)
    Y, _, _ = capi.denoise(np.asfortranarray(frames), p)
    np.testing.assert_array_equal(out, np.transpose(np.clip(Y, 0, 65535).astype(np.uint16),
                                                    (2, 0, 1)))


@pytest.mark.gpu
def test_cli_boolean_without_trailing_comment_reads_false(capi, pkg, tmp_path):
    """ParseParameters (utils.hpp:70-89) appends a space to a value that ends
    its line, so StrToBool sees "true " and returns false; the reference's
    example files put a comment after every value.  Reproduced: a bare
    "motion_estimation : true" runs without motion estimation."""
    noisy, _, _ = pkg.synth.workload("arps_256", seed=7, side=32, nt=16)
    frames = np.clip(np.round(noisy), 0, 65535).astype(np.uint16)
    write_tiff(tmp_path / "s.tif", np.transpose(frames, (2, 0, 1)))
    (tmp_path / "p.svt").write_text(
        "filename : ./s.tif # in\nstart_frame : 1 # a\nend_frame : 16 # b\n"
        "optimize_pgure : false # c\nlambda : 0.2 # d\nnoise_alpha : 0.1 # e\n"
        "noise_mu : 0.1 # f\nnoise_sigma : 0.1 # g\nmotion_estimation : true\n")
    r = run(tmp_path / "p.svt", tmp_path)
    assert r.returncode == 0, r.stderr
    out = read_tiff16(tmp_path / "s-CLEANED.tif")
    kw = dict(median_size=5, optimize_pgure=0, lambda_=0.2, alpha=0.1, mu=0.1, sigma=0.1,
              max_iter=1000)
    Yoff, _, _ = capi.denoise(np.asfortranarray(frames), capi.default_params(motion_estimation=0, **kw))
    ref = np.transpose(np.clip(Yoff, 0, 65535).astype(np.uint16), (2, 0, 1))
    np.testing.assert_array_equal(out, ref)

"""The frame decoders take bytes from files: a damaged file must give a
status (or, where the damage leaves a valid stream, an image), never a
crash or a read outside the input.  Seeded mutations of valid PNG and JPEG
files (bit flips, byte overwrites, insertions, truncations, planted
markers) through vh_decode_depth_png, vh_decode_colour_png and
vh_decode_colour_jpeg.  Host only (no GPU)."""
import zlib

import numpy as np
import pytest

from jpeg_writer import encode_jpeg, exif_segment
from png_writer import encode_png
from vhsdf import VhError, decode_colour_jpeg, decode_colour_png, decode_depth_png
from vhsdf import _native as N


def _image(w=40, h=30):
    y, x = np.mgrid[0:h, 0:w]
    img = np.stack([x * 6, y * 8, (x * y) % 256], axis=2)
    return (img + np.random.default_rng(0).integers(0, 30, img.shape)).clip(0, 255).astype(np.uint8)


def _mutate(data, rng):
    d = bytearray(data)
    for _ in range(int(rng.integers(1, 9))):
        at = int(rng.integers(0, len(d)))
        kind = int(rng.integers(0, 5))
        if kind == 0:
            d[at] ^= 1 << int(rng.integers(0, 8))
        elif kind == 1:
            d[at] = int(rng.integers(0, 256))
        elif kind == 2 and at > 2:
            del d[at:]
        elif kind == 3:
            d.insert(at, int(rng.integers(0, 256)))
        elif kind == 4 and at + 4 < len(d):
            d[at], d[at + 1] = 0xFF, 0xC0 + int(rng.integers(0, 64))
        if len(d) < 4:
            break
    return bytes(d)


def _decodes_or_fails_cleanly(fn, data):
    try:
        out = fn(data)
    except VhError as e:
        assert e.status in (N.VH_ERR_INVALID_ARG, N.VH_ERR_UNSUPPORTED), e.status
        return False
    assert out.dtype in (np.uint8, np.uint16) and out.size > 0
    return True


@pytest.mark.parametrize("kind", ["jpeg_420_restart", "jpeg_gray", "jpeg_separate_q16",
                                  "png_rgb", "png_depth16"])
def test_mutated_files(kind):
    img = _image()
    if kind == "jpeg_420_restart":
        seed, fns = encode_jpeg(img, sampling=((2, 2), (1, 1), (1, 1)), restart=3,
                                app1=exif_segment(6)).data, [decode_colour_jpeg]
    elif kind == "jpeg_gray":
        seed, fns = encode_jpeg(img[:, :, 0]).data, [decode_colour_jpeg]
    elif kind == "jpeg_separate_q16":
        seed, fns = encode_jpeg(img, interleaved=False, q16=True).data, [decode_colour_jpeg]
    elif kind == "png_rgb":
        seed, fns = encode_png(img, depth=8, filters=[0, 1, 2, 3, 4]), [decode_colour_png]
    else:
        depth = img[:, :, 0].astype(np.uint16) * 200
        seed, fns = encode_png(depth, depth=16, filters=[4], level=1), \
            [decode_depth_png, decode_colour_png]
    for fn in fns:
        assert _decodes_or_fails_cleanly(fn, seed)
    rng = np.random.default_rng(zlib.crc32(kind.encode()))
    rejected = 0
    for _ in range(2000):
        data = _mutate(seed, rng)
        for fn in fns:
            rejected += not _decodes_or_fails_cleanly(fn, data)
    assert rejected > 0  # the damage is seen


def test_mutations_under_address_sanitizer(tmp_path):
    """The decoders' and the resize's sources built with AddressSanitizer
    and UndefinedBehaviorSanitizer (tests/decoder_fuzz_driver.cpp), 20000
    mutations of each seed: no report, exit 0."""
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ is absent")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    csrc = os.path.join(repo, "voxel-hashing-sdf_gb300", "csrc")
    exe = str(tmp_path / "fuzz")
    build = subprocess.run(
        [gxx, "-O1", "-g", "-std=c++17", "-fsanitize=address,undefined",
         "-fno-sanitize-recover=undefined", "-I", os.path.join(repo, "include"),
         os.path.join(repo, "tests", "decoder_fuzz_driver.cpp"),
         os.path.join(csrc, "vh_png.cpp"), os.path.join(csrc, "vh_jpeg.cpp"),
         os.path.join(csrc, "vh_frames.cpp"), "-o", exe],
        capture_output=True, text=True)
    if build.returncode != 0:
        if "asan" in build.stderr.lower() or "ubsan" in build.stderr.lower():
            pytest.skip("the sanitizer runtimes are absent")
        raise AssertionError(build.stderr)
    img = _image()
    seeds = {
        "a.jpg": encode_jpeg(img, sampling=((2, 2), (1, 1), (1, 1)), restart=3,
                             app1=exif_segment(6)).data,
        "f.jpg": encode_jpeg(img, app1=exif_segment(7, big_endian=True)).data,
        "b.jpg": encode_jpeg(img[:, :, 0]).data,
        "c.jpg": encode_jpeg(img, interleaved=False, q16=True, sampling=((1, 2), (1, 1),
                                                                         (1, 1))).data,
        "d.png": encode_png(img, depth=8, filters=[0, 1, 2, 3, 4]),
        "e.png": encode_png(img[:, :, 0].astype(np.uint16) * 200, depth=16, filters=[4],
                            level=1),
    }
    paths = []
    for name, data in seeds.items():
        (tmp_path / name).write_bytes(data)
        paths.append(str(tmp_path / name))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1")
    run = subprocess.run([exe, "20000"] + paths, capture_output=True, text=True, env=env,
                         timeout=600)
    assert run.returncode == 0 and "ERROR" not in run.stderr, run.stderr[-4000:]
    assert "decoded" in run.stdout

"""vh_decode_colour_jpeg: the <i>.jpg colour frames the reference loads with
cv::imread(IMREAD_COLOR) and swaps to RGB (src/SaveFrame.cpp:164,
src/main.cpp:273), decoded by the library into RGB bytes.  Host only (no
GPU).

- Files from the test-side writer (tests/jpeg_writer.py) over every layout
  the decoder reads decode to the numpy restatement of decoding the written
  coefficients, within one level (the two evaluate the same exact inverse
  DCT in different orders, which can round a half-way sample apart), and,
  at near-lossless quantisation, to the image that was encoded within a
  few levels.
- Two photographs written by an independent encoder (scikit-learn's sample
  images, baseline 4:4:4 with optimised Huffman tables; skipped where
  scikit-learn is absent) decode with every code valid and every bit of
  the entropy data used, into an image whose 8 x 8 block edges do not
  stand out from its other pixel steps (a wrong zig-zag order, coefficient
  sign or transform shows there at once).
- Truncated, reordered and unsupported files give a status, never a crash.
"""
import ctypes as C
import os

import numpy as np
import pytest

from jpeg_writer import ZIGZAG, encode_jpeg, exif_segment, expected_decode
from vhsdf import VhError, decode_colour_jpeg, synth
from vhsdf import _native as N


def test_zigzag_table_is_the_anti_diagonal_walk():
    walk = []
    for s in range(15):
        rows = range(max(0, s - 7), min(s, 7) + 1)
        for r in (rows if s % 2 else reversed(rows)):
            walk.append(r * 8 + (s - r))
    assert list(ZIGZAG) == walk and sorted(walk) == list(range(64))


def noisy(w, h, seed):
    """A smooth image with texture: gradients, a few edges and noise."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    base = np.stack([x * 255.0 / max(w - 1, 1), y * 255.0 / max(h - 1, 1),
                     128 + 100 * np.sin(x / 5.0) * np.cos(y / 7.0)], axis=2)
    base[(x // 11 + y // 13) % 3 == 0] *= 0.4
    img = base + rng.normal(0, 12, base.shape)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


CASES = {
    "444": dict(sampling=((1, 1), (1, 1), (1, 1))),
    "422": dict(sampling=((2, 1), (1, 1), (1, 1))),
    "420": dict(sampling=((2, 2), (1, 1), (1, 1))),
    "440": dict(sampling=((1, 2), (1, 1), (1, 1))),
    "411": dict(sampling=((4, 1), (1, 1), (1, 1))),
    "420_restart1": dict(sampling=((2, 2), (1, 1), (1, 1)), restart=1),
    "420_restart7": dict(sampling=((2, 2), (1, 1), (1, 1)), restart=7),
    "420_separate_scans": dict(sampling=((2, 2), (1, 1), (1, 1)), interleaved=False),
    "444_separate_scans_restart3": dict(interleaved=False, restart=3),
    "420_q16_extended": dict(sampling=((2, 2), (1, 1), (1, 1)), q16=True, extended=True),
    "adobe_rgb": dict(rgb_mode="adobe"),
    "rgb_ids": dict(rgb_mode="ids"),
    "420_coarse": dict(sampling=((2, 2), (1, 1), (1, 1)), quality_table=12),
    "444_table": dict(quality_table=np.add.outer(np.arange(8), np.arange(8)) * 3 + 2),
}


def check_against_restatement(enc):
    got = decode_colour_jpeg(enc.data)
    want = expected_decode(enc)
    assert got.shape == want.shape == (enc.height, enc.width, 3) and got.dtype == np.uint8
    diff = np.abs(got.astype(np.int64) - want)
    assert diff.max() <= 1, diff.max()
    assert (diff > 0).mean() < 0.01
    return got


@pytest.mark.parametrize("name", sorted(CASES))
def test_layouts_match_the_restatement(name):
    kw = CASES[name]
    for (w, h), seed in (((96, 72), 0), ((37, 29), 1)):
        img = noisy(w, h, seed)
        enc = encode_jpeg(img, **kw)
        got = check_against_restatement(enc)
        if kw.get("quality_table") is None and kw.get("sampling", ((1, 1),) * 3)[0] == (1, 1):
            # near-lossless and full-resolution chroma: the encoded image back
            assert np.abs(got.astype(np.int64) - img).max() <= 3


def test_grayscale_and_tiny_images():
    rng = np.random.default_rng(4)
    g = rng.integers(0, 256, (19, 23), dtype=np.uint8)
    for kw in (dict(), dict(restart=2), dict(quality_table=6)):
        enc = encode_jpeg(g, **kw)
        got = check_against_restatement(enc)
        if not kw.get("quality_table"):
            assert np.abs(got[:, :, 0].astype(np.int64) - g).max() <= 1
        assert np.array_equal(got[:, :, 0], got[:, :, 1]) and np.array_equal(got[:, :, 0], got[:, :, 2])
    for shape in [(1, 1, 3), (1, 17, 3), (17, 1, 3), (9, 9, 3)]:
        img = rng.integers(0, 256, shape, dtype=np.uint8)
        for kw in (CASES["444"], CASES["420"], CASES["422"]):
            check_against_restatement(encode_jpeg(img, **kw))


def test_chroma_siting_at_4_2_0():
    """Smooth colour at 4:2:0 comes back within a level on average: the
    decoder places each chroma sample at the centre of the 2 x 2 luma
    pixels it was averaged from.  Replicating chroma, or siting it on the
    top-left luma pixel, gives ~2.8 levels on this image."""
    y, x = np.mgrid[0:120, 0:160]
    img = np.stack([128 + 100 * np.sin(x / 9.0 + y / 17.0), 128 + 90 * np.cos(y / 8.0),
                    128 + 80 * np.sin((x - y) / 11.0)], axis=2)
    img = np.clip(np.rint(img), 0, 255).astype(np.uint8)
    enc = encode_jpeg(img, sampling=((2, 2), (1, 1), (1, 1)))
    got = check_against_restatement(enc)
    assert np.abs(got.astype(np.int64) - img).mean() < 1.0


def sample_jpegs():
    sklearn = pytest.importorskip("sklearn")
    d = os.path.join(os.path.dirname(sklearn.__file__), "datasets", "images")
    paths = [os.path.join(d, f) for f in ("china.jpg", "flower.jpg")]
    if not all(os.path.exists(p) for p in paths):
        pytest.skip("scikit-learn's sample images are absent")
    return paths


def test_photographs_from_another_encoder():
    for path in sample_jpegs():
        with open(path, "rb") as f:
            data = f.read()
        img = decode_colour_jpeg(data)
        assert img.shape == (427, 640, 3) and img.dtype == np.uint8
        a = img.astype(np.int64)
        step = np.abs(np.diff(a, axis=1)).sum(axis=2)  # (427, 639): between x and x + 1
        cols = np.arange(step.shape[1])
        at_edges = step[:, cols % 8 == 7].mean()       # across a block edge
        inside = step[:, cols % 8 != 7].mean()
        # decoded right, block edges are no steeper than the rest (1.01x and
        # 1.10x on these two); a wrong coefficient order gives several times
        assert at_edges < 1.25 * inside, (path, at_edges, inside)
        vstep = np.abs(np.diff(a, axis=0)).sum(axis=2)
        rows = np.arange(vstep.shape[0])
        assert vstep[rows % 8 == 7].mean() < 1.25 * vstep[rows % 8 != 7].mean()
        assert 20 < a.mean() < 235 and a.std() > 20
        # every truncation inside the entropy data is caught
        for cut in (len(data) // 2, len(data) - 3):
            with pytest.raises(VhError) as e:
                decode_colour_jpeg(data[:cut])
            assert e.value.status == N.VH_ERR_INVALID_ARG


def test_size_query_and_capacity():
    enc = encode_jpeg(noisy(40, 30, 2), sampling=((2, 2), (1, 1), (1, 1)))
    buf = np.frombuffer(enc.data, np.uint8)
    L = N.lib()
    w, h = C.c_int32(), C.c_int32()
    assert L.vh_decode_colour_jpeg(buf.ctypes.data, buf.size, None, 0, C.byref(w),
                                   C.byref(h)) == N.VH_OK
    assert (w.value, h.value) == (40, 30)
    small = np.zeros(40 * 30 * 3 - 1, np.uint8)
    assert L.vh_decode_colour_jpeg(buf.ctypes.data, buf.size, small.ctypes.data, small.size,
                                   C.byref(w), C.byref(h)) == N.VH_ERR_CAPACITY


def _replace_marker(data, old, new):
    i = data.index(bytes([0xFF, old]))
    return data[:i] + bytes([0xFF, new]) + data[i + 2:]


def test_malformed_and_unsupported_files():
    enc = encode_jpeg(noisy(40, 30, 3), sampling=((2, 2), (1, 1), (1, 1)), restart=2)
    good = enc.data
    assert decode_colour_jpeg(good).shape == (30, 40, 3)

    def status(data):
        with pytest.raises(VhError) as e:
            decode_colour_jpeg(data)
        return e.value.status

    for bad in (b"\xff\xd8", b"not a jpeg", good[:-2],          # no EOI
                good[:len(good) // 2] + b"\xff\xd9",            # scan cut short
                _replace_marker(good, 0xD0, 0xD1),              # restart out of order
                good[:2] + good[2:].replace(b"\xff\xc4", b"\xff\xfe", 1)):  # a table missing
        assert status(bad) == N.VH_ERR_INVALID_ARG
    assert status(_replace_marker(good, 0xC0, 0xC2)) == N.VH_ERR_UNSUPPORTED  # progressive
    assert status(_replace_marker(good, 0xC0, 0xC9)) == N.VH_ERR_UNSUPPORTED  # arithmetic
    i = good.index(b"\xff\xc0")
    twelve = good[:i + 4] + bytes([12]) + good[i + 5:]
    assert status(twelve) == N.VH_ERR_UNSUPPORTED
    cmyk = (b"\xff\xd8\xff\xc0\x00\x14\x08\x00\x08\x00\x08\x04" +
            b"".join(bytes([c, 0x11, 0]) for c in range(1, 5)) + b"\xff\xd9")
    assert status(cmyk) == N.VH_ERR_UNSUPPORTED


def test_frame_folder_reads_jpeg_colour(tmp_path):
    from test_frames import write_frame
    from vhsdf import FrameFolder
    scene = synth.Scene(kind=1, seed=0, num_frames=2, width=64, height=48)
    depth, rgb, c2w = scene.render(0)
    root = str(tmp_path / "seq")
    write_frame(root, 0, depth, rgb, c2w)
    os.remove(os.path.join(root, "RGB", "0.png"))
    big = np.repeat(np.repeat(rgb, 2, axis=0), 2, axis=1)  # 128 x 96, as a camera's larger colour
    enc = encode_jpeg(big, sampling=((2, 2), (1, 1), (1, 1)))
    with open(os.path.join(root, "RGB", "0.jpg"), "wb") as f:
        f.write(enc.data)
    fr = FrameFolder(root).load(0)
    from vhsdf import resize_colour
    assert np.array_equal(fr.rgb, resize_colour(decode_colour_jpeg(enc.data), 64, 48))
    assert np.array_equal(fr.depth, depth)


# Exif orientation -> the displayed image, by the tag's definitions:
# mirrored, rotated 180, flipped, transposed, rotated 90 clockwise to show,
# transversed (mirrored, then rotated 90 clockwise), rotated 90 anticlockwise
ORIENTED = {
    1: lambda a: a,
    2: np.fliplr,
    3: lambda a: np.rot90(a, 2),
    4: np.flipud,
    5: lambda a: np.rot90(np.fliplr(a), 1),
    6: lambda a: np.rot90(a, -1),
    7: lambda a: np.rot90(np.fliplr(a), -1),
    8: lambda a: np.rot90(a, 1),
}


@pytest.mark.parametrize("orientation", range(1, 9))
@pytest.mark.parametrize("big_endian", [False, True])
def test_exif_orientation(orientation, big_endian):
    """cv::imread(IMREAD_COLOR) shows a JPEG the way its Exif Orientation
    tag says; the decoder does the same, size query included."""
    img = noisy(37, 22, 5)
    plain = decode_colour_jpeg(encode_jpeg(img, sampling=((2, 2), (1, 1), (1, 1))).data)
    data = encode_jpeg(img, sampling=((2, 2), (1, 1), (1, 1)),
                       app1=exif_segment(orientation, big_endian)).data
    got = decode_colour_jpeg(data)
    want = np.ascontiguousarray(ORIENTED[orientation](plain))
    assert got.shape == want.shape and np.array_equal(got, want)
    buf = np.frombuffer(data, np.uint8)
    w, h = C.c_int32(), C.c_int32()
    assert N.lib().vh_decode_colour_jpeg(buf.ctypes.data, buf.size, None, 0, C.byref(w),
                                         C.byref(h)) == N.VH_OK
    assert (h.value, w.value) == want.shape[:2]


def test_exif_ignored_when_malformed_or_late():
    img = noisy(21, 13, 6)
    plain = decode_colour_jpeg(encode_jpeg(img).data)
    seg = exif_segment(6)
    cut = seg[:2] + bytes([0, len(seg) - 2 - 12]) + seg[4:-12]   # directory cut short
    for kw in (dict(app1=cut), dict(app1_after_frame=seg),
               dict(app1=seg[:10] + b"XX" + seg[12:])):               # no byte-order mark
        assert np.array_equal(decode_colour_jpeg(encode_jpeg(img, **kw).data), plain)

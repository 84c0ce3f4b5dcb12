"""Colour frames and the reference's frame folders, on the host (no GPU).

- vh_decode_colour_png: RGB, RGBA, grayscale and grayscale + alpha PNGs
  with 8- or 16-bit samples (tests/png_writer.py) decode to the RGB bytes
  the reference's cv::imread(IMREAD_COLOR) and BGR-to-RGB swap give
  (src/SaveFrame.cpp:164, src/main.cpp:273): 16-bit samples keep the high
  byte, grayscale fills all three channels, alpha is dropped.  PNGs that
  other encoders wrote (this machine's package images, where present)
  decode to exactly the pixels they were filtered from.
- vh_resize_colour: equal, byte for byte, to a numpy restatement of the
  bilinear map cv::resize applies to the reference's colour frames
  (src/SaveFrame.cpp:171).
- vhsdf.FrameFolder: the RGB/ depth/ tcw/ layout of src/SaveFrame.cpp:44-52
  read back into the arrays the engine takes, and the frame schedule of
  src/main.cpp:242-258.
"""
import os

import numpy as np
import pytest

from png_writer import encode_png
from vhsdf import Frame, FrameFolder, VhError, decode_colour_png, resize_colour, synth
from vhsdf import _native as N


def colour_frame(w=96, h=72, seed=0):
    _, rgb, _ = synth.Scene(kind=1, seed=seed, num_frames=2, width=w, height=h).render(0)
    return rgb


@pytest.mark.parametrize("filters", [[0], [1], [2], [3], [4], [0, 1, 2, 3, 4]])
def test_rgb8_every_filter(filters):
    rgb = colour_frame()
    assert rgb.dtype == np.uint8 and rgb.shape == (72, 96, 3) and rgb.std() > 10
    out = decode_colour_png(encode_png(rgb, depth=8, filters=filters, idat_parts=2))
    assert out.dtype == np.uint8 and np.array_equal(out, rgb)


def test_colour_types_and_sample_depths():
    rng = np.random.default_rng(3)
    rgb = rng.integers(0, 256, (23, 31, 3), dtype=np.uint8)
    alpha = rng.integers(0, 256, (23, 31, 1), dtype=np.uint8)
    gray = rng.integers(0, 256, (23, 31), dtype=np.uint8)
    f = [0, 1, 2, 3, 4]
    # RGBA: alpha dropped
    assert np.array_equal(decode_colour_png(encode_png(np.concatenate([rgb, alpha], 2),
                                                       depth=8, filters=f)), rgb)
    # grayscale and grayscale + alpha: the gray level in R, G and B
    g3 = np.repeat(gray[:, :, None], 3, 2)
    assert np.array_equal(decode_colour_png(encode_png(gray, depth=8, filters=f)), g3)
    assert np.array_equal(decode_colour_png(encode_png(np.stack([gray, gray ^ 0x5A], 2),
                                                       depth=8, filters=f)), g3)
    # 16-bit samples: the high byte
    rgb16 = rng.integers(0, 65536, (23, 31, 3), dtype=np.uint16)
    out = decode_colour_png(encode_png(rgb16, depth=16, filters=f))
    assert np.array_equal(out, (rgb16 >> 8).astype(np.uint8))
    rgba16 = rng.integers(0, 65536, (5, 7, 4), dtype=np.uint16)
    out = decode_colour_png(encode_png(rgba16, depth=16, filters=f))
    assert np.array_equal(out, (rgba16[:, :, :3] >> 8).astype(np.uint8))
    for shape in [(1, 1, 3), (1, 9, 3), (9, 1, 3)]:
        img = rng.integers(0, 256, shape, dtype=np.uint8)
        assert np.array_equal(decode_colour_png(encode_png(img, depth=8, filters=[4])), img)


def test_colour_errors():
    import ctypes as C
    rgb = colour_frame(16, 12)
    png = np.frombuffer(encode_png(rgb, depth=8), np.uint8)
    L = N.lib()
    w, h = C.c_int32(), C.c_int32()
    assert L.vh_decode_colour_png(png.ctypes.data, png.size, None, 0, C.byref(w),
                                  C.byref(h)) == N.VH_OK
    assert (w.value, h.value) == (16, 12)
    small = np.zeros(16 * 12 * 3 - 1, np.uint8)
    assert L.vh_decode_colour_png(png.ctypes.data, png.size, small.ctypes.data, small.size,
                                  C.byref(w), C.byref(h)) == N.VH_ERR_CAPACITY
    with pytest.raises(VhError) as e:  # palette colour type
        decode_colour_png(encode_png(rgb[:, :, 0], depth=8, colour=3))
    assert e.value.status == N.VH_ERR_UNSUPPORTED
    with pytest.raises(VhError) as e:
        decode_colour_png(encode_png(rgb, depth=8, interlace=1))
    assert e.value.status == N.VH_ERR_UNSUPPORTED
    good = encode_png(rgb, depth=8, filters=[1, 4])
    for data in (good[:-12], good[:50], b"\x89PNG\r\n\x1a\n"):
        with pytest.raises(VhError) as e:
            decode_colour_png(data)
        assert e.value.status == N.VH_ERR_INVALID_ARG
    # the depth decoder still takes grayscale only
    from vhsdf import decode_depth_png
    with pytest.raises(VhError) as e:
        decode_depth_png(good)
    assert e.value.status == N.VH_ERR_UNSUPPORTED


def resize_restated(src, w, h):
    """The bilinear map of vh_resize_colour restated in numpy, in the same
    operation order: centres at half-integers, clamped borders, weights in
    double, rounded to the nearest level."""
    sh, sw, _ = src.shape

    def taps(n_src, n_dst):
        f = (np.arange(n_dst, dtype=np.float64) + 0.5) * (n_src / n_dst) - 0.5
        i = np.floor(f).astype(np.int64)
        a = f - i
        a = np.where(i < 0, 0.0, a)
        i = np.maximum(i, 0)
        a = np.where(i >= n_src - 1, 0.0, a)
        i = np.minimum(i, n_src - 1)
        return i, np.minimum(i + 1, n_src - 1), a

    x0, x1, ax = taps(sw, w)
    y0, y1, ay = taps(sh, h)
    s = src.astype(np.float64)
    axc = ax[None, :, None]
    top = (1.0 - axc) * s[y0][:, x0] + axc * s[y0][:, x1]
    bot = (1.0 - axc) * s[y1][:, x0] + axc * s[y1][:, x1]
    ayc = ay[:, None, None]
    return np.floor((1.0 - ayc) * top + ayc * bot + 0.5).astype(np.uint8)


@pytest.mark.parametrize("src_size,dst_size", [((1296, 968), (640, 480)), ((320, 240), (640, 480)),
                                               ((97, 61), (40, 33)), ((1, 1), (5, 3)),
                                               ((7, 1), (3, 4)), ((640, 480), (640, 480))])
def test_resize_matches_restatement(src_size, dst_size):
    rng = np.random.default_rng(sum(src_size) + sum(dst_size))
    sw, sh = src_size
    src = rng.integers(0, 256, (sh, sw, 3), dtype=np.uint8)
    out = resize_colour(src, *dst_size)
    assert out.shape == (dst_size[1], dst_size[0], 3)
    assert np.array_equal(out, resize_restated(src, *dst_size))
    if src_size == dst_size:
        assert np.array_equal(out, src)


def test_resize_halves_by_averaging_pairs():
    """An exact 2:1 reduction samples halfway between each pair of source
    pixels: the mean of the 2 x 2 block, rounded half up."""
    src = np.random.default_rng(5).integers(0, 256, (8, 10, 3), dtype=np.uint8)
    out = resize_colour(src, 5, 4)
    s = src.astype(np.int64)
    mean4 = (s[0::2, 0::2] + s[0::2, 1::2] + s[1::2, 0::2] + s[1::2, 1::2])
    assert np.array_equal(out, ((mean4 + 2) // 4).astype(np.uint8))


def test_resize_errors():
    src = np.zeros((4, 4, 3), np.uint8)
    for w, h in [(0, 4), (4, 0), (40000, 4)]:
        with pytest.raises(VhError) as e:
            resize_colour(src, w, h)
        assert e.value.status == N.VH_ERR_INVALID_ARG
    with pytest.raises(ValueError):
        resize_colour(np.zeros((4, 4), np.uint8), 2, 2)


def write_frame(root, i, depth, rgb, c2w, colour_ext=".png"):
    for d in ("RGB", "depth", "tcw"):
        os.makedirs(os.path.join(root, d), exist_ok=True)
    with open(os.path.join(root, "depth", f"{i}.png"), "wb") as f:
        f.write(encode_png(depth, depth=16, filters=[4, 1]))
    with open(os.path.join(root, "RGB", f"{i}{colour_ext}"), "wb") as f:
        f.write(encode_png(rgb, depth=8, filters=[2, 4]))
    with open(os.path.join(root, "tcw", f"{i}.txt"), "w") as f:
        for r in range(4):
            f.write(" ".join(repr(float(v)) for v in c2w[r]) + "\n")


def test_frame_folder_reads_the_reference_layout(tmp_path):
    scene = synth.Scene(kind=1, seed=0, num_frames=60, width=80, height=60)
    root = str(tmp_path / "seq")
    big = {}
    for i in (0, 20, 40):
        depth, rgb, c2w = scene.render(i)
        rgb_big = resize_colour(rgb, 160, 120)  # colour stored larger than depth
        big[i] = (depth, rgb_big, c2w)
        write_frame(root, i, depth, rgb_big, c2w)
    folder = FrameFolder(root)
    fr = folder.load(20)
    assert isinstance(fr, Frame) and fr.frame_id == 20
    depth, rgb_big, c2w = big[20]
    assert fr.depth.dtype == np.uint16 and np.array_equal(fr.depth, depth)
    assert fr.rgb.shape == (60, 80, 3)
    assert np.array_equal(fr.rgb, resize_colour(rgb_big, 80, 60))
    assert fr.c2w.dtype == np.float32
    assert np.array_equal(fr.c2w, np.asarray(c2w, np.float32).reshape(4, 4))
    assert folder.load(10) is None
    assert [f.frame_id for f in folder.frames()] == [0, 20, 40]


def test_frame_schedule_stops_after_missing_frames(tmp_path):
    scene = synth.Scene(kind=1, seed=0, num_frames=2, width=16, height=12)
    depth, rgb, c2w = scene.render(0)
    root = str(tmp_path / "seq")
    present = [0, 20, 60, 100, 160, 180]  # missing: 40, 80, 120, 140, then 200 ...
    for i in present:
        write_frame(root, i, depth, rgb, c2w)
    folder = FrameFolder(root)
    # the count of missing frames is not reset by a frame that loads: the
    # walk ends when the fifth missing frame (200) has been seen
    assert [f.frame_id for f in folder.frames()] == [0, 20, 60, 100, 160, 180]
    assert [f.frame_id for f in folder.frames(max_missing=2)] == [0, 20, 60]
    assert [f.frame_id for f in folder.frames(start=20, step=40, stop=200)] == [20, 60, 100, 180]
    with pytest.raises(ValueError):
        next(folder.frames(step=0))
    # decoding ahead on threads: the same frames in the same order
    for workers in (1, 3, 8):
        for kw in (dict(), dict(max_missing=2), dict(start=20, step=40, stop=200)):
            seq = list(folder.frames(**kw))
            par = list(folder.frames(workers=workers, **kw))
            assert [f.frame_id for f in par] == [f.frame_id for f in seq]
            for a, b in zip(seq, par):
                assert np.array_equal(a.depth, b.depth) and np.array_equal(a.rgb, b.rgb)
                assert np.array_equal(a.c2w, b.c2w)
    walk = folder.frames(workers=2)  # left early: the walk closes cleanly
    assert next(walk).frame_id == 0
    walk.close()


def test_frame_folder_file_rules(tmp_path):
    scene = synth.Scene(kind=1, seed=0, num_frames=2, width=16, height=12)
    depth, rgb, c2w = scene.render(0)
    root = str(tmp_path / "seq")
    write_frame(root, 0, depth, rgb, c2w, colour_ext=".jpg")  # PNG bytes under .jpg
    write_frame(root, 1, depth, rgb, c2w)
    folder = FrameFolder(root)
    assert folder.paths(0)[0].endswith("0.jpg") and folder.paths(1)[0].endswith("1.png")
    assert np.array_equal(folder.load(0).rgb, rgb)  # decoded by content, not by name
    # a JPEG start of image with nothing valid after it, and a file that
    # is neither JPEG nor PNG
    with open(os.path.join(root, "RGB", "0.jpg"), "wb") as f:
        f.write(b"\xff\xd8\xff\xe0" + bytes(60))
    with pytest.raises(VhError) as e:
        folder.load(0)
    assert e.value.status == N.VH_ERR_INVALID_ARG
    with open(os.path.join(root, "RGB", "0.jpg"), "wb") as f:
        f.write(b"GIF89a" + bytes(60))
    with pytest.raises(VhError) as e:
        folder.load(0)
    assert e.value.status == N.VH_ERR_UNSUPPORTED
    with pytest.raises(VhError):  # the error reaches the caller from a worker too
        list(folder.frames(start=0, step=1, stop=2, workers=2))
    # missing depth or pose: the frame is missing
    os.remove(os.path.join(root, "tcw", "1.txt"))
    assert folder.load(1) is None
    write_frame(root, 2, depth, rgb, c2w)
    os.remove(os.path.join(root, "depth", "2.png"))
    assert folder.load(2) is None


def test_pose_text(tmp_path):
    """tcw/<i>.txt: 16 numbers separated by any white space, each the
    nearest float to its decimal (the reference reads them with
    operator>>), the last row set to 0 0 0 1; fewer numbers or a
    non-finite one are errors."""
    scene = synth.Scene(kind=1, seed=0, num_frames=2, width=16, height=12)
    depth, rgb, c2w = scene.render(0)
    root = str(tmp_path / "seq")
    write_frame(root, 0, depth, rgb, c2w)
    folder = FrameFolder(root)
    pose = os.path.join(root, "tcw", "0.txt")
    with open(pose, "w") as f:
        f.write("1 0 0 0.5\n0 1\t0 -1e-3\n0 0 1 2.0000001\n7 7 7 7\n")
    m = folder.load(0).c2w
    assert m.dtype == np.float32 and m.shape == (4, 4)
    assert np.array_equal(m[3], [0, 0, 0, 1]) and m[0, 3] == np.float32(0.5)
    assert m[1, 3] == np.float32(-1e-3) and m[2, 3] == np.float32("2.0000001")
    for text, status in (("1 2 3", N.VH_ERR_INVALID_ARG),
                         ("1 0 0 x 0 1 0 0 0 0 1 0 0 0 0 1", N.VH_ERR_INVALID_ARG),
                         (" ".join(["nan"] * 16), N.VH_ERR_NOT_FINITE),
                         ("1e39 " * 16, N.VH_ERR_NOT_FINITE)):
        with open(pose, "w") as f:
            f.write(text)
        with pytest.raises(VhError) as e:
            folder.load(0)
        assert e.value.status == status, text


def _system_pngs():
    """PNG files that other encoders wrote (icons and documentation images
    of this machine's packages), or none."""
    import glob
    found = []
    for pattern in ("/usr/share/**/*.png", "/usr/local/cuda*/**/*.png", "/opt/nvidia/**/*.png",
                    "/usr/local/lib/python3*/dist-packages/*/**/*.png"):
        found += glob.glob(pattern, recursive=True)
    return sorted(found)[:400]


def test_pngs_from_other_encoders_decode_exactly():
    """Files written by other PNG encoders (libpng with adaptive filters,
    zlib at their levels): the decoded pixels, filtered again row by row
    with the file's own filter types (tests/png_writer.py's filters), give
    back exactly the filtered bytes of the file, so they are the pixels
    the encoder started from.  Lossless cases: 8-bit RGB through
    vh_decode_colour_png, 8- and 16-bit grayscale through
    vh_decode_depth_png."""
    import struct
    import zlib
    from png_writer import _filter_row
    from vhsdf import decode_depth_png
    checked = 0
    for path in _system_pngs():
        with open(path, "rb") as f:
            data = f.read()
        if data[:8] != b"\x89PNG\r\n\x1a\n":
            continue
        w, h, depth, colour, _, _, interlace = struct.unpack(">IIBBBBB", data[16:29])
        if interlace or (colour, depth) not in ((2, 8), (0, 8), (0, 16)):
            continue
        pos, idat = 8, b""
        while pos + 8 <= len(data):
            n = struct.unpack(">I", data[pos:pos + 4])[0]
            if data[pos + 4:pos + 8] == b"IDAT":
                idat += data[pos + 8:pos + 8 + n]
            pos += n + 12
        if colour == 2:
            img = decode_colour_png(data)
            raw = img.reshape(h, w * 3)
            bpp = 3
        else:
            img = decode_depth_png(data)
            raw = img.astype(">u2").view(np.uint8).reshape(h, 2 * w) if depth == 16 else \
                img.astype(np.uint8)
            bpp = depth // 8
        stride = raw.shape[1]
        filtered = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, stride + 1)
        prev = np.zeros(stride, np.int64)
        for y in range(h):
            cur = raw[y].astype(np.int64)
            again = _filter_row(int(filtered[y, 0]), cur, prev, bpp)
            assert np.array_equal(again, filtered[y, 1:]), (path, y, int(filtered[y, 0]))
            prev = cur
        checked += 1
    if checked == 0:
        pytest.skip("no RGB or grayscale PNG from another encoder on this machine")


def test_load_frame_c_abi(tmp_path):
    """vh_load_frame called directly: the size query, the buffers, the
    status of a missing frame and of bad arguments."""
    import ctypes as C
    scene = synth.Scene(kind=1, seed=0, num_frames=2, width=32, height=24)
    depth, rgb, c2w = scene.render(0)
    root = str(tmp_path / "seq")
    write_frame(root, 3, depth, resize_colour(rgb, 64, 48), c2w)
    L = N.lib()
    w, h = C.c_int32(), C.c_int32()
    r = root.encode()
    assert L.vh_load_frame(r, 3, None, 0, None, 0, None, C.byref(w), C.byref(h)) == N.VH_OK
    assert (w.value, h.value) == (32, 24)
    d = np.zeros((24, 32), np.uint16)
    c = np.zeros((24, 32, 3), np.uint8)
    m = np.zeros(16, np.float32)
    args = (d.ctypes.data, d.size, c.ctypes.data, c.size, m.ctypes.data, C.byref(w), C.byref(h))
    assert L.vh_load_frame(r, 3, *args) == N.VH_OK
    assert np.array_equal(d, depth) and np.array_equal(m.reshape(4, 4), c2w)
    assert np.array_equal(c, resize_colour(resize_colour(rgb, 64, 48), 32, 24))
    assert L.vh_load_frame(r, 4, *args) == N.VH_ERR_IO                       # missing
    assert L.vh_load_frame(b"/nonexistent-dir", 3, *args) == N.VH_ERR_IO
    assert L.vh_load_frame(r, -1, *args) == N.VH_ERR_INVALID_ARG
    assert L.vh_load_frame(None, 3, *args) == N.VH_ERR_INVALID_ARG
    assert L.vh_load_frame(r, 3, d.ctypes.data, d.size - 1, c.ctypes.data, c.size,
                           m.ctypes.data, C.byref(w), C.byref(h)) == N.VH_ERR_CAPACITY
    assert L.vh_load_frame(r, 3, d.ctypes.data, d.size, c.ctypes.data, c.size - 1,
                           m.ctypes.data, C.byref(w), C.byref(h)) == N.VH_ERR_CAPACITY
    assert L.vh_load_frame(r, 3, d.ctypes.data, d.size, None, 0, m.ctypes.data,
                           C.byref(w), C.byref(h)) == N.VH_ERR_INVALID_ARG
    assert L.vh_load_frame(r, 3, d.ctypes.data, d.size, c.ctypes.data, c.size, None,
                           C.byref(w), C.byref(h)) == N.VH_ERR_INVALID_ARG

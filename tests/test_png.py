"""vh_decode_depth_png: grayscale PNG depth frames (the reference reads its
depth frames with cv::imread(path, -1), src/SaveFrame.cpp:174-180) decoded
by the library into uint16.  The PNGs are written here by a small encoder
over Python's zlib: every filter type, stored / fixed-Huffman / dynamic
blocks, several IDAT chunks, 8- and 16-bit samples (tests/png_writer.py);
the decoded image must equal the encoder's input exactly.  Corrupt and
unsupported files give a status, never a crash.  Host only (no GPU)."""
import struct
import zlib

import numpy as np
import pytest

from png_writer import chunk as _chunk
from png_writer import encode_png
from vhsdf import VhError, decode_depth_png, synth
from vhsdf import _native as N


def depth_frame(w=160, h=120):
    d, _, _ = synth.Scene(kind=1, seed=0, num_frames=2, width=w, height=h).render(0)
    return d


@pytest.mark.parametrize("filters", [[0], [1], [2], [3], [4], [0, 1, 2, 3, 4], [4, 3, 2, 1, 0]])
def test_every_filter_type(filters):
    img = depth_frame()
    assert img.dtype == np.uint16 and img.max() > 1000
    out = decode_depth_png(encode_png(img, filters=filters))
    assert out.dtype == np.uint16 and np.array_equal(out, img)


@pytest.mark.parametrize("level,strategy", [(0, zlib.Z_DEFAULT_STRATEGY),
                                            (1, zlib.Z_DEFAULT_STRATEGY),
                                            (9, zlib.Z_DEFAULT_STRATEGY),
                                            (6, zlib.Z_FIXED),
                                            (6, zlib.Z_HUFFMAN_ONLY),
                                            (6, zlib.Z_RLE)])
def test_block_kinds(level, strategy):
    """Stored blocks (level 0), fixed-Huffman blocks (Z_FIXED), literal-only
    and run-length streams, and dynamic blocks."""
    rng = np.random.default_rng(level * 10 + strategy)
    img = depth_frame()
    img[rng.random(img.shape) < 0.05] = 0  # dropouts, as real depth has
    out = decode_depth_png(encode_png(img, filters=[0, 1, 2, 3, 4], level=level,
                                      strategy=strategy, idat_parts=3))
    assert np.array_equal(out, img)


def test_full_size_frame_and_noise():
    img = depth_frame(640, 480)
    assert np.array_equal(decode_depth_png(encode_png(img, filters=[4, 1])), img)
    noise = np.random.default_rng(7).integers(0, 65536, (37, 53), dtype=np.uint16)
    assert np.array_equal(decode_depth_png(encode_png(noise, filters=[0, 1, 2, 3, 4])), noise)


def test_eight_bit_and_tiny_images():
    g = np.random.default_rng(1).integers(0, 256, (9, 13)).astype(np.uint8)
    out = decode_depth_png(encode_png(g, depth=8, filters=[0, 1, 2, 3, 4]))
    assert out.dtype == np.uint16 and np.array_equal(out, g.astype(np.uint16))
    for shape in [(1, 1), (1, 17), (17, 1)]:
        img = np.arange(np.prod(shape), dtype=np.uint16).reshape(shape) * 977
        assert np.array_equal(decode_depth_png(encode_png(img, filters=[4])), img)


def test_size_query_and_capacity():
    import ctypes as C
    img = depth_frame(64, 48)
    png = np.frombuffer(encode_png(img), np.uint8)
    L = N.lib()
    w, h = C.c_int32(), C.c_int32()
    assert L.vh_decode_depth_png(png.ctypes.data, png.size, None, 0, C.byref(w),
                                 C.byref(h)) == N.VH_OK
    assert (w.value, h.value) == (64, 48)
    small = np.zeros(100, np.uint16)
    assert L.vh_decode_depth_png(png.ctypes.data, png.size, small.ctypes.data, small.size,
                                 C.byref(w), C.byref(h)) == N.VH_ERR_CAPACITY


def test_corrupt_and_unsupported_files():
    img = depth_frame(64, 48)
    good = encode_png(img, filters=[0, 1, 2, 3, 4])
    bad_crc = bytearray(good)
    bad_crc[40] ^= 0x01  # inside IHDR/tEXt/IDAT: its chunk CRC no longer matches
    cases = [b"not a png at all", good[:7], good[:60], good[:-12], bytes(bad_crc)]
    for data in cases:
        with pytest.raises(VhError) as e:
            decode_depth_png(data)
        assert e.value.status == N.VH_ERR_INVALID_ARG
    for kw in (dict(interlace=1), dict(colour=2)):
        with pytest.raises(VhError) as e:
            decode_depth_png(encode_png(img, **kw))
        assert e.value.status == N.VH_ERR_UNSUPPORTED
    # damaged compressed data with valid chunk CRCs: the Adler-32 or the
    # inflater rejects it
    z = zlib.compress(b"\x00" + b"\x01" * 10)
    broken = z[:2] + bytes([z[2] ^ 0xFF]) + z[3:]
    ihdr = struct.pack(">IIBBBBB", 5, 1, 16, 0, 0, 0, 0)
    png = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", broken) +
           _chunk(b"IEND", b""))
    with pytest.raises(VhError) as e:
        decode_depth_png(png)
    assert e.value.status == N.VH_ERR_INVALID_ARG

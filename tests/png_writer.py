"""A small PNG writer for the decoder tests (test side only): grayscale,
grayscale + alpha, RGB and RGBA images with 8- or 16-bit samples, every
filter type, any zlib level and strategy, the image data split over several
IDAT chunks.  Filters follow the PNG specification; compression is Python's
zlib."""
import struct
import zlib

import numpy as np

COLOUR_TYPE = {1: 0, 2: 4, 3: 2, 4: 6}  # channels -> PNG colour type


def chunk(kind, data):
    body = kind + data
    return struct.pack(">I", len(data)) + body + struct.pack(">I", zlib.crc32(body) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_row(ft, cur, prev, bpp):
    """PNG filter `ft` of one row of bytes (cur, prev: int arrays)."""
    left = np.concatenate([np.zeros(bpp, np.int64), cur[:-bpp]])
    upleft = np.concatenate([np.zeros(bpp, np.int64), prev[:-bpp]])
    if ft == 0:
        pred = np.zeros_like(cur)
    elif ft == 1:
        pred = left
    elif ft == 2:
        pred = prev
    elif ft == 3:
        pred = (left + prev) >> 1
    else:
        pred = _paeth(left, prev, upleft)
    return ((cur - pred) & 0xFF).astype(np.uint8)


def encode_png(img, depth=16, filters=None, level=6, strategy=zlib.Z_DEFAULT_STRATEGY,
               idat_parts=1, interlace=0, colour=None):
    """A PNG of `img` ((h, w) grayscale or (h, w, channels) with 2, 3 or 4
    channels); filters: one filter type per row, cycled; colour: the IHDR
    colour type to write (default: the one the channel count implies)."""
    img = np.asarray(img)
    if img.ndim == 2:
        img = img[:, :, None]
    h, w, ch = img.shape
    if colour is None:
        colour = COLOUR_TYPE[ch]
    if depth == 16:
        raw = img.astype(">u2").view(np.uint8).reshape(h, 2 * w * ch)
    else:
        raw = img.astype(np.uint8).reshape(h, w * ch)
    bpp = ch * depth // 8
    filters = filters or [0]
    rows = []
    prev = np.zeros(raw.shape[1], np.int64)
    for y in range(h):
        cur = raw[y].astype(np.int64)
        ft = filters[y % len(filters)]
        rows.append(bytes([ft]) + _filter_row(ft, cur, prev, bpp).tobytes())
        prev = cur
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
    z = co.compress(b"".join(rows)) + co.flush()
    parts = [z[i * len(z) // idat_parts:(i + 1) * len(z) // idat_parts] for i in range(idat_parts)]
    ihdr = struct.pack(">IIBBBBB", w, h, depth, colour, 0, 0, interlace)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"tEXt", b"k\x00v") +
            b"".join(chunk(b"IDAT", p) for p in parts) + chunk(b"IEND", b""))

"""A small sequential JPEG writer for the decoder tests (test side only),
after ITU-T T.81: forward DCT of level-shifted 8 x 8 blocks, quantisation,
zig-zag order, DC differences and AC run/size symbols coded with Huffman
tables built from the symbol counts of the image (code lengths limited to
16 bits, the all-ones code left unused), byte stuffing, restart markers.
Options cover what the decoder reads: grayscale and YCbCr with 4:4:4,
4:2:2 and 4:2:0 sampling (or any whole ratios), RGB components (Adobe
marker or 'R', 'G', 'B' ids), interleaved or one-scan-per-component
layouts, 8- or 16-bit quantisation tables, baseline or extended frame
markers.

`expected_decode` restates the decoding of the written coefficients in
numpy (exact inverse DCT, triangle-filter chroma upsampling, JFIF colour
transform) for the comparison with the library's decoder.
"""
import heapq
import struct

import numpy as np

# the zig-zag scan order as the standard tabulates it (natural index of the
# k-th coefficient)
ZIGZAG = np.array([
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5,
    12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14, 21, 28,
    35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
    58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])


def dct_matrix():
    """C[u, x] = c(u) / 2 * cos((2x + 1) u pi / 16), c(0) = 1 / sqrt(2)."""
    u = np.arange(8)[:, None]
    x = np.arange(8)[None, :]
    c = np.where(u == 0, np.sqrt(0.5), 1.0)
    return c * 0.5 * np.cos((2 * x + 1) * u * np.pi / 16)


DCT = dct_matrix()


def _segment(marker, data):
    return bytes([0xFF, marker]) + struct.pack(">H", len(data) + 2) + data


def _category(v):
    return int(abs(int(v))).bit_length()


def _code_lengths(freq):
    """Huffman code lengths (<= 16) for the symbols with nonzero counts; a
    reserved pseudo-symbol of count 1 leaves one code of the tree unused,
    as JPEG encoders do to keep the all-ones code free."""
    freq = dict(freq)
    while True:
        items = [(f, i, (s,)) for i, (s, f) in enumerate(sorted(freq.items()))]
        items.append((1, len(items), (-1,)))  # reserved
        heapq.heapify(items)
        length = {s: 0 for s in list(freq) + [-1]}
        if len(items) == 1:
            length[items[0][2][0]] = 1
        tie = len(items)
        while len(items) > 1:
            f1, _, a = heapq.heappop(items)
            f2, _, b = heapq.heappop(items)
            for s in a + b:
                length[s] += 1
            heapq.heappush(items, (f1 + f2, tie, a + b))
            tie += 1
        if max(length.values()) <= 16:
            break
        freq = {s: f // 2 + 1 for s, f in freq.items()}  # flatten and retry
    del length[-1]
    return length


class HuffTable:
    def __init__(self, freq):
        length = _code_lengths(freq)
        order = sorted(length, key=lambda s: (length[s], s))
        self.counts = [0] * 16
        for s in order:
            self.counts[length[s] - 1] += 1
        self.symbols = order
        self.code = {}
        code, k = 0, 0
        for ln in range(1, 17):
            for _ in range(self.counts[ln - 1]):
                self.code[order[k]] = (code, ln)
                code += 1
                k += 1
            code <<= 1

    def dht(self, tc, th):
        return bytes([(tc << 4) | th]) + bytes(self.counts) + bytes(self.symbols)


class BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, nbits):
        for i in range(nbits - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0x00)
                self.acc = 0
                self.n = 0

    def pad(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def rgb_to_ycbcr(rgb):
    r, g, b = (rgb[..., i].astype(np.float64) for i in range(3))
    y = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128.0
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128.0
    return [y, cb, cr]


def _pad_to(plane, ph, pw):
    h, w = plane.shape
    return np.pad(plane, ((0, ph - h), (0, pw - w)), mode="edge")


class Encoded:
    """What the writer produced: the file and the quantised coefficients per
    component (block grid, zig-zag order) that the decoder must recover."""

    def __init__(self, data, comps, qtables, width, height, hmax, vmax, rgb_components):
        self.data = data
        self.comps = comps  # list of dict(h, v, w, ht, coef (bh, bw, 64) int, tq)
        self.qtables = qtables
        self.width, self.height = width, height
        self.hmax, self.vmax = hmax, vmax
        self.rgb_components = rgb_components


def exif_segment(orientation, big_endian=False):
    """An Exif APP1 segment whose first image file directory holds the
    Orientation tag (0x0112, one SHORT) and one more tag before it."""
    e = ">" if big_endian else "<"
    tiff = (b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, 8)
    ifd = struct.pack(e + "H", 2)
    ifd += struct.pack(e + "HHI", 0x010F, 2, 4) + b"cam\x00"          # Make, ASCII, inline
    ifd += struct.pack(e + "HHIH", 0x0112, 3, 1, orientation) + b"\x00\x00"
    ifd += struct.pack(e + "I", 0)                                      # no next directory
    return _segment(0xE1, b"Exif\x00\x00" + tiff + ifd)


def encode_jpeg(img, sampling=((1, 1), (1, 1), (1, 1)), quality_table=None, restart=0,
                interleaved=True, q16=False, extended=False, rgb_mode=None, app1=b"",
                app1_after_frame=b""):
    """A JPEG of `img` ((h, w) grayscale or (h, w, 3) RGB uint8).
    sampling: (h, v) per component; quality_table: a scalar or an 8 x 8 table
    (natural order) of quantiser steps (default 1: near lossless);
    rgb_mode: None (YCbCr), "adobe" or "ids" (samples stored as R, G, B);
    app1 / app1_after_frame: segments written before the quantisation
    tables / right after the frame header."""
    img = np.asarray(img)
    gray = img.ndim == 2
    height, width = img.shape[:2]
    if gray:
        planes = [img.astype(np.float64)]
        sampling = ((1, 1),)
    elif rgb_mode:
        planes = [img[..., i].astype(np.float64) for i in range(3)]
    else:
        planes = rgb_to_ycbcr(img)
    hmax = max(s[0] for s in sampling)
    vmax = max(s[1] for s in sampling)
    mcux = -(-width // (8 * hmax))
    mcuy = -(-height // (8 * vmax))
    q = np.ones((8, 8)) if quality_table is None else np.broadcast_to(
        np.asarray(quality_table, np.float64), (8, 8))
    qz = np.asarray(q, np.int64).reshape(64)[ZIGZAG]  # zig-zag order
    qtables = [qz, np.maximum(qz, 1)]
    comps = []
    for ci, (plane, (h, v)) in enumerate(zip(planes, sampling)):
        rx, ry = hmax // h, vmax // v
        cw, ch = -(-width * h // hmax), -(-height * v // vmax)
        # box-average downsampling over rx x ry source pixels (edge-extended)
        src = _pad_to(plane, ch * ry, cw * rx)
        down = src.reshape(ch, ry, cw, rx).mean(axis=(1, 3))
        pw, ph = mcux * h * 8, mcuy * v * 8
        full = _pad_to(down, ph, pw) - 128.0
        blocks = full.reshape(ph // 8, 8, pw // 8, 8).transpose(0, 2, 1, 3)
        # F[a, b, u, v] = sum_x sum_y C[u, x] B[x, y] C[v, y]: u is the row
        # (vertical) frequency, v the column frequency, natural index u*8+v
        F = np.einsum("ux,abxy,vy->abuv", DCT, blocks, DCT)
        tq = 0 if ci == 0 else 1
        qnat = np.empty(64, np.int64)
        qnat[ZIGZAG] = qtables[tq]
        coef_nat = np.rint(F.reshape(ph // 8, pw // 8, 64) / qnat).astype(np.int64)
        comps.append(dict(h=h, v=v, w=cw, ht=ch, tq=tq, coef=coef_nat[..., ZIGZAG]))

    ncomp = len(comps)
    ids = [ord("R"), ord("G"), ord("B")] if rgb_mode == "ids" else [1, 2, 3]
    # scans: all components interleaved, or one per component
    scans = [list(range(ncomp))] if (interleaved and ncomp > 1) else [[c] for c in range(ncomp)]

    def scan_units(sc):
        """(component, block row, block col) in coding order, with MCU starts."""
        units, starts = [], []
        if len(sc) == 1:
            c = comps[sc[0]]
            bw, bh = -(-c["w"] // 8), -(-c["ht"] // 8)
            for by in range(bh):
                for bx in range(bw):
                    starts.append(len(units))
                    units.append((sc[0], by, bx))
        else:
            for my in range(mcuy):
                for mx in range(mcux):
                    starts.append(len(units))
                    for ci in sc:
                        c = comps[ci]
                        for vv in range(c["v"]):
                            for hh in range(c["h"]):
                                units.append((ci, my * c["v"] + vv, mx * c["h"] + hh))
        return units, starts

    # symbol statistics for the Huffman tables (0: luma, 1: chroma)
    dc_freq = [dict(), dict()]
    ac_freq = [dict(), dict()]

    def symbols(sc):
        units, starts = scan_units(sc)
        start_set = set(starts)
        mcu_index = {s: i for i, s in enumerate(starts)}
        pred = {c: 0 for c in sc}
        out = []  # (kind, table, symbol, bits, nbits) or ("rst", m)
        for ui, (ci, by, bx) in enumerate(units):
            if ui in start_set and restart and mcu_index[ui] and mcu_index[ui] % restart == 0:
                out.append(("rst", (mcu_index[ui] // restart - 1) % 8))
                pred = {c: 0 for c in sc}
            t = 0 if ci == 0 else 1
            zz = comps[ci]["coef"][by, bx]
            diff = int(zz[0]) - pred[ci]
            pred[ci] = int(zz[0])
            s = _category(diff)
            out.append(("dc", t, s, diff if diff >= 0 else diff + (1 << s) - 1, s))
            run = 0
            last = max([k for k in range(1, 64) if zz[k] != 0], default=0)
            for k in range(1, last + 1):
                a = int(zz[k])
                if a == 0:
                    run += 1
                    continue
                while run > 15:
                    out.append(("ac", t, 0xF0, 0, 0))
                    run -= 16
                s = _category(a)
                out.append(("ac", t, (run << 4) | s, a if a >= 0 else a + (1 << s) - 1, s))
                run = 0
            if last < 63:
                out.append(("ac", t, 0x00, 0, 0))
        return out

    scan_syms = [symbols(sc) for sc in scans]
    for syms in scan_syms:
        for e in syms:
            if e[0] == "dc":
                dc_freq[e[1]][e[2]] = dc_freq[e[1]].get(e[2], 0) + 1
            elif e[0] == "ac":
                ac_freq[e[1]][e[2]] = ac_freq[e[1]].get(e[2], 0) + 1
    ntab = 1 if ncomp == 1 else 2
    dct_tabs = [HuffTable(dc_freq[t]) for t in range(ntab)]
    act_tabs = [HuffTable(ac_freq[t]) for t in range(ntab)]

    out = bytearray(b"\xFF\xD8")
    out += _segment(0xE0, b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00")
    out += app1
    if rgb_mode == "adobe":
        out += _segment(0xEE, b"Adobe" + bytes([0, 100, 0, 0, 0, 0, 0]))
    for t in range(ntab):
        if q16:
            out += _segment(0xDB, bytes([0x10 | t]) + b"".join(
                struct.pack(">H", int(x)) for x in qtables[t]))
        else:
            out += _segment(0xDB, bytes([t]) + bytes(int(x) for x in qtables[t]))
    sof = struct.pack(">BHHB", 8, height, width, ncomp)
    for ci, c in enumerate(comps):
        sof += bytes([ids[ci], (c["h"] << 4) | c["v"], c["tq"]])
    out += _segment(0xC1 if extended else 0xC0, sof)
    out += app1_after_frame
    for t in range(ntab):
        out += _segment(0xC4, dct_tabs[t].dht(0, t))
        out += _segment(0xC4, act_tabs[t].dht(1, t))
    if restart:
        out += _segment(0xDD, struct.pack(">H", restart))
    for sc, syms in zip(scans, scan_syms):
        sos = bytes([len(sc)])
        for ci in sc:
            t = 0 if ci == 0 else 1
            sos += bytes([ids[ci], (t << 4) | t])
        sos += bytes([0, 63, 0])
        out += _segment(0xDA, sos)
        bw = BitWriter()
        for e in syms:
            if e[0] == "rst":
                bw.pad()
                bw.out += bytes([0xFF, 0xD0 + e[1]])
                continue
            tab = (dct_tabs if e[0] == "dc" else act_tabs)[e[1]]
            code, ln = tab.code[e[2]]
            bw.put(code, ln)
            if e[4]:
                bw.put(e[3], e[4])
        bw.pad()
        out += bw.out
    out += b"\xFF\xD9"
    return Encoded(bytes(out), comps, qtables, width, height, hmax, vmax, bool(rgb_mode))


def _upsample(plane, cw, ch, rx, ry, width, height):
    """Full-resolution samples from a component plane: the triangle filter
    (3/4, 1/4 per axis, clamped) for a ratio of 2, copies for 1,
    replication otherwise."""
    p = plane[:ch, :cw].astype(np.int64)

    def taps(n_out, r, n_in):
        i = np.arange(n_out)
        if r == 1:
            return i, i, 4, 0
        if r == 2:
            main = i >> 1
            other = np.where(i & 1, np.minimum(main + 1, n_in - 1), np.maximum(main - 1, 0))
            return main, other, 3, 1
        return np.minimum(i // r, n_in - 1), None, None, None

    ym, yo, wy0, wy1 = taps(height, ry, ch)
    xm, xo, wx0, wx1 = taps(width, rx, cw)
    if yo is None or xo is None:  # replication
        return p[np.minimum(np.arange(height) // ry, ch - 1)][:, np.minimum(
            np.arange(width) // rx, cw - 1)].astype(np.uint8)
    acc = (wy0 * (wx0 * p[ym][:, xm] + wx1 * p[ym][:, xo]) +
           wy1 * (wx0 * p[yo][:, xm] + wx1 * p[yo][:, xo]))
    return ((acc + 8) >> 4).astype(np.uint8)


def expected_decode(enc):
    """The decoding of `enc`'s coefficients restated in numpy."""
    planes = []
    for c in enc.comps:
        qz = enc.qtables[c["tq"]]
        zz = c["coef"] * qz  # dequantised, zig-zag order
        bh, bw = zz.shape[:2]
        nat = np.zeros((bh, bw, 64), np.float64)
        nat[..., ZIGZAG] = zz
        F = nat.reshape(bh, bw, 8, 8)
        blocks = np.einsum("ux,abuv,vy->abxy", DCT, F, DCT)
        samples = np.clip(np.floor(blocks + 128.0 + 0.5), 0, 255).astype(np.uint8)
        plane = samples.transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8)
        rx, ry = enc.hmax // c["h"], enc.vmax // c["v"]
        planes.append(_upsample(plane, c["w"], c["ht"], rx, ry, enc.width, enc.height))
    if len(planes) == 1:
        return np.repeat(planes[0][:, :, None], 3, axis=2)
    if enc.rgb_components:
        return np.stack(planes, axis=2)
    y, cb, cr = (p.astype(np.float64) for p in planes)
    r = y + 1.402 * (cr - 128)
    g = y + (-0.34414 * (cb - 128)) + (-0.71414 * (cr - 128))
    b = y + 1.772 * (cb - 128)
    return np.clip(np.floor(np.stack([r, g, b], axis=2) + 0.5), 0, 255).astype(np.uint8)

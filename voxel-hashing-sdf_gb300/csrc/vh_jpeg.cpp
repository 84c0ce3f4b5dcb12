// vh_jpeg.cpp - JPEG colour frames to interleaved RGB u8 (vh_decode_colour_jpeg).
//
// The reference loads each colour frame with cv::imread(<i>.jpg,
// IMREAD_COLOR) and swaps BGR to RGB before fusing it (src/SaveFrame.cpp:164,
// src/main.cpp:273).  This decoder reads the sequential Huffman-coded JPEG
// those files are (ITU-T T.81: baseline and extended sequential, 8-bit
// samples, one or three components, any of the 1..4 sampling factors whose
// ratios are whole, interleaved or single-component scans, restart
// intervals) and writes the RGB bytes vh_integrate takes.  Progressive,
// lossless, arithmetic-coded, 12-bit and four-component (CMYK) files are
// reported as VH_ERR_UNSUPPORTED.
//
// Stages, each from its published definition:
//   entropy decoding - canonical Huffman codes from the DHT code-length
//     counts (T.81 Annex C), a 9-bit lookahead table with the
//     code-by-length search behind it, DC differences, AC run/size symbols
//     with end-of-block and 16-zero runs, stuffed 0xFF 0x00 bytes, restart
//     markers (T.81 F.2);
//   inverse DCT - the 8 x 8 type-III DCT of T.81 A.3.3 evaluated separably in
//     double, rounded to the nearest level after the +128 level shift;
//   chroma upsampling - for a ratio of 2 the triangle filter of centred
//     chroma siting (weights 3/4 and 1/4 per axis, edges clamped), for
//     other ratios replication;
//   colour - the JFIF YCbCr to RGB transform (R = Y + 1.402 Cr',
//     G = Y - 0.34414 Cb' - 0.71414 Cr', B = Y + 1.772 Cb', with
//     Cb' = Cb - 128 and Cr' = Cr - 128), or none for an Adobe file
//     marked RGB or components named 'R', 'G', 'B';
//   orientation - an Exif Orientation tag (APP1, before the frame header)
//     turns and mirrors the image into its displayed orientation, as
//     cv::imread does for IMREAD_COLOR.
// libjpeg's integer IDCT and fixed-point colour tables can land one level
// away from these exact forms on some pixels.  Every read is
// bounds-checked; a stream whose codes run past the end of its data is
// rejected.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/vhsdf.h"

namespace {

// natural (row-major) index of the k-th coefficient in zig-zag order: the
// anti-diagonals r + c = s, walked with the row rising for odd s and
// falling for even s
struct Zigzag {
  uint8_t v[64];
  Zigzag() {
    int k = 0;
    for (int s = 0; s < 15; ++s) {
      const int lo = s > 7 ? s - 7 : 0, hi = s < 7 ? s : 7;
      if (s & 1)
        for (int r = lo; r <= hi; ++r) v[k++] = (uint8_t)(r * 8 + (s - r));
      else
        for (int r = hi; r >= lo; --r) v[k++] = (uint8_t)(r * 8 + (s - r));
    }
  }
};
const Zigzag kZig;

// c[x][u] = C(u) / 2 * cos((2x + 1) u pi / 16), C(0) = 1 / sqrt(2), else 1;
// t[u][x] = c[x][u]
struct IdctBasis {
  double c[8][8], t[8][8];
  IdctBasis() {
    const double pi = 3.14159265358979323846;
    for (int x = 0; x < 8; ++x)
      for (int u = 0; u < 8; ++u) {
        c[x][u] = (u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 * std::cos((2 * x + 1) * u * pi / 16.0);
        t[u][x] = c[x][u];
      }
  }
};
const IdctBasis kBasis;

constexpr int kLook = 9;

struct Huffman {
  bool defined = false;
  uint8_t look_len[1 << kLook];  // 0: the code is longer than kLook bits
  uint8_t look_sym[1 << kLook];
  int32_t mincode[17], maxcode[17], valptr[17];
  uint8_t vals[256];

  bool build(const uint8_t counts[16], const uint8_t *symbols, int total) {
    std::memcpy(vals, symbols, (size_t)total);
    std::memset(look_len, 0, sizeof(look_len));
    int32_t code = 0, k = 0;
    for (int len = 1; len <= 16; ++len) {
      const int n = counts[len - 1];
      valptr[len] = k;
      mincode[len] = code;
      maxcode[len] = n ? code + n - 1 : -1;
      for (int i = 0; i < n; ++i, ++k, ++code) {
        if (code >= (1 << len)) return false;  // over-subscribed
        if (len <= kLook) {
          const int shift = kLook - len;
          for (int f = code << shift; f < ((code + 1) << shift); ++f) {
            look_len[f] = (uint8_t)len;
            look_sym[f] = vals[k];
          }
        }
      }
      code <<= 1;
    }
    defined = true;
    return true;
  }
};

// Entropy-coded data, most significant bit first.  A marker (0xFF followed
// by anything but 0x00) ends the data: zero bits are fed after it, and a
// read that reaches them marks the stream as overrun.
struct BitReader {
  const uint8_t *p = nullptr;
  size_t n = 0, pos = 0;
  uint64_t buf = 0;  // the next bit is bit 63
  int cnt = 0;       // bits in buf
  int real = 0;      // of those, bits that came from the data
  bool at_marker = false, overrun = false;

  void fill() {
    while (cnt <= 56) {
      uint64_t b = 0;
      if (!at_marker && pos < n) {
        if (p[pos] != 0xFF) {
          b = p[pos++];
          real += 8;
        } else if (pos + 1 < n && p[pos + 1] == 0x00) {
          b = 0xFF;  // a stuffed byte
          pos += 2;
          real += 8;
        } else {
          at_marker = true;  // pos stays on the 0xFF
        }
      }
      buf |= b << (56 - cnt);
      cnt += 8;
    }
  }
  void consume(int k) {
    buf <<= k;
    cnt -= k;
    if (k > real) overrun = true;
    real = k > real ? 0 : real - k;
  }
  uint32_t bits(int k) {  // 0 <= k <= 16
    if (k == 0) return 0;
    if (cnt < k) fill();
    const uint32_t v = (uint32_t)(buf >> (64 - k));
    consume(k);
    return v;
  }
  int decode(const Huffman &h) {
    if (cnt < 16) fill();
    const uint32_t look = (uint32_t)(buf >> (64 - kLook));
    if (h.look_len[look]) {
      const int len = h.look_len[look];
      consume(len);
      return h.look_sym[look];
    }
    for (int len = kLook + 1; len <= 16; ++len) {
      const int32_t code = (int32_t)(buf >> (64 - len));
      if (code <= h.maxcode[len]) {
        consume(len);
        return h.vals[h.valptr[len] + code - h.mincode[len]];
      }
    }
    return -1;
  }
  // drops the buffered bits (the rest of the last byte is padding) and
  // leaves pos on the next marker's 0xFF, or at the end
  void to_marker() {
    buf = 0;
    cnt = real = 0;
    at_marker = false;
    while (pos + 1 < n && !(p[pos] == 0xFF && p[pos + 1] != 0x00 && p[pos + 1] != 0xFF)) ++pos;
    if (pos + 1 >= n) pos = n;
  }
};

// the value of an s-bit magnitude v (T.81 F.2.2.1: EXTEND)
inline int32_t extend(uint32_t v, int s) {
  return s == 0 ? 0 : (v < (1u << (s - 1)) ? (int32_t)v - (1 << s) + 1 : (int32_t)v);
}

struct Component {
  int id = 0, h = 1, v = 1, tq = 0;
  int w = 0, ht = 0;        // samples of this component
  int pw = 0, ph = 0;       // plane size (whole MCUs)
  bool scanned = false;
  std::vector<uint8_t> plane;
};

struct Decoder {
  uint32_t width = 0, height = 0;
  int ncomp = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
  Component comp[3];
  uint16_t qt[4][64];  // zig-zag order
  bool qt_defined[4] = {false, false, false, false};
  Huffman dc[4], ac[4];
  uint32_t restart = 0;
  int orientation = 1;  // Exif orientation, 1..8
  bool have_frame = false, adobe_rgb = false, ids_rgb = false;

  // the size the image is delivered in: orientations 5..8 swap the axes
  uint32_t out_width() const { return orientation >= 5 ? height : width; }
  uint32_t out_height() const { return orientation >= 5 ? width : height; }

  // one 8 x 8 block: coefficients -> samples at (bx, by) of the plane.
  // Coefficients beyond row rmax or column cmax are zero and left out of
  // the sums (adding their zero products would not change them).
  static void idct_store(const int32_t *coef, bool ac_zero, int rmax, int cmax, uint8_t *dst,
                         int stride) {
    if (ac_zero) {  // constant block: F(0,0) * C(0)^2 / 4 = F(0,0) / 8
      const double val = std::floor(coef[0] / 8.0 + 128.0 + 0.5);
      const uint8_t s = (uint8_t)(val < 0 ? 0 : (val > 255 ? 255 : val));
      for (int y = 0; y < 8; ++y) std::memset(dst + (size_t)y * stride, s, 8);
      return;
    }
    // tmp[v][x] = sum_u F(v, u) c[x][u], rows of zeros skipped; then
    // s(y, x) = sum_v c[y][v] tmp[v][x].  Each sum runs in ascending u or
    // v; the eight columns x are the inner loop, so they vectorise.
    double tmp[8][8];
    bool nz[8];
    for (int v = 0; v <= rmax; ++v) {
      const int32_t *row = coef + v * 8;
      nz[v] = (row[0] | row[1] | row[2] | row[3] | row[4] | row[5] | row[6] | row[7]) != 0;
      if (!nz[v]) continue;
      double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int u = 0; u <= cmax; ++u) {
        const double f = (double)row[u];
        for (int x = 0; x < 8; ++x) acc[x] += kBasis.t[u][x] * f;
      }
      for (int x = 0; x < 8; ++x) tmp[v][x] = acc[x];
    }
    for (int y = 0; y < 8; ++y) {
      double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int v = 0; v <= rmax; ++v) {
        if (!nz[v]) continue;
        const double c = kBasis.c[y][v];
        for (int x = 0; x < 8; ++x) acc[x] += c * tmp[v][x];
      }
      uint8_t *out = dst + (size_t)y * stride;
      for (int x = 0; x < 8; ++x) {
        const double val = std::floor(acc[x] + 128.0 + 0.5);
        out[x] = (uint8_t)(val < 0 ? 0 : (val > 255 ? 255 : val));
      }
    }
  }

  static bool block(BitReader &br, const Huffman &hd, const Huffman &ha, const uint16_t *q,
                    int32_t &pred, uint8_t *dst, int stride) {
    int32_t coef[64];
    std::memset(coef, 0, sizeof(coef));
    const int t = br.decode(hd);
    if (t < 0 || t > 11) return false;
    pred += extend(br.bits(t), t);
    coef[0] = pred * (int32_t)q[0];
    bool ac_zero = true;
    int rmax = 0, cmax = 0;
    for (int k = 1; k < 64;) {
      const int rs = br.decode(ha);
      if (rs < 0) return false;
      const int r = rs >> 4, s = rs & 15;
      if (s == 0) {
        if (r != 15) break;  // end of block
        k += 16;             // sixteen zeros
        continue;
      }
      k += r;
      if (k > 63 || s > 10) return false;
      const int at = kZig.v[k];
      coef[at] = extend(br.bits(s), s) * (int32_t)q[k];
      rmax = (at >> 3) > rmax ? (at >> 3) : rmax;
      cmax = (at & 7) > cmax ? (at & 7) : cmax;
      ac_zero = false;
      ++k;
    }
    if (br.overrun) return false;
    idct_store(coef, ac_zero, rmax, cmax, dst, stride);
    return true;
  }

  vh_status frame(const uint8_t *d, size_t len, bool extended) {
    (void)extended;
    if (have_frame || len < 6) return VH_ERR_INVALID_ARG;
    const int precision = d[0];
    height = ((uint32_t)d[1] << 8) | d[2];
    width = ((uint32_t)d[3] << 8) | d[4];
    ncomp = d[5];
    if (precision != 8) return VH_ERR_UNSUPPORTED;
    if (height == 0) return VH_ERR_UNSUPPORTED;  // height given by a DNL marker
    if (width == 0 || width > 32768 || height > 32768 ||
        (uint64_t)width * height > ((uint64_t)1 << 26))
      return VH_ERR_INVALID_ARG;
    if (ncomp == 4) return VH_ERR_UNSUPPORTED;
    if ((ncomp != 1 && ncomp != 3) || len != 6 + 3 * (size_t)ncomp) return VH_ERR_INVALID_ARG;
    hmax = vmax = 1;
    for (int c = 0; c < ncomp; ++c) {
      Component &k = comp[c];
      k.id = d[6 + 3 * c];
      k.h = d[7 + 3 * c] >> 4;
      k.v = d[7 + 3 * c] & 15;
      k.tq = d[8 + 3 * c];
      if (k.h < 1 || k.h > 4 || k.v < 1 || k.v > 4 || k.tq > 3) return VH_ERR_INVALID_ARG;
      for (int o = 0; o < c; ++o)
        if (comp[o].id == k.id) return VH_ERR_INVALID_ARG;
      if (ncomp == 1) k.h = k.v = 1;  // one component: one block per MCU
      hmax = k.h > hmax ? k.h : hmax;
      vmax = k.v > vmax ? k.v : vmax;
    }
    for (int c = 0; c < ncomp; ++c)
      if (hmax % comp[c].h || vmax % comp[c].v) return VH_ERR_UNSUPPORTED;
    // component ids 'R', 'G', 'B' mark RGB samples (ids 1, 2, 3: YCbCr)
    ids_rgb = ncomp == 3 && comp[0].id == 'R' && comp[1].id == 'G' && comp[2].id == 'B';
    mcux = (int)((width + 8u * hmax - 1) / (8u * hmax));
    mcuy = (int)((height + 8u * vmax - 1) / (8u * vmax));
    for (int c = 0; c < ncomp; ++c) {
      Component &k = comp[c];
      k.w = (int)((width * (uint32_t)k.h + hmax - 1) / hmax);
      k.ht = (int)((height * (uint32_t)k.v + vmax - 1) / vmax);
      k.pw = mcux * k.h * 8;
      k.ph = mcuy * k.v * 8;
    }
    have_frame = true;
    return VH_OK;
  }

  vh_status tables_q(const uint8_t *d, size_t len) {
    size_t o = 0;
    while (o < len) {
      const int pq = d[o] >> 4, tq = d[o] & 15;
      if (pq > 1 || tq > 3) return VH_ERR_INVALID_ARG;
      const size_t need = 1 + 64 * (size_t)(pq + 1);
      if (len - o < need) return VH_ERR_INVALID_ARG;
      for (int k = 0; k < 64; ++k)
        qt[tq][k] = pq ? (uint16_t)((d[o + 1 + 2 * k] << 8) | d[o + 2 + 2 * k]) : d[o + 1 + k];
      qt_defined[tq] = true;
      o += need;
    }
    return VH_OK;
  }

  vh_status tables_h(const uint8_t *d, size_t len) {
    size_t o = 0;
    while (o < len) {
      if (len - o < 17) return VH_ERR_INVALID_ARG;
      const int tc = d[o] >> 4, th = d[o] & 15;
      if (tc > 1 || th > 3) return VH_ERR_INVALID_ARG;
      int total = 0;
      for (int i = 0; i < 16; ++i) total += d[o + 1 + i];
      if (total > 256 || len - o - 17 < (size_t)total) return VH_ERR_INVALID_ARG;
      Huffman &h = tc ? ac[th] : dc[th];
      if (!h.build(d + o + 1, d + o + 17, total)) return VH_ERR_INVALID_ARG;
      o += 17 + (size_t)total;
    }
    return VH_OK;
  }

  // one scan: header d[0..len), entropy data from `data`; on return *next
  // is the offset of the marker after the data
  vh_status scan(const uint8_t *d, size_t len, const uint8_t *data, size_t avail, size_t *next) {
    if (!have_frame || len < 1) return VH_ERR_INVALID_ARG;
    const int ns = d[0];
    if (ns < 1 || ns > ncomp || len != 4 + 2 * (size_t)ns) return VH_ERR_INVALID_ARG;
    int idx[3], td[3], ta[3], units = 0;
    for (int i = 0; i < ns; ++i) {
      const int cs = d[1 + 2 * i];
      idx[i] = -1;
      for (int c = 0; c < ncomp; ++c)
        if (comp[c].id == cs) idx[i] = c;
      if (idx[i] < 0) return VH_ERR_INVALID_ARG;
      for (int o = 0; o < i; ++o)
        if (idx[o] == idx[i]) return VH_ERR_INVALID_ARG;
      td[i] = d[2 + 2 * i] >> 4;
      ta[i] = d[2 + 2 * i] & 15;
      if (td[i] > 3 || ta[i] > 3 || !dc[td[i]].defined || !ac[ta[i]].defined ||
          !qt_defined[comp[idx[i]].tq])
        return VH_ERR_INVALID_ARG;
      units += comp[idx[i]].h * comp[idx[i]].v;
    }
    const int ss = d[1 + 2 * ns], se = d[2 + 2 * ns], ahl = d[3 + 2 * ns];
    if (ss != 0 || se != 63 || ahl != 0 || (ns > 1 && units > 10)) return VH_ERR_INVALID_ARG;
    for (int i = 0; i < ns; ++i) {
      Component &k = comp[idx[i]];
      if (k.plane.empty()) k.plane.assign((size_t)k.pw * (size_t)k.ph, 0);
      k.scanned = true;
    }
    // MCU grid: whole-image MCUs when interleaved, the component's own
    // blocks when it is alone in the scan
    const int bw = ns == 1 ? (comp[idx[0]].w + 7) / 8 : mcux;
    const int bh = ns == 1 ? (comp[idx[0]].ht + 7) / 8 : mcuy;
    const int64_t mcus = (int64_t)bw * bh;
    BitReader br;
    br.p = data;
    br.n = avail;
    int32_t pred[3] = {0, 0, 0};
    int expect_rst = 0;
    for (int64_t m = 0; m < mcus; ++m) {
      if (restart && m > 0 && m % restart == 0) {
        br.to_marker();
        if (br.pos + 1 >= br.n || br.p[br.pos + 1] != 0xD0 + expect_rst) return VH_ERR_INVALID_ARG;
        br.pos += 2;
        expect_rst = (expect_rst + 1) & 7;
        pred[0] = pred[1] = pred[2] = 0;
      }
      const int mx = (int)(m % bw), my = (int)(m / bw);
      for (int i = 0; i < ns; ++i) {
        Component &k = comp[idx[i]];
        const uint16_t *q = qt[k.tq];
        const int hs = ns == 1 ? 1 : k.h, vs = ns == 1 ? 1 : k.v;
        for (int v = 0; v < vs; ++v)
          for (int h = 0; h < hs; ++h) {
            const int bx = mx * hs + h, by = my * vs + v;
            uint8_t *dst = k.plane.data() + (size_t)by * 8 * k.pw + (size_t)bx * 8;
            if (!block(br, dc[td[i]], ac[ta[i]], q, pred[i], dst, k.pw)) return VH_ERR_INVALID_ARG;
          }
      }
    }
    br.to_marker();
    if (br.pos >= br.n) return VH_ERR_INVALID_ARG;  // no EOI or next segment
    *next = br.pos;
    return VH_OK;
  }

  // one output row of component c, at full resolution (cs: scratch of the
  // component's width)
  void upsample_row(const Component &k, uint32_t y, uint8_t *out, int32_t *cs) const {
    const int rx = hmax / k.h, ry = vmax / k.v;
    const uint8_t *pl = k.plane.data();
    const int cw = k.w, ch = k.ht;
    if (rx == 1 && ry == 1) {  // full resolution: the row itself
      std::memcpy(out, pl + (size_t)y * k.pw, width);
      return;
    }
    if ((rx != 1 && rx != 2) || (ry != 1 && ry != 2)) {  // replication
      const uint8_t *row = pl + (size_t)(y / ry < (uint32_t)ch ? y / ry : ch - 1) * k.pw;
      for (uint32_t x = 0; x < width; ++x) {
        const int sx = (int)(x / rx);
        out[x] = row[sx < cw ? sx : cw - 1];
      }
      return;
    }
    // rows: the nearer source row weighs 3, the farther 1 (ratio 2), or
    // one row weighing 4 (ratio 1); columns alike; 16 in all
    int r0, r1, w0, w1;
    if (ry == 1) {
      r0 = r1 = (int)y;
      w0 = 4;
      w1 = 0;
    } else {
      r0 = (int)(y >> 1);
      r1 = (y & 1) ? (r0 + 1 < ch ? r0 + 1 : ch - 1) : (r0 > 0 ? r0 - 1 : 0);
      w0 = 3;
      w1 = 1;
    }
    if (r0 >= ch) r0 = ch - 1;
    // the rows blended first (cs, weights summing to 4), then the columns
    // (weights 3 and 1, or 4): the same integer sums as weighting each
    // of the four samples by its product of weights
    const uint8_t *a = pl + (size_t)r0 * k.pw, *b = pl + (size_t)r1 * k.pw;
    for (int i = 0; i < cw; ++i) cs[i] = w0 * a[i] + w1 * b[i];
    if (rx == 1) {
      for (uint32_t x = 0; x < width; ++x) out[x] = (uint8_t)((4 * cs[x] + 8) >> 4);
      return;
    }
    for (int i = 0; i < cw; ++i) {  // output columns 2i and 2i + 1
      const int mid = 3 * cs[i];
      const int left = cs[i > 0 ? i - 1 : 0], right = cs[i + 1 < cw ? i + 1 : cw - 1];
      const uint32_t x = 2u * (uint32_t)i;
      out[x] = (uint8_t)((mid + left + 8) >> 4);
      if (x + 1 < width) out[x + 1] = (uint8_t)((mid + right + 8) >> 4);
    }
  }

  void write_rgb(uint8_t *rgb) const {
    std::vector<uint8_t> rows((size_t)width * 3);
    uint8_t *r[3] = {rows.data(), rows.data() + width, rows.data() + 2 * (size_t)width};
    std::vector<int32_t> cs((size_t)width + 1);
    double cr_r[256], cb_g[256], cr_g[256], cb_b[256];
    for (int i = 0; i < 256; ++i) {
      cr_r[i] = 1.402 * (i - 128);
      cb_g[i] = -0.34414 * (i - 128);
      cr_g[i] = -0.71414 * (i - 128);
      cb_b[i] = 1.772 * (i - 128);
    }
    auto level = [](double v) {
      const double f = std::floor(v + 0.5);
      return (uint8_t)(f < 0 ? 0 : (f > 255 ? 255 : f));
    };
    for (uint32_t y = 0; y < height; ++y) {
      for (int c = 0; c < ncomp; ++c) upsample_row(comp[c], y, r[c], cs.data());
      uint8_t *out = rgb + (size_t)y * width * 3;
      if (ncomp == 1) {
        for (uint32_t x = 0; x < width; ++x) out[3 * x] = out[3 * x + 1] = out[3 * x + 2] = r[0][x];
      } else if (adobe_rgb || ids_rgb) {
        for (uint32_t x = 0; x < width; ++x) {
          out[3 * x] = r[0][x];
          out[3 * x + 1] = r[1][x];
          out[3 * x + 2] = r[2][x];
        }
      } else {
        for (uint32_t x = 0; x < width; ++x) {
          const double yy = r[0][x];
          const uint8_t cb = r[1][x], cr = r[2][x];
          out[3 * x] = level(yy + cr_r[cr]);
          out[3 * x + 1] = level(yy + cb_g[cb] + cr_g[cr]);
          out[3 * x + 2] = level(yy + cb_b[cb]);
        }
      }
    }
  }
};

inline uint32_t be16(const uint8_t *p) { return ((uint32_t)p[0] << 8) | p[1]; }

// The Orientation tag (0x0112) of an Exif APP1 segment's first image file
// directory (TIFF layout, either byte order), 1 when absent or malformed.
int exif_orientation(const uint8_t *t, size_t n) {
  if (n < 8) return 1;
  const bool le = t[0] == 'I' && t[1] == 'I';
  if (!le && !(t[0] == 'M' && t[1] == 'M')) return 1;
  auto u16 = [&](size_t o) -> uint32_t {
    return le ? (uint32_t)t[o] | ((uint32_t)t[o + 1] << 8) : ((uint32_t)t[o] << 8) | t[o + 1];
  };
  auto u32 = [&](size_t o) -> uint32_t {
    return le ? u16(o) | (u16(o + 2) << 16) : (u16(o) << 16) | u16(o + 2);
  };
  if (u16(2) != 42) return 1;
  const size_t ifd = u32(4);
  if (ifd > n - 2) return 1;
  const size_t entries = u16(ifd);
  for (size_t k = 0; k < entries; ++k) {
    const size_t e = ifd + 2 + 12 * k;
    if (e + 12 > n) return 1;
    if (u16(e) == 0x0112 && u16(e + 2) == 3 && u32(e + 4) == 1) {  // one SHORT
      const uint32_t v = u16(e + 8);
      return v >= 1 && v <= 8 ? (int)v : 1;
    }
  }
  return 1;
}

}  // namespace

extern "C" vh_status vh_decode_colour_jpeg(const uint8_t *jpg, int64_t bytes, uint8_t *rgb,
                                           int64_t capacity, int32_t *width, int32_t *height) {
  if (!jpg || bytes < 4 || capacity < 0 || !width || !height) return VH_ERR_INVALID_ARG;
  if (jpg[0] != 0xFF || jpg[1] != 0xD8) return VH_ERR_INVALID_ARG;
  const size_t n = (size_t)bytes;
  Decoder dec;
  size_t pos = 2;
  bool have_end = false;
  while (pos < n) {
    if (jpg[pos] != 0xFF) return VH_ERR_INVALID_ARG;
    while (pos < n && jpg[pos] == 0xFF) ++pos;  // fill bytes before a marker
    if (pos >= n) return VH_ERR_INVALID_ARG;
    const uint8_t m = jpg[pos++];
    if (m == 0xD9) {
      have_end = true;
      break;
    }
    if (m == 0x01) continue;                                    // TEM: no segment
    if (m == 0x00 || m == 0xD8 || (m >= 0xD0 && m <= 0xD7)) return VH_ERR_INVALID_ARG;
    if (pos + 2 > n) return VH_ERR_INVALID_ARG;
    const size_t seg = be16(jpg + pos);
    if (seg < 2 || seg > n - pos) return VH_ERR_INVALID_ARG;
    const uint8_t *d = jpg + pos + 2;
    const size_t len = seg - 2;
    vh_status s = VH_OK;
    if (m == 0xC0 || m == 0xC1) {
      s = dec.frame(d, len, m == 0xC1);
      if (s == VH_OK && !rgb) {  // size query: the frame header is enough
        *width = (int32_t)dec.out_width();
        *height = (int32_t)dec.out_height();
        return VH_OK;
      }
      if (s == VH_OK && capacity < 3 * (int64_t)dec.width * (int64_t)dec.height) {
        *width = (int32_t)dec.out_width();
        *height = (int32_t)dec.out_height();
        return VH_ERR_CAPACITY;
      }
    } else if ((m >= 0xC2 && m <= 0xCF && m != 0xC4 && m != 0xC8) || m == 0xDC) {
      s = VH_ERR_UNSUPPORTED;  // progressive, lossless, arithmetic coding, DNL
    } else if (m == 0xC4) {
      s = dec.tables_h(d, len);
    } else if (m == 0xDB) {
      s = dec.tables_q(d, len);
    } else if (m == 0xDD) {
      if (len != 2) return VH_ERR_INVALID_ARG;
      dec.restart = be16(d);
    } else if (m == 0xE1 && !dec.have_frame && len >= 6 && std::memcmp(d, "Exif\0\0", 6) == 0) {
      dec.orientation = exif_orientation(d + 6, len - 6);  // only before the frame header
    } else if (m == 0xEE && len >= 12 && std::memcmp(d, "Adobe", 5) == 0) {
      dec.adobe_rgb = d[11] == 0;  // colour transform 0: the components are R, G, B
    } else if (m == 0xDA) {
      if (!rgb) return VH_ERR_INVALID_ARG;  // a scan before any frame header
      size_t next = 0;
      s = dec.scan(d, len, jpg + pos + seg, n - pos - seg, &next);
      if (s != VH_OK) return s;
      pos = pos + seg + next;
      continue;
    }
    if (s != VH_OK) return s;
    pos += seg;  // APPn, COM and other segments are skipped
  }
  if (!dec.have_frame) return VH_ERR_INVALID_ARG;
  if (!have_end) return VH_ERR_INVALID_ARG;
  for (int c = 0; c < dec.ncomp; ++c)
    if (!dec.comp[c].scanned) return VH_ERR_INVALID_ARG;
  *width = (int32_t)dec.out_width();
  *height = (int32_t)dec.out_height();
  if (dec.orientation == 1) {
    dec.write_rgb(rgb);
    return VH_OK;
  }
  // stored image -> displayed image: output pixel (ox, oy) takes stored
  // pixel (sx, sy) of the W x H image, per Exif orientation
  std::vector<uint8_t> stored((size_t)dec.width * dec.height * 3);
  dec.write_rgb(stored.data());
  const int64_t W = dec.width, H = dec.height, ow = dec.out_width(), oh = dec.out_height();
  for (int64_t oy = 0; oy < oh; ++oy)
    for (int64_t ox = 0; ox < ow; ++ox) {
      int64_t sx = ox, sy = oy;
      switch (dec.orientation) {
        case 2: sx = W - 1 - ox; break;                      // mirrored left-right
        case 3: sx = W - 1 - ox; sy = H - 1 - oy; break;     // rotated 180
        case 4: sy = H - 1 - oy; break;                      // mirrored top-bottom
        case 5: sx = oy; sy = ox; break;                     // transposed
        case 6: sx = oy; sy = H - 1 - ox; break;             // rotate 90 clockwise to show
        case 7: sx = W - 1 - oy; sy = H - 1 - ox; break;     // transversed
        case 8: sx = W - 1 - oy; sy = ox; break;             // rotate 90 anticlockwise to show
        default: break;
      }
      std::memcpy(rgb + (size_t)(oy * ow + ox) * 3, stored.data() + (size_t)(sy * W + sx) * 3, 3);
    }
  return VH_OK;
}

// vh_png.cpp - PNG frames for the integration inputs: grayscale depth images
// to uint16 (vh_decode_depth_png) and colour images to interleaved RGB u8
// (vh_decode_colour_png).
//
// The reference loads each depth frame with cv::imread(path, -1), a 16-bit
// grayscale PNG of millimetres, and converts it to float metres
// (src/SaveFrame.cpp:174-180).  Here the PNG is decoded into the uint16
// millimetre image that vh_integrate takes as VH_DEPTH_U16_MM, so the scale
// to metres happens inside the allocation kernel and the host never holds a
// float copy.  Its colour frames go through cv::imread(path, IMREAD_COLOR)
// and a BGR-to-RGB swap (src/SaveFrame.cpp:164, src/main.cpp:273); the
// colour decoder gives the RGB bytes directly.  The decoder follows the PNG specification (chunk layout,
// CRC-32, filter types 0-4 with the Paeth predictor) and RFC 1950/1951
// (zlib wrapper with Adler-32, DEFLATE stored / fixed / dynamic Huffman
// blocks); every read is bounds-checked and the output size is fixed by the
// header before anything is inflated.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/vhsdf.h"

namespace {

// ---- CRC-32 (PNG chunks) and Adler-32 (zlib stream) ----------------------
// v[0] is the byte-at-a-time table of the reflected polynomial 0xEDB88320;
// v[k][i] is the CRC of byte i followed by k zero bytes, which lets eight
// bytes be folded in per step (slicing-by-8, Kounavis and Berry 2005).
struct CrcTable {
  uint32_t v[8][256];
  CrcTable() {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      v[0][i] = c;
    }
    for (int k = 1; k < 8; ++k)
      for (int i = 0; i < 256; ++i) v[k][i] = (v[k - 1][i] >> 8) ^ v[0][v[k - 1][i] & 0xFFu];
  }
};

inline uint32_t le32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

uint32_t crc32_of(const uint8_t *p, size_t n) {
  static const CrcTable t;  // built once, thread-safe
  uint32_t c = 0xFFFFFFFFu;
  for (; n >= 8; p += 8, n -= 8) {
    const uint32_t lo = c ^ le32(p), hi = le32(p + 4);
    c = t.v[7][lo & 0xFFu] ^ t.v[6][(lo >> 8) & 0xFFu] ^ t.v[5][(lo >> 16) & 0xFFu] ^
        t.v[4][lo >> 24] ^ t.v[3][hi & 0xFFu] ^ t.v[2][(hi >> 8) & 0xFFu] ^
        t.v[1][(hi >> 16) & 0xFFu] ^ t.v[0][hi >> 24];
  }
  for (; n; ++p, --n) c = t.v[0][(c ^ *p) & 0xFFu] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

uint32_t adler32_of(const uint8_t *p, size_t n) {
  uint32_t a = 1, b = 0;
  while (n) {  // 5552 bytes keep b below 2^32 before the reduction
    const size_t k = n < 5552 ? n : 5552;
    for (size_t i = 0; i < k; ++i) {
      a += p[i];
      b += a;
    }
    a %= 65521u;
    b %= 65521u;
    p += k;
    n -= k;
  }
  return (b << 16) | a;
}

uint32_t be32(const uint8_t *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

// ---- DEFLATE (RFC 1951) ---------------------------------------------------
// Bits least significant first, through a 64-bit buffer; reading past the
// end pads with zeros and marks the reader bad.
struct BitReader {
  const uint8_t *p;
  size_t n;
  size_t pos = 0;         // next byte to load
  uint64_t buf = 0;       // loaded, unconsumed bits
  int cnt = 0;            // bits in buf
  uint64_t consumed = 0;  // bits consumed from the start
  bool bad = false;
  void refill() {
    while (cnt <= 56) {
      if (pos < n) buf |= (uint64_t)p[pos] << cnt;
      ++pos;  // past the end: zeros, caught by the consumed count
      cnt += 8;
    }
  }
  uint32_t peek(int count) {  // count <= 32
    refill();
    return (uint32_t)(buf & ((1ull << count) - 1ull));
  }
  void drop(int count) {
    buf >>= count;
    cnt -= count;
    consumed += (uint64_t)count;
    if (consumed > 8ull * n) bad = true;
  }
  int get(int count) {  // count <= 32
    if (count == 0) return 0;
    const uint32_t v = peek(count);
    drop(count);
    return (int)v;
  }
  void align() {
    const int r = (int)(consumed & 7u);
    if (r) drop(8 - r);
  }
  // `len` whole bytes at a byte boundary, copied straight from the input
  bool copy_bytes(size_t len, std::vector<uint8_t> &out) {
    const size_t at = (size_t)(consumed >> 3);
    if ((consumed & 7u) || at > n || len > n - at) return false;
    out.insert(out.end(), p + at, p + at + len);
    consumed += 8ull * len;
    pos = at + len;  // reload from here: the buffered bits are past it
    buf = 0;
    cnt = 0;
    return true;
  }
};

// Canonical Huffman code from code lengths: a table indexed by the next
// kFastBits input bits for the codes that short, and the count of codes per
// length with the symbols ordered by (length, symbol) for the longer ones.
constexpr int kFastBits = 9;
struct Huffman {
  uint16_t count[16] = {};
  std::vector<uint16_t> symbol;
  uint16_t fast[1 << kFastBits] = {};  // symbol << 4 | length, 0 = longer code
  // false for an over-subscribed set of lengths
  bool build(const uint8_t *len, int n) {
    std::memset(count, 0, sizeof(count));
    std::memset(fast, 0, sizeof(fast));
    for (int s = 0; s < n; ++s) count[len[s]]++;
    count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
      left <<= 1;
      left -= count[l];
      if (left < 0) return false;
    }
    uint16_t offs[16] = {};
    for (int l = 1; l < 15; ++l) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
    symbol.assign((size_t)n, 0);
    for (int s = 0; s < n; ++s)
      if (len[s]) symbol[offs[len[s]]++] = (uint16_t)s;
    // canonical codes (RFC 1951 3.2.2), stored most significant bit first in
    // the stream: the table index is the code's bits reversed
    uint32_t next[16] = {};
    uint32_t code = 0;
    for (int l = 1; l < 16; ++l) {
      code = (code + count[l - 1]) << 1;
      next[l] = code;
    }
    for (int s = 0; s < n; ++s) {
      const int l = len[s];
      if (!l) continue;
      const uint32_t c = next[l]++;
      if (l > kFastBits) continue;
      uint32_t rev = 0;
      for (int i = 0; i < l; ++i) rev |= ((c >> i) & 1u) << (l - 1 - i);
      for (uint32_t k = rev; k < (1u << kFastBits); k += 1u << l)
        fast[k] = (uint16_t)((s << 4) | l);
    }
    return true;
  }
  // one symbol, or -1 when the input ends or matches no code
  int decode(BitReader &br) const {
    const uint16_t e = fast[br.peek(kFastBits)];
    if (e) {
      br.drop(e & 15);
      return br.bad ? -1 : (int)(e >> 4);
    }
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= br.get(1);
      if (br.bad) return -1;
      const int c = count[l];
      if (code - first < c) return symbol[(size_t)(index + code - first)];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    return -1;
  }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                               2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,    2,    3,    4,    5,    7,     9,     13,    17,  25,
                                33,   49,   65,   97,   129,  193,   257,   385,   513, 769,
                                1025, 1537, 2049, 3073, 4097, 6145,  8193,  12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

// Inflates a raw DEFLATE stream into out, which must end up exactly `want`
// bytes long (more output is an error: the size comes from the PNG header).
bool inflate(BitReader &br, std::vector<uint8_t> &out, size_t want) {
  out.clear();
  out.reserve(want < ((size_t)1 << 26) ? want : ((size_t)1 << 26));
  Huffman fixed_lit, fixed_dist;
  {
    uint8_t l[288];
    for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8));
    fixed_lit.build(l, 288);
    uint8_t d[30];
    for (int s = 0; s < 30; ++s) d[s] = 5;
    fixed_dist.build(d, 30);
  }
  for (;;) {
    const int last = br.get(1);
    const int type = br.get(2);
    if (br.bad) return false;
    if (type == 0) {  // stored: byte-aligned LEN, ~LEN, then LEN raw bytes
      br.align();
      const uint32_t len = (uint32_t)br.get(16), nlen = (uint32_t)br.get(16);
      if (br.bad || (len ^ 0xFFFFu) != nlen || out.size() + len > want) return false;
      if (!br.copy_bytes(len, out)) return false;
    } else if (type == 1 || type == 2) {
      Huffman dyn_lit, dyn_dist;
      const Huffman *lit = &fixed_lit, *dist = &fixed_dist;
      if (type == 2) {
        const int hlit = br.get(5) + 257, hdist = br.get(5) + 1, hclen = br.get(4) + 4;
        static const uint8_t order[19] = {16, 17, 18, 0, 8,  7, 9,  6, 10, 5,
                                          11, 4,  12, 3, 13, 2, 14, 1, 15};
        uint8_t cl[19] = {};
        for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)br.get(3);
        if (br.bad || hlit > 286 || hdist > 30) return false;
        Huffman clh;
        if (!clh.build(cl, 19)) return false;
        uint8_t lens[286 + 30] = {};
        int k = 0;
        while (k < hlit + hdist) {
          const int sym = clh.decode(br);
          if (sym < 0) return false;
          if (sym < 16) {
            lens[k++] = (uint8_t)sym;
            continue;
          }
          int rep = 0;
          uint8_t val = 0;
          if (sym == 16) {
            if (k == 0) return false;
            val = lens[k - 1];
            rep = 3 + br.get(2);
          } else if (sym == 17) {
            rep = 3 + br.get(3);
          } else {
            rep = 11 + br.get(7);
          }
          if (br.bad || k + rep > hlit + hdist) return false;
          while (rep--) lens[k++] = val;
        }
        if (lens[256] == 0) return false;  // no end-of-block code
        if (!dyn_lit.build(lens, hlit) || !dyn_dist.build(lens + hlit, hdist)) return false;
        lit = &dyn_lit;
        dist = &dyn_dist;
      }
      for (;;) {
        const int sym = lit->decode(br);
        if (sym < 0) return false;
        if (sym < 256) {
          if (out.size() >= want) return false;
          out.push_back((uint8_t)sym);
        } else if (sym == 256) {
          break;
        } else {
          const int li = sym - 257;
          if (li >= 29) return false;
          const size_t len = kLenBase[li] + (size_t)br.get(kLenExtra[li]);
          const int di = dist->decode(br);
          if (di < 0 || di >= 30) return false;
          const size_t d = kDistBase[di] + (size_t)br.get(kDistExtra[di]);
          if (br.bad || d > out.size() || out.size() + len > want) return false;
          const size_t from = out.size() - d;
          for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);  // may overlap
        }
      }
    } else {
      return false;
    }
    if (last) return out.size() == want;
  }
}

// The Paeth predictor: of a (left), b (above) and c (above-left), the one
// nearest to a + b - c, ties in the order a, b, c.  With p = a + b - c the
// distances are |p - a| = |b - c|, |p - b| = |a - c|, |p - c| = |a + b - 2c|.
inline int paeth(int a, int b, int c) {
  const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
  const int ab = pb < pa ? b : a, dab = pb < pa ? pb : pa;
  return pc < dab ? c : ab;
}

// Undoes one row's PNG filter in place: cur holds the filtered bytes, up the
// previous row's unfiltered bytes (zeros above the first row), k the bytes
// per pixel (a: the byte k to the left, b: above, c: above-left).
bool unfilter_row(uint8_t *cur, const uint8_t *up, size_t stride, size_t k, int ft) {
  switch (ft) {
    case 0:
      return true;
    case 1:
      for (size_t i = k; i < stride; ++i) cur[i] = (uint8_t)(cur[i] + cur[i - k]);
      return true;
    case 2:
      for (size_t i = 0; i < stride; ++i) cur[i] = (uint8_t)(cur[i] + up[i]);
      return true;
    case 3:
      for (size_t i = 0; i < stride; ++i)
        cur[i] = (uint8_t)(cur[i] + (((i >= k ? cur[i - k] : 0) + up[i]) >> 1));
      return true;
    case 4:
      for (size_t i = 0; i < stride; ++i)
        cur[i] = (uint8_t)(cur[i] + paeth(i >= k ? cur[i - k] : 0, up[i], i >= k ? up[i - k] : 0));
      return true;
    default:
      return false;
  }
}

// One decoded PNG: rows of `stride` unfiltered bytes, each after its filter
// byte at raw[y * (stride + 1) + 1]; samples big-endian as in the file.
struct PngImage {
  uint32_t w = 0, h = 0;
  int depth = 0, channels = 0;
  size_t stride = 0;
  std::vector<uint8_t> raw;
  const uint8_t *row(uint32_t y) const { return raw.data() + (size_t)y * (stride + 1) + 1; }
};

// Channels of a PNG colour type that the decoder reads (grayscale, RGB,
// grayscale + alpha, RGBA), 0 for the palette type and unknown ones.
int png_channels(int colour) {
  switch (colour) {
    case 0: return 1;
    case 2: return 3;
    case 4: return 2;
    case 6: return 4;
    default: return 0;
  }
}

// Parses the chunks, checks every CRC, and (pixels == true) inflates and
// unfilters the image data.  `gray_only` admits colour type 0 alone.  Only
// 8- and 16-bit samples, without interlacing, are read.  With pixels ==
// false it returns after IHDR, having filled w, h, depth and channels.
vh_status png_decode(const uint8_t *png, int64_t bytes, bool gray_only, bool pixels,
                     PngImage &img) {
  static const uint8_t kSig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  if (!png || bytes < 8) return VH_ERR_INVALID_ARG;
  if (std::memcmp(png, kSig, 8) != 0) return VH_ERR_INVALID_ARG;
  const size_t n = (size_t)bytes;
  size_t pos = 8;
  bool have_header = false, have_end = false;
  std::vector<uint8_t> idat;
  while (pos + 12 <= n) {
    const uint32_t len = be32(png + pos);
    if (len > n - pos - 12) return VH_ERR_INVALID_ARG;
    const uint8_t *type = png + pos + 4, *data = png + pos + 8;
    if (crc32_of(type, (size_t)len + 4) != be32(data + len)) return VH_ERR_INVALID_ARG;
    if (std::memcmp(type, "IHDR", 4) == 0) {
      if (len != 13 || have_header) return VH_ERR_INVALID_ARG;
      img.w = be32(data);
      img.h = be32(data + 4);
      img.depth = data[8];
      const int colour = data[9], compression = data[10], filter = data[11], interlace = data[12];
      if (img.w == 0 || img.h == 0 || img.w > 32768 || img.h > 32768 ||
          (uint64_t)img.w * img.h > ((uint64_t)1 << 26))
        return VH_ERR_INVALID_ARG;
      img.channels = png_channels(colour);
      if (img.channels == 0 || (gray_only && colour != 0) || (img.depth != 8 && img.depth != 16) ||
          compression != 0 || filter != 0 || interlace != 0)
        return VH_ERR_UNSUPPORTED;
      img.stride = (size_t)img.w * (size_t)(img.channels * img.depth / 8);
      have_header = true;
      if (!pixels) return VH_OK;  // size query: the header is enough
    } else if (std::memcmp(type, "IDAT", 4) == 0) {
      if (!have_header) return VH_ERR_INVALID_ARG;
      idat.insert(idat.end(), data, data + len);
    } else if (std::memcmp(type, "IEND", 4) == 0) {
      have_end = true;
      break;
    } else if (!(type[0] & 0x20)) {  // an unknown critical chunk
      return VH_ERR_UNSUPPORTED;
    }
    pos += (size_t)len + 12;
  }
  if (!have_header || !have_end || idat.size() < 6) return VH_ERR_INVALID_ARG;
  // zlib wrapper: CM 8 with a window of at most 32 KiB, no preset dictionary
  const uint8_t cmf = idat[0], flg = idat[1];
  if ((cmf & 0x0F) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20))
    return VH_ERR_INVALID_ARG;
  BitReader br{idat.data() + 2, idat.size() - 6};  // between the zlib header and Adler-32
  if (!inflate(br, img.raw, (size_t)img.h * (img.stride + 1))) return VH_ERR_INVALID_ARG;
  if (adler32_of(img.raw.data(), img.raw.size()) != be32(idat.data() + idat.size() - 4))
    return VH_ERR_INVALID_ARG;
  const std::vector<uint8_t> zeros(img.stride, 0);
  const size_t k = (size_t)(img.channels * img.depth / 8);
  for (uint32_t y = 0; y < img.h; ++y) {
    uint8_t *filt = img.raw.data() + (size_t)y * (img.stride + 1);
    const uint8_t *up = y ? filt - img.stride : zeros.data();
    if (!unfilter_row(filt + 1, up, img.stride, k, filt[0])) return VH_ERR_INVALID_ARG;
  }
  return VH_OK;
}

}  // namespace

extern "C" vh_status vh_decode_depth_png(const uint8_t *png, int64_t bytes, uint16_t *out,
                                         int64_t capacity, int32_t *width, int32_t *height) {
  if (capacity < 0 || !width || !height) return VH_ERR_INVALID_ARG;
  PngImage img;
  vh_status s = png_decode(png, bytes, true, false, img);
  if (s != VH_OK) return s;
  if (out && capacity < (int64_t)img.w * (int64_t)img.h) {
    *width = (int32_t)img.w;  // the size is reported with the capacity error
    *height = (int32_t)img.h;
    return VH_ERR_CAPACITY;
  }
  if (out && (s = png_decode(png, bytes, true, true, img)) != VH_OK) return s;
  *width = (int32_t)img.w;
  *height = (int32_t)img.h;
  if (!out) return VH_OK;
  for (uint32_t y = 0; y < img.h; ++y) {  // big-endian samples to native uint16
    const uint8_t *src = img.row(y);
    uint16_t *dst = out + (size_t)y * img.w;
    if (img.depth == 16)
      for (uint32_t x = 0; x < img.w; ++x)
        dst[x] = (uint16_t)(((uint32_t)src[2 * x] << 8) | src[2 * x + 1]);
    else
      for (uint32_t x = 0; x < img.w; ++x) dst[x] = src[x];
  }
  return VH_OK;
}

extern "C" vh_status vh_decode_colour_png(const uint8_t *png, int64_t bytes, uint8_t *rgb,
                                          int64_t capacity, int32_t *width, int32_t *height) {
  if (capacity < 0 || !width || !height) return VH_ERR_INVALID_ARG;
  PngImage img;
  vh_status s = png_decode(png, bytes, false, false, img);
  if (s != VH_OK) return s;
  if (rgb && capacity < 3 * (int64_t)img.w * (int64_t)img.h) {
    *width = (int32_t)img.w;
    *height = (int32_t)img.h;
    return VH_ERR_CAPACITY;
  }
  if (rgb && (s = png_decode(png, bytes, false, true, img)) != VH_OK) return s;
  *width = (int32_t)img.w;
  *height = (int32_t)img.h;
  if (!rgb) return VH_OK;
  // 16-bit samples keep their high byte; grayscale is repeated into R, G and
  // B; alpha is dropped
  const int step = img.depth / 8, px = img.channels * step;
  const int c1 = img.channels >= 3 ? step : 0, c2 = img.channels >= 3 ? 2 * step : 0;
  for (uint32_t y = 0; y < img.h; ++y) {
    const uint8_t *src = img.row(y);
    uint8_t *dst = rgb + (size_t)y * img.w * 3;
    for (uint32_t x = 0; x < img.w; ++x, src += px, dst += 3) {
      dst[0] = src[0];
      dst[1] = src[c1];
      dst[2] = src[c2];
    }
  }
  return VH_OK;
}

// vh_oracle.cpp - CPU oracle of the voxel-hashing TSDF path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
// smoke check and the CPU-baseline leg of the benchmark call it; the product
// library never links, loads or calls it.
//
// It restates, in plain C++, the per-frame algorithm of the reference
// (E-BAO/Voxel-Hashing-SDF, src/tsdf.cu and include/tsdf.cuh):
//   * camera math        frame2cam / cam2frame / base2cam / cam2base
//                        (src/tsdf.cu:67-106)
//   * voxel centres      voxel2world, index * voxel_size, no +0.5
//                        (src/tsdf.cu:24-30, 621-623)
//   * integration        the tests and running average of IntegrateHashKernel
//                        (src/tsdf.cu:706-745)
//   * marching cubes     corner order idxMap (include/tsdf.cuh:234-241),
//                        edgeTable/triTable (include/tsdf.cuh:243-534),
//                        "every corner block must exist" (src/tsdf.cu:930-969),
//                        cubeIndex (src/tsdf.cu:978-986), VertexInterp
//                        (src/tsdf.cu:1640-1660), degenerate-triangle rule
//                        (src/tsdf.cu:1055-1057)
// and the block allocation of the engine's canonical mode: every pixel's
// truncation band [d - T, d + T] walked block by block.  The reference walks
// whole subsampled rays instead (HashAssignKernel, src/tsdf.cu:2088-2238);
// its integration and MC rules are unchanged by that choice.
//
// Precision: every decision that selects a pixel, a block, a cube case or a
// degenerate triangle is computed in IEEE fp32 in the reference's operation
// order (build with -ffp-contract=off so no FMA is formed).  The accumulated
// sdf / weight / colour use Acc = float (bit-exact mode) or double (FP64
// mode); MC vertices are produced in fp32 and, in parallel, in fp64 from
// the same fp32 voxel values.
//
// Deliberate differences from the reference, shared with the GPU engine:
//   * sdf running average uses the old weight: (sdf*w_old + dist)/w_new.
//     The reference multiplies by the already-incremented weight
//     (src/tsdf.cu:739-742); colour already uses w_old there (:743-745).
//   * a NaN depth is invalid (the reference's `d <= 0 || d > max` test lets
//     NaN through, src/tsdf.cu:716).
//   * MC may also require every corner weight >= mc_min_weight (0 keeps the
//     reference rule).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kB = 8;
constexpr int kB3 = kB * kB * kB;
constexpr int kBias = 1 << 20;

struct OParams {
  int32_t width, height;
  float fx, fy, cx, cy;
  float min_depth, max_depth;
  float voxel_size, trunc, mc_min_weight;
};

inline uint64_t okey(int x, int y, int z) {
  return (uint64_t)(uint32_t)(x + kBias) | ((uint64_t)(uint32_t)(y + kBias) << 21) |
         ((uint64_t)(uint32_t)(z + kBias) << 42);
}
inline void ounkey(uint64_t k, int &x, int &y, int &z) {
  x = (int)(k & 0x1FFFFF) - kBias;
  y = (int)((k >> 21) & 0x1FFFFF) - kBias;
  z = (int)((k >> 42) & 0x1FFFFF) - kBias;
}

// ---- camera (src/tsdf.cu:67-106) -----------------------------------------
// frame2cam (src/tsdf.cu:67-74): ((u - cx) * z) / fx
inline void frame2cam(int u, int v, float z, const OParams &p, float cam[3]) {
  cam[2] = z;
  cam[0] = (((float)u - p.cx) * z) / p.fx;
  cam[1] = (((float)v - p.cy) * z) / p.fy;
}
// cam2base (src/tsdf.cu:95-106): ((c0*R0 + c1*R1) + c2*R2) + t
inline void cam2base(const float cam[3], const float *c2w, float w[3]) {
  for (int r = 0; r < 3; ++r) {
    float a = cam[0] * c2w[r * 4 + 0];
    a = a + cam[1] * c2w[r * 4 + 1];
    a = a + cam[2] * c2w[r * 4 + 2];
    w[r] = a + c2w[r * 4 + 3];
  }
}
// base2cam (src/tsdf.cu:81-93): tmp = p - t; cam_c = ((R0c*t0 + R1c*t1) + R2c*t2)
inline void base2cam(const float pw[3], const float *c2w, float cam[3]) {
  float t0 = pw[0] - c2w[3], t1 = pw[1] - c2w[7], t2 = pw[2] - c2w[11];
  for (int c = 0; c < 3; ++c) {
    float a = c2w[0 * 4 + c] * t0;
    a = a + c2w[1 * 4 + c] * t1;
    a = a + c2w[2 * 4 + c] * t2;
    cam[c] = a;
  }
}

// ---- canonical band allocation --------------------------------------------
// Continuous block coordinate of a world point: ((p / V) + 0.5) / 8, so that
// block b holds the voxel centres 8b .. 8b+7 (centre of voxel i is i*V).
constexpr float kGridLimit = 1048000.0f;  // |g| bound keeping keys in range

struct Dda {
  int c[3], e[3], step[3], rem[3];
  float tmax[3], tdelta[3];
};

// Starts a 6-connected block walk from gA to gB. Returns false if out of range.
inline bool dda_begin(const float ga[3], const float gb[3], Dda &s) {
  for (int a = 0; a < 3; ++a) {
    if (!(std::fabs(ga[a]) < kGridLimit) || !(std::fabs(gb[a]) < kGridLimit)) return false;
  }
  for (int a = 0; a < 3; ++a) {
    s.c[a] = (int)std::floor(ga[a]);
    s.e[a] = (int)std::floor(gb[a]);
    float dir = gb[a] - ga[a];
    if (s.e[a] > s.c[a]) {
      s.step[a] = 1;
      s.rem[a] = s.e[a] - s.c[a];
      s.tdelta[a] = 1.0f / dir;
      s.tmax[a] = ((float)(s.c[a] + 1) - ga[a]) / dir;
    } else if (s.e[a] < s.c[a]) {
      s.step[a] = -1;
      s.rem[a] = s.c[a] - s.e[a];
      float nd = -dir;
      s.tdelta[a] = 1.0f / nd;
      s.tmax[a] = (ga[a] - (float)s.c[a]) / nd;
    } else {
      s.step[a] = 0;
      s.rem[a] = 0;
      s.tdelta[a] = 0.0f;
      s.tmax[a] = 0.0f;
    }
  }
  return true;
}
// Advances to the next cell: the axis with the smallest tmax among axes that
// still have cells to cross (ties: x, then y, then z). Returns false at end.
inline bool dda_next(Dda &s) {
  int best = -1;
  for (int a = 0; a < 3; ++a) {
    if (s.rem[a] == 0) continue;
    if (best < 0 || s.tmax[a] < s.tmax[best]) best = a;
  }
  if (best < 0) return false;
  s.c[best] += s.step[best];
  s.rem[best] -= 1;
  s.tmax[best] = s.tmax[best] + s.tdelta[best];
  return true;
}

inline void world_to_grid(const float w[3], float voxel, float g[3]) {
  for (int a = 0; a < 3; ++a) {
    float q = w[a] / voxel;
    q = q + 0.5f;
    g[a] = q * 0.125f;
  }
}

// Appends the band blocks of pixel (u, v) with depth d. Returns false when a
// block coordinate leaves the key range.
inline bool band_blocks(int u, int v, float d, const OParams &p, const float *c2w,
                        std::vector<uint64_t> &out) {
  if (!(d > 0.0f && d <= p.max_depth)) return true;
  float z0 = d - p.trunc;
  if (z0 < p.min_depth) z0 = p.min_depth;
  float z1 = d + p.trunc;
  if (!(z1 > z0)) return true;
  float ca[3], cb[3], wa[3], wb[3], ga[3], gb[3];
  frame2cam(u, v, z0, p, ca);
  frame2cam(u, v, z1, p, cb);
  cam2base(ca, c2w, wa);
  cam2base(cb, c2w, wb);
  world_to_grid(wa, p.voxel_size, ga);
  world_to_grid(wb, p.voxel_size, gb);
  Dda s;
  if (!dda_begin(ga, gb, s)) return false;
  do {
    out.push_back(okey(s.c[0], s.c[1], s.c[2]));
  } while (dda_next(s));
  return true;
}

// ---- volume ----------------------------------------------------------------
template <typename Acc>
struct Block {
  Acc sdf[kB3];
  Acc w[kB3];
  uint8_t rgb[kB3 * 3];
};

struct Tables {
  int idx[8][3];
  int edge[256];
  int tri[256][16];
};

template <typename Acc>
struct Volume {
  OParams p;
  Tables t;
  std::unordered_map<uint64_t, int32_t> index;
  std::vector<uint64_t> keys;
  std::vector<Block<Acc>> blocks;
  std::vector<int32_t> frame;  // block indices of the last frame, key-sorted
  int64_t last_new = 0;
  int64_t last_updated = 0;

  int32_t get_or_add(uint64_t k, bool *created) {
    auto it = index.find(k);
    if (it != index.end()) {
      *created = false;
      return it->second;
    }
    int32_t id = (int32_t)blocks.size();
    blocks.emplace_back();
    Block<Acc> &b = blocks.back();
    std::memset(&b, 0, sizeof(b));
    keys.push_back(k);
    index.emplace(k, id);
    *created = true;
    return id;
  }
  int32_t find(uint64_t k) const {
    auto it = index.find(k);
    return it == index.end() ? -1 : it->second;
  }
};

// Integration of one voxel (src/tsdf.cu:690-745 with the w_old fix).
template <typename Acc>
inline bool integrate_voxel(const OParams &p, const float *c2w, const float *depth,
                            const uint8_t *rgb, int ix, int iy, int iz, Acc &sdf, Acc &w,
                            uint8_t *col) {
  float pw[3] = {(float)ix * p.voxel_size, (float)iy * p.voxel_size, (float)iz * p.voxel_size};
  float cam[3];
  base2cam(pw, c2w, cam);
  if (!(cam[2] > 0.0f)) return false;  // src/tsdf.cu:706-707
  // cam2frame (src/tsdf.cu:75-79)
  float uf = std::round(p.fx * (cam[0] / cam[2]) + p.cx);
  float vf = std::round(p.fy * (cam[1] / cam[2]) + p.cy);
  if (!(uf >= 0.0f && uf < (float)p.width && vf >= 0.0f && vf < (float)p.height))
    return false;  // src/tsdf.cu:710-711
  int pix = (int)vf * p.width + (int)uf;
  float d = depth[pix];
  if (!(d > 0.0f && d <= p.max_depth)) return false;  // src/tsdf.cu:715-716
  float diff = d - cam[2];
  if (diff <= -p.trunc) return false;  // src/tsdf.cu:720-721
  float dist = std::fmin(1.0f, diff / p.trunc);  // src/tsdf.cu:737
  Acc w_old = w;
  Acc w_new = w_old + (Acc)1;
  sdf = (sdf * w_old + (Acc)dist) / w_new;
  for (int c = 0; c < 3; ++c) {
    Acc v = ((Acc)col[c] * w_old + (Acc)rgb[3 * pix + c]) / w_new;
    col[c] = (uint8_t)v;  // truncation, as the float-to-uchar store
  }
  w = w_new;
  return true;
}

// VertexInterp (src/tsdf.cu:1640-1660), fp32.  fabs(v) < 0.00001 compares a
// float against a double literal; the fp32 test below is the same predicate.
struct V32 {
  float x, y, z;
  uint8_t r, g, b;
};
struct V64 {
  double x, y, z;
};

inline bool snap(float a) { return (double)std::fabs(a) < 0.00001; }

inline void vinterp(const V32 &p1, const V32 &p2, float v1, float v2, V32 &o, V64 &o64) {
  if (snap(0.0f - v1)) {
    o = p1;
    o64 = {p1.x, p1.y, p1.z};
    return;
  }
  if (snap(0.0f - v2)) {
    o = p2;
    o64 = {p2.x, p2.y, p2.z};
    return;
  }
  if (snap(v1 - v2)) {
    o = p1;
    o64 = {p1.x, p1.y, p1.z};
    return;
  }
  float mu = (0.0f - v1) / (v2 - v1);
  o.x = p1.x + mu * (p2.x - p1.x);
  o.y = p1.y + mu * (p2.y - p1.y);
  o.z = p1.z + mu * (p2.z - p1.z);
  o.r = (uint8_t)((float)p1.r + mu * (float)((int)p2.r - (int)p1.r));
  o.g = (uint8_t)((float)p1.g + mu * (float)((int)p2.g - (int)p1.g));
  o.b = (uint8_t)((float)p1.b + mu * (float)((int)p2.b - (int)p1.b));
  double mu64 = (0.0 - (double)v1) / ((double)v2 - (double)v1);
  o64.x = (double)p1.x + mu64 * ((double)p2.x - (double)p1.x);
  o64.y = (double)p1.y + mu64 * ((double)p2.y - (double)p1.y);
  o64.z = (double)p1.z + mu64 * ((double)p2.z - (double)p1.z);
}

inline bool veq(const V32 &a, const V32 &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

static const int kEdgeCorners[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                        {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

struct Tri {
  float xyz[9];
  uint8_t rgb[9];
  double xyz64[9];
  int32_t cube[4];  // voxel x, y, z and triangle index within the cube
};

// Marching cubes of one block (src/tsdf.cu:884-1061).
template <typename Acc>
void mc_block(const Volume<Acc> &V, int32_t bid, std::vector<Tri> &out) {
  int bx, by, bz;
  ounkey(V.keys[bid], bx, by, bz);
  const Block<Acc> *nb[8];
  for (int n = 0; n < 8; ++n) {
    int32_t id = V.find(okey(bx + (n & 1), by + ((n >> 1) & 1), bz + ((n >> 2) & 1)));
    nb[n] = id < 0 ? nullptr : &V.blocks[id];
  }
  const float minw = V.p.mc_min_weight;
  for (int z = 0; z < kB; ++z)
    for (int y = 0; y < kB; ++y)
      for (int x = 0; x < kB; ++x) {
        float val[8];
        V32 pt[8];
        bool ok = true;
        for (int k = 0; k < 8 && ok; ++k) {
          int cx = x + V.t.idx[k][0], cy = y + V.t.idx[k][1], cz = z + V.t.idx[k][2];
          int n = (cx >> 3) | ((cy >> 3) << 1) | ((cz >> 3) << 2);
          const Block<Acc> *b = nb[n];
          if (!b) {
            ok = false;  // src/tsdf.cu:969
            break;
          }
          int li = (cx & 7) + 8 * (cy & 7) + 64 * (cz & 7);
          if ((float)b->w[li] < minw) {
            ok = false;
            break;
          }
          val[k] = (float)b->sdf[li];
          pt[k].x = (float)(bx * kB + cx);
          pt[k].y = (float)(by * kB + cy);
          pt[k].z = (float)(bz * kB + cz);
          pt[k].r = b->rgb[3 * li + 0];
          pt[k].g = b->rgb[3 * li + 1];
          pt[k].b = b->rgb[3 * li + 2];
        }
        if (!ok) continue;
        int ci = 0;
        for (int k = 0; k < 8; ++k)
          if (val[k] < 0.0f) ci |= 1 << k;  // src/tsdf.cu:978-986
        int em = V.t.edge[ci];
        if (em == 0) continue;
        V32 vl[12];
        V64 vl64[12];
        for (int e = 0; e < 12; ++e)
          if (em & (1 << e)) {
            int a = kEdgeCorners[e][0], b = kEdgeCorners[e][1];
            vinterp(pt[a], pt[b], val[a], val[b], vl[e], vl64[e]);
          }
        int count = 0;
        for (int ti = 0; V.t.tri[ci][ti] != -1; ti += 3, ++count) {
          const int e0 = V.t.tri[ci][ti], e1 = V.t.tri[ci][ti + 1], e2 = V.t.tri[ci][ti + 2];
          // src/tsdf.cu:1055-1057 tests p0==p1 || p1==p2 || p0==p1.
          if (veq(vl[e0], vl[e1]) || veq(vl[e1], vl[e2])) continue;
          Tri t;
          const int es[3] = {e0, e1, e2};
          for (int j = 0; j < 3; ++j) {
            t.xyz[3 * j + 0] = vl[es[j]].x;
            t.xyz[3 * j + 1] = vl[es[j]].y;
            t.xyz[3 * j + 2] = vl[es[j]].z;
            t.rgb[3 * j + 0] = vl[es[j]].r;
            t.rgb[3 * j + 1] = vl[es[j]].g;
            t.rgb[3 * j + 2] = vl[es[j]].b;
            t.xyz64[3 * j + 0] = vl64[es[j]].x;
            t.xyz64[3 * j + 1] = vl64[es[j]].y;
            t.xyz64[3 * j + 2] = vl64[es[j]].z;
          }
          t.cube[0] = bx * kB + x;
          t.cube[1] = by * kB + y;
          t.cube[2] = bz * kB + z;
          t.cube[3] = count;
          out.push_back(t);
        }
      }
}

struct Handle {
  int precision;  // 32 or 64
  Volume<float> *v32 = nullptr;
  Volume<double> *v64 = nullptr;
  std::vector<Tri> tris;
  int64_t alloc_errors = 0;
};

template <typename Acc>
int64_t integrate_frame(Volume<Acc> &V, const float *depth, const uint8_t *rgb, const float *c2w,
                        int64_t *range_errors) {
  const OParams &p = V.p;
  const int W = p.width, H = p.height;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  std::vector<std::vector<uint64_t>> per(nt);
  int64_t errs = 0;
#pragma omp parallel reduction(+ : errs)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<uint64_t> &mine = per[tid];
#pragma omp for schedule(static)
    for (int v = 0; v < H; ++v) {
      for (int u = 0; u < W; ++u) {
        if (!band_blocks(u, v, depth[(size_t)v * W + u], p, c2w, mine)) errs += 1;
      }
      // keep the per-thread lists short
      if ((v & 7) == 7) {
        std::sort(mine.begin(), mine.end());
        mine.erase(std::unique(mine.begin(), mine.end()), mine.end());
      }
    }
    std::sort(mine.begin(), mine.end());
    mine.erase(std::unique(mine.begin(), mine.end()), mine.end());
  }
  std::vector<uint64_t> all;
  for (auto &m : per) all.insert(all.end(), m.begin(), m.end());
  std::sort(all.begin(), all.end());
  all.erase(std::unique(all.begin(), all.end()), all.end());
  V.frame.clear();
  V.last_new = 0;
  for (uint64_t k : all) {
    bool created = false;
    V.frame.push_back(V.get_or_add(k, &created));
    V.last_new += created;
  }
  int64_t updated = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : updated)
  for (int64_t i = 0; i < (int64_t)V.frame.size(); ++i) {
    Block<Acc> &b = V.blocks[V.frame[i]];
    int bx, by, bz;
    ounkey(V.keys[V.frame[i]], bx, by, bz);
    for (int li = 0; li < kB3; ++li) {
      int x = li & 7, y = (li >> 3) & 7, z = li >> 6;
      updated += integrate_voxel<Acc>(p, c2w, depth, rgb, bx * kB + x, by * kB + y, bz * kB + z,
                                      b.sdf[li], b.w[li], &b.rgb[3 * li]);
    }
  }
  V.last_updated = updated;
  if (range_errors) *range_errors = errs;
  return (int64_t)V.frame.size();
}

template <typename Acc>
int64_t run_mc(Volume<Acc> &V, int scope_all, std::vector<Tri> &tris) {
  std::vector<int32_t> list;
  if (scope_all) {
    std::vector<std::pair<uint64_t, int32_t>> order;
    order.reserve(V.keys.size());
    for (size_t i = 0; i < V.keys.size(); ++i) order.push_back({V.keys[i], (int32_t)i});
    std::sort(order.begin(), order.end());
    for (auto &o : order) list.push_back(o.second);
  } else {
    list = V.frame;
  }
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  std::vector<std::vector<Tri>> per((size_t)list.size());
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
  for (int64_t i = 0; i < (int64_t)list.size(); ++i) mc_block<Acc>(V, list[i], per[i]);
  tris.clear();
  for (auto &v : per) tris.insert(tris.end(), v.begin(), v.end());
  return (int64_t)tris.size();
}

template <typename Acc>
int64_t export_blocks(const Volume<Acc> &V, int scope_frame, int32_t *xyz, float *sdf, float *w,
                      uint8_t *rgb, double *sdf64, double *w64) {
  std::vector<std::pair<uint64_t, int32_t>> order;
  if (scope_frame) {
    for (int32_t id : V.frame) order.push_back({V.keys[id], id});
  } else {
    for (size_t i = 0; i < V.keys.size(); ++i) order.push_back({V.keys[i], (int32_t)i});
  }
  std::sort(order.begin(), order.end());
  for (size_t i = 0; i < order.size(); ++i) {
    const Block<Acc> &b = V.blocks[order[i].second];
    int x, y, z;
    ounkey(order[i].first, x, y, z);
    if (xyz) {
      xyz[3 * i] = x;
      xyz[3 * i + 1] = y;
      xyz[3 * i + 2] = z;
    }
    for (int li = 0; li < kB3; ++li) {
      if (sdf) sdf[i * kB3 + li] = (float)b.sdf[li];
      if (w) w[i * kB3 + li] = (float)b.w[li];
      if (sdf64) sdf64[i * kB3 + li] = (double)b.sdf[li];
      if (w64) w64[i * kB3 + li] = (double)b.w[li];
    }
    if (rgb) std::memcpy(rgb + i * kB3 * 3, b.rgb, kB3 * 3);
  }
  return (int64_t)order.size();
}

template <typename Acc>
void import_blocks(Volume<Acc> &V, const int32_t *xyz, const float *sdf, const float *w,
                   const uint8_t *rgb, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    bool created;
    int32_t id = V.get_or_add(okey(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), &created);
    Block<Acc> &b = V.blocks[id];
    for (int li = 0; li < kB3; ++li) {
      b.sdf[li] = (Acc)sdf[i * kB3 + li];
      b.w[li] = (Acc)w[i * kB3 + li];
    }
    std::memcpy(b.rgb, rgb + i * kB3 * 3, kB3 * 3);
  }
}

// Ray casting of the fused surface, the same march as the engine's
// vh_raycast in FP64 (no reference counterpart: the reference draws its
// mesh with OpenGL, src/tsdf.cu:1710-1758): step T through unknown space,
// 0.8 * T * phi (at least half a voxel) through known positive space, half
// a voxel through negative space not entered from positive space, the first
// + -> - change interpolated linearly; depth is camera z.
template <typename Acc>
void raycast64(const Volume<Acc> &V, const double *P, double min_w, double *depth, double *normal) {
  const OParams &p = V.p;
  const double T = p.trunc, vs = p.voxel_size;
  for (int v = 0; v < p.height; ++v)
    for (int u = 0; u < p.width; ++u) {
      const double dx = (u - (double)p.cx) / p.fx, dy = (v - (double)p.cy) / p.fy;
      const double w[3] = {P[0] * dx + P[1] * dy + P[2], P[4] * dx + P[5] * dy + P[6],
                           P[8] * dx + P[9] * dy + P[10]};
      const double len = std::sqrt(dx * dx + dy * dy + 1.0);
      const double far_step = T / len, min_step = 0.5 * vs / len;
      const int max_steps = (int)((p.max_depth - p.min_depth) / min_step) + 2;
      double t = p.min_depth, prev_t = 0, prev_phi = 0, t_hit = 0, g[3] = {0, 0, 0};
      bool prev_ok = false, hit = false;
      for (int it = 0; it < max_steps && t <= p.max_depth; ++it) {
        double phi, gs[3];
        if (!sample64(V, P[3] + t * w[0], P[7] + t * w[1], P[11] + t * w[2], min_w, &phi, gs)) {
          prev_ok = false;
          t += far_step;
          continue;
        }
        if (phi <= 0) {
          if (prev_ok) {
            t_hit = prev_t + (t - prev_t) * (prev_phi / (prev_phi - phi));
            hit = true;
            std::memcpy(g, gs, sizeof(g));
            break;
          }
          t += min_step;  // negative space not entered from positive space: cross it
          continue;
        }
        prev_ok = true;
        prev_phi = phi;
        prev_t = t;
        std::memcpy(g, gs, sizeof(g));
        t += std::max(0.8 * phi * T / len, min_step);
      }
      const size_t i = (size_t)v * p.width + u;
      depth[i] = hit ? t_hit : 0.0;
      double n[3] = {0, 0, 0};
      if (hit) {
        double phi, gs[3];
        if (sample64(V, P[3] + t_hit * w[0], P[7] + t_hit * w[1], P[11] + t_hit * w[2], min_w, &phi,
                     gs))
          std::memcpy(g, gs, sizeof(g));
        const double gn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        if (gn > 0)
          for (int a = 0; a < 3; ++a) n[a] = g[a] / gn;
      }
      for (int a = 0; a < 3; ++a) normal[3 * i + a] = n[a];
    }
}

}  // namespace

extern "C" {

// params: width, height, fx, fy, cx, cy, min_depth, max_depth, voxel_size,
// trunc, mc_min_weight.  tables: idxMap[8][3], edgeTable[256], triTable[256][16].
void *vho_create(const float *fp, const int32_t *ip, const int32_t *idx_map,
                 const int32_t *edge_table, const int32_t *tri_table, int32_t precision) {
  OParams p;
  p.width = ip[0];
  p.height = ip[1];
  p.fx = fp[0];
  p.fy = fp[1];
  p.cx = fp[2];
  p.cy = fp[3];
  p.min_depth = fp[4];
  p.max_depth = fp[5];
  p.voxel_size = fp[6];
  p.trunc = fp[7];
  p.mc_min_weight = fp[8];
  Tables t;
  std::memcpy(t.idx, idx_map, sizeof(t.idx));
  std::memcpy(t.edge, edge_table, sizeof(t.edge));
  std::memcpy(t.tri, tri_table, sizeof(t.tri));
  Handle *h = new Handle();
  h->precision = precision == 64 ? 64 : 32;
  if (h->precision == 64) {
    h->v64 = new Volume<double>();
    h->v64->p = p;
    h->v64->t = t;
  } else {
    h->v32 = new Volume<float>();
    h->v32->p = p;
    h->v32->t = t;
  }
  return h;
}

void vho_destroy(void *hp) {
  Handle *h = (Handle *)hp;
  delete h->v32;
  delete h->v64;
  delete h;
}

void vho_set_threads(int32_t n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int32_t vho_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// depth in metres (fp32), rgb H*W*3, c2w 16 floats row-major.
// Returns the number of blocks in the frame's block list.
int64_t vho_integrate(void *hp, const float *depth, const uint8_t *rgb, const float *c2w) {
  Handle *h = (Handle *)hp;
  int64_t errs = 0, n;
  if (h->precision == 64)
    n = integrate_frame(*h->v64, depth, rgb, c2w, &errs);
  else
    n = integrate_frame(*h->v32, depth, rgb, c2w, &errs);
  h->alloc_errors += errs;
  return n;
}

// Band blocks of one frame without integrating (sorted unique keys as int32
// triples); returns the count, writes at most `cap` triples.
int64_t vho_band_blocks(const float *fp, const int32_t *ip, const float *depth, const float *c2w,
                        int32_t *xyz, int64_t cap) {
  OParams p;
  p.width = ip[0];
  p.height = ip[1];
  p.fx = fp[0];
  p.fy = fp[1];
  p.cx = fp[2];
  p.cy = fp[3];
  p.min_depth = fp[4];
  p.max_depth = fp[5];
  p.voxel_size = fp[6];
  p.trunc = fp[7];
  std::vector<uint64_t> keys;
  for (int v = 0; v < p.height; ++v)
    for (int u = 0; u < p.width; ++u) band_blocks(u, v, depth[(size_t)v * p.width + u], p, c2w, keys);
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  for (int64_t i = 0; i < (int64_t)keys.size() && i < cap; ++i) {
    int x, y, z;
    ounkey(keys[i], x, y, z);
    xyz[3 * i] = x;
    xyz[3 * i + 1] = y;
    xyz[3 * i + 2] = z;
  }
  return (int64_t)keys.size();
}

int64_t vho_num_blocks(void *hp) {
  Handle *h = (Handle *)hp;
  return h->precision == 64 ? (int64_t)h->v64->keys.size() : (int64_t)h->v32->keys.size();
}
int64_t vho_frame_blocks(void *hp) {
  Handle *h = (Handle *)hp;
  return h->precision == 64 ? (int64_t)h->v64->frame.size() : (int64_t)h->v32->frame.size();
}
// [new blocks, updated voxels, range errors] of the last frame.
void vho_last_counts(void *hp, int64_t *out3) {
  Handle *h = (Handle *)hp;
  if (h->precision == 64) {
    out3[0] = h->v64->last_new;
    out3[1] = h->v64->last_updated;
  } else {
    out3[0] = h->v32->last_new;
    out3[1] = h->v32->last_updated;
  }
  out3[2] = h->alloc_errors;
}

// Copies blocks sorted by packed key (scope_frame: the last frame's list).
int64_t vho_export(void *hp, int32_t scope_frame, int32_t *xyz, float *sdf, float *w, uint8_t *rgb,
                   double *sdf64, double *w64) {
  Handle *h = (Handle *)hp;
  if (h->precision == 64) return export_blocks(*h->v64, scope_frame, xyz, sdf, w, rgb, sdf64, w64);
  return export_blocks(*h->v32, scope_frame, xyz, sdf, w, rgb, sdf64, w64);
}

void vho_import(void *hp, const int32_t *xyz, const float *sdf, const float *w, const uint8_t *rgb,
                int64_t n) {
  Handle *h = (Handle *)hp;
  if (h->precision == 64)
    import_blocks(*h->v64, xyz, sdf, w, rgb, n);
  else
    import_blocks(*h->v32, xyz, sdf, w, rgb, n);
}

// Marks the given keys as the current block list (for per-frame MC of an
// imported volume).
void vho_set_frame(void *hp, const int32_t *xyz, int64_t n) {
  Handle *h = (Handle *)hp;
  std::vector<std::pair<uint64_t, int32_t>> order;
  auto fill = [&](auto &V) {
    V.frame.clear();
    for (int64_t i = 0; i < n; ++i) {
      uint64_t k = okey(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
      int32_t id = V.find(k);
      if (id >= 0) order.push_back({k, id});
    }
    std::sort(order.begin(), order.end());
    for (auto &o : order) V.frame.push_back(o.second);
  };
  if (h->precision == 64)
    fill(*h->v64);
  else
    fill(*h->v32);
}

// Runs MC; returns the triangle count (kept in the handle).
int64_t vho_mc(void *hp, int32_t scope_all) {
  Handle *h = (Handle *)hp;
  if (h->precision == 64) return run_mc(*h->v64, scope_all, h->tris);
  return run_mc(*h->v32, scope_all, h->tris);
}

// Copies the last MC result (any pointer may be NULL).
int64_t vho_mc_copy(void *hp, float *xyz, uint8_t *rgb, double *xyz64, int32_t *cube,
                    int64_t cap) {
  Handle *h = (Handle *)hp;
  int64_t n = std::min<int64_t>(cap, (int64_t)h->tris.size());
  for (int64_t i = 0; i < n; ++i) {
    const Tri &t = h->tris[i];
    if (xyz) std::memcpy(xyz + 9 * i, t.xyz, sizeof(t.xyz));
    if (rgb) std::memcpy(rgb + 9 * i, t.rgb, sizeof(t.rgb));
    if (xyz64) std::memcpy(xyz64 + 9 * i, t.xyz64, sizeof(t.xyz64));
    if (cube) std::memcpy(cube + 4 * i, t.cube, sizeof(t.cube));
  }
  return (int64_t)h->tris.size();
}

}  // extern "C"

// ---- hooks for the golden-vector tests (reference host functions) -----------
extern "C" {

// frame2base (src/tsdf.cu:108-116) with K = [fx 0 cx; 0 fy cy; 0 0 1].
void vho_frame2base(int32_t u, int32_t v, float z, const float *K, const float *c2w, float *out3) {
  OParams p{};
  p.fx = K[0];
  p.cx = K[2];
  p.fy = K[4];
  p.cy = K[5];
  float cam[3];
  frame2cam(u, v, z, p, cam);
  cam2base(cam, c2w, out3);
}

void vho_base2cam(const float *pw, const float *c2w, float *out3) { base2cam(pw, c2w, out3); }

// cam2frame (src/tsdf.cu:75-79): rounded pixel as int.
void vho_cam2frame(const float *cam, const float *K, int32_t *out2) {
  out2[0] = (int32_t)std::round(K[0] * (cam[0] / cam[2]) + K[2]);
  out2[1] = (int32_t)std::round(K[4] * (cam[1] / cam[2]) + K[5]);
}

// VertexInterp at iso 0 (src/tsdf.cu:1640-1660). p: x1 y1 z1 x2 y2 z2; c: r1 g1 b1 r2 g2 b2.
void vho_vertex_interp(const float *p, const uint8_t *c, float v1, float v2, float *out3,
                       uint8_t *rgb3) {
  V32 a{p[0], p[1], p[2], c[0], c[1], c[2]}, b{p[3], p[4], p[5], c[3], c[4], c[5]}, o;
  V64 o64;
  vinterp(a, b, v1, v2, o, o64);
  out3[0] = o.x;
  out3[1] = o.y;
  out3[2] = o.z;
  rgb3[0] = o.r;
  rgb3[1] = o.g;
  rgb3[2] = o.b;
}

}  // extern "C"

// ---- differentiable queries (no reference counterpart) ------------------------
namespace {

// Trilinear TSDF value and gradient at a world point, in double precision,
// over the oracle's stored voxels (corners need weight >= min_w).
template <typename Acc>
bool sample64(const Volume<Acc> &V, double x, double y, double z, double min_w, double *phi,
              double g[3]) {
  const double vs = V.p.voxel_size;
  const double q[3] = {x / vs, y / vs, z / vs};
  long b[3];
  double f[3];
  for (int a = 0; a < 3; ++a) {
    const double fl = std::floor(q[a]);
    b[a] = (long)fl;
    f[a] = q[a] - fl;
  }
  double val[8];
  for (int c = 0; c < 8; ++c) {
    const long ix = b[0] + (c & 1), iy = b[1] + ((c >> 1) & 1), iz = b[2] + (c >> 2);
    const long bx = ix >= 0 ? ix / 8 : -((-ix + 7) / 8), by = iy >= 0 ? iy / 8 : -((-iy + 7) / 8),
               bz = iz >= 0 ? iz / 8 : -((-iz + 7) / 8);
    const int32_t id = V.find(okey((int)bx, (int)by, (int)bz));
    if (id < 0) return false;
    const int li = (int)(ix - 8 * bx) + 8 * (int)(iy - 8 * by) + 64 * (int)(iz - 8 * bz);
    if ((double)V.blocks[id].w[li] < min_w) return false;
    val[c] = (double)V.blocks[id].sdf[li];
  }
  double p = 0, gx = 0, gy = 0, gz = 0;
  for (int c = 0; c < 8; ++c) {
    const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
    const double wx = dx ? f[0] : 1 - f[0], wy = dy ? f[1] : 1 - f[1], wz = dz ? f[2] : 1 - f[2];
    p += wx * wy * wz * val[c];
    gx += (dx ? 1.0 : -1.0) * wy * wz * val[c];
    gy += wx * (dy ? 1.0 : -1.0) * wz * val[c];
    gz += wx * wy * (dz ? 1.0 : -1.0) * val[c];
  }
  *phi = p;
  g[0] = gx / vs;
  g[1] = gy / vs;
  g[2] = gz / vs;
  return true;
}

template <typename Acc>
void pose_terms64(const Volume<Acc> &V, const float *depth, const double *P, int stride,
                  double min_w, double *out) {
  for (int k = 0; k < 29; ++k) out[k] = 0;
  const OParams &p = V.p;
  for (int v = 0; v < p.height; v += stride)
    for (int u = 0; u < p.width; u += stride) {
      const double d = depth[(size_t)v * p.width + u];
      if (!(d > p.min_depth && d <= p.max_depth)) continue;
      const double cx = (u - (double)p.cx) * d / p.fx, cy = (v - (double)p.cy) * d / p.fy;
      double X[3];
      for (int r = 0; r < 3; ++r) X[r] = cx * P[4 * r] + cy * P[4 * r + 1] + d * P[4 * r + 2] + P[4 * r + 3];
      double phi, g[3];
      if (!sample64(V, X[0], X[1], X[2], min_w, &phi, g) || !(std::fabs(phi) < 1.0)) continue;
      const double T = p.trunc;
      const double J[6] = {T * g[0], T * g[1], T * g[2], T * (X[1] * g[2] - X[2] * g[1]),
                           T * (X[2] * g[0] - X[0] * g[2]), T * (X[0] * g[1] - X[1] * g[0])};
      const double r = T * phi;
      int k = 0;
      for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b) out[k++] += J[a] * J[b];
      for (int a = 0; a < 6; ++a) out[21 + a] += J[a] * r;
      out[27] += r * r;
      out[28] += 1;
    }
}

}  // namespace

extern "C" {

// phi (units of T) and d phi / d point at n world points; valid[i] = 0/1.
void vho_sample(void *hp, const double *xyz, int64_t n, double min_w, double *phi, double *grad,
                uint8_t *valid) {
  Handle *h = (Handle *)hp;
  for (int64_t i = 0; i < n; ++i) {
    double g[3] = {0, 0, 0}, f = 0;
    const bool ok = h->precision == 64
                        ? sample64(*h->v64, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], min_w, &f, g)
                        : sample64(*h->v32, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], min_w, &f, g);
    phi[i] = ok ? f : 0;
    for (int a = 0; a < 3; ++a) grad[3 * i + a] = ok ? g[a] : 0;
    valid[i] = ok;
  }
}

// FP64 ray cast of the fused surface: camera-z depth (0 = no hit) and unit
// normals per pixel; P: 12 doubles, row-major camera-to-world 3x4.
void vho_raycast(void *hp, const double *P, double min_w, double *depth, double *normal) {
  Handle *h = (Handle *)hp;
  if (h->precision == 64)
    raycast64(*h->v64, P, min_w, depth, normal);
  else
    raycast64(*h->v32, P, min_w, depth, normal);
}

// Normal-equation terms (same layout as the engine) in double precision;
// P: 12 doubles, row-major camera-to-world 3x4.
void vho_pose_terms(void *hp, const float *depth, const double *P, int32_t stride, double min_w,
                    double *out29) {
  Handle *h = (Handle *)hp;
  if (h->precision == 64)
    pose_terms64(*h->v64, depth, P, stride, min_w, out29);
  else
    pose_terms64(*h->v32, depth, P, stride, min_w, out29);
}

}  // extern "C"

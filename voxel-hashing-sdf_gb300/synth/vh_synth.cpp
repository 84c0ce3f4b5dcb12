// vh_synth.cpp - deterministic synthetic RGB-D streams.
//
// The reference fuses ScanNet frames read by SaveFrame::frameLoad
// (src/SaveFrame.cpp:154-218: RGB jpg, uint16 millimetre depth png, 4x4 pose
// text).  Those frames are not available, so this generator ray-casts seeded
// analytic scenes instead and emits the same formats: uint16 depth in
// millimetres, interleaved 8-bit RGB and a row-major camera-to-world matrix
// (the layout PointCloudGenerator::Reproject hands to processFrame,
// src/PointCloudGenerator.cpp:118-127).
//
// Camera model: pinhole, OpenCV axes (x right, y down, z forward), pixel
// (u, v) centred at integer coordinates, depth = camera-frame z of the hit.
// World: z up.  Noise: depth += N(0, (1.5e-3 * z^2)^2) m, then clipped to
// [0.3, 4.0] m (0 = invalid) and rounded to millimetres.
//
// Scene kinds
//   1  4x4x3 m box room, 3 spheres r in U[0.3,0.6], camera on a 1.5 m circle
//      at 1.4 m height looking at the room centre.
//   2  8x8x3 m room, 40 seeded boxes / spheres / cylinders, closed
//      Catmull-Rom trajectory walked at 0.5 m/s and 30 Hz.
//   3  room of seeded extent in [1, 8] m with 2..20 objects and a circular
//      trajectory scaled to the room (one of many uneven batched scenes).
//   4  20x20x4 m floor of 4x4 rooms (5x5 m): interior walls 0.1 m thick
//      with a 1.2 m wide, 2.2 m high door in every wall between two rooms,
//      4 seeded objects per room; the camera walks a closed loop through all
//      16 rooms and their doors at 0.5 m/s and 30 Hz, 1.5 m high.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

inline uint64_t mix3(uint64_t a, uint64_t b, uint64_t c) {
  SplitMix m(a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull) * 0xD1B54A32D192ED03ull ^ c);
  m.next();
  return m.next();
}

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 normalize(V3 a) {
  double n = std::sqrt(dot(a, a));
  return a * (1.0 / n);
}

enum PrimKind { kSphere = 0, kBox = 1, kCylinder = 2 };

struct Prim {
  int kind;
  V3 a, b;    // sphere: a = centre, b.x = radius; box: min, max; cylinder: a = (x, y, z0), b = (r, z1, -)
  uint8_t col[3];
};

struct Pose {
  double R[3][3];  // columns = camera axes in world
  V3 t;
};

struct Scene {
  int kind;
  int width, height;
  double fx, fy, cx, cy;
  V3 room_min, room_max;
  std::vector<Prim> prims;
  std::vector<Pose> poses;
  uint64_t noise_seed;
  double clip_near = 0.3, clip_far = 4.0;
};

Pose look_at(V3 eye, V3 target) {
  V3 f = normalize(target - eye);
  V3 up = {0, 0, 1};
  V3 r = normalize(cross(f, up));
  V3 d = cross(f, r);
  Pose p;
  for (int i = 0; i < 3; ++i) {
    double rc[3] = {r.x, r.y, r.z}, dc[3] = {d.x, d.y, d.z}, fc[3] = {f.x, f.y, f.z};
    p.R[i][0] = rc[i];
    p.R[i][1] = dc[i];
    p.R[i][2] = fc[i];
  }
  p.t = eye;
  return p;
}

V3 catmull(V3 p0, V3 p1, V3 p2, V3 p3, double t) {
  double t2 = t * t, t3 = t2 * t;
  return (p1 * 2.0 + (p2 - p0) * t + (p0 * 2.0 - p1 * 5.0 + p2 * 4.0 - p3) * t2 +
          (p1 * 3.0 - p0 - p2 * 3.0 + p3) * t3) *
         0.5;
}

uint8_t clamp8(double v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

void random_colour(SplitMix &r, uint8_t c[3]) {
  for (int i = 0; i < 3; ++i) c[i] = (uint8_t)(40 + (r.next() % 200));
}

// Places `n` random primitives inside [lo, hi] keeping `clear` distance (xy)
// from every point of `path`.
void place_objects(Scene &s, SplitMix &r, int n, V3 lo, V3 hi, const std::vector<V3> &path,
                   double clear) {
  int placed = 0;
  for (int attempt = 0; attempt < n * 200 && placed < n; ++attempt) {
    Prim p;
    p.kind = (int)(r.next() % 3);
    double sx = hi.x - lo.x, sy = hi.y - lo.y, sz = hi.z - lo.z;
    double sc = std::fmin(1.0, std::fmin(sx, sy) / 4.0);  // smaller objects in small rooms
    double x = r.uniform(lo.x + 0.3 * sc, hi.x - 0.3 * sc);
    double y = r.uniform(lo.y + 0.3 * sc, hi.y - 0.3 * sc);
    double reach = 0;
    if (p.kind == kSphere) {
      double rad = r.uniform(0.15, 0.5) * sc;
      double z = r.uniform(lo.z + rad, std::fmin(hi.z - rad, lo.z + 0.85 * sz));
      p.a = {x, y, z};
      p.b = {rad, 0, 0};
      reach = rad;
    } else if (p.kind == kBox) {
      double hx = r.uniform(0.15, 0.6) * sc, hy = r.uniform(0.15, 0.6) * sc;
      double h = r.uniform(0.2, 1.5) * sc;
      p.a = {x - hx, y - hy, lo.z};
      p.b = {x + hx, y + hy, lo.z + h};
      reach = std::sqrt(hx * hx + hy * hy);
    } else {
      double rad = r.uniform(0.1, 0.4) * sc;
      double h = r.uniform(0.3, 2.5) * sc;
      p.a = {x, y, lo.z};
      p.b = {rad, lo.z + std::fmin(h, 0.9 * sz), 0};
      reach = rad;
    }
    bool ok = true;
    for (const V3 &q : path) {
      double dx = q.x - x, dy = q.y - y;
      if (std::sqrt(dx * dx + dy * dy) < reach + clear) {
        ok = false;
        break;
      }
    }
    if (!ok) continue;
    random_colour(r, p.col);
    s.prims.push_back(p);
    ++placed;
  }
}

// Arc-length parametrised closed Catmull-Rom loop through `ctrl`, sampled
// densely; returns the samples and their cumulative lengths.
void dense_loop(const std::vector<V3> &ctrl, int per, std::vector<V3> &dense,
                std::vector<double> &cum) {
  const size_t n = ctrl.size();
  dense.clear();
  for (size_t k = 0; k < n; ++k)
    for (int i = 0; i < per; ++i)
      dense.push_back(catmull(ctrl[(k + n - 1) % n], ctrl[k], ctrl[(k + 1) % n], ctrl[(k + 2) % n],
                              (double)i / per));
  cum.assign(dense.size() + 1, 0.0);
  for (size_t i = 0; i < dense.size(); ++i) {
    V3 d = dense[(i + 1) % dense.size()] - dense[i];
    cum[i + 1] = cum[i] + std::sqrt(dot(d, d));
  }
}

Prim wall_box(V3 lo, V3 hi, SplitMix &r) {
  Prim p;
  p.kind = kBox;
  p.a = lo;
  p.b = hi;
  random_colour(r, p.col);
  return p;
}

// Scene kind 4: the multi-room floor (see the kinds above).
void build_floor(Scene &s, SplitMix &r, int num_frames) {
  const double half = 10.0, room = 5.0, wall = 0.05, door = 0.6, door_h = 2.2, h = 4.0;
  s.room_min = {-half, -half, 0};
  s.room_max = {half, half, h};
  // interior walls on x = -5, 0, 5 (running along y) and y = -5, 0, 5
  for (int axis = 0; axis < 2; ++axis)
    for (int k = 1; k < 4; ++k) {
      const double c = -half + room * k;
      double from = -half;
      for (int j = 0; j < 4; ++j) {
        const double dc = -half + room * (j + 0.5);  // door centre along the wall
        const double seg[3][2] = {{from, dc - door}, {dc - door, dc + door}, {dc + door, 0}};
        for (int q = 0; q < 2; ++q) {
          const double a0 = seg[q][0], a1 = seg[q][1];
          const double z0 = q == 0 ? 0.0 : door_h;  // q == 1: lintel above the door
          V3 lo = axis == 0 ? V3{c - wall, a0, z0} : V3{a0, c - wall, z0};
          V3 hi = axis == 0 ? V3{c + wall, a1, h} : V3{a1, c + wall, h};
          s.prims.push_back(wall_box(lo, hi, r));
        }
        from = dc + door;
      }
      V3 lo = axis == 0 ? V3{c - wall, from, 0} : V3{from, c - wall, 0};
      V3 hi = axis == 0 ? V3{c + wall, half, h} : V3{half, c + wall, h};
      s.prims.push_back(wall_box(lo, hi, r));
    }
  // closed loop through all 16 rooms (a Hamiltonian cycle of the 4x4 grid),
  // passing each shared wall through its door
  const int cyc[16][2] = {{0, 0}, {1, 0}, {2, 0}, {3, 0}, {3, 1}, {2, 1}, {1, 1}, {1, 2},
                          {2, 2}, {3, 2}, {3, 3}, {2, 3}, {1, 3}, {0, 3}, {0, 2}, {0, 1}};
  const double cam_z = 1.5;
  std::vector<V3> ctrl;
  for (int k = 0; k < 16; ++k) {
    const int *a = cyc[k], *b = cyc[(k + 1) % 16];
    V3 ca = {-half + room * (a[0] + 0.5), -half + room * (a[1] + 0.5), cam_z};
    V3 cb = {-half + room * (b[0] + 0.5), -half + room * (b[1] + 0.5), cam_z};
    V3 mid = (ca + cb) * 0.5;
    V3 dir = normalize(cb - ca);
    ctrl.push_back(ca);
    ctrl.push_back(mid - dir * 0.8);  // straight through the door
    ctrl.push_back(mid + dir * 0.8);
  }
  std::vector<V3> dense;
  std::vector<double> cum;
  dense_loop(ctrl, 100, dense, cum);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      V3 lo = {-half + room * i + 0.2, -half + room * j + 0.2, 0};
      V3 hi = {-half + room * (i + 1) - 0.2, -half + room * (j + 1) - 0.2, h};
      place_objects(s, r, 4, lo, hi, dense, 0.7);
    }
  const double total = cum.back(), ds = 0.5 / 30.0;
  size_t seg = 0;
  for (int f = 0; f < num_frames; ++f) {
    double sarc = std::fmod(f * ds, total);
    while (!(cum[seg] <= sarc && sarc < cum[seg + 1])) seg = (seg + 1) % dense.size();
    double a = (sarc - cum[seg]) / (cum[seg + 1] - cum[seg]);
    V3 p0 = dense[seg], p1 = dense[(seg + 1) % dense.size()];
    V3 eye = p0 + (p1 - p0) * a;
    V3 fwd = normalize(normalize(p1 - p0) + V3{0, 0, -0.25});
    s.poses.push_back(look_at(eye, eye + fwd));
  }
}

void build_scene(Scene &s, int kind, uint64_t seed, int num_frames) {
  SplitMix r(seed * 0x2545F4914F6CDD1Dull + 17);
  s.kind = kind;
  s.noise_seed = seed + 1;
  if (kind == 1) {
    s.room_min = {-2, -2, 0};
    s.room_max = {2, 2, 3};
    for (int i = 0; i < 3; ++i) {
      Prim p;
      p.kind = kSphere;
      double rad = r.uniform(0.3, 0.6);
      double lim = 1.5 - rad - 0.3;
      p.a = {r.uniform(-lim, lim), r.uniform(-lim, lim), r.uniform(rad, 3.0 - rad)};
      p.b = {rad, 0, 0};
      random_colour(r, p.col);
      s.prims.push_back(p);
    }
    V3 centre = {0, 0, 1.5};
    for (int i = 0; i < num_frames; ++i) {
      double th = 2.0 * M_PI * i / num_frames;
      s.poses.push_back(look_at({1.5 * std::cos(th), 1.5 * std::sin(th), 1.4}, centre));
    }
    return;
  }
  if (kind == 4) {
    build_floor(s, r, num_frames);
    return;
  }
  double ex = 8, ey = 8, ez = 3;
  int nobj = 40;
  if (kind == 3) {
    ex = r.uniform(1.0, 8.0);
    ey = r.uniform(1.0, 8.0);
    ez = r.uniform(2.2, 3.2);
    nobj = 2 + (int)(r.next() % 19);
  }
  s.room_min = {-ex / 2, -ey / 2, 0};
  s.room_max = {ex / 2, ey / 2, ez};
  // Closed Catmull-Rom loop through 8 jittered control points.
  std::vector<V3> ctrl;
  double rx = 0.28 * ex, ry = 0.28 * ey;
  for (int k = 0; k < 8; ++k) {
    double th = 2.0 * M_PI * k / 8;
    double j = r.uniform(0.85, 1.15);
    ctrl.push_back({rx * j * std::cos(th), ry * j * std::sin(th), r.uniform(1.2, 1.7) * ez / 3.0});
  }
  std::vector<V3> dense;
  const int per = 200;
  for (int k = 0; k < 8; ++k)
    for (int i = 0; i < per; ++i)
      dense.push_back(catmull(ctrl[(k + 7) % 8], ctrl[k], ctrl[(k + 1) % 8], ctrl[(k + 2) % 8],
                              (double)i / per));
  std::vector<double> cum(dense.size() + 1, 0.0);
  for (size_t i = 0; i < dense.size(); ++i) {
    V3 d = dense[(i + 1) % dense.size()] - dense[i];
    cum[i + 1] = cum[i] + std::sqrt(dot(d, d));
  }
  const double total = cum.back();
  place_objects(s, r, nobj, s.room_min, s.room_max, dense, kind == 3 ? 0.35 * std::fmin(1.0, std::fmin(ex, ey) / 4.0) + 0.15 : 0.5);
  const double ds = 0.5 / 30.0;  // 0.5 m/s at 30 Hz
  size_t seg = 0;
  for (int f = 0; f < num_frames; ++f) {
    double sarc = std::fmod(f * ds, total);
    while (!(cum[seg] <= sarc && sarc < cum[seg + 1])) seg = (seg + 1) % dense.size();
    double a = (sarc - cum[seg]) / (cum[seg + 1] - cum[seg]);
    V3 p0 = dense[seg], p1 = dense[(seg + 1) % dense.size()];
    V3 eye = p0 + (p1 - p0) * a;
    V3 tan = normalize(p1 - p0);
    V3 inward = normalize(V3{-eye.x, -eye.y, 0} + V3{1e-9, 0, 0});
    V3 fwd = normalize(tan * 0.6 + inward * 0.4);
    fwd = normalize(fwd + V3{0, 0, -0.18});
    s.poses.push_back(look_at(eye, eye + fwd));
  }
}

// Nearest hit along o + t*d (t > 1e-6); returns t or +inf and the surface id.
inline double hit_room(const Scene &s, V3 o, V3 d, int *face) {
  double best = INFINITY;
  const double lo[3] = {s.room_min.x, s.room_min.y, s.room_min.z};
  const double hi[3] = {s.room_max.x, s.room_max.y, s.room_max.z};
  const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
  for (int a = 0; a < 3; ++a) {
    if (dd[a] > 0) {
      double t = (hi[a] - oo[a]) / dd[a];
      if (t < best) {
        best = t;
        *face = 2 * a + 1;
      }
    } else if (dd[a] < 0) {
      double t = (lo[a] - oo[a]) / dd[a];
      if (t < best) {
        best = t;
        *face = 2 * a;
      }
    }
  }
  return best;
}

inline double hit_prim(const Prim &p, V3 o, V3 d) {
  if (p.kind == kSphere) {
    V3 oc = o - p.a;
    double b = dot(oc, d), c = dot(oc, oc) - p.b.x * p.b.x, aa = dot(d, d);
    double disc = b * b - aa * c;
    if (disc < 0) return INFINITY;
    double sq = std::sqrt(disc);
    double t = (-b - sq) / aa;
    if (t > 1e-6) return t;
    t = (-b + sq) / aa;
    return t > 1e-6 ? t : INFINITY;
  }
  if (p.kind == kBox) {
    double t0 = -INFINITY, t1 = INFINITY;
    const double lo[3] = {p.a.x, p.a.y, p.a.z}, hi[3] = {p.b.x, p.b.y, p.b.z};
    const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    for (int a = 0; a < 3; ++a) {
      if (dd[a] == 0) {
        if (oo[a] < lo[a] || oo[a] > hi[a]) return INFINITY;
        continue;
      }
      double ta = (lo[a] - oo[a]) / dd[a], tb = (hi[a] - oo[a]) / dd[a];
      if (ta > tb) std::swap(ta, tb);
      if (ta > t0) t0 = ta;
      if (tb < t1) t1 = tb;
    }
    if (t0 > t1 || t1 < 1e-6) return INFINITY;
    return t0 > 1e-6 ? t0 : INFINITY;
  }
  // vertical cylinder with caps: centre (a.x, a.y), z in [a.z, b.y], radius b.x
  double best = INFINITY;
  double ox = o.x - p.a.x, oy = o.y - p.a.y;
  double A = d.x * d.x + d.y * d.y, B = ox * d.x + oy * d.y, C = ox * ox + oy * oy - p.b.x * p.b.x;
  if (A > 0) {
    double disc = B * B - A * C;
    if (disc >= 0) {
      double sq = std::sqrt(disc);
      for (double t : {(-B - sq) / A, (-B + sq) / A}) {
        if (t > 1e-6) {
          double z = o.z + t * d.z;
          if (z >= p.a.z && z <= p.b.y && t < best) best = t;
        }
      }
    }
  }
  if (d.z != 0) {
    for (double zc : {p.a.z, p.b.y}) {
      double t = (zc - o.z) / d.z;
      if (t > 1e-6 && t < best) {
        double x = ox + t * d.x, y = oy + t * d.y;
        if (x * x + y * y <= p.b.x * p.b.x) best = t;
      }
    }
  }
  return best;
}

void render(const Scene &s, int f, uint16_t *depth, uint8_t *rgb, float *c2w, int noise) {
  const Pose &P = s.poses[f];
  if (c2w) {
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) c2w[i * 4 + j] = (float)P.R[i][j];
    }
    c2w[3] = (float)P.t.x;
    c2w[7] = (float)P.t.y;
    c2w[11] = (float)P.t.z;
    c2w[12] = c2w[13] = c2w[14] = 0.0f;
    c2w[15] = 1.0f;
  }
  const int W = s.width, H = s.height;
#pragma omp parallel for schedule(static)
  for (int v = 0; v < H; ++v) {
    for (int u = 0; u < W; ++u) {
      V3 dc = {(u - s.cx) / s.fx, (v - s.cy) / s.fy, 1.0};
      V3 d = {P.R[0][0] * dc.x + P.R[0][1] * dc.y + P.R[0][2] * dc.z,
              P.R[1][0] * dc.x + P.R[1][1] * dc.y + P.R[1][2] * dc.z,
              P.R[2][0] * dc.x + P.R[2][1] * dc.y + P.R[2][2] * dc.z};
      int face = 0;
      double t = hit_room(s, P.t, d, &face);
      int obj = -1;
      for (size_t i = 0; i < s.prims.size(); ++i) {
        double ti = hit_prim(s.prims[i], P.t, d);
        if (ti < t) {
          t = ti;
          obj = (int)i;
        }
      }
      size_t pix = (size_t)v * W + u;
      double z = t;  // dc.z == 1 so the ray parameter is the z-depth
      if (noise) {
        uint64_t h = mix3(s.noise_seed, (uint64_t)f, pix);
        double u1 = ((h >> 11) + 1.0) * (1.0 / 9007199254740993.0);
        double u2 = (double)(mix3(s.noise_seed ^ 0xABCDEFull, (uint64_t)f, pix) >> 11) *
                    (1.0 / 9007199254740992.0);
        double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
        z += g * 1.5e-3 * z * z;
      }
      uint16_t dmm = 0;
      if (std::isfinite(z) && z >= s.clip_near && z <= s.clip_far) {
        double mm = std::floor(z * 1000.0 + 0.5);
        dmm = (uint16_t)(mm > 65535 ? 0 : mm);
      }
      depth[pix] = dmm;
      V3 hp = P.t + d * t;
      uint8_t base[3] = {180, 180, 170};
      if (obj >= 0) {
        std::memcpy(base, s.prims[obj].col, 3);
      } else {
        static const uint8_t walls[6][3] = {{200, 120, 100}, {110, 190, 120}, {120, 130, 210},
                                            {210, 200, 110}, {150, 150, 150}, {230, 230, 220}};
        std::memcpy(base, walls[face], 3);
      }
      long cxq = (long)std::floor(hp.x * 10.0), cyq = (long)std::floor(hp.y * 10.0),
           czq = (long)std::floor(hp.z * 10.0);
      double shade = ((cxq + cyq + czq) & 1) ? 1.0 : 0.75;
      for (int c = 0; c < 3; ++c) rgb[3 * pix + c] = clamp8(base[c] * shade);
    }
  }
}

}  // namespace

extern "C" {

void *vhs_create(int32_t kind, uint64_t seed, int32_t width, int32_t height, float fx, float fy,
                 float cx, float cy, int32_t num_frames) {
  if (kind < 1 || kind > 4 || width <= 0 || height <= 0 || num_frames <= 0) return nullptr;
  Scene *s = new Scene();
  s->width = width;
  s->height = height;
  s->fx = fx;
  s->fy = fy;
  s->cx = cx;
  s->cy = cy;
  build_scene(*s, kind, seed, num_frames);
  return s;
}

void vhs_destroy(void *p) { delete (Scene *)p; }

int32_t vhs_num_frames(void *p) { return (int32_t)((Scene *)p)->poses.size(); }

int32_t vhs_num_objects(void *p) { return (int32_t)((Scene *)p)->prims.size(); }

// room_min xyz, room_max xyz
void vhs_bounds(void *p, float *out6) {
  Scene *s = (Scene *)p;
  out6[0] = (float)s->room_min.x;
  out6[1] = (float)s->room_min.y;
  out6[2] = (float)s->room_min.z;
  out6[3] = (float)s->room_max.x;
  out6[4] = (float)s->room_max.y;
  out6[5] = (float)s->room_max.z;
}

// Renders frame `f` (depth uint16 mm H*W, rgb H*W*3, c2w 16 floats).
int32_t vhs_render(void *p, int32_t f, uint16_t *depth, uint8_t *rgb, float *c2w, int32_t noise) {
  Scene *s = (Scene *)p;
  if (f < 0 || f >= (int32_t)s->poses.size()) return -1;
  render(*s, f, depth, rgb, c2w, noise);
  return 0;
}

}  // extern "C"

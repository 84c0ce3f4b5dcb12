// ref_golden.cu - runs the reference's own host-callable code on the CPU and
// prints golden vectors as JSON.
//
// TEST INFRASTRUCTURE ONLY (fixture generator).  It is linked against the
// reference's unmodified src/tsdf.cu, compiled from where it lies by
// oracle/ref_golden/Makefile into oracle/_ref/.  Only __host__ code runs:
//   * ark::BlockHasher                     include/tsdf.cuh:144-156
//   * frame2cam / cam2frame / base2cam /   src/tsdf.cu:67-116
//     cam2base / frame2base
//   * ark::VertexInterp                    src/tsdf.cu:1640-1660
//   * MarchingCubeParam tables             include/tsdf.cuh:234-534
//   * vhashing::HashTable, host memspace   include/vhashing.h:205-484,622-684
// Floats are printed as their IEEE-754 bit patterns.

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "tsdf.cuh"

namespace ark {
// Defined with external linkage in src/tsdf.cu; declared here for host calls.
void frame2cam(int *pt_pix, float pt_cam_z, float *pt_cam, float *K_);
void cam2frame(float *pt_cam, int *pt_pix, float *K);
void base2cam(float *pt_base, float *pt_cam, float *c2w_);
void cam2base(float *pt_cam, float *pt_base, float *c2w_);
float3 frame2base(int pt_pix_x, int pt_pix_y, float pt_cam_z, float *K_, float *c2w_,
                  MarchingCubeParam *param);
}  // namespace ark

// The reference links src/safecall.cpp, which needs glog; these definitions
// stand in for it (only reached on a CUDA error, never on the host path).
void __cudaSafeCall(cudaError err, const char *file, const int line) {
  if (err != cudaSuccess) {
    std::fprintf(stderr, "cuda error %d at %s:%d\n", (int)err, file, line);
    throw "CUDA Error";
  }
}
void __cudaCheckError(const char *, const int) {}
void __cudaCheckKernel(const char *, const int) {}
void __cudaCheckKernelStream(cudaStream_t, const char *, const int) {}
void __cudaCheckMemory(const char *, const int) {}

namespace {

struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  float uni(float a, float b) { return a + (b - a) * (float)((next() >> 40) * (1.0 / 16777216.0)); }
  int irange(int a, int b) { return a + (int)(next() % (uint64_t)(b - a + 1)); }
};

uint32_t fb(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

// Orthonormal rotation from an axis-angle, row-major into c2w[0..11].
void random_pose(Rng &r, float *c2w) {
  double ax = r.uni(-1, 1), ay = r.uni(-1, 1), az = r.uni(-1, 1);
  double n = std::sqrt(ax * ax + ay * ay + az * az) + 1e-12;
  ax /= n;
  ay /= n;
  az /= n;
  double th = r.uni(-3.1f, 3.1f), c = std::cos(th), s = std::sin(th), C = 1 - c;
  double R[3][3] = {{c + ax * ax * C, ax * ay * C - az * s, ax * az * C + ay * s},
                    {ay * ax * C + az * s, c + ay * ay * C, ay * az * C - ax * s},
                    {az * ax * C - ay * s, az * ay * C + ax * s, c + az * az * C}};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) c2w[i * 4 + j] = (float)R[i][j];
    c2w[i * 4 + 3] = r.uni(-3, 3);
  }
  c2w[12] = c2w[13] = c2w[14] = 0.0f;
  c2w[15] = 1.0f;
}

void print_floats(const char *name, const float *v, int n, bool last = false) {
  std::printf("\"%s\": [", name);
  for (int i = 0; i < n; ++i) std::printf("%s%u", i ? "," : "", fb(v[i]));
  std::printf("]%s\n", last ? "" : ",");
}

}  // namespace

int main() {
  Rng r{12345};
  std::printf("{\n");

  // ---- BlockHasher + bucket (vhashing.h:151-152 uses hash % num_buckets) ----
  {
    ark::BlockHasher h;
    std::vector<int> keys;
    std::vector<unsigned long long> hv;
    for (int i = 0; i < 256; ++i) {
      int3 k;
      if (i < 27) {
        k = make_int3(i % 3 - 1, (i / 3) % 3 - 1, i / 9 - 1);
      } else if (i < 200) {
        k = make_int3(r.irange(-300, 300), r.irange(-300, 300), r.irange(-300, 300));
      } else {
        k = make_int3(r.irange(-1048576, 1048575), r.irange(-1048576, 1048575),
                      r.irange(-1048576, 1048575));
      }
      keys.push_back(k.x);
      keys.push_back(k.y);
      keys.push_back(k.z);
      hv.push_back((unsigned long long)h(k));
    }
    std::printf("\"hash_keys\": [");
    for (size_t i = 0; i < keys.size(); ++i) std::printf("%s%d", i ? "," : "", keys[i]);
    std::printf("],\n\"hash_values\": [");
    for (size_t i = 0; i < hv.size(); ++i) std::printf("%s\"%llu\"", i ? "," : "", hv[i]);
    std::printf("],\n");
  }

  // ---- camera math --------------------------------------------------------
  {
    const int N = 512;
    std::vector<float> K(9 * N), P(16 * N), in(4 * N), f2b(3 * N), wpt(3 * N), b2c(3 * N),
        c2b(3 * N);
    std::vector<int> pix(2 * N), c2f(2 * N);
    for (int i = 0; i < N; ++i) {
      float *k = &K[9 * i];
      std::memset(k, 0, 9 * sizeof(float));
      k[0] = r.uni(300, 800);
      k[4] = r.uni(300, 800);
      k[2] = r.uni(150, 400);
      k[5] = r.uni(100, 300);
      k[8] = 1.0f;
      float *c2w = &P[16 * i];
      random_pose(r, c2w);
      int u = r.irange(0, 639), v = r.irange(0, 479);
      float z = r.uni(0.1f, 6.0f);
      pix[2 * i] = u;
      pix[2 * i + 1] = v;
      in[4 * i + 0] = z;
      float3 w = ark::frame2base(u, v, z, k, c2w, nullptr);
      f2b[3 * i] = w.x;
      f2b[3 * i + 1] = w.y;
      f2b[3 * i + 2] = w.z;
      // a world point near the camera's view: project it back
      float pw[3] = {w.x + r.uni(-0.05f, 0.05f), w.y + r.uni(-0.05f, 0.05f),
                     w.z + r.uni(-0.05f, 0.05f)};
      std::memcpy(&wpt[3 * i], pw, sizeof(pw));
      float cam[3];
      ark::base2cam(pw, cam, c2w);
      std::memcpy(&b2c[3 * i], cam, sizeof(cam));
      int pp[2] = {0, 0};
      ark::cam2frame(cam, pp, k);
      c2f[2 * i] = pp[0];
      c2f[2 * i + 1] = pp[1];
      float back[3];
      ark::cam2base(cam, back, c2w);
      std::memcpy(&c2b[3 * i], back, sizeof(back));
    }
    print_floats("cam_K", K.data(), 9 * N);
    print_floats("cam_c2w", P.data(), 16 * N);
    std::printf("\"cam_pix\": [");
    for (int i = 0; i < 2 * N; ++i) std::printf("%s%d", i ? "," : "", pix[i]);
    std::printf("],\n");
    std::vector<float> zs(N);
    for (int i = 0; i < N; ++i) zs[i] = in[4 * i];
    print_floats("cam_z", zs.data(), N);
    print_floats("frame2base", f2b.data(), 3 * N);
    print_floats("world_pt", wpt.data(), 3 * N);
    print_floats("base2cam", b2c.data(), 3 * N);
    std::printf("\"cam2frame\": [");
    for (int i = 0; i < 2 * N; ++i) std::printf("%s%d", i ? "," : "", c2f[i]);
    std::printf("],\n");
    print_floats("cam2base", c2b.data(), 3 * N);
  }

  // ---- VertexInterp ---------------------------------------------------------
  {
    const int N = 400;
    std::vector<float> in(8 * N), out(3 * N);
    std::vector<int> rgbin(6 * N), rgbout(3 * N);
    const float special[] = {0.0f, 1e-6f, -1e-6f, 9.9999e-6f, -9.9999e-6f, 1e-5f, -1e-5f,
                             1.0000001e-5f, 2e-5f, -2e-5f, 0.5f, -0.5f, 1.0f, -1.0f};
    const int ns = sizeof(special) / sizeof(float);
    for (int i = 0; i < N; ++i) {
      ark::Vertex p1((float)r.irange(-50, 50), (float)r.irange(-50, 50), (float)r.irange(-50, 50));
      ark::Vertex p2(p1.x + (float)r.irange(0, 1), p1.y + (float)r.irange(0, 1),
                     p1.z + (float)r.irange(0, 1));
      p1.r = (unsigned char)r.irange(0, 255);
      p1.g = (unsigned char)r.irange(0, 255);
      p1.b = (unsigned char)r.irange(0, 255);
      p2.r = (unsigned char)r.irange(0, 255);
      p2.g = (unsigned char)r.irange(0, 255);
      p2.b = (unsigned char)r.irange(0, 255);
      float v1, v2;
      if (i < ns * ns) {
        v1 = special[i % ns];
        v2 = special[i / ns];
      } else {
        v1 = r.uni(-1, 1);
        v2 = (i & 1) ? -v1 * r.uni(0.1f, 3.0f) : r.uni(-1, 1);
      }
      ark::Vertex o = ark::VertexInterp(0, p1, p2, v1, v2);
      float *q = &in[8 * i];
      q[0] = p1.x; q[1] = p1.y; q[2] = p1.z; q[3] = p2.x; q[4] = p2.y; q[5] = p2.z;
      q[6] = v1; q[7] = v2;
      rgbin[6 * i + 0] = p1.r; rgbin[6 * i + 1] = p1.g; rgbin[6 * i + 2] = p1.b;
      rgbin[6 * i + 3] = p2.r; rgbin[6 * i + 4] = p2.g; rgbin[6 * i + 5] = p2.b;
      out[3 * i] = o.x; out[3 * i + 1] = o.y; out[3 * i + 2] = o.z;
      rgbout[3 * i] = o.r; rgbout[3 * i + 1] = o.g; rgbout[3 * i + 2] = o.b;
    }
    print_floats("vi_in", in.data(), 8 * N);
    print_floats("vi_out", out.data(), 3 * N);
    std::printf("\"vi_rgb_in\": [");
    for (int i = 0; i < 6 * N; ++i) std::printf("%s%d", i ? "," : "", rgbin[i]);
    std::printf("],\n\"vi_rgb_out\": [");
    for (int i = 0; i < 3 * N; ++i) std::printf("%s%d", i ? "," : "", rgbout[i]);
    std::printf("],\n");
  }

  // ---- MC tables --------------------------------------------------------------
  {
    ark::MarchingCubeParam *mp = new ark::MarchingCubeParam();
    std::printf("\"idx_map\": [");
    for (int i = 0; i < 24; ++i) std::printf("%s%d", i ? "," : "", mp->idxMap[i / 3][i % 3]);
    std::printf("],\n\"edge_table\": [");
    for (int i = 0; i < 256; ++i) std::printf("%s%d", i ? "," : "", mp->edgeTable[i]);
    std::printf("],\n\"tri_table\": [");
    for (int i = 0; i < 256 * 16; ++i) std::printf("%s%d", i ? "," : "", mp->triTable[i / 16][i % 16]);
    std::printf("],\n");
    delete mp;
  }

  // ---- host hash table (insert / erase / find) ---------------------------------
  {
    typedef vhashing::HashTable<int3, ark::VoxelBlock, ark::BlockHasher, ark::BlockEqual,
                                vhashing::std_memspace>
        Table;
    Table t(211, 2, 600, make_int3(999999, 999999, 999999));  // 422 entries >= 300 inserts
    std::vector<int> ops;  // op, x, y, z, result
    for (int i = 0; i < 300; ++i) {
      int3 k = make_int3(r.irange(-6, 6), r.irange(-6, 6), r.irange(-2, 2));
      int before = *t.heap_counter;
      t[k];  // write-path operator[] inserts if absent (vhashing.h:205-239)
      int inserted = *t.heap_counter - before;
      ops.insert(ops.end(), {0, k.x, k.y, k.z, inserted});
    }
    for (int i = 0; i < 120; ++i) {
      int3 k = make_int3(r.irange(-6, 6), r.irange(-6, 6), r.irange(-2, 2));
      int erased = (int)t.erase(k);
      ops.insert(ops.end(), {1, k.x, k.y, k.z, erased});
    }
    for (int i = 0; i < 300; ++i) {
      int3 k = make_int3(r.irange(-7, 7), r.irange(-7, 7), r.irange(-3, 3));
      int found = t.find(k) != t.end();
      ops.insert(ops.end(), {2, k.x, k.y, k.z, found});
    }
    std::printf("\"hash_ops\": [");
    for (size_t i = 0; i < ops.size(); ++i) std::printf("%s%d", i ? "," : "", ops[i]);
    std::printf("],\n\"hash_heap_counter\": %d\n", *t.heap_counter);
  }
  std::printf("}\n");
  return 0;
}

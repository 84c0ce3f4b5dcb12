// vh_adjoint.cu - differentiable TSDF queries for pose refinement.
//
// The reference has no gradients; this file adds them on top of the fused
// volume (benchmark configuration "differentiable pose refinement"):
//   * trilinear sampling of the TSDF at world points together with its
//     analytic gradient (the adjoint of sampling);
//   * per-pixel SDF residuals of a back-projected depth frame and their
//     Jacobians with respect to a left se(3) perturbation of the camera pose,
//     reduced on the GPU to 6x6 Gauss-Newton normal equations;
//   * the same normal equations from forward-only central differences (the
//     plain FD-Jacobian method: 13 residual evaluations per step), for
//     comparison;
//   * the vector-Jacobian product of one integration update with respect to
//     the per-pixel depths and the camera pose, recomputed from the volume
//     (no per-frame tape).
//
// Voxel i is centred at i * voxel_size (the reference's convention), so the
// continuous voxel coordinate of a world point is p / voxel_size.  The TSDF
// stores sdf in units of the truncation distance T; residuals here are in
// metres (T * sdf).

#include <cmath>
#include <cstring>
#include <vector>

#include "vh_device.cuh"
#include "vh_internal.h"

namespace vh {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kTerms = 29;  // 21 (upper H) + 6 (J^T r) + sum r^2 + count

struct Sample {
  bool ok;
  float phi, gx, gy, gz;  // sdf (units of T) and d sdf / d world (per metre)
};

__device__ __forceinline__ uint32_t nb_block(const VolumeView &V, int bx, int by, int bz) {
  return key_in_range(bx, by, bz) ? block_of(V, pack_key(bx, by, bz)) : kNoBlock;
}

// Trilinear interpolation of the TSDF at world point (x, y, z) and its
// gradient.  Fails when any of the 8 corner voxels is unallocated or has a
// weight below min_w.
__device__ Sample sample_tsdf(const VolumeView &V, float inv_voxel, float min_w, float x, float y,
                              float z) {
  Sample s;
  s.ok = false;
  const float qx = x * inv_voxel, qy = y * inv_voxel, qz = z * inv_voxel;
  if (!(fabsf(qx) < 8.0e6f && fabsf(qy) < 8.0e6f && fabsf(qz) < 8.0e6f)) return s;
  const float fxb = floorf(qx), fyb = floorf(qy), fzb = floorf(qz);
  const int ix = (int)fxb, iy = (int)fyb, iz = (int)fzb;
  const float fx = qx - fxb, fy = qy - fyb, fz = qz - fzb;
  const int bx = ix >> 3, by = iy >> 3, bz = iz >> 3;  // floor division
  const int lx = ix & 7, ly = iy & 7, lz = iz & 7;
  const bool cx = lx == 7, cy = ly == 7, cz = lz == 7;  // corners cross into +1 blocks
  uint32_t b[8];
  b[0] = nb_block(V, bx, by, bz);
  b[1] = cx ? nb_block(V, bx + 1, by, bz) : b[0];
  b[2] = cy ? nb_block(V, bx, by + 1, bz) : b[0];
  b[3] = cx && cy ? nb_block(V, bx + 1, by + 1, bz) : (cx ? b[1] : b[2]);
  b[4] = cz ? nb_block(V, bx, by, bz + 1) : b[0];
  b[5] = cz ? (cx ? nb_block(V, bx + 1, by, bz + 1) : b[4]) : b[1];
  b[6] = cz ? (cy ? nb_block(V, bx, by + 1, bz + 1) : b[4]) : b[2];
  b[7] = cz ? ((cx || cy) ? nb_block(V, bx + cx, by + cy, bz + 1) : b[4]) : b[3];
  float val[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
    if (b[c] == kNoBlock) return s;
    const int li = ((lx + dx) & 7) + 8 * ((ly + dy) & 7) + 64 * ((lz + dz) & 7);
    const float *base = V.pool + (size_t)b[c] * kBlockWords;
    const float w = __ldg(base + kB3 + li);
    if (w < min_w) return s;
    val[c] = __ldg(base + li);
  }
  const float gx0 = 1.0f - fx, gy0 = 1.0f - fy, gz0 = 1.0f - fz;
  // phi = sum_c w_c val_c, w_c = (dx ? fx : 1-fx)(dy ? fy : 1-fy)(dz ? fz : 1-fz)
  const float c00 = val[0] * gx0 + val[1] * fx, c10 = val[2] * gx0 + val[3] * fx;
  const float c01 = val[4] * gx0 + val[5] * fx, c11 = val[6] * gx0 + val[7] * fx;
  const float c0 = c00 * gy0 + c10 * fy, c1 = c01 * gy0 + c11 * fy;
  s.phi = c0 * gz0 + c1 * fz;
  const float d00 = val[1] - val[0], d10 = val[3] - val[2];
  const float d01 = val[5] - val[4], d11 = val[7] - val[6];
  const float dphidx = (d00 * gy0 + d10 * fy) * gz0 + (d01 * gy0 + d11 * fy) * fz;
  const float dphidy = (c10 - c00) * gz0 + (c11 - c01) * fz;
  const float dphidz = c1 - c0;
  s.gx = dphidx * inv_voxel;
  s.gy = dphidy * inv_voxel;
  s.gz = dphidz * inv_voxel;
  s.ok = true;
  return s;
}

__global__ void __launch_bounds__(256) k_sdf_sample(VolumeView V, float inv_voxel, float min_w,
                                                    const float *__restrict__ xyz, uint32_t n,
                                                    float *__restrict__ phi,
                                                    float *__restrict__ grad,
                                                    uint8_t *__restrict__ valid) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Sample s = sample_tsdf(V, inv_voxel, min_w, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  phi[i] = s.ok ? s.phi : 0.0f;
  if (grad) {
    grad[3 * i] = s.ok ? s.gx : 0.0f;
    grad[3 * i + 1] = s.ok ? s.gy : 0.0f;
    grad[3 * i + 2] = s.ok ? s.gz : 0.0f;
  }
  if (valid) valid[i] = s.ok;
}

// Back-projected world point of pixel (u, v) with depth d under pose P
// (row-major 3x4): frame2cam then cam2base (src/tsdf.cu:67-74, 95-106).
struct Px {
  bool ok;
  float x, y, z;
};

__device__ __forceinline__ float pixel_depth(const void *depth, int fmt, int idx, float scale) {
  return fmt == 0 ? (float)__ldg(static_cast<const uint16_t *>(depth) + idx) * scale
                  : __ldg(static_cast<const float *>(depth) + idx);
}

__device__ __forceinline__ Px backproject(const CamParams &C, const float *P, int u, int v,
                                          float d) {
  Px r;
  r.ok = d > C.min_depth && d <= C.max_depth;
  const float cx = (((float)u - C.cx) * d) / C.fx;
  const float cy = (((float)v - C.cy) * d) / C.fy;
  r.x = cx * P[0] + cy * P[1] + d * P[2] + P[3];
  r.y = cx * P[4] + cy * P[5] + d * P[6] + P[7];
  r.z = cx * P[8] + cy * P[9] + d * P[10] + P[11];
  return r;
}

// Sums the kTerms values of every thread of the CTA into out[kTerms].
template <int kThreads>
__device__ __forceinline__ void cta_sum_terms(float (&v)[kTerms], float *out) {
  __shared__ float part[kThreads / 32][kTerms];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kTerms; ++k) {
    float x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
    if (lane == 0) part[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < kTerms) {
    float x = 0.0f;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) x += part[w][threadIdx.x];
    out[threadIdx.x] = x;
  }
}

// Adds r, J (6) of one residual to the normal-equation terms.
__device__ __forceinline__ void add_terms(float (&v)[kTerms], float r, const float (&J)[6]) {
  int k = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = a; b < 6; ++b) v[k++] += J[a] * J[b];
#pragma unroll
  for (int a = 0; a < 6; ++a) v[21 + a] += J[a] * r;
  v[27] += r * r;
  v[28] += 1.0f;
}

// Adjoint normal equations: per sampled pixel, r = T * sdf(X_w) and
// J = dr / d(v, w) for X_w -> X_w + v + w x X_w, i.e. T * [g ; X_w x g].
// Pixels whose sample is invalid or truncated (|sdf| >= 1) are skipped.
__global__ void __launch_bounds__(256) k_pose_terms(VolumeView V, CamParams C, const void *depth,
                                                    int fmt, const float *__restrict__ pose,
                                                    int stride, float inv_voxel,
                                                    float *__restrict__ partials) {
  float P[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = __ldg(pose + k);
  float acc[kTerms];
#pragma unroll
  for (int k = 0; k < kTerms; ++k) acc[k] = 0.0f;
  const int ws = (C.width + stride - 1) / stride, hs = (C.height + stride - 1) / stride;
  const int npx = ws * hs;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < npx; q += gridDim.x * blockDim.x) {
    const int u = (q % ws) * stride, v = (q / ws) * stride;
    const float d = pixel_depth(depth, fmt, v * C.width + u, C.depth_scale);
    const Px X = backproject(C, P, u, v, d);
    if (!X.ok) continue;
    const Sample s = sample_tsdf(V, inv_voxel, C.mc_min_weight, X.x, X.y, X.z);
    if (!s.ok || !(fabsf(s.phi) < 1.0f)) continue;
    const float T = C.trunc;
    const float J[6] = {T * s.gx, T * s.gy, T * s.gz, T * (X.y * s.gz - X.z * s.gy),
                        T * (X.z * s.gx - X.x * s.gz), T * (X.x * s.gy - X.y * s.gx)};
    add_terms(acc, T * s.phi, J);
  }
  cta_sum_terms<256>(acc, partials + (size_t)blockIdx.x * kTerms);
}

// Residuals of every sampled pixel under `np` poses (forward only): r = T *
// sdf, NaN where invalid or truncated.
__global__ void __launch_bounds__(256) k_pose_residuals(VolumeView V, CamParams C,
                                                        const void *depth, int fmt,
                                                        const float *__restrict__ poses, int np,
                                                        int stride, float inv_voxel,
                                                        float *__restrict__ res) {
  const int ws = (C.width + stride - 1) / stride, hs = (C.height + stride - 1) / stride;
  const int npx = ws * hs;
  const int pi = blockIdx.y;
  if (pi >= np) return;
  float P[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = __ldg(poses + 12 * pi + k);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < npx; q += gridDim.x * blockDim.x) {
    const int u = (q % ws) * stride, v = (q / ws) * stride;
    const float d = pixel_depth(depth, fmt, v * C.width + u, C.depth_scale);
    const Px X = backproject(C, P, u, v, d);
    float r = __int_as_float(0x7FC00000);
    if (X.ok) {
      const Sample s = sample_tsdf(V, inv_voxel, C.mc_min_weight, X.x, X.y, X.z);
      if (s.ok && fabsf(s.phi) < 1.0f) r = C.trunc * s.phi;
    }
    res[(size_t)pi * npx + q] = r;
  }
}

// Normal equations from the 13 residual vectors of the FD method: pose 0 is
// the current estimate, poses 1 + 2k and 2 + 2k are the +/- steps of
// coordinate k; pixels valid under all 13 poses contribute.
__global__ void __launch_bounds__(256) k_fd_terms(const float *__restrict__ res, int npx,
                                                  const float *__restrict__ inv2eps,
                                                  float *__restrict__ partials) {
  float acc[kTerms];
#pragma unroll
  for (int k = 0; k < kTerms; ++k) acc[k] = 0.0f;
  float ie[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) ie[k] = __ldg(inv2eps + k);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < npx; q += gridDim.x * blockDim.x) {
    const float r0 = res[q];
    bool ok = r0 == r0;
    float J[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float rp = res[(size_t)(1 + 2 * k) * npx + q], rm = res[(size_t)(2 + 2 * k) * npx + q];
      ok = ok && rp == rp && rm == rm;
      J[k] = (rp - rm) * ie[k];
    }
    if (ok) add_terms(acc, r0, J);
  }
  cta_sum_terms<256>(acc, partials + (size_t)blockIdx.x * kTerms);
}

// Sums `n` CTA partials in a fixed order (deterministic) into out[kTerms].
__global__ void k_sum_partials(const float *__restrict__ partials, int n, float *__restrict__ out) {
  const int k = threadIdx.x;
  if (k >= kTerms) return;
  float x = 0.0f;
  for (int i = 0; i < n; ++i) x += partials[(size_t)i * kTerms + k];
  out[k] = x;
}

// Vector-Jacobian product of the last integration update.  For a voxel v of
// the frame's block list that the update touched (recomputed: same tests as
// the forward pass, src/tsdf.cu:706-721), sdf_new = (sdf_old * w + dist) /
// (w + 1) with dist = min(1, (d_p - z_v) / T) and w the weight before the
// update (stored weight - 1).  Given G_v = dL/dsdf_new (frame-list order, 512
// per block, x-fastest), this accumulates
//   dL/dd_p  += G_v / ((w + 1) T)                       (unclamped voxels)
//   dL/dxi   += -G_v / ((w + 1) T) * dz_v/dxi,  dz/dv = -r3, dz/dw = r3 x X_v
// for the left perturbation c2w -> exp(xi) c2w (r3 = camera z axis in world).
// The pixel choice is piecewise constant and contributes nothing.
__global__ void __launch_bounds__(128) k_integrate_vjp(VolumeView V, CamParams C,
                                                       const void *depth, int fmt,
                                                       const float *__restrict__ pose,
                                                       const float *__restrict__ gsdf,
                                                       float *__restrict__ gdepth,
                                                       float *__restrict__ partials) {
  const uint32_t n = min(V.st->frame_count, V.frame_cap);
  float P[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = __ldg(pose + k);
  float acc[kTerms];
#pragma unroll
  for (int k = 0; k < kTerms; ++k) acc[k] = 0.0f;
  const int t = threadIdx.x;
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const ulonglong2 r = __ldg(V.frame_res + i);
    if (r.x >= kTombKey || (uint32_t)r.y == kNoBlock) continue;
    int bx, by, bz;
    unpack_key(r.x, bx, by, bz);
    const float *base = V.pool + (size_t)(uint32_t)r.y * kBlockWords;
    for (int li = t; li < kB3; li += blockDim.x) {
      const float g = __ldg(gsdf + (size_t)i * kB3 + li);
      if (g == 0.0f) continue;
      const int ix = bx * kB + (li & 7), iy = by * kB + ((li >> 3) & 7), iz = bz * kB + (li >> 6);
      const float wx = (float)ix * C.voxel, wy = (float)iy * C.voxel, wz = (float)iz * C.voxel;
      const float t0 = wx - P[3], t1 = wy - P[7], t2 = wz - P[11];
      const float x = (P[0] * t0 + P[4] * t1) + P[8] * t2;
      const float y = (P[1] * t0 + P[5] * t1) + P[9] * t2;
      const float z = (P[2] * t0 + P[6] * t1) + P[10] * t2;
      if (!(z > 0.0f)) continue;
      const float uf = roundf(C.fx * (x / z) + C.cx), vf = roundf(C.fy * (y / z) + C.cy);
      if (!(uf >= 0.0f && uf < C.wf && vf >= 0.0f && vf < C.hf)) continue;
      const int p = (int)vf * C.width + (int)uf;
      const float d = pixel_depth(depth, fmt, p, C.depth_scale);
      if (!(d > 0.0f && d <= C.max_depth)) continue;
      const float diff = d - z;
      if (diff <= -C.trunc || diff >= C.trunc) continue;  // skipped, or dist clamped at 1
      const float w_new = __ldg(base + kB3 + li);  // weight after the update
      const float k = g / (w_new * C.trunc);        // dL/ddist / T
      atomicAdd(gdepth + p, k);
      // dL/dz = -k; dz/dv = -r3, dz/dw = r3 x X  (r3 = column 2 of R)
      const float r3x = P[2], r3y = P[6], r3z = P[10];
      acc[0] += k * r3x;
      acc[1] += k * r3y;
      acc[2] += k * r3z;
      acc[3] -= k * (r3y * wz - r3z * wy);
      acc[4] -= k * (r3z * wx - r3x * wz);
      acc[5] -= k * (r3x * wy - r3y * wx);
    }
  }
  cta_sum_terms<128>(acc, partials + (size_t)blockIdx.x * kTerms);
}

}  // namespace
}  // namespace vh

// ---- host side ----------------------------------------------------------------
using namespace vh;

namespace {

// Rigid transform in double precision (pose composition happens here).
struct Pose {
  double R[3][3];
  double t[3];
};

Pose pose_from(const float *c2w) {
  Pose p;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) p.R[r][c] = c2w[4 * r + c];
    p.t[r] = c2w[4 * r + 3];
  }
  return p;
}

void pose_to(const Pose &p, float *c2w) {
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) c2w[4 * r + c] = (float)p.R[r][c];
    c2w[4 * r + 3] = (float)p.t[r];
  }
  c2w[12] = c2w[13] = c2w[14] = 0.0f;
  c2w[15] = 1.0f;
}

// exp(xi) * p for xi = (v, w): the SE(3) exponential (Rodrigues for the
// rotation, the left Jacobian for the translation).
Pose left_exp(const double xi[6], const Pose &p) {
  const double wx = xi[3], wy = xi[4], wz = xi[5];
  const double th2 = wx * wx + wy * wy + wz * wz, th = std::sqrt(th2);
  double A, B, Cc;
  if (th < 1e-6) {
    A = 1.0 - th2 / 6.0;
    B = 0.5 - th2 / 24.0;
    Cc = 1.0 / 6.0 - th2 / 120.0;
  } else {
    A = std::sin(th) / th;
    B = (1.0 - std::cos(th)) / th2;
    Cc = (th - std::sin(th)) / (th2 * th);
  }
  const double W[3][3] = {{0, -wz, wy}, {wz, 0, -wx}, {-wy, wx, 0}};
  double W2[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      W2[r][c] = 0;
      for (int k = 0; k < 3; ++k) W2[r][c] += W[r][k] * W[k][c];
    }
  double dR[3][3], Vm[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      const double I = r == c ? 1.0 : 0.0;
      dR[r][c] = I + A * W[r][c] + B * W2[r][c];
      Vm[r][c] = I + B * W[r][c] + Cc * W2[r][c];
    }
  double dt[3];
  for (int r = 0; r < 3; ++r) dt[r] = Vm[r][0] * xi[0] + Vm[r][1] * xi[1] + Vm[r][2] * xi[2];
  Pose q;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c)
      q.R[r][c] = dR[r][0] * p.R[0][c] + dR[r][1] * p.R[1][c] + dR[r][2] * p.R[2][c];
    q.t[r] = dR[r][0] * p.t[0] + dR[r][1] * p.t[1] + dR[r][2] * p.t[2] + dt[r];
  }
  return q;
}

void pose_rows(const Pose &p, float *out12) {
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) out12[4 * r + c] = (float)p.R[r][c];
    out12[4 * r + 3] = (float)p.t[r];
  }
}

// Solves (H + damp * diag(H)) x = -g for the 6x6 system given by the 29
// terms (upper triangle row by row, then g).  Returns false if singular.
bool solve_step(const double terms[29], double damp, double x[6]) {
  double H[6][6], g[6];
  int k = 0;
  for (int a = 0; a < 6; ++a)
    for (int b = a; b < 6; ++b) H[a][b] = H[b][a] = terms[k++];
  for (int a = 0; a < 6; ++a) g[a] = terms[21 + a];
  for (int a = 0; a < 6; ++a) H[a][a] *= 1.0 + damp;
  double L[6][6] = {};
  for (int i = 0; i < 6; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = H[i][j];
      for (int m = 0; m < j; ++m) s -= L[i][m] * L[j][m];
      if (i == j) {
        if (!(s > 0.0)) return false;
        L[i][i] = std::sqrt(s);
      } else {
        L[i][j] = s / L[j][j];
      }
    }
  }
  double y[6];
  for (int i = 0; i < 6; ++i) {
    double s = -g[i];
    for (int m = 0; m < i; ++m) s -= L[i][m] * y[m];
    y[i] = s / L[i][i];
  }
  for (int i = 5; i >= 0; --i) {
    double s = y[i];
    for (int m = i + 1; m < 6; ++m) s -= L[m][i] * x[m];
    x[i] = s / L[i][i];
  }
  return true;
}

struct RefineWork {
  float *poses;     // 13 x 12
  float *inv2eps;   // 6
  float *partials;  // grid x kTerms
  float *terms;     // kTerms
  float *res;       // 13 x npx (FD method)
  int grid;
  int npx;
};

vh_status refine_work(vh_handle *h, int stride, bool fd, RefineWork *w) {
  const CamParams C = vh::handle_cam(h);
  const int ws = (C.width + stride - 1) / stride, hs = (C.height + stride - 1) / stride;
  w->npx = ws * hs;
  w->grid = vh::handle_sm_count(h) * 4;
  const size_t floats = 13 * 12 + 8 + (size_t)w->grid * kTerms + 32 + (fd ? 13 * (size_t)w->npx : 0);
  void *p = nullptr;
  vh_status s = vh::handle_workspace(h, floats * sizeof(float), &p);
  if (s != VH_OK) return s;
  float *f = static_cast<float *>(p);
  w->poses = f;
  w->inv2eps = f + 13 * 12;
  w->partials = w->inv2eps + 8;
  w->terms = w->partials + (size_t)w->grid * kTerms;
  w->res = fd ? w->terms + 32 : nullptr;
  return VH_OK;
}

const double kFdStep[6] = {1e-4, 1e-4, 1e-4, 1e-4, 1e-4, 1e-4};

// One linearisation at `pose`: normal-equation terms in double.
vh_status linearise(vh_handle *h, const void *depth, int fmt, const Pose &pose, int stride,
                    int method, const RefineWork &w, double out[29]) {
  const VolumeView V = vh::handle_view(h);
  CamParams C = vh::handle_cam(h);
  C.mc_min_weight = C.mc_min_weight < 1.0f ? 1.0f : C.mc_min_weight;  // observed corners only
  const cudaStream_t st = vh::handle_stream(h);
  const float inv_voxel = 1.0f / C.voxel;
  float host[13 * 12];
  if (method == VH_REFINE_FD) {
    pose_rows(pose, host);
    for (int k = 0; k < 6; ++k)
      for (int sgn = 0; sgn < 2; ++sgn) {
        double xi[6] = {0, 0, 0, 0, 0, 0};
        xi[k] = sgn == 0 ? kFdStep[k] : -kFdStep[k];
        pose_rows(left_exp(xi, pose), host + 12 * (1 + 2 * k + sgn));
      }
    float ie[8];
    for (int k = 0; k < 6; ++k) ie[k] = (float)(0.5 / kFdStep[k]);
    if (cudaMemcpyAsync(w.poses, host, sizeof(host), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(w.inv2eps, ie, 6 * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "pose upload failed");
    const int gx = (w.npx + 255) / 256 < w.grid ? (w.npx + 255) / 256 : w.grid;
    k_pose_residuals<<<dim3(gx, 13), 256, 0, st>>>(V, C, depth, fmt, w.poses, 13, stride,
                                                     inv_voxel, w.res);
    k_fd_terms<<<w.grid, 256, 0, st>>>(w.res, w.npx, w.inv2eps, w.partials);
  } else {
    pose_rows(pose, host);
    if (cudaMemcpyAsync(w.poses, host, 12 * sizeof(float), cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "pose upload failed");
    k_pose_terms<<<w.grid, 256, 0, st>>>(V, C, depth, fmt, w.poses, stride, inv_voxel, w.partials);
  }
  k_sum_partials<<<1, 32, 0, st>>>(w.partials, w.grid, w.terms);
  float t[kTerms];
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(t, w.terms, sizeof(t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "normal equations failed");
  for (int k = 0; k < kTerms; ++k) out[k] = t[k];
  return VH_OK;
}

}  // namespace

extern "C" vh_status vh_sdf_sample(vh_handle *h, const float *xyz, int64_t n, float *phi,
                                   float *grad, uint8_t *valid, int32_t mem) {
  if (!h || n < 0 || (n && (!xyz || !phi)) || n > (1ll << 30)) return VH_ERR_INVALID_ARG;
  if (mem != VH_MEM_HOST && mem != VH_MEM_DEVICE) return VH_ERR_INVALID_ARG;
  if (!n) return VH_OK;
  const cudaStream_t st = vh::handle_stream(h);
  const CamParams C = vh::handle_cam(h);
  const float *dx = xyz;
  float *dphi = phi, *dgrad = grad;
  uint8_t *dvalid = valid;
  const size_t bytes = (size_t)n * (3 + 1 + 3) * sizeof(float) + (size_t)n + 256;
  if (mem == VH_MEM_HOST) {
    void *p = nullptr;
    vh_status s = vh::handle_workspace(h, bytes, &p);
    if (s != VH_OK) return s;
    float *f = static_cast<float *>(p);
    dx = f;
    dphi = f + 3 * n;
    dgrad = grad ? f + 4 * n : nullptr;
    dvalid = valid ? reinterpret_cast<uint8_t *>(f + 7 * n) : nullptr;
    if (cudaMemcpyAsync(f, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "point upload failed");
  }
  k_sdf_sample<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      vh::handle_view(h), 1.0f / C.voxel, C.mc_min_weight < 1.0f ? 1.0f : C.mc_min_weight, dx,
      (uint32_t)n, dphi, dgrad, dvalid);
  if (cudaGetLastError() != cudaSuccess) return vh::handle_fail(h, VH_ERR_CUDA, "sample launch");
  if (mem == VH_MEM_HOST) {
    bool ok = cudaMemcpyAsync(phi, dphi, sizeof(float) * n, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (grad)
      ok = ok && cudaMemcpyAsync(grad, dgrad, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st) ==
                     cudaSuccess;
    if (valid)
      ok = ok && cudaMemcpyAsync(valid, dvalid, (size_t)n, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (!ok) return vh::handle_fail(h, VH_ERR_CUDA, "sample download failed");
  }
  return vh::handle_sync(h);
}

extern "C" vh_status vh_pose_normal_equations(vh_handle *h, const void *depth, int32_t depth_fmt,
                                              int32_t mem, const float *c2w, int32_t stride,
                                              int32_t method, double *terms) {
  if (!h || !c2w || !terms || stride < 1 || (method != VH_REFINE_ADJOINT && method != VH_REFINE_FD))
    return VH_ERR_INVALID_ARG;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(c2w[i])) return VH_ERR_NOT_FINITE;
  const void *d = nullptr;
  vh_status s = vh::handle_stage_depth(h, depth, depth_fmt, mem, &d);
  if (s != VH_OK) return s;
  RefineWork w;
  if ((s = refine_work(h, stride, method == VH_REFINE_FD, &w)) != VH_OK) return s;
  return linearise(h, d, depth_fmt, pose_from(c2w), stride, method, w, terms);
}

extern "C" vh_status vh_pose_refine(vh_handle *h, const void *depth, int32_t depth_fmt, int32_t mem,
                                    const float *c2w_init, int32_t iterations, int32_t stride,
                                    int32_t method, float *c2w_out, vh_refine_stats *stats) {
  if (!h || !c2w_init || !c2w_out || iterations < 0 || stride < 1 ||
      (method != VH_REFINE_ADJOINT && method != VH_REFINE_FD))
    return VH_ERR_INVALID_ARG;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(c2w_init[i])) return VH_ERR_NOT_FINITE;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const cudaStream_t st = vh::handle_stream(h);
  cudaEventRecord(e0, st);
  const void *d = nullptr;
  vh_status s = vh::handle_stage_depth(h, depth, depth_fmt, mem, &d);
  RefineWork w;
  if (s == VH_OK) s = refine_work(h, stride, method == VH_REFINE_FD, &w);
  Pose pose = pose_from(c2w_init);
  double terms[29] = {0};
  double rmse0 = 0.0, rmse = 0.0;
  int valid = 0, done = 0;
  for (int it = 0; it < iterations && s == VH_OK; ++it) {
    s = linearise(h, d, depth_fmt, pose, stride, method, w, terms);
    if (s != VH_OK) break;
    valid = (int)terms[28];
    rmse = valid ? std::sqrt(terms[27] / valid) : 0.0;
    if (it == 0) rmse0 = rmse;
    double xi[6];
    if (valid < 6 || !solve_step(terms, 1e-6, xi)) break;
    pose = left_exp(xi, pose);
    ++done;
  }
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  pose_to(pose, c2w_out);
  if (stats) {
    stats->iterations = done;
    stats->valid_pixels = valid;
    stats->initial_rmse = (float)rmse0;
    stats->final_rmse = (float)rmse;
    stats->ms = ms;
  }
  return s;
}

extern "C" vh_status vh_integrate_vjp(vh_handle *h, const void *depth, int32_t depth_fmt,
                                      const float *c2w, const float *grad_sdf, float *grad_depth,
                                      float *grad_pose, int32_t mem) {
  if (!h || !c2w || !grad_sdf || !grad_depth || !grad_pose) return VH_ERR_INVALID_ARG;
  if (mem != VH_MEM_HOST && mem != VH_MEM_DEVICE) return VH_ERR_INVALID_ARG;
  const cudaStream_t st = vh::handle_stream(h);
  const VolumeView V = vh::handle_view(h);
  const CamParams C = vh::handle_cam(h);
  // frame-list length (the upstream gradient holds 512 values per entry)
  vh::DevState ds;
  if (cudaMemcpyAsync(&ds, V.st, sizeof(ds), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "state read failed");
  const size_t nb = ds.frame_count < V.frame_cap ? ds.frame_count : V.frame_cap;
  const size_t npx = (size_t)C.width * C.height;
  const void *d = nullptr;
  vh_status s = vh::handle_stage_depth(h, depth, depth_fmt, mem, &d);
  if (s != VH_OK) return s;
  const int grid = vh::handle_sm_count(h) * 8;
  const size_t floats = 16 + (size_t)grid * kTerms + 32 + npx + (mem == VH_MEM_HOST ? nb * 512 : 0);
  void *p = nullptr;
  if ((s = vh::handle_workspace(h, floats * sizeof(float), &p)) != VH_OK) return s;
  float *f = static_cast<float *>(p);
  float *dpose = f, *partials = f + 16, *terms = partials + (size_t)grid * kTerms;
  float *dgd = mem == VH_MEM_HOST ? terms + 32 : grad_depth;
  const float *dg = grad_sdf;
  if (mem == VH_MEM_HOST) {
    float *tmp = terms + 32 + npx;
    if (nb && cudaMemcpyAsync(tmp, grad_sdf, sizeof(float) * nb * 512, cudaMemcpyHostToDevice, st) !=
                  cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "gradient upload failed");
    dg = tmp;
  }
  float rows[12];
  pose_rows(pose_from(c2w), rows);
  if (cudaMemcpyAsync(dpose, rows, sizeof(rows), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(dgd, 0, sizeof(float) * npx, st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "vjp set-up failed");
  k_integrate_vjp<<<grid, 128, 0, st>>>(V, C, d, depth_fmt, dpose, dg, dgd, partials);
  k_sum_partials<<<1, 32, 0, st>>>(partials, grid, terms);
  float t[kTerms];
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(t, terms, sizeof(t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "vjp failed");
  if (mem == VH_MEM_HOST &&
      cudaMemcpyAsync(grad_depth, dgd, sizeof(float) * npx, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "vjp download failed");
  s = vh::handle_sync(h);
  for (int k = 0; k < 6; ++k) grad_pose[k] = t[k];
  return s;
}

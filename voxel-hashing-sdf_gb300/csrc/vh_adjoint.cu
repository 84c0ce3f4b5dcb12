// vh_adjoint.cu - differentiable TSDF queries for pose refinement.
//
// The reference has no gradients; this file adds them on top of the fused
// volume (benchmark configuration "differentiable pose refinement"):
//   * trilinear sampling of the TSDF at world points together with its
//     analytic gradient (the adjoint of sampling);
//   * per-pixel SDF residuals of a back-projected depth frame and their
//     Jacobians with respect to a left se(3) perturbation of the camera pose,
//     reduced on the GPU to 6x6 Gauss-Newton normal equations, solved and
//     composed with the pose on the device (FP64) so that a refinement runs
//     its steps without host round trips;
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
#include <cstdint>
#include <cstring>

#include "vh_device.cuh"
#include "vh_internal.h"

namespace vh {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kTerms = 29;  // 21 (upper H) + 6 (J^T r) + sum r^2 + count

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

// Warp sum of 32 values per lane by a transposing butterfly: at offset o a
// lane keeps the half of its remaining values selected by bit o of its lane
// index and adds its partner's copy of that half, so 16 + 8 + 4 + 2 + 1
// shuffles leave lane l with the warp sum of value l (in a fixed order).
__device__ __forceinline__ float warp_transpose_sum(float (&a)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const bool up = lane & o;
#pragma unroll
    for (int i = 0; i < o; ++i) {
      const float send = up ? a[i] : a[i + o];
      const float keep = up ? a[i + o] : a[i];
      a[i] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
  return a[0];
}

// Sums the kTerms values of every thread of the CTA into out[k * stride]:
// a transposing warp sum, then the warps' sums by warp 0 the same way.
template <int kThreads>
__device__ __forceinline__ void cta_sum_terms(float (&v)[kTerms], float *out, int stride = 1) {
  constexpr int kWarps = kThreads / 32;
  static_assert(kWarps <= 32, "one value per lane in the second stage");
  __shared__ float part[kWarps][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float a[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) a[k] = k < kTerms ? v[k] : 0.0f;
  part[warp][lane] = warp_transpose_sum(a);
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = lane < kWarps ? part[lane][k] : 0.0f;
    const float x = warp_transpose_sum(a);
    if (lane < kTerms) out[lane * stride] = x;
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

// ---- Gauss-Newton pose refinement on the device -----------------------------
//
// A pose is a row-major 3x4 camera-to-world matrix.  The master copy is FP64
// (pose composition); the kernels back-project with an FP32 copy.

__host__ __device__ constexpr double inv_factorial(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= i;
  return 1.0 / f;
}

// Coefficients A = sin t / t, B = (1 - cos t) / t^2, C = (t - sin t) / t^3 of
// the SE(3) exponential, t^2 = th2 (host, FP64).  Below t = 0.25 rad they are
// summed from their Taylor series, sum_n (-1)^n t^2n / (2n + k)! for
// k = 1, 2, 3, to seven terms (the first term left out is below 1e-20);
// larger angles use sin and cos.
inline void exp_coeffs(double th2, double &A, double &B, double &C) {
  if (th2 < 0.0625) {
    // coefficients fixed at compile time: (-1)^n / (2n + k)!
    constexpr double a0 = inv_factorial(1), a1 = -inv_factorial(3), a2 = inv_factorial(5),
                     a3 = -inv_factorial(7), a4 = inv_factorial(9), a5 = -inv_factorial(11),
                     a6 = inv_factorial(13);
    constexpr double b0 = inv_factorial(2), b1 = -inv_factorial(4), b2 = inv_factorial(6),
                     b3 = -inv_factorial(8), b4 = inv_factorial(10), b5 = -inv_factorial(12),
                     b6 = inv_factorial(14);
    constexpr double c0 = inv_factorial(3), c1 = -inv_factorial(5), c2 = inv_factorial(7),
                     c3 = -inv_factorial(9), c4 = inv_factorial(11), c5 = -inv_factorial(13),
                     c6 = inv_factorial(15);
    const double x = th2;
    A = a0 + x * (a1 + x * (a2 + x * (a3 + x * (a4 + x * (a5 + x * a6)))));
    B = b0 + x * (b1 + x * (b2 + x * (b3 + x * (b4 + x * (b5 + x * b6)))));
    C = c0 + x * (c1 + x * (c2 + x * (c3 + x * (c4 + x * (c5 + x * c6)))));
  } else {
    const double th = sqrt(th2);
    A = sin(th) / th;
    B = (1.0 - cos(th)) / th2;
    C = (th - sin(th)) / (th2 * th);
  }
}

// exp(xi) * P for xi = (v, w) (host, FP64): Rodrigues for the rotation, the
// left Jacobian of SO(3) for the translation, with W^2 = w w^T - |w|^2 I.
inline void se3_left_exp(const double xi[6], const double P[12], double Q[12]) {
  const double w[3] = {xi[3], xi[4], xi[5]};
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  double A, B, Cc;
  exp_coeffs(th2, A, B, Cc);
  const double W[3][3] = {{0, -w[2], w[1]}, {w[2], 0, -w[0]}, {-w[1], w[0], 0}};
  double dR[3][3], Vm[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      const double w2 = w[r] * w[c] - (r == c ? th2 : 0.0);
      const double I = r == c ? 1.0 : 0.0;
      dR[r][c] = I + A * W[r][c] + B * w2;
      Vm[r][c] = I + B * W[r][c] + Cc * w2;
    }
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 4; ++c)
      Q[4 * r + c] = dR[r][0] * P[c] + dR[r][1] * P[4 + c] + dR[r][2] * P[8 + c];
    Q[4 * r + 3] += Vm[r][0] * xi[0] + Vm[r][1] * xi[1] + Vm[r][2] * xi[2];
  }
}

// Solves (H + damp * diag(H)) x = -g for the 6x6 system of the kTerms layout
// (upper triangle row by row, then g) by Cholesky of the Jacobi-scaled matrix
// (unit diagonal), in FP32: a Gauss-Newton step needs no more, and FP64
// arithmetic is slow on this GPU.  False if the matrix is not positive
// definite or the step is not finite.
__device__ __forceinline__ bool solve6(const float *terms, float damp, float x[6]) {
  float H[6][6], L[6][6], inv[6], sc[6], y[6];
  int k = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = a; b < 6; ++b) H[a][b] = H[b][a] = terms[k++];
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    H[a][a] *= 1.0f + damp;
    ok = ok && H[a][a] > 0.0f;
    sc[a] = rsqrtf(H[a][a]);
  }
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      float s = H[i][j] * sc[i] * sc[j];
#pragma unroll
      for (int m = 0; m < j; ++m) s -= L[i][m] * L[j][m];
      if (i == j) {
        ok = ok && s > 0.0f;
        inv[i] = rsqrtf(s);
        L[i][i] = s * inv[i];
      } else {
        L[i][j] = s * inv[j];
      }
    }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    float s = -terms[21 + i] * sc[i];
#pragma unroll
    for (int m = 0; m < i; ++m) s -= L[i][m] * y[m];
    y[i] = s * inv[i];
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    float s = y[i];
#pragma unroll
    for (int m = i + 1; m < 6; ++m) s -= L[m][i] * x[m];
    x[i] = s * inv[i];
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    x[i] *= sc[i];
    ok = ok && fabsf(x[i]) < 1e30f;
  }
  return ok;
}

// Increment of exp(xi) for xi = (v, w) in FP32: D = dR - I (entries of the
// order of |w|, so FP32 keeps them to ~1e-9 absolute) and t = V v, with
// dR = I + A W + B W^2, V = I + B W + C W^2, W^2 = w w^T - |w|^2 I.
__device__ __forceinline__ void exp_increment(const float xi[6], float D[9], float t[3]) {
  const float w[3] = {xi[3], xi[4], xi[5]};
  const float th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  float A, B, Cc;
  if (th2 < 0.0625f) {
    constexpr float a1 = (float)-inv_factorial(3), a2 = (float)inv_factorial(5),
                    a3 = (float)-inv_factorial(7), a4 = (float)inv_factorial(9);
    constexpr float b0 = (float)inv_factorial(2), b1 = (float)-inv_factorial(4),
                    b2 = (float)inv_factorial(6), b3 = (float)-inv_factorial(8),
                    b4 = (float)inv_factorial(10);
    constexpr float c0 = (float)inv_factorial(3), c1 = (float)-inv_factorial(5),
                    c2 = (float)inv_factorial(7), c3 = (float)-inv_factorial(9),
                    c4 = (float)inv_factorial(11);
    // five terms: the first one left out is below 1e-10 for |w| < 0.25
    A = 1.0f + th2 * (a1 + th2 * (a2 + th2 * (a3 + th2 * a4)));
    B = b0 + th2 * (b1 + th2 * (b2 + th2 * (b3 + th2 * b4)));
    Cc = c0 + th2 * (c1 + th2 * (c2 + th2 * (c3 + th2 * c4)));
  } else {
    const float th = sqrtf(th2);
    A = sinf(th) / th;
    B = (1.0f - cosf(th)) / th2;
    Cc = (th - sinf(th)) / (th2 * th);
  }
  const float W[3][3] = {{0, -w[2], w[1]}, {w[2], 0, -w[0]}, {-w[1], w[0], 0}};
  for (int r = 0; r < 3; ++r) {
    float tr = 0.0f;
    for (int c = 0; c < 3; ++c) {
      const float w2 = w[r] * w[c] - (r == c ? th2 : 0.0f);
      D[3 * r + c] = A * W[r][c] + B * w2;
      tr += ((r == c ? 1.0f : 0.0f) + B * W[r][c] + Cc * w2) * xi[c];
    }
    t[r] = tr;
  }
}

constexpr int kFdPoses = 13;  // current pose, then +/- a step along each coordinate

// Device state of one refinement (or one linearisation), in HBM.
struct RefineState {
  double pose[12];            // master pose, FP64
  double terms[kTerms];       // last reduced normal-equation terms
  float fd_step[6];           // FD step per coordinate
  float inv2eps[6];           // 1 / (2 fd_step)
  float rows[kFdPoses * 12];  // FP32 poses: [0] current, [1 + 2k] / [2 + 2k] = +/- step k
  uint32_t counter;           // CTAs of the current launch that finished
  int32_t updates;            // pose updates applied
  int32_t stopped;            // a solve failed: later launches do nothing
  int32_t iter;               // launches that linearised
};

// SDF residual of one back-projected pixel under pose P: T * sdf, NaN when the
// sample is invalid or truncated.
__device__ __forceinline__ float pixel_residual(const VolumeView &V, const CamParams &C,
                                                const float *P, int u, int v, float d,
                                                float inv_voxel) {
  const Px X = backproject(C, P, u, v, d);
  if (X.ok) {
    const Sample s = sample_tsdf(V, inv_voxel, C.mc_min_weight, X.x, X.y, X.z);
    if (s.ok && fabsf(s.phi) < 1.0f) return C.trunc * s.phi;
  }
  return __int_as_float(0x7FC00000);
}

// Threads per CTA of the refinement step: one CTA per SM for the adjoint (so
// that the last CTA reduces only one partial per SM); the FD variant needs
// more registers per thread and runs three 256-thread CTAs per SM.
template <bool kFD>
struct RefineShape {
  static constexpr int kThreads = kFD ? 256 : 1024;
  static constexpr int kMinCtas = kFD ? 3 : 1;
};

// One Gauss-Newton step.  Every CTA accumulates the 29 normal-equation terms
// of its pixels (analytic Jacobians T [g ; X x g] from the sampling adjoint,
// or, for kFD, central differences of 13 residual evaluations per pixel) and
// stores them in partials[k * G + cta]; the last CTA to finish sums the
// partials in a fixed order (deterministic), and with kSolve solves the 6x6
// system and composes exp(xi) * pose (the pose itself in FP64).  No CTA waits
// for another.
//
// Jobs: with job_ctas > 0 the grid refines gridDim.x / job_ctas independent
// poses (keyframes) at once: CTA b works for job b / job_ctas as its CTA
// b % job_ctas of G = job_ctas, with the job's depth image depth_tab[job],
// state S[job], partials and history; the job's last CTA solves its pose.
// job_ctas = 0 is the single pose (G = gridDim.x, `depth`).
template <bool kFD, bool kSolve>
__global__ void __launch_bounds__(RefineShape<kFD>::kThreads, RefineShape<kFD>::kMinCtas)
    k_refine_step(VolumeView V, CamParams C, const void *depth, const void *const *depth_tab,
                  int fmt, int stride, float inv_voxel, RefineState *S,
                  float *__restrict__ partials, float2 *__restrict__ hist, int hist_cap,
                  int job_ctas) {
  constexpr int kThreads = RefineShape<kFD>::kThreads;
  constexpr int kRows = kFD ? kFdPoses : 1;
  __shared__ float rows[kRows * 12];
  __shared__ float inv2eps[6];
  __shared__ float tot[kTerms];
  __shared__ int last;
  // Thread i of the grid takes pixels i, i + threads, ...; the next depth
  // value is loaded while the current pixel is sampled.
  const int ws = (C.width + stride - 1) / stride, hs = (C.height + stride - 1) / stride;
  const int npx = ws * hs;
  const int lane = threadIdx.x & 31;
  const int job = job_ctas ? (int)blockIdx.x / job_ctas : 0;
  const int cta = job_ctas ? (int)blockIdx.x % job_ctas : (int)blockIdx.x;
  const int G = job_ctas ? job_ctas : (int)gridDim.x;
  if (depth_tab) depth = depth_tab[job];
  S += job;
  partials += (size_t)job * kTerms * G;
  if (hist) hist += (size_t)job * hist_cap;
  const int wstride = G * blockDim.x;
  const int q_first = cta * blockDim.x + (threadIdx.x & ~31);
  auto depth_at = [&](int q) {
    return q < npx ? pixel_depth(depth, fmt, ((q / ws) * stride) * C.width + (q % ws) * stride,
                                 C.depth_scale)
                   : 0.0f;
  };
  float d_next = depth_at(q_first + lane);
  // Launched as a programmatic dependent of the previous step: everything
  // above (the depth prefetch) may overlap that step's last CTA; the state
  // and the partials are touched only after it has completed.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (S->stopped) return;  // uniform: written only between launches
  for (int i = threadIdx.x; i < kRows * 12; i += blockDim.x) rows[i] = S->rows[i];
  if (kFD && threadIdx.x < 6) inv2eps[threadIdx.x] = S->inv2eps[threadIdx.x];
  __syncthreads();
  float acc[kTerms];
#pragma unroll
  for (int k = 0; k < kTerms; ++k) acc[k] = 0.0f;
  for (int q0 = q_first; q0 < npx; q0 += wstride) {
    const int q = q0 + lane;
    const float d = d_next;
    d_next = depth_at(q + wstride);
    const int u = (q % ws) * stride, v = (q / ws) * stride;
    if (!(q < npx && d > C.min_depth && d <= C.max_depth)) continue;
    if constexpr (kFD) {
      const float r0 = pixel_residual(V, C, rows, u, v, d, inv_voxel);
      if (r0 != r0) continue;
      float J[6];
      bool ok = true;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const float rp = pixel_residual(V, C, rows + 12 * (1 + 2 * k), u, v, d, inv_voxel);
        const float rm = pixel_residual(V, C, rows + 12 * (2 + 2 * k), u, v, d, inv_voxel);
        ok = ok && rp == rp && rm == rm;
        J[k] = (rp - rm) * inv2eps[k];
      }
      if (ok) add_terms(acc, r0, J);
    } else {
      const Px X = backproject(C, rows, u, v, d);
      const Sample s = sample_tsdf(V, inv_voxel, C.mc_min_weight, X.x, X.y, X.z);
      if (!s.ok || !(fabsf(s.phi) < 1.0f)) continue;
      const float T = C.trunc;
      const float J[6] = {T * s.gx, T * s.gy, T * s.gz, T * (X.y * s.gz - X.z * s.gy),
                          T * (X.z * s.gx - X.x * s.gz), T * (X.x * s.gy - X.y * s.gx)};
      add_terms(acc, T * s.phi, J);
    }
  }
  // the next step may start its CTAs on the SMs this grid releases
  asm volatile("griddepcontrol.launch_dependents;");
  cta_sum_terms<kThreads>(acc, partials + cta, G);
  __threadfence();  // this CTA's partials before its count
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&S->counter, 1u) == (uint32_t)G - 1u;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // Last CTA: warp w sums terms w, w + nwarps, ...; lane l adds partials
  // l, l + 32, ... in order, then a fixed shuffle tree (deterministic).
  const int t = threadIdx.x;
  for (int k = t >> 5; k < kTerms; k += kThreads / 32) {
    const float *pk = partials + (size_t)k * G;
    float x = 0.0f;
#pragma unroll 8
    for (int i = lane; i < G; i += 32) x += __ldcg(pk + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kFull, x, o);
    if (lane == 0) tot[k] = x;
  }
  __syncthreads();
  if (t < kTerms) S->terms[t] = (double)tot[t];
  if (!kSolve) {
    if (t == 0) {
      S->iter += 1;
      S->counter = 0;
    }
    return;
  }
  // Solve (one thread, FP32), then compose exp(xi) * pose in FP64 with one
  // thread per entry: pose + D * pose (+ t in the last column).
  __shared__ float inc[12];  // D (3x3 row-major), t
  __shared__ int solved;
  if (t == 0) {
    const int it = S->iter;
    if (it < hist_cap) hist[it] = make_float2(tot[27], tot[28]);
    float xi[6];
    solved = tot[28] >= 6.0f && solve6(tot, 1e-6f, xi);
    if (solved) {
      exp_increment(xi, inc, inc + 9);
      S->updates += 1;
    } else {
      S->stopped = 1;
    }
    S->iter = it + 1;
    S->counter = 0;
  }
  __syncthreads();
  if (!solved) return;
  __shared__ float newrows[12];
  if (t < 12) {
    const int r = t >> 2, c = t & 3;
    const double *P = S->pose;
    double q = P[t];
    q += (double)inc[3 * r] * P[c] + (double)inc[3 * r + 1] * P[4 + c] +
         (double)inc[3 * r + 2] * P[8 + c];
    if (c == 3) q += (double)inc[9 + r];
    __syncwarp(0xFFFu);  // every entry read the old pose before any is replaced
    S->pose[t] = q;
    S->rows[t] = (float)q;
    newrows[t] = (float)q;
  }
  if (!kFD) return;
  __syncthreads();
  if (t < 12) {  // FD pose t: exp(+/- step along coordinate t / 2) * pose, in FP32
    const int k = t >> 1;
    float xi[6] = {0, 0, 0, 0, 0, 0}, D[9], tt[3];
    xi[k] = (t & 1) ? -S->fd_step[k] : S->fd_step[k];
    exp_increment(xi, D, tt);
    float *out = S->rows + 12 * (1 + t);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c)
        out[4 * r + c] = newrows[4 * r + c] + (D[3 * r] * newrows[c] + D[3 * r + 1] * newrows[4 + c] +
                                               D[3 * r + 2] * newrows[8 + c]) +
                         (c == 3 ? tt[r] : 0.0f);
  }
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

namespace vh {

// Per-handle refinement buffers and the graph of the last refine call.
struct RefineCtx {
  int device = 0;
  RefineState *d_state = nullptr;
  RefineState *h_state = nullptr;  // pinned mirror
  float *d_partials = nullptr;
  int partial_cap = 0;
  float2 *d_hist = nullptr;
  float2 *h_hist = nullptr;  // pinned
  int hist_cap = 0;
  cudaEvent_t ev[4] = {};
  cudaGraphExec_t graph = nullptr;
  long long key[7] = {};  // method, stride, iterations, fmt, grid, stream, partial buffer
  // batched refinement (vh_pose_refine_batch): per-job states, partials,
  // histories, depth staging and the device table of depth images
  RefineState *d_bstate = nullptr, *h_bstate = nullptr;
  float *d_bpartials = nullptr;
  float2 *d_bhist = nullptr, *h_bhist = nullptr;
  const void **d_btab = nullptr, **h_btab = nullptr;
  char *d_bdepth = nullptr;
  size_t bstate_cap = 0, bpartial_cap = 0, bhist_cap = 0, btab_cap = 0, bdepth_cap = 0;
  cudaGraphExec_t bgraph = nullptr;
  long long bkey[9] = {};
};

void refine_ctx_free(RefineCtx *c) {
  if (!c) return;
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->bgraph) cudaGraphExecDestroy(c->bgraph);
  cudaFree(c->d_bstate);
  cudaFree(c->d_bpartials);
  cudaFree(c->d_bhist);
  cudaFree(c->d_btab);
  cudaFree(c->d_bdepth);
  if (c->h_bstate) cudaFreeHost(c->h_bstate);
  if (c->h_bhist) cudaFreeHost(c->h_bhist);
  if (c->h_btab) cudaFreeHost(c->h_btab);
  cudaFree(c->d_state);
  cudaFree(c->d_partials);
  cudaFree(c->d_hist);
  if (c->h_state) cudaFreeHost(c->h_state);
  if (c->h_hist) cudaFreeHost(c->h_hist);
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  delete c;
}

}  // namespace vh

namespace {

const double kFdStep = 1e-4;  // FD step per se(3) coordinate (metres / radians)

int refine_grid(vh_handle *h, int stride, bool fd) {
  const CamParams C = vh::handle_cam(h);
  const int ws = (C.width + stride - 1) / stride, hs = (C.height + stride - 1) / stride;
  const int threads = fd ? RefineShape<true>::kThreads : RefineShape<false>::kThreads;
  int per_sm = 0;
  const cudaError_t e =
      fd ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_refine_step<true, true>, threads, 0)
         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_refine_step<false, true>, threads, 0);
  if (e != cudaSuccess || per_sm < 1) per_sm = 1;
  const int need = (ws * hs + threads - 1) / threads;
  const int full = vh::handle_sm_count(h) * per_sm;
  return need < 1 ? 1 : (need < full ? need : full);
}

// Creates / grows the handle's refinement buffers.
vh_status refine_ctx(vh_handle *h, int grid, int iterations, RefineCtx **out) {
  RefineCtx *&c = vh::handle_refine(h);
  if (!c) {
    c = new RefineCtx();
    c->device = vh::handle_device(h);
    bool ok = cudaMalloc(&c->d_state, sizeof(RefineState)) == cudaSuccess &&
              cudaMallocHost(&c->h_state, sizeof(RefineState)) == cudaSuccess;
    for (auto &e : c->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    if (!ok) {
      refine_ctx_free(c);
      c = nullptr;
      return vh::handle_fail(h, VH_ERR_CUDA, "refinement state allocation failed");
    }
  }
  if (grid > c->partial_cap || iterations > c->hist_cap) {
    if (cudaStreamSynchronize(vh::handle_stream(h)) != cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "stream failed");
    if (c->graph) {
      cudaGraphExecDestroy(c->graph);  // holds the old buffer addresses
      c->graph = nullptr;
    }
  }
  if (grid > c->partial_cap) {
    cudaFree(c->d_partials);
    c->d_partials = nullptr;
    c->partial_cap = 0;
    if (cudaMalloc(&c->d_partials, sizeof(float) * kTerms * (size_t)grid) != cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "refinement partials allocation failed");
    c->partial_cap = grid;
  }
  if (iterations > c->hist_cap) {
    const int cap = iterations < 64 ? 64 : iterations;
    cudaFree(c->d_hist);
    if (c->h_hist) cudaFreeHost(c->h_hist);
    c->d_hist = nullptr;
    c->h_hist = nullptr;
    c->hist_cap = 0;
    if (cudaMalloc(&c->d_hist, sizeof(float2) * cap) != cudaSuccess ||
        cudaMallocHost(&c->h_hist, sizeof(float2) * cap) != cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "refinement history allocation failed");
    c->hist_cap = cap;
  }
  *out = c;
  return VH_OK;
}

// Initial state: FP64 pose from the caller's c2w, its FP32 rows (and FD steps).
void init_state(RefineState *S, const float *c2w, bool fd) {
  std::memset(S, 0, sizeof(*S));
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) S->pose[4 * r + c] = c2w[4 * r + c];
  for (int k = 0; k < 6; ++k) {
    S->fd_step[k] = (float)kFdStep;
    S->inv2eps[k] = (float)(0.5 / kFdStep);
  }
  for (int c = 0; c < 12; ++c) S->rows[c] = (float)S->pose[c];
  if (fd)
    for (int k = 0; k < 6; ++k)
      for (int sgn = 0; sgn < 2; ++sgn) {
        double xi[6] = {0, 0, 0, 0, 0, 0}, Q[12];
        xi[k] = sgn == 0 ? kFdStep : -kFdStep;
        se3_left_exp(xi, S->pose, Q);
        for (int c = 0; c < 12; ++c) S->rows[12 * (1 + 2 * k + sgn) + c] = (float)Q[c];
      }
}

// Enqueues `n` step launches of one method; every step after the first is a
// programmatic dependent launch of the one before (same stream; inside a
// capture it becomes a programmatic graph edge), so its CTAs start as the
// previous step's CTAs exit and wait in-kernel for that step to complete.
template <bool kSolve>
cudaError_t enqueue_steps(vh_handle *h, RefineCtx *c, const void *depth, int fmt, int stride,
                          bool fd, int grid, int n, cudaStream_t st) {
  const VolumeView V = vh::handle_view(h);
  CamParams C = vh::handle_cam(h);
  C.mc_min_weight = C.mc_min_weight < 1.0f ? 1.0f : C.mc_min_weight;  // observed corners only
  const float inv_voxel = 1.0f / C.voxel;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  for (int i = 0; i < n; ++i) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(fd ? RefineShape<true>::kThreads : RefineShape<false>::kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = i > 0 ? 1u : 0u;
    const cudaError_t e =
        fd ? cudaLaunchKernelEx(&cfg, k_refine_step<true, kSolve>, V, C, depth,
                                (const void *const *)nullptr, fmt, stride, inv_voxel, c->d_state,
                                c->d_partials, c->d_hist, c->hist_cap, 0)
           : cudaLaunchKernelEx(&cfg, k_refine_step<false, kSolve>, V, C, depth,
                                (const void *const *)nullptr, fmt, stride, inv_voxel, c->d_state,
                                c->d_partials, c->d_hist, c->hist_cap, 0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Enqueues `n` batched adjoint steps (jobs of job_ctas CTAs each), chained
// as programmatic dependent launches like enqueue_steps.
cudaError_t enqueue_batch_steps(vh_handle *h, RefineCtx *c, int fmt, int stride, int grid,
                                int job_ctas, int hist_cap, int n, cudaStream_t st) {
  const VolumeView V = vh::handle_view(h);
  CamParams C = vh::handle_cam(h);
  C.mc_min_weight = C.mc_min_weight < 1.0f ? 1.0f : C.mc_min_weight;
  const float inv_voxel = 1.0f / C.voxel;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  for (int i = 0; i < n; ++i) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(RefineShape<false>::kThreads);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = i > 0 ? 1u : 0u;
    const cudaError_t e = cudaLaunchKernelEx(
        &cfg, k_refine_step<false, true>, V, C, (const void *)nullptr,
        (const void *const *)c->d_btab, fmt, stride, inv_voxel, c->d_bstate, c->d_bpartials,
        c->d_bhist, hist_cap, job_ctas);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Grows the batched-refinement buffers (the cached batch graph holds their
// addresses, so it goes when one is reallocated).
vh_status refine_batch_buffers(vh_handle *h, RefineCtx *c, size_t jobs, size_t partials,
                               size_t hist, size_t depth_bytes) {
  const bool grow = jobs > c->bstate_cap || partials > c->bpartial_cap || hist > c->bhist_cap ||
                    jobs > c->btab_cap || depth_bytes > c->bdepth_cap;
  if (!grow) return VH_OK;
  if (cudaStreamSynchronize(vh::handle_stream(h)) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "stream failed");
  if (c->bgraph) {
    cudaGraphExecDestroy(c->bgraph);
    c->bgraph = nullptr;
  }
  bool ok = true;
  if (jobs > c->bstate_cap) {
    cudaFree(c->d_bstate);
    if (c->h_bstate) cudaFreeHost(c->h_bstate);
    c->d_bstate = nullptr;
    c->h_bstate = nullptr;
    c->bstate_cap = 0;
    ok = ok && cudaMalloc(&c->d_bstate, sizeof(RefineState) * jobs) == cudaSuccess &&
         cudaMallocHost(&c->h_bstate, sizeof(RefineState) * jobs) == cudaSuccess;
    if (ok) c->bstate_cap = jobs;
  }
  if (ok && jobs > c->btab_cap) {
    cudaFree(c->d_btab);
    if (c->h_btab) cudaFreeHost(c->h_btab);
    c->d_btab = nullptr;
    c->h_btab = nullptr;
    c->btab_cap = 0;
    ok = cudaMalloc(&c->d_btab, sizeof(void *) * jobs) == cudaSuccess &&
         cudaMallocHost(&c->h_btab, sizeof(void *) * jobs) == cudaSuccess;
    if (ok) c->btab_cap = jobs;
  }
  if (ok && partials > c->bpartial_cap) {
    cudaFree(c->d_bpartials);
    c->d_bpartials = nullptr;
    c->bpartial_cap = 0;
    ok = cudaMalloc(&c->d_bpartials, sizeof(float) * partials) == cudaSuccess;
    if (ok) c->bpartial_cap = partials;
  }
  if (ok && hist > c->bhist_cap) {
    cudaFree(c->d_bhist);
    if (c->h_bhist) cudaFreeHost(c->h_bhist);
    c->d_bhist = nullptr;
    c->h_bhist = nullptr;
    c->bhist_cap = 0;
    ok = cudaMalloc(&c->d_bhist, sizeof(float2) * hist) == cudaSuccess &&
         cudaMallocHost(&c->h_bhist, sizeof(float2) * hist) == cudaSuccess;
    if (ok) c->bhist_cap = hist;
  }
  if (ok && depth_bytes > c->bdepth_cap) {
    cudaFree(c->d_bdepth);
    c->d_bdepth = nullptr;
    c->bdepth_cap = 0;
    ok = cudaMalloc(&c->d_bdepth, depth_bytes) == cudaSuccess;
    if (ok) c->bdepth_cap = depth_bytes;
  }
  if (!ok) {
    cudaGetLastError();
    return vh::handle_fail(h, VH_ERR_CUDA, "batched refinement allocation failed");
  }
  return VH_OK;
}

// Stats of one refinement from its final state and linearisation history.
void fill_refine_stats(const RefineState &S, const float2 *hist, int iterations, float ms,
                       float ms_steps, vh_refine_stats *stats) {
  const int lin = S.iter < iterations ? S.iter : iterations;  // linearisations recorded
  auto rmse = [&](int i) {
    const float2 v = hist[i];
    return v.y > 0.0f ? std::sqrt(v.x / v.y) : 0.0f;
  };
  stats->iterations = S.updates;
  stats->valid_pixels = lin > 0 ? (int32_t)hist[lin - 1].y : 0;
  stats->initial_rmse = lin > 0 ? rmse(0) : 0.0f;
  stats->final_rmse = lin > 0 ? rmse(lin - 1) : 0.0f;
  stats->ms = ms;
  stats->ms_steps = ms_steps;
}

}  // namespace

extern "C" vh_status vh_sdf_sample(vh_handle *h, const float *xyz, int64_t n, float *phi,
                                   float *grad, uint8_t *valid, int32_t mem) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_sdf_sample");
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
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_pose_normal_equations");
  if (!h || !c2w || !terms || stride < 1 || (method != VH_REFINE_ADJOINT && method != VH_REFINE_FD))
    return VH_ERR_INVALID_ARG;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(c2w[i])) return VH_ERR_NOT_FINITE;
  const bool fd = method == VH_REFINE_FD;
  const cudaStream_t st = vh::handle_stream(h);
  const void *d = nullptr;
  vh_status s = vh::handle_stage_depth(h, depth, depth_fmt, mem, &d);
  if (s != VH_OK) return s;
  const int grid = refine_grid(h, stride, fd);
  RefineCtx *c = nullptr;
  if ((s = refine_ctx(h, grid, 1, &c)) != VH_OK) return s;
  init_state(c->h_state, c2w, fd);
  if (cudaMemcpyAsync(c->d_state, c->h_state, sizeof(RefineState), cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "pose upload failed");
  if (enqueue_steps<false>(h, c, d, depth_fmt, stride, fd, grid, 1, st) != cudaSuccess ||
      cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(c->h_state, c->d_state, sizeof(RefineState), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "normal equations failed");
  s = vh::handle_sync(h);
  for (int k = 0; k < kTerms; ++k) terms[k] = c->h_state->terms[k];
  return s;
}

extern "C" vh_status vh_pose_refine(vh_handle *h, const void *depth, int32_t depth_fmt, int32_t mem,
                                    const float *c2w_init, int32_t iterations, int32_t stride,
                                    int32_t method, float *c2w_out, vh_refine_stats *stats) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_pose_refine");
  if (!h || !c2w_init || !c2w_out || iterations < 0 || iterations > (1 << 16) || stride < 1 ||
      (method != VH_REFINE_ADJOINT && method != VH_REFINE_FD))
    return VH_ERR_INVALID_ARG;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(c2w_init[i])) return VH_ERR_NOT_FINITE;
  const bool fd = method == VH_REFINE_FD;
  const cudaStream_t st = vh::handle_stream(h);
  const int grid = refine_grid(h, stride, fd);
  RefineCtx *c = nullptr;
  vh_status s = refine_ctx(h, grid, iterations, &c);
  if (s != VH_OK) return s;
  cudaEventRecord(c->ev[0], st);
  const void *d = nullptr;
  if ((s = vh::handle_stage_depth(h, depth, depth_fmt, mem, &d)) != VH_OK) return s;
  init_state(c->h_state, c2w_init, fd);
  if (cudaMemcpyAsync(c->d_state, c->h_state, sizeof(RefineState), cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "pose upload failed");
  const long long key[7] = {method, stride, iterations, depth_fmt, grid, (long long)(uintptr_t)st,
                            (long long)(uintptr_t)c->d_partials};
  if (c->graph && std::memcmp(key, c->key, sizeof(key)) != 0) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  if (!c->graph && iterations > 0) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "refinement capture failed");
    const cudaError_t le = enqueue_steps<true>(h, c, d, depth_fmt, stride, fd, grid, iterations, st);
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (le != cudaSuccess || e != cudaSuccess || cudaGraphInstantiate(&c->graph, g, 0) != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      c->graph = nullptr;
      return vh::handle_fail(h, VH_ERR_CUDA, "refinement graph failed");
    }
    cudaGraphDestroy(g);
    std::memcpy(c->key, key, sizeof(key));
  }
  cudaEventRecord(c->ev[1], st);
  if (iterations > 0 && cudaGraphLaunch(c->graph, st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "refinement launch failed");
  cudaEventRecord(c->ev[2], st);
  if (cudaMemcpyAsync(c->h_state, c->d_state, sizeof(RefineState), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      (iterations > 0 && cudaMemcpyAsync(c->h_hist, c->d_hist, sizeof(float2) * iterations,
                                         cudaMemcpyDeviceToHost, st) != cudaSuccess))
    return vh::handle_fail(h, VH_ERR_CUDA, "refinement download failed");
  cudaEventRecord(c->ev[3], st);
  if ((s = vh::handle_sync(h)) != VH_OK) return s;
  const RefineState &S = *c->h_state;
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 4; ++k) c2w_out[4 * r + k] = (float)S.pose[4 * r + k];
  c2w_out[12] = c2w_out[13] = c2w_out[14] = 0.0f;
  c2w_out[15] = 1.0f;
  if (stats) {
    float ms = 0.0f, ms_steps = 0.0f;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[3]);
    cudaEventElapsedTime(&ms_steps, c->ev[1], c->ev[2]);
    fill_refine_stats(S, c->h_hist, iterations, ms, ms_steps, stats);
  }
  return VH_OK;
}

extern "C" vh_status vh_pose_refine_batch(vh_handle *h, const void *const *depth,
                                          int32_t depth_fmt, int32_t mem, int32_t n,
                                          const float *c2w_init, int32_t iterations,
                                          int32_t stride, float *c2w_out,
                                          vh_refine_stats *stats) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_pose_refine_batch");
  if (!h || !depth || !c2w_init || !c2w_out || n < 1 || n > VH_REFINE_BATCH_MAX ||
      iterations < 0 || iterations > (1 << 16) || stride < 1)
    return VH_ERR_INVALID_ARG;
  if (depth_fmt != VH_DEPTH_U16_MM && depth_fmt != VH_DEPTH_F32_M) return VH_ERR_INVALID_ARG;
  if (mem != VH_MEM_HOST && mem != VH_MEM_DEVICE) return VH_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i)
    if (!depth[i]) return VH_ERR_INVALID_ARG;
  for (int i = 0; i < 16 * n; ++i)
    if (!std::isfinite(c2w_init[i])) return VH_ERR_NOT_FINITE;
  const cudaStream_t st = vh::handle_stream(h);
  const CamParams C = vh::handle_cam(h);
  const size_t img = (size_t)C.width * C.height * (depth_fmt == VH_DEPTH_U16_MM ? 2 : 4);
  const int full = refine_grid(h, stride, false);
  const int job_ctas = full / n > 0 ? full / n : 1;
  const int grid = n * job_ctas;
  const int hcap = iterations > 0 ? iterations : 1;  // per-job history entries
  RefineCtx *c = nullptr;
  vh_status s = refine_ctx(h, full, iterations, &c);
  if (s != VH_OK) return s;
  s = refine_batch_buffers(h, c, (size_t)n, (size_t)kTerms * grid, (size_t)n * hcap,
                           mem == VH_MEM_HOST ? img * n : 0);
  if (s != VH_OK) return s;
  cudaEventRecord(c->ev[0], st);
  // depth images: the caller's device buffers, or staged host images
  for (int i = 0; i < n; ++i) {
    if (mem == VH_MEM_DEVICE) {
      c->h_btab[i] = depth[i];
    } else {
      if (cudaMemcpyAsync(c->d_bdepth + img * i, depth[i], img, cudaMemcpyHostToDevice, st) !=
          cudaSuccess)
        return vh::handle_fail(h, VH_ERR_CUDA, "depth upload failed");
      c->h_btab[i] = c->d_bdepth + img * i;
    }
    init_state(c->h_bstate + i, c2w_init + 16 * i, false);
  }
  if (cudaMemcpyAsync(c->d_btab, c->h_btab, sizeof(void *) * n, cudaMemcpyHostToDevice, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(c->d_bstate, c->h_bstate, sizeof(RefineState) * n, cudaMemcpyHostToDevice,
                      st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "pose upload failed");
  const long long key[9] = {n, stride, iterations, depth_fmt, grid, (long long)(uintptr_t)st,
                            (long long)(uintptr_t)c->d_bpartials,
                            (long long)(uintptr_t)c->d_bstate, (long long)(uintptr_t)c->d_bhist};
  if (c->bgraph && std::memcmp(key, c->bkey, sizeof(key)) != 0) {
    cudaGraphExecDestroy(c->bgraph);
    c->bgraph = nullptr;
  }
  if (!c->bgraph && iterations > 0) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return vh::handle_fail(h, VH_ERR_CUDA, "refinement capture failed");
    const cudaError_t le =
        enqueue_batch_steps(h, c, depth_fmt, stride, grid, job_ctas, hcap, iterations, st);
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (le != cudaSuccess || e != cudaSuccess ||
        cudaGraphInstantiate(&c->bgraph, g, 0) != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      c->bgraph = nullptr;
      return vh::handle_fail(h, VH_ERR_CUDA, "refinement graph failed");
    }
    cudaGraphDestroy(g);
    std::memcpy(c->bkey, key, sizeof(key));
  }
  cudaEventRecord(c->ev[1], st);
  if (iterations > 0 && cudaGraphLaunch(c->bgraph, st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "refinement launch failed");
  cudaEventRecord(c->ev[2], st);
  if (cudaMemcpyAsync(c->h_bstate, c->d_bstate, sizeof(RefineState) * n, cudaMemcpyDeviceToHost,
                      st) != cudaSuccess ||
      cudaMemcpyAsync(c->h_bhist, c->d_bhist, sizeof(float2) * n * hcap, cudaMemcpyDeviceToHost,
                      st) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "refinement download failed");
  cudaEventRecord(c->ev[3], st);
  if ((s = vh::handle_sync(h)) != VH_OK) return s;
  float ms = 0.0f, ms_steps = 0.0f;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[3]);
  cudaEventElapsedTime(&ms_steps, c->ev[1], c->ev[2]);
  for (int i = 0; i < n; ++i) {
    const RefineState &S = c->h_bstate[i];
    float *out = c2w_out + 16 * i;
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 4; ++k) out[4 * r + k] = (float)S.pose[4 * r + k];
    out[12] = out[13] = out[14] = 0.0f;
    out[15] = 1.0f;
    if (stats) fill_refine_stats(S, c->h_bhist + (size_t)i * hcap, iterations, ms, ms_steps, stats + i);
  }
  return VH_OK;
}

extern "C" vh_status vh_integrate_vjp(vh_handle *h, const void *depth, int32_t depth_fmt,
                                      const float *c2w, const float *grad_sdf, float *grad_depth,
                                      float *grad_pose, int32_t mem) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_integrate_vjp");
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
  std::memcpy(rows, c2w, sizeof(rows));  // rows 0-2 of the row-major 4x4
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

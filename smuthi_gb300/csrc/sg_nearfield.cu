// Electric and magnetic field of a plane-wave expansion at points (near-field evaluation).
//
// Replaces the FP32 kernels electric_field / magnetic_field of smuthi/fields/expansions_cuda.py:5-421
// (one thread per point; for every (kappa, alpha) node expf, sinf, cosf of the full phase and the
// polarisation vectors, nested trapezoids) run by PlaneWaveExpansion.electric_field /
// magnetic_field (smuthi/fields/expansions.py:660-708, 734-770). The field is
//
//   F(r) = 1/omega_F sum_k w_k kappa_k e^{i kz_k z} sum_a w_a I(kappa_k, alpha_a) e^{i kappa_k (cos a x + sin a y)}
//
// (w: trapezoid weights of the kappa contour and of the alpha grid; omega_F = 1 for E, omega for H).
// The point-independent part is hoisted: a prep kernel forms Q_c[k][a] = w_a I_c(k, a) for the three
// Cartesian components (E: TE (-sin a, cos a, 0) g_TE + TM (cos a kz/k, sin a kz/k, -kappa/k) g_TM;
// H: TE (-kz cos a, -kz sin a, kappa) g_TE + TM (-k sin a, k cos a, 0) g_TM) and P[k] = w_k kappa_k /
// omega_F. The field kernel then needs per (point, kappa) one e^{i kz z} and per (point, kappa, alpha)
// one sincos (plus one exp only where kappa is complex) and three complex multiply-adds. A block
// holds 32 points (one per lane) and 8 warps that split the kappa nodes; cos / sin alpha sit in
// shared memory; kappa ranges of a larger split go to further blocks and a reduce kernel sums them
// in a fixed order. FP64 throughout.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cmath>

#include "sg_internal.h"

namespace sg {

static constexpr int kNfWarps = 8;

struct PweArgs {
  const double *x, *y, *z;  // [np] relative to the expansion's reference point
  const double2 *kp, *kz;   // [nk]
  const double2 *Q;         // [3][nk][na]
  const double2 *P;         // [nk]
  const double *alpha;      // [na]
  double2 *partial;         // [ksplit][3][np]
  int np, nk, na, ksplit;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

__global__ void pwe_prep_kernel(int field, const double2 *g, const double2 *kp, const double2 *kz, const double *alpha,
                                int nk, int na, double2 kk, double omega, double2 *Q, double2 *P) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t plane = (size_t)nk * na;
  if (idx >= plane) return;
  const int k = (int)(idx / na), a = (int)(idx - (size_t)k * na);
  const double wa = 0.5 * ((a > 0 ? alpha[a] - alpha[a - 1] : 0.0) + (a < na - 1 ? alpha[a + 1] - alpha[a] : 0.0));
  double s, c;
  sincos(alpha[a], &s, &c);
  const double2 gte = g[idx], gtm = g[plane + idx];
  double2 ix, iy, iz;
  if (field == 0) {
    const double2 t = cmul(cdiv(kz[k], kk), gtm);
    ix = make_double2(-s * gte.x + c * t.x, -s * gte.y + c * t.y);
    iy = make_double2(c * gte.x + s * t.x, c * gte.y + s * t.y);
    const double2 u = cmul(cdiv(kp[k], kk), gtm);
    iz = make_double2(-u.x, -u.y);
  } else {
    const double2 t = cmul(kz[k], gte), u = cmul(kk, gtm);
    ix = make_double2(-c * t.x - s * u.x, -c * t.y - s * u.y);
    iy = make_double2(-s * t.x + c * u.x, -s * t.y + c * u.y);
    iz = cmul(kp[k], gte);
  }
  Q[idx] = make_double2(wa * ix.x, wa * ix.y);
  Q[plane + idx] = make_double2(wa * iy.x, wa * iy.y);
  Q[2 * plane + idx] = make_double2(wa * iz.x, wa * iz.y);
  if (a == 0) {
    double2 wk = make_double2(0.0, 0.0);
    if (k > 0) wk = make_double2(wk.x + 0.5 * (kp[k].x - kp[k - 1].x), wk.y + 0.5 * (kp[k].y - kp[k - 1].y));
    if (k < nk - 1) wk = make_double2(wk.x + 0.5 * (kp[k + 1].x - kp[k].x), wk.y + 0.5 * (kp[k + 1].y - kp[k].y));
    const double2 pk = cmul(wk, kp[k]);
    const double inv = field == 0 ? 1.0 : 1.0 / omega;
    P[k] = make_double2(pk.x * inv, pk.y * inv);
  }
}

__global__ void __launch_bounds__(32 * kNfWarps) pwe_field_kernel(const PweArgs A) {
  extern __shared__ double nf_trig[];  // cos alpha [na], sin alpha [na]
  __shared__ double2 red[kNfWarps][3][32];
  double *ca = nf_trig, *sa = nf_trig + A.na;
  for (int a = threadIdx.x; a < A.na; a += blockDim.x) sincos(A.alpha[a], &sa[a], &ca[a]);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = blockIdx.x * 32 + lane;
  const bool valid = p < A.np;
  const double x = valid ? A.x[p] : 0.0, y = valid ? A.y[p] : 0.0, z = valid ? A.z[p] : 0.0;
  const int per = (A.nk + A.ksplit - 1) / A.ksplit;
  const int k0 = blockIdx.y * per, k1 = min(A.nk, k0 + per);
  const size_t plane = (size_t)A.nk * A.na;
  double2 tot[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
  for (int k = k0 + warp; k < k1; k += kNfWarps) {
    const double2 kp = A.kp[k], kz = A.kz[k];
    double s, c;
    sincos(kz.x * z, &s, &c);
    const double mz = exp(-kz.y * z);
    const double2 f = cmul(A.P[k], make_double2(mz * c, mz * s));  // P_k e^{i kz z}
    const double2 *q0 = A.Q + (size_t)k * A.na, *q1 = q0 + plane, *q2 = q1 + plane;
    double2 acc[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    const bool complex_kp = kp.y != 0.0;
    for (int a = 0; a < A.na; ++a) {
      const double u = ca[a] * x + sa[a] * y;
      sincos(kp.x * u, &s, &c);
      if (complex_kp) {
        const double m = exp(-kp.y * u);
        s *= m;
        c *= m;
      }
      const double2 v0 = __ldg(q0 + a), v1 = __ldg(q1 + a), v2 = __ldg(q2 + a);
      acc[0].x = fma(v0.x, c, fma(-v0.y, s, acc[0].x));
      acc[0].y = fma(v0.x, s, fma(v0.y, c, acc[0].y));
      acc[1].x = fma(v1.x, c, fma(-v1.y, s, acc[1].x));
      acc[1].y = fma(v1.x, s, fma(v1.y, c, acc[1].y));
      acc[2].x = fma(v2.x, c, fma(-v2.y, s, acc[2].x));
      acc[2].y = fma(v2.x, s, fma(v2.y, c, acc[2].y));
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double2 t = cmul(f, acc[q]);
      tot[q].x += t.x;
      tot[q].y += t.y;
    }
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) red[warp][q][lane] = tot[q];
  __syncthreads();
  if (warp == 0 && valid) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double sr = 0.0, si = 0.0;
      for (int w = 0; w < kNfWarps; ++w) {
        sr += red[w][q][lane].x;
        si += red[w][q][lane].y;
      }
      A.partial[((size_t)blockIdx.y * 3 + q) * A.np + p] = make_double2(sr, si);
    }
  }
}

__global__ void pwe_reduce_kernel(const double2 *partial, int np, int ksplit, double2 *out) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)3 * np) return;
  double sr = 0.0, si = 0.0;
  for (int s = 0; s < ksplit; ++s) {
    const double2 v = partial[(size_t)s * 3 * np + idx];
    sr += v.x;
    si += v.y;
  }
  out[idx] = make_double2(sr, si);
}

int pwe_field(int field, int np, const double *x, const double *y, const double *z, int nk, const double2 *kp,
              const double2 *kz, int na, const double *alpha, const double2 *g, double2 k, double omega, double2 *out,
              cudaStream_t st) {
  SG_REQUIRE(field == 0 || field == 1, "field must be 0 (electric) or 1 (magnetic)");
  SG_REQUIRE(np >= 1 && nk >= 2 && na >= 2, "need points, >= 2 kappa nodes and >= 2 azimuthal angles");
  SG_REQUIRE(na <= 8192, "at most 8192 azimuthal angles");
  SG_REQUIRE(field == 0 || (omega > 0 && std::isfinite(omega)), "omega must be positive");
  SG_REQUIRE(k.x != 0.0 || k.y != 0.0, "wavenumber must be nonzero");
  const size_t plane = (size_t)nk * na;
  DevBuf<double2> Q, P, partial;
  Q.reserve(3 * plane);
  P.reserve(nk);
  pwe_prep_kernel<<<(unsigned)((plane + 255) / 256), 256, 0, st>>>(field, g, kp, kz, alpha, nk, na, k, omega, Q.ptr,
                                                                   P.ptr);
  SG_CUDA(cudaGetLastError());
  const int bx = (np + 31) / 32;
  int ksplit = (4 * sm_count() + bx - 1) / bx;  // about four blocks of 256 threads per SM
  const int maxs = nk / kNfWarps > 0 ? nk / kNfWarps : 1;  // keep >= one kappa node per warp
  ksplit = ksplit < 1 ? 1 : (ksplit > maxs ? maxs : ksplit);
  partial.reserve((size_t)ksplit * 3 * np);
  PweArgs A{x, y, z, kp, kz, Q.ptr, P.ptr, alpha, partial.ptr, np, nk, na, ksplit};
  const size_t smem = 2 * (size_t)na * sizeof(double);
  static bool attr_set[64] = {};
  if (first_on_device(attr_set))
    SG_CUDA(cudaFuncSetAttribute(pwe_field_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(2 * 8192 * sizeof(double))));
  pwe_field_kernel<<<dim3(bx, ksplit), 32 * kNfWarps, smem, st>>>(A);
  SG_CUDA(cudaGetLastError());
  pwe_reduce_kernel<<<(unsigned)((3 * (size_t)np + 255) / 256), 256, 0, st>>>(partial.ptr, np, ksplit, out);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));  // the scratch buffers are released on return
  return 3;
}

// ------------------------------------------------------------------ plane waves -> regular SWE at points
// out[q][p][n] = sum_c amp[q][c][n] exp(i (kx (x_p - x0) + ky (y_p - y0) + kz (z_p - z0))) for the
// discrete plane-wave components c of wave q (wavevector kx, ky real, kz complex; reference point
// r0), i.e. the regular spherical-wave coefficients of every wave at every point, the closed-form
// PVWF -> SVWF transformation of a single plane-wave component. The per-n factors amp carry the
// angular part (smuthi/fields/transformations.py:77-131 with one k point) and are formed by the
// caller; this is the particle-dependent part. One thread per (wave, point); FP64.
static constexpr int kPwsMaxComponents = 4;

__global__ void plane_wave_swe_kernel(const double *xyz, int np, int nq, int nc, const double *kr, int bs,
                                      const double2 *amp, double2 *out) {
  const size_t total = (size_t)nq * np;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int q = (int)(e / np), p = (int)(e - (size_t)q * np);
    const double x = xyz[3 * (size_t)p], y = xyz[3 * (size_t)p + 1], z = xyz[3 * (size_t)p + 2];
    double2 ph[kPwsMaxComponents];
    for (int c = 0; c < nc; ++c) {
      const double *w = kr + ((size_t)q * nc + c) * 7;
      const double dz = z - w[6];
      const double arg = w[0] * (x - w[4]) + w[1] * (y - w[5]) + w[2] * dz;
      const double damp = exp(-w[3] * dz);
      double sn, cs;
      sincos(arg, &sn, &cs);
      ph[c] = make_double2(damp * cs, damp * sn);
    }
    double2 *o = out + e * bs;
    for (int n = 0; n < bs; ++n) {
      double re = 0.0, im = 0.0;
      for (int c = 0; c < nc; ++c) {
        const double2 a = amp[((size_t)q * nc + c) * bs + n];
        re = fma(a.x, ph[c].x, fma(-a.y, ph[c].y, re));
        im = fma(a.x, ph[c].y, fma(a.y, ph[c].x, im));
      }
      o[n] = make_double2(re, im);
    }
  }
}

int plane_wave_swe(int np, const double *xyz, int nq, int nc, const double *kr, int bs, const double2 *amp,
                   double2 *out, cudaStream_t st) {
  SG_REQUIRE(np >= 1 && nq >= 1 && bs >= 1, "plane-wave SWE: sizes must be positive");
  SG_REQUIRE(nc >= 1 && nc <= kPwsMaxComponents, "plane-wave SWE: 1 to 4 plane-wave components per wave");
  const size_t total = (size_t)nq * np;
  const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, (size_t)sm_count() * 8);
  plane_wave_swe_kernel<<<grid, 256, 0, st>>>(xyz, np, nq, nc, kr, bs, amp, out);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));
  return 1;
}

}  // namespace sg

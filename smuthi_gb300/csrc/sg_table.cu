// GPU part of the radial lookup-table build: the Bessel factors of the Sommerfeld integral.
//
// The layer-mediated table (smuthi/linearsystem/particlecoupling/prepare_lookup.py:343-459) is, for
// every |m2 - m1| = n, a contraction over the Sommerfeld contour kappa_k of
//   J_n(kappa_k rho_r) * jac_k   (rho_r on the radial grid)
// with a small per-(n1, n2) integrand. Evaluating J_n at len_rho x len_kappa complex arguments
// dominates the host build (scipy.special.jv: ~18 s of 19.5 s for 14 000 x 279 x 9 values at 2 nm);
// this kernel computes all orders 0..nmax of one argument per thread:
//
// * |z| <= 2: the power series J_n(z) = (z/2)^n sum_k (-z^2/4)^k / (k! (n+k)!), 30 terms;
// * |z| > 2: Miller's backward recurrence f_{n-1} = (2n/z) f_n - f_{n+1}, started at
//   N = |z| + 10 |z|^(1/3) + 30 (even) from f_{N+1} = 0, f_N = 1e-280, rescaled when it grows past
//   1e250. It gives the ratios J_n / J_0 for every complex z; they are normalised
//   - for |z| <= 25 by the Neumann identity J_0 + 2 sum_k J_2k = 1,
//   - for |z| > 25 by J_0 or J_1 (the larger of the two recurrence values) from Hankel's asymptotic
//     expansion J_v(z) = sqrt(2/(pi z)) (P cos chi - Q sin chi), chi = z - (v/2 + 1/4) pi, summed until
//     the terms stop decreasing or fall below 1e-17 (at |z| > 25 the smallest term is far below that),
//     which avoids the cancellation of the Neumann sum when Im z is not small.
// Negative rho uses J_n(-z) = (-1)^n J_n(z). Output layout: out[n][r][k] = J_n(kappa_k rho_r) jac_k.
#include <cuda_runtime.h>
#include <math.h>

#include "sg_internal.h"

namespace sg {

struct cz {
  double x, y;
};
__device__ __forceinline__ cz cmul(cz a, cz b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cz cadd(cz a, cz b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cz csub(cz a, cz b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cz cscale(cz a, double s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ double cabs2(cz a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ cz cdiv(cz a, cz b) {
  // Smith's algorithm
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, d = b.x + b.y * r;
    return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
  }
  const double r = b.x / b.y, d = b.x * r + b.y;
  return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
}
__device__ __forceinline__ cz csqrt_principal(cz a) {
  const double m = sqrt(sqrt(cabs2(a)));
  const double th = 0.5 * atan2(a.y, a.x);
  double s, c;
  sincos(th, &s, &c);
  return {m * c, m * s};
}

// J_v(z), v in {0, 1}, |z| > 25, Re z > 0: Hankel's asymptotic expansion
__device__ cz bessel_j01_asym(int v, cz z) {
  const double mu = 4.0 * v * v;
  const cz inv8z = cdiv(cz{1.0, 0.0}, cscale(z, 8.0));
  cz term = {1.0, 0.0};  // a_k / (8z)^k with the running product
  cz P = {1.0, 0.0}, Q = {0.0, 0.0};
  double prev = 1.0;
  for (int k = 1; k <= 60; ++k) {
    const double f = (mu - (double)(2 * k - 1) * (2 * k - 1)) / (double)k;
    term = cscale(cmul(term, inv8z), f);
    const double mag = cabs2(term);
    if (mag > prev) break;  // the asymptotic series has started to diverge
    prev = mag;
    // k odd -> Q with sign (-1)^((k-1)/2); k even -> P with sign (-1)^(k/2)
    if (k & 1) Q = ((k >> 1) & 1) ? csub(Q, term) : cadd(Q, term);
    else P = ((k >> 1) & 1) ? csub(P, term) : cadd(P, term);
    if (mag < 1e-36) break;
  }
  const double phase = (0.5 * v + 0.25) * M_PI;
  const double a = z.x - phase, b = z.y;
  double sa, ca;
  sincos(a, &sa, &ca);
  const double chb = cosh(b), shb = sinh(b);
  const cz cosc = {ca * chb, -sa * shb};
  const cz sinc = {sa * chb, ca * shb};
  const cz pre = csqrt_principal(cdiv(cz{2.0 / M_PI, 0.0}, z));
  return cmul(pre, csub(cmul(P, cosc), cmul(Q, sinc)));
}

static constexpr int kMaxOrder = 32;  // |m2 - m1| <= 2 * 16

__global__ void bessel_jac_kernel(const double2 *kp, const double2 *jac, int nk, const double *rho, int nr, int nmax,
                                  double2 *out) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)nr * nk) return;
  const int r = (int)(idx / nk), k = (int)(idx - (size_t)r * nk);
  const double rr = rho[r];
  const double sgn = rr < 0.0 ? -1.0 : 1.0;
  const cz z = {kp[k].x * fabs(rr), kp[k].y * fabs(rr)};
  const double az = sqrt(cabs2(z));
  cz J[kMaxOrder + 2];
  const int nk_orders = nmax < 1 ? 1 : nmax;  // orders kept internally (J_1 is needed for normalisation)
  if (az <= 2.0) {
    // power series
    const cz h = cscale(z, 0.5);
    const cz mq = cmul(h, h);  // (z/2)^2
    cz hn = {1.0, 0.0};        // (z/2)^n / n!
    for (int n = 0; n <= nk_orders; ++n) {
      if (n > 0) hn = cscale(cmul(hn, h), 1.0 / n);
      cz sum = {0.0, 0.0}, t = {1.0, 0.0};
      for (int kk = 0; kk < 30; ++kk) {
        sum = cadd(sum, t);
        t = cscale(cmul(t, mq), -1.0 / ((double)(kk + 1) * (double)(n + kk + 1)));
      }
      J[n] = cmul(hn, sum);
    }
  } else {
    int N = (int)(az + 10.0 * cbrt(az) + 30.0);
    if (N < nk_orders + 20) N = nk_orders + 20;
    N += N & 1;
    const cz zi = cdiv(cz{1.0, 0.0}, z);
    cz fn1 = {0.0, 0.0}, fn = {1e-280, 0.0};
    cz S = (N % 2 == 0) ? cscale(fn, 2.0) : cz{0.0, 0.0};
    for (int n = 0; n <= nk_orders; ++n) J[n] = {0.0, 0.0};
    for (int n = N; n >= 1; --n) {
      const cz fm = csub(cscale(cmul(zi, fn), 2.0 * n), fn1);  // f_{n-1}
      fn1 = fn;
      fn = fm;
      const int m = n - 1;
      if (m == 0) S = cadd(S, fn);
      else if ((m & 1) == 0) S = cadd(S, cscale(fn, 2.0));
      if (m <= nk_orders) J[m] = fn;
      if (cabs2(fn) > 1e300) {  // |f| > 1e150: rescale everything kept so far
        const double s = 1e-250;
        fn = cscale(fn, s);
        fn1 = cscale(fn1, s);
        S = cscale(S, s);
        for (int q = 0; q <= nk_orders; ++q) J[q] = cscale(J[q], s);
      }
    }
    cz norm;  // multiply every f_n by this
    if (az <= 25.0) {
      norm = cdiv(cz{1.0, 0.0}, S);
    } else {
      // scale by whichever of J_0, J_1 the recurrence found larger (they never vanish together); the
      // recurrence values can be ~1e-260 here, so compare 1-norms (their squares would underflow)
      const bool use1 = fabs(J[1].x) + fabs(J[1].y) > fabs(J[0].x) + fabs(J[0].y);
      const cz exact = bessel_j01_asym(use1 ? 1 : 0, z);
      norm = cdiv(exact, use1 ? J[1] : J[0]);
    }
    for (int n = 0; n <= nk_orders; ++n) J[n] = cmul(J[n], norm);
  }
  const cz w = {jac[k].x, jac[k].y};
  for (int n = 0; n <= nmax; ++n) {
    cz v = cmul(J[n], w);
    if (sgn < 0.0 && (n & 1)) v = cscale(v, -1.0);
    out[((size_t)n * nr + r) * nk + k] = make_double2(v.x, v.y);
  }
}

// ------------------------------------------------------------------ Sommerfeld contraction
// out[r * out_stride + cols[j]] = factor * sum_k a[r][k] g[k][j]: the layer-mediated table's trapezoid
// over the contour for the columns (n1, n2) of one |m1 - m2|, a = J_|dm|(kappa_k rho_r) jac_k (the
// Bessel factors, resident on the device), g[k][j] the per-column integrand times the trapezoid
// weights. A tiled FP64 complex GEMM: 64 rows x 32 columns per block of 256 threads, each thread
// 4 x 2 outputs, K in steps of 16 through shared memory; the sum over k runs in order on the FP64 pipe.
static constexpr int kCtTM = 64, kCtTN = 32, kCtTK = 16;

__global__ void __launch_bounds__(256) contract_kernel(const double2 *__restrict__ a, int nr, int nk,
                                                       const double2 *__restrict__ g, int ncols,
                                                       const int *__restrict__ cols, double2 factor,
                                                       double2 *__restrict__ out, long long out_stride) {
  __shared__ double2 As[kCtTM][kCtTK + 1];
  __shared__ double2 Bs[kCtTK][kCtTN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads
  const int r0 = blockIdx.y * kCtTM, c0 = blockIdx.x * kCtTN;
  double2 acc[4][2];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) acc[u][v] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < nk; k0 += kCtTK) {
    for (int e = threadIdx.x; e < kCtTM * kCtTK; e += 256) {
      const int rr = e / kCtTK, kk = e - rr * kCtTK;
      const int r = r0 + rr, k = k0 + kk;
      As[rr][kk] = (r < nr && k < nk) ? a[(size_t)r * nk + k] : make_double2(0.0, 0.0);
    }
    for (int e = threadIdx.x; e < kCtTK * kCtTN; e += 256) {
      const int kk = e / kCtTN, cc = e - kk * kCtTN;
      const int k = k0 + kk, c = c0 + cc;
      Bs[kk][cc] = (k < nk && c < ncols) ? g[(size_t)k * ncols + c] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kCtTK; ++kk) {
      double2 av[4], bv[2];
#pragma unroll
      for (int u = 0; u < 4; ++u) av[u] = As[ty + 16 * u][kk];
#pragma unroll
      for (int v = 0; v < 2; ++v) bv[v] = Bs[kk][tx + 16 * v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          acc[u][v].x = fma(av[u].x, bv[v].x, fma(-av[u].y, bv[v].y, acc[u][v].x));
          acc[u][v].y = fma(av[u].x, bv[v].y, fma(av[u].y, bv[v].x, acc[u][v].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int r = r0 + ty + 16 * u, c = c0 + tx + 16 * v;
      if (r < nr && c < ncols) {
        const double2 s = acc[u][v];
        out[(size_t)r * out_stride + cols[c]] =
            make_double2(factor.x * s.x - factor.y * s.y, factor.x * s.y + factor.y * s.x);
      }
    }
}

void lookup_contract(const double2 *a, int nr, int nk, const double2 *g, int ncols, const int *cols, double2 factor,
                     double2 *out, long long out_stride, cudaStream_t st) {
  SG_REQUIRE(nr >= 1 && nk >= 1 && ncols >= 1, "empty contraction");
  SG_REQUIRE(out_stride >= 1, "bad output row stride");
  dim3 grid((ncols + kCtTN - 1) / kCtTN, (nr + kCtTM - 1) / kCtTM);
  SG_REQUIRE(grid.y <= 65535, "too many radial points for one contraction launch");
  contract_kernel<<<grid, 256, 0, st>>>(a, nr, nk, g, ncols, cols, factor, out, out_stride);
  SG_CUDA(cudaGetLastError());
}

void bessel_jac_table(const double2 *kp, const double2 *jac, int nk, const double *rho, int nr, int nmax,
                      double2 *out, cudaStream_t st) {
  SG_REQUIRE(nk >= 1 && nr >= 1, "empty contour or radial grid");
  SG_REQUIRE(nmax >= 0 && nmax <= kMaxOrder, "Bessel order must be in [0, 32]");
  const size_t total = (size_t)nr * nk;
  bessel_jac_kernel<<<(unsigned)((total + 127) / 128), 128, 0, st>>>(kp, jac, nk, rho, nr, nmax, out);
  SG_CUDA(cudaGetLastError());
}

}  // namespace sg

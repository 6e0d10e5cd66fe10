// Particle sum of the scattered field's plane-wave expansion, for the cross sections.
//
// The far field of N particles at one height (smuthi/postprocessing/far_field.py:363-427, through
// smuthi/postprocessing/scattered_field.py:80-150 and smuthi/fields/transformations.py:133-233)
// needs, for every in-plane wavenumber kappa_k and azimuth alpha_a, the sum over particles
//
//   g[r][p][k][a] = sum_i exp(-i kappa_k (cos alpha_a x_i + sin alpha_a y_i))
//                         sum_n c[i][n][r] S[n][p][k] exp(i m(n) alpha_a)
//
// (S: the SVWF -> plane-wave transformation coefficient of multipole n and polarisation p at
// kappa_k, computed on the host; the k-dependent prefactor and the layer response are applied on
// the host afterwards). Particles at different heights carry a per-particle factor
// zphase[k][i] = exp(+-i k_z,k (z_ref - z_i)) inside the sum (null: all at one height, the factor is
// part of the host prefactor). On the host this is a dense N-long contraction for every (k, a, r, p):
// 72 s for 1000 particles and one RHS on the default angular grid, so hours at 10 000 particles and
// 16 RHS. Here one thread owns one azimuth a of one kappa_k and a tile of CT (r, p) columns; a block
// stages, for a chunk of CH particles, the m-resolved data D[m][i][col] = sum_{n: m(n) = m}
// c[i][n][r] S[n][p][k] in shared memory (computed once per block and chunk), and every thread then
// applies its lateral phase and exp(i m alpha_a). All arithmetic is FP64.
#include <cuda_runtime.h>
#include <math.h>

#include "sg_internal.h"

namespace sg {

static constexpr int kFfThreads = 128;  // azimuths per block
static constexpr int kFfCH = 32;        // particles per staged chunk
static constexpr int kFfCT = 8;         // (r, p) columns per block
static constexpr int kFfMaxM = 16;

struct FfArgs {
  const double2 *xy;     // [N]
  const double2 *coef;   // [N][B][R]
  const double2 *S;      // [B][2][K]
  const double *kpar;    // [K]
  const double *alpha;   // [A]
  const int *moff;       // [nm + 1] CSR over m = -mmax..mmax of the n with that m
  const int *mlist;      // [B]
  const double2 *zph;    // [K][N] per-particle height factor, or null
  double2 *out;          // [R][2][K][A]
  int N, B, R, K, A, mmax;
};

__global__ void __launch_bounds__(kFfThreads) ff_sum_kernel(const FfArgs f) {
  extern __shared__ double2 ff_smem[];
  const int nm = 2 * f.mmax + 1;
  double2 *D = ff_smem;  // [nm][CH][CT]
  const int k = blockIdx.x;
  const int a = blockIdx.y * kFfThreads + threadIdx.x;
  const int c0 = blockIdx.z * kFfCT;
  const int ncol = 2 * f.R;
  const double kap = f.kpar[k];
  double ca = 1.0, sa = 0.0;
  double2 em[2 * kFfMaxM + 1];
  if (a < f.A) {
    sincos(f.alpha[a], &sa, &ca);
    for (int mi = 0; mi < nm; ++mi) {
      double s, c;
      sincos((double)(mi - f.mmax) * f.alpha[a], &s, &c);
      em[mi] = make_double2(c, s);
    }
  }
  double2 acc[kFfCT];
#pragma unroll
  for (int c = 0; c < kFfCT; ++c) acc[c] = make_double2(0.0, 0.0);

  for (int i0 = 0; i0 < f.N; i0 += kFfCH) {
    __syncthreads();
    for (int e = threadIdx.x; e < nm * kFfCH * kFfCT; e += kFfThreads) {
      const int mi = e / (kFfCH * kFfCT), rem = e - mi * kFfCH * kFfCT;
      const int ii = rem / kFfCT, c = rem - ii * kFfCT;
      const int i = i0 + ii, col = c0 + c;
      double2 v = make_double2(0.0, 0.0);
      if (i < f.N && col < ncol) {
        const int p = col / f.R, r = col - p * f.R;
        for (int q = f.moff[mi]; q < f.moff[mi + 1]; ++q) {
          const int n = f.mlist[q];
          const double2 cv = f.coef[((size_t)i * f.B + n) * f.R + r];
          const double2 sv = f.S[((size_t)n * 2 + p) * f.K + k];
          v.x = fma(cv.x, sv.x, fma(-cv.y, sv.y, v.x));
          v.y = fma(cv.x, sv.y, fma(cv.y, sv.x, v.y));
        }
        if (f.zph) {
          const double2 zp = f.zph[(size_t)k * f.N + i];
          v = make_double2(v.x * zp.x - v.y * zp.y, v.x * zp.y + v.y * zp.x);
        }
      }
      D[e] = v;
    }
    __syncthreads();
    if (a < f.A) {
      const int nch = min(kFfCH, f.N - i0);
      for (int ii = 0; ii < nch; ++ii) {
        const double2 pos = f.xy[i0 + ii];
        double s, c;
        sincos(-kap * (ca * pos.x + sa * pos.y), &s, &c);  // lateral phase exp(-i kappa (cos a x + sin a y))
        for (int mi = 0; mi < nm; ++mi) {
          const double wr = c * em[mi].x - s * em[mi].y, wi = c * em[mi].y + s * em[mi].x;
          const double2 *d = D + ((size_t)mi * kFfCH + ii) * kFfCT;
#pragma unroll
          for (int cc = 0; cc < kFfCT; ++cc) {
            const double2 dv = d[cc];
            acc[cc].x = fma(wr, dv.x, fma(-wi, dv.y, acc[cc].x));
            acc[cc].y = fma(wr, dv.y, fma(wi, dv.x, acc[cc].y));
          }
        }
      }
    }
  }
  if (a < f.A) {
#pragma unroll
    for (int cc = 0; cc < kFfCT; ++cc) {
      const int col = c0 + cc;
      if (col < ncol) {
        const int p = col / f.R, r = col - p * f.R;
        f.out[(((size_t)r * 2 + p) * f.K + k) * f.A + a] = acc[cc];
      }
    }
  }
}

void farfield_sum(const double2 *xy, int n, int bs, int nrhs, const double2 *coef, int mmax, const int *mofn_host,
                  int nk, const double *kpar, const double2 *S, int na, const double *alpha, const double2 *zphase,
                  double2 *out, cudaStream_t st) {
  SG_REQUIRE(n >= 1 && bs >= 1 && nrhs >= 1 && nk >= 1 && na >= 1, "empty far-field problem");
  SG_REQUIRE(mmax >= 0 && mmax <= kFfMaxM, "m_max must be in [0, 16]");
  const int nm = 2 * mmax + 1;
  std::vector<int> moff(nm + 1, 0), mlist;
  for (int mi = 0; mi < nm; ++mi) {
    for (int q = 0; q < bs; ++q) {
      SG_REQUIRE(mofn_host[q] >= -mmax && mofn_host[q] <= mmax, "m_of_n outside [-m_max, m_max]");
      if (mofn_host[q] == mi - mmax) mlist.push_back(q);
    }
    moff[mi + 1] = (int)mlist.size();
  }
  DevBuf<int> d_moff, d_mlist;
  d_moff.reserve(nm + 1);
  d_mlist.reserve(bs);
  SG_CUDA(cudaMemcpyAsync(d_moff.ptr, moff.data(), (nm + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  SG_CUDA(cudaMemcpyAsync(d_mlist.ptr, mlist.data(), bs * sizeof(int), cudaMemcpyHostToDevice, st));
  FfArgs f{xy, coef, S, kpar, alpha, d_moff.ptr, d_mlist.ptr, zphase, out, n, bs, nrhs, nk, na, mmax};
  const size_t smem = (size_t)nm * kFfCH * kFfCT * sizeof(double2);
  SG_CUDA(cudaFuncSetAttribute(ff_sum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(nk, (na + kFfThreads - 1) / kFfThreads, (2 * nrhs + kFfCT - 1) / kFfCT);
  ff_sum_kernel<<<grid, kFfThreads, smem, st>>>(f);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));  // the staging buffers above are released on return
}

}  // namespace sg

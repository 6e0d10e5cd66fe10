// Radial-lookup coupling matvec kernels and lookup-table preparation for sm_103a.
//
// Replaces the per-unknown kernels of smuthi/linearsystem/linear_system_cuda.py:273-405
// (one thread per row, sqrt/atan2/sincos per matrix element, split re/im float tables)
// with a pair-level formulation:
//
//   y_i[n1] = sum_j e^{-i m1 phi_ij} sum_n2 L_{n1 n2}(rho_ij) e^{i m2 phi_ij} x_j[n2]
//
// One CTA owns receiving particle i (optionally a slice of the emitters j), each warp
// streams emitters j; per pair the warp computes rho, the interval index and the
// phases e^{i m phi} once, stages the phase-multiplied x_j block in shared memory and
// every lane (row n1) runs the B-long n2 loop: Horner interpolation of the interval's
// coefficients (coalesced: coefficients are stored [interval][coef][n2][n1]) followed
// by the complex multiply-accumulate over the RHS tile.
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "sg_df64.h"
#include "sg_internal.h"

namespace sg {

template <typename Real>
struct CT;
template <>
struct CT<df64> {
  typedef df64x2 T;  // 16 bytes: (re.hi, re.lo, im.hi, im.lo)
};
template <>
struct CT<double> {
  typedef double2 T;
};
template <>
struct CT<float> {
  typedef float2 T;
};

static constexpr int kThreads = 256;

// read-only cached coefficient loads
__device__ __forceinline__ double2 ldc(const double2 *p) { return __ldg(p); }
__device__ __forceinline__ float2 ldc(const float2 *p) { return __ldg(p); }
__device__ __forceinline__ df64x2 ldc(const df64x2 *p) {
  const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
  df64x2 r;
  r.x = df64(v.x, v.y);
  r.y = df64(v.z, v.w);
  return r;
}

int coef_count(int kind) { return kind == SG_LINEAR ? 2 : 4; }

// ------------------------------------------------------------------ epilogue
// red: shared [bs][RT] reduced coupling sums for receiver i and RHS r0..r0+RT-1.
__device__ void coupling_epilogue(const CouplingLaunch &L, int i, int r0, int RT, const double2 *red) {
  const int bs = L.bs, R = L.nrhs;
  for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
    const int n1 = e / RT, r = e - n1 * RT;
    const size_t o = ((size_t)i * bs + n1) * R + r0 + r;
    double2 v = red[e];
    if (L.master) {
      const int ty = L.ptype[i];
      double2 tw;
      if (L.t_diag) {
        const double2 t = L.t[(size_t)ty * bs + n1];
        tw = make_double2(t.x * v.x - t.y * v.y, t.x * v.y + t.y * v.x);
      } else {
        const double2 *trow = L.t + ((size_t)ty * bs + n1) * bs;
        double ar = 0.0, ai = 0.0;
        for (int n2 = 0; n2 < bs; ++n2) {
          const double2 t = trow[n2];
          const double2 a = red[n2 * RT + r];
          ar = fma(t.x, a.x, fma(-t.y, a.y, ar));
          ai = fma(t.x, a.y, fma(t.y, a.x, ai));
        }
        tw = make_double2(ar, ai);
      }
      const double2 xv = L.x[o];
      v = make_double2(xv.x - tw.x, xv.y - tw.y);
    }
    L.y[o] = v;
  }
}

// ------------------------------------------------------------------ main kernel
template <typename Real, int NC, int RT, int P, bool PAIRS>
__global__ void __launch_bounds__(kThreads) coupling_kernel(const CouplingLaunch L, int nsplit) {
  typedef typename CT<Real>::T cplx;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int bs = L.bs, R = L.nrhs, N = L.n;
  const int i = blockIdx.x, split = blockIdx.y, r0 = blockIdx.z * RT;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  cplx *ubuf = reinterpret_cast<cplx *>(smem_raw) + (size_t)warp * bs * RT;
  double2 *red = reinterpret_cast<double2 *>(smem_raw + (size_t)nw * bs * RT * sizeof(cplx));

  const int j0 = (int)(((long long)N * split) / nsplit);
  const int j1 = (int)(((long long)N * (split + 1)) / nsplit);
  const cplx *coef = reinterpret_cast<const cplx *>(L.coef);
  const size_t bs2 = (size_t)bs * bs;

  int nrow[P], nrowc[P], mrow[P];
  bool valid[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    nrow[q] = lane + 32 * q;
    valid[q] = nrow[q] < bs;
    nrowc[q] = valid[q] ? nrow[q] : bs - 1;
    mrow[q] = L.mofn[nrowc[q]];
  }
  Real acc_re[P][RT], acc_im[P][RT];
#pragma unroll
  for (int q = 0; q < P; ++q)
#pragma unroll
    for (int r = 0; r < RT; ++r) acc_re[q][r] = acc_im[q][r] = Real(0);

  const double xi = L.pos[i].x, yi = L.pos[i].y;
  for (int j = j0 + warp; j < j1; j += nw) {
    int k;
    Real t, c, s;
    if (PAIRS) {
      const int4 pd = L.pairs[(size_t)i * N + j];
      k = pd.x;
      t = (Real)__int_as_float(pd.y);
      c = (Real)__int_as_float(pd.z);
      s = (Real)__int_as_float(pd.w);
    } else {
      const double dx = xi - L.pos[j].x, dy = yi - L.pos[j].y;
      const double rho = sqrt(dx * dx + dy * dy);
      const double sidx = (rho - L.rho_min) / L.res;
      const double fl = floor(sidx);
      k = (int)fl;
      t = (Real)(sidx - fl);
      if (rho > 0.0) {
        c = (Real)(dx / rho);
        s = (Real)(dy / rho);
      } else {
        c = Real(1);
        s = Real(0);
      }
      k = k < 0 ? 0 : (k > L.n_int - 1 ? L.n_int - 1 : k);
    }
    // phases e^{i m phi} of this lane's rows
    Real ph_re[P], ph_im[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const int am = mrow[q] < 0 ? -mrow[q] : mrow[q];
      Real pr = Real(1), pi = Real(0);
      for (int a = 0; a < am; ++a) {
        const Real nr = pr * c - pi * s;
        pi = pr * s + pi * c;
        pr = nr;
      }
      ph_re[q] = pr;
      ph_im[q] = mrow[q] < 0 ? -pi : pi;
    }
    // stage u[n2][r] = e^{i m2 phi} x_j[n2][r]
#pragma unroll
    for (int q = 0; q < P; ++q) {
      if (valid[q]) {
        const size_t xo = ((size_t)j * bs + nrow[q]) * R + r0;
#pragma unroll
        for (int r = 0; r < RT; ++r) {
          Real xr, xim;
          if constexpr (sizeof(Real) == sizeof(float)) {
            if (L.x32) {
              const float2 xv = L.x32[xo + r];
              xr = xv.x;
              xim = xv.y;
            } else {
              const double2 xv = L.x[xo + r];
              xr = (Real)xv.x;
              xim = (Real)xv.y;
            }
          } else if constexpr (std::is_same<Real, df64>::value) {
            const df64x2 xv = ldc(reinterpret_cast<const df64x2 *>(L.xdf) + xo + r);
            xr = xv.x;
            xim = xv.y;
          } else {
            const double2 xv = L.x[xo + r];
            xr = (Real)xv.x;
            xim = (Real)xv.y;
          }
          cplx u;
          u.x = ph_re[q] * xr - ph_im[q] * xim;
          u.y = ph_re[q] * xim + ph_im[q] * xr;
          // FP64: [r][n2] (lane-consecutive writes); FP32: [n2][r] (the n2 loop reads the RHS tile
          // with vector loads, which matters more than the write conflicts); double-float with an
          // even tile: [n2][RHS pair][re.hi x2, re.lo x2, im.hi x2, im.lo x2] for the packed path
          if constexpr (std::is_same<Real, df64>::value && RT % 2 == 0) {
            float *f = reinterpret_cast<float *>(ubuf) + ((size_t)nrow[q] * (RT / 2) + r / 2) * 8 + (r & 1);
            f[0] = u.x.hi;
            f[2] = u.x.lo;
            f[4] = u.y.hi;
            f[6] = u.y.lo;
          } else if (sizeof(Real) == sizeof(double)) {
            ubuf[r * bs + nrow[q]] = u;
          } else {
            ubuf[nrow[q] * RT + r] = u;
          }
        }
      }
    }
    __syncwarp();
    Real pa_re[P][RT], pa_im[P][RT];
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
      for (int r = 0; r < RT; ++r) pa_re[q][r] = pa_im[q][r] = Real(0);
    const cplx *cbase = coef + (size_t)k * NC * bs2;
    if constexpr (std::is_same<Real, double>::value) {
      for (int n2 = 0; n2 < bs; ++n2) {
        cplx u[RT];
#pragma unroll
        for (int r = 0; r < RT; ++r) u[r] = ubuf[r * bs + n2];
#pragma unroll
        for (int q = 0; q < P; ++q) {
          const cplx *cp = cbase + (size_t)n2 * bs + nrowc[q];
          cplx cc = ldc(cp + (NC - 1) * bs2);
          Real lr = cc.x, li = cc.y;
#pragma unroll
          for (int ci = NC - 2; ci >= 0; --ci) {
            const cplx d = ldc(cp + ci * bs2);
            lr = fma(lr, t, d.x);
            li = fma(li, t, d.y);
          }
#pragma unroll
          for (int r = 0; r < RT; ++r) {
            pa_re[q][r] = fma(lr, u[r].x, pa_re[q][r]);
            pa_re[q][r] = fma(-li, u[r].y, pa_re[q][r]);
            pa_im[q][r] = fma(lr, u[r].y, pa_im[q][r]);
            pa_im[q][r] = fma(li, u[r].x, pa_im[q][r]);
          }
        }
      }
    } else if constexpr (std::is_same<Real, df64>::value && RT % 2 == 0) {
      // double-float, RHS in pairs on the packed FP32x2 instructions (fma_p: the scalar operations
      // on two values at once); coefficients of the next column are fetched while this one is applied
      df64p pp_re[P][RT / 2], pp_im[P][RT / 2];
#pragma unroll
      for (int q = 0; q < P; ++q)
#pragma unroll
        for (int h = 0; h < RT / 2; ++h) {
          pp_re[q][h].hi = pp_re[q][h].lo = pp_im[q][h].hi = pp_im[q][h].lo = make_float2(0.f, 0.f);
        }
      cplx cf[P][NC];
#pragma unroll
      for (int q = 0; q < P; ++q)
#pragma unroll
        for (int ci = 0; ci < NC; ++ci) cf[q][ci] = ldc(cbase + ci * bs2 + nrowc[q]);
      const float4 *ub = reinterpret_cast<const float4 *>(ubuf);
      for (int n2 = 0; n2 < bs; ++n2) {
        const int n2n = n2 + 1 < bs ? n2 + 1 : n2;
        cplx nf[P][NC];
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
          for (int ci = 0; ci < NC; ++ci) nf[q][ci] = ldc(cbase + ci * bs2 + (size_t)n2n * bs + nrowc[q]);
        df64p ure[RT / 2], uim[RT / 2];
#pragma unroll
        for (int h = 0; h < RT / 2; ++h) {
          const float4 a0 = ub[((size_t)n2 * (RT / 2) + h) * 2], a1 = ub[((size_t)n2 * (RT / 2) + h) * 2 + 1];
          ure[h].hi = make_float2(a0.x, a0.y);
          ure[h].lo = make_float2(a0.z, a0.w);
          uim[h].hi = make_float2(a1.x, a1.y);
          uim[h].lo = make_float2(a1.z, a1.w);
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
          Real lr = cf[q][NC - 1].x, li = cf[q][NC - 1].y;
#pragma unroll
          for (int ci = NC - 2; ci >= 0; --ci) {
            lr = fma(lr, t, cf[q][ci].x);
            li = fma(li, t, cf[q][ci].y);
          }
          const df64b blr = dfw::df_bcast(lr), bli = dfw::df_bcast(li), bnli = dfw::df_bcast(-li);
#pragma unroll
          for (int h = 0; h < RT / 2; ++h) {
            pp_re[q][h] = dfw::fma_p(blr, ure[h], pp_re[q][h]);
            pp_re[q][h] = dfw::fma_p(bnli, uim[h], pp_re[q][h]);
            pp_im[q][h] = dfw::fma_p(blr, uim[h], pp_im[q][h]);
            pp_im[q][h] = dfw::fma_p(bli, ure[h], pp_im[q][h]);
          }
#pragma unroll
          for (int ci = 0; ci < NC; ++ci) cf[q][ci] = nf[q][ci];
        }
      }
#pragma unroll
      for (int q = 0; q < P; ++q)
#pragma unroll
        for (int h = 0; h < RT / 2; ++h) {
          pa_re[q][2 * h] = df64(pp_re[q][h].hi.x, pp_re[q][h].lo.x);
          pa_re[q][2 * h + 1] = df64(pp_re[q][h].hi.y, pp_re[q][h].lo.y);
          pa_im[q][2 * h] = df64(pp_im[q][h].hi.x, pp_im[q][h].lo.x);
          pa_im[q][2 * h + 1] = df64(pp_im[q][h].hi.y, pp_im[q][h].lo.y);
        }
    } else {
      // FP32 and double-float: the coefficient loads are L2-latency bound, so the next column's
      // coefficients are fetched into registers while the current column is applied (the last
      // iteration re-reads its own column, which stays in bounds)
      cplx cf[P][NC];
#pragma unroll
      for (int q = 0; q < P; ++q)
#pragma unroll
        for (int ci = 0; ci < NC; ++ci) cf[q][ci] = ldc(cbase + ci * bs2 + nrowc[q]);
      for (int n2 = 0; n2 < bs; ++n2) {
        const int n2n = n2 + 1 < bs ? n2 + 1 : n2;
        cplx nf[P][NC];
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
          for (int ci = 0; ci < NC; ++ci) nf[q][ci] = ldc(cbase + ci * bs2 + (size_t)n2n * bs + nrowc[q]);
        cplx u[RT];
#pragma unroll
        for (int r = 0; r < RT; ++r) u[r] = (sizeof(Real) == sizeof(double)) ? ubuf[r * bs + n2] : ubuf[n2 * RT + r];
#pragma unroll
        for (int q = 0; q < P; ++q) {
          Real lr = cf[q][NC - 1].x, li = cf[q][NC - 1].y;
#pragma unroll
          for (int ci = NC - 2; ci >= 0; --ci) {
            lr = fma(lr, t, cf[q][ci].x);
            li = fma(li, t, cf[q][ci].y);
          }
#pragma unroll
          for (int r = 0; r < RT; ++r) {
            pa_re[q][r] = fma(lr, u[r].x, pa_re[q][r]);
            pa_re[q][r] = fma(-li, u[r].y, pa_re[q][r]);
            pa_im[q][r] = fma(lr, u[r].y, pa_im[q][r]);
            pa_im[q][r] = fma(li, u[r].x, pa_im[q][r]);
          }
#pragma unroll
          for (int ci = 0; ci < NC; ++ci) cf[q][ci] = nf[q][ci];
        }
      }
    }
    __syncwarp();
    // output phase e^{-i m1 phi}
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        acc_re[q][r] = fma(ph_re[q], pa_re[q][r], fma(ph_im[q], pa_im[q][r], acc_re[q][r]));
        acc_im[q][r] = fma(ph_re[q], pa_im[q][r], fma(-ph_im[q], pa_re[q][r], acc_im[q][r]));
      }
  }

  // cross-warp reduction through shared memory (FP64 sums)
  __syncthreads();
  double2 *wsum = reinterpret_cast<double2 *>(smem_raw);  // [nw][bs][RT] fits in ubuf region only for
  // double; for float the region is half as large, so float partials are stored as float2.
  if (sizeof(Real) == sizeof(double)) {
#pragma unroll
    for (int q = 0; q < P; ++q)
      if (valid[q])
#pragma unroll
        for (int r = 0; r < RT; ++r)
          wsum[((size_t)warp * bs + nrow[q]) * RT + r] = make_double2((double)acc_re[q][r], (double)acc_im[q][r]);
  } else {
    float2 *fs = reinterpret_cast<float2 *>(smem_raw);
#pragma unroll
    for (int q = 0; q < P; ++q)
      if (valid[q])
#pragma unroll
        for (int r = 0; r < RT; ++r)
          fs[((size_t)warp * bs + nrow[q]) * RT + r] = make_float2((float)acc_re[q][r], (float)acc_im[q][r]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int w = 0; w < nw; ++w) {
      if (sizeof(Real) == sizeof(double)) {
        const double2 v = wsum[(size_t)w * bs * RT + e];
        sr += v.x;
        si += v.y;
      } else {
        const float2 v = reinterpret_cast<const float2 *>(smem_raw)[(size_t)w * bs * RT + e];
        sr += (double)v.x;
        si += (double)v.y;
      }
    }
    red[e] = make_double2(sr, si);
  }
  __syncthreads();
  if (nsplit > 1) {
    for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
      const int n1 = e / RT, r = e - n1 * RT;
      L.partial[(((size_t)split * N + i) * bs + n1) * R + r0 + r] = red[e];
    }
  } else {
    coupling_epilogue(L, i, r0, RT, red);
  }
}

// sums the j-split partials of receiver i, then applies the epilogue
__global__ void __launch_bounds__(kThreads) split_reduce_kernel(const CouplingLaunch L, int nsplit, int RT) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *red = reinterpret_cast<double2 *>(smem_raw);
  const int i = blockIdx.x, r0 = blockIdx.z * RT, bs = L.bs, R = L.nrhs, N = L.n;
  for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
    const int n1 = e / RT, r = e - n1 * RT;
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < nsplit; ++s) {
      const double2 v = L.partial[(((size_t)s * N + i) * bs + n1) * R + r0 + r];
      sr += v.x;
      si += v.y;
    }
    red[e] = make_double2(sr, si);
  }
  __syncthreads();
  coupling_epilogue(L, i, r0, RT, red);
}

// ------------------------------------------------------------------ dispatch
template <typename Real, int NC, int RT, int P, bool PAIRS>
static void launch_t(const CouplingLaunch &L, int nsplit, cudaStream_t st) {
  typedef typename CT<Real>::T cplx;
  const int nw = kThreads / 32;
  const size_t smem = (size_t)nw * L.bs * RT * sizeof(cplx) + (size_t)L.bs * RT * sizeof(double2);
  // the cross-warp reduction reuses the u buffers; they must hold nw*bs*RT partials
  static bool attr_done[64] = {};
  if (first_on_device(attr_done))
    SG_CUDA(cudaFuncSetAttribute(coupling_kernel<Real, NC, RT, P, PAIRS>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  dim3 grid(L.n, nsplit, L.nrhs / RT);
  coupling_kernel<Real, NC, RT, P, PAIRS><<<grid, kThreads, smem, st>>>(L, nsplit);
  SG_CUDA(cudaGetLastError());
  if (nsplit > 1) {
    dim3 g2(L.n, 1, L.nrhs / RT);
    split_reduce_kernel<<<g2, kThreads, (size_t)L.bs * RT * sizeof(double2), st>>>(L, nsplit, RT);
    SG_CUDA(cudaGetLastError());
  }
}

template <typename Real, int NC, int RT, bool PAIRS>
static void launch_p(const CouplingLaunch &L, int nsplit, cudaStream_t st) {
  const int P = (L.bs + 31) / 32;
  if (P == 1) launch_t<Real, NC, RT, 1, PAIRS>(L, nsplit, st);
  else if (P == 2) launch_t<Real, NC, RT, 2, PAIRS>(L, nsplit, st);
  else launch_t<Real, NC, RT, 3, PAIRS>(L, nsplit, st);
}

template <typename Real, int NC, bool PAIRS>
static void launch_r(const CouplingLaunch &L, int nsplit, cudaStream_t st) {
  const int R = L.nrhs;
  if (L.rt > 0) {  // tile chosen by the autotuner (FP32 path)
    SG_REQUIRE(R % L.rt == 0, "RHS tile must divide nrhs");
    if constexpr (std::is_same<Real, float>::value) {
      if (L.rt == 16) return launch_p<Real, NC, 16, PAIRS>(L, nsplit, st);
    }
    if (L.rt == 8) return launch_p<Real, NC, 8, PAIRS>(L, nsplit, st);
    if (L.rt == 4) return launch_p<Real, NC, 4, PAIRS>(L, nsplit, st);
    if (L.rt == 2) return launch_p<Real, NC, 2, PAIRS>(L, nsplit, st);
    if (L.rt == 1) return launch_p<Real, NC, 1, PAIRS>(L, nsplit, st);
    SG_REQUIRE(false, "unsupported RHS tile");
  }
  if (R % 8 == 0) launch_p<Real, NC, 8, PAIRS>(L, nsplit, st);
  else if (R % 4 == 0) launch_p<Real, NC, 4, PAIRS>(L, nsplit, st);
  else if (R % 2 == 0) launch_p<Real, NC, 2, PAIRS>(L, nsplit, st);
  else launch_p<Real, NC, 1, PAIRS>(L, nsplit, st);
}

int choose_split(int n_particles, int nrhs) {
  const int target = 2 * sm_count();
  int s = (target + n_particles - 1) / n_particles;
  if (s < 1) s = 1;
  const int maxs = n_particles / 8 > 0 ? n_particles / 8 : 1;  // keep >= 8 emitters per CTA
  if (s > maxs) s = maxs;
  (void)nrhs;
  return s;
}

// FP64-grade coupling sums in double-float arithmetic on the FP32 pipe; L.coef holds the FP64
// coefficients split into two FP32 words (df64x2), positions and vectors stay FP64.
int launch_coupling_df64(const CouplingLaunch &L, int nsplit, cudaStream_t st) {
  SG_REQUIRE(L.bs >= 1 && L.bs <= 96, "blocksize must be in [1, 96]");
  SG_REQUIRE(L.ncoef == 2 || L.ncoef == 4, "bad coefficient count");
  const int R = L.nrhs;
  if (L.rt == 8) {  // wider RHS tile chosen by the double-float autotuner
    SG_REQUIRE(R % 8 == 0, "RHS tile must divide nrhs");
    if (L.ncoef == 2) launch_p<df64, 2, 8, false>(L, nsplit, st);
    else launch_p<df64, 4, 8, false>(L, nsplit, st);
    return nsplit > 1 ? 2 : 1;
  }
  if (L.ncoef == 2) {
    if (R % 4 == 0) launch_p<df64, 2, 4, false>(L, nsplit, st);
    else if (R % 2 == 0) launch_p<df64, 2, 2, false>(L, nsplit, st);
    else launch_p<df64, 2, 1, false>(L, nsplit, st);
  } else {
    if (R % 4 == 0) launch_p<df64, 4, 4, false>(L, nsplit, st);
    else if (R % 2 == 0) launch_p<df64, 4, 2, false>(L, nsplit, st);
    else launch_p<df64, 4, 1, false>(L, nsplit, st);
  }
  return nsplit > 1 ? 2 : 1;
}

// df64x2 copy of the FP64 coefficients
__global__ void coef_to_df64_kernel(const double2 *src, df64x2 *dst, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) dst[e] = df_from_double2(src[e]);
}

void build_coefficients_df64(const double2 *coef64, void *coefdf, size_t n, cudaStream_t st) {
  coef_to_df64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(coef64, reinterpret_cast<df64x2 *>(coefdf), n);
  SG_CUDA(cudaGetLastError());
}

// df64x2 copy of an FP64 vector (the double-float kernel's input)
void k_to_df64(const double2 *x, void *xdf, size_t n, cudaStream_t st) { build_coefficients_df64(x, xdf, n, st); }

int launch_coupling(const CouplingLaunch &L, bool fp32, int nsplit, cudaStream_t st) {
  SG_REQUIRE(L.bs >= 1 && L.bs <= 96, "blocksize must be in [1, 96]");
  SG_REQUIRE(L.ncoef == 2 || L.ncoef == 4, "bad coefficient count");
  if (fp32) {
    SG_REQUIRE(L.pairs != nullptr, "FP32 path needs the pair table");
    if (L.ncoef == 2) launch_r<float, 2, true>(L, nsplit, st);
    else launch_r<float, 4, true>(L, nsplit, st);
  } else {
    if (L.ncoef == 2) launch_r<double, 2, false>(L, nsplit, st);
    else launch_r<double, 4, false>(L, nsplit, st);
  }
  return nsplit > 1 ? 2 : 1;
}

// ------------------------------------------------------------------ table preparation
// Interior tridiagonal [1 4 1] solve of the not-a-knot spline, one thread per column.
// Msc = h^2 * (second derivative) at every knot; raw/Msc are [len_rho][bs*bs] complex.
__global__ void spline_solve_kernel(const double2 *raw, double2 *msc, int len_rho, int ncol, const double *invden) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int n = len_rho;
#define Y(i) raw[(size_t)(i) * ncol + col]
#define M(i) msc[(size_t)(i) * ncol + col]
  auto rhs = [&](int i) {
    const double2 a = Y(i - 1), b = Y(i), c = Y(i + 1);
    return make_double2(6.0 * (c.x - 2.0 * b.x + a.x), 6.0 * (c.y - 2.0 * b.y + a.y));
  };
  // decoupled end equations of the not-a-knot conditions
  const double2 r1 = rhs(1), rl = rhs(n - 2);
  const double2 m1 = make_double2(r1.x / 6.0, r1.y / 6.0);
  const double2 ml = make_double2(rl.x / 6.0, rl.y / 6.0);
  M(1) = m1;
  M(n - 2) = ml;
  const int nin = n - 4;  // unknowns at knots 2 .. n-3
  if (nin > 0) {
    // forward sweep (store d' in msc)
    double2 dprev = make_double2(0.0, 0.0);
    for (int a = 0; a < nin; ++a) {
      const int kn = a + 2;
      double2 d = rhs(kn);
      if (a == 0) {
        d.x -= m1.x;
        d.y -= m1.y;
      }
      if (a == nin - 1) {
        d.x -= ml.x;
        d.y -= ml.y;
      }
      const double g = invden[a];
      const double2 dp = make_double2((d.x - dprev.x) * g, (d.y - dprev.y) * g);
      M(kn) = dp;
      dprev = dp;
    }
    // back substitution: x_a = d'_a - c'_a x_{a+1}, c'_a = invden[a]
    double2 xn = M(nin - 1 + 2);
    for (int a = nin - 2; a >= 0; --a) {
      const int kn = a + 2;
      const double2 dp = M(kn);
      const double g = invden[a];
      const double2 xv = make_double2(dp.x - g * xn.x, dp.y - g * xn.y);
      M(kn) = xv;
      xn = xv;
    }
  }
  // not-a-knot extrapolation to the end knots
  const double2 m2 = M(2), ml1 = M(n - 3);
  M(0) = make_double2(2.0 * m1.x - m2.x, 2.0 * m1.y - m2.y);
  M(n - 1) = make_double2(2.0 * ml.x - ml1.x, 2.0 * ml.y - ml1.y);
#undef Y
#undef M
}

// One thread per (interval k, n1, n2): writes coefficients [k][c][n2][n1] (FP64 and FP32).
__global__ void coef_kernel(int kind, const double2 *raw, const double2 *msc, int len_rho, int bs, double2 *c64,
                            float2 *c32) {
  const size_t bs2 = (size_t)bs * bs;
  const size_t n_int = (size_t)len_rho - 1;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_int * bs2) return;
  const size_t k = idx / bs2;
  const int e = (int)(idx - k * bs2);  // raw element index n1*bs + n2
  const int n1 = e / bs, n2 = e - n1 * bs;
  const size_t out = (size_t)n2 * bs + n1;
  double2 cf[4];
  int nc;
  const double2 y0 = raw[k * bs2 + e], y1 = raw[(k + 1) * bs2 + e];
  if (kind == SG_LINEAR) {
    nc = 2;
    cf[0] = y0;
    cf[1] = make_double2(y1.x - y0.x, y1.y - y0.y);
  } else if (kind == SG_CUBIC) {
    nc = 4;
    const double2 m0 = msc[k * bs2 + e], m1 = msc[(k + 1) * bs2 + e];
    cf[0] = y0;
    cf[1] = make_double2((y1.x - y0.x) - (2.0 * m0.x + m1.x) / 6.0, (y1.y - y0.y) - (2.0 * m0.y + m1.y) / 6.0);
    cf[2] = make_double2(m0.x / 2.0, m0.y / 2.0);
    cf[3] = make_double2((m1.x - m0.x) / 6.0, (m1.y - m0.y) / 6.0);
  } else {
    nc = 4;
    const size_t km = k > 0 ? k - 1 : 0;
    const size_t kp2 = (k + 2 < (size_t)len_rho) ? k + 2 : (size_t)len_rho - 1;
    const double2 ym = raw[km * bs2 + e], y2 = raw[kp2 * bs2 + e];
    cf[0] = y0;
    cf[1] = make_double2(0.5 * (y1.x - ym.x), 0.5 * (y1.y - ym.y));
    cf[2] = make_double2(0.5 * (2.0 * ym.x - 5.0 * y0.x + 4.0 * y1.x - y2.x),
                         0.5 * (2.0 * ym.y - 5.0 * y0.y + 4.0 * y1.y - y2.y));
    cf[3] = make_double2(0.5 * (-ym.x + 3.0 * y0.x - 3.0 * y1.x + y2.x), 0.5 * (-ym.y + 3.0 * y0.y - 3.0 * y1.y + y2.y));
  }
  for (int c = 0; c < nc; ++c) {
    const size_t o = (k * nc + c) * bs2 + out;
    c64[o] = cf[c];
    c32[o] = make_float2((float)cf[c].x, (float)cf[c].y);
  }
}

void build_coefficients(int kind, const double2 *raw, int len_rho, int bs, double2 *coef64, float2 *coef32,
                        double2 *work, cudaStream_t st) {
  const int ncol = bs * bs;
  DevBuf<double> invden;
  if (kind == SG_CUBIC) {
    SG_REQUIRE(len_rho >= 4, "cubic interpolation needs at least 4 lookup points");
    const int nin = len_rho - 4;
    std::vector<double> h(nin > 0 ? nin : 1);
    double cprev = 0.0;
    for (int a = 0; a < nin; ++a) {
      const double den = 4.0 - cprev;
      h[a] = 1.0 / den;
      cprev = h[a];
    }
    invden.reserve(h.size());
    SG_CUDA(cudaMemcpyAsync(invden.ptr, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    spline_solve_kernel<<<(ncol + 127) / 128, 128, 0, st>>>(raw, work, len_rho, ncol, invden.ptr);
    SG_CUDA(cudaGetLastError());
  }
  const size_t total = (size_t)(len_rho - 1) * ncol;
  coef_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(kind, raw, work, len_rho, bs, coef64, coef32);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));  // invden is released on return
}

__global__ void pairs_kernel(const double2 *pos, int n, double rho_min, double res, int n_int, int4 *pairs) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * n) return;
  const int i = (int)(idx / n), j = (int)(idx - (size_t)i * n);
  const double dx = pos[i].x - pos[j].x, dy = pos[i].y - pos[j].y;
  const double rho = sqrt(dx * dx + dy * dy);
  const double sidx = (rho - rho_min) / res;
  const double fl = floor(sidx);
  int k = (int)fl;
  k = k < 0 ? 0 : (k > n_int - 1 ? n_int - 1 : k);
  const float t = (float)(sidx - fl);
  float c = 1.0f, s = 0.0f;
  if (rho > 0.0) {
    c = (float)(dx / rho);
    s = (float)(dy / rho);
  }
  pairs[idx] = make_int4(k, __float_as_int(t), __float_as_int(c), __float_as_int(s));
}

void build_pairs(const double2 *pos, int n, double rho_min, double res, int n_int, int4 *pairs, cudaStream_t st) {
  const size_t total = (size_t)n * n;
  pairs_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(pos, n, rho_min, res, n_int, pairs);
  SG_CUDA(cudaGetLastError());
}

}  // namespace sg

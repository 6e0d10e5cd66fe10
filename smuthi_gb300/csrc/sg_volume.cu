// Volume-lookup coupling matvec (particles at different heights) for sm_103a.
//
// Replaces the per-unknown kernels of smuthi/linearsystem/linear_system_cuda.py:26-272 (one thread
// per row; per matrix element sqrt, atan2, cosf/sinf and 8 or 32 scattered float gathers from two
// [rho][z][n1][n2] tables) and the host matvec of CouplingMatrixVolumeLookupCPU
// (smuthi/linearsystem/linear_system.py:592-667):
//
//   y_i[n1] = sum_j e^{-i m1 phi_ij} sum_n2 (P_{n1 n2}(rho_ij, z_i + z_j) + M_{n1 n2}(rho_ij, z_i - z_j))
//                                          e^{i m2 phi_ij} x_j[n2]
//
// with P, M interpolated on the uniform 2-D grids (rho_min + a res, sz_min / dz_min + b res).
// Same pair-level organisation as the radial kernel: one CTA per receiving particle i (optionally a
// slice of the emitters), one warp per emitter j; per pair the warp computes rho, phi, the two
// height coordinates and the separable tap weights once, stages e^{i m2 phi} x_j in shared memory,
// and each lane (row n1) runs the n2 loop over coalesced table reads (tables are stored
// [rho][z][q][n2][n1], n1 fastest).
//
// Interpolation kinds (tap weights per axis):
//   SG_LINEAR        bilinear, 2 x 2 taps (RectBivariateSpline kx = ky = 1 of the CPU class and the
//                    reference CUDA linear kernel);
//   SG_CUBIC         tensor-product not-a-knot cubic spline (RectBivariateSpline kx = ky = 3 of the CPU
//                    class) in moment form: per node the value f and the scaled second derivatives
//                    h^2 f_rr, h^2 f_zz and h^4 f_rrzz (q = 0..3), 2 x 2 nodes;
//   SG_CUBIC_HERMITE 4 x 4-tap Catmull-Rom of the reference CUDA cubic kernel
//                    (linear_system_cuda.py:158-189).
#include <cuda_runtime.h>
#include <math.h>

#include <vector>

#include "sg_internal.h"

#include <type_traits>

namespace sg {

template <typename Real>
struct VC;
template <>
struct VC<double> {
  typedef double2 T;
};
template <>
struct VC<float> {
  typedef float2 T;
};

__device__ __forceinline__ double2 vld(const double2 *p) { return __ldg(p); }
__device__ __forceinline__ float2 vld(const float2 *p) { return __ldg(p); }

static constexpr int kVolThreads = 256;

// Taps along one axis: returns the first tap index (all taps inside [0, len)) and the value weights
// wv[0..NT) (and, for the spline, the moment weights wm[0..2)). The caller guarantees that every
// coordinate lies inside the grid's interior (the host checks the grid against the particles);
// clamping only keeps the reads in bounds.
template <int KIND>
__device__ __forceinline__ int axis_taps(double coord, double origin, double res, int len, double *wv, double *wm) {
  const double u = (coord - origin) / res;
  int i = (int)floor(u);
  if (KIND == SG_CUBIC_HERMITE) {
    i = i < 1 ? 1 : (i > len - 3 ? len - 3 : i);
    const double w = u - i;
    wv[0] = 0.5 * (-w * w * w + 2.0 * w * w - w);
    wv[1] = 0.5 * (3.0 * w * w * w - 5.0 * w * w + 2.0);
    wv[2] = 0.5 * (-3.0 * w * w * w + 4.0 * w * w + w);
    wv[3] = 0.5 * (w * w * w - w * w);
    return i - 1;
  }
  i = i < 0 ? 0 : (i > len - 2 ? len - 2 : i);
  const double t = u - i;
  wv[0] = 1.0 - t;
  wv[1] = t;
  if (KIND == SG_CUBIC) {
    const double s = 1.0 - t;
    wm[0] = (s * s * s - s) / 6.0;
    wm[1] = (t * t * t - t) / 6.0;
  }
  return i;
}

// The same taps for the FP32 operator: only the grid coordinate u = (coord - origin) / res and its
// integer part are formed in FP64 (they set which cells are read); the weights, polynomials of the
// fraction t in [0, 1), are evaluated in FP32, so the FP64 pipe (1/59 of the FP32 rate on GB300)
// carries a few operations per pair instead of the whole tap set.
template <int KIND>
__device__ __forceinline__ int axis_taps_f32(double coord, double origin, double inv_res, int len, float *wv,
                                             float *wm) {
  const double u = (coord - origin) * inv_res;
  int i = (int)floor(u);
  if (KIND == SG_CUBIC_HERMITE) {
    i = i < 1 ? 1 : (i > len - 3 ? len - 3 : i);
    const float w = (float)(u - i);
    wv[0] = 0.5f * (-w * w * w + 2.f * w * w - w);
    wv[1] = 0.5f * (3.f * w * w * w - 5.f * w * w + 2.f);
    wv[2] = 0.5f * (-3.f * w * w * w + 4.f * w * w + w);
    wv[3] = 0.5f * (w * w * w - w * w);
    return i - 1;
  }
  i = i < 0 ? 0 : (i > len - 2 ? len - 2 : i);
  const float t = (float)(u - i);
  wv[0] = 1.f - t;
  wv[1] = t;
  if (KIND == SG_CUBIC) {
    const float s = 1.f - t;
    wm[0] = (s * s * s - s) * (1.f / 6.f);
    wm[1] = (t * t * t - t) * (1.f / 6.f);
  } else {
    wm[0] = wm[1] = 0.f;
  }
  return i;
}

// W(n1, n2) of one table: rows = NT pointers (one per rho tap, already offset to the first z tap and
// to n2 * bs + n1), zs = elements between z taps, qs = elements between the q planes (spline)
template <typename Real, int KIND, int NT>
__device__ __forceinline__ typename VC<Real>::T table_value(const typename VC<Real>::T *const *rows, int zs, int qs,
                                                            const Real *wr, const Real *wrm, const Real *wz,
                                                            const Real *wzm) {
  typedef typename VC<Real>::T cplx;
  Real sr = 0, si = 0;
#pragma unroll
  for (int a = 0; a < NT; ++a) {
    Real vr = 0, vi = 0;  // value-weighted sum along z
    Real mr = 0, mi = 0;  // spline: rho-moment part
#pragma unroll
    for (int b = 0; b < NT; ++b) {
      const cplx f = vld(rows[a] + b * zs);
      vr += wz[b] * f.x;
      vi += wz[b] * f.y;
      if (KIND == SG_CUBIC) {
        const cplx fzz = vld(rows[a] + b * zs + 2 * qs);
        const cplx frr = vld(rows[a] + b * zs + qs);
        const cplx frrzz = vld(rows[a] + b * zs + 3 * qs);
        vr += wzm[b] * fzz.x;
        vi += wzm[b] * fzz.y;
        mr += wz[b] * frr.x + wzm[b] * frrzz.x;
        mi += wz[b] * frr.y + wzm[b] * frrzz.y;
      }
    }
    sr += wr[a] * vr;
    si += wr[a] * vi;
    if (KIND == SG_CUBIC) {
      sr += wrm[a] * mr;
      si += wrm[a] * mi;
    }
  }
  cplx out;
  out.x = sr;
  out.y = si;
  return out;
}

struct VolumeLaunch {
  CouplingLaunch c;   // positions, m(n), vectors, T-matrices, split scratch (pair table unused)
  const double *z;    // [N] particle heights
  const void *tpl;    // [len_rho][len_z][nq][bs][bs] complex, n1 fastest: z1 + z2 table
  const void *tmn;    // the same for the z1 - z2 table
  int len_rho, len_z, nq;
  double rho_min, sz_min, dz_min, res;
};

// red: shared [bs][RT] reduced coupling sums of receiver i for columns r0 .. r0 + nr - 1
__device__ void volume_epilogue(const CouplingLaunch &L, int i, int r0, int RT, int nr, const double2 *red) {
  const int bs = L.bs, R = L.nrhs;
  for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
    const int n1 = e / RT, r = e - n1 * RT;
    if (r >= nr) continue;
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

template <typename Real, int KIND, int NB1, int RT>
__global__ void __launch_bounds__(kVolThreads) volume_kernel(const VolumeLaunch V, int nsplit) {
  typedef typename VC<Real>::T cplx;
  constexpr int NT = KIND == SG_CUBIC_HERMITE ? 4 : 2;
  extern __shared__ __align__(16) unsigned char vsmem[];
  const CouplingLaunch &L = V.c;
  const int bs = L.bs, R = L.nrhs, N = L.n;
  const int i = blockIdx.x, split = blockIdx.y, r0 = blockIdx.z * RT;
  const int nr = min(RT, R - r0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  cplx *xs = reinterpret_cast<cplx *>(vsmem) + (size_t)warp * bs * RT;
  double2 *wacc = reinterpret_cast<double2 *>(vsmem + (size_t)nw * bs * RT * sizeof(cplx));
  double2 *myacc = wacc + (size_t)warp * bs * RT;
  for (int e = lane; e < bs * RT; e += 32) myacc[e] = make_double2(0.0, 0.0);

  const size_t bs2 = (size_t)bs * bs;
  const int qs = (int)bs2, zs = V.nq * (int)bs2;
  const size_t rs = (size_t)V.len_z * zs;
  const cplx *Tp = reinterpret_cast<const cplx *>(V.tpl);
  const cplx *Tm = reinterpret_cast<const cplx *>(V.tmn);
  const double2 pi = L.pos[i];
  const double zi = V.z[i];
  int m1[NB1];
#pragma unroll
  for (int s = 0; s < NB1; ++s) {
    const int n1 = lane + 32 * s;
    m1[s] = n1 < bs ? L.mofn[n1] : 0;
  }
  const int per = (N + nsplit - 1) / nsplit;
  const int j0 = split * per, j1 = min(N, j0 + per);
  constexpr bool F32 = std::is_same<Real, float>::value;
  // FP32 operator: the rotated pair sums accumulate in registers across the warp's pairs
  float2 tot[NB1][RT];
#pragma unroll
  for (int s = 0; s < NB1; ++s)
#pragma unroll
    for (int r = 0; r < RT; ++r) tot[s][r] = make_float2(0.f, 0.f);
  const double inv_res = 1.0 / V.res;
  if constexpr (F32) {
  for (int j = j0 + warp; j < j1; j += nw) {
    const double2 pj = L.pos[j];
    const double dx = pi.x - pj.x, dy = pi.y - pj.y;
    const double rho = sqrt(dx * dx + dy * dy);
    const double zj = V.z[j];
    float wr[NT], wrm[2], wp[NT], wpm[2], wn[NT], wnm[2];
    const int ir = axis_taps_f32<KIND>(rho, V.rho_min, inv_res, V.len_rho, wr, wrm);
    const int ip = axis_taps_f32<KIND>(zi + zj, V.sz_min, inv_res, V.len_z, wp, wpm);
    const int im = axis_taps_f32<KIND>(zi - zj, V.dz_min, inv_res, V.len_z, wn, wnm);
    float c = 1.f, sn = 0.f;
    if (rho > 0.0) {
      const double ir_ = 1.0 / rho;
      c = (float)(dx * ir_);
      sn = (float)(dy * ir_);
    }
    // e^{i m phi} of the lane's rows by repeated multiplication; x_j (FP32 copy) staged with e^{i m2 phi}
    float pr[NB1], pim[NB1];
#pragma unroll
    for (int s = 0; s < NB1; ++s) {
      const int am = m1[s] < 0 ? -m1[s] : m1[s];
      float a = 1.f, b = 0.f;
      for (int q = 0; q < am; ++q) {
        const float na = a * c - b * sn;
        b = a * sn + b * c;
        a = na;
      }
      pr[s] = a;
      pim[s] = m1[s] < 0 ? -b : b;
    }
#pragma unroll
    for (int s = 0; s < NB1; ++s) {
      const int n2 = lane + 32 * s;
      if (n2 < bs) {
        const float2 *xr = L.x32 + ((size_t)j * bs + n2) * R + r0;
#pragma unroll
        for (int r = 0; r < RT; ++r) {
          cplx v;
          if (r < nr) {
            const float2 xv = __ldg(xr + r);
            v.x = pr[s] * xv.x - pim[s] * xv.y;
            v.y = pr[s] * xv.y + pim[s] * xv.x;
          } else {
            v.x = 0;
            v.y = 0;
          }
          xs[n2 * RT + r] = v;
        }
      }
    }
    __syncwarp();
    const cplx *rp[NT], *rm[NT];
#pragma unroll
    for (int a = 0; a < NT; ++a) {
      rp[a] = Tp + (size_t)(ir + a) * rs + (size_t)ip * zs;
      rm[a] = Tm + (size_t)(ir + a) * rs + (size_t)im * zs;
    }
    cplx acc[NB1][RT];
#pragma unroll
    for (int s = 0; s < NB1; ++s)
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        acc[s][r].x = 0;
        acc[s][r].y = 0;
      }
    for (int n2 = 0; n2 < bs; ++n2) {
#pragma unroll
      for (int s = 0; s < NB1; ++s) {
        const int n1 = lane + 32 * s;
        if (n1 < bs) {
          const cplx *pa[NT], *ma[NT];
#pragma unroll
          for (int a = 0; a < NT; ++a) {
            pa[a] = rp[a] + n2 * bs + n1;
            ma[a] = rm[a] + n2 * bs + n1;
          }
          const cplx wpl = table_value<Real, KIND, NT>(pa, zs, qs, wr, wrm, wp, wpm);
          const cplx wmn = table_value<Real, KIND, NT>(ma, zs, qs, wr, wrm, wn, wnm);
          const Real wre = wpl.x + wmn.x, wim = wpl.y + wmn.y;
#pragma unroll
          for (int r = 0; r < RT; ++r) {
            const cplx xv = xs[n2 * RT + r];
            acc[s][r].x += wre * xv.x - wim * xv.y;
            acc[s][r].y += wre * xv.y + wim * xv.x;
          }
        }
      }
    }
    // rotate by e^{-i m1 phi} into the register accumulator
#pragma unroll
    for (int s = 0; s < NB1; ++s)
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        const float ar = (float)acc[s][r].x, ai = (float)acc[s][r].y;
        tot[s][r].x += pr[s] * ar + pim[s] * ai;
        tot[s][r].y += pr[s] * ai - pim[s] * ar;
      }
    __syncwarp();  // xs is rewritten by the next pair
  }
#pragma unroll
  for (int s = 0; s < NB1; ++s) {
    const int n1 = lane + 32 * s;
    if (n1 < bs)
#pragma unroll
      for (int r = 0; r < RT; ++r) myacc[n1 * RT + r] = make_double2((double)tot[s][r].x, (double)tot[s][r].y);
  }
  } else {
  for (int j = j0 + warp; j < j1; j += nw) {
    const double2 pj = L.pos[j];
    const double dx = pi.x - pj.x, dy = pi.y - pj.y;
    const double rho = sqrt(dx * dx + dy * dy);
    const double phi = atan2(dy, dx);
    const double zj = V.z[j];
    double wv[4], wm[2];
    Real wr[NT], wrm[2], wp[NT], wpm[2], wn[NT], wnm[2];
    const int ir = axis_taps<KIND>(rho, V.rho_min, V.res, V.len_rho, wv, wm);
#pragma unroll
    for (int a = 0; a < NT; ++a) wr[a] = (Real)wv[a];
    wrm[0] = (Real)(KIND == SG_CUBIC ? wm[0] : 0.0);
    wrm[1] = (Real)(KIND == SG_CUBIC ? wm[1] : 0.0);
    const int ip = axis_taps<KIND>(zi + zj, V.sz_min, V.res, V.len_z, wv, wm);
#pragma unroll
    for (int a = 0; a < NT; ++a) wp[a] = (Real)wv[a];
    wpm[0] = (Real)(KIND == SG_CUBIC ? wm[0] : 0.0);
    wpm[1] = (Real)(KIND == SG_CUBIC ? wm[1] : 0.0);
    const int im = axis_taps<KIND>(zi - zj, V.dz_min, V.res, V.len_z, wv, wm);
#pragma unroll
    for (int a = 0; a < NT; ++a) wn[a] = (Real)wv[a];
    wnm[0] = (Real)(KIND == SG_CUBIC ? wm[0] : 0.0);
    wnm[1] = (Real)(KIND == SG_CUBIC ? wm[1] : 0.0);

    // e^{i m phi} of the lane's rows; x_j staged with e^{i m2 phi}
    double ec[NB1], es[NB1];
#pragma unroll
    for (int s = 0; s < NB1; ++s) sincos((double)m1[s] * phi, &es[s], &ec[s]);
#pragma unroll
    for (int s = 0; s < NB1; ++s) {
      const int n2 = lane + 32 * s;
      if (n2 < bs) {
        const double2 *xr = L.x + ((size_t)j * bs + n2) * R + r0;
#pragma unroll
        for (int r = 0; r < RT; ++r) {
          cplx v;
          if (r < nr) {
            const double2 xv = xr[r];
            v.x = (Real)(ec[s] * xv.x - es[s] * xv.y);
            v.y = (Real)(ec[s] * xv.y + es[s] * xv.x);
          } else {
            v.x = 0;
            v.y = 0;
          }
          xs[n2 * RT + r] = v;
        }
      }
    }
    __syncwarp();

    const cplx *rp[NT], *rm[NT];
#pragma unroll
    for (int a = 0; a < NT; ++a) {
      rp[a] = Tp + (size_t)(ir + a) * rs + (size_t)ip * zs;
      rm[a] = Tm + (size_t)(ir + a) * rs + (size_t)im * zs;
    }
    cplx acc[NB1][RT];
#pragma unroll
    for (int s = 0; s < NB1; ++s)
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        acc[s][r].x = 0;
        acc[s][r].y = 0;
      }
    for (int n2 = 0; n2 < bs; ++n2) {
#pragma unroll
      for (int s = 0; s < NB1; ++s) {
        const int n1 = lane + 32 * s;
        if (n1 < bs) {
          const cplx *pa[NT], *ma[NT];
#pragma unroll
          for (int a = 0; a < NT; ++a) {
            pa[a] = rp[a] + n2 * bs + n1;
            ma[a] = rm[a] + n2 * bs + n1;
          }
          const cplx wpl = table_value<Real, KIND, NT>(pa, zs, qs, wr, wrm, wp, wpm);
          const cplx wmn = table_value<Real, KIND, NT>(ma, zs, qs, wr, wrm, wn, wnm);
          const Real wre = wpl.x + wmn.x, wim = wpl.y + wmn.y;
#pragma unroll
          for (int r = 0; r < RT; ++r) {
            const cplx xv = xs[n2 * RT + r];
            acc[s][r].x += wre * xv.x - wim * xv.y;
            acc[s][r].y += wre * xv.y + wim * xv.x;
          }
        }
      }
    }
    // rotate by e^{-i m1 phi} and add to the warp's accumulator (each lane owns its rows)
#pragma unroll
    for (int s = 0; s < NB1; ++s) {
      const int n1 = lane + 32 * s;
      if (n1 < bs) {
#pragma unroll
        for (int r = 0; r < RT; ++r) {
          const double ar = (double)acc[s][r].x, ai = (double)acc[s][r].y;
          double2 &o = myacc[n1 * RT + r];
          o.x += ec[s] * ar + es[s] * ai;
          o.y += ec[s] * ai - es[s] * ar;
        }
      }
    }
    __syncwarp();  // xs is rewritten by the next pair
  }
  }
  __syncthreads();
  double2 *red = reinterpret_cast<double2 *>(vsmem);  // reuses the staging area
  for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int w = 0; w < nw; ++w) {
      const double2 v = wacc[(size_t)w * bs * RT + e];
      sr += v.x;
      si += v.y;
    }
    red[e] = make_double2(sr, si);
  }
  __syncthreads();
  if (nsplit > 1) {
    for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
      const int n1 = e / RT, r = e - n1 * RT;
      if (r < nr) L.partial[(((size_t)split * N + i) * bs + n1) * R + r0 + r] = red[e];
    }
  } else {
    volume_epilogue(L, i, r0, RT, nr, red);
  }
}

// sums the emitter-split partials of receiver i, then applies the epilogue
__global__ void __launch_bounds__(kVolThreads) volume_reduce_kernel(const CouplingLaunch L, int nsplit, int RT) {
  extern __shared__ __align__(16) unsigned char vsmem[];
  double2 *red = reinterpret_cast<double2 *>(vsmem);
  const int i = blockIdx.x, r0 = blockIdx.z * RT, bs = L.bs, R = L.nrhs, N = L.n;
  const int nr = min(RT, R - r0);
  for (int e = threadIdx.x; e < bs * RT; e += blockDim.x) {
    const int n1 = e / RT, r = e - n1 * RT;
    double sr = 0.0, si = 0.0;
    if (r < nr)
      for (int s = 0; s < nsplit; ++s) {
        const double2 v = L.partial[(((size_t)s * N + i) * bs + n1) * R + r0 + r];
        sr += v.x;
        si += v.y;
      }
    red[e] = make_double2(sr, si);
  }
  __syncthreads();
  volume_epilogue(L, i, r0, RT, nr, red);
}

template <typename Real, int KIND, int NB1, int RT>
static void launch_vt(const VolumeLaunch &V, int nsplit, cudaStream_t st) {
  typedef typename VC<Real>::T cplx;
  const int nw = kVolThreads / 32, bs = V.c.bs;
  const size_t smem = (size_t)nw * bs * RT * (sizeof(cplx) + sizeof(double2));
  // the opt-in limit is set once per device for the largest blocksize this instantiation serves
  const size_t smem_max = (size_t)nw * (NB1 == 1 ? 32 : 96) * RT * (sizeof(cplx) + sizeof(double2));
  static bool attr_set[64] = {};
  if (smem_max > 48 * 1024 && first_on_device(attr_set))
    SG_CUDA(cudaFuncSetAttribute(volume_kernel<Real, KIND, NB1, RT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem_max));
  const dim3 grid(V.c.n, nsplit, (V.c.nrhs + RT - 1) / RT);
  volume_kernel<Real, KIND, NB1, RT><<<grid, kVolThreads, smem, st>>>(V, nsplit);
  SG_CUDA(cudaGetLastError());
  if (nsplit > 1) {
    volume_reduce_kernel<<<dim3(V.c.n, 1, grid.z), kVolThreads, (size_t)bs * RT * sizeof(double2), st>>>(V.c, nsplit,
                                                                                                        RT);
    SG_CUDA(cudaGetLastError());
  }
}

template <typename Real, int KIND>
static void launch_vk(const VolumeLaunch &V, int nsplit, cudaStream_t st) {
  const bool one_slot = V.c.bs <= 32;
  if (V.c.nrhs == 1) {
    if (one_slot) launch_vt<Real, KIND, 1, 1>(V, nsplit, st);
    else launch_vt<Real, KIND, 3, 1>(V, nsplit, st);
  } else if (one_slot) {
    launch_vt<Real, KIND, 1, 8>(V, nsplit, st);
  } else {
    launch_vt<Real, KIND, 3, 4>(V, nsplit, st);
  }
}

template <typename Real>
static void launch_vr(const VolumeLaunch &V, int kind, int nsplit, cudaStream_t st) {
  if (kind == SG_LINEAR) launch_vk<Real, SG_LINEAR>(V, nsplit, st);
  else if (kind == SG_CUBIC) launch_vk<Real, SG_CUBIC>(V, nsplit, st);
  else launch_vk<Real, SG_CUBIC_HERMITE>(V, nsplit, st);
}

// ------------------------------------------------------------------ table preparation
// Node moments h^2 f'' of the not-a-knot cubic spline along one axis, one thread per column:
// element k of column (o, c) sits at src[o * so + k * sk + c], c < ninner, o < nouter.
__global__ void vol_moments_kernel(const double2 *src, double2 *dst, int n, size_t sk, int ninner, int nouter,
                                   size_t so, const double *invden) {
  const size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= (size_t)ninner * nouter) return;
  const size_t o = col / ninner, c = col - o * ninner;
  const double2 *Y = src + o * so + c;
  double2 *M = dst + o * so + c;
  auto rhs = [&](int k) {
    const double2 a = Y[(size_t)(k - 1) * sk], b = Y[(size_t)k * sk], d = Y[(size_t)(k + 1) * sk];
    return make_double2(6.0 * (d.x - 2.0 * b.x + a.x), 6.0 * (d.y - 2.0 * b.y + a.y));
  };
  // the not-a-knot conditions make the second and the second-to-last moments explicit
  const double2 r1 = rhs(1), rl = rhs(n - 2);
  const double2 m1 = make_double2(r1.x / 6.0, r1.y / 6.0), ml = make_double2(rl.x / 6.0, rl.y / 6.0);
  M[sk] = m1;
  M[(size_t)(n - 2) * sk] = ml;
  const int nin = n - 4;  // [1 4 1] system for the moments of nodes 2 .. n-3
  if (nin > 0) {
    double2 dprev = make_double2(0.0, 0.0);
    for (int a = 0; a < nin; ++a) {
      double2 d = rhs(a + 2);
      if (a == 0) {
        d.x -= m1.x;
        d.y -= m1.y;
      }
      if (a == nin - 1) {
        d.x -= ml.x;
        d.y -= ml.y;
      }
      const double g = invden[a];
      dprev = make_double2((d.x - dprev.x) * g, (d.y - dprev.y) * g);
      M[(size_t)(a + 2) * sk] = dprev;
    }
    double2 xn = M[(size_t)(nin + 1) * sk];
    for (int a = nin - 2; a >= 0; --a) {
      const double2 dp = M[(size_t)(a + 2) * sk];
      const double g = invden[a];
      xn = make_double2(dp.x - g * xn.x, dp.y - g * xn.y);
      M[(size_t)(a + 2) * sk] = xn;
    }
  }
  const double2 m2 = M[2 * sk], ml1 = M[(size_t)(n - 3) * sk];
  M[0] = make_double2(2.0 * m1.x - m2.x, 2.0 * m1.y - m2.y);
  M[(size_t)(n - 1) * sk] = make_double2(2.0 * ml.x - ml1.x, 2.0 * ml.y - ml1.y);
}

// planes[q] ([len_rho][len_z][bs][bs], n2 fastest) -> out[rho][z][q][n2][n1] in FP64 and FP32
__global__ void vol_pack_kernel(const double2 *p0, const double2 *p1, const double2 *p2, const double2 *p3, int nq,
                                size_t nodes, int bs, double2 *o64, float2 *o32) {
  const size_t bs2 = (size_t)bs * bs;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nodes * nq * bs2) return;
  const size_t node = idx / (nq * bs2);
  const size_t rem = idx - node * nq * bs2;
  const int q = (int)(rem / bs2);
  const int e = (int)(rem - (size_t)q * bs2);  // output element n2 * bs + n1
  const int n2 = e / bs, n1 = e - n2 * bs;
  const double2 *src = q == 0 ? p0 : (q == 1 ? p1 : (q == 2 ? p2 : p3));
  const double2 v = src[node * bs2 + (size_t)n1 * bs + n2];
  o64[idx] = v;
  o32[idx] = make_float2((float)v.x, (float)v.y);
}

static std::vector<double> thomas_invden(int n) {
  const int nin = n - 4;
  std::vector<double> h(nin > 0 ? nin : 1);
  double cprev = 0.0;
  for (int a = 0; a < nin; ++a) {
    h[a] = 1.0 / (4.0 - cprev);
    cprev = h[a];
  }
  return h;
}

void build_volume_table(int kind, const double2 *raw, int len_rho, int len_z, int bs, double2 *out64, float2 *out32,
                        cudaStream_t st) {
  const size_t nodes = (size_t)len_rho * len_z, bs2 = (size_t)bs * bs;
  const int nq = kind == SG_CUBIC ? 4 : 1;
  DevBuf<double2> frr, fzz, frrzz;
  DevBuf<double> inv_r, inv_z;
  if (kind == SG_CUBIC) {
    frr.reserve(nodes * bs2);
    fzz.reserve(nodes * bs2);
    frrzz.reserve(nodes * bs2);
    const std::vector<double> hr = thomas_invden(len_rho), hz = thomas_invden(len_z);
    inv_r.reserve(hr.size());
    inv_z.reserve(hz.size());
    SG_CUDA(cudaMemcpyAsync(inv_r.ptr, hr.data(), hr.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    SG_CUDA(cudaMemcpyAsync(inv_z.ptr, hz.data(), hz.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    const size_t zrow = (size_t)len_z * bs2;
    // along rho: columns (z, n1, n2) are contiguous
    const size_t ncol_r = zrow;
    vol_moments_kernel<<<(unsigned)((ncol_r + 127) / 128), 128, 0, st>>>(raw, frr.ptr, len_rho, zrow, (int)ncol_r, 1,
                                                                        0, inv_r.ptr);
    SG_CUDA(cudaGetLastError());
    // along z, per rho row, of the values and of the rho moments
    const size_t ncol_z = (size_t)len_rho * bs2;
    vol_moments_kernel<<<(unsigned)((ncol_z + 127) / 128), 128, 0, st>>>(raw, fzz.ptr, len_z, bs2, (int)bs2, len_rho,
                                                                        zrow, inv_z.ptr);
    SG_CUDA(cudaGetLastError());
    vol_moments_kernel<<<(unsigned)((ncol_z + 127) / 128), 128, 0, st>>>(frr.ptr, frrzz.ptr, len_z, bs2, (int)bs2,
                                                                        len_rho, zrow, inv_z.ptr);
    SG_CUDA(cudaGetLastError());
  }
  const size_t total = nodes * nq * bs2;
  vol_pack_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(raw, frr.ptr, fzz.ptr, frrzz.ptr, nq, nodes, bs,
                                                                   out64, out32);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));  // the scratch planes are released on return
}

int launch_volume(sg_context *c, const double2 *x, double2 *y, int R, bool master, bool fp32, cudaStream_t st) {
  SG_REQUIRE(c->bs >= 1 && c->bs <= 96, "blocksize must be in [1, 96]");
  VolumeLaunch V{};
  CouplingLaunch &L = V.c;
  L.pos = c->pos.ptr;
  L.mofn = c->mofn.ptr;
  L.n = c->n;
  L.bs = c->bs;
  L.x = x;
  L.y = y;
  L.nrhs = R;
  L.master = master ? 1 : 0;
  L.t = c->tmat.ptr;
  L.ptype = c->ptype.ptr;
  L.t_diag = c->t_diag;
  int extra = 0;
  if (fp32) {  // one FP32 copy of the input: the kernel stages x_j from it
    const size_t len = (size_t)c->n * c->bs * R;
    c->bk_x32.reserve(len);
    k_to_f32(x, c->bk_x32.ptr, len, st);
    L.x32 = c->bk_x32.ptr;
    extra = 1;
  }
  V.z = c->vz.ptr;
  V.tpl = fp32 ? (const void *)c->vpl32.ptr : (const void *)c->vpl64.ptr;
  V.tmn = fp32 ? (const void *)c->vmn32.ptr : (const void *)c->vmn64.ptr;
  V.len_rho = c->len_rho;
  V.len_z = c->v_len_z;
  V.nq = c->v_nq;
  V.rho_min = c->rho_min;
  V.sz_min = c->v_sz_min;
  V.dz_min = c->v_dz_min;
  V.res = c->res;
  const int ns = choose_split(c->n, R);
  if (ns > 1) {
    c->w_partial.reserve((size_t)ns * c->n * c->bs * R);
    L.partial = c->w_partial.ptr;
  }
  if (fp32) launch_vr<float>(V, c->kind, ns, st);
  else launch_vr<double>(V, c->kind, ns, st);
  return (ns > 1 ? 2 : 1) + extra;
}

}  // namespace sg

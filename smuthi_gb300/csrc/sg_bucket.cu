// Interval-bucketed FP32 coupling matvec (the mixed-precision operator).
//
// The per-receiver kernel of sg_coupling.cu re-reads an interval's interpolation coefficients
// (4 x B^2 complex) from L2 for every ordered pair, which makes its FP32 form L2-bound. Here the
// receivers are grouped into tiles of T spatially adjacent particles (Morton order) and each
// tile's pairs (i in tile, any j) are sorted by lookup interval once per geometry. A CTA owns one
// tile and a range of intervals: for every non-empty interval it stages the coefficient block in
// shared memory once, and its warps apply it to all of that interval's pairs, accumulating the
// receivers' rows in shared memory (FP32, shared-memory atomics); at the end of its interval range
// the CTA adds its partial rows into an FP64 accumulator with global atomics. A final epilogue
// kernel forms W x or x - T W x in FP64.
//
// Summation order across CTAs follows the hardware's atomic order, so results may differ run to
// run in the last FP64 bits of the accumulated FP32 partials; this operator only drives the
// correction solves of the FP64 iterative refinement.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "sg_internal.h"

namespace sg {

static constexpr int kBThreads = 256;
static constexpr int kSegIntervals = 512;  // intervals per CTA segment

// ------------------------------------------------------------------ plan construction
__global__ void bucket_keys_kernel(const double2 *pos, const int *members, int n, int T, int n_tiles,
                                   double rho_min, double res, int n_int, int kbits, unsigned *keys, unsigned *vals,
                                   int *counts) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)n_tiles * T * n;
  if (p >= total) return;
  const size_t slot = p / n;
  const int j = (int)(p - slot * n);
  const int i = members[slot];
  if (i < 0) {
    keys[p] = 0xFFFFFFFFu;
    vals[p] = 0u;
    return;
  }
  const int tile = (int)(slot / T), a = (int)(slot - (size_t)tile * T);
  const double dx = pos[i].x - pos[j].x, dy = pos[i].y - pos[j].y;
  const double sidx = (sqrt(dx * dx + dy * dy) - rho_min) / res;
  int k = (int)floor(sidx);
  k = k < 0 ? 0 : (k > n_int - 1 ? n_int - 1 : k);
  keys[p] = ((unsigned)tile << kbits) | (unsigned)k;
  vals[p] = ((unsigned)a << 16) | (unsigned)j;
  atomicAdd(&counts[(size_t)tile * n_int + k], 1);
}

__global__ void bucket_records_kernel(const double2 *pos, const int *members, int T, int kbits,
                                      const unsigned *keys, const unsigned *vals, size_t count, double rho_min,
                                      double res, int n_int, int4 *rec) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  const unsigned v = vals[p], key = keys[p];
  const int tile = (int)(key >> kbits), a = (int)(v >> 16), j = (int)(v & 0xFFFFu);
  const int i = members[(size_t)tile * T + a];
  const double dx = pos[i].x - pos[j].x, dy = pos[i].y - pos[j].y;
  const double rho = sqrt(dx * dx + dy * dy);
  const double sidx = (rho - rho_min) / res;
  const double fl = floor(sidx);
  int k = (int)fl;
  const int kc = k < 0 ? 0 : (k > n_int - 1 ? n_int - 1 : k);
  const double t = sidx - (double)kc;  // kc == k inside the table
  float c = 1.0f, s = 0.0f;
  if (rho > 0.0) {
    c = (float)(dx / rho);
    s = (float)(dy / rho);
  }
  rec[p] = make_int4((int)v, __float_as_int((float)t), __float_as_int(c), __float_as_int(s));
}

static unsigned morton2(unsigned x, unsigned y) {
  auto spread = [](unsigned v) {
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
  };
  return spread(x) | (spread(y) << 1);
}

bool bucket_supported(const sg_context *c) { return c->n <= 65536 && c->n_int <= (1 << 16); }

void build_bucket_plan(sg_context *c, cudaStream_t st) {
  SG_REQUIRE(bucket_supported(c), "bucketed FP32 operator needs <= 65536 particles and <= 65536 intervals");
  const int n = c->n, n_int = c->n_int;
  const int T = c->bs <= 32 ? 16 : 8;
  const int n_tiles = (n + T - 1) / T;
  int kbits = 1;
  while ((1 << kbits) < n_int) ++kbits;
  SG_REQUIRE(kbits + 32 - __builtin_clz((unsigned)std::max(1, n_tiles)) <= 32, "bucket key does not fit 32 bits");
  // Morton order of the receivers
  std::vector<double2> pos(n);
  SG_CUDA(cudaMemcpy(pos.data(), c->pos.ptr, n * sizeof(double2), cudaMemcpyDeviceToHost));
  double x0 = pos[0].x, x1 = pos[0].x, y0 = pos[0].y, y1 = pos[0].y;
  for (auto &p : pos) {
    x0 = std::min(x0, p.x);
    x1 = std::max(x1, p.x);
    y0 = std::min(y0, p.y);
    y1 = std::max(y1, p.y);
  }
  const double sx = x1 > x0 ? 65535.0 / (x1 - x0) : 0.0, sy = y1 > y0 ? 65535.0 / (y1 - y0) : 0.0;
  std::vector<unsigned> code(n);
  for (int i = 0; i < n; ++i) code[i] = morton2((unsigned)((pos[i].x - x0) * sx), (unsigned)((pos[i].y - y0) * sy));
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return code[a] < code[b]; });
  std::vector<int> members((size_t)n_tiles * T, -1);
  for (int q = 0; q < n; ++q) members[q] = perm[q];
  c->bk_members.reserve(members.size());
  SG_CUDA(cudaMemcpyAsync(c->bk_members.ptr, members.data(), members.size() * sizeof(int), cudaMemcpyHostToDevice,
                          st));
  // keys, counts, stable sort, records, offsets
  const size_t total = (size_t)n_tiles * T * n, valid = (size_t)n * n;
  const size_t nbins = (size_t)n_tiles * n_int;
  DevBuf<unsigned> keys, vals, keys2, vals2;
  keys.reserve(total);
  vals.reserve(total);
  keys2.reserve(total);
  vals2.reserve(total);
  c->bk_offs.reserve(nbins + 1);
  SG_CUDA(cudaMemsetAsync(c->bk_offs.ptr, 0, (nbins + 1) * sizeof(int), st));
  bucket_keys_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c->pos.ptr, c->bk_members.ptr, n, T, n_tiles,
                                                                      c->rho_min, c->res, n_int, kbits, keys.ptr,
                                                                      vals.ptr, c->bk_offs.ptr);
  SG_CUDA(cudaGetLastError());
  size_t tmp_bytes = 0, scan_bytes = 0;
  SG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.ptr, keys2.ptr, vals.ptr, vals2.ptr,
                                          (int64_t)total, 0, 32, st));
  SG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, c->bk_offs.ptr, c->bk_offs.ptr, (int64_t)(nbins + 1),
                                        st));
  DevBuf<unsigned char> tmp;
  tmp.reserve(std::max(tmp_bytes, scan_bytes));
  SG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.ptr, tmp_bytes, keys.ptr, keys2.ptr, vals.ptr, vals2.ptr,
                                          (int64_t)total, 0, 32, st));
  SG_CUDA(cub::DeviceScan::ExclusiveSum(tmp.ptr, scan_bytes, c->bk_offs.ptr, c->bk_offs.ptr, (int64_t)(nbins + 1),
                                        st));
  c->bk_rec.reserve(valid);
  bucket_records_kernel<<<(unsigned)((valid + 255) / 256), 256, 0, st>>>(c->pos.ptr, c->bk_members.ptr, T, kbits,
                                                                         keys2.ptr, vals2.ptr, valid, c->rho_min,
                                                                         c->res, n_int, c->bk_rec.ptr);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));  // temporaries are released on return
  c->bk_T = T;
  c->bk_tiles = n_tiles;
  c->bk_S = (n_int + kSegIntervals - 1) / kSegIntervals;
  c->launches += 4;
}

// ------------------------------------------------------------------ matvec kernels
__global__ void to_f32_kernel(const double2 *x, float2 *y, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) y[e] = make_float2((float)x[e].x, (float)x[e].y);
}

void k_to_f32(const double2 *x, float2 *y, size_t n, cudaStream_t st) {
  to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, y, n);
  SG_CUDA(cudaGetLastError());
}

struct BucketArgs {
  const int *members;
  const int4 *rec;
  const int *offs;
  const float2 *coef;  // [n_int][NC][bs][bs], n1 fastest
  const int *mofn;
  const float2 *x32;   // [N][bs][R]
  double2 *yacc;       // [N][bs][R]
  int n, bs, n_int, T, S, R;
};

template <int NC, int RT, int P>
__global__ void __launch_bounds__(kBThreads) bucket_kernel(const BucketArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int bs = a.bs, R = a.R, T = a.T;
  const size_t bs2 = (size_t)bs * bs;
  float2 *coef_s = reinterpret_cast<float2 *>(smem_raw);
  float2 *acc_s = coef_s + NC * bs2;                 // [T][RT][bs]: lane-consecutive rows, no bank conflicts
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  float2 *ubuf = acc_s + (size_t)T * bs * RT + (size_t)warp * bs * RT;
  const int tile = blockIdx.x / a.S, seg = blockIdx.x - tile * a.S;
  const int r0 = blockIdx.y * RT;
  const int k0 = seg * kSegIntervals, k1 = min(a.n_int, k0 + kSegIntervals);
  for (int e = threadIdx.x; e < T * bs * RT; e += blockDim.x) acc_s[e] = make_float2(0.f, 0.f);

  int nrow[P], nrowc[P], mrow[P];
  bool valid[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    nrow[q] = lane + 32 * q;
    valid[q] = nrow[q] < bs;
    nrowc[q] = valid[q] ? nrow[q] : bs - 1;
    mrow[q] = a.mofn[nrowc[q]];
  }
  const int *offs = a.offs + (size_t)tile * a.n_int;
  for (int k = k0; k < k1; ++k) {
    const int p0 = offs[k], p1 = offs[k + 1];
    if (p0 == p1) continue;
    __syncthreads();  // previous interval's readers are done with coef_s
    {
      const float4 *src = reinterpret_cast<const float4 *>(a.coef + (size_t)k * NC * bs2);
      float4 *dst = reinterpret_cast<float4 *>(coef_s);
      const int n4 = (int)(NC * bs2 / 2);
      for (int e = threadIdx.x; e < n4; e += blockDim.x) dst[e] = __ldg(src + e);
    }
    __syncthreads();
    for (int p = p0 + warp; p < p1; p += nw) {
      const int4 rd = a.rec[p];
      const unsigned v = (unsigned)rd.x;
      const int ai = (int)(v >> 16), j = (int)(v & 0xFFFFu);
      const float t = __int_as_float(rd.y), c = __int_as_float(rd.z), s = __int_as_float(rd.w);
      float ph_re[P], ph_im[P];
#pragma unroll
      for (int q = 0; q < P; ++q) {
        const int am = mrow[q] < 0 ? -mrow[q] : mrow[q];
        float pr = 1.f, pi = 0.f;
        for (int b = 0; b < am; ++b) {
          const float nr = pr * c - pi * s;
          pi = pr * s + pi * c;
          pr = nr;
        }
        ph_re[q] = pr;
        ph_im[q] = mrow[q] < 0 ? -pi : pi;
        if (valid[q]) {
          const float2 *xs = a.x32 + ((size_t)j * bs + nrow[q]) * R + r0;
#pragma unroll
          for (int r = 0; r < RT; ++r) {
            const float2 xv = xs[r];
            ubuf[r * bs + nrow[q]] = make_float2(pr * xv.x - ph_im[q] * xv.y, pr * xv.y + ph_im[q] * xv.x);
          }
        }
      }
      __syncwarp();
      float pa_re[P][RT], pa_im[P][RT];
#pragma unroll
      for (int q = 0; q < P; ++q)
#pragma unroll
        for (int r = 0; r < RT; ++r) pa_re[q][r] = pa_im[q][r] = 0.f;
      for (int n2 = 0; n2 < bs; ++n2) {
        float2 u[RT];
#pragma unroll
        for (int r = 0; r < RT; ++r) u[r] = ubuf[r * bs + n2];
#pragma unroll
        for (int q = 0; q < P; ++q) {
          const float2 *cp = coef_s + (size_t)n2 * bs + nrowc[q];
          float2 cc = cp[(NC - 1) * bs2];
          float lr = cc.x, li = cc.y;
#pragma unroll
          for (int ci = NC - 2; ci >= 0; --ci) {
            const float2 d = cp[ci * bs2];
            lr = fmaf(lr, t, d.x);
            li = fmaf(li, t, d.y);
          }
#pragma unroll
          for (int r = 0; r < RT; ++r) {
            pa_re[q][r] = fmaf(lr, u[r].x, pa_re[q][r]);
            pa_re[q][r] = fmaf(-li, u[r].y, pa_re[q][r]);
            pa_im[q][r] = fmaf(lr, u[r].y, pa_im[q][r]);
            pa_im[q][r] = fmaf(li, u[r].x, pa_im[q][r]);
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < P; ++q) {
        if (!valid[q]) continue;
        float2 *dst = acc_s + (size_t)ai * RT * bs + nrow[q];
#pragma unroll
        for (int r = 0; r < RT; ++r) {
          atomicAdd(&dst[r * bs].x, ph_re[q] * pa_re[q][r] + ph_im[q] * pa_im[q][r]);
          atomicAdd(&dst[r * bs].y, ph_re[q] * pa_im[q][r] - ph_im[q] * pa_re[q][r]);
        }
      }
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < T * bs * RT; e += blockDim.x) {
    const int ai = e / (bs * RT), rem = e - ai * bs * RT;
    const int r = rem / bs, n1 = rem - r * bs;
    const int i = a.members[(size_t)tile * T + ai];
    if (i < 0) continue;
    const float2 v = acc_s[e];
    if (v.x == 0.f && v.y == 0.f) continue;
    double2 *dst = a.yacc + ((size_t)i * bs + n1) * R + r0 + r;
    atomicAdd(&dst->x, (double)v.x);
    atomicAdd(&dst->y, (double)v.y);
  }
}

// y = yacc (coupling) or x - T yacc (master), FP64
__global__ void bucket_epilogue_kernel(const double2 *yacc, const double2 *x, const double2 *t, const int *ptype,
                                       int t_diag, int master, int n, int bs, int R, double2 *y) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t len = (size_t)n * bs * R;
  if (e >= len) return;
  if (!master) {
    y[e] = yacc[e];
    return;
  }
  const int r = (int)(e % R);
  const size_t row = e / R;
  const int i = (int)(row / bs), n1 = (int)(row - (size_t)i * bs);
  const int ty = ptype[i];
  double ar, ai;
  if (t_diag) {
    const double2 tv = t[(size_t)ty * bs + n1], w = yacc[e];
    ar = tv.x * w.x - tv.y * w.y;
    ai = tv.x * w.y + tv.y * w.x;
  } else {
    ar = 0.0;
    ai = 0.0;
    const double2 *trow = t + ((size_t)ty * bs + n1) * bs;
    for (int n2 = 0; n2 < bs; ++n2) {
      const double2 tv = trow[n2], w = yacc[((size_t)i * bs + n2) * R + r];
      ar = fma(tv.x, w.x, fma(-tv.y, w.y, ar));
      ai = fma(tv.x, w.y, fma(tv.y, w.x, ai));
    }
  }
  y[e] = make_double2(x[e].x - ar, x[e].y - ai);
}

template <int NC, int RT, int P>
static void launch_bucket_t(const BucketArgs &a, cudaStream_t st) {
  const size_t smem = ((size_t)NC * a.bs * a.bs + (size_t)a.T * a.bs * RT + (size_t)(kBThreads / 32) * a.bs * RT) *
                      sizeof(float2);
  SG_REQUIRE(smem <= 220 * 1024, "bucketed operator: shared memory request too large");
  static bool attr[64] = {};
  if (first_on_device(attr))
    SG_CUDA(cudaFuncSetAttribute(bucket_kernel<NC, RT, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
  dim3 grid(a.T > 0 ? (unsigned)((size_t)((a.n + a.T - 1) / a.T) * a.S) : 0u, a.R / RT);
  bucket_kernel<NC, RT, P><<<grid, kBThreads, smem, st>>>(a);
  SG_CUDA(cudaGetLastError());
}

template <int NC, int RT>
static void launch_bucket_p(const BucketArgs &a, cudaStream_t st) {
  const int P = (a.bs + 31) / 32;
  if (P == 1) launch_bucket_t<NC, RT, 1>(a, st);
  else if (P == 2) launch_bucket_t<NC, RT, 2>(a, st);
  else launch_bucket_t<NC, RT, 3>(a, st);
}

template <int NC>
static void launch_bucket_r(const BucketArgs &a, int RT, cudaStream_t st) {
  switch (RT) {
    case 16: launch_bucket_p<NC, 16>(a, st); break;
    case 8: launch_bucket_p<NC, 8>(a, st); break;
    case 4: launch_bucket_p<NC, 4>(a, st); break;
    case 2: launch_bucket_p<NC, 2>(a, st); break;
    default: launch_bucket_p<NC, 1>(a, st); break;
  }
}

// Returns the number of kernels launched.
int launch_bucket_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  const size_t len = (size_t)c->n * c->bs * R;
  c->bk_x32.reserve(len);
  c->bk_yacc.reserve(len);
  to_f32_kernel<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(x, c->bk_x32.ptr, len);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaMemsetAsync(c->bk_yacc.ptr, 0, len * sizeof(double2), st));
  int RT = 1;
  for (int cand : {16, 8, 4, 2, 1})
    if (R % cand == 0) {
      RT = cand;
      break;
    }
  // keep the shared-memory footprint inside the opt-in limit for the large blocksizes
  while (RT > 1 && ((size_t)c->ncoef * c->bs * c->bs + (size_t)c->bk_T * c->bs * RT + 8 * (size_t)c->bs * RT) *
                           sizeof(float2) > 220 * 1024)
    RT /= 2;
  BucketArgs a{c->bk_members.ptr, c->bk_rec.ptr, c->bk_offs.ptr, c->coef32.ptr, c->mofn.ptr, c->bk_x32.ptr,
               c->bk_yacc.ptr, c->n, c->bs, c->n_int, c->bk_T, c->bk_S, R};
  if (c->ncoef == 2) launch_bucket_r<2>(a, RT, st);
  else launch_bucket_r<4>(a, RT, st);
  bucket_epilogue_kernel<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(
      c->bk_yacc.ptr, x, c->tmat.ptr, c->ptype.ptr, c->t_diag, master ? 1 : 0, c->n, c->bs, R, y);
  SG_CUDA(cudaGetLastError());
  return 3;
}

}  // namespace sg

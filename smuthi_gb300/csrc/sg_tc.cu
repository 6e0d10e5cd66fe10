// Tensor-core (tcgen05, 3xTF32) form of the FP32 coupling operator for batched right-hand sides.
//
// Per ordered pair (i, j) the full coupling block W_ij = e^{-i m1 phi} L(rho_ij) e^{i m2 phi}
// (B x B complex, B <= 32) is a dense contraction with the RHS panel x_j (B x R complex):
//
//   [Re W; Im W] (2 x 32 rows, K = 32) x [Re x_j | Im x_j] (K = 32, N = 2R columns)
//     = [[Wr xr, Wr xi], [Wi xr, Wi xi]]
//   Re y_i = Wr xr - Wi xi,  Im y_i = Wr xi + Wi xr.
//
// One CTA owns two receiving particles (M = 128 accumulator rows: receiver 0 in rows 0-63,
// receiver 1 in rows 64-127) and streams every emitter j. For each j the CUDA cores interpolate
// the interval's coefficients (FP32 Horner), fold in the phase e^{i (m2 - m1) phi}, split every
// value into a TF32 high part and an FP32 remainder (3xTF32: hi*hi + hi*lo + lo*hi) and store the
// block into shared memory in the canonical no-swizzle K-major layout; x_j's pre-split panel is
// copied next to it. One thread issues the tcgen05.mma instructions (kind::tf32, M=128, N=2R, K=8
// each) that accumulate into tensor memory across all j; the A/x stages are double-buffered and
// freed by tcgen05.commit arrivals on an mbarrier. Every mbarrier wait is bounded by a clock
// budget: on expiry the kernel records an error, waits (bounded) for its issued MMAs, frees its
// tensor memory and returns. The epilogue reads the accumulators with tcgen05.ld, combines real and
// imaginary parts in FP64 and applies the master epilogue x - T (W x).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sg_internal.h"

namespace sg {

static constexpr int kTcThreads = 256;
static constexpr int kBP = 32;         // padded block size (K of the contraction and rows per part)
static constexpr int kKC = kBP / 4;    // 16-byte core-matrix columns along K
static constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz per wait

// float offset of element (row, k) in a canonical no-swizzle K-major tile with kKC core columns:
// core matrix (row / 8, k / 4) is 8 rows x 16 bytes, stored contiguously (128 bytes); core
// matrices adjacent in K are 128 bytes apart (LBO), adjacent 8-row groups kKC * 128 bytes (SBO).
__device__ __forceinline__ int tc_off(int row, int k) {
  return (((row >> 3) * kKC + (k >> 2)) << 5) + ((row & 7) << 2) + (k & 3);
}

__device__ __forceinline__ float tf32_hi(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start, LBO = 128 B, SBO = kKC * 128 B, no swizzle, version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)(((kKC * 128) >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kWaitCycles) return false;
  }
}

struct TcArgs {
  const int4 *pairs;    // [N][N] (interval, t, cos phi, sin phi)
  const float2 *coef;   // FP32 coefficients [interval][c][n2][n1]
  const int *mofn;      // [bs]
  const float *xop;     // pre-split panels: per particle [hi | lo] tiles of 2R x kBP floats
  const double2 *x;     // FP64 input (master epilogue), padded [N][bs][R]
  double2 *y;
  const double2 *t;     // T blocks (diagonal)
  const int *ptype;
  int master;
  int n, bs, R, ncoef;
  int dmax;             // largest |m2 - m1| (phase-table length - 1), <= 32
  int *err;             // set to 1 when a wait runs out
};

// Pre-split panels: xop[j][h][tc_off(c, n2)] = hi/lo of (c < R ? Re : Im) x[j][n2][c mod R]
__global__ void tc_split_x_kernel(const double2 *x, float *xop, int n, int bs, int R) {
  const int NN = 2 * R;
  const size_t tile = (size_t)NN * kBP;
  const size_t total = (size_t)n * tile;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / tile);
    const int rem = (int)(e - (size_t)j * tile);
    const int c = rem / kBP, n2 = rem - c * kBP;
    float v = 0.f;
    if (n2 < bs) {
      const double2 xv = x[((size_t)j * bs + n2) * R + (c < R ? c : c - R)];
      v = (float)(c < R ? xv.x : xv.y);
    }
    const float hi = tf32_hi(v);
    float *base = xop + (size_t)j * 2 * tile;
    base[tc_off(c, n2)] = hi;
    base[tile + tc_off(c, n2)] = v - hi;
  }
}

template <int NC, int R>
__global__ void __launch_bounds__(kTcThreads, 1) tc_coupling_kernel(const TcArgs a) {
  constexpr int NN = 2 * R;             // MMA N
  constexpr int ATILE = 128 * kBP;      // floats per A tile (one of hi / lo)
  constexpr int XTILE = NN * kBP;       // floats per x tile
  // Tensor-memory columns. The hi*hi products accumulate in one accumulator, the two correction
  // products (hi*lo, lo*hi, ~2^-11 smaller) in another, and even and odd emitters use separate
  // accumulator pairs: the tensor core's accumulation into tensor memory loses precision roughly
  // in proportion to the number of instructions accumulated (measured: one accumulator 1.3e-5,
  // main/correction split 4.4e-6, plus even/odd split 2.2e-6 relative at 60 emitters), so shorter
  // chains and the FP64 sum of the four accumulators in the epilogue keep it FP32-like.
  constexpr int NCOLS = 4 * NN;  // 64, 128 or 256
  static_assert(NCOLS >= 32 && NCOLS <= 256, "tensor-memory columns");
  static_assert(NN == 16 || NN == 32 || NN == 64, "2R must be 16, 32 or 64");
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  float *As = reinterpret_cast<float *>(tc_smem);             // [2 stages][hi, lo][ATILE]
  float *Xs = As + 4 * ATILE;                                 // [2 stages][hi, lo][XTILE]
  float2 *ph = reinterpret_cast<float2 *>(Xs + 4 * XTILE);    // [2 bufs][2 receivers][33] e^{i d phi}
  int *pk = reinterpret_cast<int *>(ph + 2 * 2 * 33);         // [2 bufs][2]
  float *pt = reinterpret_cast<float *>(pk + 4);              // [2 bufs][2]
  // 2 stage mbarriers and one for the final commit after a timeout (8-byte aligned: offsets are multiples of 8)
  uint64_t *bars = reinterpret_cast<uint64_t *>(pt + 4 + 2);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 3);
  int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int bs = a.bs, N = a.n, bs2 = bs * bs;
  const int i0 = 2 * blockIdx.x;
  const int nrecv = (i0 + 1 < N) ? 2 : 1;

  // zero both A stages (padding rows and columns stay zero) and set up barriers
  for (int e = tid; e < 4 * ATILE; e += kTcThreads) As[e] = 0.f;
  if (tid == 0) {
    *abort_flag = 0;
    for (int s = 0; s < 3; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // pair data and phase tables of emitter 0
  auto pair_setup = [&](int j, int buf) {
    if (tid < 2) {
      const int i = (tid < nrecv) ? i0 + tid : i0;
      const int4 pd = a.pairs[(size_t)i * N + j];
      pk[buf * 2 + tid] = pd.x;
      pt[buf * 2 + tid] = __int_as_float(pd.y);
      const float c = __int_as_float(pd.z), s = __int_as_float(pd.w);
      float2 *p = ph + (buf * 2 + tid) * 33;
      float pr = 1.f, pi = 0.f;
      p[0] = make_float2(1.f, 0.f);
      for (int d = 1; d <= a.dmax; ++d) {
        const float nr = pr * c - pi * s;
        pi = pr * s + pi * c;
        pr = nr;
        p[d] = make_float2(pr, pi);
      }
    }
  };
  pair_setup(0, 0);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

  // lane -> (8 rows x 4 columns) core tile; warp -> tiles (receiver, row block, column block)
  const int l_n1 = lane & 7, l_n2 = lane >> 3;
  int jj = 0;
  for (; jj < N; ++jj) {
    const int s = jj & 1, buf = jj & 1;
    if (jj >= 2) {
      if (!mbar_wait(smem_u32(&bars[s]), (uint32_t)(((jj - 2) >> 1) & 1))) *abort_flag = 1;
    }
    __syncthreads();  // every thread sees the abort flag and the freed stage
    if (*abort_flag) break;
    float *Ah = As + (size_t)s * 2 * ATILE, *Al = Ah + ATILE;
    // 2 receivers x 4 row blocks x 8 column blocks = 64 core tiles over 8 warps; all coefficient
    // loads of a warp's 8 tiles are issued before any is used (one L2 latency per emitter)
    {
      float2 cf[8][NC];
      int nn1[8], nn2[8], rr[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int tile = warp + 8 * u;
        rr[u] = tile >> 5;
        nn1[u] = ((tile >> 3) & 3) * 8 + l_n1;
        nn2[u] = (tile & 7) * 4 + l_n2;
        const bool in = nn1[u] < bs && nn2[u] < bs;
        const int k = pk[buf * 2 + rr[u]];
        const float2 *cp = a.coef + (size_t)k * NC * bs2 + (size_t)(in ? nn2[u] : 0) * bs + (in ? nn1[u] : 0);
#pragma unroll
        for (int ci = 0; ci < NC; ++ci) cf[u][ci] = __ldg(cp + ci * bs2);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int n1 = nn1[u], n2 = nn2[u], r = rr[u];
        if (n1 < bs && n2 < bs) {
          const float t = pt[buf * 2 + r];
          float lr = cf[u][NC - 1].x, li = cf[u][NC - 1].y;
#pragma unroll
          for (int ci = NC - 2; ci >= 0; --ci) {
            lr = fmaf(lr, t, cf[u][ci].x);
            li = fmaf(li, t, cf[u][ci].y);
          }
          const int dm = a.mofn[n2] - a.mofn[n1];
          float2 e = ph[(buf * 2 + r) * 33 + (dm < 0 ? -dm : dm)];
          if (dm < 0) e.y = -e.y;
          const float wr = lr * e.x - li * e.y, wi = lr * e.y + li * e.x;
          const float wrh = tf32_hi(wr), wih = tf32_hi(wi);
          const int row = r * 64 + n1;
          Ah[tc_off(row, n2)] = wrh;
          Al[tc_off(row, n2)] = wr - wrh;
          Ah[tc_off(row + 32, n2)] = wih;
          Al[tc_off(row + 32, n2)] = wi - wih;
        }
      }
    }
    // x_j panel (hi, lo) into stage s
    {
      const float4 *src = reinterpret_cast<const float4 *>(a.xop + (size_t)jj * 2 * XTILE);
      float4 *dst = reinterpret_cast<float4 *>(Xs + (size_t)s * 2 * XTILE);
      for (int e = tid; e < 2 * XTILE / 4; e += kTcThreads) dst[e] = __ldg(src + e);
    }
    if (jj + 1 < N) pair_setup(jj + 1, buf ^ 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_hi = smem_u32(Ah), a_lo = smem_u32(Al);
      const uint32_t x_hi = smem_u32(Xs + (size_t)s * 2 * XTILE), x_lo = x_hi + XTILE * 4;
#pragma unroll
      for (int ks = 0; ks < kBP / 8; ++ks) {
        const uint32_t koff = ks * 256;  // two 128-byte core matrices per K step of 8
#pragma unroll
        for (int prod = 0; prod < 3; ++prod) {
          const uint32_t aa = (prod == 2 ? a_lo : a_hi) + koff;
          const uint32_t bb = (prod == 1 ? x_lo : x_hi) + koff;
          const uint32_t acc = (jj > 1 || ks > 0 || prod > 1) ? 1u : 0u;
          const uint32_t dcol = tmem + (uint32_t)((jj & 1) * 2 * NN + (prod == 0 ? 0 : NN));
          asm volatile(
              "{\n\t.reg .pred p;\n\t"
              "setp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dcol),
              "l"(tc_desc(aa)), "l"(tc_desc(bb)), "r"(idesc), "r"(acc)
              : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bars[s]))
                   : "memory");
    }
  }
  // drain: wait for the last commit of each stage that was used (bounded)
  const int issued = jj;  // emitters whose MMAs were issued
  bool ok = true;
  for (int s = 0; s < 2; ++s) {
    const int ns = issued > s ? (issued - s + 1) / 2 : 0;  // commits on stage s
    if (ns > 0 && !mbar_wait(smem_u32(&bars[s]), (uint32_t)((ns - 1) & 1))) ok = false;
  }
  ok = __syncthreads_and(ok) != 0;  // one verdict for the whole CTA (the epilogue's loads are warp-collective)
  if (!ok) {
    // a drain wait ran out: MMAs of this CTA may still be running. One more commit tracks every
    // tcgen05 operation the issuing thread started; wait for it (bounded) before the tensor memory
    // is freed, so that no MMA writes columns that another CTA may allocate next. The output of this
    // launch is undefined either way and the error flag is set.
    if (tid == 0)
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bars[2]))
                   : "memory");
    (void)mbar_wait(smem_u32(&bars[2]), 0u);
    __syncthreads();
  }
  if (!ok || *abort_flag) {
    if (tid == 0) atomicExch(a.err, 1);
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool good = ok && issued == N;
  // epilogue: warps 0-3 read their 32 accumulator lanes into shared memory (the A stages are free)
  double *Ds = reinterpret_cast<double *>(As);  // [128][NN] FP64 sum of the accumulators (64 KB at NN = 64)
  const int nparts = N > 1 ? 4 : 2;  // the odd-emitter accumulators exist only when N > 1
  for (int part = 0; part < nparts && good && warp < 4; ++part) {
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(part * NN);
    float v[NN];
    if constexpr (NN == 16) {
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
            "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
          : "r"(taddr));
    } else {
#pragma unroll
      for (int c0 = 0; c0 < NN; c0 += 32) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=f"(v[c0 + 0]), "=f"(v[c0 + 1]), "=f"(v[c0 + 2]), "=f"(v[c0 + 3]), "=f"(v[c0 + 4]), "=f"(v[c0 + 5]),
              "=f"(v[c0 + 6]), "=f"(v[c0 + 7]), "=f"(v[c0 + 8]), "=f"(v[c0 + 9]), "=f"(v[c0 + 10]),
              "=f"(v[c0 + 11]), "=f"(v[c0 + 12]), "=f"(v[c0 + 13]), "=f"(v[c0 + 14]), "=f"(v[c0 + 15]),
              "=f"(v[c0 + 16]), "=f"(v[c0 + 17]), "=f"(v[c0 + 18]), "=f"(v[c0 + 19]), "=f"(v[c0 + 20]),
              "=f"(v[c0 + 21]), "=f"(v[c0 + 22]), "=f"(v[c0 + 23]), "=f"(v[c0 + 24]), "=f"(v[c0 + 25]),
              "=f"(v[c0 + 26]), "=f"(v[c0 + 27]), "=f"(v[c0 + 28]), "=f"(v[c0 + 29]), "=f"(v[c0 + 30]),
              "=f"(v[c0 + 31])
            : "r"(taddr + (uint32_t)c0));
      }
    }
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int row = warp * 32 + lane;
#pragma unroll
    for (int c = 0; c < NN; ++c) Ds[row * NN + c] = (part ? Ds[row * NN + c] : 0.0) + (double)v[c];
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS) : "memory");
  }
  if (!good) return;
  for (int e = tid; e < nrecv * bs * R; e += kTcThreads) {
    const int r = e / (bs * R), rem = e - r * bs * R, n1 = rem / R, c = rem - n1 * R;
    const int i = i0 + r;
    const double *d0 = Ds + (size_t)(r * 64 + n1) * NN, *d1 = Ds + (size_t)(r * 64 + 32 + n1) * NN;
    const double yr = d0[c] - d1[R + c];
    const double yi = d0[R + c] + d1[c];
    const size_t o = ((size_t)i * bs + n1) * R + c;
    if (a.master) {
      const double2 tv = a.t[(size_t)a.ptype[i] * bs + n1];
      const double2 xv = a.x[o];
      a.y[o] = make_double2(xv.x - (tv.x * yr - tv.y * yi), xv.y - (tv.x * yi + tv.y * yr));
    } else {
      a.y[o] = make_double2(yr, yi);
    }
  }
}

bool tc_supported(const sg_context *c, int R) {
  return c->bs <= kBP && c->uniform && c->t_diag && (R == 8 || R == 16 || R == 32) && c->pairs_ready;
}

template <int NC, int R>
static void tc_launch_t(const TcArgs &a, cudaStream_t st) {
  constexpr int NN = 2 * R;
  const size_t smem = (size_t)(4 * 128 * kBP + 4 * NN * kBP) * sizeof(float) + 2 * 2 * 33 * sizeof(float2) +
                      4 * sizeof(int) + 6 * sizeof(float) + 3 * sizeof(uint64_t) + 2 * sizeof(uint32_t) + 64;
  static bool attr_done[64] = {};
  if (first_on_device(attr_done))
    SG_CUDA(cudaFuncSetAttribute(tc_coupling_kernel<NC, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tc_coupling_kernel<NC, R><<<(a.n + 1) / 2, kTcThreads, smem, st>>>(a);
  SG_CUDA(cudaGetLastError());
}

// y = M x or W x with the tensor-core operator; returns the number of kernels launched
int launch_tc_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  SG_REQUIRE(tc_supported(c, R), "tensor-core operator: needs blocksize <= 32, uniform diagonal T, nrhs in {8,16,32}");
  const size_t xop_len = (size_t)c->n * 2 * (2 * R) * kBP;
  c->tc_xop.reserve(xop_len);
  c->tc_err.reserve(1);
  if (!c->tc_err_init) {
    SG_CUDA(cudaMemsetAsync(c->tc_err.ptr, 0, sizeof(int), st));
    c->tc_err_init = true;
  }
  const size_t total = (size_t)c->n * (2 * R) * kBP;
  tc_split_x_kernel<<<(unsigned)std::min<size_t>((total + 255) / 256, (size_t)sm_count() * 16), 256, 0, st>>>(x, c->tc_xop.ptr, c->n,
                                                                                              c->bs, R);
  SG_CUDA(cudaGetLastError());
  TcArgs a{};
  a.pairs = c->pairs.ptr;
  a.coef = c->coef32.ptr;
  a.mofn = c->mofn.ptr;
  a.xop = c->tc_xop.ptr;
  a.x = x;
  a.y = y;
  a.t = c->tmat.ptr;
  a.ptype = c->ptype.ptr;
  a.master = master ? 1 : 0;
  a.n = c->n;
  a.bs = c->bs;
  a.R = R;
  a.ncoef = c->ncoef;
  int mmax = 0;
  for (int m : c->h_mofn) mmax = std::max(mmax, m < 0 ? -m : m);
  a.dmax = 2 * mmax;
  a.err = c->tc_err.ptr;
  if (c->ncoef == 2) {
    if (R == 8) tc_launch_t<2, 8>(a, st);
    else if (R == 16) tc_launch_t<2, 16>(a, st);
    else tc_launch_t<2, 32>(a, st);
  } else {
    if (R == 8) tc_launch_t<4, 8>(a, st);
    else if (R == 16) tc_launch_t<4, 16>(a, st);
    else tc_launch_t<4, 32>(a, st);
  }
  return 2;
}

// reads and clears the tensor-core kernels' error flag (synchronises the stream)
bool tc_check_error(sg_context *c, cudaStream_t st) {
  if (!c->tc_err_init) return false;
  int h = 0;
  SG_CUDA(cudaMemcpyAsync(&h, c->tc_err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (h) SG_CUDA(cudaMemsetAsync(c->tc_err.ptr, 0, sizeof(int), st));
  return h != 0;
}

}  // namespace sg

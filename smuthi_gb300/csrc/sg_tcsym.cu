// Pair-symmetric tensor-core (tcgen05, 3xTF32) FP32 coupling operator for 16 or 32 right-hand sides
// and blocksize <= 32.
//
// For particles at one height the block of the reverse pair is the same interpolated block with
// signs, W_ji = S W_ij S with S = diag((-1)^{m(n)}), so one interpolated block W_ij serves both
// directions: y_i += W_ij x_j and y_j += S (W_ij (S x_i)). This kernel builds every unordered
// pair's block once (the operator of sg_tc.cu builds it once per ordered pair, so this halves the
// producer work and the coefficient stream).
//
// A CTA owns a pair of receiving particles i1 = 2I, i2 = 2I + 1 and a run of emitters j (a work
// item). For each emitter the producer warps build A = [Re W_i1j; Im W_i1j; Re W_i2j; Im W_i2j]
// (128 rows, K = 32, TF32 hi and lo) exactly as sg_tc.cu does, and one thread issues two MMA groups
// on it (M = 128, K = 8 steps, hi*hi + hi*lo + lo*hi):
//
//   * direction 1: D1 += A x [Re x_j | Im x_j] (N = 2R), accumulated over the item's emitters in
//     tensor memory and drained into an FP32 total every `win` emitters (as in sg_tc.cu);
//   * direction 2 (emitters j >= 2I + 2 only): D2 = A x [S x_i1 | S x_i2] (N = 4R, both receivers'
//     sign-flipped panels side by side, staged once per item). Its diagonal blocks
//     W_i1j S x_i1 (rows 0-63, columns 0..2R-1) and W_i2j S x_i2 (rows 64-127, columns 2R..4R-1)
//     sum to W_i1j S x_i1 + W_i2j S x_i2; the off-diagonal blocks are not used. Four drain warps read
//     the two blocks out of tensor memory (D2 is double-buffered), add them, combine real and
//     imaginary parts, apply S and add the result to y_j with 16-byte FP32 vector atomics.
//
// The emitters 2I and 2I + 1 of the first item of a receiver pair are applied in direction 1 only
// (all four ordered pairs of the block, self pairs included); emitters j < 2I belong to the CTAs of
// j's receiver pair. D1 is added to y_i1, y_i2 with vector atomics at the end of the item; the FP32
// epilogue kernel forms W x or x - T W x in FP64.
//
// Every wait is bounded. The four drain warps take every decision to continue or stop together
// (barrier reductions over the 128 threads), so none waits at their named barrier for a warp that
// has left. After a timeout the kernel records an error, waits (bounded) for its own MMAs and bulk
// copies, frees its tensor memory and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "sg_internal.h"
#include "sg_tcgen05.h"

namespace sg {

static constexpr int kTsRoles = 6;       // 4 drain warps, 1 MMA warp, 1 copy warp
static constexpr int kTsProducers = 16;  // four 8 x 4 tiles each (64 per emitter; 24 warps measured slower)
static constexpr int kTsThreads = 32 * (kTsRoles + kTsProducers);
static constexpr int kTsChunk = 256;     // emitters per work item
static constexpr int kTsBP = 32;         // padded blocksize

struct TsArgs {
  const int4 *pairs;   // [N][N] (interval, t, cos phi, sin phi)
  const float2 *coef;  // FP32 coefficients [interval][c][n2][n1]
  const int *mofn;     // [bs]
  const float *xop;    // per particle [hi | lo] panels of [Re x | Im x] (2R rows x 32)
  const float *xops;   // the same with row n2 multiplied by (-1)^{m(n2)}
  const int4 *items;   // (I, first emitter, end emitter, 0)
  float2 *yacc;        // W x in FP32, [N][bs][R], zero on entry
  int n, bs, dmax, win;
  int *err;
};

template <int R>
struct TsShape {
  static constexpr int BP = kTsBP, KC = BP / 4, KSTEPS = BP / 8;
  static constexpr int NN = 2 * R;   // direction 1 MMA N
  static constexpr int N2 = 2 * NN;  // direction 2 MMA N (both receivers' signed panels)
  static constexpr int ATILE = 128 * BP, XTILE = NN * BP, SXTILE = N2 * BP;
  static constexpr int STAGE = 2 * (ATILE + XTILE);
  static constexpr int EROW = NN + 1;            // staging row stride (floats)
  static constexpr int ETILE = 64 * EROW;        // one 64-row staging block
  static constexpr int FIXED = 2 * SXTILE + 2 * ETILE;
  static constexpr int MISC = 1024;
  static constexpr int S0 = (kTcSmemBudget - MISC - FIXED * 4) / (STAGE * 4);
  static constexpr int S = S0 > 4 ? 4 : S0;
  static constexpr int TPR = (BP / 8) * (BP / 4), TILES = 2 * TPR;
  static constexpr int UNR = (TILES + kTsProducers - 1) / kTsProducers;
  static constexpr int G = 16;                   // lanes per receiver in the phase exchange
  static constexpr int COLS = 3 * NN + 2 * N2;   // D1 (two accumulators, total), D2 (two buffers)
  static constexpr int NCOLS = COLS <= 128 ? 128 : (COLS <= 256 ? 256 : 512);
  static constexpr size_t smem() { return (size_t)(S * STAGE + FIXED) * 4 + MISC; }
  static_assert(S >= 2, "two stages must fit");
  static_assert(UNR <= 4, "tiles per producer");
  static_assert(COLS <= 512, "tensor-memory columns");
  static_assert(N2 <= 256 && N2 % 16 == 0, "MMA N");
  static_assert(128 * (NN + 1) <= S * STAGE, "epilogue staging fits in the stages");
  static_assert(8 * (3 * S + 11) + 8 + 4 * BP <= MISC, "barrier area");
  static_assert(ETILE % 2 == 0, "8-byte alignment of the barriers");
};

// all threads of named barrier `id` (n threads) get the AND of their predicates
__device__ __forceinline__ bool ts_bar_and(int id, int n, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.and.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void ts_bar(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

template <int NC, int R>
__global__ void __launch_bounds__(kTsThreads, 1) tcsym_kernel(const TsArgs a) {
  using Sh = TsShape<R>;
  constexpr int NN = Sh::NN, N2 = Sh::N2, KC = Sh::KC, S = Sh::S, BP = Sh::BP;
  extern __shared__ __align__(1024) unsigned char ts_smem[];
  float *stages = reinterpret_cast<float *>(ts_smem);
  float *sx = stages + (size_t)S * Sh::STAGE;  // [hi | lo] of [S x_i1 ; S x_i2] (N2 rows x BP)
  float *Ea = sx + 2 * Sh::SXTILE;             // D2 rows 0-63, columns 0..NN-1
  float *Eb = Ea + Sh::ETILE;                  // D2 rows 64-127, columns NN..2NN-1
  uint64_t *bars = reinterpret_cast<uint64_t *>(Eb + Sh::ETILE);
  uint64_t *full_a = bars, *full_x = bars + S, *empty = bars + 2 * S;
  uint64_t *acc_full = bars + 3 * S, *acc_empty = acc_full + 2, *acc2_full = acc_full + 4, *acc2_empty = acc_full + 6;
  uint64_t *sx_full = acc_full + 8, *fin = acc_full + 9;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_full + 10);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  int *mofn_s = reinterpret_cast<int *>(tmem_slot + 2);  // [BP]

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int bs = a.bs, N = a.n, bs2 = bs * bs;
  const int4 item = a.items[blockIdx.x];
  const int i0 = 2 * item.x, jb = item.y, je = item.z;
  const int nsteps = je - jb;
  const int d0 = max(jb, i0 + 2);  // first emitter applied in both directions
  const int nwin = (nsteps + a.win - 1) / a.win;

  for (int e = tid; e < (S * Sh::STAGE + 2 * Sh::SXTILE) / 4; e += kTsThreads)
    reinterpret_cast<float4 *>(stages)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int e = tid; e < BP; e += kTsThreads) mofn_s[e] = e < bs ? a.mofn[e] : 0;
  if (tid == 0) {
    *abort_flag = 0;
    for (int s = 0; s < S; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_a[s])), "r"(kTsProducers) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_x[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])) : "memory");
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(smem_u32(&acc_empty[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc2_full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(smem_u32(&acc2_empty[b])) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(sx_full)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(fin)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(Sh::NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp >= kTsRoles) {
    // ------------------------------------------------------------------ producers (as in sg_tc.cu)
    const int p = warp - kTsRoles;
    const int grp = lane / Sh::G;
    const int gi = i0 + grp;
    const bool gvalid = gi < N;
    int coff[Sh::UNR], sinfo[Sh::UNR];
#pragma unroll
    for (int u = 0; u < Sh::UNR; ++u) {
      const int tile = p + kTsProducers * u;
      const int r = (tile / Sh::TPR) & 1, tr = tile % Sh::TPR;
      const int n1 = (tr / (BP / 4)) * 8 + (lane & 7), n2 = (tr % (BP / 4)) * 4 + (lane >> 3);
      const bool valid = tile < Sh::TILES && i0 + r < N && n1 < bs && n2 < bs;
      const int dm = valid ? mofn_s[n2] - mofn_s[n1] : 0;
      coff[u] = valid ? n2 * bs + n1 : -1;
      sinfo[u] = tc_off<KC>(r * 2 * BP + n1, n2) | ((r * Sh::G + (dm < 0 ? -dm : dm)) << 16) | ((dm < 0 ? 1 : 0) << 21) |
                 ((r * Sh::G) << 22);
    }
    const size_t plane = (size_t)bs2, block = (size_t)NC * bs2;
    int4 pd_next = gvalid ? __ldg(&a.pairs[(size_t)gi * N + jb]) : make_int4(0, 0, 0x3f800000, 0);
    for (int st = 0; st < nsteps; ++st) {
      if (__shfl_sync(kTcFull, *abort_flag, 0)) break;
      const int j = jb + st;
      const int s = st % S, q = st / S;
      const int4 pd = pd_next;
      if (st + 1 < nsteps && gvalid) pd_next = __ldg(&a.pairs[(size_t)gi * N + j + 1]);
      float pr = 1.f, pim = 0.f;
      {
        const int d = min(lane % Sh::G, a.dmax);
        const float c = __int_as_float(pd.z), sn = __int_as_float(pd.w);
        for (int it = 0; it < d; ++it) {
          const float nr = pr * c - pim * sn;
          pim = pr * sn + pim * c;
          pr = nr;
        }
      }
      float *Ah = stages + (size_t)s * Sh::STAGE;
      float2 cf[Sh::UNR][NC];
      float tt[Sh::UNR];
#pragma unroll
      for (int u = 0; u < Sh::UNR; ++u) {
        const int ks = (sinfo[u] >> 22) & 31;
        const int k = __shfl_sync(kTcFull, pd.x, ks);
        tt[u] = __shfl_sync(kTcFull, __int_as_float(pd.y), ks);
        const int off = coff[u];
        const float2 *cp = a.coef + ((size_t)k * block + (off < 0 ? 0 : off));
#pragma unroll
        for (int ci = 0; ci < NC; ++ci) cf[u][ci] = off >= 0 ? __ldg(cp + ci * plane) : make_float2(0.f, 0.f);
      }
      if (q > 0 && !tc_waitw(smem_u32(&empty[s]), (uint32_t)((q - 1) & 1))) {
        if (lane == 0) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
        }
        break;
      }
#pragma unroll
      for (int u = 0; u < Sh::UNR; ++u) {
        if (p + kTsProducers * u >= Sh::TILES) continue;  // warp-uniform: this warp has no such tile
        const int si = sinfo[u];
        const int src = (si >> 16) & 31;
        const float er = __shfl_sync(kTcFull, pr, src);
        float ei = __shfl_sync(kTcFull, pim, src);
        if (si & (1 << 21)) ei = -ei;
        if (coff[u] < 0) continue;  // padding stays zero
        float lr = cf[u][NC - 1].x, li = cf[u][NC - 1].y;
#pragma unroll
        for (int ci = NC - 2; ci >= 0; --ci) {
          lr = fmaf(lr, tt[u], cf[u][ci].x);
          li = fmaf(li, tt[u], cf[u][ci].y);
        }
        const float wr = lr * er - li * ei, wi = lr * ei + li * er;
        const float wrh = tf32_hi(wr), wih = tf32_hi(wi);
        float *dst = Ah + (si & 0xFFFF);
        dst[0] = wrh;
        dst[Sh::ATILE] = wr - wrh;
        dst[BP * BP] = wih;
        dst[Sh::ATILE + BP * BP] = wi - wih;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) tc_arrive(smem_u32(&full_a[s]));
    }
  } else if (warp == 5) {
    // ------------------------------------------------------------------ copies
    if (lane == 0) {
      constexpr uint32_t pbytes = (uint32_t)Sh::XTILE * 4u;  // one hi or lo panel
      bool sx_armed = false;
      if (je > d0) {
        // [S x_i1 ; S x_i2] hi and lo, once per item (a missing second receiver stays zero)
        const int nrec = i0 + 1 < N ? 2 : 1;
        const uint32_t bar = smem_u32(sx_full);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(2u * nrec * pbytes)
                     : "memory");
        for (int r = 0; r < nrec; ++r)
          for (int h = 0; h < 2; ++h) {
            const float *src = a.xops + ((size_t)(i0 + r) * 2 + h) * Sh::XTILE;
            const uint32_t dst = smem_u32(sx + (size_t)h * Sh::SXTILE + (size_t)r * Sh::XTILE);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                "l"(src), "r"(pbytes), "r"(bar)
                : "memory");
          }
        sx_armed = true;
      }
      int armed = 0;
      for (int st = 0; st < nsteps; ++st) {
        if (*abort_flag) break;
        const int s = st % S, q = st / S;
        if (q > 0 && !tc_wait1(smem_u32(&empty[s]), (uint32_t)((q - 1) & 1))) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
          break;
        }
        const uint32_t bar = smem_u32(&full_x[s]);
        const uint32_t dst = smem_u32(stages + (size_t)s * Sh::STAGE + 2 * Sh::ATILE);
        const float *src = a.xop + (size_t)(jb + st) * 2 * Sh::XTILE;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(2u * pbytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
            "l"(src), "r"(2u * pbytes), "r"(bar)
            : "memory");
        armed = st + 1;
      }
      for (int s = 0; s < S; ++s) {
        const int uses = armed > s ? (armed - s + S - 1) / S : 0;
        if (uses > 0 && !tc_wait1(smem_u32(&full_x[s]), (uint32_t)((uses - 1) & 1))) atomicExch(a.err, 1);
      }
      if (sx_armed && !tc_wait1(smem_u32(sx_full), 0u)) atomicExch(a.err, 1);
    }
  } else if (warp == 4) {
    // ------------------------------------------------------------------ MMA issue
    if (lane == 0) {
      const uint32_t idesc1 =
          (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
      const uint32_t idesc2 =
          (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N2 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
      const uint32_t sx_hi = smem_u32(sx), sx_lo = sx_hi + Sh::SXTILE * 4;
      bool issued = false;
      for (int st = 0; st < nsteps; ++st) {
        if (*abort_flag) break;
        const int j = jb + st;
        const int s = st % S, q = st / S;
        const int w = st / a.win, b = w & 1;
        const bool first = (st % a.win) == 0;
        const bool two = j >= d0;
        const int q2 = j - d0, b2 = q2 & 1;
        bool ok = tc_wait1(smem_u32(&full_x[s]), (uint32_t)(q & 1)) &&
                  tc_wait1(smem_u32(&full_a[s]), (uint32_t)(q & 1));
        if (ok && first && w >= 2) ok = tc_wait1(smem_u32(&acc_empty[b]), (uint32_t)(((w >> 1) - 1) & 1));
        if (ok && two && q2 == 0) ok = tc_wait1(smem_u32(sx_full), 0u);
        if (ok && two && q2 >= 2) ok = tc_wait1(smem_u32(&acc2_empty[b2]), (uint32_t)(((q2 >> 1) - 1) & 1));
        if (!ok) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a_hi = smem_u32(stages + (size_t)s * Sh::STAGE), a_lo = a_hi + Sh::ATILE * 4;
        const uint32_t x_hi = a_hi + 2 * Sh::ATILE * 4, x_lo = x_hi + Sh::XTILE * 4;
        const uint32_t d1 = tmem + (uint32_t)(b * NN);
        const uint32_t d2 = tmem + (uint32_t)(3 * NN + b2 * N2);
#pragma unroll
        for (int ks = 0; ks < Sh::KSTEPS; ++ks) {
          const uint32_t koff = ks * 256;
#pragma unroll
          for (int prod = 0; prod < 3; ++prod) {
            const uint32_t aa = (prod == 2 ? a_lo : a_hi) + koff;
            const uint32_t bb = (prod == 1 ? x_lo : x_hi) + koff;
            const uint32_t acc = (first && ks == 0 && prod == 0) ? 0u : 1u;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d1),
                "l"(tc_desc<KC>(aa)), "l"(tc_desc<KC>(bb)), "r"(idesc1), "r"(acc)
                : "memory");
          }
        }
        if (two) {
#pragma unroll
          for (int ks = 0; ks < Sh::KSTEPS; ++ks) {
            const uint32_t koff = ks * 256;
#pragma unroll
            for (int prod = 0; prod < 3; ++prod) {
              const uint32_t aa = (prod == 2 ? a_lo : a_hi) + koff;
              const uint32_t bb = (prod == 1 ? sx_lo : sx_hi) + koff;
              const uint32_t acc = (ks == 0 && prod == 0) ? 0u : 1u;
              asm volatile(
                  "{\n\t.reg .pred p;\n\t"
                  "setp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d2),
                  "l"(tc_desc<KC>(aa)), "l"(tc_desc<KC>(bb)), "r"(idesc2), "r"(acc)
                  : "memory");
            }
          }
        }
        issued = true;
        tc_commit(smem_u32(&empty[s]));
        if (two) tc_commit(smem_u32(&acc2_full[b2]));
        if ((st % a.win) == a.win - 1 || st == nsteps - 1) tc_commit(smem_u32(&acc_full[b]));
      }
      if (issued) {
        tc_commit(smem_u32(fin));
        if (!tc_wait1(smem_u32(fin), 0u)) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
        }
      }
    }
  } else {
    // ------------------------------------------------------------------ drain warps 0-3
    // every continue/stop decision is taken by all 128 threads together (barrier reductions), so
    // no warp waits at named barrier 1 for one that has left
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const int row = warp * 32 + lane;
    for (int st = 0; st < nsteps; ++st) {
      const int j = jb + st;
      if (!ts_bar_and(1, 128, *abort_flag == 0)) break;
      if (j >= d0) {
        // direction 2 of this emitter: y_j += S (W_i1j S x_i1 + W_i2j S x_i2)
        const int q2 = j - d0, b2 = q2 & 1;
        bool ok = tc_waitw(smem_u32(&acc2_full[b2]), (uint32_t)((q2 >> 1) & 1));
        if (!ok && lane == 0) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
        }
        if (!ts_bar_and(1, 128, ok)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // rows 0-63 read columns 0..NN-1 (receiver 1's panel), rows 64-127 columns NN..2NN-1
        const uint32_t base = lane_base + (uint32_t)(3 * NN + b2 * N2 + (warp < 2 ? 0 : NN));
        float *E = (warp < 2 ? Ea : Eb) + (size_t)(row & 63) * Sh::EROW;
#pragma unroll 1
        for (int c0 = 0; c0 < NN; c0 += 16) {
          float v[16];
          tmem_ld16(base + (uint32_t)c0, v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int e = 0; e < 16; ++e) E[c0 + e] = v[e];
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) tc_arrive(smem_u32(&acc2_empty[b2]));
        ts_bar(1, 128);
        // (n1, pair of RHS) per thread: Re y = Wr xr - Wi xi, Im y = Wr xi + Wi xr, times s(n1)
        float2 *yj = a.yacc + (size_t)j * bs * R;
        for (int e = tid; e < bs * (R / 2); e += 128) {
          const int n1 = e / (R / 2), rr = 2 * (e - n1 * (R / 2));
          const float *ar = Ea + (size_t)n1 * Sh::EROW, *ai = Ea + (size_t)(BP + n1) * Sh::EROW;
          const float *br = Eb + (size_t)n1 * Sh::EROW, *bi = Eb + (size_t)(BP + n1) * Sh::EROW;
          const float sg = (mofn_s[n1] & 1) ? -1.f : 1.f;
          float4 v;
          v.x = sg * ((ar[rr] + br[rr]) - (ai[R + rr] + bi[R + rr]));
          v.y = sg * ((ar[R + rr] + br[R + rr]) + (ai[rr] + bi[rr]));
          v.z = sg * ((ar[rr + 1] + br[rr + 1]) - (ai[R + rr + 1] + bi[R + rr + 1]));
          v.w = sg * ((ar[R + rr + 1] + br[R + rr + 1]) + (ai[rr + 1] + bi[rr + 1]));
          atomicAdd(reinterpret_cast<float4 *>(yj + (size_t)n1 * R + rr), v);
        }
        ts_bar(1, 128);  // Ea / Eb are rewritten by the next emitter
      }
      if ((st % a.win) == a.win - 1 || st == nsteps - 1) {
        const int w = st / a.win, b = w & 1;
        bool ok = tc_waitw(smem_u32(&acc_full[b]), (uint32_t)((w >> 1) & 1));
        if (!ok && lane == 0) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
        }
        if (!ts_bar_and(1, 128, ok)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
        for (int c0 = 0; c0 < NN; c0 += 16) {
          float v[16], t[16];
          tmem_ld16(lane_base + (uint32_t)(b * NN + c0), v);
          if (w > 0) {
            tmem_ld16(lane_base + (uint32_t)(2 * NN + c0), t);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int e = 0; e < 16; ++e) t[e] += v[e];
          } else {
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int e = 0; e < 16; ++e) t[e] = v[e];
          }
          tmem_st16(lane_base + (uint32_t)(2 * NN + c0), t);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) tc_arrive(smem_u32(&acc_empty[b]));
      }
    }
    (void)nwin;
  }

  // ------------------------------------------------------------------ direction 1 -> y_i1, y_i2
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool good = !*abort_flag;
  float *Ds = stages;  // [128][NN + 1]
  if (good && warp < 4) {
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const int row = warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < NN; c0 += 16) {
      float v[16];
      tmem_ld16(lane_base + (uint32_t)(2 * NN + c0), v);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int e = 0; e < 16; ++e) Ds[row * (NN + 1) + c0 + e] = v[e];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Sh::NCOLS) : "memory");
  }
  if (!good) return;
  const int nrecv = min(2, N - i0);
  for (int e = tid; e < nrecv * bs * (R / 2); e += kTsThreads) {
    const int r = e / (bs * (R / 2)), rem = e - r * bs * (R / 2), n1 = rem / (R / 2), c = 2 * (rem - n1 * (R / 2));
    const float *d0r = Ds + (size_t)(r * 2 * BP + n1) * (NN + 1);
    const float *d1r = Ds + (size_t)(r * 2 * BP + BP + n1) * (NN + 1);
    const float4 v = make_float4(d0r[c] - d1r[R + c], d0r[R + c] + d1r[c], d0r[c + 1] - d1r[R + c + 1],
                                 d0r[R + c + 1] + d1r[c + 1]);
    atomicAdd(reinterpret_cast<float4 *>(a.yacc + ((size_t)(i0 + r) * bs + n1) * R + c), v);
  }
}

// Pre-split panels of x and of S x: xop[j][h][tc_off(c, n2)] = hi/lo of (c < R ? Re : Im) x[j][n2][c mod R],
// xops the same with (-1)^{m(n2)} x
__global__ void tcsym_split_x_kernel(const double2 *x, const int *mofn, float *xop, float *xops, int n, int bs, int R) {
  const int NN = 2 * R;
  const size_t tile = (size_t)NN * kTsBP;
  const size_t total = (size_t)n * tile;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / tile);
    const int rem = (int)(e - (size_t)j * tile);
    const int c = rem / kTsBP, n2 = rem - c * kTsBP;
    float v = 0.f;
    int sgn = 0;
    if (n2 < bs) {
      const double2 xv = x[((size_t)j * bs + n2) * R + (c < R ? c : c - R)];
      v = (float)(c < R ? xv.x : xv.y);
      sgn = mofn[n2] & 1;
    }
    const float hi = tf32_hi(v), lo = v - hi;
    const size_t o = (size_t)j * 2 * tile + tc_off<kTsBP / 4>(c, n2);
    xop[o] = hi;
    xop[o + tile] = lo;
    xops[o] = sgn ? -hi : hi;
    xops[o + tile] = sgn ? -lo : lo;
  }
}

bool tcsym_supported(const sg_context *c, int R) {
  if (c->vol || c->bs < 2 || c->bs > kTsBP || !(R == 16 || R == 32) || !c->pairs_ready || c->n < 2) return false;
  int mmax = 0;
  for (int m : c->h_mofn) mmax = std::max(mmax, m < 0 ? -m : m);
  return 2 * mmax < 16;  // phase powers are exchanged within 16 lanes
}

// work items: receiver pair I, emitters [jb, je) with jb >= 2I, runs of kTsChunk, longest first
static void build_tcsym_items(sg_context *c) {
  std::vector<int4> items;
  const int n = c->n, npair = (n + 1) / 2;
  for (int I = 0; I < npair; ++I)
    for (int jb = 2 * I; jb < n; jb += kTsChunk) items.push_back(make_int4(I, jb, std::min(n, jb + kTsChunk), 0));
  std::stable_sort(items.begin(), items.end(), [](const int4 &a, const int4 &b) { return a.z - a.y > b.z - b.y; });
  c->tcs_items.reserve(items.size());
  SG_CUDA(cudaMemcpy(c->tcs_items.ptr, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
  c->tcs_n_items = (int)items.size();
  c->tcs_items_n = n;
}

template <int NC, int R>
static void tcsym_launch_t(sg_context *c, const TsArgs &a, cudaStream_t st) {
  using Sh = TsShape<R>;
  static bool attr_done[64] = {};
  if (first_on_device(attr_done))
    SG_CUDA(cudaFuncSetAttribute(tcsym_kernel<NC, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Sh::smem()));
  tcsym_kernel<NC, R><<<c->tcs_n_items, kTsThreads, Sh::smem(), st>>>(a);
  SG_CUDA(cudaGetLastError());
}

// y = M x or W x with the pair-symmetric tensor-core operator; returns the number of kernels launched
int launch_tcsym_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  SG_REQUIRE(tcsym_supported(c, R),
             "pair-symmetric tensor-core operator: needs the radial lookup, blocksize <= 32 and nrhs in {16, 32}");
  SG_REQUIRE(c->tc_win >= 1, "tensor-core operator: the drain window must be positive");
  if (c->tcs_items_n != c->n || c->tcs_n_items == 0) build_tcsym_items(c);
  const size_t plen = (size_t)c->n * 2 * (2 * R) * kTsBP;
  c->tc_xop.reserve(plen);
  c->tc_xops.reserve(plen);
  c->tc_err.reserve(1);
  if (!c->tc_err_init) {
    SG_CUDA(cudaMemsetAsync(c->tc_err.ptr, 0, sizeof(int), st));
    c->tc_err_init = true;
  }
  const size_t total = (size_t)c->n * (2 * R) * kTsBP;
  const unsigned sgrid = (unsigned)std::min<size_t>((total + 255) / 256, (size_t)sm_count() * 16);
  tcsym_split_x_kernel<<<sgrid, 256, 0, st>>>(x, c->mofn.ptr, c->tc_xop.ptr, c->tc_xops.ptr, c->n, c->bs, R);
  SG_CUDA(cudaGetLastError());
  const size_t len = (size_t)c->n * c->bs * R;
  c->sym_yacc.reserve(len);
  SG_CUDA(cudaMemsetAsync(c->sym_yacc.ptr, 0, len * sizeof(float2), st));
  TsArgs a{};
  a.pairs = c->pairs.ptr;
  a.coef = c->coef32.ptr;
  a.mofn = c->mofn.ptr;
  a.xop = c->tc_xop.ptr;
  a.xops = c->tc_xops.ptr;
  a.items = c->tcs_items.ptr;
  a.yacc = c->sym_yacc.ptr;
  a.n = c->n;
  a.bs = c->bs;
  int mmax = 0;
  for (int m : c->h_mofn) mmax = std::max(mmax, m < 0 ? -m : m);
  a.dmax = 2 * mmax;
  a.win = c->tc_win;
  a.err = c->tc_err.ptr;
  if (c->ncoef == 2) {
    if (R == 16) tcsym_launch_t<2, 16>(c, a, st);
    else tcsym_launch_t<2, 32>(c, a, st);
  } else {
    if (R == 16) tcsym_launch_t<4, 16>(c, a, st);
    else tcsym_launch_t<4, 32>(c, a, st);
  }
  launch_fp32_epilogue(c, x, y, R, master, st);
  return 3;  // split, coupling, epilogue (the memset is not a kernel of this library)
}

}  // namespace sg

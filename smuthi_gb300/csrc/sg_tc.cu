// Tensor-core (tcgen05, 3xTF32) form of the FP32 coupling operator for batched right-hand sides.
//
// Per ordered pair (i, j) the coupling block W_ij = e^{-i m1 phi} L(rho_ij) e^{i m2 phi} (B x B
// complex, B <= 48, padded to BP in {16, 32, 48}) is contracted with the RHS panel x_j (B x R
// complex, R in {16, 32, 64}) as one real product
//
//   [Re W; Im W] (2 BP rows, K = BP) x [Re x_j | Im x_j] (K = BP, N = 2R columns)
//     = [[Wr xr, Wr xi], [Wi xr, Wi xi]],   Re y_i = Wr xr - Wi xi,  Im y_i = Wr xi + Wi xr,
//
// on the MMA datapath's 128 rows: a CTA owns 128 / (2 BP) receiving particles (four at BP = 16, two
// at BP = 32, one at BP = 48 with rows 96-127 zero) and streams every emitter j in index order, so
// that all CTAs read the same x_j panels at about the same time (one DRAM read per panel per wave
// of CTAs). The CTA is warp-specialised and pipelined over S shared-memory stages:
//
//   * 16 or 24 producer warps (two to four 8 x 4 tiles each) interpolate the interval's coefficients (FP32 Horner), fold in the phase
//     e^{i (m2 - m1) phi} (powers computed per emitter by one lane each and exchanged by shuffles),
//     split every value into a TF32 high part and an FP32 remainder and store the block into the
//     stage in the canonical no-swizzle K-major layout (one 8 x 4 core tile per warp instruction,
//     128 contiguous bytes, no bank conflicts); the coefficient loads of all tiles of a thread are
//     in flight together;
//   * one thread copies x_j's pre-split panel (hi | lo, contiguous) into the stage with one
//     cp.async.bulk completing on the stage's mbarrier;
//   * one thread issues the tcgen05.mma instructions (kind::tf32, M = 128, N = 2R, K = 8; hi*hi +
//     hi*lo + lo*hi per K step) and frees the stage with tcgen05.commit;
//   * four drain warps fold the accumulator into a running total held in tensor memory every `win`
//     emitters. The tensor core's accumulation into tensor memory is not round-to-nearest FP32: its
//     error grows with the number of MMAs accumulated into one accumulator, so every accumulator
//     takes only `win` emitters (two accumulators alternate, so the MMAs do not wait for a drain)
//     and the total is summed with round-to-nearest FP32 additions on the CUDA cores.
//
// Every mbarrier wait is bounded by a clock budget: on expiry the kernel records an error, stops
// every role, waits (bounded) for its own MMAs and bulk copies, frees its tensor memory and returns
// without writing output. The result is W x in FP32 ([n][bs][R] complex); the FP32 epilogue kernel
// turns it into FP64 W x or x - T (W x) for diagonal or dense T blocks.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sg_internal.h"
#include "sg_tcgen05.h"

namespace sg {

static constexpr int kTcRoles = 6;                        // 4 drain warps, 1 MMA warp, 1 copy warp
struct TcArgs {
  const int4 *pairs;   // [N][N] (interval, t, cos phi, sin phi)
  const float2 *coef;  // FP32 coefficients [interval][c][n2][n1]
  const int *mofn;     // [bs]
  const float *xop;    // pre-split panels: per particle [hi | lo] tiles of 2R x BP floats
  float2 *yacc;        // W x in FP32, [N][bs][R]
  int n, bs, dmax, win;
  int *err;  // set to 1 when a wait runs out
};

template <int BP, int R>
struct TcShape {
  static constexpr int NN = 2 * R;                                 // MMA N
  static constexpr int RPC = (2 * BP <= 64) ? 128 / (2 * BP) : 1;  // receivers per CTA
  static constexpr int KC = BP / 4;
  static constexpr int KSTEPS = BP / 8;
  static constexpr int ATILE = 128 * BP;             // floats per A tile (hi or lo)
  static constexpr int XTILE = NN * BP;              // floats per x tile (hi or lo)
  static constexpr int STAGE = 2 * (ATILE + XTILE);  // floats per stage
  static constexpr int MISC = 1024;                  // barriers, tensor-memory slot, flag, m(n)
  static constexpr int S0 = (kTcSmemBudget - MISC) / (STAGE * 4);
  static constexpr int S = S0 > 4 ? 4 : S0;            // pipeline stages
  static constexpr int TPR = (BP / 8) * (BP / 4);      // 8 x 4 core tiles per receiver
  static constexpr int TILES = RPC * TPR;
  // producer warps: three 8 x 4 tiles each at BP = 48 (30 warps), four at BP = 32, two at BP = 16;
  // more warps hide more of the coefficient stream's latency (960 threads is the largest multiple)
  static constexpr int NPROD = TILES % 24 == 0 ? 24 : 16;
  static constexpr int THREADS = 32 * (kTcRoles + NPROD);
  static constexpr int UNR = (TILES + NPROD - 1) / NPROD;
  static constexpr int GRP = UNR < 4 ? UNR : 4;  // tiles whose loads are in flight together
  static constexpr int G = 32 / RPC;             // lanes per receiver in the phase exchange
  static constexpr int COLS = 3 * NN;            // two accumulators and the total
  static constexpr int NCOLS = COLS <= 32 ? 32 : (COLS <= 64 ? 64 : (COLS <= 128 ? 128 : (COLS <= 256 ? 256 : 512)));
  static constexpr size_t smem() { return (size_t)S * STAGE * 4 + MISC; }
  static_assert(S >= 2, "two stages must fit");
  static_assert(NN % 16 == 0 && NN >= 16 && NN <= 256, "MMA N");
  static_assert(128 * (NN + 1) <= S * STAGE, "epilogue staging fits in the stages");
  static_assert(8 * (3 * S + 5) + 8 + 4 * BP <= MISC, "barrier area");
};

template <int NC, int BP, int R>
__global__ void __launch_bounds__(TcShape<BP, R>::THREADS, 1) tc_coupling_kernel(const TcArgs a) {
  using Sh = TcShape<BP, R>;
  constexpr int kTcThreads = Sh::THREADS, kTcProducers = Sh::NPROD;
  constexpr int NN = Sh::NN, RPC = Sh::RPC, KC = Sh::KC, S = Sh::S;
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  float *stages = reinterpret_cast<float *>(tc_smem);
  uint64_t *bars = reinterpret_cast<uint64_t *>(tc_smem + (size_t)S * Sh::STAGE * 4);
  uint64_t *full_a = bars, *full_x = bars + S, *empty = bars + 2 * S;
  uint64_t *acc_full = bars + 3 * S, *acc_empty = acc_full + 2, *fin = acc_full + 4;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(fin + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  int *mofn_s = reinterpret_cast<int *>(tmem_slot + 2);  // [BP]

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int bs = a.bs, N = a.n, bs2 = bs * bs;
  const int i0 = RPC * blockIdx.x;
  const int nwin = (N + a.win - 1) / a.win;

  // zero every stage (padding rows and columns stay zero), copy m(n), set up barriers
  for (int e = tid; e < S * Sh::STAGE / 4; e += kTcThreads)
    reinterpret_cast<float4 *>(stages)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int e = tid; e < BP; e += kTcThreads) mofn_s[e] = e < bs ? a.mofn[e] : 0;
  if (tid == 0) {
    *abort_flag = 0;
    for (int s = 0; s < S; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_a[s])), "r"(kTcProducers)
                   : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_x[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])) : "memory");
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(smem_u32(&acc_empty[b])) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(fin)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(Sh::NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the zeroed stages, for the tensor core
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp >= kTcRoles) {
    // ------------------------------------------------------------------ producers
    const int p = warp - kTcRoles;
    const int grp = lane / Sh::G;  // receiver whose pair data and phase powers this lane holds
    const int gi = i0 + grp;
    const bool gvalid = grp < RPC && gi < N;
    // Per-thread invariants of every tile this warp builds (the same for all emitters):
    // coff = element offset n2 * bs + n1 within a coefficient plane (-1: padding or no receiver);
    // sinfo = store offset tc_off(row, n2) (bits 0-15) | phase source lane r * G + |dm| (bits 16-20)
    //         | conjugate flag dm < 0 (bit 21) | pair-data source lane r * G (bits 22-26).
    int coff[Sh::UNR], sinfo[Sh::UNR];
#pragma unroll
    for (int u = 0; u < Sh::UNR; ++u) {
      const int tile = p + kTcProducers * u;
      const int r = (tile / Sh::TPR) % RPC, tr = tile % Sh::TPR;
      const int n1 = (tr / (BP / 4)) * 8 + (lane & 7), n2 = (tr % (BP / 4)) * 4 + (lane >> 3);
      const bool valid = tile < Sh::TILES && i0 + r < N && n1 < bs && n2 < bs;
      const int dm = valid ? mofn_s[n2] - mofn_s[n1] : 0;
      coff[u] = valid ? n2 * bs + n1 : -1;
      sinfo[u] = tc_off<KC>(r * 2 * BP + n1, n2) | ((r * Sh::G + (dm < 0 ? -dm : dm)) << 16) | ((dm < 0 ? 1 : 0) << 21) |
                 ((r * Sh::G) << 22);
    }
    const size_t plane = (size_t)bs2, block = (size_t)NC * bs2;
    int4 pd_next = gvalid ? __ldg(&a.pairs[(size_t)gi * N]) : make_int4(0, 0, 0x3f800000, 0);
    for (int jj = 0; jj < N; ++jj) {
      if (__shfl_sync(kTcFull, *abort_flag, 0)) break;  // one decision per warp
      const int s = jj % S, q = jj / S;
      const int4 pd = pd_next;
      if (jj + 1 < N && gvalid) pd_next = __ldg(&a.pairs[(size_t)gi * N + jj + 1]);
      // phase power e^{i d phi}, d = this lane's index within its receiver group (<= dmax)
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
      bool waited = (q == 0);
#pragma unroll
      for (int g0 = 0; g0 < Sh::UNR; g0 += Sh::GRP) {
        float2 cf[Sh::GRP][NC];
        float tt[Sh::GRP];
#pragma unroll
        for (int u = 0; u < Sh::GRP; ++u) {
          if (g0 + u >= Sh::UNR) continue;
          const int ks = (sinfo[g0 + u] >> 22) & 31;
          const int k = __shfl_sync(kTcFull, pd.x, ks);
          tt[u] = __shfl_sync(kTcFull, __int_as_float(pd.y), ks);
          const int off = coff[g0 + u];
          const float2 *cp = a.coef + ((size_t)k * block + (off < 0 ? 0 : off));
#pragma unroll
          for (int ci = 0; ci < NC; ++ci) cf[u][ci] = off >= 0 ? __ldg(cp + ci * plane) : make_float2(0.f, 0.f);
        }
        if (!waited) {
          if (!tc_waitw(smem_u32(&empty[s]), (uint32_t)((q - 1) & 1))) {
            if (lane == 0) {
              *abort_flag = 1;
              atomicExch(a.err, 1);
            }
            break;
          }
          waited = true;
        }
#pragma unroll
        for (int u = 0; u < Sh::GRP; ++u) {
          if (g0 + u >= Sh::UNR || p + kTcProducers * (g0 + u) >= Sh::TILES) continue;  // warp-uniform
          const int si = sinfo[g0 + u];
          const int src = (si >> 16) & 31;
          const float er = __shfl_sync(kTcFull, pr, src);
          float ei = __shfl_sync(kTcFull, pim, src);
          if (si & (1 << 21)) ei = -ei;
          if (coff[g0 + u] < 0) continue;  // padding stays zero
          float lr = cf[u][NC - 1].x, li = cf[u][NC - 1].y;
#pragma unroll
          for (int ci = NC - 2; ci >= 0; --ci) {
            lr = fmaf(lr, tt[u], cf[u][ci].x);
            li = fmaf(li, tt[u], cf[u][ci].y);
          }
          // the self pair (rho = 0) is not zero: it is the particle's coupling to itself through the layers
          const float wr = lr * er - li * ei, wi = lr * ei + li * er;
          const float wrh = tf32_hi(wr), wih = tf32_hi(wi);
          float *dst = Ah + (si & 0xFFFF);  // Re W in row n1, Im W in row BP + n1 (BP * BP floats further)
          dst[0] = wrh;
          dst[Sh::ATILE] = wr - wrh;
          dst[BP * BP] = wih;
          dst[Sh::ATILE + BP * BP] = wi - wih;
        }
      }
      if (!waited) break;  // the wait above ran out
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) tc_arrive(smem_u32(&full_a[s]));
    }
  } else if (warp == 5) {
    // ------------------------------------------------------------------ x panel copies
    if (lane == 0) {
      constexpr uint32_t bytes = 2u * Sh::XTILE * 4u;
      int armed = 0;
      for (int jj = 0; jj < N; ++jj) {
        if (*abort_flag) break;
        const int s = jj % S, q = jj / S;
        if (q > 0 && !tc_wait1(smem_u32(&empty[s]), (uint32_t)((q - 1) & 1))) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
          break;
        }
        const uint32_t bar = smem_u32(&full_x[s]);
        const uint32_t dst = smem_u32(stages + (size_t)s * Sh::STAGE + 2 * Sh::ATILE);
        const float *src = a.xop + (size_t)jj * 2 * Sh::XTILE;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
            "l"(src), "r"(bytes), "r"(bar)
            : "memory");
        armed = jj + 1;
      }
      // no copy of this CTA may still be in flight when it exits: wait (bounded) for the last
      // armed phase of every stage
      for (int s = 0; s < S; ++s) {
        const int uses = armed > s ? (armed - s + S - 1) / S : 0;
        if (uses > 0 && !tc_wait1(smem_u32(&full_x[s]), (uint32_t)((uses - 1) & 1))) atomicExch(a.err, 1);
      }
    }
  } else if (warp == 4) {
    // ------------------------------------------------------------------ MMA issue
    if (lane == 0) {
      const uint32_t idesc =
          (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
      bool issued = false;
      for (int jj = 0; jj < N; ++jj) {
        if (*abort_flag) break;
        const int s = jj % S, q = jj / S;
        const int w = jj / a.win, b = w & 1;
        const bool first = (jj % a.win) == 0;
        bool ok = tc_wait1(smem_u32(&full_x[s]), (uint32_t)(q & 1)) &&
                  tc_wait1(smem_u32(&full_a[s]), (uint32_t)(q & 1));
        if (ok && first && w >= 2) ok = tc_wait1(smem_u32(&acc_empty[b]), (uint32_t)(((w >> 1) - 1) & 1));
        if (!ok) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a_hi = smem_u32(stages + (size_t)s * Sh::STAGE), a_lo = a_hi + Sh::ATILE * 4;
        const uint32_t x_hi = a_hi + 2 * Sh::ATILE * 4, x_lo = x_hi + Sh::XTILE * 4;
        const uint32_t dcol = tmem + (uint32_t)(b * NN);
#pragma unroll
        for (int ks = 0; ks < Sh::KSTEPS; ++ks) {
          const uint32_t koff = ks * 256;  // two 128-byte core matrices per K step of 8
#pragma unroll
          for (int prod = 0; prod < 3; ++prod) {
            const uint32_t aa = (prod == 2 ? a_lo : a_hi) + koff;
            const uint32_t bb = (prod == 1 ? x_lo : x_hi) + koff;
            const uint32_t acc = (first && ks == 0 && prod == 0) ? 0u : 1u;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dcol),
                "l"(tc_desc<KC>(aa)), "l"(tc_desc<KC>(bb)), "r"(idesc), "r"(acc)
                : "memory");
          }
        }
        issued = true;
        tc_commit(smem_u32(&empty[s]));
        if ((jj % a.win) == a.win - 1 || jj == N - 1) tc_commit(smem_u32(&acc_full[b]));
      }
      // every MMA of this CTA has completed before the tensor memory is read for the last time or freed
      if (issued) {
        tc_commit(smem_u32(fin));
        if (!tc_wait1(smem_u32(fin), 0u)) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
        }
      }
    }
  } else {
    // ------------------------------------------------------------------ drain (warps 0-3)
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int w = 0; w < nwin; ++w) {
      if (__shfl_sync(kTcFull, *abort_flag, 0)) break;  // one decision per warp
      const int b = w & 1;
      if (!tc_waitw(smem_u32(&acc_full[b]), (uint32_t)((w >> 1) & 1))) {
        if (lane == 0) {
          *abort_flag = 1;
          atomicExch(a.err, 1);
        }
        break;
      }
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

  // ------------------------------------------------------------------ epilogue
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool good = !*abort_flag;
  float *Ds = stages;  // [128][NN + 1] FP32 totals (every stage is free now)
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
  const int nrecv = min(RPC, N - i0);
  for (int e = tid; e < nrecv * bs * R; e += kTcThreads) {
    const int r = e / (bs * R), rem = e - r * bs * R, n1 = rem / R, c = rem - n1 * R;
    const float *d0 = Ds + (size_t)(r * 2 * BP + n1) * (NN + 1);
    const float *d1 = Ds + (size_t)(r * 2 * BP + BP + n1) * (NN + 1);
    a.yacc[((size_t)(i0 + r) * bs + n1) * R + c] = make_float2(d0[c] - d1[R + c], d0[R + c] + d1[c]);
  }
}

// Pre-split panels: xop[j][h][tc_off(c, n2)] = hi/lo of (c < R ? Re : Im) x[j][n2][c mod R]
template <int BP>
__global__ void tc_split_x_kernel(const double2 *x, float *xop, int n, int bs, int R) {
  const int NN = 2 * R;
  const size_t tile = (size_t)NN * BP;
  const size_t total = (size_t)n * tile;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / tile);
    const int rem = (int)(e - (size_t)j * tile);
    const int c = rem / BP, n2 = rem - c * BP;
    float v = 0.f;
    if (n2 < bs) {
      const double2 xv = x[((size_t)j * bs + n2) * R + (c < R ? c : c - R)];
      v = (float)(c < R ? xv.x : xv.y);
    }
    const float hi = tf32_hi(v);
    float *base = xop + (size_t)j * 2 * tile;
    base[tc_off<BP / 4>(c, n2)] = hi;
    base[tile + tc_off<BP / 4>(c, n2)] = v - hi;
  }
}

static int tc_bp(int bs) { return bs <= 16 ? 16 : (bs <= 32 ? 32 : 48); }

bool tc_supported(const sg_context *c, int R) {
  if (c->vol || c->bs < 2 || c->bs > 48 || !(R == 16 || R == 32 || R == 64) || !c->pairs_ready || c->n < 1) return false;
  // the phase powers e^{i d phi}, d <= 2 max|m|, are exchanged within 32 / (receivers per CTA) lanes
  int mmax = 0;
  for (int m : c->h_mofn) mmax = std::max(mmax, m < 0 ? -m : m);
  const int bp = tc_bp(c->bs), rpc = 2 * bp <= 64 ? 128 / (2 * bp) : 1;
  return 2 * mmax < 32 / rpc;
}

template <int NC, int BP, int R>
static void tc_launch_t(const TcArgs &a, cudaStream_t st) {
  using Sh = TcShape<BP, R>;
  static bool attr_done[64] = {};
  if (first_on_device(attr_done))
    SG_CUDA(cudaFuncSetAttribute(tc_coupling_kernel<NC, BP, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)Sh::smem()));
  const unsigned grid = (unsigned)((a.n + Sh::RPC - 1) / Sh::RPC);
  tc_coupling_kernel<NC, BP, R><<<grid, Sh::THREADS, Sh::smem(), st>>>(a);
  SG_CUDA(cudaGetLastError());
}

template <int NC, int BP>
static void tc_launch_r(const TcArgs &a, int R, cudaStream_t st) {
  if (R == 16) tc_launch_t<NC, BP, 16>(a, st);
  else if (R == 32) tc_launch_t<NC, BP, 32>(a, st);
  else tc_launch_t<NC, BP, 64>(a, st);
}

// y = M x or W x with the tensor-core operator; returns the number of kernels launched
int launch_tc_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  SG_REQUIRE(tc_supported(c, R),
             "tensor-core operator: needs the radial lookup, blocksize <= 48 and nrhs in {16, 32, 64}");
  SG_REQUIRE(c->tc_win >= 1, "tensor-core operator: the drain window must be positive");
  const int BP = tc_bp(c->bs);
  const size_t xop_len = (size_t)c->n * 2 * (2 * R) * BP;
  c->tc_xop.reserve(xop_len);
  c->tc_err.reserve(1);
  if (!c->tc_err_init) {
    SG_CUDA(cudaMemsetAsync(c->tc_err.ptr, 0, sizeof(int), st));
    c->tc_err_init = true;
  }
  const size_t total = (size_t)c->n * (2 * R) * BP;
  const unsigned sgrid = (unsigned)std::min<size_t>((total + 255) / 256, (size_t)sm_count() * 16);
  if (BP == 16) tc_split_x_kernel<16><<<sgrid, 256, 0, st>>>(x, c->tc_xop.ptr, c->n, c->bs, R);
  else if (BP == 32) tc_split_x_kernel<32><<<sgrid, 256, 0, st>>>(x, c->tc_xop.ptr, c->n, c->bs, R);
  else tc_split_x_kernel<48><<<sgrid, 256, 0, st>>>(x, c->tc_xop.ptr, c->n, c->bs, R);
  SG_CUDA(cudaGetLastError());
  c->sym_yacc.reserve((size_t)c->n * c->bs * R);
  TcArgs a{};
  a.pairs = c->pairs.ptr;
  a.coef = c->coef32.ptr;
  a.mofn = c->mofn.ptr;
  a.xop = c->tc_xop.ptr;
  a.yacc = c->sym_yacc.ptr;
  a.n = c->n;
  a.bs = c->bs;
  int mmax = 0;
  for (int m : c->h_mofn) mmax = std::max(mmax, m < 0 ? -m : m);
  a.dmax = 2 * mmax;
  a.win = c->tc_win;
  a.err = c->tc_err.ptr;
  if (c->ncoef == 2) {
    if (BP == 16) tc_launch_r<2, 16>(a, R, st);
    else if (BP == 32) tc_launch_r<2, 32>(a, R, st);
    else tc_launch_r<2, 48>(a, R, st);
  } else {
    if (BP == 16) tc_launch_r<4, 16>(a, R, st);
    else if (BP == 32) tc_launch_r<4, 32>(a, R, st);
    else tc_launch_r<4, 48>(a, R, st);
  }
  launch_fp32_epilogue(c, x, y, R, master, st);
  return 3;  // split, coupling, epilogue
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

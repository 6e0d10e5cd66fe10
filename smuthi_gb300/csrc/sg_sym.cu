// Pair-symmetric FP32 coupling matvec (the mixed-precision operator for batched right-hand sides).
//
// For particles at one height the radial lookup gives, for an ordered pair (i, j) at distance rho
// and azimuth phi (of the vector from j to i),
//
//   W_ij[n1][n2] = L_{n1 n2}(rho) e^{i (m2 - m1) phi},
//
// and the reverse pair (j, i) has the same rho and phi + pi, so
//
//   W_ji[n1][n2] = s(n1) s(n2) W_ij[n1][n2],   s(n) = (-1)^{m(n)}.
//
// One interpolation of L at rho_ij therefore serves both directions: this kernel visits every
// unordered pair once, reads its interval's coefficient block once for all RHS of the tile and
// applies it to x_j (for y_i) and to s x_i (for y_j). The per-receiver kernel of sg_coupling.cu
// reads the block once per ordered pair and RHS tile, and waits on it through L2 latency.
//
// Coefficient stream: each warp streams its pairs' coefficient blocks through a private ring of
// kSymStages shared-memory stages with cp.async.bulk copies (one elected lane issues them, an
// mbarrier per stage counts the bytes). A stage holds CH columns n2 of one pair's block, all
// interpolation coefficients; the copies run up to kSymStages - 1 chunks ahead of the arithmetic,
// across pair boundaries, so the L2 latency is hidden by copies in flight rather than by resident
// warps or registers. Every mbarrier wait is bounded by a clock budget; on expiry the warp flags the
// error, stops computing, waits (bounded) for its copies in flight and leaves.
//
// Work decomposition: a CTA has 8 warps; SPLIT warps (1 or 2) serve one receiver, each with its own
// slice of the CTA's RHS tile, and share that receiver's coefficient ring (the copies are issued by
// the first warp of the slot once both have finished a stage), so particles are grouped in tiles of
// T = 8 / SPLIT. With SPLIT = 2 two CTAs fit on an SM (16 warps) and each coefficient chunk still
// serves all RHS of the tile. A work item is a receiver tile I and a run of up to kSymChunk emitter
// tiles J >= I. Slot w owns receiver i = T I + w and keeps y_i in registers over the whole item.
// For an off-diagonal tile J the slots walk its T emitters in a staggered order (slot w takes
// emitter (w + s) mod T at step s, one CTA barrier per step), so at every step each emitter's y_j
// partial sum in shared memory is updated by exactly one slot; after the T steps the tile's y_J
// partials go to an FP32 accumulator in global memory with vector atomics. The diagonal tile J = I
// is applied one-directionally (all ordered pairs, the self pair included). A final kernel forms
// W x or x - T W x in FP64.
//
// Arithmetic: for RHS slices of two or more the complex multiply-adds run as packed FP32x2 FMAs on
// pairs of right-hand sides; the staged vectors are stored per RHS pair as (re_r, re_r+1, im_r, im_r+1)
// so that one 16-byte shared-memory load feeds four packed FMAs without shuffles.
//
// Summation order across CTAs follows the hardware's atomic order, so results may differ run to run
// in the last FP32 bits; this operator only drives the correction solves of the FP64 iterative
// refinement, whose residuals use an FP64-grade operator.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "sg_internal.h"

namespace sg {

static constexpr int kSymWarps = 8;  // warps per CTA
static constexpr int kSymThreads = kSymWarps * 32;
static constexpr int kSymChunk = 8;   // emitter tiles per work item
static constexpr int kSymStages = 3;  // coefficient ring stages per warp
static constexpr long long kSymWaitCycles = 2000000000LL;  // ~1 s at 2 GHz per wait
static constexpr size_t kSymSmemMax = 227 * 1024;
static constexpr unsigned kFull = 0xffffffffu;

struct SymLaunch {
  const int4 *pairs;    // [N][N] (interval, t, cos phi, sin phi) of the ordered pair (i, j)
  const int *mofn;      // [bs]
  const float2 *coef;   // [n_int][NC][bs][bs], n1 fastest
  const float2 *x32;    // [N][bs][R]
  float2 *yacc;         // [N][bs][R], zero on entry
  const int4 *items;    // (I, J0, J1, 0)
  int *err;             // set to 1 when a bounded wait ran out
  int n, bs, nrhs;
  int ch, nch;          // columns per ring stage, stages per pair
  int ring_f2;          // float2 per receiver ring (kSymStages * NC * ch * bs)
};

template <int RT>
struct SymPad {
  static constexpr int v = RT >= 2 ? RT + 2 : 1;  // staging row stride (float2): conflict-free vector stores
};

__device__ __forceinline__ uint32_t sym_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// staged row of RT complex values: for RT >= 2 stored per RHS pair as (re_r, re_r+1, im_r, im_r+1)
// (float4 blocks), for RT = 1 as one complex value
template <int RT>
__device__ __forceinline__ void stage_put_t(float2 *row, int r, float2 v) {
  if constexpr (RT >= 2) {
    float *f = reinterpret_cast<float *>(row) + 4 * (r >> 1) + (r & 1);
    f[0] = v.x;
    f[2] = v.y;
  } else {
    row[r] = v;
  }
}

__device__ __forceinline__ void red_add2(float2 *p, float2 a, float2 b) {
  // 16-byte aligned: two consecutive complex values
  atomicAdd(reinterpret_cast<float4 *>(p), make_float4(a.x, a.y, b.x, b.y));
}

// d = a * b + c on two FP32 lanes at once (one packed instruction, sm_100 and later)
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

// all lanes poll; true when the phase of `parity` has completed, false when the budget ran out
__device__ __forceinline__ bool sym_wait(uint32_t bar, uint32_t parity) {
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
    if (__all_sync(kFull, ok)) return true;
    const int late = (clock64() - t0 > kSymWaitCycles) ? 1 : 0;
    if (__shfl_sync(kFull, late, 0)) return false;
  }
}

template <int NC, int RTW, int P, int SPLIT>
__global__ void __launch_bounds__(kSymThreads, SPLIT) sym_kernel(const SymLaunch L) {
  constexpr int T = kSymWarps / SPLIT;   // receivers per CTA = particles per tile
  constexpr int RT = RTW * SPLIT;        // RHS per CTA
  constexpr int RTP = SymPad<RT>::v;
  constexpr int D = kSymStages;
  constexpr int RV = RTW >= 2 ? RTW / 2 : 1;  // float4 (two complex) per warp row; RTW = 1: one float2
  auto stage_put = [](float2 *row, int r, float2 v) { stage_put_t<RT>(row, r, v); };
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int bs = L.bs, N = L.n, R = L.nrhs, CH = L.ch, NCH = L.nch;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = warp % T, half = warp / T;  // receiver slot, RHS slice of the slot
  const bool producer = half == 0;
  const int4 item = L.items[blockIdx.x];
  const int I = item.x, J0 = item.y, J1 = item.z;
  const int r0 = blockIdx.y * RT;   // the CTA's RHS tile in the vectors
  const int rw = half * RTW;        // this warp's slice within the tile
  // shared memory: [rings][x_J][s x_i per slot][y_J][phase tables per warp][mbarriers][abort flags]
  float2 *ring = reinterpret_cast<float2 *>(smem_raw) + (size_t)slot * L.ring_f2;
  float2 *xJ = reinterpret_cast<float2 *>(smem_raw) + (size_t)T * L.ring_f2;  // [T][bs][RT]
  float2 *xs = xJ + (size_t)T * bs * RT + (size_t)slot * bs * RT;             // [bs][RT]
  float2 *yJ = xJ + (size_t)2 * T * bs * RT;                                  // [T][bs][RTP]
  float2 *ph2 = yJ + (size_t)T * bs * RTP + (size_t)warp * bs;                // [bs] e^{i m(n) phi}
  uint64_t *bars0 = reinterpret_cast<uint64_t *>(yJ + (size_t)T * bs * RTP + (size_t)kSymWarps * bs);
  uint64_t *bars = bars0 + slot * D;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(bars0 + T * D) + slot;
  const int ytile = T * bs * RTP;
  for (int e = threadIdx.x; e < ytile; e += blockDim.x) yJ[e] = make_float2(0.f, 0.f);
  if (producer && lane == 0) {
    for (int s = 0; s < D; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sym_smem(&bars[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = 0;
  }
  // the slot's warps meet after every consumed chunk (the producer then refills that stage)
  auto slot_sync = [&]() {
    if constexpr (SPLIT == 2) {
      asm volatile("bar.sync %0, %1;" ::"r"(1 + slot), "r"(64) : "memory");
    } else {
      __syncwarp();
    }
  };

  const int i = I * T + slot;
  const bool has_i = i < N;
  int nrow[P], nrowc[P], mrow[P];
  bool valid[P];
  float sgn[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    nrow[q] = lane + 32 * q;
    valid[q] = nrow[q] < bs;
    nrowc[q] = valid[q] ? nrow[q] : bs - 1;
    mrow[q] = L.mofn[nrowc[q]];
    sgn[q] = (mrow[q] & 1) ? -1.f : 1.f;
  }
  // s(n) x_i for the reverse direction, once per item (each warp its own RHS slice)
  if (has_i) {
    for (int e = lane; e < bs * RTW; e += 32) {
      const int n = e / RTW, r = e - n * RTW;
      const float sg = (L.mofn[n] & 1) ? -1.f : 1.f;
      const float2 a = L.x32[((size_t)i * bs + n) * R + r0 + rw + r];
      stage_put(xs + (size_t)n * RT, rw + r, make_float2(sg * a.x, sg * a.y));
    }
  }
  // accumulators: AR[q][p] = (re_2p, re_2p+1), AI[q][p] = (im_2p, im_2p+1) for RHS slices >= 2
  float2 AR[P][RV], AI[P][RV];
#pragma unroll
  for (int q = 0; q < P; ++q)
#pragma unroll
    for (int p = 0; p < RV; ++p) AR[q][p] = AI[q][p] = make_float2(0.f, 0.f);

  // the slot's pairs q = 0 .. nq-1 in order: tile J0 + q / T, step q % T
  const int nq = (J1 - J0) * T;
  auto pair_jl = [&](int q) {
    const int J = J0 + q / T, s = q % T;
    return J == I ? s : ((slot + s) % T);
  };
  auto pair_ok = [&](int q) { return has_i && (J0 + q / T) * T + pair_jl(q) < N; };
  auto next_ok = [&](int q) {
    while (q < nq && !pair_ok(q)) ++q;
    return q;
  };
  // pair data of tile J in lanes 0..T-1 (lane l: emitter T J + l); cur = consumer's tile, nxt = the one after
  auto load_tile = [&](int J) {
    int4 v = make_int4(0, 0, 0, 0);
    if (has_i && lane < T && J < J1) {
      const int j = J * T + lane;
      if (j < N) v = L.pairs[(size_t)i * N + j];
    }
    return v;
  };
  int4 cur = load_tile(J0), nxt = load_tile(J0 + 1);
  int curJ = J0;
  __syncthreads();

  // producer: next chunk to copy (pair pq, chunk pc); chunks are numbered in issue order, and every
  // warp of the slot keeps the same counters
  int pq = next_ok(0), pc = 0;
  unsigned issued = 0, consumed = 0;
  bool aborted = false;
  const size_t bs2 = (size_t)bs * bs;
  auto issue = [&]() {
    if (pq >= nq) return;
    const int J = J0 + pq / T;
    const int k = __shfl_sync(kFull, J == curJ ? cur.x : nxt.x, pair_jl(pq));
    const int st = (int)(issued % D);
    if (producer && lane == 0) {
      const int n2a = pc * CH, cols = min(CH, bs - n2a);
      const uint32_t bytes = (uint32_t)(cols * bs * (int)sizeof(float2));
      const uint32_t bar = sym_smem(&bars[st]);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the slot's reads of this stage are done
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes * NC) : "memory");
      float2 *dst = ring + (size_t)st * NC * CH * bs;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const float2 *src = L.coef + ((size_t)k * NC + c) * bs2 + (size_t)n2a * bs;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                sym_smem(dst + (size_t)c * CH * bs)),
            "l"(src), "r"(bytes), "r"(bar)
            : "memory");
      }
    }
    ++issued;
    if (++pc == NCH) {
      pc = 0;
      pq = next_ok(pq + 1);
    }
  };
  for (int d = 0; d < D; ++d) issue();

  for (int q = 0; q < nq; ++q) {
    const int J = J0 + q / T, s = q % T;
    const bool diag = (J == I);
    if (s == 0) {
      if (J != curJ) {
        cur = nxt;
        curJ = J;
        nxt = load_tile(J + 1);
      }
      // the tile's emitter vectors x_J[jl][n][r] (all warps read them); the previous tile's readers
      // have passed the barrier that ended their last step
      for (int e = threadIdx.x; e < T * bs * RT; e += blockDim.x) {
        const int jj = e / (bs * RT), rem = e - jj * bs * RT;
        const int n = rem / RT, r = rem - n * RT;
        const int jg = J * T + jj;
        stage_put(xJ + ((size_t)jj * bs + n) * RT, r,
                  jg < N ? L.x32[((size_t)jg * bs + n) * R + r0 + r] : make_float2(0.f, 0.f));
      }
      __syncthreads();
    }
    const int jl = pair_jl(q);
    const float t = __int_as_float(__shfl_sync(kFull, cur.y, jl));
    const float c = __int_as_float(__shfl_sync(kFull, cur.z, jl));
    const float sn = __int_as_float(__shfl_sync(kFull, cur.w, jl));
    if (pair_ok(q) && !aborted) {
      // e^{i m phi} of this lane's rows (repeated multiplication, |m| <= m_max); the same values
      // indexed by column form the per-pair table ph2[n2]
      float ph_re[P], ph_im[P];
#pragma unroll
      for (int qq = 0; qq < P; ++qq) {
        const int am = mrow[qq] < 0 ? -mrow[qq] : mrow[qq];
        float pr = 1.f, pi = 0.f;
        for (int a = 0; a < am; ++a) {
          const float nr = pr * c - pi * sn;
          pi = pr * sn + pi * c;
          pr = nr;
        }
        ph_re[qq] = pr;
        ph_im[qq] = mrow[qq] < 0 ? -pi : pi;
        if (valid[qq]) ph2[nrow[qq]] = make_float2(ph_re[qq], ph_im[qq]);
      }
      __syncwarp();
      const float2 *xjw = xJ + (size_t)jl * bs * RT + rw;  // this warp's slice of x_j, row stride RT
      const float2 *xsw = xs + rw;
      float2 BR[P][RV], BI[P][RV];  // y_j partials of this pair, the same layout as AR, AI
#pragma unroll
      for (int qq = 0; qq < P; ++qq)
#pragma unroll
        for (int pp = 0; pp < RV; ++pp) BR[qq][pp] = BI[qq][pp] = make_float2(0.f, 0.f);
      // W''[n1][n2] = e^{i (m2 - m1) phi} L(t) of this lane's rows at column n2 of a staged chunk
      auto wcoef = [&](const float2 *chunk, int col, int n2, float (&lr)[P], float (&li)[P]) {
        const float2 p2 = ph2[n2];
#pragma unroll
        for (int qq = 0; qq < P; ++qq) {
          const float2 *cp = chunk + (size_t)col * bs + nrowc[qq];
          const float2 cc = cp[(size_t)(NC - 1) * CH * bs];
          float a = cc.x, b = cc.y;
#pragma unroll
          for (int ci = NC - 2; ci >= 0; --ci) {
            const float2 d = cp[(size_t)ci * CH * bs];
            a = fmaf(a, t, d.x);
            b = fmaf(b, t, d.y);
          }
          // p = conj(e^{i m1 phi}) e^{i m2 phi}
          const float pr = fmaf(ph_re[qq], p2.x, ph_im[qq] * p2.y);
          const float pi = fmaf(ph_re[qq], p2.y, -ph_im[qq] * p2.x);
          lr[qq] = fmaf(pr, a, -pi * b);
          li[qq] = fmaf(pr, b, pi * a);
        }
      };
      for (int ch = 0; ch < NCH; ++ch) {
        const int st = (int)(consumed % D);
        if (!sym_wait(sym_smem(&bars[st]), (consumed / D) & 1u)) {
          *abort_flag = 1;
          if (lane == 0) atomicExch(L.err, 1);
        }
        __syncwarp();
        if (!*abort_flag) {
          const float2 *chunk = ring + (size_t)st * NC * CH * bs;
          const int n2a = ch * CH, cols = min(CH, bs - n2a);
          // software pipeline over the chunk's columns: the next column's W'' and x rows are read
          // while this column's multiply-adds run
          float lr[P], li[P];
          wcoef(chunk, 0, n2a, lr, li);
          float4 U[RV], V[RV];
          if constexpr (RTW >= 2) {
#pragma unroll
            for (int rp = 0; rp < RV; ++rp) {
              U[rp] = *reinterpret_cast<const float4 *>(xjw + (size_t)n2a * RT + 2 * rp);
              V[rp] = *reinterpret_cast<const float4 *>(xsw + (size_t)n2a * RT + 2 * rp);
            }
          }
          for (int col = 0; col < cols; ++col) {
            const int n2 = n2a + col;
            const int coln = col + 1 < cols ? col + 1 : col;  // the last column re-reads itself
            float lrn[P], lin[P];
            wcoef(chunk, coln, n2a + coln, lrn, lin);
            if constexpr (RTW >= 2) {
              // (re, re') += lr (ux, ux') - li (uy, uy');  (im, im') += lr (uy, uy') + li (ux, ux')
              float2 LRp[P], LIp[P], NLIp[P];
#pragma unroll
              for (int qq = 0; qq < P; ++qq) {
                LRp[qq] = make_float2(lr[qq], lr[qq]);
                LIp[qq] = make_float2(li[qq], li[qq]);
                NLIp[qq] = make_float2(-li[qq], -li[qq]);
              }
#pragma unroll
              for (int rp = 0; rp < RV; ++rp) {
                const float4 u = U[rp], v = V[rp];
                U[rp] = *reinterpret_cast<const float4 *>(xjw + (size_t)(n2a + coln) * RT + 2 * rp);
                V[rp] = *reinterpret_cast<const float4 *>(xsw + (size_t)(n2a + coln) * RT + 2 * rp);
                const float2 ux = make_float2(u.x, u.y), uy = make_float2(u.z, u.w);
                const float2 vx = make_float2(v.x, v.y), vy = make_float2(v.z, v.w);
#pragma unroll
                for (int qq = 0; qq < P; ++qq) {
                  AR[qq][rp] = ffma2(NLIp[qq], uy, ffma2(LRp[qq], ux, AR[qq][rp]));
                  AI[qq][rp] = ffma2(LIp[qq], ux, ffma2(LRp[qq], uy, AI[qq][rp]));
                  if (!diag) {
                    BR[qq][rp] = ffma2(NLIp[qq], vy, ffma2(LRp[qq], vx, BR[qq][rp]));
                    BI[qq][rp] = ffma2(LIp[qq], vx, ffma2(LRp[qq], vy, BI[qq][rp]));
                  }
                }
              }
            } else {
              const float2 u = xjw[(size_t)n2 * RT], v = xsw[(size_t)n2 * RT];
#pragma unroll
              for (int qq = 0; qq < P; ++qq) {
                AR[qq][0].x = fmaf(lr[qq], u.x, fmaf(-li[qq], u.y, AR[qq][0].x));
                AI[qq][0].x = fmaf(lr[qq], u.y, fmaf(li[qq], u.x, AI[qq][0].x));
                if (!diag) {
                  BR[qq][0].x = fmaf(lr[qq], v.x, fmaf(-li[qq], v.y, BR[qq][0].x));
                  BI[qq][0].x = fmaf(lr[qq], v.y, fmaf(li[qq], v.x, BI[qq][0].x));
                }
              }
            }
#pragma unroll
            for (int qq = 0; qq < P; ++qq) {
              lr[qq] = lrn[qq];
              li[qq] = lin[qq];
            }
          }
        }
        slot_sync();  // every warp of the slot is done with this stage (and has seen the abort flag)
        ++consumed;
        aborted = *abort_flag != 0;
        if (aborted) break;
        issue();
      }
      if (!diag && !aborted) {
#pragma unroll
        for (int qq = 0; qq < P; ++qq) {
          if (!valid[qq]) continue;
          float2 *yr = yJ + ((size_t)jl * bs + nrow[qq]) * RTP + rw;
          if constexpr (RTW >= 2) {
#pragma unroll
            for (int pp = 0; pp < RV; ++pp) {
              float4 v = *reinterpret_cast<float4 *>(yr + 2 * pp);
              v.x = fmaf(sgn[qq], BR[qq][pp].x, v.x);
              v.y = fmaf(sgn[qq], BI[qq][pp].x, v.y);
              v.z = fmaf(sgn[qq], BR[qq][pp].y, v.z);
              v.w = fmaf(sgn[qq], BI[qq][pp].y, v.w);
              *reinterpret_cast<float4 *>(yr + 2 * pp) = v;
            }
          } else {
            float2 v = yr[0];
            v.x = fmaf(sgn[qq], BR[qq][0].x, v.x);
            v.y = fmaf(sgn[qq], BI[qq][0].x, v.y);
            yr[0] = v;
          }
        }
      }
      __syncwarp();  // ph2 is rewritten by the next pair
    }
    if (!diag) __syncthreads();  // emitter slot jl is taken by slot w - 1 at the next step
    if (s == T - 1) {
      if (!diag) {
        // this tile's y_J partials -> global accumulator; clear for the next tile
        const int per = bs * RT;
        if constexpr (RT >= 2) {
          for (int e = threadIdx.x; e < T * per / 2; e += blockDim.x) {
            const int jj = (2 * e) / per, rem = 2 * e - jj * per;
            const int n1 = rem / RT, r = rem - n1 * RT;
            const int jg = J * T + jj;
            float2 *src = yJ + ((size_t)jj * bs + n1) * RTP + r;
            if (jg < N) red_add2(L.yacc + ((size_t)jg * bs + n1) * R + r0 + r, src[0], src[1]);
            src[0] = make_float2(0.f, 0.f);
            src[1] = make_float2(0.f, 0.f);
          }
        } else {
          for (int e = threadIdx.x; e < T * per; e += blockDim.x) {
            const int jj = e / per, n1 = e - jj * per;
            const int jg = J * T + jj;
            float2 *src = yJ + ((size_t)jj * bs + n1) * RTP;
            if (jg < N) {
              atomicAdd(&L.yacc[((size_t)jg * bs + n1) * R + r0].x, src[0].x);
              atomicAdd(&L.yacc[((size_t)jg * bs + n1) * R + r0].y, src[0].y);
            }
            src[0] = make_float2(0.f, 0.f);
          }
        }
      }
      __syncthreads();  // x_J and y_J are rewritten for the next tile
    }
  }
  if (aborted) {
    // copies still in flight land in this CTA's shared memory: the producer waits for them (bounded)
    // before the CTA leaves
    if (producer) {
      while (consumed < issued) {
        if (!sym_wait(sym_smem(&bars[consumed % D]), (consumed / D) & 1u)) break;
        ++consumed;
      }
      if (lane == 0) L.yacc[0].x = __int_as_float(0x7fc00000);  // the result is undefined: make it NaN
    }
    return;
  }
  if (has_i) {
#pragma unroll
    for (int qq = 0; qq < P; ++qq) {
      if (!valid[qq]) continue;
      float2 *dst = L.yacc + ((size_t)i * bs + nrow[qq]) * R + r0 + rw;
      if constexpr (RTW >= 2) {
#pragma unroll
        for (int pp = 0; pp < RV; ++pp)
          red_add2(dst + 2 * pp, make_float2(AR[qq][pp].x, AI[qq][pp].x), make_float2(AR[qq][pp].y, AI[qq][pp].y));
      } else {
        atomicAdd(&dst[0].x, AR[qq][0].x);
        atomicAdd(&dst[0].y, AI[qq][0].x);
      }
    }
  }
}

// y = W x (FP64 from the FP32 sums) or x - T W x; one thread per padded element
__global__ void sym_epilogue_kernel(const float2 *yacc, const double2 *x, double2 *y, int n, int bs, int R, int master,
                                    const double2 *t, const int *ptype, int t_diag) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)n * bs * R;
  if (e >= total) return;
  const int r = (int)(e % R);
  const size_t ib = e / R;
  const int n1 = (int)(ib % bs);
  const int i = (int)(ib / bs);
  const float2 w = yacc[e];
  double2 v = make_double2((double)w.x, (double)w.y);
  if (master) {
    const int ty = ptype[i];
    double2 tw;
    if (t_diag) {
      const double2 tt = t[(size_t)ty * bs + n1];
      tw = make_double2(tt.x * v.x - tt.y * v.y, tt.x * v.y + tt.y * v.x);
    } else {
      const double2 *trow = t + ((size_t)ty * bs + n1) * bs;
      const float2 *wrow = yacc + (size_t)i * bs * R + r;
      double ar = 0.0, ai = 0.0;
      for (int n2 = 0; n2 < bs; ++n2) {
        const double2 tt = trow[n2];
        const float2 a = wrow[(size_t)n2 * R];
        ar = fma(tt.x, (double)a.x, fma(-tt.y, (double)a.y, ar));
        ai = fma(tt.x, (double)a.y, fma(tt.y, (double)a.x, ai));
      }
      tw = make_double2(ar, ai);
    }
    const double2 xv = x[e];
    v = make_double2(xv.x - tw.x, xv.y - tw.y);
  }
  y[e] = v;
}

// ------------------------------------------------------------------ plan and dispatch
bool sym_supported(const sg_context *c) { return !c->vol && c->bs >= 2 && c->bs <= 64 && c->n >= 1; }

int sym_max_tile(const sg_context *c) { return c->bs <= 32 ? 16 : 8; }

// work items: receiver tile I with emitter tiles [J0, J1), J0 >= I (tiles of T particles); full runs first
static void build_sym_items(sg_context *c, int T) {
  const int nt = (c->n + T - 1) / T;
  std::vector<int4> full, part;
  for (int I = 0; I < nt; ++I)
    for (int J0 = I; J0 < nt; J0 += kSymChunk) {
      const int J1 = std::min(nt, J0 + kSymChunk);
      (J1 - J0 == kSymChunk ? full : part).push_back(make_int4(I, J0, J1, 0));
    }
  std::stable_sort(part.begin(), part.end(), [](const int4 &a, const int4 &b) { return a.z - a.y > b.z - b.y; });
  full.insert(full.end(), part.begin(), part.end());
  c->sym_items.reserve(full.size());
  SG_CUDA(cudaMemcpy(c->sym_items.ptr, full.data(), full.size() * sizeof(int4), cudaMemcpyHostToDevice));
  c->sym_n_items = (int)full.size();
  c->sym_items_n = c->n;
  c->sym_items_T = T;
}

template <int NC, int RTW, int P, int SPLIT>
static void launch_sym_t(sg_context *c, SymLaunch L, cudaStream_t st) {
  constexpr int T = kSymWarps / SPLIT;
  constexpr int RT = RTW * SPLIT;
  constexpr int RTP = SymPad<RT>::v;
  if (c->sym_items_n != c->n || c->sym_items_T != T || c->sym_n_items == 0) build_sym_items(c, T);
  L.items = c->sym_items.ptr;
  const int bs = L.bs;
  // shared memory per CTA (SPLIT CTAs per SM): rings, x_J, s x_i per slot, y_J partials, phase tables,
  // mbarriers, abort flags; the ring stage size takes what is left
  const size_t budget = SPLIT == 1 ? kSymSmemMax : kSymSmemMax / 2 - 1024;
  const size_t fixed = ((size_t)2 * T * bs * RT + (size_t)T * bs * RTP + (size_t)kSymWarps * bs) * sizeof(float2) +
                       (size_t)T * kSymStages * sizeof(uint64_t) + 16 * sizeof(int);
  const size_t col_bytes = (size_t)NC * bs * sizeof(float2);
  SG_REQUIRE(fixed + (size_t)T * kSymStages * col_bytes <= budget,
             "symmetric FP32 kernel: blocksize too large for its shared memory");
  int ch = (int)((budget - fixed) / ((size_t)T * kSymStages * col_bytes));
  ch = std::min(ch, bs);
  const int nch = (bs + ch - 1) / ch;
  ch = (bs + nch - 1) / nch;  // equal chunks
  L.ch = ch;
  L.nch = nch;
  L.ring_f2 = kSymStages * NC * ch * bs;
  const size_t smem = fixed + (size_t)T * L.ring_f2 * sizeof(float2);
  static bool attr_done[64] = {};
  if (first_on_device(attr_done))
    SG_CUDA(cudaFuncSetAttribute(sym_kernel<NC, RTW, P, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kSymSmemMax));
  dim3 grid(c->sym_n_items, L.nrhs / RT);
  sym_kernel<NC, RTW, P, SPLIT><<<grid, kSymThreads, smem, st>>>(L);
  SG_CUDA(cudaGetLastError());
}

// RHS tile rt per CTA, served by one warp per receiver (split 1: tiles of 8 particles, one CTA per SM)
// or by two warps per receiver with half the tile each (split 2, rt >= 4: tiles of 4, two CTAs per SM)
template <int NC, int P>
static void launch_sym_r(sg_context *c, const SymLaunch &L, int rt, int split, cudaStream_t st) {
  if (split == 2) {
    if constexpr (P == 1) {
      if (rt == 16) return launch_sym_t<NC, 8, P, 2>(c, L, st);
    }
    if (rt == 8) return launch_sym_t<NC, 4, P, 2>(c, L, st);
    if (rt == 4) return launch_sym_t<NC, 2, P, 2>(c, L, st);
  } else {
    if constexpr (P == 1) {
      if (rt == 16) return launch_sym_t<NC, 16, P, 1>(c, L, st);
    }
    if (rt == 8) return launch_sym_t<NC, 8, P, 1>(c, L, st);
    if (rt == 4) return launch_sym_t<NC, 4, P, 1>(c, L, st);
    if (rt == 2) return launch_sym_t<NC, 2, P, 1>(c, L, st);
    if (rt == 1) return launch_sym_t<NC, 1, P, 1>(c, L, st);
  }
  SG_REQUIRE(false, "unsupported RHS tile for the symmetric FP32 kernel");
}

int launch_sym_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, int rt, int split,
                      cudaStream_t st) {
  SG_REQUIRE(sym_supported(c), "symmetric FP32 kernel: radial lookup with blocksize <= 64 required");
  SG_REQUIRE(split == 1 || (split == 2 && rt >= 4), "symmetric FP32 kernel: two warps per receiver need a tile >= 4");
  SG_REQUIRE(c->pairs_ready, "symmetric FP32 kernel: the pair table is not built");
  SG_REQUIRE(rt >= 1 && R % rt == 0 && rt <= sym_max_tile(c), "symmetric FP32 kernel: bad RHS tile");
  SG_REQUIRE(R / rt <= 65535, "symmetric FP32 kernel: too many RHS tiles");
  if (!c->sym_err_init) {
    c->sym_err.reserve(1);
    SG_CUDA(cudaMemsetAsync(c->sym_err.ptr, 0, sizeof(int), st));
    c->sym_err_init = true;
  }
  const size_t len = (size_t)c->n * c->bs * R;
  c->bk_x32.reserve(len);
  k_to_f32(x, c->bk_x32.ptr, len, st);
  c->sym_yacc.reserve(len);
  SG_CUDA(cudaMemsetAsync(c->sym_yacc.ptr, 0, len * sizeof(float2), st));
  SymLaunch L{};
  L.pairs = c->pairs.ptr;
  L.mofn = c->mofn.ptr;
  L.coef = c->coef32.ptr;
  L.x32 = c->bk_x32.ptr;
  L.yacc = c->sym_yacc.ptr;
  L.err = c->sym_err.ptr;
  L.n = c->n;
  L.bs = c->bs;
  L.nrhs = R;
  const int P = (c->bs + 31) / 32;
  if (c->ncoef == 2) {
    if (P == 1) launch_sym_r<2, 1>(c, L, rt, split, st);
    else launch_sym_r<2, 2>(c, L, rt, split, st);
  } else {
    if (P == 1) launch_sym_r<4, 1>(c, L, rt, split, st);
    else launch_sym_r<4, 2>(c, L, rt, split, st);
  }
  launch_fp32_epilogue(c, x, y, R, master, st);
  return 3;  // conversion, coupling, epilogue (the memset is not a kernel of this library)
}

void launch_fp32_epilogue(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  const size_t len = (size_t)c->n * c->bs * R;
  sym_epilogue_kernel<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(c->sym_yacc.ptr, x, y, c->n, c->bs, R,
                                                                     master ? 1 : 0, c->tmat.ptr, c->ptype.ptr,
                                                                     c->t_diag);
  SG_CUDA(cudaGetLastError());
}

// reads and clears the pair-symmetric kernel's error flag (synchronises the stream)
bool sym_check_error(sg_context *c, cudaStream_t st) {
  if (!c->sym_err_init) return false;
  int h = 0;
  SG_CUDA(cudaMemcpyAsync(&h, c->sym_err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (h) SG_CUDA(cudaMemsetAsync(c->sym_err.ptr, 0, sizeof(int), st));
  return h != 0;
}

}  // namespace sg

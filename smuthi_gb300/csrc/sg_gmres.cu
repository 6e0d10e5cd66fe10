// GMRES(m) on the master operator M = 1 - T W, on the device.
//
// Mirrors the control flow of scipy.sparse.linalg.gmres as called by the reference
// (smuthi/linearsystem/linear_system.py:285): x0 = given, restart m, stop when
// ||b - M x|| <= rtol ||b||, Givens-rotated Hessenberg least squares, adaptive inner
// tolerance, explicit residual at every restart. Differences: orthogonalisation is
// classical Gram-Schmidt applied twice (CGS2; as stable as scipy's MGS and four
// batched kernels instead of 2(j+1) dependent ones), and nrhs > 1 right-hand sides
// run independent Krylov spaces in lockstep that share one block matvec per step.
//
// Vectors live in the padded layout [particle][blocksize][nrhs] (double2).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <vector>

#include "sg_internal.h"

namespace sg {

typedef std::complex<double> cd;
static constexpr int kMaxVec = 130;  // restart <= 128, plus w and one spare
static constexpr int kHcol = 2 * kMaxVec + 4;  // per-rhs slots of the Arnoldi scalar buffer

struct VecList {
  const double2 *v[kMaxVec];
};

// partial[blk][k][r] = sum_{rows in blk} conj(V_k[row][r]) * w[row][r]
__global__ void dots_partial_kernel(VecList V, int nvec, const double2 *w, size_t rows, int R, double2 *partial) {
  extern __shared__ double2 sd[];
  const int tpr = blockDim.x / R;  // threads per rhs column (blockDim.x is a multiple of R)
  const int r = threadIdx.x % R, lr = threadIdx.x / R;
  const size_t nblk = gridDim.x;
  for (int k = 0; k < nvec; ++k) {
    double sr = 0.0, si = 0.0;
    for (size_t row = blockIdx.x * (size_t)tpr + lr; row < rows; row += nblk * tpr) {
      const double2 a = V.v[k][row * R + r], b = w[row * R + r];
      sr = fma(a.x, b.x, fma(a.y, b.y, sr));
      si = fma(a.x, b.y, fma(-a.y, b.x, si));
    }
    sd[threadIdx.x] = make_double2(sr, si);
    __syncthreads();
    // reduce over lr for each r (tree over the lr index)
    for (int s = tpr / 2; s > 0; s >>= 1) {
      if (lr < s) {
        const double2 o = sd[threadIdx.x + s * R];
        sd[threadIdx.x].x += o.x;
        sd[threadIdx.x].y += o.y;
      }
      __syncthreads();
    }
    if (lr == 0) partial[((size_t)blockIdx.x * nvec + k) * R + r] = sd[r];
    __syncthreads();
  }
}

__global__ void dots_final_kernel(const double2 *partial, int nblk, int nvec, int R, double2 *out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nvec * R) return;
  double sr = 0.0, si = 0.0;
  for (int b = 0; b < nblk; ++b) {
    const double2 v = partial[(size_t)b * nvec * R + e];
    sr += v.x;
    si += v.y;
  }
  out[e] = make_double2(sr, si);
}

// y[row][r] += sign * sum_k V_k[row][r] * c[k][r]
__global__ void combine_kernel(VecList V, int nvec, const double2 *c, double sign, double2 *y, size_t rows, int R) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * R) return;
  const int r = (int)(e % R);
  double2 acc = y[e];
  for (int k = 0; k < nvec; ++k) {
    const double2 a = V.v[k][e], h = c[k * R + r];
    acc.x = fma(sign * a.x, h.x, fma(-sign * a.y, h.y, acc.x));
    acc.y = fma(sign * a.x, h.y, fma(sign * a.y, h.x, acc.y));
  }
  y[e] = acc;
}

// y = x * s[r] (real scale per rhs)
__global__ void scale_kernel(const double2 *x, const double *s, double2 *y, size_t rows, int R) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * R) return;
  const double f = s[e % R];
  y[e] = make_double2(x[e].x * f, x[e].y * f);
}

// r = b - r (residual from a master-matvec result)
__global__ void sub_from_kernel(const double2 *b, double2 *r, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  r[e] = make_double2(b[e].x - r[e].x, b[e].y - r[e].y);
}

// x += d * mask[r]
__global__ void add_masked_kernel(double2 *x, const double2 *d, const double *mask, size_t rows, int R) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * R) return;
  const double f = mask[e % R];
  x[e].x += f * d[e].x;
  x[e].y += f * d[e].y;
}

__global__ void zero_kernel(double2 *p, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) p[e] = make_double2(0.0, 0.0);
}

__global__ void gather_kernel(const double2 *src, double2 *dst, const int *map, int nu, int R) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)nu * R) return;
  const int u = (int)(e / R), r = (int)(e % R);
  dst[(size_t)map[u] * R + r] = src[e];
}

__global__ void scatter_kernel(const double2 *src, double2 *dst, const int *map, int nu, int R) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)nu * R) return;
  const int u = (int)(e / R), r = (int)(e % R);
  dst[e] = src[(size_t)map[u] * R + r];
}

static inline unsigned nblocks(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

void k_zero(double2 *p, size_t n, cudaStream_t st) {
  if (!n) return;
  zero_kernel<<<nblocks(n), 256, 0, st>>>(p, n);
  SG_CUDA(cudaGetLastError());
}
void k_gather(const double2 *src, double2 *dst, const int *map, int nu, int R, cudaStream_t st) {
  gather_kernel<<<nblocks((size_t)nu * R), 256, 0, st>>>(src, dst, map, nu, R);
  SG_CUDA(cudaGetLastError());
}
void k_scatter(const double2 *src, double2 *dst, const int *map, int nu, int R, cudaStream_t st) {
  scatter_kernel<<<nblocks((size_t)nu * R), 256, 0, st>>>(src, dst, map, nu, R);
  SG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------ operator + dots
void apply_padded(sg_context *c, const double2 *x, double2 *y, int R, bool master, bool fp32, cudaStream_t st);

struct Solver {
  sg_context *c;
  cudaStream_t st;
  int R;
  size_t rows;  // padded rows = n * bs
  int64_t *launches;

  size_t len() const { return rows * R; }

  // y = M x on padded vectors with the FP64 or FP32 operator
  void master(const double2 *x, double2 *y, bool fp32) { apply_padded(c, x, y, R, true, fp32, st); }
  // y = M x with FP64-grade sums: the FP64 operator, or its double-float twin when df64 is set
  void master_true(const double2 *x, double2 *y, bool df64) {
    if (df64) apply_padded_df64(c, x, y, R, true, st);
    else apply_padded(c, x, y, R, true, false, st);
  }

  // out[k][r] = <V_k, w> for k < nvec (device), copied to host h (nvec * R)
  void dots(const VecList &V, int nvec, const double2 *w, double2 *dout) {
    int tpb = 256;
    const int tpr = std::max(1, tpb / R);
    int p2 = 1;
    while (p2 * 2 <= tpr) p2 *= 2;
    tpb = p2 * R;
    const int nblk = (int)std::min<size_t>((size_t)sm_count() * 2, (rows + p2 - 1) / p2);
    c->w_tmp.reserve((size_t)nblk * nvec * R);
    dots_partial_kernel<<<nblk, tpb, tpb * sizeof(double2), st>>>(V, nvec, w, rows, R, c->w_tmp.ptr);
    SG_CUDA(cudaGetLastError());
    dots_final_kernel<<<nblocks((size_t)nvec * R), 256, 0, st>>>(c->w_tmp.ptr, nblk, nvec, R, dout);
    SG_CUDA(cudaGetLastError());
    *launches += 2;
  }

  void combine(const VecList &V, int nvec, const double2 *coef, double sign, double2 *y) {
    combine_kernel<<<nblocks(len()), 256, 0, st>>>(V, nvec, coef, sign, y, rows, R);
    SG_CUDA(cudaGetLastError());
    *launches += 1;
  }
};

// LAPACK zlartg convention: [c s; -conj(s) c] [f; g] = [r; 0], c real.
static void lartg(cd f, cd g, double &cs, cd &sn, cd &r) {
  const double af = std::abs(f), ag = std::abs(g);
  if (ag == 0.0) {
    cs = 1.0;
    sn = 0.0;
    r = f;
    return;
  }
  if (af == 0.0) {
    cs = 0.0;
    sn = std::conj(g) / ag;
    r = ag;
    return;
  }
  const double nrm = std::hypot(af, ag);
  cs = af / nrm;
  const cd fs = f / af;
  sn = fs * std::conj(g) / nrm;
  r = fs * nrm;
}

struct GmresResult {
  int inner_iters = 0;
  int cycles = 0;
  int matvecs = 0;
  bool breakdown = false;
  std::vector<double> relres;  // per rhs: final ||b - M x|| / ||b|| with the solve's operator
  std::vector<char> conv;
};

// Lockstep GMRES on padded device vectors. b, x: len(); x holds x0 (zero_x0 = x0 is zero).
// stall_cycles > 0 stops a right-hand side whose explicit residual fell by less than 5% over that many
// consecutive restart cycles (used for the FP32-operator correction solves, whose residual has a noise
// floor near the FP32 operator error); 0 keeps scipy's semantics.
// precond = true runs flexible GMRES with the learned right preconditioner P: the Arnoldi step applies
// M to z_k = P v_k, and the update is x += Z y.
static GmresResult gmres_lockstep(Solver &S, const double2 *b, double2 *x, double rtol, int restart, int maxiter,
                                  bool fp32, bool zero_x0, const std::vector<char> &skip, int stall_cycles = 0,
                                  bool precond = false) {
  sg_context *c = S.c;
  const int R = S.R;
  const size_t len = S.len();
  restart = std::max(1, std::min(restart, (int)std::min<size_t>(S.rows, kMaxVec - 2)));
  c->w_basis.reserve((size_t)(restart + 1) * len);
  if (precond) c->w_z.reserve((size_t)restart * len);
  auto Zk = [&](int k) { return c->w_z.ptr + (size_t)k * len; };
  c->w_w.reserve(len);
  c->w_r.reserve(len);
  c->w_hcol.reserve((size_t)kHcol * R);
  c->w_red.reserve((size_t)4 * R + 4);
  double2 *V0 = c->w_basis.ptr;
  double2 *w = c->w_w.ptr;
  double2 *r = c->w_r.ptr;
  double2 *dh = c->w_hcol.ptr;
  auto Vk = [&](int k) { return V0 + (size_t)k * len; };
  const double eps = 2.220446049250313e-16;
  GmresResult res;
  res.relres.assign(R, 0.0);
  res.conv.assign(R, 0);

  // ||b||
  std::vector<double2> hb((size_t)kHcol * R);
  VecList L1{};
  L1.v[0] = b;
  S.dots(L1, 1, b, dh);
  SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
  SG_CUDA(cudaStreamSynchronize(S.st));
  std::vector<double> bnrm(R), atol(R), ptol(R), pfac(R, 1.0), presid(R, 0.0), rnorm(R, 0.0);
  std::vector<char> active(R, 1);
  for (int q = 0; q < R; ++q) {
    bnrm[q] = std::sqrt(std::max(0.0, hb[q].x));
    atol[q] = rtol * bnrm[q];
    if (bnrm[q] == 0.0 || (!skip.empty() && skip[q])) {
      active[q] = 0;
      res.conv[q] = 1;
    }
  }
  // r = b - M x0; like scipy, an all-zero x0 skips the operator application
  if (!zero_x0) {
    L1.v[0] = x;
    S.dots(L1, 1, x, dh);
    SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
    SG_CUDA(cudaStreamSynchronize(S.st));
    bool allzero = true;
    for (int q = 0; q < R; ++q) allzero &= hb[q].x == 0.0;
    zero_x0 = allzero;
  }
  if (zero_x0) {
    SG_CUDA(cudaMemcpyAsync(r, b, len * sizeof(double2), cudaMemcpyDeviceToDevice, S.st));
  } else {
    S.master(x, r, fp32);
    res.matvecs++;
    sub_from_kernel<<<nblocks(len), 256, 0, S.st>>>(b, r, len);
    SG_CUDA(cudaGetLastError());
    // already converged at x0?
    L1.v[0] = r;
    S.dots(L1, 1, r, dh);
    SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
    SG_CUDA(cudaStreamSynchronize(S.st));
    for (int q = 0; q < R; ++q) {
      rnorm[q] = std::sqrt(std::max(0.0, hb[q].x));
      if (active[q] && rnorm[q] < atol[q]) {
        active[q] = 0;
        res.conv[q] = 1;
      }
    }
  }
  for (int q = 0; q < R; ++q) ptol[q] = bnrm[q] * std::min(1.0, bnrm[q] > 0 ? atol[q] / bnrm[q] : 1.0);

  std::vector<cd> H((size_t)restart * (restart + 1) * R), G((size_t)restart * R), Sv((size_t)(restart + 1) * R);
  std::vector<double> Gc((size_t)restart * R);
  std::vector<double> hscale(R), hmask(R);
  std::vector<int> colstop(R);
  std::vector<char> inner_done(R), breakdown(R);
  std::vector<int> stalls(R, 0);
  int inner_iter = 0;
  c->w_d.reserve(len);

  for (int cycle = 0; cycle < maxiter; ++cycle) {
    bool any = false;
    for (int q = 0; q < R; ++q) any |= active[q] != 0;
    if (!any) break;
    res.cycles++;
    // v0 = r / ||r||
    L1.v[0] = r;
    S.dots(L1, 1, r, dh);
    SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
    SG_CUDA(cudaStreamSynchronize(S.st));
    for (int q = 0; q < R; ++q) {
      const double nr = std::sqrt(std::max(0.0, hb[q].x));
      hscale[q] = nr > 0 ? 1.0 / nr : 0.0;
      for (int k = 0; k <= restart; ++k) Sv[(size_t)k * R + q] = 0.0;
      Sv[q] = nr;
      inner_done[q] = active[q] ? 0 : 1;
      breakdown[q] = 0;
      colstop[q] = -1;
      if (active[q] && nr == 0.0) inner_done[q] = 1;
    }
    double *dscale = c->w_red.ptr;
    SG_CUDA(cudaMemcpyAsync(dscale, hscale.data(), R * sizeof(double), cudaMemcpyHostToDevice, S.st));
    scale_kernel<<<nblocks(len), 256, 0, S.st>>>(r, dscale, Vk(0), S.rows, R);
    SG_CUDA(cudaGetLastError());

    int col = 0;
    for (col = 0; col < restart; ++col) {
      bool all_done = true;
      for (int q = 0; q < R; ++q) all_done &= inner_done[q] != 0;
      if (all_done) break;
      // w = M v_col (flexible: w = M z_col, z_col = P v_col)
      if (precond) {
        precond_apply(c, Vk(col), Zk(col), R, S.st);
        S.master(Zk(col), w, fp32);
      } else {
        S.master(Vk(col), w, fp32);
      }
      res.matvecs++;
      // pass 1: dots with V_0..V_col and w itself (h0^2)
      VecList L{};
      for (int k = 0; k <= col; ++k) L.v[k] = Vk(k);
      L.v[col + 1] = w;
      S.dots(L, col + 2, w, dh);
      S.combine(L, col + 1, dh, -1.0, w);
      // pass 2: re-orthogonalise, then ||w||^2
      double2 *dh2 = dh + (size_t)(col + 2) * R;
      S.dots(L, col + 1, w, dh2);
      S.combine(L, col + 1, dh2, -1.0, w);
      double2 *dn = dh2 + (size_t)(col + 1) * R;
      L1.v[0] = w;
      S.dots(L1, 1, w, dn);
      const size_t nh = (size_t)(2 * col + 4) * R;
      SG_CUDA(cudaMemcpyAsync(hb.data(), dh, nh * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
      SG_CUDA(cudaStreamSynchronize(S.st));
      inner_iter++;
      for (int q = 0; q < R; ++q) {
        cd *h = &H[((size_t)q * restart + col) * (restart + 1)];
        const double h0 = std::sqrt(std::max(0.0, hb[(size_t)(col + 1) * R + q].x));
        for (int k = 0; k <= col; ++k) {
          const double2 a = hb[(size_t)k * R + q], a2 = hb[(size_t)(col + 2 + k) * R + q];
          h[k] = cd(a.x + a2.x, a.y + a2.y);
        }
        const double h1 = std::sqrt(std::max(0.0, hb[(size_t)(2 * col + 3) * R + q].x));
        h[col + 1] = h1;
        hscale[q] = (h1 > 0) ? 1.0 / h1 : 0.0;
        if (inner_done[q]) continue;
        bool bd = false;
        if (h1 <= eps * h0) {
          h[col + 1] = 0.0;
          bd = true;
        }
        // apply previous rotations
        for (int k = 0; k < col; ++k) {
          const double cs = Gc[(size_t)q * restart + k];
          const cd sn = G[(size_t)q * restart + k];
          const cd n0 = h[k], n1 = h[k + 1];
          h[k] = cs * n0 + sn * n1;
          h[k + 1] = -std::conj(sn) * n0 + cs * n1;
        }
        double cs;
        cd sn, rr;
        lartg(h[col], h[col + 1], cs, sn, rr);
        Gc[(size_t)q * restart + col] = cs;
        G[(size_t)q * restart + col] = sn;
        h[col] = rr;
        h[col + 1] = 0.0;
        const cd tmp = -std::conj(sn) * Sv[(size_t)col * R + q];
        Sv[(size_t)col * R + q] = cs * Sv[(size_t)col * R + q];
        Sv[(size_t)(col + 1) * R + q] = tmp;
        presid[q] = std::abs(tmp);
        colstop[q] = col;
        if (presid[q] <= ptol[q] || bd) {
          inner_done[q] = 1;
          breakdown[q] = bd;
        }
      }
      // v_{col+1} = w / h1
      SG_CUDA(cudaMemcpyAsync(dscale, hscale.data(), R * sizeof(double), cudaMemcpyHostToDevice, S.st));
      scale_kernel<<<nblocks(len), 256, 0, S.st>>>(w, dscale, Vk(col + 1), S.rows, R);
      SG_CUDA(cudaGetLastError());
    }
    // y = H^{-1} S per rhs; x += V y
    std::vector<double2> ycoef((size_t)(restart + 1) * R, make_double2(0, 0));
    int maxcol = -1;
    for (int q = 0; q < R; ++q) {
      if (!active[q] || colstop[q] < 0) continue;
      const int cq = colstop[q];
      maxcol = std::max(maxcol, cq);
      auto hq = [&](int cc, int k) -> cd & { return H[((size_t)q * restart + cc) * (restart + 1) + k]; };
      std::vector<cd> y(cq + 1);
      if (hq(cq, cq) == 0.0) Sv[(size_t)cq * R + q] = 0.0;
      for (int k = 0; k <= cq; ++k) y[k] = Sv[(size_t)k * R + q];
      for (int k = cq; k > 0; --k) {
        if (y[k] != 0.0) {
          y[k] /= hq(k, k);
          const cd t = y[k];
          for (int a = 0; a < k; ++a) y[a] -= t * hq(k, a);
        }
      }
      if (y[0] != 0.0) y[0] /= hq(0, 0);
      for (int k = 0; k <= cq; ++k) ycoef[(size_t)k * R + q] = make_double2(y[k].real(), y[k].imag());
    }
    if (maxcol >= 0) {
      SG_CUDA(cudaMemcpyAsync(dh, ycoef.data(), (size_t)(maxcol + 1) * R * sizeof(double2), cudaMemcpyHostToDevice,
                              S.st));
      VecList L{};
      for (int k = 0; k <= maxcol; ++k) L.v[k] = precond ? Zk(k) : Vk(k);
      S.combine(L, maxcol + 1, dh, 1.0, x);
    }
    // explicit residual r = b - M x
    S.master(x, r, fp32);
    res.matvecs++;
    sub_from_kernel<<<nblocks(len), 256, 0, S.st>>>(b, r, len);
    SG_CUDA(cudaGetLastError());
    L1.v[0] = r;
    S.dots(L1, 1, r, dh);
    SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
    SG_CUDA(cudaStreamSynchronize(S.st));
    for (int q = 0; q < R; ++q) {
      const double before = rnorm[q];
      rnorm[q] = std::sqrt(std::max(0.0, hb[q].x));
      if (!active[q]) continue;
      if (rnorm[q] <= atol[q]) {
        active[q] = 0;
        res.conv[q] = 1;
        continue;
      }
      if (breakdown[q]) {
        active[q] = 0;
        continue;
      }
      if (stall_cycles > 0) {
        const double ref = cycle == 0 ? bnrm[q] : before;
        stalls[q] = (rnorm[q] > 0.95 * ref) ? stalls[q] + 1 : 0;
        if (stalls[q] >= stall_cycles) {
          active[q] = 0;
          continue;
        }
      }
      if (presid[q] <= ptol[q]) pfac[q] = std::max(eps, 0.25 * pfac[q]);
      else pfac[q] = std::min(1.0, 1.5 * pfac[q]);
      ptol[q] = presid[q] * std::min(pfac[q], atol[q] / rnorm[q]);
    }
  }
  res.inner_iters = inner_iter;
  for (int q = 0; q < R; ++q) {
    if (bnrm[q] > 0) res.relres[q] = rnorm[q] / bnrm[q];
    if (bnrm[q] == 0.0) res.conv[q] = 1;
  }
  return res;
}

// ------------------------------------------------------------------ block GMRES
// One block Krylov space for all active right-hand sides: block Arnoldi with classical Gram-Schmidt
// applied twice, CholeskyQR2 for each new block, and the block-Hessenberg least-squares problem
// solved by incrementally applied complex Householder reflectors on the host. Columns that already
// meet the tolerance are compacted out at every restart.

// partial[blk][i][a][b] = sum_{rows in blk} conj(V_i[row][a]) * W[row][b]   (16 x 16 (a, b) tiles)
__global__ void gram_partial_kernel(VecList V, int nv, const double2 *W, size_t rows, int Ra, double2 *partial) {
  __shared__ double2 vs[32][17], ws[32][17];
  const int i = blockIdx.y;
  const int ntile = (Ra + 15) / 16;
  const int ta0 = (blockIdx.z / ntile) * 16, tb0 = (blockIdx.z % ntile) * 16;
  const int tid = threadIdx.x, ta = tid / 16, tb = tid % 16;
  const int a = ta0 + ta, b = tb0 + tb;
  double sr = 0.0, si = 0.0;
  const double2 *Vi = V.v[i];
  for (size_t r0 = (size_t)blockIdx.x * 32; r0 < rows; r0 += (size_t)gridDim.x * 32) {
    for (int e = tid; e < 32 * 16; e += blockDim.x) {
      const int rr = e / 16, cc = e % 16;
      const size_t row = r0 + rr;
      const bool ok = row < rows;
      vs[rr][cc] = (ok && ta0 + cc < Ra) ? Vi[row * Ra + ta0 + cc] : make_double2(0.0, 0.0);
      ws[rr][cc] = (ok && tb0 + cc < Ra) ? W[row * Ra + tb0 + cc] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 8
    for (int rr = 0; rr < 32; ++rr) {
      const double2 p = vs[rr][ta], q = ws[rr][tb];
      sr = fma(p.x, q.x, fma(p.y, q.y, sr));
      si = fma(p.x, q.y, fma(-p.y, q.x, si));
    }
    __syncthreads();
  }
  if (a < Ra && b < Ra) partial[(((size_t)blockIdx.x * nv + i) * Ra + a) * Ra + b] = make_double2(sr, si);
}

// out[e] = sum over blk of partial[blk][e], e < n
__global__ void sum_partials_kernel(const double2 *partial, int nblk, size_t n, double2 *out) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double sr = 0.0, si = 0.0;
  for (int k = 0; k < nblk; ++k) {
    const double2 v = partial[(size_t)k * n + e];
    sr += v.x;
    si += v.y;
  }
  out[e] = make_double2(sr, si);
}

// W[row][b] += sign * sum_i sum_a V_i[row][a] * C[i][a][b]; V blocks have Ra columns, W and C have Rc
__global__ void block_combine_kernel(VecList V, int nv, int Ra, const double2 *C, int Rc, double sign, double2 *W,
                                     size_t rows) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * Rc) return;
  const size_t row = e / Rc;
  const int b = (int)(e - row * Rc);
  double ar = 0.0, ai = 0.0;
  for (int i = 0; i < nv; ++i) {
    const double2 *vr = V.v[i] + row * Ra;
    const double2 *ci = C + (size_t)i * Ra * Rc + b;
    for (int a = 0; a < Ra; ++a) {
      const double2 v = vr[a], h = ci[(size_t)a * Rc];
      ar = fma(v.x, h.x, fma(-v.y, h.y, ar));
      ai = fma(v.x, h.y, fma(v.y, h.x, ai));
    }
  }
  W[e].x += sign * ar;
  W[e].y += sign * ai;
}

// out[row][b] = sum_a W[row][a] * Mt[a][b]   (Ra x Ra)
__global__ void right_mult_kernel(const double2 *W, const double2 *Mt, size_t rows, int Ra, double2 *out) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * Ra) return;
  const size_t row = e / Ra;
  const int b = (int)(e - row * Ra);
  double ar = 0.0, ai = 0.0;
  for (int a = 0; a < Ra; ++a) {
    const double2 w = W[row * Ra + a], m = Mt[(size_t)a * Ra + b];
    ar = fma(w.x, m.x, fma(-w.y, m.y, ar));
    ai = fma(w.x, m.y, fma(w.y, m.x, ai));
  }
  out[e] = make_double2(ar, ai);
}

// dst[row][q] = src[row][cols[q]] (gather) or dst[row][cols[q]] += src[row][q] (scatter-add)
__global__ void cols_kernel(const double2 *src, double2 *dst, const int *cols, size_t rows, int Rwide, int Ra,
                            int scatter_add) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * Ra) return;
  const size_t row = e / Ra;
  const int q = (int)(e - row * Ra);
  if (scatter_add) {
    double2 &d = dst[row * Rwide + cols[q]];
    d.x += src[e].x;
    d.y += src[e].y;
  } else {
    dst[e] = src[row * Rwide + cols[q]];
  }
}

struct BlockOps {
  Solver &S;
  sg_context *c;
  size_t rows;
  std::vector<cd> host;

  // H[i] (Ra x Ra) = V_i^H W for i < nv, result on the host (row-major [i][a][b])
  void gram(const VecList &V, int nv, const double2 *W, int Ra, std::vector<cd> &H) {
    const int ntile = (Ra + 15) / 16;
    const int nblk = (int)std::min<size_t>((size_t)sm_count(), (rows + 31) / 32);
    const size_t n = (size_t)nv * Ra * Ra;
    c->w_tmp.reserve((size_t)nblk * n + n);
    dim3 grid(nblk, nv, ntile * ntile);
    gram_partial_kernel<<<grid, 256, 0, S.st>>>(V, nv, W, rows, Ra, c->w_tmp.ptr);
    SG_CUDA(cudaGetLastError());
    double2 *out = c->w_tmp.ptr + (size_t)nblk * n;
    sum_partials_kernel<<<nblocks(n), 256, 0, S.st>>>(c->w_tmp.ptr, nblk, n, out);
    SG_CUDA(cudaGetLastError());
    *S.launches += 2;
    std::vector<double2> h(n);
    SG_CUDA(cudaMemcpyAsync(h.data(), out, n * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
    SG_CUDA(cudaStreamSynchronize(S.st));
    H.resize(n);
    for (size_t e = 0; e < n; ++e) H[e] = cd(h[e].x, h[e].y);
  }

  // W += sign * sum_i V_i C_i with C on the host ([i][a][b], Ra x Rc blocks)
  void combine(const VecList &V, int nv, int Ra, const std::vector<cd> &C, int Rc, double sign, double2 *W) {
    std::vector<double2> h(C.size());
    for (size_t e = 0; e < C.size(); ++e) h[e] = make_double2(C[e].real(), C[e].imag());
    c->w_hcol.reserve(std::max<size_t>(c->w_hcol.n, h.size()));
    SG_CUDA(cudaMemcpyAsync(c->w_hcol.ptr, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, S.st));
    block_combine_kernel<<<nblocks(rows * Rc), 256, 0, S.st>>>(V, nv, Ra, c->w_hcol.ptr, Rc, sign, W, rows);
    SG_CUDA(cudaGetLastError());
    *S.launches += 1;
  }

  // CholeskyQR2: W (rows x Ra) -> orthonormal Q in place, Rf (Ra x Ra upper, row-major). false on breakdown.
  bool cholqr2(double2 *W, double2 *tmp, int Ra, std::vector<cd> &Rf) {
    std::vector<cd> Rtot(Ra * Ra, 0.0);
    for (int a = 0; a < Ra; ++a) Rtot[a * Ra + a] = 1.0;
    for (int pass = 0; pass < 2; ++pass) {
      VecList L{};
      L.v[0] = W;
      std::vector<cd> G;
      gram(L, 1, W, Ra, G);
      // Cholesky G = U^H U (U upper)
      std::vector<cd> U(Ra * Ra, 0.0);
      double gmax = 0.0;
      for (int a = 0; a < Ra; ++a) gmax = std::max(gmax, G[a * Ra + a].real());
      for (int a = 0; a < Ra; ++a) {
        cd d = G[a * Ra + a];
        for (int k = 0; k < a; ++k) d -= std::conj(U[k * Ra + a]) * U[k * Ra + a];
        if (!(d.real() > 1e-24 * std::max(gmax, 1e-300))) return false;
        const double ua = std::sqrt(d.real());
        U[a * Ra + a] = ua;
        for (int b = a + 1; b < Ra; ++b) {
          cd v = G[a * Ra + b];
          for (int k = 0; k < a; ++k) v -= std::conj(U[k * Ra + a]) * U[k * Ra + b];
          U[a * Ra + b] = v / ua;
        }
      }
      // Uinv (upper) by back substitution
      std::vector<cd> Ui(Ra * Ra, 0.0);
      for (int col = 0; col < Ra; ++col) {
        for (int a = Ra - 1; a >= 0; --a) {
          cd v = (a == col) ? cd(1.0) : cd(0.0);
          for (int k = a + 1; k < Ra; ++k) v -= U[a * Ra + k] * Ui[k * Ra + col];
          Ui[a * Ra + col] = v / U[a * Ra + a];
        }
      }
      std::vector<double2> h(Ra * Ra);
      for (int e = 0; e < Ra * Ra; ++e) h[e] = make_double2(Ui[e].real(), Ui[e].imag());
      c->w_red.reserve(std::max<size_t>(c->w_red.n, 2 * (size_t)Ra * Ra));
      double2 *dm = reinterpret_cast<double2 *>(c->w_red.ptr);
      SG_CUDA(cudaMemcpyAsync(dm, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, S.st));
      right_mult_kernel<<<nblocks(rows * Ra), 256, 0, S.st>>>(W, dm, rows, Ra, tmp);
      SG_CUDA(cudaGetLastError());
      SG_CUDA(cudaMemcpyAsync(W, tmp, rows * Ra * sizeof(double2), cudaMemcpyDeviceToDevice, S.st));
      *S.launches += 1;
      SG_CUDA(cudaStreamSynchronize(S.st));
      // Rtot = U * Rtot
      std::vector<cd> Rn(Ra * Ra, 0.0);
      for (int a = 0; a < Ra; ++a)
        for (int b = 0; b < Ra; ++b) {
          cd v = 0.0;
          for (int k = a; k < Ra; ++k) v += U[a * Ra + k] * Rtot[k * Ra + b];
          Rn[a * Ra + b] = v;
        }
      Rtot.swap(Rn);
    }
    Rf.swap(Rtot);
    return true;
  }
};

// Complex Householder reflector for x (length len): returns v (v[0] set) and beta; H x = beta e1,
// H = I - 2 v v^H / (v^H v).
static void householder(cd *x, int len, std::vector<cd> &v, cd &beta) {
  double nrm = 0.0;
  for (int k = 0; k < len; ++k) nrm += std::norm(x[k]);
  nrm = std::sqrt(nrm);
  v.assign(x, x + len);
  if (nrm == 0.0) {
    beta = 0.0;
    return;
  }
  const double ax = std::abs(x[0]);
  const cd ph = ax > 0 ? x[0] / ax : cd(1.0);
  beta = -ph * nrm;
  v[0] = x[0] - beta;
}

static void apply_reflector(const std::vector<cd> &v, cd *y, int len) {
  cd vh_y = 0.0;
  double vv = 0.0;
  for (int k = 0; k < len; ++k) {
    vh_y += std::conj(v[k]) * y[k];
    vv += std::norm(v[k]);
  }
  if (vv == 0.0) return;
  const cd f = 2.0 * vh_y / vv;
  for (int k = 0; k < len; ++k) y[k] -= f * v[k];
}

// Block GMRES on padded device vectors (nrhs = S.R); x holds x0 (zero_x0: x0 == 0). Returns the
// per-RHS explicit residual of the final iterate with the solve's operator.
static GmresResult block_gmres(Solver &S, const double2 *b, double2 *x, double rtol, int restart, int max_cycles,
                               bool fp32, bool zero_x0, const std::vector<char> &skip) {
  sg_context *c = S.c;
  const int R = S.R;
  const size_t rows = S.rows, len = S.len();
  restart = std::max(1, std::min(restart, 20));
  BlockOps ops{S, c, rows, {}};
  GmresResult res;
  res.relres.assign(R, 0.0);
  res.conv.assign(R, 0);
  c->w_basis.reserve((size_t)(restart + 1) * len);
  c->w_w.reserve(len);
  c->w_r.reserve(len);
  c->w_d.reserve(len);
  c->w_b.reserve(std::max<size_t>(c->w_b.n, len));
  double2 *r = c->w_r.ptr, *W = c->w_w.ptr, *tmp = c->w_d.ptr;
  std::vector<double2> hb((size_t)kHcol * R);
  auto col_norms = [&](const double2 *v, std::vector<double> &out) {
    VecList L{};
    L.v[0] = v;
    S.dots(L, 1, v, c->w_hcol.ptr);
    SG_CUDA(cudaMemcpyAsync(hb.data(), c->w_hcol.ptr, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
    SG_CUDA(cudaStreamSynchronize(S.st));
    out.resize(R);
    for (int q = 0; q < R; ++q) out[q] = std::sqrt(std::max(0.0, hb[q].x));
  };
  c->w_hcol.reserve((size_t)kHcol * R);
  std::vector<double> bnrm, rn;
  col_norms(b, bnrm);
  if (zero_x0) {
    SG_CUDA(cudaMemcpyAsync(r, b, len * sizeof(double2), cudaMemcpyDeviceToDevice, S.st));
  } else {
    S.master(x, r, fp32);
    res.matvecs++;
    sub_from_kernel<<<nblocks(len), 256, 0, S.st>>>(b, r, len);
    SG_CUDA(cudaGetLastError());
  }
  DevBuf<int> dcols;
  dcols.reserve(R);
  for (int cycle = 0; cycle < max_cycles; ++cycle) {
    col_norms(r, rn);
    std::vector<int> cols;
    for (int q = 0; q < R; ++q) {
      if (bnrm[q] > 0) res.relres[q] = rn[q] / bnrm[q];
      const bool ok = rn[q] <= rtol * bnrm[q] || bnrm[q] == 0.0;
      res.conv[q] = ok ? 1 : 0;
      if (!ok && (skip.empty() || !skip[q])) cols.push_back(q);
    }
    if (cols.empty()) break;
    res.cycles++;
    const int Ra = (int)cols.size();
    const size_t blen = rows * Ra;
    auto Vk = [&](int k) { return c->w_basis.ptr + (size_t)k * blen; };
    SG_CUDA(cudaMemcpyAsync(dcols.ptr, cols.data(), Ra * sizeof(int), cudaMemcpyHostToDevice, S.st));
    cols_kernel<<<nblocks(blen), 256, 0, S.st>>>(r, Vk(0), dcols.ptr, rows, R, Ra, 0);
    SG_CUDA(cudaGetLastError());
    std::vector<cd> beta;
    if (!ops.cholqr2(Vk(0), tmp, Ra, beta)) {
      res.breakdown = true;
      break;
    }
    // G = Q^H E1 beta, Rfac = triangular factor, reflectors per column
    const int maxrow = (restart + 1) * Ra;
    std::vector<cd> G((size_t)maxrow * Ra, 0.0);  // row-major [row][q]
    for (int a = 0; a < Ra; ++a)
      for (int q = 0; q < Ra; ++q) G[(size_t)a * Ra + q] = beta[a * Ra + q];
    std::vector<std::vector<cd>> refl;                    // reflector for column c acts on rows c..c+Ra
    std::vector<cd> Rcol((size_t)restart * Ra * maxrow);  // column-major columns of the triangular factor
    int jdone = 0;
    bool stop = false;
    for (int j = 0; j < restart && !stop; ++j) {
      // W = M V_j on the compacted block
      S.R = Ra;
      S.master(Vk(j), W, fp32);
      S.R = R;
      res.matvecs++;
      VecList L{};
      for (int k = 0; k <= j; ++k) L.v[k] = Vk(k);
      std::vector<cd> H1, H2;
      ops.gram(L, j + 1, W, Ra, H1);
      ops.combine(L, j + 1, Ra, H1, Ra, -1.0, W);
      ops.gram(L, j + 1, W, Ra, H2);
      ops.combine(L, j + 1, Ra, H2, Ra, -1.0, W);
      for (size_t e = 0; e < H1.size(); ++e) H1[e] += H2[e];
      std::vector<cd> Hs;
      const bool ok = ops.cholqr2(W, tmp, Ra, Hs);
      if (ok) SG_CUDA(cudaMemcpyAsync(Vk(j + 1), W, blen * sizeof(double2), cudaMemcpyDeviceToDevice, S.st));
      // new block column: rows 0 .. (j+2)Ra
      const int nr = (j + 2) * Ra;
      for (int cc = 0; cc < Ra; ++cc) {
        cd *col = &Rcol[(size_t)(j * Ra + cc) * maxrow];
        for (int rr = 0; rr < maxrow; ++rr) col[rr] = 0.0;
        for (int i = 0; i <= j; ++i)
          for (int a = 0; a < Ra; ++a) col[i * Ra + a] = H1[((size_t)i * Ra + a) * Ra + cc];
        for (int a = 0; a < Ra; ++a) col[(j + 1) * Ra + a] = ok ? Hs[a * Ra + cc] : cd(0.0);
        // previous reflectors
        for (size_t k = 0; k < refl.size(); ++k) apply_reflector(refl[k], col + k, (int)refl[k].size());
      }
      // new reflectors for columns j*Ra .. (j+1)*Ra-1
      for (int cc = 0; cc < Ra; ++cc) {
        const int cidx = j * Ra + cc;
        cd *col = &Rcol[(size_t)cidx * maxrow];
        const int l = std::min(Ra + 1, nr - cidx);
        std::vector<cd> v;
        cd bet;
        householder(col + cidx, l, v, bet);
        col[cidx] = bet;
        for (int k = 1; k < l; ++k) col[cidx + k] = 0.0;
        for (int c2 = cc + 1; c2 < Ra; ++c2) apply_reflector(v, &Rcol[(size_t)(j * Ra + c2) * maxrow] + cidx, l);
        // apply to G columns
        for (int q = 0; q < Ra; ++q) {
          std::vector<cd> g(l);
          for (int k = 0; k < l; ++k) g[k] = G[(size_t)(cidx + k) * Ra + q];
          apply_reflector(v, g.data(), l);
          for (int k = 0; k < l; ++k) G[(size_t)(cidx + k) * Ra + q] = g[k];
        }
        refl.push_back(v);
      }
      jdone = j + 1;
      res.inner_iters++;
      // implicit residual per active column: rows (j+1)Ra .. (j+2)Ra of G
      bool all = true;
      for (int q = 0; q < Ra; ++q) {
        double s2 = 0.0;
        for (int a = 0; a < Ra; ++a) s2 += std::norm(G[(size_t)((j + 1) * Ra + a) * Ra + q]);
        if (std::sqrt(s2) > rtol * bnrm[cols[q]]) all = false;
      }
      if (all || !ok) stop = true;
    }
    // Y = Rfac^{-1} G[0 : jdone*Ra]
    const int K = jdone * Ra;
    std::vector<cd> Y((size_t)K * Ra, 0.0);
    for (int q = 0; q < Ra; ++q)
      for (int rr = K - 1; rr >= 0; --rr) {
        cd v = G[(size_t)rr * Ra + q];
        for (int k = rr + 1; k < K; ++k) v -= Rcol[(size_t)k * maxrow + rr] * Y[(size_t)k * Ra + q];
        const cd d = Rcol[(size_t)rr * maxrow + rr];
        Y[(size_t)rr * Ra + q] = d != 0.0 ? v / d : cd(0.0);
      }
    // dx = V Y (compact), x[:, cols] += dx
    VecList L{};
    for (int k = 0; k < jdone; ++k) L.v[k] = Vk(k);
    k_zero(tmp, blen, S.st);
    ops.combine(L, jdone, Ra, Y, Ra, 1.0, tmp);
    cols_kernel<<<nblocks(blen), 256, 0, S.st>>>(tmp, x, dcols.ptr, rows, R, Ra, 1);
    SG_CUDA(cudaGetLastError());
    // explicit residual
    S.master(x, r, fp32);
    res.matvecs++;
    sub_from_kernel<<<nblocks(len), 256, 0, S.st>>>(b, r, len);
    SG_CUDA(cudaGetLastError());
  }
  col_norms(r, rn);
  for (int q = 0; q < R; ++q) {
    if (bnrm[q] > 0) res.relres[q] = rn[q] / bnrm[q];
    res.conv[q] = (rn[q] <= rtol * bnrm[q] || bnrm[q] == 0.0) ? 1 : 0;
  }
  return res;
}

// Mixed precision: FP32-operator GMRES corrections inside FP64 iterative refinement.
// precond = true makes the correction solves flexible GMRES with the learned preconditioner; a
// correction that leaves some right-hand side's residual no smaller than it started is redone without
// it, and a refinement step that fails to halve the FP64 residual turns the preconditioner off for the
// rest of the solve (both counted in `fallbacks`), so a poor preconditioner costs time, not the answer.
static GmresResult refine_mixed(Solver &S, const double2 *b, double2 *x, double rtol, int restart, int maxiter,
                                int &fp64_mv, int &fp32_mv, int &steps, bool block, bool precond, int &fallbacks,
                                bool df64) {
  sg_context *c = S.c;
  const int R = S.R;
  const size_t len = S.len();
  c->w_b.reserve(len);  // residual (rhs of the correction solve)
  c->w_x.reserve(len);  // correction
  double2 *rr = c->w_b.ptr, *d = c->w_x.ptr;
  std::vector<double2> hb(2 * R);
  GmresResult out;
  out.relres.assign(R, 0.0);
  out.conv.assign(R, 0);
  c->w_hcol.reserve((size_t)kHcol * R);
  c->w_red.reserve((size_t)4 * R + 4);
  double2 *dh = c->w_hcol.ptr;
  VecList L1{};
  L1.v[0] = b;
  S.dots(L1, 1, b, dh);
  SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
  SG_CUDA(cudaStreamSynchronize(S.st));
  std::vector<double> bnrm(R);
  for (int q = 0; q < R; ++q) bnrm[q] = std::sqrt(std::max(0.0, hb[q].x));
  std::vector<char> done(R, 0);
  std::vector<double> mask(R);
  const int max_steps = 40;
  const int inner_cap_cycles = std::max(4, 4000 / std::max(1, restart));  // <= ~4000 iterations per correction
  int inner_total = 0, no_progress = 0;
  double prev_worst = 0.0;
  L1.v[0] = x;
  S.dots(L1, 1, x, dh);
  SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
  SG_CUDA(cudaStreamSynchronize(S.st));
  bool x0_zero = true;
  for (int q = 0; q < R; ++q) x0_zero &= hb[q].x == 0.0;
  for (steps = 0; steps <= max_steps; ++steps) {
    // FP64 true residual (r = b exactly when x0 == 0)
    if (steps == 0 && x0_zero) {
      SG_CUDA(cudaMemcpyAsync(rr, b, len * sizeof(double2), cudaMemcpyDeviceToDevice, S.st));
    } else {
      S.master_true(x, rr, df64);
      fp64_mv++;
      sub_from_kernel<<<nblocks(len), 256, 0, S.st>>>(b, rr, len);
      SG_CUDA(cudaGetLastError());
    }
    L1.v[0] = rr;
    S.dots(L1, 1, rr, dh);
    SG_CUDA(cudaMemcpyAsync(hb.data(), dh, R * sizeof(double2), cudaMemcpyDeviceToHost, S.st));
    SG_CUDA(cudaStreamSynchronize(S.st));
    double worst = 0.0;
    std::vector<double> rn(R);
    for (int q = 0; q < R; ++q) {
      rn[q] = std::sqrt(std::max(0.0, hb[q].x));
      const double rel = bnrm[q] > 0 ? rn[q] / bnrm[q] : 0.0;
      out.relres[q] = rel;
      done[q] = rel <= rtol ? 1 : 0;
      out.conv[q] = done[q];
      if (!done[q]) worst = std::max(worst, rel);
    }
    if (worst == 0.0 || steps == max_steps || inner_total >= maxiter) break;
    // refinement must contract the FP64 residual; two steps without halving it end the solve
    if (steps > 0 && worst > 0.5 * prev_worst) {
      if (precond) {
        // the preconditioned corrections stopped contracting the FP64 residual: finish without them
        precond = false;
        fallbacks++;
      } else if (++no_progress >= 2) {
        break;
      }
    } else {
      no_progress = 0;
    }
    prev_worst = worst;
    // correction solve with the FP32 operator: tolerance relative to the current residual
    double tau = 0.3 * rtol / worst;
    tau = std::max(1e-6, std::min(0.5, tau));
    k_zero(d, len, S.st);
    const int cycles = std::max(1, std::min(inner_cap_cycles, (maxiter - inner_total) / restart + 1));
    GmresResult g;
    bool use_block = block && R > 1;
    if (use_block) {
      const int brestart = std::min(restart, 20);
      g = block_gmres(S, rr, d, tau, brestart, std::max(1, std::min(inner_cap_cycles, 200)), true, true, done);
      if (g.breakdown && g.inner_iters == 0) {
        k_zero(d, len, S.st);
        use_block = false;
      }
    }
    if (!use_block) {
      g = gmres_lockstep(S, rr, d, tau, restart, cycles, true, true, done, 2, precond);
      if (precond) {
        bool failed = false;
        for (int q = 0; q < R; ++q) failed |= !done[q] && !(g.relres[q] < 1.0);
        if (failed) {
          fallbacks++;
          fp32_mv += g.matvecs;
          inner_total += g.inner_iters;
          out.inner_iters += g.inner_iters;
          out.cycles += g.cycles;
          k_zero(d, len, S.st);
          g = gmres_lockstep(S, rr, d, tau, restart, cycles, true, true, done, 2, false);
        }
      }
    }
    fp32_mv += g.matvecs;
    inner_total += g.inner_iters;
    out.inner_iters += g.inner_iters;
    out.cycles += g.cycles;
    for (int q = 0; q < R; ++q) mask[q] = done[q] ? 0.0 : 1.0;
    dh = c->w_hcol.ptr;
    double *dm = c->w_red.ptr;
    SG_CUDA(cudaMemcpyAsync(dm, mask.data(), R * sizeof(double), cudaMemcpyHostToDevice, S.st));
    add_masked_kernel<<<nblocks(len), 256, 0, S.st>>>(x, d, dm, S.rows, R);
    SG_CUDA(cudaGetLastError());
  }
  return out;
}

// Public driver used by the C ABI: padded device vectors b, x (x holds x0).
void solve_padded(sg_context *c, const double2 *b, double2 *x, int R, double rtol, int restart, int maxiter,
                  int precision, sg_solve_info *info, cudaStream_t st) {
  Solver S{c, st, R, (size_t)c->n * c->bs, &c->launches};
  if (maxiter <= 0) maxiter = 10 * c->n_unknowns;
  if (restart <= 0) restart = 20;
  const auto t0 = std::chrono::steady_clock::now();
  cudaEvent_t ev0, ev1;
  SG_CUDA(cudaEventCreate(&ev0));
  SG_CUDA(cudaEventCreate(&ev1));
  SG_CUDA(cudaEventRecord(ev0, st));
  GmresResult g;
  int fp64_mv = 0, fp32_mv = 0, steps = 0, fallbacks = 0;
  if (precision & SG_FP32) {
    g = refine_mixed(S, b, x, rtol, restart, maxiter * restart, fp64_mv, fp32_mv, steps,
                     (precision & SG_BLOCK_GMRES) != 0, (precision & SG_PRECOND) != 0, fallbacks,
                     (precision & SG_DF64) != 0);
  } else {
    g = gmres_lockstep(S, b, x, rtol, restart, maxiter, false, false, std::vector<char>());
    fp64_mv = g.matvecs;
    steps = g.cycles;
  }
  SG_CUDA(cudaEventRecord(ev1, st));
  SG_CUDA(cudaStreamSynchronize(st));
  const auto t1 = std::chrono::steady_clock::now();
  float dev_ms = 0.f;
  SG_CUDA(cudaEventElapsedTime(&dev_ms, ev0, ev1));
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (info) {
    info->iterations = g.inner_iters;
    info->restarts = steps;
    info->fp64_matvecs = fp64_mv;
    info->fp32_matvecs = fp32_mv;
    int nc = 0;
    double mx = 0.0;
    for (int q = 0; q < R; ++q) {
      nc += g.conv[q] ? 1 : 0;
      mx = std::max(mx, g.relres[q]);
    }
    info->converged = nc;
    info->precond_fallbacks = fallbacks;
    info->max_rel_residual = mx;
    info->seconds = std::chrono::duration<double>(t1 - t0).count();
    info->device_seconds = dev_ms * 1e-3;
  }
}

// y = M x or W x on padded vectors (public matvec entry points)
// One CUDA-event-timed run of each FP32 kernel on the live operands; the faster one is cached per
// RHS count. Runs once per (context, nrhs) and synchronises the stream, so it must not be reached
// inside a stream capture.
static void launch_receiver_fp32(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st,
                                 int rt = 0) {
  CouplingLaunch L{};
  L.pos = c->pos.ptr;
  L.mofn = c->mofn.ptr;
  L.coef = c->coef32.ptr;
  L.pairs = c->pairs.ptr;
  L.n = c->n;
  L.bs = c->bs;
  L.n_int = c->n_int;
  L.ncoef = c->ncoef;
  L.rho_min = c->rho_min;
  L.res = c->res;
  L.x = x;
  const size_t len = (size_t)c->n * c->bs * R;
  c->bk_x32.reserve(len);
  k_to_f32(x, c->bk_x32.ptr, len, st);
  c->launches += 1;
  L.x32 = c->bk_x32.ptr;
  L.y = y;
  L.nrhs = R;
  L.rt = rt;
  L.master = master ? 1 : 0;
  L.t = c->tmat.ptr;
  L.ptype = c->ptype.ptr;
  L.t_diag = c->t_diag;
  const int ns = choose_split(c->n, R);
  if (ns > 1) {
    c->w_partial.reserve((size_t)ns * c->n * c->bs * R);
    L.partial = c->w_partial.ptr;
  }
  c->launches += launch_coupling(L, true, ns, st);
}

static int autotune_fp32(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  // candidates: the per-receiver kernel with the three largest RHS tiles that divide R (16 only for
  // the FP32 path), and the bucketed kernel when its plan exists; each is warmed once (first
  // launches carry one-time set-up) and timed once with CUDA events on the live operands
  std::vector<int> tiles;
  for (int rt : {16, 8, 4, 2, 1})
    if (R % rt == 0 && tiles.size() < 3) tiles.push_back(rt);
  cudaEvent_t e0, e1;
  SG_CUDA(cudaEventCreate(&e0));
  SG_CUDA(cudaEventCreate(&e1));
  auto time_it = [&](auto &&launch) {
    launch();
    SG_CUDA(cudaEventRecord(e0, st));
    launch();
    SG_CUDA(cudaEventRecord(e1, st));
    SG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    SG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    return ms;
  };
  float best_rec = -1.f;
  int best_rt = tiles.front();
  for (int rt : tiles) {
    const float ms = time_it([&] { launch_receiver_fp32(c, x, y, R, master, st, rt); });
    if (best_rec < 0.f || ms < best_rec) {
      best_rec = ms;
      best_rt = rt;
    }
  }
  float ms_bucket = -1.f;
  if (c->use_bucket) ms_bucket = time_it([&] { c->launches += launch_bucket_matvec(c, x, y, R, master, st); });
  // the pair-symmetric kernel at the two largest RHS tiles that divide R within its register budget,
  // with one warp per receiver and (tiles >= 4) with two
  float ms_sym = -1.f;
  int sym_rt = 0, sym_split = 1;
  if (sym_supported(c)) {
    int ntile = 0;
    for (int rt : {16, 8, 4, 2, 1}) {
      if (rt > sym_max_tile(c) || R % rt != 0 || ntile == 2) continue;
      ++ntile;
      for (int split : {1, 2}) {
        if (split == 2 && rt < 4) continue;
        const float ms = time_it([&] { c->launches += launch_sym_matvec(c, x, y, R, master, rt, split, st); });
        if (ms_sym < 0.f || ms < ms_sym) {
          ms_sym = ms;
          sym_rt = rt;
          sym_split = split;
        }
      }
    }
  }
  // the tensor-core operator (3xTF32, accumulators drained every few emitters)
  float ms_tc = -1.f, ms_tcs = -1.f;
  if (tc_supported(c, R)) ms_tc = time_it([&] { c->launches += launch_tc_matvec(c, x, y, R, master, st); });
  if (tcsym_supported(c, R))
    ms_tcs = time_it([&] { c->launches += launch_tcsym_matvec(c, x, y, R, master, st); });
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int v = 0;
  float best = best_rec;
  if (ms_bucket >= 0.f && ms_bucket < best) {
    v = 1;
    best = ms_bucket;
  }
  if (ms_sym >= 0.f && ms_sym < best) {
    v = sym_split == 2 ? 3 : 2;
    best = ms_sym;
  }
  if (ms_tc >= 0.f && ms_tc < best) {
    v = 4;
    best = ms_tc;
  }
  if (ms_tcs >= 0.f && ms_tcs < best) v = 5;
  c->tuned.push_back({R, v, best_rt, best_rec, ms_bucket, sym_rt, ms_sym, ms_tc, ms_tcs});
  return v;
}

void apply_padded(sg_context *c, const double2 *x, double2 *y, int R, bool master, bool fp32, cudaStream_t st) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->profiling) {
    SG_CUDA(cudaEventCreate(&e0));
    SG_CUDA(cudaEventCreate(&e1));
    SG_CUDA(cudaEventRecord(e0, st));
  }
  int variant = 0, rt = 0, sym_rt = 0;
  if (c->vol) {
    c->launches += launch_volume(c, x, y, R, master, fp32, st);
    variant = -1;
  } else if (fp32) {
    variant = -1;
    for (const auto &t : c->tuned)
      if (t.nrhs == R) {
        variant = t.variant;
        rt = t.rt;
        sym_rt = t.sym_rt;
      }
    if (variant < 0) {
      variant = autotune_fp32(c, x, y, R, master, st);
      rt = c->tuned.back().rt;
      sym_rt = c->tuned.back().sym_rt;
    }
  }
  if (variant == 5) {
    c->launches += launch_tcsym_matvec(c, x, y, R, master, st);
  } else if (variant == 4) {
    c->launches += launch_tc_matvec(c, x, y, R, master, st);
  } else if (variant == 2 || variant == 3) {
    c->launches += launch_sym_matvec(c, x, y, R, master, sym_rt, variant == 3 ? 2 : 1, st);
  } else if (variant == 1) {
    c->launches += launch_bucket_matvec(c, x, y, R, master, st);
  } else if (variant == 0) {
    CouplingLaunch L{};
    L.pos = c->pos.ptr;
    L.mofn = c->mofn.ptr;
    L.coef = fp32 ? (const void *)c->coef32.ptr : (const void *)c->coef64.ptr;
    L.pairs = fp32 ? c->pairs.ptr : nullptr;
    L.n = c->n;
    L.bs = c->bs;
    L.n_int = c->n_int;
    L.ncoef = c->ncoef;
    L.rho_min = c->rho_min;
    L.res = c->res;
    L.x = x;
    if (fp32) {  // one FP32 copy of the input instead of an FP64->FP32 conversion per pair
      const size_t len = (size_t)c->n * c->bs * R;
      c->bk_x32.reserve(len);
      k_to_f32(x, c->bk_x32.ptr, len, st);
      c->launches += 1;
      L.x32 = c->bk_x32.ptr;
      L.rt = rt;
    }
    L.y = y;
    L.nrhs = R;
    L.master = master ? 1 : 0;
    L.t = c->tmat.ptr;
    L.ptype = c->ptype.ptr;
    L.t_diag = c->t_diag;
    const int ns = choose_split(c->n, R);
    if (ns > 1) {
      c->w_partial.reserve((size_t)ns * c->n * c->bs * R);
      L.partial = c->w_partial.ptr;
    }
    c->launches += launch_coupling(L, fp32, ns, st);
  }
  if (c->profiling) {
    SG_CUDA(cudaEventRecord(e1, st));
    c->events.push_back({e0, e1, fp32 ? 1 : 0});
  }
}

static void launch_df64(sg_context *c, const double2 *x, double2 *y, int R, bool master, int rt, cudaStream_t st);

// The double-float kernel's RHS tile (4 or 8): chosen once per RHS count by timing both on the live
// operands (only when 8 divides R), then cached.
static int df64_tile(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  for (const auto &t : c->tuned_df)
    if (t.first == R) return t.second;
  int best = 0;
  if (R % 8 == 0) {
    cudaEvent_t e[4];
    for (auto &ev : e) SG_CUDA(cudaEventCreate(&ev));
    SG_CUDA(cudaEventRecord(e[0], st));
    launch_df64(c, x, y, R, master, 0, st);
    SG_CUDA(cudaEventRecord(e[1], st));
    SG_CUDA(cudaEventRecord(e[2], st));
    launch_df64(c, x, y, R, master, 8, st);
    SG_CUDA(cudaEventRecord(e[3], st));
    SG_CUDA(cudaEventSynchronize(e[3]));
    float m0 = 0.f, m1 = 0.f;
    SG_CUDA(cudaEventElapsedTime(&m0, e[0], e[1]));
    SG_CUDA(cudaEventElapsedTime(&m1, e[2], e[3]));
    for (auto &ev : e) cudaEventDestroy(ev);
    best = m1 < m0 ? 8 : 0;
  }
  c->tuned_df.push_back({R, best});
  return best;
}

void apply_padded_df64(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st) {
  const size_t ncoef_total = (size_t)c->n_int * c->ncoef * c->bs * c->bs;
  if (!c->df_ready) {
    c->coefdf.reserve(ncoef_total);
    build_coefficients_df64(c->coef64.ptr, c->coefdf.ptr, ncoef_total, st);
    c->launches += 1;
    c->df_ready = true;
  }
  const int rt = df64_tile(c, x, y, R, master, st);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->profiling) {
    SG_CUDA(cudaEventCreate(&e0));
    SG_CUDA(cudaEventCreate(&e1));
    SG_CUDA(cudaEventRecord(e0, st));
  }
  launch_df64(c, x, y, R, master, rt, st);
  if (c->profiling) {
    SG_CUDA(cudaEventRecord(e1, st));
    c->events.push_back({e0, e1, 2});
  }
}

static void launch_df64(sg_context *c, const double2 *x, double2 *y, int R, bool master, int rt, cudaStream_t st) {
  CouplingLaunch L{};
  L.rt = rt;
  L.pos = c->pos.ptr;
  L.mofn = c->mofn.ptr;
  L.coef = c->coefdf.ptr;
  L.pairs = nullptr;
  L.n = c->n;
  L.bs = c->bs;
  L.n_int = c->n_int;
  L.ncoef = c->ncoef;
  L.rho_min = c->rho_min;
  L.res = c->res;
  L.x = x;
  const size_t len = (size_t)c->n * c->bs * R;
  c->xdf.reserve(len);
  k_to_df64(x, c->xdf.ptr, len, st);
  c->launches += 1;
  L.xdf = c->xdf.ptr;
  L.y = y;
  L.nrhs = R;
  L.master = master ? 1 : 0;
  L.t = c->tmat.ptr;
  L.ptype = c->ptype.ptr;
  L.t_diag = c->t_diag;
  const int ns = choose_split(c->n, R);
  if (ns > 1) {
    c->w_partial.reserve((size_t)ns * c->n * c->bs * R);
    L.partial = c->w_partial.ptr;
  }
  c->launches += launch_coupling_df64(L, ns, st);
}

}  // namespace sg

namespace sg {

__global__ void residual_kernel_sub(const double2 *b, double2 *r, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) r[e] = make_double2(b[e].x - r[e].x, b[e].y - r[e].y);
}

// rel[q] = ||b_q - M x_q|| / ||b_q|| with the FP64 operator (padded device vectors)
void residual_norms(sg_context *c, const double2 *b, const double2 *x, int R, double *rel, cudaStream_t st) {
  Solver S{c, st, R, (size_t)c->n * c->bs, &c->launches};
  const size_t len = S.len();
  c->w_r.reserve(len);
  c->w_hcol.reserve((size_t)kHcol * R);
  S.master(x, c->w_r.ptr, false);
  residual_kernel_sub<<<nblocks(len), 256, 0, st>>>(b, c->w_r.ptr, len);
  SG_CUDA(cudaGetLastError());
  VecList L{};
  L.v[0] = b;
  L.v[1] = c->w_r.ptr;
  S.dots(L, 1, b, c->w_hcol.ptr);
  VecList L2{};
  L2.v[0] = c->w_r.ptr;
  S.dots(L2, 1, c->w_r.ptr, c->w_hcol.ptr + R);
  std::vector<double2> h(2 * R);
  SG_CUDA(cudaMemcpyAsync(h.data(), c->w_hcol.ptr, 2 * R * sizeof(double2), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  for (int q = 0; q < R; ++q) {
    const double bn = std::sqrt(std::max(0.0, h[q].x)), rn = std::sqrt(std::max(0.0, h[R + q].x));
    rel[q] = bn > 0 ? rn / bn : rn;
  }
}

}  // namespace sg

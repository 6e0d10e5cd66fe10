// Learned right preconditioner: a message-passing network over each particle's k nearest
// neighbours, with hand-written forward, backward and Adam kernels (BF16 weights, FP32 math).
//
// Graph: slot 0 of every particle is the particle itself, slots 1..k its k nearest neighbours.
// Messages use the physical near-field coupling G[i][s] = T_i W_{i, nbr(i,s)} (B x B complex,
// interpolated from the lookup coefficients), so that with zero output weights and alpha = 1 the
// network is the 3-term Neumann series of the near-field operator, (I - T W_near)^{-1} ~ I + A + A^2 + A^3.
//
// For a batch of S vectors v (padded layout [N][B][S], complex):
//   s_q = ||v_q||,  u = v / s,  h_0 = u
//   layer l = 0..2:  a = A h_l                (A h)_i = sum_s G[i][s] h_{nbr(i,s)}
//                    f = [Re a, Im a, Re h_l, Im h_l]       (4B features per (particle, sample))
//                    p = W1 f + b1 (128 wide),  g = W2 relu(p) + b2 (2B wide)
//                    h_{l+1} = u + alpha_l a + g            (alpha_l complex, g read as [re | im])
//   z = s * h_3
// Parameters (one flat FP32 vector), per layer: W1[128][4B], b1[128], W2[2B][128], b2[2B],
// alpha[2] (re, im). Forward and backward use BF16 copies of W1 and W2; Adam updates the FP32
// master copy. Training loss per sample: ||h_3 - e/s||^2 / ||e/s||^2 (mean over the batch), where
// e = M^{-1} v is the target.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sg_internal.h"

namespace sg {

static constexpr int kHid = 128;
static constexpr int kLayers = 3;     // the default network depth (sg_precond_param_count)
static constexpr int kMaxLayers = 8;  // deeper networks: the parameter count sets the depth

static int per_layer_count(int bs) {
  const int F = 4 * bs, O = 2 * bs;
  return kHid * F + kHid + O * kHid + O + 2;
}

int precond_param_count(int bs) { return kLayers * per_layer_count(bs); }

// layers of a parameter vector of `count` floats (0 when the count fits no depth 1..kMaxLayers)
int precond_layers(int bs, int count) {
  const int per = per_layer_count(bs);
  if (count <= 0 || count % per != 0 || count / per > kMaxLayers) return 0;
  return count / per;
}

struct LayerOff {
  size_t w1, b1, w2, b2, al;
};
static LayerOff layer_offsets(int bs, int l) {
  const int F = 4 * bs, O = 2 * bs;
  const size_t per = (size_t)kHid * F + kHid + (size_t)O * kHid + O + 2;
  LayerOff o;
  o.w1 = per * l;
  o.b1 = o.w1 + (size_t)kHid * F;
  o.w2 = o.b1 + kHid;
  o.b2 = o.w2 + (size_t)O * kHid;
  o.al = o.b2 + O;
  return o;
}

static inline unsigned nb(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------------ graph blocks
// G[e][n1][n2] = T_i[n1] e^{-i m1 phi} L_{n1 n2}(rho) e^{i m2 phi}, edge e = i*k1 + s, j = nbr[e]
__global__ void pc_blocks_kernel(const double2 *pos, const int *mofn, const double2 *coef, int ncoef, int n_int,
                                 double rho_min, double res, int bs, int k1, const int *nbr, const double2 *tdiag,
                                 const int *ptype, float2 *G) {
  const int e = blockIdx.x;
  const int i = e / k1;
  const int j = nbr[e];
  __shared__ double ph_re[33], ph_im[33];
  __shared__ int sk;
  __shared__ double st;
  if (threadIdx.x == 0) {
    const double dx = pos[i].x - pos[j].x, dy = pos[i].y - pos[j].y;
    const double rho = sqrt(dx * dx + dy * dy);
    const double sidx = (rho - rho_min) / res;
    int k = (int)floor(sidx);
    k = k < 0 ? 0 : (k > n_int - 1 ? n_int - 1 : k);
    sk = k;
    st = sidx - (double)k;
    double c = 1.0, s = 0.0;
    if (rho > 0.0) {
      c = dx / rho;
      s = dy / rho;
    }
    double pr = 1.0, pi = 0.0;
    ph_re[16] = 1.0;
    ph_im[16] = 0.0;
    for (int m = 1; m <= 16; ++m) {
      const double nr = pr * c - pi * s;
      pi = pr * s + pi * c;
      pr = nr;
      ph_re[16 + m] = pr;
      ph_im[16 + m] = pi;
      ph_re[16 - m] = pr;
      ph_im[16 - m] = -pi;
    }
  }
  __syncthreads();
  const size_t bs2 = (size_t)bs * bs;
  const double t = st;
  const double2 *cb = coef + (size_t)sk * ncoef * bs2;
  const double2 *tv = tdiag + (size_t)ptype[i] * bs;
  for (int el = threadIdx.x; el < bs * bs; el += blockDim.x) {
    const int n1 = el / bs, n2 = el - n1 * bs;
    const size_t off = (size_t)n2 * bs + n1;  // coefficients are stored [c][n2][n1]
    double lr = cb[(ncoef - 1) * bs2 + off].x, li = cb[(ncoef - 1) * bs2 + off].y;
    for (int c = ncoef - 2; c >= 0; --c) {
      lr = fma(lr, t, cb[c * bs2 + off].x);
      li = fma(li, t, cb[c * bs2 + off].y);
    }
    // e^{i (m2 - m1) phi} = e^{i m2 phi} e^{-i m1 phi}  (|m| <= 16)
    const double ar = ph_re[16 + mofn[n2]], ai = ph_im[16 + mofn[n2]];
    const double br = ph_re[16 + mofn[n1]], bi = -ph_im[16 + mofn[n1]];
    const double er = ar * br - ai * bi, ei = ar * bi + ai * br;
    const double wr = lr * er - li * ei, wi = lr * ei + li * er;
    const double2 tt = tv[n1];
    G[(size_t)e * bs2 + (size_t)n1 * bs + n2] =
        make_float2((float)(tt.x * wr - tt.y * wi), (float)(tt.x * wi + tt.y * wr));
  }
}

// out[i][n1][q] = sum_s sum_n2 G[i*k1+s][n1][n2] in[nbr(i,s)][n2][q]
__global__ void pc_apply_kernel(const float2 *G, const int *nbr, int k1, int bs, int S, const float2 *in, float2 *out) {
  const int i = blockIdx.x;
  const size_t bs2 = (size_t)bs * bs;
  for (int t = threadIdx.x; t < bs * S; t += blockDim.x) {
    const int n1 = t / S, q = t - n1 * S;
    float ar = 0.f, ai = 0.f;
    for (int s = 0; s < k1; ++s) {
      const int j = nbr[i * k1 + s];
      const float2 *g = G + (size_t)(i * k1 + s) * bs2 + (size_t)n1 * bs;
      const float2 *x = in + (size_t)j * bs * S + q;
      for (int n2 = 0; n2 < bs; ++n2) {
        const float2 gv = g[n2], xv = x[(size_t)n2 * S];
        ar = fmaf(gv.x, xv.x, fmaf(-gv.y, xv.y, ar));
        ai = fmaf(gv.x, xv.y, fmaf(gv.y, xv.x, ai));
      }
    }
    out[((size_t)i * bs + n1) * S + q] = make_float2(ar, ai);
  }
}

// out[j][n2][q] = sum_{(i,s): nbr(i,s) = j} sum_n1 conj(G[i*k1+s][n1][n2]) in[i][n1][q]
__global__ void pc_adjoint_kernel(const float2 *G, const int *rev_off, const int *rev_idx, int k1, int bs, int S,
                                  const float2 *in, float2 *out) {
  const int j = blockIdx.x;
  const size_t bs2 = (size_t)bs * bs;
  for (int t = threadIdx.x; t < bs * S; t += blockDim.x) {
    const int n2 = t / S, q = t - n2 * S;
    float ar = 0.f, ai = 0.f;
    for (int r = rev_off[j]; r < rev_off[j + 1]; ++r) {
      const int e = rev_idx[r];
      const int i = e / k1;
      const float2 *g = G + (size_t)e * bs2 + n2;
      const float2 *y = in + (size_t)i * bs * S + q;
      for (int n1 = 0; n1 < bs; ++n1) {
        const float2 gv = g[(size_t)n1 * bs], yv = y[(size_t)n1 * S];
        ar = fmaf(gv.x, yv.x, fmaf(gv.y, yv.y, ar));
        ai = fmaf(gv.x, yv.y, fmaf(-gv.y, yv.x, ai));
      }
    }
    out[((size_t)j * bs + n2) * S + q] = make_float2(ar, ai);
  }
}

// out[q] += sum_rows |v[row][q]|^2 (FP32 vectors [rows][S], len = rows * S elements)
__global__ void pc_sqnorm_kernel(const float2 *v, size_t len, int S, float *out) {
  extern __shared__ float sh[];
  for (int q = threadIdx.x; q < S; q += blockDim.x) sh[q] = 0.f;
  __syncthreads();
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (size_t)gridDim.x * blockDim.x) {
    const float2 x = v[e];
    atomicAdd(&sh[e % S], x.x * x.x + x.y * x.y);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < S; q += blockDim.x) atomicAdd(&out[q], sh[q]);
}

__global__ void pc_f64_to_f32_kernel(const double2 *v, float2 *y, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) y[e] = make_float2((float)v[e].x, (float)v[e].y);
}

__global__ void pc_scale_kernel(const float2 *x, float2 *y, size_t len, int S, const float *sq) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  const float s = sqrtf(sq[e % S]);
  const float inv = s > 0.f ? 1.f / s : 0.f;
  y[e] = make_float2(x[e].x * inv, x[e].y * inv);
}

__global__ void pc_from_f32_scaled(const float2 *h, double2 *z, size_t len, int S, const float *sq) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  const double s = sqrt((double)sq[e % S]);
  z[e] = make_double2((double)h[e].x * s, (double)h[e].y * s);
}

__global__ void pc_to_bf16(const float *src, __nv_bfloat16 *dst, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) dst[e] = __float2bfloat16(src[e]);
}

// feature k of (particle i, sample q) from a and h ([N][B][S] complex FP32)
__device__ __forceinline__ float pc_feature(const float2 *a, const float2 *h, int i, int q, int k, int bs, int S) {
  const int part = k / bs, n = k - part * bs;
  const size_t idx = ((size_t)i * bs + n) * S + q;
  switch (part) {
    case 0: return a[idx].x;
    case 1: return a[idx].y;
    case 2: return h[idx].x;
    default: return h[idx].y;
  }
}

// p[row][hid] = b1 + W1 f(row), row = i*S + q; a block of kHid threads handles 8 rows
__global__ void pc_mlp1_kernel(const float2 *a, const float2 *h, const __nv_bfloat16 *W1, const float *b1, int n, int bs,
                               int S, float *p) {
  extern __shared__ float fs[];  // [8][4B]
  const int F = 4 * bs;
  const size_t rows = (size_t)n * S;
  const size_t r0 = (size_t)blockIdx.x * 8;
  for (int t = threadIdx.x; t < 8 * F; t += blockDim.x) {
    const int rr = t / F, k = t - rr * F;
    const size_t row = r0 + rr;
    fs[t] = row < rows ? pc_feature(a, h, (int)(row / S), (int)(row % S), k, bs, S) : 0.f;
  }
  __syncthreads();
  const int hid = threadIdx.x;
  float acc[8];
  for (int rr = 0; rr < 8; ++rr) acc[rr] = b1[hid];
  const __nv_bfloat16 *w = W1 + (size_t)hid * F;
  for (int k = 0; k < F; ++k) {
    const float wv = __bfloat162float(w[k]);
    for (int rr = 0; rr < 8; ++rr) acc[rr] = fmaf(wv, fs[rr * F + k], acc[rr]);
  }
  for (int rr = 0; rr < 8; ++rr)
    if (r0 + rr < rows) p[(r0 + rr) * kHid + hid] = acc[rr];
}

// g = b2 + W2 relu(p); h_out = u + alpha a + g; a block of 2B threads handles 8 rows
__global__ void pc_mlp2_kernel(const float *p, const __nv_bfloat16 *W2, const float *b2, const float *alpha,
                               const float2 *u, const float2 *a, int n, int bs, int S, float2 *hout) {
  __shared__ float qs[8][kHid];
  const size_t rows = (size_t)n * S;
  const size_t r0 = (size_t)blockIdx.x * 8;
  for (int t = threadIdx.x; t < 8 * kHid; t += blockDim.x) {
    const int rr = t / kHid, hh = t - rr * kHid;
    qs[rr][hh] = (r0 + rr < rows) ? fmaxf(p[(r0 + rr) * kHid + hh], 0.f) : 0.f;
  }
  __syncthreads();
  const int o = threadIdx.x;
  if (o >= 2 * bs) return;
  const __nv_bfloat16 *w = W2 + (size_t)o * kHid;
  float acc[8];
  for (int rr = 0; rr < 8; ++rr) acc[rr] = b2[o];
  for (int hh = 0; hh < kHid; ++hh) {
    const float wv = __bfloat162float(w[hh]);
    for (int rr = 0; rr < 8; ++rr) acc[rr] = fmaf(wv, qs[rr][hh], acc[rr]);
  }
  const int nrow = o < bs ? o : o - bs;
  const float alr = alpha[0], ali = alpha[1];
  for (int rr = 0; rr < 8; ++rr) {
    const size_t row = r0 + rr;
    if (row >= rows) break;
    const int i = (int)(row / S), q = (int)(row % S);
    const size_t idx = ((size_t)i * bs + nrow) * S + q;
    const float2 av = a[idx], uv = u[idx];
    if (o < bs) hout[idx].x = uv.x + alr * av.x - ali * av.y + acc[rr];
    else hout[idx].y = uv.y + alr * av.y + ali * av.x + acc[rr];
  }
}

// loss += sum_q ||h3 - e/s||^2 / (||e/s||^2 S);  dh = 2 (h3 - e/s) / (||e/s||^2 S)
__global__ void pc_loss_kernel(const float2 *h3, const double2 *e, const float *sq_v, const float *sq_e, size_t len,
                               int S, float2 *dh, float *loss) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  float contrib = 0.f;
  if (idx < len) {
    const int q = (int)(idx % S);
    const float s = sqrtf(sq_v[q]);
    const float inv = s > 0.f ? 1.f / s : 0.f;
    const float en2 = sq_e[q] * inv * inv;
    const float w = en2 > 0.f ? 1.f / (en2 * S) : 0.f;
    const float dr = h3[idx].x - (float)e[idx].x * inv, di = h3[idx].y - (float)e[idx].y * inv;
    contrib = (dr * dr + di * di) * w;
    dh[idx] = make_float2(2.f * dr * w, 2.f * di * w);
  }
  __shared__ float red[256];
  red[threadIdx.x] = contrib;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if (threadIdx.x < s2) red[threadIdx.x] += red[threadIdx.x + s2];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// dalpha += sum conj(a) dh (complex); da = conj(alpha) dh
__global__ void pc_alpha_back_kernel(const float2 *a, const float2 *dh, const float *alpha, size_t len, float2 *da,
                                     float *dalpha) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  float gr = 0.f, gi = 0.f;
  if (e < len) {
    const float2 av = a[e], d = dh[e];
    gr = av.x * d.x + av.y * d.y;
    gi = av.x * d.y - av.y * d.x;
    da[e] = make_float2(alpha[0] * d.x + alpha[1] * d.y, alpha[0] * d.y - alpha[1] * d.x);
  }
  __shared__ float r0[256], r1[256];
  r0[threadIdx.x] = gr;
  r1[threadIdx.x] = gi;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if (threadIdx.x < s2) {
      r0[threadIdx.x] += r0[threadIdx.x + s2];
      r1[threadIdx.x] += r1[threadIdx.x + s2];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&dalpha[0], r0[0]);
    atomicAdd(&dalpha[1], r1[0]);
  }
}

// dg[row][o] from dh; dp[row][hid] = (sum_o W2[o][hid] dg) * (p > 0); kHid threads, 8 rows per block
__global__ void pc_mlp2_back_kernel(const float2 *dh, const float *p, const __nv_bfloat16 *W2, int n, int bs, int S,
                                    float *dg, float *dp) {
  __shared__ float gs[8][128];
  const int O = 2 * bs;
  const size_t rows = (size_t)n * S;
  const size_t r0 = (size_t)blockIdx.x * 8;
  for (int t = threadIdx.x; t < 8 * O; t += blockDim.x) {
    const int rr = t / O, o = t - rr * O;
    const size_t row = r0 + rr;
    float v = 0.f;
    if (row < rows) {
      const int i = (int)(row / S), q = (int)(row % S);
      const int nrow = o < bs ? o : o - bs;
      const float2 d = dh[((size_t)i * bs + nrow) * S + q];
      v = o < bs ? d.x : d.y;
      dg[row * O + o] = v;
    }
    gs[rr][o] = v;
  }
  __syncthreads();
  const int hid = threadIdx.x;
  for (int rr = 0; rr < 8; ++rr) {
    const size_t row = r0 + rr;
    if (row >= rows) break;
    float acc = 0.f;
    for (int o = 0; o < O; ++o) acc = fmaf(__bfloat162float(W2[(size_t)o * kHid + hid]), gs[rr][o], acc);
    dp[row * kHid + hid] = p[row * kHid + hid] > 0.f ? acc : 0.f;
  }
}

// df = W1^T dp per row; the a part is added into da, the h part written to dh_prev
__global__ void pc_mlp1_back_kernel(const float *dp, const __nv_bfloat16 *W1, int n, int bs, int S, float2 *da,
                                    float2 *dh_prev) {
  __shared__ float ps[8][kHid];
  const int F = 4 * bs;
  const size_t rows = (size_t)n * S;
  const size_t r0 = (size_t)blockIdx.x * 8;
  for (int t = threadIdx.x; t < 8 * kHid; t += blockDim.x) {
    const int rr = t / kHid, hh = t - rr * kHid;
    ps[rr][hh] = (r0 + rr < rows) ? dp[(r0 + rr) * kHid + hh] : 0.f;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < F; k += blockDim.x) {
    float acc[8];
    for (int rr = 0; rr < 8; ++rr) acc[rr] = 0.f;
    for (int hh = 0; hh < kHid; ++hh) {
      const float wv = __bfloat162float(W1[(size_t)hh * F + k]);
      for (int rr = 0; rr < 8; ++rr) acc[rr] = fmaf(wv, ps[rr][hh], acc[rr]);
    }
    const int part = k / bs, nn = k - part * bs;
    for (int rr = 0; rr < 8; ++rr) {
      const size_t row = r0 + rr;
      if (row >= rows) break;
      const int i = (int)(row / S), q = (int)(row % S);
      const size_t idx = ((size_t)i * bs + nn) * S + q;
      switch (part) {
        case 0: da[idx].x += acc[rr]; break;
        case 1: da[idx].y += acc[rr]; break;
        case 2: dh_prev[idx].x = acc[rr]; break;
        default: dh_prev[idx].y = acc[rr]; break;
      }
    }
  }
}

// dW2[o][hid] += sum_rows dg[row][o] relu(p[row][hid]); db2[o] += sum_rows dg[row][o]
__global__ void pc_wgrad2_kernel(const float *dg, const float *p, size_t rows, int O, float *dW2, float *db2) {
  const int o = blockIdx.x;
  const int hid = threadIdx.x;
  float acc = 0.f, accb = 0.f;
  for (size_t row = 0; row < rows; ++row) {
    const float d = dg[row * O + o];
    acc = fmaf(d, fmaxf(p[row * kHid + hid], 0.f), acc);
    accb += d;
  }
  dW2[(size_t)o * kHid + hid] += acc;
  if (hid == 0) db2[o] += accb;
}

// dW1[hid][k] += sum_rows dp[row][hid] f(row, k); db1[hid] += sum_rows dp[row][hid]
__global__ void pc_wgrad1_kernel(const float *dp, const float2 *a, const float2 *h, size_t rows, int bs, int S,
                                 float *dW1, float *db1) {
  const int hid = blockIdx.x;
  const int F = 4 * bs;
  for (int k = threadIdx.x; k < F; k += blockDim.x) {
    float acc = 0.f, accb = 0.f;
    for (size_t row = 0; row < rows; ++row) {
      const float d = dp[row * kHid + hid];
      acc = fmaf(d, pc_feature(a, h, (int)(row / S), (int)(row % S), k, bs, S), acc);
      accb += d;
    }
    dW1[(size_t)hid * F + k] += acc;
    if (k == 0) db1[hid] += accb;
  }
}

__global__ void pc_add_kernel(float2 *dst, const float2 *src, size_t n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) {
    dst[e].x += src[e].x;
    dst[e].y += src[e].y;
  }
}

__global__ void pc_adam_kernel(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
                               float eps, float c1, float c2) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float gg = g[e];
  m[e] = b1 * m[e] + (1.f - b1) * gg;
  v[e] = b2 * v[e] + (1.f - b2) * gg * gg;
  w[e] -= lr * (m[e] / c1) / (sqrtf(v[e] / c2) + eps);
}

// ------------------------------------------------------------------ host side
void precond_add_graph(sg_context *c, int k, const int *nbr_host, int *graph_id, cudaStream_t st) {
  SG_REQUIRE(c->t_ready && c->t_diag, "the learned preconditioner needs diagonal T-matrices (sg_set_tmatrix)");
  SG_REQUIRE(c->kind >= 0, "sg_set_lookup must precede the preconditioner graph");
  SG_REQUIRE(!c->vol, "the learned preconditioner needs a radial lookup (particles at one height)");
  SG_REQUIRE(k >= 0 && k <= 64, "k must be in [0, 64]");
  SG_REQUIRE(c->bs <= 64, "the learned preconditioner supports blocksize <= 64");
  SG_REQUIRE(c->uniform, "the learned preconditioner works on uniform particle blocks");
  const int n = c->n, k1 = k + 1, bs = c->bs;
  for (size_t e = 0; e < (size_t)n * k1; ++e)
    SG_REQUIRE(nbr_host[e] >= 0 && nbr_host[e] < n, "neighbour index out of range");
  for (int i = 0; i < n; ++i) SG_REQUIRE(nbr_host[(size_t)i * k1] == i, "slot 0 of every particle must be itself");
  auto g = std::make_unique<sg_context::PGraph>();
  g->n = n;
  g->bs = bs;
  g->k1 = k1;
  g->nbr.reserve((size_t)n * k1);
  SG_CUDA(cudaMemcpyAsync(g->nbr.ptr, nbr_host, (size_t)n * k1 * sizeof(int), cudaMemcpyHostToDevice, st));
  // reverse adjacency (edges ending at each particle) for the adjoint
  std::vector<int> cnt(n + 1, 0), idx((size_t)n * k1);
  for (size_t e = 0; e < (size_t)n * k1; ++e) cnt[nbr_host[e] + 1]++;
  for (int j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (size_t e = 0; e < (size_t)n * k1; ++e) idx[fill[nbr_host[e]]++] = (int)e;
  g->rev_off.reserve(n + 1);
  g->rev_idx.reserve((size_t)n * k1);
  SG_CUDA(cudaMemcpyAsync(g->rev_off.ptr, cnt.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  SG_CUDA(cudaMemcpyAsync(g->rev_idx.ptr, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  g->G.reserve((size_t)n * k1 * bs * bs);
  pc_blocks_kernel<<<(unsigned)((size_t)n * k1), 256, 0, st>>>(c->pos.ptr, c->mofn.ptr, c->coef64.ptr, c->ncoef,
                                                               c->n_int, c->rho_min, c->res, bs, k1, g->nbr.ptr,
                                                               c->tmat.ptr, c->ptype.ptr, g->G.ptr);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));  // host staging vectors are released on return
  c->launches += 1;
  c->pgraphs.push_back(std::move(g));
  *graph_id = (int)c->pgraphs.size() - 1;
}

void precond_set_params(sg_context *c, int bs, const float *params, int count, cudaStream_t st) {
  SG_REQUIRE(bs >= 1 && bs <= 64 && precond_layers(bs, count) > 0,
             "parameter count does not match a network of 1..8 layers for this blocksize");
  c->p_w.reserve(count);
  c->p_wb.reserve(count);
  c->p_g.reserve(count);
  c->p_m.reserve(count);
  c->p_v.reserve(count);
  SG_CUDA(cudaMemcpyAsync(c->p_w.ptr, params, count * sizeof(float), cudaMemcpyHostToDevice, st));
  SG_CUDA(cudaMemsetAsync(c->p_m.ptr, 0, count * sizeof(float), st));
  SG_CUDA(cudaMemsetAsync(c->p_v.ptr, 0, count * sizeof(float), st));
  pc_to_bf16<<<nb(count), 256, 0, st>>>(c->p_w.ptr, c->p_wb.ptr, count);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaStreamSynchronize(st));
  c->p_bs = bs;
  c->p_count = count;
  c->p_layers = precond_layers(bs, count);
  c->launches += 1;
}

struct Fwd {
  float2 *u, *a[kMaxLayers], *h[kMaxLayers + 1];
  float *p[kMaxLayers];
  float *sq;
};

// Forward pass of a batch of S vectors on graph g (double2 input, padded [N][B][S]); keeps the
// activations the backward pass needs.
static void forward(sg_context *c, const sg_context::PGraph &g, const double2 *v, int S, Fwd &f, cudaStream_t st) {
  SG_REQUIRE(S >= 1 && S <= 64, "the preconditioner handles 1..64 vectors per call");
  SG_REQUIRE(c->p_layers > 0 && c->p_bs == g.bs, "preconditioner parameters are not set for this blocksize");
  const int nl = c->p_layers;
  const int n = g.n, bs = g.bs;
  const size_t len = (size_t)n * bs * S, rows = (size_t)n * S;
  c->p_act.reserve(len * 2 * (2 * nl + 2) + rows * kHid * nl + 64);
  float *base = c->p_act.ptr;
  size_t off = 0;
  f.u = reinterpret_cast<float2 *>(base + off);
  off += len * 2;
  for (int l = 0; l < nl; ++l) {
    f.a[l] = reinterpret_cast<float2 *>(base + off);
    off += len * 2;
  }
  for (int l = 0; l <= nl; ++l) {
    f.h[l] = reinterpret_cast<float2 *>(base + off);
    off += len * 2;
  }
  for (int l = 0; l < nl; ++l) {
    f.p[l] = base + off;
    off += rows * kHid;
  }
  f.sq = base + off;
  c->p_tmp.reserve(len);
  float2 *vf = c->p_tmp.ptr;
  SG_CUDA(cudaMemsetAsync(f.sq, 0, 64 * sizeof(float), st));
  pc_f64_to_f32_kernel<<<nb(len), 256, 0, st>>>(v, vf, len);
  pc_sqnorm_kernel<<<std::min<unsigned>(nb(len), 1024), 256, S * sizeof(float), st>>>(vf, len, S, f.sq);
  pc_scale_kernel<<<nb(len), 256, 0, st>>>(vf, f.u, len, S, f.sq);
  SG_CUDA(cudaGetLastError());
  SG_CUDA(cudaMemcpyAsync(f.h[0], f.u, len * sizeof(float2), cudaMemcpyDeviceToDevice, st));
  for (int l = 0; l < nl; ++l) {
    const LayerOff o = layer_offsets(bs, l);
    pc_apply_kernel<<<n, 256, 0, st>>>(g.G.ptr, g.nbr.ptr, g.k1, bs, S, f.h[l], f.a[l]);
    pc_mlp1_kernel<<<nb(rows, 8), kHid, 8 * 4 * bs * sizeof(float), st>>>(f.a[l], f.h[l], c->p_wb.ptr + o.w1,
                                                                            c->p_w.ptr + o.b1, n, bs, S, f.p[l]);
    pc_mlp2_kernel<<<nb(rows, 8), 2 * bs, 0, st>>>(f.p[l], c->p_wb.ptr + o.w2, c->p_w.ptr + o.b2, c->p_w.ptr + o.al,
                                                   f.u, f.a[l], n, bs, S, f.h[l + 1]);
    SG_CUDA(cudaGetLastError());
  }
  c->launches += 3 + 3 * nl;
}

// z = P(v) with the selected graph (double2 vectors, padded [N][B][S])
void precond_apply(sg_context *c, const double2 *v, double2 *z, int S, cudaStream_t st) {
  SG_REQUIRE(c->p_active >= 0 && c->p_active < (int)c->pgraphs.size(), "no preconditioner graph selected");
  const sg_context::PGraph &g = *c->pgraphs[c->p_active];
  SG_REQUIRE(g.n == c->n && g.bs == c->bs, "the selected preconditioner graph does not match the particles");
  Fwd f;
  forward(c, g, v, S, f, st);
  const int nl = c->p_layers;
  const size_t rows = (size_t)g.n * S, len = rows * g.bs;
  pc_from_f32_scaled<<<nb(len), 256, 0, st>>>(f.h[nl], z, len, S, f.sq);
  SG_CUDA(cudaGetLastError());
  c->launches += 1;
}

// One training step on graph gid: forward, loss, backward; an Adam update when lr > 0.
void precond_train(sg_context *c, int gid, const double2 *v, const double2 *e, int S, float lr, int step,
                   double *loss_out, float *grad_host, cudaStream_t st) {
  SG_REQUIRE(gid >= 0 && gid < (int)c->pgraphs.size(), "bad preconditioner graph id");
  const sg_context::PGraph &g = *c->pgraphs[gid];
  const int n = g.n, bs = g.bs, O = 2 * bs;
  const size_t rows = (size_t)n * S, len = rows * bs;
  Fwd f;
  forward(c, g, v, S, f, st);
  const int nl = c->p_layers;
  // dh, da, dhp, tmp (float2 x len each), dg (rows x O), dp (rows x kHid), sq_e (64), loss (1)
  c->p_back.reserve(len * 2 * 4 + rows * O + rows * kHid + 128);
  float *b = c->p_back.ptr;
  float2 *dh = reinterpret_cast<float2 *>(b), *da = dh + len, *dhp = da + len, *tmp = dhp + len;
  float *dg = b + len * 8, *dp = dg + rows * O, *sq_e = dp + rows * kHid, *loss = sq_e + 64;
  SG_CUDA(cudaMemsetAsync(sq_e, 0, 65 * sizeof(float), st));
  pc_f64_to_f32_kernel<<<nb(len), 256, 0, st>>>(e, tmp, len);
  pc_sqnorm_kernel<<<std::min<unsigned>(nb(len), 1024), 256, S * sizeof(float), st>>>(tmp, len, S, sq_e);
  pc_loss_kernel<<<nb(len), 256, 0, st>>>(f.h[nl], e, f.sq, sq_e, len, S, dh, loss);
  SG_CUDA(cudaGetLastError());
  const int count = c->p_count;
  SG_CUDA(cudaMemsetAsync(c->p_g.ptr, 0, count * sizeof(float), st));
  for (int l = nl - 1; l >= 0; --l) {
    const LayerOff o = layer_offsets(bs, l);
    pc_alpha_back_kernel<<<nb(len), 256, 0, st>>>(f.a[l], dh, c->p_w.ptr + o.al, len, da, c->p_g.ptr + o.al);
    pc_mlp2_back_kernel<<<nb(rows, 8), kHid, 0, st>>>(dh, f.p[l], c->p_wb.ptr + o.w2, n, bs, S, dg, dp);
    pc_wgrad2_kernel<<<O, kHid, 0, st>>>(dg, f.p[l], rows, O, c->p_g.ptr + o.w2, c->p_g.ptr + o.b2);
    pc_wgrad1_kernel<<<kHid, 128, 0, st>>>(dp, f.a[l], f.h[l], rows, bs, S, c->p_g.ptr + o.w1, c->p_g.ptr + o.b1);
    pc_mlp1_back_kernel<<<nb(rows, 8), 128, 0, st>>>(dp, c->p_wb.ptr + o.w1, n, bs, S, da, dhp);
    pc_adjoint_kernel<<<n, 256, 0, st>>>(g.G.ptr, g.rev_off.ptr, g.rev_idx.ptr, g.k1, bs, S, da, tmp);
    pc_add_kernel<<<nb(len), 256, 0, st>>>(dhp, tmp, len);
    SG_CUDA(cudaGetLastError());
    std::swap(dh, dhp);
  }
  c->launches += 3 + 7 * nl;
  float hl = 0.f;
  SG_CUDA(cudaMemcpyAsync(&hl, loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  if (grad_host) SG_CUDA(cudaMemcpyAsync(grad_host, c->p_g.ptr, count * sizeof(float), cudaMemcpyDeviceToHost, st));
  if (lr > 0.f) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    pc_adam_kernel<<<nb(count), 256, 0, st>>>(c->p_w.ptr, c->p_g.ptr, c->p_m.ptr, c->p_v.ptr, count, lr, b1, b2, 1e-8f,
                                              c1, c2);
    pc_to_bf16<<<nb(count), 256, 0, st>>>(c->p_w.ptr, c->p_wb.ptr, count);
    SG_CUDA(cudaGetLastError());
    c->launches += 2;
  }
  SG_CUDA(cudaStreamSynchronize(st));
  if (loss_out) *loss_out = hl;
}

void precond_get_params(sg_context *c, float *params, int count, cudaStream_t st) {
  SG_REQUIRE(count == c->p_count, "parameter count mismatch");
  SG_CUDA(cudaMemcpyAsync(params, c->p_w.ptr, count * sizeof(float), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
}

void precond_export_blocks(sg_context *c, int gid, float *G_host, cudaStream_t st) {
  SG_REQUIRE(gid >= 0 && gid < (int)c->pgraphs.size(), "bad preconditioner graph id");
  const sg_context::PGraph &g = *c->pgraphs[gid];
  SG_CUDA(cudaMemcpyAsync(G_host, g.G.ptr, (size_t)g.n * g.k1 * g.bs * g.bs * sizeof(float2), cudaMemcpyDeviceToHost,
                          st));
  SG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace sg

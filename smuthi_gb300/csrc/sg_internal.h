// Internal declarations of the smuthi_gb300 CUDA library.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/smuthi_gb300.h"

struct sg_context;

namespace sg {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
void clear_error();

struct Error {
  int code;
  std::string msg;
};

#define SG_CUDA(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) throw ::sg::Error{SG_ERR_CUDA, std::string(#call) + ": " +          \
                                                              cudaGetErrorString(e_)};          \
  } while (0)

#define SG_REQUIRE(cond, msg)                                   \
  do {                                                          \
    if (!(cond)) throw ::sg::Error{SG_ERR_ARG, std::string(msg)}; \
  } while (0)

// ---------------------------------------------------------------- device buffers
template <typename T>
struct DevBuf {
  T *ptr = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    n = 0;
  }
  // grow-only allocation; contents are not preserved
  void reserve(size_t count) {
    if (count <= n && ptr) return;
    release();
    if (count == 0) return;
    SG_CUDA(cudaMalloc(&ptr, count * sizeof(T)));
    n = count;
  }
};

// ---------------------------------------------------------------- coupling launch parameters
// Vectors handled by the kernels are "padded": [particle][blocksize][nrhs] complex double.
struct CouplingLaunch {
  const double2 *pos;   // [N] particle (x, y)
  const int *mofn;      // [bs]
  const void *coef;     // [n_int][ncoef][bs][bs] complex (double2 or float2), n1 fastest
  const int4 *pairs;    // FP32 path: [N][N] (k, t, cos phi, sin phi) or null
  int n, bs, n_int, ncoef;
  double rho_min, res;
  const double2 *x;     // padded input
  const float2 *x32;    // FP32 path: FP32 copy of x (read by the emitter loop; null = convert per pair)
  const void *xdf;      // double-float path: df64x2 copy of x (required)
  double2 *y;           // padded output (or split partials)
  double2 *partial;     // [nsplit][N][bs][R] scratch when nsplit > 1
  int nrhs;             // R (leading dimension of x, y)
  int rt;               // RHS tile per CTA (0 = default choice; the FP32 autotuner sets it)
  int master;           // 0: y = W x; 1: y = x - T W x
  const double2 *t;     // T blocks: diag [types][bs] or full [types][bs][bs]
  const int *ptype;     // [N]
  int t_diag;
};

// launch the coupling matvec on padded vectors; returns number of kernels launched
int launch_coupling(const CouplingLaunch &L, bool fp32, int nsplit, cudaStream_t st);
// the same in double-float arithmetic (L.coef = df64 coefficients from build_coefficients_df64)
int launch_coupling_df64(const CouplingLaunch &L, int nsplit, cudaStream_t st);
void build_coefficients_df64(const double2 *coef64, void *coefdf, size_t n, cudaStream_t st);
void k_to_df64(const double2 *x, void *xdf, size_t n, cudaStream_t st);
// tensor-core (tcgen05, 3xTF32) FP32-grade operator for batched RHS (sg_tc.cu)
bool tc_supported(const sg_context *c, int R);
int launch_tc_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st);
bool tc_check_error(sg_context *c, cudaStream_t st);  // reads and clears the timeout flag (synchronises)
bool tcsym_supported(const sg_context *c, int R);
int launch_tcsym_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st);
// FP32 W x in c->sym_yacc -> FP64 W x or x - T (W x) (diagonal or dense T); one launch
void launch_fp32_epilogue(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st);
// y = M x or W x in double-float arithmetic (FP64-grade; builds the df64 coefficients on first use)
void apply_padded_df64(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st);
// padded-vector operator application and solver (sg_gmres.cu)
void apply_padded(sg_context *c, const double2 *x, double2 *y, int R, bool master, bool fp32, cudaStream_t st);
void solve_padded(sg_context *c, const double2 *b, double2 *x, int R, double rtol, int restart, int maxiter,
                  int precision, sg_solve_info *info, cudaStream_t st);
void residual_norms(sg_context *c, const double2 *b, const double2 *x, int R, double *rel, cudaStream_t st);
// choose the j-split for a problem (>= 1)
int choose_split(int n_particles, int nrhs);

// ---------------------------------------------------------------- table preparation
// Build interpolation coefficients from a raw FP64 table [len_rho][bs][bs] (n2 fastest).
void build_coefficients(int kind, const double2 *raw, int len_rho, int bs, double2 *coef64, float2 *coef32,
                        double2 *work, cudaStream_t st);
int coef_count(int kind);
// interval-bucketed FP32 operator (sg_bucket.cu)
bool bucket_supported(const sg_context *c);
void build_bucket_plan(sg_context *c, cudaStream_t st);
int launch_bucket_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, cudaStream_t st);
// pair-symmetric FP32 operator (sg_sym.cu): each unordered pair's interpolated block serves both directions
bool sym_supported(const sg_context *c);
int sym_max_tile(const sg_context *c);
int launch_sym_matvec(sg_context *c, const double2 *x, double2 *y, int R, bool master, int rt, int split,
                      cudaStream_t st);
bool sym_check_error(sg_context *c, cudaStream_t st);  // reads and clears the timeout flag (synchronises)
// FP32 per-pair data (interval index, t, cos, sin) for all ordered pairs.
void build_pairs(const double2 *pos, int n, double rho_min, double res, int n_int, int4 *pairs, cudaStream_t st);

// ---------------------------------------------------------------- BLAS-1 style kernels (padded vectors)
void k_gather(const double2 *src, double2 *dst, const int *map, int n_unknowns, int nrhs, cudaStream_t st);
void k_scatter(const double2 *src, double2 *dst, const int *map, int n_unknowns, int nrhs, cudaStream_t st);
void k_zero(double2 *p, size_t n, cudaStream_t st);
void k_to_f32(const double2 *x, float2 *y, size_t n, cudaStream_t st);

// cudaFuncSetAttribute acts on the current device: true the first time a given kernel's attribute is
// needed on the current device (the caller keeps one flag array per kernel instantiation)
inline bool first_on_device(bool (&done)[64]) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return true;
  if (done[dev]) return false;
  done[dev] = true;
  return true;
}

// number of SMs of the current device (queried once per device; grid sizes scale with it)
inline int sm_count() {
  static int cache[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  if (cache[dev] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
    cache[dev] = v;
  }
  return cache[dev];
}

// FMA-throughput probe (TFLOP/s) of the FP64 or FP32 pipe
double fma_peak(int fp64, cudaStream_t st);

// volume lookup (sg_volume.cu): raw [len_rho][len_z][bs][bs] (n2 fastest) -> interpolation planes
// [len_rho][len_z][nq][bs][bs] (n1 fastest; nq = 4 for SG_CUBIC, else 1) in FP64 and FP32
void build_volume_table(int kind, const double2 *raw, int len_rho, int len_z, int bs, double2 *out64, float2 *out32,
                        cudaStream_t st);
// y = W x or x - T W x with the volume lookup on padded vectors; returns the number of kernels launched
int launch_volume(sg_context *c, const double2 *x, double2 *y, int R, bool master, bool fp32, cudaStream_t st);

// field of a plane-wave expansion at points (sg_nearfield.cu); synchronous, returns kernels launched
// regular SWE coefficients of plane waves at points (device buffers); returns the number of launches
int plane_wave_swe(int np, const double *xyz, int nq, int nc, const double *kr, int bs, const double2 *amp,
                   double2 *out, cudaStream_t st);
int pwe_field(int field, int np, const double *x, const double *y, const double *z, int nk, const double2 *kp,
              const double2 *kz, int na, const double *alpha, const double2 *g, double2 k, double omega, double2 *out,
              cudaStream_t st);

// Bessel factors of the layer-mediated lookup table (sg_table.cu)
void bessel_jac_table(const double2 *kp, const double2 *jac, int nk, const double *rho, int nr, int nmax,
                      double2 *out, cudaStream_t st);
// out[r * out_stride + cols[j]] = factor * sum_k a[r][k] g[k][j] (FP64 tiled complex GEMM, sg_table.cu)
void lookup_contract(const double2 *a, int nr, int nk, const double2 *g, int ncols, const int *cols, double2 factor,
                     double2 *out, long long out_stride, cudaStream_t st);

// particle sum of the scattered plane-wave expansion (sg_farfield.cu); synchronous
void farfield_sum(const double2 *xy, int n, int bs, int nrhs, const double2 *coef, int mmax, const int *mofn_host,
                  int nk, const double *kpar, const double2 *S, int na, const double *alpha, const double2 *zphase,
                  double2 *out, cudaStream_t st);

// ---------------------------------------------------------------- learned preconditioner (sg_precond.cu)
int precond_param_count(int bs);   // the default (3-layer) network
int precond_layers(int bs, int count);  // depth of a parameter vector (0: no valid depth)
void precond_add_graph(sg_context *c, int k, const int *nbr_host, int *graph_id, cudaStream_t st);
void precond_set_params(sg_context *c, int bs, const float *params, int count, cudaStream_t st);
void precond_get_params(sg_context *c, float *params, int count, cudaStream_t st);
// z = P v for S padded vectors with the selected graph
void precond_apply(sg_context *c, const double2 *v, double2 *z, int S, cudaStream_t st);
void precond_train(sg_context *c, int gid, const double2 *v, const double2 *e, int S, float lr, int step,
                   double *loss_out, float *grad_host, cudaStream_t st);
void precond_export_blocks(sg_context *c, int gid, float *G_host, cudaStream_t st);

}  // namespace sg

// ---------------------------------------------------------------- context
struct sg_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;

  // particles
  int n = 0, bs = 0, n_unknowns = 0;
  bool uniform = true;  // reference layout == padded layout
  sg::DevBuf<double2> pos;
  sg::DevBuf<int> map;  // [n_unknowns] -> padded index
  sg::DevBuf<int> mofn;
  std::vector<int> h_mofn;

  // lookup
  int kind = -1, len_rho = 0, n_int = 0, ncoef = 0;
  double rho_min = 0, res = 0;
  sg::DevBuf<double2> coef64;
  sg::DevBuf<float2> coef32;
  sg::DevBuf<int4> pairs;
  sg::DevBuf<double2> coefdf;  // FP64 coefficients split into two FP32 words each (16 bytes per complex)
  bool df_ready = false;
  sg::DevBuf<double2> xdf;  // double-float copy of the operator input (16 bytes per complex)
  sg::DevBuf<float> tc_xop;  // tensor-core operator: pre-split TF32 hi/lo RHS panels
  sg::DevBuf<float> tc_xops;  // pair-symmetric tensor-core operator: the same panels of S x
  sg::DevBuf<int4> tcs_items; // pair-symmetric tensor-core operator: (receiver pair, emitter run)
  int tcs_n_items = 0, tcs_items_n = -1;
  sg::DevBuf<int> tc_err;    // tensor-core operator: set when a bounded wait ran out
  bool tc_err_init = false;
  int tc_win = 8;            // tensor-core operator: emitters per accumulator before it is drained
  bool pairs_ready = false;  // FP32 operator data (bucket plan or pair table) is built

  // volume lookup (particles at different heights): replaces the radial table when set; `kind`,
  // `len_rho`, `rho_min` and `res` describe its rho axis
  bool vol = false;
  int v_len_z = 0, v_nq = 1;
  double v_sz_min = 0, v_dz_min = 0;
  sg::DevBuf<double> vz;                // [N] particle heights
  sg::DevBuf<double2> vpl64, vmn64;     // z1 + z2 and z1 - z2 tables, [rho][z][q][n2][n1]
  sg::DevBuf<float2> vpl32, vmn32;

  // interval-bucketed FP32 operator (sg_bucket.cu)
  bool use_bucket = false;  // the bucket plan exists
  // FP32 kernel autotuner: per RHS count, the fastest of the per-receiver, the bucketed and the
  // pair-symmetric kernel
  struct Tuned {
    int nrhs, variant;  // 0 per-receiver, 1 bucketed, 2 pair-symmetric, 3 pair-symmetric (2 warps per receiver),
                        // 4 tensor cores (3xTF32), 5 pair-symmetric tensor cores
    int rt;             // per-receiver kernel: RHS tile per CTA
    float ms_receiver, ms_bucket;  // best per-receiver tile, bucketed (< 0: not a candidate)
    int sym_rt;         // pair-symmetric kernel: RHS tile per CTA
    float ms_sym;       // best pair-symmetric tile and layout (< 0: not a candidate)
    float ms_tc;        // tensor-core operator (< 0: not a candidate)
    float ms_tcs;       // pair-symmetric tensor-core operator (< 0: not a candidate)
  };
  std::vector<Tuned> tuned;
  std::vector<std::pair<int, int>> tuned_df;  // double-float kernel: (nrhs, RHS tile)
  int bk_T = 0, bk_tiles = 0, bk_S = 0;
  sg::DevBuf<int> bk_members, bk_offs;
  sg::DevBuf<int4> bk_rec;
  sg::DevBuf<float2> bk_x32;
  sg::DevBuf<double2> bk_yacc;
  // pair-symmetric FP32 operator: work items (receiver tile, emitter-tile run) and FP32 accumulator
  sg::DevBuf<int4> sym_items;
  int sym_n_items = 0, sym_items_n = -1, sym_items_T = 0;
  sg::DevBuf<float2> sym_yacc;
  sg::DevBuf<int> sym_err;  // set when a bounded wait of the pair-symmetric kernel ran out
  bool sym_err_init = false;

  // T-matrices
  int n_types = 0, t_diag = 1;
  sg::DevBuf<double2> tmat;
  sg::DevBuf<int> ptype;
  bool t_ready = false;

  // work buffers
  sg::DevBuf<double2> io_in, io_out, pad_in, pad_out, sol_b, sol_x;
  sg::DevBuf<double2> w_partial, w_b, w_x, w_r, w_w, w_basis, w_tmp, w_d;
  sg::DevBuf<double> w_red;
  sg::DevBuf<double2> w_hcol;
  std::vector<double> h_red;

  // learned preconditioner: k-nearest-neighbour graphs with their near-field blocks T_i W_ij
  struct PGraph {
    int n = 0, bs = 0, k1 = 0;  // k1 = neighbours + self
    sg::DevBuf<int> nbr;        // [n][k1], slot 0 = self
    sg::DevBuf<int> rev_off, rev_idx;  // edges grouped by their source particle (adjoint)
    sg::DevBuf<float2> G;       // [n][k1][bs][bs], n2 fastest
  };
  std::vector<std::unique_ptr<PGraph>> pgraphs;
  int p_active = -1, p_bs = 0, p_count = 0, p_layers = 0;
  sg::DevBuf<float> p_w, p_g, p_m, p_v;  // FP32 master weights, gradient, Adam moments
  sg::DevBuf<__nv_bfloat16> p_wb;        // BF16 copy used by the forward and backward kernels
  sg::DevBuf<float> p_act, p_back;       // activations, backward scratch
  sg::DevBuf<float2> p_tmp;
  sg::DevBuf<double2> w_z;               // flexible-GMRES basis Z = P V

  // instrumentation
  int64_t launches = 0;
  bool profiling = false;
  struct Timed {
    cudaEvent_t e0, e1;
    int fp32;
  };
  std::vector<Timed> events;
  int64_t coupling_launches[4] = {0, 0, 0, 0};  // [fp64, fp32, df64, tf32x3]
  double coupling_ms[4] = {0.0, 0.0, 0.0, 0.0};

  size_t padded(int nrhs) const { return (size_t)n * bs * nrhs; }
};

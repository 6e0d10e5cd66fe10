// C ABI of the smuthi_gb300 library: context, uploads, validation and entry points.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "sg_internal.h"

static thread_local std::string g_last_error;

namespace sg {
void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
}  // namespace sg

template <class F>
static int guarded(F &&f) {
  sg::clear_error();
  try {
    return f();
  } catch (const sg::Error &e) {
    sg::set_error(e.msg);
    return e.code;
  } catch (const std::exception &e) {
    sg::set_error(std::string("internal error: ") + e.what());
    return SG_ERR_CUDA;
  } catch (...) {
    sg::set_error("internal error");
    return SG_ERR_CUDA;
  }
}

static void use_device(sg_context *c) { SG_CUDA(cudaSetDevice(c->device)); }

static void require_ready(sg_context *c, bool need_t) {
  SG_REQUIRE(c != nullptr, "null context");
  SG_REQUIRE(c->n > 0, "sg_set_particles has not been called");
  SG_REQUIRE(c->kind >= 0, "sg_set_lookup has not been called");
  if (need_t) SG_REQUIRE(c->t_ready, "sg_set_tmatrix has not been called");
}

// FP32 operator data: the pair table of the per-receiver kernel and, when the sizes allow it, the
// interval-bucketed plan; the autotuner picks between the two kernels per RHS count.
static void ensure_pairs(sg_context *c, cudaStream_t st) {
  if (c->pairs_ready || c->vol) return;  // the volume kernel needs no pair table
  c->pairs.reserve((size_t)c->n * c->n);
  sg::build_pairs(c->pos.ptr, c->n, c->rho_min, c->res, c->n_int, c->pairs.ptr, st);
  c->launches += 1;
  c->use_bucket = false;
  if (sg::bucket_supported(c)) {
    sg::build_bucket_plan(c, st);
    c->use_bucket = true;
  }
  c->tuned.clear();
  c->pairs_ready = true;
}

static bool all_finite(const double *p, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

extern "C" {

const char *sg_last_error(void) { return g_last_error.c_str(); }

const char *sg_version(void) { return "smuthi_gb300 0.1 (sm_103a)"; }

int sg_create(int device, sg_context **out) {
  return guarded([&]() -> int {
    SG_REQUIRE(out != nullptr, "null output pointer");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
      cudaGetLastError();
      throw sg::Error{SG_ERR_NO_DEVICE, "no CUDA device available"};
    }
    SG_REQUIRE(device >= 0 && device < count, "device index out of range");
    SG_CUDA(cudaSetDevice(device));
    sg_context *c = new sg_context();
    c->device = device;
    // a blocking stream: work on it is ordered with the legacy default stream, so callers that queue
    // their inputs there (and pass NULL for "the context's stream") need no extra synchronisation
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamDefault);
    if (e != cudaSuccess) {
      delete c;
      throw sg::Error{SG_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)};
    }
    c->own_stream = true;
    *out = c;
    return SG_OK;
  });
}

int sg_destroy(sg_context *ctx) {
  return guarded([&]() -> int {
    if (!ctx) return SG_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &ev : ctx->events) {
      cudaEventDestroy(ev.e0);
      cudaEventDestroy(ev.e1);
    }
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SG_OK;
  });
}

int sg_set_particles(sg_context *ctx, int n_particles, const double *xy, int n_unknowns,
                     const int32_t *unknown_particle, const int32_t *unknown_n, int blocksize,
                     const int32_t *m_of_n) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    SG_REQUIRE(n_particles >= 1, "need at least one particle");
    SG_REQUIRE(blocksize >= 1 && blocksize <= 96, "blocksize must be in [1, 96]");
    SG_REQUIRE(n_unknowns >= 1 && (long long)n_unknowns <= (long long)n_particles * blocksize,
               "n_unknowns must be in [1, n_particles * blocksize]");
    SG_REQUIRE(xy && unknown_particle && unknown_n && m_of_n, "null input array");
    SG_REQUIRE(all_finite(xy, 2 * (size_t)n_particles), "particle positions must be finite");
    use_device(ctx);
    std::vector<char> seen((size_t)n_particles * blocksize, 0);
    std::vector<int> map(n_unknowns);
    bool uniform = (long long)n_unknowns == (long long)n_particles * blocksize;
    for (int u = 0; u < n_unknowns; ++u) {
      const int p = unknown_particle[u], n = unknown_n[u];
      SG_REQUIRE(p >= 0 && p < n_particles, "unknown_particle out of range");
      SG_REQUIRE(n >= 0 && n < blocksize, "unknown_n out of range");
      const size_t pad = (size_t)p * blocksize + n;
      SG_REQUIRE(!seen[pad], "duplicate (particle, n) pair in the unknown list");
      seen[pad] = 1;
      map[u] = (int)pad;
      if ((size_t)u != pad) uniform = false;
    }
    int mmax = 0;
    for (int n = 0; n < blocksize; ++n) mmax = std::max(mmax, std::abs((int)m_of_n[n]));
    SG_REQUIRE(mmax <= 16, "|m| must be <= 16");
    ctx->n = n_particles;
    ctx->bs = blocksize;
    ctx->n_unknowns = n_unknowns;
    ctx->uniform = uniform;
    std::vector<double2> pos(n_particles);
    for (int i = 0; i < n_particles; ++i) pos[i] = make_double2(xy[2 * i], xy[2 * i + 1]);
    ctx->pos.reserve(n_particles);
    SG_CUDA(cudaMemcpy(ctx->pos.ptr, pos.data(), n_particles * sizeof(double2), cudaMemcpyHostToDevice));
    ctx->h_mofn.assign(m_of_n, m_of_n + blocksize);
    ctx->mofn.reserve(blocksize);
    SG_CUDA(cudaMemcpy(ctx->mofn.ptr, ctx->h_mofn.data(), blocksize * sizeof(int), cudaMemcpyHostToDevice));
    if (!uniform) {
      ctx->map.reserve(n_unknowns);
      SG_CUDA(cudaMemcpy(ctx->map.ptr, map.data(), n_unknowns * sizeof(int), cudaMemcpyHostToDevice));
    }
    ctx->pairs_ready = false;
    ctx->tuned_df.clear();
    ctx->kind = -1;  // the table must be re-uploaded for a new geometry
    ctx->vol = false;
    ctx->t_ready = false;
    ctx->pgraphs.clear();  // preconditioner graphs belong to the old particles
    ctx->p_active = -1;
    return SG_OK;
  });
}

int sg_set_lookup(sg_context *ctx, int kind, int len_rho, double rho_min, double resolution, const double *table) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    SG_REQUIRE(ctx->n > 0, "sg_set_particles must precede sg_set_lookup");
    SG_REQUIRE(kind == SG_LINEAR || kind == SG_CUBIC || kind == SG_CUBIC_HERMITE, "unknown interpolation kind");
    SG_REQUIRE(len_rho >= (kind == SG_LINEAR ? 2 : 4), "lookup table too short for this interpolation kind");
    SG_REQUIRE(resolution > 0 && std::isfinite(resolution) && std::isfinite(rho_min), "bad lookup grid");
    SG_REQUIRE(table != nullptr, "null table");
    const int bs = ctx->bs;
    const size_t count = (size_t)len_rho * bs * bs;
    if (!all_finite(table, 2 * count)) throw sg::Error{SG_ERR_NAN, "lookup table holds NaN or Inf"};
    // the grid must cover every pair distance: largest rho must sit in an interval
    std::vector<double2> pos(ctx->n);
    use_device(ctx);
    SG_CUDA(cudaMemcpy(pos.data(), ctx->pos.ptr, ctx->n * sizeof(double2), cudaMemcpyDeviceToHost));
    double r2max = 0.0;
    for (int i = 0; i < ctx->n; ++i)
      for (int j = i + 1; j < ctx->n; ++j) {
        const double dx = pos[i].x - pos[j].x, dy = pos[i].y - pos[j].y;
        r2max = std::max(r2max, dx * dx + dy * dy);
      }
    const double rmax = std::sqrt(r2max);
    const int need = kind == SG_CUBIC_HERMITE ? 3 : 2;
    SG_REQUIRE(rho_min <= 0.0 && std::floor((rmax - rho_min) / resolution) + need <= len_rho,
               "lookup grid does not cover [0, largest particle distance]");
    const int ncoef = sg::coef_count(kind);
    const int n_int = len_rho - 1;
    cudaStream_t st = ctx->stream;
    sg::DevBuf<double2> raw, work;
    raw.reserve(count);
    if (kind == SG_CUBIC) work.reserve(count);
    SG_CUDA(cudaMemcpyAsync(raw.ptr, table, count * sizeof(double2), cudaMemcpyHostToDevice, st));
    ctx->coef64.reserve((size_t)n_int * ncoef * bs * bs);
    ctx->coef32.reserve((size_t)n_int * ncoef * bs * bs);
    sg::build_coefficients(kind, raw.ptr, len_rho, bs, ctx->coef64.ptr, ctx->coef32.ptr, work.ptr, st);
    ctx->launches += kind == SG_CUBIC ? 2 : 1;
    ctx->kind = kind;
    ctx->vol = false;
    ctx->len_rho = len_rho;
    ctx->n_int = n_int;
    ctx->ncoef = ncoef;
    ctx->rho_min = rho_min;
    ctx->res = resolution;
    ctx->pairs_ready = false;
    ctx->df_ready = false;
    ctx->tuned_df.clear();
    ctx->pgraphs.clear();  // their near-field blocks came from the old table
    ctx->p_active = -1;
    return SG_OK;
  });
}

int sg_set_volume_lookup(sg_context *ctx, int kind, const double *z, int len_rho, double rho_min, int len_z,
                         double sz_min, double dz_min, double resolution, const double *table_plus,
                         const double *table_minus) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    SG_REQUIRE(ctx->n > 0, "sg_set_particles must precede sg_set_volume_lookup");
    SG_REQUIRE(kind == SG_LINEAR || kind == SG_CUBIC || kind == SG_CUBIC_HERMITE, "unknown interpolation kind");
    const int need_len = kind == SG_LINEAR ? 2 : 4;
    SG_REQUIRE(len_rho >= need_len && len_z >= need_len, "lookup grid too short for this interpolation kind");
    SG_REQUIRE(resolution > 0 && std::isfinite(resolution) && std::isfinite(rho_min) && std::isfinite(sz_min) &&
                   std::isfinite(dz_min),
               "bad lookup grid");
    SG_REQUIRE(z && table_plus && table_minus, "null input array");
    const int bs = ctx->bs, N = ctx->n;
    SG_REQUIRE(all_finite(z, N), "particle heights must be finite");
    const size_t count = (size_t)len_rho * len_z * bs * bs;
    if (!all_finite(table_plus, 2 * count) || !all_finite(table_minus, 2 * count))
      throw sg::Error{SG_ERR_NAN, "lookup table holds NaN or Inf"};
    // every pair's (rho, z_i + z_j, z_i - z_j) must lie where all taps are on the grid
    std::vector<double2> pos(N);
    use_device(ctx);
    SG_CUDA(cudaMemcpy(pos.data(), ctx->pos.ptr, N * sizeof(double2), cudaMemcpyDeviceToHost));
    double r2max = 0.0, zmin = z[0], zmax = z[0];
    for (int i = 0; i < N; ++i) {
      zmin = std::min(zmin, z[i]);
      zmax = std::max(zmax, z[i]);
      for (int j = i + 1; j < N; ++j) {
        const double dx = pos[i].x - pos[j].x, dy = pos[i].y - pos[j].y;
        r2max = std::max(r2max, dx * dx + dy * dy);
      }
    }
    const int lo = kind == SG_CUBIC_HERMITE ? 1 : 0, hi = kind == SG_CUBIC_HERMITE ? 3 : 2;
    auto covers = [&](double origin, double a, double b, int len) {
      return std::floor((a - origin) / resolution) >= lo && std::floor((b - origin) / resolution) + hi <= len;
    };
    SG_REQUIRE(covers(rho_min, 0.0, std::sqrt(r2max), len_rho),
               "lookup grid does not cover [0, largest lateral particle distance]");
    SG_REQUIRE(covers(sz_min, 2 * zmin, 2 * zmax, len_z), "z1 + z2 grid does not cover the particle heights");
    SG_REQUIRE(covers(dz_min, zmin - zmax, zmax - zmin, len_z), "z1 - z2 grid does not cover the particle heights");
    cudaStream_t st = ctx->stream;
    const int nq = kind == SG_CUBIC ? 4 : 1;
    sg::DevBuf<double2> raw;
    raw.reserve(count);
    ctx->vpl64.reserve(count * nq);
    ctx->vmn64.reserve(count * nq);
    ctx->vpl32.reserve(count * nq);
    ctx->vmn32.reserve(count * nq);
    SG_CUDA(cudaMemcpyAsync(raw.ptr, table_plus, count * sizeof(double2), cudaMemcpyHostToDevice, st));
    sg::build_volume_table(kind, raw.ptr, len_rho, len_z, bs, ctx->vpl64.ptr, ctx->vpl32.ptr, st);
    SG_CUDA(cudaMemcpyAsync(raw.ptr, table_minus, count * sizeof(double2), cudaMemcpyHostToDevice, st));
    sg::build_volume_table(kind, raw.ptr, len_rho, len_z, bs, ctx->vmn64.ptr, ctx->vmn32.ptr, st);
    ctx->launches += 2 * (kind == SG_CUBIC ? 4 : 1);
    ctx->vz.reserve(N);
    SG_CUDA(cudaMemcpy(ctx->vz.ptr, z, N * sizeof(double), cudaMemcpyHostToDevice));
    ctx->kind = kind;
    ctx->vol = true;
    ctx->len_rho = len_rho;
    ctx->rho_min = rho_min;
    ctx->res = resolution;
    ctx->v_len_z = len_z;
    ctx->v_nq = nq;
    ctx->v_sz_min = sz_min;
    ctx->v_dz_min = dz_min;
    ctx->n_int = 0;
    ctx->ncoef = 0;
    ctx->pairs_ready = false;
    ctx->use_bucket = false;
    ctx->tuned.clear();
    ctx->df_ready = false;
    ctx->tuned_df.clear();
    ctx->pgraphs.clear();
    ctx->p_active = -1;
    return SG_OK;
  });
}

int sg_set_tmatrix(sg_context *ctx, int n_types, const double *t, const int32_t *particle_type, int diagonal) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    SG_REQUIRE(ctx->n > 0, "sg_set_particles must precede sg_set_tmatrix");
    SG_REQUIRE(n_types >= 1 && t && particle_type, "bad T-matrix arguments");
    const int bs = ctx->bs;
    const size_t full = (size_t)n_types * bs * bs;
    if (!all_finite(t, 2 * full)) throw sg::Error{SG_ERR_NAN, "T-matrix holds NaN or Inf"};
    for (int i = 0; i < ctx->n; ++i)
      SG_REQUIRE(particle_type[i] >= 0 && particle_type[i] < n_types, "particle_type out of range");
    use_device(ctx);
    const double2 *tc = reinterpret_cast<const double2 *>(t);
    if (diagonal) {
      std::vector<double2> d((size_t)n_types * bs);
      for (int ty = 0; ty < n_types; ++ty)
        for (int a = 0; a < bs; ++a) {
          for (int b2 = 0; b2 < bs; ++b2)
            if (b2 != a) {
              const double2 v = tc[((size_t)ty * bs + a) * bs + b2];
              SG_REQUIRE(v.x == 0.0 && v.y == 0.0, "T-matrix declared diagonal has off-diagonal entries");
            }
          d[(size_t)ty * bs + a] = tc[((size_t)ty * bs + a) * bs + a];
        }
      ctx->tmat.reserve(d.size());
      SG_CUDA(cudaMemcpy(ctx->tmat.ptr, d.data(), d.size() * sizeof(double2), cudaMemcpyHostToDevice));
    } else {
      ctx->tmat.reserve(full);
      SG_CUDA(cudaMemcpy(ctx->tmat.ptr, tc, full * sizeof(double2), cudaMemcpyHostToDevice));
    }
    ctx->ptype.reserve(ctx->n);
    SG_CUDA(cudaMemcpy(ctx->ptype.ptr, particle_type, ctx->n * sizeof(int), cudaMemcpyHostToDevice));
    ctx->n_types = n_types;
    ctx->t_diag = diagonal ? 1 : 0;
    ctx->t_ready = true;
    ctx->pgraphs.clear();  // their near-field blocks hold the old T-matrices
    ctx->p_active = -1;
    return SG_OK;
  });
}

// reference-layout device vector -> padded device vector (returns the padded pointer)
static const double2 *to_padded(sg_context *c, const double2 *src, sg::DevBuf<double2> &pad, int R, cudaStream_t st) {
  if (c->uniform) return src;
  pad.reserve(c->padded(R));
  sg::k_zero(pad.ptr, c->padded(R), st);
  sg::k_gather(src, pad.ptr, c->map.ptr, c->n_unknowns, R, st);
  c->launches += 2;
  return pad.ptr;
}

static void matvec_dev(sg_context *c, const double2 *x, double2 *y, int R, int precision, bool master,
                       cudaStream_t st) {
  require_ready(c, master);
  SG_REQUIRE(R >= 1 && R <= 256, "nrhs must be in [1, 256]");
  SG_REQUIRE(precision == SG_FP64 || precision == SG_FP32 || precision == SG_DF64 || precision == SG_TF32X3,
             "unknown precision");
  SG_REQUIRE(!c->vol || precision == SG_FP64 || precision == SG_FP32,
             "a volume lookup supports SG_FP64 and SG_FP32 only");
  use_device(c);
  const bool fp32 = precision == SG_FP32;
  if (fp32 || precision == SG_TF32X3) ensure_pairs(c, st);
  const double2 *xp = to_padded(c, x, c->pad_in, R, st);
  double2 *yp = y;
  if (!c->uniform) {
    c->pad_out.reserve(c->padded(R));
    yp = c->pad_out.ptr;
  }
  if (precision == SG_DF64) {
    sg::apply_padded_df64(c, xp, yp, R, master, st);
  } else if (precision == SG_TF32X3) {
    SG_REQUIRE(sg::tc_supported(c, R),
               "SG_TF32X3 needs the radial lookup, blocksize <= 48 and nrhs in {16, 32, 64}");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (c->profiling) {
      SG_CUDA(cudaEventCreate(&e0));
      SG_CUDA(cudaEventCreate(&e1));
      SG_CUDA(cudaEventRecord(e0, st));
    }
    c->launches += sg::launch_tc_matvec(c, xp, yp, R, master, st);
    if (c->profiling) {
      SG_CUDA(cudaEventRecord(e1, st));
      c->events.push_back({e0, e1, 3});
    }
    if (sg::tc_check_error(c, st)) throw sg::Error{SG_ERR_CUDA, "tensor-core operator: a bounded wait ran out"};
  } else {
    sg::apply_padded(c, xp, yp, R, master, fp32, st);
  }
  if (!c->uniform) {
    sg::k_scatter(yp, y, c->map.ptr, c->n_unknowns, R, st);
    c->launches += 1;
  }
}

static int matvec_host(sg_context *ctx, const double *x, double *y, int nrhs, int precision, bool master) {
  return guarded([&]() -> int {
    require_ready(ctx, master);
    SG_REQUIRE(x && y, "null vector");
    SG_REQUIRE(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
    const size_t len = (size_t)ctx->n_unknowns * nrhs;
    if (!all_finite(x, 2 * len)) throw sg::Error{SG_ERR_NAN, "input vector holds NaN or Inf"};
    use_device(ctx);
    cudaStream_t st = ctx->stream;
    ctx->io_in.reserve(len);
    ctx->io_out.reserve(len);
    SG_CUDA(cudaMemcpyAsync(ctx->io_in.ptr, x, len * sizeof(double2), cudaMemcpyHostToDevice, st));
    matvec_dev(ctx, ctx->io_in.ptr, ctx->io_out.ptr, nrhs, precision, master, st);
    SG_CUDA(cudaMemcpyAsync(y, ctx->io_out.ptr, len * sizeof(double2), cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    if (precision == SG_FP32 && sg::sym_check_error(ctx, st))
      throw sg::Error{SG_ERR_CUDA, "pair-symmetric FP32 operator: a bounded wait ran out"};
    if (precision == SG_FP32 && sg::tc_check_error(ctx, st))
      throw sg::Error{SG_ERR_CUDA, "tensor-core operator: a bounded wait ran out"};
    return SG_OK;
  });
}

int sg_coupling_matvec(sg_context *ctx, const double *x, double *y, int nrhs, int precision) {
  return matvec_host(ctx, x, y, nrhs, precision, false);
}

int sg_master_matvec(sg_context *ctx, const double *x, double *y, int nrhs, int precision) {
  return matvec_host(ctx, x, y, nrhs, precision, true);
}

int sg_coupling_matvec_dev(sg_context *ctx, const void *x, void *y, int nrhs, int precision, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(x && y, "null vector");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    matvec_dev(ctx, (const double2 *)x, (double2 *)y, nrhs, precision, false, st);
    return SG_OK;
  });
}

int sg_master_matvec_dev(sg_context *ctx, const void *x, void *y, int nrhs, int precision, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(x && y, "null vector");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    matvec_dev(ctx, (const double2 *)x, (double2 *)y, nrhs, precision, true, st);
    return SG_OK;
  });
}

static int solve_dev_impl(sg_context *ctx, const double2 *b, double2 *x, int nrhs, double rtol, int restart,
                          int maxiter, int precision, sg_solve_info *info, cudaStream_t st) {
  require_ready(ctx, true);
  SG_REQUIRE(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
  SG_REQUIRE(rtol > 0 && std::isfinite(rtol), "rtol must be positive");
  SG_REQUIRE(restart >= 0 && restart <= 128, "restart must be in [0, 128] (0 = 20)");
  SG_REQUIRE(precision == SG_FP64 ||
                 ((precision & SG_FP32) && !(precision & ~(SG_FP32 | SG_BLOCK_GMRES | SG_PRECOND | SG_DF64)) &&
                  !((precision & SG_BLOCK_GMRES) && (precision & SG_PRECOND))),
             "unknown precision / solver flags");
  SG_REQUIRE(!ctx->vol || !(precision & (SG_PRECOND | SG_DF64)),
             "a volume lookup supports SG_FP64 and SG_FP32 (| SG_BLOCK_GMRES) solves only");
  if (precision & SG_PRECOND) {
    SG_REQUIRE(ctx->p_active >= 0, "SG_PRECOND needs a preconditioner graph (sg_precond_select)");
    SG_REQUIRE(ctx->p_layers > 0 && ctx->p_bs == ctx->bs, "SG_PRECOND needs parameters (sg_precond_set_params)");
    SG_REQUIRE(nrhs <= 64, "SG_PRECOND handles at most 64 right-hand sides per solve");
  }
  use_device(ctx);
  if (precision & SG_FP32) ensure_pairs(ctx, st);
  const size_t plen = ctx->padded(nrhs);
  const double2 *bp = b;
  double2 *xp = x;
  if (!ctx->uniform) {
    ctx->sol_b.reserve(plen);
    ctx->sol_x.reserve(plen);
    sg::k_zero(ctx->sol_b.ptr, plen, st);
    sg::k_zero(ctx->sol_x.ptr, plen, st);
    sg::k_gather(b, ctx->sol_b.ptr, ctx->map.ptr, ctx->n_unknowns, nrhs, st);
    sg::k_gather(x, ctx->sol_x.ptr, ctx->map.ptr, ctx->n_unknowns, nrhs, st);
    ctx->launches += 4;
    bp = ctx->sol_b.ptr;
    xp = ctx->sol_x.ptr;
  }
  sg_solve_info local{};
  sg::solve_padded(ctx, bp, xp, nrhs, rtol, restart, maxiter, precision, &local, st);
  if (!ctx->uniform) {
    sg::k_scatter(xp, x, ctx->map.ptr, ctx->n_unknowns, nrhs, st);
    ctx->launches += 1;
  }
  if (info) *info = local;
  if ((precision & SG_FP32) && sg::sym_check_error(ctx, st))
    throw sg::Error{SG_ERR_CUDA, "pair-symmetric FP32 operator: a bounded wait ran out"};
  if ((precision & SG_FP32) && sg::tc_check_error(ctx, st))
    throw sg::Error{SG_ERR_CUDA, "tensor-core operator: a bounded wait ran out"};
  if (!std::isfinite(local.max_rel_residual)) throw sg::Error{SG_ERR_NAN, "solver produced NaN or Inf"};
  if (local.converged < nrhs) {
    sg::set_error("GMRES did not reach the tolerance for every right-hand side");
    return SG_ERR_NOT_CONVERGED;
  }
  return SG_OK;
}

int sg_gmres_solve(sg_context *ctx, const double *b, double *x, int nrhs, double rtol, int restart, int maxiter,
                   int precision, sg_solve_info *info) {
  return guarded([&]() -> int {
    require_ready(ctx, true);
    SG_REQUIRE(b && x, "null vector");
    SG_REQUIRE(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
    const size_t len = (size_t)ctx->n_unknowns * nrhs;
    if (!all_finite(b, 2 * len) || !all_finite(x, 2 * len))
      throw sg::Error{SG_ERR_NAN, "right-hand side or initial guess holds NaN or Inf"};
    use_device(ctx);
    cudaStream_t st = ctx->stream;
    ctx->io_in.reserve(len);
    ctx->io_out.reserve(len);
    SG_CUDA(cudaMemcpyAsync(ctx->io_in.ptr, b, len * sizeof(double2), cudaMemcpyHostToDevice, st));
    SG_CUDA(cudaMemcpyAsync(ctx->io_out.ptr, x, len * sizeof(double2), cudaMemcpyHostToDevice, st));
    int rc = solve_dev_impl(ctx, ctx->io_in.ptr, ctx->io_out.ptr, nrhs, rtol, restart, maxiter, precision, info, st);
    SG_CUDA(cudaMemcpyAsync(x, ctx->io_out.ptr, len * sizeof(double2), cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    return rc;
  });
}

int sg_gmres_solve_dev(sg_context *ctx, const void *b, void *x, int nrhs, double rtol, int restart, int maxiter,
                       int precision, sg_solve_info *info, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(b && x, "null vector");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return solve_dev_impl(ctx, (const double2 *)b, (double2 *)x, nrhs, rtol, restart, maxiter, precision, info, st);
  });
}

int sg_true_residual(sg_context *ctx, const double *b, const double *x, int nrhs, double *rel_residual) {
  return guarded([&]() -> int {
    require_ready(ctx, true);
    SG_REQUIRE(b && x && rel_residual, "null argument");
    SG_REQUIRE(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
    const size_t len = (size_t)ctx->n_unknowns * nrhs;
    use_device(ctx);
    cudaStream_t st = ctx->stream;
    ctx->io_in.reserve(len);
    ctx->io_out.reserve(len);
    SG_CUDA(cudaMemcpyAsync(ctx->io_in.ptr, b, len * sizeof(double2), cudaMemcpyHostToDevice, st));
    SG_CUDA(cudaMemcpyAsync(ctx->io_out.ptr, x, len * sizeof(double2), cudaMemcpyHostToDevice, st));
    const double2 *bp = to_padded(ctx, ctx->io_in.ptr, ctx->sol_b, nrhs, st);
    const double2 *xp = to_padded(ctx, ctx->io_out.ptr, ctx->sol_x, nrhs, st);
    sg::residual_norms(ctx, bp, xp, nrhs, rel_residual, st);
    return SG_OK;
  });
}

int sg_profile(sg_context *ctx, int enable) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    ctx->profiling = enable != 0;
    return SG_OK;
  });
}

int sg_kernel_timing(sg_context *ctx, int precision, double *total_ms, int64_t *count, int reset) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    SG_REQUIRE(precision == -1 || precision == SG_FP64 || precision == SG_FP32 || precision == SG_DF64 ||
                   precision == SG_TF32X3,
               "precision must be SG_FP64, SG_FP32, SG_DF64, SG_TF32X3 or -1 (all)");
    use_device(ctx);
    for (auto &ev : ctx->events) {
      SG_CUDA(cudaEventSynchronize(ev.e1));
      float ms = 0.f;
      SG_CUDA(cudaEventElapsedTime(&ms, ev.e0, ev.e1));
      ctx->coupling_ms[ev.fp32] += ms;
      ctx->coupling_launches[ev.fp32] += 1;
      cudaEventDestroy(ev.e0);
      cudaEventDestroy(ev.e1);
    }
    ctx->events.clear();
    const int slot = precision == SG_DF64 ? 2 : (precision == SG_TF32X3 ? 3 : precision);
    const int lo = precision < 0 ? 0 : slot, hi = precision < 0 ? 3 : slot;
    double ms = 0.0;
    int64_t n = 0;
    for (int p = lo; p <= hi; ++p) {
      ms += ctx->coupling_ms[p];
      n += ctx->coupling_launches[p];
    }
    if (total_ms) *total_ms = ms;
    if (count) *count = n;
    if (reset) {
      for (int p = 0; p < 4; ++p) {
        ctx->coupling_ms[p] = 0.0;
        ctx->coupling_launches[p] = 0;
      }
    }
    return SG_OK;
  });
}

int sg_measure_fma_peak(sg_context *ctx, int precision, double *tflops) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && tflops, "null argument");
    SG_REQUIRE(precision == SG_FP64 || precision == SG_FP32, "unknown precision");
    use_device(ctx);
    *tflops = sg::fma_peak(precision == SG_FP64 ? 1 : 0, ctx->stream);
    ctx->launches += 4;
    return SG_OK;
  });
}

int sg_fp32_autotune(sg_context *ctx, int nrhs, int *variant, int *rhs_tile, double *ms_receiver,
                     double *ms_bucket, double *ms_symmetric, double *ms_tensor, double *ms_tensor_symmetric) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && variant, "null argument");
    for (const auto &t : ctx->tuned)
      if (t.nrhs == nrhs) {
        *variant = t.variant;
        if (rhs_tile) *rhs_tile = t.variant >= 4 ? nrhs : (t.variant >= 2 ? t.sym_rt : t.rt);
        if (ms_receiver) *ms_receiver = t.ms_receiver;
        if (ms_bucket) *ms_bucket = t.ms_bucket;
        if (ms_symmetric) *ms_symmetric = t.ms_sym;
        if (ms_tensor) *ms_tensor = t.ms_tc;
        if (ms_tensor_symmetric) *ms_tensor_symmetric = t.ms_tcs;
        return SG_OK;
      }
    *variant = -1;
    return SG_OK;
  });
}

int sg_tc_set_window(sg_context *ctx, int emitters) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx, "null context");
    SG_REQUIRE(emitters >= 1, "the drain window must be at least one emitter");
    ctx->tc_win = emitters;
    return SG_OK;
  });
}

int sg_fp32_set_kernel(sg_context *ctx, int nrhs, int variant, int rhs_tile) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx, "null context");
    SG_REQUIRE(nrhs >= 1, "nrhs must be >= 1");
    SG_REQUIRE(!ctx->vol && ctx->kind >= 0, "a radial lookup must be set");
    SG_REQUIRE(variant >= 0 && variant <= 5, "variant must be 0, 1, 2, 3, 4 or 5");
    use_device(ctx);
    ensure_pairs(ctx, ctx->stream);  // builds the FP32 operator data now (it would clear the choice later)
    sg_context::Tuned t{nrhs, variant, 0, -1.f, -1.f, 0, -1.f, -1.f, -1.f};
    if (variant == 0) {
      SG_REQUIRE(rhs_tile == 1 || rhs_tile == 2 || rhs_tile == 4 || rhs_tile == 8 || rhs_tile == 16,
                 "per-receiver RHS tile must be 1, 2, 4, 8 or 16");
      SG_REQUIRE(nrhs % rhs_tile == 0, "RHS tile must divide nrhs");
      t.rt = rhs_tile;
    } else if (variant == 1) {
      SG_REQUIRE(ctx->use_bucket, "the bucketed kernel has no plan for this geometry");
    } else if (variant == 4) {
      SG_REQUIRE(sg::tc_supported(ctx, nrhs), "the tensor-core operator needs blocksize <= 48 and nrhs in {16, 32, 64}");
      SG_REQUIRE(rhs_tile == nrhs, "the tensor-core operator takes all right-hand sides at once (rhs_tile = nrhs)");
    } else if (variant == 5) {
      SG_REQUIRE(sg::tcsym_supported(ctx, nrhs),
                 "the pair-symmetric tensor-core operator needs blocksize <= 32 and nrhs in {16, 32}");
      SG_REQUIRE(rhs_tile == nrhs, "the tensor-core operators take all right-hand sides at once (rhs_tile = nrhs)");
    } else {
      SG_REQUIRE(sg::sym_supported(ctx), "the pair-symmetric kernel needs blocksize <= 64");
      SG_REQUIRE(rhs_tile >= 1 && rhs_tile <= sg::sym_max_tile(ctx) && (rhs_tile & (rhs_tile - 1)) == 0,
                 "pair-symmetric RHS tile must be a power of two within the kernel's register budget");
      SG_REQUIRE(nrhs % rhs_tile == 0, "RHS tile must divide nrhs");
      SG_REQUIRE(variant == 2 || rhs_tile >= 4, "two warps per receiver need an RHS tile >= 4");
      t.sym_rt = rhs_tile;
    }
    for (auto &e : ctx->tuned)
      if (e.nrhs == nrhs) {
        e = t;
        return SG_OK;
      }
    ctx->tuned.push_back(t);
    return SG_OK;
  });
}

int sg_bessel_jac_table(sg_context *ctx, const void *kappa, const void *jac, int nk, const void *rho, int nr,
                        int nmax, void *out, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && kappa && jac && rho && out, "null argument");
    use_device(ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    sg::bessel_jac_table((const double2 *)kappa, (const double2 *)jac, nk, (const double *)rho, nr, nmax,
                         (double2 *)out, st);
    ctx->launches += 1;
    return SG_OK;
  });
}

int sg_lookup_contract(sg_context *ctx, const void *a, int nr, int nk, const void *g, int ncols, const int *cols,
                       double factor_re, double factor_im, void *out, long long out_stride, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && a && g && cols && out, "null argument");
    use_device(ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    sg::lookup_contract((const double2 *)a, nr, nk, (const double2 *)g, ncols, cols,
                        make_double2(factor_re, factor_im), (double2 *)out, out_stride, st);
    ctx->launches += 1;
    return SG_OK;
  });
}

int sg_farfield_sum_heights(sg_context *ctx, int n_particles, const void *xy, int blocksize, int nrhs,
                            const void *coef, int m_max, const int32_t *m_of_n, int nk, const void *kpar,
                            const void *S, int na, const void *alpha, const void *zphase, void *out, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && xy && coef && m_of_n && kpar && S && alpha && out, "null argument");
    use_device(ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    sg::farfield_sum((const double2 *)xy, n_particles, blocksize, nrhs, (const double2 *)coef, m_max, m_of_n, nk,
                     (const double *)kpar, (const double2 *)S, na, (const double *)alpha, (const double2 *)zphase,
                     (double2 *)out, st);
    ctx->launches += 1;
    return SG_OK;
  });
}

int sg_farfield_sum(sg_context *ctx, int n_particles, const void *xy, int blocksize, int nrhs, const void *coef,
                    int m_max, const int32_t *m_of_n, int nk, const void *kpar, const void *S, int na,
                    const void *alpha, void *out, void *stream) {
  return sg_farfield_sum_heights(ctx, n_particles, xy, blocksize, nrhs, coef, m_max, m_of_n, nk, kpar, S, na, alpha,
                                 nullptr, out, stream);
}

int sg_pwe_field(sg_context *ctx, int field, int n_points, const void *x, const void *y, const void *z, int nk,
                 const void *kpar, const void *kz, int na, const void *alpha, const void *g, double k_re, double k_im,
                 double omega, void *out, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && x && y && z && kpar && kz && alpha && g && out, "null argument");
    use_device(ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    ctx->launches += sg::pwe_field(field, n_points, (const double *)x, (const double *)y, (const double *)z, nk,
                                   (const double2 *)kpar, (const double2 *)kz, na, (const double *)alpha,
                                   (const double2 *)g, make_double2(k_re, k_im), omega, (double2 *)out, st);
    return SG_OK;
  });
}

int sg_plane_wave_swe(sg_context *ctx, int n_points, const void *xyz, int nwaves, int ncomp, const void *kr,
                      int blocksize, const void *amp, void *out, void *stream) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && xyz && kr && amp && out, "null argument");
    use_device(ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    ctx->launches += sg::plane_wave_swe(n_points, (const double *)xyz, nwaves, ncomp, (const double *)kr, blocksize,
                                        (const double2 *)amp, (double2 *)out, st);
    return SG_OK;
  });
}

int sg_precond_param_count(int blocksize) {
  if (blocksize < 1 || blocksize > 64) return -1;
  return sg::precond_param_count(blocksize);
}

int sg_precond_add_graph(sg_context *ctx, int k, const int32_t *nbr, int *graph_id) {
  return guarded([&]() -> int {
    require_ready(ctx, true);
    SG_REQUIRE(nbr && graph_id, "null argument");
    use_device(ctx);
    sg::precond_add_graph(ctx, k, nbr, graph_id, ctx->stream);
    return SG_OK;
  });
}

int sg_precond_select(sg_context *ctx, int graph_id) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    SG_REQUIRE(graph_id >= -1 && graph_id < (int)ctx->pgraphs.size(), "bad preconditioner graph id");
    ctx->p_active = graph_id;
    return SG_OK;
  });
}

int sg_precond_clear(sg_context *ctx) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx != nullptr, "null context");
    use_device(ctx);
    SG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->pgraphs.clear();
    ctx->p_active = -1;
    return SG_OK;
  });
}

int sg_precond_set_params(sg_context *ctx, int blocksize, const float *params, int count) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && params, "null argument");
    for (int i = 0; i < count; ++i) SG_REQUIRE(std::isfinite(params[i]), "parameters hold NaN or Inf");
    use_device(ctx);
    sg::precond_set_params(ctx, blocksize, params, count, ctx->stream);
    return SG_OK;
  });
}

int sg_precond_get_params(sg_context *ctx, float *params, int count) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && params, "null argument");
    use_device(ctx);
    sg::precond_get_params(ctx, params, count, ctx->stream);
    return SG_OK;
  });
}

int sg_precond_apply_dev(sg_context *ctx, const void *v, void *z, int nvec, void *stream) {
  return guarded([&]() -> int {
    require_ready(ctx, true);
    SG_REQUIRE(v && z, "null vector");
    SG_REQUIRE(ctx->uniform, "the learned preconditioner works on uniform particle blocks");
    use_device(ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    sg::precond_apply(ctx, (const double2 *)v, (double2 *)z, nvec, st);
    return SG_OK;
  });
}

int sg_precond_train_step(sg_context *ctx, int graph_id, const void *v, const void *e, int nvec, float lr, int step,
                          double *loss, float *grad) {
  return guarded([&]() -> int {
    require_ready(ctx, true);
    SG_REQUIRE(v && e, "null vector");
    SG_REQUIRE(ctx->uniform, "the learned preconditioner works on uniform particle blocks");
    SG_REQUIRE(lr >= 0.f && std::isfinite(lr), "lr must be >= 0");
    SG_REQUIRE(lr == 0.f || step >= 1, "step must be >= 1 for an Adam update");
    use_device(ctx);
    sg::precond_train(ctx, graph_id, (const double2 *)v, (const double2 *)e, nvec, lr, step, loss, grad,
                      ctx->stream);
    return SG_OK;
  });
}

int sg_precond_export_blocks(sg_context *ctx, int graph_id, float *blocks) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && blocks, "null argument");
    use_device(ctx);
    sg::precond_export_blocks(ctx, graph_id, blocks, ctx->stream);
    return SG_OK;
  });
}

int sg_launch_count(sg_context *ctx, int64_t *count) {
  return guarded([&]() -> int {
    SG_REQUIRE(ctx && count, "null argument");
    *count = ctx->launches;
    return SG_OK;
  });
}

}  // extern "C"

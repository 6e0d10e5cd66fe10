/*
 * smuthi_gb300 -- C ABI of the GB300-native radial-lookup coupling solve path.
 *
 * Drop-in boundary for SMUTHI's CouplingMatrixRadialLookupCUDA and the GMRES
 * loop that drives it. Every entry point returns an int status (SG_OK = 0);
 * no exception crosses the ABI. Host buffers are owned by the caller and are
 * read or written only during the call; device buffers are owned by the
 * context. One context serves one host thread at a time.
 *
 * Complex numbers are interleaved (re, im) pairs of double. A "system vector"
 * uses the reference layout: particle-major, each particle's block ordered
 * by its own multi index n(tau, l, m) (smuthi/fields/__init__.py:29-80).
 * Multi-RHS arrays are [unknown][rhs] (the rhs index runs fastest).
 */
#ifndef SMUTHI_GB300_H
#define SMUTHI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SG_OK 0
#define SG_ERR_ARG 1          /* invalid argument or call order */
#define SG_ERR_CUDA 2         /* CUDA runtime error or out of device memory */
#define SG_ERR_NOT_CONVERGED 3 /* solver hit its iteration limit; outputs hold the last iterate */
#define SG_ERR_NAN 4          /* NaN/Inf detected in an input or an iterate */
#define SG_ERR_NO_DEVICE 5    /* no CUDA device available */

/* lookup interpolation kinds */
#define SG_LINEAR 0           /* scipy interp1d(kind='linear') */
#define SG_CUBIC 1            /* scipy interp1d(kind='cubic'): not-a-knot cubic spline */
#define SG_CUBIC_HERMITE 2    /* 4-tap Catmull-Rom of the reference CUDA kernel */

/* arithmetic of an operator application */
#define SG_FP64 0
#define SG_FP32 1
/* solver flag, OR-ed into sg_gmres_solve's precision with SG_FP32: the correction solves of the
 * mixed form use one block Krylov space for all right-hand sides (block GMRES, restart <= 20)
 * instead of independent lockstep Krylov spaces */
#define SG_BLOCK_GMRES 2
/* solver flag, OR-ed into sg_gmres_solve's precision with SG_FP32: the correction solves are
 * right-preconditioned flexible GMRES with the learned preconditioner selected by
 * sg_precond_select; a correction solve that fails to reduce its residual is redone without it */
#define SG_PRECOND 4
/* double-float arithmetic: every sum of the coupling operator in two FP32 words (about 48
 * significant bits) on the FP32 pipe, with the FP64 table split into two FP32 words. As a matvec
 * precision it is an FP64-grade operator (it agrees with SG_FP64 to ~1e-13 relative); OR-ed into
 * sg_gmres_solve's precision with SG_FP32, the refinement's true residuals use it in place of the
 * FP64 operator. No counterpart in the reference. */
#define SG_DF64 8
/* matvec precision: the coupling operator on the tensor cores (tcgen05.mma kind::tf32, each
 * operand split into a TF32 high part and a remainder, three products), for the radial lookup with
 * blocksize <= 48 and nrhs in {16, 32, 64}. Each tensor-memory accumulator takes a few emitters
 * before it is added into an FP32 total (round-to-nearest), which bounds the error of the tensor
 * core's accumulation. It is also variant 4 of the FP32 operator (sg_fp32_autotune /
 * sg_fp32_set_kernel), the inner operator of the mixed-precision solve when it is the fastest.
 * No counterpart in the reference. */
#define SG_TF32X3 16

typedef struct sg_context sg_context;

/* Text of the last error on the calling thread ("" if none). */
const char *sg_last_error(void);

/* Library version string. */
const char *sg_version(void);

/* Create / destroy a context on CUDA device `device`. The context owns a blocking CUDA stream
 * (ordered with the legacy default stream); a NULL stream argument below means that stream.
 * Replaces the PyCUDA autoinit + gpuarray set-up of
 * smuthi/linearsystem/linear_system.py:829-882. */
int sg_create(int device, sg_context **out);
int sg_destroy(sg_context *ctx);

/* Particles and unknowns (smuthi/linearsystem/linear_system.py:848-869).
 * xy[2*i+{0,1}]: particle i lateral position (all particles share one z).
 * unknown_particle[u], unknown_n[u]: particle number and global lookup index
 * n(tau, l, m; l_max, m_max) of system-vector entry u, u < n_unknowns.
 * m_of_n[n]: multipole order m of global lookup index n, n < blocksize. */
int sg_set_particles(sg_context *ctx, int n_particles, const double *xy, int n_unknowns,
                     const int32_t *unknown_particle, const int32_t *unknown_n, int blocksize,
                     const int32_t *m_of_n);

/* Radial lookup table w[rho][n1][n2] (complex, len_rho x blocksize^2) on the
 * grid rho_k = rho_min + k * resolution, with interpolation `kind`.
 * Replaces the table upload and kernel compile of
 * smuthi/linearsystem/linear_system.py:838-881 (which cast to float32);
 * the table is kept in FP64 and also rounded once to FP32 for SG_FP32. */
int sg_set_lookup(sg_context *ctx, int kind, int len_rho, double rho_min, double resolution,
                  const double *table);

/* Volume lookup for particles at different heights in one layer, replacing the radial table
 * (the table upload and kernel compile of CouplingMatrixVolumeLookupCUDA,
 * smuthi/linearsystem/linear_system.py:700-770, and the interpolators of
 * CouplingMatrixVolumeLookupCPU, :592-667). z[i]: height of particle i (the xy of sg_set_particles).
 * table_plus[rho][s][n1][n2] is the z1 + z2 table on rho_min + a * resolution, sz_min + s * resolution;
 * table_minus[rho][d][n1][n2] the z1 - z2 table (direct + layer-mediated) on dz_min + d * resolution
 * (complex, len_rho x len_z x blocksize^2 each; the layout and grids of
 * smuthi/linearsystem/particlecoupling/prepare_lookup.py:16-250). kind: SG_LINEAR (bilinear),
 * SG_CUBIC (tensor-product not-a-knot cubic spline = RectBivariateSpline(kx=ky=3) of the CPU class)
 * or SG_CUBIC_HERMITE (the 4 x 4-tap Catmull-Rom of the reference CUDA kernel). The grids must
 * cover every pair's (rho, z_i + z_j, z_i - z_j) with all interpolation taps. With a volume lookup
 * the operator supports SG_FP64 and SG_FP32 (solves: SG_FP64, SG_FP32 [| SG_BLOCK_GMRES]); a later
 * sg_set_lookup or sg_set_particles drops it. */
int sg_set_volume_lookup(sg_context *ctx, int kind, const double *z, int len_rho, double rho_min, int len_z,
                         double sz_min, double dz_min, double resolution, const double *table_plus,
                         const double *table_minus);

/* Per-particle T-matrices (smuthi/linearsystem/linear_system.py:410-424):
 * n_types distinct blocks t[type][n1][n2] in the global lookup index space
 * (blocksize x blocksize complex); particle_type[i] picks particle i's block.
 * diagonal != 0 declares every block diagonal (Mie spheres). */
int sg_set_tmatrix(sg_context *ctx, int n_types, const double *t, const int32_t *particle_type, int diagonal);

/* y = W x, the coupling matvec (host buffers, n_unknowns x nrhs complex).
 * Replaces CouplingMatrixRadialLookupCUDA.linear_operator.matvec,
 * smuthi/linearsystem/linear_system.py:888-900. */
int sg_coupling_matvec(sg_context *ctx, const double *x, double *y, int nrhs, int precision);

/* y = x - T W x, the master operator (smuthi/linearsystem/linear_system.py:402-407). */
int sg_master_matvec(sg_context *ctx, const double *x, double *y, int nrhs, int precision);

/* Device-pointer variants: x, y are device buffers in the reference layout;
 * `stream` is a cudaStream_t (NULL = the context's stream). Asynchronous. */
int sg_coupling_matvec_dev(sg_context *ctx, const void *x, void *y, int nrhs, int precision, void *stream);
int sg_master_matvec_dev(sg_context *ctx, const void *x, void *y, int nrhs, int precision, void *stream);

/* Solver report. */
typedef struct sg_solve_info {
  int32_t iterations;      /* inner (Arnoldi) iterations, max over rhs */
  int32_t restarts;        /* restart cycles (plain) or refinement steps (mixed) */
  int32_t fp64_matvecs;    /* FP64 operator applications */
  int32_t fp32_matvecs;    /* FP32 operator applications */
  int32_t converged;       /* number of rhs that met the tolerance */
  int32_t precond_fallbacks; /* SG_PRECOND: correction solves redone without the preconditioner */
  double max_rel_residual; /* max over rhs of ||b - M x|| / ||b|| (FP64 operator) */
  double seconds;          /* host wall time of the solve call */
  double device_seconds;   /* CUDA-event time of the solve on the context's stream */
} sg_solve_info;

/* GMRES(restart) on the master operator, scipy semantics of the call at
 * smuthi/linearsystem/linear_system.py:285 (x0 = given x, restart default 20, at most 128,
 * stop when ||b - M x|| <= rtol ||b||, explicit residual at every restart).
 * b, x: host buffers n_unknowns x nrhs; x holds x0 on entry and the solution
 * on return. nrhs > 1 runs independent Krylov spaces in lockstep, sharing one
 * block matvec per iteration. precision = SG_FP64 (plain drop-in) or
 * SG_FP32 (mixed: FP32 operator inside FP64 iterative refinement with FP64
 * true residuals and FP64 Arnoldi). maxiter <= 0 selects 10 * n_unknowns. */
int sg_gmres_solve(sg_context *ctx, const double *b, double *x, int nrhs, double rtol, int restart,
                   int maxiter, int precision, sg_solve_info *info);

/* Device-pointer variant of sg_gmres_solve (b, x device buffers). */
int sg_gmres_solve_dev(sg_context *ctx, const void *b, void *x, int nrhs, double rtol, int restart,
                       int maxiter, int precision, sg_solve_info *info, void *stream);

/* ||b - M x|| / ||b|| per rhs with the FP64 operator (host buffers). */
int sg_true_residual(sg_context *ctx, const double *b, const double *x, int nrhs, double *rel_residual);

/* Kernel instrumentation. sg_profile(ctx, 1) brackets every coupling-kernel
 * launch with CUDA events on its stream; sg_kernel_timing synchronises and
 * returns the summed event time (ms) and the number of bracketed launches
 * of the given precision (SG_FP64, SG_FP32, SG_DF64, SG_TF32X3, or -1 for all) since the last
 * reset. sg_launch_count returns the number of kernels this context has
 * launched since it was created. */
int sg_profile(sg_context *ctx, int enable);
int sg_kernel_timing(sg_context *ctx, int precision, double *total_ms, int64_t *count, int reset);
int sg_launch_count(sg_context *ctx, int64_t *count);

/* FP32-operator autotuner result for an RHS count: variant 0 = per-receiver kernel, 1 =
 * interval-bucketed kernel, 2 = pair-symmetric kernel (one interpolation per unordered pair serves
 * both directions; one warp per receiver), 3 = the pair-symmetric kernel with two warps per receiver
 * (each half of the RHS tile), 4 = the tensor-core operator (SG_TF32X3), 5 = the pair-symmetric
 * tensor-core operator (one interpolated block per unordered pair on tcgen05; blocksize <= 32 and
 * 16 or 32 RHS), -1 = not tuned yet; rhs_tile = the chosen kernel's RHS tile per CTA (nrhs for
 * variants 4 and 5); with the CUDA-event times (ms) of one run of the best per-receiver tile, of the
 * bucketed kernel, of the best pair-symmetric tile and of the two tensor-core operators (-1 when not
 * a candidate; any output pointer may be NULL).
 * The first FP32 application for a new RHS count times every candidate on the live operands
 * (synchronising the stream) and keeps the fastest. No counterpart in the reference. */
int sg_fp32_autotune(sg_context *ctx, int nrhs, int *variant, int *rhs_tile, double *ms_receiver,
                     double *ms_bucket, double *ms_symmetric, double *ms_tensor, double *ms_tensor_symmetric);

/* Fixes the FP32 operator for an RHS count instead of timing the candidates: variant 0 =
 * per-receiver kernel (rhs_tile 1, 2, 4, 8 or 16 dividing nrhs), 1 = interval-bucketed kernel
 * (rhs_tile ignored; needs its plan), 2 = pair-symmetric kernel (rhs_tile a power of two dividing
 * nrhs, at most 16 for blocksize <= 32 and 8 for blocksize <= 64), 3 = pair-symmetric kernel with two
 * warps per receiver (the same tiles, at least 4), 4 = tensor-core operator (rhs_tile = nrhs, in
 * {16, 32, 64}; blocksize <= 48), 5 = pair-symmetric tensor-core operator (rhs_tile = nrhs, in
 * {16, 32}; blocksize <= 32). Replaces an earlier choice for
 * that RHS count; set_particles / set_lookup clear it. For tests and measurements of one kernel; no
 * counterpart in the reference. */
int sg_fp32_set_kernel(sg_context *ctx, int nrhs, int variant, int rhs_tile);

/* Emitters accumulated into one tensor-memory accumulator of the tensor-core operator before it is
 * added into the FP32 total (default 8). Fewer emitters bound the tensor core's accumulation error
 * more tightly at the cost of more drains. No counterpart in the reference. */
int sg_tc_set_window(sg_context *ctx, int emitters);

/* FMA throughput (TFLOP/s, 2 flops per FMA) of the FP64 or FP32 pipe of the
 * context's device, measured with a dependent-chain probe kernel. Used to
 * state pipe rooflines; no counterpart in the reference. */
int sg_measure_fma_peak(sg_context *ctx, int precision, double *tflops);

/* Allocation-free FP64 coupling matvec y = W x with linear interpolation, for callers that
 * cannot call cudaMalloc while they compute (code running inside another framework's device
 * memory pool, or loops with a fixed memory budget after start-up). No counterpart in the
 * reference. Every argument is a caller-owned device buffer: xy = double2[n_particles] lateral
 * positions, m_of_n = int32[blocksize], table = complex128[len_rho][blocksize][blocksize] on the
 * grid rho_k = rho_min + k * resolution (the reference layout; it must cover every particle
 * distance), x, y = complex128[n_particles][blocksize][nrhs] (uniform blocks). The call allocates
 * nothing: its scratch is a static 16 MiB device array, so n_particles * blocksize * nrhs must be
 * <= 1048576 and nrhs <= 65535 (larger sizes return SG_ERR_ARG). CUDA loads device code lazily:
 * the first call on a device (and the first after a cudaDeviceReset) loads the code holding the
 * array, which allocates its 16 MiB then and keeps them until exit, and looks its address up. Make
 * that first call at start-up, before a memory pool claims the device and before any stream
 * capture; later calls allocate nothing. `device` must be the current device. Every call shares the
 * array: calls that overlap on the GPU race on it. Asynchronous on `stream` (a cudaStream_t, NULL =
 * legacy default stream). */
int sg_coupling_matvec_linear_noalloc(int device, int n_particles, const void *xy, int blocksize,
                                      const void *m_of_n, int len_rho, double rho_min, double resolution,
                                      const void *table, const void *x, void *y, int nrhs, void *stream);

/* Bessel factors of the layer-mediated lookup table, the GPU part of the table build (the reference
 * evaluates scipy.special.jv on the host inside smuthi/linearsystem/particlecoupling/
 * prepare_lookup.py:343-459): out[n][r][k] = J_n(kappa_k * rho_r) * jac_k for n = 0..nmax
 * (nmax <= 32). kappa, jac: complex128[nk]; rho: float64[nr]; out: complex128[(nmax+1) * nr * nk];
 * all device buffers on the context's device. Asynchronous on `stream` (NULL = context stream). */
int sg_bessel_jac_table(sg_context *ctx, const void *kappa, const void *jac, int nk, const void *rho, int nr,
                        int nmax, void *out, void *stream);

/* Sommerfeld contraction of the layer-mediated lookup table on the GPU (the reference's GPU helper
 * smuthi/linearsystem/particlecoupling/prepare_lookup_cuda.py:55-95, driven at prepare_lookup.py:439-456,
 * integrates each (n1, n2) column over the contour per radial point):
 * out[r * out_stride + cols[j]] = (factor_re + i factor_im) * sum_k a[r][k] * g[k][j] for r < nr,
 * j < ncols. a: complex128[nr][nk] (one order of sg_bessel_jac_table's output), g: complex128[nk][ncols]
 * (integrand times trapezoid weights of the columns of one |m1 - m2|), cols: int32[ncols] output
 * columns, out: complex128 rows of out_stride; all device buffers on the context's device. FP64
 * throughout, the k sum in order. Asynchronous on `stream` (NULL = context stream). */
int sg_lookup_contract(sg_context *ctx, const void *a, int nr, int nk, const void *g, int ncols, const int *cols,
                       double factor_re, double factor_im, void *out, long long out_stride, void *stream);

/* Regular spherical-wave coefficients of plane waves at points (the initial field at every particle
 * for a batch of plane waves; the reference converts each wave per particle on the host:
 * smuthi/initial_field.py:284-329 through smuthi/fields/transformations.py:77-131):
 *   out[q][p][n] = sum_c amp[q][c][n] exp(i (kx (x_p - x0) + ky (y_p - y0) + kz (z_p - z0)))
 * with kr[q][c] = (kx, ky, Re kz, Im kz, x0, y0, z0) for the plane-wave components c (at most 4) of
 * wave q in the points' layer, and amp[q][c][n] the per-index factors of the transformation
 * (4 sum_pol B^dagger(n, pol) e^{-i m alpha} g_pol). Device buffers: xyz float64[n_points][3],
 * kr float64[nwaves][ncomp][7], amp complex128[nwaves][ncomp][blocksize],
 * out complex128[nwaves][n_points][blocksize]. FP64; synchronous on `stream` (NULL = the context's
 * stream). */
int sg_plane_wave_swe(sg_context *ctx, int n_points, const void *xyz, int nwaves, int ncomp, const void *kr,
                      int blocksize, const void *amp, void *out, void *stream);

/* Particle sum of the scattered field's plane-wave expansion for the cross sections (the reference
 * converts each particle's expansion on the host: smuthi/postprocessing/far_field.py:363-427,
 * smuthi/postprocessing/scattered_field.py:80-150, smuthi/fields/transformations.py:133-233):
 *   out[r][p][k][a] = sum_i exp(-i kpar_k (cos alpha_a x_i + sin alpha_a y_i))
 *                     sum_n coef[i][n][r] S[n][p][k] exp(i m_of_n[n] alpha_a)
 * Device buffers: xy double2[n_particles], coef complex128[n_particles][blocksize][nrhs],
 * kpar float64[nk] (real), S complex128[blocksize][2][nk], alpha float64[na],
 * out complex128[nrhs][2][nk][na]; m_of_n is a host array int32[blocksize] with |m| <= m_max <= 16.
 * FP64 throughout. Synchronous on `stream` (NULL = the context's stream). */
int sg_farfield_sum(sg_context *ctx, int n_particles, const void *xy, int blocksize, int nrhs, const void *coef,
                    int m_max, const int32_t *m_of_n, int nk, const void *kpar, const void *S, int na,
                    const void *alpha, void *out, void *stream);

/* Electric (field = 0) or magnetic (field = 1) field of a plane-wave expansion at n_points points,
 * replacing the GPU branches of PlaneWaveExpansion.electric_field / magnetic_field
 * (smuthi/fields/expansions.py:660-708, 734-770; FP32 kernels of smuthi/fields/expansions_cuda.py:5-421):
 *   F(r) = 1/omega_F int dkappa kappa int dalpha sum_pol g_pol(kappa, alpha) Phi_pol e^{i k.r}
 * with the reference's trapezoid rules over the alpha grid and the (complex) kappa contour;
 * omega_F = 1 for E and omega for H. Device buffers: x, y, z float64[n_points] relative to the
 * expansion's reference point; kpar, kz complex128[nk] (kz signed by the expansion's kind: + upgoing,
 * - downgoing); alpha float64[na]; g complex128[2][nk][na] (TE, TM); out complex128[3][n_points]
 * (x, y, z components). k = k_re + i k_im is the medium's wavenumber. nk >= 2, 2 <= na <= 8192.
 * FP64 throughout. Synchronous on `stream` (NULL = the context's stream). */
int sg_pwe_field(sg_context *ctx, int field, int n_points, const void *x, const void *y, const void *z, int nk,
                 const void *kpar, const void *kz, int na, const void *alpha, const void *g, double k_re, double k_im,
                 double omega, void *out, void *stream);

/* The same for particles at different heights: zphase complex128[nk][n_particles] (device) multiplies
 * particle i's term at kpar_k (exp(+-i k_z (z_ref - z_i)) of the up- or downgoing expansion; the
 * reference applies it per particle in smuthi/fields/transformations.py:133-233). NULL = no factor. */
int sg_farfield_sum_heights(sg_context *ctx, int n_particles, const void *xy, int blocksize, int nrhs,
                            const void *coef, int m_max, const int32_t *m_of_n, int nk, const void *kpar,
                            const void *S, int na, const void *alpha, const void *zphase, void *out, void *stream);

/* ---------------------------------------------------------------------------------------------
 * Learned preconditioner for the mixed solve (no counterpart in the reference, whose GMRES call
 * at smuthi/linearsystem/linear_system.py:285 is unpreconditioned). A message-passing network on
 * the k-nearest-neighbour graph of the particles: three layers, each a near-field coupling
 * a = sum_s T_i W_{i,nbr(i,s)} h followed by an MLP (4*blocksize -> 128 -> 2*blocksize, BF16
 * weights, FP32 accumulation), h <- u + alpha a + MLP([a, h]) with u the normalised input. With
 * zero output weights and alpha = 1 it is the Neumann series (I - T W_near)^{-1} ~ I + A + A^2 + A^3.
 * It needs diagonal T-matrices (sg_set_tmatrix, diagonal = 1), uniform blocks and blocksize <= 64.
 * Parameters are one flat float32 vector of sg_precond_param_count(blocksize) entries; per layer
 * W1[128][4B], b1[128], W2[2B][128], b2[2B], alpha[2] (B = blocksize). */
int sg_precond_param_count(int blocksize);

/* Add a graph for the current particles: nbr[i*(k+1) + s], slot 0 = i itself, then k neighbours.
 * Builds the near-field blocks from the lookup coefficients (sg_set_lookup first). Returns its id. */
int sg_precond_add_graph(sg_context *ctx, int k, const int32_t *nbr, int *graph_id);
/* Select the graph used by SG_PRECOND solves and sg_precond_apply_dev (-1 = none). */
int sg_precond_select(sg_context *ctx, int graph_id);
/* Drop every graph (the particle set changed). */
int sg_precond_clear(sg_context *ctx);
int sg_precond_set_params(sg_context *ctx, int blocksize, const float *params, int count);
int sg_precond_get_params(sg_context *ctx, float *params, int count);
/* z = P v for nvec <= 64 vectors (device buffers, reference layout n_unknowns x nvec). */
int sg_precond_apply_dev(sg_context *ctx, const void *v, void *z, int nvec, void *stream);
/* One training step on graph graph_id with nvec <= 64 pairs (v, e = M^{-1} v) (device buffers,
 * reference layout): loss = mean_q ||P(v_q)/|v_q| - e_q/|v_q|||^2 / ||e_q/|v_q|||^2. Writes the loss,
 * the gradient (if grad != NULL, param_count floats) and, when lr > 0, takes an Adam step
 * (beta1 0.9, beta2 0.999, eps 1e-8; step = 1, 2, ... for the bias corrections). Synchronous. */
int sg_precond_train_step(sg_context *ctx, int graph_id, const void *v, const void *e, int nvec, float lr,
                          int step, double *loss, float *grad);
/* Copy a graph's near-field blocks (complex64 [n][k+1][B][B], n2 fastest) to the host. */
int sg_precond_export_blocks(sg_context *ctx, int graph_id, float *blocks);

#ifdef __cplusplus
}
#endif
#endif /* SMUTHI_GB300_H */

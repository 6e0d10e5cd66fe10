// FP64 linear-interpolation coupling matvec that allocates no device memory.
//
// Some callers cannot call cudaMalloc while they compute: code running inside another
// framework's memory pool (which owns all device memory and forbids foreign allocations), or a
// host loop with a fixed memory budget that must not allocate after start-up. For them,
// sg_coupling_matvec_linear_noalloc takes every input and output as caller-owned device buffers
// and keeps its scratch -- the per-split partial sums of the emitter-split coupling kernel -- in
// the file-scope static device array below (16 MiB, held by every device that loads it until the
// process exits). CUDA loads a library's device code lazily: the 16 MiB are allocated when this
// file's code is first loaded onto a device, which is inside the first call of this entry point
// on that device (the address lookup below). A caller whose memory pool claims the device's memory
// must therefore make one call at start-up, before the pool takes the memory and before any stream
// capture; later calls on that device allocate nothing.
//
// The scratch array is shared by all calls: it keeps the last call's contents, every call
// overwrites the part it reads before reading it, and calls whose executions overlap on the GPU
// (different streams, or different host threads) race on it.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "sg_internal.h"

namespace {

constexpr size_t kNoAllocScratchElems = (size_t)1 << 20;  // double2 elements = 16 MiB
static __device__ __align__(256) double2 g_noalloc_scratch[kNoAllocScratchElems];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
struct ScratchAddr {
  void *ctx;     // CUDA context the address belongs to
  double2 *ptr;  // device address of g_noalloc_scratch in that context
};
ScratchAddr g_scratch[kMaxDevices] = {};

// The calling thread's current CUDA context (a driver call, reached through the runtime so that the
// library links only the runtime); null when it cannot be resolved.
void *current_context() {
  typedef int (*GetCurrentFn)(void **);
  static GetCurrentFn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<GetCurrentFn>(f);
  }();
  void *ctx = nullptr;
  if (fn && fn(&ctx) != 0) ctx = nullptr;
  return ctx;
}

// Device address of the static scratch on `device`, which must be current. Looked up once per
// device and context: the first call on a device (or after a cudaDeviceReset replaced its context)
// performs this set-up, which loads the module holding the array.
double2 *scratch_on(int device) {
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  void *ctx = current_context();
  if (g_scratch[device].ptr && ctx && g_scratch[device].ctx == ctx) return g_scratch[device].ptr;
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess)
    throw sg::Error{SG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e)};
  if (ctx == nullptr) ctx = current_context();  // the lookup initialised the context
  g_scratch[device] = {ctx, reinterpret_cast<double2 *>(p)};
  return g_scratch[device].ptr;
}

constexpr int kThreads = 256;

// Partial W x over emitter slice `blockIdx.y` for receiver `blockIdx.x` and RHS `blockIdx.z`,
// linear interpolation read straight from the reference-layout table w[rho][n1][n2].
template <int P>
__global__ void __launch_bounds__(kThreads)
    noalloc_partial_kernel(const double2 *pos, const int *mofn, const double2 *table, int n, int bs, int len_rho,
                           double rho_min, double res, const double2 *x, int nrhs, int nsplit, double2 *scratch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int i = blockIdx.x, split = blockIdx.y, r = blockIdx.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double2 *ubuf = reinterpret_cast<double2 *>(smem_raw) + (size_t)warp * bs;
  double2 *wsum = reinterpret_cast<double2 *>(smem_raw);
  const int j0 = (int)(((long long)n * split) / nsplit), j1 = (int)(((long long)n * (split + 1)) / nsplit);
  const size_t bs2 = (size_t)bs * bs;
  int nrow[P], nrowc[P], mrow[P];
  bool valid[P];
  double acc_re[P], acc_im[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    nrow[q] = lane + 32 * q;
    valid[q] = nrow[q] < bs;
    nrowc[q] = valid[q] ? nrow[q] : bs - 1;
    mrow[q] = mofn[nrowc[q]];
    acc_re[q] = acc_im[q] = 0.0;
  }
  const double xi = pos[i].x, yi = pos[i].y;
  for (int j = j0 + warp; j < j1; j += nw) {
    const double dx = xi - pos[j].x, dy = yi - pos[j].y;
    const double rho = sqrt(dx * dx + dy * dy);
    const double sidx = (rho - rho_min) / res;
    const double fl = floor(sidx);
    int k = (int)fl;
    k = k < 0 ? 0 : (k > len_rho - 2 ? len_rho - 2 : k);
    const double t = sidx - fl;
    double c = 1.0, s = 0.0;
    if (rho > 0.0) {
      c = dx / rho;
      s = dy / rho;
    }
    double ph_re[P], ph_im[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const int am = mrow[q] < 0 ? -mrow[q] : mrow[q];
      double pr = 1.0, pi = 0.0;
      for (int a = 0; a < am; ++a) {
        const double nr = pr * c - pi * s;
        pi = pr * s + pi * c;
        pr = nr;
      }
      ph_re[q] = pr;
      ph_im[q] = mrow[q] < 0 ? -pi : pi;
      if (valid[q]) {
        const double2 xv = x[((size_t)j * bs + nrow[q]) * nrhs + r];
        ubuf[nrow[q]] = make_double2(pr * xv.x - ph_im[q] * xv.y, pr * xv.y + ph_im[q] * xv.x);
      }
    }
    __syncwarp();
    const double2 *t0 = table + (size_t)k * bs2, *t1 = t0 + bs2;
    double pa_re[P], pa_im[P];
#pragma unroll
    for (int q = 0; q < P; ++q) pa_re[q] = pa_im[q] = 0.0;
    for (int n2 = 0; n2 < bs; ++n2) {
      const double2 u = ubuf[n2];
#pragma unroll
      for (int q = 0; q < P; ++q) {
        const size_t e = (size_t)nrowc[q] * bs + n2;
        const double2 a = t0[e], b = t1[e];
        const double lr = fma(t, b.x - a.x, a.x), li = fma(t, b.y - a.y, a.y);
        pa_re[q] = fma(lr, u.x, fma(-li, u.y, pa_re[q]));
        pa_im[q] = fma(lr, u.y, fma(li, u.x, pa_im[q]));
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < P; ++q) {
      acc_re[q] = fma(ph_re[q], pa_re[q], fma(ph_im[q], pa_im[q], acc_re[q]));
      acc_im[q] = fma(ph_re[q], pa_im[q], fma(-ph_im[q], pa_re[q], acc_im[q]));
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < P; ++q)
    if (valid[q]) wsum[(size_t)warp * bs + nrow[q]] = make_double2(acc_re[q], acc_im[q]);
  __syncthreads();
  for (int n1 = threadIdx.x; n1 < bs; n1 += blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int w = 0; w < nw; ++w) {
      sr += wsum[(size_t)w * bs + n1].x;
      si += wsum[(size_t)w * bs + n1].y;
    }
    scratch[(((size_t)split * n + i) * bs + n1) * nrhs + r] = make_double2(sr, si);
  }
}

__global__ void noalloc_reduce_kernel(const double2 *scratch, int n, int bs, int nrhs, int nsplit, double2 *y) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t len = (size_t)n * bs * nrhs;
  if (e >= len) return;
  double sr = 0.0, si = 0.0;
  for (int s = 0; s < nsplit; ++s) {
    const double2 v = scratch[(size_t)s * len + e];
    sr += v.x;
    si += v.y;
  }
  y[e] = make_double2(sr, si);
}

}  // namespace

extern "C" int sg_coupling_matvec_linear_noalloc(int device, int n_particles, const void *xy, int blocksize,
                                                 const void *m_of_n, int len_rho, double rho_min, double resolution,
                                                 const void *table, const void *x, void *y, int nrhs,
                                                 void *stream) {
  sg::clear_error();
  try {
    SG_REQUIRE(n_particles >= 1 && blocksize >= 1 && blocksize <= 96 && nrhs >= 1, "bad sizes");
    SG_REQUIRE(nrhs <= 65535, "nrhs must be <= 65535 (one grid row per right-hand side)");
    SG_REQUIRE(len_rho >= 2 && resolution > 0, "bad lookup grid");
    SG_REQUIRE(xy && m_of_n && table && x && y, "null buffer");
    SG_REQUIRE(device >= 0 && device < kMaxDevices, "device index out of range");
    int current = -1;
    SG_CUDA(cudaGetDevice(&current));
    SG_REQUIRE(current == device, "device must be the calling thread's current CUDA device");
    const size_t len = (size_t)n_particles * blocksize * nrhs;
    if (len > kNoAllocScratchElems)
      throw sg::Error{SG_ERR_ARG, "n_particles * blocksize * nrhs exceeds the 1048576-element (16 MiB) static "
                                  "scratch of sg_coupling_matvec_linear_noalloc"};
    int nsplit = sg::choose_split(n_particles, nrhs);
    const int fit = (int)(kNoAllocScratchElems / len);
    if (nsplit > fit) nsplit = fit;
    if (nsplit < 1) nsplit = 1;
    double2 *scratch = scratch_on(device);
    cudaStream_t st = (cudaStream_t)stream;
    const int P = (blocksize + 31) / 32;
    const size_t smem = (size_t)(kThreads / 32) * blocksize * sizeof(double2);
    dim3 grid(n_particles, nsplit, nrhs);
    const double2 *pos = (const double2 *)xy;
    const double2 *tab = (const double2 *)table;
    const double2 *xv = (const double2 *)x;
    const int *mo = (const int *)m_of_n;
    if (P == 1)
      noalloc_partial_kernel<1><<<grid, kThreads, smem, st>>>(pos, mo, tab, n_particles, blocksize, len_rho, rho_min,
                                                             resolution, xv, nrhs, nsplit, scratch);
    else if (P == 2)
      noalloc_partial_kernel<2><<<grid, kThreads, smem, st>>>(pos, mo, tab, n_particles, blocksize, len_rho, rho_min,
                                                             resolution, xv, nrhs, nsplit, scratch);
    else
      noalloc_partial_kernel<3><<<grid, kThreads, smem, st>>>(pos, mo, tab, n_particles, blocksize, len_rho, rho_min,
                                                             resolution, xv, nrhs, nsplit, scratch);
    SG_CUDA(cudaGetLastError());
    noalloc_reduce_kernel<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(scratch, n_particles, blocksize, nrhs,
                                                                        nsplit, (double2 *)y);
    SG_CUDA(cudaGetLastError());
    return SG_OK;
  } catch (const sg::Error &e) {
    sg::set_error(e.msg);
    return e.code;
  } catch (...) {
    sg::set_error("internal error");
    return SG_ERR_CUDA;
  }
}

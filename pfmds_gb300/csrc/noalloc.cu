// pfmd_rjl_forces_noalloc: rjl forces and energy of a caller-owned system that
// allocate no device memory.
//
// Some callers cannot call cudaMalloc: an MD host code whose device memory is
// all reserved up front by its own pool allocator, or a driver loop that
// interleaves work on several streams and cannot take the device-wide
// synchronisation that cudaMalloc/cudaFree imply.  The context-based API
// (pfmd_create_from_files) allocates its lists and scratch at set-up; this entry
// point takes positions, a neighbour list and output buffers that the caller
// already owns, and keeps the one piece of scratch it needs (1/Eb per atom and
// the per-block energy partials) in a fixed array that is part of the loaded
// library image.
//
// The arithmetic is the plain (FP64) rjl form of forces_rjl.cu
// (RosatoGuillopeLegrand.f90:23-94 of the reference): pass 1 forms
// Eb_i = sqrt(sum exp(-2q(r/r0-1)) fc) and the row energy A0*Er - xi*Eb, pass 2
// gathers F_i -= (a - b (1/Eb_i + 1/Eb_j)) dr with the pair terms recomputed
// (no per-entry cache), pass 3 sums the block partials of the energy in a fixed
// order.
#include <math_constants.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/pfmd.h"
#include "forces.cuh"

namespace pfmd {

// Largest system the entry point accepts.  The scratch array below is sized for
// it: 8 MiB of 1/Eb values plus 32 KiB of block partials, held by every GPU that
// loads the library until the process exits.
static constexpr int kNoAllocMaxAtoms = 1 << 20;
static constexpr int kNoAllocBlock = 256;
static constexpr int kNoAllocMaxBlocks = kNoAllocMaxAtoms / kNoAllocBlock;

// [0, kNoAllocMaxAtoms): 1/Eb per atom; then kNoAllocMaxBlocks energy partials.
// Every call writes each value it later reads, so nothing here needs clearing.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxAtoms + kNoAllocMaxBlocks];

static constexpr int kNoAllocMaxDevices = 64;
// The address is cached per device together with the id of the CUDA context it
// was looked up in: a device reset, or a caller's own driver-API context, makes
// the next call look it up again in the context that is current then.
static double* g_noalloc_ptr[kNoAllocMaxDevices] = {};
static unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};
static std::mutex g_noalloc_mu;

__device__ __forceinline__ double4_32a na_pos(const double* __restrict__ pos, int i) {
  return make_double4_32a(pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2], 0.0);
}

// One thread per atom.  Counts above max_nbr are cut to max_nbr and entries
// outside [0, n) are skipped, so a malformed list cannot read out of bounds; a
// cut row gets NaN for its 1/Eb and its energy, so the error shows in the
// energy and in the forces of the row and of its partners.
__global__ void __launch_bounds__(kNoAllocBlock)
    k_na_rjl_density(int n, const double* __restrict__ pos, Box B, RJLc<double> c, const int* __restrict__ nnum,
                     const int* __restrict__ nbr, int max_nbr, double* __restrict__ scratch, int energy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double erow[1] = {0.0};
  if (i < n) {
    const double4_32a pi = na_pos(pos, i);
    const int m = min(max(nnum[i], 0), max_nbr);
    const int* row = nbr + (size_t)i * max_nbr;
    double eb2 = 0.0, er = 0.0;
    for (int p = 0; p < m; ++p) {
      const int j = row[p];
      if ((unsigned)j >= (unsigned)n) continue;
      double dr[3];
      const double r = sqrt(mi_exact(pi, na_pos(pos, j), B, dr));
      if (r <= c.R2) {
        double fc, dfc;
        fdfcut_cos(r, c.R1, c.R2, fc, dfc);
        const double x = r * c.inv_r0 - 1.0;
        eb2 += exp(c.m2q * x) * fc;
        er += exp(c.mp * x) * fc;
      }
    }
    const double eb = sqrt(eb2);
    const bool cut = nnum[i] > max_nbr;
    scratch[i] = cut ? CUDART_NAN : 1.0 / eb;
    erow[0] = cut ? CUDART_NAN : c.A0 * er - c.xi * eb;
  }
  if (energy) {
    block_sum<1>(erow);
    if (threadIdx.x == 0) scratch[kNoAllocMaxAtoms + blockIdx.x] = erow[0];
  }
}

__global__ void __launch_bounds__(kNoAllocBlock)
    k_na_rjl_force(int n, const double* __restrict__ pos, Box B, RJLc<double> c, const int* __restrict__ nnum,
                   const int* __restrict__ nbr, int max_nbr, const double* __restrict__ scratch,
                   double* __restrict__ frc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a pi = na_pos(pos, i);
  const int m = min(max(nnum[i], 0), max_nbr);
  const int* row = nbr + (size_t)i * max_nbr;
  const double ieb_i = scratch[i];
  double f[3] = {0.0, 0.0, 0.0};
  for (int p = 0; p < m; ++p) {
    const int j = row[p];
    if ((unsigned)j >= (unsigned)n) continue;
    double dr[3];
    const double r = sqrt(mi_exact(pi, na_pos(pos, j), B, dr));
    if (r <= c.R2) {
      double fc, dfc;
      fdfcut_cos(r, c.R1, c.R2, fc, dfc);
      const double x = r * c.inv_r0 - 1.0;
      const double ep = exp(c.mp * x), eq = exp(c.m2q * x), ir = 1.0 / r;
      const double a = c.a2 * (c.pr0 * fc - dfc * r) * ep * ir;
      const double b = c.xi * (c.qr0 * fc - dfc * 0.5 * r) * eq * ir;
      const double k = a - b * (ieb_i + scratch[j]);
      f[0] -= k * dr[0];
      f[1] -= k * dr[1];
      f[2] -= k * dr[2];
    }
  }
  if (nnum[i] > max_nbr) f[0] = f[1] = f[2] = CUDART_NAN;  // a cut row
  frc[3 * (size_t)i] = f[0];
  frc[3 * (size_t)i + 1] = f[1];
  frc[3 * (size_t)i + 2] = f[2];
}

// One block: thread t sums partials t, t + blockDim.x, ..., then the block tree.
__global__ void __launch_bounds__(kNoAllocBlock)
    k_na_energy(int blocks, const double* __restrict__ scratch, double* __restrict__ energy) {
  double v[1] = {0.0};
  for (int b = threadIdx.x; b < blocks; b += blockDim.x) v[0] += scratch[kNoAllocMaxAtoms + b];
  block_sum<1>(v);
  if (threadIdx.x == 0) *energy = v[0];
}

// Id of the CUDA context current on this thread (0 when none is), through the
// driver entry point the runtime hands out; no driver library is linked.
static unsigned long long current_ctx_id() {
  using GetCur = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCur get_cur = nullptr;
  static GetId get_id = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<GetCur>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_cur && get_id && get_cur(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of the scratch array in the current device's current context,
// looked up once per device and context.  Host code cannot use
// g_noalloc_scratch's name as a device pointer.
static cudaError_t noalloc_scratch(double** out, int* dev) {
  cudaError_t err = cudaGetDevice(dev);
  if (err != cudaSuccess) return err;
  if (*dev < 0 || *dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  unsigned long long ctx = current_ctx_id();
  if (!g_noalloc_ptr[*dev] || ctx == 0 || ctx != g_noalloc_ctx[*dev]) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess) return err;
    g_noalloc_ptr[*dev] = static_cast<double*>(p);
    g_noalloc_ctx[*dev] = ctx ? ctx : current_ctx_id();  // the lookup made the primary context current
  }
  *out = g_noalloc_ptr[*dev];
  return cudaSuccess;
}

}  // namespace pfmd

static int na_fail(char* err, int err_len, int code, const char* fmt, ...) __attribute__((format(printf, 4, 5)));
static int na_fail(char* err, int err_len, int code, const char* fmt, ...) {
  if (err && err_len > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, static_cast<size_t>(err_len), fmt, ap);
    va_end(ap);
  }
  return code;
}

extern "C" int pfmd_rjl_forces_noalloc(int n_atoms, const double* pos, const double box[3], const double params[7],
                                       const int* nnum, const int* nbr, int max_nbr, double* frc, double* energy,
                                       void* stream, char* err, int err_len) {
  using namespace pfmd;
  if (err && err_len > 0) err[0] = '\0';
  if (n_atoms < 0 || n_atoms > kNoAllocMaxAtoms)
    return na_fail(err, err_len, PFMD_E_PARAM,
                   "pfmd_rjl_forces_noalloc: n_atoms = %d is outside 0..%d, the size of its fixed scratch", n_atoms,
                   kNoAllocMaxAtoms);
  if (max_nbr < 0) return na_fail(err, err_len, PFMD_E_PARAM, "pfmd_rjl_forces_noalloc: max_nbr = %d < 0", max_nbr);
  if (!box || !params) return na_fail(err, err_len, PFMD_E_PARAM, "pfmd_rjl_forces_noalloc: box or params is NULL");
  if (n_atoms > 0 && (!pos || !nnum || !frc || (max_nbr > 0 && !nbr)))
    return na_fail(err, err_len, PFMD_E_PARAM, "pfmd_rjl_forces_noalloc: a device buffer is NULL");
  for (int k = 0; k < 3; ++k)
    if (!(box[k] > 0.0)) return na_fail(err, err_len, PFMD_E_PARAM, "pfmd_rjl_forces_noalloc: box[%d] <= 0", k);
  if (!(params[4] > 0.0) || !(params[6] > params[5]))
    return na_fail(err, err_len, PFMD_E_PARAM, "pfmd_rjl_forces_noalloc: need r0 > 0 and R2 > R1");

  // an error left by the caller's earlier work is reported as such (and not
  // cleared), not as a failure of this call's launches
  cudaError_t ce = cudaPeekAtLastError();
  if (ce != cudaSuccess)
    return na_fail(err, err_len, PFMD_E_CUDA, "pfmd_rjl_forces_noalloc: a CUDA error was pending before the call: %s",
                   cudaGetErrorString(ce));
  double* scratch = nullptr;
  int dev = -1;
  ce = noalloc_scratch(&scratch, &dev);
  if (ce != cudaSuccess)
    return na_fail(err, err_len, PFMD_E_CUDA, "pfmd_rjl_forces_noalloc: scratch address on device %d: %s", dev,
                   cudaGetErrorString(ce));

  RJLPar P{params[0], params[1], params[2], params[3], params[4], params[5], params[6], {}, {}};
  derive(P);
  Box B{};
  for (int k = 0; k < 3; ++k) {
    B.L[k] = box[k];
    B.h[k] = 0.5 * box[k];
    B.qinv[k] = 4294967296.0 / box[k];
    B.qs[k] = static_cast<float>(box[k] / 4294967296.0);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n_atoms == 0) {
    if (energy) ce = cudaMemsetAsync(energy, 0, sizeof(double), s);
  } else {
    const int blocks = (n_atoms + kNoAllocBlock - 1) / kNoAllocBlock;
    k_na_rjl_density<<<blocks, kNoAllocBlock, 0, s>>>(n_atoms, pos, B, P.d, nnum, nbr, max_nbr, scratch,
                                                      energy ? 1 : 0);
    k_na_rjl_force<<<blocks, kNoAllocBlock, 0, s>>>(n_atoms, pos, B, P.d, nnum, nbr, max_nbr, scratch, frc);
    if (energy) k_na_energy<<<1, kNoAllocBlock, 0, s>>>(blocks, scratch, energy);
    ce = cudaGetLastError();
  }
  if (ce != cudaSuccess)
    return na_fail(err, err_len, PFMD_E_CUDA, "pfmd_rjl_forces_noalloc: launch: %s", cudaGetErrorString(ce));
  return PFMD_OK;
}

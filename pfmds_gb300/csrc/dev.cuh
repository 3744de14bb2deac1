// Device-side building blocks shared by the PFMDS kernels (sm_103a).
//
// * Box / minimum image: find_distance of md_general.f90:423-441 in two forms.
//   mi_exact evaluates the reference expression with round-to-nearest intrinsics
//   (no FMA contraction), so d r^2 and the list predicate `dr2 < r_cut*r_cut`
//   (md_neighbours.f90:77) come out bit for bit as in an uncontracted FP64 build.
//   mi_f32 is the same formula in FP32 for the precision form.
// * Cut-off switches of cut_off_function.f90 (cosine, truncated pi) and
//   cut_off_poly.f90 (quintic, f_dfr_cut with its missing 1/(R2-R1)).
// * Ctl: the device-resident control block (status, step counter, energies,
//   reduction scratch) that lets a whole step sequence run without the host.
// * Deterministic grid reductions: per-block partials, the last block to finish
//   sums them in block order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifndef PFMD_MAX_INTER
#define PFMD_MAX_INTER 16
#endif
#define PFMD_MAX_LISTS (3 * PFMD_MAX_INTER)
#define PFMD_MAX_GROUPS 64
#define PFMD_MAX_NHC 8
#define PFMD_MAX_CHAIN 16
#define PFMD_RED_SLOTS 32
#define PFMD_PARTIALS (1 << 16)

namespace pfmd {

// status codes (include/pfmd.h)
enum : int {
  ST_OK = 0,
  ST_NLIST_OVERFLOW = 1,
  ST_OUT_OF_CELL = 2,
  ST_GR_NN = 3,
  ST_PARAM = 4,
  ST_CUDA = 5,
  ST_TIMEOUT = 6
};

// Error detail kinds recorded next to the status code.
enum : int {
  EK_NONE = 0,
  EK_OVERFLOW = 1,      // info: list id, row (1-based), count
  EK_OOB = 2,           // info: atom (1-based)
  EK_GR_TOO_MANY = 3,   // info: row (1-based)
  EK_GR_NOT_ENOUGH = 4, // info: row (1-based)
  EK_L1 = 5,            // 'l1>3'
  EK_CONVERSE_OVF = 6,  // info: list id, row (1-based), count
  EK_NMAX_CAP = 7       // nmax above the build kernel's capacity
};

struct NHCDev {
  int M, L;
  double T, s, e;
  double x[PFMD_MAX_CHAIN], v[PFMD_MAX_CHAIN], q[PFMD_MAX_CHAIN];
  double iq[PFMD_MAX_CHAIN];  // 1/q, formed on the host
};

// Control block in device memory.  The host reads it back after a segment.
struct Ctl {
  // status: `stop` is non-zero once an error or the nvms exit happened; every
  // kernel returns immediately when it is set.
  int stop;
  int error;
  int err_kind;
  int err_info[3];
  long long err_step;
  int pending_oob;  // an atom left the cell in the last drift; checked at step start
  int oob_atom;     // smallest offending atom (0-based) of the pending check
  int converged;    // nvms exit
  // the same flag for a drift fused into the previous step's force kernel, by the
  // parity of the step it begins (the kernel that sets one slot tests the other)
  int pending_fused[2];
  int pad0;
  long long md_step;  // the step being executed
  // energies
  double pe_last, pe_prev;
  double e_inter[PFMD_MAX_INTER];
  double ke, temperature, e_nhc, total, conserved;
  // group sizes (device resident so captured graphs survive group changes)
  int group_n[PFMD_MAX_GROUPS];
  // Nose-Hoover chains
  NHCDev nhc[PFMD_MAX_NHC];
  // chain 0's second-half scale when the pair kernel also ran the next step's
  // first half: the next kick-drift applies it, then nhc[0].s
  double nhc_sa;
  // small reduction results
  double red[PFMD_RED_SLOTS];
  int maxnnum[PFMD_MAX_LISTS];
  // skin-triggered rebuilds (precision form): list_need[id] is 1 when list id must
  // be rebuilt at its next update step; skin_done counts the blocks of the kernel
  // that records a rebuild
  int list_need[PFMD_MAX_LISTS];
  // two-level lists: outer_need[id] is 1 when list id's outer list (a wider list
  // its rows are filtered from) must be rebuilt too
  int outer_need[PFMD_MAX_LISTS];
  unsigned int skin_done[PFMD_MAX_LISTS];
  // squared displacements (float bits): since the build, over the last period,
  // since the outer list's build
  unsigned int skin_max[PFMD_MAX_LISTS][3];
  long long list_builds[PFMD_MAX_LISTS];     // rebuilds of each skin-managed list
  unsigned int counter[PFMD_RED_SLOTS];
  double partial[PFMD_PARTIALS];  // per-block partial sums of the grid reductions
};

// An out-of-cell verdict of the last drift waits to be raised.
__device__ __forceinline__ bool oob_pending(const Ctl* ctl) {
  return ctl->pending_oob || ctl->pending_fused[0] || ctl->pending_fused[1];
}

// Velocity Verlet pieces shared by the integration kernels and the fused force
// epilogue.  kt = dt/2/(m*mass_coef) formed once per atom: one FMA per component.
__device__ __forceinline__ double kick1_fast(double v, double f, double kt) { return fma(f, kt, v); }
// One shift back into [0, L] (md_integrators.f90:19-24): x > L and x < 0.0 decided
// on the bit patterns (L > 0; the patterns of x >= +0 order like the values,
// x < 0.0 is a set sign bit other than -0.0).  NaN stays NaN either way.
__device__ __forceinline__ double wrap1(double x, double L) {
  const long long b = __double_as_longlong(x);
  if (b > __double_as_longlong(L))
    x = x - L;
  else if (b < 0 && b != (long long)0x8000000000000000ULL)
    x = x + L;
  return x;
}
// the precision form's drift: one FMA, then the shift
__device__ __forceinline__ double drift1_fast(double x, double v, double ts1, double L) {
  return wrap1(fma(v, ts1, x), L);
}
// !(x > -tol .and. x < L + tol) with tol = 1e-7 (md_general.f90:346), evaluated
// on the bit patterns with integer compares (GB300's FP64 pipe is narrow).  For
// x >= +0 the patterns order like the values; a negative x (sign bit set, -0.0
// included) is inside iff its magnitude is below tol.  NaN is outside either way.
__device__ __forceinline__ bool out_of_cell(double x, double Ltol) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b >= __double_as_longlong(Ltol)
                : (unsigned long long)b >= (unsigned long long)__double_as_longlong(-0.0000001);
}

// A skin-managed list whose atoms all stayed within half the skin since its last
// build keeps its rows: its build kernels return at once.
// A list's rebuild kernels return at once when the skin test keeps it: skin is
// the list's id, or PFMD_MAX_LISTS + id for the outer list of list id.
__device__ __forceinline__ bool skin_keep(const Ctl* ctl, int skin) {
  if (skin < 0) return false;
  return skin >= PFMD_MAX_LISTS ? ctl->outer_need[skin - PFMD_MAX_LISTS] == 0 : ctl->list_need[skin] == 0;
}

// Box lengths, halves, and the fixed-point scales of the force-side positions:
// a coordinate is stored as round(x * 2^32 / L) modulo 2^32 (posq), so the
// difference of two stored coordinates, taken modulo 2^32 as a signed 32-bit
// integer, is the minimum-image separation in units of L / 2^32.
struct Box {
  double L[3], h[3];
  double qinv[3];  // 2^32 / L
  float qs[3];     // L / 2^32
  double Ltol[3];  // L + 1e-7, the upper bound of the out-of-cell test (md_general.f90:346)
  // 2^32 / L as qm * 2^(qe - 64) with qm in [2^63, 2^64): quantize_int's reciprocal
  unsigned long long qm[3];
  int qe[3];
};

// ---------------------------------------------------------------------------
// minimum image
// ---------------------------------------------------------------------------

// d - h*(sign(1,d-h)+sign(1,d+h)), rounded exactly as written.  The sum of
// signs is 2 when d >= h, -2 when d < -h and 0 otherwise (a rounded d -+ h is
// zero only when exactly zero, and otherwise keeps its sign), and h*2 is exact,
// so the expression is d - 2h, d + 2h or d itself, bit for bit.  The two
// comparisons run on the doubles' bit patterns as integers (h > 0: the order of
// non-negative doubles is that of their patterns), which leaves one FP64 add per
// axis on this GPU's narrow FP64 pipe instead of five operations.
__device__ __forceinline__ double mi_axis_exact(double d, double h) {
  const long long bd = __double_as_longlong(d), bh = __double_as_longlong(h);
  const bool up = bd >= bh;                                    // d >= h
  const bool dn = bd < 0 && (bd & 0x7FFFFFFFFFFFFFFFLL) > bh;  // d < -h
  const double w = up ? -(h + h) : (h + h);
  const double r = __dadd_rn(d, w);
  return (up || dn) ? r : d;
}
// dr = b - a with the minimum image; returns dr.dr evaluated as
// (dx*dx + dy*dy) + dz*dz without contraction.
__device__ __forceinline__ double mi_exact(const double4_32a& a, const double4_32a& b, const Box& B, double dr[3]) {
  dr[0] = mi_axis_exact(__dsub_rn(b.x, a.x), B.h[0]);
  dr[1] = mi_axis_exact(__dsub_rn(b.y, a.y), B.h[1]);
  dr[2] = mi_axis_exact(__dsub_rn(b.z, a.z), B.h[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(dr[0], dr[0]), __dmul_rn(dr[1], dr[1])), __dmul_rn(dr[2], dr[2]));
}
// Fixed-point coordinate of x (wraps modulo 2^32, i.e. periodically).
__device__ __forceinline__ int quantize(double x, double qinv) {
  return (int)(unsigned int)(unsigned long long)__double2ll_rn(x * qinv);
}
// The same fixed-point coordinate from integer arithmetic on the double's bits,
// for kernels bound by GB300's narrow FP64 pipe: with x = m 2^(e-1075) (m the
// 53-bit significand) and 2^32/L = qm 2^(qe-64), x 2^32/L = (m qm / 2^64) 2^(e+qe-1075);
// the high word of m*qm is one 64x64 integer multiply.  Rounds half up on the
// truncated product, so it can differ from quantize() by one unit (L/2^32) at
// near-ties; callers use one or the other consistently per run.
__device__ __forceinline__ int quantize_int(double x, const Box& B, int k) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0;
  const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const unsigned long long hi = __umul64hi(m, B.qm[k]);
  const int sh = e + B.qe[k] - 1075;
  unsigned long long r;
  if (sh >= 0)
    r = sh < 64 ? hi << sh : 0ull;
  else if (sh > -64)
    r = (hi + (1ull << (-sh - 1))) >> (-sh);
  else
    r = 0ull;
  const unsigned int u = (unsigned int)r;
  return (int)(b < 0 ? 0u - u : u);
}

// Minimum-image b - a from fixed-point coordinates, in FP32 (precision form and
// the list-build prefilter).  Resolution L / 2^32; the relative error of dr is
// that of one int->float conversion and one multiply.
__device__ __forceinline__ float mi_q(const int4& a, const int4& b, const Box& B, float dr[3]) {
  dr[0] = (float)(int)((unsigned int)b.x - (unsigned int)a.x) * B.qs[0];
  dr[1] = (float)(int)((unsigned int)b.y - (unsigned int)a.y) * B.qs[1];
  dr[2] = (float)(int)((unsigned int)b.z - (unsigned int)a.z) * B.qs[2];
  return dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
}
// Cell of a fixed-point coordinate on a grid of nc cells: floor(frac * nc), exact.
__device__ __forceinline__ int cell_q(int xq, int nc) {
  return (int)(((unsigned long long)(unsigned int)xq * (unsigned long long)nc) >> 32);
}

// ---------------------------------------------------------------------------
// cut-off switches
// ---------------------------------------------------------------------------
#define PFMD_PI_TRUNC 3.14159265358979

// cut_off_function.f90:6-16
__device__ __forceinline__ double fcut_cos(double r, double R1, double R2) {
  if (r < R1) return 1.0;
  if (r < R2) return (1.0 + cos(PFMD_PI_TRUNC * (r - R1) / (R2 - R1))) * 0.5;
  return 0.0;
}
// cut_off_function.f90:18-28 (returns f'/r)
__device__ __forceinline__ double dfcut_cos(double r, double R1, double R2) {
  if (r < R1) return 0.0;
  if (r < R2) return -sin(PFMD_PI_TRUNC * (r - R1) / (R2 - R1)) * PFMD_PI_TRUNC / (R2 - R1) / r * 0.5;
  return 0.0;
}
// both at once: fc and f'/r
__device__ __forceinline__ void fdfcut_cos(double r, double R1, double R2, double& f, double& df) {
  if (r < R1) {
    f = 1.0;
    df = 0.0;
  } else if (r < R2) {
    double s, c;
    sincos(PFMD_PI_TRUNC * (r - R1) / (R2 - R1), &s, &c);
    f = (1.0 + c) * 0.5;
    df = -s * PFMD_PI_TRUNC / (R2 - R1) / r * 0.5;
  } else {
    f = 0.0;
    df = 0.0;
  }
}
// The same switch for the FP64 kernels without FP64 divides (each a
// multi-instruction sequence on this GPU's narrow FP64 pipe): the argument as
// (r - R1) inv_w with inv_w = 1/(R2 - R1) formed on the host, f'/r through the
// caller's 1/r, and sin and cos of pi_t x as sincospi of x pi_t/pi (its
// reduction is exact).  The results differ from the divided form in the last
// bits only.
constexpr double kPiTruncOverPi = PFMD_PI_TRUNC / 3.14159265358979323846;
__device__ __forceinline__ double fcut_cos_w(double r, double R1, double R2, double inv_w) {
  if (r < R1) return 1.0;
  if (r < R2) return (1.0 + cospi((r - R1) * inv_w * kPiTruncOverPi)) * 0.5;
  return 0.0;
}
__device__ __forceinline__ void fdfcut_cos_w(double r, double ir, double R1, double R2, double inv_w, double& f,
                                             double& df) {
  if (r < R1) {
    f = 1.0;
    df = 0.0;
  } else if (r < R2) {
    double s, c;
    sincospi((r - R1) * inv_w * kPiTruncOverPi, &s, &c);
    f = (1.0 + c) * 0.5;
    df = -s * (0.5 * PFMD_PI_TRUNC) * inv_w * ir;
  } else {
    f = 0.0;
    df = 0.0;
  }
}
__device__ __forceinline__ void fdfcut_cos_f(float r, float R1, float R2, float inv_w, float& f, float& df) {
  if (r < R1) {
    f = 1.0f;
    df = 0.0f;
  } else if (r < R2) {
    float s, c;
    __sincosf(3.14159265358979f * (r - R1) * inv_w, &s, &c);
    f = (1.0f + c) * 0.5f;
    df = -s * 3.14159265358979f * inv_w / r * 0.5f;
  } else {
    f = 0.0f;
    df = 0.0f;
  }
}
// The same switch with r*df in place of df (no divide): f and r*df/dr.
__device__ __forceinline__ void fdfrcut_cos_f(float r, float R1, float R2, float inv_w, float& f, float& rdf) {
  if (r < R1) {
    f = 1.0f;
    rdf = 0.0f;
  } else if (r < R2) {
    float s, c;
    __sincosf(3.14159265358979f * (r - R1) * inv_w, &s, &c);
    f = (1.0f + c) * 0.5f;
    rdf = -s * 3.14159265358979f * inv_w * 0.5f;
  } else {
    f = 0.0f;
    rdf = 0.0f;
  }
}
// cut_off_poly.f90:6-17
__device__ __forceinline__ double fcut_poly(double r, double R1, double R2) {
  if (r > R1 && r < R2) {
    double a = r - R1, w = R2 - R1;
    double a3 = a * a * a, w2 = w * w;
    return 1.0 + (-10.0 * a3 * w2 + 15.0 * (a3 * a) * w - 6.0 * (a3 * a * a)) / (w2 * w2 * w);
  }
  if (r <= R1) return 1.0;
  return 0.0;
}
// cut_off_poly.f90:30-43 (dfr lacks 1/(R2-R1), as in the reference); x as
// (t - R1) inv_w with inv_w = 1/(R2 - R1) formed on the host (no divide)
template <class T>
__device__ __forceinline__ void f_dfr_cut(T r, T R1, T R2, T inv_w, T& f, T& dfr) {
  T t = r < R1 ? R1 : r;
  t = t > R2 ? R2 : t;
  T x = (t - R1) * inv_w;
  T x2 = x * x;
  f = T(1) + x2 * x * (T(-10) + T(15) * x - T(6) * x2);
  dfr = t * x2 * (T(-30) + T(60) * x - T(30) * x2);
}

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sums K values over the block; result valid in thread 0.  blockDim.x <= 1024.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K]) {
  __shared__ double sh[K][32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][w] = v[k];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double t = lane < nw ? sh[k][lane] : 0.0;
      v[k] = warp_sum(t);
    }
  }
}

// Grid-wide deterministic sum of K doubles per block.  Every block calls it with
// its block-partial values; returns true in thread 0 of the last block to arrive,
// with out[k] holding the grid totals.  The last block sums the partials with all
// its threads: thread t takes partials t, t + blockDim.x, ... in order, then the
// block tree sums those -- a fixed order, so the result does not depend on which
// block arrived last.  `slot` selects the arrival counter; the last block resets
// it, so graphs can replay the kernel.
template <int K>
__device__ __forceinline__ bool grid_finish(Ctl* ctl, int slot, double (&v)[K], double (&out)[K]);
template <int K>
__device__ __forceinline__ bool grid_sum(Ctl* ctl, int slot, double (&v)[K], double (&out)[K]) {
  block_sum<K>(v);
  return grid_finish<K>(ctl, slot, v, out);
}
// grid_sum from block totals already formed (valid in thread 0); every thread of
// every block calls it.
template <int K>
__device__ __forceinline__ bool grid_finish(Ctl* ctl, int slot, double (&v)[K], double (&out)[K]) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) ctl->partial[(size_t)blockIdx.x * K + k] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(&ctl->counter[slot], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double w[K];
#pragma unroll
  for (int k = 0; k < K; ++k) w[k] = 0.0;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < K; ++k) w[k] += ((volatile double*)ctl->partial)[(size_t)b * K + k];
  __syncthreads();  // block_sum's shared scratch is reused
  block_sum<K>(w);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = w[k];
    ctl->counter[slot] = 0u;
  }
  return threadIdx.x == 0;
}

// Ctl::stop as one verdict for the whole block (it is a block barrier): a kernel
// with block barriers after its stop test uses it, so that no warp of a block
// returns while another goes on to a barrier after a thread of this grid set
// the flag in between their reads.  Every thread of the block calls it.
__device__ __forceinline__ bool block_stop(const Ctl* ctl) {
  return __syncthreads_or(*reinterpret_cast<const volatile int*>(&ctl->stop) != 0) != 0;
}

// Records the first error (later ones are dropped) at md_step `step` and stops
// the device step loop.
__device__ __forceinline__ void set_error_at(Ctl* ctl, int code, int kind, int a, int b, int c, long long step) {
  if (atomicCAS(&ctl->error, 0, code) == 0) {
    ctl->err_kind = kind;
    ctl->err_info[0] = a;
    ctl->err_info[1] = b;
    ctl->err_info[2] = c;
    ctl->err_step = step;
  }
  ctl->stop = 1;
}
__device__ __forceinline__ void set_error(Ctl* ctl, int code, int kind, int a, int b, int c) {
  set_error_at(ctl, code, kind, a, b, c, ctl->md_step);
}

// Kahan-compensated accumulation (precision form).
struct Kahan3 {
  float s[3], c[3];
  __device__ __forceinline__ Kahan3() {
    s[0] = s[1] = s[2] = 0.f;
    c[0] = c[1] = c[2] = 0.f;
  }
  __device__ __forceinline__ void add(float x, float y, float z) {
    float in[3] = {x, y, z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float yk = in[k] - c[k];
      float t = s[k] + yk;
      c[k] = (t - s[k]) - yk;
      s[k] = t;
    }
  }
  __device__ __forceinline__ double get(int k) const { return (double)s[k] - (double)c[k]; }
};

}  // namespace pfmd

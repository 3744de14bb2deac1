// Shared pieces of the force kernels (forces_*.cu).
//
// Every force kernel is a full-list gather: TPA threads own one list row (one
// thread per row for large systems), split its entries, recompute the
// minimum-image vector to each partner from positions (the reference stores it
// per entry and refreshes it every step, md_neighbours.f90:104-124), reduce the
// row's force across the group and add it to the row's atom once.  No atomics.
// Energies are folded into the force pass at energy steps and reduced
// deterministically.
//
// PREC=false: FP64 throughout; tests like `r < R2` use the exact FP64 distance,
// so the set of interacting pairs equals the reference's.
// PREC=true : the precision form -- separations from the fixed-point positions,
// FP32 pair terms, per-thread Kahan sums merged across the group with an
// error-free TwoSum, FP64 per-atom force update and FP64 energy reduction.
#pragma once

#include <type_traits>

#include "kernels.h"

namespace pfmd {

template <bool PREC>
struct RT;
template <>
struct RT<false> {
  using R = double;
  using P4 = double4_32a;
  static __device__ __forceinline__ P4 load(const Atoms& A, int i) { return A.pos[i]; }
  // the exact minimum image (as the lists use it); r^2 with fused multiply-adds
  // (two FP64 instructions fewer than the uncontracted sum the list predicate
  // needs; the forces differ from it in the last bits only)
  static __device__ __forceinline__ R d2(const P4& a, const P4& b, const Box& B, R dr[3]) {
    dr[0] = mi_axis_exact(__dsub_rn(b.x, a.x), B.h[0]);
    dr[1] = mi_axis_exact(__dsub_rn(b.y, a.y), B.h[1]);
    dr[2] = mi_axis_exact(__dsub_rn(b.z, a.z), B.h[2]);
    return fma(dr[2], dr[2], fma(dr[1], dr[1], dr[0] * dr[0]));
  }
};
template <>
struct RT<true> {
  using R = float;
  using P4 = int4;
  static __device__ __forceinline__ P4 load(const Atoms& A, int i) { return A.posq[i]; }
  static __device__ __forceinline__ R d2(const P4& a, const P4& b, const Box& B, R dr[3]) {
    return mi_q(a, b, B, dr);
  }
};

// Rows are spread over the lanes of a warp so that consecutive rows sit on
// consecutive lanes: a warp holds 32/TPA rows, and the TPA threads of a row are
// lanes r, r + 32/TPA, r + 2*32/TPA, ...  Thread `sub` of a row takes slots
// sub, sub + TPA, ...; its partial sums are combined by xor-shuffles over
// offsets 16, 8, ..., 32/TPA.
template <int TPA>
struct Grp {
  int row, sub;
  __device__ __forceinline__ Grp() {
    constexpr int RPW = 32 / TPA;  // rows per warp
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = g & 31;
    row = (g >> 5) * RPW + (lane % RPW);
    sub = lane / RPW;
  }
};
template <int TPA>
__device__ __forceinline__ double gsum(double v) {
#pragma unroll
  for (int o = 16; o >= 32 / TPA; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Compensated merge of per-lane Kahan pairs (value = s - c) across the group:
// TwoSum(s1, s2) = t + e exactly, so (s1 - c1) + (s2 - c2) = t - (c1 + c2 - e).
template <int TPA>
__device__ __forceinline__ void gmerge(float& s, float& c) {
#pragma unroll
  for (int o = 16; o >= 32 / TPA; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
    const float t = s + s2;
    const float bb = t - s;
    const float e = (s - (t - bb)) + (s2 - bb);
    c = (c + c2) - e;
    s = t;
  }
}

// Per-thread accumulators: plain FP64, or FP32 with Kahan compensation.
template <bool PREC>
struct Acc3;
template <>
struct Acc3<false> {
  double s[3] = {0.0, 0.0, 0.0};
  __device__ __forceinline__ void add(double x, double y, double z) {
    s[0] += x;
    s[1] += y;
    s[2] += z;
  }
  template <int TPA>
  __device__ __forceinline__ void reduce() {
#pragma unroll
    for (int k = 0; k < 3; ++k) s[k] = gsum<TPA>(s[k]);
  }
  __device__ __forceinline__ double get(int k) const { return s[k]; }
};
template <>
struct Acc3<true> {
  Kahan3 k;
  __device__ __forceinline__ void add(float x, float y, float z) { k.add(x, y, z); }
  template <int TPA>
  __device__ __forceinline__ void reduce() {
#pragma unroll
    for (int c = 0; c < 3; ++c) gmerge<TPA>(k.s[c], k.c[c]);
  }
  // the compensated sum rounded to FP32 (one conversion to FP64 per component)
  __device__ __forceinline__ double get(int c) const { return (double)(k.s[c] - k.c[c]); }
};
template <bool PREC>
struct Acc1;
template <>
struct Acc1<false> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  template <int TPA>
  __device__ __forceinline__ void reduce() {
    s = gsum<TPA>(s);
  }
  __device__ __forceinline__ double get() const { return s; }
};
template <>
struct Acc1<true> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  template <int TPA>
  __device__ __forceinline__ void reduce() {
    gmerge<TPA>(s, c);
  }
  __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

template <bool PREC>
__device__ __forceinline__ void fdfc(typename RT<PREC>::R r, typename RT<PREC>::R R1, typename RT<PREC>::R R2,
                                     typename RT<PREC>::R inv_w, typename RT<PREC>::R& f,
                                     typename RT<PREC>::R& df) {
  if constexpr (PREC)
    fdfcut_cos_f(r, R1, R2, inv_w, f, df);
  else
    fdfcut_cos_w(r, 1.0 / r, R1, R2, inv_w, f, df);
}
// The same with the caller's 1/r (the FP64 form then divides nowhere).
template <bool PREC>
__device__ __forceinline__ void fdfc(typename RT<PREC>::R r, typename RT<PREC>::R ir, typename RT<PREC>::R R1,
                                     typename RT<PREC>::R R2, typename RT<PREC>::R inv_w, typename RT<PREC>::R& f,
                                     typename RT<PREC>::R& df) {
  if constexpr (PREC)
    fdfcut_cos_f(r, R1, R2, inv_w, f, df);
  else
    fdfcut_cos_w(r, ir, R1, R2, inv_w, f, df);
}
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R fc_only(typename RT<PREC>::R r, typename RT<PREC>::R R1,
                                                        typename RT<PREC>::R R2, typename RT<PREC>::R inv_w) {
  if constexpr (PREC) {
    if (r < R1) return 1.0f;
    if (r < R2) return (1.0f + __cosf(3.14159265358979f * (r - R1) * inv_w)) * 0.5f;
    return 0.0f;
  } else {
    return fcut_cos_w(r, R1, R2, inv_w);
  }
}
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R xexp(typename RT<PREC>::R x) {
  if constexpr (PREC)
    return __expf(x);
  else
    return exp(x);
}
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R xpow(typename RT<PREC>::R x, typename RT<PREC>::R y) {
  if constexpr (PREC)
    return x > 0.0f ? exp2f(y * __log2f(x)) : 0.0f;
  else
    return pow(x, y);
}
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R xsqrt(typename RT<PREC>::R x) {
  if constexpr (PREC)
    return sqrtf(x);
  else
    return sqrt(x);
}
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R dot3(const typename RT<PREC>::R* a, const typename RT<PREC>::R* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

__device__ __forceinline__ void add_force(const Atoms& A, int ai, double fx, double fy, double fz) {
  double4_32a f = A.frc[ai];
  f.x += fx;
  f.y += fy;
  f.z += fz;
  A.frc[ai] = f;
}

__device__ __forceinline__ double kick_component(double v, double f, double m, double kc, double ts2, int exact) {
  // the plain form keeps the reference's f/m/mass_coef*dt/2 (md_integrators.f90:70)
  return exact ? __dadd_rn(v, __dmul_rn(__ddiv_rn(__ddiv_rn(f, m), 1.6605389217 / 1.6021765654 * 100.0), ts2))
               : v + f * kc * ts2;
}
// Stores or adds the row's force, then (Epi::kick) applies the second half-kick:
// the reference's expression in the plain form (exact), one FMA per component
// with kc*dt/2 formed once per atom otherwise.
__device__ __forceinline__ void finish_force(const Atoms& A, const Epi& E, int ai, double fx, double fy, double fz) {
  double4_32a f;
  if (E.store) {
    f = make_double4_32a(fx, fy, fz, 0.0);
  } else {
    f = A.frc[ai];
    f.x += fx;
    f.y += fy;
    f.z += fz;
  }
  A.frc[ai] = f;
  if (E.kick) {
    const unsigned char m = E.mflag[ai] & 3;  // bit 1: xyz-moving, bit 2: z-moving
    if (m) {
      double4_32a v = A.vel[ai];
      if (E.exact) {
        const double ms = A.mass[ai], kc = A.kc[ai];
        if (m & 1) {
          v.x = kick_component(v.x, f.x, ms, kc, E.ts2, 1);
          v.y = kick_component(v.y, f.y, ms, kc, E.ts2, 1);
        }
        v.z = kick_component(v.z, f.z, ms, kc, E.ts2, 1);
      } else {
        const double kt = A.kc[ai] * E.ts2;
        if (m & 1) {
          v.x = fma(f.x, kt, v.x);
          v.y = fma(f.y, kt, v.y);
        }
        v.z = fma(f.z, kt, v.z);
      }
      A.vel[ai] = v;
    }
  }
}

// finish_force, then (E.drift) the next step's first half-kick and drift of the
// atom, fused into this kernel: the same FMAs as k_kick_drift, so a run is the
// same bit for bit either way.  The previous drift's out-of-cell verdict is read
// first (set before this kernel started): a pending one stops the run at the
// next step's begin, with this step complete.  The new verdict goes to the other
// parity slot, which no thread of this kernel reads.
__device__ __forceinline__ void finish_force_drift(const Atoms& A, const Epi& E, const Box& B, Ctl* ctl, int ai,
                                                   double fx, double fy, double fz) {
  finish_force(A, E, ai, fx, fy, fz);
  if (!E.drift) return;
  const long long s = ctl->md_step;
  if (ctl->pending_oob || ctl->pending_fused[s & 1]) {
    set_error_at(ctl, ST_OUT_OF_CELL, EK_OOB, ctl->oob_atom + 1, 0, 0, s + 1);
    return;
  }
  const int4 q = A.posq[ai];
  if (!(E.mflag[ai] & 1)) {  // not moving: the same position in the next buffer
    E.posq_next[ai] = make_int4(q.x, q.y, q.z, 0);
    return;
  }
  const double4_32a f = A.frc[ai];
  double4_32a v = A.vel[ai], p = A.pos[ai];
  const double kt = A.kc[ai] * E.ts2;
  v.x = kick1_fast(v.x, f.x, kt);
  v.y = kick1_fast(v.y, f.y, kt);
  v.z = kick1_fast(v.z, f.z, kt);
  A.vel[ai] = v;
  p.x = drift1_fast(p.x, v.x, E.ts1, B.L[0]);
  p.y = drift1_fast(p.y, v.y, E.ts1, B.L[1]);
  p.z = drift1_fast(p.z, v.z, E.ts1, B.L[2]);
  A.pos[ai] = p;
  E.posq_next[ai] = make_int4(quantize_int(p.x, B, 0), quantize_int(p.y, B, 1), quantize_int(p.z, B, 2), 0);
  if (out_of_cell(p.x, B.Ltol[0]) || out_of_cell(p.y, B.Ltol[1]) || out_of_cell(p.z, B.Ltol[2])) {
    atomicMin(&ctl->oob_atom, ai);
    ctl->pending_fused[(s + 1) & 1] = 1;
  }
}

// Grid sum of K values held as float-float pairs (value = s - c, the form gmerge
// merges): every block's thread 0 passes its block totals, which go to
// Ctl::partial as two floats per value; the last block to arrive merges all
// partials with FP32 TwoSum steps in a fixed order (threads over blocks, then a
// warp and block tree) and returns the totals in FP64 in thread 0.  No FP64
// arithmetic runs in the tree: on this GPU's narrow FP64 pipe each FP64
// instruction of a warp costs a full warp's issue.  Every thread of every block
// calls it; the relative error is about 2^-46.
template <int K>
__device__ __forceinline__ bool grid_finish_ff(Ctl* ctl, int slot, const float (&s)[K], const float (&c)[K],
                                               double (&out)[K]) {
  __shared__ bool last;
  __shared__ float ss[K][32], sc[K][32];
  float2* part = reinterpret_cast<float2*>(ctl->partial);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) part[(size_t)blockIdx.x * K + k] = make_float2(s[k], c[k]);
    __threadfence();
    const unsigned int t = atomicAdd(&ctl->counter[slot], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  float ws[K], wc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) ws[k] = wc[k] = 0.f;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const float2 p = __ldcg(&part[(size_t)b * K + k]);  // written by other blocks: from L2
      float s2 = p.x, c2 = p.y;  // merge (s2, c2) into (ws, wc)
      const float t = ws[k] + s2, bb = t - ws[k];
      const float e = (ws[k] - (t - bb)) + (s2 - bb);
      wc[k] = (wc[k] + c2) - e;
      ws[k] = t;
    }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    gmerge<32>(ws[k], wc[k]);
    if (lane == 0) {
      ss[k][w] = ws[k];
      sc[k][w] = wc[k];
    }
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      ws[k] = lane < nw ? ss[k][lane] : 0.f;
      wc[k] = lane < nw ? sc[k][lane] : 0.f;
      gmerge<32>(ws[k], wc[k]);
    }
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = (double)ws[k] - (double)wc[k];
    ctl->counter[slot] = 0u;
  }
  return threadIdx.x == 0;
}

// Reduction slot (Ctl::counter) of the all-pairs kernel k_pair_atoms.
constexpr int kPairSlot = 20;
constexpr double kMassCoef = 1.6605389217 / 1.6021765654 * 100.0;  // amu A^2/fs^2 -> eV (md_integrators.f90:62)
constexpr double kKtPerKelvin = 1.3806488 / 1.6021765654 * 1e-4;   // k_B in eV/K (md_general.f90:304)

// Kinetic energy of atom i (calculate_kinetic_energy's term, md_general.f90:161-180).
__device__ __forceinline__ double ke_of(const Atoms& A, int i) {
  const double4_32a v = A.vel[i];
  return A.mass[i] * (v.x * v.x + v.y * v.y + v.z * v.z) / 2 * kMassCoef;
}

// e^x for the chain's scale factors, whose arguments (a thermostat velocity times
// a fraction of the time step) are small: below |x| = 2^-6 the Taylor series to
// x^8 (Horner, 8 FMAs; the first omitted term is under 2e-22), else exp().  One
// thread evaluates these on an FP64 pipe where each instruction costs a full
// warp's issue, so the short series is several times faster than the general
// function.
__device__ __forceinline__ double exp_small(double x) {
  if (fabs(x) >= 0.015625) return exp(x);
  double p = 1.0 / 40320.0;
  p = fma(p, x, 1.0 / 5040.0);
  p = fma(p, x, 1.0 / 720.0);
  p = fma(p, x, 1.0 / 120.0);
  p = fma(p, x, 1.0 / 24.0);
  p = fma(p, x, 1.0 / 6.0);
  p = fma(p, x, 0.5);
  p = fma(p, x, 1.0);
  return fma(p, x, 1.0);
}

// The chain part of integrate_nose_hoover_chain (md_integrators.f90:200-245)
// for the group's kinetic energy ke: both half-updates of the chain and the
// scale factor s (k_scale / k_kick_drift apply it).  One thread.  GB300's FP64
// pipe makes every FP64 instruction of this one thread cost a full warp's issue,
// so the update uses the host-formed 1/q instead of dividing, and the second
// sweep reuses the first sweep's factors b_i = exp(-v_{i+1} ts4): v_{i+1} is not
// touched between the two, so they are the same numbers the reference forms
// again (the divisions become multiplications by 1/q, a last-bit difference).
__device__ __forceinline__ void nhc_chain_update(NHCDev& hd, double ke, double ts2, double ts3, double ts4) {
  NHCDev h = hd;  // one set of independent loads, not a chain of dependent ones
  const double kt = kKtPerKelvin * h.T;
  const int M = h.M;
  double kedif = 2.0 * ke - 3.0 * h.L * kt;
  double bb[PFMD_MAX_CHAIN];
  if (M == 1) {
    h.v[0] = h.v[0] + kedif * h.iq[0] * ts3;
  } else {
    h.v[M - 1] = h.v[M - 1] + (h.q[M - 2] * (h.v[M - 2] * h.v[M - 2]) - kt) * h.iq[M - 1] * ts3;
    for (int i = M - 2; i >= 1; --i) {
      const double b = exp_small(-h.v[i + 1] * ts4);
      bb[i] = b;
      h.v[i] = h.v[i] * (b * b) + (h.q[i - 1] * (h.v[i - 1] * h.v[i - 1]) - kt) * h.iq[i] * ts3 * b;
    }
    bb[0] = exp_small(-h.v[1] * ts4);
    h.v[0] = h.v[0] * (bb[0] * bb[0]) + kedif * h.iq[0] * ts3 * bb[0];
  }
  h.s = exp_small(-h.v[0] * ts2);
  kedif = 2.0 * ke * (h.s * h.s) - 3.0 * h.L * kt;
  for (int i = 0; i < M; ++i) h.x[i] = h.x[i] + h.v[i] * ts2;
  if (M == 1) {
    h.v[0] = h.v[0] + kedif * h.iq[0] * ts3;
  } else {
    h.v[0] = h.v[0] * (bb[0] * bb[0]) + kedif * h.iq[0] * ts3 * bb[0];
    for (int i = 1; i <= M - 2; ++i)
      h.v[i] = h.v[i] * (bb[i] * bb[i]) + (h.q[i - 1] * (h.v[i - 1] * h.v[i - 1]) - kt) * h.iq[i] * ts3 * bb[i];
    h.v[M - 1] = h.v[M - 1] + (h.q[M - 2] * (h.v[M - 2] * h.v[M - 2]) - kt) * h.iq[M - 1] * ts3;
  }
  hd = h;
}

// Energy of one row into the interaction's total (every thread of the grid calls it).
__device__ __forceinline__ void energy_reduce(Ctl* ctl, int eslot, int ekey, double erow) {
  double v[1] = {erow}, out[1];
  if (grid_sum<1>(ctl, eslot, v, out)) ctl->e_inter[ekey] = out[0];
}

// The same for a row energy formed in FP32 (precision form): the block's rows are
// summed in FP32 with error-free TwoSum merges (value = s - c), and the block
// total goes to FP64 once, so the reduction issues no FP64 shuffles.
__device__ __forceinline__ void energy_reduce_f(Ctl* ctl, int eslot, int ekey, float erow) {
  __shared__ float ss[32], sc[32];
  float s = erow, c = 0.f;
  gmerge<32>(s, c);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) {
    ss[w] = s;
    sc[w] = c;
  }
  __syncthreads();
  double v[1] = {0.0}, out[1];
  if (w == 0) {
    s = lane < nw ? ss[lane] : 0.f;
    c = lane < nw ? sc[lane] : 0.f;
    gmerge<32>(s, c);
    v[0] = (double)s - (double)c;
  }
  if (grid_finish<1>(ctl, eslot, v, out)) ctl->e_inter[ekey] = out[0];
}

// The constants of a parameter set in the kernel's precision.
template <bool PREC>
__device__ __forceinline__ const LJc<typename RT<PREC>::R>& cst(const LJPar& p) {
  if constexpr (PREC) return p.f; else return p.d;
}
template <bool PREC>
__device__ __forceinline__ const Cosc<typename RT<PREC>::R>& cst(const CosPar& p) {
  if constexpr (PREC) return p.f; else return p.d;
}
template <bool PREC>
__device__ __forceinline__ const RJLc<typename RT<PREC>::R>& cst(const RJLPar& p) {
  if constexpr (PREC) return p.f; else return p.d;
}
template <bool PREC>
__device__ __forceinline__ const TBc<typename RT<PREC>::R>& cst(const TBPar& p) {
  if constexpr (PREC) return p.f; else return p.dd;
}
// 1/sqrt(x): the FP64 reciprocal square root (no divide) or rsqrtf
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R xrsqrt(typename RT<PREC>::R x) {
  if constexpr (PREC) return rsqrtf(x); else return rsqrt(x);
}
// 1/x: one divide per pair in FP64 (the plain form), the fast reciprocal in FP32
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R xrcp(typename RT<PREC>::R x) {
  if constexpr (PREC) return __frcp_rn(x); else return 1.0 / x;
}

static inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

// Launches with programmatic stream serialisation: the grid is set up while the
// previous kernel on the stream drains, and waits in griddepcontrol.wait (its
// first statement) until that kernel has completed and its writes are visible.
// The rjl passes trigger no dependents early: an early trigger let the next
// grid's blocks take SM slots from the running one (38.3 us per MD step against
// 32.1 on the 65,536-atom slab).  The fused pair kernel triggers after its
// epilogue, before the last block's reduction and chain update, so the next
// kick-drift is set up during that one-block tail.
template <class K, class... Args>
static inline void launch_dependent(K kern, int grid, int block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

// Entry `p` of list row `row` (slot-major storage).
__device__ __forceinline__ int ent(const ListDev& L, int row, int p) { return L.nlist[(size_t)p * L.stride + row]; }
__device__ __forceinline__ int ent(const RowList& L, int row, int p) { return L.nlist[(size_t)p * L.stride + row]; }

// 2^x by the ex2.approx instruction (relative error about 2^-22).
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// 1/sqrt(x) by the rsqrt.approx instruction, denormals flushed (list distances
// are never denormal).
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// sin and cos of x by the sin.approx / cos.approx instructions (absolute error
// about 2^-21 for |x| <= pi, the range the cosine switch uses).
__device__ __forceinline__ void sincos_approx(float x, float& s, float& c) {
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(x));
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(c) : "f"(x));
}

// Calls F with an integral_constant for the list's threads-per-row.
template <class F>
static inline void with_tpa(int tpa, F f) {
  switch (tpa) {
    case 1: f(std::integral_constant<int, 1>()); break;
    case 2: f(std::integral_constant<int, 2>()); break;
    case 4: f(std::integral_constant<int, 4>()); break;
    case 8: f(std::integral_constant<int, 8>()); break;
    case 16: f(std::integral_constant<int, 16>()); break;
    default: f(std::integral_constant<int, 32>()); break;
  }
}
template <class F>
static inline void with_bool(bool b, F f) {
  if (b)
    f(std::true_type());
  else
    f(std::false_type());
}

}  // namespace pfmd

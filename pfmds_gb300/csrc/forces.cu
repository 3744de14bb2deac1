// Forces and energies of the six PFMDS interactions on the device.
//
// Every kernel is a full-list gather: one thread owns one list row, recomputes the
// minimum-image vector to each neighbour from positions (the reference stores it
// per entry and refreshes it every step, md_neighbours.f90:104-124), sums the
// row's force in registers and adds it to its atom once.  No atomics: the
// half-list lj1g of the reference (Newton's third law with per-thread force
// copies, LennardJones_1g.f90:54-103) becomes a full-list gather with the same
// pair weights.  Energies are folded into the force pass at energy steps and
// reduced deterministically (block partials summed in block order).
//
// PREC=false: FP64 throughout; the `r < R2` style tests use the exact FP64
// distance, so the set of interacting pairs equals the reference's.
// PREC=true : the precision form -- separations from the fixed-point positions,
// FP32 pair terms, per-row Kahan sums in FP32, FP64 per-atom force update and
// FP64 energy reduction.
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
  static __device__ __forceinline__ R d2(const P4& a, const P4& b, const Box& B, R dr[3]) {
    return mi_exact(a, b, B, dr);
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

// Per-row accumulators: plain FP64, or FP32 with Kahan compensation.
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
  __device__ __forceinline__ double get(int k) const { return s[k]; }
};
template <>
struct Acc3<true> {
  Kahan3 k;
  __device__ __forceinline__ void add(float x, float y, float z) { k.add(x, y, z); }
  __device__ __forceinline__ double get(int c) const { return k.get(c); }
};
template <bool PREC>
struct Acc1;
template <>
struct Acc1<false> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
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
  __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

template <bool PREC>
__device__ __forceinline__ void fdfc(typename RT<PREC>::R r, typename RT<PREC>::R R1, typename RT<PREC>::R R2,
                                     typename RT<PREC>::R inv_w, typename RT<PREC>::R& f,
                                     typename RT<PREC>::R& df) {
  if constexpr (PREC)
    fdfcut_cos_f(r, R1, R2, inv_w, f, df);
  else
    fdfcut_cos(r, R1, R2, f, df);
}
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R fc_only(typename RT<PREC>::R r, typename RT<PREC>::R R1,
                                                        typename RT<PREC>::R R2, typename RT<PREC>::R inv_w) {
  if constexpr (PREC) {
    if (r < R1) return 1.0f;
    if (r < R2) return (1.0f + __cosf(3.14159265358979f * (r - R1) * inv_w)) * 0.5f;
    return 0.0f;
  } else {
    return fcut_cos(r, R1, R2);
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

__device__ __forceinline__ void add_force(const Atoms& A, int ai, double fx, double fy, double fz) {
  double4_32a f = A.frc[ai];
  f.x += fx;
  f.y += fy;
  f.z += fz;
  A.frc[ai] = f;
}

// Energy of one row into the interaction's total (all threads of the grid call it).
__device__ __forceinline__ void energy_reduce(Ctl* ctl, int eslot, int ekey, double erow) {
  double v[1] = {erow}, out[1];
  if (grid_sum<1>(ctl, eslot, v, out)) ctl->e_inter[ekey] = out[0];
}

// ---------------------------------------------------------------------------
// lj: LennardJones.f90:23-69 (cosine switch, full list, force on the row atom)
// ---------------------------------------------------------------------------
template <bool PREC, bool ENERGY>
__global__ void __launch_bounds__(256) k_lj(ListDev L, LJPar P, Atoms A, Box B, Ctl* ctl, int eslot, int ekey) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double erow = 0.0;
  if (i < L.rows) {
    const int n = L.nnum[i];
    if (n > 0) {
      const int ai = L.pidx[i];
      const auto pi = T::load(A, ai);
      const R sig = (R)P.sig, R1 = (R)P.R1, R2 = (R)P.R2, eps4 = (R)(4.0 * P.eps), inv_w = (R)(1.0 / (P.R2 - P.R1));
      Acc3<PREC> acc;
      Acc1<PREC> e;
      for (int p = 0; p < n; ++p) {
        const int aj = L.col_idx[L.nlist[(size_t)p * L.stride + i]];
        R dr[3];
        const R r = xsqrt<PREC>(T::d2(pi, T::load(A, aj), B, dr));
        if (r < R2) {
          const R x = sig / r, x2 = x * x, V = x2 * x2 * x2;
          R fc, dfc;
          fdfc<PREC>(r, R1, R2, inv_w, fc, dfc);
          const R c = eps4 * (V * (R(12) * V - R(6)) / (r * r) * fc - V * (V - R(1)) * dfc);
          acc.add(-c * dr[0], -c * dr[1], -c * dr[2]);
          if (ENERGY) e.add(eps4 * V * (V - R(1)) * fc);
        }
      }
      add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
      erow = e.get();
    }
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

// ---------------------------------------------------------------------------
// lj1g: LennardJones_1g.f90:28-117.  The reference walks the half list
// p <= lessnnum(i) and applies -fp to i and +fp to the partner.  Gathering over the
// full list, atom i receives -F(r) dr once for every pair in its own half list and
// once for every pair whose half list holds i; with a group in ascending atom order
// every pair is in exactly one of the two half lists (weight 1).  GENERAL keeps the
// weights for any group order: w = [p < lessnnum(i)] + [i < bnd(j)].
// Requires list groups g1 == g2, as the reference's particle_index(nlist(p,i)) does.
// ---------------------------------------------------------------------------
template <bool PREC, bool ENERGY, bool GENERAL>
__global__ void __launch_bounds__(256) k_lj1g(ListDev L, LJPar P, Atoms A, Box B, Ctl* ctl, int eslot, int ekey) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double erow = 0.0;
  if (i < L.rows) {
    const int n = L.nnum[i];
    if (n > 0) {
      const int ai = L.pidx[i];
      const int less = L.lessnnum[i];
      const auto pi = T::load(A, ai);
      const R R1 = (R)P.R1, R2 = (R)P.R2, c6 = (R)P.c6, c12 = (R)P.c12, c6t6 = (R)P.c6t6, c12t12 = (R)P.c12t12;
      Acc3<PREC> acc;
      Acc1<PREC> e;
      for (int p = 0; p < n; ++p) {
        const int jnd = L.nlist[(size_t)p * L.stride + i];
        const int aj = L.col_idx[jnd];
        R dr[3];
        const R r = xsqrt<PREC>(T::d2(pi, T::load(A, aj), B, dr));
        if (r < R2) {
          R w = R(1);
          if (GENERAL) w = R((p < less ? 1 : 0) + (i < L.bnd[jnd] ? 1 : 0));
          const R invr2 = R(1) / (r * r);
          const R U = invr2 * invr2 * invr2;
          R fcut, dfr;
          f_dfr_cut<R>(r, R1, R2, fcut, dfr);
          const R F = w * (U * invr2 * ((c12t12 * U - c6t6) * fcut - (c12 * U - c6) * dfr));
          acc.add(-F * dr[0], -F * dr[1], -F * dr[2]);
          if (ENERGY && p < less) {
            R Ue;
            if constexpr (PREC)
              Ue = U;
            else
              Ue = 1.0 / (r * r * r * r * r * r);
            R fp;
            if constexpr (PREC) {
              R x = (r - R1) / (R2 - R1);
              fp = r <= R1 ? R(1) : R(1) + x * x * x * (R(-10) + R(15) * x - R(6) * x * x);
            } else {
              fp = fcut_poly(r, R1, R2);
            }
            e.add(Ue * (c12 * Ue - c6) * fp);
          }
        }
      }
      add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
      erow = e.get();
    }
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

// ---------------------------------------------------------------------------
// rjl: RosatoGuillopeLegrand.f90:23-94.  Pass 1 (density) forms
// Eb_i = sqrt(sum exp(-2q(r/r0-1)) fc) and, at energy steps, the row energy
// A0*Er - xi*Eb; pass 2 gathers the pair forces with 1/Eb_i + 1/Eb_j.
// Requires g1 == g2 (Eb is indexed by the neighbour's list index).
// ---------------------------------------------------------------------------
// inv_eb holds 1/Eb per row: double for the plain form, float for the precision form.
template <bool PREC, bool ENERGY>
__global__ void __launch_bounds__(256) k_rjl_density(ListDev L, RJLPar P, Atoms A, Box B, void* inv_eb, Ctl* ctl,
                                                     int eslot, int ekey) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double erow = 0.0;
  if (i < L.rows) {
    const int n = L.nnum[i];
    const int ai = L.pidx[i];
    Acc1<PREC> eb2, er;
    if (n > 0) {
      const auto pi = T::load(A, ai);
      const R R1 = (R)P.R1, R2 = (R)P.R2, inv_r0 = (R)(1.0 / P.r0), m2q = (R)(-2.0 * P.q), mp = (R)(-P.p),
              inv_w = (R)(1.0 / (P.R2 - P.R1));
      for (int p = 0; p < n; ++p) {
        const int aj = L.col_idx[L.nlist[(size_t)p * L.stride + i]];
        R dr[3];
        const R r = xsqrt<PREC>(T::d2(pi, T::load(A, aj), B, dr));
        if (r <= R2) {
          const R fc = fc_only<PREC>(r, R1, R2, inv_w);
          R x;
          if constexpr (PREC)
            x = r * inv_r0 - 1.0f;
          else
            x = r / P.r0 - 1.0;
          eb2.add(xexp<PREC>(m2q * x) * fc);
          if (ENERGY) er.add(xexp<PREC>(mp * x) * fc);
        }
      }
    }
    const double s = eb2.get();
    const double eb = sqrt(s);
    if constexpr (PREC)
      static_cast<float*>(inv_eb)[i] = (float)(1.0 / eb);
    else
      static_cast<double*>(inv_eb)[i] = 1.0 / eb;
    if (ENERGY) erow = P.A0 * er.get() - P.xi * eb;
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

template <bool PREC>
__global__ void __launch_bounds__(256) k_rjl_force(ListDev L, RJLPar P, Atoms A, Box B, const void* inv_eb,
                                                   Ctl* ctl) {
  using IE = typename std::conditional<PREC, float, double>::type;
  const IE* ieb = static_cast<const IE*>(inv_eb);
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.rows) return;
  const int n = L.nnum[i];
  if (n == 0) return;
  const int ai = L.pidx[i];
  const auto pi = T::load(A, ai);
  const R R1 = (R)P.R1, R2 = (R)P.R2, inv_r0 = (R)(1.0 / P.r0), m2q = (R)(-2.0 * P.q), mp = (R)(-P.p),
          inv_w = (R)(1.0 / (P.R2 - P.R1));
  const R a2 = (R)(2.0 * P.A0), pr0 = (R)(P.p / P.r0), qr0 = (R)(P.q / P.r0), xi = (R)P.xi;
  const R ieb_i = ieb[i];
  Acc3<PREC> acc;
  for (int p = 0; p < n; ++p) {
    const int jnd = L.nlist[(size_t)p * L.stride + i];
    const int aj = L.col_idx[jnd];
    R dr[3];
    const R r = xsqrt<PREC>(T::d2(pi, T::load(A, aj), B, dr));
    if (r <= R2) {
      R fc, dfc;
      fdfc<PREC>(r, R1, R2, inv_w, fc, dfc);
      R x;
      if constexpr (PREC)
        x = r * inv_r0 - 1.0f;
      else
        x = r / P.r0 - 1.0;
      const R ep = xexp<PREC>(mp * x), eq = xexp<PREC>(m2q * x);
      const R T1 = a2 * (pr0 * fc - dfc * r) * ep;
      const R T2 = xi * (qr0 * fc - dfc * R(0.5) * r) * (ieb_i + ieb[jnd]) * eq;
      const R c = (T1 - T2) / r;
      acc.add(-c * dr[0], -c * dr[1], -c * dr[2]);
    }
  }
  add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
}

// ---------------------------------------------------------------------------
// tb: TersoffBrenner.f90:26-150.  Pass 1: bond orders B(p,i); pass 2: forces with
// the angular terms of i's and of each neighbour j's environment, and (energy
// steps) the bond energies for j > i.  Requires g1 == g2.
// ---------------------------------------------------------------------------
template <bool PREC>
__device__ __forceinline__ typename RT<PREC>::R dot3(const typename RT<PREC>::R* a, const typename RT<PREC>::R* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

template <bool PREC>
__global__ void __launch_bounds__(128) k_tb_bond(ListDev L, TBPar P, Atoms A, Box B, double* Bb, Ctl* ctl) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.rows) return;
  const int n = L.nnum[i];
  const int ai = L.pidx[i];
  const auto pi = T::load(A, ai);
  const R R1 = (R)P.R1, R2 = (R)P.R2, a0 = (R)P.a0, c02 = (R)P.c02, d02 = (R)P.d02, delt = (R)P.delt,
          inv_w = (R)(1.0 / (P.R2 - P.R1));
  for (int p = 0; p < n; ++p) {
    R dp[3];
    const R rp = xsqrt<PREC>(T::d2(pi, T::load(A, L.col_idx[L.nlist[(size_t)p * L.stride + i]]), B, dp));
    R b = R(0);
    if (rp < R2) {
      for (int q = 0; q < n; ++q) {
        if (q == p) continue;
        R dq[3];
        const R rq = xsqrt<PREC>(T::d2(pi, T::load(A, L.col_idx[L.nlist[(size_t)q * L.stride + i]]), B, dq));
        if (rq < R2) {
          const R cs = dot3<PREC>(dp, dq) / (rp * rq);
          b += fc_only<PREC>(rq, R1, R2, inv_w) * (R(1) + c02 / d02 - c02 / (d02 + (R(1) + cs) * (R(1) + cs)));
        }
      }
      b = xpow<PREC>(R(1) + a0 * b, -delt);
    }
    Bb[(size_t)p * L.stride + i] = (double)b;
  }
}

template <bool PREC, bool ENERGY>
__global__ void __launch_bounds__(128) k_tb_force(ListDev L, TBPar P, Atoms A, Box B, const double* Bb, Ctl* ctl,
                                                  int eslot, int ekey) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double erow = 0.0;
  if (i < L.rows && L.nnum[i] > 0) {
    const int n = L.nnum[i];
    const int ai = L.pidx[i];
    const auto pi = T::load(A, ai);
    const R R1 = (R)P.R1, R2 = (R)P.R2, a0 = (R)P.a0, c02 = (R)P.c02, d02 = (R)P.d02, delt = (R)P.delt,
            d = (R)P.d, s = (R)P.s, bb = (R)P.b, r0 = (R)P.r0, inv_w = (R)(1.0 / (P.R2 - P.R1));
    const R ex = (R)(1.0 / P.delt + 1.0);
    const R sq2s = (R)sqrt(2.0 * P.s), sq2os = (R)sqrt(2.0 / P.s);
    const R pre_e = d / (s - R(1));
    Acc3<PREC> acc;
    Acc1<PREC> e;
    for (int p = 0; p < n; ++p) {
      const int j = L.nlist[(size_t)p * L.stride + i];
      const int aj = L.col_idx[j];
      R dp[3];
      const R rp = xsqrt<PREC>(T::d2(pi, T::load(A, aj), B, dp));
      R dB[3] = {R(0), R(0), R(0)};
      for (int q = 0; q < n; ++q) {
        if (q == p) continue;
        R dq[3];
        const R rq = xsqrt<PREC>(T::d2(pi, T::load(A, L.col_idx[L.nlist[(size_t)q * L.stride + i]]), B, dq));
        const R rr = R(1) / rp / rq;
        const R cosi = dot3<PREC>(dp, dq) * rr;
        const R t = d02 + (R(1) + cosi) * (R(1) + cosi);
        R fq, dfq;
        fdfc<PREC>(rq, R1, R2, inv_w, fq, dfq);
        const R g1 = fq * R(2) * a0 * c02 * (R(1) + cosi) / (t * t);
        const R g2 = dfq * a0 * (R(1) + c02 / d02 - c02 / t);
#pragma unroll
        for (int k = 0; k < 3; ++k)
          dB[k] += g1 * ((dp[k] + dq[k]) * rr - cosi * (dp[k] / (rp * rp) + dq[k] / (rq * rq))) + g2 * dq[k];
      }
      const R Bpi = (R)Bb[(size_t)p * L.stride + i];
      const R bpe = xpow<PREC>(Bpi, ex);
#pragma unroll
      for (int k = 0; k < 3; ++k) dB[k] *= bpe;
      // i's slot l in j's row, and j's environment
      const int nj = L.nnum[j];
      const auto pj = T::load(A, aj);
      int l = 0;
      for (; l < nj; ++l)
        if (L.nlist[(size_t)l * L.stride + j] == i) break;
      R dl[3] = {R(0), R(0), R(0)};
      R rl = R(0), Blj = R(0);
      if (l < nj) {
        rl = xsqrt<PREC>(T::d2(pj, pi, B, dl));
        Blj = (R)Bb[(size_t)l * L.stride + j];
      }
      const R blpe = xpow<PREC>(Blj, ex);
      for (int q = 0; q < nj && l < nj; ++q) {
        if (q == l) continue;
        R dq[3];
        const R rq = xsqrt<PREC>(T::d2(pj, T::load(A, L.col_idx[L.nlist[(size_t)q * L.stride + j]]), B, dq));
        const R rr = R(1) / rl / rq;
        const R cosi = dot3<PREC>(dl, dq) * rr;
        const R t = d02 + (R(1) + cosi) * (R(1) + cosi);
        const R g = blpe * fc_only<PREC>(rq, R1, R2, inv_w) * R(2) * a0 * c02 * (R(1) + cosi) / (t * t);
#pragma unroll
        for (int k = 0; k < 3; ++k) dB[k] += g * (-dq[k] * rr + cosi * dl[k] / (rl * rl));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) dB[k] = dB[k] * (-delt) * R(0.5);
      if (rp < R2) {
        R fc, dfc;
        fdfc<PREC>(rp, R1, R2, inv_w, fc, dfc);
        const R dff = dfc / fc;
        const R a = -sq2s * bb * (rp - r0);
        const R ea = xexp<PREC>(a), eas = xexp<PREC>(a / s);
        const R c1 = sq2s * bb / rp, c2 = sq2os * bb / rp;
        const R pre = fc * d / (s - R(1));
        const R bavg = (Bpi + Blj) * R(0.5);
        R f[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
          f[k] = pre * ((dp[k] * dff - c1 * dp[k]) * ea - (dB[k] + bavg * (dp[k] * dff - c2 * dp[k])) * s * eas);
        acc.add(f[0], f[1], f[2]);
        if (ENERGY && j > i) e.add(fc * pre_e * (ea - bavg * s * eas));
      }
      if (l < nj) {
        R fl, dfl;
        fdfc<PREC>(rl, R1, R2, inv_w, fl, dfl);
        for (int q = 0; q < nj; ++q) {
          if (q == l) continue;
          R dq[3];
          const R rq = xsqrt<PREC>(T::d2(pj, T::load(A, L.col_idx[L.nlist[(size_t)q * L.stride + j]]), B, dq));
          const R rr = R(1) / rl / rq;
          const R cosi = dot3<PREC>(dl, dq) * rr;
          const R t = d02 + (R(1) + cosi) * (R(1) + cosi);
          const R t1 = fl * R(2) * a0 * c02 * (R(1) + cosi) / (t * t);
          const R t2 = dfl * a0 * (R(1) + c02 / d02 - c02 / t);
          const R pre = delt * R(0.5) * xpow<PREC>((R)Bb[(size_t)q * L.stride + j], ex);
          const R post = fc_only<PREC>(rq, R1, R2, inv_w) * d / (s - R(1)) * s * xexp<PREC>(-sq2s * bb * (rq - r0) / s);
          R f[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) f[k] = pre * (t1 * (-dq[k] * rr + cosi * dl[k] / (rl * rl)) + dp[k] * t2) * post;
          acc.add(f[0], f[1], f[2]);
        }
      }
    }
    add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
    erow = e.get();
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

// ---------------------------------------------------------------------------
// ljc / morsec: LennardJonesCosine.f90 and MorseCosine.f90 (26-139).
// Graphene side (rows of nl(1)): the pair term with the row's normal plus, unless
// `simplified`, the term through the normals of its three nearest neighbours j
// (dn_j/dr_i).  Metal side (rows of nl(2)): the pair term with the neighbour's
// normal; morsec divides that cosine by |n| (MorseCosine.f90:127), ljc does not.
// ---------------------------------------------------------------------------
template <bool PREC, bool MORSE>
__device__ __forceinline__ void cos_pair(const CosPar& P, typename RT<PREC>::R r, const typename RT<PREC>::R* dr,
                                         const typename RT<PREC>::R* nv, typename RT<PREC>::R nnorm, bool metal,
                                         typename RT<PREC>::R& X, typename RT<PREC>::R& Y, typename RT<PREC>::R& E) {
  using R = typename RT<PREC>::R;
  const R R1 = (R)P.R1, R2 = (R)P.R2, delt = (R)P.delt, inv_w = (R)(1.0 / (P.R2 - P.R1));
  const R nd = nv[0] * dr[0] + nv[1] * dr[1] + nv[2] * dr[2];
  R fc, dfc;
  fdfc<PREC>(r, R1, R2, inv_w, fc, dfc);
  if (!MORSE) {
    const R x = (R)P.sig / r, x2 = x * x, V2 = x2 * x2 * x2, V1 = V2 * V2;
    const R V3 = xpow<PREC>(fabs(nd) / r, delt);
    X = (R(12) * V1 - (R(6) + delt) * V2 * V3) / (r * r) * fc - (V1 - V2 * V3) * dfc;
    Y = delt * V2 * V3 / nd * fc;
    E = (V1 - V2 * V3) * fc;
  } else {
    const R a = (R)P.a;
    const R V2 = xexp<PREC>(-a * (r - (R)P.r0)), V1 = V2 * V2;
    const R V3 = xpow<PREC>(metal ? fabs(nd) / (nnorm * r) : fabs(nd) / r, delt);
    X = R(2) * (a * V1 - (a + delt / r) * V2 * V3) / r * fc - (V1 - R(2) * V2 * V3) * dfc;
    Y = R(2) * delt * V2 * V3 / nd * fc;
    E = (V1 - R(2) * V2 * V3) * fc;
  }
}

template <bool PREC, bool ENERGY, bool MORSE>
__global__ void __launch_bounds__(128) k_cos_graphene(ListDev nl, ListDev nn, CosPar P, const double4_32a* norm, Atoms A,
                                                      Box B, Ctl* ctl, int eslot, int ekey) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double erow = 0.0;
  if (i < nl.rows) {
    const int ai = nl.pidx[i];
    const auto pi = T::load(A, ai);
    const R R2 = (R)P.R2;
    const R pref = MORSE ? (R)P.D : (R)(4.0 * P.eps);
    Acc3<PREC> acc;
    Acc1<PREC> e;
    const double4_32a ni = norm[i];
    const R nv[3] = {(R)ni.x, (R)ni.y, (R)ni.z};
    const int n = nl.nnum[i];
    for (int p = 0; p < n; ++p) {
      const int aj = nl.col_idx[nl.nlist[(size_t)p * nl.stride + i]];
      R dr[3];
      const R r = xsqrt<PREC>(T::d2(pi, T::load(A, aj), B, dr));
      if (r < R2) {
        R X, Y, E;
        cos_pair<PREC, MORSE>(P, r, dr, nv, R(1), false, X, Y, E);
        acc.add(-pref * (X * dr[0] + Y * nv[0]), -pref * (X * dr[1] + Y * nv[1]), -pref * (X * dr[2] + Y * nv[2]));
        if (ENERGY) e.add(pref * E);
      }
    }
    if (!P.simplified) {
      const R R1 = (R)P.R1, delt = (R)P.delt, inv_w = (R)(1.0 / (P.R2 - P.R1));
      for (int q = 0; q < 3; ++q) {
        const int j = nn.nlist[(size_t)q * nn.stride + i];
        if (j < 0 || j >= nn.rows || j >= nl.rows || j >= nn.row_cap) {
          // a neighbour outside the graphene rows (groups 5/6 of the list differ)
          set_error(ctl, ST_PARAM, EK_NONE, i + 1, j + 1, 0);
          break;
        }
        int l1 = 0;
        for (; l1 < 3; ++l1)
          if (nn.nlist[(size_t)l1 * nn.stride + j] == i) break;
        if (l1 >= 3) {
          set_error(ctl, ST_GR_NN, EK_L1, i + 1, j + 1, 0);
          break;
        }
        const int l2 = (l1 + 1) % 3, l3 = (l1 + 2) % 3;
        const int aj = nn.row_idx[j];
        const auto pj = T::load(A, aj);
        R dl[3][3];
#pragma unroll
        for (int l = 0; l < 3; ++l) T::d2(pj, T::load(A, nn.col_idx[nn.nlist[(size_t)l * nn.stride + j]]), B, dl[l]);
        R d12[3], d31[3], d23[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          d12[k] = dl[l2][k] - dl[l1][k];
          d31[k] = dl[l1][k] - dl[l3][k];
          d23[k] = dl[l3][k] - dl[l2][k];
        }
        const R Aa = dot3<PREC>(d12, d12) * dot3<PREC>(d31, d31) - dot3<PREC>(d12, d31) * dot3<PREC>(d12, d31);
        const R s2331 = dot3<PREC>(d23, d31), s2312 = dot3<PREC>(d23, d12);
        R w[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) w[k] = d12[k] * s2331 - d31[k] * s2312;
        const double4_32a nj4 = norm[j];
        const R nj[3] = {(R)nj4.x, (R)nj4.y, (R)nj4.z};
        const auto pg = T::load(A, nl.pidx[j]);
        const int m = nl.nnum[j];
        for (int p = 0; p < m; ++p) {
          const int am = nl.col_idx[nl.nlist[(size_t)p * nl.stride + j]];
          R dr[3];
          const R r = xsqrt<PREC>(T::d2(pg, T::load(A, am), B, dr));
          if (r < R2) {
            const R nd = nj[0] * dr[0] + nj[1] * dr[1] + nj[2] * dr[2];
            const R V3 = xpow<PREC>(fabs(nd) / r, delt);
            const R fc = fc_only<PREC>(r, R1, R2, inv_w);
            R V2;
            if (MORSE)
              V2 = xexp<PREC>(-(R)P.a * (r - (R)P.r0));
            else {
              const R x = (R)P.sig / r, x2 = x * x;
              V2 = x2 * x2 * x2;
            }
            const R C = dr[0] * w[0] + dr[1] * w[1] + dr[2] * w[2];
            const R coef = (MORSE ? R(2) * pref : pref) * delt * V2 * V3 * fc / Aa / nd;
            acc.add(-coef * nj[0] * C, -coef * nj[1] * C, -coef * nj[2] * C);
          }
        }
      }
    }
    add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
    erow = e.get();
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

template <bool PREC, bool MORSE>
__global__ void __launch_bounds__(128) k_cos_metal(ListDev nl, CosPar P, const double4_32a* norm, Atoms A, Box B,
                                                   Ctl* ctl) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl.rows) return;
  const int n = nl.nnum[i];
  if (n == 0) return;
  const int ai = nl.pidx[i];
  const auto pi = T::load(A, ai);
  const R R2 = (R)P.R2;
  const R pref = MORSE ? (R)P.D : (R)(4.0 * P.eps);
  Acc3<PREC> acc;
  for (int p = 0; p < n; ++p) {
    const int jnd = nl.nlist[(size_t)p * nl.stride + i];
    const int aj = nl.col_idx[jnd];
    R dr[3];
    const R r = xsqrt<PREC>(T::d2(pi, T::load(A, aj), B, dr));
    if (r < R2) {
      const double4_32a g = norm[jnd];
      const R nv[3] = {(R)g.x, (R)g.y, (R)g.z};
      const R nn = xsqrt<PREC>(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
      R X, Y, E;
      cos_pair<PREC, MORSE>(P, r, dr, nv, nn, true, X, Y, E);
      acc.add(-pref * (X * dr[0] + Y * nv[0]), -pref * (X * dr[1] + Y * nv[1]), -pref * (X * dr[2] + Y * nv[2]));
    }
  }
  add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }

void launch_lj(bool prec, bool energy, const ListDev& L, const LJPar& P, const Atoms& A, const Box& B, Ctl* ctl,
               int eslot, int ekey, cudaStream_t s) {
  if (L.rows == 0) {
    if (energy) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int g = nblk(L.rows, 256);
  if (prec) {
    if (energy)
      { k_lj<true, true><<<g, 256, 0, s>>>(L, P, A, B, ctl, eslot, ekey); ++g_kernel_launches; }
    else
      { k_lj<true, false><<<g, 256, 0, s>>>(L, P, A, B, ctl, eslot, ekey); ++g_kernel_launches; }
  } else {
    if (energy)
      { k_lj<false, true><<<g, 256, 0, s>>>(L, P, A, B, ctl, eslot, ekey); ++g_kernel_launches; }
    else
      { k_lj<false, false><<<g, 256, 0, s>>>(L, P, A, B, ctl, eslot, ekey); ++g_kernel_launches; }
  }
}

void launch_lj1g(bool prec, bool energy, bool general, const ListDev& L, const LJPar& P, const Atoms& A,
                 const Box& B, Ctl* ctl, int eslot, int ekey, cudaStream_t s) {
  if (L.rows == 0) {
    if (energy) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int g = nblk(L.rows, 256);
#define PFMD_LJ1G(PR, EN, GE) \
  (k_lj1g<PR, EN, GE><<<g, 256, 0, s>>>(L, P, A, B, ctl, eslot, ekey), ++g_kernel_launches)
  if (prec) {
    if (energy) {
      if (general) PFMD_LJ1G(true, true, true); else PFMD_LJ1G(true, true, false);
    } else {
      if (general) PFMD_LJ1G(true, false, true); else PFMD_LJ1G(true, false, false);
    }
  } else {
    if (energy) {
      if (general) PFMD_LJ1G(false, true, true); else PFMD_LJ1G(false, true, false);
    } else {
      if (general) PFMD_LJ1G(false, false, true); else PFMD_LJ1G(false, false, false);
    }
  }
#undef PFMD_LJ1G
}

void launch_rjl(bool prec, bool energy, const ListDev& L, const RJLPar& P, const Atoms& A, const Box& B, void* Eb,
                Ctl* ctl, int eslot, int ekey, cudaStream_t s, int parts) {
  if (L.rows == 0) {
    if (energy) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int g = nblk(L.rows, 256);
  if (!(parts & 1)) {
    if (prec) { k_rjl_force<true><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl); ++g_kernel_launches; }
    else { k_rjl_force<false><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl); ++g_kernel_launches; }
    return;
  }
  if (prec) {
    if (energy)
      { k_rjl_density<true, true><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl, eslot, ekey); ++g_kernel_launches; }
    else
      { k_rjl_density<true, false><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl, eslot, ekey); ++g_kernel_launches; }
    if (parts & 2) { k_rjl_force<true><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl); ++g_kernel_launches; }
  } else {
    if (energy)
      { k_rjl_density<false, true><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl, eslot, ekey); ++g_kernel_launches; }
    else
      { k_rjl_density<false, false><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl, eslot, ekey); ++g_kernel_launches; }
    if (parts & 2) { k_rjl_force<false><<<g, 256, 0, s>>>(L, P, A, B, Eb, ctl); ++g_kernel_launches; }
  }
}

void launch_tb(bool prec, bool energy, const ListDev& L, const TBPar& P, const Atoms& A, const Box& B, double* Bb,
               Ctl* ctl, int eslot, int ekey, cudaStream_t s, int parts) {
  if (L.rows == 0) {
    if (energy) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int g = nblk(L.rows, 128);
  if (prec) {
    if (parts & 1) { k_tb_bond<true><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl); ++g_kernel_launches; }
    if (!(parts & 2)) return;
    if (energy)
      { k_tb_force<true, true><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl, eslot, ekey); ++g_kernel_launches; }
    else
      { k_tb_force<true, false><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl, eslot, ekey); ++g_kernel_launches; }
  } else {
    if (parts & 1) { k_tb_bond<false><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl); ++g_kernel_launches; }
    if (!(parts & 2)) return;
    if (energy)
      { k_tb_force<false, true><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl, eslot, ekey); ++g_kernel_launches; }
    else
      { k_tb_force<false, false><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl, eslot, ekey); ++g_kernel_launches; }
  }
}

void launch_cos(bool prec, bool energy, bool morse, const ListDev& nl1, const ListDev& nl2, const ListDev& nn,
                const CosPar& P, const double4_32a* norm, const Atoms& A, const Box& B, Ctl* ctl, int eslot, int ekey,
                cudaStream_t s, int parts) {
  if (nl1.rows > 0 && (parts & 1)) {
    const int g = nblk(nl1.rows, 128);
#define PFMD_COSG(PR, EN, MO) \
  (k_cos_graphene<PR, EN, MO><<<g, 128, 0, s>>>(nl1, nn, P, norm, A, B, ctl, eslot, ekey), ++g_kernel_launches)
    if (prec) {
      if (energy) {
        if (morse) PFMD_COSG(true, true, true); else PFMD_COSG(true, true, false);
      } else {
        if (morse) PFMD_COSG(true, false, true); else PFMD_COSG(true, false, false);
      }
    } else {
      if (energy) {
        if (morse) PFMD_COSG(false, true, true); else PFMD_COSG(false, true, false);
      } else {
        if (morse) PFMD_COSG(false, false, true); else PFMD_COSG(false, false, false);
      }
    }
#undef PFMD_COSG
  } else if (energy && (parts & 1)) {
    cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
  }
  if (nl2.rows > 0 && (parts & 2)) {
    const int g = nblk(nl2.rows, 128);
    if (prec) {
      if (morse)
        { k_cos_metal<true, true><<<g, 128, 0, s>>>(nl2, P, norm, A, B, ctl); ++g_kernel_launches; }
      else
        { k_cos_metal<true, false><<<g, 128, 0, s>>>(nl2, P, norm, A, B, ctl); ++g_kernel_launches; }
    } else {
      if (morse)
        { k_cos_metal<false, true><<<g, 128, 0, s>>>(nl2, P, norm, A, B, ctl); ++g_kernel_launches; }
      else
        { k_cos_metal<false, false><<<g, 128, 0, s>>>(nl2, P, norm, A, B, ctl); ++g_kernel_launches; }
    }
  }
}

}  // namespace pfmd

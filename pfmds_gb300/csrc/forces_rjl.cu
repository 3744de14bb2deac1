// rjl (Rosato-Guillope-Legrand, second-moment tight binding) forces and energy,
// RosatoGuillopeLegrand.f90:23-94.  Pass 1 (density) forms
// Eb_i = sqrt(sum exp(-2q(r/r0-1)) fc), stores 1/Eb per atom and, at energy steps,
// the row energy A0*Er - xi*Eb; pass 2 gathers the pair forces with
// 1/Eb_i + 1/Eb_j.  See forces.cuh for the execution scheme.
//
// Pass 1 also keeps the pair terms of each list slot,
//   a = 2 A0 (p/r0 fc - f' ) e_p / r,   b = xi (q/r0 fc - f'/2) e_q / r,
// so pass 2 only needs the separation vector: F_i -= (a - b (1/Eb_i + 1/Eb_j)) dr.
// That replaces two exponentials, a sine/cosine, a square root and a reciprocal
// per pair with one coalesced load: 16 bytes per slot (double2) in the plain form,
// 8 bytes (float2) in the precision form.  The precision form keeps 1/Eb_i in the
// spare w word of the atom's fixed-point position, so pass 2 fetches a partner's
// position and 1/Eb with a single 16-byte gather.
#include "forces.cuh"

namespace pfmd {

// inv_eb holds 1/Eb per atom: double for the plain form, float for the precision form.
template <bool PREC, bool ENERGY, int TPA>
__global__ void __launch_bounds__(256) k_rjl_density(ListDev L, RJLPar P, Atoms A, Box B, void* inv_eb,
                                                     double2* pair, Ctl* ctl, int eslot, int ekey, double* eatom,
                                                     int begin) {
  using T = RT<PREC>;
  using R = typename T::R;
  asm volatile("griddepcontrol.wait;" ::: "memory");  // see launch_dependent
  if (ctl->stop) return;
  if (begin && blockIdx.x == 0 && threadIdx.x == 0) {
    // nothing else in this launch reads these two
    ctl->md_step = ctl->md_step + 1;
    ctl->pe_prev = ctl->pe_last;
  }
  const Grp<TPA> g;
  const bool valid = g.row < L.rows;
  const int n = valid ? L.nnum[g.row] : 0;
  const int ai = valid ? L.pidx[g.row] : 0;
  const auto& c = cst<PREC>(P);
  Acc1<PREC> eb2, er;
  if (n > 0) {
    const auto pi = T::load(A, ai);
    // the next slot's partner index is loaded one iteration ahead, so its load
    // overlaps this slot's gather instead of preceding the next one (14.6 -> 14.4 us
    // on the 65,536-atom slab); precision: no unrolling measured fastest (14.4 us
    // against 15.6 with 4)
    int aj = g.sub < n ? ent(L, g.row, g.sub) : ai;
#pragma unroll(PREC ? 1 : 4)
    for (int p = g.sub; p < n; p += TPA) {
      R dr[3];
      const int pn = p + TPA;
      const int aj_next = pn < n ? ent(L, g.row, pn) : ai;
      const R r2 = T::d2(pi, T::load(A, aj), B, dr);
      aj = aj_next;
      if constexpr (PREC) {
        // r and 1/r from one reciprocal square root
        const float ir = rsqrt_approx(r2), r = r2 * ir;
        // the cosine switch without branches: t is 0 below R1 and 1 from R2 on; entries
        // beyond R2 (about a fifth of the 5.5 A list) are masked, not skipped, so the
        // warp stays converged
        const float t = __saturatef(fmaf(r, c.inv_w, c.tb));
        float sn, cs;
        sincos_approx(3.14159265358979f * t, sn, cs);  // argument in [0, pi]
        const float in = r <= c.R2 ? 1.f : 0.f;
        const float fc = (0.5f + 0.5f * cs) * in;
        const float rdfc = sn * c.dsw * in;
        // each exponential is one FMA into the hardware's base-2 exponential
        const float eq = ex2_approx(fmaf(c.eqa, r, c.eqb)), ep = ex2_approx(fmaf(c.epa, r, c.epb));
        eb2.add(eq * fc);
        if (ENERGY) er.add(ep * fc);
        float2 ab;
        ab.x = c.a2 * (c.pr0 * fc - rdfc) * ep * ir;
        ab.y = c.xi * (c.qr0 * fc - 0.5f * rdfc) * eq * ir;
        reinterpret_cast<float2*>(pair)[(size_t)p * L.stride + g.row] = ab;
      } else {
        // r and 1/r from one reciprocal square root (no FP64 divide: each FP64
        // instruction costs a full warp's issue on this GPU's FP64 pipe)
        const R ir = rsqrt(r2), r = r2 * ir;
        double2 ab = make_double2(0.0, 0.0);
        if (r <= c.R2) {
          R fc, dfc;
          fdfc<PREC>(r, ir, c.R1, c.R2, c.inv_w, fc, dfc);
          const R x = r * c.inv_r0 - R(1);
          const R eq = xexp<PREC>(c.m2q * x), ep = xexp<PREC>(c.mp * x);
          eb2.add(eq * fc);
          if (ENERGY) er.add(ep * fc);
          ab.x = c.a2 * (c.pr0 * fc - dfc * r) * ep * ir;
          ab.y = c.xi * (c.qr0 * fc - dfc * R(0.5) * r) * eq * ir;
        }
        pair[(size_t)p * L.stride + g.row] = ab;
      }
    }
  }
  eb2.template reduce<TPA>();
  if (ENERGY) er.template reduce<TPA>();
  double erow = 0.0;
  float erowf = 0.f;
  if (valid && g.sub == 0) {
    if constexpr (PREC) {
      // 1/Eb from the FP32-rounded sum (no FP64 square root on the step), kept in
      // the w word of the atom's fixed-point position
      const float e2 = eb2.s - eb2.c, ie = rsqrtf(e2);
      reinterpret_cast<int*>(A.posq + ai)[3] = __float_as_int(ie);
      if (ENERGY) erowf = c.A0 * (er.s - er.c) - c.xi * (e2 > 0.f ? e2 * ie : 0.f);
    } else {
      const double eb = sqrt(eb2.get());
      static_cast<double*>(inv_eb)[ai] = 1.0 / eb;
      if (ENERGY) erow = P.A0 * er.get() - P.xi * eb;
    }
  }
  if constexpr (ENERGY) {
    if (eatom && valid && g.sub == 0) eatom[ai] = PREC ? (double)erowf : erow;
    if constexpr (PREC)
      energy_reduce_f(ctl, eslot, ekey, erowf);
    else
      energy_reduce(ctl, eslot, ekey, erow);
  }
}

// Blocks of 32 rows (32 x TPA threads): the row sums go through shared memory to
// one full warp, which runs the FP64 epilogue (force store, kick, the next
// step's kick and drift) with all 32 lanes busy.  Finishing each row on its own
// sub-0 lane instead keeps TPA - 1 of every TPA lanes idle on the FP64 pipe, which
// is what held the kernel at 2 threads per row.
template <bool PREC, int TPA>
__global__ void __launch_bounds__(32 * TPA) k_rjl_force(ListDev L, RJLPar P, Atoms A, Box B, const void* inv_eb,
                                                        const double2* pair, Ctl* ctl, Epi E) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // see launch_dependent
  using T = RT<PREC>;
  using R = typename T::R;
  using IE = typename std::conditional<PREC, float, double>::type;
  constexpr int RPW = 32 / TPA;
  __shared__ double s_f[3][32];
  const IE* ieb = static_cast<const IE*>(inv_eb);
  if (block_stop(ctl)) return;
  const Grp<TPA> g;
  const bool valid = g.row < L.rows;
  const int n = valid ? L.nnum[g.row] : 0;
  const int ai = valid ? L.pidx[g.row] : 0;
  const auto& c = cst<PREC>(P);
  Acc3<PREC> acc;
  if (n > 0) {
    const auto pi = T::load(A, ai);
    R ieb_i;
    if constexpr (PREC)
      ieb_i = __int_as_float(pi.w);
    else
      ieb_i = ieb[ai];
    // the partner index is loaded one iteration ahead, as in the density pass
    int aj = g.sub < n ? ent(L, g.row, g.sub) : ai;
#pragma unroll 2
    for (int p = g.sub; p < n; p += TPA) {
      const int pn = p + TPA;
      const int aj_next = pn < n ? ent(L, g.row, pn) : ai;
      R dr[3];
      if constexpr (PREC) {
        const int4 pj = A.posq[aj];
        T::d2(pi, pj, B, dr);
        const float2 ab = reinterpret_cast<const float2*>(pair)[(size_t)p * L.stride + g.row];
        const float k = ab.x - ab.y * (ieb_i + __int_as_float(pj.w));
        acc.add(-k * dr[0], -k * dr[1], -k * dr[2]);
      } else {
        const double2 ab = pair[(size_t)p * L.stride + g.row];
        T::d2(pi, T::load(A, aj), B, dr);
        const R k = ab.x - ab.y * (ieb_i + ieb[aj]);
        acc.add(-k * dr[0], -k * dr[1], -k * dr[2]);
      }
      aj = aj_next;
    }
  }
  acc.template reduce<TPA>();
  const int lane = threadIdx.x & 31, slot = (threadIdx.x >> 5) * RPW + lane % RPW;
  if (g.sub == 0) {
    s_f[0][slot] = acc.get(0);
    s_f[1][slot] = acc.get(1);
    s_f[2][slot] = acc.get(2);
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int r = blockIdx.x * 32 + threadIdx.x;
    if (r < L.rows) {
      const int ar = L.pidx[r];
      if (L.nnum[r] > 0 || E.store || E.kick) {
        if constexpr (PREC)
          finish_force_drift(A, E, B, ctl, ar, s_f[0][threadIdx.x], s_f[1][threadIdx.x], s_f[2][threadIdx.x]);
        else
          finish_force(A, E, ar, s_f[0][threadIdx.x], s_f[1][threadIdx.x], s_f[2][threadIdx.x]);
      }
    }
  }
}

void launch_rjl(bool prec, bool energy, const ListDev& L, const RJLPar& P, const Atoms& A, const Box& B, void* Eb,
                double2* pair, Ctl* ctl, int eslot, int ekey, cudaStream_t s, int parts, const Epi& E) {
  if (L.rows == 0) {
    if (energy && (parts & 1)) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    if (E.begin && (parts & 1)) launch_step_begin_fused(ctl, s);
    return;
  }
  with_bool(prec, [&](auto pr) {
    constexpr bool PR = decltype(pr)::value;
    if (parts & 1) {
      const int tpa1 = L.tpa1 > 0 ? L.tpa1 : L.tpa;
      const int grid = nblk((long long)L.rows * tpa1, 256);
      with_tpa(tpa1, [&](auto t) {
        constexpr int TP = decltype(t)::value;
        if (energy)
          launch_dependent(k_rjl_density<PR, true, TP>, grid, 256, s, L, P, A, B, Eb, pair, ctl, eslot, ekey,
                           E.eatom, E.begin);
        else
          launch_dependent(k_rjl_density<PR, false, TP>, grid, 256, s, L, P, A, B, Eb, pair, ctl, eslot, ekey,
                           (double*)nullptr, E.begin);
        ++g_kernel_launches;
      });
    }
    if (parts & 2) {
      // 32 rows per block
      const int grid = nblk(L.rows, 32);
      with_tpa(L.tpa, [&](auto t) {
        constexpr int TP = decltype(t)::value;
        launch_dependent(k_rjl_force<PR, TP>, grid, 32 * TP, s, L, P, A, B, (const void*)Eb, (const double2*)pair,
                         ctl, E);
        ++g_kernel_launches;
      });
    }
  });
}

}  // namespace pfmd

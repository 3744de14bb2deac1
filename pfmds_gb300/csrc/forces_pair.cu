// lj and lj1g pair forces (see forces.cuh for the execution scheme).
#include "forces.cuh"

namespace pfmd {

// lj: LennardJones.f90:23-69 (cosine switch, full list, force on the row atom)
template <bool PREC, bool ENERGY, int TPA>
__global__ void __launch_bounds__(256) k_lj(ListDev L, LJPar P, Atoms A, Box B, Ctl* ctl, int eslot, int ekey,
                                            Epi E) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const Grp<TPA> g;
  const bool valid = g.row < L.rows;
  const int n = valid ? L.nnum[g.row] : 0;
  const int ai = valid ? L.pidx[g.row] : 0;
  const auto& c = cst<PREC>(P);
  Acc3<PREC> acc;
  Acc1<PREC> e;
  if (n > 0) {
    const auto pi = T::load(A, ai);
#pragma unroll 4
    for (int p = g.sub; p < n; p += TPA) {
      R dr[3];
      const R r = xsqrt<PREC>(T::d2(pi, T::load(A, ent(L, g.row, p)), B, dr));
      if (r < c.R2) {
        const R ir = xrcp<PREC>(r);
        const R x = c.sig * ir, x2 = x * x, V = x2 * x2 * x2;
        R fc, dfc;
        fdfc<PREC>(r, c.R1, c.R2, c.inv_w, fc, dfc);
        const R k = c.eps4 * (V * (R(12) * V - R(6)) * (ir * ir) * fc - V * (V - R(1)) * dfc);
        acc.add(-k * dr[0], -k * dr[1], -k * dr[2]);
        if (ENERGY) e.add(c.eps4 * V * (V - R(1)) * fc);
      }
    }
  }
  acc.template reduce<TPA>();
  if (ENERGY) e.template reduce<TPA>();
  if (valid && (n > 0 || E.store || E.kick) && g.sub == 0) finish_force(A, E, ai, acc.get(0), acc.get(1), acc.get(2));
  if (ENERGY) energy_reduce(ctl, eslot, ekey, (n > 0 && g.sub == 0) ? e.get() : 0.0);
}

// lj1g: LennardJones_1g.f90:28-117.  The reference walks the half list
// p <= lessnnum(i) and applies -fp to i and +fp to the partner.  Gathering over the
// full list, atom i receives -F(r) dr once for every pair in its own half list and
// once for every pair whose half list holds i; with a group in ascending atom order
// every pair is in exactly one of the two half lists (weight 1).  GENERAL keeps the
// weights for any group order: w = [p < lessnnum(i)] + [i < bnd(j)].
// Requires list groups g1 == g2, as the reference's particle_index(nlist(p,i)) does.
template <bool PREC, bool ENERGY, bool GENERAL, int TPA>
__global__ void __launch_bounds__(256) k_lj1g(ListDev L, LJPar P, Atoms A, Box B, Ctl* ctl, int eslot, int ekey,
                                              Epi E) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const Grp<TPA> g;
  const bool valid = g.row < L.rows;
  const int n = valid ? L.nnum[g.row] : 0;
  const int ai = valid ? L.pidx[g.row] : 0;
  const auto& c = cst<PREC>(P);
  Acc3<PREC> acc;
  Acc1<PREC> e;
  if (n > 0) {
    const int less = L.lessnnum[g.row];
    const auto pi = T::load(A, ai);
#pragma unroll 4
    for (int p = g.sub; p < n; p += TPA) {
      const int aj = ent(L, g.row, p);
      R dr[3];
      const R r2 = T::d2(pi, T::load(A, aj), B, dr);
      const R r = xsqrt<PREC>(r2);
      if (r < c.R2) {  // beyond R2 the clamped switch makes force and energy exactly zero
        R w = R(1);
        if (GENERAL) w = R((p < less ? 1 : 0) + (g.row < L.bnd[L.row_of[aj]] ? 1 : 0));
        const R invr2 = xrcp<PREC>(r2);
        const R U = invr2 * invr2 * invr2;
        R fcut, dfr;
        f_dfr_cut<R>(r, c.R1, c.R2, fcut, dfr);
        const R F = w * (U * invr2 * ((c.c12t12 * U - c.c6t6) * fcut - (c.c12 * U - c.c6) * dfr));
        acc.add(-F * dr[0], -F * dr[1], -F * dr[2]);
        // the half list p <= lessnnum(i); in a row kept in cell order (groups in
        // atom order only) that is the partners with a smaller atom index
        if (ENERGY && (L.sorted ? p < less : aj < ai)) {
          R fp;
          if constexpr (PREC) {
            const R x = (r - c.R1) * c.inv_w;
            fp = r <= c.R1 ? R(1) : R(1) + x * x * x * (R(-10) + R(15) * x - R(6) * x * x);
          } else {
            fp = fcut_poly(r, c.R1, c.R2);
          }
          e.add(U * (c.c12 * U - c.c6) * fp);
        }
      }
    }
  }
  acc.template reduce<TPA>();
  if (ENERGY) e.template reduce<TPA>();
  if (valid && (n > 0 || E.store || E.kick) && g.sub == 0) finish_force(A, E, ai, acc.get(0), acc.get(1), acc.get(2));
  if (ENERGY) energy_reduce(ctl, eslot, ekey, (n > 0 && g.sub == 0) ? e.get() : 0.0);
}

void launch_lj(bool prec, bool energy, const ListDev& L, const LJPar& P, const Atoms& A, const Box& B, Ctl* ctl,
               int eslot, int ekey, cudaStream_t s, const Epi& E) {
  if (L.rows == 0) {
    if (energy) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int grid = nblk((long long)L.rows * L.tpa, 256);
  with_bool(prec, [&](auto pr) {
    with_bool(energy, [&](auto en) {
      with_tpa(L.tpa, [&](auto t) {
        k_lj<decltype(pr)::value, decltype(en)::value, decltype(t)::value>
            <<<grid, 256, 0, s>>>(L, P, A, B, ctl, eslot, ekey, E);
        ++g_kernel_launches;
      });
    });
  });
}

void launch_lj1g(bool prec, bool energy, bool general, const ListDev& L, const LJPar& P, const Atoms& A,
                 const Box& B, Ctl* ctl, int eslot, int ekey, cudaStream_t s, const Epi& E) {
  if (L.rows == 0) {
    if (energy) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int grid = nblk((long long)L.rows * L.tpa, 256);
  with_bool(prec, [&](auto pr) {
    with_bool(energy, [&](auto en) {
      with_bool(general, [&](auto ge) {
        with_tpa(L.tpa, [&](auto t) {
          k_lj1g<decltype(pr)::value, decltype(en)::value, decltype(ge)::value, decltype(t)::value>
              <<<grid, 256, 0, s>>>(L, P, A, B, ctl, eslot, ekey, E);
          ++g_kernel_launches;
        });
      });
    });
  });
}

}  // namespace pfmd

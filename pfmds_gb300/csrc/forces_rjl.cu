// rjl (Rosato-Guillope-Legrand, second-moment tight binding) forces and energy,
// RosatoGuillopeLegrand.f90:23-94.  Pass 1 (density) forms
// Eb_i = sqrt(sum exp(-2q(r/r0-1)) fc), stores 1/Eb per atom and, at energy steps,
// the row energy A0*Er - xi*Eb; pass 2 gathers the pair forces with
// 1/Eb_i + 1/Eb_j.  See forces.cuh for the execution scheme.
#include "forces.cuh"

namespace pfmd {

// inv_eb holds 1/Eb per atom: double for the plain form, float for the precision form.
template <bool PREC, bool ENERGY, int TPA>
__global__ void __launch_bounds__(256) k_rjl_density(ListDev L, RJLPar P, Atoms A, Box B, void* inv_eb, Ctl* ctl,
                                                     int eslot, int ekey) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const Grp<TPA> g;
  const bool valid = g.row < L.rows;
  const int n = valid ? L.nnum[g.row] : 0;
  const int ai = valid ? L.pidx[g.row] : 0;
  Acc1<PREC> eb2, er;
  if (n > 0) {
    const auto pi = T::load(A, ai);
    const R R1 = (R)P.R1, R2 = (R)P.R2, inv_r0 = (R)(1.0 / P.r0), m2q = (R)(-2.0 * P.q), mp = (R)(-P.p),
            inv_w = (R)(1.0 / (P.R2 - P.R1));
    for (int p = g.sub; p < n; p += TPA) {
      R dr[3];
      const R r = xsqrt<PREC>(T::d2(pi, T::load(A, ent(L, g.row, p)), B, dr));
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
  eb2.template reduce<TPA>();
  if (ENERGY) er.template reduce<TPA>();
  double erow = 0.0;
  if (valid && g.sub == 0) {
    const double eb = sqrt(eb2.get());
    if constexpr (PREC)
      static_cast<float*>(inv_eb)[ai] = (float)(1.0 / eb);
    else
      static_cast<double*>(inv_eb)[ai] = 1.0 / eb;
    if (ENERGY) erow = P.A0 * er.get() - P.xi * eb;
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

template <bool PREC, int TPA>
__global__ void __launch_bounds__(256) k_rjl_force(ListDev L, RJLPar P, Atoms A, Box B, const void* inv_eb,
                                                   Ctl* ctl) {
  using T = RT<PREC>;
  using R = typename T::R;
  using IE = typename std::conditional<PREC, float, double>::type;
  const IE* ieb = static_cast<const IE*>(inv_eb);
  if (ctl->stop) return;
  const Grp<TPA> g;
  const int n = g.row < L.rows ? L.nnum[g.row] : 0;
  const int ai = n > 0 ? L.pidx[g.row] : 0;
  Acc3<PREC> acc;
  if (n > 0) {
    const auto pi = T::load(A, ai);
    const R R1 = (R)P.R1, R2 = (R)P.R2, inv_r0 = (R)(1.0 / P.r0), m2q = (R)(-2.0 * P.q), mp = (R)(-P.p),
            inv_w = (R)(1.0 / (P.R2 - P.R1));
    const R a2 = (R)(2.0 * P.A0), pr0 = (R)(P.p / P.r0), qr0 = (R)(P.q / P.r0), xi = (R)P.xi;
    const R ieb_i = ieb[ai];
    for (int p = g.sub; p < n; p += TPA) {
      const int aj = ent(L, g.row, p);
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
        const R T2 = xi * (qr0 * fc - dfc * R(0.5) * r) * (ieb_i + (R)ieb[aj]) * eq;
        const R c = (T1 - T2) / r;
        acc.add(-c * dr[0], -c * dr[1], -c * dr[2]);
      }
    }
  }
  acc.template reduce<TPA>();
  if (n > 0 && g.sub == 0) add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
}

void launch_rjl(bool prec, bool energy, const ListDev& L, const RJLPar& P, const Atoms& A, const Box& B, void* Eb,
                Ctl* ctl, int eslot, int ekey, cudaStream_t s, int parts) {
  if (L.rows == 0) {
    if (energy && (parts & 1)) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int grid = nblk((long long)L.rows * L.tpa, 256);
  with_bool(prec, [&](auto pr) {
    with_tpa(L.tpa, [&](auto t) {
      constexpr bool PR = decltype(pr)::value;
      constexpr int TP = decltype(t)::value;
      if (parts & 1) {
        if (energy)
          k_rjl_density<PR, true, TP><<<grid, 256, 0, s>>>(L, P, A, B, Eb, ctl, eslot, ekey);
        else
          k_rjl_density<PR, false, TP><<<grid, 256, 0, s>>>(L, P, A, B, Eb, ctl, eslot, ekey);
        ++g_kernel_launches;
      }
      if (parts & 2) {
        k_rjl_force<PR, TP><<<grid, 256, 0, s>>>(L, P, A, B, Eb, ctl);
        ++g_kernel_launches;
      }
    });
  });
}

}  // namespace pfmd

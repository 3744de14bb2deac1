// ljc / morsec: LennardJonesCosine.f90 and MorseCosine.f90 (26-139).
// Graphene side (rows of nl(1)): the pair term with the row's normal plus, unless
// `simplified`, the term through the normals of its three nearest neighbours j
// (dn_j/dr_i).  Metal side (rows of nl(2)): the pair term with the neighbour's
// normal; morsec divides that cosine by |n| (MorseCosine.f90:127), ljc does not.
// Normals are stored per atom.  See forces.cuh for the execution scheme.
#include "forces.cuh"

namespace pfmd {

// The cosine power V3 = (|n.d| / (|n| r))^delta (|n| only where `scaled`:
// morsec's metal side) and V3 / (n.d).  For delta = 2, the parameter files'
// value (Cosc::idelt), both are products (no FP64 divide, no pow); otherwise pow
// and a divide as written.  (At n.d = 0 the written quotient is 0/0 where the
// product gives 0: the partner would lie in the plane through the atom normal
// to n, which a sheet coupled to a slab never forms.)
template <bool PREC>
__device__ __forceinline__ void cos_v3(const Cosc<typename RT<PREC>::R>& c, typename RT<PREC>::R nd,
                                       typename RT<PREC>::R ir, typename RT<PREC>::R inn2, bool scaled,
                                       typename RT<PREC>::R& V3, typename RT<PREC>::R& V3n) {
  using R = typename RT<PREC>::R;
  if (c.idelt == 2) {
    const R u = nd * ir, s = scaled ? inn2 : R(1);
    V3 = u * u * s;
    V3n = u * ir * s;
  } else {
    const R x = fabs(nd) * ir;
    V3 = xpow<PREC>(scaled ? x * xsqrt<PREC>(inn2) : x, c.delt);
    V3n = V3 / nd;
  }
}

// One pair (r, its reciprocal ir, dr, the normal nv; inn2 = 1/|nv|^2 on morsec's
// metal side): X, Y with F = pref (X dr + Y nv), and the energy E.
template <bool PREC, bool MORSE>
__device__ __forceinline__ void cos_pair(const CosPar& P, typename RT<PREC>::R r, typename RT<PREC>::R ir,
                                         const typename RT<PREC>::R* dr, const typename RT<PREC>::R* nv,
                                         typename RT<PREC>::R inn2, bool metal, typename RT<PREC>::R& X,
                                         typename RT<PREC>::R& Y, typename RT<PREC>::R& E) {
  using R = typename RT<PREC>::R;
  const auto& c = cst<PREC>(P);
  const R R1 = c.R1, R2 = c.R2, delt = c.delt, inv_w = c.inv_w;
  const R nd = nv[0] * dr[0] + nv[1] * dr[1] + nv[2] * dr[2];
  R fc, dfc;
  fdfc<PREC>(r, ir, R1, R2, inv_w, fc, dfc);
  R V3, V3n;
  if (!MORSE) {
    const R x = c.sig * ir, x2 = x * x, V2 = x2 * x2 * x2, V1 = V2 * V2;
    cos_v3<PREC>(c, nd, ir, R(1), false, V3, V3n);
    X = (R(12) * V1 - (R(6) + delt) * V2 * V3) * (ir * ir) * fc - (V1 - V2 * V3) * dfc;
    Y = delt * V2 * V3n * fc;
    E = (V1 - V2 * V3) * fc;
  } else {
    const R a = c.a;
    const R V2 = xexp<PREC>(-a * (r - c.r0)), V1 = V2 * V2;
    cos_v3<PREC>(c, nd, ir, inn2, metal, V3, V3n);
    X = R(2) * (a * V1 - (a + delt * ir) * V2 * V3) * ir * fc - (V1 - R(2) * V2 * V3) * dfc;
    Y = R(2) * delt * V2 * V3n * fc;
    E = (V1 - R(2) * V2 * V3) * fc;
  }
}

// Graphene side, the pair terms.  Unless `simplified`, each row also stores
// G_i = sum_p pref Y_ip dr_ip (Y the pair's normal coefficient, dr to partner p):
// the normal-derivative term of every row i' with i among its three nearest
// neighbours is a function of G_i and of the geometry of i's three neighbours
// only (k_cos_nderiv), so the partners are visited once instead of four times.
template <bool PREC, bool ENERGY, bool MORSE, int TPA>
__global__ void __launch_bounds__(256) k_cos_graphene(ListDev nl, CosPar P, const double4_32a* norm,
                                                      double4_32a* gsum, Atoms A, Box B, Ctl* ctl, int eslot,
                                                      int ekey) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const Grp<TPA> g;
  const bool valid = g.row < nl.rows;
  const int i = g.row;
  Acc3<PREC> acc, gacc;
  Acc1<PREC> e;
  const int ai = valid ? nl.pidx[i] : 0;
  const auto& c = cst<PREC>(P);
  const R pref = c.pref;
  if (valid) {
    const auto pi = T::load(A, ai);
    const R R2 = c.R2;
    const double4_32a ni = norm[ai];
    const R nv[3] = {(R)ni.x, (R)ni.y, (R)ni.z};
    const int n = nl.nnum[i];
    for (int p = g.sub; p < n; p += TPA) {
      R dr[3];
      const R r2 = T::d2(pi, T::load(A, ent(nl, i, p)), B, dr);
      const R ir = xrsqrt<PREC>(r2), r = r2 * ir;
      if (r < R2) {
        R X, Y, E;
        cos_pair<PREC, MORSE>(P, r, ir, dr, nv, R(1), false, X, Y, E);
        acc.add(-pref * (X * dr[0] + Y * nv[0]), -pref * (X * dr[1] + Y * nv[1]), -pref * (X * dr[2] + Y * nv[2]));
        const R py = pref * Y;
        gacc.add(py * dr[0], py * dr[1], py * dr[2]);
        if (ENERGY) e.add(pref * E);
      }
    }
  }
  acc.template reduce<TPA>();
  if (!P.simplified) gacc.template reduce<TPA>();
  if (ENERGY) e.template reduce<TPA>();
  if (valid && g.sub == 0) {
    add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
    if (!P.simplified) gsum[i] = double4_32a{gacc.get(0), gacc.get(1), gacc.get(2), 0.0};
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, (valid && g.sub == 0) ? e.get() : 0.0);
}

// The normal-derivative term of the graphene side (the dn_j/dr_i part of
// LennardJonesCosine.f90 / MorseCosine.f90 when not simplified).  For each of
// row i's three nearest neighbours j, j's partners p contribute
// -(pref Y_jp / A_ij) (dr_jp . w_ij) n_j, with A_ij and w_ij formed from the
// positions of j's three neighbours (i among them); A_ij and w_ij do not depend
// on p, so the sum over p is -((w_ij . G_j) / A_ij) n_j with k_cos_graphene's
// G_j.  One thread per row; the force adds to the pair terms'.
template <bool PREC>
__global__ void __launch_bounds__(256) k_cos_nderiv(ListDev nl, ListDev nn, const double4_32a* norm,
                                                    const double4_32a* gsum, Atoms A, Box B, Ctl* ctl) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl.rows) return;
  const int ai = nl.pidx[i];
  double f[3] = {0.0, 0.0, 0.0};
  for (int q = 0; q < 3; ++q) {
    const int j = ent(nn, i, q);
    if (j < 0 || j >= nn.rows || j >= nl.rows || j >= nn.row_cap) {
      // a neighbour outside the graphene rows (groups 5/6 of the list differ)
      set_error(ctl, ST_PARAM, EK_NONE, i + 1, j + 1, 0);
      break;
    }
    int l1 = 0;
    for (; l1 < 3; ++l1)
      if (ent(nn, j, l1) == i) break;
    if (l1 >= 3) {
      set_error(ctl, ST_GR_NN, EK_L1, i + 1, j + 1, 0);
      break;
    }
    const int l2 = (l1 + 1) % 3, l3 = (l1 + 2) % 3;
    const int aj = nn.row_idx[j];
    const auto pj = T::load(A, aj);
    R dl[3][3];
#pragma unroll
    for (int l = 0; l < 3; ++l) T::d2(pj, T::load(A, nn.col_idx[ent(nn, j, l)]), B, dl[l]);
    R d12[3], d31[3], d23[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      d12[k] = dl[l2][k] - dl[l1][k];
      d31[k] = dl[l1][k] - dl[l3][k];
      d23[k] = dl[l3][k] - dl[l2][k];
    }
    const R Aa = dot3<PREC>(d12, d12) * dot3<PREC>(d31, d31) - dot3<PREC>(d12, d31) * dot3<PREC>(d12, d31);
    const R s2331 = dot3<PREC>(d23, d31), s2312 = dot3<PREC>(d23, d12);
    const double4_32a G = gsum[j];
    double wg = 0.0;
    wg += (double)(d12[0] * s2331 - d31[0] * s2312) * G.x;
    wg += (double)(d12[1] * s2331 - d31[1] * s2312) * G.y;
    wg += (double)(d12[2] * s2331 - d31[2] * s2312) * G.z;
    const double k = wg / (double)Aa;
    const double4_32a nj = norm[nl.pidx[j]];
    f[0] -= k * (double)(R)nj.x;
    f[1] -= k * (double)(R)nj.y;
    f[2] -= k * (double)(R)nj.z;
  }
  add_force(A, ai, f[0], f[1], f[2]);
}

template <bool PREC, bool MORSE, int TPA>
__global__ void __launch_bounds__(256) k_cos_metal(ListDev nl, CosPar P, const double4_32a* norm, Atoms A, Box B,
                                                   Ctl* ctl) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const Grp<TPA> g;
  const int n = g.row < nl.rows ? nl.nnum[g.row] : 0;
  const int ai = n > 0 ? nl.pidx[g.row] : 0;
  Acc3<PREC> acc;
  if (n > 0) {
    const auto pi = T::load(A, ai);
    const auto& c = cst<PREC>(P);
    const R R2 = c.R2;
    const R pref = c.pref;
    for (int p = g.sub; p < n; p += TPA) {
      const int aj = ent(nl, g.row, p);
      R dr[3];
      const R r2 = T::d2(pi, T::load(A, aj), B, dr);
      const R ir = xrsqrt<PREC>(r2), r = r2 * ir;
      if (r < R2) {
        const double4_32a gn = norm[aj];
        const R nv[3] = {(R)gn.x, (R)gn.y, (R)gn.z};
        const R inn2 = MORSE ? (R)gn.w : R(1);  // 1/|n|^2, formed with the normal
        R X, Y, E;
        cos_pair<PREC, MORSE>(P, r, ir, dr, nv, inn2, true, X, Y, E);
        acc.add(-pref * (X * dr[0] + Y * nv[0]), -pref * (X * dr[1] + Y * nv[1]), -pref * (X * dr[2] + Y * nv[2]));
      }
    }
  }
  acc.template reduce<TPA>();
  if (n > 0 && g.sub == 0) add_force(A, ai, acc.get(0), acc.get(1), acc.get(2));
}

void launch_cos(bool prec, bool energy, bool morse, const ListDev& nl1, const ListDev& nl2, const ListDev& nn,
                const CosPar& P, const double4_32a* norm, double4_32a* gsum, const Atoms& A, const Box& B, Ctl* ctl,
                int eslot, int ekey, cudaStream_t s, int parts) {
  with_bool(prec, [&](auto pr) {
    with_bool(morse, [&](auto mo) {
      constexpr bool PR = decltype(pr)::value, MO = decltype(mo)::value;
      if (parts & 1) {
        if (nl1.rows > 0) {
          const int grid = nblk((long long)nl1.rows * nl1.tpa, 256);
          with_tpa(nl1.tpa, [&](auto t) {
            constexpr int TP = decltype(t)::value;
            if (energy)
              k_cos_graphene<PR, true, MO, TP><<<grid, 256, 0, s>>>(nl1, P, norm, gsum, A, B, ctl, eslot, ekey);
            else
              k_cos_graphene<PR, false, MO, TP><<<grid, 256, 0, s>>>(nl1, P, norm, gsum, A, B, ctl, eslot, ekey);
            ++g_kernel_launches;
          });
          if (!P.simplified) {
            k_cos_nderiv<PR><<<nblk(nl1.rows, 256), 256, 0, s>>>(nl1, nn, norm, gsum, A, B, ctl);
            ++g_kernel_launches;
          }
        } else if (energy) {
          cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
        }
      }
      if ((parts & 2) && nl2.rows > 0) {
        const int grid = nblk((long long)nl2.rows * nl2.tpa, 256);
        with_tpa(nl2.tpa, [&](auto t) {
          k_cos_metal<PR, MO, decltype(t)::value><<<grid, 256, 0, s>>>(nl2, P, norm, A, B, ctl);
          ++g_kernel_launches;
        });
      }
    });
  });
}

}  // namespace pfmd

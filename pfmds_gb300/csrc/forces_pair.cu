// lj and lj1g pair forces (see forces.cuh for the execution scheme).
#include "forces.cuh"

namespace pfmd {

// One list row of lj: thread `sub` of the row's TPA threads adds its share of
// the row's force to acc and (ENERGY) of its energy to e.
template <bool PREC, bool ENERGY, int TPA, class LT>
__device__ __forceinline__ void lj_row(const LT& L, const LJc<typename RT<PREC>::R>& c, const Atoms& A,
                                       const Box& B, int row, int sub, int n, const typename RT<PREC>::P4& pi,
                                       Acc3<PREC>& acc, Acc1<PREC>& e) {
  using T = RT<PREC>;
  using R = typename T::R;
#pragma unroll 4
  for (int p = sub; p < n; p += TPA) {
    R dr[3];
    const R r2 = T::d2(pi, T::load(A, ent(L, row, p)), B, dr);
    // plain: r and 1/r from one reciprocal square root (no FP64 divide)
    R r, ir;
    if constexpr (PREC) {
      r = xsqrt<PREC>(r2);
      ir = xrcp<PREC>(r);
    } else {
      ir = rsqrt(r2);
      r = r2 * ir;
    }
    if (r < c.R2) {
      const R x = c.sig * ir, x2 = x * x, V = x2 * x2 * x2;
      R fc, dfc;
      fdfc<PREC>(r, ir, c.R1, c.R2, c.inv_w, fc, dfc);
      const R k = c.eps4 * (V * (R(12) * V - R(6)) * (ir * ir) * fc - V * (V - R(1)) * dfc);
      acc.add(-k * dr[0], -k * dr[1], -k * dr[2]);
      if (ENERGY) e.add(c.eps4 * V * (V - R(1)) * fc);
    }
  }
}

// One list row of lj1g (row atom ai), as lj_row.
template <bool PREC, bool ENERGY, bool GENERAL, int TPA, class LT>
__device__ __forceinline__ void lj1g_row(const LT& L, const LJc<typename RT<PREC>::R>& c, const Atoms& A,
                                         const Box& B, int row, int sub, int n, int ai,
                                         const typename RT<PREC>::P4& pi, Acc3<PREC>& acc, Acc1<PREC>& e) {
  using T = RT<PREC>;
  using R = typename T::R;
  const int less = L.lessnnum[row];
#pragma unroll 4
  for (int p = sub; p < n; p += TPA) {
    const int aj = ent(L, row, p);
    R dr[3];
    const R r2 = T::d2(pi, T::load(A, aj), B, dr);
    R r, invr2;
    if constexpr (PREC) {
      r = xsqrt<PREC>(r2);
    } else {  // r and 1/r^2 from one reciprocal square root (no FP64 divide)
      const R ir = rsqrt(r2);
      r = r2 * ir;
      invr2 = ir * ir;
    }
    if (r < c.R2) {  // beyond R2 the clamped switch makes force and energy exactly zero
      R w = R(1);
      if (GENERAL) w = R((p < less ? 1 : 0) + (row < L.bnd[L.row_of[aj]] ? 1 : 0));
      if constexpr (PREC) invr2 = xrcp<PREC>(r2);
      const R U = invr2 * invr2 * invr2;
      R fcut, dfr;
      f_dfr_cut<R>(r, c.R1, c.R2, c.inv_w, fcut, dfr);
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
  if (n > 0) lj_row<PREC, ENERGY, TPA>(L, c, A, B, g.row, g.sub, n, T::load(A, ai), acc, e);
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
  if (n > 0) lj1g_row<PREC, ENERGY, GENERAL, TPA>(L, c, A, B, g.row, g.sub, n, ai, T::load(A, ai), acc, e);
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

// All lj / lj1g lists in one launch, atom-major (see PairSet).  A block takes
// (256 / 32) * (32 / TPA) consecutive atoms per pass, TPA threads per atom; the
// atoms of a warp may head different numbers of rows, so every thread loops to
// the warp's largest task count and the shuffles of the reductions see the
// whole warp.  The per-atom epilogue (FP64 force store, kick, kinetic energy) is
// the FP64 pipe's work, which is scarce on this GPU: the reduced forces go
// through shared memory and the epilogue runs with one atom per thread, so a
// warp's FP64 instructions serve 32 atoms instead of 32 / TPA.  Energies (per
// interaction) and the chain's kinetic energy go through one grid reduction;
// its last block stores the energies and updates the chain.
// Register budgets by resident blocks per SM: the precision variants at three
// (80 registers, no spills, where the compiler's own choice of 64 registers
// spilled 536 bytes: the 4,000-atom gas step 34.3 us against 32.8), the plain
// variants at two (at most 128 registers, as the 106 they took before).
template <bool PREC, bool ENERGY, int TPA>
__global__ void __launch_bounds__(256, PREC ? 3 : 2) k_pair_atoms(PairSet S, Atoms A, Box B, Ctl* ctl, Epi E, int chain,
                                                    double ts2, double ts3, double ts4, int ahead) {
  using T = RT<PREC>;
  constexpr int RPW = 32 / TPA, APB = 8 * RPW;  // atoms per warp, per block pass (256 threads)
  __shared__ double s_f[3][APB];
  __shared__ double s_e[ENERGY ? kMaxPairKeys : 1][APB];
  __shared__ PairSlot s_slot[kMaxPairSlots];
  const int lane = threadIdx.x & 31, sub = lane / RPW, w = threadIdx.x >> 5;
  const int slot = w * RPW + lane % RPW;
  // The slot table and the atoms' task ranges are set up once per system and
  // written by no kernel of the step: they are read before the wait on the
  // previous kernel, whose tail they then overlap.
  {
    constexpr int W = sizeof(PairSlot) / sizeof(int);
    static_assert(sizeof(PairSlot) % sizeof(int) == 0, "PairSlot copies as ints");
    const int* src = reinterpret_cast<const int*>(S.slots);
    int* dst = reinterpret_cast<int*>(s_slot);
    for (int k = threadIdx.x; k < S.nslot * W; k += blockDim.x) dst[k] = src[k];
  }
  const int a_first = blockIdx.x * APB + slot;
  const int t0_first = a_first < S.natoms ? S.task_off[a_first] : 0;
  const int t1_first = a_first < S.natoms ? S.task_off[a_first + 1] : 0;
  asm volatile("griddepcontrol.wait;" ::: "memory");  // see launch_dependent
  if (block_stop(ctl)) return;  // (its barrier also publishes s_slot)
  double red[kMaxPairKeys + 1] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int bbase = blockIdx.x * APB; bbase < S.natoms; bbase += gridDim.x * APB) {  // uniform over the block
    const int a = bbase + slot;
    const bool valid = a < S.natoms;
    const bool first = bbase == blockIdx.x * APB;
    const int t0 = first ? t0_first : (valid ? S.task_off[a] : 0);
    const int nt = first ? t1_first - t0_first : (valid ? S.task_off[a + 1] - t0 : 0);
    int ntw = nt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ntw = max(ntw, __shfl_xor_sync(0xffffffffu, ntw, o));
    Acc3<PREC> acc;
    Acc1<PREC> e[kMaxPairKeys];
    const auto pi = T::load(A, valid ? a : 0);
    for (int t = 0; t < ntw; ++t) {
      if (t >= nt) continue;
      const int2 tk = S.task[t0 + t];
      // the slot's list and constants into registers once per row
      const PairSlot& sl = s_slot[tk.x];
      const RowList L = sl.L;
      const auto c = cst<PREC>(sl.P);
      const int kind = sl.kind, general = sl.general, ekey = sl.ekey;
      const int n = L.nnum[tk.y];
      Acc1<PREC> et;
      if (kind == 0)
        lj_row<PREC, ENERGY, TPA>(L, c, A, B, tk.y, sub, n, pi, acc, et);
      else if (general)
        lj1g_row<PREC, ENERGY, true, TPA>(L, c, A, B, tk.y, sub, n, a, pi, acc, et);
      else
        lj1g_row<PREC, ENERGY, false, TPA>(L, c, A, B, tk.y, sub, n, a, pi, acc, et);
      if (ENERGY && ekey >= 0) {
#pragma unroll
        for (int k = 0; k < kMaxPairKeys; ++k)
          if (k == ekey) e[k].add(static_cast<typename T::R>(et.get()));
      }
    }
    acc.template reduce<TPA>();
    if (ENERGY) {
#pragma unroll
      for (int k = 0; k < kMaxPairKeys; ++k) e[k].template reduce<TPA>();
    }
    if (sub == 0) {
      s_f[0][slot] = acc.get(0);
      s_f[1][slot] = acc.get(1);
      s_f[2][slot] = acc.get(2);
      if (ENERGY) {
#pragma unroll
        for (int k = 0; k < kMaxPairKeys; ++k) s_e[k][slot] = e[k].get();
      }
    }
    __syncthreads();
    if (threadIdx.x < APB) {
      const int ae = bbase + threadIdx.x;
      if (ae < S.natoms) {
        finish_force(A, E, ae, s_f[0][threadIdx.x], s_f[1][threadIdx.x], s_f[2][threadIdx.x]);
        if (ENERGY) {
#pragma unroll
          for (int k = 0; k < kMaxPairKeys; ++k) red[k] += s_e[k][threadIdx.x];
        }
        if (chain >= 0 && (E.mflag[ae] & 4)) red[kMaxPairKeys] += ke_of(A, ae);
      }
    }
    __syncthreads();  // s_f is rewritten by the next pass
  }
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (!ENERGY && chain < 0) return;
  // only the epilogue threads (the first APB of the block) hold sums: each
  // splits its FP64 sums into float-float pairs, and their warps merge them in
  // FP32 (no FP64 shuffles; each FP64 instruction costs a full warp's issue on
  // this GPU's FP64 pipe), then the grid sum runs in float-float as well
  constexpr int EW = (APB + 31) / 32;
  float fs[kMaxPairKeys + 1], fcmp[kMaxPairKeys + 1];
#pragma unroll
  for (int k = 0; k <= kMaxPairKeys; ++k) {
    fs[k] = (float)red[k];
    fcmp[k] = (float)((double)fs[k] - red[k]);  // value = fs - fcmp
  }
  if (w < EW) {
#pragma unroll
    for (int k = 0; k <= kMaxPairKeys; ++k) gmerge<32>(fs[k], fcmp[k]);
  }
  if constexpr (EW > 1) {
    __shared__ float s_rs[kMaxPairKeys + 1][EW], s_rc[kMaxPairKeys + 1][EW];
    if (w < EW && lane == 0) {
#pragma unroll
      for (int k = 0; k <= kMaxPairKeys; ++k) {
        s_rs[k][w] = fs[k];
        s_rc[k][w] = fcmp[k];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k <= kMaxPairKeys; ++k)
        for (int q = 1; q < EW; ++q) {
          const float s2 = s_rs[k][q], c2 = s_rc[k][q];
          const float t = fs[k] + s2, bb = t - fs[k];
          const float e = (fs[k] - (t - bb)) + (s2 - bb);
          fcmp[k] = (fcmp[k] + c2) - e;
          fs[k] = t;
        }
    }
  }
  double out[kMaxPairKeys + 1];
  if (!grid_finish_ff<kMaxPairKeys + 1>(ctl, kPairSlot, fs, fcmp, out)) return;
  if (ENERGY) {
#pragma unroll
    for (int k = 0; k < kMaxPairKeys; ++k)
      if (k < S.nkey) ctl->e_inter[S.keys[k]] = out[k];
  }
  if (chain >= 0) {
    nhc_chain_update(ctl->nhc[chain], out[kMaxPairKeys], ts2, ts3, ts4);
    if (ahead) {
      // the next step's first half-update: its kinetic energy is this one's after
      // the scaling, s^2 ke (the form the chain's own second part uses); the next
      // kick-drift applies s_a, then the new s, to the velocities
      const double sa = ctl->nhc[chain].s;
      ctl->nhc_sa = sa;
      nhc_chain_update(ctl->nhc[chain], out[kMaxPairKeys] * (sa * sa), ts2, ts3, ts4);
    }
  }
}

void launch_pair_atoms(bool prec, bool energy, const PairSet& S, const Atoms& A, const Box& B, Ctl* ctl,
                       cudaStream_t s, const Epi& E, int chain, double ts2, double ts3, double ts4, bool ahead) {
  if (S.natoms <= 0) return;
  // at most 4096 blocks: their partials of the grid reduction fit Ctl::partial
  const long long blocks = nblk((long long)S.natoms * S.tpa, 256);  // 256 threads = 8 * 32 / TPA atoms
  const int grid = static_cast<int>(blocks < 4096 ? blocks : 4096);
  with_bool(prec, [&](auto pr) {
    with_bool(energy, [&](auto en) {
      with_tpa(S.tpa, [&](auto t) {
        launch_dependent(k_pair_atoms<decltype(pr)::value, decltype(en)::value, decltype(t)::value>, grid, 256, s, S,
                         A, B, ctl, E, chain, ts2, ts3, ts4, ahead ? 1 : 0);
        ++g_kernel_launches;
      });
    });
  });
}

}  // namespace pfmd

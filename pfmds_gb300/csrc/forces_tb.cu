// tb (Tersoff-Brenner bond order) forces and energy, TersoffBrenner.f90:26-150.
// Pass 1: bond orders B(p,i) per list slot; pass 2: forces with the angular terms
// of i's and of each neighbour j's environment and, at energy steps, the bond
// energies for j > i.  Lists hold ~3 partners, so one thread owns a row.
// Requires g1 == g2: a partner's row is row_of[atom].
#include "forces.cuh"

namespace pfmd {

// Pass 1: B(p,i) = (1 + a0 sum_q fc(r_q) g(cos))^-delta for every bond of row i,
// and beside it (at slot nmax + p) B^(1/delta + 1) = B / (1 + a0 sum), the power
// of B the force pass takes (no pow there).  Distances through one reciprocal
// square root per bond (no FP64 divide but the angular term's).
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
  const auto& c = cst<PREC>(P);
  const R R1 = c.R1, R2 = c.R2, a0 = c.a0, c02 = c.c02, d02 = c.d02, delt = c.delt, inv_w = c.inv_w;
  const size_t ex_off = (size_t)L.nmax * L.stride;
  for (int p = 0; p < n; ++p) {
    R dp[3];
    const R r2p = T::d2(pi, T::load(A, ent(L, i, p)), B, dp);
    const R irp = xrsqrt<PREC>(r2p), rp = r2p * irp;
    R b = R(0), bex = R(0);
    if (rp < R2) {
      for (int q = 0; q < n; ++q) {
        if (q == p) continue;
        R dq[3];
        const R r2q = T::d2(pi, T::load(A, ent(L, i, q)), B, dq);
        const R irq = xrsqrt<PREC>(r2q), rq = r2q * irq;
        if (rq < R2) {
          const R cs = dot3<PREC>(dp, dq) * (irp * irq);
          b += fc_only<PREC>(rq, R1, R2, inv_w) * (R(1) + c.c02d02 - c02 / (d02 + (R(1) + cs) * (R(1) + cs)));
        }
      }
      const R base = R(1) + a0 * b;
      b = xpow<PREC>(base, -delt);
      bex = b / base;
    }
    Bb[(size_t)p * L.stride + i] = (double)b;
    Bb[ex_off + (size_t)p * L.stride + i] = (double)bex;
  }
}

template <bool PREC, bool ENERGY>
__global__ void __launch_bounds__(128) k_tb_force(ListDev L, TBPar P, Atoms A, Box B, const double* Bb, Ctl* ctl,
                                                  int eslot, int ekey, Epi E) {
  using T = RT<PREC>;
  using R = typename T::R;
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double erow = 0.0;
  if (i < L.rows && (L.nnum[i] > 0 || E.store || E.kick)) {
    const int n = L.nnum[i];
    const int ai = L.pidx[i];
    const auto pi = T::load(A, ai);
    const auto& c = cst<PREC>(P);
    const R R1 = c.R1, R2 = c.R2, a0 = c.a0, c02 = c.c02, d02 = c.d02, delt = c.delt, s = c.s, bb = c.b,
            r0 = c.r0, inv_w = c.inv_w, sq2s = c.sq2s, sq2os = c.sq2os, pre_e = c.pre_e, is = c.is;
    const size_t ex_off = (size_t)L.nmax * L.stride;
    Acc3<PREC> acc;
    Acc1<PREC> e, eh;
    // Entries at or beyond R2 contribute exactly zero (every term carries fc or
    // its derivative of that bond), so they are skipped: a list longer than the
    // bonds (the learned form's descriptor list) costs little.
    for (int p = 0; p < n; ++p) {
      const int aj = ent(L, i, p);
      R dp[3];
      const R r2p = T::d2(pi, T::load(A, aj), B, dp);
      const R irp = xrsqrt<PREC>(r2p), rp = r2p * irp;
      if (!(rp < R2)) continue;
      const R irp2 = irp * irp;
      const int j = L.row_of[aj];
      R dB[3] = {R(0), R(0), R(0)};
      for (int q = 0; q < n; ++q) {
        if (q == p) continue;
        R dq[3];
        const R r2q = T::d2(pi, T::load(A, ent(L, i, q)), B, dq);
        const R irq = xrsqrt<PREC>(r2q), rq = r2q * irq;
        if (!(rq < R2)) continue;
        const R rr = irp * irq;
        const R cosi = dot3<PREC>(dp, dq) * rr;
        const R it = R(1) / (d02 + (R(1) + cosi) * (R(1) + cosi));
        R fq, dfq;
        fdfc<PREC>(rq, irq, R1, R2, inv_w, fq, dfq);
        const R g1 = fq * R(2) * a0 * c02 * (R(1) + cosi) * (it * it);
        const R g2 = dfq * a0 * (R(1) + c.c02d02 - c02 * it);
        const R irq2 = irq * irq;
#pragma unroll
        for (int k = 0; k < 3; ++k)
          dB[k] += g1 * ((dp[k] + dq[k]) * rr - cosi * (dp[k] * irp2 + dq[k] * irq2)) + g2 * dq[k];
      }
      const R Bpi = (R)Bb[(size_t)p * L.stride + i];
      const R bpe = (R)Bb[ex_off + (size_t)p * L.stride + i];
#pragma unroll
      for (int k = 0; k < 3; ++k) dB[k] *= bpe;
      // i's slot l in j's row, and j's environment
      const int nj = L.nnum[j];
      const auto pj = T::load(A, aj);
      int l = 0;
      for (; l < nj; ++l)
        if (ent(L, j, l) == ai) break;
      R dl[3] = {R(0), R(0), R(0)};
      R rl = R(0), irl = R(0), Blj = R(0), blpe = R(0);
      if (l < nj) {
        const R r2l = T::d2(pj, pi, B, dl);
        irl = xrsqrt<PREC>(r2l);
        rl = r2l * irl;
        Blj = (R)Bb[(size_t)l * L.stride + j];
        blpe = (R)Bb[ex_off + (size_t)l * L.stride + j];
      }
      const R irl2 = irl * irl;
      for (int q = 0; q < nj && l < nj; ++q) {
        if (q == l) continue;
        R dq[3];
        const R r2q = T::d2(pj, T::load(A, ent(L, j, q)), B, dq);
        const R irq = xrsqrt<PREC>(r2q), rq = r2q * irq;
        if (!(rq < R2)) continue;
        const R rr = irl * irq;
        const R cosi = dot3<PREC>(dl, dq) * rr;
        const R it = R(1) / (d02 + (R(1) + cosi) * (R(1) + cosi));
        const R g = blpe * fc_only<PREC>(rq, R1, R2, inv_w) * R(2) * a0 * c02 * (R(1) + cosi) * (it * it);
#pragma unroll
        for (int k = 0; k < 3; ++k) dB[k] += g * (-dq[k] * rr + cosi * dl[k] * irl2);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) dB[k] = dB[k] * (-delt) * R(0.5);
      {
        R fc, dfc;
        fdfc<PREC>(rp, irp, R1, R2, inv_w, fc, dfc);
        const R dff = dfc / fc;
        const R a = -sq2s * bb * (rp - r0);
        const R ea = xexp<PREC>(a), eas = xexp<PREC>(a * is);
        const R c1 = sq2s * bb * irp, c2 = sq2os * bb * irp;
        const R pre = fc * pre_e;  // fc d / (s - 1)
        const R bavg = (Bpi + Blj) * R(0.5);
        R f[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
          f[k] = pre * ((dp[k] * dff - c1 * dp[k]) * ea - (dB[k] + bavg * (dp[k] * dff - c2 * dp[k])) * s * eas);
        acc.add(f[0], f[1], f[2]);
        if (ENERGY && j > i) e.add(fc * pre_e * (ea - bavg * s * eas));
        if (ENERGY && E.eatom) eh.add(R(0.5) * fc * pre_e * (ea - bavg * s * eas));
      }
      if (l < nj) {
        R fl, dfl;
        fdfc<PREC>(rl, irl, R1, R2, inv_w, fl, dfl);
        for (int q = 0; q < nj; ++q) {
          if (q == l) continue;
          R dq[3];
          const R r2q = T::d2(pj, T::load(A, ent(L, j, q)), B, dq);
          const R irq = xrsqrt<PREC>(r2q), rq = r2q * irq;
          if (!(rq < R2)) continue;
          const R rr = irl * irq;
          const R cosi = dot3<PREC>(dl, dq) * rr;
          const R it = R(1) / (d02 + (R(1) + cosi) * (R(1) + cosi));
          const R t1 = fl * R(2) * a0 * c02 * (R(1) + cosi) * (it * it);
          const R t2 = dfl * a0 * (R(1) + c.c02d02 - c02 * it);
          const R pre = delt * R(0.5) * (R)Bb[ex_off + (size_t)q * L.stride + j];
          const R post = fc_only<PREC>(rq, R1, R2, inv_w) * pre_e * s * xexp<PREC>(-sq2s * bb * (rq - r0) * is);
          R f[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) f[k] = pre * (t1 * (-dq[k] * rr + cosi * dl[k] * irl2) + dp[k] * t2) * post;
          acc.add(f[0], f[1], f[2]);
        }
      }
    }
    finish_force(A, E, ai, acc.get(0), acc.get(1), acc.get(2));
    erow = e.get();
    if (ENERGY && E.eatom) E.eatom[ai] = eh.get();
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

void launch_tb(bool prec, bool energy, const ListDev& L, const TBPar& P, const Atoms& A, const Box& B, double* Bb,
               Ctl* ctl, int eslot, int ekey, cudaStream_t s, int parts, const Epi& E) {
  if (L.rows == 0) {
    if (energy && (parts & 2)) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int g = nblk(L.rows, 128);
  with_bool(prec, [&](auto pr) {
    constexpr bool PR = decltype(pr)::value;
    if (parts & 1) {
      k_tb_bond<PR><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl);
      ++g_kernel_launches;
    }
    if (parts & 2) {
      if (energy)
        k_tb_force<PR, true><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl, eslot, ekey, E);
      else
        k_tb_force<PR, false><<<g, 128, 0, s>>>(L, P, A, B, Bb, ctl, eslot, ekey, E);
      ++g_kernel_launches;
    }
  });
}

}  // namespace pfmd

// Batched form: many independent replicas stepped together on one GPU.
//
// The reference runs independent systems one per MPI rank, each rank calling md()
// on one entry of a settings list (run_md_simulation_mpi.f90:68-88).  Here all the
// replicas of such a list live in one device state -- atoms concatenated replica
// by replica, each replica with its own box, cell grid and parameters -- and one
// persistent cooperative kernel advances all of them through K MD steps: kick and
// drift, cell binning and list build at the list period, the rjl density pass, the
// force pass with the second half-kick fused in, and per-replica FP64 energies at
// the energy period.  Phases are separated by a grid barrier whose spin is
// bounded (status PFMD_E_TIMEOUT when it gives up), so no launch boundary or host
// round trip falls between phases, and replicas of very different sizes share the
// GPU through one flat row space: a replica of 500 atoms and one of 20,000 atoms
// cost one warp-tile per 32/TPA rows each.
//
// Arithmetic is the precision form: fixed-point positions per replica box, FP32
// pair terms with compensated sums, FP64 positions, velocities and energies.
// Supported replicas (the systems of the batched configuration): a binary LJ gas
// (lj1g A-A, lj1g B-B, lj A-B, as LennardJones_1g.f90 / LennardJones.f90) or an
// rjl slab (RosatoGuillopeLegrand.f90), integrated with nve or with nvt under one
// Nose-Hoover chain per replica (md_integrators.f90:182-260): each half of the
// chain is a per-replica reduction of its group's kinetic energy (one warp per
// replica over its tiles' partials) and a chain update, and the scaling it
// implies rides on the next phase that touches the velocities.  The merged LJ list
// holds every partner within r_cut; same-species pairs take the lj1g terms
// (quintic switch, energy once per pair) and cross pairs the lj terms (cosine
// switch, energy on the A rows, the reference's nl(1)), so the sums equal the
// reference's three interactions.  Per-species-class counts are checked against
// each list's nmax ('error: too many neighbours', md_neighbours.f90:80).
//
// Work tiles: a warp owns 32/TPA rows of one replica; TPA (threads per row) is
// chosen per size bucket (kind x {< 2,000, < 8,000, larger} atoms) by an
// autotuner that times the persistent kernel with each candidate on a saved copy of
// the state and restores it afterwards.
#include <cuda_runtime.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pfmd.h"
#include "forces.cuh"
#include "settings.h"

namespace pfmd {
namespace batch {

static constexpr int kThreads = 256;
static constexpr int kBuckets = 6;
static constexpr int kHistCols = 5;  // energy history: 3 interaction classes, kinetic, chain
enum Kind : int { KIND_LJ = 0, KIND_RJL = 1 };

struct Rep {
  int atom0, n, kind, par;
  int cell0, nc[3];
  int tile0, ntile;
  int nmax_same, nmax_cross;  // list capacities: same-species and cross-species partners
  float rc2;                  // list radius squared (fixed-point FP32 test)
  float qs[3];
  double L[3], Ltol[3], qinv[3];
  double ts1, ts2;  // dt, dt/2
  double ts3, ts4;  // dt/4, dt/8 (the chain's substeps)
  int nvt;          // 1: the replica integrates nvt with one Nose-Hoover chain
};
struct LJSet {
  LJc<float> aa, bb, ab;
};
struct Tile {
  int row0, nrows, rep, tpa;
};

struct Dev {
  int N, R, T, ncell, nslot, stride;
  int rebuild_period, energy_period, hist_cap, zero_momentum_period;
  double* vcm;  // per replica centre-of-mass velocity (zero_momentum)
  double4_32a *pos, *vel, *frc;
  int4* posq;
  double *mass, *kc;
  unsigned char *species, *moving;
  int* rep_of;
  int *nnum, *nlist;
  float2* pair;
  int *ccount, *cstart, *ccursor, *cell_of, *catom;
  int4* cposq;
  int* scan_part;
  const Rep* rep;
  const LJSet* lj;
  const RJLc<float>* rjl;
  const Tile* tile;
  double *tile_e, *tile_k, *e_pot, *e_kin, *hist;  // tile_e, e_pot: 3 interaction classes each
  double* tile_kc;  // per tile: kinetic energy of the chain group's atoms (nvt replicas)
  NHCDev* nhc;      // per replica: its chain (nvt replicas)
  double* e_nhc;    // per replica: the chain's energy at the last energy step
  int any_nvt;      // some replica integrates nvt
  unsigned int *bar_count, *bar_gen, *bar_flag;  // bar_flag: status when the last block arrived
  unsigned int spin_limit;                        // polls before a barrier gives up
  unsigned int bar_extra;                         // arrivals expected beyond the grid (0; 1 stalls)
  int* status;  // [0] code, [1] replica, [2] row, [3] info
  long long* step;
};

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fail(const Dev& D, int code, int rep, int row, int info) {
  if (atomicCAS(&D.status[0], 0, code) == 0) {
    D.status[1] = rep;
    D.status[2] = row;
    D.status[3] = info;
  }
}

// Grid barrier for a cooperative launch (all blocks co-resident).  The block
// that arrives last copies the status word into bar_flag before it releases the
// others, and every block returns that copy, so all blocks leave or pass the
// same barrier together: an error raised after the release by a fast block is
// seen by everyone at the next barrier.  The spin is bounded: after
// D.spin_limit polls a block records PFMD_E_TIMEOUT and returns false.
__device__ __forceinline__ bool barrier(const Dev& D) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = D.bar_gen;
    const unsigned int g = *gen;
    __threadfence();
    int ok;
    if (atomicAdd(D.bar_count, 1u) == gridDim.x - 1 + D.bar_extra) {
      const int st = *(volatile int*)D.status;
      *(volatile unsigned int*)D.bar_flag = static_cast<unsigned int>(st);
      *D.bar_count = 0u;
      __threadfence();
      atomicAdd(D.bar_gen, 1u);
      ok = st == 0;
    } else {
      unsigned int spins = 0;
      bool released = true;
      while (*gen == g) {
        if (++spins > D.spin_limit) {
          fail(D, PFMD_E_TIMEOUT, -1, -1, 0);
          released = false;
          break;
        }
        __nanosleep(64);
      }
      __threadfence();
      ok = released && *(volatile unsigned int*)D.bar_flag == 0u;
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool oob(double x, double Ltol) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b >= __double_as_longlong(Ltol)
                : (unsigned long long)b >= (unsigned long long)__double_as_longlong(-0.0000001);
}
__device__ __forceinline__ double wrap(double x, double L) {
  const long long b = __double_as_longlong(x);
  if (b > __double_as_longlong(L))
    x = x - L;
  else if (b < 0 && b != (long long)0x8000000000000000ULL)
    x = x + L;
  return x;
}

// Half-kick of the velocity (kt = kc*dt/2) and drift with the single-shift wrap
// (md_integrators.f90:7-97), FMA form; the fixed-point position follows.
__device__ void phase_kick_drift(const Dev& D) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < D.N; a += gridDim.x * blockDim.x) {
    const unsigned char mv = D.moving[a];
    if (mv & 4) {  // the chain's first-half scaling (scale_velocities, md_general.f90:97-112)
      const double sc = D.nhc[D.rep_of[a]].s;
      double4_32a u = D.vel[a];
      u.x *= sc;
      u.y *= sc;
      u.z *= sc;
      D.vel[a] = u;
    }
    if (!(mv & 1)) continue;
    const Rep& R = D.rep[D.rep_of[a]];
    const double kt = D.kc[a] * R.ts2;
    const double4_32a f = D.frc[a];
    double4_32a v = D.vel[a], p = D.pos[a];
    v.x = fma(f.x, kt, v.x);
    v.y = fma(f.y, kt, v.y);
    v.z = fma(f.z, kt, v.z);
    p.x = wrap(fma(v.x, R.ts1, p.x), R.L[0]);
    p.y = wrap(fma(v.y, R.ts1, p.y), R.L[1]);
    p.z = wrap(fma(v.z, R.ts1, p.z), R.L[2]);
    D.vel[a] = v;
    D.pos[a] = p;
    const int w = D.posq[a].w;
    D.posq[a] = make_int4(quantize(p.x, R.qinv[0]), quantize(p.y, R.qinv[1]), quantize(p.z, R.qinv[2]), w);
    if (oob(p.x, R.Ltol[0]) || oob(p.y, R.Ltol[1]) || oob(p.z, R.Ltol[2]))
      fail(D, PFMD_E_OUT_OF_CELL, D.rep_of[a], a - R.atom0, 0);
  }
}

// Exclusive scan of the cell counts over all replicas' cells: block b scans its
// contiguous chunk, then adds the totals of the chunks before it.
__device__ bool phase_scan(const Dev& D) {
  __shared__ int sh[kThreads];
  const int chunk = (D.ncell + gridDim.x - 1) / gridDim.x;
  const int c0 = blockIdx.x * chunk, c1 = min(D.ncell, c0 + chunk);
  int run = 0;
  for (int base = c0; base < c1; base += blockDim.x) {
    const int c = base + threadIdx.x;
    const int v = c < c1 ? D.ccount[c] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < blockDim.x; o <<= 1) {
      const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (c < c1) D.cstart[c] = run + sh[threadIdx.x] - v;
    run += sh[blockDim.x - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) D.scan_part[blockIdx.x] = run;
  if (!barrier(D)) return false;
  int off = 0;
  for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) off += D.scan_part[b];
  sh[threadIdx.x] = off;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  off = sh[0];
  for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
    D.cstart[c] += off;
    D.ccursor[c] = D.cstart[c];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) D.cstart[D.ncell] = off + run;
  return true;
}

// Ascending atom order inside every cell (the scatter order comes from atomics).
__device__ void phase_cell_sort(const Dev& D) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < D.ncell; c += nw) {
    const int s = D.cstart[c], e = D.cstart[c + 1], len = e - s;
    if (len <= 1) continue;
    if (len <= 32) {
      int key = lane < len ? D.catom[s + lane] : INT_MAX;
      const int4 q0 = lane < len ? D.cposq[s + lane] : make_int4(0, 0, 0, 0);
      int src = lane;
      for (int k = 2; k <= 32; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
          const int ok = __shfl_xor_sync(0xffffffffu, key, j);
          const int os = __shfl_xor_sync(0xffffffffu, src, j);
          const bool lower = (lane & j) == 0, up = (lane & k) == 0;
          if (lower ? ((key > ok) == up) : ((key < ok) == up)) {
            key = ok;
            src = os;
          }
        }
      int4 q;
      q.x = __shfl_sync(0xffffffffu, q0.x, src);
      q.y = __shfl_sync(0xffffffffu, q0.y, src);
      q.z = __shfl_sync(0xffffffffu, q0.z, src);
      q.w = 0;
      if (lane < len) {
        D.catom[s + lane] = key;
        D.cposq[s + lane] = q;
      }
    } else if (lane == 0) {
      for (int i = s + 1; i < e; ++i) {
        const int k = D.catom[i];
        const int4 q = D.cposq[i];
        int j = i - 1;
        while (j >= s && D.catom[j] > k) {
          D.catom[j + 1] = D.catom[j];
          D.cposq[j + 1] = D.cposq[j];
          --j;
        }
        D.catom[j + 1] = k;
        D.cposq[j + 1] = q;
      }
    }
    __syncwarp();
  }
}

// One warp per row: the x-runs of the 27 surrounding cells of the row's replica,
// partners within r_cut (fixed-point separation, FP32) appended in cell order.
__device__ void phase_build(const Dev& D) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < D.N; a += nw) {
    const int r = D.rep_of[a];
    const Rep& R = D.rep[r];
    Box B;
    B.qs[0] = R.qs[0];
    B.qs[1] = R.qs[1];
    B.qs[2] = R.qs[2];
    const int4 piq = D.posq[a];
    const int sa = D.species[a];
    const int nx = R.nc[0], ny = R.nc[1], nz = R.nc[2];
    const int cx = cell_q(piq.x, nx), cy = cell_q(piq.y, ny), cz = cell_q(piq.z, nz);
    const int my = ny < 3 ? ny : 3, mz = nz < 3 ? nz : 3;
    int cnt = 0, same = 0;
    for (int iz = 0; iz < mz; ++iz) {
      const int z = nz < 3 ? iz : (cz - 1 + iz + nz) % nz;
      for (int iy = 0; iy < my; ++iy) {
        const int y = ny < 3 ? iy : (cy - 1 + iy + ny) % ny;
        const int base = R.cell0 + (z * ny + y) * nx;
        int r0s, r0e, r1s = 0, r1e = 0;
        if (nx < 3) {
          r0s = D.cstart[base];
          r0e = D.cstart[base + nx];
        } else if (cx >= 1 && cx + 1 < nx) {
          r0s = D.cstart[base + cx - 1];
          r0e = D.cstart[base + cx + 2];
        } else if (cx == 0) {
          r0s = D.cstart[base];
          r0e = D.cstart[base + 2];
          r1s = D.cstart[base + nx - 1];
          r1e = D.cstart[base + nx];
        } else {
          r0s = D.cstart[base + nx - 2];
          r0e = D.cstart[base + nx];
          r1s = D.cstart[base];
          r1e = D.cstart[base + 1];
        }
        for (int run = 0; run < 2; ++run) {
          const int s0 = run ? r1s : r0s, e0 = run ? r1e : r0e;
          for (int k0 = s0; k0 < e0; k0 += 32) {
            const int k = k0 + lane;
            bool hit = false;
            int aj = 0;
            if (k < e0) {
              aj = D.catom[k];
              if (aj != a) {
                float d[3];
                hit = mi_q(piq, D.cposq[k], B, d) < R.rc2;
              }
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (hit) {
              const int p = cnt + __popc(m & ((1u << lane) - 1u));
              if (p < D.nslot) D.nlist[(size_t)p * D.stride + a] = aj;
            }
            same += __popc(__ballot_sync(0xffffffffu, hit && D.species[aj] == sa));
            cnt += __popc(m);
          }
        }
      }
    }
    if (lane == 0) {
      const int cross = cnt - same;
      if (same > R.nmax_same || cross > R.nmax_cross || cnt > D.nslot)
        fail(D, PFMD_E_NLIST_OVERFLOW, r, a - R.atom0, max(same, cross));
      D.nnum[a] = min(cnt, D.nslot);
    }
  }
}

template <int TPA>
__device__ __forceinline__ float tile_merge(float& s, float& c) {
  gmerge<TPA>(s, c);
  return s;
}

// rjl density of one tile (RosatoGuillopeLegrand.f90:23-94): 1/Eb into posq.w and
// the slot's pair terms (a, b).
template <int TPA>
__device__ void tile_density(const Dev& D, const Tile& t, bool energy, float& erow_sum_s, float& erow_sum_c) {
  constexpr int RPW = 32 / TPA;
  const int lane = threadIdx.x & 31;
  const int row = lane % RPW, sub = lane / RPW;
  const Rep& R = D.rep[t.rep];
  const RJLc<float> c = D.rjl[R.par];
  Box B;
  B.qs[0] = R.qs[0];
  B.qs[1] = R.qs[1];
  B.qs[2] = R.qs[2];
  const int a = t.row0 + row;
  const bool valid = row < t.nrows;
  const int n = valid ? D.nnum[a] : 0;
  Acc1<true> eb2, er;
  if (n > 0) {
    const int4 pi = D.posq[a];
    // the next slot's partner index is loaded one iteration ahead, as in the
    // single-system passes; with the same in the LJ loop below, 1.01e9 -> 1.15e9
    // atom-steps/s on the 512-replica batch
    int aj = sub < n ? D.nlist[(size_t)sub * D.stride + a] : a;
#pragma unroll 4
    for (int p = sub; p < n; p += TPA) {
      float dr[3];
      const int pn = p + TPA;
      const int ajn = pn < n ? D.nlist[(size_t)pn * D.stride + a] : a;
      const float r2 = mi_q(pi, D.posq[aj], B, dr);
      aj = ajn;
      const float ir = rsqrtf(r2), r = r2 * ir;
      float2 ab = make_float2(0.f, 0.f);
      if (r <= c.R2) {
        float fc, rdfc;
        fdfrcut_cos_f(r, c.R1, c.R2, c.inv_w, fc, rdfc);
        // (the folded ex2 form of the single-system density pass takes this
        // kernel from 64 to 80 registers and fewer resident blocks: 5.1 -> 5.9 ms
        // per step on the 512-replica batch)
        const float x = r * c.inv_r0 - 1.f;
        const float eq = __expf(c.m2q * x), ep = __expf(c.mp * x);
        eb2.add(eq * fc);
        er.add(ep * fc);
        ab.x = c.a2 * (c.pr0 * fc - rdfc) * ep * ir;
        ab.y = c.xi * (c.qr0 * fc - 0.5f * rdfc) * eq * ir;
      }
      D.pair[(size_t)p * D.stride + a] = ab;
    }
  }
  eb2.template reduce<TPA>();
  er.template reduce<TPA>();
  erow_sum_s = 0.f;
  erow_sum_c = 0.f;
  if (valid && sub == 0) {
    const float e2 = eb2.s - eb2.c, ie = rsqrtf(e2);
    reinterpret_cast<int*>(D.posq + a)[3] = __float_as_int(ie);
    if (energy) erow_sum_s = c.A0 * (er.s - er.c) - c.xi * (e2 > 0.f ? e2 * ie : 0.f);
  }
}

// Forces of one tile, the fused second half-kick, and (energy steps) the tile's
// potential and kinetic energy.
// Energy classes: LJ replicas 0 = lj1g A-A, 1 = lj1g B-B, 2 = lj A-B; rjl replicas 0.
template <int TPA>
__device__ void tile_force(const Dev& D, const Tile& t, bool kick, bool energy, float (&es)[3], float (&ec)[3],
                           double& ke, double& kc) {
  constexpr int RPW = 32 / TPA;
  const int lane = threadIdx.x & 31;
  const int row = lane % RPW, sub = lane / RPW;
  const Rep& R = D.rep[t.rep];
  Box B;
  B.qs[0] = R.qs[0];
  B.qs[1] = R.qs[1];
  B.qs[2] = R.qs[2];
  const int a = t.row0 + row;
  const bool valid = row < t.nrows;
  const int n = valid ? D.nnum[a] : 0;
  Acc3<true> acc;
  Acc1<true> e[3];
  if (n > 0) {
    const int4 pi = D.posq[a];
    if (R.kind == KIND_RJL) {
      const float ieb_i = __int_as_float(pi.w);
      int aj = sub < n ? D.nlist[(size_t)sub * D.stride + a] : a;
#pragma unroll 4
      for (int p = sub; p < n; p += TPA) {
        const int pn = p + TPA;
        const int ajn = pn < n ? D.nlist[(size_t)pn * D.stride + a] : a;
        const int4 pj = D.posq[aj];
        aj = ajn;
        float dr[3];
        mi_q(pi, pj, B, dr);
        const float2 ab = D.pair[(size_t)p * D.stride + a];
        const float k = ab.x - ab.y * (ieb_i + __int_as_float(pj.w));
        acc.add(-k * dr[0], -k * dr[1], -k * dr[2]);
      }
    } else {
      const LJSet& P = D.lj[R.par];
      const int si = D.species[a];
      int ajn = sub < n ? D.nlist[(size_t)sub * D.stride + a] : a;
#pragma unroll 2
      for (int p = sub; p < n; p += TPA) {
        const int aj = ajn;
        const int pn = p + TPA;
        ajn = pn < n ? D.nlist[(size_t)pn * D.stride + a] : a;
        float dr[3];
        const float r2 = mi_q(pi, D.posq[aj], B, dr);
        const int sj = D.species[aj];
        const float ir = rsqrtf(r2), r = r2 * ir;
        if (si == sj) {  // lj1g (LennardJones_1g.f90:28-117), quintic switch
          const LJc<float>& c = si == 0 ? P.aa : P.bb;
          if (r < c.R2) {
            const float invr2 = ir * ir, U = invr2 * invr2 * invr2;
            float fcut, dfr;
            f_dfr_cut<float>(r, c.R1, c.R2, c.inv_w, fcut, dfr);
            const float F = U * invr2 * ((c.c12t12 * U - c.c6t6) * fcut - (c.c12 * U - c.c6) * dfr);
            acc.add(-F * dr[0], -F * dr[1], -F * dr[2]);
            if (energy && aj < a) e[si].add(U * (c.c12 * U - c.c6) * fcut);
          }
        } else {  // lj (LennardJones.f90:23-69), cosine switch
          const LJc<float>& c = P.ab;
          if (r < c.R2) {
            const float x = c.sig * ir, x2 = x * x, V = x2 * x2 * x2;
            float fc, dfc;
            fdfcut_cos_f(r, c.R1, c.R2, c.inv_w, fc, dfc);
            const float k = c.eps4 * (V * (12.f * V - 6.f) * (ir * ir) * fc - V * (V - 1.f) * dfc);
            acc.add(-k * dr[0], -k * dr[1], -k * dr[2]);
            if (energy && si == 0) e[2].add(c.eps4 * V * (V - 1.f) * fc);
          }
        }
      }
    }
  }
  acc.template reduce<TPA>();
  if (energy)
#pragma unroll
    for (int k = 0; k < 3; ++k) e[k].template reduce<TPA>();
#pragma unroll
  for (int k = 0; k < 3; ++k) es[k] = ec[k] = 0.f;
  ke = 0.0;
  kc = 0.0;
  if (valid && sub == 0) {
    const double4_32a f = make_double4_32a(acc.get(0), acc.get(1), acc.get(2), 0.0);
    D.frc[a] = f;
    const unsigned char mv = D.moving[a];
    if (mv) {
      double4_32a v = D.vel[a];
      if (kick && (mv & 1)) {
        const double kt = D.kc[a] * R.ts2;
        v.x = fma(f.x, kt, v.x);
        v.y = fma(f.y, kt, v.y);
        v.z = fma(f.z, kt, v.z);
        D.vel[a] = v;
      }
      const double k2 = D.mass[a] * (v.x * v.x + v.y * v.y + v.z * v.z) / 2 * kMassCoef;
      if (energy && (mv & 2)) ke = k2;
      if (kick && (mv & 4)) kc = k2;  // the chain's second half needs it (nvt replicas)
    }
    if (energy && R.kind == KIND_LJ)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        es[k] = e[k].s;
        ec[k] = e[k].c;
      }
  }
}

template <int TPA>
__device__ void run_tile(const Dev& D, int ti, int phase, bool kick, bool energy) {
  const Tile& t = D.tile[ti];
  float s[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
  double ke = 0.0, kc = 0.0;
  if (phase == 0) {
    tile_density<TPA>(D, t, energy, s[0], c[0]);
  } else {
    tile_force<TPA>(D, t, kick, energy, s, c, ke, kc);
    if (kick && D.rep[t.rep].nvt) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) kc += __shfl_xor_sync(0xffffffffu, kc, o);
      if ((threadIdx.x & 31) == 0) D.tile_kc[ti] = kc;
    }
  }
  if (!energy) return;
  // the tile's rows sit in one warp: compensated FP32 merges of the row energies,
  // an FP64 sum of the kinetic energies
#pragma unroll
  for (int k = 0; k < 3; ++k) gmerge<32>(s[k], c[k]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ke += __shfl_xor_sync(0xffffffffu, ke, o);
  if ((threadIdx.x & 31) == 0) {
    double* te = D.tile_e + 3 * (size_t)ti;
    if (phase == 0) {  // rjl: the density pass holds the energy
      te[0] = (double)s[0] - (double)c[0];
      te[1] = te[2] = 0.0;
    } else {
      if (D.rep[t.rep].kind == KIND_LJ)
        for (int k = 0; k < 3; ++k) te[k] = (double)s[k] - (double)c[k];
      D.tile_k[ti] = ke;
    }
  }
}

__device__ void phase_tiles(const Dev& D, int phase, bool kick, bool energy) {
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ti < D.T; ti += nw) {
    const int kind = D.rep[D.tile[ti].rep].kind;
    if (phase == 0 && kind != KIND_RJL) continue;
    switch (D.tile[ti].tpa) {
      case 1: run_tile<1>(D, ti, phase, kick, energy); break;
      case 2: run_tile<2>(D, ti, phase, kick, energy); break;
      case 4: run_tile<4>(D, ti, phase, kick, energy); break;
      default: run_tile<8>(D, ti, phase, kick, energy); break;
    }
  }
}

// zero_momentum (md_general.f90:236-252) of every replica's all-atoms group: one
// warp per replica sums m*v and m in a fixed order, then every atom loses the
// centre-of-mass velocity.
__device__ bool phase_zero_momentum(const Dev& D) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < D.R; r += nw) {
    const Rep& R = D.rep[r];
    double px = 0.0, py = 0.0, pz = 0.0, m = 0.0;
    for (int i = lane; i < R.n; i += 32) {
      const double mi = D.mass[R.atom0 + i];
      const double4_32a u = D.vel[R.atom0 + i];
      px += mi * u.x;
      py += mi * u.y;
      pz += mi * u.z;
      m += mi;
    }
    px = warp_sum(px);
    py = warp_sum(py);
    pz = warp_sum(pz);
    m = warp_sum(m);
    if (lane == 0) {
      D.vcm[3 * r] = px / m;
      D.vcm[3 * r + 1] = py / m;
      D.vcm[3 * r + 2] = pz / m;
    }
  }
  if (!barrier(D)) return false;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < D.N; a += gridDim.x * blockDim.x) {
    const int r = D.rep_of[a];
    double4_32a v = D.vel[a];
    v.x = v.x - D.vcm[3 * r];
    v.y = v.y - D.vcm[3 * r + 1];
    v.z = v.z - D.vcm[3 * r + 2];
    D.vel[a] = v;
  }
  return true;
}

// One warp per nvt replica: the chain's kinetic energy from its tiles' partials
// (a fixed order) and integrate_nose_hoover_chain's chain update
// (md_integrators.f90:200-245); the scaling it implies is applied by the next
// phase that touches the velocities.
__device__ void phase_chain(const Dev& D) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < D.R; r += nw) {
    const Rep& R = D.rep[r];
    if (!R.nvt) continue;
    double k = 0.0;
    for (int t = lane; t < R.ntile; t += 32) k += D.tile_kc[R.tile0 + t];
    k = warp_sum(k);
    if (lane == 0) nhc_chain_update(D.nhc[r], k, R.ts2, R.ts3, R.ts4);
  }
}

// The chain's second-half scaling of the nvt replicas' chain-group atoms, then
// per tile the kinetic energy of the chain group (for the next step's first
// half) and, at energy steps, of the temperature group -- both of the scaled
// velocities.  scale = false at step 0, which only forms the partials.
__device__ void phase_scale(const Dev& D, bool scale, bool energy) {
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  for (int ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ti < D.T; ti += nw) {
    const Tile& t = D.tile[ti];
    if (!D.rep[t.rep].nvt) continue;
    const double sc = D.nhc[t.rep].s;
    double kc = 0.0, ke = 0.0;
    if (lane < t.nrows) {
      const int a = t.row0 + lane;
      const unsigned char mv = D.moving[a];
      double4_32a v = D.vel[a];
      if (scale && (mv & 4)) {
        v.x *= sc;
        v.y *= sc;
        v.z *= sc;
        D.vel[a] = v;
      }
      const double k2 = D.mass[a] * (v.x * v.x + v.y * v.y + v.z * v.z) / 2 * kMassCoef;
      if (mv & 4) kc = k2;
      if (mv & 2) ke = k2;
    }
    kc = warp_sum(kc);
    ke = warp_sum(ke);
    if (lane == 0) {
      D.tile_kc[ti] = kc;
      if (energy) D.tile_k[ti] = ke;
    }
  }
}

// Per-replica totals in a fixed order: one warp per replica, lane-strided over its
// tiles, then the warp tree.
__device__ void phase_energy(const Dev& D, long long s) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < D.R; r += nw) {
    const Rep& R = D.rep[r];
    double ep[3] = {0.0, 0.0, 0.0}, ek = 0.0;
    for (int t = lane; t < R.ntile; t += 32) {
      for (int k = 0; k < 3; ++k) ep[k] += D.tile_e[3 * (size_t)(R.tile0 + t) + k];
      ek += D.tile_k[R.tile0 + t];
    }
    for (int k = 0; k < 3; ++k) ep[k] = warp_sum(ep[k]);
    ek = warp_sum(ek);
    if (lane == 0) {
      for (int k = 0; k < 3; ++k) D.e_pot[3 * r + k] = ep[k];
      D.e_kin[r] = ek;
      // calculate_nose_hoover_chain_energy (md_integrators.f90:247-260)
      double en = 0.0;
      if (R.nvt) {
        const NHCDev& h = D.nhc[r];
        const double kt = kKtPerKelvin * h.T;
        en = h.q[0] / 2 * (h.v[0] * h.v[0]) + 3.0 * h.L * kt * h.x[0];
        for (int i = 1; i < h.M; ++i) en = en + h.q[i] / 2 * (h.v[i] * h.v[i]) + kt * h.x[i];
      }
      D.e_nhc[r] = en;
      const long long h = s / D.energy_period;
      if (s % D.energy_period == 0 && h < D.hist_cap) {
        double* o = D.hist + (h * D.R + r) * kHistCols;
        o[0] = ep[0];
        o[1] = ep[1];
        o[2] = ep[2];
        o[3] = ek;
        o[4] = en;
      }
    }
  }
}

// K MD steps of every replica.  Step s: (s > 0) first half-kick and drift; list
// rebuild when s % period == 0; rjl density; forces and (s > 0) the second
// half-kick; energies when s % energy_period == 0 (history rows) and at the
// launch's last step (e_pot / e_kin only).
// Four blocks per SM: the register cap this implies (64) holds the kernel
// without spills, where the compiler's own choice (80 registers, 140 bytes of
// spills, three blocks per SM) ran the 512-replica batch at 5.3-5.5 ms per MD
// step against 4.4-4.5.
__global__ void __launch_bounds__(kThreads, 4) k_batch(Dev D, int nsteps) {
  const long long s0 = *D.step;
  for (int it = 0; it < nsteps; ++it) {
    const long long s = s0 + it;
    if (s > 0) {
      if (D.any_nvt) {  // the chain's first half (its scaling rides on the kick-drift)
        phase_chain(D);
        if (!barrier(D)) return;
      }
      phase_kick_drift(D);
      if (!barrier(D)) return;
    }
    if (s % D.rebuild_period == 0) {
      for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < D.ncell; c += gridDim.x * blockDim.x) D.ccount[c] = 0;
      if (!barrier(D)) return;
      for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < D.N; a += gridDim.x * blockDim.x) {
        const Rep& R = D.rep[D.rep_of[a]];
        const int4 q = D.posq[a];
        const int c = R.cell0 + (cell_q(q.z, R.nc[2]) * R.nc[1] + cell_q(q.y, R.nc[1])) * R.nc[0] +
                      cell_q(q.x, R.nc[0]);
        D.cell_of[a] = c;
        atomicAdd(&D.ccount[c], 1);
      }
      if (!barrier(D)) return;
      if (!phase_scan(D)) return;
      if (!barrier(D)) return;
      for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < D.N; a += gridDim.x * blockDim.x) {
        const int slot = atomicAdd(&D.ccursor[D.cell_of[a]], 1);
        D.catom[slot] = a;
        D.cposq[slot] = D.posq[a];
      }
      if (!barrier(D)) return;
      phase_cell_sort(D);
      if (!barrier(D)) return;
      phase_build(D);
      if (!barrier(D)) return;
    }
    if (s % D.zero_momentum_period == 0) {
      if (!phase_zero_momentum(D)) return;
      if (!barrier(D)) return;
    }
    const bool energy = s % D.energy_period == 0 || it == nsteps - 1;
    phase_tiles(D, 0, false, energy);
    if (!barrier(D)) return;
    phase_tiles(D, 1, s > 0, energy);
    if (!barrier(D)) return;
    if (D.any_nvt) {  // the chain's second half, then its scaling
      if (s > 0) {
        phase_chain(D);
        if (!barrier(D)) return;
      }
      phase_scale(D, s > 0, energy);
      if (!barrier(D)) return;
    }
    if (energy) phase_energy(D, s);
  }
  if (!barrier(D)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) *D.step = s0 + nsteps;
}

// The chain group's kinetic energy per tile of the nvt replicas from the current
// velocities (the partials the next step's first chain half reads), after the
// tiles changed.
__global__ void k_tile_kc(Dev D) {
  phase_scale(D, false, false);
}

__global__ void k_pack(Dev D) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= D.N) return;
  const Rep& R = D.rep[D.rep_of[a]];
  const double4_32a p = D.pos[a];
  D.posq[a] = make_int4(quantize(p.x, R.qinv[0]), quantize(p.y, R.qinv[1]), quantize(p.z, R.qinv[2]), 0);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
#define BCK(x)                                                                                   \
  do {                                                                                           \
    cudaError_t e_ = (x);                                                                        \
    if (e_ != cudaSuccess)                                                                       \
      throw ::pfmd::batch::Error(PFMD_E_CUDA, std::string(#x ": ") + cudaGetErrorString(e_));     \
  } while (0)

template <class T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  void alloc(size_t k) {
    n = std::max<size_t>(k, 1);
    BCK(cudaMalloc(&p, n * sizeof(T)));
  }
  void up(const std::vector<T>& v, cudaStream_t s) {
    BCK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  ~Buf() {
    if (p) cudaFree(p);
  }
};

struct HostRep {
  std::string settings, prefix;
  int kind = KIND_LJ, atom0 = 0, n = 0, nmove = 0;
  double L[3] = {0, 0, 0}, dt = 0.0;
  double rc = 0.0;
  long long period = 1, log_period = 1, steps = 0, zmp = 1;
  int nmax_same = 0, nmax_cross = 0;
  LJPar aa{}, bb{}, ab{};
  RJLPar rjl{};
  // what a settings-list run writes (md_simulation.f90:204-241, 262-300)
  std::string integ_name, log_file, xyz_file;
  long long snap_period = 1, traj_period = 1;
  int traj_group = 0, n_ke = 0, n_nhc = 0;
  // nvt: the one Nose-Hoover chain (md_integrators.f90:165-198): length, target
  // temperature, q1 and the atoms of its group
  bool nvt = false;
  int nhc_M = 0, nhc_L = 0;
  double nhc_T = 0.0, nhc_q1 = 0.0;
  std::vector<int> all_idx, traj_idx;  // group members in the reference's order (type, then atom)
  std::vector<int> inter_class;        // energy class of each interaction, settings order
  std::vector<std::string> types;
};

static int bucket_of(const HostRep& r) {
  const int cls = r.n < 2000 ? 0 : (r.n < 8000 ? 1 : 2);
  return r.kind * 3 + cls;
}

static LJPar lj_from(const std::vector<double>& p) {
  LJPar P{};
  P.eps = p[0];
  P.sig = p[1];
  P.R1 = p[2];
  P.R2 = p[3];
  const double s6 = p[1] * p[1] * p[1] * p[1] * p[1] * p[1], s12 = s6 * s6;
  P.c6 = 4.0 * p[0] * s6;
  P.c12 = 4.0 * p[0] * s12;
  P.c6t6 = 6.0 * P.c6;
  P.c12t12 = 12.0 * P.c12;
  derive(P);
  return P;
}

static bool in_group(const pfmd_io::Settings& S, int g, const std::string& type) {
  if (g < 1 || g > static_cast<int>(S.group_types.size())) return false;
  for (const auto& t : S.group_types[static_cast<size_t>(g - 1)])
    if (t == type) return true;
  return false;
}

struct Batch {
  std::vector<HostRep> reps;
  int N = 0, nslot = 0, stride = 0, ncell = 0, grid = 0;
  int tpa[kBuckets] = {2, 2, 2, 2, 2, 2};
  long long md_step = 0, hist_cap = 0;
  int rebuild_period = 10, energy_period = 10;
  long long zero_momentum_period = 1;
  int out_period = 1;
  cudaStream_t st = nullptr;
  std::string err;
  std::vector<double> mass_h;
  std::vector<int> rep_of_h;
  Buf<double4_32a> pos, vel, frc;
  Buf<int4> posq, cposq;
  Buf<double> mass, kc, tile_e, tile_k, tile_kc, e_pot, e_kin, e_nhc, hist, vcm;
  Buf<NHCDev> nhc;
  bool any_nvt = false;
  Buf<unsigned char> species, moving;
  Buf<int> rep_of, nnum, nlist, ccount, cstart, ccursor, cell_of, catom, scan_part, status;
  Buf<float2> pair;
  Buf<Rep> rep;
  Buf<LJSet> lj;
  Buf<RJLc<float>> rjl;
  Buf<Tile> tile;
  Buf<unsigned int> bar;
  Buf<long long> step;
  std::vector<Rep> rep_h;
  int ntile = 0;

  ~Batch() {
    clear_graphs();
    if (st) cudaStreamDestroy(st);
  }

  // The launches of a run of n steps in chunks, captured once as a CUDA graph and
  // replayed: the kernel reads its step counter from device memory, so a replay
  // continues where the last one stopped.  A change of tiles drops the graphs.
  std::map<std::pair<long long, int>, cudaGraphExec_t> graphs;
  bool graphs_ok = true;  // false if the driver cannot capture the cooperative launch
  void clear_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }

  void load(const std::string& input_path, const std::string& list_file) {
    fortio::ListReader lst;
    if (!lst.open(input_path + list_file)) throw Error(PFMD_E_IO, "cannot open " + input_path + list_file);
    const long long nset = fortio::to_int(lst.read_items(1)[0].s);
    if (nset < 1) throw Error(PFMD_E_PARAM, "batch: empty settings list");
    for (long long k = 0; k < nset; ++k) {
      auto it = lst.read_items(2);
      HostRep r;
      r.settings = fortio::trim(fortio::to_char(it[0].s, 128));
      r.prefix = fortio::trim(fortio::to_char(it[1].s, 128));
      reps.push_back(r);
    }
  }

  // One replica's settings into host arrays; the supported systems are described
  // at the top of this file.
  void add(HostRep& r, const pfmd_io::Settings& S, std::vector<double>& pos_h, std::vector<double>& vel_h,
           std::vector<unsigned char>& sp_h, std::vector<unsigned char>& mv_h) {
    const auto& X = S.xyz;
    r.n = X.N;
    for (int k = 0; k < 3; ++k) r.L[k] = X.box[k];
    // the integrators that run (md_simulation.f90:121-136 skips those of length 0)
    std::vector<const pfmd_io::IntegratorSpec*> runs;
    for (const auto& is : S.integrators)
      if (is.l > 0) runs.push_back(&is);
    const std::string stage = runs.size() == 1 ? fortio::trim(runs[0]->name) : "";
    if (stage != "nve" && stage != "nvt")
      throw Error(PFMD_E_PARAM, r.settings + ": the batched form integrates one nve or nvt stage only");
    r.nvt = stage == "nvt";
    if (r.nvt) {
      if (S.nhc.size() != 1)
        throw Error(PFMD_E_PARAM, r.settings + ": an nvt replica of the batched form has one Nose-Hoover chain");
      const auto& h = S.nhc[0];
      r.nhc_M = h.M;
      r.nhc_T = h.temperature;
      r.nhc_q1 = h.q1;
      if (h.M < 1 || h.M > PFMD_MAX_CHAIN)
        throw Error(PFMD_E_PARAM, r.settings + ": chain length out of range");
    }
    if (S.new_velocities) throw Error(PFMD_E_PARAM, r.settings + ": the batched form takes velocities from the .xyz");
    if (!S.changes.empty() || S.invert_z_vel)
      throw Error(PFMD_E_PARAM, r.settings + ": the batched form has no group changes or z-velocity inversion");
    const auto& I = *runs[0];
    r.dt = I.dt;
    r.log_period = std::max<long long>(1, I.period_log);
    // steps 0..steps run (md_simulation.f90:113-134: the stage ends after l steps or at md_step_limit)
    r.steps = std::min<long long>(I.l, S.md_step_limit);
    r.integ_name = I.name;
    r.snap_period = std::max<long long>(1, I.period_snapshot);
    r.traj_period = std::max<long long>(1, S.period_traj);
    r.traj_group = S.traj_group;
    r.n_nhc = static_cast<int>(S.nhc.size());
    r.log_file = S.logfilename;
    r.xyz_file = S.init_xyz_filename;
    r.types = X.types;
    auto members = [&](int g) {
      std::vector<int> idx;
      if (g < 1 || g > static_cast<int>(S.group_types.size())) return idx;
      for (const auto& nm : S.group_types[static_cast<size_t>(g - 1)])
        for (int i = 0; i < X.N; ++i)
          if (X.types[static_cast<size_t>(i)] == nm) idx.push_back(i);
      return idx;
    };
    r.all_idx = members(S.all_atoms);
    r.traj_idx = members(S.traj_group);
    std::vector<const pfmd_io::InteractionSpec*> lj1g, lj, rjl;
    for (const auto& in : S.interactions) {
      if (in.kind == pfmd_io::K_LJ1G) lj1g.push_back(&in);
      else if (in.kind == pfmd_io::K_LJ) lj.push_back(&in);
      else if (in.kind == pfmd_io::K_RJL) rjl.push_back(&in);
      else throw Error(PFMD_E_PARAM, r.settings + ": interaction " + in.name + " is not in the batched form");
    }
    std::vector<unsigned char> sp(static_cast<size_t>(X.N), 255);
    if (rjl.size() == 1 && lj1g.empty() && lj.empty()) {
      r.kind = KIND_RJL;
      const auto& in = *rjl[0];
      r.rjl = RJLPar{in.p[0], in.p[1], in.p[2], in.p[3], in.p[4], in.p[5], in.p[6], {}, {}};
      derive(r.rjl);
      r.rc = in.nl[0].r_cut;
      r.period = in.nl[0].period;
      r.nmax_same = in.nl[0].nmax;
      r.nmax_cross = 0;
      for (int i = 0; i < X.N; ++i) {
        if (!in_group(S, in.nl[0].g1, X.types[static_cast<size_t>(i)]))
          throw Error(PFMD_E_PARAM, r.settings + ": the rjl group must hold every atom");
        sp[static_cast<size_t>(i)] = 0;
      }
    } else if (rjl.empty() && lj1g.size() == 2 && lj.size() == 1) {
      r.kind = KIND_LJ;
      const int ga = lj1g[0]->nl[0].g1, gb = lj1g[1]->nl[0].g1;
      r.aa = lj_from(lj1g[0]->p);
      r.bb = lj_from(lj1g[1]->p);
      r.ab = lj_from(lj[0]->p);
      r.rc = lj1g[0]->nl[0].r_cut;
      r.period = lj1g[0]->nl[0].period;
      r.nmax_same = std::max(lj1g[0]->nl[0].nmax, lj1g[1]->nl[0].nmax);
      r.nmax_cross = 0;
      for (const auto& nl : lj[0]->nl) r.nmax_cross = std::max(r.nmax_cross, nl.nmax);
      for (const auto* in : {lj1g[0], lj1g[1], lj[0]})
        for (const auto& nl : in->nl)
          if (nl.r_cut != r.rc || nl.period != r.period)
            throw Error(PFMD_E_PARAM, r.settings + ": the lists of an LJ replica need one r_cut and period");
      if (lj[0]->nl.size() < 1 || lj[0]->nl[0].g1 != ga || lj[0]->nl[0].g2 != gb)
        throw Error(PFMD_E_PARAM, r.settings + ": lj must couple the two lj1g groups, first group first");
      for (int i = 0; i < X.N; ++i) {
        const auto& t = X.types[static_cast<size_t>(i)];
        const bool a = in_group(S, ga, t), b = in_group(S, gb, t);
        if (a == b) throw Error(PFMD_E_PARAM, r.settings + ": every atom must be in exactly one lj1g group");
        sp[static_cast<size_t>(i)] = a ? 0 : 1;
      }
    } else {
      throw Error(PFMD_E_PARAM, r.settings + ": a replica is an LJ gas (lj1g, lj1g, lj) or an rjl slab");
    }
    for (const auto& in : S.interactions)
      r.inter_class.push_back(r.kind == KIND_RJL ? 0 : (&in == lj1g[0] ? 0 : (&in == lj1g[1] ? 1 : 2)));
    r.nmove = 0;
    r.zmp = S.zero_momentum_period;
    for (int i = 0; i < X.N; ++i) {
      const auto& t = X.types[static_cast<size_t>(i)];
      if (!in_group(S, S.all_atoms, t))
        throw Error(PFMD_E_PARAM, r.settings + ": the all-atoms group must hold every atom");
      if (in_group(S, S.z_moving, t))
        throw Error(PFMD_E_PARAM, r.settings + ": the batched form has no z-only moving group");
      const bool mv = in_group(S, S.xyz_moving, t), ke = in_group(S, S.all_moving, t);
      const bool ch = r.nvt && in_group(S, S.nhc[0].group, t);
      mv_h.push_back(static_cast<unsigned char>((mv ? 1 : 0) | (ke ? 2 : 0) | (ch ? 4 : 0)));
      r.nhc_L += ch ? 1 : 0;
      r.nmove += mv ? 1 : 0;
      r.n_ke += ke ? 1 : 0;
      sp_h.push_back(sp[static_cast<size_t>(i)]);
      mass_h.push_back(X.mass[static_cast<size_t>(i)]);
      for (int k = 0; k < 3; ++k) {
        pos_h.push_back(X.pos[static_cast<size_t>(3 * i + k)]);
        vel_h.push_back(X.vel[static_cast<size_t>(3 * i + k)]);
      }
    }
  }

  void build_tiles() {
    clear_graphs();
    std::vector<Tile> t;
    for (size_t r = 0; r < reps.size(); ++r) {
      const int T = tpa[bucket_of(reps[r])], rpw = 32 / T;
      rep_h[r].tile0 = static_cast<int>(t.size());
      for (int a = 0; a < reps[r].n; a += rpw)
        t.push_back(Tile{reps[r].atom0 + a, std::min(rpw, reps[r].n - a), static_cast<int>(r), T});
      rep_h[r].ntile = static_cast<int>(t.size()) - rep_h[r].tile0;
    }
    if (static_cast<int>(t.size()) > ntile) {
      ntile = static_cast<int>(t.size());
      tile = Buf<Tile>();
      tile.alloc(t.size());
      tile_e = Buf<double>();
      tile_e.alloc(3 * t.size());
      tile_k = Buf<double>();
      tile_k.alloc(t.size());
      tile_kc = Buf<double>();
      tile_kc.alloc(t.size());
      BCK(cudaMemsetAsync(tile_kc.p, 0, tile_kc.n * sizeof(double), st));
      BCK(cudaMemsetAsync(tile_e.p, 0, tile_e.n * sizeof(double), st));  // 3 classes per tile
      BCK(cudaMemsetAsync(tile_k.p, 0, tile_k.n * sizeof(double), st));
    }
    ntile_used = static_cast<int>(t.size());
    tile.up(t, st);
    rep.up(rep_h, st);
    if (any_nvt && nhc.p) {  // new tiles: their chain partials from the current velocities
      k_tile_kc<<<(ntile_used + 7) / 8, 256, 0, st>>>(dev_view());
      BCK(cudaGetLastError());
    }
  }
  int ntile_used = 0;

  // entries: the list's (settings file, prefix) pairs when not read from list_file
  void create(const std::string& input_path, const std::string& list_file, const pfmd_options& o,
              const std::vector<std::pair<std::string, std::string>>* entries = nullptr) {
    BCK(cudaSetDevice(o.device));
    BCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    if (entries) {
      if (entries->empty()) throw Error(PFMD_E_PARAM, "batch: empty settings list");
      for (const auto& e : *entries) {
        HostRep r;
        r.settings = fortio::trim(e.first);
        r.prefix = fortio::trim(e.second);
        reps.push_back(r);
      }
    } else {
      load(input_path, list_file);
    }
    std::vector<double> pos_h, vel_h;
    std::vector<unsigned char> sp_h, mv_h;
    for (auto& r : reps) {
      pfmd_io::Settings S;
      try {
        pfmd_io::read_settings(input_path, r.settings, S);
      } catch (const fortio::ReadError& e) {
        throw Error(PFMD_E_IO, r.settings + ": " + e.what());
      }
      r.atom0 = N;
      add(r, S, pos_h, vel_h, sp_h, mv_h);
      N += r.n;
      for (int i = 0; i < r.n; ++i) rep_of_h.push_back(static_cast<int>(&r - reps.data()));
    }
    rebuild_period = static_cast<int>(reps[0].period);
    energy_period = static_cast<int>(reps[0].log_period);
    zero_momentum_period = reps[0].zmp;
    for (const auto& r : reps) {
      if (r.period != rebuild_period)
        throw Error(PFMD_E_PARAM, "batch: every replica needs the same list period");
      if (r.zmp != zero_momentum_period)
        throw Error(PFMD_E_PARAM, "batch: every replica needs the same zero_momentum_period");
      // every replica's log steps are history rows
      energy_period = static_cast<int>(std::gcd<long long>(energy_period, r.log_period));
      nslot = std::max(nslot, r.nmax_same + r.nmax_cross);
    }
    // energies also at the output period of md_simulation.f90:188 when it is not every step
    // (every step is covered by the energies of a launch's last step)
    if (o.out_period > 1) energy_period = std::gcd(energy_period, o.out_period);
    energy_period = std::max(1, energy_period);
    out_period = std::max(1, o.out_period);
    stride = (N + 31) / 32 * 32;
    // replica table, cell grids
    std::vector<LJSet> ljs;
    std::vector<RJLc<float>> rjls;
    for (auto& r : reps) {
      Rep d{};
      d.atom0 = r.atom0;
      d.n = r.n;
      d.kind = r.kind;
      d.nmax_same = r.nmax_same;
      d.nmax_cross = r.nmax_cross;
      d.rc2 = static_cast<float>(r.rc * r.rc);
      const double maxL = std::max(r.L[0], std::max(r.L[1], r.L[2]));
      const double margin = 1e-3 * r.rc + 2e-3 + 4e-6 * maxL;
      d.cell0 = ncell;
      int nc = 1;
      for (int k = 0; k < 3; ++k) {
        if (!(r.L[k] > 2.0 * r.rc)) throw Error(PFMD_E_PARAM, r.settings + ": box length must exceed 2 r_cut");
        d.nc[k] = std::max(1, static_cast<int>(std::floor(r.L[k] / (r.rc + margin))));
        nc *= d.nc[k];
        d.L[k] = r.L[k];
        d.Ltol[k] = r.L[k] + 0.0000001;
        d.qinv[k] = 4294967296.0 / r.L[k];
        d.qs[k] = static_cast<float>(r.L[k] / 4294967296.0);
      }
      ncell += nc;
      d.ts1 = r.dt;
      d.ts2 = r.dt / 2;
      d.ts3 = r.dt / 4;
      d.ts4 = r.dt / 8;
      d.nvt = r.nvt ? 1 : 0;
      if (r.nvt && r.nhc_L < 1) throw Error(PFMD_E_PARAM, r.settings + ": wrong nhc parameters");
      if (r.kind == KIND_LJ) {
        d.par = static_cast<int>(ljs.size());
        ljs.push_back(LJSet{r.aa.f, r.bb.f, r.ab.f});
      } else {
        d.par = static_cast<int>(rjls.size());
        rjls.push_back(r.rjl.f);
      }
      rep_h.push_back(d);
    }
    // device state
    const size_t n = static_cast<size_t>(N);
    pos.alloc(n);
    vel.alloc(n);
    frc.alloc(n);
    posq.alloc(n);
    mass.alloc(n);
    kc.alloc(n);
    species.alloc(n);
    moving.alloc(n);
    rep_of.alloc(n);
    nnum.alloc(n);
    nlist.alloc(static_cast<size_t>(nslot) * stride);
    pair.alloc(static_cast<size_t>(nslot) * stride);
    ccount.alloc(static_cast<size_t>(ncell));
    cstart.alloc(static_cast<size_t>(ncell) + 1);
    ccursor.alloc(static_cast<size_t>(ncell));
    cell_of.alloc(n);
    catom.alloc(n);
    cposq.alloc(n);
    rep.alloc(reps.size());
    lj.alloc(ljs.size());
    rjl.alloc(rjls.size());
    e_pot.alloc(3 * reps.size());
    e_kin.alloc(reps.size());
    e_nhc.alloc(reps.size());
    BCK(cudaMemsetAsync(e_nhc.p, 0, reps.size() * sizeof(double), st));
    // the chains (set_nose_hoover_chain, md_integrators.f90:182-198)
    {
      std::vector<NHCDev> ch(reps.size());
      for (size_t k = 0; k < reps.size(); ++k) {
        NHCDev& h = ch[k];
        std::memset(&h, 0, sizeof(h));
        h.s = 1.0;
        const HostRep& r = reps[k];
        if (!r.nvt) continue;
        any_nvt = true;
        h.M = r.nhc_M;
        h.L = r.nhc_L;
        h.T = r.nhc_T;
        h.q[0] = r.nhc_q1;
        for (int i = 1; i < h.M; ++i) h.q[i] = h.q[0] / (3.0 * h.L);
        for (int i = 0; i < h.M; ++i) h.iq[i] = 1.0 / h.q[i];
      }
      nhc.alloc(reps.size());
      nhc.up(ch, st);
    }
    vcm.alloc(3 * reps.size());
    status.alloc(4);
    bar.alloc(3);
    step.alloc(1);
    std::vector<double4_32a> p4(n), v4(n);
    std::vector<double> kc_h(n);
    for (size_t i = 0; i < n; ++i) {
      p4[i] = make_double4_32a(pos_h[3 * i], pos_h[3 * i + 1], pos_h[3 * i + 2], 0.0);
      v4[i] = make_double4_32a(vel_h[3 * i], vel_h[3 * i + 1], vel_h[3 * i + 2], 0.0);
      kc_h[i] = 1.0 / (mass_h[i] * kMassCoef);
    }
    pos.up(p4, st);
    vel.up(v4, st);
    mass.up(mass_h, st);
    kc.up(kc_h, st);
    species.up(sp_h, st);
    moving.up(mv_h, st);
    rep_of.up(rep_of_h, st);
    if (!ljs.empty()) lj.up(ljs, st);
    if (!rjls.empty()) rjl.up(rjls, st);
    BCK(cudaMemsetAsync(frc.p, 0, n * sizeof(double4_32a), st));
    BCK(cudaMemsetAsync(nnum.p, 0, n * sizeof(int), st));
    BCK(cudaMemsetAsync(status.p, 0, 4 * sizeof(int), st));
    BCK(cudaMemsetAsync(bar.p, 0, 3 * sizeof(unsigned int), st));
    BCK(cudaMemsetAsync(step.p, 0, sizeof(long long), st));
    BCK(cudaMemsetAsync(e_pot.p, 0, 3 * reps.size() * sizeof(double), st));
    BCK(cudaMemsetAsync(e_kin.p, 0, reps.size() * sizeof(double), st));
    long long max_steps = 0;
    for (const auto& r : reps) max_steps = std::max(max_steps, r.steps);
    hist_cap = max_steps / energy_period + 2;
    hist.alloc(static_cast<size_t>(hist_cap) * reps.size() * kHistCols);
    BCK(cudaMemsetAsync(hist.p, 0, hist.n * sizeof(double), st));
    // threads per row: a heuristic start (the autotuner refines it)
    for (int b = 0; b < kBuckets; ++b) tpa[b] = (b / 3 == KIND_RJL) ? 2 : 2;
    build_tiles();
    // co-resident blocks for the cooperative launch
    int dev = 0, sms = 0, per_sm = 0;
    BCK(cudaGetDevice(&dev));
    BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kThreads, 0));
    if (per_sm < 1) throw Error(PFMD_E_CUDA, "batch: the persistent kernel does not fit on an SM");
    // every co-resident block; a small batch takes one block per SM (its grid
    // barriers are shorter, and every SM still gets work)
    const long long want = std::max<long long>((N + kThreads - 1) / kThreads, sms);
    grid = static_cast<int>(std::min<long long>(static_cast<long long>(sms) * per_sm, want));
    scan_part.alloc(static_cast<size_t>(grid));
    k_pack<<<(N + 255) / 256, 256, 0, st>>>(dev_view());
    BCK(cudaGetLastError());
    BCK(cudaStreamSynchronize(st));
  }

  Dev dev_view() {
    Dev D{};
    D.N = N;
    D.R = static_cast<int>(reps.size());
    D.T = ntile_used;
    D.ncell = ncell;
    D.nslot = nslot;
    D.stride = stride;
    D.rebuild_period = rebuild_period;
    D.energy_period = energy_period;
    D.zero_momentum_period = static_cast<int>(std::min<long long>(zero_momentum_period, 1LL << 30));
    D.vcm = vcm.p;
    D.hist_cap = static_cast<int>(hist_cap);
    D.pos = pos.p;
    D.vel = vel.p;
    D.frc = frc.p;
    D.posq = posq.p;
    D.mass = mass.p;
    D.kc = kc.p;
    D.species = species.p;
    D.moving = moving.p;
    D.rep_of = rep_of.p;
    D.nnum = nnum.p;
    D.nlist = nlist.p;
    D.pair = pair.p;
    D.ccount = ccount.p;
    D.cstart = cstart.p;
    D.ccursor = ccursor.p;
    D.cell_of = cell_of.p;
    D.catom = catom.p;
    D.cposq = cposq.p;
    D.scan_part = scan_part.p;
    D.rep = rep.p;
    D.lj = lj.p;
    D.rjl = rjl.p;
    D.tile = tile.p;
    D.tile_e = tile_e.p;
    D.tile_k = tile_k.p;
    D.tile_kc = tile_kc.p;
    D.nhc = nhc.p;
    D.e_nhc = e_nhc.p;
    D.any_nvt = any_nvt ? 1 : 0;
    D.e_pot = e_pot.p;
    D.e_kin = e_kin.p;
    D.hist = hist.p;
    D.bar_count = bar.p;
    D.bar_gen = bar.p + 1;
    D.bar_flag = bar.p + 2;
    D.spin_limit = g_wait_hook.spin_limit ? g_wait_hook.spin_limit : (1u << 22);
    D.bar_extra = g_wait_hook.stall ? 1u : 0u;
    D.status = status.p;
    D.step = step.p;
    return D;
  }

  void launch(int nsteps) {
    Dev D = dev_view();
    void* args[] = {&D, &nsteps};
    BCK(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(k_batch), dim3(grid), dim3(kThreads), args, 0, st));
    ++g_kernel_launches;
  }

  void check_status() {
    int s[4];
    BCK(cudaMemcpyAsync(s, status.p, sizeof(s), cudaMemcpyDeviceToHost, st));
    BCK(cudaStreamSynchronize(st));
    if (s[0] == 0) return;
    const std::string where = s[1] >= 0 ? " (replica " + std::to_string(s[1] + 1) + " '" +
                                              reps[static_cast<size_t>(s[1])].settings + "', atom " +
                                              std::to_string(s[2] + 1) + ")"
                                        : "";
    switch (s[0]) {
      case PFMD_E_NLIST_OVERFLOW: throw Error(s[0], "error: too many neighbours" + where);
      case PFMD_E_OUT_OF_CELL: throw Error(s[0], "particle out of cell" + where);
      case PFMD_E_TIMEOUT: throw Error(s[0], "batch: a grid barrier gave up waiting");
      default: throw Error(s[0], "batch: device error " + std::to_string(s[0]));
    }
  }

  // Advances every replica by nsteps MD steps in chunks of at most `chunk` steps
  // per launch; *ms = device time of the launches.
  double run(long long nsteps, int chunk = 100) {
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    auto launches = [&] {
      for (long long done = 0; done < nsteps;) {
        const int k = static_cast<int>(std::min<long long>(chunk, nsteps - done));
        launch(k);
        done += k;
      }
    };
    const auto key = std::make_pair(nsteps, chunk);
    // while the wait test hook is set, launch directly: a graph would keep the
    // launch arguments of its capture
    const bool hooked = g_wait_hook.spin_limit != 0 || g_wait_hook.stall != 0;
    auto it = hooked ? graphs.end() : graphs.find(key);
    if (it == graphs.end() && graphs_ok && !hooked) {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        const long long before = g_kernel_launches;
        for (long long done = 0; done < nsteps && ok;) {
          int k = static_cast<int>(std::min<long long>(chunk, nsteps - done));
          Dev D = dev_view();
          void* args[] = {&D, &k};
          ok = cudaLaunchCooperativeKernel(reinterpret_cast<void*>(k_batch), dim3(grid), dim3(kThreads), args, 0,
                                           st) == cudaSuccess;
          done += k;
        }
        g_kernel_launches = before;  // counted when the graph runs
        ok = (cudaStreamEndCapture(st, &g) == cudaSuccess) && ok && g != nullptr;
        if (ok) ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
      }
      if (ok) {
        it = graphs.emplace(key, ge).first;
      } else {
        cudaGetLastError();  // not capturable here: launch directly from now on
        graphs_ok = false;
      }
    }
    BCK(cudaEventRecord(e0, st));
    if (it != graphs.end()) {
      BCK(cudaGraphLaunch(it->second, st));
      g_kernel_launches += (nsteps + chunk - 1) / chunk;
    } else {
      launches();
    }
    BCK(cudaEventRecord(e1, st));
    BCK(cudaEventSynchronize(e1));
    float ms = 0.f;
    BCK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    md_step += nsteps;
    check_status();
    return ms;
  }

  // Autotuner: for every bucket, time `steps` MD steps with each candidate threads
  // per row on a saved copy of the state (restored afterwards): one untimed run
  // (it also captures the run's graph), then the fastest of three; keep the
  // fastest candidate.  A single timing per candidate picked worse splits.
  void tune(int steps) {
    const size_t n = static_cast<size_t>(N);
    Buf<double4_32a> sp, sv, sf;
    Buf<int4> sq;
    sp.alloc(n);
    sv.alloc(n);
    sf.alloc(n);
    sq.alloc(n);
    long long step_saved = 0;
    BCK(cudaMemcpyAsync(&step_saved, step.p, sizeof(long long), cudaMemcpyDeviceToHost, st));
    BCK(cudaMemcpyAsync(sp.p, pos.p, n * sizeof(double4_32a), cudaMemcpyDeviceToDevice, st));
    BCK(cudaMemcpyAsync(sv.p, vel.p, n * sizeof(double4_32a), cudaMemcpyDeviceToDevice, st));
    BCK(cudaMemcpyAsync(sf.p, frc.p, n * sizeof(double4_32a), cudaMemcpyDeviceToDevice, st));
    BCK(cudaMemcpyAsync(sq.p, posq.p, n * sizeof(int4), cudaMemcpyDeviceToDevice, st));
    Buf<NHCDev> sh;
    sh.alloc(reps.size());
    BCK(cudaMemcpyAsync(sh.p, nhc.p, reps.size() * sizeof(NHCDev), cudaMemcpyDeviceToDevice, st));
    BCK(cudaStreamSynchronize(st));
    auto restore = [&]() {
      BCK(cudaMemcpyAsync(nhc.p, sh.p, reps.size() * sizeof(NHCDev), cudaMemcpyDeviceToDevice, st));
      BCK(cudaMemcpyAsync(pos.p, sp.p, n * sizeof(double4_32a), cudaMemcpyDeviceToDevice, st));
      BCK(cudaMemcpyAsync(vel.p, sv.p, n * sizeof(double4_32a), cudaMemcpyDeviceToDevice, st));
      BCK(cudaMemcpyAsync(frc.p, sf.p, n * sizeof(double4_32a), cudaMemcpyDeviceToDevice, st));
      BCK(cudaMemcpyAsync(posq.p, sq.p, n * sizeof(int4), cudaMemcpyDeviceToDevice, st));
      // restart at the list period so the trial run rebuilds its lists
      const long long s0 = step_saved - step_saved % rebuild_period;
      BCK(cudaMemcpyAsync(step.p, &s0, sizeof(long long), cudaMemcpyHostToDevice, st));
      if (any_nvt) {  // the chain partials of the restored velocities
        k_tile_kc<<<(ntile_used + 7) / 8, 256, 0, st>>>(dev_view());
        BCK(cudaGetLastError());
      }
      BCK(cudaStreamSynchronize(st));
    };
    const long long md_saved = md_step;
    bool present[kBuckets] = {false};
    for (const auto& r : reps) present[bucket_of(r)] = true;
    for (int b = 0; b < kBuckets; ++b) {
      if (!present[b]) continue;
      int best = tpa[b];
      double best_ms = 1e300;
      for (int cand : {1, 2, 4, 8}) {
        tpa[b] = cand;
        build_tiles();
        restore();
        run(steps, steps);
        double ms = 1e300;
        for (int rep = 0; rep < 3; ++rep) {
          restore();
          ms = std::min(ms, run(steps, steps));
        }
        if (ms < best_ms) {
          best_ms = ms;
          best = cand;
        }
      }
      tpa[b] = best;
    }
    build_tiles();
    restore();
    md_step = md_saved;
  }
};

// A settings-list run on the batched kernel: every entry of the list advanced
// together, and per entry the files of its own run (md_simulation.f90:204-241 and
// 278-297) -- log lines at the log period, snapshots, trajectory frames, the
// closing record (also to all_out_fd, as run_md_simulation.f90:52-62 collects
// them) and final_<xyz>.  Entries must run the same number of steps.
static void write_text(const std::string& fn, const std::string& text, const char* mode) {
  FILE* f = std::fopen(fn.c_str(), mode);
  if (!f) throw Error(PFMD_E_IO, "cannot open " + fn);
  std::fputs(text.c_str(), f);
  std::fclose(f);
}

static void run_list(Batch& B, const std::string& out_path, int all_out_fd, double* device_ms) {
  const long long L = B.reps[0].steps;
  for (const auto& r : B.reps)
    if (r.steps != L)
      throw Error(PFMD_E_PARAM, "batch: every list entry must run the same number of steps (" + r.settings +
                                    ": " + std::to_string(r.steps) + ", first entry: " + std::to_string(L) + ")");
  if (B.md_step != 0) throw Error(PFMD_E_STATE, "batch: a list run starts at step 0");
  const size_t R = B.reps.size();
  // steps after which some entry writes a trajectory frame or a snapshot
  std::vector<long long> ev;
  for (const auto& r : B.reps) {
    for (long long s = 0; s <= L; s += r.traj_period) ev.push_back(s);
    for (long long s = r.snap_period; s <= L; s += r.snap_period) ev.push_back(s);
  }
  std::sort(ev.begin(), ev.end());
  ev.erase(std::unique(ev.begin(), ev.end()), ev.end());
  double ms = 0.0;
  std::vector<double4_32a> p4(static_cast<size_t>(B.N)), v4(static_cast<size_t>(B.N));
  std::vector<double> hp, hv;
  auto state_of = [&](const HostRep& r) {
    hp.resize(3 * static_cast<size_t>(r.n));
    hv.resize(3 * static_cast<size_t>(r.n));
    for (int i = 0; i < r.n; ++i) {
      const double4_32a& p = p4[static_cast<size_t>(r.atom0 + i)];
      const double4_32a& v = v4[static_cast<size_t>(r.atom0 + i)];
      hp[3 * i] = p.x, hp[3 * i + 1] = p.y, hp[3 * i + 2] = p.z;
      hv[3 * i] = v.x, hv[3 * i + 1] = v.y, hv[3 * i + 2] = v.z;
    }
  };
  auto fetch = [&] {
    BCK(cudaMemcpyAsync(p4.data(), B.pos.p, p4.size() * sizeof(double4_32a), cudaMemcpyDeviceToHost, B.st));
    BCK(cudaMemcpyAsync(v4.data(), B.vel.p, v4.size() * sizeof(double4_32a), cudaMemcpyDeviceToHost, B.st));
    BCK(cudaStreamSynchronize(B.st));
  };
  for (const long long e : ev) {
    if (e + 1 > B.md_step) ms += B.run(e + 1 - B.md_step);
    fetch();
    for (const auto& r : B.reps) {
      const std::string prefix = out_path + r.prefix;
      const bool snap = e != 0 && e % r.snap_period == 0, traj = e % r.traj_period == 0;
      if (!snap && !traj) continue;
      state_of(r);
      const std::vector<double>& mass = B.mass_h;
      const double* m = mass.data() + r.atom0;
      if (snap)
        write_text(prefix + "snapshot_" + fortio::fmt_i0pad(e, 6, 6) + ".xyz",
                   pfmd_io::xyz_snapshot_text(r.L, static_cast<int>(r.all_idx.size()), r.all_idx.data(), hp.data(),
                                              hv.data(), m, r.types),
                   "w");
      if (traj) {
        const std::string t = pfmd_io::xyz_traj_frame_text(r.L, static_cast<int>(r.traj_idx.size()),
                                                           r.traj_idx.data(), hp.data(), hv.data(), m, r.types, e);
        if (!t.empty())
          write_text(prefix + "traj_" + fortio::fmt_i0pad(r.traj_group, 2, 2) + ".xyz", t, "a");
      }
    }
  }
  if (L + 1 > B.md_step) ms += B.run(L + 1 - B.md_step);
  fetch();
  // energies: the history rows and the last step's totals
  const long long rows = std::min<long long>(B.hist_cap, L / B.energy_period + 1);
  std::vector<double> hist(static_cast<size_t>(rows) * R * kHistCols), ep(3 * R), ek(R);
  BCK(cudaMemcpyAsync(hist.data(), B.hist.p, hist.size() * sizeof(double), cudaMemcpyDeviceToHost, B.st));
  BCK(cudaMemcpyAsync(ep.data(), B.e_pot.p, ep.size() * sizeof(double), cudaMemcpyDeviceToHost, B.st));
  BCK(cudaMemcpyAsync(ek.data(), B.e_kin.p, ek.size() * sizeof(double), cudaMemcpyDeviceToHost, B.st));
  BCK(cudaStreamSynchronize(B.st));
  const double kt_a_degree = 1.3806488 / 1.6021765654 * 1e-4;  // md_general.f90:304
  for (size_t k = 0; k < R; ++k) {
    const HostRep& r = B.reps[k];
    const std::string prefix = out_path + r.prefix;
    // (potential per interaction in settings order, potential, kinetic, temperature)
    auto energies = [&](const double* cls, double ke, std::vector<double>& inter, double& pe, double& temp) {
      inter.clear();
      pe = 0.0;
      for (int c : r.inter_class) {
        inter.push_back(cls[c]);
        pe += cls[c];
      }
      temp = 2 * ke / kt_a_degree / static_cast<double>(3 * std::max(r.n_ke, 1));
    };
    std::string log;
    double sim_time = 0.0;  // accumulated one step at a time, as md_simulation.f90:243 does
    std::vector<double> inter;
    double pe = 0.0, temp = 0.0;
    for (long long s = 0; s <= L; ++s) {
      if (s != 0) sim_time = sim_time + r.dt;
      if (s % r.log_period != 0) continue;
      const double* h = hist.data() + (static_cast<size_t>(s / B.energy_period) * R + k) * kHistCols;
      energies(h, h[3], inter, pe, temp);
      // the chain's energy (0 under nve, where md() leaves it at its initial 0)
      const double en = r.nvt ? h[4] : 0.0;
      fortio::Rec q;
      q.a(fortio::trim(r.integ_name), 6).i(s, 9);
      q.f(sim_time, 24, 6).f(pe + h[3] + en, 24, 6).f(en, 24, 6).f(pe + h[3], 24, 6).f(pe, 24, 6);
      q.f(h[3], 24, 6).f(temp, 24, 6);
      for (double v : inter) q.f(v, 20, 9);
      for (int j = 0; j < r.n_nhc; ++j) q.f(j == 0 ? en : 0.0, 20, 9);
      log += q.s + "\n";
    }
    // the closing record holds the energies of the last energy step (md_simulation.f90:188)
    long long last = L;
    if (B.out_period > 1) {
      last = -1;
      for (long long s = L; s >= 0 && last < 0; --s)
        if (s % r.log_period == 0 || s % B.out_period == 0) last = s;
    }
    const double* cls;
    double ke;
    if (last == L) {
      cls = ep.data() + 3 * k;
      ke = ek[k];
    } else {
      const double* h = hist.data() + (static_cast<size_t>(last / B.energy_period) * R + k) * kHistCols;
      cls = h;
      ke = h[3];
    }
    energies(cls, ke, inter, pe, temp);
    fortio::Rec c;
    c.a(fortio::trim(prefix), 32).i(L, 9).f(sim_time, 20, 9);
    c.f(pe + ke, 20, 9).f(pe, 20, 9).f(ke, 20, 9).f(temp, 20, 9);
    for (double v : inter) c.f(v, 20, 9);
    if (all_out_fd >= 0) {
      const std::string line = c.s + "\n";
      ssize_t w = ::write(all_out_fd, line.data(), line.size());
      (void)w;
    }
    write_text(prefix + fortio::trim(r.log_file), log + c.s + "\n", "w");
    state_of(r);
    write_text(prefix + "final_" + fortio::trim(r.xyz_file),
               pfmd_io::xyz_snapshot_text(r.L, static_cast<int>(r.all_idx.size()), r.all_idx.data(), hp.data(),
                                          hv.data(), B.mass_h.data() + r.atom0, r.types),
               "w");
  }
  if (device_ms) *device_ms = ms;
}

}  // namespace batch
}  // namespace pfmd

using pfmd::batch::Batch;

struct pfmd_batch {
  std::unique_ptr<Batch> b;
  std::string msg;
};

template <class F>
static int bguard(pfmd_batch* c, F f) {
  try {
    f();
    return PFMD_OK;
  } catch (const pfmd::batch::Error& e) {
    if (c) c->msg = e.what();
    return e.code;
  } catch (const fortio::ReadError& e) {
    if (c) c->msg = e.what();
    return PFMD_E_IO;
  } catch (const std::exception& e) {
    if (c) c->msg = e.what();
    return PFMD_E_PARAM;
  }
}

extern "C" {

int pfmd_batch_create(const char* input_path, const char* list_file, const pfmd_options* opt, pfmd_batch** out) {
  if (!out) return PFMD_E_PARAM;
  auto* c = new pfmd_batch();
  *out = c;
  c->b.reset(new Batch());
  pfmd_options o;
  pfmd_default_options(&o);
  if (opt) o = *opt;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    c->msg = "no CUDA device";
    return PFMD_E_CUDA;
  }
  return bguard(c, [&] { c->b->create(input_path ? input_path : "", list_file ? list_file : "", o); });
}

int pfmd_batch_create_entries(const char* input_path, int n, const char* const* settings,
                              const char* const* prefixes, const pfmd_options* opt, pfmd_batch** out) {
  if (!out) return PFMD_E_PARAM;
  auto* c = new pfmd_batch();
  *out = c;
  c->b.reset(new Batch());
  if (n < 1 || !settings || !prefixes) {
    c->msg = "batch: no entries";
    return PFMD_E_PARAM;
  }
  pfmd_options o;
  pfmd_default_options(&o);
  if (opt) o = *opt;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    c->msg = "no CUDA device";
    return PFMD_E_CUDA;
  }
  std::vector<std::pair<std::string, std::string>> e;
  for (int k = 0; k < n; ++k) e.emplace_back(settings[k] ? settings[k] : "", prefixes[k] ? prefixes[k] : "");
  return bguard(c, [&] { c->b->create(input_path ? input_path : "", "", o, &e); });
}

int pfmd_batch_accepts(const char* input_path, const char* settings, long long* steps, int* list_period,
                       long long* zero_momentum_period, char* why, int why_len) {
  if (why && why_len > 0) why[0] = '\0';
  try {
    pfmd_io::Settings S;
    pfmd_io::read_settings(input_path ? input_path : "", settings ? settings : "", S);
    Batch B;
    pfmd::batch::HostRep r;
    r.settings = settings ? settings : "";
    std::vector<double> p, v;
    std::vector<unsigned char> sp, mv;
    B.add(r, S, p, v, sp, mv);
    if (steps) *steps = r.steps;
    if (list_period) *list_period = static_cast<int>(r.period);
    if (zero_momentum_period) *zero_momentum_period = r.zmp;
    return PFMD_OK;
  } catch (const pfmd::batch::Error& e) {
    if (why && why_len > 0) std::snprintf(why, static_cast<size_t>(why_len), "%s", e.what());
    return e.code;
  } catch (const std::exception& e) {
    if (why && why_len > 0) std::snprintf(why, static_cast<size_t>(why_len), "%s", e.what());
    return PFMD_E_IO;
  }
}

void pfmd_batch_destroy(pfmd_batch* c) { delete c; }

const char* pfmd_batch_errmsg(const pfmd_batch* c) { return c ? c->msg.c_str() : "no batch"; }

int pfmd_batch_info(const pfmd_batch* c, int* n_replicas, long long* n_atoms, long long* md_step) {
  if (!c || !c->b) return PFMD_E_STATE;
  if (n_replicas) *n_replicas = static_cast<int>(c->b->reps.size());
  if (n_atoms) *n_atoms = c->b->N;
  if (md_step) *md_step = c->b->md_step;
  return PFMD_OK;
}

int pfmd_batch_replica(const pfmd_batch* c, int r, int* atom0, int* n, int* kind) {
  if (!c || !c->b) return PFMD_E_STATE;
  if (r < 0 || r >= static_cast<int>(c->b->reps.size())) return PFMD_E_PARAM;
  const auto& R = c->b->reps[static_cast<size_t>(r)];
  if (atom0) *atom0 = R.atom0;
  if (n) *n = R.n;
  if (kind) *kind = R.kind;
  return PFMD_OK;
}

int pfmd_batch_run(pfmd_batch* c, long long nsteps, double* device_ms) {
  if (!c || !c->b) return PFMD_E_STATE;
  return bguard(c, [&] {
    const double ms = c->b->run(nsteps);
    if (device_ms) *device_ms = ms;
  });
}

int pfmd_batch_run_list(pfmd_batch* c, const char* out_path, int all_out_fd, double* device_ms) {
  if (!c || !c->b) return PFMD_E_STATE;
  return bguard(c, [&] { pfmd::batch::run_list(*c->b, fortio::trim(out_path ? out_path : ""), all_out_fd, device_ms); });
}

int pfmd_batch_graphs(const pfmd_batch* c, int* n) {
  if (!c || !c->b || !n) return PFMD_E_STATE;
  *n = c->b->graphs_ok ? static_cast<int>(c->b->graphs.size()) : -1;
  return PFMD_OK;
}

int pfmd_batch_tune(pfmd_batch* c, int steps, int* tpa) {
  if (!c || !c->b) return PFMD_E_STATE;
  return bguard(c, [&] {
    if (c->b->md_step % c->b->rebuild_period != 0)
      throw pfmd::batch::Error(PFMD_E_STATE, "batch: tune at a list-period boundary");
    c->b->tune(std::max(steps, 1));
    if (tpa)
      for (int b = 0; b < pfmd::batch::kBuckets; ++b) tpa[b] = c->b->tpa[b];
  });
}

int pfmd_batch_set_tpa(pfmd_batch* c, const int* tpa) {
  if (!c || !c->b || !tpa) return PFMD_E_STATE;
  return bguard(c, [&] {
    for (int b = 0; b < pfmd::batch::kBuckets; ++b)
      if (tpa[b] != 1 && tpa[b] != 2 && tpa[b] != 4 && tpa[b] != 8)
        throw pfmd::batch::Error(PFMD_E_PARAM, "batch: threads per row must be 1, 2, 4 or 8");
    for (int b = 0; b < pfmd::batch::kBuckets; ++b) c->b->tpa[b] = tpa[b];
    c->b->build_tiles();
    BCK(cudaStreamSynchronize(c->b->st));
  });
}

int pfmd_batch_get_state(pfmd_batch* c, int r, double* pos, double* vel, double* frc) {
  if (!c || !c->b) return PFMD_E_STATE;
  return bguard(c, [&] {
    auto& B = *c->b;
    if (r < 0 || r >= static_cast<int>(B.reps.size())) throw pfmd::batch::Error(PFMD_E_PARAM, "batch: replica out of range");
    const auto& R = B.reps[static_cast<size_t>(r)];
    std::vector<double4_32a> t(static_cast<size_t>(R.n));
    auto get = [&](double4_32a* src, double* dst) {
      if (!dst) return;
      BCK(cudaMemcpyAsync(t.data(), src + R.atom0, t.size() * sizeof(double4_32a), cudaMemcpyDeviceToHost, B.st));
      BCK(cudaStreamSynchronize(B.st));
      for (size_t i = 0; i < t.size(); ++i) {
        dst[3 * i] = t[i].x;
        dst[3 * i + 1] = t[i].y;
        dst[3 * i + 2] = t[i].z;
      }
    };
    get(B.pos.p, pos);
    get(B.vel.p, vel);
    get(B.frc.p, frc);
  });
}

int pfmd_batch_energies(pfmd_batch* c, double* e_pot, double* e_kin) {
  if (!c || !c->b) return PFMD_E_STATE;
  return bguard(c, [&] {
    auto& B = *c->b;
    const size_t R = B.reps.size();
    std::vector<double> ep(3 * R);
    BCK(cudaMemcpyAsync(ep.data(), B.e_pot.p, ep.size() * sizeof(double), cudaMemcpyDeviceToHost, B.st));
    if (e_kin) BCK(cudaMemcpyAsync(e_kin, B.e_kin.p, R * sizeof(double), cudaMemcpyDeviceToHost, B.st));
    BCK(cudaStreamSynchronize(B.st));
    if (e_pot)
      for (size_t r = 0; r < R; ++r) e_pot[r] = ep[3 * r] + ep[3 * r + 1] + ep[3 * r + 2];
  });
}

int pfmd_batch_energy_history(pfmd_batch* c, double* hist, long long* rows, int* period) {
  if (!c || !c->b) return PFMD_E_STATE;
  return bguard(c, [&] {
    auto& B = *c->b;
    const long long avail = std::min<long long>(B.hist_cap, B.md_step == 0 ? 0 : (B.md_step - 1) / B.energy_period + 1);
    if (rows) *rows = avail;
    if (period) *period = B.energy_period;
    if (hist && avail > 0)
      BCK(cudaMemcpyAsync(hist, B.hist.p, static_cast<size_t>(avail) * B.reps.size() * pfmd::batch::kHistCols * sizeof(double),
                          cudaMemcpyDeviceToHost, B.st));
    BCK(cudaStreamSynchronize(B.st));
  });
}

}  // extern "C"

// Neighbour lists on the device: cell binning, list build, graphene nearest
// neighbours and normals.
//
// Reference: find_neighbours (md_neighbours.f90:56-100) tests every pair of the two
// groups; converce_neighbour_list (md_neighbours.f90:128-160) transposes a list every
// step; find_gr_nearest_neighbors / find_norm_in_graphene (graphenenorm.f90:8-56).
//
// Here the candidates come from a cell grid over the column group (cells at least
// r_cut wide, so the 27 surrounding cells hold every partner).  Binning writes
// cell-ordered copies of each candidate's group-2 index, atom index and
// fixed-point position, so one warp per row streams its candidates contiguously.
// The row is sorted by group-2 index before it is written, so it holds exactly the
// reference's entries in the reference's order; the entries stored are the atom
// indexes of those partners (the force kernels need nothing else) and the
// reference's group-2 indexes are recovered on read-back.  In the plain form an
// FP32 prefilter with a safety margin discards far candidates and the survivors
// are tested with the exact FP64 predicate (mi_exact); the precision form uses the
// fixed-point separation alone.  The converse list is built the same way with the
// groups swapped at the source list's rebuild steps: its membership equals the
// transpose because dr.dr is symmetric bit for bit.  Distances are not stored:
// every force kernel recomputes them from positions.
#include <climits>

#include "kernels.h"

namespace pfmd {

static constexpr int kBuildWarps = 8;

__global__ void k_pack_posq(Atoms A, Box B) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.N) {
    double4_32a p = A.pos[i];
    A.posq[i] = make_int4(quantize(p.x, B.qinv[0]), quantize(p.y, B.qinv[1]), quantize(p.z, B.qinv[2]), 0);
  }
}

__global__ void k_bin_count(ListDev L, CellGrid cg, Atoms A, Ctl* ctl) {
  if (ctl->stop || skin_keep(ctl, L.skin)) return;
  int n2 = ctl->group_n[L.col_group];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n2) return;
  int4 p = A.posq[L.col_idx[j]];
  int c = (cell_q(p.z, cg.nc[2]) * cg.nc[1] + cell_q(p.y, cg.nc[1])) * cg.nc[0] + cell_q(p.x, cg.nc[0]);
  cg.cell_of[j] = c;
  atomicAdd(&cg.count[c], 1);
}

// Exclusive scan of the cell counts by one block of 1024 threads: 1024 cells per
// pass (coalesced), shuffles within each warp, a second shuffle level over the 32
// warp totals, and a carry from pass to pass.
__global__ void __launch_bounds__(1024) k_bin_scan(CellGrid cg, int skin, Ctl* ctl) {
  if (ctl->stop || skin_keep(ctl, skin)) return;
  __shared__ int wsum[32];
  __shared__ int carry_s;
  const int n = cg.ncell, t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) carry_s = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int c = base + t;
    const int v = c < n ? cg.count[c] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int s = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      wsum[lane] = s;
    }
    __syncthreads();
    const int carry = carry_s;
    const int excl = carry + (w ? wsum[w - 1] : 0) + x - v;
    if (c < n) {
      cg.start[c] = excl;
      cg.cursor[c] = excl;
    }
    __syncthreads();  // every thread has read carry_s and wsum
    if (t == 1023) carry_s = carry + wsum[31];
    __syncthreads();
  }
  if (t == 0) cg.start[n] = carry_s;
}

__global__ void k_bin_scatter(ListDev L, CellGrid cg, Atoms A, Ctl* ctl) {
  if (ctl->stop || skin_keep(ctl, L.skin)) return;
  int n2 = ctl->group_n[L.col_group];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n2) return;
  int slot = atomicAdd(&cg.cursor[cg.cell_of[j]], 1);
  const int a = L.col_idx[j];
  cg.jnd[slot] = j;
  cg.atom[slot] = a;
  cg.posq[slot] = A.posq[a];
}

// Puts every cell's atoms in ascending group-2 order, so rows built from the
// cell order (no per-row sort) are the same on every run.  One warp per cell;
// cells of more than 32 atoms (rare: large or sparse cells) use an insertion
// sort by one lane.
__global__ void k_cell_sort(CellGrid cg, int skin, Ctl* ctl) {
  if (ctl->stop || skin_keep(ctl, skin)) return;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= cg.ncell) return;
  const int s = cg.start[c], e = cg.start[c + 1], len = e - s;
  if (len <= 1) return;
  if (len <= 32) {
    int key = lane < len ? cg.jnd[s + lane] : INT_MAX;
    int src = lane;
    const int atom = lane < len ? cg.atom[s + lane] : 0;
    const int4 pq = lane < len ? cg.posq[s + lane] : make_int4(0, 0, 0, 0);
    for (int k = 2; k <= 32; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        const int ok = __shfl_xor_sync(0xffffffffu, key, j);
        const int os = __shfl_xor_sync(0xffffffffu, src, j);
        const bool lower = (lane & j) == 0, up = (lane & k) == 0;
        const bool take = lower ? ((key > ok) == up) : ((key < ok) == up);
        if (take) {
          key = ok;
          src = os;
        }
      }
    }
    const int a = __shfl_sync(0xffffffffu, atom, src);
    int4 q;
    q.x = __shfl_sync(0xffffffffu, pq.x, src);
    q.y = __shfl_sync(0xffffffffu, pq.y, src);
    q.z = __shfl_sync(0xffffffffu, pq.z, src);
    q.w = 0;
    if (lane < len) {
      cg.jnd[s + lane] = key;
      cg.atom[s + lane] = a;
      cg.posq[s + lane] = q;
    }
  } else if (lane == 0) {
    for (int i = s + 1; i < e; ++i) {
      const int k = cg.jnd[i], a = cg.atom[i];
      const int4 q = cg.posq[i];
      int j = i - 1;
      while (j >= s && cg.jnd[j] > k) {
        cg.jnd[j + 1] = cg.jnd[j];
        cg.atom[j + 1] = cg.atom[j];
        cg.posq[j + 1] = cg.posq[j];
        --j;
      }
      cg.jnd[j + 1] = k;
      cg.atom[j + 1] = a;
      cg.posq[j + 1] = q;
    }
  }
}

// One warp per row.  CAP >= nmax rounded up to a power of two.  SORT: sort the
// row by group-2 index (the reference's order; needed for bit-exact lists and for
// lessnnum in groups that are not in atom order).  Without SORT the row keeps the
// cell-scan order, which the per-cell sort makes deterministic.
template <bool PREC, int CAP, bool SORT>
__global__ void __launch_bounds__(kBuildWarps * 32) k_build(ListDev L, CellGrid cg, Atoms A, Box B, double rc2,
                                                             float rcp2, int converse, int src_rows, Ctl* ctl) {
  __shared__ int sbuf[kBuildWarps][CAP];
  if (ctl->stop || skin_keep(ctl, L.skin)) return;
  const int n1 = ctl->group_n[L.row_group];
  const int n2 = ctl->group_n[L.col_group];
  if (!converse) {
    // update_neighbour_list only acts when both groups and the list are non-empty
    if (n1 == 0 || n2 == 0 || L.rows == 0) return;
  } else {
    // converce_neighbour_list acts when group 2, the source list and itself are
    if (n1 == 0 || src_rows == 0 || L.rows == 0) return;
  }
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int row = blockIdx.x * kBuildWarps + wib;
  if (row == 0 && lane == 0 && n1 > L.rows) set_error(ctl, ST_PARAM, EK_NONE, L.id, n1, L.rows);
  if (row >= L.rows) return;
  if (row >= n1) {
    // rows past the group: the converse list clears them, a regular list keeps them
    if (converse && lane == 0) L.nnum[row] = 0;
    return;
  }
  int* buf = sbuf[wib];
  const int ai = L.row_idx[row];
  const int4 piq = A.posq[ai];
  double4_32a pi = make_double4_32a(0, 0, 0, 0);
  if (!PREC) pi = A.pos[ai];
  const int c0[3] = {cell_q(piq.x, cg.nc[0]), cell_q(piq.y, cg.nc[1]), cell_q(piq.z, cg.nc[2])};
  int lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (cg.nc[k] < 3) {
      lo[k] = 0;
      hi[k] = cg.nc[k] - 1;
    } else {
      lo[k] = c0[k] - 1;
      hi[k] = c0[k] + 1;
    }
  }
  int cnt = 0;
  int nless = 0;  // entries with a smaller atom index (lessnnum of an unsorted row)
  const int nx = cg.nc[0];
  for (int z = lo[2]; z <= hi[2]; ++z) {
    const int cz = (z + cg.nc[2]) % cg.nc[2];
    for (int y = lo[1]; y <= hi[1]; ++y) {
      const int cy = (y + cg.nc[1]) % cg.nc[1];
      const int base = (cz * cg.nc[1] + cy) * nx;
      // the x-cells of this (y,z) row as at most two contiguous candidate runs
      int r0s, r0e, r1s = 0, r1e = 0;
      if (nx < 3) {
        r0s = cg.start[base];
        r0e = cg.start[base + nx];
      } else if (c0[0] >= 1 && c0[0] + 1 < nx) {
        r0s = cg.start[base + c0[0] - 1];
        r0e = cg.start[base + c0[0] + 2];
      } else if (c0[0] == 0) {
        r0s = cg.start[base];
        r0e = cg.start[base + 2];
        r1s = cg.start[base + nx - 1];
        r1e = cg.start[base + nx];
      } else {
        r0s = cg.start[base + nx - 2];
        r0e = cg.start[base + nx];
        r1s = cg.start[base];
        r1e = cg.start[base + 1];
      }
      for (int run = 0; run < 2; ++run) {
        const int s0 = run ? r1s : r0s, e0 = run ? r1e : r0e;
        for (int k0 = s0; k0 < e0; k0 += 32) {
          const int k = k0 + lane;
          bool hit = false;
          int jnd = 0, aj = 0;
          if (k < e0) {
            aj = cg.atom[k];
            if (aj != ai) {
              float d[3];
              const float r2f = mi_q(piq, cg.posq[k], B, d);
              if (PREC) {
                hit = r2f < rcp2;
              } else if (r2f < rcp2) {
                double dd[3];
                hit = mi_exact(pi, A.pos[aj], B, dd) < rc2;
              }
              if (hit) jnd = cg.jnd[k];
            }
          }
          const unsigned m = __ballot_sync(0xffffffffu, hit);
          if (hit) {
            const int p = cnt + __popc(m & ((1u << lane) - 1u));
            if (SORT) {
              if (p < CAP) buf[p] = jnd;
            } else if (p < L.nmax) {
              L.nlist[(size_t)p * L.stride + row] = aj;
            }
          }
          if (!SORT) nless += __popc(__ballot_sync(0xffffffffu, hit && aj < ai));
          cnt += __popc(m);
        }
      }
    }
  }
  __syncwarp();
  if (cnt > L.nmax) {
    // 'error: too many neighbours', ind, nnumind  (md_neighbours.f90:80, :151)
    if (lane == 0) set_error(ctl, ST_NLIST_OVERFLOW, converse ? EK_CONVERSE_OVF : EK_OVERFLOW, L.id, row + 1, L.nmax + 1);
    return;
  }
  if (!SORT) {
    if (lane == 0) {
      L.nnum[row] = cnt;
      L.pidx[row] = ai;
      L.lessnnum[row] = converse ? 0 : nless;
      L.bnd[row] = INT_MAX;
    }
    return;
  }
  // bitonic sort of buf[0..n) ascending, padded with INT_MAX
  int n = 1;
  while (n < cnt) n <<= 1;
  for (int p = cnt + lane; p < n; p += 32) buf[p] = INT_MAX;
  __syncwarp();
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const int a = buf[i], b = buf[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[ixj] = a;
          }
        }
      }
      __syncwarp();
    }
  }
  // lessnnum: entries before the first neighbour with a larger atom index
  // (md_neighbours.f90:78); the converse list leaves it at zero as the reference does
  int less = cnt;
  for (int p0 = 0; p0 < cnt; p0 += 32) {
    const int p = p0 + lane;
    const int aj = p < cnt ? L.col_idx[buf[p]] : 0;
    if (p < cnt) L.nlist[(size_t)p * L.stride + row] = aj;
    if (!converse && less == cnt) {
      const unsigned m = __ballot_sync(0xffffffffu, p < cnt && ai < aj);
      if (m) less = p0 + __ffs(m) - 1;
    }
  }
  if (lane == 0) {
    L.nnum[row] = cnt;
    L.pidx[row] = ai;
    L.lessnnum[row] = converse ? 0 : less;
    L.bnd[row] = (less < cnt) ? buf[less] : INT_MAX;
  }
}

// Self lists (row group == column group) without sorting: one warp per cell,
// four cells per block.  The warp stages the candidates of the surrounding cells
// (the same x-runs, in the same order, as k_build) in its share of shared memory,
// then each lane takes one of the cell's rows and scans the staged candidates in
// order; every lane reads the same candidate at once (a shared-memory broadcast),
// so a (row, candidate) test costs about a dozen instructions for up to 32 rows.
// A lane appends its hits in candidate order: rows and entries come out exactly as
// k_build<PREC, CAP, false> writes them.  lessnnum is not kept (no kernel reads
// it for unsorted rows).  On the 65,536-atom slab (6,615 cells) a rebuild takes as
// long as with one 4-warp block per cell and a warp per row, and a list kept by
// the skin test launches a quarter of the blocks.
static constexpr int kCellWarps = 4;
static constexpr int kWarpCand = 256;  // candidates staged per pass, per warp

__global__ void __launch_bounds__(kCellWarps * 32) k_build_cells(ListDev L, CellGrid cg, Box B, float rcp2, Ctl* ctl) {
  __shared__ float4 s_rel_all[kCellWarps][kWarpCand];  // candidate relative to the cell corner, atom in w
  __shared__ int s_off_all[kCellWarps][19];             // prefix offsets of up to 18 candidate runs
  __shared__ int s_beg_all[kCellWarps][18];             // run starts in the cell-ordered arrays
  if (ctl->stop || skin_keep(ctl, L.skin)) return;
  const int n1 = ctl->group_n[L.row_group];
  // update_neighbour_list only acts when the group and the list are non-empty
  if (n1 == 0 || L.rows == 0) return;
  if (n1 > L.rows) {  // rows are indexed by group index: nothing is written past L.rows
    if (blockIdx.x == 0 && threadIdx.x == 0) set_error(ctl, ST_PARAM, EK_NONE, L.id, n1, L.rows);
    return;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = blockIdx.x * kCellWarps + w;
  if (c >= cg.ncell) return;
  const int r0 = cg.start[c], nr = cg.start[c + 1] - r0;
  if (nr == 0) return;
  float4* s_rel = s_rel_all[w];
  int* s_off = s_off_all[w];
  int* s_beg = s_beg_all[w];
  const int nx = cg.nc[0], ny = cg.nc[1], nz = cg.nc[2];
  const int cx = c % nx, cy = (c / nx) % ny, cz = c / (nx * ny);
  // run t: (y, z) row t/2 of the 3x3 (fewer when a dimension has < 3 cells), z
  // outer, y inner; x-run t&1
  int len = 0;
  if (lane < 18) {
    const int t = lane, which = t & 1, yz = t >> 1;
    const int my = ny < 3 ? ny : 3, mz = nz < 3 ? nz : 3;
    int b = 0, e = 0;
    if (yz < my * mz) {
      const int iy = yz % my, iz = yz / my;
      const int y = ny < 3 ? iy : (cy - 1 + iy + ny) % ny;
      const int z = nz < 3 ? iz : (cz - 1 + iz + nz) % nz;
      const int base = (z * ny + y) * nx;
      if (nx < 3) {
        if (!which) { b = cg.start[base]; e = cg.start[base + nx]; }
      } else if (cx >= 1 && cx + 1 < nx) {
        if (!which) { b = cg.start[base + cx - 1]; e = cg.start[base + cx + 2]; }
      } else if (cx == 0) {
        if (!which) { b = cg.start[base]; e = cg.start[base + 2]; }
        else { b = cg.start[base + nx - 1]; e = cg.start[base + nx]; }
      } else {
        if (!which) { b = cg.start[base + nx - 2]; e = cg.start[base + nx]; }
        else { b = cg.start[base]; e = cg.start[base + 1]; }
      }
    }
    s_beg[t] = b;
    len = e - b;
  }
  // exclusive prefix of the run lengths over lanes 0..17
  int incl = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane < 18) s_off[lane + 1] = incl;
  if (lane == 0) s_off[0] = 0;
  __syncwarp();
  const int total = s_off[18];
  // Positions relative to this cell's lower corner, as FP32: every candidate lies
  // within one cell of the corner cell, so with at least 4 cells per dimension
  // (cells at most L/4 wide) the fixed-point difference is the minimum image and a
  // pair's separation is the plain difference of two relative positions.  Grids
  // with fewer cells keep the per-pair minimum image.
  const bool rel_ok = nx >= 4 && ny >= 4 && nz >= 4;
  const unsigned int ref[3] = {(unsigned int)(((unsigned long long)cx << 32) / (unsigned long long)nx),
                               (unsigned int)(((unsigned long long)cy << 32) / (unsigned long long)ny),
                               (unsigned int)(((unsigned long long)cz << 32) / (unsigned long long)nz)};
  for (int rg = 0; rg < nr; rg += 32) {
    const bool has_row = rg + lane < nr;
    const int kr = r0 + rg + (has_row ? lane : 0);
    const int ai = cg.atom[kr], row = cg.jnd[kr];
    const int4 piq = cg.posq[kr];
    const float ix = (float)(int)((unsigned int)piq.x - ref[0]) * B.qs[0];
    const float iy = (float)(int)((unsigned int)piq.y - ref[1]) * B.qs[1];
    const float iz = (float)(int)((unsigned int)piq.z - ref[2]) * B.qs[2];
    int cnt = 0;
    for (int b0 = 0; b0 < total; b0 += kWarpCand) {
      const int nb = min(kWarpCand, total - b0);
      __syncwarp();  // the previous pass is done with the staged candidates
      int r = 0;
#pragma unroll 4
      for (int v = lane; v < nb; v += 32) {
        const int g = b0 + v;
        while (s_off[r + 1] <= g) ++r;  // g < total = s_off[18], so r < 18
        {
          const int k = s_beg[r] + (g - s_off[r]);
          const int4 q = cg.posq[k];
          float4 rp;
          if (rel_ok) {
            rp.x = (float)(int)((unsigned int)q.x - ref[0]) * B.qs[0];
            rp.y = (float)(int)((unsigned int)q.y - ref[1]) * B.qs[1];
            rp.z = (float)(int)((unsigned int)q.z - ref[2]) * B.qs[2];
          } else {  // the raw fixed-point coordinates, for the per-pair minimum image
            rp.x = __int_as_float(q.x);
            rp.y = __int_as_float(q.y);
            rp.z = __int_as_float(q.z);
          }
          rp.w = __int_as_float(cg.atom[k]);
          s_rel[v] = rp;
        }
      }
      __syncwarp();
      if (has_row) {
        if (rel_ok) {
#pragma unroll 4
          for (int k = 0; k < nb; ++k) {
            const float4 q = s_rel[k];
            const int aj = __float_as_int(q.w);
            const float dx = q.x - ix, dy = q.y - iy, dz = q.z - iz;
            if (aj != ai && dx * dx + dy * dy + dz * dz < rcp2) {
              if (cnt < L.nmax) L.nlist[(size_t)cnt * L.stride + row] = aj;
              ++cnt;
            }
          }
        } else {
          for (int k = 0; k < nb; ++k) {
            const float4 q = s_rel[k];
            const int aj = __float_as_int(q.w);
            float d[3];
            if (aj != ai &&
                mi_q(piq, make_int4(__float_as_int(q.x), __float_as_int(q.y), __float_as_int(q.z), 0), B, d) < rcp2) {
              if (cnt < L.nmax) L.nlist[(size_t)cnt * L.stride + row] = aj;
              ++cnt;
            }
          }
        }
      }
    }
    if (has_row) {
      if (cnt > L.nmax) {
        // 'error: too many neighbours', ind, nnumind  (md_neighbours.f90:80)
        set_error(ctl, ST_NLIST_OVERFLOW, EK_OVERFLOW, L.id, row + 1, L.nmax + 1);
      } else {
        L.nnum[row] = cnt;
        L.pidx[row] = ai;
        L.bnd[row] = INT_MAX;  // lessnnum of an unsorted row is formed when it is read back
      }
    }
  }
}

// tb entries are atoms; the nn list keeps tb row indexes (tb lists have g1 == g2)
template <bool PREC>
__global__ void k_nn_select(ListDev tb, ListDev nn, double rcnn, Atoms A, Box B, Ctl* ctl) {
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= tb.rows) return;
  const int ai = tb.row_idx[i];
  const int n = tb.nnum[i];

  int k = 0;
  bool bad = false;
  for (int p = 0; p < n; ++p) {
    const int aj = tb.nlist[(size_t)p * tb.stride + i];
    bool in;
    if (PREC) {
      float d[3];
      float r2 = mi_q(A.posq[ai], A.posq[aj], B, d);
      in = sqrtf(r2) < (float)rcnn;
    } else {
      double d[3];
      double r2 = mi_exact(A.pos[ai], A.pos[aj], B, d);
      in = sqrt(r2) < rcnn;
    }
    if (in) {
      k = k + 1;
      if (k <= 3) {
        nn.nlist[(size_t)(k - 1) * nn.stride + i] = tb.row_of[aj];
      } else {
        set_error(ctl, ST_GR_NN, EK_GR_TOO_MANY, i + 1, 0, 0);
        bad = true;
        break;
      }
    }
  }
  if (!bad && k != 3) set_error(ctl, ST_GR_NN, EK_GR_NOT_ENOUGH, i + 1, k, 0);
  nn.nnum[i] = 3;
}

// Normals of the nn rows, stored per atom (norm[atom]); nn entries are group
// indexes of nn.col_idx (tb rows, or group 6 of the list without tb).
template <bool PREC>
__global__ void k_normals(ListDev nn, double4_32a* norm, int simplified, Atoms A, Box B, Ctl* ctl) {
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn.rows || i >= nn.row_cap) return;  // rows past the row group have no atom
  const int ai = nn.row_idx[i];
  if (simplified) {
    norm[ai] = make_double4_32a(0.0, 0.0, 1.0, 1.0);
    return;
  }
  const int cnt = nn.nnum[i];
  double d[3][3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    d[q][0] = d[q][1] = d[q][2] = 0.0;
    if (q < cnt) {
      const int aj = nn.col_idx[nn.nlist[(size_t)q * nn.stride + i]];
      if (PREC) {
        float df[3];
        mi_q(A.posq[ai], A.posq[aj], B, df);
        d[q][0] = df[0];
        d[q][1] = df[1];
        d[q][2] = df[2];
      } else {
        mi_exact(A.pos[ai], A.pos[aj], B, d[q]);
      }
    }
  }
  double d12[3], d31[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    d12[k] = d[1][k] - d[0][k];
    d31[k] = d[0][k] - d[2][k];
  }
  double g0 = d12[1] * d31[2] - d12[2] * d31[1];
  double g1 = d12[2] * d31[0] - d12[0] * d31[2];
  double g2 = d12[0] * d31[1] - d12[1] * d31[0];
  if (g2 < 0.0) {
    g0 = -g0;
    g1 = -g1;
    g2 = -g2;
  }
  const double nr = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
  const double nx = g0 / nr, ny = g1 / nr, nz = g2 / nr;
  // w: 1/|n|^2 of the stored components (1 up to rounding), which morsec's metal
  // side divides by for every pair (MorseCosine.f90:127)
  norm[ai] = make_double4_32a(nx, ny, nz, 1.0 / (nx * nx + ny * ny + nz * nz));
}

__global__ void k_nnum_max(ListDev L, Ctl* ctl) {
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.rows; i += gridDim.x * blockDim.x) m = max(m, L.nnum[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(&ctl->maxnnum[L.id], m);
}

// ---------------- launchers ----------------
static inline int blocks_for(long long n, int bs) { return (int)((n + bs - 1) / bs); }

void launch_pack_posq(const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s) {
  (void)ctl;
  if (A.N > 0) { k_pack_posq<<<blocks_for(A.N, 256), 256, 0, s>>>(A, B); ++g_kernel_launches; }
}

// Skin-triggered rebuilds (precision form).  At a list's update step every atom of
// its groups records its displacement since the list was built (xref) and over
// the last period (xprev, then updated), as maxima of the squares; the last block
// of k_skin_check to finish (or k_skin_decide, for empty groups) asks for a
// rebuild when the two maxima add up to more than half the skin, so the list
// stays complete through the next period if no atom moves faster than in the
// last one.  Maxima by atomicMax on the bits of non-negative floats: the same
// result in any order.
//
// Two-level lists (xout non-null): the list's rows are filtered from an outer
// list built with a radius `margin` wider.  Every pair now within the list's
// radius was within it plus twice the largest displacement at the outer build,
// so the outer list is rebuilt (binning and the cell kernels) only when a
// rebuild is due and some atom moved more than half the margin since the outer
// build; otherwise a rebuild is the filter pass alone.
// The decision from the recorded maxima (read atomically: the blocks that
// recorded them may still be in flight on other SMs until their fences), then the
// maxima cleared for the next update step.
__device__ __forceinline__ void skin_decide(Ctl* ctl, int id, float half_skin, float half_margin, bool outer) {
  const float b = sqrtf(__uint_as_float(atomicMax(&ctl->skin_max[id][0], 0u)));
  const float p = sqrtf(__uint_as_float(atomicMax(&ctl->skin_max[id][1], 0u)));
  const bool need = ctl->list_need[id] != 0 || !(b + p <= half_skin);
  if (need) ctl->list_need[id] = 1;
  if (outer) {
    const float o = sqrtf(__uint_as_float(atomicMax(&ctl->skin_max[id][2], 0u)));
    if (ctl->outer_need[id] != 0 || (need && !(o <= half_margin))) ctl->outer_need[id] = 1;
  }
  ctl->skin_max[id][0] = 0u;
  ctl->skin_max[id][1] = 0u;
  ctl->skin_max[id][2] = 0u;
}

__global__ void k_skin_check(ListDev L, Atoms A, Box B, const int4* xref, int4* xprev, const int4* xout, int both,
                             float half_skin, float half_margin, Ctl* ctl) {
  if (block_stop(ctl)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nr = ctl->group_n[L.row_group], nc = ctl->group_n[L.col_group];
  int a = -1;
  if (i < L.row_cap) {
    if (i < nr) a = L.row_idx[i];
  } else if (both && i - L.row_cap < nc) {
    a = L.col_idx[i - L.row_cap];
  }
  unsigned int ub = 0u, up = 0u, uo = 0u;
  if (a >= 0) {
    const int4 q = A.posq[a];
    float d[3];
    ub = __float_as_uint(mi_q(xref[a], q, B, d));
    up = __float_as_uint(mi_q(xprev[a], q, B, d));
    if (xout) uo = __float_as_uint(mi_q(xout[a], q, B, d));
    xprev[a] = q;
  }
  // one atomic per warp
  ub = __reduce_max_sync(0xffffffffu, ub);
  up = __reduce_max_sync(0xffffffffu, up);
  uo = __reduce_max_sync(0xffffffffu, uo);
  if ((threadIdx.x & 31) == 0) {
    if (ub) atomicMax(&ctl->skin_max[L.skin][0], ub);
    if (up) atomicMax(&ctl->skin_max[L.skin][1], up);
    if (uo) atomicMax(&ctl->skin_max[L.skin][2], uo);
    __threadfence();  // the maxima are visible before this block is counted
  }
  // the last block to finish reads the maxima and decides (as k_skin_decide):
  // one launch fewer per update step (30.60 -> 30.33 us per MD step on the
  // 65,536-atom slab, with the kept-list return in k_skin_commit)
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(&ctl->skin_done[L.skin], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  skin_decide(ctl, L.skin, half_skin, half_margin, xout != nullptr);
  ctl->skin_done[L.skin] = 0u;
}
__global__ void k_skin_decide(int id, float half_skin, float half_margin, int outer, Ctl* ctl) {
  if (ctl->stop) return;
  skin_decide(ctl, id, half_skin, half_margin, outer != 0);
}
// After the update step: a rebuilt list's atoms give the new reference positions
// (and a rebuilt outer list's, the outer reference); the last block to finish
// clears the flags (every block has read them by then).
__global__ void k_skin_commit(ListDev L, Atoms A, int4* xref, int4* xout, Ctl* ctl) {
  if (block_stop(ctl)) return;
  __shared__ int need, oneed;
  if (threadIdx.x == 0) {
    need = ctl->list_need[L.skin];
    oneed = xout ? ctl->outer_need[L.skin] : 0;
  }
  __syncthreads();
  if (!need && !oneed) return;  // nothing rebuilt: the flags are already clear
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.N; a += gridDim.x * blockDim.x) {
    const int4 q = A.posq[a];
    if (need) xref[a] = q;
    if (oneed) xout[a] = q;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int done = atomicAdd(&ctl->skin_done[L.skin], 1u);
    if (done == gridDim.x - 1) {
      if (need) ctl->list_builds[L.skin] += 1;
      ctl->list_need[L.skin] = 0;
      ctl->outer_need[L.skin] = 0;
      ctl->skin_done[L.skin] = 0;
    }
  }
}

void launch_skin_check(const ListDev& L, const Atoms& A, const Box& B, const int4* xref, int4* xprev,
                       const int4* xout, double half_skin, double half_margin, Ctl* ctl, cudaStream_t s) {
  if (L.skin < 0) return;
  const int both = L.row_group != L.col_group ? 1 : 0;  // a self list checks its rows once
  const int n = L.row_cap + (both ? L.col_cap : 0);
  if (n > 0) {
    k_skin_check<<<blocks_for(n, 256), 256, 0, s>>>(L, A, B, xref, xprev, xout, both, static_cast<float>(half_skin),
                                                   static_cast<float>(half_margin), ctl);
    ++g_kernel_launches;
  } else {
    k_skin_decide<<<1, 1, 0, s>>>(L.skin, static_cast<float>(half_skin), static_cast<float>(half_margin),
                                  xout ? 1 : 0, ctl);
    ++g_kernel_launches;
  }
}
void launch_skin_commit(const ListDev& L, const Atoms& A, int4* xref, int4* xout, Ctl* ctl, cudaStream_t s) {
  if (L.skin < 0) return;
  const int grid = std::max(1, std::min(blocks_for(A.N, 256), 152));
  k_skin_commit<<<grid, 256, 0, s>>>(L, A, xref, xout, ctl);
  ++g_kernel_launches;
}

// The rows of a two-level list from its outer list O (same rows): the entries of
// each outer row within rc, in the outer row's order.  kFilterTpa threads per
// row, lanes laid out as in the force kernels (row = lane % rows-per-warp), so a
// warp reads 8 rows' slots coalesced; each round the hits of a row's lanes are
// ranked by one ballot and appended in slot order.
static constexpr int kFilterTpa = 4;
__global__ void __launch_bounds__(256) k_filter_outer(ListDev L, ListDev O, const int4* __restrict__ posq, Box B,
                                                      float rcp2, Ctl* ctl) {
  if (ctl->stop || skin_keep(ctl, L.skin)) return;
  const int n1 = ctl->group_n[L.row_group];
  if (n1 == 0 || L.rows == 0) return;
  constexpr int RPW = 32 / kFilterTpa;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int row = (gt >> 5) * RPW + (lane % RPW);
  const int sub = lane / RPW;
  const bool valid = row < n1 && row < L.rows;
  const int n = valid ? O.nnum[row] : 0;
  const int ai = valid ? O.pidx[row] : 0;
  const int4 pi = posq[ai];
  int nw = n;  // every lane of the warp runs the same number of rounds
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nw = max(nw, __shfl_xor_sync(0xffffffffu, nw, o));
  unsigned rowmask = 0u;
#pragma unroll
  for (int k = 0; k < kFilterTpa; ++k) rowmask |= 1u << (lane % RPW + k * RPW);
  const unsigned below = rowmask & ((1u << lane) - 1u);
  int cnt = 0;
  int ajn = sub < n ? O.nlist[(size_t)sub * O.stride + row] : ai;
  for (int base = 0; base < nw; base += kFilterTpa) {
    const int p = base + sub;
    bool hit = false;
    const int aj = ajn;
    const int pn = p + kFilterTpa;
    ajn = pn < n ? O.nlist[(size_t)pn * O.stride + row] : ai;
    if (p < n) {
      float d[3];
      hit = mi_q(pi, posq[aj], B, d) < rcp2;
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (hit) {
      const int q = cnt + __popc(m & below);
      if (q < L.nmax) L.nlist[(size_t)q * L.stride + row] = aj;
    }
    cnt += __popc(m & rowmask);
  }
  if (valid && sub == 0) {
    if (cnt > L.nmax) {
      // 'error: too many neighbours', ind, nnumind  (md_neighbours.f90:80)
      set_error(ctl, ST_NLIST_OVERFLOW, EK_OVERFLOW, L.id, row + 1, L.nmax + 1);
    } else {
      L.nnum[row] = cnt;
      L.pidx[row] = ai;
      L.bnd[row] = INT_MAX;  // lessnnum of an unsorted row is formed when it is read back
    }
  }
}

void launch_filter_outer(const ListDev& L, const ListDev& O, const Atoms& A, const Box& B, double rc, Ctl* ctl,
                         cudaStream_t s) {
  if (L.rows == 0) return;
  const long long threads = (long long)L.rows * kFilterTpa;
  k_filter_outer<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(L, O, A.posq, B, (float)(rc * rc), ctl);
  ++g_kernel_launches;
}

void launch_bin(const ListDev& L, const CellGrid& cg, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  cudaMemsetAsync(cg.count, 0, sizeof(int) * (size_t)cg.ncell, s);
  if (L.col_cap > 0) { k_bin_count<<<blocks_for(L.col_cap, 256), 256, 0, s>>>(L, cg, A, ctl); ++g_kernel_launches; }
  { k_bin_scan<<<1, 1024, 0, s>>>(cg, L.skin, ctl); ++g_kernel_launches; }
  if (L.col_cap > 0) { k_bin_scatter<<<blocks_for(L.col_cap, 256), 256, 0, s>>>(L, cg, A, ctl); ++g_kernel_launches; }
}

template <bool PREC, bool SORT>
static void build_dispatch(const ListDev& L, const CellGrid& cg, const Atoms& A, const Box& B, double rc2,
                           float rcp2, int converse, int src_rows, Ctl* ctl, cudaStream_t s) {
  const int grid = blocks_for(L.rows, kBuildWarps);
  const int bs = kBuildWarps * 32;
  if (grid == 0) return;
  if (L.nmax <= 64)
    k_build<PREC, 64, SORT><<<grid, bs, 0, s>>>(L, cg, A, B, rc2, rcp2, converse, src_rows, ctl);
  else if (L.nmax <= 128)
    k_build<PREC, 128, SORT><<<grid, bs, 0, s>>>(L, cg, A, B, rc2, rcp2, converse, src_rows, ctl);
  else if (L.nmax <= 256)
    k_build<PREC, 256, SORT><<<grid, bs, 0, s>>>(L, cg, A, B, rc2, rcp2, converse, src_rows, ctl);
  else if (L.nmax <= 512)
    k_build<PREC, 512, SORT><<<grid, bs, 0, s>>>(L, cg, A, B, rc2, rcp2, converse, src_rows, ctl);
  else
    k_build<PREC, 1024, SORT><<<grid, bs, 0, s>>>(L, cg, A, B, rc2, rcp2, converse, src_rows, ctl);
  ++g_kernel_launches;
}

void launch_build_list(bool prec, const ListDev& L, const CellGrid& cg, const Atoms& A, const Box& B, double rc,
                       double prefilter_margin, int converse, int src_rows, Ctl* ctl, cudaStream_t s) {
  const double rc2 = rc * rc;
  if (!L.sorted) {
    { k_cell_sort<<<blocks_for((long long)cg.ncell * 32, 256), 256, 0, s>>>(cg, L.skin, ctl); ++g_kernel_launches; }
  }
  if (prec) {
    if (L.sorted)
      build_dispatch<true, true>(L, cg, A, B, rc2, (float)rc2, converse, src_rows, ctl, s);
    else if (!converse && L.row_group == L.col_group && cg.ncell > 0)
      { k_build_cells<<<(cg.ncell + kCellWarps - 1) / kCellWarps, kCellWarps * 32, 0, s>>>(L, cg, B, (float)rc2, ctl); ++g_kernel_launches; }
    else
      build_dispatch<true, false>(L, cg, A, B, rc2, (float)rc2, converse, src_rows, ctl, s);
  } else {
    const double rp = rc + prefilter_margin;
    if (L.sorted)
      build_dispatch<false, true>(L, cg, A, B, rc2, (float)(rp * rp), converse, src_rows, ctl, s);
    else
      build_dispatch<false, false>(L, cg, A, B, rc2, (float)(rp * rp), converse, src_rows, ctl, s);
  }
}

void launch_nn_select(bool prec, const ListDev& tb, const ListDev& nn, double rc_nn, const Atoms& A,
                      const Box& B, Ctl* ctl, cudaStream_t s) {
  if (tb.rows == 0) return;
  if (prec)
    { k_nn_select<true><<<blocks_for(tb.rows, 128), 128, 0, s>>>(tb, nn, rc_nn, A, B, ctl); ++g_kernel_launches; }
  else
    { k_nn_select<false><<<blocks_for(tb.rows, 128), 128, 0, s>>>(tb, nn, rc_nn, A, B, ctl); ++g_kernel_launches; }
}

void launch_normals(bool prec, const ListDev& nn, double4_32a* norm, int simplified, const Atoms& A, const Box& B,
                    Ctl* ctl, cudaStream_t s) {
  if (nn.rows == 0) return;
  if (prec)
    { k_normals<true><<<blocks_for(nn.rows, 128), 128, 0, s>>>(nn, norm, simplified, A, B, ctl); ++g_kernel_launches; }
  else
    { k_normals<false><<<blocks_for(nn.rows, 128), 128, 0, s>>>(nn, norm, simplified, A, B, ctl); ++g_kernel_launches; }
}

void launch_nnum_max(const ListDev& L, Ctl* ctl, cudaStream_t s) {
  if (L.rows == 0) return;
  int g = blocks_for(L.rows, 256);
  if (g > 256) g = 256;
  { k_nnum_max<<<g, 256, 0, s>>>(L, ctl); ++g_kernel_launches; }
}

}  // namespace pfmd

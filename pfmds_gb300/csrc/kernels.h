// Launch interface between the host engine and the CUDA kernels.
//
// Layouts in HBM:
//   atoms      double4_32a pos/vel/frc [N] (w unused), double mass [N],
//              int4 posq [N]: fixed-point box fractions (x*2^32/L mod 2^32) used
//              by the precision form's forces, the list-build prefilter and the
//              cell binning
//   groups     int idx[cap] (0-based atom indexes); current sizes live in
//              Ctl::group_n so captured graphs survive change_particle_group_N
//   lists      slot-major: nlist[slot*stride + row] (stride = rows rounded up to
//              32), a row's entries in the reference's order (ascending group-2
//              index).  Main lists store the partner's atom index; the graphene
//              nearest-neighbour list stores tb row indexes.  Consecutive rows sit
//              on consecutive lanes, so a warp reading one slot of its rows is
//              coalesced, and in an ordered crystal slot p of neighbouring rows
//              points at neighbouring atoms (a near-coalesced position gather).
//              nnum/pidx/lessnnum/bnd [rows]; row_of[N]: row of an atom (-1 if
//              none) for lists whose kernels address the partner's row
//   cells      per list: cell_start[ncell+1]; cell-ordered jnd/atom/posq copies of
//              the column group [cap2]; cell_of[cap2]; cell_count/cursor[ncell]
#pragma once

#include <cuda_runtime.h>

#include "dev.cuh"

namespace pfmd {

// Kernels launched by this library (incremented by every launcher, also while a
// stream is being captured into a graph).
extern thread_local long long g_kernel_launches;  // launches made by this host thread

// Bounded device waits (the batched kernel's grid barrier, the tensor-core
// kernels' mbarrier waits) read these at launch time.  spin_limit != 0 replaces
// their built-in poll limits; stall != 0 makes the waits impossible (the grid
// barrier expects one arrival more than the grid has, the tensor-core kernels
// wait for an mbarrier phase that no MMA completes), so that tests can make
// them run out.  Set by pfmd_debug_waits.
struct WaitHook {
  unsigned int spin_limit = 0;
  int stall = 0;
};
extern WaitHook g_wait_hook;

struct Atoms {
  int N;
  double4_32a* pos;
  double4_32a* vel;
  double4_32a* frc;
  double* mass;
  int4* posq;
  double* kc;  // 1/(m*mass_coef) per atom: the precision form's kick factor
};

struct ListDev {
  int id;            // index into Ctl::maxnnum
  int rows;          // nl%N
  int nmax, stride;  // nlist[slot*stride + row]
  int tpa;           // threads per row in the force kernels (1..32, power of two)
  int tpa1;          // threads per row of the rjl density pass (no force write-back: it
                     // runs best with more, shorter threads)
  int sorted;        // rows kept in the reference's order (ascending group-2 index)
  int* nnum;
  int* nlist;
  int* pidx;
  int* lessnnum;
  int* bnd;          // first group-2 index whose atom index exceeds the row's atom
  const int* row_idx;  // row group indexes (particle_index source)
  const int* col_idx;  // column group indexes
  const int* row_of;   // atom -> row (g1 == g2 lists that need it), else null
  int row_group, col_group;  // 0-based group numbers (sizes in Ctl::group_n)
  int row_cap, col_cap;
  int skin;  // index into Ctl::list_need when its rebuilds are skin-triggered, else -1
};

struct CellGrid {
  int nc[3];
  int ncell;
  int* start;   // [ncell+1]
  int* count;   // [ncell]
  int* cursor;  // [ncell]
  int* jnd;     // [col_cap] group-2 index, cell order
  int* atom;    // [col_cap] atom index, cell order
  int4* posq;   // [col_cap] fixed-point position, cell order
  int* cell_of; // [col_cap]
};

struct GroupRef {
  const int* idx;
  int g;    // 0-based group number
  int cap;  // capacity (launch size)
};

// Potential parameters.  Every constant a kernel needs is derived on the host
// (both precisions), so no thread spends FP64 divides on parameter algebra.
template <class R>
struct LJc {
  R eps4, sig, R1, R2, inv_w;     // lj (cosine switch)
  R c6, c12, c6t6, c12t12;        // lj1g (LennardJones_1g.f90:21-24)
};
struct LJPar {
  double eps, sig, R1, R2, c6, c12, c6t6, c12t12;
  LJc<double> d;
  LJc<float> f;
};
template <class R>
struct Cosc {
  R sig, delt, a, r0, R1, R2, inv_w;
  R pref;     // 4 eps (ljc) or D (morsec)
  int idelt;  // 2 when delta is exactly 2 (the cosine power then runs as products), else 0
};
struct CosPar {  // ljc: eps sig delt; morsec: D r0 a delt
  double eps, sig, delt, D, r0, a, R1, R2;
  int simplified;
  Cosc<double> d;
  Cosc<float> f;
};
template <class R>
struct RJLc {
  R A0, xi, R1, R2, inv_w, inv_r0, m2q, mp, a2, pr0, qr0;
  // the two exponents in base 2 as linear functions of r: -2q (r/r0 - 1) log2(e)
  // = eqa r + eqb, and -p (r/r0 - 1) log2(e) = epa r + epb
  R eqa, eqb, epa, epb;
  // the switch argument t = (r - R1)/(R2 - R1) = r inv_w + tb; dsw = -pi/2 inv_w
  R tb, dsw;
};
struct RJLPar {
  double A0, xi, p, q, r0, R1, R2;
  RJLc<double> d;
  RJLc<float> f;
};
template <class R>
struct TBc {
  R d, s, b, r0, delt, a0, c02, d02, R1, R2, inv_w, ex, sq2s, sq2os, pre_e, c02d02;
  R is;  // 1/s
};
struct TBPar {
  double d, s, b, r0, delt, a0, c0, d0, R1, R2, c02, d02;
  TBc<double> dd;
  TBc<float> f;
};
// rebosc, REBOsolidcarbon.f90:7-9: A Q alpha / B(3) / beta(3) / T / g(6) / R1 R2.
struct REBOPar {
  double A, Q, alpha, B[3], beta[3], T, g[6], R1, R2;
};
// Fill the derived constants of a parameter set.
void derive(LJPar& P);
void derive(CosPar& P, bool morse);
void derive(RJLPar& P);
void derive(TBPar& P);

struct ChangeSpec {
  int from, to;  // 0-based groups
  long long ts1, ts2, frec;
  int to_cap;
};

enum Integ { I_NVE = 0, I_NVT = 1, I_NVMS = 2 };

// How a force kernel finishes an atom's force.  store: the kernel is the first
// and only writer of every atom of the all-atoms group, so it stores instead of
// adding (zero_forces is skipped).  kick: it is the last writer of every moving
// atom, so it also applies the second half-kick (v += f/m/mass_coef*dt/2 for the
// xyz group, z only for the z group; flags bit 0 / bit 1).
struct Epi {
  int store, kick, exact;
  double ts2;
  const unsigned char* mflag;
  double* eatom;  // energy steps: per-atom energy of the interaction (rjl: the row energy;
                  // tb: half of every bond), or null
  // drift (precision rjl force kernel, nve): after the second half-kick also the
  // next step's first half-kick and drift of the row's atom, its fixed-point
  // position into posq_next (the buffer the next step reads)
  int drift = 0;
  double ts1 = 0.0;
  int4* posq_next = nullptr;
  // begin (rjl density pass): its first thread also opens the step (the step
  // counter and the previous potential energy, as k_step_begin_fused), for a step
  // whose kick and drift ran in the previous force kernel and that launches
  // nothing before the density pass
  int begin = 0;
};

// ---------------- neighbour lists (nlist.cu) ----------------
void launch_pack_posq(const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s);
void launch_bin(const ListDev& L, const CellGrid& cg, const Atoms& A, Ctl* ctl, cudaStream_t s);
// Skin-triggered rebuilds (L.skin >= 0): the displacement test before a list's
// update step and the reference update after it.
// xout (or null): the positions at the outer list's build, for a two-level list.
void launch_skin_check(const ListDev& L, const Atoms& A, const Box& B, const int4* xref, int4* xprev,
                       const int4* xout, double half_skin, double half_margin, Ctl* ctl, cudaStream_t s);
void launch_skin_commit(const ListDev& L, const Atoms& A, int4* xref, int4* xout, Ctl* ctl, cudaStream_t s);
// A two-level list's rows from its outer list O: the entries within rc.
void launch_filter_outer(const ListDev& L, const ListDev& O, const Atoms& A, const Box& B, double rc, Ctl* ctl,
                         cudaStream_t s);
// Regular list (converse=0), or the converse of a list with src_rows rows
// (converse=1, built at the source list's rebuild steps).  The plain form tests
// candidates with an FP32 prefilter at r_cut + prefilter_margin, then exactly.
void launch_build_list(bool prec, const ListDev& L, const CellGrid& cg, const Atoms& A, const Box& B, double rc,
                       double prefilter_margin, int converse, int src_rows, Ctl* ctl, cudaStream_t s);
// graphene nearest neighbours picked from a tb list (graphenenorm.f90:8-36)
void launch_nn_select(bool prec, const ListDev& tb, const ListDev& nn, double rc_nn, const Atoms& A,
                      const Box& B, Ctl* ctl, cudaStream_t s);
// graphene normals (graphenenorm.f90:38-56); norm is double4_32a[rows]
void launch_normals(bool prec, const ListDev& nn, double4_32a* norm, int simplified, const Atoms& A,
                    const Box& B, Ctl* ctl, cudaStream_t s);
void launch_nnum_max(const ListDev& L, Ctl* ctl, cudaStream_t s);

// ---------------- forces and energies (forces.cu) ----------------
void launch_lj(bool prec, bool energy, const ListDev& L, const LJPar& P, const Atoms& A, const Box& B,
               Ctl* ctl, int eslot, int ekey, cudaStream_t s, const Epi& E = Epi{0, 0, 0, 0.0, nullptr});
void launch_lj1g(bool prec, bool energy, bool general, const ListDev& L, const LJPar& P, const Atoms& A,
                 const Box& B, Ctl* ctl, int eslot, int ekey, cudaStream_t s,
                 const Epi& E = Epi{0, 0, 0, 0.0, nullptr});
// All lj and lj1g lists of a system in one launch (k_pair_atoms): TPA threads
// own an atom and gather over every list row the atom heads -- its tasks, as
// (slot, row) pairs in slot order -- so each atom's force is formed in one
// place and stored (no zero_forces), kicked (Epi::kick) and, for a
// Nose-Hoover chain (mflag bit 4 marks its group), the chain's kinetic energy
// is reduced and the chain updated by the last block.
// The fields of one list that the pair row loops read.
struct RowList {
  const int* nnum;
  const int* nlist;
  const int* lessnnum;
  const int* bnd;
  const int* row_of;
  int stride, sorted;
};
struct PairSlot {  // device memory, one per list
  RowList L;
  LJPar P;
  int kind;     // 0: lj, 1: lj1g
  int general;  // lj1g rows with half-list weights (group not in atom order)
  int ekey;     // index into PairSet::keys of the energy this list adds to, or -1
};
constexpr int kMaxPairSlots = 6, kMaxPairKeys = 4;
struct PairSet {
  int nslot, nkey, natoms, tpa;
  const PairSlot* slots;   // nslot, device memory
  int keys[kMaxPairKeys];  // e_inter indexes
  const int* task_off;     // natoms + 1
  const int2* task;        // (slot, row)
};
// chain >= 0: the chain's kinetic energy is reduced and its second half-update
// run by the last block; with ahead, also the next step's first half-update
// (Ctl::nhc_sa keeps the second half's scale for the next kick-drift).
void launch_pair_atoms(bool prec, bool energy, const PairSet& S, const Atoms& A, const Box& B, Ctl* ctl,
                       cudaStream_t s, const Epi& E, int chain, double ts2, double ts3, double ts4, bool ahead = false);

// Multi-kernel interactions take `parts`, a bit mask of their kernels (all by
// default; single kernels are launched alone only for timing).
// inv_eb: 1/Eb per atom (double[N] plain, float[N] precision); pair: the plain
// form's per-slot force coefficients (double2[nmax*stride]) written by the density
// pass.  parts: 1 density, 2 force
void launch_rjl(bool prec, bool energy, const ListDev& L, const RJLPar& P, const Atoms& A, const Box& B,
                void* inv_eb, double2* pair, Ctl* ctl, int eslot, int ekey, cudaStream_t s, int parts = 3,
                const Epi& E = Epi{0, 0, 0, 0.0, nullptr});
// parts: 1 bond orders, 2 force
void launch_tb(bool prec, bool energy, const ListDev& L, const TBPar& P, const Atoms& A, const Box& B,
               double* Bbuf, Ctl* ctl, int eslot, int ekey, cudaStream_t s, int parts = 3,
               const Epi& E = Epi{0, 0, 0, 0.0, nullptr});
// rebosc (FP64 in both forms).  S3: 3 x nmax x stride doubles (per slot bsp,
// dbsp/dS, bdh).  parts: 1 bond terms, 2 force
void launch_rebo(bool energy, const ListDev& L, const REBOPar& P, const Atoms& A, const Box& B, double* S3, Ctl* ctl,
                 int eslot, int ekey, cudaStream_t s, int parts = 3, const Epi& E = Epi{0, 0, 0, 0.0, nullptr});
// parts: 1 graphene side, 2 metal side
// gsum: one record per graphene row (the per-row sums the normal-derivative
// term reads), unused when P.simplified
void launch_cos(bool prec, bool energy, bool morse, const ListDev& nl1, const ListDev& nl2, const ListDev& nn,
                const CosPar& P, const double4_32a* norm, double4_32a* gsum, const Atoms& A, const Box& B, Ctl* ctl,
                int eslot, int ekey, cudaStream_t s, int parts = 3);

// ---------------- state transfer (integrate.cu) ----------------
// xyz-interleaved doubles (the reference's (3,N) arrays, as the host passes them)
// to / from the device's 32-byte atom records, on the device.
// xyz-interleaved <-> double4 records, up to three arrays in one launch (null
// entries skipped)
// positions and velocities (either may be null) from xyz-interleaved doubles into
// the records, positions also into the fixed-point records
void launch_state_in(int n, const double* pos, const double* vel, const Atoms& A, const Box& B, cudaStream_t s);
void launch_d4_to_xyz(int n, const double4_32a* const d4[3], double* const xyz[3], cudaStream_t s);

// ---------------- integration and reductions (integrate.cu) ----------------
// phase: 0 = group changes + out-of-cell check, 1 = nvms exit test, 2 = both
void launch_step_begin(int phase, int n_changes, const ChangeSpec* changes, int nvms, double ms_de,
                       Ctl* ctl, cudaStream_t s);
void launch_check_all(const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s);
void launch_invert_z(const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s);
// exact: the reference's f/m/mass_coef*dt/2 with round-to-nearest divides (plain form);
// otherwise f*kc*dt/2 (precision form)
void launch_kick(const GroupRef& g, bool xyz, double ts2, bool exact, const Atoms& A, Ctl* ctl, cudaStream_t s);
void launch_drift(const GroupRef& g, bool xyz, double ts1, bool write_posq, const Atoms& A, const Box& B,
                  Ctl* ctl, cudaStream_t s);
// The step-begin bookkeeping of a step whose kick and drift ran in the previous
// step's force kernel: the step counter and the previous potential energy.
void launch_step_begin_fused(Ctl* ctl, cudaStream_t s);
// nhc_scale = chain + 1 scales the velocities by that chain's s first (nhc_pre:
// by Ctl::nhc_sa, then s); begin opens the step (counter, previous energy).
void launch_kick_drift(const GroupRef& g, double ts1, double ts2, bool write_posq, int nhc_scale, bool exact,
                       const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s, bool begin = false,
                       bool nhc_pre = false, bool early = false);
void launch_nhc(int chain, const GroupRef& g, double ts2, double ts3, double ts4, const Atoms& A, Ctl* ctl,
                cudaStream_t s, int prescale = 0, int ahead = 0);
// the xyz-moving group's second half-kick with the half-update of the chain over
// the same group (ahead: and the next step's first half, as launch_nhc)
void launch_kick_nhc(const GroupRef& g, double kts2, bool exact, int chain, double ts2, double ts3, double ts4,
                     bool ahead, const Atoms& A, Ctl* ctl, cudaStream_t s);
void launch_scale(int chain, const GroupRef& g, const Atoms& A, Ctl* ctl, cudaStream_t s);
void launch_ms(const GroupRef& g, bool xyz, const Atoms& A, Ctl* ctl, cudaStream_t s);
void launch_zero_forces(const GroupRef& g, const Atoms& A, Ctl* ctl, cudaStream_t s);
void launch_zero_momentum(const GroupRef& g, const Atoms& A, Ctl* ctl, cudaStream_t s);
// energies at log/out/nvms steps: KE and temperature of the all-moving group,
// Nose-Hoover energies (when nvt), potential/total/conserved sums
// One log record's values (the log line of md_simulation.f90:204-207) copied
// from the control block into row: conserved, chain energy, total, potential,
// kinetic, temperature, the interactions' energies (kLogInter), the chains'
// energies (kLogChains).  Log steps inside a segment write rows that the host
// turns into log lines at the segment's end.
constexpr int kLogInter = PFMD_MAX_INTER, kLogChains = PFMD_MAX_NHC, kLogCols = 6 + kLogInter + kLogChains;
void launch_log_row(const Ctl* ctl, double* row, cudaStream_t s);
void launch_energy_finalize(const GroupRef& moving, int n_inter, int n_nhc, int nvt, const Atoms& A,
                            Ctl* ctl, cudaStream_t s);
// output-block sums: force sum, mass-weighted position and velocity sums and the
// mass of the all-atoms group; largest |v|^2 over every atom (red[0..8])
void launch_out_reduce(const GroupRef& all, const Atoms& A, Ctl* ctl, cudaStream_t s);

}  // namespace pfmd

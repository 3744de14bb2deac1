// CPU oracle for the PFMDS MD hot path -- TEST INFRASTRUCTURE ONLY.
//
// FP64 restatement of run_md_simulation -> md() of PFMDS (Fortran 90 + OpenMP),
// routine by routine, each function citing the reference file:line it follows.
// It keeps the reference's algorithms, including the O(N1*N2) neighbour search and
// the quirks listed in the comments, and it is built with -ffp-contract=off so the
// neighbour-list predicate evaluates exactly as written.
//
// PARITY UNPINNED: no Fortran compiler exists on either machine and the reference
// has no tests or fixtures, so this restatement cannot be run against the reference
// itself.  It is checked against physics invariants and hand-derived known answers.
//
// Only tests, the smoke entry point and the benchmark's CPU baseline use it.

#include "oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../pfmds_gb300/csrc/settings.h"

namespace orc {

using pfmd_io::InteractionSpec;
using pfmd_io::Settings;

enum {
  E_OK = 0,
  E_NLIST_OVERFLOW = 1,
  E_OUT_OF_CELL = 2,
  E_GR_NN = 3,
  E_PARAM = 4,
  E_CUDA = 5,
  E_TIMEOUT = 6,
  E_IO = 7
};

struct Stop : std::runtime_error {
  int code;
  Stop(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Constants exactly as the reference folds them (left to right, FP64).
static const double MASS_COEF = 1.6605389217 / 1.6021765654 * 100.0;   // md_integrators.f90:62
static const double KT_A_DEGREE = 1.3806488 / 1.6021765654 * 1e-4;     // md_general.f90:304
static const double MOMENTA_COEF = 1.3806488 / 1.6605389217 * 1e-6;    // md_general.f90:144
static const double PI_TRUNC = 3.14159265358979;                        // cut_off_function.f90:8

// ---------------------------------------------------------------------------
// Types, md_general.f90:5-41
// ---------------------------------------------------------------------------
struct Cell {
  double box[3], half[3];
};
struct Particles {
  int N = 0;
  std::vector<double> pos, vel, mass, frc;  // (3,N) column-major == xyz interleaved
  std::vector<std::string> types;
};
struct Group {
  int N = 0;
  std::vector<int> idx;  // 0-based atom indexes; size() == size(indexes)
};
struct NL {
  int N = 0, nmax = 0;
  long long period = 1;
  double rc = 0.0;
  std::vector<int> nlist, nnum, lessnnum, pidx;  // nlist[i*nmax+p]: 0-based group-2 index
  std::vector<double> dr, moddr;                 // dr[(i*nmax+p)*3+k]
  int& L(int p, int i) { return nlist[static_cast<size_t>(i) * nmax + p]; }
  int L(int p, int i) const { return nlist[static_cast<size_t>(i) * nmax + p]; }
  double* D(int p, int i) { return &dr[(static_cast<size_t>(i) * nmax + p) * 3]; }
  const double* D(int p, int i) const { return &dr[(static_cast<size_t>(i) * nmax + p) * 3]; }
  double& R(int p, int i) { return moddr[static_cast<size_t>(i) * nmax + p]; }
  double R(int p, int i) const { return moddr[static_cast<size_t>(i) * nmax + p]; }
};
struct NHC {
  int M = 0, L = 0, group_num = 0;
  std::vector<double> x, v, q;
  double temperature = 0, s = 1, e = 0;
};
struct TimeSteps {
  double ts[4] = {0, 0, 0, 0};
  double simulation_time = 0;
};
struct Integrator {
  std::string name;
  double dt = 0;
  long long l = 0, period_snapshot = 1, period_log = 1;
};
struct Interaction {
  InteractionSpec spec;
  int nl_n = 0;
  std::vector<int> group_nums;  // 1-based, 2*nl_n
  std::vector<NL> nl;
  double energy = 0;
  std::vector<double> gr_norm;  // ljc / morsec: (3, nl(3)%N)
  // lj1g derived constants, LennardJones_1g.f90:21-24
  double c6 = 0, c12 = 0, c6t6 = 0, c12t12 = 0;
  // tb derived constants, TersoffBrenner.f90:22-23
  double c02 = 0, d02 = 0;
};

static inline double fsign1(double x) { return std::signbit(x) ? -1.0 : 1.0; }  // sign(1.,x)
static inline double pow6(double x) {
  double x2 = x * x;
  return x2 * x2 * x2;
}

// find_distance, md_general.f90:423-441: minimum image in all three axes.
static inline void find_distance(double dr[3], double& dr2, const double* v1, const double* v2,
                                 const Cell& c) {
  dr[0] = v2[0] - v1[0];
  dr[1] = v2[1] - v1[1];
  dr[2] = v2[2] - v1[2];
  dr[0] = dr[0] - c.half[0] * (fsign1(dr[0] - c.half[0]) + fsign1(dr[0] + c.half[0]));
  dr[1] = dr[1] - c.half[1] * (fsign1(dr[1] - c.half[1]) + fsign1(dr[1] + c.half[1]));
  dr[2] = dr[2] - c.half[2] * (fsign1(dr[2] - c.half[2]) + fsign1(dr[2] + c.half[2]));
  dr2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
}

// cut_off_function.f90:6-28 (cosine switch; df_cut returns f'/r)
static inline double f_cut_cos(double r, double R1, double R2) {
  if (r < R1) return 1.0;
  if (r < R2) return (1.0 + std::cos(PI_TRUNC * (r - R1) / (R2 - R1))) / 2;
  return 0.0;
}
static inline double df_cut_cos(double r, double R1, double R2) {
  if (r < R1) return 0.0;
  if (r < R2) return -std::sin(PI_TRUNC * (r - R1) / (R2 - R1)) * PI_TRUNC / (R2 - R1) / r / 2;
  return 0.0;
}
// REBOsc_energy, REBOsolidcarbon.f90:27-92, over any list (the full one or a
// truncated one); serial, rows in order.  P: A Q alpha B(3) beta(3) T g(6) R1 R2.
static double rebosc_energy(const NL& nl, const std::vector<double>& P) {
  const double A = P[0], Q = P[1], al = P[2], T = P[9], R1 = P[16], R2 = P[17];
  const double* B = &P[3];
  const double* be = &P[6];
  const double* g = &P[10];
  const size_t M = static_cast<size_t>(nl.nmax);
  std::vector<double> bsp(M * nl.N, 0.0), bdh(M * nl.N, 0.0);
  auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  for (int i = 0; i < nl.N; ++i) {
    for (int p = 0; p < nl.nnum[i]; ++p) {
      if (!(nl.R(p, i) < R2)) continue;
      const int j = nl.L(p, i);
      double s = 0.0, h = 0.0;
      for (int q = 0; q < nl.nnum[i]; ++q) {
        if (p == q || !(nl.R(q, i) < R2)) continue;
        const double c = dot(nl.D(p, i), nl.D(q, i)) / (nl.R(p, i) * nl.R(q, i));
        s = s + f_cut_cos(nl.R(q, i), R1, R2) *
                    (g[0] + g[1] * c + g[2] * c * c + g[3] * c * c * c + g[4] * c * c * c * c + g[5] * c * c * c * c * c);
        for (int l = 0; l < nl.nnum[j]; ++l) {
          if (nl.L(l, j) == i || !(nl.R(l, j) < R2)) continue;
          const double aa = nl.R(p, i) * nl.R(p, i);
          const double ab = dot(nl.D(p, i), nl.D(q, i)), ac = dot(nl.D(p, i), nl.D(l, j));
          const double bc = dot(nl.D(q, i), nl.D(l, j));
          const double D = aa * bc - ab * ac;
          h = h + f_cut_cos(nl.R(q, i), R1, R2) * f_cut_cos(nl.R(l, j), R1, R2) *
                      (1.0 - D * D / (aa * nl.R(q, i) * nl.R(q, i) - ab * ab) /
                                 (aa * nl.R(l, j) * nl.R(l, j) - ac * ac));
        }
      }
      bsp[i * M + p] = std::pow(1.0 + s, -0.5);
      bdh[i * M + p] = T * h;
    }
  }
  double e = 0.0;
  for (int i = 0; i < nl.N; ++i) {
    for (int p = 0; p < nl.nnum[i]; ++p) {
      const double r = nl.R(p, i);
      if (!(r < R2)) continue;
      const int j = nl.L(p, i);
      if (j <= i) continue;
      int q = 0;
      for (; q < nl.nnum[j]; ++q)
        if (nl.L(q, j) == i) break;
      const double bq = q < nl.nmax ? bsp[j * M + q] : 0.0;
      e = e + f_cut_cos(r, R1, R2) *
                  ((1.0 + Q / r) * A * std::exp(-al * r) -
                   ((bsp[i * M + p] + bq) / 2 + bdh[i * M + p]) *
                       (B[0] * std::exp(-be[0] * r) + B[1] * std::exp(-be[1] * r) + B[2] * std::exp(-be[2] * r)));
    }
  }
  return e;
}

// cut_off_poly.f90:6-17 (quintic switch used by the lj1g energy)
static inline double ipow(double x, int n) {
  double r = 1.0;
  for (int k = 0; k < n; ++k) r *= x;
  return r;
}
static inline double f_cut_poly(double r, double R1, double R2) {
  if (r > R1 && r < R2)
    return 1.0 + (-10.0 * ipow(r - R1, 3) * ipow(R2 - R1, 2) + 15.0 * ipow(r - R1, 4) * (R2 - R1) -
                  6.0 * ipow(r - R1, 5)) /
                     ipow(R2 - R1, 5);
  if (r <= R1) return 1.0;
  return 0.0;
}
// cut_off_poly.f90:30-43.  Quirk kept: dfr lacks the 1/(R2-R1) factor of the
// derivative, so lj1g forces equal -dE/dr only when R2-R1 = 1.
static inline void f_dfr_cut(double& f, double& dfr, double r, double R1, double R2) {
  double tempr = r;
  tempr = std::max(tempr, R1);
  tempr = std::min(tempr, R2);
  double x = (tempr - R1) / (R2 - R1);
  double x2 = x * x;
  f = 1.0 + x2 * x * (-10.0 + 15.0 * x - 6.0 * x2);
  dfr = tempr * x2 * (-30.0 + 60.0 * x - 30.0 * x2);
}

// ---------------------------------------------------------------------------
// The simulation object: md() state plus the loop body.
// ---------------------------------------------------------------------------
class Sim {
 public:
  Settings S;
  Cell cell;
  TimeSteps dt;
  Particles atoms;
  std::vector<Group> groups;
  std::vector<Interaction> inters;
  std::vector<Integrator> integrators;  // index 0 is 'none'
  std::vector<NHC> nhc;
  std::vector<int> change_from, change_to;
  std::vector<long long> change_ts1, change_ts2, change_frec;

  std::string input_path, settings_filename, output_prefix;
  int out_period = 1, num_threads = 1, rand_seed = 1;
  bool write_files = true;
  std::string out;  // output unit text
  FILE* out_file = nullptr;
  FILE* all_out_file = nullptr;  // same as out when null
  std::string logname;
  std::FILE* log = nullptr;

  long long md_step = 0;
  int integrator_index = 0;
  std::string integrator_name;
  double potential_energy = 0, prev_potential_energy = 0, kinetic_energy = 0, temperature = 0,
         total_energy = 0, conserved_energy = 0, nose_hoover_energy = 0;
  double exe_time_start = 0, exe_time_md = 0, exe_time_pos_vel = 0, exe_time_nlists = 0,
         exe_time_nlsearch = 0, exe_time_nldistance = 0, exe_time_forces = 0, exe_time_energy = 0;
  bool finished = false;
  std::string errmsg;

  ~Sim() {
    if (log) std::fclose(log);
  }

  void emit(const std::string& s) {
    if (out_file) {
      std::fputs(s.c_str(), out_file);
    } else {
      out += s;
    }
  }
  void line(const std::string& s) { emit(s + "\n"); }
  void all_emit(const std::string& s) {
    if (all_out_file)
      std::fputs(s.c_str(), all_out_file);
    else
      emit(s);
  }

  // ---------------- md_general.f90 ----------------
  void init_time_steps(double delta_t) {  // :45-55
    for (int i = 0; i < 4; ++i) dt.ts[i] = delta_t / static_cast<double>(1 << i);
  }
  void create_particle_group(Group& g, const std::vector<std::string>& names) {  // :57-80
    g.N = 0;
    for (const auto& nm : names)
      for (int i = 0; i < atoms.N; ++i)
        if (atoms.types[i] == nm) ++g.N;
    g.idx.clear();
    for (const auto& nm : names)
      for (int i = 0; i < atoms.N; ++i)
        if (atoms.types[i] == nm) g.idx.push_back(i);
  }
  void change_particle_group_N(Group& g, long long step, long long ts1, long long ts2,
                               long long frec, const Group& init) {  // :82-95
    if (step <= ts1) {
      g.N = init.N;
      if (step == ts1) g.N = g.N + 1;
    } else {
      if (step < ts2 && (step - ts1) % frec == 0) g.N = g.N + 1;
    }
    if (g.N > static_cast<int>(g.idx.size())) g.N = static_cast<int>(g.idx.size());
  }
  void scale_velocities(const Group& g, double s) {  // :97-112
#pragma omp parallel for schedule(static)
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      for (int k = 0; k < 3; ++k) atoms.vel[3 * i + k] = atoms.vel[3 * i + k] * s;
    }
  }
  // Reductions below sum per-thread partials in thread order (the reference adds
  // them with OMP ATOMIC in arrival order).
  template <class F>
  double reduce_group(const Group& g, F f) const {
    int nt = omp_get_max_threads();
    std::vector<double> part(static_cast<size_t>(nt), 0.0);
#pragma omp parallel
    {
      int t = omp_get_thread_num();
      double acc = 0.0;
#pragma omp for schedule(static)
      for (int ind = 0; ind < g.N; ++ind) acc = acc + f(g.idx[ind]);
      part[t] = acc;
    }
    double s = 0.0;
    for (double v : part) s = s + v;
    return s;
  }
  double calculate_kinetic_energy(const Group& g) const {  // :161-180
    return reduce_group(g, [&](int i) {
      const double* v = &atoms.vel[3 * i];
      return atoms.mass[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / 2 * MASS_COEF;
    });
  }
  double calculate_masses_sum(const Group& g) const {  // :254-273
    return reduce_group(g, [&](int i) { return atoms.mass[i]; });
  }
  void weighted_sum(const Group& g, const std::vector<double>& a, bool by_mass, double r[3]) const {
    for (int k = 0; k < 3; ++k)
      r[k] = reduce_group(g, [&](int i) { return (by_mass ? atoms.mass[i] : 1.0) * a[3 * i + k]; });
  }
  void calculate_mass_center(double mc[3], const Group& g) const {  // :183-207
    weighted_sum(g, atoms.pos, true, mc);
    double totm = calculate_masses_sum(g);
    for (int k = 0; k < 3; ++k) mc[k] = mc[k] / totm;
  }
  void calculate_mass_center_velocity(double mcv[3], const Group& g) const {  // :210-233
    weighted_sum(g, atoms.vel, true, mcv);
    double totm = calculate_masses_sum(g);
    for (int k = 0; k < 3; ++k) mcv[k] = mcv[k] / totm;
  }
  void zero_momentum(const Group& g) {  // :236-252
    double mcv[3];
    calculate_mass_center_velocity(mcv, g);
#pragma omp parallel for schedule(static)
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      for (int k = 0; k < 3; ++k) atoms.vel[3 * i + k] = atoms.vel[3 * i + k] - mcv[k];
    }
  }
  void calculate_force_sum(double fs[3], const Group& g) const {  // :277-298
    weighted_sum(g, atoms.frc, false, fs);
  }
  void calculate_temperature(double& temp, double& ke, const Group& g) const {  // :301-310
    ke = calculate_kinetic_energy(g);
    temp = 2 * ke / KT_A_DEGREE / static_cast<double>(3 * g.N);
  }
  // random_velocities / random_momenta / set_new_temperature, :114-159 and :328-340.
  // The per-thread srand/rand stream of the reference is replaced by one serial
  // minimal-standard stream in atom order (see pfmd_io::MinStd).
  void set_new_temperature(const Group& g, double temp, int seed) {
    pfmd_io::MinStd rng(seed);
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      for (int k = 0; k < 3; ++k) {
        double a1 = 0, a2 = 0, b = 2.0;
        while (b >= 1.0) {
          a1 = 2.0 * rng.next() - 1.0;
          a2 = 2.0 * rng.next() - 1.0;
          b = a1 * a1 + a2 * a2;
        }
        atoms.vel[3 * i + k] = a1 * std::sqrt(-2.0 * std::log(b) / b);
      }
    }
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      for (int k = 0; k < 3; ++k)
        atoms.vel[3 * i + k] = atoms.vel[3 * i + k] * std::sqrt(MOMENTA_COEF / atoms.mass[i]);
    }
    zero_momentum(g);
    double t, ke;
    calculate_temperature(t, ke, g);
    scale_velocities(g, std::sqrt(temp / t));
  }
  void check_positions() {  // :342-364
    const double tolerance = 0.0000001;
    std::vector<std::string> msgs;
    for (int i = 0; i < atoms.N; ++i)
      for (int k = 0; k < 3; ++k) {
        double x = atoms.pos[3 * i + k];
        if (!(x > (0.0 - tolerance) && x < (cell.box[k] + tolerance))) {
          std::string m = fortio::list_int(i + 1) + " particle out of cell " +
                          fortio::list_real(atoms.pos[3 * i]) +
                          fortio::list_real(atoms.pos[3 * i + 1]) +
                          fortio::list_real(atoms.pos[3 * i + 2]);
          msgs.push_back(m);
        }
      }
    if (!msgs.empty()) {
      for (auto& m : msgs) line(m);
      throw Stop(E_OUT_OF_CELL, "particle out of cell");
    }
  }
  double find_max_velocity() const {  // :366-380
    double maxvel2 = -1.0;
    for (int i = 0; i < atoms.N; ++i) {
      const double* v = &atoms.vel[3 * i];
      double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      if (maxvel2 < v2) maxvel2 = v2;
    }
    return std::sqrt(maxvel2);
  }
  void invert_z_velocities(double lo, double hi) {  // :382-398
#pragma omp parallel for schedule(static)
    for (int i = 0; i < atoms.N; ++i) {
      double z = atoms.pos[3 * i + 2];
      double& vz = atoms.vel[3 * i + 2];
      if ((z > lo && z < (lo + hi) / 2 && vz > 0.0) || (z < hi && z > (lo + hi) / 2 && vz < 0.0))
        vz = -vz;
    }
  }

  // ---------------- md_neighbours.f90 ----------------
  static void create_neighbour_list(NL& nl) {  // :9-28
    if (nl.N > 0) {
      size_t n = static_cast<size_t>(nl.N), m = static_cast<size_t>(std::max(nl.nmax, 0));
      nl.pidx.assign(n, -1);
      nl.nnum.assign(n, 0);
      nl.lessnnum.assign(n, 0);
      nl.nlist.assign(n * m, 0);
      nl.dr.assign(n * m * 3, 0.0);
      nl.moddr.assign(n * m, 0.0);
    }
  }
  void find_neighbours(NL& nl, const Group& g1, const Group& g2) {  // :56-100
    if (g1.N > nl.N)
      throw Stop(E_PARAM, "error: group1%N>nl%N " + std::to_string(g1.N) + " " + std::to_string(nl.N));
    int bad_ind = -1, bad_n = 0;
    const double rc2 = nl.rc * nl.rc;
#pragma omp parallel for schedule(dynamic, 16)
    for (int ind = 0; ind < g1.N; ++ind) {
      int i = g1.idx[ind];
      nl.pidx[ind] = i;
      int nnumind = 0, lessnnumind = -1;
      for (int jnd = 0; jnd < g2.N; ++jnd) {
        int j = g2.idx[jnd];
        if (i != j) {
          double dr[3], dr2;
          find_distance(dr, dr2, &atoms.pos[3 * i], &atoms.pos[3 * j], cell);
          if (dr2 < rc2) {
            if (lessnnumind == -1 && i < j) lessnnumind = nnumind;
            nnumind = nnumind + 1;
            if (nnumind > nl.nmax) {
#pragma omp critical
              {
                if (bad_ind < 0 || ind < bad_ind) {
                  bad_ind = ind;
                  bad_n = nnumind;
                }
              }
              break;
            }
            int p = nnumind - 1;
            nl.L(p, ind) = jnd;
            double* d = nl.D(p, ind);
            d[0] = dr[0];
            d[1] = dr[1];
            d[2] = dr[2];
            nl.R(p, ind) = std::sqrt(dr2);
          }
        }
      }
      nl.lessnnum[ind] = (lessnnumind == -1) ? nnumind : lessnnumind;
      nl.nnum[ind] = nnumind;
    }
    if (bad_ind >= 0)
      throw Stop(E_NLIST_OVERFLOW, "error: too many neighbours " + std::to_string(bad_ind + 1) + " " +
                                       std::to_string(bad_n));
  }
  void find_neighbour_distances(NL& nl, const Group& g1, const Group& g2) {  // :104-124
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      for (int p = 0; p < nl.nnum[i]; ++p) {
        double dr2;
        find_distance(nl.D(p, i), dr2, &atoms.pos[3 * g1.idx[i]], &atoms.pos[3 * g2.idx[nl.L(p, i)]],
                      cell);
        nl.R(p, i) = std::sqrt(dr2);
      }
    }
  }
  void converce_neighbour_list(NL& cnl, const Group& g2, const NL& nl) {  // :128-160
    if (g2.N > 0 && nl.N > 0 && cnl.N > 0) {
      if (g2.N > cnl.N)
        throw Stop(E_PARAM, "error: group2%N>cnl%N " + std::to_string(g2.N) + " " + std::to_string(cnl.N));
      for (int i = 0; i < g2.N; ++i) cnl.pidx[i] = g2.idx[i];
      for (int i = 0; i < cnl.N; ++i) cnl.nnum[i] = 0;
      for (int i = 0; i < nl.N; ++i) {  // serial, as in the reference
        for (int p = 0; p < nl.nnum[i]; ++p) {
          int j = nl.L(p, i);
          cnl.nnum[j] = cnl.nnum[j] + 1;
          if (cnl.nnum[j] > cnl.nmax)
            throw Stop(E_NLIST_OVERFLOW, "error: too many neighbours " + std::to_string(j + 1) + " " +
                                             std::to_string(cnl.nnum[j]));
          int q = cnl.nnum[j] - 1;
          cnl.L(q, j) = i;
          const double* s = nl.D(p, i);
          double* d = cnl.D(q, j);
          d[0] = -s[0];
          d[1] = -s[1];
          d[2] = -s[2];
          cnl.R(q, j) = nl.R(p, i);
        }
      }
    }
  }
  void update_neighbour_list(long long step, NL& nl, const Group& g1, const Group& g2) {  // :32-52
    if (g1.N > 0 && g2.N > 0 && nl.N > 0) {
      double t = omp_get_wtime();
      if (step % nl.period == 0) {
        find_neighbours(nl, g1, g2);
        exe_time_nlsearch += omp_get_wtime() - t;
      } else {
        find_neighbour_distances(nl, g1, g2);
        exe_time_nldistance += omp_get_wtime() - t;
      }
    }
  }

  // ---------------- graphenenorm.f90 ----------------
  void find_gr_nearest_neighbors(NL& nn, const NL& nl) {  // :8-36
    const int nnum_nn = 3;
    if (nn.nmax != nnum_nn) throw Stop(E_GR_NN, "error: nl_nn%neighb_num_max/=nnum_nn");
    if (nl.N > nn.N) throw Stop(E_GR_NN, "error: graphene nearest-neighbour list is shorter than the tb list");
    std::string err;
    int err_code = 0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      int k = 0;
      bool bad = false;
      for (int p = 0; p < nl.nnum[i] && !bad; ++p) {
        if (nl.R(p, i) < nn.rc) {
          k = k + 1;
          if (k <= nnum_nn) {
            nn.L(k - 1, i) = nl.L(p, i);
            nn.R(k - 1, i) = nl.R(p, i);
            const double* s = nl.D(p, i);
            double* d = nn.D(k - 1, i);
            d[0] = s[0];
            d[1] = s[1];
            d[2] = s[2];
          } else {
#pragma omp critical
            if (err.empty()) err = "error: too many gr nearest neibs " + std::to_string(i + 1);
            bad = true;
          }
        }
      }
      if (!bad && k != nnum_nn) {
#pragma omp critical
        if (err.empty()) err = "error: not enough gr nearest neibs " + std::to_string(i + 1);
        bad = true;
      }
      nn.nnum[i] = nnum_nn;
      (void)err_code;
    }
    if (!err.empty()) throw Stop(E_GR_NN, err);
  }
  static void find_norm_in_graphene(std::vector<double>& gr_norm, const NL& nn) {  // :38-56
    int n = static_cast<int>(gr_norm.size() / 3);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      double d12[3], d31[3];
      const double* a = nn.D(0, i);
      const double* b = nn.D(1, i);
      const double* c = nn.D(2, i);
      for (int k = 0; k < 3; ++k) {
        d12[k] = b[k] - a[k];
        d31[k] = a[k] - c[k];
      }
      double* g = &gr_norm[3 * static_cast<size_t>(i)];
      g[0] = d12[1] * d31[2] - d12[2] * d31[1];
      g[1] = d12[2] * d31[0] - d12[0] * d31[2];
      g[2] = d12[0] * d31[1] - d12[1] * d31[0];
      if (g[2] < 0.0) {
        g[0] = -g[0];
        g[1] = -g[1];
        g[2] = -g[2];
      }
      double nrm = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
      g[0] = g[0] / nrm;
      g[1] = g[1] / nrm;
      g[2] = g[2] / nrm;
    }
  }
  void update_nearest_neighbours_in_graphene(long long step, NL& nn, const NL& nl,
                                             const Group& g) {  // :58-70
    if (step % nl.period == 0)
      find_gr_nearest_neighbors(nn, nl);
    else
      find_neighbour_distances(nn, g, g);
  }

  // ---------------- md_interactions.f90 ----------------
  Group& G(int num) {
    if (num < 1 || num > static_cast<int>(groups.size()))
      throw Stop(E_PARAM, "error: group number " + std::to_string(num) + " out of range");
    return groups[static_cast<size_t>(num - 1)];
  }
  void create_interactions() {  // :59-136
    for (const auto& sp : S.interactions) {
      Interaction in;
      in.spec = sp;
      in.nl_n = sp.nl_n;
      const auto& p = sp.p;
      if (sp.kind == pfmd_io::K_LJ1G) {
        double s6 = ipow(p[1], 6), s12 = ipow(p[1], 12);
        in.c6 = 4.0 * p[0] * s6;
        in.c12 = 4.0 * p[0] * s12;
        in.c6t6 = 6.0 * 4.0 * p[0] * s6;
        in.c12t12 = 12.0 * 4.0 * p[0] * s12;
      }
      if (sp.kind == pfmd_io::K_TB) {
        in.c02 = p[6] * p[6];
        in.d02 = p[7] * p[7];
      }
      for (int j = 0; j < sp.nl_n; ++j) {
        const auto& ls = sp.nl[static_cast<size_t>(j)];
        in.group_nums.push_back(ls.g1);
        in.group_nums.push_back(ls.g2);
        NL nl;
        nl.nmax = ls.nmax;
        nl.rc = ls.r_cut;
        nl.period = ls.period;
        if (nl.period < 1) throw Stop(E_PARAM, "error: neighbour list update period must be positive");
        if (nl.nmax < 0) throw Stop(E_PARAM, "error: negative neighb_num_max");
        nl.N = G(ls.g1).N;
        G(ls.g2);
        create_neighbour_list(nl);
        in.nl.push_back(nl);
      }
      inters.push_back(std::move(in));
    }
    // allocate_graphene_norm, :180-193
    for (auto& in : inters)
      if (in.spec.kind == pfmd_io::K_LJC || in.spec.kind == pfmd_io::K_MORSEC)
        in.gr_norm.assign(3 * static_cast<size_t>(in.nl[2].N), 0.0);
  }
  void update_interactions_neighbour_lists(long long step) {  // :138-178
    for (size_t i = 0; i < inters.size(); ++i) {
      Interaction& in = inters[i];
      update_neighbour_list(step, in.nl[0], G(in.group_nums[0]), G(in.group_nums[1]));
      int k = in.spec.kind;
      if (k == pfmd_io::K_LJ || k == pfmd_io::K_LJC || k == pfmd_io::K_MORSEC)
        converce_neighbour_list(in.nl[1], G(in.group_nums[1]), in.nl[0]);
      if (k == pfmd_io::K_LJC || k == pfmd_io::K_MORSEC) {
        size_t j = 0;
        for (; j < inters.size(); ++j)
          if (inters[j].spec.kind == pfmd_io::K_TB || inters[j].spec.kind == pfmd_io::K_REBOSC) break;
        if (j < inters.size()) {
          update_nearest_neighbours_in_graphene(step, in.nl[2], inters[j].nl[0],
                                                G(inters[j].group_nums[0]));
        } else {
          update_neighbour_list(step, in.nl[2], G(in.group_nums[4]), G(in.group_nums[5]));
        }
      }
    }
    // update_norm_in_graphene, :195-208
    for (auto& in : inters)
      if (in.spec.kind == pfmd_io::K_LJC || in.spec.kind == pfmd_io::K_MORSEC)
        find_norm_in_graphene(in.gr_norm, in.nl[2]);
  }

  // ---------------- potentials: forces ----------------
  void LJ_forces(const NL& nl, const Interaction& in) {  // LennardJones.f90:48-69
    const double eps = in.spec.p[0], sig = in.spec.p[1], R1 = in.spec.p[2], R2 = in.spec.p[3];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      for (int p = 0; p < nl.nnum[i]; ++p) {
        double r = nl.R(p, i);
        if (r < R2) {
          double V = pow6(sig / r);
          double A = V * (12.0 * V - 6.0) / (r * r) * f_cut_cos(r, R1, R2) -
                     V * (V - 1.0) * df_cut_cos(r, R1, R2);
          const double* d = nl.D(p, i);
          double* f = &atoms.frc[3 * nl.pidx[i]];
          for (int k = 0; k < 3; ++k) f[k] = f[k] - 4.0 * eps * A * d[k];
        }
      }
    }
  }
  static double scalar_lj_force(double r, double R1, double R2, double c12, double c6, double c12t12,
                                double c6t6) {  // LennardJones_1g.f90:105-117
    double invr2 = 1.0 / (r * r);
    double U = invr2 * invr2 * invr2;
    double fcut, dfrcut;
    f_dfr_cut(fcut, dfrcut, r, R1, R2);
    return U * invr2 * ((c12t12 * U - c6t6) * fcut - (c12 * U - c6) * dfrcut);
  }
  void LJ1g_forces(const NL& nl, const Interaction& in) {  // LennardJones_1g.f90:54-103
    const double R1 = in.spec.p[2], R2 = in.spec.p[3];
    int nt = omp_get_max_threads();
    std::vector<std::vector<double>> priv(static_cast<size_t>(nt));
#pragma omp parallel
    {
      int t = omp_get_thread_num();
      std::vector<double>& pf = priv[t];
      pf.assign(3 * static_cast<size_t>(atoms.N), 0.0);
#pragma omp for schedule(dynamic, 16)
      for (int i = 0; i < nl.N; ++i) {
        for (int p = 0; p < nl.lessnnum[i]; ++p) {
          double F = scalar_lj_force(nl.R(p, i), R1, R2, in.c12, in.c6, in.c12t12, in.c6t6);
          const double* d = nl.D(p, i);
          double fp0 = F * d[0], fp1 = F * d[1], fp2 = F * d[2];
          int ind = nl.pidx[i];
          int jnd = nl.pidx[nl.L(p, i)];  // the list index mapped through particle_index
          pf[3 * ind] -= fp0;
          pf[3 * ind + 1] -= fp1;
          pf[3 * ind + 2] -= fp2;
          pf[3 * jnd] += fp0;
          pf[3 * jnd + 1] += fp1;
          pf[3 * jnd + 2] += fp2;
        }
      }
    }
    for (int t = 0; t < nt; ++t)
      for (size_t k = 0; k < atoms.frc.size(); ++k) atoms.frc[k] = atoms.frc[k] + priv[t][k];
  }
  static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
  // ljc (kind 0) and morsec (kind 1), graphene side: LennardJonesCosine.f90:53-110,
  // MorseCosine.f90:53-110.
  void cosine_forces_for_graphene(const NL& nl, const NL& nn, Interaction& in, bool morse) {
    if (nl.N != nn.N && nl.N != 0)
      throw Stop(E_PARAM, "error: nl%N/=nl_nn%N " + std::to_string(nl.N) + " " + std::to_string(nn.N));
    const auto& P = in.spec.p;
    int nnum_nn = 3;
    if (in.spec.simplified) {
      nnum_nn = 0;
      for (size_t k = 0; k < in.gr_norm.size(); ++k) in.gr_norm[k] = (k % 3 == 2) ? 1.0 : 0.0;
    }
    const double R1 = morse ? P[4] : P[3], R2 = morse ? P[5] : P[4];
    const double delt = morse ? P[3] : P[2];
    const std::vector<double>& gn = in.gr_norm;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      for (int p = 0; p < nl.nnum[i]; ++p) {
        double r = nl.R(p, i);
        if (r < R2) {
          const double* d = nl.D(p, i);
          const double* n = &gn[3 * static_cast<size_t>(i)];
          double nd = dot3(n, d);
          double fc = f_cut_cos(r, R1, R2), dfc = df_cut_cos(r, R1, R2);
          double* f = &atoms.frc[3 * nl.pidx[i]];
          if (!morse) {
            const double eps = P[0], sig = P[1];
            double V2 = pow6(sig / r), V1 = V2 * V2;
            double V3 = std::pow(std::fabs(nd) / r, delt);
            double X = (12.0 * V1 - (6.0 + delt) * V2 * V3) / (r * r) * fc - (V1 - V2 * V3) * dfc;
            double Y = delt * V2 * V3 / nd * fc;
            for (int k = 0; k < 3; ++k) f[k] = f[k] - 4.0 * eps * (X * d[k] + Y * n[k]);
          } else {
            const double D = P[0], r0 = P[1], a = P[2];
            double V2 = std::exp(-a * (r - r0)), V1 = V2 * V2;
            double V3 = std::pow(std::fabs(nd) / r, delt);
            double X = 2.0 * (a * V1 - (a + delt / r) * V2 * V3) / r * fc - (V1 - 2.0 * V2 * V3) * dfc;
            double Y = 2.0 * delt * V2 * V3 / nd * fc;
            for (int k = 0; k < 3; ++k) f[k] = f[k] - D * (X * d[k] + Y * n[k]);
          }
        }
      }
    }
    std::string err;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      for (int q = 0; q < nnum_nn; ++q) {
        int j = nn.L(q, i);
        int l1 = 0;
        for (; l1 < nnum_nn; ++l1)
          if (nn.L(l1, j) == i) break;
        if (l1 >= 3) {
#pragma omp critical
          if (err.empty()) err = "l1>3";
          break;
        }
        int l2 = (l1 + 1) % 3, l3 = (l1 + 2) % 3;  // 0-based form of mod(l1,3)+1, mod(l1+1,3)+1
        double d12[3], d31[3], d23[3];
        const double *a = nn.D(l1, j), *b = nn.D(l2, j), *c = nn.D(l3, j);
        for (int k = 0; k < 3; ++k) {
          d12[k] = b[k] - a[k];
          d31[k] = a[k] - c[k];
          d23[k] = c[k] - b[k];
        }
        double A = dot3(d12, d12) * dot3(d31, d31) - dot3(d12, d31) * dot3(d12, d31);
        double s2331 = dot3(d23, d31), s2312 = dot3(d23, d12);
        const double* n = &gn[3 * static_cast<size_t>(j)];
        for (int p = 0; p < nl.nnum[j]; ++p) {
          double r = nl.R(p, j);
          if (r < R2) {
            const double* d = nl.D(p, j);
            double nd = dot3(n, d);
            double V3 = std::pow(std::fabs(nd) / r, delt);
            double fc = f_cut_cos(r, R1, R2);
            double w[3];
            for (int k = 0; k < 3; ++k) w[k] = d12[k] * s2331 - d31[k] * s2312;
            double C = d[0] * w[0] + d[1] * w[1] + d[2] * w[2];
            double* f = &atoms.frc[3 * nl.pidx[i]];
            double coef;
            if (!morse) {
              const double eps = P[0], sig = P[1];
              double V2 = pow6(sig / r);
              coef = 4.0 * eps * delt * V2 * V3 * fc / A / nd;
            } else {
              const double D = P[0], r0 = P[1], a0 = P[2];
              double V2 = std::exp(-a0 * (r - r0));
              coef = 2.0 * D * delt * V2 * V3 * fc / A / nd;
            }
            for (int k = 0; k < 3; ++k) f[k] = f[k] - coef * n[k] * C;
          }
        }
      }
    }
    if (!err.empty()) throw Stop(E_GR_NN, err);
  }
  // metal side: LennardJonesCosine.f90:112-139, MorseCosine.f90:112-139
  void cosine_forces_for_other_atoms(const NL& nl, const Interaction& in, bool morse) {
    const auto& P = in.spec.p;
    const double R1 = morse ? P[4] : P[3], R2 = morse ? P[5] : P[4];
    const double delt = morse ? P[3] : P[2];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      for (int p = 0; p < nl.nnum[i]; ++p) {
        double r = nl.R(p, i);
        if (r < R2) {
          const double* n = &in.gr_norm[3 * static_cast<size_t>(nl.L(p, i))];
          const double* d = nl.D(p, i);
          double nd = dot3(n, d);
          double fc = f_cut_cos(r, R1, R2), dfc = df_cut_cos(r, R1, R2);
          double* f = &atoms.frc[3 * nl.pidx[i]];
          if (!morse) {
            const double eps = P[0], sig = P[1];
            double V2 = pow6(sig / r), V1 = V2 * V2;
            double V3 = std::pow(std::fabs(nd) / r, delt);
            double X = (12.0 * V1 - (6.0 + delt) * V2 * V3) / (r * r) * fc - (V1 - V2 * V3) * dfc;
            double Y = delt * V2 * V3 / nd * fc;
            for (int k = 0; k < 3; ++k) f[k] = f[k] - 4.0 * eps * (X * d[k] + Y * n[k]);
          } else {
            const double D = P[0], r0 = P[1], a = P[2];
            double V2 = std::exp(-a * (r - r0)), V1 = V2 * V2;
            double V3 = std::pow(std::fabs(nd) / (std::sqrt(dot3(n, n)) * r), delt);
            double X = 2.0 * (a * V1 - (a + delt / r) * V2 * V3) / r * fc - (V1 - 2.0 * V2 * V3) * dfc;
            double Y = 2.0 * delt * V2 * V3 / nd * fc;
            for (int k = 0; k < 3; ++k) f[k] = f[k] - D * (X * d[k] + Y * n[k]);
          }
        }
      }
    }
  }
  void RJL_forces(const NL& nl, const Interaction& in) {  // RosatoGuillopeLegrand.f90:51-94
    const auto& P = in.spec.p;
    const double A0 = P[0], xi = P[1], pp = P[2], qq = P[3], r0 = P[4], R1 = P[5], R2 = P[6];
    size_t M = static_cast<size_t>(nl.nmax);
    std::vector<double> Eb(static_cast<size_t>(nl.N)), expp(M * nl.N), expq(M * nl.N);
#pragma omp parallel
    {
#pragma omp for schedule(static)
      for (int i = 0; i < nl.N; ++i)
        for (int p = 0; p < nl.nnum[i]; ++p) {
          double r = nl.R(p, i);
          if (r <= R2) {
            expq[i * M + p] = std::exp(-2.0 * qq * (r / r0 - 1.0));
            expp[i * M + p] = std::exp(-pp * (r / r0 - 1.0));
          }
        }
#pragma omp for schedule(static)
      for (int i = 0; i < nl.N; ++i) {
        double e = 0.0;
        for (int p = 0; p < nl.nnum[i]; ++p) {
          double r = nl.R(p, i);
          if (r <= R2) e = e + expq[i * M + p] * f_cut_cos(r, R1, R2);
        }
        Eb[i] = std::sqrt(e);
      }
#pragma omp for schedule(static)
      for (int i = 0; i < nl.N; ++i) {
        double* f = &atoms.frc[3 * nl.pidx[i]];
        for (int p = 0; p < nl.nnum[i]; ++p) {
          double r = nl.R(p, i);
          if (r <= R2) {
            double fc = f_cut_cos(r, R1, R2), dfc = df_cut_cos(r, R1, R2);
            double T1 = 2.0 * A0 * (pp / r0 * fc - dfc * r) * expp[i * M + p];
            double T2 = xi * (qq / r0 * fc - dfc / 2.0 * r) * (1.0 / Eb[i] + 1.0 / Eb[nl.L(p, i)]) *
                        expq[i * M + p];
            const double* d = nl.D(p, i);
            for (int k = 0; k < 3; ++k) f[k] = f[k] - (T1 - T2) / r * d[k];
          }
        }
      }
    }
  }
  // B(p,i) of TersoffBrenner.f90:78-92 (forces) / :33-45 (energy)
  void tb_bond_order(const NL& nl, const Interaction& in, std::vector<double>& B) const {
    const auto& P = in.spec.p;
    const double a0 = P[5], delt = P[4], R1 = P[8], R2 = P[9];
    size_t M = static_cast<size_t>(nl.nmax);
    B.assign(M * nl.N, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      for (int p = 0; p < nl.nnum[i]; ++p) {
        double b = 0.0;
        if (nl.R(p, i) < R2) {
          for (int q = 0; q < nl.nnum[i]; ++q) {
            if (p != q && nl.R(q, i) < R2) {
              double cs = dot3(nl.D(p, i), nl.D(q, i)) / (nl.R(p, i) * nl.R(q, i));
              b = b + f_cut_cos(nl.R(q, i), R1, R2) *
                          (1.0 + in.c02 / in.d02 - in.c02 / (in.d02 + (1.0 + cs) * (1.0 + cs)));
            }
          }
          b = std::pow(1.0 + a0 * b, -delt);
        }
        B[i * M + p] = b;
      }
    }
  }
  void TB_forces(const NL& nl, const Interaction& in) {  // TersoffBrenner.f90:74-150
    const auto& P = in.spec.p;
    const double d = P[0], s = P[1], bb = P[2], r0 = P[3], delt = P[4], a0 = P[5], R1 = P[8], R2 = P[9];
    const double c02 = in.c02, d02 = in.d02;
    size_t M = static_cast<size_t>(nl.nmax);
    std::vector<double> B;
    tb_bond_order(nl, in, B);
    const double ex = 1.0 / delt + 1.0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nl.N; ++i) {
      double* F = &atoms.frc[3 * nl.pidx[i]];
      for (int p = 0; p < nl.nnum[i]; ++p) {
        const double* dp = nl.D(p, i);
        const double rp = nl.R(p, i);
        double dB[3] = {0, 0, 0};
        for (int q = 0; q < nl.nnum[i]; ++q) {
          if (p != q) {
            const double* dq = nl.D(q, i);
            const double rq = nl.R(q, i);
            double rr = 1.0 / rp / rq;
            double cosi = dot3(dp, dq) * rr;
            double g1 = f_cut_cos(rq, R1, R2) * 2.0 * a0 * c02 * (1.0 + cosi) /
                        ((d02 + (1.0 + cosi) * (1.0 + cosi)) * (d02 + (1.0 + cosi) * (1.0 + cosi)));
            double g2 = df_cut_cos(rq, R1, R2) * a0 *
                        (1.0 + c02 / d02 - c02 / (d02 + (1.0 + cosi) * (1.0 + cosi)));
            for (int k = 0; k < 3; ++k)
              dB[k] = dB[k] + g1 * ((dp[k] + dq[k]) * rr - cosi * (dp[k] / (rp * rp) + dq[k] / (rq * rq))) +
                      g2 * dq[k];
          }
        }
        double bpe = std::pow(B[i * M + p], ex);
        for (int k = 0; k < 3; ++k) dB[k] = dB[k] * bpe;
        int j = nl.L(p, i);
        int l = 0;
        for (; l < nl.nnum[j]; ++l)
          if (nl.L(l, j) == i) break;
        // l == nnum(j) when i is missing from j's list (reference reads past the row)
        const double* dl = (l < nl.nmax) ? nl.D(l, j) : nullptr;
        const double rl = (l < nl.nmax) ? nl.R(l, j) : 0.0;
        const double Blj = (l < nl.nmax) ? B[j * M + l] : 0.0;
        for (int q = 0; q < nl.nnum[j]; ++q) {
          if (q != l) {
            const double* dq = nl.D(q, j);
            const double rq = nl.R(q, j);
            double rr = 1.0 / rl / rq;
            double cosi = dot3(dl, dq) * rr;
            double g = std::pow(Blj, ex) * f_cut_cos(rq, R1, R2) * 2.0 * a0 * c02 * (1.0 + cosi) /
                       ((d02 + (1.0 + cosi) * (1.0 + cosi)) * (d02 + (1.0 + cosi) * (1.0 + cosi)));
            for (int k = 0; k < 3; ++k) dB[k] = dB[k] + g * (-dq[k] * rr + cosi * dl[k] / (rl * rl));
          }
        }
        for (int k = 0; k < 3; ++k) dB[k] = dB[k] * (-delt) / 2.0;
        if (rp < R2) {
          double fc = f_cut_cos(rp, R1, R2);
          double dff = df_cut_cos(rp, R1, R2) / fc;
          double a = -std::sqrt(2.0 * s) * bb * (rp - r0);
          double ea = std::exp(a), eas = std::exp(a / s);
          double c1 = std::sqrt(2.0 * s) * bb / rp, c2 = std::sqrt(2.0 / s) * bb / rp;
          double pre = fc * d / (s - 1.0);
          double bavg = (B[i * M + p] + Blj) / 2;
          for (int k = 0; k < 3; ++k)
            F[k] = F[k] + pre * ((dp[k] * dff - c1 * dp[k]) * ea -
                                 (dB[k] + bavg * (dp[k] * dff - c2 * dp[k])) * s * eas);
        }
        for (int q = 0; q < nl.nnum[j]; ++q) {
          if (q != l) {
            double fc = f_cut_cos(rl, R1, R2), dfc = df_cut_cos(rl, R1, R2);
            const double* dq = nl.D(q, j);
            const double rq = nl.R(q, j);
            double rr = 1.0 / rl / rq;
            double cosi = dot3(dl, dq) * rr;
            double t1 = fc * 2.0 * a0 * c02 * (1.0 + cosi) /
                        ((d02 + (1.0 + cosi) * (1.0 + cosi)) * (d02 + (1.0 + cosi) * (1.0 + cosi)));
            double t2 = dfc * a0 * (1.0 + c02 / d02 - c02 / (d02 + (1.0 + cosi) * (1.0 + cosi)));
            double pre = delt / 2 * std::pow(B[j * M + q], ex);
            double post = f_cut_cos(rq, R1, R2) * d / (s - 1.0) * s *
                          std::exp(-std::sqrt(2.0 * s) * bb * (rq - r0) / s);
            for (int k = 0; k < 3; ++k)
              F[k] = F[k] + pre * (t1 * (-dq[k] * rr + cosi * dl[k] / (rl * rl)) + dp[k] * t2) * post;
          }
        }
      }
    }
  }
  // calculate_truncated_nl, md_interactions.f90:333-375: row i and the rows within
  // n-1 list steps of it in full, the rows at step n with one entry (back to the
  // first row that lists them).  `has` stands for particle_index /= 0.
  static void calculate_truncated_nl(NL& t, const NL& nl, int i, int n, std::vector<char>& has) {
    std::fill(t.nnum.begin(), t.nnum.end(), 0);
    std::fill(has.begin(), has.end(), 0);
    auto copy_row = [&](int q) {
      for (int p = 0; p < nl.nnum[q]; ++p) {
        t.L(p, q) = nl.L(p, q);
        for (int k = 0; k < 3; ++k) t.D(p, q)[k] = nl.D(p, q)[k];
        t.R(p, q) = nl.R(p, q);
      }
      t.pidx[q] = nl.pidx[q];
      has[q] = 1;
    };
    copy_row(i);
    t.nnum[i] = nl.nnum[i];
    for (int ni = 1; ni <= n; ++ni) {
      if (ni < n) {
        for (int j = 0; j < t.N; ++j)
          for (int p = 0; p < t.nnum[j]; ++p) {
            const int q = t.L(p, j);
            if (t.nnum[q] == 0) copy_row(q);
          }
        for (int j = 0; j < t.N; ++j)
          if (has[j]) t.nnum[j] = nl.nnum[j];
      } else {
        for (int j = 0; j < t.N; ++j)
          for (int p = 0; p < t.nnum[j]; ++p) {
            const int q = t.L(p, j);
            if (t.nnum[q] == 0) {
              t.nnum[q] = t.nnum[q] + 1;
              const int s = t.nnum[q] - 1;
              t.L(s, q) = j;
              for (int k = 0; k < 3; ++k) t.D(s, q)[k] = -nl.D(p, j)[k];
              t.R(s, q) = nl.R(p, j);
              t.pidx[q] = nl.pidx[q];
              has[q] = 1;
            }
          }
      }
    }
  }
  // shift_drs, md_interactions.f90:377-399 (nl_n == 1): atom row inl moved by -dx along k
  static void shift_drs(NL& t, int inl, int k, double dx) {
    for (int p = 0; p < t.nnum[inl]; ++p) {
      double* d = t.D(p, inl);
      d[k] = d[k] - dx;
      t.R(p, inl) = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    }
    for (int j = 0; j < t.N; ++j)
      for (int p = 0; p < t.nnum[j]; ++p)
        if (t.L(p, j) == inl) {
          double* d = t.D(p, j);
          d[k] = d[k] + dx;
          t.R(p, j) = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        }
  }
  // calculate_forces_numerically, md_interactions.f90:273-310 (rebosc: neib_order 3)
  void calculate_forces_numerically() {
    const double dx = 1e-6;  // 10.**(-6)
    for (auto& in : inters) {
      if (in.spec.kind != pfmd_io::K_REBOSC) continue;
      for (auto& nl : in.nl) {
#pragma omp parallel
        {
          NL t;
          t.N = nl.N;
          t.nmax = nl.nmax;
          create_neighbour_list(t);
          std::vector<char> has(static_cast<size_t>(t.N), 0);
#pragma omp for schedule(static)
          for (int inl = 0; inl < nl.N; ++inl) {
            calculate_truncated_nl(t, nl, inl, 3, has);
            for (int k = 0; k < 3; ++k) {
              shift_drs(t, inl, k, -dx);
              const double e1 = rebosc_energy(t, in.spec.p);
              shift_drs(t, inl, k, 2 * dx);
              const double e2 = rebosc_energy(t, in.spec.p);
              if (k != 2) shift_drs(t, inl, k, -dx);
              double& f = atoms.frc[3 * static_cast<size_t>(nl.pidx[inl]) + k];
              f = f + (e1 - e2) / 2 / dx;
            }
          }
        }
      }
    }
  }
  void calculate_forces() {  // md_interactions.f90:210-242
    for (auto& in : inters) {
      switch (in.spec.kind) {
        case pfmd_io::K_LJ:
          LJ_forces(in.nl[0], in);
          LJ_forces(in.nl[1], in);
          break;
        case pfmd_io::K_LJ1G:
          LJ1g_forces(in.nl[0], in);
          break;
        case pfmd_io::K_LJC:
          cosine_forces_for_graphene(in.nl[0], in.nl[2], in, false);
          cosine_forces_for_other_atoms(in.nl[1], in, false);
          break;
        case pfmd_io::K_MORSEC:
          cosine_forces_for_graphene(in.nl[0], in.nl[2], in, true);
          cosine_forces_for_other_atoms(in.nl[1], in, true);
          break;
        case pfmd_io::K_TB:
          TB_forces(in.nl[0], in);
          break;
        case pfmd_io::K_RJL:
          RJL_forces(in.nl[0], in);
          break;
        case pfmd_io::K_REBOSC:  // numerical: calculate_forces_numerically
          break;
      }
    }
  }

  // ---------------- potentials: energies ----------------
  template <class F>
  double reduce_rows(int n, F f) const {
    int nt = omp_get_max_threads();
    std::vector<double> part(static_cast<size_t>(nt), 0.0);
#pragma omp parallel
    {
      int t = omp_get_thread_num();
      double acc = 0.0;
#pragma omp for schedule(static)
      for (int i = 0; i < n; ++i) acc = acc + f(i);
      part[t] = acc;
    }
    double s = 0.0;
    for (double v : part) s = s + v;
    return s;
  }
  double energy(const Interaction& in) const {  // md_interactions.f90:244-261 over nl(1)
    const NL& nl = in.nl[0];
    const auto& P = in.spec.p;
    switch (in.spec.kind) {
      case pfmd_io::K_LJ:  // LennardJones.f90:23-46
        return reduce_rows(nl.N, [&](int i) {
          double e = 0.0;
          for (int p = 0; p < nl.nnum[i]; ++p) {
            double r = nl.R(p, i);
            if (r < P[3]) {
              double V = pow6(P[1] / r);
              e = e + 4.0 * P[0] * V * (V - 1.0) * f_cut_cos(r, P[2], P[3]);
            }
          }
          return e;
        });
      case pfmd_io::K_LJ1G:  // LennardJones_1g.f90:28-52
        return reduce_rows(nl.N, [&](int i) {
          double e = 0.0;
          for (int p = 0; p < nl.lessnnum[i]; ++p) {
            double r = nl.R(p, i);
            double U = 1.0 / (r * r * r * r * r * r);
            e = e + U * (in.c12 * U - in.c6) * f_cut_poly(r, P[2], P[3]);
          }
          return e;
        });
      case pfmd_io::K_LJC:  // LennardJonesCosine.f90:26-51
      case pfmd_io::K_MORSEC: {  // MorseCosine.f90:26-51
        bool morse = in.spec.kind == pfmd_io::K_MORSEC;
        const double R1 = morse ? P[4] : P[3], R2 = morse ? P[5] : P[4];
        const double delt = morse ? P[3] : P[2];
        return reduce_rows(nl.N, [&](int i) {
          double e = 0.0;
          const double* n = &in.gr_norm[3 * static_cast<size_t>(i)];
          for (int p = 0; p < nl.nnum[i]; ++p) {
            double r = nl.R(p, i);
            if (r < R2) {
              double V3 = std::pow(std::fabs(dot3(n, nl.D(p, i))) / r, delt);
              if (!morse) {
                double V2 = pow6(P[1] / r), V1 = V2 * V2;
                e = e + 4.0 * P[0] * (V1 - V2 * V3) * f_cut_cos(r, R1, R2);
              } else {
                double V2 = std::exp(-P[2] * (r - P[1])), V1 = V2 * V2;
                e = e + P[0] * (V1 - 2.0 * V2 * V3) * f_cut_cos(r, R1, R2);
              }
            }
          }
          return e;
        });
      }
      case pfmd_io::K_RJL:  // RosatoGuillopeLegrand.f90:23-49
        return reduce_rows(nl.N, [&](int i) {
          double Eb2 = 0.0, Er = 0.0;
          for (int p = 0; p < nl.nnum[i]; ++p) {
            double r = nl.R(p, i);
            if (r <= P[6]) {
              Eb2 = Eb2 + std::exp(-2.0 * P[3] * (r / P[4] - 1.0)) * f_cut_cos(r, P[5], P[6]);
              Er = Er + std::exp(-P[2] * (r / P[4] - 1.0)) * f_cut_cos(r, P[5], P[6]);
            }
          }
          return P[0] * Er - P[1] * std::sqrt(Eb2);
        });
      case pfmd_io::K_REBOSC:
        return rebosc_energy(nl, P);
      case pfmd_io::K_TB: {  // TersoffBrenner.f90:26-72
        std::vector<double> B;
        tb_bond_order(nl, in, B);
        size_t M = static_cast<size_t>(nl.nmax);
        const double d = P[0], s = P[1], bb = P[2], r0 = P[3], R1 = P[8], R2 = P[9];
        return reduce_rows(nl.N, [&](int i) {
          double e = 0.0;
          for (int p = 0; p < nl.nnum[i]; ++p) {
            double r = nl.R(p, i);
            if (r < R2) {
              int j = nl.L(p, i);
              if (j > i) {
                int q = 0;
                for (; q < nl.nnum[j]; ++q)
                  if (nl.L(q, j) == i) break;
                double Bqj = (q < nl.nmax) ? B[j * M + q] : 0.0;
                double a = -std::sqrt(2.0 * s) * bb * (r - r0);
                e = e + f_cut_cos(r, R1, R2) * d / (s - 1.0) *
                            (std::exp(a) - (B[i * M + p] + Bqj) / 2 * s * std::exp(a / s));
              }
            }
          }
          return e;
        });
      }
    }
    return 0.0;
  }
  void calculate_potential_energies() {  // md_interactions.f90:263-271
    for (auto& in : inters) in.energy = energy(in);
  }

  // ---------------- md_integrators.f90 ----------------
  void integrate_verlet_positions(const Group& g, bool xyz) {  // :7-56
    int k0 = xyz ? 0 : 2;
#pragma omp parallel for schedule(static)
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      for (int k = k0; k < 3; ++k) {
        double& x = atoms.pos[3 * i + k];
        x = x + atoms.vel[3 * i + k] * dt.ts[0];
        if (x > cell.box[k])
          x = x - cell.box[k];
        else if (x < 0.0)
          x = x + cell.box[k];
      }
    }
  }
  void integrate_verlet_velocities(const Group& g, bool xyz) {  // :58-97
    int k0 = xyz ? 0 : 2;
#pragma omp parallel for schedule(static)
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      for (int k = k0; k < 3; ++k)
        atoms.vel[3 * i + k] =
            atoms.vel[3 * i + k] + atoms.frc[3 * i + k] / atoms.mass[i] / MASS_COEF * dt.ts[1];
    }
  }
  void molecular_static_xyz_velocities(const Group& g) {  // :99-123
#pragma omp parallel for schedule(static)
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      const double* f = &atoms.frc[3 * i];
      double* v = &atoms.vel[3 * i];
      double fv = f[0] * v[0] + f[1] * v[1] + f[2] * v[2];
      double ff = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
      if (fv > 0.0 && ff > 1e-12) {
        for (int k = 0; k < 3; ++k) v[k] = fv / ff * f[k];
      } else {
        v[0] = v[1] = v[2] = 0.0;
      }
    }
  }
  void molecular_static_1D_velocities(const Group& g) {  // :125-145
#pragma omp parallel for schedule(static)
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      const double* f = &atoms.frc[3 * i];
      double* v = &atoms.vel[3 * i];
      double fv = f[0] * v[0] + f[1] * v[1] + f[2] * v[2];
      if (!(fv > 0.0)) v[0] = v[1] = v[2] = 0.0;
    }
  }
  void zero_forces(const Group& g) {  // :147-163
#pragma omp parallel for schedule(static)
    for (int ind = 0; ind < g.N; ++ind) {
      int i = g.idx[ind];
      atoms.frc[3 * i] = atoms.frc[3 * i + 1] = atoms.frc[3 * i + 2] = 0.0;
    }
  }
  void integrate_nose_hoover_chain(NHC& h, const Group& g) {  // :200-245
    double ke = calculate_kinetic_energy(g);
    double kt = KT_A_DEGREE * h.temperature;
    double kedif = 2.0 * ke - 3.0 * h.L * kt;
    const double ts2 = dt.ts[1], ts3 = dt.ts[2], ts4 = dt.ts[3];
    const int M = h.M;
    auto& v = h.v;
    auto& q = h.q;
    double b = 0.0;
    if (M == 1) {
      v[0] = v[0] + kedif / q[0] * ts3;
    } else {
      v[M - 1] = v[M - 1] + (q[M - 2] * (v[M - 2] * v[M - 2]) - kt) / q[M - 1] * ts3;
      for (int i = M - 2; i >= 1; --i) {
        b = std::exp(-v[i + 1] * ts4);
        v[i] = v[i] * (b * b) + (q[i - 1] * (v[i - 1] * v[i - 1]) - kt) / q[i] * ts3 * b;
      }
      b = std::exp(-v[1] * ts4);
      v[0] = v[0] * (b * b) + kedif / q[0] * ts3 * b;
    }
    h.s = std::exp(-v[0] * ts2);
    scale_velocities(g, h.s);
    kedif = 2.0 * ke * (h.s * h.s) - 3.0 * h.L * kt;
    for (int i = 0; i < M; ++i) h.x[i] = h.x[i] + v[i] * ts2;
    if (M == 1) {
      v[0] = v[0] + kedif / q[0] * ts3;
    } else {
      v[0] = v[0] * (b * b) + kedif / q[0] * ts3 * b;
      for (int i = 1; i <= M - 2; ++i) {
        b = std::exp(-v[i + 1] * ts4);
        v[i] = v[i] * (b * b) + (q[i - 1] * (v[i - 1] * v[i - 1]) - kt) / q[i] * ts3 * b;
      }
      v[M - 1] = v[M - 1] + (q[M - 2] * (v[M - 2] * v[M - 2]) - kt) / q[M - 1] * ts3;
    }
  }
  void calculate_nose_hoover_chain_energy(NHC& h) {  // :247-260
    double kt = KT_A_DEGREE * h.temperature;
    h.e = h.q[0] / 2 * (h.v[0] * h.v[0]) + 3.0 * h.L * kt * h.x[0];
    for (int i = 1; i < h.M; ++i) h.e = h.e + h.q[i] / 2 * (h.v[i] * h.v[i]) + kt * h.x[i];
  }

  // ---------------- md_simulation.f90 ----------------
  void setup() {  // :44-113
    exe_time_start = omp_get_wtime();
    try {
      pfmd_io::read_settings(input_path, settings_filename, S);
    } catch (...) {
      emit(S.echo);
      throw;
    }
    emit(S.echo);
    cell.box[0] = S.xyz.box[0];
    cell.box[1] = S.xyz.box[1];
    cell.box[2] = S.xyz.box[2];
    for (int k = 0; k < 3; ++k) cell.half[k] = 0.5 * cell.box[k];
    atoms.N = S.xyz.N;
    atoms.pos = S.xyz.pos;
    atoms.vel = S.xyz.vel;
    atoms.mass = S.xyz.mass;
    atoms.types = S.xyz.types;
    atoms.frc.assign(3 * static_cast<size_t>(atoms.N), 0.0);
    for (const auto& names : S.group_types) {
      Group g;
      create_particle_group(g, names);
      groups.push_back(g);
    }
    for (const auto& c : S.changes) {
      change_from.push_back(c.from);
      change_to.push_back(c.to);
      change_ts1.push_back(c.ts1);
      change_ts2.push_back(c.ts2);
      change_frec.push_back(c.frec);
      G(c.from);
      G(c.to);
      if (c.frec < 1) throw Stop(E_PARAM, "error: group change frequency must be positive");
    }
    integrators.push_back(Integrator{"none", 0.0, 0, 1, 1});
    for (const auto& is : S.integrators) {
      if (is.period_log < 1 || is.period_snapshot < 1)
        throw Stop(E_PARAM, "error: integrator output periods must be positive");
      integrators.push_back(Integrator{is.name, is.dt, is.l, is.period_snapshot, is.period_log});
    }
    for (const auto& h : S.nhc) {
      NHC c;  // create_nose_hoover_chain, md_integrators.f90:165-180
      c.M = h.M;
      if (c.M < 1) throw Stop(E_PARAM, "error: wrong nhc parameters");
      c.x.assign(static_cast<size_t>(c.M), 0.0);
      c.v.assign(static_cast<size_t>(c.M), 0.0);
      c.q.assign(static_cast<size_t>(c.M), 0.0);
      c.e = 0.0;
      c.s = 1.0;
      // set_nose_hoover_chain, md_integrators.f90:182-198
      c.group_num = h.group;
      c.L = G(h.group).N;
      c.temperature = h.temperature;
      c.q[0] = h.q1;
      for (int i = 1; i < c.M; ++i) c.q[i] = c.q[0] / (3.0 * c.L);
      nhc.push_back(c);
    }
    double t0 = S.initial_temperature;
    if (t0 < 0.0) t0 = 0.0;
    G(S.all_moving);
    G(S.xyz_moving);
    G(S.z_moving);
    G(S.all_atoms);
    G(S.traj_group);
    if (S.period_traj < 1 || S.zero_momentum_period < 1)
      throw Stop(E_PARAM, "error: output and momentum periods must be positive");
    if (S.new_velocities) set_new_temperature(G(S.all_moving), t0, rand_seed);
    create_interactions();
    if (write_files) {
      logname = output_prefix + fortio::trim(S.logfilename);
      log = std::fopen(logname.c_str(), "w");
      if (!log) throw Stop(E_IO, "cannot open log file " + logname);
    }
    line(fortio::Rec().a("PREPARATIONS TIME: ", 24).f(omp_get_wtime() - exe_time_start, 10, 2).a(" S ").s);
    line(fortio::Rec().a("RUNNING ON ", 24).i(num_threads, 6).a(" OPENMP THREADS").s);
    line("");
    exe_time_md = omp_get_wtime();
    integrator_index = 0;
    dt.simulation_time = 0.0;
    md_step = 0;
  }

  void log_write(const std::string& s) {
    if (log) std::fputs(s.c_str(), log);
  }

  // One pass of the loop body for md_step (md_simulation.f90:116-241).  Sets
  // `finished` when the loop exits at this md_step.
  void step() {
    if (finished) return;
    if (md_step > S.md_step_limit) {
      finished = true;
      return;
    }
    for (size_t i = 0; i < change_to.size(); ++i)
      change_particle_group_N(G(change_to[i]), md_step, change_ts1[i], change_ts2[i], change_frec[i],
                              G(change_from[i]));
    const int integrators_num = static_cast<int>(integrators.size()) - 1;
    long long lsum = 0;
    for (int k = 0; k <= integrator_index && k <= integrators_num; ++k) lsum += integrators[k].l;
    if (md_step - 1 == lsum || integrator_index == 0) {
      integrator_index = integrator_index + 1;
      int i = integrator_index;
      for (; i <= integrators_num; ++i) {
        if (integrators[i].l > 0) {
          integrator_name = integrators[i].name;
          init_time_steps(integrators[i].dt);
          break;
        }
      }
      if (i > integrators_num || (i == integrators_num && integrators[integrators_num].l < 1)) {
        line(" no more integrators");
        finished = true;
        return;
      }
      integrator_index = i;
    }
    double exe_t = omp_get_wtime();
    check_positions();
    if (S.invert_z_vel) invert_z_velocities(0.8 * cell.box[2], 0.9 * cell.box[2]);
    if (md_step != 0) {
      if (integrator_name == "nvms") {
        if (std::fabs(potential_energy - prev_potential_energy) <= S.ms_de) {
          line(" potential energy diffrence is small enough");
          finished = true;
          return;
        }
      }
      if (integrator_name == "nvt")
        for (auto& h : nhc) integrate_nose_hoover_chain(h, G(h.group_num));
      integrate_verlet_velocities(G(S.xyz_moving), true);
      integrate_verlet_velocities(G(S.z_moving), false);
      integrate_verlet_positions(G(S.xyz_moving), true);
      integrate_verlet_positions(G(S.z_moving), false);
    }
    prev_potential_energy = potential_energy;
    exe_time_pos_vel += omp_get_wtime() - exe_t;

    exe_t = omp_get_wtime();
    update_interactions_neighbour_lists(md_step);
    exe_time_nlists += omp_get_wtime() - exe_t;
    exe_t = omp_get_wtime();
    if (md_step % S.zero_momentum_period == 0) zero_momentum(G(S.all_atoms));
    zero_forces(G(S.all_atoms));
    calculate_forces();
    calculate_forces_numerically();
    exe_time_forces += omp_get_wtime() - exe_t;

    exe_t = omp_get_wtime();
    if (md_step != 0) {
      integrate_verlet_velocities(G(S.xyz_moving), true);
      integrate_verlet_velocities(G(S.z_moving), false);
      if (integrator_name == "nvt")
        for (auto& h : nhc) integrate_nose_hoover_chain(h, G(h.group_num));
      if (integrator_name == "nvms") {
        molecular_static_xyz_velocities(G(S.xyz_moving));
        molecular_static_1D_velocities(G(S.z_moving));
      }
      dt.simulation_time = dt.simulation_time + dt.ts[0];
    }
    exe_time_pos_vel += omp_get_wtime() - exe_t;

    const Integrator& I = integrators[static_cast<size_t>(integrator_index)];
    if (md_step % I.period_log == 0 || md_step % out_period == 0 || integrator_name == "nvms") {
      exe_t = omp_get_wtime();
      calculate_potential_energies();
      potential_energy = 0.0;
      for (auto& in : inters) potential_energy = potential_energy + in.energy;
      calculate_temperature(temperature, kinetic_energy, G(S.all_moving));
      if (integrator_name == "nvt")
        for (auto& h : nhc) calculate_nose_hoover_chain_energy(h);
      nose_hoover_energy = 0.0;
      for (auto& h : nhc) nose_hoover_energy = nose_hoover_energy + h.e;
      total_energy = potential_energy + kinetic_energy;
      conserved_energy = total_energy + nose_hoover_energy;
      exe_time_energy += omp_get_wtime() - exe_t;
      if (md_step % I.period_log == 0) {
        fortio::Rec r;
        r.a(fortio::trim(integrator_name), 6).i(md_step, 9);
        r.f(dt.simulation_time, 24, 6).f(conserved_energy, 24, 6).f(nose_hoover_energy, 24, 6);
        r.f(total_energy, 24, 6).f(potential_energy, 24, 6).f(kinetic_energy, 24, 6).f(temperature, 24, 6);
        for (auto& in : inters) r.f(in.energy, 20, 9);
        for (auto& h : nhc) r.f(h.e, 20, 9);
        log_write(r.s + "\n");
      }
      if (md_step % out_period == 0) {
        double fs[3], mc[3], mcv[3];
        calculate_force_sum(fs, G(S.all_atoms));
        calculate_mass_center(mc, G(S.all_atoms));
        calculate_mass_center_velocity(mcv, G(S.all_atoms));
        double fsn = std::sqrt(fs[0] * fs[0] + fs[1] * fs[1] + fs[2] * fs[2]);
        double mcvn = std::sqrt(mcv[0] * mcv[0] + mcv[1] * mcv[1] + mcv[2] * mcv[2]);
        line(fortio::Rec().a("exe time (s) = ").f(omp_get_wtime() - exe_time_start, 10, 2).s);
        line(fortio::Rec().a("step = ").i(md_step, 12).a(" integrator = ").a(fortio::trim(integrator_name), 6).s);
        line(fortio::Rec().a("conserved energy (eV) = ").es(conserved_energy, 21, 9).s);
        line(fortio::Rec().a("forces sum (eV/A) = ").es(fsn, 16, 6).s);
        line(fortio::Rec().a("c.o.m. velocity (A/fs) = ").es(mcvn, 16, 6).s);
        line(fortio::Rec().a("c.o.m. position (A) = ").f(mc[0], 12, 6).f(mc[1], 12, 6).f(mc[2], 12, 6).s);
        line(fortio::Rec().a("maximum velocity (A/fs) = ").f(find_max_velocity(), 12, 6).s);
        nlists_load();
        if (integrator_name != "nvms" && fsn > 1e-14) line(" WARNING: forces sum is too big");
        if (integrator_name == "nvt" && S.xyz_moving == S.all_atoms && mcvn > 1e-14)
          line(" WARNING: center of mass velocity is too big");
        line("");
      }
    }
    if (md_step % I.period_snapshot == 0 && md_step != 0 && write_files) {
      std::string fn = output_prefix + "snapshot_" + fortio::fmt_i0pad(md_step, 6, 6) + ".xyz";
      const Group& g = G(S.all_atoms);
      write_text(fn, pfmd_io::xyz_snapshot_text(cell.box, g.N, g.idx.data(), atoms.pos.data(),
                                               atoms.vel.data(), atoms.mass.data(), atoms.types),
                 false);
    }
    if (md_step % S.period_traj == 0 && write_files) {
      std::string fn = output_prefix + "traj_" + fortio::fmt_i0pad(S.traj_group, 2, 2) + ".xyz";
      const Group& g = G(S.traj_group);
      write_text(fn, pfmd_io::xyz_traj_frame_text(cell.box, g.N, g.idx.data(), atoms.pos.data(),
                                                 atoms.vel.data(), atoms.mass.data(), atoms.types, md_step),
                 true);
    }
    md_step = md_step + 1;
  }
  void nlists_load() {  // md_interactions.f90:427-444
    if (!inters.empty()) line("neib lists load:");
    for (auto& in : inters)
      for (int j = 0; j < in.nl_n; ++j) {
        const NL& nl = in.nl[static_cast<size_t>(j)];
        int mx = 0;
        if (nl.N > 0) mx = *std::max_element(nl.nnum.begin(), nl.nnum.end());
        line(fortio::Rec().a(fortio::trim(in.spec.name), 8).i(j + 1, 3).i(mx, 6).a(" /").i(nl.nmax, 6).s);
      }
  }
  void write_text(const std::string& fn, const std::string& text, bool append) {
    FILE* f = std::fopen(fn.c_str(), append ? "a" : "w");
    if (!f) throw Stop(E_IO, "cannot open " + fn);
    std::fputs(text.c_str(), f);
    std::fclose(f);
  }
  void finish() {  // :245-272
    exe_time_md = omp_get_wtime() - exe_time_md;
    if (integrator_name == "nvms")
      line(" potential energy difference: " + fortio::list_real(potential_energy - prev_potential_energy));
    line(" steps number:" + fortio::list_int(md_step - 1));
    line("");
    line(" PERFOMANCE:");
    auto perf = [&](const char* name, double t) {
      line(fortio::Rec().a(name, 24).f(t, 10, 2).a(" S ").f(t / exe_time_md * 100, 10, 2).a("%").s);
    };
    perf("MD:", exe_time_md);
    perf("POSITION AND VELOCITY:", exe_time_pos_vel);
    perf("NEIGHBOURS:", exe_time_nlists);
    perf("NEIGHBOURS SEARCH:", exe_time_nlsearch);
    perf("NEIGHBOURS DISTANCE:", exe_time_nldistance);
    perf("FORCES:", exe_time_forces);
    perf("ENERGY:", exe_time_energy);
    perf("REST:", exe_time_md - exe_time_pos_vel - exe_time_nlists - exe_time_forces - exe_time_energy);
    line(fortio::Rec().a("TIME STEPS PER HOUR:", 24).f(static_cast<double>(md_step) / exe_time_md * 3600, 16, 2).s);
    line("");
    fortio::Rec r;
    r.a(fortio::trim(output_prefix), 32).i(md_step - 1, 9).f(dt.simulation_time, 20, 9);
    r.f(total_energy, 20, 9).f(potential_energy, 20, 9).f(kinetic_energy, 20, 9).f(temperature, 20, 9);
    for (auto& in : inters) r.f(in.energy, 20, 9);
    all_emit(r.s);  // the record stays open (advance='no'); the runner ends it
    log_write(r.s + "\n");
    if (md_step != 0 && write_files) {
      std::string fn = output_prefix + "final_" + fortio::trim(S.init_xyz_filename);
      const Group& g = G(S.all_atoms);
      write_text(fn, pfmd_io::xyz_snapshot_text(cell.box, g.N, g.idx.data(), atoms.pos.data(),
                                               atoms.vel.data(), atoms.mass.data(), atoms.types),
                 false);
    }
    if (log) {
      std::fclose(log);
      log = nullptr;
    }
  }
};

}  // namespace orc

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
struct orc_sim {
  std::unique_ptr<orc::Sim> s;
  std::string err;
};

template <class F>
static int guarded(orc_sim* h, F f) {
  try {
    f();
    return 0;
  } catch (const orc::Stop& e) {
    h->err = e.what();
    return e.code;
  } catch (const fortio::ReadError& e) {
    h->err = e.what();
    return orc::E_IO;
  } catch (const std::exception& e) {
    h->err = e.what();
    return orc::E_PARAM;
  }
}

extern "C" {

int orc_create(const char* input_path, const char* settings_filename, const char* output_prefix,
               int out_period, int num_threads, int rand_seed, int write_files, orc_sim** out) {
  auto* h = new orc_sim();
  h->s.reset(new orc::Sim());
  orc::Sim& s = *h->s;
  s.input_path = input_path ? input_path : "";
  s.settings_filename = settings_filename ? settings_filename : "md_run_settings.txt";
  s.output_prefix = output_prefix ? output_prefix : "";
  s.out_period = out_period > 0 ? out_period : 1;
  s.num_threads = num_threads > 0 ? num_threads : omp_get_max_threads();
  s.rand_seed = rand_seed;
  s.write_files = write_files != 0;
  omp_set_num_threads(s.num_threads);
  *out = h;
  return guarded(h, [&] { s.setup(); });
}

int orc_step(orc_sim* h, int* finished) {
  int rc = guarded(h, [&] { h->s->step(); });
  if (finished) *finished = h->s->finished ? 1 : 0;
  return rc;
}

int orc_run(orc_sim* h, long long nsteps, int* finished) {
  int rc = guarded(h, [&] {
    for (long long k = 0; k < nsteps && !h->s->finished; ++k) h->s->step();
  });
  if (finished) *finished = h->s->finished ? 1 : 0;
  return rc;
}

int orc_finish(orc_sim* h) {
  return guarded(h, [&] { h->s->finish(); });
}
void orc_destroy(orc_sim* h) { delete h; }
long long orc_md_step(const orc_sim* h) { return h->s->md_step; }
int orc_natoms(const orc_sim* h) { return h->s->atoms.N; }
void orc_get_state(const orc_sim* h, double* pos, double* vel, double* frc) {
  const auto& a = h->s->atoms;
  size_t n = 3 * static_cast<size_t>(a.N);
  if (pos) std::memcpy(pos, a.pos.data(), n * sizeof(double));
  if (vel) std::memcpy(vel, a.vel.data(), n * sizeof(double));
  if (frc) std::memcpy(frc, a.frc.data(), n * sizeof(double));
}
void orc_set_state(orc_sim* h, const double* pos, const double* vel) {
  auto& a = h->s->atoms;
  size_t n = 3 * static_cast<size_t>(a.N);
  if (pos) std::memcpy(a.pos.data(), pos, n * sizeof(double));
  if (vel) std::memcpy(a.vel.data(), vel, n * sizeof(double));
}
double orc_sim_time(const orc_sim* h) { return h->s->dt.simulation_time; }
int orc_ninteractions(const orc_sim* h) { return static_cast<int>(h->s->inters.size()); }
int orc_nl_shape(const orc_sim* h, int inter, int list, int* n_rows, int* nmax) {
  const auto& s = *h->s;
  if (inter < 0 || inter >= static_cast<int>(s.inters.size())) return orc::E_PARAM;
  const auto& in = s.inters[static_cast<size_t>(inter)];
  if (list < 0 || list >= in.nl_n) return orc::E_PARAM;
  *n_rows = in.nl[static_cast<size_t>(list)].N;
  *nmax = in.nl[static_cast<size_t>(list)].nmax;
  return 0;
}
int orc_get_nl(const orc_sim* h, int inter, int list, int* nnum, int* lessnnum, int* pidx, int* nlist,
               double* moddr) {
  int n, m;
  int rc = orc_nl_shape(h, inter, list, &n, &m);
  if (rc) return rc;
  const auto& nl = h->s->inters[static_cast<size_t>(inter)].nl[static_cast<size_t>(list)];
  if (n == 0) return 0;
  if (nnum) std::memcpy(nnum, nl.nnum.data(), sizeof(int) * static_cast<size_t>(n));
  if (lessnnum) std::memcpy(lessnnum, nl.lessnnum.data(), sizeof(int) * static_cast<size_t>(n));
  if (pidx) std::memcpy(pidx, nl.pidx.data(), sizeof(int) * static_cast<size_t>(n));
  if (nlist) std::memcpy(nlist, nl.nlist.data(), sizeof(int) * static_cast<size_t>(n) * m);
  if (moddr) std::memcpy(moddr, nl.moddr.data(), sizeof(double) * static_cast<size_t>(n) * m);
  return 0;
}
int orc_get_gr_norm(const orc_sim* h, int inter, double* norm) {
  const auto& s = *h->s;
  if (inter < 0 || inter >= static_cast<int>(s.inters.size())) return orc::E_PARAM;
  const auto& g = s.inters[static_cast<size_t>(inter)].gr_norm;
  if (g.empty()) return orc::E_PARAM;
  std::memcpy(norm, g.data(), g.size() * sizeof(double));
  return 0;
}
int orc_energies(const orc_sim* h, double* e_inter, double* pe, double* ke, double* temp,
                 double* e_nhc, double* e_conserved) {
  const auto& s = *h->s;
  if (e_inter)
    for (size_t i = 0; i < s.inters.size(); ++i) e_inter[i] = s.inters[i].energy;
  if (pe) *pe = s.potential_energy;
  if (ke) *ke = s.kinetic_energy;
  if (temp) *temp = s.temperature;
  if (e_nhc) *e_nhc = s.nose_hoover_energy;
  if (e_conserved) *e_conserved = s.conserved_energy;
  return 0;
}
int orc_eval(orc_sim* h, int rebuild, double* e_inter) {
  return guarded(h, [&] {
    auto& s = *h->s;
    // a step number that is (rebuild) or is not (refresh) a multiple of every period
    // step 0 is a multiple of every period; a large prime is a multiple of none
    // (lists with period 1 rebuild either way)
    long long step = rebuild ? 0 : 1000003;
    s.update_interactions_neighbour_lists(step);
    s.zero_forces(s.G(s.S.all_atoms));
    s.calculate_forces();
    s.calculate_forces_numerically();
    s.calculate_potential_energies();
    if (e_inter)
      for (size_t i = 0; i < s.inters.size(); ++i) e_inter[i] = s.inters[i].energy;
  });
}
const char* orc_errmsg(const orc_sim* h) { return h->err.c_str(); }
const char* orc_output(const orc_sim* h) { return h->s->out.c_str(); }

double orc_f_cut_cos(double r, double R1, double R2) { return orc::f_cut_cos(r, R1, R2); }
double orc_df_cut_cos(double r, double R1, double R2) { return orc::df_cut_cos(r, R1, R2); }
double orc_f_cut_poly(double r, double R1, double R2) { return orc::f_cut_poly(r, R1, R2); }
void orc_f_dfr_cut(double r, double R1, double R2, double* f, double* dfr) {
  orc::f_dfr_cut(*f, *dfr, r, R1, R2);
}
void orc_find_distance(const double* v1, const double* v2, const double* box, double* dr, double* dr2) {
  orc::Cell c;
  for (int k = 0; k < 3; ++k) {
    c.box[k] = box[k];
    c.half[k] = 0.5 * box[k];
  }
  orc::find_distance(dr, *dr2, v1, v2, c);
}

}  // extern "C"

// run_md_simulation.f90:1-77 -- the command-line runner around md().
extern "C" int orc_run_md_simulation(int argc, const char* const* argv) {
  using fortio::Rec;
  const std::string line(80, '_');
  int out_period = 1;
  std::string settings_files_list, settings_filename = "md_run_settings.txt",
                                   all_out_file = "all_out.txt", output_prefix, input_path, out_path;
  int num_threads = omp_get_max_threads();
  std::printf("%s\n", line.c_str());
  for (int i = 1; i < argc; ++i) {
    std::string arg = fortio::to_char(argv[i], 32);
    auto next = [&]() -> std::string { return (i + 1 < argc) ? std::string(argv[++i]) : std::string(); };
    if (arg == "-i" || arg == "--input") {
      settings_filename = next();
    } else if (arg == "-p" || arg == "--prefix") {
      output_prefix = next();
      std::printf("output_prefix:  %s\n", fortio::trim(output_prefix).c_str());
    } else if (arg == "-op" || arg == "--out_period") {
      std::string s = next();
      std::printf("out_period:         %s\n", fortio::trim(s).c_str());
      out_period = static_cast<int>(fortio::to_int(s));
    } else if (arg == "-omp_n" || arg == "--openmp_threads_num") {
      std::string s = next();
      std::printf("openmp_threads_num: %s\n", fortio::trim(s).c_str());
      num_threads = static_cast<int>(fortio::to_int(s));
    } else if (arg == "-ipath" || arg == "--input_path") {
      input_path = next();
      std::printf("input_path:         %s\n", fortio::trim(input_path).c_str());
    } else if (arg == "-ilist" || arg == "--input_list") {
      settings_files_list = next();
      std::printf("input_list:         %s\n", fortio::trim(settings_files_list).c_str());
    } else if (arg == "-opath" || arg == "--out_path") {
      out_path = next();
      std::printf("out_path:           %s\n", fortio::trim(out_path).c_str());
    } else if (arg == "-ofile" || arg == "--all_out_file") {
      all_out_file = next();
      std::printf("all_out_file:   %s\n", fortio::trim(all_out_file).c_str());
    }
  }
  auto run_one = [&](const std::string& settings, const std::string& prefix, FILE* all_out) -> int {
    orc::Sim s;
    s.input_path = input_path;
    s.settings_filename = settings;
    s.output_prefix = prefix;
    s.out_period = out_period;
    s.num_threads = num_threads;
    s.rand_seed = 1;
    s.write_files = true;
    s.out_file = stdout;
    s.all_out_file = all_out;
    omp_set_num_threads(num_threads);
    try {
      s.setup();
      while (!s.finished) s.step();
      s.finish();
    } catch (const orc::Stop& e) {
      std::fflush(stdout);
      std::fprintf(stdout, " %s\n", e.what());
      return e.code;
    } catch (const std::exception& e) {
      std::fprintf(stdout, " %s\n", e.what());
      return orc::E_IO;
    }
    std::fflush(stdout);
    return 0;
  };
  int rc = 0;
  if (!settings_files_list.empty()) {
    fortio::ListReader lst;
    if (!lst.open(input_path + settings_files_list)) {
      std::fprintf(stderr, "cannot open %s\n", (input_path + settings_files_list).c_str());
      return orc::E_IO;
    }
    FILE* all_out = std::fopen((out_path + all_out_file).c_str(), "w");
    if (!all_out) return orc::E_IO;
    long long set_num = fortio::to_int(lst.read_items(1)[0].s);
    for (long long k = 1; k <= set_num && rc == 0; ++k) {
      auto it = lst.read_items(2);
      std::string sf = fortio::to_char(it[0].s, 128), str = fortio::to_char(it[1].s, 128);
      std::string prefix = fortio::trim(out_path) + fortio::trim(str);
      std::printf("%s\n", line.c_str());
      std::printf("%s\n", Rec().i(k, 6).a("\t").a(sf, 32, 128).a(prefix, 32, 128).s.c_str());
      rc = run_one(sf, prefix, all_out);
      std::fputs("\n", all_out);
      std::printf("%s\n", line.c_str());
    }
    std::fclose(all_out);
  } else {
    std::printf("%s\n", line.c_str());
    rc = run_one(settings_filename, output_prefix, nullptr);
    std::printf("\n");
    std::printf("%s\n", line.c_str());
  }
  std::printf("%s\n", line.c_str());
  std::fflush(stdout);
  return rc;
}

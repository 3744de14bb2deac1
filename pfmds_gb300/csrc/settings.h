// PFMDS input files: the fixed-order settings file, the potential parameter files
// and the extended .xyz file.
//
// The read order follows md() in md_simulation.f90:48-94 item by item, including the
// reads done inside create_groups (md_interactions.f90:38-57), create_interactions
// (md_interactions.f90:59-136), read_integrator_params (md_read_write.f90:10-16),
// read_box_size / read_particles (md_read_write.f90:22-61) and the
// read_*_parameters routines of the six supported interactions.  The text md()
// echoes to its output unit while it reads is rebuilt here byte for byte, so a
// driver only has to print `echo`.  Parameter names in the settings file are not
// checked, only their order matters (as in the reference).
#pragma once

#include <algorithm>
#include <cmath>
#include <string>
#include <thread>
#include <vector>

#include "fortio.h"

namespace pfmd_io {

struct NLSpec {
  int g1 = 0, g2 = 0;  // 1-based group numbers
  int nmax = 0;
  double r_cut = 0.0;
  long long period = 1;
};

enum InterKind { K_LJ = 0, K_LJ1G = 1, K_LJC = 2, K_MORSEC = 3, K_RJL = 4, K_TB = 5, K_REBOSC = 6 };

struct InteractionSpec {
  std::string name;        // lj lj1g ljc morsec rjl tb
  std::string param_file;  // as written in the settings file
  InterKind kind = K_LJ;
  int nl_n = 0;
  std::vector<NLSpec> nl;
  // parameters in the order of the parameter file:
  //  lj, lj1g : eps sig R1 R2
  //  ljc      : eps sig delt R1 R2
  //  morsec   : d r a delt R1 R2
  //  rjl      : A0 xi p q r0 R1 R2
  //  tb       : d s b r0 delt a0 c0 d0 R1 R2
  std::vector<double> p;
  bool simplified = false;  // ljc / morsec
};

struct IntegratorSpec {
  std::string name;  // nve nvt nvms (anything else behaves as nve)
  double dt = 0.0;
  long long l = 0, period_snapshot = 1, period_log = 1;
};

struct NHCSpec {
  int group = 0;
  double temperature = 0.0;
  int M = 1;
  double q1 = 0.0;
};

struct GroupChange {
  int from = 0, to = 0;
  long long ts1 = 0, ts2 = 0, frec = 1;
};

struct XYZ {
  int N = 0;
  double box[3] = {0, 0, 0};
  std::vector<double> pos, vel, mass;  // pos/vel: xyz interleaved, 3*N
  std::vector<std::string> types;
};

struct Settings {
  long long md_step_limit = 0;
  std::string logfilename, init_xyz_filename;
  bool new_velocities = false;
  long long zero_momentum_period = 1;
  int particle_types_num = 0;
  std::vector<std::vector<std::string>> group_types;  // [group][type]
  int all_moving = 0, xyz_moving = 0, z_moving = 0, all_atoms = 0, traj_group = 0;
  long long period_traj = 1;
  std::vector<GroupChange> changes;
  bool invert_z_vel = false;
  std::vector<IntegratorSpec> integrators;  // 1..n (index 0 of the reference is implicit)
  double ms_de = 0.0;
  std::vector<NHCSpec> nhc;
  double initial_temperature = 0.0;
  std::vector<InteractionSpec> interactions;
  XYZ xyz;
  std::string echo;  // what md() writes to its output unit while reading
};

inline int count_group(const XYZ& x, const std::vector<std::string>& names) {
  int n = 0;
  for (const auto& nm : names)
    for (const auto& t : x.types)
      if (t == nm) ++n;
  return n;
}

// read_box_size + read_particles (md_read_write.f90:22-61)
inline XYZ read_xyz(const std::string& path) {
  XYZ x;
  fortio::ListReader r;
  if (!r.open(path)) throw fortio::ReadError("cannot open " + path);
  {
    r.skip_record();
    auto it = r.read_items(10);
    double bm[9];
    for (int k = 0; k < 9; ++k) bm[k] = it[k + 1].set ? fortio::to_real(it[k + 1].s) : 0.0;
    x.box[0] = bm[0];
    x.box[1] = bm[4];
    x.box[2] = bm[8];
  }
  fortio::ListReader r2;
  r2.open(path);
  auto n = r2.read_items(1);
  x.N = static_cast<int>(fortio::to_int(n[0].s));
  if (x.N < 0) throw fortio::ReadError("negative particle count in " + path);
  x.pos.resize(3 * static_cast<size_t>(x.N));
  x.vel.resize(3 * static_cast<size_t>(x.N));
  x.mass.resize(static_cast<size_t>(x.N));
  x.types.resize(static_cast<size_t>(x.N));
  r2.skip_record();
  for (int i = 0; i < x.N; ++i) {
    auto it = r2.read_items(8);
    for (int k = 0; k < 3; ++k) x.pos[3 * i + k] = fortio::to_real(it[k].s);
    for (int k = 0; k < 3; ++k) x.vel[3 * i + k] = fortio::to_real(it[3 + k].s);
    x.mass[i] = fortio::to_real(it[6].s);
    x.types[i] = fortio::to_char(it[7].s, 32);
  }
  return x;
}

inline void read_params(InteractionSpec& in, const std::string& path) {
  fortio::ListReader r;
  if (!r.open(path)) throw fortio::ReadError("cannot open " + path);
  auto reals = [&](size_t n) {
    auto it = r.read_items(n);
    for (size_t k = 0; k < n; ++k) in.p.push_back(it[k].set ? fortio::to_real(it[k].s) : 0.0);
  };
  switch (in.kind) {
    case K_LJ:
    case K_LJ1G:  // LennardJones.f90:12-20, LennardJones_1g.f90:14-26
      reals(2);
      reals(2);
      break;
    case K_LJC:  // LennardJonesCosine.f90:14-24
      reals(3);
      reals(2);
      in.simplified = fortio::to_logical(r.read_items(1)[0].s);
      break;
    case K_MORSEC:  // MorseCosine.f90:14-24
      reals(4);
      reals(2);
      in.simplified = fortio::to_logical(r.read_items(1)[0].s);
      break;
    case K_RJL:  // RosatoGuillopeLegrand.f90:12-21
      reals(5);
      reals(2);
      break;
    case K_TB:  // TersoffBrenner.f90:13-24
      reals(8);
      reals(2);
      break;
    case K_REBOSC:  // REBOsolidcarbon.f90:12-25: A Q alpha / B / beta / T / g / R1 R2
      reals(3);
      reals(3);
      reals(3);
      reals(1);
      reals(6);
      reals(2);
      break;
  }
}

// The settings file, in md()'s read order.  Throws fortio::ReadError on malformed
// input and std::runtime_error with the reference's message on semantic errors.
// `S` is filled as reading proceeds, so S.echo holds what md() had echoed when a
// read fails.
inline void read_settings(const std::string& input_path, const std::string& settings_filename, Settings& S) {
  using namespace fortio;
  std::string& E = S.echo;
  auto nl = [&](const std::string& s) { E += s + "\n"; };
  ListReader r;
  if (!r.open(input_path + settings_filename))
    throw ReadError("cannot open settings file " + input_path + settings_filename);
  nl(std::string("settings_filename: ") + trim(settings_filename));
  auto str128 = [](const std::string& t) { return to_char(t, 128); };
  {
    auto it = r.read_items(2);
    S.md_step_limit = to_int(it[1].s);
    nl(Rec().a(str128(it[0].s), 32, 128).i(S.md_step_limit, 12).s);
  }
  {
    auto it = r.read_items(2);
    S.logfilename = to_char(it[1].s, 128);
    nl(Rec().a(str128(it[0].s), 32, 128).a("\t").a(trim(S.logfilename)).s);
  }
  {
    auto it = r.read_items(2);
    S.init_xyz_filename = to_char(it[1].s, 128);
    nl(Rec().a(str128(it[0].s), 32, 128).a("\t").a(trim(S.init_xyz_filename)).s);
  }
  S.xyz = read_xyz(input_path + S.init_xyz_filename);
  nl(Rec().a("box_size: ").f(S.xyz.box[0], 16, 6).f(S.xyz.box[1], 16, 6).f(S.xyz.box[2], 16, 6).s);
  nl(Rec().a("particles_num: ").i(S.xyz.N, 12).s);
  {
    auto it = r.read_items(2);
    S.new_velocities = to_logical(it[1].s);
    nl(Rec().a(str128(it[0].s), 32, 128).l(S.new_velocities, 8).s);
  }
  {
    auto it = r.read_items(2);
    S.zero_momentum_period = to_int(it[1].s);
    nl(Rec().a(str128(it[0].s), 32, 128).i(S.zero_momentum_period, 12).s);
  }
  // create_groups (md_interactions.f90:38-57)
  int groups_num = 0;
  {
    auto it = r.read_items(2);
    S.particle_types_num = static_cast<int>(to_int(it[1].s));
    nl(Rec().a(str128(it[0].s), 32, 128).i(S.particle_types_num, 12).s);
    auto it2 = r.read_items(2);
    groups_num = static_cast<int>(to_int(it2[1].s));
    nl(Rec().a(str128(it2[0].s), 32, 128).i(groups_num, 12).s);
  }
  for (int g = 0; g < groups_num; ++g) {
    auto it = r.read_items(1 + static_cast<size_t>(S.particle_types_num));
    std::vector<std::string> names;
    for (int t = 0; t < S.particle_types_num; ++t) names.push_back(to_char(it[1 + t].s, 32));
    S.group_types.push_back(names);
    Rec rec;
    rec.i(g + 1, 6).a(" ");
    for (const auto& n : names) rec.a(n, 12, 32);
    rec.i(count_group(S.xyz, names), 9);
    nl(rec.s);
  }
  auto read_int_line = [&](long long& v) {
    auto it = r.read_items(2);
    v = to_int(it[1].s);
    nl(Rec().a(str128(it[0].s), 32, 128).i(v, 12).s);
  };
  long long t;
  read_int_line(t);
  S.all_moving = static_cast<int>(t);
  read_int_line(t);
  S.xyz_moving = static_cast<int>(t);
  read_int_line(t);
  S.z_moving = static_cast<int>(t);
  read_int_line(t);
  S.all_atoms = static_cast<int>(t);
  read_int_line(t);
  S.traj_group = static_cast<int>(t);
  read_int_line(S.period_traj);
  long long change_group_num = 0;
  read_int_line(change_group_num);
  for (long long c = 0; c < change_group_num; ++c) {
    GroupChange gc;
    auto it = r.read_items(3);
    gc.from = static_cast<int>(to_int(it[1].s));
    gc.to = static_cast<int>(to_int(it[2].s));
    nl(Rec().a(str128(it[0].s), 32, 128).i(gc.from, 12).i(gc.to, 12).s);
    auto it2 = r.read_items(4);
    gc.ts1 = to_int(it2[1].s);
    gc.ts2 = to_int(it2[2].s);
    gc.frec = to_int(it2[3].s);
    nl(Rec().a(str128(it2[0].s), 32, 128).i(gc.ts1, 12).i(gc.ts2, 12).i(gc.frec, 12).s);
    S.changes.push_back(gc);
  }
  {
    auto it = r.read_items(2);
    S.invert_z_vel = to_logical(it[1].s);
    nl(Rec().a(str128(it[0].s), 32, 128).l(S.invert_z_vel, 8).s);
  }
  long long integrators_num = 0;
  read_int_line(integrators_num);
  {
    std::string hdr = r.read_line();
    nl(fmt_a(to_char(hdr, 128), -1, 128));
  }
  for (long long k = 0; k < integrators_num; ++k) {
    IntegratorSpec is;
    auto it = r.read_items(5);
    is.name = to_char(it[0].s, 32);
    is.dt = to_real(it[1].s);
    is.l = to_int(it[2].s);
    is.period_snapshot = to_int(it[3].s);
    is.period_log = to_int(it[4].s);
    nl(Rec()
           .a("  ")
           .a(is.name, 6, 32)
           .f(is.dt, 10, 5)
           .i(is.l, 9)
           .i(is.period_snapshot, 9)
           .i(is.period_log, 9)
           .s);
    S.integrators.push_back(is);
  }
  {
    auto it = r.read_items(2);
    S.ms_de = to_real(it[1].s);
    nl(Rec().a(str128(it[0].s), 32, 128).es(S.ms_de, 16, 6).s);
  }
  long long nhc_num = 0;
  read_int_line(nhc_num);
  for (long long k = 0; k < nhc_num; ++k) {
    NHCSpec h;
    auto it = r.read_items(4);
    h.group = static_cast<int>(to_int(it[0].s));
    h.temperature = to_real(it[1].s);
    h.M = static_cast<int>(to_int(it[2].s));
    h.q1 = to_real(it[3].s);
    nl(Rec().i(h.group, 6).f(h.temperature, 16, 6).i(h.M, 6).f(h.q1, 16, 6).s);
    int L = (h.group >= 1 && h.group <= groups_num)
                ? count_group(S.xyz, S.group_types[static_cast<size_t>(h.group - 1)])
                : 0;
    // set_nose_hoover_chain (md_integrators.f90:187)
    if (L < 1 || h.q1 < 0.0 || h.temperature < 0.0) {
      S.nhc.push_back(h);
      throw std::runtime_error("error: wrong nhc parameters");
    }
    S.nhc.push_back(h);
  }
  {
    auto it = r.read_items(2);
    S.initial_temperature = to_real(it[1].s);
    nl(Rec().a(str128(it[0].s), 32, 128).f(S.initial_temperature, 16, 6).s);
  }
  // create_interactions (md_interactions.f90:59-136)
  long long inter_n = 0;
  read_int_line(inter_n);
  for (long long k = 0; k < inter_n; ++k) {
    InteractionSpec in;
    auto it = r.read_items(2);
    in.name = to_char(it[0].s, 32);
    in.param_file = to_char(it[1].s, 32);
    if (in.name == "lj") {
      in.kind = K_LJ;
      in.nl_n = 2;
    } else if (in.name == "lj1g") {
      in.kind = K_LJ1G;
      in.nl_n = 1;
    } else if (in.name == "ljc") {
      in.kind = K_LJC;
      in.nl_n = 3;
    } else if (in.name == "morsec") {
      in.kind = K_MORSEC;
      in.nl_n = 3;
    } else if (in.name == "tb") {
      in.kind = K_TB;
      in.nl_n = 1;
    } else if (in.name == "rjl") {
      in.kind = K_RJL;
      in.nl_n = 1;
    } else if (in.name == "rebosc") {
      in.kind = K_REBOSC;
      in.nl_n = 1;
    } else {
      // md_interactions.f90:119-120 prints this and carries on with an unset list
      // count; here the run stops instead.
      throw std::runtime_error("error: unknown interaction name");
    }
    read_params(in, input_path + in.param_file);
    nl(Rec().a(in.name, 32, 32).a(in.param_file, 32, 32).i(in.nl_n, 6).s);
    for (int j = 0; j < in.nl_n; ++j) {
      NLSpec s;
      auto li = r.read_items(5);
      s.g1 = static_cast<int>(to_int(li[0].s));
      s.g2 = static_cast<int>(to_int(li[1].s));
      s.nmax = static_cast<int>(to_int(li[2].s));
      s.r_cut = to_real(li[3].s);
      s.period = to_int(li[4].s);
      nl(Rec().i(s.g1, 6).i(s.g2, 6).i(s.nmax, 6).f(s.r_cut, 16, 6).i(s.period, 9).s);
      in.nl.push_back(s);
    }
    S.interactions.push_back(in);
  }
}

// Fw.d appended to out (fortio::fmt_f without temporaries).
inline void put_f(std::string& out, double x, int w, int d) {
  if (!std::isfinite(x)) {
    out += fortio::fmt_f(x, w, d);
    return;
  }
  char buf[512];
  int n = std::snprintf(buf, sizeof buf, "%.*f", d, x);
  const char* s = buf;
  if (n > w) {  // drop the optional leading zero of "0.xxx" / "-0.xxx"
    if (buf[0] == '0' && buf[1] == '.') {
      ++s;
      --n;
    } else if (buf[0] == '-' && buf[1] == '0' && buf[2] == '.') {
      buf[1] = '-';
      ++s;
      --n;
    }
  }
  if (n > w) {
    out.append(static_cast<size_t>(w), '*');
    return;
  }
  out.append(static_cast<size_t>(w - n), ' ');
  out.append(s, static_cast<size_t>(n));
}

// The per-atom lines of a file, line(k, out) for k = 0..n-1, formatted by up to
// 16 threads in contiguous chunks when n is large; the text is that of one pass.
template <class F>
inline std::string atom_lines(int n, F line) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = n < 8192 ? 1 : static_cast<int>(std::min(16u, hw));
  std::vector<std::string> part(static_cast<size_t>(nt));
  auto run = [&](int t) {
    const int k0 = static_cast<int>(static_cast<long long>(n) * t / nt);
    const int k1 = static_cast<int>(static_cast<long long>(n) * (t + 1) / nt);
    part[static_cast<size_t>(t)].reserve(static_cast<size_t>(k1 - k0) * 240);
    for (int k = k0; k < k1; ++k) line(k, part[static_cast<size_t>(t)]);
  };
  if (nt == 1) {
    run(0);
    return std::move(part[0]);
  }
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(run, t);
  run(0);
  for (auto& x : th) x.join();
  size_t tot = 0;
  for (const auto& p : part) tot += p.size();
  std::string out;
  out.reserve(tot);
  for (const auto& p : part) out += p;
  return out;
}

// write_particle_group (md_read_write.f90:65-83): a new .xyz file with a group's atoms.
inline std::string xyz_snapshot_text(const double box[3], int n, const int* idx, const double* pos,
                                     const double* vel, const double* mass,
                                     const std::vector<std::string>& types) {
  using namespace fortio;
  std::string out;
  out += list_int(n) + "\n";
  Rec h;
  h.a("Lattice=\"");
  h.f(box[0], 16, 6).f(0.0, 16, 6).f(0.0, 16, 6).f(0.0, 16, 6).f(box[1], 16, 6);
  h.f(0.0, 16, 6).f(0.0, 16, 6).f(0.0, 16, 6).f(box[2], 16, 6);
  h.a(" \" Properties=pos:R:3:vel:R:3:mass:R:1:species:S:1");
  out += h.s + "\n";
  out += atom_lines(n, [&](int k, std::string& o) {
    const int i = idx[k];
    for (int c = 0; c < 3; ++c) put_f(o, pos[3 * i + c], 27, 16);
    for (int c = 0; c < 3; ++c) put_f(o, vel[3 * i + c], 27, 16);
    put_f(o, mass[i], 27, 16);
    o += "    ";
    o += fmt_a(types[static_cast<size_t>(i)], -1, 32);
    o += "\n";
  });
  return out;
}

// write_particle_group_append (md_read_write.f90:86-107): one trajectory frame.
inline std::string xyz_traj_frame_text(const double box[3], int n, const int* idx,
                                       const double* pos, const double* vel, const double* mass,
                                       const std::vector<std::string>& types, long long md_step) {
  using namespace fortio;
  std::string out;
  if (n <= 0) return out;
  out += list_int(n) + "\n";
  Rec h;
  h.a("time_step: ").i(md_step, 9).a("    Lattice=\"");
  h.f(box[0], 10, 4).f(0.0, 10, 4).f(0.0, 10, 4).f(0.0, 10, 4).f(box[1], 10, 4);
  h.f(0.0, 10, 4).f(0.0, 10, 4).f(0.0, 10, 4).f(box[2], 10, 4);
  h.a(" \" Properties=pos:R:3:vel:R:3:mass:R:1:species:S:1");
  out += h.s + "\n";
  out += atom_lines(n, [&](int k, std::string& o) {
    const int i = idx[k];
    for (int c = 0; c < 3; ++c) put_f(o, pos[3 * i + c], 10, 4);
    for (int c = 0; c < 3; ++c) put_f(o, vel[3 * i + c], 10, 4);
    put_f(o, mass[i], 10, 4);
    o += "    ";
    o += trim(types[static_cast<size_t>(i)]);
    o += "\n";
  });
  return out;
}

}  // namespace pfmd_io

namespace pfmd_io {

// Seeded uniform generator for new Maxwell velocities: the Park-Miller "minimal
// standard" multiplicative congruential generator (Park & Miller, CACM 31(10), 1988),
// x <- 16807 x mod (2^31 - 1), returning x / (2^31 - 1).  PFMDS draws from the
// compiler's RAND intrinsic from every OpenMP thread (md_general.f90:120-136), so
// its velocities depend on the thread count; this generator is one serial stream
// in atom order and is shared by the engine and the oracle.
struct MinStd {
  long long x;
  explicit MinStd(long long seed) {
    x = seed % 2147483647LL;
    if (x <= 0) x += 2147483646LL;
  }
  double next() {
    x = (16807LL * x) % 2147483647LL;
    return static_cast<double>(x) / 2147483647.0;
  }
};

}  // namespace pfmd_io

// The reference's graphene-on-copper analysis and moire fitting programs on top
// of pfmd_md:
//
//  * gr_on_cu_analysis (graphene_on_surface_analysis.f90:8-29): z statistics
//    (mean, minimum, maximum above a height z; position_analysis,
//    md_general.f90:400-421) of the carbon types 'C', 'C_a', 'C_b' and of the
//    copper types 'CU', 'CU_fixed' of an .xyz file;
//  * run_gr_analysis (runners/run_gr_analysis.f90:1-46): that analysis over a
//    list of files;
//  * run_gr_moire_fitting (runners/run_gr_moire_fitting.f90:1-110 with
//    fit_gr_moire.f90:16-184): a golden-section fit, parameter by parameter, of
//    the ljc or morsec coupling to a binding energy per carbon atom and the
//    graphene corrugation of two systems.
//
// Each error evaluation runs two md() simulations.  Evaluations that do not
// depend on each other run at the same time, each md() on its own host thread
// with its own context and stream on the GPU: the two systems of one evaluation,
// and the four evaluations that open the search of each parameter.  The
// reference stages an evaluation's inputs by renaming files (its structure and
// its parameter file under the names the settings use); here every run gets the
// same contents under the same names through a per-thread input overlay
// (fortio::t_overlay), so concurrent runs never share a file.  Their standard
// output is captured per run and written in the reference's order.
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pfmd.h"
#include "settings.h"

namespace pfmd {
namespace fit {

using fortio::Rec;

// Fortran character comparison: the shorter operand is padded with blanks.
static bool feq(const std::string& a, const std::string& b) {
  const size_t n = std::max(a.size(), b.size());
  for (size_t i = 0; i < n; ++i) {
    const char x = i < a.size() ? a[i] : ' ', y = i < b.size() ? b[i] : ' ';
    if (x != y) return false;
  }
  return true;
}

// read_particles (md_read_write.f90:42-61): the count, a skipped record, then per
// atom position, velocity, mass and type.
struct Particles {
  std::vector<double> pos;
  std::vector<std::string> types;
};
static Particles read_particles(const std::string& path) {
  fortio::ListReader r;
  if (!r.open(path)) throw fortio::ReadError("cannot open " + path);
  Particles p;
  const long long n = fortio::to_int(r.read_items(1)[0].s);
  r.skip_record();
  for (long long i = 0; i < n; ++i) {
    auto it = r.read_items(8);
    for (int k = 0; k < 3; ++k) p.pos.push_back(fortio::to_real(it[static_cast<size_t>(k)].s));
    p.types.push_back(fortio::to_char(it[7].s, 32));
  }
  return p;
}

// create_particle_group (md_general.f90:57-80): type by type, atoms in file order.
static std::vector<int> group_of(const Particles& p, const std::vector<std::string>& names) {
  std::vector<int> idx;
  for (const auto& nm : names)
    for (size_t i = 0; i < p.types.size(); ++i)
      if (feq(p.types[i], nm)) idx.push_back(static_cast<int>(i));
  return idx;
}

// position_analysis (md_general.f90:400-421) along z.
static void position_analysis(const Particles& p, const std::vector<int>& g, double minimum, double maximum,
                              double& av, double& mi, double& ma) {
  long long k = 0;
  av = 0.0;
  mi = maximum;
  ma = minimum;
  for (int i : g) {
    const double z = p.pos[3 * static_cast<size_t>(i) + 2];
    if (z < maximum && z > minimum) {
      av = av + z;
      ++k;
      if (z > ma) ma = z;
      if (z < mi) mi = z;
    }
  }
  av = av / static_cast<double>(k);
}

static void gr_on_cu_analysis(const std::string& path, double z, double arr1[3], double arr2[3]) {
  const Particles p = read_particles(path);
  position_analysis(p, group_of(p, {"C", "C_a", "C_b"}), z, 1000.0, arr1[0], arr1[1], arr1[2]);
  position_analysis(p, group_of(p, {"CU", "CU_fixed", "#"}), z, 1000.0, arr2[0], arr2[1], arr2[2]);
}

// ---------------------------------------------------------------------------
// the fitting run
// ---------------------------------------------------------------------------
struct Eval {
  long long sim = 0;
  double params[4] = {0, 0, 0, 0};
  bool from_init = true;
  double error = 0.0;
  std::string out;  // standard output of this evaluation, in the reference's order
  int rc = PFMD_OK;
};

struct Fit {
  std::string input_path, out_path, interaction, prefix, param_file;
  std::string settings[2], start_xyz[2], final_file[2], xyz_file[2];
  long long c_num[2] = {0, 0};
  double zero_level[2] = {0, 0}, grd0[2] = {0, 0}, rcut[2] = {0, 0};
  double z = 0.0, be0 = 0.0;
  bool simplified = false;
  double init_min[4] = {0, 0, 0, 0}, init_max[4] = {0, 0, 0, 0};
  long long sim_num = 0;
  int out_period = 1, threads = 1;
  pfmd_options base{};
  FILE* oid = nullptr;
  std::string line = std::string(80, '_');

  static void say(const std::string& s) { std::fputs((s + "\n").c_str(), stdout); }

  // set_fitting_parameters (fit_gr_moire.f90:121-182)
  void setup(const std::string& fpfn) {
    fortio::ListReader r;
    if (!r.open(fpfn)) throw fortio::ReadError("cannot open " + fpfn);
    auto fixed16 = [&](std::string& label, std::string& value) {  // '(A16,A)'
      const std::string ln = r.read_line();
      label = ln.substr(0, std::min<size_t>(16, ln.size()));
      value = ln.size() > 16 ? ln.substr(16) : std::string();
      say(" " + fortio::trim(label) + "  " + fortio::trim(value));
    };
    std::string lab;
    fixed16(lab, input_path);
    fixed16(lab, out_path);
    input_path = fortio::trim(input_path);
    out_path = fortio::trim(out_path);
    auto str = [&](std::string& v) {
      auto it = r.read_items(2);
      v = fortio::trim(fortio::to_char(it[1].s, 256));
      say(" " + fortio::trim(fortio::to_char(it[0].s, 256)) + "  " + v);
    };
    auto num = [&](double& v) {
      auto it = r.read_items(2);
      v = fortio::to_real(it[1].s);
      say(" " + fortio::trim(fortio::to_char(it[0].s, 256)) + "  " + fortio::list_real(v));
    };
    auto inum = [&](long long& v) {
      auto it = r.read_items(2);
      v = fortio::to_int(it[1].s);
      say(" " + fortio::trim(fortio::to_char(it[0].s, 256)) + "  " + fortio::list_int(v));
    };
    str(interaction);
    str(prefix);
    for (int i = 0; i < 2; ++i) {
      str(settings[i]);
      str(start_xyz[i]);
      inum(c_num[i]);
      num(zero_level[i]);
      str(final_file[i]);
    }
    std::string min_file, max_file;
    str(min_file);
    str(max_file);
    num(z);
    num(be0);
    num(grd0[0]);
    num(grd0[1]);
    if (interaction != "ljc" && interaction != "morsec")
      throw fortio::ReadError("the fitted interaction must be ljc or morsec, not " + interaction);
    simplified = false;
    {
      fortio::ListReader m;
      if (!m.open(input_path + min_file)) throw fortio::ReadError("cannot open " + input_path + min_file);
      auto it = m.read_items(interaction == "ljc" ? 3 : 4);
      if (interaction == "ljc") {
        init_min[2] = fortio::to_real(it[0].s), init_min[0] = fortio::to_real(it[1].s);
        init_min[1] = fortio::to_real(it[2].s), init_min[3] = 0.0;
      } else {
        init_min[2] = fortio::to_real(it[0].s), init_min[0] = fortio::to_real(it[1].s);
        init_min[3] = fortio::to_real(it[2].s), init_min[1] = fortio::to_real(it[3].s);
      }
      auto rc = m.read_items(2);
      rcut[0] = fortio::to_real(rc[0].s);
      rcut[1] = fortio::to_real(rc[1].s);
    }
    {
      fortio::ListReader m;
      if (!m.open(input_path + max_file)) throw fortio::ReadError("cannot open " + input_path + max_file);
      auto it = m.read_items(interaction == "ljc" ? 3 : 4);
      if (interaction == "ljc") {
        init_max[2] = fortio::to_real(it[0].s), init_max[0] = fortio::to_real(it[1].s);
        init_max[1] = fortio::to_real(it[2].s), init_max[3] = 0.0;
      } else {
        init_max[2] = fortio::to_real(it[0].s), init_max[0] = fortio::to_real(it[1].s);
        init_max[3] = fortio::to_real(it[2].s), init_max[1] = fortio::to_real(it[3].s);
      }
    }
    sim_num = 0;
    // the structure file of each system (third record of its settings) and, from
    // the first settings file, the parameter file of the fitted interaction
    for (int i = 0; i < 2; ++i) {
      fortio::ListReader s;
      if (!s.open(input_path + settings[i])) throw fortio::ReadError("cannot open " + input_path + settings[i]);
      s.skip_record();
      s.skip_record();
      xyz_file[i] = fortio::trim(fortio::to_char(s.read_items(2)[1].s, 256));
      if (i != 0) continue;
      for (;;) {
        std::string ln = s.read_line();
        ln.resize(std::max<size_t>(ln.size(), 128), ' ');
        int skip = 0;
        if (feq(ln.substr(0, 3), interaction)) skip = 3;
        else if (feq(ln.substr(0, 6), interaction)) skip = 6;
        if (skip) {
          fortio::ListReader t;
          t.from_string(ln.substr(static_cast<size_t>(skip)));
          param_file = fortio::trim(fortio::to_char(t.read_items(1)[0].s, 256));
          break;
        }
      }
    }
  }

  std::string op_of(long long sim) const {
    return out_path + prefix + fortio::fmt_i0pad(sim, 6, 6) + "_";
  }

  // The parameter file an evaluation writes (fit_gr_moire.f90:27-45), under the
  // name the reference renames it to when the evaluation ends (:108).
  void write_params(const Eval& e) const {
    const std::string fn = input_path + fortio::fmt_i0pad(e.sim, 6, 6) + param_file;
    std::string t = " ";
    if (interaction == "ljc")
      t += fortio::list_real(e.params[2]) + fortio::list_real(e.params[0]) + fortio::list_real(e.params[1]);
    else
      t += fortio::list_real(e.params[2]) + fortio::list_real(e.params[0]) + fortio::list_real(e.params[3]) +
           fortio::list_real(e.params[1]);
    t += "\n " + fortio::list_real(rcut[0]) + fortio::list_real(rcut[1]) + "\n" + fortio::list_logical(simplified) +
         "\n";
    FILE* f = std::fopen(fn.c_str(), "w");
    if (!f) throw fortio::ReadError("cannot open " + fn);
    std::fputs(t.c_str(), f);
    std::fclose(f);
  }

  // One md() of evaluation e, system i (fit_gr_moire.f90:50-70), on the calling
  // thread: its inputs through the overlay, its output text into *text.
  int run_md(const Eval& e, int i, std::string* text) const {
    const std::string start =
        e.from_init ? input_path + start_xyz[i] : op_of(e.sim - 1) + "final_" + xyz_file[i];
    fortio::t_overlay.clear();
    fortio::t_overlay.emplace_back(input_path + xyz_file[i], start);
    fortio::t_overlay.emplace_back(input_path + param_file,
                                   input_path + fortio::fmt_i0pad(e.sim, 6, 6) + param_file);
    const std::string op = op_of(e.sim);
    FILE* fin = std::fopen((op + final_file[i]).c_str(), "w");
    FILE* cap = std::tmpfile();
    int rc = PFMD_E_IO;
    if (fin && cap) {
      pfmd_options o = base;
      o.out_fd = fileno(cap);
      o.all_out_fd = fileno(fin);
      o.output_prefix = op.c_str();
      o.write_files = 1;
      o.out_period = out_period;
      o.num_threads = threads;
      rc = pfmd_md(input_path.c_str(), settings[i].c_str(), &o);
      std::fflush(cap);
      std::rewind(cap);
      char buf[1 << 16];
      size_t k;
      while ((k = std::fread(buf, 1, sizeof buf, cap)) > 0) text->append(buf, k);
    } else {
      *text += " cannot open " + op + final_file[i] + "\n";
    }
    if (cap) std::fclose(cap);
    if (fin) std::fclose(fin);
    fortio::t_overlay.clear();
    return rc;
  }

  // calc_error (fit_gr_moire.f90:16-111) for a set of independent evaluations.
  void evaluate(std::vector<Eval>& ev) {
    for (auto& e : ev) {
      e.sim = ++sim_num;
      write_params(e);
    }
    std::vector<std::string> text(2 * ev.size());
    std::vector<int> rc(2 * ev.size(), PFMD_OK);
    {
      std::vector<std::thread> th;
      for (size_t k = 0; k < ev.size(); ++k)
        for (int i = 0; i < 2; ++i)
          th.emplace_back([&, k, i] { rc[2 * k + i] = run_md(ev[k], i, &text[2 * k + i]); });
      for (auto& t : th) t.join();
    }
    for (size_t k = 0; k < ev.size(); ++k) {
      Eval& e = ev[k];
      std::string& out = e.out;
      Rec fl;  // this evaluation's line of fit_out.txt
      out += "\n " + input_path + param_file + "\n";
      if (interaction == "ljc") {
        out += fortio::list_int(e.sim) + fortio::list_real(e.params[2]) + fortio::list_real(e.params[0]) +
               fortio::list_real(e.params[1]) + "\n";
        fl.i(e.sim, 6).f(e.params[2], 21, 6).f(e.params[0], 21, 6).f(e.params[1], 21, 6);
      } else {
        out += fortio::list_int(e.sim) + fortio::list_real(e.params[2]) + fortio::list_real(e.params[0]) +
               fortio::list_real(e.params[3]) + fortio::list_real(e.params[1]) + "\n";
        fl.i(e.sim, 6).f(e.params[2], 21, 6).f(e.params[0], 21, 6).f(e.params[3], 21, 6).f(e.params[1], 21, 6);
      }
      double error = 0.0;
      for (int i = 0; i < 2; ++i) {
        out += line + "\n" + text[2 * k + i] + line + "\n";
        if (rc[2 * k + i] != PFMD_OK) {
          e.rc = rc[2 * k + i];
          return;
        }
        const std::string op = op_of(e.sim);
        double arr1[3], arr2[3];
        gr_on_cu_analysis(op + "final_" + xyz_file[i], z, arr1, arr2);
        out += " gr_on_cu_analysis:";
        for (double v : arr1) out += fortio::list_real(v);
        for (double v : arr2) out += fortio::list_real(v);
        out += "\n";
        // the analysis goes on the record md() left open in the final file; the
        // total energy is read back from it ('(A61,f20.9,A)')
        {
          FILE* f = std::fopen((op + final_file[i]).c_str(), "a");
          if (!f) throw fortio::ReadError("cannot open " + op + final_file[i]);
          const std::string r =
              Rec().f(arr1[0] - arr2[0], 16, 6).f(arr1[1] - arr2[0], 16, 6).f(arr1[2] - arr2[0], 16, 6).s + "\n";
          std::fputs(r.c_str(), f);
          std::fclose(f);
        }
        fortio::ListReader back;
        if (!back.open(op + final_file[i])) throw fortio::ReadError("cannot open " + op + final_file[i]);
        std::string rec = back.read_line();
        rec.resize(std::max<size_t>(rec.size(), 81), ' ');
        double be = fortio::to_real(rec.substr(61, 20));
        const double bd = arr1[0] - arr2[0];
        const double grd = arr1[2] - arr1[1];
        be = (be - zero_level[i]) / static_cast<double>(c_num[i]);
        fl.f(be, 21, 6).f(bd, 21, 6).f(grd, 21, 6);
        if (i == 0) {
          const double t1 = (be / be0 - 1.0) * (be / be0 - 1.0), t2 = (grd / grd0[0] - 1.0) * (grd / grd0[0] - 1.0);
          error = t1 + t2;
          fl.f(t1, 21, 6).f(t2, 21, 6);
        } else {
          const double t3 = (grd / grd0[1] - 1.0) * (grd / grd0[1] - 1.0);
          error = error + t3;
          fl.f(t3, 21, 6);
        }
      }
      fl.f(error, 21, 6);
      e.error = error;
      std::fputs((fl.s + "\n").c_str(), oid);
      std::fflush(oid);
    }
  }

  // run_gr_moire_fitting.f90:47-101
  int run(double delta_error_gold, double delta_error_fit) {
    const double gold = (std::sqrt(5.0) - 1.0) / (std::sqrt(5.0) + 1.0);
    double min_p[4], max_p[4], params[4], err_arr[4] = {0, 0, 0, 0};
    double error = 0.0, prev_error_fit = 0.0;
    for (int k = 0; k < 4; ++k) {
      min_p[k] = init_min[k];
      max_p[k] = init_max[k];
      params[k] = (init_min[k] + init_max[k]) / 2;
    }
    auto delta = [&] {
      double mx = err_arr[0], mn = err_arr[0];
      for (double v : err_arr) mx = std::max(mx, v), mn = std::min(mn, v);
      return mx - mn;
    };
    // evaluates the given parameter sets (independent of each other) and emits
    // their output in order; returns false on an md() error
    int rc = PFMD_OK;
    auto eval = [&](std::vector<Eval> ev, std::vector<double*> dst) {
      evaluate(ev);
      for (size_t k = 0; k < ev.size(); ++k) {
        std::fputs(ev[k].out.c_str(), stdout);
        if (ev[k].rc != PFMD_OK) {
          rc = ev[k].rc;
          return false;
        }
        *dst[k] = ev[k].error;
      }
      std::fflush(stdout);
      return true;
    };
    auto with = [&](int k, double v, bool from_init) {
      Eval e;
      for (int j = 0; j < 4; ++j) e.params[j] = params[j];
      e.params[k] = v;
      e.from_init = from_init;
      return e;
    };
    while (std::fabs(prev_error_fit - error) > delta_error_fit || sim_num == 0) {
      for (int k = 0; k < 3; ++k) {
        prev_error_fit = error;
        if (sim_num == 0) prev_error_fit = 1000000.0;
        min_p[k] = init_min[k];
        max_p[k] = init_max[k];
        // the four opening points are independent: one concurrent set
        if (!eval({with(k, min_p[k], true), with(k, max_p[k], true),
                   with(k, min_p[k] + (max_p[k] - min_p[k]) * gold, true),
                   with(k, max_p[k] - (max_p[k] - min_p[k]) * gold, true)},
                  {&err_arr[0], &err_arr[3], &err_arr[1], &err_arr[2]}))
          return rc;
        params[k] = max_p[k] - (max_p[k] - min_p[k]) * gold;  // the last point the reference set
        double de = delta();
        say("  delta_error: " + fortio::list_real(de));
        int gold_i = 0;
        while (de > delta_error_gold && gold_i <= 20) {
          ++gold_i;
          if (err_arr[1] < err_arr[2]) {
            err_arr[3] = err_arr[2];
            err_arr[2] = err_arr[1];
            max_p[k] = max_p[k] - (max_p[k] - min_p[k]) * gold;
            params[k] = min_p[k] + (max_p[k] - min_p[k]) * gold;
            if (!eval({with(k, params[k], false)}, {&err_arr[1]})) return rc;
          } else {
            err_arr[0] = err_arr[1];
            err_arr[1] = err_arr[2];
            min_p[k] = min_p[k] + (max_p[k] - min_p[k]) * gold;
            params[k] = max_p[k] - (max_p[k] - min_p[k]) * gold;
            if (!eval({with(k, params[k], false)}, {&err_arr[2]})) return rc;
          }
          de = delta();
          say("  delta_error: " + fortio::list_real(de));
        }
        int loc = 0;  // minloc: the first minimum
        for (int j = 1; j < 4; ++j)
          if (err_arr[j] < err_arr[loc]) loc = j;
        error = err_arr[loc];
        switch (loc) {
          case 1: params[k] = min_p[k] + (max_p[k] - min_p[k]) * gold; break;
          case 2: params[k] = max_p[k] - (max_p[k] - min_p[k]) * gold; break;
          case 0: params[k] = min_p[k]; break;
          default: params[k] = max_p[k]; break;
        }
        std::string s = "  parameters: ";
        for (double v : params) s += fortio::list_real(v);
        say(s);
      }
    }
    return PFMD_OK;
  }
};

}  // namespace fit
}  // namespace pfmd

extern "C" {

int pfmd_gr_on_cu_analysis(const char* xyz_path, double z, double* arr1, double* arr2) {
  if (!xyz_path || !arr1 || !arr2) return PFMD_E_PARAM;
  try {
    pfmd::fit::gr_on_cu_analysis(xyz_path, z, arr1, arr2);
  } catch (const std::exception&) {
    return PFMD_E_IO;
  }
  return PFMD_OK;
}

int pfmd_run_gr_analysis(int argc, const char* const* argv) {
  std::string path, filelist = "filelist.txt", outfilename = "outfilename.txt";
  double z = 0.0;
  for (int i = 1; i < argc; ++i) {
    const std::string arg = fortio::to_char(argv[i], 32);
    auto next = [&]() -> std::string { return (i + 1 < argc) ? std::string(argv[++i]) : std::string(); };
    if (arg == "-path") path = next();
    else if (arg == "-fl") filelist = next();
    else if (arg == "-o") outfilename = next();
    else if (arg == "-z") z = fortio::to_real(next());
  }
  path = fortio::trim(path);
  std::printf(" %s\n %s\n", (path + filelist).c_str(), (path + outfilename).c_str());
  try {
    fortio::ListReader in;
    if (!in.open(path + filelist)) throw fortio::ReadError("cannot open " + path + filelist);
    FILE* out = std::fopen((path + outfilename).c_str(), "w");
    if (!out) throw fortio::ReadError("cannot open " + path + outfilename);
    const long long n = fortio::to_int(in.read_items(1)[0].s);
    std::printf("%s\n", fortio::list_int(n).c_str());
    for (long long i = 1; i <= n; ++i) {
      const std::string fn = fortio::trim(fortio::to_char(in.read_items(1)[0].s, 256));
      double a1[3], a2[3];
      pfmd::fit::gr_on_cu_analysis(path + fn, z, a1, a2);
      std::printf("%s", fortio::fmt_i(i, 10).c_str());
      std::string r = " " + fn + "    ";
      for (double v : a1) r += fortio::list_real(v - a2[0]);
      std::fputs((r + "\n").c_str(), out);
    }
    std::fclose(out);
  } catch (const std::exception& e) {
    std::fflush(stdout);
    std::fprintf(stderr, "%s\n", e.what());
    return PFMD_E_IO;
  }
  std::fflush(stdout);
  return PFMD_OK;
}

int pfmd_run_gr_moire_fitting(int argc, const char* const* argv) {
  pfmd::fit::Fit F;
  pfmd_default_options(&F.base);
  std::string fpfn;
  double de_gold = 0.0, de_fit = 0.0;
  for (int i = 1; i < argc; ++i) {
    const std::string arg = fortio::to_char(argv[i], 32);
    auto next = [&]() -> std::string { return (i + 1 < argc) ? std::string(argv[++i]) : std::string(); };
    try {
      if (arg == "-op" || arg == "--out_period") {
        const std::string s = next();
        F.out_period = static_cast<int>(fortio::to_int(s));
        std::printf("out_period: %s\n", fortio::trim(s).c_str());
      } else if (arg == "-omp_n" || arg == "--openmp_threads_num") {
        const std::string s = next();
        F.threads = static_cast<int>(fortio::to_int(s));
        std::printf("openmp_threads_num: %s\n", fortio::trim(s).c_str());
      } else if (arg == "-fpfn") {
        fpfn = next();
        std::printf("fitting_parameters_file_name: %s\n", fortio::trim(fpfn).c_str());
      } else if (arg == "-delta_error_gold") {
        const std::string s = next();
        de_gold = fortio::to_real(s);
        std::printf("delta_error_gold: %s\n", fortio::trim(s).c_str());
      } else if (arg == "-delta_error_fit") {
        const std::string s = next();
        de_fit = fortio::to_real(s);
        std::printf("delta_error_fit: %s\n", fortio::trim(s).c_str());
      } else if (arg == "-form") {
        F.base.form = next() == "precision" ? PFMD_FORM_PRECISION : PFMD_FORM_PLAIN;
      } else if (arg == "-device") {
        F.base.device = static_cast<int>(fortio::to_int(next()));
      }
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return PFMD_E_PARAM;
    }
  }
  int rc = PFMD_OK;
  try {
    F.setup(fpfn);
    const std::string fo = F.out_path + F.prefix + "fit_out.txt";
    F.oid = std::fopen(fo.c_str(), "w");
    if (!F.oid) throw fortio::ReadError("cannot open " + fo);
    F.say(F.line);
    std::fflush(stdout);
    rc = F.run(de_gold, de_fit);
    std::fclose(F.oid);
    F.oid = nullptr;
  } catch (const std::exception& e) {
    if (F.oid) std::fclose(F.oid);
    std::fflush(stdout);
    std::fprintf(stderr, "%s\n", e.what());
    return PFMD_E_IO;
  }
  F.say(F.line);
  std::fflush(stdout);
  return rc;
}

}  // extern "C"

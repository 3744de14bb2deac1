// run_md_simulation (runners/run_md_simulation.f90:1-77) on top of pfmd_md: the
// same options (-i -p -op -omp_n -ipath -ilist -opath -ofile), the same banner
// lines and the same single-file and list modes.  Extra options of this
// implementation: -form plain|precision (arithmetic form), -graphs 0|1,
// -device n, and -batch, which runs a whole list as one batch on the batched
// kernel (pfmd_batch_run_list: the same files per entry; no per-step output
// blocks).
#include <unistd.h>

#include <cstdio>
#include <string>

#include "../../include/pfmd.h"
#include "settings.h"

extern "C" int pfmd_run_md_simulation(int argc, const char* const* argv) {
  using fortio::Rec;
  const std::string line(80, '_');
  pfmd_options o;
  pfmd_default_options(&o);
  o.out_fd = 1;
  o.write_files = 1;
  std::string settings_files_list, settings_filename = "md_run_settings.txt", all_out_file = "all_out.txt",
                                   output_prefix, input_path, out_path;
  bool batched = false;
  std::string banner;
  auto say = [&](const std::string& s) {
    std::fputs((s + "\n").c_str(), stdout);
  };
  say(line);
  for (int i = 1; i < argc; ++i) {
    std::string arg = fortio::to_char(argv[i], 32);
    auto next = [&]() -> std::string { return (i + 1 < argc) ? std::string(argv[++i]) : std::string(); };
    try {
      if (arg == "-i" || arg == "--input") {
        settings_filename = next();
      } else if (arg == "-p" || arg == "--prefix") {
        output_prefix = next();
        say("output_prefix:  " + fortio::trim(output_prefix));
      } else if (arg == "-op" || arg == "--out_period") {
        std::string s = next();
        say("out_period:         " + fortio::trim(s));
        o.out_period = static_cast<int>(fortio::to_int(s));
      } else if (arg == "-omp_n" || arg == "--openmp_threads_num") {
        std::string s = next();
        say("openmp_threads_num: " + fortio::trim(s));
        o.num_threads = static_cast<int>(fortio::to_int(s));
      } else if (arg == "-ipath" || arg == "--input_path") {
        input_path = next();
        say("input_path:         " + fortio::trim(input_path));
      } else if (arg == "-ilist" || arg == "--input_list") {
        settings_files_list = next();
        say("input_list:         " + fortio::trim(settings_files_list));
      } else if (arg == "-opath" || arg == "--out_path") {
        out_path = next();
        say("out_path:           " + fortio::trim(out_path));
      } else if (arg == "-ofile" || arg == "--all_out_file") {
        all_out_file = next();
        say("all_out_file:   " + fortio::trim(all_out_file));
      } else if (arg == "-form") {
        std::string s = next();
        o.form = (s == "precision") ? PFMD_FORM_PRECISION : PFMD_FORM_PLAIN;
      } else if (arg == "-graphs") {
        o.use_graphs = static_cast<int>(fortio::to_int(next()));
      } else if (arg == "-device") {
        o.device = static_cast<int>(fortio::to_int(next()));
      } else if (arg == "-skin") {
        o.skin_lists = static_cast<int>(fortio::to_int(next()));
      } else if (arg == "-fuse") {
        o.fuse_steps = static_cast<int>(fortio::to_int(next()));
      } else if (arg == "-async_io") {
        o.async_io = static_cast<int>(fortio::to_int(next()));
      } else if (arg == "-batch") {
        batched = true;
      }
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return PFMD_E_PARAM;
    }
  }
  std::fflush(stdout);
  int rc = PFMD_OK;
  if (batched && !settings_files_list.empty()) {
    FILE* all_out = std::fopen((out_path + all_out_file).c_str(), "w");
    if (!all_out) return PFMD_E_IO;
    pfmd_batch* b = nullptr;
    rc = pfmd_batch_create(input_path.c_str(), settings_files_list.c_str(), &o, &b);
    double ms = 0.0;
    if (rc == PFMD_OK) rc = pfmd_batch_run_list(b, out_path.c_str(), fileno(all_out), &ms);
    if (rc == PFMD_OK) {
      int reps = 0;
      long long atoms = 0, steps = 0;
      pfmd_batch_info(b, &reps, &atoms, &steps);
      say(line);
      say(Rec().a("BATCH: ").i(reps, 6).a(" entries").i(atoms, 12).a(" atoms").i(steps, 12).a(" steps").s);
      say(Rec().a("DEVICE TIME: ", 24).f(ms / 1000.0, 10, 2).a(" S ").s);
    } else {
      std::fprintf(stderr, "%s\n", pfmd_batch_errmsg(b));
    }
    pfmd_batch_destroy(b);
    std::fclose(all_out);
  } else if (!settings_files_list.empty()) {
    fortio::ListReader lst;
    if (!lst.open(input_path + settings_files_list)) {
      std::fprintf(stderr, "cannot open %s\n", (input_path + settings_files_list).c_str());
      return PFMD_E_IO;
    }
    FILE* all_out = std::fopen((out_path + all_out_file).c_str(), "w");
    if (!all_out) return PFMD_E_IO;
    long long set_num = 0;
    try {
      set_num = fortio::to_int(lst.read_items(1)[0].s);
    } catch (const std::exception& e) {
      std::fclose(all_out);
      return PFMD_E_IO;
    }
    for (long long k = 1; k <= set_num && rc == PFMD_OK; ++k) {
      std::string sf, str;
      try {
        auto it = lst.read_items(2);
        sf = fortio::to_char(it[0].s, 128);
        str = fortio::to_char(it[1].s, 128);
      } catch (const std::exception& e) {
        rc = PFMD_E_IO;
        break;
      }
      std::string prefix = fortio::trim(out_path) + fortio::trim(str);
      say(line);
      say(Rec().i(k, 6).a("\t").a(sf, 32, 128).a(prefix, 32, 128).s);
      std::fflush(stdout);
      std::fflush(all_out);
      o.output_prefix = prefix.c_str();
      o.all_out_fd = fileno(all_out);
      rc = pfmd_md(input_path.c_str(), sf.c_str(), &o);
      std::fputs("\n", all_out);
      std::fflush(all_out);
      say(line);
    }
    std::fclose(all_out);
  } else {
    say(line);
    std::fflush(stdout);
    o.output_prefix = output_prefix.c_str();
    o.all_out_fd = -1;
    rc = pfmd_md(input_path.c_str(), settings_filename.c_str(), &o);
    std::fflush(stdout);
    say("");
    say(line);
  }
  say(line);
  std::fflush(stdout);
  return rc;
}

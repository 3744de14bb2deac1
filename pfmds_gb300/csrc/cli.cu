// run_md_simulation (runners/run_md_simulation.f90:1-77) on top of pfmd_md: the
// same options (-i -p -op -omp_n -ipath -ilist -opath -ofile), the same banner
// lines and the same single-file and list modes.  Extra options of this
// implementation: -form plain|precision (arithmetic form), -graphs 0|1,
// -device n, and -batch, which runs the entries of a list that the batched
// kernel takes as batches on it (pfmd_batch_run_list: the same files per entry;
// no per-step output blocks) and the others (graphene/Cu, nvms, several chains)
// as independent md() runs, -streams n of them at a time (default 16), each on
// its own host thread with its own stream and graphs; their standard output is
// held and written in list order, as list mode writes it.
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <map>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

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
  int streams = 16;
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
      } else if (arg == "-streams") {
        streams = static_cast<int>(fortio::to_int(next()));
        if (streams < 1) streams = 1;
      }
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return PFMD_E_PARAM;
    }
  }
  std::fflush(stdout);
  int rc = PFMD_OK;
  if (batched && !settings_files_list.empty()) {
    // the entries the batched kernel takes run together, one batch per shared
    // (steps, list period, zero_momentum_period); the others run one by one as
    // in list mode.  Closing records go to all_out in list order.
    fortio::ListReader lst;
    if (!lst.open(input_path + settings_files_list)) {
      std::fprintf(stderr, "cannot open %s\n", (input_path + settings_files_list).c_str());
      return PFMD_E_IO;
    }
    std::vector<std::pair<std::string, std::string>> entries;
    try {
      const long long set_num = fortio::to_int(lst.read_items(1)[0].s);
      for (long long k = 0; k < set_num; ++k) {
        auto it = lst.read_items(2);
        entries.emplace_back(fortio::trim(fortio::to_char(it[0].s, 128)), fortio::trim(fortio::to_char(it[1].s, 128)));
      }
    } catch (const std::exception& e) {
      return PFMD_E_IO;
    }
    const size_t n = entries.size();
    std::vector<std::string> recs(n);
    std::map<std::tuple<long long, int, long long>, std::vector<size_t>> groups;
    std::vector<size_t> single;
    for (size_t k = 0; k < n; ++k) {
      long long steps = 0, zmp = 0;
      int per = 0;
      char why[256];
      if (pfmd_batch_accepts(input_path.c_str(), entries[k].first.c_str(), &steps, &per, &zmp, why, sizeof why) ==
          PFMD_OK)
        groups[std::make_tuple(steps, per, zmp)].push_back(k);
      else
        single.push_back(k);
    }
    auto read_back = [](FILE* f) {
      std::string t;
      std::rewind(f);
      char buf[4096];
      size_t m;
      while ((m = std::fread(buf, 1, sizeof buf, f)) > 0) t.append(buf, m);
      return t;
    };
    for (auto& g : groups) {
      std::vector<const char*> sf, pf;
      for (size_t k : g.second) {
        sf.push_back(entries[k].first.c_str());
        pf.push_back(entries[k].second.c_str());
      }
      FILE* tmp = std::tmpfile();
      if (!tmp) return PFMD_E_IO;
      pfmd_batch* b = nullptr;
      rc = pfmd_batch_create_entries(input_path.c_str(), static_cast<int>(sf.size()), sf.data(), pf.data(), &o, &b);
      double ms = 0.0;
      if (rc == PFMD_OK) rc = pfmd_batch_run_list(b, out_path.c_str(), fileno(tmp), &ms);
      if (rc == PFMD_OK) {
        int reps = 0;
        long long atoms = 0, steps = 0;
        pfmd_batch_info(b, &reps, &atoms, &steps);
        say(line);
        say(Rec().a("BATCH: ").i(reps, 6).a(" entries").i(atoms, 12).a(" atoms").i(steps, 12).a(" steps").s);
        say(Rec().a("DEVICE TIME: ", 24).f(ms / 1000.0, 10, 2).a(" S ").s);
        std::fflush(tmp);
        const std::string t = read_back(tmp);
        size_t pos = 0;
        for (size_t k : g.second) {  // one line per entry, in the batch's order
          const size_t e = t.find('\n', pos);
          recs[k] = t.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
          pos = e == std::string::npos ? t.size() : e + 1;
        }
      } else {
        std::fprintf(stderr, "%s\n", pfmd_batch_errmsg(b));
      }
      pfmd_batch_destroy(b);
      std::fclose(tmp);
      if (rc != PFMD_OK) return rc;
    }
    // The other entries are independent md() runs (run_md_simulation_mpi.f90:74-85
    // gives each its own rank): up to `streams` at a time, each on a host thread
    // with its own engine, stream and graphs, so that small systems fill the GPU
    // together.  No new entry starts after one has failed; the output stops at
    // the first failed entry in list order, as in a one-by-one run.
    struct Single {
      std::string prefix, text;
      int rc = PFMD_OK;
      bool ran = false;
    };
    std::vector<Single> sg(single.size());
    std::atomic<size_t> next_j{0};
    std::atomic<bool> failed{false};
    auto worker = [&] {
      for (size_t j; !failed.load() && (j = next_j.fetch_add(1)) < single.size();) {
        const size_t k = single[j];
        Single& s = sg[j];
        s.ran = true;
        s.prefix = fortio::trim(out_path) + entries[k].second;
        FILE* cap = std::tmpfile();
        FILE* rec = std::tmpfile();
        if (cap && rec) {
          pfmd_options oj = o;
          oj.output_prefix = s.prefix.c_str();
          oj.out_fd = fileno(cap);
          oj.all_out_fd = fileno(rec);
          s.rc = pfmd_md(input_path.c_str(), entries[k].first.c_str(), &oj);
          std::fflush(cap);
          std::fflush(rec);
          s.text = read_back(cap);
          recs[k] = read_back(rec);
          while (!recs[k].empty() && recs[k].back() == '\n') recs[k].pop_back();
        } else {
          s.rc = PFMD_E_IO;
        }
        if (cap) std::fclose(cap);
        if (rec) std::fclose(rec);
        if (s.rc != PFMD_OK) failed.store(true);
      }
    };
    {
      std::vector<std::thread> th;
      const size_t nt = std::min(single.size(), static_cast<size_t>(streams));
      for (size_t t = 0; t < nt; ++t) th.emplace_back(worker);
      for (auto& t : th) t.join();
    }
    for (size_t j = 0; j < single.size(); ++j) {
      const size_t k = single[j];
      const Single& s = sg[j];
      if (!s.ran) return PFMD_E_IO;  // not started: an earlier entry failed
      say(line);
      say(Rec().i(static_cast<long long>(k + 1), 6).a("\t").a(entries[k].first, 32, 128).a(s.prefix, 32, 128).s);
      std::fputs(s.text.c_str(), stdout);
      say(line);
      if (s.rc != PFMD_OK) return s.rc;
    }
    FILE* all_out = std::fopen((out_path + all_out_file).c_str(), "w");
    if (!all_out) return PFMD_E_IO;
    for (const auto& r : recs) std::fputs((r + "\n").c_str(), all_out);
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

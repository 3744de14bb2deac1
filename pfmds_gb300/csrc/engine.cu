// Host engine: md() of PFMDS (md_simulation.f90:19-274) on one GPU.
//
// Set-up reads the reference's input files (settings.h), builds the groups
// (create_particle_group, md_general.f90:57-80), the Nose-Hoover chains, new
// Maxwell velocities when asked, the interactions and their neighbour lists, and
// uploads everything.  The step loop then runs on the device: the host plans runs
// of consecutive steps between host events (log line, output block, snapshot,
// trajectory frame, integrator switch), launches each step's kernels in the
// reference's order -- or replays a captured CUDA graph when the same run of
// steps was seen before -- and synchronises only at the end of a run.  Errors and
// the nvms exit are raised on the device (Ctl::stop) and reported after the run
// with the reference's messages.
#include <unistd.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pfmd.h"
#include "kernels.h"
#include "learned.h"
#include "settings.h"

namespace pfmd {

thread_local long long g_kernel_launches = 0;
WaitHook g_wait_hook;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(call)                                                                                     \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess)                                                                           \
      throw ::pfmd::Error(PFMD_E_CUDA, std::string("CUDA error ") + cudaGetErrorString(e_) + " at " #call); \
  } while (0)

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) CK(cudaMalloc(&p, sizeof(T) * count));
  }
  void zero(cudaStream_t s) {
    if (n) CK(cudaMemsetAsync(p, 0, sizeof(T) * n, s));
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    if (count) CK(cudaMemcpyAsync(p, h, sizeof(T) * count, cudaMemcpyHostToDevice, s));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
};

static const double MASS_COEF = 1.6605389217 / 1.6021765654 * 100.0;
static const double KT_A_DEGREE = 1.3806488 / 1.6021765654 * 1e-4;
static const double MOMENTA_COEF = 1.3806488 / 1.6605389217 * 1e-6;

// Threads per list row: enough threads to fill the GPU (~152 SMs x 32 resident
// warps) when rows are few, but at least ~2 entries per thread, and one thread
// per row for large lists so that a warp reads 32 consecutive rows' slots.
// Two-level lists: the outer list is this much (A) wider than the list, and it
// is rebuilt when an atom moved more than half of it, less a tolerance for the
// FP32 displacement test, since its build.
static constexpr double kOuterMargin = 1.0;
static constexpr double kOuterTol = 1e-3;

static int auto_tpa(int rows, double mean_entries, bool prec) {
  const double want = 152.0 * 32 * 32 / std::max(rows, 1);
  int t = 1;
  // FP32 kernels: the power of two nearest the target (in ratio): 2 for the
  // 65,536-row slab (target 2.4), 8 for the 20,456 graphene rows of the moire's
  // morsec lists (target 7.6; every list at 8 took that step from 337 to 274 us,
  // against 4); FP64 kernels hide pipe latency with more threads: the smallest
  // power of two above the target
  if (prec)
    while (t < 32 && t * 1.4142135623730951 < want) t <<= 1;
  else
    while (t < want && t < 32) t <<= 1;
  while (t > 1 && t > mean_entries / 2.0) t >>= 1;
  // long rows: at most 32 entries per thread, so a thread's chain of dependent
  // gathers stays short
  while (t < 32 && mean_entries / t > 32.0) t <<= 1;
  return t;
}

// The rjl density pass of the precision form has no force write-back and a short
// body: twice the force pass's threads per row (measured faster on the Cu slab at
// 2 -> 4), within the same entries-per-thread floor.
static int pass1_tpa(int tpa, double mean_entries, bool prec) {
  if (!prec) return tpa;
  const int t = std::min(32, 2 * tpa);
  return t > mean_entries / 4.0 ? tpa : t;
}

template <class R>
static void fill_lj(LJc<R>& c, const LJPar& P) {
  c.eps4 = (R)(4.0 * P.eps);
  c.sig = (R)P.sig;
  c.R1 = (R)P.R1;
  c.R2 = (R)P.R2;
  c.inv_w = (R)(1.0 / (P.R2 - P.R1));
  c.c6 = (R)P.c6;
  c.c12 = (R)P.c12;
  c.c6t6 = (R)P.c6t6;
  c.c12t12 = (R)P.c12t12;
}
void derive(LJPar& P) {
  fill_lj(P.d, P);
  fill_lj(P.f, P);
}
template <class R>
static void fill_cos(Cosc<R>& c, const CosPar& P, bool morse) {
  c.sig = (R)P.sig;
  c.delt = (R)P.delt;
  c.a = (R)P.a;
  c.r0 = (R)P.r0;
  c.R1 = (R)P.R1;
  c.R2 = (R)P.R2;
  c.inv_w = (R)(1.0 / (P.R2 - P.R1));
  c.pref = (R)(morse ? P.D : 4.0 * P.eps);
  c.idelt = P.delt == 2.0 ? 2 : 0;
}
void derive(CosPar& P, bool morse) {
  fill_cos(P.d, P, morse);
  fill_cos(P.f, P, morse);
}
template <class R>
static void fill_rjl(RJLc<R>& c, const RJLPar& P) {
  c.A0 = (R)P.A0;
  c.xi = (R)P.xi;
  c.R1 = (R)P.R1;
  c.R2 = (R)P.R2;
  c.inv_w = (R)(1.0 / (P.R2 - P.R1));
  c.inv_r0 = (R)(1.0 / P.r0);
  c.m2q = (R)(-2.0 * P.q);
  c.mp = (R)(-P.p);
  c.a2 = (R)(2.0 * P.A0);
  c.pr0 = (R)(P.p / P.r0);
  c.qr0 = (R)(P.q / P.r0);
  const double log2e = 1.4426950408889634;
  c.eqa = (R)(-2.0 * P.q * log2e / P.r0);
  c.eqb = (R)(2.0 * P.q * log2e);
  c.epa = (R)(-P.p * log2e / P.r0);
  c.epb = (R)(P.p * log2e);
  c.tb = (R)(-P.R1 / (P.R2 - P.R1));
  c.dsw = (R)(-0.5 * 3.14159265358979323846 / (P.R2 - P.R1));
}
void derive(RJLPar& P) {
  fill_rjl(P.d, P);
  fill_rjl(P.f, P);
}
template <class R>
static void fill_tb(TBc<R>& c, const TBPar& P) {
  c.d = (R)P.d;
  c.s = (R)P.s;
  c.b = (R)P.b;
  c.r0 = (R)P.r0;
  c.delt = (R)P.delt;
  c.a0 = (R)P.a0;
  c.c02 = (R)P.c02;
  c.d02 = (R)P.d02;
  c.R1 = (R)P.R1;
  c.R2 = (R)P.R2;
  c.inv_w = (R)(1.0 / (P.R2 - P.R1));
  c.ex = (R)(1.0 / P.delt + 1.0);
  c.sq2s = (R)std::sqrt(2.0 * P.s);
  c.sq2os = (R)std::sqrt(2.0 / P.s);
  c.pre_e = (R)(P.d / (P.s - 1.0));
  c.c02d02 = (R)(P.c02 / P.d02);
  c.is = (R)(1.0 / P.s);
}
void derive(TBPar& P) {
  fill_tb(P.dd, P);
  fill_tb(P.f, P);
}

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct GroupH {
  std::vector<int> idx;  // 0-based atoms
  int n0 = 0;            // size at creation
  DBuf<int> d;
};

enum ListKind { L_REGULAR = 0, L_CONVERSE = 1, L_NN_TB = 2 };

struct ListH {
  ListKind kind = L_REGULAR;
  ListDev d{};
  CellGrid cg{};
  DBuf<int> nnum, nlist, pidx, less, bnd, row_of, cstart, ccount, ccursor, cjnd, catom, ccell;
  DBuf<int4> cposq;
  std::vector<int> col_inv;  // host: atom -> column-group index (reading lists back)
  double rc = 0.0;
  long long period = 1;
  int src = -1;  // converse: source list; nn: the tb list
  bool has_grid = false;
  double half_skin = 0.0;  // skin-triggered rebuilds: half of r_cut minus the interaction's cut-off
  DBuf<int4> xref, xprev;  // fixed-point positions at the last build / the last update step (skin >= 0)
  // two-level list: the wider list this list's rows are filtered from, and the
  // positions at its last build
  std::unique_ptr<ListH> outer;
  DBuf<int4> xout;
};

struct InterH {
  pfmd_io::InteractionSpec spec;
  int lists[3] = {-1, -1, -1};
  LJPar lj{};
  CosPar cp{};
  RJLPar rjl{};
  TBPar tb{};
  REBOPar rebo{};
  bool general = false;  // lj1g weights for a group not in ascending atom order
  DBuf<double> scratch;  // rjl 1/Eb, tb bond orders
  DBuf<double2> pair;    // rjl plain form: per-slot force coefficients
  DBuf<double4_32a> norm;    // ljc / morsec graphene normals
  DBuf<double4_32a> gsum;    // ljc / morsec: per graphene row, the sum the normal-derivative term reads
  int tb_inter = -1;     // ljc / morsec: the first tb interaction
  double rc_nn = 0.0;
};

struct StepPlan {
  long long step;
  bool first, energy, out, zero_mom, check_all;
  std::vector<char> rebuild;  // per list
  // the next step's kick and drift fused into this step's force kernel / this
  // step's kick and drift done by the previous step's
  bool drift_next = false, drifted = false;
  // nvt with the pair kernel's fused chain: the chain's second-half scaling is
  // left to the next step's k_nhc (same segment, no energy or output step)
  bool nhc_defer = false;
  // the same, with the pair kernel also running the next step's first
  // half-update (nhc_ahead); the next step (nhc_done) launches no k_nhc for the
  // chain, and its kick-drift opens the step and applies both scales
  bool nhc_ahead = false, nhc_done = false;
  // a log step inside the segment: its record's row in the device log ring,
  // turned into the log line at the segment's end (-1: none)
  int log_row = -1;
};

// Snapshot and trajectory files (md_read_write.f90:65-107) are formatted and
// written by one worker thread, in submission order, while the device runs the
// next steps.  The state is copied to the host before a job is queued, so each
// file holds its own step.  At most four jobs wait (the submitter blocks beyond
// that); the first write error is kept for the engine to raise.
class FileWriter {
 public:
  using Format = std::function<std::string()>;
  FileWriter() : th_([this] { loop(); }) {}
  ~FileWriter() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    if (th_.joinable()) th_.join();
  }
  void submit(std::string path, bool append, Format f) {
    std::unique_lock<std::mutex> lk(mu_);
    room_.wait(lk, [&] { return q_.size() < kMaxPending; });
    q_.push_back(Job{std::move(path), append, std::move(f)});
    cv_.notify_one();
  }
  // Waits for every queued job; returns the first error ("" if none).
  std::string drain() {
    std::unique_lock<std::mutex> lk(mu_);
    room_.wait(lk, [&] { return q_.empty() && !busy_; });
    return err_;
  }
  std::string error() {
    std::lock_guard<std::mutex> lk(mu_);
    return err_;
  }
  // Formats and writes one file on the calling thread (what the worker does).
  static std::string write(const std::string& path, bool append, const Format& f) {
    const std::string text = f();
    if (text.empty()) return "";
    FILE* fp = std::fopen(path.c_str(), append ? "a" : "w");
    if (!fp) return "cannot open " + path;
    std::fputs(text.c_str(), fp);
    std::fclose(fp);
    return "";
  }

 private:
  struct Job {
    std::string path;
    bool append = false;
    Format f;
  };
  void loop() {
    for (;;) {
      Job j;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || !q_.empty(); });
        if (q_.empty()) return;
        j = std::move(q_.front());
        q_.pop_front();
        busy_ = true;
      }
      room_.notify_all();
      const std::string e = write(j.path, j.append, j.f);
      {
        std::lock_guard<std::mutex> lk(mu_);
        busy_ = false;
        if (!e.empty() && err_.empty()) err_ = e;
      }
      room_.notify_all();
    }
  }
  static constexpr size_t kMaxPending = 4;
  std::mutex mu_;
  std::condition_variable cv_, room_;
  std::deque<Job> q_;
  bool stop_ = false, busy_ = false;
  std::string err_;
  std::thread th_;  // declared last: starts once the members above exist
};

class Engine {
 public:
  pfmd_options opt{};
  std::string input_path, settings_filename, prefix;
  pfmd_io::Settings S;
  int N = 0;
  Box box{};
  Atoms A{};
  DBuf<double4_32a> pos, vel, frc;
  DBuf<double> stage;  // 9 N doubles: xyz-interleaved positions, velocities, forces in transfer
  DBuf<double> mass, kc;
  DBuf<int4> posq, posq2;  // fixed-point positions; two buffers when kick-drift fuses into the forces
  int posq_cur = 0;         // which buffer A.posq is (0: posq, 1: posq2)
  bool fuse_drift = false;  // the precision rjl force kernel may run the next step's kick and drift
  void flip_posq() {
    posq_cur ^= 1;
    A.posq = posq_cur ? posq2.p : posq.p;
  }
  std::vector<GroupH> groups;
  std::vector<ListH> lists;
  std::vector<InterH> inters;
  std::vector<ChangeSpec> changes;
  // learned form: a network per tb / rjl interaction (see learned.h)
  struct Lrn {
    bool on = false;
    bool tc = false;  // network on the tensor cores (BF16)
    learned::Model model;
    DBuf<learned::DescPar> d;
    DBuf<learned::Net> net;
    DBuf<float> G, g, e, part, grad, m, v;
    DBuf<float4> leg, cforce;
    DBuf<double> t, lpart, loss;
    int adam_step = 0;
  };
  std::vector<Lrn> lrn;        // per interaction
  bool learned_active = false;  // learned kernels in place of the classical ones
  long long check_period = 0;
  double max_rmse = 0.0, last_rmse = -1.0;
  int checks = 0;
  bool fallen_back = false;
  DBuf<double4_32a> fsave;
  DBuf<double> fdiff, eatom;
  double* eatom_out = nullptr;  // set while per-atom energies are recorded
  void learned_setup(const std::vector<learned::Model>& ms);
  void learned_upload_desc(Lrn& L);
  double learned_check(bool switch_on_fail);
  void learned_train(const std::string& model_in, const std::string& model_out, int frames, int stride, int iters, int flags,
                     float* grad_out, double* loss_out, double* grad_ms,
                     double lr, double force_weight, double* rmse_out, double* force_rmse);
  DBuf<double4_32a> fref;
  DBuf<float4> fres;
  void clear_graphs();
  void ensure_lists();
  Ctl* ctl = nullptr;
  Ctl* hctl = nullptr;  // pinned host copy (header part)
  // log records of the log steps inside a segment (kLogCols doubles each)
  DBuf<double> log_ring;
  double* hlog = nullptr;  // pinned host copy
  size_t log_cap = 0;      // rows
  size_t ctl_head = 0;
  // hctl equals the device's header: set by read_ctl, cleared when an API call
  // that may launch work starts (energies reads the copy while it holds)
  bool ctl_fresh = false;
  cudaStream_t st = nullptr;
  bool prec = false;
  bool fuse_kick_drift = true;
  int fused_nhc_chain = -1;  // chain whose scaling folds into the first kick
  // force-phase fusion (Epi): the first force kernel stores instead of adding,
  // the last one applies the second half-kick
  bool store_first = false, kick_last = false;
  DBuf<unsigned char> mflag;  // per atom: bit 0 in the xyz group, bit 1 in the z group, bit 2 in chain 0's
  // all lj / lj1g lists in one atom-major launch (k_pair_atoms)
  bool pair_fused = false;
  int pair_tpa = 1;
  DBuf<int> pair_off;
  DBuf<int2> pair_task;
  DBuf<PairSlot> pair_slots;
  bool nhc_fused = false;    // the pair kernel reduces chain 0's kinetic energy and updates it
  bool nhc_pending = false;  // chain 0's last scaling still to be applied (by the next k_nhc)
  bool nhc_ahead = false;    // the pair launch being enqueued also runs the next first half-update
  void plan_pair_fusion();
  // Forces on two streams: with one ljc / morsec coupling whose two sides' rows
  // are disjoint atom sets, and every other interaction's rows inside one side
  // (tb on the sheet, rjl in the slab), the kernels that write one side's atoms
  // run on st and the others on st2 (non-energy steps: the energy variants share
  // the grid-reduction scratch).  Every force kernel writes only its own rows.
  void plan_force_split();
  bool force_split = false;
  std::vector<int> force_side;  // per interaction: 1 (st), 2 (st2), 3 (the coupling: both)
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  PairSet pair_set() const;
  bool need_check_all = true;

  // md() loop state
  long long md_step = 0;  // next step to execute
  int integrator_index = 0;
  std::string integrator_name;
  int integ = I_NVE;
  double ts[4] = {0, 0, 0, 0};
  double sim_time = 0.0;
  bool finished = false;
  bool finished_called = false;
  bool tpa_tuned = false;

  // output
  std::string obuf;
  FILE* log = nullptr;
  double t_start = 0, t_md = 0;
  std::string err;
  bool printed = false;  // the failure's message already went to the output unit

  // graphs
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;
    int seen = 0;
  };
  std::map<std::string, GraphEntry> graphs;
  long long launches = 0;
  // device timing of advance (events recorded on st around the enqueued work)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timing = false, timing_started = false;
  DBuf<unsigned char> flush_buf;
  int flush_seq = 0;

  ~Engine();
  void create(const std::string& ip, const std::string& sf, const pfmd_options& o);
  void advance(long long max_steps, int* fin);
  void finish();
  void compute(bool rebuild, double* e_inter);
  double time_kernel(const std::string& name, int reps, double* bytes);
  double kernel_bytes(const std::string& name);

  // helpers
  void out(const std::string& s) { obuf += s; }
  void outln(const std::string& s) { obuf += s + "\n"; }
  void flush_out();
  void write_all_out(const std::string& s);
  GroupRef gref(int g1based) const {
    const GroupH& g = groups[static_cast<size_t>(g1based - 1)];
    return GroupRef{g.d.p, g1based - 1, static_cast<int>(g.idx.size())};
  }
  int group_checked(int num) const {
    if (num < 1 || num > static_cast<int>(groups.size()))
      throw Error(PFMD_E_PARAM, "error: group number " + std::to_string(num) + " out of range");
    return num;
  }
  void read_ctl();
  void tune_tpa();
  void upload_ctl_groups();
  void raise_device_error();
  bool switch_needed(long long s) const;
  bool do_switch();  // false: no more integrators
  StepPlan plan(long long s) const;
  bool is_event(const StepPlan& p) const;
  void enqueue_step(const StepPlan& p);
  void enqueue_lists(const StepPlan& p);
  void alloc_list(ListH& L);
  void enqueue_forces(bool energy, bool kick = false, bool drift_next = false, bool begin = false);
  void plan_fusion();
  void refresh_mflag();
  void run_plans(const std::vector<StepPlan>& plans);
  void host_events(const StepPlan& p, bool log_line = true);
  bool log_step(const StepPlan& p) const;
  bool hard_event(const StepPlan& p) const;
  void write_log_line(long long s, double t, const double* row);
  void get_state_host(std::vector<double>& p, std::vector<double>& v, std::vector<double>* f);
  void get_state_to(double* p, double* v, double* f);
  std::unique_ptr<FileWriter> writer;  // snapshot / trajectory files (opt.async_io)
  void emit_file(const std::string& path, bool append, FileWriter::Format f);
  void check_writer(bool wait);
  std::string nlists_load_text();
};

Engine::~Engine() {
  writer.reset();  // its queued jobs read this engine's groups and types
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (st2) cudaStreamDestroy(st2);
  for (auto& kv : graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  if (log) std::fclose(log);
  if (ctl) cudaFree(ctl);
  if (hctl) cudaFreeHost(hctl);
  if (hlog) cudaFreeHost(hlog);
  if (st) cudaStreamDestroy(st);
}

void Engine::flush_out() {
  if (obuf.empty()) return;
  if (opt.out_fd >= 0) {
    size_t off = 0;
    while (off < obuf.size()) {
      ssize_t w = ::write(opt.out_fd, obuf.data() + off, obuf.size() - off);
      if (w <= 0) break;
      off += static_cast<size_t>(w);
    }
  }
  obuf.clear();
}

void Engine::write_all_out(const std::string& s) {
  int fd = opt.all_out_fd >= 0 ? opt.all_out_fd : opt.out_fd;
  if (fd == opt.out_fd) {
    out(s);
    return;
  }
  flush_out();
  if (fd >= 0) {
    ssize_t w = ::write(fd, s.data(), s.size());
    (void)w;
  }
}

// ---------------------------------------------------------------------------
// set-up
// ---------------------------------------------------------------------------
void Engine::create(const std::string& ip, const std::string& sf, const pfmd_options& o) {
  opt = o;
  input_path = ip;
  settings_filename = sf;
  prefix = o.output_prefix ? o.output_prefix : "";
  prec = opt.form == PFMD_FORM_PRECISION;
  t_start = now_s();
  {
    const int t = opt.threads_per_row;
    if (t < 0 || t > 32 || (t & (t - 1)) != 0)
      throw Error(PFMD_E_PARAM, "threads_per_row must be 0 (automatic) or a power of two up to 32");
  }
  try {
    pfmd_io::read_settings(input_path, settings_filename, S);
  } catch (const fortio::ReadError& e) {
    out(S.echo);
    throw Error(PFMD_E_IO, e.what());
  } catch (const std::exception& e) {
    out(S.echo);
    throw Error(PFMD_E_PARAM, e.what());
  }
  out(S.echo);
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    throw Error(PFMD_E_CUDA, "no CUDA device: this library runs its MD step on the GPU only");
  CK(cudaSetDevice(opt.device));
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));

  N = S.xyz.N;
  for (int k = 0; k < 3; ++k) {
    box.L[k] = S.xyz.box[k];
    box.h[k] = 0.5 * S.xyz.box[k];
    box.qinv[k] = 4294967296.0 / box.L[k];
    box.qs[k] = static_cast<float>(box.L[k] / 4294967296.0);
    box.Ltol[k] = box.L[k] + 0.0000001;
    {  // 2^32 / L = qm * 2^(qe - 64), qm in [2^63, 2^64)
      int ex = 0;
      const double fr = std::frexp(box.qinv[k], &ex);  // qinv = fr * 2^ex, fr in [0.5, 1)
      box.qm[k] = static_cast<unsigned long long>(std::ldexp(fr, 64));
      box.qe[k] = ex;
    }
  }
  // groups: create_particle_group (md_general.f90:57-80)
  if (S.group_types.size() > PFMD_MAX_GROUPS) throw Error(PFMD_E_PARAM, "error: too many groups");
  for (const auto& names : S.group_types) {
    GroupH g;
    for (const auto& nm : names)
      for (int i = 0; i < N; ++i)
        if (S.xyz.types[static_cast<size_t>(i)] == nm) g.idx.push_back(i);
    g.n0 = static_cast<int>(g.idx.size());
    groups.push_back(std::move(g));
  }
  for (const auto& c : S.changes) {
    ChangeSpec cs{};
    cs.from = group_checked(c.from) - 1;
    cs.to = group_checked(c.to) - 1;
    cs.ts1 = c.ts1;
    cs.ts2 = c.ts2;
    cs.frec = c.frec;
    if (c.frec < 1) throw Error(PFMD_E_PARAM, "error: group change frequency must be positive");
    cs.to_cap = static_cast<int>(groups[static_cast<size_t>(cs.to)].idx.size());
    changes.push_back(cs);
  }
  if (changes.size() > 8) throw Error(PFMD_E_PARAM, "error: at most 8 group changes are supported");
  group_checked(S.all_moving);
  group_checked(S.xyz_moving);
  group_checked(S.z_moving);
  group_checked(S.all_atoms);
  group_checked(S.traj_group);
  if (S.period_traj < 1 || S.zero_momentum_period < 1)
    throw Error(PFMD_E_PARAM, "error: output and momentum periods must be positive");
  for (const auto& is : S.integrators)
    if (is.period_log < 1 || is.period_snapshot < 1)
      throw Error(PFMD_E_PARAM, "error: integrator output periods must be positive");
  if (S.nhc.size() > PFMD_MAX_NHC) throw Error(PFMD_E_PARAM, "error: too many Nose-Hoover chains");
  for (const auto& h : S.nhc) {
    group_checked(h.group);
    if (h.M < 1 || h.M > PFMD_MAX_CHAIN) throw Error(PFMD_E_PARAM, "error: wrong nhc parameters");
  }

  // host copies of the state
  std::vector<double> hp = S.xyz.pos, hv = S.xyz.vel;
  const std::vector<double>& hm = S.xyz.mass;
  if (S.new_velocities) {
    // set_new_temperature (md_general.f90:328-340) with the serial seeded stream
    const GroupH& g = groups[static_cast<size_t>(S.all_moving - 1)];
    double t0 = S.initial_temperature < 0.0 ? 0.0 : S.initial_temperature;
    pfmd_io::MinStd rng(opt.rand_seed);
    for (int i : g.idx)
      for (int k = 0; k < 3; ++k) {
        double a1 = 0, a2 = 0, b = 2.0;
        while (b >= 1.0) {
          a1 = 2.0 * rng.next() - 1.0;
          a2 = 2.0 * rng.next() - 1.0;
          b = a1 * a1 + a2 * a2;
        }
        hv[3 * i + k] = a1 * std::sqrt(-2.0 * std::log(b) / b);
      }
    for (int i : g.idx)
      for (int k = 0; k < 3; ++k) hv[3 * i + k] = hv[3 * i + k] * std::sqrt(MOMENTA_COEF / hm[i]);
    double mv[3] = {0, 0, 0}, mt = 0;
    for (int k = 0; k < 3; ++k)
      for (int i : g.idx) mv[k] = mv[k] + hm[i] * hv[3 * i + k];
    for (int i : g.idx) mt = mt + hm[i];
    for (int k = 0; k < 3; ++k) mv[k] = mv[k] / mt;
    for (int i : g.idx)
      for (int k = 0; k < 3; ++k) hv[3 * i + k] = hv[3 * i + k] - mv[k];
    double ke = 0;
    for (int i : g.idx) {
      const double* v = &hv[3 * i];
      ke = ke + hm[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / 2 * MASS_COEF;
    }
    double temp = 2 * ke / KT_A_DEGREE / static_cast<double>(3 * static_cast<int>(g.idx.size()));
    double sc = std::sqrt(t0 / temp);
    for (int i : g.idx)
      for (int k = 0; k < 3; ++k) hv[3 * i + k] = hv[3 * i + k] * sc;
  }

  // interactions and their lists (create_interactions, md_interactions.f90:59-136)
  if (S.interactions.size() > PFMD_MAX_INTER) throw Error(PFMD_E_PARAM, "error: too many interactions");
  // the first tb or rebosc interaction gives ljc / morsec their graphene
  // neighbours (md_interactions.f90:158-164)
  int first_tb = -1;
  for (size_t k = 0; k < S.interactions.size(); ++k)
    if (S.interactions[k].kind == pfmd_io::K_TB || S.interactions[k].kind == pfmd_io::K_REBOSC) {
      first_tb = static_cast<int>(k);
      break;
    }
  auto new_list = [&](ListKind kind, int row_g, int col_g, int rows, int nmax, double rc, long long period) {
    ListH L;
    L.kind = kind;
    L.rc = rc;
    L.period = period;
    L.d.id = static_cast<int>(lists.size());
    L.d.rows = rows;
    L.d.nmax = nmax;
    L.d.stride = ((std::max(rows, 1) + 31) / 32) * 32;
    // the plain form keeps the reference's row order (bit-exact lists); the
    // precision form keeps the deterministic cell-scan order
    L.d.sorted = prec ? 0 : 1;
    L.d.tpa = opt.threads_per_row > 0 ? opt.threads_per_row : auto_tpa(rows, std::max(nmax, 2) / 2.0, opt.form == PFMD_FORM_PRECISION);
    L.d.tpa1 = opt.threads_per_row > 0 ? opt.threads_per_row
                                       : pass1_tpa(L.d.tpa, std::max(nmax, 2) / 2.0, opt.form == PFMD_FORM_PRECISION);
    L.d.row_group = row_g - 1;
    L.d.col_group = col_g - 1;
    L.d.skin = -1;
    L.d.row_cap = static_cast<int>(groups[static_cast<size_t>(row_g - 1)].idx.size());
    L.d.col_cap = static_cast<int>(groups[static_cast<size_t>(col_g - 1)].idx.size());
    if (nmax < 0) throw Error(PFMD_E_PARAM, "error: negative neighb_num_max");
    if (nmax > 1024) throw Error(PFMD_E_PARAM, "error: neighb_num_max above 1024 is not supported");
    if (period < 1) throw Error(PFMD_E_PARAM, "error: neighbour list update period must be positive");
    lists.push_back(std::move(L));
    if (lists.size() > PFMD_MAX_LISTS) throw Error(PFMD_E_PARAM, "error: too many neighbour lists");
    return static_cast<int>(lists.size()) - 1;
  };
  for (size_t k = 0; k < S.interactions.size(); ++k) {
    const auto& sp = S.interactions[k];
    InterH I;
    I.spec = sp;
    const auto& p = sp.p;
    for (const auto& ls : sp.nl) {
      group_checked(ls.g1);
      group_checked(ls.g2);
    }
    const auto& l1 = sp.nl[0];
    const int rows1 = static_cast<int>(groups[static_cast<size_t>(l1.g1 - 1)].idx.size());
    I.lists[0] = new_list(L_REGULAR, l1.g1, l1.g2, rows1, l1.nmax, l1.r_cut, l1.period);
    switch (sp.kind) {
      case pfmd_io::K_LJ:
      case pfmd_io::K_LJ1G:
        I.lj.eps = p[0];
        I.lj.sig = p[1];
        I.lj.R1 = p[2];
        I.lj.R2 = p[3];
        {
          double s6 = p[1] * p[1] * p[1] * p[1] * p[1] * p[1], s12 = s6 * s6;
          I.lj.c6 = 4.0 * p[0] * s6;
          I.lj.c12 = 4.0 * p[0] * s12;
          I.lj.c6t6 = 6.0 * 4.0 * p[0] * s6;
          I.lj.c12t12 = 12.0 * 4.0 * p[0] * s12;
        }
        break;
      case pfmd_io::K_LJC:
        I.cp.eps = p[0];
        I.cp.sig = p[1];
        I.cp.delt = p[2];
        I.cp.R1 = p[3];
        I.cp.R2 = p[4];
        I.cp.simplified = sp.simplified ? 1 : 0;
        break;
      case pfmd_io::K_MORSEC:
        I.cp.D = p[0];
        I.cp.r0 = p[1];
        I.cp.a = p[2];
        I.cp.delt = p[3];
        I.cp.R1 = p[4];
        I.cp.R2 = p[5];
        I.cp.simplified = sp.simplified ? 1 : 0;
        break;
      case pfmd_io::K_RJL:
        I.rjl = RJLPar{p[0], p[1], p[2], p[3], p[4], p[5], p[6], {}, {}};
        derive(I.rjl);
        break;
      case pfmd_io::K_TB:
        I.tb = TBPar{p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9], p[6] * p[6], p[7] * p[7], {}, {}};
        derive(I.tb);
        break;
      case pfmd_io::K_REBOSC:
        I.rebo = REBOPar{p[0], p[1], p[2], {p[3], p[4], p[5]}, {p[6], p[7], p[8]}, p[9],
                         {p[10], p[11], p[12], p[13], p[14], p[15]}, p[16], p[17]};
        break;
    }
    if (sp.kind == pfmd_io::K_LJ || sp.kind == pfmd_io::K_LJ1G) derive(I.lj);
    if (sp.kind == pfmd_io::K_LJC || sp.kind == pfmd_io::K_MORSEC) derive(I.cp, sp.kind == pfmd_io::K_MORSEC);
    if (sp.kind == pfmd_io::K_LJ1G || sp.kind == pfmd_io::K_RJL || sp.kind == pfmd_io::K_TB ||
        sp.kind == pfmd_io::K_REBOSC) {
      // the reference indexes these lists' partners through the row arrays
      // (particle_index(nlist), Eb(nlist), nl%nlist(:,j)), which needs g1 == g2
      if (l1.g1 != l1.g2)
        throw Error(PFMD_E_PARAM, "error: " + fortio::trim(sp.name) + " needs the same group on both sides of its list");
      if (sp.kind == pfmd_io::K_LJ1G) {
        const auto& gi = groups[static_cast<size_t>(l1.g1 - 1)].idx;
        for (size_t a = 1; a < gi.size(); ++a)
          if (gi[a] <= gi[a - 1]) I.general = true;
      }
    }
    if (sp.kind == pfmd_io::K_LJ || sp.kind == pfmd_io::K_LJC || sp.kind == pfmd_io::K_MORSEC) {
      const auto& l2 = sp.nl[1];
      const int rows2 = static_cast<int>(groups[static_cast<size_t>(l2.g1 - 1)].idx.size());
      // rows hold nl(1)'s group-2 atoms, entries are nl(1) rows (its group 1)
      int c = new_list(L_CONVERSE, l1.g2, l1.g1, rows2, l2.nmax, l1.r_cut, l1.period);
      lists[static_cast<size_t>(c)].src = I.lists[0];
      I.lists[1] = c;
    }
    if (sp.kind == pfmd_io::K_LJC || sp.kind == pfmd_io::K_MORSEC) {
      const auto& l3 = sp.nl[2];
      const int rows3 = static_cast<int>(groups[static_cast<size_t>(l3.g1 - 1)].idx.size());
      I.tb_inter = first_tb;
      I.rc_nn = l3.r_cut;
      if (first_tb >= 0) {
        const auto& tl = S.interactions[static_cast<size_t>(first_tb)].nl[0];
        int c = new_list(L_NN_TB, tl.g1, tl.g1, rows3, l3.nmax, l3.r_cut, tl.period);
        I.lists[2] = c;
      } else {
        I.lists[2] = new_list(L_REGULAR, l3.g1, l3.g2, rows3, l3.nmax, l3.r_cut, l3.period);
      }
      if (rows1 != rows3 && rows1 != 0)
        throw Error(PFMD_E_PARAM, "error: nl%N/=nl_nn%N " + std::to_string(rows1) + " " + std::to_string(rows3));
    }
    inters.push_back(std::move(I));
  }
  // the tb list an nn list reads
  for (auto& I : inters)
    if (I.tb_inter >= 0) lists[static_cast<size_t>(I.lists[2])].src = inters[static_cast<size_t>(I.tb_inter)].lists[0];
  for (auto& I : inters)
    if (I.tb_inter >= 0) {
      const ListH& tb = lists[static_cast<size_t>(lists[static_cast<size_t>(I.lists[2])].src)];
      if (tb.d.rows > lists[static_cast<size_t>(I.lists[2])].d.rows)
        throw Error(PFMD_E_PARAM, "error: the graphene nearest-neighbour list is shorter than the tb list");
    }
  // rows of every list must name distinct atoms (forces are added without atomics)
  {
    std::vector<char> seen(static_cast<size_t>(N));
    for (auto& L : lists) {
      if (L.kind == L_NN_TB) continue;
      std::fill(seen.begin(), seen.end(), 0);
      for (int a : groups[static_cast<size_t>(L.d.row_group)].idx) {
        if (seen[static_cast<size_t>(a)])
          throw Error(PFMD_E_PARAM, "error: an atom appears twice in a group that rows a neighbour list");
        seen[static_cast<size_t>(a)] = 1;
      }
    }
  }
  // kick and drift fuse when the xyz and z groups share no atom
  {
    std::vector<char> in_xyz(static_cast<size_t>(N), 0);
    for (int a : groups[static_cast<size_t>(S.xyz_moving - 1)].idx) in_xyz[static_cast<size_t>(a)] = 1;
    for (int a : groups[static_cast<size_t>(S.z_moving - 1)].idx)
      if (in_xyz[static_cast<size_t>(a)]) fuse_kick_drift = false;
    if (S.xyz_moving == S.z_moving && !groups[static_cast<size_t>(S.xyz_moving - 1)].idx.empty())
      fuse_kick_drift = false;
  }
  // a single chain over exactly the xyz group folds its scaling into the first kick
  if (S.nhc.size() == 1 && S.nhc[0].group == S.xyz_moving && fuse_kick_drift) fused_nhc_chain = 0;

  // ---- device ----
  pos.alloc(static_cast<size_t>(std::max(N, 1)));
  vel.alloc(static_cast<size_t>(std::max(N, 1)));
  frc.alloc(static_cast<size_t>(std::max(N, 1)));
  mass.alloc(static_cast<size_t>(std::max(N, 1)));
  posq.alloc(static_cast<size_t>(std::max(N, 1)));
  {
    std::vector<double4_32a> tp(static_cast<size_t>(N)), tv(static_cast<size_t>(N));
    for (int i = 0; i < N; ++i) {
      tp[static_cast<size_t>(i)] = make_double4_32a(hp[3 * i], hp[3 * i + 1], hp[3 * i + 2], 0.0);
      tv[static_cast<size_t>(i)] = make_double4_32a(hv[3 * i], hv[3 * i + 1], hv[3 * i + 2], 0.0);
    }
    pos.upload(tp.data(), tp.size(), st);
    vel.upload(tv.data(), tv.size(), st);
    frc.zero(st);
    mass.upload(hm.data(), hm.size(), st);
    std::vector<double> hk(hm.size());
    for (size_t i = 0; i < hm.size(); ++i) hk[i] = 1.0 / (hm[i] * MASS_COEF);
    kc.alloc(std::max<size_t>(hk.size(), 1));
    kc.upload(hk.data(), hk.size(), st);
    CK(cudaStreamSynchronize(st));
  }
  A = Atoms{N, pos.p, vel.p, frc.p, mass.p, posq.p, kc.p};
  for (auto& g : groups) {
    g.d.alloc(std::max<size_t>(g.idx.size(), 1));
    g.d.upload(g.idx.data(), g.idx.size(), st);
  }
  for (auto& L : lists) alloc_list(L);
  for (auto& I : inters) {
    const ListH& L1 = lists[static_cast<size_t>(I.lists[0])];
    if (I.spec.kind == pfmd_io::K_RJL) {
      I.scratch.alloc(static_cast<size_t>(std::max(N, 1)));  // 1/Eb per atom (plain form)
      // pair terms per list slot: double2 (plain) or float2 (precision)
      const size_t slots = static_cast<size_t>(L1.d.nmax) * L1.d.stride;
      I.pair.alloc(std::max<size_t>(prec ? (slots + 1) / 2 : slots, 1));
    }
    if (I.spec.kind == pfmd_io::K_TB)
      // B and B^(1/delta + 1) per list slot
      I.scratch.alloc(std::max<size_t>(2 * static_cast<size_t>(L1.d.nmax) * L1.d.stride, 1));
    if (I.spec.kind == pfmd_io::K_REBOSC)  // bsp, dbsp/dS and bdh per list slot
      I.scratch.alloc(std::max<size_t>(3 * static_cast<size_t>(L1.d.nmax) * L1.d.stride, 1));
    if (I.lists[2] >= 0) {
      I.norm.alloc(static_cast<size_t>(std::max(N, 1)));  // normals per atom
      I.norm.zero(st);
      I.gsum.alloc(static_cast<size_t>(std::max(N, 1)));  // at most one graphene row per atom
      I.gsum.zero(st);
    }
    // lj1g in a group that is not in atom order needs lessnnum in the reference's order
    if (I.spec.kind == pfmd_io::K_LJ1G && I.general) lists[static_cast<size_t>(I.lists[0])].d.sorted = 1;
    // lists whose kernels address a partner's row: tb (and the nn selection that
    // reads it), lj1g in a group that is not in ascending atom order
    std::vector<int> need;
    if (I.spec.kind == pfmd_io::K_TB || I.spec.kind == pfmd_io::K_REBOSC || (I.spec.kind == pfmd_io::K_LJ1G && I.general))
      need.push_back(I.lists[0]);
    for (int li : need) {
      ListH& L = lists[static_cast<size_t>(li)];
      if (L.row_of.p) continue;
      std::vector<int> ro(static_cast<size_t>(N), -1);
      const auto& rg = groups[static_cast<size_t>(L.d.row_group)].idx;
      for (size_t k = 0; k < rg.size(); ++k) ro[static_cast<size_t>(rg[k])] = static_cast<int>(k);
      L.row_of.alloc(ro.size());
      L.row_of.upload(ro.data(), ro.size(), st);
      L.d.row_of = L.row_of.p;
    }
  }
  // skin-triggered rebuilds (precision form): at an update step a list keeps its
  // rows when no atom of its groups moved more than half of (r_cut - the
  // interaction's cut-off) since it was built; its converse list follows it
  if (prec && opt.skin_lists && changes.empty()) {
    for (auto& I : inters) {
      double rint = -1.0;
      switch (I.spec.kind) {
        case pfmd_io::K_LJ:
        case pfmd_io::K_LJ1G: rint = I.lj.R2; break;
        case pfmd_io::K_LJC:
        case pfmd_io::K_MORSEC: rint = I.cp.R2; break;
        case pfmd_io::K_RJL: rint = I.rjl.R2; break;
        case pfmd_io::K_TB: rint = I.tb.R2; break;
        case pfmd_io::K_REBOSC: rint = I.rebo.R2; break;
      }
      ListH& L1 = lists[static_cast<size_t>(I.lists[0])];
      if (!(rint > 0.0) || !(L1.rc > rint)) continue;
      L1.d.skin = L1.d.id;
      L1.half_skin = 0.5 * (L1.rc - rint);
      L1.xref.alloc(static_cast<size_t>(std::max(N, 1)));
      L1.xprev.alloc(static_cast<size_t>(std::max(N, 1)));
      L1.xref.zero(st);
      L1.xprev.zero(st);
      if (I.lists[1] >= 0) lists[static_cast<size_t>(I.lists[1])].d.skin = L1.d.id;
      // two-level: a self list built by cells gets an outer list kOuterMargin
      // wider (its own cell grid, four times the slots), and a rebuild filters
      // the outer rows while no atom moved more than half the margin since the
      // outer build
      // (only where four times the slots fit the kernels' 1,024, so the outer
      // list cannot overflow where the list itself would not)
      if (L1.kind == L_REGULAR && !L1.d.sorted && L1.d.row_group == L1.d.col_group && L1.has_grid && N > 0 &&
          4 * L1.d.nmax <= 1024) {
        auto O = std::make_unique<ListH>();
        O->kind = L_REGULAR;
        O->rc = L1.rc + kOuterMargin;
        O->period = L1.period;
        O->d = L1.d;
        O->d.nmax = 4 * std::max(L1.d.nmax, 1);
        O->d.skin = PFMD_MAX_LISTS + L1.d.id;
        alloc_list(*O);
        L1.outer = std::move(O);
        L1.xout.alloc(static_cast<size_t>(N));
        L1.xout.zero(st);
      }
    }
  }
  plan_fusion();
  plan_pair_fusion();
  plan_force_split();
  // the next step's kick and drift in the force kernel: precision form, one rjl
  // interaction whose rows are every atom and which kicks last, an xyz-moving group
  // and no z-moving one, no group changes or z-velocity inversion
  if (prec && opt.fuse_steps && fuse_kick_drift && inters.size() == 1 && inters[0].spec.kind == pfmd_io::K_RJL &&
      kick_last &&
      changes.empty() && !S.invert_z_vel && groups[static_cast<size_t>(S.xyz_moving - 1)].idx.size() > 0 &&
      groups[static_cast<size_t>(S.z_moving - 1)].idx.empty() &&
      lists[static_cast<size_t>(inters[0].lists[0])].d.rows == N) {
    fuse_drift = true;
    posq2.alloc(static_cast<size_t>(std::max(N, 1)));
  }
  // control block
  CK(cudaMalloc(&ctl, sizeof(Ctl)));
  CK(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
  ctl_head = offsetof(Ctl, partial);
  CK(cudaMallocHost(&hctl, ctl_head));
  std::memset(hctl, 0, ctl_head);
  hctl->md_step = -1;
  hctl->oob_atom = INT_MAX;
  for (size_t g = 0; g < groups.size(); ++g) hctl->group_n[g] = static_cast<int>(groups[g].idx.size());
  for (int l = 0; l < PFMD_MAX_LISTS; ++l) hctl->list_need[l] = hctl->outer_need[l] = 1;  // every list is built first
  for (size_t c = 0; c < S.nhc.size(); ++c) {
    const auto& h = S.nhc[c];
    NHCDev& d = hctl->nhc[c];
    d.M = h.M;
    d.L = static_cast<int>(groups[static_cast<size_t>(h.group - 1)].idx.size());
    d.T = h.temperature;
    d.s = 1.0;
    d.e = 0.0;
    d.q[0] = h.q1;
    for (int i = 1; i < d.M; ++i) d.q[i] = d.q[0] / (3.0 * d.L);
    for (int i = 0; i < d.M; ++i) d.iq[i] = 1.0 / d.q[i];
  }
  CK(cudaMemcpyAsync(ctl, hctl, ctl_head, cudaMemcpyHostToDevice, st));
  launch_pack_posq(A, box, ctl, st);
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());

  if (opt.write_files) {
    std::string ln = prefix + fortio::trim(S.logfilename);
    log = std::fopen(ln.c_str(), "w");
    if (!log) throw Error(PFMD_E_IO, "cannot open log file " + ln);
    if (opt.async_io) writer.reset(new FileWriter());
  }
  outln(fortio::Rec().a("PREPARATIONS TIME: ", 24).f(now_s() - t_start, 10, 2).a(" S ").s);
  outln(fortio::Rec().a("RUNNING ON ", 24).i(opt.num_threads, 6).a(" OPENMP THREADS").s);
  outln("");
  flush_out();
  t_md = now_s();
  md_step = 0;
  integrator_index = 0;
  sim_time = 0.0;
}

// Threads per row of each list's force kernels once the first build's mean
// neighbour count is known (a deterministic choice, so repeated runs stay
// bit-identical).
void Engine::tune_tpa() {
  tpa_tuned = true;
  if (opt.threads_per_row > 0) return;
  bool changed = false;
  for (auto& L : lists) {
    if (L.kind == L_NN_TB || L.d.rows == 0) continue;
    std::vector<int> n(static_cast<size_t>(L.d.rows));
    CK(cudaMemcpyAsync(n.data(), L.nnum.p, sizeof(int) * n.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // the mean over the rows that have entries: in a coupling list most rows
    // can be empty (the Cu atoms below the surface layer of the moire) while
    // the rest hold about 150 partners each
    double tot = 0;
    int filled = 0;
    for (int v : n) {
      tot += v;
      filled += v > 0 ? 1 : 0;
    }
    const double mean = tot / std::max(filled, 1);
    const int t = auto_tpa(L.d.rows, mean, prec);
    const int t1 = pass1_tpa(t, mean, prec);
    if (t != L.d.tpa || t1 != L.d.tpa1) {
      L.d.tpa = t;
      L.d.tpa1 = t1;
      changed = true;
    }
  }
  if (pair_fused) {
    // the all-pairs kernel: threads per atom from the entries an atom heads in all
    double tot = 0;
    for (const auto& I : inters)
      for (int j = 0; j < (I.spec.kind == pfmd_io::K_LJ ? 2 : 1); ++j) {
        const ListH& L = lists[static_cast<size_t>(I.lists[j])];
        std::vector<int> n(static_cast<size_t>(std::max(L.d.rows, 0)));
        if (n.empty()) continue;
        CK(cudaMemcpyAsync(n.data(), L.nnum.p, sizeof(int) * n.size(), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int v : n) tot += v;
      }
    const int t = auto_tpa(N, tot / std::max(N, 1), prec);
    if (t != pair_tpa) {
      pair_tpa = t;
      changed = true;
    }
  }
  if (changed) {
    for (auto& kv : graphs)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    graphs.clear();
  }
}

void Engine::alloc_list(ListH& L) {
  const double maxL = std::max(box.L[0], std::max(box.L[1], box.L[2]));
  const size_t rows = static_cast<size_t>(std::max(L.d.rows, 1));
  L.nnum.alloc(rows);
  L.nnum.zero(st);
  L.nlist.alloc(std::max<size_t>(static_cast<size_t>(L.d.nmax), 1) * static_cast<size_t>(L.d.stride));
  L.nlist.zero(st);
  L.pidx.alloc(rows);
  L.pidx.zero(st);
  L.less.alloc(rows);
  L.less.zero(st);
  L.bnd.alloc(rows);
  L.bnd.zero(st);
  L.d.nnum = L.nnum.p;
  L.d.nlist = L.nlist.p;
  L.d.pidx = L.pidx.p;
  L.d.lessnnum = L.less.p;
  L.d.bnd = L.bnd.p;
  L.d.row_idx = groups[static_cast<size_t>(L.d.row_group)].d.p;
  L.d.col_idx = groups[static_cast<size_t>(L.d.col_group)].d.p;
  L.d.row_of = nullptr;
  {
    const auto& cg = groups[static_cast<size_t>(L.d.col_group)].idx;
    L.col_inv.assign(static_cast<size_t>(N), -1);
    for (size_t k = 0; k < cg.size(); ++k) L.col_inv[static_cast<size_t>(cg[k])] = static_cast<int>(k);
  }
  if (L.kind != L_NN_TB) {
    // cells at least r_cut (+ a margin for FP32 binning) wide
    const double margin = 1e-3 * L.rc + 2e-3 + 4e-6 * maxL;
    long long ncell = 1;
    for (int k = 0; k < 3; ++k) {
      int nc = static_cast<int>(std::floor(box.L[k] / (L.rc + margin)));
      L.cg.nc[k] = std::max(1, nc);
    }
    const long long cap = 8LL * std::max(L.d.col_cap, 1) + 64;
    for (;;) {
      ncell = 1LL * L.cg.nc[0] * L.cg.nc[1] * L.cg.nc[2];
      if (ncell <= cap) break;
      int k = 0;
      for (int a = 1; a < 3; ++a)
        if (L.cg.nc[a] > L.cg.nc[k]) k = a;
      L.cg.nc[k] = std::max(1, L.cg.nc[k] / 2);
    }
    L.cg.ncell = static_cast<int>(ncell);
    L.cstart.alloc(static_cast<size_t>(ncell) + 1);
    L.ccount.alloc(static_cast<size_t>(ncell));
    L.ccursor.alloc(static_cast<size_t>(ncell));
    L.cjnd.alloc(std::max<size_t>(static_cast<size_t>(L.d.col_cap), 1));
    L.catom.alloc(std::max<size_t>(static_cast<size_t>(L.d.col_cap), 1));
    L.cposq.alloc(std::max<size_t>(static_cast<size_t>(L.d.col_cap), 1));
    L.ccell.alloc(std::max<size_t>(static_cast<size_t>(L.d.col_cap), 1));
    L.cg.start = L.cstart.p;
    L.cg.count = L.ccount.p;
    L.cg.cursor = L.ccursor.p;
    L.cg.jnd = L.cjnd.p;
    L.cg.atom = L.catom.p;
    L.cg.posq = L.cposq.p;
    L.cg.cell_of = L.ccell.p;
    L.has_grid = true;
  }
}

void Engine::read_ctl() {
  CK(cudaMemcpyAsync(hctl, ctl, ctl_head, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  ctl_fresh = true;
}

void Engine::upload_ctl_groups() {
  CK(cudaMemcpyAsync(ctl->group_n, hctl->group_n, sizeof(hctl->group_n), cudaMemcpyHostToDevice, st));
}

// Reports a device-side stop with the reference's messages and throws.
void Engine::raise_device_error() {
  const Ctl& c = *hctl;
  md_step = c.err_step;  // the loop stopped inside this step, as the reference's stop does
  std::string msg;
  switch (c.err_kind) {
    case EK_OVERFLOW:
    case EK_CONVERSE_OVF:
      msg = "error: too many neighbours" + fortio::list_int(c.err_info[1]) + fortio::list_int(c.err_info[2]);
      break;
    case EK_OOB: {
      std::vector<double> p, v;
      get_state_host(p, v, nullptr);
      for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
          double x = p[3 * i + k];
          if (!(x > (0.0 - 0.0000001) && x < (box.L[k] + 0.0000001)))
            outln(fortio::list_int(i + 1) + " particle out of cell " + fortio::list_real(p[3 * i]) +
                  fortio::list_real(p[3 * i + 1]) + fortio::list_real(p[3 * i + 2]));
        }
      msg = "particle out of cell";
      break;
    }
    case EK_GR_TOO_MANY:
      msg = "error: too many gr nearest neibs" + fortio::list_int(c.err_info[0]);
      break;
    case EK_GR_NOT_ENOUGH:
      msg = "error: not enough gr nearest neibs" + fortio::list_int(c.err_info[0]);
      break;
    case EK_L1:
      msg = "l1>3";
      break;
    default:
      if (c.error == PFMD_E_PARAM)
        msg = "error: group1%N>nl%N" + fortio::list_int(c.err_info[1]) + fortio::list_int(c.err_info[2]);
      else if (c.error == PFMD_E_TIMEOUT)
        msg = "error: a bounded device wait gave up (block" + fortio::list_int(c.err_info[0]) + ")";
      else
        msg = "device error";
  }
  if (c.err_kind != EK_OOB) outln(" " + msg);
  flush_out();
  printed = true;
  throw Error(c.error ? c.error : PFMD_E_STATE, msg + " (md_step " + std::to_string(c.err_step) + ")");
}

// ---------------------------------------------------------------------------
// step planning
// ---------------------------------------------------------------------------
bool Engine::switch_needed(long long s) const {
  if (integrator_index == 0) return true;
  long long sum = 0;
  for (int k = 1; k <= integrator_index && k <= static_cast<int>(S.integrators.size()); ++k)
    sum += S.integrators[static_cast<size_t>(k - 1)].l;
  return s - 1 == sum;
}

// md_simulation.f90:121-136
bool Engine::do_switch() {
  const int n = static_cast<int>(S.integrators.size());
  integrator_index = integrator_index + 1;
  int i = integrator_index;
  for (; i <= n; ++i) {
    const auto& is = S.integrators[static_cast<size_t>(i - 1)];
    if (is.l > 0) {
      integrator_name = is.name;
      for (int k = 0; k < 4; ++k) ts[k] = is.dt / static_cast<double>(1 << k);
      integ = (fortio::trim(is.name) == "nvt") ? I_NVT : (fortio::trim(is.name) == "nvms") ? I_NVMS : I_NVE;
      break;
    }
  }
  if (i > n) return false;
  integrator_index = i;
  return true;
}

StepPlan Engine::plan(long long s) const {
  StepPlan p;
  p.step = s;
  p.first = (s == 0);
  const auto& I = S.integrators[static_cast<size_t>(integrator_index - 1)];
  p.energy = (s % I.period_log == 0) || (s % opt.out_period == 0) || integ == I_NVMS;
  p.out = (s % opt.out_period == 0) && opt.out_fd >= 0;
  p.zero_mom = (s % S.zero_momentum_period == 0);
  p.check_all = need_check_all;
  p.rebuild.resize(lists.size());
  for (size_t k = 0; k < lists.size(); ++k) {
    const ListH& L = lists[k];
    long long per = L.period;
    if (L.kind == L_CONVERSE) per = lists[static_cast<size_t>(L.src)].period;
    // after set_state the first step also updates the lists
    p.rebuild[k] = (s % per == 0 || need_check_all) ? 1 : 0;
  }
  return p;
}

bool Engine::is_event(const StepPlan& p) const { return log_step(p) || hard_event(p); }

bool Engine::log_step(const StepPlan& p) const {
  const auto& I = S.integrators[static_cast<size_t>(integrator_index - 1)];
  return log && p.step % I.period_log == 0;
}

// Events that need the host between steps (output block, files, the learned
// form's check).  A log line does not: log steps record their values on the
// device and the lines are written at the segment's end, in step order.
bool Engine::hard_event(const StepPlan& p) const {
  const auto& I = S.integrators[static_cast<size_t>(integrator_index - 1)];
  if (learned_active && check_period > 0 && p.step > 0 && p.step % check_period == 0) return true;
  if (p.out) return true;
  if (opt.write_files && p.step % I.period_snapshot == 0 && p.step != 0) return true;
  if (opt.write_files && p.step % S.period_traj == 0) return true;
  return false;
}

void Engine::enqueue_lists(const StepPlan& p) {
  for (auto& I : inters) {
    ListH& L1 = lists[static_cast<size_t>(I.lists[0])];
    const bool skin = L1.d.skin >= 0 && p.rebuild[static_cast<size_t>(I.lists[0])];
    ListH* O = (skin && L1.outer) ? L1.outer.get() : nullptr;
    if (skin)
      launch_skin_check(L1.d, A, box, L1.xref.p, L1.xprev.p, O ? L1.xout.p : nullptr, L1.half_skin,
                        0.5 * kOuterMargin - kOuterTol, ctl, st);
    if (p.rebuild[static_cast<size_t>(I.lists[0])]) {
      const double pm = 1e-3 + 4e-6 * std::max(box.L[0], std::max(box.L[1], box.L[2]));
      if (O) {
        // the outer list's kernels return at once unless it must be rebuilt too
        launch_bin(O->d, O->cg, A, ctl, st);
        launch_build_list(prec, O->d, O->cg, A, box, O->rc, pm, 0, 0, ctl, st);
        launch_filter_outer(L1.d, O->d, A, box, L1.rc, ctl, st);
      } else {
        launch_bin(L1.d, L1.cg, A, ctl, st);
        launch_build_list(prec, L1.d, L1.cg, A, box, L1.rc, pm, 0, 0, ctl, st);
      }
    }
    if (I.lists[1] >= 0 && p.rebuild[static_cast<size_t>(I.lists[1])]) {
      ListH& L2 = lists[static_cast<size_t>(I.lists[1])];
      launch_bin(L2.d, L2.cg, A, ctl, st);
      launch_build_list(prec, L2.d, L2.cg, A, box, L2.rc, 1e-3 + 4e-6 * std::max(box.L[0], std::max(box.L[1], box.L[2])),
                        1, L1.d.rows, ctl, st);
    }
    if (skin) launch_skin_commit(L1.d, A, L1.xref.p, O ? L1.xout.p : nullptr, ctl, st);
    if (I.lists[2] >= 0 && p.rebuild[static_cast<size_t>(I.lists[2])]) {
      ListH& L3 = lists[static_cast<size_t>(I.lists[2])];
      if (L3.kind == L_NN_TB) {
        if (L3.d.nmax != 3) {
          // find_gr_nearest_neighbors checks this on every selection (graphenenorm.f90:13)
          throw Error(PFMD_E_GR_NN, "error: nl_nn%neighb_num_max/=nnum_nn");
        }
        launch_nn_select(prec, lists[static_cast<size_t>(L3.src)].d, L3.d, I.rc_nn, A, box, ctl, st);
      } else {
        launch_bin(L3.d, L3.cg, A, ctl, st);
        launch_build_list(prec, L3.d, L3.cg, A, box, L3.rc, 1e-3 + 4e-6 * std::max(box.L[0], std::max(box.L[1], box.L[2])),
                          0, 0, ctl, st);
      }
    }
  }
  for (auto& I : inters)
    if (I.lists[2] >= 0)
      launch_normals(prec, lists[static_cast<size_t>(I.lists[2])].d, I.norm.p, I.cp.simplified, A, box, ctl, st);
}

// The force kernels that write forces, in launch order, and whether the first
// may store (its rows are exactly the all-atoms group, the only group zero_forces
// clears) and the last may kick (its rows hold every xyz and z atom).
void Engine::plan_fusion() {
  struct W {
    int list;
    bool epi;
  };
  std::vector<W> w;
  for (auto& I : inters) {
    switch (I.spec.kind) {
      case pfmd_io::K_LJ:
        w.push_back({I.lists[0], true});
        w.push_back({I.lists[1], true});
        break;
      case pfmd_io::K_LJC:
      case pfmd_io::K_MORSEC:
        w.push_back({I.lists[0], false});
        w.push_back({I.lists[1], false});
        break;
      default:
        w.push_back({I.lists[0], true});
    }
  }
  if (w.empty() || !changes.empty()) return;
  auto rows_set = [&](int li) {
    const ListH& L = lists[static_cast<size_t>(li)];
    std::vector<char> s(static_cast<size_t>(N), 0);
    const auto& g = groups[static_cast<size_t>(L.d.row_group)].idx;
    for (size_t r = 0; r < g.size() && r < static_cast<size_t>(L.d.rows); ++r) s[static_cast<size_t>(g[r])] = 1;
    return s;
  };
  const auto& all = groups[static_cast<size_t>(S.all_atoms - 1)].idx;
  {
    const ListH& L0 = lists[static_cast<size_t>(w.front().list)];
    const auto& g0 = groups[static_cast<size_t>(L0.d.row_group)].idx;
    std::vector<char> sa(static_cast<size_t>(N), 0);
    for (int a : all) sa[static_cast<size_t>(a)] = 1;
    store_first = w.front().epi && L0.d.rows == static_cast<int>(g0.size()) && rows_set(w.front().list) == sa;
  }
  if (fuse_kick_drift && w.back().epi) {
    const auto s = rows_set(w.back().list);
    bool cover = true;
    std::vector<unsigned char> fl(static_cast<size_t>(N), 0);
    for (int a : groups[static_cast<size_t>(S.xyz_moving - 1)].idx) fl[static_cast<size_t>(a)] |= 1;
    for (int a : groups[static_cast<size_t>(S.z_moving - 1)].idx) fl[static_cast<size_t>(a)] |= 2;
    for (int a = 0; a < N; ++a)
      if (fl[static_cast<size_t>(a)] && !s[static_cast<size_t>(a)]) cover = false;
    if (cover) {
      kick_last = true;
      mflag.alloc(static_cast<size_t>(std::max(N, 1)));
      mflag.upload(fl.data(), fl.size(), st);
    }
  }
}

// The per-atom moving flags that the force kernels' fused kick reads, from the
// current sizes of the xyz- and z-moving groups (pfmd_set_group_n changes them
// between steps, as change_particle_group_N does inside md()).
void Engine::refresh_mflag() {
  if (!kick_last || !mflag.p) return;
  std::vector<unsigned char> fl(static_cast<size_t>(N), 0);
  auto mark = [&](int g1based, unsigned char bit) {
    const auto& idx = groups[static_cast<size_t>(g1based - 1)].idx;
    const int cap = static_cast<int>(idx.size());
    const int n = hctl ? std::min<int>(hctl->group_n[g1based - 1], cap) : cap;
    for (int k = 0; k < n; ++k) fl[static_cast<size_t>(idx[static_cast<size_t>(k)])] |= bit;
  };
  mark(S.xyz_moving, 1);
  mark(S.z_moving, 2);
  if (nhc_fused) mark(S.nhc[0].group, 4);
  mflag.upload(fl.data(), fl.size(), st);
}

// All-pairs fusion: every interaction is lj or lj1g (at most kMaxPairSlots lists
// and kMaxPairKeys interactions), the all-atoms group holds every atom, the
// moving groups are disjoint and no group changes size.  One atom-major kernel
// then forms, stores and kicks every atom's force.  Chain 0 fuses in as well
// when it is the only chain and no z-velocity inversion runs between the steps.
void Engine::plan_pair_fusion() {
  if (!opt.fuse_steps || inters.empty() || !changes.empty() || N == 0 || !fuse_kick_drift) return;
  int nslot = 0;
  for (const auto& I : inters) {
    if (I.spec.kind == pfmd_io::K_LJ)
      nslot += 2;
    else if (I.spec.kind == pfmd_io::K_LJ1G)
      nslot += 1;
    else
      return;
  }
  if (nslot > kMaxPairSlots || static_cast<int>(inters.size()) > kMaxPairKeys) return;
  if (static_cast<int>(groups[static_cast<size_t>(S.all_atoms - 1)].idx.size()) != N) return;
  // an atom's tasks: the rows it heads, in slot order (lj rows before lj1g rows
  // in the usual settings, so the kinds agree across a warp); and the slot table:
  // the fields of each list the row loops read (list buffers keep their
  // addresses for the life of the engine) and the parameters
  std::vector<std::vector<int2>> t(static_cast<size_t>(N));
  std::vector<PairSlot> slots;
  double cap = 0.0;
  int key = 0;
  for (const auto& I : inters) {
    const int nl = I.spec.kind == pfmd_io::K_LJ ? 2 : 1;
    for (int j = 0; j < nl; ++j) {
      const ListH& L = lists[static_cast<size_t>(I.lists[j])];
      const auto& g = groups[static_cast<size_t>(L.d.row_group)].idx;
      const int slot = static_cast<int>(slots.size());
      for (int r = 0; r < L.d.rows && r < static_cast<int>(g.size()); ++r) {
        t[static_cast<size_t>(g[static_cast<size_t>(r)])].push_back(make_int2(slot, r));
        cap += 0.5 * std::max(L.d.nmax, 2);
      }
      PairSlot sl{};
      sl.L = RowList{L.d.nnum, L.d.nlist, L.d.lessnnum, L.d.bnd, L.d.row_of, L.d.stride, L.d.sorted};
      sl.P = I.lj;
      sl.kind = I.spec.kind == pfmd_io::K_LJ ? 0 : 1;
      sl.general = I.general ? 1 : 0;
      sl.ekey = j == 0 ? key : -1;  // lj's energy is that of its first list (LennardJones.f90:23-46)
      slots.push_back(sl);
    }
    ++key;
  }
  std::vector<int> off(static_cast<size_t>(N) + 1, 0);
  std::vector<int2> flat;
  for (int a = 0; a < N; ++a) {
    off[static_cast<size_t>(a) + 1] = off[static_cast<size_t>(a)] + static_cast<int>(t[static_cast<size_t>(a)].size());
    for (const int2& x : t[static_cast<size_t>(a)]) flat.push_back(x);
  }
  pair_off.alloc(off.size());
  pair_off.upload(off.data(), off.size(), st);
  pair_task.alloc(std::max<size_t>(flat.size(), 1));
  if (!flat.empty()) pair_task.upload(flat.data(), flat.size(), st);
  pair_slots.alloc(slots.size());
  pair_slots.upload(slots.data(), slots.size(), st);
  pair_fused = true;
  store_first = true;
  kick_last = true;
  nhc_fused = S.nhc.size() == 1 && !S.invert_z_vel;
  mflag.alloc(static_cast<size_t>(std::max(N, 1)));
  refresh_mflag();
  // until tune_tpa measures the rows: half of each headed row's capacity
  pair_tpa = opt.threads_per_row > 0 ? opt.threads_per_row : auto_tpa(N, cap / N, prec);
  CK(cudaStreamSynchronize(st));
}

void Engine::plan_force_split() {
  force_split = false;
  if (pair_fused || N == 0 || inters.size() < 2) return;
  int cos = -1;
  for (size_t k = 0; k < inters.size(); ++k) {
    const int kind = inters[k].spec.kind;
    if (kind == pfmd_io::K_LJC || kind == pfmd_io::K_MORSEC) {
      if (cos >= 0) return;
      cos = static_cast<int>(k);
    } else if (kind != pfmd_io::K_RJL && kind != pfmd_io::K_TB && kind != pfmd_io::K_LJ1G) {
      return;  // kernels not known to write only their own rows
    }
  }
  if (cos < 0) return;
  std::vector<char> side(static_cast<size_t>(N), 0);
  auto mark = [&](int g, char s) {
    for (int a : groups[static_cast<size_t>(g)].idx) {
      if (side[static_cast<size_t>(a)] && side[static_cast<size_t>(a)] != s) return false;
      side[static_cast<size_t>(a)] = s;
    }
    return true;
  };
  const InterH& C = inters[static_cast<size_t>(cos)];
  if (!mark(lists[static_cast<size_t>(C.lists[0])].d.row_group, 1) ||
      !mark(lists[static_cast<size_t>(C.lists[1])].d.row_group, 2))
    return;
  std::vector<int> fs(inters.size(), 0);
  fs[static_cast<size_t>(cos)] = 3;
  for (size_t k = 0; k < inters.size(); ++k) {
    if (static_cast<int>(k) == cos) continue;
    char s = 0;
    for (int a : groups[static_cast<size_t>(lists[static_cast<size_t>(inters[k].lists[0])].d.row_group)].idx) {
      const char t = side[static_cast<size_t>(a)];
      if (t == 0 || (s != 0 && t != s)) return;
      s = t;
    }
    if (s == 0) return;
    fs[k] = s;
  }
  if (!st2) CK(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking));
  if (!ev_fork) CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
  if (!ev_join) CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  force_side = fs;
  force_split = true;
}

PairSet Engine::pair_set() const {
  PairSet P{};
  P.natoms = N;
  P.tpa = pair_tpa;
  P.task_off = pair_off.p;
  P.task = pair_task.p;
  P.slots = pair_slots.p;
  int slot = 0;
  for (size_t k = 0; k < inters.size(); ++k) {
    slot += inters[k].spec.kind == pfmd_io::K_LJ ? 2 : 1;
    P.keys[k] = static_cast<int>(k);
  }
  P.nslot = slot;
  P.nkey = static_cast<int>(inters.size());
  return P;
}

void Engine::enqueue_forces(bool energy, bool kick, bool drift_next, bool begin) {
  if (pair_fused && !learned_active) {
    // every lj / lj1g list in one launch: stores every force, kicks (second half)
    // and, under nvt, reduces and updates chain 0
    Epi e{1, kick ? 1 : 0, prec ? 0 : 1, ts[1], mflag.p, eatom_out};
    const int chain = (kick && nhc_fused && integ == I_NVT) ? 0 : -1;
    launch_pair_atoms(prec, energy, pair_set(), A, box, ctl, st, e, chain, ts[1], ts[2], ts[3],
                      chain == 0 && nhc_ahead);
    return;
  }
  // which launch is the first / last force writer
  const int nint = static_cast<int>(inters.size());
  auto epi = [&](bool first, bool last) {
    Epi e{0, 0, prec ? 0 : 1, ts[1], mflag.p, eatom_out};
    e.store = (first && store_first) ? 1 : 0;
    e.kick = (last && kick && kick_last) ? 1 : 0;
    if (last && e.kick && drift_next) {
      e.drift = 1;
      e.ts1 = ts[0];
      e.posq_next = posq_cur ? posq.p : posq2.p;
    }
    e.begin = (first && begin) ? 1 : 0;
    return e;
  };
  const bool split = force_split && !energy;
  if (split) {
    CK(cudaEventRecord(ev_fork, st));
    CK(cudaStreamWaitEvent(st2, ev_fork, 0));
  }
  for (int k = 0; k < nint; ++k) {
    InterH& I = inters[static_cast<size_t>(k)];
    const int key = k;
    const int eslot = 4 + (k % 16);
    const bool first = k == 0, last = k == nint - 1;
    const ListDev& L1 = lists[static_cast<size_t>(I.lists[0])].d;
    cudaStream_t sk = (split && force_side[static_cast<size_t>(k)] == 2) ? st2 : st;
    if (learned_active && k < static_cast<int>(lrn.size()) && lrn[static_cast<size_t>(k)].on) {
      Lrn& M = lrn[static_cast<size_t>(k)];
      // (each model's kernels write its own buffers and its rows' forces only)
      learned::launch_desc(L1, M.d.p, A, box, M.G.p, ctl, sk);
      if (M.tc)
        learned::launch_mlp_tc(L1.rows, M.G.p, M.d.p, M.net.p, M.e.p, M.g.p, ctl, sk);
      else
        learned::launch_mlp(L1.rows, M.G.p, M.d.p, M.net.p, M.e.p, M.g.p, ctl, sk);
      learned::launch_force(L1, M.d.p, M.g.p, M.e.p, M.leg.p, M.cforce.p, energy, A, box, ctl, eslot, key, sk,
                            epi(first, last), learned::core_radius(M.model.kind));
      continue;
    }
    switch (I.spec.kind) {
      case pfmd_io::K_LJ:
        launch_lj(prec, energy, L1, I.lj, A, box, ctl, eslot, key, st, epi(first, false));
        launch_lj(prec, false, lists[static_cast<size_t>(I.lists[1])].d, I.lj, A, box, ctl, eslot, key, st,
                  epi(false, last));
        break;
      case pfmd_io::K_LJ1G:
        launch_lj1g(prec, energy, I.general, L1, I.lj, A, box, ctl, eslot, key, sk, epi(first, last));
        break;
      case pfmd_io::K_RJL:
        launch_rjl(prec, energy, L1, I.rjl, A, box, I.scratch.p, I.pair.p, ctl, eslot, key, sk, 3,
                   epi(first, last));
        break;
      case pfmd_io::K_TB:
        launch_tb(prec, energy, L1, I.tb, A, box, I.scratch.p, ctl, eslot, key, sk, 3, epi(first, last));
        break;
      case pfmd_io::K_REBOSC:
        launch_rebo(energy, L1, I.rebo, A, box, I.scratch.p, ctl, eslot, key, st, 3, epi(first, last));
        break;
      case pfmd_io::K_LJC:
      case pfmd_io::K_MORSEC: {
        const bool morse = I.spec.kind == pfmd_io::K_MORSEC;
        const ListDev& L2 = lists[static_cast<size_t>(I.lists[1])].d;
        const ListDev& L3 = lists[static_cast<size_t>(I.lists[2])].d;
        if (split) {  // the sheet's side on st, the metal's on st2
          launch_cos(prec, energy, morse, L1, L2, L3, I.cp, I.norm.p, I.gsum.p, A, box, ctl, eslot, key, st, 1);
          launch_cos(prec, energy, morse, L1, L2, L3, I.cp, I.norm.p, I.gsum.p, A, box, ctl, eslot, key, st2, 2);
        } else {
          launch_cos(prec, energy, morse, L1, L2, L3, I.cp, I.norm.p, I.gsum.p, A, box, ctl, eslot, key, st);
        }
        break;
      }
    }
  }
  if (split) {
    CK(cudaEventRecord(ev_join, st2));
    CK(cudaStreamWaitEvent(st, ev_join, 0));
  }
}

// One pass of md()'s loop body on the device (md_simulation.f90:116-231).
void Engine::enqueue_step(const StepPlan& p) {
  const bool nvms = integ == I_NVMS, nvt = integ == I_NVT;
  if (p.check_all) launch_check_all(A, box, ctl, st);
  // an nve step without group changes lets the kick-drift kernel open the step
  // (nvt too when the previous step ran this step's chain half-update: then the
  // kick-drift is the step's first kernel)
  const bool fused_begin = !p.first && (integ == I_NVE || (nvt && p.nhc_done)) && changes.empty() &&
                           !S.invert_z_vel && fuse_kick_drift &&
                           groups[static_cast<size_t>(S.xyz_moving - 1)].idx.size() > 0;
  // a drifted step (its kick and drift ran in the previous step's force kernel)
  // that launches nothing before a single rjl interaction opens in that
  // interaction's density pass
  bool begin_in_forces = false;
  if (p.drifted) {
    bool rebuilds = false;
    for (char r : p.rebuild) rebuilds = rebuilds || r;
    begin_in_forces = !rebuilds && !p.zero_mom && store_first && inters.size() == 1 &&
                      inters[0].spec.kind == pfmd_io::K_RJL && inters[0].lists[2] < 0 && !learned_active;
    if (!begin_in_forces) launch_step_begin_fused(ctl, st);
  } else if (fused_begin) {
    // (nothing: k_kick_drift below)
  } else if (S.invert_z_vel) {
    launch_step_begin(0, static_cast<int>(changes.size()), changes.data(), 0, S.ms_de, ctl, st);
    launch_invert_z(A, box, ctl, st);
    launch_step_begin(1, 0, nullptr, nvms ? 1 : 0, S.ms_de, ctl, st);
  } else {
    launch_step_begin(2, static_cast<int>(changes.size()), changes.data(), nvms ? 1 : 0, S.ms_de, ctl, st);
  }
  const GroupRef gx = gref(S.xyz_moving), gz = gref(S.z_moving);
  if (!p.first) {
    int scale_chain = 0;
    if (nvt)
      for (size_t c = 0; c < S.nhc.size(); ++c) {
        const GroupRef gc = gref(S.nhc[c].group);
        if (c == 0 && p.nhc_done) {  // updated by the previous step's pair kernel
          scale_chain = 1;
          continue;
        }
        // a pending scaling of chain 0 (the previous step's second half) comes first
        launch_nhc(static_cast<int>(c), gc, ts[1], ts[2], ts[3], A, ctl, st, (c == 0 && nhc_pending) ? 1 : 0);
        if (c == 0) nhc_pending = false;
        if (static_cast<int>(c) == fused_nhc_chain)
          scale_chain = static_cast<int>(c) + 1;
        else
          launch_scale(static_cast<int>(c), gc, A, ctl, st);
      }
    if (p.drifted) {
      // (done)
    } else if (fuse_kick_drift) {
      // the fused pair kernel may start early: it reads its static tables while
      // this one runs (a kernel between them is an ordinary launch and waits)
      launch_kick_drift(gx, ts[0], ts[1], true, scale_chain, !prec, A, box, ctl, st, fused_begin, p.nhc_done,
                        pair_fused && !learned_active);
      if (gz.cap > 0) {
        launch_kick(gz, false, ts[1], !prec, A, ctl, st);
        launch_drift(gz, false, ts[0], true, A, box, ctl, st);
      }
    } else {
      launch_kick(gx, true, ts[1], !prec, A, ctl, st);
      launch_kick(gz, false, ts[1], !prec, A, ctl, st);
      launch_drift(gx, true, ts[0], true, A, box, ctl, st);
      launch_drift(gz, false, ts[0], true, A, box, ctl, st);
    }
  }
  enqueue_lists(p);
  const GroupRef gall = gref(S.all_atoms);
  if (p.zero_mom) launch_zero_momentum(gall, A, ctl, st);
  if (!store_first) launch_zero_forces(gall, A, ctl, st);
  nhc_ahead = p.nhc_ahead;
  enqueue_forces(p.energy, !p.first, p.drift_next, begin_in_forces);
  nhc_ahead = false;
  if (p.drift_next) flip_posq();  // the next step reads the positions written by this one
  if (!p.first) {
    // the chain's group is the kicked one and nothing else is kicked: the kick
    // and the chain's half-update run as one kernel
    const bool kick_nhc = !kick_last && nvt && fused_nhc_chain == 0 && gz.cap == 0 &&
                          !(nhc_fused && pair_fused && !learned_active);
    if (kick_nhc) {
      launch_kick_nhc(gx, ts[1], !prec, 0, ts[1], ts[2], ts[3], p.nhc_ahead, A, ctl, st);
      if (!p.nhc_ahead) launch_scale(0, gx, A, ctl, st);
    } else if (!kick_last) {
      launch_kick(gx, true, ts[1], !prec, A, ctl, st);
      if (gz.cap > 0) launch_kick(gz, false, ts[1], !prec, A, ctl, st);
    }
    if (nvt && !kick_nhc)
      for (size_t c = 0; c < S.nhc.size(); ++c) {
        const GroupRef gc = gref(S.nhc[c].group);
        if (c == 0 && nhc_fused && pair_fused && !learned_active) {
          // the pair kernel reduced the kinetic energy and updated the chain
          if (p.nhc_ahead)
            ;  // and the next step's first half: the next kick-drift scales
          else if (p.nhc_defer)
            nhc_pending = true;
          else
            launch_scale(0, gc, A, ctl, st);
          continue;
        }
        if (c == 0 && p.nhc_ahead) {  // with the next first half; the next kick-drift scales
          launch_nhc(0, gc, ts[1], ts[2], ts[3], A, ctl, st, 0, 1);
          continue;
        }
        launch_nhc(static_cast<int>(c), gc, ts[1], ts[2], ts[3], A, ctl, st);
        launch_scale(static_cast<int>(c), gc, A, ctl, st);
      }
    if (nvms) {
      launch_ms(gx, true, A, ctl, st);
      if (gz.cap > 0) launch_ms(gz, false, A, ctl, st);
    }
  }
  if (p.energy)
    launch_energy_finalize(gref(S.all_moving), static_cast<int>(inters.size()), static_cast<int>(S.nhc.size()),
                           nvt ? 1 : 0, A, ctl, st);
  if (p.log_row >= 0) launch_log_row(ctl, log_ring.p + static_cast<size_t>(p.log_row) * kLogCols, st);
  if (p.out) {
    launch_out_reduce(gall, A, ctl, st);
    CK(cudaMemsetAsync(ctl->maxnnum, 0, sizeof(int) * PFMD_MAX_LISTS, st));
    for (auto& L : lists) launch_nnum_max(L.d, ctl, st);
  }
}

static std::string plan_key(const StepPlan& p) {
  std::string k;
  k.reserve(8 + p.rebuild.size());
  k.push_back(static_cast<char>('A' + (p.first ? 1 : 0) + 2 * (p.energy ? 1 : 0) + 4 * (p.out ? 1 : 0) +
                                8 * (p.zero_mom ? 1 : 0) + 16 * (p.check_all ? 1 : 0)));
  k.push_back(static_cast<char>('a' + (p.drift_next ? 1 : 0) + 2 * (p.drifted ? 1 : 0) + 4 * (p.nhc_defer ? 1 : 0) +
                                8 * (p.nhc_ahead ? 1 : 0)));
  k.push_back(p.nhc_done ? 'd' : '-');
  // (a log step's row is its rank among the segment's log steps, which the
  // key's earlier steps fix)
  k.push_back(p.log_row >= 0 ? 'L' : '-');
  for (char r : p.rebuild) k.push_back(r ? '1' : '0');
  k.push_back('|');
  return k;
}

void Engine::run_plans(const std::vector<StepPlan>& plans) {
  if (timing && !timing_started) {
    CK(cudaEventRecord(ev0, st));
    timing_started = true;
  }
  struct RecordEnd {
    Engine* e;
    ~RecordEnd() {
      if (e->timing) cudaEventRecord(e->ev1, e->st);
    }
  } record_end{this};
  // the key carries the positions buffer the segment starts from: a graph replays
  // the buffer pointers it captured
  std::string key = std::to_string(integrator_index) + ":" + std::to_string(posq_cur) + ":";
  int flips = 0;
  for (const auto& p : plans) {
    key += plan_key(p);
    flips += p.drift_next ? 1 : 0;
  }
  GraphEntry* ge = nullptr;
  if (opt.use_graphs && plans.size() >= 2) {
    ge = &graphs[key];
    ge->seen++;
  }
  if (ge && ge->exec) {
    CK(cudaGraphLaunch(ge->exec, st));
    launches += ge->kernels;
    if (flips & 1) flip_posq();  // as enqueue_step did while the graph was captured
  } else if (ge && ge->seen >= 2) {
    if (graphs.size() > 64) {  // keep the cache bounded
      for (auto it = graphs.begin(); it != graphs.end();) {
        if (it->second.exec && it->first != key) {
          cudaGraphExecDestroy(it->second.exec);
          it = graphs.erase(it);
        } else {
          ++it;
        }
      }
      ge = &graphs[key];
    }
    cudaGraph_t g = nullptr;
    const long long before = g_kernel_launches;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      for (const auto& p : plans) enqueue_step(p);
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    CK(cudaStreamEndCapture(st, &g));
    ge->kernels = g_kernel_launches - before;
    CK(cudaGraphInstantiate(&ge->exec, g, 0));
    cudaGraphDestroy(g);
    CK(cudaGraphLaunch(ge->exec, st));
    launches += ge->kernels;
  } else {
    const long long before = g_kernel_launches;
    for (const auto& p : plans) enqueue_step(p);
    launches += g_kernel_launches - before;
  }
  need_check_all = false;
}

// A device view of a host array of n doubles, or null.  Page-locked host memory
// (cudaHostAlloc, cudaHostRegister, or a pinned tensor) is reached by the GPU
// over NVLink-C2C / PCIe, so the conversion kernels read and write it in place
// instead of going through a staging copy.  Both ends of the array must lie in
// page-locked memory with a device address; anything else (pageable memory)
// takes the staging copy.
static const double* host_view(const void* h, size_t n) {
  if (!h || n == 0) return nullptr;
  cudaPointerAttributes a0, a1;
  const double* last = static_cast<const double*>(h) + (n - 1);
  if (cudaPointerGetAttributes(&a0, h) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  const double* d = static_cast<const double*>(a0.devicePointer);
  if (static_cast<const double*>(a1.devicePointer) != d + (n - 1)) return nullptr;
  return d;
}

// The state as xyz-interleaved doubles, converted on the device and written
// straight into the destinations (any of them may be null): in place when the
// destination is page-locked, else through a staging copy.
void Engine::get_state_to(double* p, double* v, double* f) {
  if (N <= 0) return;
  const size_t n3 = 3 * static_cast<size_t>(N);
  double* dst[3] = {p, v, f};
  const double4_32a* src[3] = {pos.p, vel.p, frc.p};
  double* out[3] = {nullptr, nullptr, nullptr};
  bool staged[3] = {false, false, false};
  for (int k = 0; k < 3; ++k) {
    if (!dst[k]) continue;
    out[k] = const_cast<double*>(host_view(dst[k], n3));
    if (!out[k]) {
      if (!stage.p) stage.alloc(3 * n3);
      out[k] = stage.p + k * n3;
      staged[k] = true;
    }
  }
  launch_d4_to_xyz(N, src, out, st);
  for (int k = 0; k < 3; ++k)
    if (staged[k])
      CK(cudaMemcpyAsync(dst[k], stage.p + k * n3, sizeof(double) * n3, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
}

void Engine::get_state_host(std::vector<double>& p, std::vector<double>& v, std::vector<double>* f) {
  p.resize(3 * static_cast<size_t>(N));
  v.resize(3 * static_cast<size_t>(N));
  if (f) f->resize(3 * static_cast<size_t>(N));
  get_state_to(p.data(), v.data(), f ? f->data() : nullptr);
}

std::string Engine::nlists_load_text() {  // md_interactions.f90:427-444
  std::string s;
  if (!inters.empty()) s += "neib lists load:\n";
  for (auto& I : inters) {
    const int nl_n = I.spec.nl_n;
    for (int j = 0; j < nl_n; ++j) {
      const ListH& L = lists[static_cast<size_t>(I.lists[j])];
      int mx = L.d.rows > 0 ? hctl->maxnnum[L.d.id] : 0;
      s += fortio::Rec().a(fortio::trim(I.spec.name), 8).i(j + 1, 3).i(mx, 6).a(" /").i(L.d.nmax, 6).s + "\n";
    }
  }
  return s;
}

// Host work after an event step: log line, output block, snapshot, trajectory
// (md_simulation.f90:204-241).
// The log line (A6,i9,7f24.6 then the interactions' and chains' energies,
// md_simulation.f90:204-207) of step s at simulation time t from a log record.
void Engine::write_log_line(long long s, double t, const double* row) {
  fortio::Rec r;
  r.a(fortio::trim(integrator_name), 6).i(s, 9);
  r.f(t, 24, 6).f(row[0], 24, 6).f(row[1], 24, 6).f(row[2], 24, 6).f(row[3], 24, 6);
  r.f(row[4], 24, 6).f(row[5], 24, 6);
  for (size_t k = 0; k < inters.size(); ++k) r.f(row[6 + k], 20, 9);
  for (size_t k = 0; k < S.nhc.size(); ++k) r.f(row[6 + kLogInter + k], 20, 9);
  std::string line = r.s + "\n";
  std::fputs(line.c_str(), log);
}

void Engine::host_events(const StepPlan& p, bool log_line) {
  const long long s = p.step;
  const auto& I = S.integrators[static_cast<size_t>(integrator_index - 1)];
  const Ctl& c = *hctl;
  if (log_line && log && s % I.period_log == 0) {
    double row[kLogCols];
    row[0] = c.conserved;
    row[1] = c.e_nhc;
    row[2] = c.total;
    row[3] = c.pe_last;
    row[4] = c.ke;
    row[5] = c.temperature;
    for (int k = 0; k < kLogInter; ++k) row[6 + k] = c.e_inter[k];
    for (int k = 0; k < kLogChains; ++k) row[6 + kLogInter + k] = c.nhc[k].e;
    write_log_line(s, sim_time, row);
  }
  if (p.out) {
    const double fs = std::sqrt(c.red[0] * c.red[0] + c.red[1] * c.red[1] + c.red[2] * c.red[2]);
    const double mv[3] = {c.red[6] / c.red[9], c.red[7] / c.red[9], c.red[8] / c.red[9]};
    const double mcv = std::sqrt(mv[0] * mv[0] + mv[1] * mv[1] + mv[2] * mv[2]);
    outln(fortio::Rec().a("exe time (s) = ").f(now_s() - t_start, 10, 2).s);
    outln(fortio::Rec().a("step = ").i(s, 12).a(" integrator = ").a(fortio::trim(integrator_name), 6).s);
    outln(fortio::Rec().a("conserved energy (eV) = ").es(c.conserved, 21, 9).s);
    outln(fortio::Rec().a("forces sum (eV/A) = ").es(fs, 16, 6).s);
    outln(fortio::Rec().a("c.o.m. velocity (A/fs) = ").es(mcv, 16, 6).s);
    outln(fortio::Rec()
              .a("c.o.m. position (A) = ")
              .f(c.red[3] / c.red[9], 12, 6)
              .f(c.red[4] / c.red[9], 12, 6)
              .f(c.red[5] / c.red[9], 12, 6)
              .s);
    outln(fortio::Rec().a("maximum velocity (A/fs) = ").f(std::sqrt(c.red[10]), 12, 6).s);
    out(nlists_load_text());
    if (integ != I_NVMS && fs > 1e-14) outln(" WARNING: forces sum is too big");
    if (integ == I_NVT && S.xyz_moving == S.all_atoms && mcv > 1e-14)
      outln(" WARNING: center of mass velocity is too big");
    outln("");
  }
  const bool snap = opt.write_files && s % I.period_snapshot == 0 && s != 0;
  const bool traj = opt.write_files && s % S.period_traj == 0;
  check_writer(false);
  if (snap || traj) {
    // the step's state, shared by the jobs that format it
    auto st8 = std::make_shared<std::pair<std::vector<double>, std::vector<double>>>();
    get_state_host(st8->first, st8->second, nullptr);
    const std::array<double, 3> L3 = {box.L[0], box.L[1], box.L[2]};
    const double* mass = S.xyz.mass.data();
    const std::vector<std::string>* types = &S.xyz.types;
    if (snap) {
      const auto& g = groups[static_cast<size_t>(S.all_atoms - 1)];
      const int gn = hctl->group_n[S.all_atoms - 1];
      const int* idx = g.idx.data();
      emit_file(prefix + "snapshot_" + fortio::fmt_i0pad(s, 6, 6) + ".xyz", false, [=] {
        return pfmd_io::xyz_snapshot_text(L3.data(), gn, idx, st8->first.data(), st8->second.data(), mass, *types);
      });
    }
    if (traj) {
      const auto& g = groups[static_cast<size_t>(S.traj_group - 1)];
      const int gn = hctl->group_n[S.traj_group - 1];
      const int* idx = g.idx.data();
      emit_file(prefix + "traj_" + fortio::fmt_i0pad(S.traj_group, 2, 2) + ".xyz", true, [=] {
        return pfmd_io::xyz_traj_frame_text(L3.data(), gn, idx, st8->first.data(), st8->second.data(), mass, *types,
                                            s);
      });
    }
  }
}

void Engine::emit_file(const std::string& path, bool append, FileWriter::Format f) {
  if (writer) {
    writer->submit(path, append, std::move(f));
    return;
  }
  const std::string e = FileWriter::write(path, append, f);
  if (!e.empty()) throw Error(PFMD_E_IO, e);
}

// Raises the background writer's first error; wait: after the queued files are written.
void Engine::check_writer(bool wait) {
  if (!writer) return;
  const std::string e = wait ? writer->drain() : writer->error();
  if (!e.empty()) throw Error(PFMD_E_IO, e);
}

void Engine::advance(long long max_steps, int* fin) {
  long long done = 0;
  const size_t seg_cap = 4096;
  while (!finished && done < max_steps) {
    const long long s = md_step;
    if (s > S.md_step_limit) {
      finished = true;
      break;
    }
    if (switch_needed(s)) {
      if (!do_switch()) {
        outln(" no more integrators");
        finished = true;
        break;
      }
    }
    std::vector<StepPlan> plans;
    for (long long t = s; t <= S.md_step_limit; ++t) {
      if (t != s && switch_needed(t)) break;
      plans.push_back(plan(t));
      need_check_all = false;  // only the first planned step runs the full check
      if (hard_event(plans.back()) || plans.size() >= seg_cap ||
          done + static_cast<long long>(plans.size()) >= max_steps)
        break;
    }
    // log steps record their values on the device; the lines follow at the end
    int log_rows = 0;
    for (auto& p : plans)
      if (log_step(p)) p.log_row = log_rows++;
    if (static_cast<size_t>(log_rows) > log_cap) {
      log_cap = static_cast<size_t>(log_rows);
      log_ring.alloc(log_cap * kLogCols);
      clear_graphs();  // captured segments hold the old ring's address
      if (hlog) cudaFreeHost(hlog);
      hlog = nullptr;
      CK(cudaMallocHost(&hlog, sizeof(double) * log_cap * kLogCols));
    }
    need_check_all = plans.front().check_all;
    // each force kernel also runs the next step's kick and drift when both steps
    // are nve steps of this segment and the first computes no energies or output
    if (fuse_drift && integ == I_NVE && !learned_active)
      for (size_t i = 0; i + 1 < plans.size(); ++i) {
        StepPlan& a = plans[i];
        StepPlan& b = plans[i + 1];
        if (a.first || a.energy || a.out || b.first || b.check_all) continue;
        a.drift_next = b.drifted = true;
      }
    // chain 0's second-half scaling waits for the next step's k_nhc when both
    // steps are in this segment and the first computes no energies or output
    if (nhc_fused && pair_fused && integ == I_NVT && !learned_active)
      for (size_t i = 0; i + 1 < plans.size(); ++i) {
        StepPlan& a = plans[i];
        if (!a.first && !a.energy && !a.out) a.nhc_defer = true;
        // with chain 0's scaling in the kick-drift, the pair kernel runs the next
        // step's first half-update as well
        if (a.nhc_defer && fused_nhc_chain == 0) {
          a.nhc_ahead = true;
          plans[i + 1].nhc_done = true;
        }
      }
    // other interactions: the second half's k_nhc runs the next first half too,
    // and the next kick-drift applies both scalings (no k_scale, no k_nhc there)
    if (!pair_fused && S.nhc.size() == 1 && !S.invert_z_vel && integ == I_NVT && !learned_active &&
        fused_nhc_chain == 0 && changes.empty())
      for (size_t i = 0; i + 1 < plans.size(); ++i) {
        StepPlan& a = plans[i];
        if (a.first || a.energy || a.out || plans[i + 1].first) continue;
        a.nhc_ahead = true;
        plans[i + 1].nhc_done = true;
      }
    run_plans(plans);
    if (log_rows > 0)
      CK(cudaMemcpyAsync(hlog, log_ring.p, sizeof(double) * static_cast<size_t>(log_rows) * kLogCols,
                         cudaMemcpyDeviceToHost, st));
    read_ctl();
    if (log_rows > 0) {
      // the log lines of the steps that completed (a stop inside the segment
      // ends it at err_step), with the simulation time of each
      const long long done_to = (hctl->error || hctl->converged) ? hctl->err_step : plans.back().step + 1;
      double t = sim_time;
      for (const auto& p : plans) {
        if (p.step >= done_to) break;
        if (p.step != 0) t = t + ts[0];
        if (p.log_row >= 0) write_log_line(p.step, t, hlog + static_cast<size_t>(p.log_row) * kLogCols);
      }
    }
    if (hctl->error) raise_device_error();
    if (!tpa_tuned) tune_tpa();
    const long long executed_to = hctl->converged ? hctl->err_step : plans.back().step + 1;
    for (long long t = s; t < executed_to; ++t)
      if (t != 0) sim_time = sim_time + ts[0];
    if (hctl->converged) {
      outln(" potential energy diffrence is small enough");
      md_step = hctl->err_step;
      finished = true;
      done += md_step - s;
      break;
    }
    md_step = plans.back().step + 1;
    done += static_cast<long long>(plans.size());
    if (hard_event(plans.back())) {
      host_events(plans.back(), plans.back().log_row < 0);
      const long long ls = plans.back().step;
      if (learned_active && check_period > 0 && ls > 0 && ls % check_period == 0) learned_check(true);
    }
    flush_out();
  }
  if (md_step > S.md_step_limit) finished = true;
  flush_out();
  if (log) std::fflush(log);
  if (fin) *fin = finished ? 1 : 0;
}

// md_simulation.f90:245-272
void Engine::finish() {
  if (finished_called) throw Error(PFMD_E_STATE, "pfmd_finish was already called");
  finished_called = true;
  read_ctl();
  const double exe = now_s() - t_md;
  const Ctl& c = *hctl;
  if (integ == I_NVMS) outln(" potential energy difference: " + fortio::list_real(c.pe_last - c.pe_prev));
  outln(" steps number:" + fortio::list_int(md_step - 1));
  outln("");
  outln(" PERFOMANCE:");
  auto perf = [&](const char* name, double t) {
    outln(fortio::Rec().a(name, 24).f(t, 10, 2).a(" S ").f(t / exe * 100, 10, 2).a("%").s);
  };
  // phases run back to back on the device inside one stream; only the loop's
  // wall time is measured
  perf("MD:", exe);
  perf("POSITION AND VELOCITY:", 0.0);
  perf("NEIGHBOURS:", 0.0);
  perf("NEIGHBOURS SEARCH:", 0.0);
  perf("NEIGHBOURS DISTANCE:", 0.0);
  perf("FORCES:", 0.0);
  perf("ENERGY:", 0.0);
  perf("REST:", exe);
  outln(fortio::Rec().a("TIME STEPS PER HOUR:", 24).f(static_cast<double>(md_step) / exe * 3600, 16, 2).s);
  outln("");
  fortio::Rec r;
  r.a(fortio::trim(prefix), 32).i(md_step - 1, 9).f(sim_time, 20, 9);
  r.f(c.total, 20, 9).f(c.pe_last, 20, 9).f(c.ke, 20, 9).f(c.temperature, 20, 9);
  for (size_t k = 0; k < inters.size(); ++k) r.f(c.e_inter[k], 20, 9);
  write_all_out(r.s);
  if (log) std::fputs((r.s + "\n").c_str(), log);
  check_writer(true);  // every snapshot and trajectory frame is on disk
  if (md_step != 0 && opt.write_files) {
    std::vector<double> hp, hv;
    get_state_host(hp, hv, nullptr);
    std::string fn = prefix + "final_" + fortio::trim(S.init_xyz_filename);
    const auto& g = groups[static_cast<size_t>(S.all_atoms - 1)];
    std::string text = pfmd_io::xyz_snapshot_text(box.L, hctl->group_n[S.all_atoms - 1], g.idx.data(), hp.data(),
                                                  hv.data(), S.xyz.mass.data(), S.xyz.types);
    FILE* f = std::fopen(fn.c_str(), "w");
    if (!f) throw Error(PFMD_E_IO, "cannot open " + fn);
    std::fputs(text.c_str(), f);
    std::fclose(f);
  }
  if (log) {
    std::fclose(log);
    log = nullptr;
  }
  flush_out();
}

void Engine::clear_graphs() {
  for (auto& kv : graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  graphs.clear();
}

void Engine::learned_setup(const std::vector<learned::Model>& ms) {
  lrn.clear();
  lrn.resize(inters.size());
  int used = 0;
  for (size_t k = 0; k < inters.size(); ++k) {
    const int kind = inters[k].spec.kind == pfmd_io::K_TB ? 0 : (inters[k].spec.kind == pfmd_io::K_RJL ? 1 : -1);
    if (kind < 0) continue;
    const learned::Model* m = nullptr;
    for (const auto& x : ms)
      if (x.kind == kind) {
        m = &x;
        break;
      }
    if (!m) continue;
    Lrn& M = lrn[k];
    M.on = true;
    M.model = *m;
    ListH& L = lists[static_cast<size_t>(inters[k].lists[0])];
    // the descriptors reach past the interaction's own cut-off: its list is rebuilt
    // at every update step again
    if (L.d.skin >= 0) {
      L.d.skin = -1;
      clear_graphs();
    }
    if (L.rc < std::max(m->d.rc_rad, m->d.rc_ang))
      throw Error(PFMD_E_PARAM, "learned form: the " + inters[k].spec.name + " list needs r_cut >= " +
                                    std::to_string(std::max(m->d.rc_rad, m->d.rc_ang)) + " A for its descriptors");
    const size_t rows = static_cast<size_t>(std::max(L.d.rows, 1));
    M.d.alloc(1);
    M.net.alloc(1);
    M.G.alloc(rows * learned::NG);
    M.g.alloc(rows * learned::NG);
    M.e.alloc(rows);
    M.t.alloc(rows);
    M.leg.alloc(static_cast<size_t>(std::max(L.d.nmax, 1)) * static_cast<size_t>(std::max(L.d.stride, 1)));
    M.cforce.alloc(rows);
    M.d.upload(&M.model.d, 1, st);
    M.net.upload(&M.model.n, 1, st);
    if (!L.row_of.p) {  // the force gather reads a partner's row
      std::vector<int> ro(static_cast<size_t>(N), -1);
      const auto& rg = groups[static_cast<size_t>(L.d.row_group)].idx;
      for (size_t q = 0; q < rg.size(); ++q) ro[static_cast<size_t>(rg[q])] = static_cast<int>(q);
      L.row_of.alloc(ro.size());
      L.row_of.upload(ro.data(), ro.size(), st);
      L.d.row_of = L.row_of.p;
    }
    ++used;
  }
  if (!used) throw Error(PFMD_E_PARAM, "learned form: no tb or rjl interaction matches the model file");
  if (!fsave.p) {
    fsave.alloc(static_cast<size_t>(std::max(N, 1)));
    fdiff.alloc(2 * 256 + 2);
  }
  clear_graphs();
  CK(cudaStreamSynchronize(st));
}

// Learned and classical forces at the current positions: RMSE over all atoms
// (eV/A).  With switch_on_fail the learned form stays on below max_rmse and falls
// back to the classical kernels (keeping their forces) above it.
// A run that has not taken its first step has no lists yet: build them.
void Engine::ensure_lists() {
  if (md_step != 0) return;
  StepPlan p;
  p.step = 0;
  p.first = true;
  p.energy = true;
  p.out = p.zero_mom = p.check_all = false;
  p.rebuild.assign(lists.size(), 1);
  enqueue_lists(p);
}

double Engine::learned_check(bool switch_on_fail) {
  ctl_fresh = false;  // launches the classical kernels
  const bool was = learned_active;
  ensure_lists();
  const GroupRef gall = gref(S.all_atoms);
  learned_active = true;
  if (!store_first) launch_zero_forces(gall, A, ctl, st);
  enqueue_forces(false, false);
  CK(cudaMemcpyAsync(fsave.p, frc.p, sizeof(double4_32a) * static_cast<size_t>(N), cudaMemcpyDeviceToDevice, st));
  learned_active = false;
  if (!store_first) launch_zero_forces(gall, A, ctl, st);
  enqueue_forces(false, false);
  learned::launch_force_diff(N, fsave.p, frc.p, fdiff.p, fdiff.p + 512, st);
  double out[2] = {0.0, 0.0};
  CK(cudaMemcpyAsync(out, fdiff.p + 512, sizeof(out), cudaMemcpyDeviceToHost, st));
  read_ctl();
  if (hctl->error) raise_device_error();
  const double rmse = std::sqrt(out[0] / (3.0 * std::max(N, 1)));
  ++checks;
  last_rmse = rmse;
  bool keep = was;
  if (switch_on_fail && was && rmse > max_rmse) {
    keep = false;
    fallen_back = true;
    clear_graphs();
  }
  learned_active = keep;
  if (keep)
    CK(cudaMemcpyAsync(frc.p, fsave.p, sizeof(double4_32a) * static_cast<size_t>(N), cudaMemcpyDeviceToDevice, st));
  CK(cudaStreamSynchronize(st));
  return rmse;
}

// Online training from this (plain-form) run: every `stride` steps the plain tb and
// rjl kernels give per-atom energies of the current configuration; each network
// takes `iters` Adam steps on its atoms' descriptors.  rmse_out[k] (per
// interaction, NaN where no network) = per-atom energy RMSE of the last frame.
// grad_out: the gradient mode -- one frame, the loss gradient of each network into
// grad_out (NET_FLOATS each) and its summed squared energy error into loss_out,
// no update and nothing saved.
void Engine::learned_train(const std::string& model_in, const std::string& model_out, int frames, int stride,
                           int iters, int flags, float* grad_out, double* loss_out, double* grad_ms, double lr,
                           double force_weight, double* rmse_out, double* force_rmse) {
  const bool tc = (flags & PFMD_LEARNED_TENSOR_CORES) != 0;
  if (grad_out) {
    frames = 1;
    stride = 0;
    iters = 1;
  }
  if (prec) throw Error(PFMD_E_STATE, "learned training runs on the plain form (FP64 targets)");
  std::vector<learned::Model> ms;
  const bool fresh = model_in.empty();
  if (fresh) {
    for (const auto& I : inters) {
      if (I.spec.kind == pfmd_io::K_TB) ms.push_back(learned::default_model(0, static_cast<unsigned>(opt.rand_seed)));
      if (I.spec.kind == pfmd_io::K_RJL) {
        // the rjl repulsion is the model's baseline; the network learns the rest
        learned::Model m = learned::default_model(1, static_cast<unsigned>(opt.rand_seed));
        m.d.bA = static_cast<float>(I.rjl.A0);
        m.d.bp = static_cast<float>(I.rjl.p);
        m.d.br0 = static_cast<float>(I.rjl.r0);
        m.d.bR1 = static_cast<float>(I.rjl.R1);
        m.d.bR2 = static_cast<float>(I.rjl.R2);
        ms.push_back(m);
      }
    }
  } else {
    ms = learned::load_models(model_in);
  }
  iters = std::max(1, iters);
  learned_setup(ms);
  learned_active = false;
  if (!eatom.p) eatom.alloc(static_cast<size_t>(std::max(N, 1)));
  for (auto& M : lrn) {
    if (!M.on) continue;
    const int rows = static_cast<int>(M.e.n);
    const int blocks = std::max(learned::train_blocks(rows), learned::train_tc_grid(rows));
    M.part.alloc(static_cast<size_t>(blocks) * learned::NET_FLOATS);
    M.lpart.alloc(static_cast<size_t>(blocks));
    M.grad.alloc(learned::NET_FLOATS);
    M.m.alloc(learned::NET_FLOATS);
    M.v.alloc(learned::NET_FLOATS);
    M.m.zero(st);
    M.v.zero(st);
    M.loss.alloc(2);
    M.adam_step = 0;
  }
  const bool fm = force_weight > 0.0;  // force matching
  std::vector<DBuf<float>> U(lrn.size());
  if (fm) {
    fref.alloc(static_cast<size_t>(std::max(N, 1)));
    fres.alloc(static_cast<size_t>(std::max(N, 1)));
    for (size_t k = 0; k < lrn.size(); ++k)
      if (lrn[k].on) U[k].alloc(lrn[k].G.n);
  }
  const GroupRef gall = gref(S.all_atoms);
  // learned forces at this configuration into frc, residuals against fref, and
  // the force-matching directions of every network
  auto learned_residuals = [&]() {
    learned_active = true;
    if (!store_first) launch_zero_forces(gall, A, ctl, st);
    enqueue_forces(false, false);
    learned_active = false;
    learned::launch_residual(N, frc.p, fref.p, fres.p, st);
    for (size_t k = 0; k < lrn.size(); ++k)
      if (lrn[k].on)
        learned::launch_desc_vjp(lists[static_cast<size_t>(inters[k].lists[0])].d, lrn[k].d.p, A, box, fres.p,
                                 U[k].p, ctl, st);
  };
  for (int f = 0; f < frames; ++f) {
    if (stride > 0) {
      int fin = 0;
      advance(stride, &fin);
      if (finished) break;
    }
    // per-atom energies of the classical interactions at this configuration
    ensure_lists();
    eatom_out = eatom.p;
    if (!store_first) launch_zero_forces(gall, A, ctl, st);
    enqueue_forces(true, false);
    eatom_out = nullptr;
    if (fm)
      CK(cudaMemcpyAsync(fref.p, frc.p, sizeof(double4_32a) * static_cast<size_t>(N), cudaMemcpyDeviceToDevice, st));
    for (size_t k = 0; k < lrn.size(); ++k) {
      Lrn& M = lrn[k];
      if (!M.on) continue;
      const ListH& L = lists[static_cast<size_t>(inters[k].lists[0])];
      const int rows = L.d.rows;
      learned::launch_gather_rows(L.d, eatom.p, M.t.p, st);
      learned::launch_core_sub(L.d, M.d.p, A, box, learned::core_radius(M.model.kind), M.t.p, st);
      if (fresh && f == 0) {
        // descriptor normalisation and the energy offset from the first frame
        for (int q = 0; q < learned::NG; ++q) {
          M.model.d.mean[q] = 0.f;
          M.model.d.inv_std[q] = 1.f;
        }
        M.d.upload(&M.model.d, 1, st);
        learned::launch_desc(L.d, M.d.p, A, box, M.G.p, ctl, st);
        std::vector<float> G(static_cast<size_t>(rows) * learned::NG);
        std::vector<double> t(static_cast<size_t>(rows));
        CK(cudaMemcpyAsync(G.data(), M.G.p, sizeof(float) * G.size(), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(t.data(), M.t.p, sizeof(double) * t.size(), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int q = 0; q < learned::NG; ++q) {
          double s = 0.0, s2 = 0.0;
          for (int r = 0; r < rows; ++r) {
            const double x = G[static_cast<size_t>(r) * learned::NG + q];
            s += x;
            s2 += x * x;
          }
          const double mu = s / std::max(rows, 1), var = std::max(s2 / std::max(rows, 1) - mu * mu, 0.0);
          M.model.d.mean[q] = static_cast<float>(mu);
          // a floor on the spread: a function that is (nearly) constant on the first
          // frame must not amplify later fluctuations
          M.model.d.inv_std[q] = static_cast<float>(1.0 / std::max(std::sqrt(var), 0.05));
        }
        double tm = 0.0;
        for (double x : t) tm += x;
        M.model.n.b3 = static_cast<float>(tm / std::max(rows, 1));
        M.d.upload(&M.model.d, 1, st);
        M.net.upload(&M.model.n, 1, st);
      }
    }
    for (int it = 0; it < iters; ++it) {
      if (fm) learned_residuals();  // also refreshes every network's descriptors
      for (size_t k = 0; k < lrn.size(); ++k) {
        Lrn& M = lrn[k];
        if (!M.on) continue;
        const ListH& L = lists[static_cast<size_t>(inters[k].lists[0])];
        const int rows = L.d.rows;
        if (!fm && it == 0) learned::launch_desc(L.d, M.d.p, A, box, M.G.p, ctl, st);
        learned::TrainBuf T;
        T.part = M.part.p;
        T.lpart = M.lpart.p;
        T.part_blocks = learned::train_blocks(rows);
        T.grad = M.grad.p;
        T.m = M.m.p;
        T.v = M.v.p;
        T.loss = M.loss.p;
        if (grad_out && grad_ms) {
          if (!ev0) {
            CK(cudaEventCreate(&ev0));
            CK(cudaEventCreate(&ev1));
          }
          CK(cudaEventRecord(ev0, st));
        }
        if (tc)
          learned::launch_train_grad_tc(rows, M.G.p, fm ? U[k].p : nullptr, M.t.p, 1.0f,
                                        static_cast<float>(force_weight), M.net.p, T, ctl, st);
        else
          learned::launch_train_grad(rows, M.G.p, fm ? U[k].p : nullptr, M.t.p, 1.0f,
                                     static_cast<float>(force_weight), M.net.p, T, st);
        if (grad_out && grad_ms) {
          CK(cudaEventRecord(ev1, st));
          CK(cudaEventSynchronize(ev1));
          float ms = 0.f;
          CK(cudaEventElapsedTime(&ms, ev0, ev1));
          *grad_ms += ms;
        }
        if (grad_out) {
          int slot = 0;
          for (size_t q = 0; q < k; ++q) slot += lrn[q].on ? 1 : 0;
          CK(cudaMemcpyAsync(grad_out + static_cast<size_t>(slot) * learned::NET_FLOATS, M.grad.p,
                             sizeof(float) * learned::NET_FLOATS, cudaMemcpyDeviceToHost, st));
          if (loss_out) CK(cudaMemcpyAsync(loss_out + slot, M.loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
          continue;
        }
        ++M.adam_step;
        learned::launch_adam(M.net.p, T, M.adam_step, static_cast<float>(lr), st);
      }
    }
    // the dynamics goes on with the classical forces of this configuration
    if (fm)
      CK(cudaMemcpyAsync(frc.p, fref.p, sizeof(double4_32a) * static_cast<size_t>(N), cudaMemcpyDeviceToDevice, st));
    read_ctl();
    if (hctl->error) raise_device_error();
  }
  if (grad_out) {
    CK(cudaStreamSynchronize(st));
    read_ctl();
    if (hctl->error) raise_device_error();
    clear_graphs();
    return;
  }
  // the error of the final networks on the last frame
  for (size_t k = 0; k < inters.size(); ++k) {
    if (rmse_out) rmse_out[k] = std::nan("");
    if (k >= lrn.size() || !lrn[k].on) continue;
    Lrn& M = lrn[k];
    const ListH& L = lists[static_cast<size_t>(inters[k].lists[0])];
    learned::TrainBuf T;
    T.part = M.part.p;
    T.lpart = M.lpart.p;
    T.part_blocks = learned::train_blocks(L.d.rows);
    T.grad = M.grad.p;
    T.loss = M.loss.p;
    learned::launch_desc(L.d, M.d.p, A, box, M.G.p, ctl, st);
    learned::launch_train_grad(L.d.rows, M.G.p, nullptr, M.t.p, 1.0f, 0.0f, M.net.p, T, st);
    double loss[2] = {0.0, 0.0};
    CK(cudaMemcpyAsync(loss, M.loss.p, sizeof(loss), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&M.model.n, M.net.p, sizeof(learned::Net), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (rmse_out) rmse_out[k] = std::sqrt(loss[0] / std::max(loss[1], 1.0));
  }
  if (force_rmse) {
    // learned against classical forces on the last configuration (all atoms)
    const double r = learned_check(false);
    *force_rmse = r;
  }
  std::vector<learned::Model> out;
  for (auto& M : lrn)
    if (M.on) out.push_back(M.model);
  if (!model_out.empty()) learned::save_models(model_out, out);
  clear_graphs();
}

void Engine::compute(bool rebuild, double* e_inter) {
  StepPlan p;
  p.step = 0;
  p.first = true;
  p.energy = true;
  p.out = false;
  p.zero_mom = false;
  p.check_all = false;
  p.rebuild.assign(lists.size(), rebuild ? 1 : 0);
  enqueue_lists(p);
  launch_zero_forces(gref(S.all_atoms), A, ctl, st);
  enqueue_forces(true);
  read_ctl();
  if (hctl->error) raise_device_error();
  if (e_inter)
    for (size_t k = 0; k < inters.size(); ++k) e_inter[k] = hctl->e_inter[k];
}

static long long host_nnz(const ListH& L, cudaStream_t st) {
  std::vector<int> n(static_cast<size_t>(L.d.rows));
  if (!n.empty()) CK(cudaMemcpyAsync(n.data(), L.nnum.p, sizeof(int) * n.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  long long t = 0;
  for (int v : n) t += v;
  return t;
}

// Algorithmic HBM bytes of one launch: list entries (4 B each), per-row list data
// (nnum, pidx: 8 B), the row atom's position (32 B plain, 16 B fixed-point), its
// force update (read + write of a double4: 64 B) and kernel-specific per-row
// arrays.  Neighbour positions and neighbour per-row data are counted as cache
// resident (they are re-read by many rows).
double Engine::kernel_bytes(const std::string& name) {
  const double P = prec ? 16.0 : 32.0, F = 64.0, IE = prec ? 4.0 : 8.0;
  auto row_bytes = [&](const ListH& L, double extra_row, double extra_entry) {
    const double R = L.d.rows, nnz = static_cast<double>(host_nnz(L, st));
    return 8.0 * R + 4.0 * nnz + P * R + extra_row * R + extra_entry * nnz;
  };
  double b = 0.0;
  for (auto& I : inters) {
    const ListH& L1 = lists[static_cast<size_t>(I.lists[0])];
    const int k = I.spec.kind;
    if (k == pfmd_io::K_LJ && (name == "lj" || name == "forces")) {
      b += row_bytes(L1, F, 0) + row_bytes(lists[static_cast<size_t>(I.lists[1])], F, 0);
      if (name == "lj") return b;
    }
    if (k == pfmd_io::K_LJ1G && (name == "lj1g" || name == "forces")) {
      b += row_bytes(L1, F + 4.0, 0);
      if (name == "lj1g") return b;
    }
    if (k == pfmd_io::K_RJL) {
      // the density pass writes two pair coefficients per entry (FP64 plain, FP32
      // precision) and the force pass reads them back
      const double PC = prec ? 8.0 : 16.0;
      if (name == "rjl_density") return row_bytes(L1, IE, PC);
      // with the next step's kick and drift fused in: k_kick_drift's 160 B per moving atom
      if (name == "rjl_force")
        return row_bytes(L1, IE + F, PC) +
               (fuse_drift ? 160.0 * static_cast<double>(groups[static_cast<size_t>(S.xyz_moving - 1)].idx.size())
                           : 0.0);
      if (name == "forces") b += row_bytes(L1, IE, PC) + row_bytes(L1, IE + F, PC);
    }
    if (k == pfmd_io::K_REBOSC) {
      if (name == "rebo_bond") return row_bytes(L1, 0, 24.0);
      if (name == "rebo_force") return row_bytes(L1, F, 24.0);
      if (name == "forces") b += row_bytes(L1, 0, 24.0) + row_bytes(L1, F, 24.0);
    }
    if (k == pfmd_io::K_TB) {
      if (name == "tb_bond") return row_bytes(L1, 0, 8.0);
      if (name == "tb_force") return row_bytes(L1, F, 8.0);
      if (name == "forces") b += row_bytes(L1, 0, 8.0) + row_bytes(L1, F, 8.0);
    }
    if (k == pfmd_io::K_LJC || k == pfmd_io::K_MORSEC) {
      const ListH& L2 = lists[static_cast<size_t>(I.lists[1])];
      if (name == "cos_graphene") return row_bytes(L1, F + 32.0, 0);
      if (name == "cos_metal") return row_bytes(L2, F, 0);
      if (name == "forces") b += row_bytes(L1, F + 32.0, 0) + row_bytes(L2, F, 0);
    }
  }
  if (name == "forces") {
    b += 32.0 * static_cast<double>(groups[static_cast<size_t>(S.all_atoms - 1)].idx.size());  // zero_forces
    return b;
  }
  if (name == "kick_drift")  // force, velocity, position, kc read; velocity, position, posq written
    return 160.0 * static_cast<double>(groups[static_cast<size_t>(S.xyz_moving - 1)].idx.size());
  if (name == "lists") {
    for (auto& L : lists) {
      if (L.kind == L_NN_TB) continue;
      const double C = L.d.col_cap, R = L.d.rows, nnz = static_cast<double>(host_nnz(L, st));
      // binning: posq + cell id + count + scatter; build: posq, list entries, row data
      b += 28.0 * C + P * R + 4.0 * nnz + 16.0 * R;
    }
    return b;
  }
  return b;
}

// Launches `reps` times one kernel group between two events on st.
double Engine::time_kernel(const std::string& name, int reps, double* bytes) {
  if (reps < 1) reps = 1;
  if (!ev0) {
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
  }
  auto once = [&]() -> bool {
    if (name == "forces") {
      launch_zero_forces(gref(S.all_atoms), A, ctl, st);
      enqueue_forces(false);
      return true;
    }
    if (name == "kick_drift") {
      // zero time steps: the same loads, FP64 work and stores, the state unchanged
      launch_kick_drift(gref(S.xyz_moving), 0.0, 0.0, true, 0, !prec, A, box, ctl, st, false);
      return true;
    }
    if (name == "lists") {
      // every list rebuilt, skin-triggered or not
      CK(cudaMemsetAsync(ctl->list_need, 1, sizeof(ctl->list_need), st));
      StepPlan p;
      p.step = 0;
      p.first = true;
      p.energy = p.out = p.zero_mom = p.check_all = false;
      p.rebuild.assign(lists.size(), 1);
      enqueue_lists(p);
      return true;
    }
    for (size_t k = 0; k < inters.size(); ++k) {
      InterH& I = inters[k];
      const ListDev& L1 = lists[static_cast<size_t>(I.lists[0])].d;
      const int kind = I.spec.kind;
      const int eslot = 4;
      if (kind == pfmd_io::K_LJ && name == "lj") {
        launch_lj(prec, false, L1, I.lj, A, box, ctl, eslot, 0, st);
        launch_lj(prec, false, lists[static_cast<size_t>(I.lists[1])].d, I.lj, A, box, ctl, eslot, 0, st);
        return true;
      }
      if (kind == pfmd_io::K_LJ1G && name == "lj1g") {
        launch_lj1g(prec, false, I.general, L1, I.lj, A, box, ctl, eslot, 0, st);
        return true;
      }
      if (kind == pfmd_io::K_RJL && (name == "rjl_density" || name == "rjl_force")) {
        // the force pass as the step runs it: with the kick and, when steps fuse, the
        // next step's kick and drift -- here with zero time steps, so the state keeps
        // its values
        Epi e{0, 0, prec ? 0 : 1, 0.0, mflag.p, nullptr};
        if (name == "rjl_force" && kick_last && mflag.p) {
          e.kick = 1;
          if (fuse_drift) {
            e.drift = 1;
            e.ts1 = 0.0;
            e.posq_next = posq_cur ? posq.p : posq2.p;
          }
        }
        launch_rjl(prec, false, L1, I.rjl, A, box, I.scratch.p, I.pair.p, ctl, eslot, 0, st,
                   name == "rjl_density" ? 1 : 2, e);
        return true;
      }
      if (kind == pfmd_io::K_REBOSC && (name == "rebo_bond" || name == "rebo_force")) {
        launch_rebo(false, L1, I.rebo, A, box, I.scratch.p, ctl, eslot, 0, st, name == "rebo_bond" ? 1 : 2);
        return true;
      }
      if (kind == pfmd_io::K_TB && (name == "tb_bond" || name == "tb_force")) {
        launch_tb(prec, false, L1, I.tb, A, box, I.scratch.p, ctl, eslot, 0, st, name == "tb_bond" ? 1 : 2);
        return true;
      }
      if ((kind == pfmd_io::K_LJC || kind == pfmd_io::K_MORSEC) && (name == "cos_graphene" || name == "cos_metal")) {
        launch_cos(prec, false, kind == pfmd_io::K_MORSEC, L1, lists[static_cast<size_t>(I.lists[1])].d,
                   lists[static_cast<size_t>(I.lists[2])].d, I.cp, I.norm.p, I.gsum.p, A, box, ctl, eslot, 0, st,
                   name == "cos_graphene" ? 1 : 2);
        return true;
      }
    }
    return false;
  };
  if (!once()) throw Error(PFMD_E_PARAM, "no kernel named '" + name + "' in this system");
  CK(cudaStreamSynchronize(st));
  CK(cudaEventRecord(ev0, st));
  for (int r = 0; r < reps; ++r) once();
  CK(cudaEventRecord(ev1, st));
  CK(cudaEventSynchronize(ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ev0, ev1));
  // restore the forces of the current positions
  launch_zero_forces(gref(S.all_atoms), A, ctl, st);
  enqueue_forces(false);
  read_ctl();
  if (hctl->error) raise_device_error();
  if (bytes) *bytes = kernel_bytes(name);
  return static_cast<double>(ms) / reps;
}

}  // namespace pfmd

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct pfmd_ctx {
  std::unique_ptr<pfmd::Engine> e;
  std::string err;
};

template <class F>
static int guard_keep(pfmd_ctx* c, F f);

template <class F>
static int guard(pfmd_ctx* c, F f) {
  if (c && c->e) c->e->ctl_fresh = false;  // the call may launch work
  return guard_keep(c, f);
}

// For calls that launch nothing that writes the control block.
template <class F>
static int guard_keep(pfmd_ctx* c, F f) {
  try {
    f();
    return PFMD_OK;
  } catch (const pfmd::Error& e) {
    if (c) c->err = e.what();
    return e.code;
  } catch (const fortio::ReadError& e) {
    if (c) c->err = e.what();
    return PFMD_E_IO;
  } catch (const std::exception& e) {
    if (c) c->err = e.what();
    return PFMD_E_PARAM;
  }
}

extern "C" {

void pfmd_default_options(pfmd_options* o) {
  if (!o) return;
  o->form = PFMD_FORM_PLAIN;
  o->rand_seed = 1;
  o->out_period = 1;
  o->out_fd = -1;
  o->all_out_fd = -1;
  o->write_files = 0;
  o->output_prefix = "";
  o->num_threads = 1;
  o->device = 0;
  o->use_graphs = 1;
  o->threads_per_row = 0;
  o->async_io = 1;
  o->skin_lists = 1;
  o->fuse_steps = 1;
}

int pfmd_create_from_files(const char* input_path, const char* settings_filename, const pfmd_options* opt,
                           pfmd_ctx** out) {
  if (!out) return PFMD_E_PARAM;
  auto* c = new pfmd_ctx();
  c->e.reset(new pfmd::Engine());
  *out = c;
  pfmd_options o;
  pfmd_default_options(&o);
  if (opt) o = *opt;
  if (o.out_period < 1) o.out_period = 1;
  int rc = guard(c, [&] {
    c->e->create(input_path ? input_path : "", settings_filename ? settings_filename : "md_run_settings.txt", o);
  });
  c->e->flush_out();
  return rc;
}

void pfmd_destroy(pfmd_ctx* c) { delete c; }
const char* pfmd_errmsg(const pfmd_ctx* c) { return c ? c->err.c_str() : "null context"; }
const char* pfmd_strerror(int code) {
  switch (code) {
    case PFMD_OK: return "PFMD_OK";
    case PFMD_E_NLIST_OVERFLOW: return "PFMD_E_NLIST_OVERFLOW";
    case PFMD_E_OUT_OF_CELL: return "PFMD_E_OUT_OF_CELL";
    case PFMD_E_GR_NN: return "PFMD_E_GR_NN";
    case PFMD_E_PARAM: return "PFMD_E_PARAM";
    case PFMD_E_CUDA: return "PFMD_E_CUDA";
    case PFMD_E_TIMEOUT: return "PFMD_E_TIMEOUT";
    case PFMD_E_IO: return "PFMD_E_IO";
    case PFMD_E_STATE: return "PFMD_E_STATE";
  }
  return "PFMD_E_UNKNOWN";
}

int pfmd_advance(pfmd_ctx* c, long long max_steps, int* finished) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] { c->e->advance(max_steps, finished); });
}

int pfmd_finish(pfmd_ctx* c) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] { c->e->finish(); });
}

int pfmd_md(const char* input_path, const char* settings_filename, const pfmd_options* opt) {
  pfmd_ctx* c = nullptr;
  int rc = pfmd_create_from_files(input_path, settings_filename, opt, &c);
  if (rc == PFMD_OK) {
    int fin = 0;
    rc = pfmd_advance(c, LLONG_MAX, &fin);
    if (rc == PFMD_OK) rc = pfmd_finish(c);
  }
  if (rc != PFMD_OK && c && c->e && !c->e->printed) {
    c->e->outln(" " + c->err);
    c->e->flush_out();
  }
  pfmd_destroy(c);
  return rc;
}

int pfmd_natoms(const pfmd_ctx* c, int* n) {
  if (!c || !c->e || !n) return PFMD_E_STATE;
  *n = c->e->N;
  return PFMD_OK;
}

int pfmd_md_step(const pfmd_ctx* c, long long* s, double* t) {
  if (!c || !c->e) return PFMD_E_STATE;
  if (s) *s = c->e->md_step;
  if (t) *t = c->e->sim_time;
  return PFMD_OK;
}

int pfmd_get_state(pfmd_ctx* c, double* pos, double* vel, double* frc) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard_keep(c, [&] { c->e->get_state_to(pos, vel, frc); });
}

int pfmd_set_state(pfmd_ctx* c, const double* pos, const double* vel) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] {
    pfmd::Engine& e = *c->e;
    const int N = e.N;
    const size_t n3 = 3 * static_cast<size_t>(N);
    // read in place when page-locked, else copied as given; converted on the device
    const double* in[3] = {nullptr, nullptr, nullptr};
    const double* h[2] = {pos, vel};
    for (int k = 0; k < 2 && N; ++k) {
      if (!h[k]) continue;
      in[k] = pfmd::host_view(h[k], n3);
      if (!in[k]) {
        if (!e.stage.p) e.stage.alloc(3 * n3);
        CK(cudaMemcpyAsync(e.stage.p + k * n3, h[k], sizeof(double) * n3, cudaMemcpyHostToDevice, e.st));
        in[k] = e.stage.p + k * n3;
      }
    }
    pfmd::launch_state_in(N, in[0], in[1], e.A, e.box, e.st);
    if (pos && N) e.need_check_all = true;  // also rebuilds the lists (skin-triggered ones if needed) at the next step
    CK(cudaStreamSynchronize(e.st));
  });
}

int pfmd_energies(pfmd_ctx* c, double* e_inter, double* pe, double* ke, double* temp, double* e_nhc,
                  double* e_cons) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard_keep(c, [&] {
    pfmd::Engine& e = *c->e;
    if (!e.ctl_fresh) e.read_ctl();
    if (e_inter)
      for (size_t k = 0; k < e.inters.size(); ++k) e_inter[k] = e.hctl->e_inter[k];
    if (pe) *pe = e.hctl->pe_last;
    if (ke) *ke = e.hctl->ke;
    if (temp) *temp = e.hctl->temperature;
    if (e_nhc) *e_nhc = e.hctl->e_nhc;
    if (e_cons) *e_cons = e.hctl->conserved;
  });
}

int pfmd_compute(pfmd_ctx* c, int rebuild, double* e_inter) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] { c->e->compute(rebuild != 0, e_inter); });
}

int pfmd_ninteractions(const pfmd_ctx* c, int* n) {
  if (!c || !c->e || !n) return PFMD_E_STATE;
  *n = static_cast<int>(c->e->inters.size());
  return PFMD_OK;
}

static int list_of(const pfmd_ctx* c, int inter, int list) {
  const auto& e = *c->e;
  if (inter < 0 || inter >= static_cast<int>(e.inters.size())) return -1;
  if (list < 0 || list >= 3) return -1;
  return e.inters[static_cast<size_t>(inter)].lists[list];
}

int pfmd_nlist_shape(const pfmd_ctx* c, int inter, int list, int* n_rows, int* nmax) {
  if (!c || !c->e) return PFMD_E_STATE;
  int l = list_of(c, inter, list);
  if (l < 0) return PFMD_E_PARAM;
  const auto& L = c->e->lists[static_cast<size_t>(l)];
  if (n_rows) *n_rows = L.d.rows;
  if (nmax) *nmax = L.d.nmax;
  return PFMD_OK;
}

int pfmd_get_nlist(pfmd_ctx* c, int inter, int list, int* nnum, int* lessnnum, int* pidx, int* nlist) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  int l = list_of(c, inter, list);
  if (l < 0) return PFMD_E_PARAM;
  return guard(c, [&] {
    auto& e = *c->e;
    const auto& L = e.lists[static_cast<size_t>(l)];
    const size_t rows = static_cast<size_t>(L.d.rows), nmax = static_cast<size_t>(L.d.nmax),
                 stride = static_cast<size_t>(L.d.stride);
    if (rows == 0) return;
    if (nnum) CK(cudaMemcpyAsync(nnum, L.nnum.p, sizeof(int) * rows, cudaMemcpyDeviceToHost, e.st));
    if (lessnnum) CK(cudaMemcpyAsync(lessnnum, L.less.p, sizeof(int) * rows, cudaMemcpyDeviceToHost, e.st));
    if (pidx) CK(cudaMemcpyAsync(pidx, L.pidx.p, sizeof(int) * rows, cudaMemcpyDeviceToHost, e.st));
    // unsorted (cell-order) rows of a regular list: lessnnum is formed here as the
    // reference defines it, the position (in ascending group-2 order) of the
    // first partner with a larger atom index (md_neighbours.f90:78)
    const bool count_less = lessnnum && !L.d.sorted && L.kind == pfmd::L_REGULAR && nmax;
    std::vector<int> t, hn, hp;
    if ((nlist || count_less) && nmax) {
      t.resize(nmax * stride);
      CK(cudaMemcpyAsync(t.data(), L.nlist.p, sizeof(int) * t.size(), cudaMemcpyDeviceToHost, e.st));
    }
    if (count_less) {
      hn.resize(rows);
      hp.resize(rows);
      CK(cudaMemcpyAsync(hn.data(), L.nnum.p, sizeof(int) * rows, cudaMemcpyDeviceToHost, e.st));
      CK(cudaMemcpyAsync(hp.data(), L.pidx.p, sizeof(int) * rows, cudaMemcpyDeviceToHost, e.st));
    }
    CK(cudaStreamSynchronize(e.st));
    if (count_less) {
      std::vector<std::pair<int, int>> row;  // (group-2 index, atom)
      for (size_t r = 0; r < rows; ++r) {
        const size_t n = std::min(static_cast<size_t>(std::max(hn[r], 0)), nmax);
        row.clear();
        for (size_t p = 0; p < n; ++p) {
          const int v = t[p * stride + r];
          row.emplace_back(v >= 0 && v < e.N ? L.col_inv[static_cast<size_t>(v)] : v, v);
        }
        std::sort(row.begin(), row.end());
        int k = static_cast<int>(n);
        for (size_t p = 0; p < n; ++p)
          if (hp[r] < row[p].second) {
            k = static_cast<int>(p);
            break;
          }
        lessnnum[r] = k;
      }
    }
    // main lists hold partner atoms: report the reference's group-2 indexes
    const bool atoms = L.kind != pfmd::L_NN_TB;
    if (nlist && nmax)
      for (size_t r = 0; r < rows; ++r)
        for (size_t p = 0; p < nmax; ++p) {
          const int v = t[p * stride + r];
          nlist[r * nmax + p] = (atoms && v >= 0 && v < e.N) ? L.col_inv[static_cast<size_t>(v)] : v;
        }
  });
}

int pfmd_nlist_load(pfmd_ctx* c, int* maxnnum, int* count) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] {
    auto& e = *c->e;
    CK(cudaMemsetAsync(e.ctl->maxnnum, 0, sizeof(int) * PFMD_MAX_LISTS, e.st));
    for (auto& L : e.lists) pfmd::launch_nnum_max(L.d, e.ctl, e.st);
    e.read_ctl();
    int k = 0;
    for (auto& I : e.inters)
      for (int j = 0; j < I.spec.nl_n; ++j) {
        const auto& L = e.lists[static_cast<size_t>(I.lists[j])];
        if (maxnnum) maxnnum[k] = e.hctl->maxnnum[L.d.id];
        ++k;
      }
    if (count) *count = k;
  });
}

int pfmd_nlist_builds(pfmd_ctx* c, long long* builds, int* count) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] {
    auto& e = *c->e;
    e.read_ctl();
    int k = 0;
    for (auto& I : e.inters)
      for (int j = 0; j < I.spec.nl_n; ++j) {
        const auto& L = e.lists[static_cast<size_t>(I.lists[j])];
        // a converse list follows its source's rebuilds
        if (builds) builds[k] = (L.d.skin >= 0) ? e.hctl->list_builds[L.d.skin] : -1;
        ++k;
      }
    if (count) *count = k;
  });
}

int pfmd_get_gr_norm(pfmd_ctx* c, int inter, double* norm) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  auto& e = *c->e;
  if (inter < 0 || inter >= static_cast<int>(e.inters.size())) return PFMD_E_PARAM;
  auto& I = e.inters[static_cast<size_t>(inter)];
  if (!I.norm.p) return PFMD_E_PARAM;
  return guard(c, [&] {
    // normals are kept per atom; gr_norm is indexed by the nn list's rows
    const auto& L3 = e.lists[static_cast<size_t>(I.lists[2])];
    const size_t rows = static_cast<size_t>(L3.d.rows);
    const auto& rg = e.groups[static_cast<size_t>(L3.d.row_group)].idx;
    std::vector<double4_32a> t(static_cast<size_t>(std::max(e.N, 1)));
    if (e.N) CK(cudaMemcpyAsync(t.data(), I.norm.p, sizeof(double4_32a) * e.N, cudaMemcpyDeviceToHost, e.st));
    CK(cudaStreamSynchronize(e.st));
    for (size_t r = 0; r < rows; ++r) {
      const double nan = std::nan("");
      const bool has = r < rg.size();
      norm[3 * r] = has ? t[static_cast<size_t>(rg[r])].x : nan;
      norm[3 * r + 1] = has ? t[static_cast<size_t>(rg[r])].y : nan;
      norm[3 * r + 2] = has ? t[static_cast<size_t>(rg[r])].z : nan;
    }
  });
}

int pfmd_set_group_n(pfmd_ctx* c, int group, int n) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  auto& e = *c->e;
  if (group < 1 || group > static_cast<int>(e.groups.size())) return PFMD_E_PARAM;
  return guard(c, [&] {
    e.read_ctl();
    const int cap = static_cast<int>(e.groups[static_cast<size_t>(group - 1)].idx.size());
    e.hctl->group_n[group - 1] = std::max(0, std::min(n, cap));
    e.upload_ctl_groups();
    e.refresh_mflag();
    // rows change with the group: skin-triggered lists (and outer lists) rebuild at
    // their next update step
    CK(cudaMemsetAsync(e.ctl->list_need, 1, sizeof(e.ctl->list_need), e.st));
    CK(cudaMemsetAsync(e.ctl->outer_need, 1, sizeof(e.ctl->outer_need), e.st));
    CK(cudaStreamSynchronize(e.st));
  });
}

int pfmd_get_stream(pfmd_ctx* c, void** stream) {
  if (!c || !c->e || !stream) return PFMD_E_STATE;
  *stream = c->e->st;
  return PFMD_OK;
}

int pfmd_advance_timed(pfmd_ctx* c, long long max_steps, int* finished, double* device_ms) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] {
    pfmd::Engine& e = *c->e;
    if (!e.ev0) {
      CK(cudaEventCreate(&e.ev0));
      CK(cudaEventCreate(&e.ev1));
    }
    e.timing = true;
    e.timing_started = false;
    try {
      e.advance(max_steps, finished);
    } catch (...) {
      e.timing = false;
      throw;
    }
    e.timing = false;
    float ms = 0.f;
    if (e.timing_started) {
      CK(cudaEventSynchronize(e.ev1));
      CK(cudaEventElapsedTime(&ms, e.ev0, e.ev1));
    }
    if (device_ms) *device_ms = ms;
  });
}

int pfmd_time_kernel(pfmd_ctx* c, const char* name, int reps, double* ms, double* bytes) {
  if (!c || !c->e || !c->e->ctl || !name) return PFMD_E_STATE;
  return guard(c, [&] {
    double t = c->e->time_kernel(name, reps, bytes);
    if (ms) *ms = t;
  });
}

int pfmd_flush_l2(pfmd_ctx* c, long long bytes) {
  if (!c || !c->e || !c->e->ctl || bytes <= 0) return PFMD_E_STATE;
  return guard(c, [&] {
    pfmd::Engine& e = *c->e;
    if (e.flush_buf.n < static_cast<size_t>(bytes)) e.flush_buf.alloc(static_cast<size_t>(bytes));
    CK(cudaMemsetAsync(e.flush_buf.p, (++e.flush_seq) & 0xff, static_cast<size_t>(bytes), e.st));
  });
}

int pfmd_learned_train(pfmd_ctx* c, const char* model_in, const char* model_out, int frames, int stride, int iters,
                       double lr, double force_weight, int flags, double* rmse, double* force_rmse) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  if (frames < 1 || stride < 0 || !(lr > 0.0) || force_weight < 0.0) return PFMD_E_PARAM;
  return guard(c, [&] {
    c->e->learned_train(model_in ? model_in : "", model_out ? model_out : "", frames, stride, iters, flags, nullptr,
                        nullptr, nullptr, lr, force_weight, rmse, force_rmse);
  });
}

int pfmd_learned_gradient(pfmd_ctx* c, const char* model_in, double force_weight, int flags, float* grad,
                          double* loss, double* device_ms) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  if (!grad || force_weight < 0.0) return PFMD_E_PARAM;
  if (device_ms) *device_ms = 0.0;
  return guard(c, [&] {
    c->e->learned_train(model_in ? model_in : "", "", 1, 0, 1, flags, grad, loss, device_ms, 1e-3, force_weight,
                        nullptr, nullptr);
  });
}

int pfmd_learned_use(pfmd_ctx* c, const char* model_path, long long check_period, double max_rmse, int flags) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  if (!model_path || check_period < 0) return PFMD_E_PARAM;
  return guard(c, [&] {
    auto& e = *c->e;
    std::vector<pfmd::learned::Model> ms;
    try {
      ms = pfmd::learned::load_models(model_path);
    } catch (const std::runtime_error& x) {
      throw ::pfmd::Error(PFMD_E_IO, x.what());
    }
    e.learned_setup(ms);
    for (auto& M : e.lrn) M.tc = (flags & PFMD_LEARNED_TENSOR_CORES) != 0;
    e.learned_active = true;
    e.check_period = check_period;
    e.max_rmse = max_rmse;
    e.checks = 0;
    e.last_rmse = -1.0;
    e.fallen_back = false;
  });
}

int pfmd_learned_check(pfmd_ctx* c, double* rmse) {
  if (!c || !c->e || !c->e->ctl) return PFMD_E_STATE;
  return guard(c, [&] {
    if (c->e->lrn.empty()) throw ::pfmd::Error(PFMD_E_STATE, "learned form: no model loaded");
    const double r = c->e->learned_check(false);
    if (rmse) *rmse = r;
  });
}

int pfmd_learned_status(const pfmd_ctx* c, int* active, int* checks, double* last_rmse, int* fallen_back) {
  if (!c || !c->e) return PFMD_E_STATE;
  const auto& e = *c->e;
  if (active) *active = e.learned_active ? 1 : 0;
  if (checks) *checks = e.checks;
  if (last_rmse) *last_rmse = e.last_rmse;
  if (fallen_back) *fallen_back = e.fallen_back ? 1 : 0;
  return PFMD_OK;
}

int pfmd_kernel_launches(const pfmd_ctx* c, long long* n) {
  if (!c || !c->e || !n) return PFMD_E_STATE;
  *n = c->e->launches;
  return PFMD_OK;
}

int pfmd_debug_waits(unsigned int spin_limit, int stall) {
  pfmd::g_wait_hook.spin_limit = spin_limit;
  pfmd::g_wait_hook.stall = stall ? 1 : 0;
  return PFMD_OK;
}

}  // extern "C"

// Test shim: exposes the Fortran-format helpers of pfmds_gb300/csrc/fortio.h and
// the settings reader through a C interface for the CPU tests.
#include <cstring>
#include <string>

#include "../../pfmds_gb300/csrc/settings.h"

static void put(const std::string& s, char* out, int cap) {
  std::strncpy(out, s.c_str(), static_cast<size_t>(cap) - 1);
  out[cap - 1] = 0;
}

extern "C" {
void sh_fmt_f(double x, int w, int d, char* out, int cap) { put(fortio::fmt_f(x, w, d), out, cap); }
// the allocation-free Fw.d of the .xyz writers
void sh_put_f(double x, int w, int d, char* out, int cap) {
  std::string s;
  pfmd_io::put_f(s, x, w, d);
  put(s, out, cap);
}
// a snapshot of n atoms at x = k*scale, formatted by the threaded writer, against
// the same lines built one by one with fmt_f; returns 1 when equal
int sh_snapshot_matches(int n, double scale) {
  std::vector<double> pos(3 * static_cast<size_t>(n)), vel(3 * static_cast<size_t>(n)), mass(static_cast<size_t>(n));
  std::vector<int> idx(static_cast<size_t>(n));
  std::vector<std::string> types(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) {
    for (int c = 0; c < 3; ++c) {
      pos[3 * i + c] = (i * 3 + c) * scale - 0.37;
      vel[3 * i + c] = -(i + c) * scale * 1e-3;
    }
    mass[i] = 12.011 + i % 3;
    idx[i] = n - 1 - i;
    types[i] = i % 2 ? "C" : "CU_fixed";
  }
  const double box[3] = {10.0, 20.0, 30.0};
  const std::string got = pfmd_io::xyz_snapshot_text(box, n, idx.data(), pos.data(), vel.data(), mass.data(), types);
  std::string want;
  for (int k = 0; k < n; ++k) {
    const int i = idx[k];
    fortio::Rec a;
    for (int c = 0; c < 3; ++c) a.f(pos[3 * i + c], 27, 16);
    for (int c = 0; c < 3; ++c) a.f(vel[3 * i + c], 27, 16);
    a.f(mass[i], 27, 16).a("    ").a(types[static_cast<size_t>(i)], -1, 32);
    want += a.s + "\n";
  }
  return got.size() >= want.size() && got.compare(got.size() - want.size(), want.size(), want) == 0 ? 1 : 0;
}
void sh_fmt_es(double x, int w, int d, char* out, int cap) { put(fortio::fmt_es(x, w, d), out, cap); }
void sh_fmt_i(long long v, int w, char* out, int cap) { put(fortio::fmt_i(v, w), out, cap); }
void sh_fmt_i0(long long v, int w, int m, char* out, int cap) { put(fortio::fmt_i0pad(v, w, m), out, cap); }
void sh_fmt_a(const char* s, int w, int decl, char* out, int cap) { put(fortio::fmt_a(s, w, decl), out, cap); }
void sh_fmt_l(int v, int w, char* out, int cap) { put(fortio::fmt_l(v != 0, w), out, cap); }
void sh_list_int(long long v, char* out, int cap) { put(fortio::list_int(v), out, cap); }
void sh_list_real(double v, char* out, int cap) { put(fortio::list_real(v), out, cap); }
double sh_to_real(const char* s) { return fortio::to_real(s); }
// list-directed read of `n` items from `text`; items joined with '|', unset ones as '<unset>'
int sh_read_items(const char* text, int n, char* out, int cap) {
  try {
    fortio::ListReader r;
    r.from_string(text);
    auto it = r.read_items(static_cast<size_t>(n));
    std::string s;
    for (size_t k = 0; k < it.size(); ++k) {
      if (k) s += "|";
      s += it[k].set ? it[k].s : "<unset>";
    }
    put(s, out, cap);
    return 0;
  } catch (const std::exception& e) {
    put(e.what(), out, cap);
    return 1;
  }
}
}

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

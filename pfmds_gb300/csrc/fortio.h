// Fortran-style text I/O used by PFMDS's input and output files.
//
// PFMDS reads its settings, parameter and .xyz files with list-directed READ
// statements (md_simulation.f90:48-94, md_read_write.f90:10-61, the
// read_*_parameters routines) and writes its log, snapshot and trajectory files
// with explicit edit descriptors (md_simulation.f90:205-268,
// md_read_write.f90:65-107).  This header reproduces both halves in C++ so a
// drop-in driver consumes and produces the same files:
//
//   * ListReader: one READ statement consumes items from the current record and,
//     when it runs out, from the following records; whatever is left of the last
//     record it touched is discarded.  Undelimited character items end at a blank,
//     comma or end of record; a slash ends the whole statement.  'd'/'D' exponents
//     and the logical forms T/F/.true./.false. are accepted.
//   * fmt_* writers: Aw, Iw, Fw.d, ESw.d and Lw with Fortran's justification,
//     overflow-to-asterisks and exponent rules, plus gfortran's list-directed forms.
//
// Header-only; no CUDA, no allocation beyond std::string.
#pragma once

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace fortio {

struct ReadError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------------------
// List-directed reader over the records (lines) of one file.
// ---------------------------------------------------------------------------
// Per-thread input overlay: while a path is listed here, ListReader::open reads
// the file it maps to instead.  Concurrent md() runs of the fitting runner use it
// to read their own structure and parameter files under the names their settings
// give.
inline thread_local std::vector<std::pair<std::string, std::string>> t_overlay;
inline const std::string& overlaid(const std::string& path) {
  for (const auto& kv : t_overlay)
    if (kv.first == path) return kv.second;
  return path;
}

class ListReader {
 public:
  ListReader() = default;
  explicit ListReader(const std::string& path) { open(path); }

  bool open(const std::string& path) {
    std::ifstream f(overlaid(path));
    if (!f) return false;
    lines_.clear();
    std::string s;
    while (std::getline(f, s)) {
      if (!s.empty() && s.back() == '\r') s.pop_back();
      lines_.push_back(s);
    }
    rec_ = 0;
    path_ = path;
    return true;
  }
  void from_string(const std::string& text) {
    lines_.clear();
    std::istringstream f(text);
    std::string s;
    while (std::getline(f, s)) {
      if (!s.empty() && s.back() == '\r') s.pop_back();
      lines_.push_back(s);
    }
    rec_ = 0;
  }
  const std::string& path() const { return path_; }
  bool eof() const { return rec_ >= lines_.size(); }

  // read(u,'(A)') str : the whole next record.
  std::string read_line() {
    if (rec_ >= lines_.size()) throw ReadError("end of file in " + path_);
    return lines_[rec_++];
  }
  // read(u,*) with no items: skip one record.
  void skip_record() {
    if (rec_ >= lines_.size()) throw ReadError("end of file in " + path_);
    ++rec_;
  }

  // One list-directed READ statement for n items.  Returns the raw tokens, which
  // the caller converts with to_real / to_int / to_logical / to_char; a slash, or a
  // null value between two commas, leaves an item unset.
  struct Item {
    bool set = false;
    std::string s;
  };
  std::vector<Item> read_items(size_t n) {
    std::vector<Item> out(n);
    if (rec_ >= lines_.size()) throw ReadError("end of file in " + path_);
    size_t pos = 0;
    const std::string* line = &lines_[rec_];
    size_t k = 0;
    bool after_value = false;  // a comma right after a value is only its separator
    while (k < n) {
      while (pos < line->size() && is_blank((*line)[pos])) ++pos;
      if (pos >= line->size()) {  // end of record: a separator, go on to the next one
        ++rec_;
        if (rec_ >= lines_.size()) throw ReadError("end of file in " + path_);
        line = &lines_[rec_];
        pos = 0;
        continue;
      }
      char c = (*line)[pos];
      if (c == ',') {
        ++pos;
        if (after_value) {
          after_value = false;
        } else {
          ++k;  // null value: the item keeps its previous value
        }
        continue;
      }
      if (c == '/') break;  // slash: the statement ends here
      std::string tok;
      bool slash = false;
      if (c == '\'' || c == '"') {
        char q = c;
        ++pos;
        for (;;) {
          if (pos >= line->size()) {  // a delimited string may continue on the next record
            ++rec_;
            if (rec_ >= lines_.size()) throw ReadError("unterminated string in " + path_);
            line = &lines_[rec_];
            pos = 0;
            continue;
          }
          if ((*line)[pos] == q) {
            if (pos + 1 < line->size() && (*line)[pos + 1] == q) {
              tok.push_back(q);
              pos += 2;
              continue;
            }
            ++pos;
            break;
          }
          tok.push_back((*line)[pos++]);
        }
      } else {
        while (pos < line->size() && !is_blank((*line)[pos]) && (*line)[pos] != ',' &&
               (*line)[pos] != '/')
          tok.push_back((*line)[pos++]);
        if (pos < line->size() && (*line)[pos] == '/') slash = true;
      }
      out[k].set = true;
      out[k].s = tok;
      ++k;
      after_value = true;
      if (slash) break;
    }
    ++rec_;  // the rest of the last record is skipped
    return out;
  }

 private:
  static bool is_blank(char c) { return c == ' ' || c == '\t'; }
  std::vector<std::string> lines_;
  size_t rec_ = 0;
  std::string path_;
};

// Fortran numeric input conversion (list-directed, F editing rules).
inline double to_real(const std::string& t) {
  std::string s;
  s.reserve(t.size() + 1);
  bool seen_digit = false;
  for (size_t i = 0; i < t.size(); ++i) {
    char c = t[i];
    if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
    // "1.5-3" means 1.5e-3 : a sign after a digit of the mantissa starts an exponent
    if ((c == '+' || c == '-') && seen_digit && !s.empty() && s.back() != 'e' && s.back() != 'E')
      s.push_back('e');
    if (std::isdigit(static_cast<unsigned char>(c))) seen_digit = true;
    s.push_back(c);
  }
  char* end = nullptr;
  double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') throw ReadError("bad real value '" + t + "'");
  return v;
}
inline long long to_int(const std::string& t) {
  char* end = nullptr;
  long long v = std::strtoll(t.c_str(), &end, 10);
  if (end == t.c_str() || *end != '\0') throw ReadError("bad integer value '" + t + "'");
  return v;
}
inline bool to_logical(const std::string& t) {
  size_t i = 0;
  if (i < t.size() && t[i] == '.') ++i;
  if (i >= t.size()) throw ReadError("bad logical value '" + t + "'");
  char c = static_cast<char>(std::toupper(static_cast<unsigned char>(t[i])));
  if (c == 'T') return true;
  if (c == 'F') return false;
  throw ReadError("bad logical value '" + t + "'");
}
// character(len=n) assignment: truncate to n (trailing blanks are implicit)
inline std::string to_char(const std::string& t, size_t len = 32) {
  return t.size() > len ? t.substr(0, len) : t;
}

// ---------------------------------------------------------------------------
// Edit-descriptor writers.
// ---------------------------------------------------------------------------
inline std::string stars(int w) { return std::string(static_cast<size_t>(w), '*'); }

// Aw with a character entity of length len(s): right-justified when shorter than w,
// leftmost w characters when longer.  Fortran variables carry trailing blanks up to
// their declared length: pass `declared_len` to reproduce a padded variable.
inline std::string fmt_a(const std::string& s, int w = -1, int declared_len = -1) {
  std::string v = s;
  if (declared_len >= 0 && static_cast<int>(v.size()) < declared_len)
    v.append(static_cast<size_t>(declared_len) - v.size(), ' ');
  if (w < 0) return v;
  if (static_cast<int>(v.size()) >= w) return v.substr(0, static_cast<size_t>(w));
  return std::string(static_cast<size_t>(w) - v.size(), ' ') + v;
}

inline std::string fmt_i(long long v, int w) {
  std::string s = std::to_string(v);
  if (static_cast<int>(s.size()) > w) return stars(w);
  return std::string(static_cast<size_t>(w) - s.size(), ' ') + s;
}

// Iw.m : at least m digits
inline std::string fmt_i0pad(long long v, int w, int m) {
  char buf[64];
  if (v < 0)
    std::snprintf(buf, sizeof buf, "-%0*lld", m, -v);
  else
    std::snprintf(buf, sizeof buf, "%0*lld", m, v);
  std::string s(buf);
  if (static_cast<int>(s.size()) > w) return stars(w);
  return std::string(static_cast<size_t>(w) - s.size(), ' ') + s;
}

inline std::string fmt_l(bool v, int w) {
  return std::string(static_cast<size_t>(w > 0 ? w - 1 : 0), ' ') + (v ? "T" : "F");
}

// Fw.d : fixed point, correctly rounded; a leading zero is kept only when the field
// has room for it; no room for the digits gives w asterisks.
inline std::string fmt_f(double x, int w, int d) {
  if (std::isnan(x)) return std::string(static_cast<size_t>(w > 3 ? w - 3 : 0), ' ') + "NaN";
  if (std::isinf(x)) {
    std::string s = x < 0 ? "-Infinity" : "Infinity";
    if (static_cast<int>(s.size()) > w) s = x < 0 ? "-Inf" : "Inf";
    if (static_cast<int>(s.size()) > w) return stars(w);
    return std::string(static_cast<size_t>(w) - s.size(), ' ') + s;
  }
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.*f", d, x);
  std::string s(buf);
  if (static_cast<int>(s.size()) > w) {
    // drop the optional leading zero of "0.xxx" / "-0.xxx"
    if (s.rfind("0.", 0) == 0)
      s.erase(0, 1);
    else if (s.rfind("-0.", 0) == 0)
      s.erase(1, 1);
  }
  if (static_cast<int>(s.size()) > w) return stars(w);
  return std::string(static_cast<size_t>(w) - s.size(), ' ') + s;
}

// ESw.d : scientific with one nonzero digit before the point; exponent E+dd, or
// +ddd without the letter when |exponent| > 99.
inline std::string fmt_es(double x, int w, int d) {
  if (std::isnan(x) || std::isinf(x)) return fmt_f(x, w, d);
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.*E", d, x);
  std::string s(buf);
  size_t e = s.find('E');
  std::string mant = s.substr(0, e);
  int ex = std::atoi(s.c_str() + e + 1);
  char eb[16];
  if (std::abs(ex) <= 99)
    std::snprintf(eb, sizeof eb, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  else
    std::snprintf(eb, sizeof eb, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  s = mant + eb;
  if (static_cast<int>(s.size()) > w) return stars(w);
  return std::string(static_cast<size_t>(w) - s.size(), ' ') + s;
}

// gfortran list-directed output items.  Every record starts with one blank; a
// default INTEGER occupies 12 columns including its separator; a REAL(8) is written
// as G26.17 (F form with 17 significant digits and 4 trailing blanks when
// 0.1 <= |x| < 1e17, otherwise ES with a three-digit exponent).
inline std::string list_int(long long v) { return fmt_i(v, 12); }
inline std::string list_real(double x) {
  double ax = std::fabs(x);
  if (x == 0.0) return fmt_f(0.0, 22, 17 - 1) + "    ";
  if (ax >= 0.1 && ax < 1e17) {
    int digits_before = static_cast<int>(std::floor(std::log10(ax))) + 1;
    if (digits_before < 0) digits_before = 0;
    int d = 17 - digits_before;
    if (d < 0) d = 0;
    return fmt_f(x, 22, d) + "    ";
  }
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.16E", x);
  std::string s(buf);
  size_t e = s.find('E');
  int ex = std::atoi(s.c_str() + e + 1);
  char eb[16];
  std::snprintf(eb, sizeof eb, "E%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  s = s.substr(0, e) + eb;
  return std::string(s.size() < 26 ? 26 - s.size() : 0, ' ') + s;
}
inline std::string list_logical(bool v) { return v ? " T" : " F"; }

// Helper for building one formatted record.
struct Rec {
  std::string s;
  Rec& a(const std::string& v, int w = -1, int declared = -1) {
    s += fmt_a(v, w, declared);
    return *this;
  }
  Rec& i(long long v, int w) {
    s += fmt_i(v, w);
    return *this;
  }
  Rec& f(double v, int w, int d) {
    s += fmt_f(v, w, d);
    return *this;
  }
  Rec& es(double v, int w, int d) {
    s += fmt_es(v, w, d);
    return *this;
  }
  Rec& l(bool v, int w) {
    s += fmt_l(v, w);
    return *this;
  }
};

// Fortran TRIM: drop trailing blanks.
inline std::string trim(const std::string& s) {
  size_t n = s.size();
  while (n > 0 && s[n - 1] == ' ') --n;
  return s.substr(0, n);
}

}  // namespace fortio

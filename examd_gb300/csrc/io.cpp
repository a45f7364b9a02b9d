// io.cpp -- the reference's particle file, exaMD_particles.dat.
//
// Format (SRC/exaMD_input_formats.f90:128-208, written by
// exaMD_write_particles :211-235): Fortran list-directed text.
//   record 1: natms_tot              (Read(50,*) natms_tot, :139)
//   record 2: globalbox(1:3)         (Read(50,*) globalbox, :140)
//   then natms_tot records: x y z    (Read(50,*) posxyz, :169)
// Each READ starts at a new record and may continue onto the next ones until
// its items are read; the rest of its last record is skipped.  Items are
// separated by blanks or commas; reals may use E, D or Q exponents; an item
// may carry a repeat count r*value.  Positions are returned as read: the
// reference assigns blocks from them as they are (exaMD_identify_block), and
// the library wraps or rejects them when the atoms are set.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "../../include/examd_gb300.h"

namespace {

class ListReader {
 public:
  explicit ListReader(std::FILE* f) : f_(f) {}

  // Read n values starting at a new record; false at end of file or on a
  // malformed item.
  bool read_reals(double* out, int n) {
    int got = 0;
    while (got < n) {
      if (!next_record()) return false;
      size_t p = 0;
      std::string tok;
      while (got < n && next_token(p, tok)) {
        int rep = 1;
        const size_t star = tok.find('*');
        if (star != std::string::npos) {
          char* end = nullptr;
          const long r = std::strtol(tok.substr(0, star).c_str(), &end, 10);
          if (star == 0 || *end != '\0' || r < 1) return false;
          rep = (int)r;
          tok = tok.substr(star + 1);
          if (tok.empty()) return false;  // null values are not used by this format
        }
        double v;
        if (!parse_real(tok, v)) return false;
        for (int k = 0; k < rep && got < n; ++k) out[got++] = v;
      }
    }
    return true;
  }

  bool read_int64(int64_t* out) {
    if (!next_record()) return false;
    size_t p = 0;
    std::string tok;
    if (!next_token(p, tok)) return false;
    char* end = nullptr;
    errno = 0;
    const long long v = std::strtoll(tok.c_str(), &end, 10);
    if (errno != 0 || end == tok.c_str() || *end != '\0') return false;
    *out = v;
    return true;
  }

 private:
  bool next_record() {
    line_.clear();
    int c;
    bool any = false;
    while ((c = std::fgetc(f_)) != EOF) {
      any = true;
      if (c == '\n') break;
      line_.push_back((char)c);
    }
    return any;
  }

  bool next_token(size_t& p, std::string& tok) {
    while (p < line_.size() && (line_[p] == ' ' || line_[p] == '\t' || line_[p] == '\r')) ++p;
    if (p < line_.size() && line_[p] == ',') ++p;  // one separator comma
    while (p < line_.size() && (line_[p] == ' ' || line_[p] == '\t' || line_[p] == '\r')) ++p;
    if (p >= line_.size()) return false;
    const size_t b = p;
    while (p < line_.size() && line_[p] != ' ' && line_[p] != '\t' && line_[p] != '\r' && line_[p] != ',') ++p;
    tok = line_.substr(b, p - b);
    return true;
  }

  static bool parse_real(std::string s, double& v) {
    for (char& ch : s)
      if (ch == 'd' || ch == 'D' || ch == 'q' || ch == 'Q') ch = 'e';
    char* end = nullptr;
    errno = 0;
    v = std::strtod(s.c_str(), &end);
    return errno == 0 && end != s.c_str() && *end == '\0' && std::isfinite(v);
  }

  std::FILE* f_;
  std::string line_;
};

}  // namespace

extern "C" int examd_read_particles(const char* path, int64_t* natoms, double* L, double* pos, int64_t capacity) {
  if (!path || !natoms || !L) return EXAMD_ERR_ARG;
  std::FILE* f = std::fopen(path, "r");
  if (!f) return EXAMD_ERR_IO;
  ListReader rd(f);
  int64_t n = 0;
  double box[3];
  int rc = EXAMD_OK;
  if (!rd.read_int64(&n) || n < 0 || !rd.read_reals(box, 3)) {
    rc = EXAMD_ERR_IO;
  } else {
    *natoms = n;
    for (int a = 0; a < 3; ++a) L[a] = box[a];
    if (pos) {
      if (capacity < n) {
        rc = EXAMD_ERR_ARG;
      } else {
        for (int64_t i = 0; i < n; ++i)
          if (!rd.read_reals(pos + 3 * i, 3)) {
            rc = EXAMD_ERR_IO;
            break;
          }
      }
    }
  }
  std::fclose(f);
  return rc;
}

extern "C" int examd_write_particles(const char* path, int64_t natoms, const double* L, const double* pos) {
  if (!path || natoms < 0 || !L || (natoms > 0 && !pos)) return EXAMD_ERR_ARG;
  std::FILE* f = std::fopen(path, "w");
  if (!f) return EXAMD_ERR_IO;
  // 17 significant digits: a list-directed Read gives back the same doubles
  bool ok = std::fprintf(f, " %lld\n", (long long)natoms) > 0 &&
            std::fprintf(f, " %.17g %.17g %.17g\n", L[0], L[1], L[2]) > 0;
  for (int64_t i = 0; ok && i < natoms; ++i)
    ok = std::fprintf(f, " %.17g %.17g %.17g\n", pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]) > 0;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? EXAMD_OK : EXAMD_ERR_IO;
}

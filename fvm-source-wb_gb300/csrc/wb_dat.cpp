// wb_dat.cpp -- the reference's text snapshot format, '(7(1PE12.5,1X))': the number
// formatter shared by the 2D and 1D writers (output_file, 2d/benchmark_2d_dg.f90:468-495
// and benchmark_1d.f90:69-100) and the reader (the np.loadtxt of get_image,
// post_processing2d.py:55-64, which cannot parse the three-digit-exponent form).
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wb_capi.h"
#include "wb_tables.h"

namespace wb {

// Fortran 1PE12.5: one digit before the point, five after, exponent E+dd (or +ddd with
// the E dropped when the exponent needs three digits), right-justified in 12 columns.
void fortran_1pe12_5(double v, char *out) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.5E", v);
  char *e = std::strchr(buf, 'E');
  if (e) {
    int ex = std::atoi(e + 1);
    if (ex >= 100 || ex <= -100) std::snprintf(e, 8, "%c%03d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
  }
  std::snprintf(out, 16, "%12s", buf);
}

// One edit-descriptor field: a plain number (1.23456E-03, NaN, Infinity) or the
// three-digit-exponent form with the E dropped (1.23456-100).  False if the token is not
// a number.
bool parse_fortran_real(const char *tok, double *v) {
  errno = 0;
  char *end = nullptr;
  double m = std::strtod(tok, &end);
  if (end == tok) return false;
  if (*end == '\0') {
    *v = m;
    return true;
  }
  if ((*end == '+' || *end == '-') && end != tok) {
    char *e2 = nullptr;
    long ex = std::strtol(end, &e2, 10);
    if (*e2 != '\0' || e2 == end + 1) return false;
    std::string s = std::string(tok, end - tok) + "E" + std::to_string(ex);
    char *e3 = nullptr;
    *v = std::strtod(s.c_str(), &e3);
    return *e3 == '\0';
  }
  return false;
}

}  // namespace wb

extern "C" int wb_read_dat(const char *path, int32_t ncols, double *values, int64_t capacity,
                           int64_t *nrows) {
  if (!path || ncols < 1 || capacity < 0 || (capacity > 0 && !values) || !nrows) return WB_ERR_ARG;
  *nrows = 0;
  FILE *f = std::fopen(path, "r");
  if (!f) return WB_ERR_ARG;
  // A record of ncols values fills ceil(ncols / 7) lines: 7 values per line (the
  // descriptor's repeat count), the remainder on the last.
  std::vector<char> line(4096);
  int64_t row = 0;
  int col = 0;
  int rc = WB_OK;
  while (std::fgets(line.data(), (int)line.size(), f)) {
    size_t len = std::strlen(line.data());
    if (len + 1 == line.size() && line[len - 1] != '\n') {
      rc = WB_ERR_ARG;  // longer than any record of this format
      break;
    }
    int on_line = 0;
    bool record_ended = false;  // a record ended on this line: nothing may follow it
    char *save = nullptr;
    for (char *tok = strtok_r(line.data(), " \t\r\n", &save); tok;
         tok = strtok_r(nullptr, " \t\r\n", &save)) {
      double v;
      if (record_ended || !wb::parse_fortran_real(tok, &v) || row >= capacity) {
        rc = WB_ERR_ARG;
        break;
      }
      values[row * ncols + col] = v;
      ++on_line;
      if (++col == ncols) {
        col = 0;
        ++row;
        record_ended = true;
      }
    }
    if (rc) break;
    if (on_line == 0) continue;  // blank line
    // every line holds 7 values, except the last line of a record
    if (on_line > 7 || (on_line < 7 && !record_ended)) {
      rc = WB_ERR_ARG;
      break;
    }
  }
  std::fclose(f);
  if (rc == WB_OK && col != 0) rc = WB_ERR_ARG;  // a record cut short
  *nrows = row;
  return rc;
}

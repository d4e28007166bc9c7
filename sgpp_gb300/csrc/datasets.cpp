// Host-side dataset ingest: ARFF and CSV text read exactly as the reference's readers read it
// (datadriven/src/sgpp/datadriven/tools/ARFFTools.cpp, CSVTools.cpp), so a data set read here
// and handed to sgmev_create gives the same matrix and targets as the reference's Dataset.
// C ABI in include/sgmev.h (sgdata_*). Text parsing stays on the host: it is a single pass over
// bytes, far cheaper than the copy of the parsed matrix to the device (and the bounding-box
// transform happens on the device at staging).
//
// Reading rules (both readers, ARFFTools.cpp readARFFSize/readARFF, CSVTools.cpp
// readCSVSize/readCSV):
//   * the text is split at '\n'; a final piece after the last '\n' is a line too (an input
//     ending in '\n' gives a last, empty line), '\r' is kept (values parse through it);
//   * ARFF: every line containing '%' or '@' anywhere is skipped, then every empty line;
//   * CSV: the size pass skips empty lines before it consumes the optional header line, the read
//     pass consumes the header line first (the reference's two passes differ here, and so do
//     these);
//   * the first data line fixes the dimension: its number of commas (+1 without targets); while
//     that count is 0 the next data line fixes it again; every later data line must have the
//     same number of commas, else "Columns missing in line <instances so far>";
//   * values are the fields between commas parsed with strtod (atof: leading blanks skipped,
//     trailing text ignored, an empty field is 0);
//   * with targets the last field is the target; a non-empty target filter keeps the rows whose
//     target lies within 0.001 of one of its values (a ragged line fails even when filtered);
//   * an instance cutoff keeps the first rows; a column selection picks and orders columns
//     (an index at or beyond the dimension fails, and so does a selected column missing from a
//     shorter data line);
//   * a cutoff of 0 gives no rows (the reference writes row 0 of its empty matrix there).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sgmev.h"

namespace sgmev {
extern thread_local std::string g_last_error;
}

namespace {

int data_fail(int code, const std::string& msg) {
  sgmev::g_last_error = msg;
  return code;
}

struct Line {
  const char* p;
  size_t n;
  bool empty() const { return n == 0; }
  bool has(char c) const { return std::memchr(p, c, n) != nullptr; }
  int64_t commas() const {
    int64_t k = 0;
    for (size_t i = 0; i < n; ++i) k += p[i] == ',';
    return k;
  }
};

std::vector<Line> split_lines(const char* text, int64_t len) {
  std::vector<Line> lines;
  size_t start = 0;
  const size_t n = static_cast<size_t>(len);
  for (size_t i = 0; i < n; ++i) {
    if (text[i] == '\n') {
      lines.push_back(Line{text + start, i - start});
      start = i + 1;
    }
  }
  lines.push_back(Line{text + start, n - start});
  return lines;
}

double parse_field(const char* p, size_t n) {
  const std::string s(p, n);  // strtod needs a terminated string
  return std::strtod(s.c_str(), nullptr);
}

// fields of a line, split at every ',' (an empty field is a value too)
void parse_line(const Line& l, std::vector<double>& out) {
  out.clear();
  size_t start = 0;
  for (size_t i = 0; i <= l.n; ++i) {
    if (i == l.n || l.p[i] == ',') {
      out.push_back(parse_field(l.p + start, i - start));
      start = i + 1;
    }
  }
}

double last_field(const Line& l) {
  size_t i = l.n;
  while (i > 0 && l.p[i - 1] != ',') --i;
  return parse_field(l.p + i, l.n - i);
}

bool selected(double target, const double* targets, int n_targets) {
  if (n_targets <= 0) return true;
  for (int k = 0; k < n_targets; ++k)
    if (std::fabs(target - targets[k]) < 0.001) return true;
  return false;
}

struct Options {
  int format;
  bool has_targets;
  bool skip_first_line;
  const double* targets;
  int n_targets;
};

// readARFFSize / readCSVSize
int size_pass(const std::vector<Line>& lines, const Options& o, int64_t* n_instances,
              int64_t* dim) {
  int64_t d = 0, n = 0;
  bool skip = o.skip_first_line;
  const int64_t extra = o.has_targets ? 0 : 1;
  for (const Line& l : lines) {
    if (o.format == SGDATA_ARFF) {
      if (l.has('%') || l.has('@')) continue;
      if (l.empty()) continue;
    } else {
      if (l.empty()) continue;
      if (skip) {
        skip = false;
        continue;
      }
    }
    const int64_t c = l.commas();
    if (d == 0) {
      d = c + extra;
    } else if (d - c != extra) {
      return data_fail(SGMEV_ERR_INVALID,
                       std::string(o.format == SGDATA_ARFF ? "readARFFSize" : "readCSVSize") +
                           ": Columns missing in line " + std::to_string(n));
    }
    if (o.has_targets && o.n_targets > 0) {
      if (selected(last_field(l), o.targets, o.n_targets)) ++n;
    } else {
      ++n;
    }
  }
  *n_instances = n;
  *dim = d;
  return SGMEV_OK;
}

int check_format(int format) {
  if (format != SGDATA_ARFF && format != SGDATA_CSV)
    return data_fail(SGMEV_ERR_INVALID, "format must be SGDATA_ARFF or SGDATA_CSV");
  return SGMEV_OK;
}

}  // namespace

extern "C" {

SGMEV_API int sgdata_size(int format, const char* text, int64_t len, int has_targets,
                          int skip_first_line, const double* targets, int n_targets,
                          int64_t* n_instances, int64_t* dim) {
  sgmev::g_last_error.clear();
  int rc = check_format(format);
  if (rc != SGMEV_OK) return rc;
  if ((!text && len > 0) || len < 0 || !n_instances || !dim || (n_targets > 0 && !targets))
    return data_fail(SGMEV_ERR_INVALID, "sgdata_size: bad arguments");
  const Options o{format, has_targets != 0, skip_first_line != 0, targets, n_targets};
  return size_pass(split_lines(text ? text : "", len), o, n_instances, dim);
}

SGMEV_API int sgdata_read(int format, const char* text, int64_t len, int has_targets,
                          int skip_first_line, int64_t cutoff, const int64_t* cols, int n_cols,
                          const double* targets, int n_targets, double* data, double* y,
                          int64_t n_cap, int64_t* n_read, int64_t* dim_out) {
  sgmev::g_last_error.clear();
  int rc = check_format(format);
  if (rc != SGMEV_OK) return rc;
  if ((!text && len > 0) || len < 0 || !n_read || !dim_out || (n_cols > 0 && !cols) ||
      (n_targets > 0 && !targets) || n_cap < 0)
    return data_fail(SGMEV_ERR_INVALID, "sgdata_read: bad arguments");
  const std::vector<Line> lines = split_lines(text ? text : "", len);
  const Options o{format, has_targets != 0, skip_first_line != 0, targets, n_targets};
  int64_t max_inst = 0, max_dim = 0;
  rc = size_pass(lines, o, &max_inst, &max_dim);
  if (rc != SGMEV_OK) return rc;
  int64_t dim = max_dim;
  if (n_cols > 0) {
    for (int k = 0; k < n_cols; ++k) {
      if (cols[k] < 0 || cols[k] >= max_dim)
        return data_fail(SGMEV_ERR_INVALID, format == SGDATA_ARFF
                                                ? "readCSVPartial invalid col selection"
                                                : "readCSV invalid column selection");
    }
    dim = n_cols;
  }
  const int64_t n_inst = cutoff < 0 ? max_inst : std::min(max_inst, cutoff);
  if (n_inst > n_cap)
    return data_fail(SGMEV_ERR_INVALID, "sgdata_read: n_cap is smaller than the instances");
  if (n_inst > 0 && dim > 0 && !data)
    return data_fail(SGMEV_ERR_INVALID, "sgdata_read: data is NULL");
  if (n_inst > 0 && has_targets && !y) return data_fail(SGMEV_ERR_INVALID, "sgdata_read: y is NULL");
  *dim_out = dim;
  *n_read = 0;
  if (n_inst == 0) return SGMEV_OK;  // the reference would write into an empty matrix here
  bool skip = o.skip_first_line;
  int64_t row = 0;
  std::vector<double> vals;
  for (const Line& l : lines) {
    if (o.format == SGDATA_ARFF) {
      if (l.has('%') || l.has('@')) continue;
      if (l.empty()) continue;
    } else {
      if (skip) {
        skip = false;
        continue;
      }
      if (l.empty()) continue;
    }
    parse_line(l, vals);
    if (o.has_targets) {
      const double t = vals.back();
      vals.pop_back();
      if (!selected(t, targets, n_targets)) continue;
      y[row] = t;
    }
    double* out = data + row * dim;
    for (int64_t i = 0; i < dim; ++i) out[i] = 0.0;  // as the reference's zero-filled matrix
    if (n_cols == 0) {
      // every line has the first line's field count, so vals.size() == dim
      for (int64_t i = 0; i < dim && i < static_cast<int64_t>(vals.size()); ++i) out[i] = vals[i];
    } else {
      for (int k = 0; k < n_cols; ++k) {
        // a line with fewer fields than the first one (possible only through the rules above,
        // e.g. a "\r" line before the first data line) fails as the reference's vector::at does
        if (cols[k] >= static_cast<int64_t>(vals.size()))
          return data_fail(SGMEV_ERR_INVALID, "selected column " + std::to_string(cols[k]) +
                                                  " is missing in data line " +
                                                  std::to_string(row));
        out[k] = vals[cols[k]];
      }
    }
    ++row;
    if (row >= n_inst) break;
  }
  *n_read = row;
  return SGMEV_OK;
}

}  // extern "C"

// Host-side entry points of the C ABI: variogram string parsing and the
// nugget-only check. Pure C++ (no device code); errors are status codes.
#include <cuda_runtime.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "spinterps_gb300.h"

namespace {

bool is_space(char c) {
  return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f';
}

std::string strip(const std::string& s) {
  size_t b = 0, e = s.size();
  while (b < e && is_space(s[b])) ++b;
  while (e > b && is_space(s[e - 1])) --e;
  return s.substr(b, e - b);
}

// Python bytes.split(sep) with a one-character separator.
std::vector<std::string> split(const std::string& s, char sep) {
  std::vector<std::string> out;
  size_t start = 0;
  for (size_t i = 0; i <= s.size(); ++i) {
    if (i == s.size() || s[i] == sep) {
      out.push_back(s.substr(start, i - start));
      start = i + 1;
    }
  }
  return out;
}

bool is_digit(char c) { return c >= '0' && c <= '9'; }

// Python float() of a bytes token. ASCII whitespace may surround it; the
// rest must be, in full, [sign] followed by
//   digitpart ["." [digitpart]] | "." digitpart, then [("e"|"E") [sign] digitpart],
// with digitpart = digit (["_"] digit)*, or by "inf", "infinity" or "nan" in
// any case. No hexadecimal, no "nan(...)". The token without its
// underscores then goes to strtod, which rounds correctly as Python does.
bool py_float(const std::string& tok, double* out) {
  const std::string t = strip(tok);
  const size_t n = t.size();
  size_t i = 0;
  std::string clean;
  bool neg = false;
  if (i < n && (t[i] == '+' || t[i] == '-')) {
    neg = t[i] == '-';
    clean += t[i++];
  }
  std::string word;
  for (size_t j = i; j < n; ++j) word += (char)std::tolower((unsigned char)t[j]);
  if (word == "inf" || word == "infinity") {
    *out = neg ? -HUGE_VAL : HUGE_VAL;
    return true;
  }
  if (word == "nan") {
    *out = std::copysign(std::nan(""), neg ? -1.0 : 1.0);
    return true;
  }
  auto digitpart = [&]() {
    if (i >= n || !is_digit(t[i])) return false;
    clean += t[i++];
    while (i < n) {
      if (is_digit(t[i])) {
        clean += t[i++];
      } else if (t[i] == '_' && i + 1 < n && is_digit(t[i + 1])) {
        ++i;
      } else {
        break;
      }
    }
    return true;
  };
  const bool whole = digitpart();
  if (i < n && t[i] == '.') {
    clean += t[i++];
    const bool frac = digitpart();
    if (!whole && !frac) return false;
  } else if (!whole) {
    return false;
  }
  if (i < n && (t[i] == 'e' || t[i] == 'E')) {
    clean += t[i++];
    if (i < n && (t[i] == '+' || t[i] == '-')) clean += t[i++];
    if (!digitpart()) return false;
  }
  if (i != n) return false;
  *out = std::strtod(clean.c_str(), nullptr);
  return true;
}

int model_code(const std::string& name) {
  static const char* names[] = {"Rng", "Nug", "Sph", "Exp", "Lin", "Gau", "Pow", "Hol"};
  for (int i = 0; i < 8; ++i)
    if (name == names[i]) return i;
  return -1;
}

}  // namespace

// cyth/interpmthds.pyx:174-184: split on '+', strip, split on ' ' into
// exactly (sill, 'Name(range'), split on '(' into exactly (Name, 'range)'),
// range = part before ')', clamped to max(1e-5, range).
extern "C" int spi_parse_vg(const char* vg_str, spi_vg_t* out) {
  if (!vg_str || !out) return SPI_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  std::vector<std::string> parts = split(std::string(vg_str), '+');
  if (parts.size() > SPI_MAX_VG_COMP) return SPI_ERR_TOO_LARGE;
  int k = 0;
  for (const std::string& raw : parts) {
    std::string p = strip(raw);
    std::vector<std::string> a = split(p, ' ');
    if (a.size() != 2) return SPI_ERR_VG;
    std::vector<std::string> b = split(a[1], '(');
    if (b.size() != 2) return SPI_ERR_VG;
    std::string rs = split(b[1], ')')[0];
    int code = model_code(b[0]);
    if (code < 0) return SPI_ERR_VG;
    double sill, rng;
    if (!py_float(a[0], &sill) || !py_float(rs, &rng)) return SPI_ERR_VG;
    out->code[k] = code;
    out->sill[k] = sill;
    out->range[k] = std::fmax(1e-5, rng);
    if (std::isnan(rng)) out->range[k] = 1e-5;  // Python max(1e-5, nan) is 1e-5
    ++k;
  }
  out->n_comp = k;
  return SPI_OK;
}

// misc.py:1074-1105.
extern "C" int spi_check_full_nuggetness(const char* vg_str, double min_vg_val, int32_t* out) {
  if (!vg_str || !out) return SPI_ERR_ARG;
  std::string in(vg_str);
  *out = 0;
  if (in == "nan") return SPI_OK;
  std::vector<std::string> models = split(in, '+');
  double sill = 0.0, rng = 0.0;
  for (const std::string& raw : models) {
    std::string sub = strip(raw);
    std::string head = strip(split(sub, '(')[0]);
    if (head.size() < 3) return SPI_ERR_VG;
    double s;
    if (!py_float(head.substr(0, head.size() - 3), &s)) return SPI_ERR_VG;
    sill += s;
    std::vector<std::string> b = split(sub, '(');
    if (b.size() < 2) return SPI_ERR_VG;
    double r;
    if (!py_float(split(b[1], ')')[0], &r)) return SPI_ERR_VG;
    rng = std::fmax(rng, r);
  }
  if (sill <= min_vg_val || rng <= min_vg_val) *out = 1;
  return SPI_OK;
}

extern "C" const char* spi_version(void) { return "spinterps_gb300 0.1 (sm_103a)"; }

namespace spi {
static thread_local cudaError_t g_cuda_error = cudaSuccess;
void record_cuda_error(cudaError_t e) { g_cuda_error = e; }
}  // namespace spi

extern "C" const char* spi_cuda_error(void) {
  static thread_local char buf[256];
  cudaError_t e = spi::g_cuda_error;
  spi::g_cuda_error = cudaSuccess;
  if (e == cudaSuccess) e = cudaPeekAtLastError();
  if (e == cudaSuccess) return "";
  std::snprintf(buf, sizeof(buf), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
  return buf;
}

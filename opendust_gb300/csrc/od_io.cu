// od_io.cu — trajectory dumps of OpenDust.simulate() (opendust.py:1071-1098): one XYZ frame
// appended per call, or one CSV file per frame; and the restart file (opendust.py:1099-1115,
// read back at :452-466). Host code only. The reference formats every
// coordinate with Python's "{}".format (the shortest decimal string that reads back to the same
// double, in fixed notation for decimal exponents -4 .. 15 and scientific notation outside);
// the same text is produced here from std::to_chars, formatted in parallel host threads, so that
// the files are byte-identical and a frame of 2^20 ions takes a fraction of a second instead of
// several seconds of Python.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "od_internal.h"

namespace {

// Python's repr of a double: shortest round-trip digits; fixed notation when the decimal
// exponent e (value = d.ddd x 10^e) satisfies -4 <= e < 16, with at least one digit after the
// point; otherwise d[.ddd]e(+|-)XX with at least two exponent digits. Returns the length.
int repr_double(double v, char* out) {
  if (std::isnan(v)) { std::memcpy(out, "nan", 3); return 3; }
  if (std::isinf(v)) {
    if (v < 0) { std::memcpy(out, "-inf", 4); return 4; }
    std::memcpy(out, "inf", 3);
    return 3;
  }
  char sci[64];
  const auto r = std::to_chars(sci, sci + sizeof(sci), v, std::chars_format::scientific);
  const char* p = sci;
  const char* end = r.ptr;
  int n = 0;
  if (*p == '-') { out[n++] = '-'; p++; }
  // mantissa digits without the point, then the exponent
  char dig[32];
  int k = 0;
  while (p < end && *p != 'e') {
    if (*p != '.') dig[k++] = *p;
    p++;
  }
  int e = 0;  // "e+06" -> 6, "e-05" -> -5 (to_chars writes no terminating NUL)
  if (p < end) {
    p++;
    const bool neg = *p == '-';
    if (*p == '-' || *p == '+') p++;
    for (; p < end; p++) e = 10 * e + (*p - '0');
    if (neg) e = -e;
  }
  if (e >= -4 && e < 16) {
    const int point = e + 1;  // digits before the decimal point
    if (point <= 0) {
      out[n++] = '0';
      out[n++] = '.';
      for (int i = 0; i < -point; i++) out[n++] = '0';
      for (int i = 0; i < k; i++) out[n++] = dig[i];
    } else if (point < k) {
      for (int i = 0; i < point; i++) out[n++] = dig[i];
      out[n++] = '.';
      for (int i = point; i < k; i++) out[n++] = dig[i];
    } else {
      for (int i = 0; i < k; i++) out[n++] = dig[i];
      for (int i = k; i < point; i++) out[n++] = '0';
      out[n++] = '.';
      out[n++] = '0';
    }
  } else {
    out[n++] = dig[0];
    if (k > 1) {
      out[n++] = '.';
      for (int i = 1; i < k; i++) out[n++] = dig[i];
    }
    out[n++] = 'e';
    out[n++] = e < 0 ? '-' : '+';
    const int a = e < 0 ? -e : e;
    if (a >= 100) out[n++] = (char)('0' + a / 100);
    out[n++] = (char)('0' + (a / 10) % 10);
    out[n++] = (char)('0' + a % 10);
  }
  return n;
}

void append_repr(std::string& s, double v) {
  char b[40];
  s.append(b, (size_t)repr_double(v, b));
}

// Lines for ions [0, n) formatted by line(i0, i1, out) into pieces, in parallel host threads
// for large n (each thread its own contiguous range), returned in ion order.
template <class F>
std::vector<std::string> format_lines(int64_t n, size_t bytes_per_line, F line) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t parts = std::max<int64_t>(1, std::min<int64_t>({(int64_t)hw, 16, n / 16384}));
  std::vector<std::string> out((size_t)parts);
  std::vector<char> failed((size_t)parts, 0);
  auto work = [&](int64_t p) {
    const int64_t i0 = n * p / parts, i1 = n * (p + 1) / parts;
    try {
      out[(size_t)p].reserve((size_t)(i1 - i0) * bytes_per_line);
      line(i0, i1, out[(size_t)p]);
    } catch (...) {  // host memory exhausted: reported as a failed write
      failed[(size_t)p] = 1;
    }
  };
  if (parts == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int64_t p = 1; p < parts; p++) th.emplace_back(work, p);
    work(0);
    for (auto& t : th) t.join();
  }
  for (char f : failed)
    if (f) return {};
  return out;
}

bool write_all(const char* path, const char* mode, const std::string& head,
               const std::vector<std::string>& body) {
  FILE* f = std::fopen(path, mode);
  if (!f) return false;
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
  for (const auto& b : body) ok = ok && std::fwrite(b.data(), 1, b.size(), f) == b.size();
  return std::fclose(f) == 0 && ok;
}

}  // namespace

extern "C" int32_t od_format_double(double v, char* buf) {
  if (!buf) return 0;
  const int n = repr_double(v, buf);
  buf[n] = '\0';
  return n;
}

extern "C" od_status od_write_xyz_frame(const char* path, const double* xyz_nm, int64_t n,
                                        int64_t frame) {
  if (!path || (n > 0 && !xyz_nm) || n < 0)
    return od_fail_nohandle(OD_ERR_INVALID, "od_write_xyz_frame: NULL path or positions");
  const std::string head = std::to_string(n) + "\n" + std::to_string(frame) + "\n";
  const auto body = format_lines(n, 64, [xyz_nm](int64_t i0, int64_t i1, std::string& s) {
    for (int64_t i = i0; i < i1; i++) {
      s += "Ar\t";
      append_repr(s, xyz_nm[3 * i]);
      s += '\t';
      append_repr(s, xyz_nm[3 * i + 1]);
      s += '\t';
      append_repr(s, xyz_nm[3 * i + 2]);
      s += '\n';
    }
  });
  if ((n > 0 && body.empty()) || !write_all(path, "ab", head, body))
    return od_fail_nohandle(OD_ERR_INVALID, std::string("cannot append to ") + path);
  return OD_OK;
}

extern "C" od_status od_write_csv_frame(const char* path, const double* xyz_nm, int64_t n,
                                        double density, double mass) {
  if (!path || (n > 0 && !xyz_nm) || n < 0)
    return od_fail_nohandle(OD_ERR_INVALID, "od_write_csv_frame: NULL path or positions");
  // Python's csv.writer: comma separated, "\r\n" line ends, floats as repr
  std::string tail = ",";
  append_repr(tail, density);
  tail += ',';
  append_repr(tail, mass);
  tail += "\r\n";
  const auto body = format_lines(n, 80, [xyz_nm, &tail](int64_t i0, int64_t i1, std::string& s) {
    for (int64_t i = i0; i < i1; i++) {
      append_repr(s, xyz_nm[3 * i]);
      s += ',';
      append_repr(s, xyz_nm[3 * i + 1]);
      s += ',';
      append_repr(s, xyz_nm[3 * i + 2]);
      s += tail;
    }
  });
  if ((n > 0 && body.empty()) || !write_all(path, "wb", "x,y,z,density,mass\r\n", body))
    return od_fail_nohandle(OD_ERR_INVALID, std::string("cannot write ") + path);
  return OD_OK;
}

extern "C" od_status od_write_restart(const char* path, const double* pos_nm,
                                      const double* vel_nmps, int64_t n) {
  if (!path || (n > 0 && (!pos_nm || !vel_nmps)) || n < 0)
    return od_fail_nohandle(OD_ERR_INVALID, "od_write_restart: NULL path or arrays");
  const auto body = format_lines(n, 128, [pos_nm, vel_nmps](int64_t i0, int64_t i1,
                                                             std::string& s) {
    for (int64_t i = i0; i < i1; i++) {
      for (int c = 0; c < 3; c++) {
        append_repr(s, pos_nm[3 * i + c]);
        s += '\t';
      }
      for (int c = 0; c < 3; c++) {
        append_repr(s, vel_nmps[3 * i + c]);
        s += c < 2 ? '\t' : '\n';
      }
    }
  });
  if ((n > 0 && body.empty()) || !write_all(path, "wb", std::string(), body))
    return od_fail_nohandle(OD_ERR_INVALID, std::string("cannot write ") + path);
  return OD_OK;
}

extern "C" od_status od_read_restart(const char* path, int64_t n, double* pos_nm,
                                     double* vel_nmps) {
  if (!path || (n > 0 && (!pos_nm || !vel_nmps)) || n < 0)
    return od_fail_nohandle(OD_ERR_INVALID, "od_read_restart: NULL path or arrays");
  FILE* f = std::fopen(path, "rb");
  if (!f) return od_fail_nohandle(OD_ERR_INVALID, std::string("cannot open ") + path);
  std::string buf;
  char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.append(chunk, got);
  std::fclose(f);
  // the first n lines, six tab-separated numbers each (the reference's float() per field)
  const char* p = buf.c_str();
  const char* end = p + buf.size();
  for (int64_t i = 0; i < n; i++) {
    for (int c = 0; c < 6; c++) {
      char* q = nullptr;
      const double v = std::strtod(p, &q);
      if (q == p)
        return od_fail_nohandle(OD_ERR_INVALID, std::string(path) + ": line " +
                                                    std::to_string(i + 1) + " holds fewer than 6 numbers"
                                                    " (or the file fewer lines than ions)");
      (c < 3 ? pos_nm[3 * i + c] : vel_nmps[3 * i + c - 3]) = v;
      p = q;
      if (c < 5) {
        if (p < end && *p == '\t') p++;
      }
    }
    while (p < end && *p != '\n') p++;  // rest of the line
    if (p < end) p++;
  }
  return OD_OK;
}

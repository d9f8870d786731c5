// Host side of d2bi's output files: the .dat header (src/d2bi.f90:1429-1455) in Fortran
// F and I editing, and the PNG container of 16-bit greyscale levels (the file libpng
// writes for src/Lib_Greyscale.c:162-260: IHDR bit depth 16, colour type 0, no
// interlace; the pixel rows behind filter byte 0).  The image data is compressed as
// zlib "stored" blocks: any PNG decoder returns the same pixels as from d2bi's files.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/stem.h"

namespace {

// Fortran Fw.d: rounded to d decimals, right-justified in w characters, a '-' for
// negative values, at least one integer digit when it fits, a trailing '.' for d = 0,
// w asterisks when the number does not fit.
std::string fortran_f(double x, int w, int d) {
  std::string s;
  if (std::isnan(x)) {
    s = "NaN";
  } else if (std::isinf(x)) {
    s = x > 0 ? "Infinity" : "-Infinity";
  } else {
    char buf[400];
    std::snprintf(buf, sizeof buf, "%.*f", d, std::fabs(x));
    s = buf;
    if (d == 0) s += ".";
    if (std::signbit(x)) s = "-" + s;
    if ((int)s.size() > w) {  // the leading zero of |x| < 1 is optional
      const size_t z = s[0] == '-' ? 1 : 0;
      if (s.compare(z, 2, "0.") == 0) s.erase(z, 1);
    }
  }
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

std::string fortran_i(long long v, int w) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%lld", v);
  std::string s = buf;
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
  for (uint32_t n = 0; n < 256; ++n) {
    uint32_t c = n;
    for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    crc_table[n] = c;
  }
  crc_ready = true;
}

uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0xFFFFFFFFu) {
  for (size_t i = 0; i < n; ++i) crc = crc_table[(crc ^ p[i]) & 255] ^ (crc >> 8);
  return crc;
}

void put32(uint8_t* p, uint32_t v) {
  p[0] = (uint8_t)(v >> 24);
  p[1] = (uint8_t)(v >> 16);
  p[2] = (uint8_t)(v >> 8);
  p[3] = (uint8_t)v;
}

}  // namespace

extern "C" int st_format_dat_header(const st_dat_header* h, int32_t nx, int32_t ny, char* buf, int64_t cap,
                                    int64_t* len) {
  if (!h || !buf || cap < 1 || nx < 0 || ny < 0) return ST_ERR_ARG;
  if (h->nM < 0 || h->nM > 3) return ST_ERR_ARG;
  std::string t;
  char ver[33];
  std::memcpy(ver, h->version, 32);
  ver[32] = 0;
  t += "# d2bi v." + std::string(ver) + "\n";
  const int nv = h->miller4 ? 4 : 3;
  t += "# k       ";
  for (int i = 0; i < nv; ++i) t += fortran_f(h->k[i], 10, 3);
  t += "\n# g       ";
  for (int i = 0; i < nv; ++i) t += fortran_f(h->g[i], 10, 3);
  t += fortran_f(h->modg, 12, 5) + "\n";
  t += "# M       ";
  for (int i = 0; i < h->nM; ++i) t += fortran_i(h->M[i], 8);
  t += "\n# V (keV) " + fortran_f(h->V, 10, 0) + "\n";
  t += "# xi (A)  " + fortran_f(h->xi0, 12, 5) + fortran_f(h->xig, 12, 5) + "\n";
  if (h->has_ng) t += "# n_g     " + fortran_f(h->ng, 8, 3) + "\n";
  t += "# s_g (1/A)    " + fortran_f(h->sg, 12, 5) + "\n";
  t += "# img space (A)";
  for (int i = 0; i < 3; ++i) t += fortran_f(h->xmax[i], 12, 3);
  t += "\n# scale (A/px) " + fortran_f(h->aperpx, 12, 5) + "\n";
  t += "# rotation ";
  for (int i = 0; i < 9; ++i) t += fortran_f(h->rotation[i], 12, 6);
  t += "\n" + fortran_i(nx, 8) + fortran_i(ny, 8) + "\n";
  if ((int64_t)t.size() + 1 > cap) return ST_ERR_ARG;
  std::memcpy(buf, t.c_str(), t.size() + 1);
  if (len) *len = (int64_t)t.size();
  return ST_OK;
}

extern "C" int64_t st_dat_text_bytes(int64_t n) { return n <= 0 ? 0 : n * 12 + (n + 999) / 1000; }

extern "C" int64_t st_png16_bytes(int32_t nx, int32_t ny) {
  if (nx < 1 || ny < 1) return 0;
  const int64_t raw = (int64_t)ny * (1 + 2 * (int64_t)nx);
  const int64_t blocks = (raw + 65534) / 65535;
  const int64_t zlib = 2 + raw + 5 * blocks + 4;
  return 8 + (12 + 13) + (12 + zlib) + 12;
}

extern "C" int st_encode_png16(const uint16_t* levels, int32_t nx, int32_t ny, uint8_t* out, int64_t cap,
                               int64_t* len) {
  if (!levels || !out || nx < 1 || ny < 1) return ST_ERR_ARG;
  const int64_t total = st_png16_bytes(nx, ny);
  const int64_t raw = (int64_t)ny * (1 + 2 * (int64_t)nx);
  if (total > cap || 2 + raw + 5 * ((raw + 65534) / 65535) + 4 > 0x7FFFFFFFLL) return ST_ERR_ARG;
  if (!crc_ready) crc_init();
  uint8_t* p = out;
  static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  std::memcpy(p, sig, 8);
  p += 8;
  // IHDR
  put32(p, 13);
  std::memcpy(p + 4, "IHDR", 4);
  put32(p + 8, (uint32_t)nx);
  put32(p + 12, (uint32_t)ny);
  p[16] = 16;  // bit depth
  p[17] = 0;   // greyscale
  p[18] = 0;   // deflate
  p[19] = 0;   // adaptive filtering (filter byte per row)
  p[20] = 0;   // no interlace
  put32(p + 21, crc32(p + 4, 17) ^ 0xFFFFFFFFu);
  p += 25;
  // IDAT: zlib header, stored blocks of the scanlines, Adler-32
  const int64_t zlen = 2 + raw + 5 * ((raw + 65534) / 65535) + 4;
  put32(p, (uint32_t)zlen);
  std::memcpy(p + 4, "IDAT", 4);
  uint8_t* z = p + 8;
  z[0] = 0x78;
  z[1] = 0x01;
  uint8_t* q = z + 2;
  uint32_t s1 = 1, s2 = 0;
  int64_t left = raw, row = 0, col = -1;  // col -1: the row's filter byte
  while (left > 0) {
    const uint32_t nb = (uint32_t)(left > 65535 ? 65535 : left);
    q[0] = left <= 65535 ? 1 : 0;  // final block flag, stored type
    q[1] = (uint8_t)(nb & 255);
    q[2] = (uint8_t)(nb >> 8);
    q[3] = (uint8_t)(~nb & 255);
    q[4] = (uint8_t)((~nb >> 8) & 255);
    q += 5;
    for (uint32_t i = 0; i < nb; ++i) {
      uint8_t b;
      if (col < 0) {
        b = 0;
      } else {
        const uint16_t lv = levels[row * nx + col / 2];
        b = (col & 1) ? (uint8_t)(lv & 255) : (uint8_t)(lv >> 8);
      }
      if (++col == 2 * (int64_t)nx) {
        col = -1;
        ++row;
      }
      *q++ = b;
      s1 += b;
      if (s1 >= 65521) s1 -= 65521;
      s2 += s1;
      if (s2 >= 65521) s2 -= 65521;
    }
    left -= nb;
  }
  put32(q, (s2 << 16) | s1);
  q += 4;
  put32(q, crc32(p + 4, (size_t)(4 + zlen)) ^ 0xFFFFFFFFu);
  p = q + 4;
  // IEND
  put32(p, 0);
  std::memcpy(p + 4, "IEND", 4);
  put32(p + 8, crc32(p + 4, 4) ^ 0xFFFFFFFFu);
  p += 12;
  if (len) *len = (int64_t)(p - out);
  return ST_OK;
}

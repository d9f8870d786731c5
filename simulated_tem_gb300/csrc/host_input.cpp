// The headers of the input files, read as the reference reads them.
//
// LAMMPS data files
// (src/Lib_XYZFiles.f90:628-716, readHeader_lammps, and :1092-1101, the box lines of
// input_lammps): up to 1000 lines, each left-adjusted; a line containing "atoms" gives the
// atom count (its first integer), one containing "atom types" the type count, lines
// containing "xlo", "ylo", "zlo" the box (their first two numbers); "Masses" is followed
// by a blank line and one line per type; "Atoms" by one more line, after which the atom
// lines start.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/stem.h"
#include "parse_number.cuh"

namespace {

bool first_integer(const std::string& s, long long& v) {
  const char* p = s.c_str();
  while (*p == ' ' || *p == '\t') ++p;
  char* e = nullptr;
  errno = 0;
  v = std::strtoll(p, &e, 10);
  return e != p && errno == 0;
}

bool first_two_reals(const std::string& s, double& a, double& b) {
  const char* p = s.c_str();
  char* e = nullptr;
  a = std::strtod(p, &e);
  if (e == p) return false;
  p = e;
  b = std::strtod(p, &e);
  return e != p;
}

}  // namespace

extern "C" int st_lammps_header(const char* path, st_lammps_info* info) {
  if (!path || !info) return ST_ERR_ARG;
  std::memset(info, 0, sizeof *info);
  FILE* f = std::fopen(path, "rb");
  if (!f) return ST_ERR_ARG;
  std::string line;
  long long offset = 0, n_atoms = -1, n_types = -1;
  bool atoms_seen = false;
  auto get = [&](std::string& out) -> bool {
    out.clear();
    int c;
    bool any = false;
    while ((c = std::fgetc(f)) != EOF) {
      any = true;
      ++offset;
      if (c == '\n') break;
      out.push_back((char)c);
    }
    if (!out.empty() && out.back() == '\r') out.pop_back();
    return any;
  };
  for (int ii = 0; ii < 1000 && get(line); ++ii) {
    const size_t b = line.find_first_not_of(" \t");
    const std::string d = b == std::string::npos ? std::string() : line.substr(b);
    if (d.find("atoms") != std::string::npos && !first_integer(d, n_atoms)) break;
    if (d.find("atom types") != std::string::npos && !first_integer(d, n_types)) break;
    const char* axes[3] = {"xlo", "ylo", "zlo"};
    for (int a = 0; a < 3; ++a)
      if (d.find(axes[a]) != std::string::npos && !first_two_reals(d, info->lo[a], info->hi[a])) {
        std::fclose(f);
        return ST_ERR_ARG;
      }
    if (d.compare(0, 6, "Masses") == 0) {
      get(line);  // blank
      for (long long k = 0; k < n_types; ++k) get(line);
    }
    if (d.compare(0, 5, "Atoms") == 0) {
      get(line);  // blank
      atoms_seen = true;
      break;
    }
  }
  std::fseek(f, 0, SEEK_END);
  const long long size = std::ftell(f);
  std::fclose(f);
  if (!atoms_seen || n_atoms < 0) return ST_ERR_ARG;
  info->n_atoms = n_atoms;
  info->n_types = (int32_t)(n_types < 0 ? 0 : n_types);
  info->data_offset = offset;
  info->file_bytes = size;
  return ST_OK;
}

extern "C" int st_parse_real(const char* text, int64_t len, double* out, int32_t* used) {
  if (!text || !out || len < 0) return ST_ERR_ARG;
  int u = 0;
  if (!stem::pn::parse_real(text, text + len, *out, u)) return ST_ERR_ARG;
  if (used) *used = u;
  return ST_OK;
}


// ---- the (extended) .xyz header (src/Lib_XYZFiles.f90:507-626 readHeader, 905-1058
// getSupercell0) with the string tools of src/NBAX_StringTokenizers.f90 -------------------

namespace {

// gfortran's real ** integer (libgcc __powidf2): square-and-multiply, then the reciprocal
// for a negative exponent
double powi(double x, int m) {
  unsigned n = m < 0 ? 0u - (unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1 / y : y;
}

bool number_char(char c) {
  return (c >= '0' && c <= '9') || c == '.' || c == '+' || c == '-' || c == 'e' || c == 'E' || c == 'd' ||
         c == 'D';
}

// Fortran substring s(a:b), 1-based, empty when b < a
std::string sub(const std::string& s, int a, int b) {
  if (b < a || a < 1) return std::string();
  return s.substr((size_t)a - 1, (size_t)(b - a + 1));
}

// ParseReal (NBAX_StringTokenizers.f90:303-420): the first run of number characters
// after leading blanks, split into aaaa.bbbb e cccc and evaluated as
// (aaaa + sum bbbb_k 0.1^k) * 10 ** cccc.  Not correctly rounded; kept for its bits.
bool fortran_parse_real(const std::string& text, double& r) {
  std::string str;
  bool in_num = false;
  for (char c : text) {
    if (!in_num && c == ' ') continue;
    if (!number_char(c)) break;
    in_num = true;
    str.push_back(c);
    if (str.size() == 64) break;
  }
  if (str.empty()) return false;
  for (char& c : str)
    if (c == 'd' || c == 'D' || c == 'E') c = 'e';
  const int n = (int)str.size();
  const size_t pd = str.find('.'), pe = str.find('e');
  const int ii = pd == std::string::npos ? 0 : (int)pd + 1, jj = pe == std::string::npos ? 0 : (int)pe + 1;
  std::string a = "0", b = "0", c = "0";
  if (ii == 1) {
    if (jj > 1) {
      b = sub(str, 2, jj - 1);
      c = sub(str, jj + 1, n);
    } else {
      b = sub(str, 2, n);
    }
  } else if (ii > 1) {
    a = sub(str, 1, ii - 1);
    if (jj > 1) {
      b = sub(str, ii + 1, jj - 1);
      c = sub(str, jj + 1, n);
    } else {
      b = sub(str, ii + 1, n);
    }
  } else {
    if (jj > 1) {
      a = sub(str, 1, jj - 1);
      c = sub(str, jj + 1, n);
    } else {
      a = sub(str, 1, n);
    }
  }
  for (std::string* s : {&a, &b, &c})
    if (s->size() > 32) s->resize(32);  // character(len=32)
  double xa = 0.0;
  for (char ch : a) {
    const int d = ch - '0';
    if (d >= 0 && d <= 9) xa = xa * 10 + d;
  }
  int ic = 0;
  for (char ch : c) {
    const int d = ch - '0';
    if (d >= 0 && d <= 9) ic = ic * 10 + d;
  }
  if (!c.empty() && c[0] == '-') ic = -ic;
  double xx = 1.0, xb = 0.0;
  for (char ch : b) {
    xx = xx * 0.1;
    xb = xb + xx * (ch - '0');
  }
  double rr = (xa + xb) * powi(10.0, ic);
  if (!a.empty() && a[0] == '-') rr = -rr;
  if (std::fabs(rr) == 0) rr = 0;
  r = rr;
  return true;
}

size_t len_trim(const std::string& s) {
  size_t k = s.size();
  while (k > 0 && s[k - 1] == ' ') --k;
  return k;
}

// StringTokenizer (NBAX_StringTokenizers.f90:111-210): nextToken on a blank-padded buffer
struct Tokenizer {
  std::string buf, delims;
  size_t max_tok;
  Tokenizer(const std::string& s, const std::string& d, size_t max_tok = 256) : delims(d), max_tok(max_tok) {
    buf = s.substr(0, std::min(len_trim(s), (size_t)1024));  // STRINGTOKENIZER_MAX_STRING
  }
  bool more() const { return len_trim(buf) > 0; }
  std::string next() {
    for (;;) {
      const size_t kk = len_trim(buf);
      if (kk == 0) return std::string();
      size_t jj = kk + 1;
      for (size_t p = 0; p < kk; ++p)
        if (delims.find(buf[p]) != std::string::npos) {
          jj = p + 1;
          break;
        }
      const size_t i = std::min(max_tok, jj - 1);
      std::string t = buf.substr(0, i);
      std::string rest = jj < kk ? buf.substr(jj, kk - jj) : std::string();
      buf = rest + std::string(jj, ' ');
      buf.resize(kk);
      if (i > 0) return t;
    }
  }
  std::string remaining() const { return buf.substr(0, len_trim(buf)); }
};

// ParseRealArray1 (:273-300): the numbers among the tokens (" ,;" tab CR NUL), at most cap
std::vector<double> parse_real_array(const std::string& s, size_t cap) {
  Tokenizer st(s.substr(0, len_trim(s)), std::string(" ,;\t\r\0", 6), 32);
  std::vector<double> out;
  for (int k = 0; k < 1000000 && st.more(); ++k) {
    double r;
    if (fortran_parse_real(st.next(), r)) {
      out.push_back(r);
      if (out.size() == cap) break;
    }
  }
  return out;
}

// parseInt (:534-564): the first run of digits, negative if a '-' came before it
bool fortran_parse_int(const std::string& s, long long& v) {
  long long ii = 0;
  bool started = false, neg = false;
  for (size_t k = 0; k < len_trim(s); ++k) {
    const char c = s[k];
    if (c >= '0' && c <= '9') {
      ii = ii * 10 + (c - '0');
      started = true;
    } else if (started) {
      break;
    } else if (c == '-') {
      neg = true;
    }
  }
  if (started) v = neg ? -ii : ii;
  return started;
}

// a list-directed integer read of one record (input0's `read(uu,*) nn`)
bool list_directed_int(const std::string& s, long long& v) {
  size_t p = 0;
  while (p < s.size() && (s[p] == ' ' || s[p] == '\t')) ++p;
  size_t q = p;
  while (q < s.size() && s[q] != ' ' && s[q] != '\t' && s[q] != ',' && s[q] != '/' && s[q] != '\r') ++q;
  const std::string tok = s.substr(p, q - p);
  if (tok.empty()) return false;
  size_t k = 0;
  if (tok[0] == '+' || tok[0] == '-') k = 1;
  if (k == tok.size()) return false;
  for (size_t m = k; m < tok.size(); ++m)
    if (tok[m] < '0' || tok[m] > '9') return false;
  v = std::strtoll(tok.c_str(), nullptr, 10);
  return true;
}

std::string adjustl(const std::string& s) {
  const size_t b = s.find_first_not_of(' ');
  return b == std::string::npos ? std::string() : s.substr(b);
}

struct LineReader {
  FILE* f;
  long long offset = 0;
  bool get(std::string& out) {  // one record, without its newline (and a trailing CR)
    out.clear();
    int c;
    bool any = false;
    while ((c = std::fgetc(f)) != EOF) {
      any = true;
      ++offset;
      if (c == '\n') break;
      out.push_back((char)c);
    }
    if (!out.empty() && out.back() == '\r') out.pop_back();
    return any;
  }
};

std::string fixed(const std::string& s, size_t n) { return s.size() > n ? s.substr(0, n) : s; }

}  // namespace

extern "C" int st_fortran_parse_real(const char* text, int64_t len, double* out, int32_t* ok) {
  if (!text || !out || !ok || len < 0) return ST_ERR_ARG;
  double r = 0.0;
  *ok = fortran_parse_real(std::string(text, (size_t)len), r) ? 1 : 0;
  if (*ok) *out = r;
  return ST_OK;
}

extern "C" int st_xyz_header(const char* path, st_xyz_info* info) {
  if (!path || !info) return ST_ERR_ARG;
  std::memset(info, 0, sizeof *info);
  for (int i = 0; i < 9; ++i) info->a_super[i] = (i % 4 == 0) ? 1.0 : 0.0;
  info->repeats[0] = info->repeats[1] = info->repeats[2] = 1;
  info->n_read = -1;
  FILE* f = std::fopen(path, "rb");
  if (!f) return ST_ERR_ARG;
  LineReader rd{f};
  std::string line;
  if (!rd.get(line)) {
    std::fclose(f);
    return ST_ERR_ARG;
  }
  if (fixed(adjustl(fixed(line, 256)), 6) == "LAMMPS") {
    std::fclose(f);
    info->lammps = 1;
    return ST_OK;
  }
  std::rewind(f);
  rd.offset = 0;
  std::vector<std::string> header;
  std::string count;
  bool found = false;
  for (int ii = 0; ii < 1000 && rd.get(line); ++ii) {
    const std::string d = adjustl(fixed(line, 256));
    const char letter = d.empty() ? ' ' : d[0];
    if (letter == '#' || letter == '%' || letter == '!') {
      header.push_back(fixed(line, 256));
      continue;
    }
    count = d;
    found = true;
    break;
  }
  std::string desc, first;
  const bool ok_desc = found && rd.get(desc);
  const long long data_offset = rd.offset;
  const bool ok_first = ok_desc && rd.get(first);
  std::fseek(f, 0, SEEK_END);
  info->file_bytes = std::ftell(f);
  if (!ok_first) {
    std::fclose(f);
    return ST_ERR_ARG;
  }
  Tokenizer ct(count, " ");
  long long n_atoms = 0;
  if (!fortran_parse_int(ct.next(), n_atoms)) {
    std::fclose(f);
    return ST_ERR_ARG;
  }
  long long nn = 0;
  info->n_read = list_directed_int(count, nn) ? nn : -1;
  Tokenizer ft(fixed(first, 4096), " ");
  ft.next();  // the species
  const std::vector<double> dat = parse_real_array(ft.remaining(), 1000);
  if (dat.size() < 3) {
    std::fclose(f);
    return ST_ERR_ARG;
  }
  info->n_atoms = n_atoms;
  info->n_columns = (int32_t)dat.size();
  info->n_header_lines = (int32_t)header.size();
  info->data_offset = data_offset;
  desc = fixed(desc, 256);
  std::memcpy(info->column_description, desc.data(), desc.size());
  // getSupercell0
  double* a = info->a_super;
  const std::string dt = desc.substr(0, len_trim(desc));
  size_t p;
  if ((p = dt.find("Lattice=\"")) != std::string::npos) {
    info->supercell_kind = ST_XYZ_SUPERCELL_LATTICE;
    const std::vector<double> v = parse_real_array(desc.substr(p + 9), 9);
    if (v.size() == 3) {
      a[0] = v[0], a[4] = v[1], a[8] = v[2];
      info->supercell_ok = 1;
    } else if (v.size() == 9) {
      for (int i = 0; i < 9; ++i) a[i] = v[i];
      info->supercell_ok = 1;
    }
  } else if ((p = dt.find("boxsize")) != std::string::npos) {
    info->supercell_kind = ST_XYZ_SUPERCELL_BOXSIZE;
    const std::vector<double> v = parse_real_array(desc.substr(p + 8), 9);
    if (v.size() >= 3) {
      a[0] = v[0], a[4] = v[1], a[8] = v[2];
      info->supercell_ok = 1;
    }
  } else {
    std::rewind(f);
    rd.offset = 0;
    for (size_t ii = 0; ii < header.size(); ++ii) {
      std::string d;
      rd.get(d);
      d = fixed(d, 256);
      const size_t j1 = d.find("supercell"), j2 = d.find("super cell");
      const long long jj = std::max(j1 == std::string::npos ? 0LL : (long long)j1 + 1,
                                    j2 == std::string::npos ? 0LL : (long long)j2 + 1);
      if (jj == 0) continue;
      info->supercell_kind = ST_XYZ_SUPERCELL_HEADER;
      const std::vector<double> rep = parse_real_array(d.size() >= (size_t)jj + 9 ? d.substr(jj + 8) : "", 9);
      double xm[3] = {1.0, 1.0, 1.0};
      if (rep.size() == 3) xm[0] = rep[0], xm[1] = rep[1], xm[2] = rep[2];
      int rp[3];
      for (int k = 0; k < 3; ++k) rp[k] = (int)std::lround(xm[k]);
      for (int kk = 0; kk < 3; ++kk) {
        std::string v3;
        rd.get(v3);
        v3 = fixed(v3, 256);
        const std::vector<double> v = parse_real_array(v3.size() > 2 ? v3.substr(2) : "", 9);
        if (v.size() == 3) {
          for (int j = 0; j < 3; ++j) a[kk + 3 * j] = v[j];  // a(kk, 1:3): a row
          if (kk == 2) {
            info->supercell_ok = 1;
            break;
          }
        } else if (v.size() == 9) {
          for (int i = 0; i < 9; ++i) a[i] = v[i];
          info->supercell_ok = 1;
          break;
        } else {
          break;
        }
      }
      if (info->supercell_ok)
        for (int j = 0; j < 3; ++j) {
          for (int i = 0; i < 3; ++i) a[i + 3 * j] = a[i + 3 * j] * rp[j];
          info->repeats[j] = rp[j];
        }
      break;
    }
  }
  std::fclose(f);
  return ST_OK;
}

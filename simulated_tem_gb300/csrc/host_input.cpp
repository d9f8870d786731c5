// The header of a LAMMPS data file, read as the reference reads it
// (src/Lib_XYZFiles.f90:628-716, readHeader_lammps, and :1092-1101, the box lines of
// input_lammps): up to 1000 lines, each left-adjusted; a line containing "atoms" gives the
// atom count (its first integer), one containing "atom types" the type count, lines
// containing "xlo", "ylo", "zlo" the box (their first two numbers); "Masses" is followed
// by a blank line and one line per type; "Atoms" by one more line, after which the atom
// lines start.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

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


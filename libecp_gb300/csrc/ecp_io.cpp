// ecp_io.cpp -- readers for the text inputs of the reference's example
// program (example/ex1.c:12-123): an xyz geometry, an ECP file and a basis
// file, into one ecpgb_system.
//
//   xyz    atom count; a comment line; per atom "symbol x y z" (the
//          coordinates are used as given, bohr, as the example does).
//   basis  per atom "index nShells"; per shell "l K"; K lines "index a d"
//          (exponent, coefficient), example/ex1.c:12-57.
//   ECP    per atom "index nCore nShells"; per shell "l K"; K term lines.
//          The example's reader takes "index a d n" (example/ex1.c:114), but
//          its own ECP file writes three numbers per term -- coefficient,
//          exponent, r power (example/test_c.ecp:3) -- which that reader
//          misparses (it takes the integer part of the coefficient as the
//          index).  Here a four-number line is read as "index a d n" and a
//          three-number line as "d a n".
// Every atom has an entry in both files (possibly with zero shells), as the
// example's readers require.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "ecp_host.h"
#include "libecp_gb300.h"

struct ecpgb_loaded {
  ecpgb_system sys;
  std::vector<double> geometry, nECP, dECP, aECP, dBS, aBS;
  std::vector<int> shellsECP, KECP, lECP, shellsBS, lBS, KBS;
  std::vector<std::string> symbols;
};

namespace {

// Reads the non-empty lines of a file.
bool read_lines(const char *path, std::vector<std::string> &out) {
  std::ifstream f(path);
  if (!f) {
    ecpgb::set_error("cannot open %s", path ? path : "(null)");
    return false;
  }
  std::string line;
  while (std::getline(f, line)) {
    bool blank = true;
    for (char ch : line)
      if (!std::isspace((unsigned char)ch)) blank = false;
    if (!blank) out.push_back(line);
  }
  return true;
}

std::vector<std::string> fields(const std::string &line) {
  std::istringstream is(line);
  std::vector<std::string> out;
  std::string w;
  while (is >> w) out.push_back(w);
  return out;
}

bool to_int(const std::string &w, int &v) {
  char *end = nullptr;
  long x = std::strtol(w.c_str(), &end, 10);
  if (end == w.c_str() || *end) return false;
  v = (int)x;
  return true;
}

bool to_double(const std::string &w, double &v) {
  char *end = nullptr;
  v = std::strtod(w.c_str(), &end);
  return end != w.c_str() && !*end;
}

struct Cursor {
  const std::vector<std::string> &lines;
  const char *path;
  size_t i = 0;
  bool next(std::vector<std::string> &f, size_t want_min, size_t want_max) {
    if (i >= lines.size()) {
      ecpgb::set_error("%s: unexpected end of file", path);
      return false;
    }
    f = fields(lines[i++]);
    if (f.size() < want_min || f.size() > want_max) {
      ecpgb::set_error("%s line %zu: expected %zu to %zu fields, found %zu", path, i, want_min, want_max,
                       f.size());
      return false;
    }
    return true;
  }
};

bool load_xyz(const char *path, ecpgb_loaded &L) {
  std::ifstream fin(path);
  if (!fin) {
    ecpgb::set_error("cannot open %s", path ? path : "(null)");
    return false;
  }
  std::vector<std::string> lines;  // every line: the comment line may be blank
  for (std::string line; std::getline(fin, line);) lines.push_back(line);
  int n = 0;
  auto head = lines.empty() ? std::vector<std::string>() : fields(lines[0]);
  if (head.size() != 1 || !to_int(head[0], n) || n < 1) {
    ecpgb::set_error("%s: first line is not a positive atom count", path);
    return false;
  }
  if (lines.size() < (size_t)n + 2) {
    ecpgb::set_error("%s: %d atoms announced, %zu atom lines follow", path, n,
                     lines.size() > 2 ? lines.size() - 2 : (size_t)0);
    return false;
  }
  for (size_t k = 2; k < 2 + (size_t)n; k++) {
    auto f = fields(lines[k]);
    double x, y, z;
    if (f.size() < 4 || !to_double(f[1], x) || !to_double(f[2], y) || !to_double(f[3], z)) {
      ecpgb::set_error("%s line %zu: expected \"symbol x y z\"", path, k + 1);
      return false;
    }
    L.symbols.push_back(f[0]);
    L.geometry.insert(L.geometry.end(), {x, y, z});
  }
  return true;
}

bool load_basis(const char *path, int nAtoms, ecpgb_loaded &L) {
  std::vector<std::string> lines;
  if (!read_lines(path, lines)) return false;
  Cursor c{lines, path};
  std::vector<std::string> f;
  for (int a = 0; a < nAtoms; a++) {
    int idx, ns;
    if (!c.next(f, 2, 2)) return false;
    if (!to_int(f[0], idx) || !to_int(f[1], ns) || ns < 0) {
      ecpgb::set_error("%s line %zu: expected \"index nShells\"", path, c.i);
      return false;
    }
    L.shellsBS.push_back(ns);
    for (int s = 0; s < ns; s++) {
      int l, K;
      if (!c.next(f, 2, 2)) return false;
      if (!to_int(f[0], l) || !to_int(f[1], K) || K < 1) {
        ecpgb::set_error("%s line %zu: expected \"l K\"", path, c.i);
        return false;
      }
      L.lBS.push_back(l);
      L.KBS.push_back(K);
      for (int k = 0; k < K; k++) {
        double ea, ed;
        if (!c.next(f, 3, 3)) return false;
        if (!to_int(f[0], idx) || !to_double(f[1], ea) || !to_double(f[2], ed)) {
          ecpgb::set_error("%s line %zu: expected \"index a d\"", path, c.i);
          return false;
        }
        L.aBS.push_back(ea);
        L.dBS.push_back(ed);
      }
    }
  }
  return true;
}

bool load_ecp(const char *path, int nAtoms, ecpgb_loaded &L) {
  std::vector<std::string> lines;
  if (!read_lines(path, lines)) return false;
  Cursor c{lines, path};
  std::vector<std::string> f;
  for (int a = 0; a < nAtoms; a++) {
    int idx, core, ns;
    if (!c.next(f, 3, 3)) return false;
    if (!to_int(f[0], idx) || !to_int(f[1], core) || !to_int(f[2], ns) || ns < 0) {
      ecpgb::set_error("%s line %zu: expected \"index nCore nShells\"", path, c.i);
      return false;
    }
    L.shellsECP.push_back(ns);
    for (int s = 0; s < ns; s++) {
      int l, K;
      if (!c.next(f, 2, 2)) return false;
      if (!to_int(f[0], l) || !to_int(f[1], K) || K < 0) {
        ecpgb::set_error("%s line %zu: expected \"l K\"", path, c.i);
        return false;
      }
      L.lECP.push_back(l);
      L.KECP.push_back(K);
      for (int k = 0; k < K; k++) {
        double ea, ed, en;
        if (!c.next(f, 3, 4)) return false;
        bool ok = f.size() == 4 ? to_int(f[0], idx) && to_double(f[1], ea) && to_double(f[2], ed) &&
                                      to_double(f[3], en)
                                : to_double(f[0], ed) && to_double(f[1], ea) && to_double(f[2], en);
        if (!ok) {
          ecpgb::set_error("%s line %zu: expected \"index a d n\" or \"d a n\"", path, c.i);
          return false;
        }
        L.aECP.push_back(ea);
        L.dECP.push_back(ed);
        L.nECP.push_back(en);
      }
    }
  }
  return true;
}

}  // namespace

extern "C" {

ecpgb_loaded *ecpgb_load_system(const char *xyzPath, const char *ecpPath, const char *basisPath) {
  auto *L = new ecpgb_loaded();
  if (!load_xyz(xyzPath, *L)) {
    delete L;
    return nullptr;
  }
  const int n = (int)L->symbols.size();
  if (!load_ecp(ecpPath, n, *L) || !load_basis(basisPath, n, *L)) {
    delete L;
    return nullptr;
  }
  // give every vector storage, so that an empty one still has a valid pointer
  for (auto *v : {&L->nECP, &L->dECP, &L->aECP, &L->dBS, &L->aBS}) v->reserve(1);
  for (auto *v : {&L->KECP, &L->lECP, &L->lBS, &L->KBS}) v->reserve(1);
  L->sys = {n, L->geometry.data(), L->shellsECP.data(), L->KECP.data(), L->lECP.data(), L->nECP.data(),
            L->dECP.data(), L->aECP.data(), L->shellsBS.data(), L->lBS.data(), L->KBS.data(),
            L->dBS.data(), L->aBS.data(), 1024, 1.0E-12, 1.0E-14, 0};
  return L;
}

const ecpgb_system *ecpgb_loaded_system(const ecpgb_loaded *L) { return L ? &L->sys : nullptr; }

const char *ecpgb_loaded_symbol(const ecpgb_loaded *L, int atom) {
  return L && atom >= 0 && atom < (int)L->symbols.size() ? L->symbols[atom].c_str() : nullptr;
}

void ecpgb_loaded_free(ecpgb_loaded *L) { delete L; }

}  // extern "C"

// basis_lib.cu -- the basis library text parsed once per context, and the
// reference's buildBasis (src/myQC/basis.f90:23-226) in C++: the flat bas /
// set / basinfo / setinfo arrays of a molecule from its atoms, so that a batch
// of thousands of molecules is set up without a host-language parse of the
// library per molecule (mq_batch_add_atoms).
#include <cmath>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"

namespace mq {

static const char *const ELEMENT_NAME[] = {"H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne"};

// tokens of every line; the first token of a line compares on its first 8
// characters, as the reference's READ of a CHARACTER(LEN=8) does
int basis_library_set(mq_ctx *c, const char *text, const char *key) {
  c->basis_rows.clear();
  std::istringstream in(text ? text : "");
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::vector<std::string> tok;
    std::string w;
    while (ls >> w) tok.push_back(w);
    c->basis_rows.push_back(tok);
  }
  c->basis_key = -1;
  for (size_t r = 0; r < c->basis_rows.size(); ++r)
    if (!c->basis_rows[r].empty() && c->basis_rows[r][0].substr(0, 8) == key) {
      c->basis_key = (int)r;
      break;
    }
  if (c->basis_key < 0 || c->basis_key + 1 >= (int)c->basis_rows.size() || c->basis_rows[c->basis_key + 1].size() < 5)
    return set_err(c, MQ_EINVAL, std::string("basis library: no ") + key + " section");
  return MQ_OK;
}

static bool to_int(const std::string &t, int &v) {
  char *end = nullptr;
  const long x = std::strtol(t.c_str(), &end, 10);
  if (!end || *end) return false;
  v = (int)x;
  return true;
}

static bool to_real(std::string t, double &v) {
  for (char &ch : t)
    if (ch == 'D' || ch == 'd') ch = 'E';
  char *end = nullptr;
  v = std::strtod(t.c_str(), &end);
  return end && !*end;
}

int basis_build(mq_ctx *c, int nnuc, const int *Z, std::vector<double> &bas, std::vector<double> &set,
                std::vector<int> &basinfo, std::vector<int> &setinfo) {
  const auto &rows = c->basis_rows;
  const int p = c->basis_key;
  if (p < 0) return set_err(c, MQ_ESTATE, "no basis library (mq_basis_library)");
  int hdr[5];
  for (int k = 0; k < 5; ++k)
    if (!to_int(rows[p + 1][k], hdr[k])) return set_err(c, MQ_EINVAL, "basis library: bad header");
  const int Omax = hdr[2], almax = hdr[3], OpS = hdr[4], setl = 3 + OpS;
  bas.assign((size_t)nnuc * almax * OpS, 0.0);
  set.assign((size_t)nnuc * almax, 0.0);
  basinfo.assign(2 + 5 * (size_t)Omax * nnuc, 0);
  setinfo.assign(2 + (size_t)nnuc * almax * setl, 0);
  int setnum = 0, orbnum = 0;
  for (int i = 0; i < nnuc; ++i) {
    if (Z[i] < 1 || Z[i] > 10) return set_err(c, MQ_EINVAL, "basis library: element out of range");
    size_t q = p;
    while (q < rows.size() && (rows[q].empty() || rows[q][0].substr(0, 8) != ELEMENT_NAME[Z[i] - 1])) ++q;
    if (q + 1 >= rows.size() || rows[q + 1].size() < 3)
      return set_err(c, MQ_EINVAL, std::string("basis library: no ") + ELEMENT_NAME[Z[i] - 1]);
    int sec, orb, nset;
    if (!to_int(rows[q + 1][0], sec) || !to_int(rows[q + 1][1], orb) || !to_int(rows[q + 1][2], nset))
      return set_err(c, MQ_EINVAL, "basis library: bad atom header");
    q += 2;
    basinfo[0] = OpS;
    basinfo[1] += orb;
    setinfo[0] += nset;
    setinfo[1] = setl;
    for (int s = 0; s < sec; ++s) {
      while (q < rows.size() && rows[q].size() < 5) ++q;
      if (q >= rows.size()) return set_err(c, MQ_EINVAL, "basis library: truncated section");
      int func, coef, pri, ang, ori;
      if (!to_int(rows[q][0], func) || !to_int(rows[q][1], coef) || !to_int(rows[q][2], pri) ||
          !to_int(rows[q][3], ang) || !to_int(rows[q][4], ori))
        return set_err(c, MQ_EINVAL, "basis library: bad section header");
      ++q;
      for (int k = 0; k < func; ++k, ++q) {
        if (q >= rows.size() || (int)rows[q].size() < coef + 1) return set_err(c, MQ_EINVAL, "basis library: short line");
        std::vector<double> v(coef + 1);
        for (int cc = 0; cc <= coef; ++cc)
          if (!to_real(rows[q][cc], v[cc])) return set_err(c, MQ_EINVAL, "basis library: bad number");
        const double tt = v[coef];
        const int sid = setnum + (int)std::floor(std::fabs(tt) + 0.5) * (tt >= 0 ? 1 : -1);
        if (sid < 0 || sid >= nnuc * almax) return set_err(c, MQ_EINVAL, "basis library: set index out of range");
        set[sid] = v[coef - 1];
        const size_t base = 1 + (size_t)sid * setl;
        int kk = setinfo[base + 1];
        setinfo[base + 3] = i;
        if (ori == -1) {
          setinfo[base + 4 + kk] = orbnum;
          bas[kk + (size_t)sid * OpS] = v[0];
          ++kk;
        } else if (ori == 2) {
          for (int m = 0; m < 3; ++m) {
            setinfo[base + 4 + kk] = orbnum + m;
            bas[kk + (size_t)sid * OpS] = v[0];
            ++kk;
          }
          setinfo[base + 2] = std::max(setinfo[base + 2], 1);
        } else {
          return set_err(c, MQ_EINVAL, "basis library: only s and p sections are supported");
        }
        setinfo[base + 1] = kk;
      }
      if (ori == -1) {
        int *bi = &basinfo[2 + 5 * (size_t)orbnum];
        bi[0] = pri, bi[1] = ang, bi[2] = ori, bi[3] = func, bi[4] = i;
        orbnum += 1;
      } else {
        for (int m = 0; m < 3; ++m) {
          int *bi = &basinfo[2 + 5 * (size_t)(orbnum + m)];
          bi[0] = pri, bi[1] = ang, bi[2] = m, bi[3] = func, bi[4] = i;
        }
        orbnum += 3;
      }
    }
    setnum = setinfo[0];
  }
  return MQ_OK;
}

}  // namespace mq

using namespace mq;

extern "C" {

int mq_basis_library(mq_ctx *c, const char *text) {
  if (!c || !text) return MQ_EINVAL;
  return basis_library_set(c, text, "STO-3G");
}

int mq_basis_build(mq_ctx *c, int nnuc, const int *Z, double *bas, double *set, int *basinfo, int *setinfo,
                   int sizes[4]) {
  if (!c || nnuc <= 0 || !Z || !sizes) return c ? set_err(c, MQ_EINVAL, "basis build: bad arguments") : MQ_EINVAL;
  std::vector<double> b, s;
  std::vector<int> bi, si;
  MQ_TRY(basis_build(c, nnuc, Z, b, s, bi, si));
  const int need[4] = {(int)b.size(), (int)s.size(), (int)bi.size(), (int)si.size()};
  const bool fit = bas && set && basinfo && setinfo && sizes[0] >= need[0] && sizes[1] >= need[1] &&
                   sizes[2] >= need[2] && sizes[3] >= need[3];
  for (int k = 0; k < 4; ++k) sizes[k] = need[k];
  if (!fit) return MQ_OK;  // sizes only
  std::memcpy(bas, b.data(), b.size() * sizeof(double));
  std::memcpy(set, s.data(), s.size() * sizeof(double));
  std::memcpy(basinfo, bi.data(), bi.size() * sizeof(int));
  std::memcpy(setinfo, si.data(), si.size() * sizeof(int));
  return MQ_OK;
}

int mq_batch_add_atoms(mq_ctx *c, int nnuc, const int *Z, const double *xyz, int nocc) {
  if (!c || nnuc <= 0 || !Z || !xyz) return c ? set_err(c, MQ_EINVAL, "batch molecule: bad arguments") : MQ_EINVAL;
  std::vector<double> b, s;
  std::vector<int> bi, si;
  MQ_TRY(basis_build(c, nnuc, Z, b, s, bi, si));
  return batch_add(c, nnuc, Z, xyz, b.data(), s.data(), bi.data(), si.data(), nocc);
}

}  // extern "C"

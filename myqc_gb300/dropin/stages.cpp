// stages.cpp -- drop-in replacements of the reference's stage executables
// parse, int1e, int2e, scf, ao2mo and mp2 (and the property stages int1p, cphf and
// props), computing through libmyqc.
//
// One binary; the stage is the name it is invoked by (symlinks parse, int1e, int2e,
// scf, ao2mo, mp2) or its first argument.  Like the reference's programs they
// work in the current directory on the reference's files (formats of
// src/parser/parser.f90, src/myQC/env.f90, basis.f90, integrals/int1e.f90, int2e.f90, scf/scf.f90,
// ao2mo/ao2mo.f90, mp2/mp2.f90):
//   ZMAT                        the input (parse)
//   envdat, nucpos, fmem        text (parse)
//   mybasis, Ftab               basis library and Boys table
//   basinfo, setinfo            text, written by int1e / int2e
//   Suv, Huv                    text (int1e)
//   XX                          gfortran unformatted record, n^4 doubles (int2e)
//   Cui, eig, MOLDEN            text (scf); Cui is also read as a guess
//   Da, Dold                    one unformatted record per spin (scf)
//   Pxuv                        text, dipole integrals x, y, z (int1p; read by cphf)
//   ijab_AA, ijab_AB, ijab_BB   one unformatted record per (i, j) pair (ao2mo, MP2)
//   ajib_AA/AB/BB, ajbi_AA/BB   one unformatted record per (j, b) pair (ao2mo, UHF CIS)
// A failure prints a message, creates the file `error` (the reference's
// signal to its driver, src/myQC/myQC.f90:30) and exits with status 1; a
// stage started while `error` exists stops at once, as the reference does.
// Environment: MYQC_MODE=tight selects accurate Boys values and true pi
// instead of the reference's table and constants; MYQC_PRECISION=bf16x3
// selects the split-BF16 tensor-core transform in ao2mo.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/myqc.h"

namespace {

bool exists(const char *p) {
  struct stat st;
  return stat(p, &st) == 0;
}

[[noreturn]] void fail(const std::string &msg) {
  std::fprintf(stdout, " %s\n", msg.c_str());
  std::fflush(stdout);
  FILE *f = std::fopen("error", "w");
  if (f) std::fclose(f);
  std::exit(1);
}

std::string slurp(const char *path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) fail(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

// all numbers of a list-directed text file (Fortran D exponents accepted)
std::vector<double> numbers(const char *path) {
  std::string s = slurp(path);
  for (char &ch : s)
    if (ch == 'D' || ch == 'd') ch = 'E';
  std::vector<double> v;
  const char *p = s.c_str();
  char *end;
  while (*p) {
    const double x = std::strtod(p, &end);
    if (end == p) {
      ++p;
      continue;
    }
    v.push_back(x);
    p = end;
  }
  return v;
}

// gfortran sequential unformatted records: int32 length, payload, int32
// length; a payload above 2^31-9 bytes is split in subrecords whose leading
// length is negative while more follow (and trailing length negative on all
// but the first)
std::vector<std::vector<char>> read_records(const char *path) {
  std::string s = slurp(path);
  std::vector<std::vector<char>> out;
  size_t pos = 0;
  while (pos + 4 <= s.size()) {
    std::vector<char> rec;
    for (;;) {
      int32_t m;
      std::memcpy(&m, s.data() + pos, 4);
      const size_t L = (size_t)std::llabs((long long)m);
      if (pos + 8 + L > s.size()) fail(std::string("truncated record in ") + path);
      rec.insert(rec.end(), s.data() + pos + 4, s.data() + pos + 4 + L);
      pos += 8 + L;
      if (m >= 0) break;
    }
    out.push_back(std::move(rec));
  }
  return out;
}

void write_record(std::ofstream &f, const void *data, size_t bytes) {
  const size_t MAXSUB = 2147483639ull;
  const char *p = (const char *)data;
  if (bytes <= MAXSUB) {
    const int32_t m = (int32_t)bytes;
    f.write((const char *)&m, 4);
    f.write(p, bytes);
    f.write((const char *)&m, 4);
    return;
  }
  size_t done = 0;
  bool first = true;
  while (done < bytes) {
    const size_t m = std::min(MAXSUB, bytes - done);
    const bool more = done + m < bytes;
    const int32_t lead = more ? -(int32_t)m : (int32_t)m, trail = first ? (int32_t)m : -(int32_t)m;
    f.write((const char *)&lead, 4);
    f.write(p + done, m);
    f.write((const char *)&trail, 4);
    done += m;
    first = false;
  }
}

void write_text(const char *path, const std::vector<const double *> &mats, size_t count) {
  FILE *f = std::fopen(path, "w");
  if (!f) fail(std::string("cannot write ") + path);
  for (const double *m : mats) {
    for (size_t i = 0; i < count; ++i) std::fprintf(f, " %.17E%s", m[i], (i % 4 == 3 || i + 1 == count) ? "\n" : "");
  }
  std::fclose(f);
}

struct Env {
  int nnuc = 0, nelcA = 0, nelcB = 0;
  std::vector<int> options, Z;
  std::vector<double> xyz;  // nnuc x 3, Fortran xyz(0:nnuc-1, 0:2)
};

Env read_env() {
  Env e;
  std::vector<double> t = numbers("envdat");
  if (t.size() < 4) fail("envdat: too short");
  e.nnuc = (int)t[0];
  e.nelcA = (int)t[1];
  e.nelcB = (int)t[2];
  const int nopt = (int)t[3];
  if ((int)t.size() < 4 + nopt) fail("envdat: options missing");
  for (int k = 0; k < nopt; ++k) e.options.push_back((int)t[4 + k]);
  std::vector<double> np = numbers("nucpos");
  if ((int)np.size() < 4 * e.nnuc) fail("nucpos: too short");
  e.xyz.assign(3 * (size_t)e.nnuc, 0.0);
  for (int a = 0; a < e.nnuc; ++a) {
    e.Z.push_back((int)np[4 * a]);
    for (int k = 0; k < 3; ++k) e.xyz[a + (size_t)e.nnuc * k] = np[4 * a + 1 + k];
  }
  return e;
}

const char *ELEM[] = {"H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne"};

// buildBasis (src/myQC/basis.f90:23-226): the flat bas, set, basinfo, setinfo
// arrays of the atoms from the mybasis library, STO-3G section
struct Basis {
  std::vector<double> bas, set;
  std::vector<int> basinfo, setinfo;
  int norb() const { return basinfo[1]; }
};

Basis build_basis(const std::vector<int> &Z) {
  std::vector<std::vector<std::string>> rows;
  {
    std::istringstream in(slurp("mybasis"));
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::vector<std::string> tok;
      std::string w;
      while (ls >> w) tok.push_back(w);
      rows.push_back(tok);
    }
  }
  auto first = [&](size_t r) { return rows[r].empty() ? std::string() : rows[r][0].substr(0, 8); };
  size_t p = 0;
  while (p < rows.size() && first(p) != "STO-3G") ++p;
  if (p + 1 >= rows.size()) fail("mybasis: no STO-3G section");
  const int Smax = std::stoi(rows[p + 1][0]), almax = std::stoi(rows[p + 1][3]), OpS = std::stoi(rows[p + 1][4]);
  (void)Smax;
  const int natm = (int)Z.size(), setl = 3 + OpS;
  const int Omax = std::stoi(rows[p + 1][2]);
  Basis b;
  b.bas.assign((size_t)natm * almax * OpS, 0.0);
  b.set.assign((size_t)natm * almax, 0.0);
  b.basinfo.assign(2 + 5 * (size_t)Omax * natm, 0);
  b.setinfo.assign(2 + (size_t)natm * almax * setl, 0);
  int setnum = 0, orbnum = 0;
  for (int i = 0; i < natm; ++i) {
    if (Z[i] < 1 || Z[i] > 10) fail("mybasis: element out of range");
    size_t q = p;
    while (q < rows.size() && first(q) != ELEM[Z[i] - 1]) ++q;
    if (q + 1 >= rows.size()) fail(std::string("mybasis: no ") + ELEM[Z[i] - 1]);
    const int sec = std::stoi(rows[q + 1][0]), orb = std::stoi(rows[q + 1][1]), nset = std::stoi(rows[q + 1][2]);
    q += 2;
    b.basinfo[0] = OpS;
    b.basinfo[1] += orb;
    b.setinfo[0] += nset;
    b.setinfo[1] = setl;
    for (int s = 0; s < sec; ++s) {
      while (q < rows.size() && rows[q].size() < 5) ++q;
      const int func = std::stoi(rows[q][0]), coef = std::stoi(rows[q][1]), pri = std::stoi(rows[q][2]),
                ang = std::stoi(rows[q][3]), ori = std::stoi(rows[q][4]);
      ++q;
      for (int k = 0; k < func; ++k, ++q) {
        std::vector<double> v;
        for (int c = 0; c <= coef; ++c) {
          std::string t = rows[q][c];
          for (char &ch : t)
            if (ch == 'D' || ch == 'd') ch = 'E';
          v.push_back(std::stod(t));
        }
        const double tt = v[coef];
        const int sid = setnum + (int)std::floor(std::fabs(tt) + 0.5) * (tt >= 0 ? 1 : -1);
        b.set[sid] = v[coef - 1];
        const size_t base = 1 + (size_t)sid * setl;
        int kk = b.setinfo[base + 1];
        b.setinfo[base + 3] = i;
        if (ori == -1) {
          b.setinfo[base + 4 + kk] = orbnum;
          b.bas[kk + (size_t)sid * OpS] = v[0];
          ++kk;
        } else if (ori == 2) {
          for (int m = 0; m < 3; ++m) {
            b.setinfo[base + 4 + kk] = orbnum + m;
            b.bas[kk + (size_t)sid * OpS] = v[0];
            ++kk;
          }
          b.setinfo[base + 2] = std::max(b.setinfo[base + 2], 1);
        } else {
          fail("mybasis: only s and p sections are supported");
        }
        b.setinfo[base + 1] = kk;
      }
      if (ori == -1) {
        int *bi = &b.basinfo[2 + 5 * (size_t)orbnum];
        bi[0] = pri, bi[1] = ang, bi[2] = ori, bi[3] = func, bi[4] = i;
        orbnum += 1;
      } else {
        for (int m = 0; m < 3; ++m) {
          int *bi = &b.basinfo[2 + 5 * (size_t)(orbnum + m)];
          bi[0] = pri, bi[1] = ang, bi[2] = m, bi[3] = func, bi[4] = i;
        }
        orbnum += 3;
      }
    }
    setnum = b.setinfo[0];
  }
  return b;
}

void write_basinfo(const Basis &b) {
  FILE *f = std::fopen("basinfo", "w");
  if (!f) fail("cannot write basinfo");
  for (int v : b.basinfo) std::fprintf(f, " %d", v);
  std::fprintf(f, "\n\n #orbitals per set, #orbitals, {principle qn., angular qn., orientation, #primatives, center "
                  "number},...\n");
  std::fclose(f);
  f = std::fopen("setinfo", "w");
  if (!f) fail("cannot write setinfo");
  for (int v : b.setinfo) std::fprintf(f, " %d", v);
  std::fprintf(f, "\n\n #sets, length of each set,{#orbitals, max ang qn., center num, [orbital 0, orbital 1, ...]},...\n");
  std::fclose(f);
}

struct Lib {
  mq_ctx *ctx = nullptr;
  Lib() {
    if (mq_init(&ctx, 0) != MQ_OK) fail("libmyqc: no CUDA device");
  }
  ~Lib() { mq_free(ctx); }
  void check(int rc, const char *what) {
    if (rc == MQ_OK) return;
    char buf[512] = {0};
    mq_last_error(ctx, buf, sizeof buf);
    fail(std::string(what) + ": " + buf);
  }
};

int mode_from_env() {
  const char *m = std::getenv("MYQC_MODE");
  return (m && std::string(m) == "tight") ? MQ_MODE_TIGHT : MQ_MODE_REFERENCE;
}

// the system of the working directory on the context; returns n
int set_system(Lib &L, const Env &e, Basis &b) {
  std::vector<double> ftab;
  const int mode = mode_from_env();
  if (mode == MQ_MODE_REFERENCE) {
    auto recs = read_records("Ftab");
    if (recs.size() != 1 || recs[0].size() != 121 * 23 * 8) fail("Ftab: expected one record of 121x23 doubles");
    ftab.resize(121 * 23);
    std::memcpy(ftab.data(), recs[0].data(), recs[0].size());
  }
  L.check(mq_set_system(L.ctx, e.nnuc, e.Z.data(), e.xyz.data(), b.bas.data(), b.set.data(), b.basinfo.data(),
                        b.setinfo.data(), ftab.empty() ? nullptr : ftab.data(), mode),
          "set_system");
  int n = 0;
  L.check(mq_norb(L.ctx, &n), "norb");
  return n;
}

std::vector<double> read_XX(int n) {
  auto recs = read_records("XX");
  const size_t want = (size_t)n * n * n * n * 8;
  if (recs.size() != 1 || recs[0].size() != want) fail("XX: expected one record of n^4 doubles");
  std::vector<double> XX((size_t)n * n * n * n);
  std::memcpy(XX.data(), recs[0].data(), want);
  return XX;
}

// ------------------------------------------------------------------ stages
// ---- parse (src/parser/parser.f90): ZMAT -> nucpos, envdat, fmem
//
// CARTESIAN input only, as the reference: a line CARTESIAN, one line per atom
// (symbol, x, y, z), END, one line skipped, then "KEY= value" option lines
// (read_options, :700-735, and the get* functions, :160-430).  The geometry is
// recentred on the centre of mass with integer masses, converted from
// angstrom to bohr unless UNITS= Bohr (build, :435-547); the electron counts
// follow from the charge and multiplicity.  Where the reference touches
// `error` (atoms closer than 0.2 A, an impossible charge and multiplicity,
// RHF for an open shell, contradicting options) the files are still written
// and the stage then fails; where the reference only STOPs (an unknown
// element, method, basis or reference, a multiplicity below 1) this stage
// also writes `error`, so that a driver polling it stops.
const double A2B = 1.8897161646320724;  // parser.f90:14

std::vector<std::string> tokens(const std::string &line) {
  std::istringstream ls(line);
  std::vector<std::string> tok;
  std::string w;
  while (ls >> w) tok.push_back(w);
  return tok;
}

// READ(chr,'(I8)'): the first 8 characters as an integer, blanks ignored
long long read_i8(const std::string &tok, const char *key) {
  std::string t;
  for (char ch : tok.substr(0, 8))
    if (ch != ' ') t.push_back(ch);
  if (t.empty()) return 0;
  char *end = nullptr;
  const long long v = std::strtoll(t.c_str(), &end, 10);
  if (!end || *end) fail(std::string("ZMAT: bad integer for ") + key + " " + tok);
  return v;
}

double read_real(std::string t) {
  for (char &ch : t)
    if (ch == 'D' || ch == 'd') ch = 'E';
  char *end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  if (!end || *end) fail("ZMAT: bad coordinate " + t);
  return v;
}

int stage_parse() {
  if (!exists("ZMAT")) fail("You need to create the input file : 'ZMAT'");
  const std::string text = slurp("ZMAT");
  std::fputs(text.c_str(), stdout);  // the reference echoes its input (cat ZMAT)
  std::printf(" \n Input parameters\n");
  std::vector<std::string> lines;
  {
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
      if (!line.empty() && line.back() == '\r') line.pop_back();
      lines.push_back(line);
    }
  }
  const int fline = (int)lines.size();
  const std::vector<std::string> head = lines.empty() ? std::vector<std::string>() : tokens(lines[0]);
  const std::string sys = head.empty() ? std::string() : head[0].substr(0, 9);
  if (sys == "INTERNAL") fail("Sorry, that input style not supported yet");
  if (sys != "CARTESIAN") fail("Bad system type input. Exiting...");
  // geometry (cartesian, :622-678)
  std::vector<int> Z;
  std::vector<double> X;  // nnuc x 3, row-major while parsing
  int i = 1;
  for (;; ++i) {
    if (i >= fline) fail("You need to put 'END' marker in ZMAT");
    const std::vector<std::string> tok = tokens(lines[i]);
    if (!tok.empty() && tok[0] == "END") break;
    if (tok.size() < 4) fail("ZMAT: bad atom line '" + lines[i] + "'");
    const std::string id = tok[0].substr(0, 2);
    int z = 0;
    for (int k = 0; k < 10; ++k)
      if (id == ELEM[k]) z = k + 1;
    if (!z) fail("Sorry, that element is not implemented yet. Exiting ...");
    Z.push_back(z);
    for (int k = 1; k <= 3; ++k) X.push_back(read_real(tok[k]));
  }
  const int nnuc = (int)Z.size();
  if (nnuc <= 0) fail("No atoms in system");
  // options (defaults as :52; read_options skips the line after END)
  long long opt[17] = {0, 0, 0, 0, 0, 1, 1000, 1, 7, 0, 1, 0, 1, 0, 0, 0, 0};
  const int nline = nnuc + 2;
  for (int l = nline + 1; l < fline; ++l) {
    const std::vector<std::string> tok = tokens(lines[l]);
    if (tok.size() < 2) continue;
    const std::string &k = tok[0], &v = tok[1];
    if (k == "CALC=") {
      if (v == "SCF" || v == "HF") opt[1] = 0;
      else if (v == "MP2") opt[1] = 1;
      else if (v == "CIS") opt[1] = 2;
      else fail("Sorry, that method has not been implimented. Exiting...");
    } else if (k == "BASIS=") {
      if (v == "STO-3G") opt[2] = 0;
      else if (v == "tester1") opt[2] = 1;
      else if (v == "tester2") opt[2] = 2;
      else if (v == "tester3") opt[2] = 3;
      else fail("Sorry, that basis has not been implimented. Exiting...");
    } else if (k == "CHARGE=") {
      opt[9] = read_i8(v, "CHARGE=");
    } else if (k == "MULTI=") {
      opt[10] = read_i8(v, "MULTI=");
      if (opt[10] <= 0) fail("bad value for multiplicity, exiting.");
    } else if (k == "REF=") {
      if (v == "RHF") opt[3] = 0;
      else if (v == "UHF") opt[3] = 1;
      else if (v == "ROHF") fail("Sorry, this reference is not implimented yet. Exiting...");
      else fail("Sorry, that reference has not been implimented. Exiting...");
    } else if (k == "PAR=") {
      opt[4] = v == "OMP" ? 2 : v == "MPI" ? 3 : 1;
    } else if (k == "NODES=") {
      std::printf(" Nodes : not implimented yet\n");
      opt[5] = 1;
    } else if (k == "MEMORY=") {
      const long long m = read_i8(v, "MEMORY=");
      if (m < 0) std::printf(" You specificed a memory less than zero.\n");
      opt[6] = m < 0 ? 1000 : m;
    } else if (k == "VERB=") {
      opt[7] = v == "1" ? 1 : v == "2" ? 2 : v == "3" ? 3 : 0;
    } else if (k == "SCF_Conv=") {
      opt[8] = read_i8(v, "SCF_Conv=");
    } else if (k == "UNITS=") {
      opt[11] = v == "Bohr" ? 1 : 0;
    } else if (k == "AO2MO=") {
      if (v != "1") std::printf(" Sorry, only slow ao2mo supported\n");
      opt[12] = 1;
    } else if (k == "EXCITE=") {
      opt[13] = (v == "CIS" || v == "1") ? 1 : 0;
    } else if (k == "ROOT_ALG=") {
      opt[14] = 0;
    } else if (k == "E_NUM=") {
      const long long m = read_i8(v, "E_NUM=");
      opt[15] = m < 0 ? 1 : m;
    } else if (k == "PROP=") {
      opt[16] = (v == "FIRST" || v == "1") ? 1 : (v == "SECOND" || v == "2") ? 2 : 0;
    } else {
      std::printf(" parser could not understand options line %12d\n", l - nline - 1);
    }
  }
  bool bad = false;
  // checkgeom (:560-600): pairs closer than 0.2 A in the input units
  for (int a = 0; a < nnuc; ++a)
    for (int b = a + 1; b < nnuc; ++b) {
      double r = 0.0;
      for (int k = 0; k < 3; ++k) r += (X[3 * a + k] - X[3 * b + k]) * (X[3 * a + k] - X[3 * b + k]);
      if (std::sqrt(r) < (opt[11] == 0 ? 0.2 : 0.2 * A2B)) {
        std::printf(" These atoms are too close (r < 0.2 A) : %12d %12d\n", a, b);
        bad = true;
      }
    }
  // centre of mass with integer masses, then angstrom -> bohr
  static const double MASS[10] = {1, 4, 7, 9, 11, 12, 14, 16, 19, 20};
  double com[3] = {0, 0, 0}, tot = 0.0;
  for (int a = 0; a < nnuc; ++a) {
    for (int k = 0; k < 3; ++k) com[k] = com[k] + MASS[Z[a] - 1] * X[3 * a + k];
    tot = tot + MASS[Z[a] - 1];
  }
  for (int k = 0; k < 3; ++k) com[k] = com[k] / tot;
  for (int a = 0; a < nnuc; ++a)
    for (int k = 0; k < 3; ++k) {
      X[3 * a + k] = X[3 * a + k] - com[k];
      if (opt[11] == 0) X[3 * a + k] = X[3 * a + k] * A2B;
    }
  // electrons
  long long nelc = -opt[9];
  for (int z : Z) nelc += z;
  const long long unpr = opt[10] - 1;
  long long nelcB = (nelc - unpr) / 2, nelcA = nelcB + unpr;
  if (nelcA + nelcB != nelc) {
    std::printf(" That charge and multiplicity is not allowed.\n");
    bad = true;
  }
  if (nelc < 0 || nelcA < 0 || nelcB < 0) {
    std::printf(" You have less than 0 electrons. :)\n");
    bad = true;
  }
  if (nelcA != nelcB && opt[3] == 0) {
    std::printf(" You cannot use RHF for open shell molecules!\n");
    bad = true;
  }
  {
    FILE *f = std::fopen("nucpos", "w");
    if (!f) fail("cannot write nucpos");
    for (int a = 0; a < nnuc; ++a)
      std::fprintf(f, " %11d %25.17E %25.17E %25.17E\n", Z[a], X[3 * a], X[3 * a + 1], X[3 * a + 2]);
    std::fclose(f);
    f = std::fopen("envdat", "w");
    if (!f) fail("cannot write envdat");
    std::fprintf(f, " %11d\n %11lld %11lld\n %11d\n", nnuc, nelcA, nelcB, 17);
    for (int k = 0; k < 17; ++k) std::fprintf(f, " %20lld", opt[k]);
    std::fprintf(f, "\n \n #number of nuclei\n #number of electrons\n #length of options array\n options array\n");
    std::fclose(f);
    f = std::fopen("fmem", "w");
    if (!f) fail("cannot write fmem");
    std::fprintf(f, " %20lld\n", opt[6]);
    std::fclose(f);
  }
  if (bad) fail("parser found an error in ZMAT");
  // check_options (:767-800)
  std::string why;
  if (opt[13] != 0 && opt[1] != 0) why += " Sorry, only SCF CIS coded\n";
  if (opt[13] != 0 && opt[3] != 1) why += " Sorry, only UHF CIS references are coded\n";
  if (opt[16] != 0 && opt[1] != 0) why += " Sorry, only SCF properties are coded\n";
  if (opt[16] != 0 && opt[3] != 0) why += " Sorry, only RHF reference properites are coded\n";
  if (!why.empty()) {
    std::fputs(why.c_str(), stdout);
    fail("===========================================\n Bad options in ZMAT");
  }
  std::printf(" ===========================================\n");
  std::printf(" nuclei %d, alpha electrons %lld, beta electrons %lld, %s, %s, SCF convergence 1e-%lld\n", nnuc, nelcA,
              nelcB, opt[3] ? "UHF" : "RHF", opt[1] == 1 ? "MP2" : opt[1] == 2 ? "CIS" : "SCF", opt[8]);
  return 0;
}

int stage_int1e() {
  std::printf("\n int1e called\n");
  Env e = read_env();
  Basis b = build_basis(e.Z);
  write_basinfo(b);
  Lib L;
  const int n = set_system(L, e, b);
  std::vector<double> S((size_t)n * n), H((size_t)n * n);
  L.check(mq_int1e(L.ctx, S.data(), H.data()), "int1e");
  write_text("Suv", {S.data()}, S.size());
  write_text("Huv", {H.data()}, H.size());
  std::printf(" One electron integrals constructed (n = %d)\n", n);
  return 0;
}

int stage_int2e() {
  std::printf("\n int2e called\n");
  Env e = read_env();
  Basis b = build_basis(e.Z);
  write_basinfo(b);
  if (exists("XX")) {  // int2e.f90:58-63
    std::printf(" Reading two electron integrals from intermediate\n");
    return 0;
  }
  std::printf(" Constructing two electron integrals\n");
  Lib L;
  const int n = set_system(L, e, b);
  std::vector<double> XX((size_t)n * n * n * n);
  L.check(mq_eri_full(L.ctx, XX.data()), "int2e");
  std::ofstream f("XX", std::ios::binary | std::ios::trunc);
  if (!f) fail("cannot write XX");
  write_record(f, XX.data(), XX.size() * sizeof(double));
  double ms = 0;
  mq_stat(L.ctx, "eri", &ms);
  std::printf(" Two electron integrals constructed in (s) %10.5f\n", ms * 1e-3);
  return 0;
}

// gfortran's list-directed REAL(8) item (1PG25.17E3): 17 significant
// digits in F form, right-justified in 20 columns and followed by 5 blanks,
// when the value rounded to 17 digits lies in [0.1, 1e17) (zero included, with
// 16 decimals); otherwise E form with one leading digit, 16 decimals and a
// three-digit exponent, right-justified in 25 columns
std::string ld_real(double x) {
  char buf[64];
  if (x == 0.0) {
    std::snprintf(buf, sizeof buf, "%20.16f     ", x);
    return buf;
  }
  std::snprintf(buf, sizeof buf, "%.16e", x);
  const int e10 = std::atoi(std::strchr(buf, 'e') + 1);
  if (e10 >= -1 && e10 <= 16) {
    std::snprintf(buf, sizeof buf, "%20.*f     ", 16 - e10, x);
    return buf;
  }
  char m[64];
  std::snprintf(m, sizeof m, "%.16E", x);  // d.dddE+XX: widen the exponent to three digits
  char *ep = std::strchr(m, 'E');
  const int ex = std::abs(std::atoi(ep + 1)) % 1000;
  const char sign = ep[1] == '-' ? '-' : '+';
  *ep = 0;
  std::snprintf(buf, sizeof buf, "%.24sE%c%03d", m, sign, ex);
  char out[64];
  std::snprintf(out, sizeof out, "%25s", buf);
  return out;
}

// MOLDEN file of the SCF orbitals in the reference writer's layout
// (makeMOLDEN, src/scf/scf.f90:1343-1466): the atoms in bohr, then per atom
// its mybasis sections as listed there (a shell letter, the primitive count,
// "1.00", then exponent and coefficient of each primitive as list-directed
// REAL(8) items), then every orbital with occupation 1 when its energy is
// negative; beta orbitals follow for UHF
void write_molden(const Env &e, int n, const std::vector<double> &C, const std::vector<double> &eps, bool uhf) {
  std::vector<std::vector<std::string>> rows;
  {
    std::istringstream in(slurp("mybasis"));
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::vector<std::string> tok;
      std::string w;
      while (ls >> w) tok.push_back(w);
      rows.push_back(tok);
    }
  }
  auto first = [&](size_t r) { return rows[r].empty() ? std::string() : rows[r][0].substr(0, 8); };
  auto real = [&](std::string t) {
    for (char &ch : t)
      if (ch == 'D' || ch == 'd') ch = 'E';
    return std::stod(t);
  };
  FILE *f = std::fopen("MOLDEN", "w");
  if (!f) fail("cannot write MOLDEN");
  std::fprintf(f, " [Molden Format]\n [ATOMS] AU\n");
  for (int a = 0; a < e.nnuc; ++a)
    std::fprintf(f, "%-2s    %3d    %3d    %15.8f    %15.8f    %15.8f\n", ELEM[e.Z[a] - 1], a + 1, e.Z[a], e.xyz[a],
                 e.xyz[a + e.nnuc], e.xyz[a + 2 * (size_t)e.nnuc]);
  std::fprintf(f, " [Molden Format]\n [GTO]\n");
  static const char SHELL[] = "spdfgh";
  size_t p = 0;
  while (p < rows.size() && first(p) != "STO-3G") ++p;
  for (int a = 0; a < e.nnuc; ++a) {
    std::fprintf(f, " %11d %11d\n", a + 1, 0);
    size_t q = p;
    while (q < rows.size() && first(q) != ELEM[e.Z[a] - 1]) ++q;
    if (q + 1 >= rows.size()) fail(std::string("mybasis: no ") + ELEM[e.Z[a] - 1]);
    const int sec = std::stoi(rows[q + 1][0]);
    q += 2;
    for (int s = 0; s < sec; ++s) {
      while (q < rows.size() && rows[q].size() < 5) ++q;
      if (q >= rows.size()) fail("mybasis: truncated section");
      const int func = std::stoi(rows[q][0]), coef = std::stoi(rows[q][1]), ang = std::stoi(rows[q][3]);
      if (ang < 0 || ang > 5 || coef < 1) fail("mybasis: bad section header");
      ++q;
      std::fprintf(f, " %c %11d 1.00\n", SHELL[ang], func);
      for (int k = 0; k < func; ++k, ++q) {
        if (q >= rows.size() || (int)rows[q].size() < coef) fail("mybasis: truncated primitive line");
        std::string line;
        for (int c = 1; c < coef; ++c) line += " " + ld_real(real(rows[q][c]));
        line += " " + ld_real(real(rows[q][0]));
        std::fprintf(f, "%s\n", line.c_str());
      }
    }
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "\n [MO]\n");
  for (int s = 0; s < (uhf ? 2 : 1); ++s)
    for (int i = 0; i < n; ++i) {
      const double en = eps[(size_t)s * n + i];
      std::fprintf(f, " Sym= A\n Ene= %15.8f\n  Spin= %s\n Occup= %s\n", en, s ? "Beta" : "Alpha",
                   en < 0 ? "1.0" : "0.0");
      for (int k = 0; k < n; ++k) std::fprintf(f, " %4d    %15.10f\n", k + 1, C[(size_t)s * n * n + k + (size_t)n * i]);
    }
  std::fclose(f);
}

int stage_scf() {
  std::printf("\n                      STARTING SCF\n ------------------------------------------------------------\n");
  Env e = read_env();
  Basis b = build_basis(e.Z);
  Lib L;
  const int n = set_system(L, e, b);
  const size_t n2 = (size_t)n * n;
  std::vector<double> S = numbers("Suv"), H = numbers("Huv");
  if (S.size() < n2 || H.size() < n2) fail("Suv/Huv: too short");
  std::vector<double> XX = read_XX(n);
  L.check(mq_eri_upload(L.ctx, XX.data()), "XX upload");
  std::vector<double>().swap(XX);
  const bool uhf = e.options.size() > 3 && e.options[3] == 1;
  const int ns = uhf ? 2 : 1;
  mq_scf_opts o;
  std::memset(&o, 0, sizeof o);
  o.uhf = uhf;
  o.nalpha = e.nelcA;
  o.nbeta = e.nelcB;
  const int cexp = e.options.size() > 8 ? e.options[8] : 7;
  o.conv = std::pow(10.0, -std::min(cexp, 12));
  std::vector<double> Cin;
  if (exists("Cui")) {
    Cin = numbers("Cui");
    if (Cin.size() >= ns * n2) {
      std::printf(" Reading MO coef from Cui\n");
      o.guess = 1;
      o.C_in = Cin.data();
    }
  }
  const int cap = uhf ? 300 : 500;
  std::vector<double> C(ns * n2), eps((size_t)ns * n), D(ns * n2), hist(2 * (size_t)cap);
  double E = 0.0;
  int iters = 0;
  const int rc = mq_scf(L.ctx, S.data(), H.data(), &o, C.data(), eps.data(), D.data(), &E, &iters, hist.data());
  if (rc != MQ_OK && rc != MQ_ENOCONV) L.check(rc, "scf");
  std::printf(" %s calculation...\n Iteration   Total Energy (hartrees)   Ediff               Ddiff\n", uhf ? "UHF" : "RHF");
  std::printf(" =========================================================================\n");
  for (int k = 0; k < iters; ++k) {
    const double Ek = hist[2 * k], dE = k ? Ek - hist[2 * (k - 1)] : 0.0;
    if (k) std::printf("    %3d    %20.15f        %15.8E    %15.8E\n", k, Ek, dE, hist[2 * k + 1]);
    else std::printf("    %3d    %20.15f\n", k, Ek);
  }
  if (rc == MQ_ENOCONV) std::printf(" SCF failed to converge.\n");
  else std::printf(" SCF has converged!\n\n Total SCF energy (a.u) %25.17f\n\n", E);
  std::printf(" =========================================================================\n Orbital eigenvalues (a.u.)\n");
  for (int s = 0; s < ns; ++s)
    for (int i = 0; i < n; ++i) std::printf("               %3d    %20.15f\n", i + 1, eps[(size_t)s * n + i]);
  std::vector<const double *> cm, em;
  for (int s = 0; s < ns; ++s) {
    cm.push_back(C.data() + s * n2);
    em.push_back(eps.data() + (size_t)s * n);
  }
  write_text("Cui", cm, n2);
  write_text("eig", em, (size_t)n);
  write_molden(e, n, C, eps, uhf);
  // the density files of the reference's loop (dens.f90 writes Da, scf.f90
  // keeps Dold): one unformatted record per spin; both hold the last
  // iteration's density here, converged to the SCF threshold
  for (const char *fn : {"Da", "Dold"}) {
    std::ofstream f(fn, std::ios::binary | std::ios::trunc);
    if (!f) fail(std::string("cannot write ") + fn);
    for (int s2 = 0; s2 < ns; ++s2) write_record(f, D.data() + s2 * n2, n2 * sizeof(double));
  }
  return 0;
}

// int1p (src/integrals/int1p.f90): dipole integrals into Pxuv (text, the x, y, z
// matrices in turn); an existing Pxuv is kept, as the reference keeps it
int stage_int1p() {
  std::printf(" int1p called\n               STARTING PROPERTY INTEGRALS\n"
              " ------------------------------------------------------------\n");
  Env e = read_env();
  if (exists("Pxuv")) {
    std::printf(" Reading Dipole integrals from Pxuv\n");
    return 0;
  }
  Basis b = build_basis(e.Z);
  Lib L;
  const int n = set_system(L, e, b);
  const size_t n2 = (size_t)n * n;
  std::vector<double> P(3 * n2);
  L.check(mq_int1p(L.ctx, P.data()), "int1p");
  write_text("Pxuv", {P.data(), P.data() + n2, P.data() + 2 * n2}, n2);
  std::printf(" Dipole moment integrals written to Pxuv\n");
  return 0;
}

// cphf (src/props/cphf.f90:80-131): the RHF dipole moment from Pxuv and Da,
// mu_c = -sum_uv D(u,v) Px(c,v,u) + sum_A Z_A R_A,c
int stage_cphf() {
  std::printf("\n cphf called\n\n");
  Env e = read_env();
  const bool uhf = e.options.size() > 3 && e.options[3] == 1;
  if (uhf) {
    std::printf(" Sorry, only RHF CPHF equations are coded\n");
    return 0;
  }
  std::vector<double> bi = numbers("basinfo");
  if (bi.size() < 2) fail("basinfo: too short");
  const size_t n = (size_t)bi[1], n2 = n * n;
  std::vector<double> P = numbers("Pxuv");
  if (P.size() < 3 * n2) fail("Pxuv: too short");
  auto recs = read_records("Da");
  if (recs.empty() || recs[0].size() != n2 * sizeof(double)) fail("Da: bad record");
  const double *D = (const double *)recs[0].data();
  double mu[3];
  for (int c = 0; c < 3; ++c) {
    double t = 0.0;
    for (size_t u = 0; u < n; ++u)
      for (size_t v = 0; v < n; ++v) t -= D[u + n * v] * P[c * n2 + v + n * u];
    for (int a = 0; a < e.nnuc; ++a) t += e.Z[a] * e.xyz[a + (size_t)e.nnuc * c];
    mu[c] = t;
  }
  std::printf("                 Dipole Moments                \n ----------------------------------------------\n"
              "        X              Y              Z        \n%15.6f%15.6f%15.6f\n"
              " ----------------------------------------------\n",
              mu[0], mu[1], mu[2]);
  return 0;
}

// props (src/props/props.f90): first- or second-order properties of an SCF
// (options(1) = 0) run int1p then cphf
int stage_props() {
  std::printf("\n               STARTING PROPERTY CALCULATIONS\n"
              " ------------------------------------------------------------\n props called\n\n");
  Env e = read_env();
  const int order = e.options.size() > 16 ? e.options[16] : 0;
  const int calc = e.options.size() > 1 ? e.options[1] : 0;
  if (order == 0) {
    std::printf(" Property order   :  none\n");
    return 0;
  }
  std::printf(" Property order   :  %s\n", order == 1 ? "first" : "second");
  if (calc != 0) {
    std::printf(" Sorry, only cphf properties for RHF available\n");
    return 0;
  }
  std::printf(" Property method  :  cphf\n");
  if (const int rc = stage_int1p()) return rc;
  return stage_cphf();
}

int precision_from_env() {
  const char *p = std::getenv("MYQC_PRECISION");
  if (!p) return MQ_PREC_FP64;
  const std::string s(p);
  if (s == "bf16x3") return MQ_PREC_SPLIT_BF16X3;
  if (s == "bf16") return MQ_PREC_SPLIT_BF16;
  return MQ_PREC_FP64;
}

// records Om(i, :, j, :) (v1 x v2, a fastest) for i < j (upper) or all (i, j)
void write_ijab(const char *path, const std::vector<double> &Om, int no1, int nv1, int no2, int nv2, bool upper) {
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) fail(std::string("cannot write ") + path);
  std::vector<double> rec((size_t)nv1 * nv2);
  for (int i = 0; i < no1; ++i)
    for (int j = upper ? i + 1 : 0; j < no2; ++j) {
      for (int b = 0; b < nv2; ++b)
        for (int a = 0; a < nv1; ++a)
          rec[a + (size_t)nv1 * b] = Om[i + (size_t)no1 * (a + (size_t)nv1 * (j + (size_t)no2 * b))];
      write_record(f, rec.data(), rec.size() * sizeof(double));
    }
}

// The UHF CIS integral blocks of slow_ao2mo_CIS_UHF (src/ao2mo/ao2mo.f90:919-1227):
// Om(x1,x2,x3,x4) = sum (uv|ld) C1(u,x1) C2(v,x2) C3(l,x3) C4(d,x4), x1 fastest,
// one record per (j, b) with the (i, a) block, a fastest:
//   ajib_AA, ajib_AB, ajib_BB   Om(a,i,j,b) over the blocks (vrt, occ, occ, vrt)
//   ajbi_AA, ajbi_BB            Om(a,b,j,i) over the blocks (vrt, vrt, occ, occ)
void cis_blocks(Lib &L, const double *CA, const double *CB, int n, int noA, int noB, int prec) {
  struct Blk {
    const char *file;
    const double *c1, *c3;  // alpha/beta coefficients of the first two and the last two indices
    int o1, o3;
    bool ajbi;
  };
  const Blk blocks[5] = {{"ajib_AA", CA, CA, noA, noA, false}, {"ajbi_AA", CA, CA, noA, noA, true},
                         {"ajib_AB", CA, CB, noA, noB, false}, {"ajib_BB", CB, CB, noB, noB, false},
                         {"ajbi_BB", CB, CB, noB, noB, true}};
  for (const Blk &k : blocks) {
    const int v1 = n - k.o1, v3 = n - k.o3;
    const double *occ1 = k.c1, *vrt1 = k.c1 + (size_t)n * k.o1, *occ3 = k.c3, *vrt3 = k.c3 + (size_t)n * k.o3;
    std::vector<double> Om((size_t)v1 * (k.ajbi ? v1 : k.o1) * k.o3 * (k.ajbi ? k.o3 : v3));
    if (!k.ajbi)
      L.check(mq_ao2mo_iajb(L.ctx, vrt1, v1, occ1, k.o1, occ3, k.o3, vrt3, v3, prec, Om.data()), "ao2mo");
    else
      L.check(mq_ao2mo_iajb(L.ctx, vrt1, v1, vrt1, v1, occ3, k.o3, occ3, k.o3, prec, Om.data()), "ao2mo");
    std::printf(" Writing to %s\n", k.file);
    std::ofstream f(k.file, std::ios::binary | std::ios::trunc);
    if (!f) fail(std::string("cannot write ") + k.file);
    std::vector<double> rec((size_t)k.o1 * v1);
    const int nj = k.o3, nb = k.ajbi ? v1 : v3;
    for (int j = 0; j < nj; ++j)
      for (int b = 0; b < nb; ++b) {
        if (!k.ajbi) {  // Om(:, :, j, b) is one contiguous (a, i) block
          const double *src = Om.data() + (size_t)v1 * k.o1 * (j + (size_t)k.o3 * b);
          std::copy(src, src + rec.size(), rec.begin());
        } else {  // Om(a, b, j, i) gathered over i, a
          for (int i = 0; i < k.o1; ++i)
            for (int a = 0; a < v1; ++a)
              rec[a + (size_t)v1 * i] = Om[a + (size_t)v1 * (b + (size_t)v1 * (j + (size_t)k.o3 * i))];
        }
        write_record(f, rec.data(), rec.size() * sizeof(double));
      }
  }
}

int stage_ao2mo() {
  std::printf("\n                STARTING AO TRANSFORM\n ------------------------------------------------------------\n");
  std::printf(" ao2mo called\n\n Starting AO to MO integral transform\n");
  Env e = read_env();
  Basis b = build_basis(e.Z);
  Lib L;
  const int n = set_system(L, e, b);
  const size_t n2 = (size_t)n * n;
  std::vector<double> XX = read_XX(n);
  L.check(mq_eri_upload(L.ctx, XX.data()), "XX upload");
  std::vector<double>().swap(XX);
  const bool uhf = e.options.size() > 3 && e.options[3] == 1;
  std::vector<double> C = numbers("Cui");
  if (C.size() < (uhf ? 2 : 1) * n2) fail("Cui: too short");
  const int prec = precision_from_env();
  // transform type as ao2mo.f90 chooses it: MP2 (options(1) = 1), SCF CIS
  // (options(13) = 1, options(1) = 0, UHF only), else an error
  const int calc = e.options.size() > 1 ? e.options[1] : 0;
  const int excite = e.options.size() > 13 ? e.options[13] : 0;
  if (calc != 1) {
    if (excite == 1 && calc == 0) {
      if (!uhf) fail("Sorry, only UHF CIS is coded");
      cis_blocks(L, C.data(), C.data() + n2, n, e.nelcA, e.nelcB, prec);
      return 0;
    }
    fail("Sorry, that transform type has not been coded yet");
  }
  struct Blk {
    const char *file;
    const double *c1, *c2;
    int o1, o2;
    bool upper;
  };
  std::vector<Blk> blocks;
  const double *CA = C.data(), *CB = uhf ? C.data() + n2 : C.data();
  blocks.push_back({"ijab_AA", CA, CA, e.nelcA, e.nelcA, true});
  if (uhf) blocks.push_back({"ijab_BB", CB, CB, e.nelcB, e.nelcB, true});
  blocks.push_back({"ijab_AB", CA, CB, e.nelcA, uhf ? e.nelcB : e.nelcA, false});
  for (const Blk &k : blocks) {
    const int v1 = n - k.o1, v2 = n - k.o2;
    std::vector<double> Om((size_t)k.o1 * v1 * k.o2 * v2);
    L.check(mq_ao2mo_iajb(L.ctx, k.c1, k.o1, k.c1 + (size_t)n * k.o1, v1, k.c2, k.o2, k.c2 + (size_t)n * k.o2, v2, prec,
                          Om.data()),
            "ao2mo");
    std::printf(" Writing to %s\n", k.file);
    write_ijab(k.file, Om, k.o1, v1, k.o2, v2, k.upper);
  }
  return 0;
}

// (ia|jb) of a file of records written by write_ijab
std::vector<double> read_ijab(const char *path, int no1, int nv1, int no2, int nv2, bool upper) {
  auto recs = read_records(path);
  std::vector<double> Om((size_t)no1 * nv1 * no2 * nv2, 0.0);
  size_t r = 0;
  for (int i = 0; i < no1; ++i)
    for (int j = upper ? i + 1 : 0; j < no2; ++j, ++r) {
      if (r >= recs.size() || recs[r].size() != (size_t)nv1 * nv2 * 8) fail(std::string(path) + ": bad record");
      const double *rec = (const double *)recs[r].data();
      for (int b = 0; b < nv2; ++b)
        for (int a = 0; a < nv1; ++a)
          Om[i + (size_t)no1 * (a + (size_t)nv1 * (j + (size_t)no2 * b))] = rec[a + (size_t)nv1 * b];
    }
  return Om;
}

int stage_mp2() {
  std::printf("\n                      STARTING MP2\n ------------------------------------------------------------\n"
              " mp2 called\n\n");
  Env e = read_env();
  const bool uhf = e.options.size() > 3 && e.options[3] == 1;
  std::vector<double> eig = numbers("eig");
  const int n = (int)(uhf ? eig.size() / 2 : eig.size());
  if (n <= 0) fail("eig: empty");
  Lib L;
  double out[2];
  if (!uhf) {
    const int no = e.nelcA, nv = n - no;
    std::vector<double> Om = read_ijab("ijab_AB", no, nv, no, nv, false);
    L.check(mq_mp2_pairs(L.ctx, Om.data(), no, nv, no, nv, eig.data(), eig.data(), 1, out), "mp2");
    std::printf(" E(AA) =  %25.17E\n E(AB) =  %25.17E\n E(MBPT2) =  %25.17E\n", out[1], out[0], 2 * out[1] + out[0]);
  } else {
    const int noA = e.nelcA, noB = e.nelcB, nvA = n - noA, nvB = n - noB;
    const double *eA = eig.data(), *eB = eig.data() + n;
    std::vector<double> AA = read_ijab("ijab_AA", noA, nvA, noA, nvA, true);
    L.check(mq_mp2_pairs(L.ctx, AA.data(), noA, nvA, noA, nvA, eA, eA, 1, out), "mp2");
    const double eaa = out[1];
    std::vector<double> BB = read_ijab("ijab_BB", noB, nvB, noB, nvB, true);
    L.check(mq_mp2_pairs(L.ctx, BB.data(), noB, nvB, noB, nvB, eB, eB, 1, out), "mp2");
    const double ebb = out[1];
    std::vector<double> AB = read_ijab("ijab_AB", noA, nvA, noB, nvB, false);
    L.check(mq_mp2_pairs(L.ctx, AB.data(), noA, nvA, noB, nvB, eA, eB, 0, out), "mp2");
    const double eab = out[0];
    std::printf(" E(AA) =  %25.17E\n E(BB) =  %25.17E\n E(AB) =  %25.17E\n E(MBPT2) =  %25.17E\n", eaa, ebb, eab,
                eaa + ebb + eab);
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  std::string name = argv[0];
  const size_t slash = name.find_last_of('/');
  if (slash != std::string::npos) name = name.substr(slash + 1);
  static const char *const stages[] = {"parse", "int1e", "int2e", "scf", "ao2mo", "mp2", "int1p", "cphf", "props"};
  bool known = false;
  for (const char *st : stages) known = known || name == st;
  if (!known) {
    if (argc < 2) {
      std::fprintf(stderr, "usage: %s parse|int1e|int2e|scf|ao2mo|mp2|int1p|cphf|props (or through a link of that name)\n",
                   argv[0]);
      return 2;
    }
    name = argv[1];
  }
  if (exists("error")) return 0;  // a previous stage failed: stop, as the reference does
  if (name == "parse") return stage_parse();
  if (name == "int1e") return stage_int1e();
  if (name == "int2e") return stage_int2e();
  if (name == "scf") return stage_scf();
  if (name == "ao2mo") return stage_ao2mo();
  if (name == "mp2") return stage_mp2();
  if (name == "int1p") return stage_int1p();
  if (name == "cphf") return stage_cphf();
  if (name == "props") return stage_props();
  std::fprintf(stderr, "unknown stage %s\n", name.c_str());
  return 2;
}

// basis.cu -- contracted shells and primitive-pair tables from the
// reference's flat basis arrays (src/myQC/basis.f90:23-226 layout), plus the
// accurate Boys table used in MQ_MODE_TIGHT.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>

#include "internal.h"

namespace mq {

static double gto_norm(int l, double a, double pi) {
  // primitive normalisation, the formula of gtoD (src/integrals/auxilary.f90:704-726)
  if (l == 0) return std::pow(2.0 * a / pi, 3.0 / 4.0);
  return std::pow(128.0 * std::pow(a, 5.0) / std::pow(pi, 3.0), 1.0 / 4.0);
}

int build_shells(mq_ctx *c, int nnuc, const int *Z, const double *xyz, const double *bas, const double *set,
                 const int *basinfo, const int *setinfo) {
  if (nnuc <= 0 || !Z || !xyz || !bas || !set || !basinfo || !setinfo) return set_err(c, MQ_EINVAL, "null system array");
  const int ops = basinfo[0], norb = basinfo[1];
  const int nset = setinfo[0], setl = setinfo[1];
  if (norb <= 0 || nset <= 0 || setl != 3 + ops) return set_err(c, MQ_EINVAL, "inconsistent basinfo/setinfo");
  c->nnuc = nnuc;
  c->Z.assign(Z, Z + nnuc);
  c->xyz.resize(3 * (size_t)nnuc);
  for (int a = 0; a < nnuc; ++a)
    for (int k = 0; k < 3; ++k) c->xyz[3 * a + k] = xyz[a + (size_t)nnuc * k];  // xyz(0:nnuc-1,0:2)
  const double pi = c->mode == MQ_MODE_REFERENCE ? PI_REF : PI_TRUE;

  // per AO: the sets that carry it and its coefficient in each
  std::vector<std::vector<std::pair<int, double>>> ao_sets(norb);
  std::vector<int> set_lmax(nset), set_ctr(nset);
  for (int s = 0; s < nset; ++s) {
    const int *si = setinfo + 1 + s * setl;  // si[1]=#AO, si[2]=lmax, si[3]=centre, si[4..]=AOs
    set_lmax[s] = si[2];
    set_ctr[s] = si[3];
    for (int k = 0; k < si[1]; ++k) {
      int o = si[4 + k];
      if (o < 0 || o >= norb) return set_err(c, MQ_EINVAL, "setinfo AO index out of range");
      ao_sets[o].push_back({s, bas[s * ops + k]});
    }
  }
  // group AOs that share atom and primitive sets into shells
  std::map<std::pair<int, std::vector<int>>, std::vector<int>> groups;
  std::vector<std::pair<int, std::vector<int>>> order;
  for (int o = 0; o < norb; ++o) {
    const int *bi = basinfo + 2 + 5 * o;  // [n, l, ori, nprim, centre]
    if (bi[1] > 1) return set_err(c, MQ_EINVAL, "only s and p functions are supported");
    std::vector<int> key;
    for (auto &pr : ao_sets[o]) key.push_back(pr.first);
    std::sort(key.begin(), key.end());
    if (key.empty() || (int)key.size() > KMAX) return set_err(c, MQ_EINVAL, "AO with 0 or too many primitives");
    auto k = std::make_pair(bi[4], key);
    if (!groups.count(k)) order.push_back(k);
    groups[k].push_back(o);
  }
  c->shells.clear();
  for (auto &k : order) {
    std::vector<int> &aos = groups[k];
    std::vector<int> s_aos, p_aos[3];
    for (int o : aos) {
      const int *bi = basinfo + 2 + 5 * o;
      if (bi[1] == 0) s_aos.push_back(o);
      else if (bi[2] >= 0 && bi[2] <= 2) p_aos[bi[2]].push_back(o);
      else return set_err(c, MQ_EINVAL, "bad p orientation");
    }
    size_t np = p_aos[0].size();
    if (p_aos[1].size() != np || p_aos[2].size() != np || np > 1)
      return set_err(c, MQ_EINVAL, "p functions must come as one x,y,z triple per primitive set group");
    size_t nsh = std::max(s_aos.size(), np);
    for (size_t t = 0; t < nsh; ++t) {
      HostShell sh{};
      sh.atom = k.first;
      sh.has_s = t < s_aos.size();
      sh.has_p = t < np;
      sh.type = sh.has_p ? 1 : 0;
      sh.nprim = (int)k.second.size();
      sh.qlmax = 0;
      int so = sh.has_s ? s_aos[t] : -1, px = sh.has_p ? p_aos[0][t] : -1;
      for (int i = 0; i < sh.nprim; ++i) {
        int s = k.second[i];
        sh.alpha[i] = set[s];
        sh.qlmax = std::max(sh.qlmax, set_lmax[s]);
        auto coef_of = [&](int o) {
          double v = 0.0;
          if (o >= 0)
            for (auto &pr : ao_sets[o])
              if (pr.first == s) v = pr.second;
          return v;
        };
        double csv = coef_of(so), cpv = coef_of(px);
        sh.cs[i] = sh.has_s ? csv * gto_norm(0, set[s], pi) : 0.0;
        sh.cp[i] = sh.has_p ? cpv * gto_norm(1, set[s], pi) : 0.0;
      }
      // AO indices: s, px, py, pz must be consecutive (the reference orders a
      // section's functions that way, basis.f90:182-192)
      if (sh.has_p && sh.has_s && (p_aos[0][t] != so + 1 || p_aos[1][t] != so + 2 || p_aos[2][t] != so + 3))
        return set_err(c, MQ_EINVAL, "sp shell AOs are not consecutive");
      if (sh.has_p && (p_aos[1][t] != px + 1 || p_aos[2][t] != px + 2))
        return set_err(c, MQ_EINVAL, "p AOs are not consecutive");
      if (!sh.has_s) return set_err(c, MQ_EINVAL, "p functions without an s function on the same primitive sets");
      sh.ao0 = so;
      c->shells.push_back(sh);
    }
  }
  c->nshell = (int)c->shells.size();
  c->nao = norb;
  return MQ_OK;
}

void free_pairs(mq_ctx *c) {
  for (void *p : c->pair_allocs) cudaFree(p);
  c->pair_allocs.clear();
  c->pt = PairTable{};
  c->schwarz_valid = 0;
}

// Shell pairs of one molecule, in class order (ss), (sp,s), (sp,sp), with
// their surviving primitive pairs.
void pairs_host(const std::vector<HostShell> &shells, const std::vector<double> &xyz, HostPairs &h) {
  h = HostPairs{};
  const int ns = (int)shells.size();
  std::vector<std::pair<int, int>> pl[3];
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b <= a; ++b) {
      int A = a, B = b;
      const HostShell &sa = shells[a], &sb = shells[b];
      if (sb.type > sa.type) std::swap(A, B);
      pl[sa.type + sb.type].push_back({A, B});
    }
  // within a class, pairs with more primitive pairs first: neighbouring quartets
  // of an integral launch (one warp) then loop over similar primitive counts
  auto live = [&](const std::pair<int, int> &ab) {
    const HostShell &A = shells[ab.first], &B = shells[ab.second];
    const double *xa = &xyz[3 * A.atom], *xb = &xyz[3 * B.atom];
    double AB2 = 0;
    for (int k = 0; k < 3; ++k) AB2 += (xa[k] - xb[k]) * (xa[k] - xb[k]);
    int cnt = 0;
    for (int i = 0; i < A.nprim; ++i)
      for (int j = 0; j < B.nprim; ++j) {
        const double a = A.alpha[i], b = B.alpha[j];
        cnt += std::exp(-a * b * AB2 / (a + b)) >= 1.0e-14;
      }
    return cnt;
  };
  for (int cl = 0; cl < 3; ++cl) {
    std::vector<std::pair<int, std::pair<int, int>>> keyed;
    for (auto &ab : pl[cl]) keyed.push_back({live(ab), ab});
    std::stable_sort(keyed.begin(), keyed.end(),
                     [](const auto &x, const auto &y) { return x.first > y.first; });
    for (size_t k = 0; k < keyed.size(); ++k) pl[cl][k] = keyed[k].second;
  }
  int idx = 0;
  for (int cl = 0; cl < 3; ++cl) {
    h.class_off[cl] = idx;
    for (auto &ab : pl[cl]) {
      const HostShell &A = shells[ab.first], &B = shells[ab.second];
      const double *xa = &xyz[3 * A.atom], *xb = &xyz[3 * B.atom];
      double AB2 = 0;
      for (int k = 0; k < 3; ++k) AB2 += (xa[k] - xb[k]) * (xa[k] - xb[k]);
      h.shA.push_back(ab.first);
      h.shB.push_back(ab.second);
      h.aoA.push_back(A.ao0);
      h.aoB.push_back(B.ao0);
      h.mol.push_back(0);
      h.off.push_back((int)h.p.size());
      // the surviving primitive pairs, K descending (stable: ties keep the
      // (i, j) order): the pairs of a ket passing the screen against one bra
      // primitive are then a prefix of the ket's list, and the integral
      // kernels visit exactly the surviving primitive quartets
      std::vector<std::pair<double, std::pair<int, int>>> live_pp;
      for (int i = 0; i < A.nprim; ++i)
        for (int j = 0; j < B.nprim; ++j) {
          const double a = A.alpha[i], b = B.alpha[j];
          const double Kab = std::exp(-a * b * AB2 / (a + b));
          // a primitive pair whose EIJ is below 1e-14 fails the reference's
          // screen EIJ*EGH < 1e-14 (int2e.f90:257; int1e.f90:238) for any
          // partner, since EGH <= 1
          if (Kab >= 1.0e-14) live_pp.push_back({Kab, {i, j}});
        }
      std::stable_sort(live_pp.begin(), live_pp.end(),
                       [](const auto &x, const auto &y) { return x.first > y.first; });
      for (const auto &lp : live_pp) {
        const int i = lp.second.first, j = lp.second.second;
        double a = A.alpha[i], b = B.alpha[j], pp = a + b;
        double Kab = lp.first;
        double P[3], PA[3], PB[3];
        for (int k = 0; k < 3; ++k) {
          P[k] = (a * xa[k] + b * xb[k]) / pp;
          PA[k] = P[k] - xa[k];
          PB[k] = P[k] - xb[k];
        }
        h.p.push_back(pp);
        h.inv2p.push_back(1.0 / (2.0 * pp));
        h.beta.push_back(b);
        h.Px.push_back(P[0]); h.Py.push_back(P[1]); h.Pz.push_back(P[2]);
        h.PAx.push_back(PA[0]); h.PAy.push_back(PA[1]); h.PAz.push_back(PA[2]);
        h.PBx.push_back(PB[0]); h.PBy.push_back(PB[1]); h.PBz.push_back(PB[2]);
        h.K.push_back(Kab);
        double ca[2] = {A.cs[i], A.cp[i]}, cb[2] = {B.cs[j], B.cp[j]};
        for (int la = 0; la < 2; ++la)
          for (int lb = 0; lb < 2; ++lb) h.c4.push_back(Kab * ca[la] * cb[lb]);
      }
      ++idx;
    }
  }
  h.class_off[3] = idx;
  h.off.push_back((int)h.p.size());
}

// Append the class-cl pairs of one molecule's table to a batch table (whose
// pairs are ordered class first, then molecule), tagging them with `mol`.
void append_pairs_class(HostPairs &dst, const HostPairs &src, int cl, int mol) {
  if (dst.off.empty()) dst.off.push_back(0);
  for (int P = src.class_off[cl]; P < src.class_off[cl + 1]; ++P) {
    dst.shA.push_back(src.shA[P]);
    dst.shB.push_back(src.shB[P]);
    dst.aoA.push_back(src.aoA[P]);
    dst.aoB.push_back(src.aoB[P]);
    dst.mol.push_back(mol);
    for (int q = src.off[P]; q < src.off[P + 1]; ++q) {
      dst.p.push_back(src.p[q]);
      dst.inv2p.push_back(src.inv2p[q]);
      dst.beta.push_back(src.beta[q]);
      dst.Px.push_back(src.Px[q]); dst.Py.push_back(src.Py[q]); dst.Pz.push_back(src.Pz[q]);
      dst.PAx.push_back(src.PAx[q]); dst.PAy.push_back(src.PAy[q]); dst.PAz.push_back(src.PAz[q]);
      dst.PBx.push_back(src.PBx[q]); dst.PBy.push_back(src.PBy[q]); dst.PBz.push_back(src.PBz[q]);
      dst.K.push_back(src.K[q]);
      for (int k = 0; k < 4; ++k) dst.c4.push_back(src.c4[4 * q + k]);
    }
    dst.off.push_back((int)dst.p.size());  // end of this pair's primitives = start of the next
  }
}

// All arrays of the table in one device block (256-byte aligned pieces),
// staged through one pinned host buffer and one copy.  allocs != null: a new
// block recorded there (batches); null: the context's reusable "pair_table"
// buffer, after the work queued on the stream (which may read the previous
// table) has finished.
int upload_pairs(mq_ctx *c, const HostPairs &h, std::vector<void *> *allocs, PairTable &t) {
  t = PairTable{};
  for (int k = 0; k < 4; ++k) t.class_off[k] = h.class_off[k];
  t.npairs = (int)h.shA.size();
  t.npp = (int)h.p.size();
  std::vector<double> ones(h.shA.size(), 1.0e300);
  std::vector<float4> pf(4 * h.p.size());
  for (size_t i = 0; i < h.p.size(); ++i) {
    pf[4 * i] = make_float4((float)h.p[i], (float)h.inv2p[i], (float)h.K[i], (float)h.Px[i]);
    pf[4 * i + 1] = make_float4((float)h.Py[i], (float)h.Pz[i], (float)h.PAx[i], (float)h.PAy[i]);
    pf[4 * i + 2] = make_float4((float)h.PAz[i], (float)h.PBx[i], (float)h.PBy[i], (float)h.PBz[i]);
    pf[4 * i + 3] = make_float4((float)h.c4[4 * i], (float)h.c4[4 * i + 1], (float)h.c4[4 * i + 2],
                                (float)h.c4[4 * i + 3]);
  }
  struct Item {
    void **dst;
    const void *src;
    size_t bytes, off;
  };
  std::vector<Item> items;
  size_t total = 0;
  auto add = [&](auto *&dst, const auto &src) {
    using T = typename std::decay<decltype(src)>::type::value_type;
    const size_t bytes = src.size() * sizeof(T);
    items.push_back({(void **)&dst, (const void *)src.data(), bytes, total});
    total += (std::max<size_t>(bytes, 1) + 255) / 256 * 256;
  };
  add(t.shA, h.shA);
  add(t.shB, h.shB);
  add(t.pp_off, h.off);
  add(t.aoA, h.aoA);
  add(t.aoB, h.aoB);
  add(t.mol, h.mol);
  add(t.schwarz, ones);
  add(t.p, h.p);
  add(t.inv2p, h.inv2p);
  add(t.beta, h.beta);
  add(t.Px, h.Px); add(t.Py, h.Py); add(t.Pz, h.Pz);
  add(t.PAx, h.PAx); add(t.PAy, h.PAy); add(t.PAz, h.PAz);
  add(t.PBx, h.PBx); add(t.PBy, h.PBy); add(t.PBz, h.PBz);
  add(t.K, h.K);
  add(t.c4, h.c4);
  add(t.pf, pf);
  char *dev = nullptr;
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  if (allocs) {
    if (cudaMalloc((void **)&dev, total) != cudaSuccess) return set_err(c, MQ_ENOMEM, "cudaMalloc pair table");
    allocs->push_back(dev);
  } else {
    dev = (char *)buf(c, "pair_table", total);
    if (!dev) return MQ_ENOMEM;
  }
  if (c->pin_bytes < total) {
    if (c->pin) cudaFreeHost(c->pin);
    c->pin = nullptr;
    c->pin_bytes = 0;
    MQ_CUDA(c, cudaHostAlloc(&c->pin, total, cudaHostAllocDefault));
    c->pin_bytes = total;
  }
  char *st = (char *)c->pin;
  for (const Item &it : items) {
    if (it.bytes) memcpy(st + it.off, it.src, it.bytes);
    *it.dst = dev + it.off;
  }
  MQ_CUDA(c, cudaMemcpyAsync(dev, st, total, cudaMemcpyHostToDevice, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));  // the staging buffer is reused by the next upload
  return MQ_OK;
}

int build_pairs(mq_ctx *c) {
  free_pairs(c);
  HostPairs h;
  pairs_host(c->shells, c->xyz, h);
  MQ_TRY(upload_pairs(c, h, nullptr, c->pt));
  c->pair_class_count = {h.class_off[1] - h.class_off[0], h.class_off[2] - h.class_off[1],
                         h.class_off[3] - h.class_off[2]};
  c->hp_shA = h.shA;
  c->hp_shB = h.shB;
  c->hp_aoA = h.aoA;
  c->hp_aoB = h.aoB;
  for (int k = 0; k < 4; ++k) c->hp_class_off[k] = h.class_off[k];
  c->qs.valid = 0;
  c->qs.tables_valid = 0;
  return MQ_OK;
}

// F_m(T) for T = 0.0, 0.1, ..., 36.0 and m = 0..12 by the power series
//   F_m(T) = e^-T sum_k (2T)^k / ((2m+1)(2m+3)...(2m+2k+1))
// at m = 12 in long double, then downward recursion F_m = (2T F_{m+1} + e^-T)/(2m+1).
// The table is a constant: computed once per process (the long-double series
// is slow where long double is a software type, as on aarch64).
static void tight_boys_compute(std::vector<double> &tab);
void tight_boys_table(std::vector<double> &tab) {
  static std::once_flag once;
  static std::vector<double> cached;
  std::call_once(once, [] { tight_boys_compute(cached); });
  tab = cached;
}

// The tight table as the kernels read it: F_m(Tk) [TIGHT_NT][TIGHT_NM], the grid
// values Tk, then for m = 0..BOYS_SCALED_M-1 the Taylor coefficients of F_m
// about Tk, F_{m+k}(Tk) / k! for k = 0..8 ([m][TIGHT_NT][9]).
void tight_boys_device_table(std::vector<double> &tab) {
  std::vector<double> f;
  tight_boys_table(f);
  tab = f;
  for (int k = 0; k < TIGHT_NT; ++k) tab.push_back(k / 10.0);
  for (int m = 0; m < BOYS_SCALED_M; ++m)
    for (int t = 0; t < TIGHT_NT; ++t) {
      double fact = 1.0;
      for (int k = 0; k < 9; ++k) {
        if (k > 0) fact *= k;
        tab.push_back(f[(size_t)t * TIGHT_NM + m + k] / fact);
      }
    }
}

static void tight_boys_compute(std::vector<double> &tab) {
  tab.assign((size_t)TIGHT_NT * TIGHT_NM, 0.0);
  for (int it = 0; it < TIGHT_NT; ++it) {
    long double T = it / 10.0L;
    const int m = TIGHT_NM - 1;
    long double term = 1.0L / (2 * m + 1), sum = term;
    for (int k = 1; k < 2000; ++k) {
      term *= 2.0L * T / (2 * m + 2 * k + 1);
      sum += term;
      if (term < 1e-22L * sum) break;
    }
    long double e = expl(-T);
    long double F[TIGHT_NM];
    F[m] = e * sum;
    for (int j = m - 1; j >= 0; --j) F[j] = (2.0L * T * F[j + 1] + e) / (2.0L * j + 1.0L);
    for (int j = 0; j < TIGHT_NM; ++j) tab[(size_t)it * TIGHT_NM + j] = (double)F[j];
  }
}

}  // namespace mq

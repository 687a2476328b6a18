/*
 * oracle.c -- CPU restatement of myQC's Hartree-Fock/MP2 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the GB300
 * library: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it.  The product path (libmyqc) never links or calls it.
 *
 * It follows the reference (jhthorpe/myQC, Fortran 90) statement for statement
 * where values depend on it, single-threaded like the reference:
 *   Boys F_j(T)          src/integrals/auxilary.f90:85-215,265-285
 *   Hermite E coeffs     src/integrals/auxilary.f90:349-536 (getcoef/lrec/rrec)
 *   pair lists (getDk)   src/integrals/auxilary.f90:541-633, gtoD :704-726
 *   R_{NLM}^{(j)}        src/integrals/auxilary.f90:22-80 (RNLMj)
 *   ERIs (proc2e)        src/integrals/int2e.f90:78-351, clmnew :618-726,
 *                        fillsym :540-613
 *   S, T, V (proc1e)     src/integrals/int1e.f90:132-582
 *   density              src/dens/dens.f90:115-124 (RHF), :213-228 (UHF)
 *   G digestion          src/I2G/RHFI2G.f90:80-90, src/I2G/UHFI2G.f90:80-93
 *   quarter transforms   src/ao2mo/ao2mo.f90:1306-1439 (idx1..idx4_trans)
 *   MP2 sums             src/mp2/mp2.f90:79-144 (RHF), :154-232 (UHF)
 *
 * Two modes:
 *   mode 0 "reference"  pi as the reference declares it (a REAL(8) PARAMETER
 *                        initialised from a default-REAL literal, i.e. the
 *                        float value 3.1415927410125732), the Boys function
 *                        from the Ftab table with the reference's three
 *                        regimes and BoysG polynomials.
 *   mode 1 "tight"      true pi and a Boys function accurate to ~1e-15
 *                        (power series + downward recursion below T=50,
 *                        erf-based F0 + upward recursion above).
 *
 * Compiled with -ffp-contract=off so that products and sums round the way the
 * reference's unfused gfortran code does.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI_REF ((double)3.1415926535897931f) /* float pi, src/integrals/auxilary.f90:169 */
#define PI_TRUE 3.14159265358979323846

static double pi_of(int mode) { return mode == 0 ? PI_REF : PI_TRUE; }

/* factR8, auxilary.f90:290-312 */
static double factR8(int n) {
  double v = 1.0;
  for (int i = n; i >= 2; --i) v = v * i;
  return v;
}

static double ipow(double x, int k) {
  double r = 1.0;
  for (int i = 0; i < k; ++i) r *= x;
  return r;
}

/* BoysG, auxilary.f90:265-285.  The reference leaves the result undefined for
 * T >= 30; this restatement uses 0.490 there (its effect on F0 is below
 * e^-30/30 ~ 3e-15). */
static double boysG(double T) {
  if (T >= 12.0 && T < 15.0)
    return 0.4999489092 - 0.2473631686 * pow(T, -1.0) + 0.321180909 * pow(T, -2.0) -
           0.3811559346 * pow(T, -3.0);
  if (T >= 15.0 && T < 18.0) return 0.4998436875 - 0.24249438 * pow(T, -1.0) + 0.24642845 * pow(T, -2.0);
  if (T >= 18.0 && T < 24.0) return 0.499093162 - 0.2152832 * pow(T, -1.0);
  return 0.490;
}

/* Boys / Boys1 / Boys2 / Boys3, auxilary.f90:85-215.  Ft is the 121x23
 * column-major table Ft(0:120,0:22) (T fastest). */
static int boys_ref(double *Fj, int Q, double T, const double *Ft) {
  if (Q > 16) return -1;
  if (T >= 0 && T < 12) {
    for (int j = 0; j <= Q; ++j) Fj[j] = 0.0;
    long Tk = lround(T * 10);
    for (int k = 0; k <= 6; ++k)
      Fj[Q] = Fj[Q] + Ft[Tk + 121 * (Q + k)] * ipow(Tk / 10.0 - T, k) / factR8(k);
    for (int j = Q - 1; j >= 0; --j) Fj[j] = (2 * T * Fj[j + 1] + exp(-T)) / (2.0 * j + 1.0);
  } else if (T >= 12 && T < 2 * Q + 36) {
    double g = boysG(T);
    Fj[0] = 0.5 * pow(PI_REF, 0.5) * pow(T, -0.5) - exp(-T) * g / T;
    for (int j = 1; j <= Q; ++j) Fj[j] = pow(2.0 * T, -1.0) * ((2.0 * (j - 1) + 1) * Fj[j - 1] - exp(-T));
  } else if (T >= 2 * Q + 36) {
    Fj[0] = 0.5 * pow(PI_REF, 0.5) * pow(T, -0.5);
    for (int j = 1; j <= Q; ++j) Fj[j] = pow(2.0 * T, -1.0) * (2.0 * (j - 1) + 1.0) * Fj[j - 1];
  } else {
    return -2;
  }
  return 0;
}

/* Accurate F_j(T), j=0..Q (oracle B).  Series
 *   F_m(T) = e^-T sum_k (2T)^k / ((2m+1)(2m+3)...(2m+2k+1))
 * for the top order then downward recursion; for T >= 50 the exact
 * F_0 = sqrt(pi/T) erf(sqrt T)/2 and upward recursion (stable for T >> m). */
static int boys_tight(double *Fj, int Q, double T) {
  if (T < 50.0) {
    double term = 1.0 / (2 * Q + 1), sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * T / (2 * Q + 2 * k + 1);
      sum += term;
      if (term < 1e-18 * sum) break;
    }
    double e = exp(-T);
    Fj[Q] = e * sum;
    for (int j = Q - 1; j >= 0; --j) Fj[j] = (2.0 * T * Fj[j + 1] + e) / (2.0 * j + 1.0);
  } else {
    double e = exp(-T);
    Fj[0] = 0.5 * sqrt(PI_TRUE / T) * erf(sqrt(T));
    for (int j = 1; j <= Q; ++j) Fj[j] = ((2.0 * j - 1.0) * Fj[j - 1] - e) / (2.0 * T);
  }
  return 0;
}

static int boys(int mode, double *Fj, int Q, double T, const double *Ft) {
  return mode == 0 ? boys_ref(Fj, Q, T, Ft) : boys_tight(Fj, Q, T);
}

/* exported for tests */
int orc_boys(int mode, double T, int Q, const double *Ft, double *Fj) { return boys(mode, Fj, Q, T, Ft); }

/* ------------------------------------------------------------------ */
/* Hermite expansion coefficients E^{j,k}_i per Cartesian axis: the values
 * getcoef/lrec/rrec (auxilary.f90:349-536) memoise.  Each (j,k) entry uses
 * the reference's own rule: j<=k raises k from (j,k-1) with PB, otherwise
 * raises j from (j-1,k) with PA.  Out-of-range i (i<0 or i>j+k) is zero.
 * The reference calls getcoef with amax=la+2 / bmax=lb+2 (int2e.f90:227,261):
 * with that reach every entry getDk reads is visited, so the values are the
 * complete standard table computed here. */
#define EJ 4            /* j,k in 0..3 */
#define EI 8            /* i in 0..7  */
typedef struct { double e[3][EI][EJ][EJ]; } ecoef_t;

static double eget(const ecoef_t *E, int l, int i, int j, int k) {
  if (i < 0 || j < 0 || k < 0 || i > j + k) return 0.0;
  return E->e[l][i][j][k];
}

static void getcoef(ecoef_t *E, const double PA[3], const double PB[3], double pp, int amax, int bmax) {
  memset(E, 0, sizeof(*E));
  for (int l = 0; l < 3; ++l) {
    E->e[l][0][0][0] = 1.0;
    for (int s = 1; s <= amax + bmax; ++s)
      for (int j = 0; j <= amax; ++j) {
        int k = s - j;
        if (k < 0 || k > bmax) continue;
        for (int i = 0; i <= s; ++i) {
          double v;
          if (j <= k)
            v = eget(E, l, i - 1, j, k - 1) / (2.0 * pp) + PB[l] * eget(E, l, i, j, k - 1) +
                (i + 1) * eget(E, l, i + 1, j, k - 1);
          else
            v = eget(E, l, i - 1, j - 1, k) / (2.0 * pp) + PA[l] * eget(E, l, i, j - 1, k) +
                (i + 1) * eget(E, l, i + 1, j - 1, k);
          E->e[l][i][j][k] = v;
        }
      }
  }
}

/* gtoD, auxilary.f90:704-726 */
static double gtoD(int l, double a, double pi) {
  if (l == 0) return pow(2.0 * a / pi, 3.0 / 4.0);
  if (l == 1) return pow(128.0 * pow(a, 5.0) / pow(pi, 3.0), 1.0 / 4.0);
  return pow(2048.0 * pow(a, 7.0) / (9.0 * pow(pi, 3.0)), 1.0 / 4.0);
}

/* ------------------------------------------------------------------ */
/* Basis bookkeeping in the reference's flat arrays (src/myQC/basis.f90):
 *   basinfo(0)=OpS, basinfo(1)=norb, then per AO [n, l, ori, nprim, centre]
 *   setinfo(0)=nset, setinfo(1)=setl, then per set [#AO, lmax, centre, AO...]
 *   bas(OpS*set + slot) contraction coefficient, set(set) exponent.         */
typedef struct {
  int nset, setl, ops, norb;
  const double *bas, *set;
  const int *basinfo, *setinfo;
  const double *xyz; /* xyz(0:nnuc-1,0:2), column-major */
  int nnuc;
  const int *atoms;
  const double *Ft;
  int mode;
} sys_t;

static int set_nao(const sys_t *s, int a) { return s->setinfo[1 + a * s->setl + 1]; }
static int set_lmax(const sys_t *s, int a) { return s->setinfo[1 + a * s->setl + 2]; }
static int set_ctr(const sys_t *s, int a) { return s->setinfo[1 + a * s->setl + 3]; }
static int set_ao(const sys_t *s, int a, int i) { return s->setinfo[1 + a * s->setl + 4 + i]; }
static int ao_l(const sys_t *s, int o) { return s->basinfo[1 + 5 * o + 2]; }
static int ao_ori(const sys_t *s, int o) { return s->basinfo[1 + 5 * o + 3]; }
static double X(const sys_t *s, int atom, int c) { return s->xyz[atom + s->nnuc * c]; }

static void ao_lmn(const sys_t *s, int o, int out[3]) {
  int ori = ao_ori(s, o), l = ao_l(s, o);
  if (ori == -1) { out[0] = out[1] = out[2] = l; }
  else { out[0] = out[1] = out[2] = 0; out[ori] = l; }
}

/* one primitive-set pair: the values proc2e builds at int2e.f90:215-229 */
typedef struct {
  double p, P[3], EIJ;
  int la, lb;
  int nk;
  double *Dk;
  int *N, *L, *M, *oa, *ob;
} pair_t;

/* getDk, auxilary.f90:541-633 */
static void getDk(const sys_t *s, const ecoef_t *E, int a, int b, double aa, double bb, double EIJ, pair_t *pr) {
  const double tol = 0.1e-15;
  double pi = pi_of(s->mode);
  int cap = 16 * 27;
  pr->Dk = (double *)malloc(sizeof(double) * cap);
  pr->N = (int *)malloc(sizeof(int) * cap * 5);
  pr->L = pr->N + cap; pr->M = pr->L + cap; pr->oa = pr->M + cap; pr->ob = pr->oa + cap;
  pr->nk = 0;
  for (int i = 0; i < set_nao(s, a); ++i) {
    int orba = set_ao(s, a, i), ll[3];
    ao_lmn(s, orba, ll);
    for (int j = 0; j < set_nao(s, b); ++j) {
      int orbb = set_ao(s, b, j), rr[3];
      ao_lmn(s, orbb, rr);
      int Nmax = ll[0] + rr[0], Lmax = ll[1] + rr[1], Mmax = ll[2] + rr[2];
      for (int M = 0; M <= Mmax; ++M) {
        if (fabs(eget(E, 2, M, ll[2], rr[2])) < tol) continue;
        for (int L = 0; L <= Lmax; ++L) {
          if (fabs(eget(E, 1, L, ll[1], rr[1])) < tol) continue;
          for (int N = 0; N <= Nmax; ++N) {
            if (fabs(eget(E, 0, N, ll[0], rr[0])) < tol) continue;
            int k = pr->nk++;
            double d = eget(E, 0, N, ll[0], rr[0]) * eget(E, 1, L, ll[1], rr[1]) * eget(E, 2, M, ll[2], rr[2]);
            d = d * EIJ * gtoD(ao_l(s, orba), aa, pi) * gtoD(ao_l(s, orbb), bb, pi);
            d = d * s->bas[a * s->ops + i] * s->bas[b * s->ops + j];
            pr->Dk[k] = d;
            pr->N[k] = N; pr->L[k] = L; pr->M[k] = M;
            pr->oa[k] = orba; pr->ob[k] = orbb;
          }
        }
      }
    }
  }
}

static void make_pair(const sys_t *s, int a, int b, int amax_extra, pair_t *pr, ecoef_t *Eout) {
  double aa = s->set[a], bb = s->set[b];
  int u = set_ctr(s, a), v = set_ctr(s, b);
  double p = aa + bb, mm = aa * bb, AB[3], PA[3], PB[3];
  for (int i = 0; i < 3; ++i) {
    AB[i] = X(s, u, i) - X(s, v, i);
    pr->P[i] = (aa * X(s, u, i) + bb * X(s, v, i)) / p;
    PA[i] = pr->P[i] - X(s, u, i);
    PB[i] = pr->P[i] - X(s, v, i);
  }
  pr->p = p;
  pr->EIJ = exp(-mm * (AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2]) / p);
  pr->la = set_lmax(s, a);
  pr->lb = set_lmax(s, b);
  ecoef_t E;
  getcoef(&E, PA, PB, p, pr->la + amax_extra, pr->lb + 2);
  getDk(s, &E, a, b, aa, bb, pr->EIJ, pr);
  if (Eout) *Eout = E;
}

static void free_pair(pair_t *pr) { free(pr->Dk); free(pr->N); }

/* R_{NLM}^{(j)} table, the values RNLMj (auxilary.f90:22-80) memoises:
 * R(0,0,0,j) = (-2 al)^j F_j and the N, then L, then M reduction. */
typedef struct { int nN, nL, nM, nJ; double *v; } rtab_t;
#define RIDX(r, N, L, M, j) ((((j) * (r)->nM + (M)) * (r)->nL + (L)) * (r)->nN + (N))

static double rget(const rtab_t *r, int N, int L, int M, int j) {
  if (N < 0 || L < 0 || M < 0) return 0.0;
  return r->v[RIDX(r, N, L, M, j)];
}

static void rfill(rtab_t *r, int Nmax, int Lmax, int Mmax, int Jmax, double a, double b, double c, double al,
                  const double *Fj) {
  r->nN = Nmax + 1; r->nL = Lmax + 1; r->nM = Mmax + 1; r->nJ = Jmax + 1;
  /* order: decreasing j so that level j+1 is complete before level j */
  for (int j = Jmax; j >= 0; --j)
    for (int M = 0; M <= Mmax; ++M)
      for (int L = 0; L <= Lmax; ++L)
        for (int N = 0; N <= Nmax; ++N) {
          if (N + L + M > Jmax - j) { r->v[RIDX(r, N, L, M, j)] = 0.0; continue; }
          double v;
          if (N == 0 && L == 0 && M == 0) v = ipow(-2.0 * al, j) * Fj[j];
          else if (N != 0) v = a * rget(r, N - 1, L, M, j + 1) + (N - 1) * rget(r, N - 2, L, M, j + 1);
          else if (L != 0) v = b * rget(r, 0, L - 1, M, j + 1) + (L - 1) * rget(r, 0, L - 2, M, j + 1);
          else v = c * rget(r, 0, 0, M - 1, j + 1) + (M - 1) * rget(r, 0, 0, M - 2, j + 1);
          r->v[RIDX(r, N, L, M, j)] = v;
        }
}

/* ------------------------------------------------------------------ */
/* proc2e + clmnew + fillsym (int2e.f90:78-351, 540-613, 618-726).
 * XX is n^4, XX(i,j,g,h) at i + n*(j + n*(g + n*h)).  Returns 0 or <0. */
int orc_int2e(int nset, int setl, int ops, int norb, const double *bas, const double *set, const int *basinfo,
              const int *setinfo, int nnuc, const double *xyz, const double *Ft, int mode, double *XX) {
  sys_t S = {nset, setl, ops, norb, bas, set, basinfo, setinfo, xyz, nnuc, NULL, Ft, mode};
  const sys_t *s = &S;
  size_t n = (size_t)norb, n4 = n * n * n * n;
  double pi = pi_of(mode);
  for (size_t i = 0; i < n4; ++i) XX[i] = 0.0;
  pair_t *pairs = (pair_t *)calloc((size_t)nset * nset, sizeof(pair_t));
  for (int a = 0; a < nset; ++a)
    for (int b = 0; b < nset; ++b) make_pair(s, a, b, 2, &pairs[a * nset + b], NULL);
  double Fj[32];
  rtab_t R;
  R.v = (double *)malloc(sizeof(double) * 5 * 5 * 5 * 13);
  for (int a = 0; a < nset; ++a)
    for (int b = 0; b < nset; ++b) {
      const pair_t *ab = &pairs[a * nset + b];
      for (int c = 0; c < nset; ++c)
        for (int d = 0; d < nset; ++d) {
          const pair_t *cd = &pairs[c * nset + d];
          if (cd->EIJ * ab->EIJ < 1.0e-14) continue; /* int2e.f90:257 */
          double p = ab->p, q = cd->p, PQ[3];
          for (int j = 0; j < 3; ++j) PQ[j] = ab->P[j] - cd->P[j];
          int Lsum = ab->la + ab->lb + cd->la + cd->lb;
          int Q = 3 * Lsum; /* Nmax+Lmax+Mmax, int2e.f90:654-658 */
          double ll = 2 * pow(pi, 2.5) / (p * q * sqrt(p + q));
          double TT = p * q * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]) / (p + q);
          if (boys(mode, Fj, Q, TT, Ft) != 0) { free(R.v); return -1; }
          rfill(&R, Lsum, Lsum, Lsum, Q, PQ[0], PQ[1], PQ[2], p * q / (p + q), Fj);
          for (int k = 0; k < ab->nk; ++k) {
            int i = ab->oa[k], j = ab->ob[k];
            if (j < i) continue;
            for (int kp = 0; kp < cd->nk; ++kp) {
              int g = cd->oa[kp], h = cd->ob[kp];
              if (h < g) continue;
              if (g * norb + h < i * norb + j) continue;
              int Np = cd->N[kp], Lp = cd->L[kp], Mp = cd->M[kp];
              double sign = ((Np + Lp + Mp) & 1) ? -1.0 : 1.0;
              double r = rget(&R, ab->N[k] + Np, ab->L[k] + Lp, ab->M[k] + Mp, 0);
              size_t idx = (size_t)i + n * ((size_t)j + n * ((size_t)g + n * (size_t)h));
              XX[idx] = XX[idx] + sign * ll * cd->Dk[kp] * r * ab->Dk[k];
            }
          }
        }
    }
  free(R.v);
  for (int i = 0; i < nset * nset; ++i) free_pair(&pairs[i]);
  free(pairs);
  /* fillsym over the canonical quartets, int2e.f90:290-304 */
#define XI(i, j, g, h) XX[(size_t)(i) + n * ((size_t)(j) + n * ((size_t)(g) + n * (size_t)(h)))]
  for (int i = 0; i < norb; ++i)
    for (int j = i; j < norb; ++j) {
      for (int h = j; h < norb; ++h) {
        int g = i;
        double v = XI(i, j, g, h);
        XI(i, j, h, g) = v; XI(j, i, g, h) = v; XI(j, i, h, g) = v;
        XI(g, h, i, j) = v; XI(g, h, j, i) = v; XI(h, g, i, j) = v; XI(h, g, j, i) = v;
      }
      for (int g = i + 1; g < norb; ++g)
        for (int h = g; h < norb; ++h) {
          double v = XI(i, j, g, h);
          XI(i, j, h, g) = v; XI(j, i, g, h) = v; XI(j, i, h, g) = v;
          XI(g, h, i, j) = v; XI(g, h, j, i) = v; XI(h, g, i, j) = v; XI(h, g, j, i) = v;
        }
    }
#undef XI
  return 0;
}

/* ------------------------------------------------------------------ */
/* proc1e: overlap, kinetic, coulomb (int1e.f90:132-582).  S and H are
 * n x n column-major. */
int orc_int1e(int nset, int setl, int ops, int norb, const double *bas, const double *set, const int *basinfo,
              const int *setinfo, int nnuc, const int *atoms, const double *xyz, const double *Ft, int mode,
              double *Sm, double *Hm) {
  sys_t S = {nset, setl, ops, norb, bas, set, basinfo, setinfo, xyz, nnuc, atoms, Ft, mode};
  const sys_t *s = &S;
  int n = norb;
  double pi = pi_of(mode);
  for (int i = 0; i < n * n; ++i) Sm[i] = Hm[i] = 0.0;
  double Fj[32];
  rtab_t R;
  R.v = (double *)malloc(sizeof(double) * 5 * 5 * 5 * 13);
  for (int a = 0; a < nset; ++a)
    for (int b = 0; b < nset; ++b) {
      pair_t pr;
      ecoef_t E;
      double aa = set[a], bb = set[b];
      /* int1e calls getcoef with amax = la, bmax = lb + 2 (int1e.f90:213-222) */
      make_pair(s, a, b, 0, &pr, &E);
      if (pr.EIJ < 1.0e-14) { free_pair(&pr); continue; } /* int1e.f90:238-241 */
      double p = pr.p, EIJ = pr.EIJ;
      for (int i = 0; i < set_nao(s, a); ++i) {
        int oa = set_ao(s, a, i), la[3];
        ao_lmn(s, oa, la);
        for (int j = 0; j < set_nao(s, b); ++j) {
          int ob = set_ao(s, b, j), lb[3];
          ao_lmn(s, ob, lb);
          double ca = bas[a * ops + i], cb = bas[b * ops + j];
          double gA = gtoD(ao_l(s, oa), aa, pi), gB = gtoD(ao_l(s, ob), bb, pi);
          /* overlap, int1e.f90:321-386 */
          double t = EIJ * pow(pi / p, 3.0 / 2.0) * ca * cb;
          t = t * gA;
          t = t * gB;
          t = t * eget(&E, 0, 0, la[0], lb[0]) * eget(&E, 1, 0, la[1], lb[1]) * eget(&E, 2, 0, la[2], lb[2]);
          Sm[oa + n * ob] += t;
          /* kinetic, int1e.f90:391-474 */
          double val = 0.0;
          for (int ax = 0; ax < 3; ++ax) {
            int nb = lb[ax], na = la[ax];
            double tt = nb * (nb - 1) * eget(&E, ax, 0, na, nb - 2);
            tt = tt - 2.0 * bb * nb * eget(&E, ax, 0, na, nb);
            tt = tt - 2.0 * bb * (nb + 1) * eget(&E, ax, 0, na, nb);
            tt = tt + 4.0 * bb * bb * eget(&E, ax, 0, na, nb + 2);
            int o1 = (ax + 1) % 3, o2 = (ax + 2) % 3;
            int lo = o1 < o2 ? o1 : o2, hi = o1 < o2 ? o2 : o1;
            tt = tt * eget(&E, lo, 0, la[lo], lb[lo]) * eget(&E, hi, 0, la[hi], lb[hi]);
            val = val + tt;
          }
          val = val * (-0.5) * EIJ * pow(pi / p, 3.0 / 2.0);
          val = val * ca * cb;
          val = val * gA;
          val = val * gB;
          Hm[oa + n * ob] += val;
        }
      }
      /* coulomb, int1e.f90:479-582 */
      int Lsum = pr.la + pr.lb, Q = 3 * Lsum;
      for (int c = 0; c < nnuc; ++c) {
        double CP[3];
        for (int i = 0; i < 3; ++i) CP[i] = X(s, c, i) - pr.P[i];
        double TT = p * (CP[0] * CP[0] + CP[1] * CP[1] + CP[2] * CP[2]);
        if (boys(mode, Fj, Q, TT, Ft) != 0) { free(R.v); free_pair(&pr); return -1; }
        rfill(&R, Lsum, Lsum, Lsum, Q, -CP[0], -CP[1], -CP[2], p, Fj);
        for (int k = 0; k < pr.nk; ++k) {
          double t = atoms[c] * (2.0 * pi / p) * rget(&R, pr.N[k], pr.L[k], pr.M[k], 0) * pr.Dk[k];
          Hm[pr.oa[k] + n * pr.ob[k]] -= t;
        }
      }
      free_pair(&pr);
    }
  free(R.v);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Dipole integrals <u| r_c |v> about the origin, int1p.f90 proc1p/dipole
 * (src/integrals/int1p.f90:150-300): every set pair (a, b) with EIJ >= 1e-14,
 * E_0 and E_1 of getcoef_dipole (auxilary.f90:649-696; the standard Hermite
 * table), P_c = EIJ (pi/p)^(3/2) c_a c_b N_a N_b E^y_0 E^z_0 (E^x_1 + P_x E^x_0)
 * for c = x and likewise for y, z.  Both pi constants of int1p are default-real
 * literals, so mode 0 uses the float-valued pi in both.  Px: 3 n x n matrices
 * (x, y, z), column-major. */
int orc_int1p(int nset, int setl, int ops, int norb, const double *bas, const double *set, const int *basinfo,
              const int *setinfo, int nnuc, const int *atoms, const double *xyz, int mode, double *Px) {
  sys_t S = {nset, setl, ops, norb, bas, set, basinfo, setinfo, xyz, nnuc, atoms, NULL, mode};
  const sys_t *s = &S;
  const int n = norb;
  const double pi = pi_of(mode);
  for (int i = 0; i < 3 * n * n; ++i) Px[i] = 0.0;
  for (int a = 0; a < nset; ++a)
    for (int b = 0; b < nset; ++b) {
      pair_t pr;
      ecoef_t E;
      const double aa = set[a], bb = set[b];
      make_pair(s, a, b, 0, &pr, &E);
      if (pr.EIJ < 1.0e-14) { free_pair(&pr); continue; } /* int1p.f90 EIJ screen */
      const double p = pr.p, EIJ = pr.EIJ;
      for (int i = 0; i < set_nao(s, a); ++i) {
        int oa = set_ao(s, a, i), la[3];
        ao_lmn(s, oa, la);
        for (int j = 0; j < set_nao(s, b); ++j) {
          int ob = set_ao(s, b, j), lb[3];
          ao_lmn(s, ob, lb);
          const double w = EIJ * pow(pi / p, 3.0 / 2.0) * bas[a * ops + i] * bas[b * ops + j] *
                           gtoD(ao_l(s, oa), aa, pi) * gtoD(ao_l(s, ob), bb, pi);
          for (int c = 0; c < 3; ++c) {
            const int o1 = (c + 1) % 3, o2 = (c + 2) % 3;
            double t = w * eget(&E, o1 < o2 ? o1 : o2, 0, la[o1 < o2 ? o1 : o2], lb[o1 < o2 ? o1 : o2]) *
                       eget(&E, o1 < o2 ? o2 : o1, 0, la[o1 < o2 ? o2 : o1], lb[o1 < o2 ? o2 : o1]);
            t = t * (eget(&E, c, 1, la[c], lb[c]) + pr.P[c] * eget(&E, c, 0, la[c], lb[c]));
            Px[(size_t)c * n * n + oa + (size_t)n * ob] += t;
          }
        }
      }
      free_pair(&pr);
    }
  return 0;
}

/* ------------------------------------------------------------------ */
/* dens.f90:115-124 (RHF, factor 2) and :213-228 (UHF) */
void orc_density(int n, int nocc, const double *C, double factor, double *D) {
  for (int v = 0; v < n; ++v)
    for (int u = 0; u < n; ++u) {
      double t = 0.0;
      for (int i = 0; i < nocc; ++i) t = t + C[u + n * i] * C[v + n * i];
      D[u + n * v] = t * factor;
    }
}

/* RHFI2G.f90:80-90 */
void orc_fock_rhf(int n, const double *XX, const double *D, double *G) {
  size_t N = (size_t)n;
#define XI(i, j, g, h) XX[(size_t)(i) + N * ((size_t)(j) + N * ((size_t)(g) + N * (size_t)(h)))]
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double t = 0.0;
      for (int l = 0; l < n; ++l)
        for (int k = 0; k < n; ++k)
          t = t + D[k + n * l] * (XI(i, j, k, l) - 0.25 * XI(i, k, j, l) - 0.25 * XI(i, l, j, k));
      G[i + n * j] = t;
    }
}

/* UHFI2G.f90:80-93 */
void orc_fock_uhf(int n, const double *XX, const double *Da, const double *Db, double *Ga, double *Gb) {
  size_t N = (size_t)n;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double ta = 0.0, tb = 0.0;
      for (int l = 0; l < n; ++l)
        for (int k = 0; k < n; ++k) {
          double dt = Da[k + n * l] + Db[k + n * l];
          ta = ta + dt * XI(i, j, k, l) - Da[k + n * l] * XI(i, k, j, l);
          tb = tb + dt * XI(i, j, k, l) - Db[k + n * l] * XI(i, k, j, l);
        }
      Ga[i + n * j] = ta;
      Gb[i + n * j] = tb;
    }
}
#undef XI

/* ------------------------------------------------------------------ */
/* (ia|jb) by the four naive quarter transforms, ao2mo.f90:1306-1439, in the
 * order the RHF/UHF drivers call them (i, a, j, b).  Ci: n x no1 (first
 * occupied block), Ca: n x nv1, Cj: n x no2, Cb: n x nv2, all column-major
 * with leading dimension n.  Out: Om(0:no1-1,0:nv1-1,0:no2-1,0:nv2-1). */
int orc_ao2mo(int n, const double *XX, const double *Ci, int no1, const double *Ca, int nv1, const double *Cj,
              int no2, const double *Cb, int nv2, double *Om) {
  size_t N = (size_t)n;
  double *Lm = (double *)malloc(sizeof(double) * no1 * N * N * N);
  double *Mm = (double *)malloc(sizeof(double) * no1 * nv1 * N * N);
  double *Nm = (double *)malloc(sizeof(double) * no1 * nv1 * no2 * N);
  if (!Lm || !Mm || !Nm) { free(Lm); free(Mm); free(Nm); return -1; }
  /* idx1: Lm(p,q,r,s) = sum_t A(t,q,r,s) x(t,p) */
  for (int p = 0; p < no1; ++p)
    for (int q = 0; q < n; ++q)
      for (int r = 0; r < n; ++r)
        for (int s = 0; s < n; ++s) {
          double t = 0.0;
          for (int u = 0; u < n; ++u) t = t + XX[u + N * (q + N * (r + N * s))] * Ci[u + N * p];
          Lm[p + no1 * (q + N * (r + N * s))] = t;
        }
  /* idx2: Mm(p,q,r,s) = sum_t Lm(p,t,r,s) x(t,q) */
  for (int p = 0; p < no1; ++p)
    for (int q = 0; q < nv1; ++q)
      for (int r = 0; r < n; ++r)
        for (int s = 0; s < n; ++s) {
          double t = 0.0;
          for (int u = 0; u < n; ++u) t = t + Lm[p + no1 * (u + N * (r + N * s))] * Ca[u + N * q];
          Mm[p + no1 * (q + nv1 * (r + N * s))] = t;
        }
  /* idx3: Nm(p,q,r,s) = sum_t Mm(p,q,t,s) x(t,r) */
  for (int p = 0; p < no1; ++p)
    for (int q = 0; q < nv1; ++q)
      for (int r = 0; r < no2; ++r)
        for (int s = 0; s < n; ++s) {
          double t = 0.0;
          for (int u = 0; u < n; ++u) t = t + Mm[p + no1 * (q + nv1 * (u + N * s))] * Cj[u + N * r];
          Nm[p + no1 * (q + nv1 * (r + no2 * s))] = t;
        }
  /* idx4: Om(p,q,r,s) = sum_t Nm(p,q,r,t) x(t,s) */
  for (int p = 0; p < no1; ++p)
    for (int q = 0; q < nv1; ++q)
      for (int r = 0; r < no2; ++r)
        for (int s = 0; s < nv2; ++s) {
          double t = 0.0;
          for (int u = 0; u < n; ++u) t = t + Nm[p + no1 * (q + nv1 * (r + no2 * u))] * Cb[u + N * s];
          Om[p + no1 * (q + nv1 * (r + no2 * s))] = t;
        }
  free(Lm); free(Mm); free(Nm);
  return 0;
}

/* mp2_rhf, mp2.f90:79-144, reading Om(i,a,j,b) in the record order the
 * reference streams ijab_AB (i outer, j inner, each record v x v, a fastest).
 * out[0] = E(AA) (sum1), out[1] = E(AB) (sum2), out[2] = E(MBPT2). */
void orc_mp2_rhf(int nocc, int nvrt, const double *eig, const double *Om, double *out) {
  int ntot = nocc + nvrt;
  double sum1 = 0.0, sum2 = 0.0;
#define OM(i, a, j, b) Om[(i) + nocc * ((a) + nvrt * ((j) + nocc * (b)))]
#define DEN(i, j, a, b) (eig[i] + eig[j] - eig[(a) + nocc] - eig[(b) + nocc])
  for (int i = 0; i <= nocc - 2; ++i) {
    for (int j = 0; j <= i; ++j)
      for (int a = 0; a < nvrt; ++a)
        for (int b = 0; b < nvrt; ++b) sum2 = sum2 + OM(i, a, j, b) * OM(i, a, j, b) / DEN(i, j, a, b);
    for (int j = i + 1; j < nocc; ++j) {
      for (int a = 0; a <= nvrt - 2; ++a) {
        for (int b = 0; b <= a; ++b) sum2 = sum2 + OM(i, a, j, b) * OM(i, a, j, b) / DEN(i, j, a, b);
        for (int b = a + 1; b < nvrt; ++b) {
          sum2 = sum2 + OM(i, a, j, b) * OM(i, a, j, b) / DEN(i, j, a, b);
          double x = OM(i, a, j, b) - OM(i, b, j, a);
          sum1 = sum1 + x * x / DEN(i, j, a, b);
        }
      }
      for (int b = 0; b < nvrt; ++b)
        sum2 = sum2 + OM(i, nvrt - 1, j, b) * OM(i, nvrt - 1, j, b) /
                          (eig[i] + eig[j] - eig[ntot - 1] - eig[b + nocc]);
    }
  }
  for (int j = 0; j < nocc; ++j)
    for (int a = 0; a < nvrt; ++a)
      for (int b = 0; b < nvrt; ++b)
        sum2 = sum2 + OM(nocc - 1, a, j, b) * OM(nocc - 1, a, j, b) / DEN(nocc - 1, j, a, b);
#undef OM
#undef DEN
  out[0] = sum1;
  out[1] = sum2;
  out[2] = 2 * sum1 + sum2;
}

/* mp2_uhf, mp2.f90:154-232.  OAA(i,a,j,b) over alpha, OBB over beta,
 * OAB(i,a,j,b) with i,a alpha and j,b beta.  out = {E(AA), E(BB), E(AB), E(MBPT2)}. */
void orc_mp2_uhf(int noA, int noB, int nvA, int nvB, const double *eA, const double *eB, const double *OAA,
                 const double *OBB, const double *OAB, double *out) {
  double s1 = 0.0, s2 = 0.0, s3 = 0.0;
  for (int i = 0; i <= noA - 2; ++i)
    for (int j = i + 1; j < noA; ++j)
      for (int a = 0; a <= nvA - 2; ++a)
        for (int b = a + 1; b < nvA; ++b) {
          double x = OAA[i + noA * (a + nvA * (j + noA * b))] - OAA[i + noA * (b + nvA * (j + noA * a))];
          s1 = s1 + x * x / (eA[i] + eA[j] - eA[a + noA] - eA[b + noA]);
        }
  for (int i = 0; i <= noB - 2; ++i)
    for (int j = i + 1; j < noB; ++j)
      for (int a = 0; a <= nvB - 2; ++a)
        for (int b = a + 1; b < nvB; ++b) {
          double x = OBB[i + noB * (a + nvB * (j + noB * b))] - OBB[i + noB * (b + nvB * (j + noB * a))];
          s2 = s2 + x * x / (eB[i] + eB[j] - eB[a + noB] - eB[b + noB]);
        }
  for (int i = 0; i < noA; ++i)
    for (int j = 0; j < noB; ++j)
      for (int a = 0; a < nvA; ++a)
        for (int b = 0; b < nvB; ++b) {
          double x = OAB[i + noA * (a + nvA * (j + noB * b))];
          s3 = s3 + x * x / (eA[i] + eB[j] - eA[a + noA] - eB[b + noB]);
        }
  out[0] = s1; out[1] = s2; out[2] = s3; out[3] = s1 + s2 + s3;
}

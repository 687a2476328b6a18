// int1e.cu -- overlap S and core Hamiltonian H = T + V over contracted s/sp
// shell pairs, FP64.  Restates proc1e (src/integrals/int1e.f90:132-280):
// overlap :321-386, kinetic :391-474, coulomb (nuclear attraction) :479-582,
// with the same Hermite coefficients, Boys regimes (Boys order 3*(la+lb)) and
// primitive screen EIJ < 1e-14 (applied when the pair table is built).
#include "boys.cuh"
#include "internal.h"

namespace mq {

struct Int1eArgs {
  PairTable t;
  const double *boys;
  const double *nuc;  // nnuc x 4 (x, y, z, Z)
  int nnuc, n, mode;
  int pOff, np;
  double *S, *H;
  const MolDesc *mols;  // batch: per-pair molecule gives n, nuclei and matrix offset (null: one system)
};

// Hermite coefficients E^{ij}_t of one axis for i <= 1, j <= 3 (kinetic needs
// j = l_b + 2), by the standard recursion the reference's lrec/rrec memoise.
__device__ __forceinline__ void axis_E(double PA, double PB, double i2p, double (&E)[2][4][5]) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int t = 0; t < 5; ++t) E[i][j][t] = 0.0;
  E[0][0][0] = 1.0;
  E[1][0][0] = PA;
  E[1][0][1] = i2p;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int t = 0; t <= i + j + 1; ++t) {
        double v = PB * E[i][j][t];
        if (t > 0) v += i2p * E[i][j][t - 1];
        if (t + 1 <= i + j) v += (t + 1) * E[i][j][t + 1];
        E[i][j + 1][t] = v;
      }
}

// One warp per contracted shell pair: the 32 lanes split the nuclei of the
// attraction integrals (nucleus cn on lane cn mod 32) and every lane contracts
// its partial V with the Hermite coefficients; lane 0 adds the overlap and
// kinetic terms, and a shuffle tree sums the lanes (fixed order).
constexpr int INT1E_WARPS = 4;

template <int LA, int LB>
__global__ void __launch_bounds__(32 * INT1E_WARPS) int1e_kernel(Int1eArgs g) {
  constexpr int NA = LA ? 4 : 1, NB = LB ? 4 : 1, L = LA + LB, QREF = 3 * L;
  const int idx = blockIdx.x * INT1E_WARPS + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (idx >= g.np) return;  // warp-uniform
  const int P = g.pOff + idx;
  const PairTable &t = g.t;
  const double *nuc = g.nuc;
  int nnuc = g.nnuc;
  size_t n = g.n;
  double *Sout = g.S, *Hout = g.H;
  if (g.mols) {
    const MolDesc md = g.mols[t.mol[P]];
    nuc += 4 * md.nuc_off;
    nnuc = md.nnuc;
    n = md.n;
    Sout += md.mat;
    Hout += md.mat;
  }
  const bool parity = g.mode == MQ_MODE_REFERENCE;
  const double pi = parity ? PI_REF : PI_TRUE;
  double s[NA][NB], h[NA][NB];
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b) s[a][b] = h[a][b] = 0.0;
  for (int ip = t.pp_off[P]; ip < t.pp_off[P + 1]; ++ip) {
    const double p = t.p[ip], i2p = t.inv2p[ip];
    const double Px = t.Px[ip], Py = t.Py[ip], Pz = t.Pz[ip];
    double Ex[2][4][5], Ey[2][4][5], Ez[2][4][5];
    axis_E(t.PAx[ip], t.PBx[ip], i2p, Ex);
    axis_E(t.PAy[ip], t.PBy[ip], i2p, Ey);
    axis_E(t.PAz[ip], t.PBz[ip], i2p, Ez);
    const double bb = t.beta[ip];  // exponent of B (the kinetic term needs it)
    const double pp32 = pow(pi / p, 1.5);
    double c[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) c[k] = t.c4[4 * ip + k];
    // nuclear attraction: R^{(0)}_{tuv}(p, P - C) for all nuclei
    double V[L + 1][L + 1][L + 1];
#pragma unroll
    for (int x = 0; x <= L; ++x)
#pragma unroll
      for (int y = 0; y <= L; ++y)
#pragma unroll
        for (int z = 0; z <= L; ++z) V[x][y][z] = 0.0;
    for (int cn = lane; cn < nnuc; cn += 32) {
      const double X = Px - nuc[4 * cn], Y = Py - nuc[4 * cn + 1], Z = Pz - nuc[4 * cn + 2];
      const double T = p * (X * X + Y * Y + Z * Z);
      double F[L + 1];
      boys<QREF, L>(g.mode, T, g.boys, F);
      const double w = -nuc[4 * cn + 3] * 2.0 * pi / p;
      // R recursion (auxilary.f90:22-80) with alpha = p
      double Rj[L + 1][L + 1][L + 1][L + 1];
      double pw = 1.0;
#pragma unroll
      for (int j = 0; j <= L; ++j) {
        Rj[j][0][0][0] = pw * F[j] * w;
        pw *= -2.0 * p;
      }
#pragma unroll
      for (int j = L - 1; j >= 0; --j)
#pragma unroll
        for (int x = 0; x <= L; ++x)
#pragma unroll
          for (int y = 0; y <= L; ++y)
#pragma unroll
            for (int z = 0; z <= L; ++z) {
              if (x + y + z == 0 || x + y + z > L - j) continue;
              double r;
              if (x > 0) {
                r = X * Rj[j + 1][x - 1][y][z];
                if (x > 1) r += (x - 1) * Rj[j + 1][x - 2][y][z];
              } else if (y > 0) {
                r = Y * Rj[j + 1][x][y - 1][z];
                if (y > 1) r += (y - 1) * Rj[j + 1][x][y - 2][z];
              } else {
                r = Z * Rj[j + 1][x][y][z - 1];
                if (z > 1) r += (z - 1) * Rj[j + 1][x][y][z - 2];
              }
              Rj[j][x][y][z] = r;
            }
#pragma unroll
      for (int x = 0; x <= L; ++x)
#pragma unroll
        for (int y = 0; y <= L; ++y)
#pragma unroll
          for (int z = 0; z <= L; ++z)
            if (x + y + z <= L) V[x][y][z] += Rj[0][x][y][z];
    }
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        const int ax = a == 1, ay = a == 2, az = a == 3, bx = b == 1, by = b == 2, bz = b == 3;
        const double cf = c[2 * (a > 0) + (b > 0)];
        const double sx = Ex[ax][bx][0], sy = Ey[ay][by][0], sz = Ez[az][bz][0];
        const double own = lane == 0 ? 1.0 : 0.0;  // overlap and kinetic terms: lane 0 only
        s[a][b] += own * cf * pp32 * sx * sy * sz;
        // kinetic: -1/2 sum_axis [nb(nb-1) E(na,nb-2) - 2b(2nb+1) E(na,nb) + 4b^2 E(na,nb+2)] * others
        auto kin = [&](const double (&E)[2][4][5], int na, int nb) {
          double v = -2.0 * bb * (2 * nb + 1) * E[na][nb][0] + 4.0 * bb * bb * E[na][nb + 2][0];
          if (nb >= 2) v += nb * (nb - 1) * E[na][nb - 2][0];
          return v;
        };
        const double tk = kin(Ex, ax, bx) * sy * sz + kin(Ey, ay, by) * sx * sz + kin(Ez, az, bz) * sx * sy;
        double v = 0.0;
#pragma unroll
        for (int x = 0; x <= ax + bx; ++x)
#pragma unroll
          for (int y = 0; y <= ay + by; ++y)
#pragma unroll
            for (int z = 0; z <= az + bz; ++z) v += Ex[ax][bx][x] * Ey[ay][by][y] * Ez[az][bz][z] * V[x][y][z];
        h[a][b] += cf * (-0.5 * own * pp32 * tk + v);
      }
  }
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        s[a][b] += __shfl_xor_sync(0xffffffffu, s[a][b], o);
        h[a][b] += __shfl_xor_sync(0xffffffffu, h[a][b], o);
      }
  if (lane != 0) return;
  const int A = t.shA[P], B = t.shB[P], i0 = t.aoA[P], j0 = t.aoB[P];
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int i = i0 + a, j = j0 + b;
      if (A == B && i < j) continue;
      Sout[i + n * j] = s[a][b];
      Sout[j + n * i] = s[a][b];
      Hout[i + n * j] = h[a][b];
      Hout[j + n * i] = h[a][b];
    }
}

// Dipole integrals about the origin, the property integrals of int1p
// (src/integrals/int1p.f90:150-300): <a| r_c |b> per primitive pair is
// K_ab c_a c_b (pi/p)^(3/2) E^{ab}_0 of the two other axes times
// (E^{ab}_1 + P_c E^{ab}_0) of axis c.  One thread per contracted shell pair;
// Px holds the x, y, z matrices one after the other (column-major n x n).
template <int LA, int LB>
__global__ void __launch_bounds__(128) dipole_kernel(PairTable t, int pOff, int np, int n, int mode,
                                                     double *__restrict__ Px) {
  constexpr int NA = LA ? 4 : 1, NB = LB ? 4 : 1;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= np) return;
  const int P = pOff + idx;
  const double pi = mode == MQ_MODE_REFERENCE ? PI_REF : PI_TRUE;
  double d[3][NA][NB];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b) d[c][a][b] = 0.0;
  for (int ip = t.pp_off[P]; ip < t.pp_off[P + 1]; ++ip) {
    const double p = t.p[ip], i2p = t.inv2p[ip];
    double E[3][2][4][5];
    axis_E(t.PAx[ip], t.PBx[ip], i2p, E[0]);
    axis_E(t.PAy[ip], t.PBy[ip], i2p, E[1]);
    axis_E(t.PAz[ip], t.PBz[ip], i2p, E[2]);
    const double Pc[3] = {t.Px[ip], t.Py[ip], t.Pz[ip]};
    const double pp32 = pow(pi / p, 1.5);
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        const int la[3] = {a == 1, a == 2, a == 3}, lb[3] = {b == 1, b == 2, b == 3};
        const double cf = t.c4[4 * ip + 2 * (a > 0) + (b > 0)] * pp32;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int o1 = (c + 1) % 3, o2 = (c + 2) % 3;
          const double e0 = E[c][la[c]][lb[c]][0], e1 = E[c][la[c]][lb[c]][1];
          d[c][a][b] += cf * E[o1][la[o1]][lb[o1]][0] * E[o2][la[o2]][lb[o2]][0] * (e1 + Pc[c] * e0);
        }
      }
  }
  const int A = t.shA[P], B = t.shB[P], i0 = t.aoA[P], j0 = t.aoB[P];
  const size_t N = n, n2 = N * N;
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int i = i0 + a, j = j0 + b;
      if (A == B && i < j) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Px[n2 * c + i + N * j] = d[c][a][b];
        Px[n2 * c + j + N * i] = d[c][a][b];
      }
    }
}

int int1p_device(mq_ctx *c, double *d_Px) {
  const size_t n = c->nao;
  MQ_CUDA(c, cudaMemsetAsync(d_Px, 0, 3 * n * n * sizeof(double), c->stream));
  for (int cl = 0; cl < 3; ++cl) {
    const int pOff = c->pt.class_off[cl], np = c->pt.class_off[cl + 1] - pOff;
    if (!np) continue;
    const dim3 grid((np + 127) / 128);
    if (cl == 0) dipole_kernel<0, 0><<<grid, 128, 0, c->stream>>>(c->pt, pOff, np, (int)n, c->mode, d_Px);
    else if (cl == 1) dipole_kernel<1, 0><<<grid, 128, 0, c->stream>>>(c->pt, pOff, np, (int)n, c->mode, d_Px);
    else dipole_kernel<1, 1><<<grid, 128, 0, c->stream>>>(c->pt, pOff, np, (int)n, c->mode, d_Px);
    c->stats.launches += 1;
    MQ_CUDA(c, cudaGetLastError());
  }
  return MQ_OK;
}

// Batch: S and H of every molecule of the batch table into the packed n x n
// arrays (offset MolDesc::mat), one launch per pair class for all molecules.
int int1e_batch_device(mq_ctx *c, const PairTable &t, const double *d_nuc, const MolDesc *d_mols, size_t mat_total,
                       double *d_S, double *d_H) {
  MQ_CUDA(c, cudaMemsetAsync(d_S, 0, mat_total * sizeof(double), c->stream));
  MQ_CUDA(c, cudaMemsetAsync(d_H, 0, mat_total * sizeof(double), c->stream));
  Int1eArgs g{};
  g.t = t;
  g.boys = c->d_boys;
  g.nuc = d_nuc;
  g.mode = MQ_MODE_TIGHT;
  g.S = d_S;
  g.H = d_H;
  g.mols = d_mols;
  for (int cl = 0; cl < 3; ++cl) {
    g.pOff = t.class_off[cl];
    g.np = t.class_off[cl + 1] - g.pOff;
    if (!g.np) continue;
    dim3 grid((g.np + INT1E_WARPS - 1) / INT1E_WARPS);
    if (cl == 0) int1e_kernel<0, 0><<<grid, 32 * INT1E_WARPS, 0, c->stream>>>(g);
    else if (cl == 1) int1e_kernel<1, 0><<<grid, 32 * INT1E_WARPS, 0, c->stream>>>(g);
    else int1e_kernel<1, 1><<<grid, 32 * INT1E_WARPS, 0, c->stream>>>(g);
    c->stats.launches += 1;
    MQ_CUDA(c, cudaGetLastError());
  }
  return MQ_OK;
}

int int1e_device(mq_ctx *c, double *d_S, double *d_H) {
  const size_t n = c->nao;
  MQ_CUDA(c, cudaMemsetAsync(d_S, 0, n * n * sizeof(double), c->stream));
  MQ_CUDA(c, cudaMemsetAsync(d_H, 0, n * n * sizeof(double), c->stream));
  Int1eArgs g{};
  g.t = c->pt;
  g.boys = c->d_boys;
  g.nuc = c->d_nuc;
  g.nnuc = c->nnuc;
  g.n = c->nao;
  g.mode = c->mode;
  g.S = d_S;
  g.H = d_H;
  for (int cl = 0; cl < 3; ++cl) {
    g.pOff = c->pt.class_off[cl];
    g.np = c->pt.class_off[cl + 1] - g.pOff;
    if (!g.np) continue;
    dim3 grid((g.np + INT1E_WARPS - 1) / INT1E_WARPS);
    if (cl == 0) int1e_kernel<0, 0><<<grid, 32 * INT1E_WARPS, 0, c->stream>>>(g);
    else if (cl == 1) int1e_kernel<1, 0><<<grid, 32 * INT1E_WARPS, 0, c->stream>>>(g);
    else int1e_kernel<1, 1><<<grid, 32 * INT1E_WARPS, 0, c->stream>>>(g);
    c->stats.launches += 1;
    MQ_CUDA(c, cudaGetLastError());
  }
  return MQ_OK;
}

}  // namespace mq

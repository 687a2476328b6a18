// guess.cu -- the learned initial density on the device: pair descriptors in
// local frames, the network's forward pass, and the assembly of the predicted
// blocks into each molecule's density, for one molecule or a whole batch in a
// few launches.  The descriptors are the ones the network was trained on
// (myqc_gb300/guess.py restates them on the host for the training set):
//
//   pairs (A, B): every unordered pair within CUTOFF (8 A) and every (A, A),
//     the heavier element first;
//   frame: e_z along A -> B (for (A, A): towards A's nearest atom), e_x the
//     first of A's six nearest atoms (skipping B, and for (A, A) the atom that
//     fixed e_z) with a component perpendicular to e_z of more than 1e-3 A,
//     else a fixed axis; e_y = e_z x e_x.  Atoms are ordered by their
//     distance rounded to 1e-6 A, ties by index;
//   features (NFEAT = 64): heavy(A), heavy(B), R, 1/R, then for A and for B
//     its K_ENV = 6 nearest other atoms (B and A excluded) as (x, y, z in the
//     pair frame, heavy flag, 1/r), nearest first, zeros where fewer;
//   outputs: the 5 x 5 block (s, s', px, py, pz; an H atom uses index 0) in
//     the local frame, standardised per block type (heavy-heavy, heavy-H,
//     H-H, heavy diagonal, H diagonal);
//   assembly: D[A, B] = R_A b R_B^T (R = identity on s, the frame on p),
//     diagonal blocks symmetrised, absent pairs zero.
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace mq {

constexpr int G_KENV = 6, G_NFEAT = 4 + 2 * G_KENV * 5, G_NOUT = 25, G_NTYPES = 5;
constexpr int G_NB = 8;  // nearest atoms kept per atom (K_ENV + the pair partner + one)
constexpr double G_CUTOFF = 8.0;
constexpr double G_BOHR = 1.8897161646320724;

struct GuessAtoms {
  const double *xyz;     // Angstrom, natoms x 3
  const int *Z;
  const int *mol;        // molecule of each atom
  const int *mol_atom0;  // first atom of each molecule (nmol + 1)
  int *nb;               // [atom][G_NB] nearest others, -1 past the molecule's size
};

__device__ __forceinline__ double gdist(const double *x, int a, int b) {
  const double dx = x[3 * a] - x[3 * b], dy = x[3 * a + 1] - x[3 * b + 1], dz = x[3 * a + 2] - x[3 * b + 2];
  return sqrt(dx * dx + dy * dy + dz * dz);
}

// each atom's G_NB nearest other atoms of its molecule: by distance rounded to
// 1e-6 A (round half to even), ties by index
__global__ void guess_neighbours_kernel(GuessAtoms g, int natoms) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= natoms) return;
  const int m = g.mol[a], b0 = g.mol_atom0[m], b1 = g.mol_atom0[m + 1];
  double key[G_NB];
  int idx[G_NB];
  int cnt = 0;
  for (int b = b0; b < b1; ++b) {
    if (b == a) continue;
    const double k = rint(gdist(g.xyz, a, b) * 1e6);
    // insertion into the sorted top list (key, then index: b ascends, so equal keys keep order)
    int pos = cnt < G_NB ? cnt : G_NB;
    while (pos > 0 && key[pos - 1] > k) --pos;
    if (pos >= G_NB) continue;
    const int last = cnt < G_NB ? cnt : G_NB - 1;
    for (int t = last; t > pos; --t) {
      key[t] = key[t - 1];
      idx[t] = idx[t - 1];
    }
    key[pos] = k;
    idx[pos] = b;
    if (cnt < G_NB) ++cnt;
  }
  for (int t = 0; t < G_NB; ++t) g.nb[(size_t)a * G_NB + t] = t < cnt ? idx[t] : -1;
}

__device__ __forceinline__ void gsub(const double *x, int a, int b, double v[3]) {  // x_b - x_a
  v[0] = x[3 * b] - x[3 * a];
  v[1] = x[3 * b + 1] - x[3 * a + 1];
  v[2] = x[3 * b + 2] - x[3 * a + 2];
}

// frames and standardised features of every pair
__global__ void guess_features_kernel(GuessAtoms g, const int2 *__restrict__ pairs, int npairs,
                                      const double *__restrict__ mu_x, const double *__restrict__ sd_x,
                                      float *__restrict__ X, double *__restrict__ Qout) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  const int A = pairs[p].x, B = pairs[p].y;
  const bool diag = A == B;
  const int *nbA = g.nb + (size_t)A * G_NB;
  const int first = nbA[0];
  double ez[3];
  if (diag) {
    if (first >= 0) gsub(g.xyz, A, first, ez);
    else ez[0] = ez[1] = 0.0, ez[2] = 1.0;  // a lone atom: any axis
  } else {
    gsub(g.xyz, A, B, ez);
  }
  {
    const double nz = sqrt(ez[0] * ez[0] + ez[1] * ez[1] + ez[2] * ez[2]);
    for (int k = 0; k < 3; ++k) ez[k] /= nz;
  }
  double ex[3] = {0.0, 0.0, 0.0};
  bool have = false;
  for (int k = 0; k < 6 && !have; ++k) {
    const int c = nbA[k];
    if (c < 0 || c == B || (diag && c == first)) continue;
    double v[3];
    gsub(g.xyz, A, c, v);
    const double dp = v[0] * ez[0] + v[1] * ez[1] + v[2] * ez[2];
    for (int j = 0; j < 3; ++j) v[j] -= dp * ez[j];
    const double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (nv > 1e-3) {
      for (int j = 0; j < 3; ++j) ex[j] = v[j] / nv;
      have = true;
    }
  }
  if (!have) {  // collinear surroundings: a fixed axis made perpendicular
    double t[3] = {fabs(ez[0]) < 0.9 ? 1.0 : 0.0, fabs(ez[0]) < 0.9 ? 0.0 : 1.0, 0.0};
    const double dp = t[0] * ez[0] + t[1] * ez[1] + t[2] * ez[2];
    double v[3];
    for (int j = 0; j < 3; ++j) v[j] = t[j] - dp * ez[j];
    const double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int j = 0; j < 3; ++j) ex[j] = v[j] / nv;
  }
  const double ey[3] = {ez[1] * ex[2] - ez[2] * ex[1], ez[2] * ex[0] - ez[0] * ex[2], ez[0] * ex[1] - ez[1] * ex[0]};
  // Q columns e_x, e_y, e_z: Q[i][j] at Qout[9 p + 3 i + j]
  double *Q = Qout + 9 * (size_t)p;
  for (int i = 0; i < 3; ++i) {
    Q[3 * i] = ex[i];
    Q[3 * i + 1] = ey[i];
    Q[3 * i + 2] = ez[i];
  }
  double f[G_NFEAT];
  for (int k = 0; k < G_NFEAT; ++k) f[k] = 0.0;
  const double R = diag ? 0.0 : gdist(g.xyz, A, B);
  f[0] = g.Z[A] > 2;
  f[1] = g.Z[B] > 2;
  f[2] = R;
  f[3] = R > 0 ? 1.0 / fmax(R, 1e-9) : 0.0;
  for (int side = 0; side < 2; ++side) {
    const int Xa = side ? B : A, other = side ? A : B;
    const int *nb = g.nb + (size_t)Xa * G_NB;
    int rank = 0;
    for (int k = 0; k < G_KENV + 1 && rank < G_KENV; ++k) {
      const int c = nb[k];
      if (c < 0 || c == other) continue;
      double v[3];
      gsub(g.xyz, Xa, c, v);
      const int base = 4 + side * G_KENV * 5 + rank * 5;
      for (int j = 0; j < 3; ++j) f[base + j] = v[0] * Q[j] + v[1] * Q[3 + j] + v[2] * Q[6 + j];  // Q^T v
      f[base + 3] = g.Z[c] > 2;
      f[base + 4] = 1.0 / gdist(g.xyz, Xa, c);
      ++rank;
    }
  }
  // standardised in FP32, as the training pipeline's FP32 statistics are applied
  float *x = X + (size_t)p * G_NFEAT;
  for (int k = 0; k < G_NFEAT; ++k) x[k] = __fdiv_rn(__fsub_rn((float)f[k], (float)mu_x[k]), (float)sd_x[k]);
}

// the predicted blocks into the densities (zeroed first), in the frame of the molecule
__global__ void guess_assemble_kernel(GuessAtoms g, const int2 *__restrict__ pairs, int npairs,
                                      const float *__restrict__ Y, int ldy, const double *__restrict__ mu_y,
                                      const double *__restrict__ sd_y, const double *__restrict__ Qin,
                                      const int *__restrict__ ao0, const long long *__restrict__ mol_mat,
                                      const int *__restrict__ mol_n, double *__restrict__ D) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  const int A = pairs[p].x, B = pairs[p].y, m = g.mol[A];
  const bool diag = A == B;
  const bool ha = g.Z[A] > 2, hb = g.Z[B] > 2;
  const int t = diag ? (ha ? 3 : 4) : (ha && hb ? 0 : (ha || hb ? 1 : 2));
  const int na = ha ? 5 : 1, nbf = hb ? 5 : 1;
  double b5[5][5];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      const int e = 5 * i + j;
      b5[i][j] = (i < na && j < nbf) ? (double)Y[(size_t)p * ldy + e] * sd_y[t * G_NOUT + e] + mu_y[t * G_NOUT + e]
                                     : 0.0;
    }
  const double *Q = Qin + 9 * (size_t)p;
  // R = identity on s (indices 0, 1), Q on p (2, 3, 4) for a heavy atom
  auto rot = [&](bool heavy, int i, int k) -> double {
    if (!heavy || i < 2 || k < 2) return i == k ? 1.0 : 0.0;
    return Q[3 * (i - 2) + (k - 2)];
  };
  double blk[5][5];
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nbf; ++j) {
      double v = 0.0;
      for (int k = 0; k < na; ++k) {
        const double rik = rot(ha, i, k);
        if (rik == 0.0) continue;
        for (int l = 0; l < nbf; ++l) v += rik * b5[k][l] * rot(hb, j, l);
      }
      blk[i][j] = v;
    }
  if (diag)
    for (int i = 0; i < na; ++i)
      for (int j = i + 1; j < na; ++j) {
        const double v = 0.5 * (blk[i][j] + blk[j][i]);
        blk[i][j] = blk[j][i] = v;
      }
  const size_t n = mol_n[m];
  double *Dm = D + mol_mat[m];
  const int ia = ao0[A], ib = ao0[B];
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nbf; ++j) {
      Dm[(ia + i) + n * (ib + j)] = blk[i][j];
      Dm[(ib + j) + n * (ia + i)] = blk[i][j];
    }
}

int guess_predict(mq_ctx *c, int nmol, const int *nnuc, const int *Z, const double *xyz, double *D_out);

}  // namespace mq

using namespace mq;

extern "C" {

int mq_guess_model(mq_ctx *c, int nin, int width, int nout, const float *params, const double *mu_x,
                   const double *sd_x, const double *mu_y, const double *sd_y) {
  if (!c || !params || !mu_x || !sd_x || !mu_y || !sd_y) return MQ_EINVAL;
  if (nin != G_NFEAT || nout != G_NOUT) return set_err(c, MQ_EINVAL, "guess model: 64 features and 25 outputs expected");
  MQ_TRY(mlp_init(c, nin, width, nout));
  MQ_TRY(mlp_set_params(c, params));
  c->guess_mu_x.assign(mu_x, mu_x + G_NFEAT);
  c->guess_sd_x.assign(sd_x, sd_x + G_NFEAT);
  c->guess_mu_y.assign(mu_y, mu_y + G_NTYPES * G_NOUT);
  c->guess_sd_y.assign(sd_y, sd_y + G_NTYPES * G_NOUT);
  return MQ_OK;
}

int mq_guess_predict(mq_ctx *c, int nmol, const int *nnuc, const int *Z, const double *xyz, double *D_out) {
  if (!c || nmol <= 0 || !nnuc || !Z || !xyz || !D_out) return c ? set_err(c, MQ_EINVAL, "guess: bad arguments") : MQ_EINVAL;
  if (c->guess_mu_x.size() != (size_t)G_NFEAT) return set_err(c, MQ_ESTATE, "guess: no model (mq_guess_model)");
  cudaSetDevice(c->device);
  // on the aux stream (highest priority): a guess asked for while the integral
  // pass is queued on the main stream does not wait for it
  MQ_TRY(ensure_aux(c));
  cudaStream_t main = c->stream;
  c->stream = c->aux;
  const int rc = guess_predict(c, nmol, nnuc, Z, xyz, D_out);
  c->stream = main;
  return rc;
}

}  // extern "C"

namespace mq {
int guess_predict(mq_ctx *c, int nmol, const int *nnuc, const int *Z, const double *xyz, double *D_out) {
  // host: atoms, molecules, AO offsets, pairs (cheap O(atoms^2) per molecule)
  std::vector<int> mol, atom0(nmol + 1, 0), ao0, moln(nmol);
  std::vector<long long> mat(nmol + 1, 0);
  std::vector<double> xa;
  std::vector<int2> pairs;
  long long ntot = 0;  // xyz is column-major over all the molecules' atoms: xyz(0:ntot-1, 0:2)
  for (int m = 0; m < nmol; ++m) ntot += nnuc[m] > 0 ? nnuc[m] : 0;
  int natoms = 0;
  for (int m = 0; m < nmol; ++m) {
    if (nnuc[m] <= 0) return set_err(c, MQ_EINVAL, "guess: a molecule without atoms");
    atom0[m] = natoms;
    int n = 0;
    for (int a = 0; a < nnuc[m]; ++a) {
      const int z = Z[natoms + a];
      if (z < 1 || z > 10) return set_err(c, MQ_EINVAL, "guess: element out of range");
      ao0.push_back(n);
      n += z <= 2 ? 1 : 5;
      mol.push_back(m);
      for (int k = 0; k < 3; ++k) xa.push_back(xyz[(size_t)(natoms + a) + (size_t)ntot * k] / G_BOHR);
    }
    moln[m] = n;
    mat[m + 1] = mat[m] + (long long)n * n;
    for (int a = 0; a < nnuc[m]; ++a)
      for (int b = a; b < nnuc[m]; ++b) {
        const int ga = natoms + a, gb = natoms + b;
        if (a != b) {
          const double dx = xa[3 * ga] - xa[3 * gb], dy = xa[3 * ga + 1] - xa[3 * gb + 1],
                       dz = xa[3 * ga + 2] - xa[3 * gb + 2];
          if (std::sqrt(dx * dx + dy * dy + dz * dz) > G_CUTOFF) continue;
        }
        const bool swap = Z[gb] > Z[ga];
        pairs.push_back(swap ? make_int2(gb, ga) : make_int2(ga, gb));
      }
    natoms += nnuc[m];
  }
  atom0[nmol] = natoms;
  const int np = (int)pairs.size();
  // device buffers, one block
  const size_t o_xyz = 0, o_z = o_xyz + 24 * (size_t)natoms, o_mol = o_z + 4 * (size_t)natoms,
               o_a0 = o_mol + 4 * (size_t)natoms, o_nb = o_a0 + 4 * (size_t)(nmol + 1),
               o_ao = o_nb + 4 * (size_t)natoms * G_NB, o_pairs = (o_ao + 4 * (size_t)natoms + 15) / 16 * 16,
               o_mat = o_pairs + 8 * (size_t)np, o_moln = o_mat + 8 * (size_t)(nmol + 1),
               o_norm = (o_moln + 4 * (size_t)nmol + 15) / 16 * 16,
               o_X = o_norm + 8 * (size_t)(2 * G_NFEAT + 2 * G_NTYPES * G_NOUT),
               o_Q = (o_X + 4 * (size_t)np * G_NFEAT + 15) / 16 * 16, o_D = o_Q + 72 * (size_t)np,
               total = o_D + 8 * (size_t)mat[nmol];
  char *d = (char *)buf(c, "guess_work", total + 64);
  if (!d) return MQ_ENOMEM;
  std::vector<char> hb(o_X);
  std::memcpy(hb.data() + o_xyz, xa.data(), 24 * (size_t)natoms);
  std::memcpy(hb.data() + o_z, Z, 4 * (size_t)natoms);
  std::memcpy(hb.data() + o_mol, mol.data(), 4 * (size_t)natoms);
  std::memcpy(hb.data() + o_a0, atom0.data(), 4 * (size_t)(nmol + 1));
  std::memcpy(hb.data() + o_ao, ao0.data(), 4 * (size_t)natoms);
  std::memcpy(hb.data() + o_pairs, pairs.data(), 8 * (size_t)np);
  std::memcpy(hb.data() + o_mat, mat.data(), 8 * (size_t)(nmol + 1));
  std::memcpy(hb.data() + o_moln, moln.data(), 4 * (size_t)nmol);
  double *norm = (double *)(hb.data() + o_norm);
  std::memcpy(norm, c->guess_mu_x.data(), 8 * G_NFEAT);
  std::memcpy(norm + G_NFEAT, c->guess_sd_x.data(), 8 * G_NFEAT);
  std::memcpy(norm + 2 * G_NFEAT, c->guess_mu_y.data(), 8 * G_NTYPES * G_NOUT);
  std::memcpy(norm + 2 * G_NFEAT + G_NTYPES * G_NOUT, c->guess_sd_y.data(), 8 * G_NTYPES * G_NOUT);
  MQ_CUDA(c, cudaMemcpyAsync(d, hb.data(), o_X, cudaMemcpyHostToDevice, c->stream));
  GuessAtoms g{(const double *)(d + o_xyz), (const int *)(d + o_z), (const int *)(d + o_mol),
               (const int *)(d + o_a0), (int *)(d + o_nb)};
  const double *dnorm = (const double *)(d + o_norm);
  float *dX = (float *)(d + o_X);
  double *dQ = (double *)(d + o_Q), *dD = (double *)(d + o_D);
  guess_neighbours_kernel<<<(natoms + 127) / 128, 128, 0, c->stream>>>(g, natoms);
  guess_features_kernel<<<(np + 127) / 128, 128, 0, c->stream>>>(g, (const int2 *)(d + o_pairs), np, dnorm,
                                                                dnorm + G_NFEAT, dX, dQ);
  MQ_CUDA(c, cudaMemsetAsync(dD, 0, 8 * (size_t)mat[nmol], c->stream));
  c->stats.launches += 2;
  MQ_CUDA(c, cudaGetLastError());
  float *dY = nullptr;
  MQ_TRY(mlp_forward_device(c, np, dX, &dY));
  guess_assemble_kernel<<<(np + 127) / 128, 128, 0, c->stream>>>(
      g, (const int2 *)(d + o_pairs), np, dY, G_NOUT, dnorm + 2 * G_NFEAT, dnorm + 2 * G_NFEAT + G_NTYPES * G_NOUT, dQ,
      (const int *)(d + o_ao), (const long long *)(d + o_mat), (const int *)(d + o_moln), dD);
  c->stats.launches += 1;
  MQ_CUDA(c, cudaGetLastError());
  MQ_CUDA(c, cudaMemcpyAsync(D_out, dD, 8 * (size_t)mat[nmol], cudaMemcpyDeviceToHost, c->stream));
  MQ_CUDA(c, cudaStreamSynchronize(c->stream));
  return MQ_OK;
}
}  // namespace mq

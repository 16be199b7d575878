// bonded.cu -- harmonic bonds and angles with their k-space (Ewald) discounts
// (src/EmDeeData.f90:443-550, src/bond_harmonic.f90, src/angle_harmonic.f90,
// src/modelClass_kspace.f90:321-334).
//
// One thread per bond or angle computes its energy, virial and force vectors
// in FP64, as the reference's statements (this file is compiled with
// -fmad=false).  The vectors go to a contribution buffer; a second kernel adds,
// for every atom, its contributions in a fixed order (bonds in the order they
// were added, then angles), so the forces are deterministic and no atomics
// touch them.  Energies and virials are reduced with the deterministic grid
// reduction.  Dihedrals are stored (they only add exclusions): the reference
// never evaluates them (src/EmDeeCode.f90:1238-1246 calls compute_bonds and
// compute_angles only).
#include <algorithm>
#include <cmath>
#include <vector>

#include "pairmath.cuh"
#include "reduce.cuh"
#include "system.hpp"

namespace emdee {

static const int BONDED_THREADS = 256;

struct BondedArgs {
  const double* R;
  double* F;
  const int4* item;     // i, j, k (-1 for bonds), kind (BK_*)
  const double2* param;  // (k, x0)
  const double* qq;     // kCoul qi qj of the pair the discount applies to (bond i-j, angle i-k)
  double* vec;          // contribution vectors, 3 doubles each
  int nbonds, nitems;
  int bonded, kspace;
  double L, invL2, alpha, beta;
  const int* first;     // per atom: [first[a], first[a+1]) entries
  const int* entry;     // vector index << 1 | negate
  int natoms;
  double* partials;
  unsigned int* ticket;
  double* result;       // [0] Ebond, [1] Wbond, [2] Eangle, [3] Wangle, [4] Ecoul discount
};

enum BondedKind : int { BK_NONE = 0, BK_HARMONIC = 1 };

// cKspaceModel_discount (src/modelClass_kspace.f90:321-334)
__device__ __forceinline__ void kspace_discount(double alpha, double beta, double rsq, double QiQj, double& E,
                                                double& W) {
  const double r = sqrt(rsq), x = alpha * r, expmx2 = exp(-x * x);
  E = -QiQj * (1.0 - uerfc(x, expmx2)) / r;
  W = E + QiQj * beta * expmx2;
}

__global__ void __launch_bounds__(BONDED_THREADS) k_bonded(BondedArgs A) {
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < A.nitems) {
    const int4 it = A.item[m];
    const double2 pr = A.param[m];
    const double half_k = 0.5 * pr.x, minus_k = -pr.x;
    if (m < A.nbonds) {   // compute_bonds, src/EmDeeData.f90:443-487
      double Rij[3];
      for (int d = 0; d < 3; d++) {
        double x = A.R[3 * it.x + d] / A.L - A.R[3 * it.y + d] / A.L;
        Rij[d] = x - round(x);
      }
      const double invR2 = A.invL2 / (Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2]);
      double W = 0.0;
      if (A.bonded) {
        double E = 0.0;
        if (it.w == BK_HARMONIC) {   // src/bond_harmonic.f90:64-75
          const double r = 1.0 / sqrt(invR2), delta = r - pr.y;
          E = half_k * (delta * delta);
          W = minus_k * delta * r;
        }
        v[0] += E;
        v[1] += W;
      }
      if (A.kspace) {
        double EL, WL;
        kspace_discount(A.alpha, A.beta, 1.0 / invR2, A.qq[m], EL, WL);
        v[4] += EL;
        W = W + WL;
      }
      double* out = A.vec + 3 * (size_t)m;
      for (int d = 0; d < 3; d++) out[d] = W * invR2 * A.L * Rij[d];
    } else {              // compute_angles, src/EmDeeData.f90:491-550
      double a[3], b[3];
      for (int d = 0; d < 3; d++) {
        const double rj = A.R[3 * it.y + d] / A.L;
        double x = A.R[3 * it.x + d] / A.L - rj, y = A.R[3 * it.z + d] / A.L - rj;
        a[d] = A.L * (x - round(x));
        b[d] = A.L * (y - round(y));
      }
      double Fi[3] = {0.0, 0.0, 0.0}, Fk[3] = {0.0, 0.0, 0.0}, Fj[3] = {0.0, 0.0, 0.0};
      if (A.bonded) {
        const double aa = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        const double bb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
        const double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
        const double theta = acos(ab / sqrt(aa * bb));
        double Ea = 0.0, Fa = 0.0;
        if (it.w == BK_HARMONIC) {   // src/angle_harmonic.f90:64-73
          const double delta = theta - pr.y;
          Ea = half_k * (delta * delta);
          Fa = minus_k * delta;
        }
        const double factor = Fa / sqrt(aa * bb - ab * ab);
        for (int d = 0; d < 3; d++) {
          Fi[d] = ((ab / aa) * a[d] - b[d]) * factor;
          Fk[d] = ((ab / bb) * b[d] - a[d]) * factor;
          Fj[d] = -(Fi[d] + Fk[d]);
        }
        v[2] += Ea;
        v[3] += (Fi[0] * a[0] + Fk[0] * b[0]) + (Fi[1] * a[1] + Fk[1] * b[1]) + (Fi[2] * a[2] + Fk[2] * b[2]);
      }
      if (A.kspace) {
        double Rik[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
        const double RikSq = Rik[0] * Rik[0] + Rik[1] * Rik[1] + Rik[2] * Rik[2];
        double EL, WL;
        kspace_discount(A.alpha, A.beta, RikSq, A.qq[m], EL, WL);
        v[4] += EL;
        for (int d = 0; d < 3; d++) {
          const double f = WL * Rik[d] / RikSq;
          Fi[d] += f;
          Fk[d] -= f;
        }
      }
      double* out = A.vec + 3 * ((size_t)A.nbonds + 3 * (size_t)(m - A.nbonds));
      for (int d = 0; d < 3; d++) {
        out[d] = Fi[d];
        out[3 + d] = Fk[d];
        out[6 + d] = Fj[d];
      }
    }
  }
  grid_reduce<5, BONDED_THREADS>(v, A.partials, A.ticket, A.result);
}

// F(a) += the atom's contributions, in list order
__global__ void __launch_bounds__(BONDED_THREADS) k_bonded_gather(BondedArgs A) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= A.natoms) return;
  const int e0 = A.first[a], e1 = A.first[a + 1];
  if (e0 == e1) return;
  double f[3] = {A.F[3 * a], A.F[3 * a + 1], A.F[3 * a + 2]};
  for (int e = e0; e < e1; e++) {
    const int code = A.entry[e];
    const double* v = A.vec + 3 * (size_t)(code >> 1);
    for (int d = 0; d < 3; d++) f[d] = (code & 1) ? f[d] - v[d] : f[d] + v[d];
  }
  for (int d = 0; d < 3; d++) A.F[3 * a + d] = f[d];
}

// Uploads the item tables, the per-atom contribution lists and, per layer, the
// discount charge products.  Runs when items were added since the last upload.
static void bonded_upload(System& s) {
  BondedTerms& B = s.bondedTerms;
  const int nb = (int)B.bonds.size(), na = (int)B.angles.size(), n = nb + na, N = s.natoms;
  std::vector<int4> item(n);
  std::vector<double2> param(n);
  std::vector<double> qq((size_t)s.nlayers * n);
  std::vector<std::vector<int>> per(N);
  for (int m = 0; m < nb; m++) {
    const BondedTerms::Item& b = B.bonds[m];
    item[m] = make_int4(b.i, b.j, -1, b.kind);
    param[m] = make_double2(b.kf, b.x0);
    per[b.i].push_back(m << 1);
    per[b.j].push_back((m << 1) | 1);
  }
  for (int q = 0; q < na; q++) {
    const BondedTerms::Item& g = B.angles[q];
    const int m = nb + q, v = nb + 3 * q;
    item[m] = make_int4(g.i, g.j, g.k, g.kind);
    param[m] = make_double2(g.kf, g.x0);
    per[g.i].push_back(v << 1);
    per[g.k].push_back((v + 1) << 1);
    per[g.j].push_back((v + 2) << 1);
  }
  for (int l = 0; l < s.nlayers; l++)
    for (int m = 0; m < n; m++) {
      const int i = item[m].x, j = m < nb ? item[m].y : item[m].z;   // src/EmDeeData.f90:474-476,537-539
      const int ti = s.atomType[i] - 1, tj = s.atomType[j] - 1;
      qq[(size_t)l * n + m] = s.P(ti, tj, l).kCoul * s.charge[i] * s.charge[j];
    }
  std::vector<int> first(N + 1, 0), entry;
  for (int a = 0; a < N; a++) {
    first[a] = (int)entry.size();
    entry.insert(entry.end(), per[a].begin(), per[a].end());
  }
  first[N] = (int)entry.size();
  const int nvec = nb + 3 * na;
  CK(cudaFree(B.dItem)); CK(cudaFree(B.dParam)); CK(cudaFree(B.dQQ)); CK(cudaFree(B.dVec));
  CK(cudaFree(B.dFirst)); CK(cudaFree(B.dEntry)); CK(cudaFree(B.dPartials));
  CK(cudaMalloc(&B.dItem, sizeof(int4) * n));
  CK(cudaMalloc(&B.dParam, sizeof(double2) * n));
  CK(cudaMalloc(&B.dQQ, sizeof(double) * qq.size()));
  CK(cudaMalloc(&B.dVec, sizeof(double) * 3 * nvec));
  CK(cudaMalloc(&B.dFirst, sizeof(int) * (N + 1)));
  CK(cudaMalloc(&B.dEntry, sizeof(int) * std::max<size_t>(entry.size(), 1)));
  const int blocks = (n + BONDED_THREADS - 1) / BONDED_THREADS;
  CK(cudaMalloc(&B.dPartials, sizeof(double) * 5 * blocks));
  CK(cudaMemcpyAsync(B.dItem, item.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, s.stream));
  CK(cudaMemcpyAsync(B.dParam, param.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, s.stream));
  CK(cudaMemcpyAsync(B.dQQ, qq.data(), sizeof(double) * qq.size(), cudaMemcpyHostToDevice, s.stream));
  CK(cudaMemcpyAsync(B.dFirst, first.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice, s.stream));
  if (!entry.empty())
    CK(cudaMemcpyAsync(B.dEntry, entry.data(), sizeof(int) * entry.size(), cudaMemcpyHostToDevice, s.stream));
  CK(cudaStreamSynchronize(s.stream));   // the host vectors above go out of scope
  B.uploaded = n;
}

bool device_bonded(System& s, double out[5]) {
  BondedTerms& B = s.bondedTerms;
  for (int q = 0; q < 5; q++) out[q] = 0.0;
  const int n = (int)(B.bonds.size() + B.angles.size());
  const int l = s.layer - 1;
  const bool bonded = s.bonded[l] != 0, kspace = s.coul[l].requires_kspace != 0;
  if (n == 0 || !(bonded || kspace)) return false;
  if (B.uploaded != n) bonded_upload(s);
  BondedArgs A;
  A.R = s.dR;
  A.F = s.F();
  A.item = B.dItem;
  A.param = B.dParam;
  A.qq = B.dQQ + (size_t)l * n;
  A.vec = B.dVec;
  A.nbonds = (int)B.bonds.size();
  A.nitems = n;
  A.bonded = bonded;
  A.kspace = kspace;
  A.L = *s.Lbox;
  A.invL2 = 1.0 / (A.L * A.L);
  A.alpha = s.ewald.alpha;
  A.beta = s.ewald.beta;
  A.first = B.dFirst;
  A.entry = B.dEntry;
  A.natoms = s.natoms;
  A.partials = B.dPartials;
  A.ticket = s.dTicket + 7;
  A.result = s.dResult + 40;
  k_bonded<<<(n + BONDED_THREADS - 1) / BONDED_THREADS, BONDED_THREADS, 0, s.stream>>>(A);
  CK(cudaGetLastError());
  k_bonded_gather<<<(s.natoms + BONDED_THREADS - 1) / BONDED_THREADS, BONDED_THREADS, 0, s.stream>>>(A);
  CK(cudaGetLastError());
  s.prof.total += 2;
  CK(cudaMemcpyAsync(s.hResult + 40, s.dResult + 40, 5 * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
  CK(cudaStreamSynchronize(s.stream));
  for (int q = 0; q < 5; q++) out[q] = s.hResult[40 + q];
  return true;
}

void bonded_free(System& s) {
  BondedTerms& B = s.bondedTerms;
  cudaFree(B.dItem); cudaFree(B.dParam); cudaFree(B.dQQ); cudaFree(B.dVec);
  cudaFree(B.dFirst); cudaFree(B.dEntry); cudaFree(B.dPartials);
  B.dItem = nullptr; B.dParam = nullptr; B.dQQ = nullptr; B.dVec = nullptr;
  B.dFirst = nullptr; B.dEntry = nullptr; B.dPartials = nullptr;
}

}  // namespace emdee

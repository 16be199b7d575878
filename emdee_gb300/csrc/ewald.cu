// ewald.cu -- Ewald k-space electrostatics for coul_long (src/kspace_ewald.f90,
// src/modelClass_kspace.f90, src/coul_long.f90).
//
// Host: the reference's set-up, statement by statement (alpha and kmax from the
// accuracy, the half k-lattice inside the sphere of radius nmax * 2pi/L, the
// prefactors, the charge list by type, the rigid-pair and self-energy
// discounts, the Coulomb constants per type pair and layer).
// Device, FP64, compiled with -fmad=false:
//   k_ewald_sf     one block per group of charged atoms: the powers
//                  exp(i 2pi m x_d / L), m = 0..nmax, by the reference's complex
//                  recursion into shared memory, then per k-vector the
//                  block's partial type structure factors S(k, t)
//   k_ewald_sigma  per k-vector: S summed over blocks in block order,
//                  sigma(k, t) = sum_u S(k, u) lambda(u, t), energy terms
//                  prefac(k) sum_t Re(S conj-free dot sigma), grid reduction
//   k_ewald_force  one thread per charged atom: its powers in shared memory,
//                  F += sum_k vec(k) (Re sigma Im qe - Re qe Im sigma),
//                  added to the pair forces (no atomics: one thread per atom)
// Arithmetic order follows the CPU oracle: q exp(i k.r) = ((q G1) G2) G3,
// structure factors summed in charge-list order (blocks in order), forces
// summed over k-vectors in order.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "reduce.cuh"
#include "system.hpp"

namespace emdee {

static const double EW_PI = 3.14159265358979324;
static const int SF_THREADS = 256;
static const int FORCE_ATOMS = 64;

struct EwArgs {
  const double* R;
  double invL;   // 1 / current box length (theta = 2 pi R / L)
  int nq, nvecs, nmax, ntypes;
  const int* item;
  const int* qtype;
  const double* value;
  const int* first;
  const int* last;
  const int4* n;
  const double* prefac;
  const double* vec;
  const double* lambda;   // this layer: [t][u]
  double2* partial;       // [block][t][v]
  double2* sigma;         // [t][v]
  int sfBlocks, qb;
  double* F;
  double* epart;
  unsigned int* ticket;
  double* result;
};

// powers exp(i 2pi m x / L), m = 0..nm, of one coordinate into table rows
// row(m) = base + m * stride (src/kspace_ewald.f90:205-243: B = Z; G(j) = B; B = B*Z)
__device__ __forceinline__ void power_table(double x, double invL, int nm, double2* base, int stride) {
  const double theta = 6.28318530717958648 * (x * invL);
  double zi, zr;
  sincos(theta, &zi, &zr);
  base[0] = make_double2(1.0, 0.0);
  double br = zr, bi = zi;
  for (int m = 1; m <= nm; m++) {
    base[(size_t)m * stride] = make_double2(br, bi);
    const double nr = br * zr - bi * zi, ni = br * zi + bi * zr;
    br = nr;
    bi = ni;
  }
}

__device__ __forceinline__ double2 table_get(const double2* row0, int stride, int m) {
  if (m >= 0) return row0[(size_t)m * stride];
  const double2 g = row0[(size_t)(-m) * stride];
  return make_double2(g.x, -g.y);
}

// q exp(i k.r) = ((q G1) G2) G3
__device__ __forceinline__ double2 qeikr(double q, double2 g1, double2 g2, double2 g3) {
  const double ar = q * g1.x, ai = q * g1.y;
  const double br = ar * g2.x - ai * g2.y, bi = ar * g2.y + ai * g2.x;
  return make_double2(br * g3.x - bi * g3.y, br * g3.y + bi * g3.x);
}

__global__ void __launch_bounds__(SF_THREADS) k_ewald_sf(EwArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int QB = A.qb, QS = QB + 1;   // row stride: odd, so rows fall in different banks
  const int nm = A.nmax, rows = nm + 1;
  double2* G = (double2*)smem;        // [d][m][a], row (d, m) at (d * rows + m) * QS
  double* qs = (double*)(G + (size_t)3 * rows * QS);
  const int a0 = blockIdx.x * QB, na = min(QB, A.nq - a0);
  for (int a = threadIdx.x; a < na; a += blockDim.x) {
    const int i = A.item[a0 + a];
    qs[a] = A.value[a0 + a];
    for (int d = 0; d < 3; d++) power_table(A.R[3 * i + d], A.invL, nm, G + (size_t)d * rows * QS + a, QS);
  }
  __syncthreads();
  for (int v = threadIdx.x; v < A.nvecs; v += blockDim.x) {
    const int4 nv = A.n[v];
    for (int t = 0; t < A.ntypes; t++) {
      const int s0 = max(A.first[t] - a0, 0), s1 = min(A.last[t] - a0, na);
      double sr = 0.0, si = 0.0;
      for (int a = s0; a < s1; a++) {
        const double2 c = qeikr(qs[a], G[(size_t)nv.x * QS + a], table_get(G + (size_t)rows * QS + a, QS, nv.y),
                                table_get(G + (size_t)2 * rows * QS + a, QS, nv.z));
        sr += c.x;
        si += c.y;
      }
      A.partial[((size_t)blockIdx.x * A.ntypes + t) * A.nvecs + v] = make_double2(sr, si);
    }
  }
}

static const int EW_MAXT = 16;   // charged atom types handled by the k-space kernels

__global__ void __launch_bounds__(256) k_ewald_sigma(EwArgs A) {
  double e[1] = {0.0};
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < A.nvecs) {
    double Sr[EW_MAXT], Si[EW_MAXT];
    for (int u = 0; u < A.ntypes; u++) {
      double sr = 0.0, si = 0.0;
      for (int b = 0; b < A.sfBlocks; b++) {
        const double2 p = A.partial[((size_t)b * A.ntypes + u) * A.nvecs + v];
        sr += p.x;
        si += p.y;
      }
      Sr[u] = sr;
      Si[u] = si;
    }
    double d = 0.0;
    for (int t = 0; t < A.ntypes; t++) {
      double r = 0.0, im = 0.0;
      for (int u = 0; u < A.ntypes; u++) {
        const double lam = A.lambda[t * A.ntypes + u];
        r += Sr[u] * lam;
        im += Si[u] * lam;
      }
      A.sigma[(size_t)t * A.nvecs + v] = make_double2(r, im);
      d += Sr[t] * r + Si[t] * im;
    }
    e[0] = A.prefac[v] * d;
  }
  grid_reduce<1, 256>(e, A.epart, A.ticket, A.result);
}

__global__ void __launch_bounds__(FORCE_ATOMS) k_ewald_force(EwArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nm = A.nmax, rows = nm + 1, QS = FORCE_ATOMS;
  double2* G = (double2*)smem;   // [d][m][a]
  const int a = threadIdx.x, j = blockIdx.x * FORCE_ATOMS + a;
  const bool active = j < A.nq;
  int i = 0, t = 0;
  double q = 0.0;
  if (active) {
    i = A.item[j];
    t = A.qtype[j];
    q = A.value[j];
    for (int d = 0; d < 3; d++) power_table(A.R[3 * i + d], A.invL, nm, G + (size_t)d * rows * QS + a, QS);
  }
  if (!active) return;
  const double2* sig = A.sigma + (size_t)t * A.nvecs;
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
  for (int v = 0; v < A.nvecs; v++) {
    const int4 nv = __ldg(&A.n[v]);
    const double2 c = qeikr(q, G[(size_t)nv.x * QS + a], table_get(G + (size_t)rows * QS + a, QS, nv.y),
                            table_get(G + (size_t)2 * rows * QS + a, QS, nv.z));
    const double2 s = __ldg(&sig[v]);
    const double x = s.x * c.y - c.x * s.y;
    f0 += __ldg(&A.vec[3 * v]) * x;
    f1 += __ldg(&A.vec[3 * v + 1]) * x;
    f2 += __ldg(&A.vec[3 * v + 2]) * x;
  }
  A.F[3 * i] += f0;
  A.F[3 * i + 1] += f1;
  A.F[3 * i + 2] += f2;
}

// ---- host -----------------------------------------------------------------------

static int symm1D(int i, int j) {   // src/math.f90:695-702 (1-based)
  int x = std::min(i, j) - 1, y = std::max(i, j) - 1;
  return x + (y + 1) * y / 2 + 1;
}

static double inverse_of_x_plus_ln_x(double y) {   // src/math.f90:642-657
  const double tol = 1.0e-12;
  double x = y > 0.5671432904097839 ? y - std::log(y) : std::exp(y);
  double x0 = x + 1.0;
  while (std::fabs(x - x0) > tol * x0) {
    x0 = x;
    x = x * (y + 1.0 - std::log(x)) / (x + 1.0);
  }
  return x;
}

// src/kspace_ewald.f90:107-170 for a cubic box of edge L
static void ewald_update(Ewald& e, double L) {
  const double unit = 2.0 * EW_PI / L, unitSq = unit * unit;
  const int nmax = (int)std::ceil(e.kmax / unit);
  if (nmax != e.nmax) {
    e.nmax = nmax;
    const long M = 2 * nmax + 1, maxnvecs = M * M * M / 2, M2 = M, M2M3 = M * M;
    const double kmaxSq = unitSq * nmax * nmax;
    e.n.clear();
    for (long i = maxnvecs + 1; i <= 2 * maxnvecs; i++) {
      const long n1 = i / M2M3, j = i - n1 * M2M3, n2 = j / M2, n3 = j - n2 * M2;
      const int k0 = (int)n1 - nmax, k1 = (int)n2 - nmax, k2 = (int)n3 - nmax;
      if (unitSq * k0 * k0 + unitSq * k1 * k1 + unitSq * k2 * k2 <= kmaxSq) {
        e.n.push_back(k0);
        e.n.push_back(k1);
        e.n.push_back(k2);
      }
    }
    e.nvecs = (int)(e.n.size() / 3);
    e.prefac.assign(e.nvecs, 0.0);
    e.vec.assign((size_t)3 * e.nvecs, 0.0);
    const double B = -0.25 / (e.alpha * e.alpha);
    e.Volume = L * L * L;
    const double fourPiByV = 4.0 * EW_PI / e.Volume;
    for (int v = 0; v < e.nvecs; v++) {
      const double k[3] = {unit * e.n[3 * v], unit * e.n[3 * v + 1], unit * e.n[3 * v + 2]};
      const double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
      e.prefac[v] = fourPiByV * std::exp(ksq * B) / ksq;
      for (int d = 0; d < 3; d++) e.vec[3 * v + d] = 2.0 * e.prefac[v] * k[d];
    }
  } else {
    const double factor = e.Volume / (L * L * L);
    for (int v = 0; v < e.nvecs; v++) {
      e.prefac[v] = factor * e.prefac[v];
      for (int d = 0; d < 3; d++) e.vec[3 * v + d] = factor * e.vec[3 * v + d];
    }
    e.Volume = L * L * L;
  }
  e.L = L;
}

void ewald_free(System& s) {
  Ewald& e = s.ewald;
  cudaFree(e.dItem);
  cudaFree(e.dQType);
  cudaFree(e.dFirst);
  cudaFree(e.dLast);
  cudaFree(e.dValue);
  cudaFree(e.dN);
  cudaFree(e.dPrefac);
  cudaFree(e.dVec);
  cudaFree(e.dLambda);
  cudaFree(e.dPartial);
  cudaFree(e.dSigma);
  cudaFree(e.dEnergyPartial);
  e.dItem = e.dQType = e.dFirst = e.dLast = nullptr;
  e.dValue = e.dPrefac = e.dVec = e.dLambda = e.dEnergyPartial = nullptr;
  e.dN = nullptr;
  e.dPartial = e.dSigma = nullptr;
}

template <typename T>
static T* upload_vec(const std::vector<T>& h) {
  T* d = nullptr;
  CK(cudaMalloc(&d, sizeof(T) * std::max<size_t>(h.size(), 1)));
  if (!h.empty()) CK(cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return d;
}

static int sf_block_atoms(int nmax) {
  // shared memory per atom: 3 (nmax + 1) powers of 16 bytes plus the charge
  const size_t perAtom = (size_t)3 * (nmax + 1) * 16 + 8;
  int qb = (int)std::min<size_t>(128, (96 * 1024) / perAtom);
  return std::max(qb, 1);
}

// src/modelClass_kspace.f90:111-243 and src/EmDeeData.f90:403-412
void ewald_initialize(System& s, double kspaceRc) {
  const char* task = "kspace model initialization";
  Ewald& e = s.ewald;
  ewald_free(s);
  e = Ewald();
  const int N = s.natoms;
  const double eps = 2.220446049250313e-16;
  std::vector<char> charged(N);
  int ncharged = 0, maxType = 0;
  for (int i = 0; i < N; i++) {
    charged[i] = std::fabs(s.charge[i]) > eps;
    if (charged[i]) {
      ncharged++;
      maxType = std::max(maxType, s.atomType[i]);
    }
  }
  if (ncharged == 0) fatal(task, "system has no charged atoms");
  std::vector<char> present(maxType + 1, 0);
  for (int i = 0; i < N; i++)
    if (charged[i]) present[s.atomType[i]] = 1;
  std::vector<int> local(maxType + 1, 0);
  for (int t = 1; t <= maxType; t++)
    if (present[t]) {
      e.type.push_back(t);
      local[t] = (int)e.type.size();
    }
  e.ntypes = (int)e.type.size();
  if (e.ntypes > EW_MAXT) fatal(task, "more than 16 types of charged atoms");
  // charge list: every atom of each charged type, type by type
  for (int t = 0; t < e.ntypes; t++) {
    e.first.push_back((int)e.item.size());
    for (int i = 0; i < N; i++)
      if (s.atomType[i] == e.type[t]) {
        e.item.push_back(i);
        e.qtype.push_back(t);
        e.value.push_back(s.charge[i]);
      }
    e.last.push_back((int)e.item.size());
  }
  e.nq = (int)e.item.size();
  // src/kspace_ewald.f90:82-103
  const double acc = s.kspace.accuracy;
  const double sp = std::sqrt(inverse_of_x_plus_ln_x(-std::log(acc)));
  e.alpha = sp / kspaceRc;
  e.kmax = 2.0 * e.alpha * sp;
  printf("KSPACE PARAMETERS: alpha = %10.5f and kmax = %10.5f\n", e.alpha, e.kmax);
  fflush(stdout);
  e.beta = 2.0 * e.alpha / std::sqrt(EW_PI);
  // rigid pairs (positions at initialization) and self energy
  e.nTypePairs = e.ntypes * (e.ntypes - 1) / 2 + e.ntypes;
  e.Erigid.assign(e.nTypePairs, 0.0);
  const double L = *s.Lbox, invL = 1.0 / L;
  std::vector<double> R((size_t)3 * N);
  CK(cudaMemcpy(R.data(), s.dR, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost));
  for (int b = 0; b < s.nbodies; b++) {
    const BodyState& B = s.hBodies[b];
    for (int ii = 0; ii < B.NP - 1; ii++) {
      const int i = s.hBodyAtom[B.first + ii];
      if (!charged[i]) continue;
      for (int jj = ii + 1; jj < B.NP; jj++) {
        const int j = s.hBodyAtom[B.first + jj];
        if (!charged[j]) continue;
        double Rij[3];
        for (int d = 0; d < 3; d++) {
          Rij[d] = R[3 * i + d] - R[3 * j + d];
          Rij[d] = Rij[d] - L * std::round(invL * Rij[d]);
        }
        const double rsq = Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2];
        // src/modelClass_kspace.f90:318-332
        const double QiQj = s.charge[i] * s.charge[j], r = std::sqrt(rsq), x = e.alpha * r, ex = std::exp(-x * x);
        const double Eij = -QiQj * (1.0 - uerfc<double>(x, ex)) / r;
        e.Erigid[symm1D(local[s.atomType[i]], local[s.atomType[j]]) - 1] += Eij;
      }
    }
  }
  for (int t = 1; t <= e.ntypes; t++) {
    double q2 = 0.0;
    for (int k = e.first[t - 1]; k < e.last[t - 1]; k++) q2 += e.value[k] * e.value[k];
    e.Erigid[symm1D(t, t) - 1] -= e.alpha * q2 / std::sqrt(EW_PI);
  }
  // Coulomb constants per type pair and layer (me%pair%kCoul)
  const int nt = e.ntypes, nl = s.nlayers;
  e.lambda.assign((size_t)nt * nt * nl, 0.0);
  e.lambda1D.assign((size_t)e.nTypePairs * nl, 0.0);
  for (int i = 1; i <= nt; i++)
    for (int j = i; j <= nt; j++)
      for (int l = 0; l < nl; l++) {
        const double lam = s.P(e.type[i - 1] - 1, e.type[j - 1] - 1, l).kCoul;
        e.lambda[((size_t)l * nt + (j - 1)) * nt + (i - 1)] = lam;
        e.lambda[((size_t)l * nt + (i - 1)) * nt + (j - 1)] = lam;
        e.lambda1D[(size_t)l * e.nTypePairs + symm1D(i, j) - 1] = lam;
      }
  ewald_update(e, L);
  // device copies
  e.dItem = upload_vec(e.item);
  e.dQType = upload_vec(e.qtype);
  e.dValue = upload_vec(e.value);
  e.dFirst = upload_vec(e.first);
  e.dLast = upload_vec(e.last);
  std::vector<int4> n4(e.nvecs);
  for (int v = 0; v < e.nvecs; v++) n4[v] = make_int4(e.n[3 * v], e.n[3 * v + 1], e.n[3 * v + 2], 0);
  e.dN = upload_vec(n4);
  e.dPrefac = upload_vec(e.prefac);
  e.dVec = upload_vec(e.vec);
  e.dLambda = upload_vec(e.lambda);
  const int qb = sf_block_atoms(e.nmax), blocks = (e.nq + qb - 1) / qb;
  CK(cudaMalloc(&e.dPartial, sizeof(double2) * std::max<size_t>((size_t)blocks * nt * e.nvecs, 1)));
  CK(cudaMalloc(&e.dSigma, sizeof(double2) * std::max<size_t>((size_t)nt * e.nvecs, 1)));
  CK(cudaMalloc(&e.dEnergyPartial, sizeof(double) * std::max(1, (e.nvecs + 255) / 256)));
  // coul_long and other models that need the k-space alpha (src/coul_long.f90:55-64,
  // src/modelClass_coul.f90:101-106)
  for (int l = 0; l < nl; l++) {
    Model& m = s.coul[l];
    if (!m.requires_kspace) continue;
    m.p.alpha = e.alpha;
    if (m.kind == MK_COUL_LONG) m.p.beta = 2.0 * e.alpha / std::sqrt(EW_PI);
  }
  s.modelsUploaded = false;
}

// k-space energy of the current layer (plus the rigid-pair and self discounts);
// forces added to the current layer's force array
double ewald_compute(System& s) {
  Ewald& e = s.ewald;
  const int l = s.layer - 1;
  EwArgs A;
  A.R = s.dR;
  A.invL = 1.0 / *s.Lbox;
  A.nq = e.nq;
  A.nvecs = e.nvecs;
  A.nmax = e.nmax;
  A.ntypes = e.ntypes;
  A.item = e.dItem;
  A.qtype = e.dQType;
  A.value = e.dValue;
  A.first = e.dFirst;
  A.last = e.dLast;
  A.n = e.dN;
  A.prefac = e.dPrefac;
  A.vec = e.dVec;
  A.lambda = e.dLambda + (size_t)l * e.ntypes * e.ntypes;
  A.partial = e.dPartial;
  A.sigma = e.dSigma;
  A.qb = sf_block_atoms(e.nmax);
  A.sfBlocks = (e.nq + A.qb - 1) / A.qb;
  A.F = s.F();
  A.epart = e.dEnergyPartial;
  A.ticket = s.dTicket + 4;
  A.result = s.dResult + 22;
  const int rows = e.nmax + 1;
  const size_t smemSF = (size_t)3 * rows * (A.qb + 1) * sizeof(double2) + (size_t)A.qb * sizeof(double);
  const size_t smemF = (size_t)3 * rows * FORCE_ATOMS * sizeof(double2);
  static size_t setSF = 0, setF = 0;
  if (smemSF > setSF) {
    CK(cudaFuncSetAttribute(k_ewald_sf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemSF));
    setSF = smemSF;
  }
  if (smemF > setF) {
    CK(cudaFuncSetAttribute(k_ewald_force, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemF));
    setF = smemF;
  }
  if (smemSF > 227 * 1024 || smemF > 227 * 1024) fatal("kspace computation", "too many k-vectors per dimension");
  k_ewald_sf<<<A.sfBlocks, SF_THREADS, smemSF, s.stream>>>(A);
  CK(cudaGetLastError());
  k_ewald_sigma<<<(e.nvecs + 255) / 256, 256, 0, s.stream>>>(A);
  CK(cudaGetLastError());
  k_ewald_force<<<(e.nq + FORCE_ATOMS - 1) / FORCE_ATOMS, FORCE_ATOMS, smemF, s.stream>>>(A);
  CK(cudaGetLastError());
  s.prof.total += 3;
  double Ek = 0.0;
  CK(cudaMemcpyAsync(&Ek, s.dResult + 22, sizeof(double), cudaMemcpyDeviceToHost, s.stream));
  CK(cudaStreamSynchronize(s.stream));
  // src/modelClass_kspace.f90:247-314, energy part
  double disc = 0.0;
  for (int k = 0; k < e.nTypePairs; k++) disc += e.lambda1D[(size_t)l * e.nTypePairs + k] * e.Erigid[k];
  return Ek + disc;
}

}  // namespace emdee

// pair_fp64.cu -- pair forces, energies and virials in FP64 with the
// reference's per-pair arithmetic (src/compute.f90:20-100).
//
// Same tiling and lists as the FP32 kernel; the halo holds the scaled FP64
// coordinates Rs = R/L and each pair goes through exactly the operations of the
// reference: Rij = Rs_i - Rs_j, Rij -= anint(Rij), r2 = sum(Rij^2),
// invR2 = invL2/r2, invR = sqrt(invR2), model and modifier, Coulomb term,
// Fij = Wsum*invR2*Rij, and finally F = L*F.  Compiled with -fmad=false so every
// operation rounds as written.  Only the order in which the pair forces of an
// atom are summed differs from the reference (full lists instead of
// Newton's-third-law half lists).
#include "reduce.cuh"
#include "system.hpp"
#include "tile.cuh"

namespace emdee {

static const int PAIR64_THREADS = 128;

struct __align__(32) D4 {
  double x, y, z, w;
};

struct PairArgsD {
  TileGeom g;
  const int2* tab;
  const double* Rs;        // slot order, double[N][3]
  const double* charge;    // API order
  const uint8_t* type8;
  const int* start;
  const int* orig;
  const uint16_t* self;
  const uint16_t* nb;
  const int* count;
  int cap, tileStride, haloCap;
  const PairEntry<double>* table;
  const NBParams<double>* coul;
  int ntypes;
  double Rc2, invL2, L;
  double* F;
  double* partials;
  unsigned int* ticket;
  double* result;
};

template <bool COMPUTE>
__global__ void __launch_bounds__(PAIR64_THREADS) k_pair_fp64(PairArgsD A) {
  extern __shared__ __align__(32) unsigned char sraw[];
  __shared__ int ws[33];
  const TileGeom g = A.g;
  const int t = blockIdx.x, cells = g.TB * g.TB * g.TB;
  D4* hpos = (D4*)sraw;   // Rs.xyz, charge
  int* off = (int*)(hpos + A.haloCap + 1);
  int* cst = off + g.haloCells + 1;
  uint8_t* htype = (uint8_t*)(cst + g.haloCells);
  halo_layout(g, t, A.tab, A.start, off, cst, (int*)nullptr, ws);
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x)
    for (int q = off[h]; q < off[h + 1]; q++) {
      int sj = cst[h] + (q - off[h]);
      hpos[q] = D4{A.Rs[3 * sj], A.Rs[3 * sj + 1], A.Rs[3 * sj + 2], A.charge[A.orig[sj]]};
      htype[q] = A.type8[sj];
    }
  __syncthreads();
  const NBParams<double> coul = *A.coul;
  const int tb = A.start[t * cells], te = A.start[(t + 1) * cells];
  double Ep = 0.0, Ec = 0.0, Wp = 0.0, Wc = 0.0;
  int within = 0;
  for (int li = threadIdx.x; li < te - tb; li += blockDim.x) {
    const int si = tb + li, qi = A.self[si];
    const D4 pi = hpos[qi];
    const int ti = htype[qi];
    const bool ich = fabs(pi.w) > 2.220446049250313e-16;
    const int n = min(A.count[si], A.cap);
    double Fi[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < n; k++) {
      const int qj = A.nb[(((size_t)t * (A.cap >> 3) + (k >> 3)) * A.tileStride + li) * 8 + (k & 7)];
      const D4 pj = hpos[qj];
      double Rij[3] = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
      for (int d = 0; d < 3; d++) Rij[d] = Rij[d] - round(Rij[d]);
      const double r2 = Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2];
      if (r2 < A.Rc2) {
        within++;
        const double invR2 = A.invL2 / r2, invR = sqrt(invR2);
        const PairEntry<double>& pe = A.table[ti * A.ntypes + htype[qj]];
        const bool ijch = ich && fabs(pj.w) > 2.220446049250313e-16;
        const double Wsum = pair_eval<double, COMPUTE>(pe, coul, ijch, pi.w, pj.w, invR, invR2, Ep, Ec, Wp, Wc);
        const double s = Wsum * invR2;
        for (int d = 0; d < 3; d++) Fi[d] += s * Rij[d];
      }
    }
    double* Fa = A.F + 3 * (size_t)A.orig[si];
    for (int d = 0; d < 3; d++) Fa[d] = A.L * Fi[d];
  }
  double v[5] = {0.5 * Ep, 0.5 * Ec, 0.5 * Wp, 0.5 * Wc, 0.5 * (double)within};
  grid_reduce<5, PAIR64_THREADS>(v, A.partials, A.ticket, A.result);
}

void device_pair_forces_fp64(System& s, bool compute, bool useInRc, double rc2scaled) {
  Grid& g = s.grid;
  const double L = *s.Lbox;
  PairArgsD A;
  A.g = make_geom(g.M, g.TB);
  A.tab = g.dHaloTab;
  A.Rs = g.dRs64;
  A.charge = s.dCharge;
  A.type8 = g.dType8;
  A.start = g.dStart;
  A.orig = g.dOrig;
  A.self = g.dSelf;
  A.nb = g.dNb;
  A.count = useInRc ? g.dNbInner : g.dNbCount;
  A.cap = g.cap;
  A.tileStride = g.tileStride;
  A.haloCap = g.maxHalo;
  A.table = s.models.d64 + (size_t)(s.layer - 1) * s.ntypes * s.ntypes;
  A.coul = s.models.coul64 + (s.layer - 1);
  A.ntypes = s.ntypes;
  A.invL2 = 1.0 / (L * L);   // src/EmDeeData.f90:658-659
  A.Rc2 = rc2scaled;
  A.L = L;
  A.F = s.F();
  A.partials = s.dPartials;
  A.ticket = s.dTicket;
  A.result = s.dResult;
  size_t smem = (size_t)(g.maxHalo + 1) * (sizeof(D4) + 1) + sizeof(int) * (2 * g.haloCells + 1) + 16;
  if (compute) {
    CK(cudaFuncSetAttribute(k_pair_fp64<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_pair_fp64<true><<<g.nTiles, PAIR64_THREADS, smem, s.stream>>>(A);
  } else {
    CK(cudaFuncSetAttribute(k_pair_fp64<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_pair_fp64<false><<<g.nTiles, PAIR64_THREADS, smem, s.stream>>>(A);
  }
  CK(cudaGetLastError());
}

}  // namespace emdee

// motion.cu -- phase-space updates (src/EmDeeData.f90:823-922) and the force
// dispatcher.
//
// boost:  P <- CP P + CF F, with the per-dimension 2KE = sum P^2/m when energies
//         are requested (src/EmDeeData.f90:864-922);
// move:   R <- CR R + CP P/m (src/EmDeeData.f90:823-860).
// FP64 throughout; compiled with -fmad=false so each update rounds exactly like
// the reference's statement.
#include "ffkick.cuh"
#include "fpconv.h"
#include "reduce.cuh"
#include <vector>

#include "system.hpp"

namespace emdee {

void device_pair_forces_mixed(System& s, bool compute, bool useInRc, double rc2scaled, int variant);
void device_pair_forces_fp64(System& s, bool compute, bool useInRc, double rc2scaled);

static const int MOTION_THREADS = 256;

// UNITCP: CP == 1, so CP*P == P exactly and is skipped; UNITM: all masses are
// 1, so multiplications by 1/m are skipped.  Both leave every rounding as in
// the reference's statements.  FMA (mixed precision only): the update is one
// fused multiply-add, which halves the work on GB300's narrow FP64 pipe; FP64
// mode keeps the reference's separately rounded statements.
template <bool KIN, bool UNITCP, bool UNITM, bool FMA>
__global__ void __launch_bounds__(MOTION_THREADS) k_boost(double* __restrict__ P, const double* __restrict__ F,
                                                          const double* __restrict__ invMass, int N, double CP,
                                                          double CF, double* partials, unsigned int* ticket,
                                                          double* twoKE) {
  double k2[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double im = (KIN && !UNITM) ? invMass[i] : 1.0;
    for (int d = 0; d < 3; d++) {
      const double base = UNITCP ? P[3 * i + d] : CP * P[3 * i + d];
      double p = FMA ? fma(CF, F[3 * i + d], base) : base + CF * F[3 * i + d];
      P[3 * i + d] = p;
      if (KIN) k2[d] += UNITM ? p * p : im * (p * p);
    }
  }
  if (KIN) grid_reduce<3, MOTION_THREADS>(k2, partials, ticket, twoKE);
}

template <bool UNITCR, bool UNITM, bool FMA>
__global__ void __launch_bounds__(MOTION_THREADS) k_move(double* __restrict__ R, const double* __restrict__ P,
                                                         const double* __restrict__ invMass, int N, double CR,
                                                         double CP) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double im = UNITM ? 1.0 : invMass[i];
  for (int d = 0; d < 3; d++) {
    const double base = UNITCR ? R[3 * i + d] : CR * R[3 * i + d];
    if (FMA) R[3 * i + d] = UNITM ? fma(CP, P[3 * i + d], base) : fma(CP * P[3 * i + d], im, base);
    else R[3 * i + d] = base + (UNITM ? CP * P[3 * i + d] : CP * P[3 * i + d] * im);
  }
}

// grid size cap of the boost kernels: 152 SMs x 8 resident blocks, grid-stride beyond
static constexpr int MOTION_MAX_BLOCKS = 1184;

static int motion_blocks(int N) {
  int b = (N + MOTION_THREADS - 1) / MOTION_THREADS;
  return b < MOTION_MAX_BLOCKS ? b : MOTION_MAX_BLOCKS;
}

// 2KE per dimension = sum over atoms of P^2/m (src/EmDeeData.f90:157-189, free
// atoms), into result[10..12] (and the pinned host copy).  The threads walk the
// flat array P[3N] with a grid stride that is a multiple of 3 (coalesced loads),
// so each thread sums one component; a few hundred blocks keep the FP64 shuffle
// reductions and the block partials few.
// COPY: the momenta come from src (the caller's pinned host buffer, read over the
// host link) and are stored into P on the way.
// SPEC (unit masses, FP32-exact forces F): also 2KE per dimension of P + cf F in
// float-float arithmetic, the kinetic sums of an identical boost that follows (the
// first half-kick of a velocity-Verlet step), into result[56..58]; the F reads ride
// along with the slower reads of src.
template <bool UNITM, bool COPY, bool SPEC>
__global__ void __launch_bounds__(MOTION_THREADS) k_kinetic(const double* __restrict__ src, double* __restrict__ P,
                                                            const double* __restrict__ invMass, int N,
                                                            double* partials, unsigned int* ticket, double* result,
                                                            double* hostResult, const double* __restrict__ F,
                                                            float cfh, float cfl, unsigned int* specTicket) {
  const size_t n3 = 3 * (size_t)N, stride = (size_t)gridDim.x * blockDim.x;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double k = 0.0;
  float sh = 0.f, sl = 0.f;
  for (size_t j = g; j < n3; j += stride) {
    const double p = src[j];
    if (COPY) P[j] = p;
    k += UNITM ? p * p : invMass[j / 3] * (p * p);
    if (SPEC) {
      const float f = ffk_round(F[j]);
      float ph, pl, h, l;
      ffk_split(p, ph, pl);
      const float q = __fmul_rn(cfh, f), qe = fmaf(cfl, f, fmaf(cfh, f, -q));
      ffk_add(ph, pl, q, qe, h, l);
      ffk_sq_acc(h, l, sh, sl);
    }
  }
  const int d = (int)(g % 3);
  double k2[3] = {d == 0 ? k : 0.0, d == 1 ? k : 0.0, d == 2 ? k : 0.0};
  grid_reduce<3, MOTION_THREADS>(k2, partials, ticket, result + 10, hostResult + 10);
  if (SPEC) {
    const float vh[3] = {d == 0 ? sh : 0.f, d == 1 ? sh : 0.f, d == 2 ? sh : 0.f};
    const float vl[3] = {d == 0 ? sl : 0.f, d == 1 ? sl : 0.f, d == 2 ? sl : 0.f};
    grid_reduce_ff2<3, MOTION_THREADS>(vh, vl, reinterpret_cast<float2*>(partials + 3 * gridDim.x), specTicket,
                                       result + 56, hostResult + 56);
  }
}

template <bool FMA>
static void boost_launch(System& s, double CP, double CF, bool kinetic) {
  int N = s.natoms, blocks = motion_blocks(N);
  if (kinetic) {
    if (s.keCap < blocks) {
      CK(cudaFree(s.dKE));
      s.keCap = blocks;
      CK(cudaMalloc(&s.dKE, sizeof(double) * 3 * blocks));
    }
    prof_begin(s, PK_BOOST);
    auto kern = CP == 1.0 ? (s.unitMass ? k_boost<true, true, true, FMA> : k_boost<true, true, false, FMA>)
                          : (s.unitMass ? k_boost<true, false, true, FMA> : k_boost<true, false, false, FMA>);
    kern<<<blocks, MOTION_THREADS, 0, s.stream>>>(s.dP, s.F(), s.dInvMass, N, CP, CF, s.dKE, s.dTicket + 1,
                                                  s.dResult + 10);
    CK(cudaGetLastError());
    prof_end(s, PK_BOOST);
    CK(cudaMemcpyAsync(s.hResult + 10, s.dResult + 10, 3 * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
  } else {
    prof_begin(s, PK_BOOST);
    auto kern = CP == 1.0 ? k_boost<false, true, true, FMA> : k_boost<false, false, true, FMA>;
    kern<<<blocks, MOTION_THREADS, 0, s.stream>>>(s.dP, s.F(), s.dInvMass, N, CP, CF, nullptr, nullptr, nullptr);
    CK(cudaGetLastError());
    prof_end(s, PK_BOOST);
  }
}

void device_boost(System& s, double CP, double CF, bool kinetic) {
  if (s.precision == 0) boost_launch<true>(s, CP, CF, kinetic);
  else boost_launch<false>(s, CP, CF, kinetic);
}

template <bool FMA>
static void move_launch(System& s, double CR, double CP) {
  int N = s.natoms;
  prof_begin(s, PK_MOVE);
  auto kern = CR == 1.0 ? (s.unitMass ? k_move<true, true, FMA> : k_move<true, false, FMA>)
                        : (s.unitMass ? k_move<false, true, FMA> : k_move<false, false, FMA>);
  kern<<<(N + MOTION_THREADS - 1) / MOTION_THREADS, MOTION_THREADS, 0, s.stream>>>(s.dR, s.dP, s.dInvMass, N, CR, CP);
  CK(cudaGetLastError());
  prof_end(s, PK_MOVE);
}

void device_move(System& s, double CR, double CP) {
  if (s.precision == 0) move_launch<true>(s, CR, CP);
  else move_launch<false>(s, CR, CP);
}

// Pending kicks applied on the way out (free atoms, CP = 1): P += CF_k F for each
// pending k in order, with the arithmetic of k_boost, into P and straight into the
// caller's pinned host buffer out.
template <int NK, bool FMA>
__global__ void __launch_bounds__(MOTION_THREADS) k_kick_out(double* __restrict__ P, const double* __restrict__ F,
                                                             size_t n3, double cf0, double cf1,
                                                             double* __restrict__ out) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n3; j += stride) {
    const double f = F[j];
    double p = P[j];
    p = FMA ? fma(cf0, f, p) : p + cf0 * f;
    if (NK == 2) p = FMA ? fma(cf1, f, p) : p + cf1 * f;
    P[j] = p;
    out[j] = p;
  }
}

void device_kick_out(System& s, double* out) {
  const size_t n3 = 3 * (size_t)s.natoms;
  const int blocks = (int)std::min<size_t>((n3 + MOTION_THREADS - 1) / MOTION_THREADS, 8 * 152);
  const double c0 = s.pendCF[0], c1 = s.pendCF[1];
  prof_begin(s, PK_BOOST);
  if (s.precision == 0) {
    if (s.npend == 1) k_kick_out<1, true><<<blocks, MOTION_THREADS, 0, s.stream>>>(s.dP, s.F(), n3, c0, c1, out);
    else k_kick_out<2, true><<<blocks, MOTION_THREADS, 0, s.stream>>>(s.dP, s.F(), n3, c0, c1, out);
  } else {
    if (s.npend == 1) k_kick_out<1, false><<<blocks, MOTION_THREADS, 0, s.stream>>>(s.dP, s.F(), n3, c0, c1, out);
    else k_kick_out<2, false><<<blocks, MOTION_THREADS, 0, s.stream>>>(s.dP, s.F(), n3, c0, c1, out);
  }
  CK(cudaGetLastError());
  prof_end(s, PK_BOOST);
  s.npend = 0;
  CK(cudaStreamSynchronize(s.stream));
}

bool device_kinetic(System& s, double* twoKE, const double* src, const double* specCF) {
  const int N = s.natoms;
  // a multiple of 3 blocks (the grid stride over P[3N] must be), at most 3 per SM
  const int blocks = std::min(3 * ((N + 3 * MOTION_THREADS - 1) / (3 * MOTION_THREADS)), 3 * 152);
  if (s.keCap < 2 * blocks) {   // FP64 partials, then the float-float ones of SPEC
    CK(cudaFree(s.dKE));
    s.keCap = 2 * blocks;
    CK(cudaMalloc(&s.dKE, sizeof(double) * 3 * s.keCap));
  }
  const bool spec = specCF != nullptr && s.unitMass;
  const float ch = spec ? (float)*specCF : 0.f, cl = spec ? (float)(*specCF - (double)ch) : 0.f;
  auto kern = spec ? (src ? k_kinetic<true, true, true> : k_kinetic<true, false, true>)
              : src ? (s.unitMass ? k_kinetic<true, true, false> : k_kinetic<false, true, false>)
                    : (s.unitMass ? k_kinetic<true, false, false> : k_kinetic<false, false, false>);
  // the last block writes the sums into the pinned hResult as well: no copy back
  kern<<<blocks, MOTION_THREADS, 0, s.stream>>>(src ? src : s.dP, s.dP, s.dInvMass, N, s.dKE, s.dTicket + 1,
                                                s.dResult, s.hResult, s.F(), ch, cl, s.dTicket + 8);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s.stream));
  for (int d = 0; d < 3; d++) twoKE[d] = s.hResult[10 + d];
  return spec;
}

// 2KE per dimension of P + cf[0] F + ... + cf[NK] F (the pending kicks and one more,
// applied in order with the fused multiply-adds of k_step_fused) without writing P:
// the kicks stay deferred.  Flat walk over P[3N] as in k_kinetic.
template <int NK, bool UNITM>
__global__ void __launch_bounds__(MOTION_THREADS) k_kinetic_pending(const double* __restrict__ P,
                                                                    const double* __restrict__ F,
                                                                    const double* __restrict__ invMass, int N,
                                                                    double cf0, double cf1, double cf2,
                                                                    double* partials, unsigned int* ticket,
                                                                    double* result, double* hostResult) {
  const size_t n3 = 3 * (size_t)N, stride = (size_t)gridDim.x * blockDim.x;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double k = 0.0;
  for (size_t j = g; j < n3; j += stride) {
    const double f = F[j];
    double p = fma(cf0, f, P[j]);
    if (NK >= 1) p = fma(cf1, f, p);
    if (NK >= 2) p = fma(cf2, f, p);
    k += UNITM ? p * p : invMass[j / 3] * (p * p);
  }
  const int d = (int)(g % 3);
  double k2[3] = {d == 0 ? k : 0.0, d == 1 ? k : 0.0, d == 2 ? k : 0.0};
  grid_reduce<3, MOTION_THREADS>(k2, partials, ticket, result + 10, hostResult + 10);
}

void device_kinetic_pending(System& s, double CF) {
  const int N = s.natoms;
  const int blocks = std::min(3 * ((N + 3 * MOTION_THREADS - 1) / (3 * MOTION_THREADS)), 3 * 152);
  if (s.keCap < blocks) {
    CK(cudaFree(s.dKE));
    s.keCap = blocks;
    CK(cudaMalloc(&s.dKE, sizeof(double) * 3 * blocks));
  }
  // the kicks in application order: pending ones first, then CF
  double c[3] = {CF, 0.0, 0.0};
  for (int k = 0; k < s.npend; k++) c[k] = s.pendCF[k];
  c[s.npend] = CF;
  prof_begin(s, PK_BOOST);
#define KP_LAUNCH(NK)                                                                                          \
  (s.unitMass ? k_kinetic_pending<NK, true> : k_kinetic_pending<NK, false>)<<<blocks, MOTION_THREADS, 0,       \
                                                                              s.stream>>>(                     \
      s.dP, s.F(), s.dInvMass, N, c[0], c[1], c[2], s.dKE, s.dTicket + 1, s.dResult, s.hResult)
  if (s.npend == 0) KP_LAUNCH(0);
  else if (s.npend == 1) KP_LAUNCH(1);
  else KP_LAUNCH(2);
#undef KP_LAUNCH
  CK(cudaGetLastError());
  prof_end(s, PK_BOOST);
  CK(cudaStreamSynchronize(s.stream));
}

// 2KE per dimension of P + CF F and of P + CF F + CF F (two kicks in sequence, as
// k_step_fused applies them), P unchanged: 4 fused multiply-adds per component.
template <bool UNITM>
__global__ void __launch_bounds__(MOTION_THREADS) k_kinetic_two(const double* __restrict__ P,
                                                                const double* __restrict__ F,
                                                                const double* __restrict__ invMass, int N, double cf,
                                                                double* partials, unsigned int* ticket, double* result,
                                                                double* hostResult, const double* skip) {
  if (skip != nullptr && __double_as_longlong(*skip) != 0) return;   // a rebuild is due: nothing to sum
  const size_t n3 = 3 * (size_t)N, stride = (size_t)gridDim.x * blockDim.x;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double k1 = 0.0, k2 = 0.0;
  for (size_t j = g; j < n3; j += stride) {
    const double f = F[j], p1 = fma(cf, f, P[j]), p2 = fma(cf, f, p1);
    if (UNITM) {
      k1 = fma(p1, p1, k1);
      k2 = fma(p2, p2, k2);
    } else {
      const double im = invMass[j / 3];
      k1 = fma(im * p1, p1, k1);
      k2 = fma(im * p2, p2, k2);
    }
  }
  const int d = (int)(g % 3);
  double v[6] = {d == 0 ? k1 : 0.0, d == 1 ? k1 : 0.0, d == 2 ? k1 : 0.0,
                 d == 0 ? k2 : 0.0, d == 1 ? k2 : 0.0, d == 2 ? k2 : 0.0};
  grid_reduce<6, MOTION_THREADS>(v, partials, ticket, result + 48, hostResult + 48);
}

// The same two sums without FP64 arithmetic, for unit masses and forces that are
// exact FP32 values (the mixed-precision pair forces), in float-float arithmetic
// (ffkick.cuh); the sums agree with the FP64 ones to ~1e-14 (relative).
constexpr int KE_FF_LOADS = 4;
__global__ void __launch_bounds__(MOTION_THREADS) k_kinetic_two_ff(const double* __restrict__ P,
                                                                   const double* __restrict__ F, int N, float cfh,
                                                                   float cfl, float2* partials, unsigned int* ticket,
                                                                   double* result, double* hostResult,
                                                                   const double* skip) {
  if (skip != nullptr && __double_as_longlong(*skip) != 0) return;   // a rebuild is due: nothing to sum
  const size_t n3 = 3 * (size_t)N, stride = (size_t)gridDim.x * blockDim.x;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  float a1h = 0.f, a1l = 0.f, a2h = 0.f, a2l = 0.f;
  // KE_FF_LOADS components per thread in flight (the stride is a multiple of 3, so
  // every component of a thread has the same dimension)
  for (size_t j0 = g; j0 < n3; j0 += KE_FF_LOADS * stride) {
    double pv[KE_FF_LOADS], fv[KE_FF_LOADS];
#pragma unroll
    for (int u = 0; u < KE_FF_LOADS; u++) {
      const size_t j = j0 + u * stride;
      pv[u] = j < n3 ? P[j] : 0.0;
      fv[u] = j < n3 ? F[j] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < KE_FF_LOADS; u++) {
      if (j0 + u * stride >= n3) break;
      ffk_two_kicks(pv[u], ffk_round(fv[u]), cfh, cfl, a1h, a1l, a2h, a2l);
    }
  }
  const int d = (int)(g % 3);
  float vh[6] = {d == 0 ? a1h : 0.f, d == 1 ? a1h : 0.f, d == 2 ? a1h : 0.f,
                 d == 0 ? a2h : 0.f, d == 1 ? a2h : 0.f, d == 2 ? a2h : 0.f};
  float vl[6] = {d == 0 ? a1l : 0.f, d == 1 ? a1l : 0.f, d == 2 ? a1l : 0.f,
                 d == 0 ? a2l : 0.f, d == 1 ? a2l : 0.f, d == 2 ? a2l : 0.f};
  grid_reduce_ff2<6, MOTION_THREADS>(vh, vl, partials, ticket, result + 48, hostResult + 48);
}

// skip: a device flag (0.0 or 1.0, tested on its bits) that makes the pass return at
// once; the pass is queued without waiting for it
static void launch_kinetic_two(System& s, double CF, const double* skip) {
  const int N = s.natoms;
  const int blocks = std::min(3 * ((N + 3 * MOTION_THREADS - 1) / (3 * MOTION_THREADS)), 3 * 152);
  // the float-float pass is latency-bound: as many blocks as fit at once (five per
  // SM at its 47 registers, rounded down to a multiple of 3), each thread with
  // KE_FF_LOADS loads in flight
  const int ffBlocks = std::min(3 * ((N + 3 * MOTION_THREADS - 1) / (3 * MOTION_THREADS)), 5 * 152 / 3 * 3);
  if (s.keCap < 2 * ffBlocks) {   // partials: 6 doubles (or float pairs) per block
    CK(cudaFree(s.dKE));
    s.keCap = 2 * ffBlocks;
    CK(cudaMalloc(&s.dKE, sizeof(double) * 3 * s.keCap));
  }
  prof_begin(s, PK_BOOST);
  static const bool fp64Only = getenv("EMDEE_KE_FP64") != nullptr;   // tuning switch: the FP64 pass
  if (s.unitMass && s.forcesF32 && !fp64Only) {
    const float ch = (float)CF, cl = (float)(CF - (double)ch);
    k_kinetic_two_ff<<<ffBlocks, MOTION_THREADS, 0, s.stream>>>(s.dP, s.F(), N, ch, cl, (float2*)s.dKE,
                                                             s.dTicket + 1, s.dResult, s.hResult, skip);
  } else {
    (s.unitMass ? k_kinetic_two<true> : k_kinetic_two<false>)<<<blocks, MOTION_THREADS, 0, s.stream>>>(
        s.dP, s.F(), s.dInvMass, N, CF, s.dKE, s.dTicket + 1, s.dResult, s.hResult, skip);
  }
  CK(cudaGetLastError());
  prof_end(s, PK_BOOST);
}

void device_kinetic_two(System& s, double CF) {
  launch_kinetic_two(s, CF, nullptr);
  CK(cudaStreamSynchronize(s.stream));
}

void flush_pending(System& s) {
  for (int k = 0; k < s.npend; k++) device_boost(s, 1.0, s.pendCF[k], false);
  s.npend = 0;
}

// Chooses the force kernel for the current layer and leaves the four sums in
// hResult[0..3] (src/EmDeeData.f90:644-685).
// single-type Lennard-Jones without charges takes the specialised kernel
bool pair_lj_only(System& s) {
  const int l = s.layer - 1;
  return s.ntypes == 1 && s.P(0, 0, l).model.kind == MK_LJ_CUT &&
         !(s.P(0, 0, l).coulomb && s.coul[l].kind != MK_COUL_NONE);
}

bool device_pair_forces(System& s, bool compute, bool speculative) {
  const int l = s.layer - 1;
  const double L = *s.Lbox, invL2 = 1.0 / (L * L);
  const bool useInRc = s.useInRc[l] != 0;
  const double rc2 = (useInRc ? s.InRcSq : s.RcSq) * invL2;   // src/EmDeeData.f90:660-667
  if (!s.pairs_exist[l]) {
    CK(cudaMemsetAsync(s.F(), 0, sizeof(double) * 3 * s.natoms, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    for (int q = 0; q < 4; q++) s.hResult[q] = 0.0;
    return true;
  }
  if (s.partialCap < s.grid.nTiles) {
    CK(cudaFree(s.dPartials));
    s.partialCap = s.grid.nTiles;
    CK(cudaMalloc(&s.dPartials, sizeof(double) * 5 * s.partialCap));
  }
  prof_begin(s, PK_PAIR);
  if (s.precision == 1) {
    device_pair_forces_fp64(s, compute, useInRc, rc2);
  } else {
    s.pairSkip = speculative ? s.dResult + 9 : nullptr;
    device_pair_forces_mixed(s, compute, useInRc, rc2, pair_lj_only(s) ? 0 : 1);
    s.pairSkip = nullptr;
  }
  prof_end(s, PK_PAIR);
  // A boost that waits for these forces (free atoms, no bond, angle or k-space forces
  // to be added to them) gets its kinetic sums from a pass queued right behind the
  // pair kernel, which skips it too when a rebuild is due
  const int l2 = s.layer - 1;
  const bool chain = s.keChainReq && s.precision == 0 && s.nbodies == 0 && s.bondedTerms.bonds.empty() &&
                     s.bondedTerms.angles.empty() && !s.coul[l2].requires_kspace;
  if (chain) launch_kinetic_two(s, s.keChainCF, speculative ? s.dResult + 9 : nullptr);
  // Mixed precision: the last block of the pair kernel wrote the sums, and the fused
  // step the skin value and rebuild flag ([8], [9]), straight into the pinned hResult,
  // so one synchronisation returns all of them.  FP64 mode copies them back.
  if (s.precision == 1)
    CK(cudaMemcpyAsync(s.hResult, s.dResult, (speculative ? 10 : 4) * sizeof(double), cudaMemcpyDeviceToHost,
                       s.stream));
  CK(cudaStreamSynchronize(s.stream));
  if (speculative && s.hResult[9] != 0.0) {
    if (chain) prof_drop_last(s);   // the kinetic pass returned at once as well
    prof_drop_last(s);
    return false;
  }
  if (chain) s.keChained = true;
  return true;
}

// Half-list statistics: entries of the current lists and pairs within the
// cut-off at the last force evaluation (used for algorithmic FLOP counts).
void device_pair_statistics(System& s, long* listed, long* within) {
  long total = 0;
  if (s.r0Valid) {
    std::vector<int> cnt(s.natoms);
    CK(cudaStreamSynchronize(s.stream));
    CK(cudaMemcpy(cnt.data(), s.grid.dNbCount, sizeof(int) * s.natoms, cudaMemcpyDeviceToHost));
    for (int c : cnt) total += c;
  }
  double w = 0.0;
  if (s.r0Valid && s.precision == 0 && s.pairs_exist[s.layer - 1]) {
    const double L = *s.Lbox;
    const bool useInRc = s.useInRc[s.layer - 1] != 0;
    device_pack(s);
    device_pair_forces_mixed(s, false, useInRc, (useInRc ? s.InRcSq : s.RcSq) / (L * L), 2);
    CK(cudaMemcpyAsync(&w, s.dResult + 4, sizeof(double), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
  } else {
    CK(cudaMemcpy(&w, s.dResult + 4, sizeof(double), cudaMemcpyDeviceToHost));
  }
  if (listed) *listed = total / 2;
  if (within) *within = (long)(w + 0.5);
}

// ---------------------------------------------------------------------------------
// EmDee_boost_noalloc: the boost + kinetic-energy kernel on caller-owned device
// arrays, with its scratch in a fixed device array instead of cudaMalloc.
//
// Who needs it: callers that must not allocate device memory at the point of
// the call -- processes whose device memory is owned by another allocator (a
// framework's caching allocator or a pool reserved at start-up), and loops that
// cannot take the device-wide synchronization that cudaMalloc/cudaFree may
// imply.  It is called from ordinary host code, like every entry point: CUDA
// forbids CUDA calls inside a stream's host function, and this one makes some.
//
// The scratch holds one partial sum per thread block (3 doubles) and the
// completion ticket of the grid reduction.  It lives in every GPU that loads
// this library until the process exits.  All calls share it: calls that
// overlap on the GPU (different streams, different host threads) race, so
// serialize them.  The first call on each device looks up the array's device
// address (cudaGetSymbolAddress); make that first call before any stream
// capture.
// ---------------------------------------------------------------------------------

namespace {

const int NOALLOC_MAX_BLOCKS = MOTION_MAX_BLOCKS;   // one partial per block of the boost grid
static_assert(NOALLOC_MAX_BLOCKS >= MOTION_MAX_BLOCKS, "the scratch must hold a partial for every block");
const long long NOALLOC_MAX_ATOMS = 715827882LL;   // 3N must fit in a signed 32-bit index
// [0, 3*MAX_BLOCKS) per-block partial sums; [3*MAX_BLOCKS] ticket (as 8 bytes)
static __device__ __align__(256) double g_noalloc_scratch[3 * NOALLOC_MAX_BLOCKS + 1];

void* noalloc_scratch_address() {
  static void* addr[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      fprintf(stderr, "Error in boost_noalloc: cannot locate the scratch array on device %d (%s).\n", dev,
              cudaGetErrorString(e));
      return nullptr;
    }
    addr[dev] = p;
  }
  return addr[dev];
}

}  // namespace

}  // namespace emdee

// P <- CP P + CF F for N atoms (device arrays double[N][3]) and, in twoKE
// (device double[3]), 2KE per dimension = sum over atoms of P^2/m with the
// updated momenta.  invMass is a device double[N] array, or NULL for unit
// masses.  Returns 0 on success, 1 for a size outside [1, 715827882] atoms or a
// NULL P, F or twoKE, 2 for a CUDA error; the reason is printed on stderr.
// Allocates no memory.
extern "C" int EmDee_boost_noalloc(double* P, const double* F, const double* invMass, int N, double CP, double CF,
                                   double* twoKE, void* stream) {
  using namespace emdee;
  if (N < 1 || (long long)N > NOALLOC_MAX_ATOMS) {
    fprintf(stderr, "Error in boost_noalloc: %d atoms is outside the supported range [1, %lld].\n", N,
            NOALLOC_MAX_ATOMS);
    return 1;
  }
  if (!P || !F || !twoKE) {
    fprintf(stderr, "Error in boost_noalloc: the momenta, forces and kinetic-energy arrays must not be NULL.\n");
    return 1;
  }
  double* scratch = (double*)noalloc_scratch_address();
  if (!scratch) return 2;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned int* ticket = (unsigned int*)(scratch + 3 * NOALLOC_MAX_BLOCKS);
  // the ticket must start at zero; partial sums are overwritten before use
  cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st);
  int blocks = motion_blocks(N);
  bool unitCP = CP == 1.0, unitM = invMass == nullptr;
  auto kern = unitCP ? (unitM ? k_boost<true, true, true, false> : k_boost<true, true, false, false>)
                     : (unitM ? k_boost<true, false, true, false> : k_boost<true, false, false, false>);
  if (e == cudaSuccess) {
    kern<<<blocks, MOTION_THREADS, 0, st>>>(P, F, invMass, N, CP, CF, scratch, ticket, twoKE);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "Error in boost_noalloc: %s.\n", cudaGetErrorString(e));
    return 2;
  }
  return 0;
}

// bodies.cu -- rigid bodies on the device: per-body force and torque, momentum
// and position updates, exact or NO_SQUISH rotation, kinetic energies, the
// rigid-body virial, and momentum assignment (src/EmDeeData.f90:157-189,
// 420-439, 823-953; src/ArBee.f90).  One thread per body, FP64, compiled with
// -fmad=false.  Free atoms of a system with bodies go through index-list
// variants of the boost and move kernels.
#include <vector>

#include "reduce.cuh"
#include "bodies.cuh"
#include "rigid.cuh"
#include "system.hpp"

namespace emdee {

static const int BODY_THREADS = 128;


// force_and_torque, then pcm and pi updates; 2KE translational (bodies) and
// rotational partial sums
__global__ void __launch_bounds__(BODY_THREADS) k_body_boost(BodyArgs A, const double* __restrict__ F, double CP,
                                                             double CF, int translate, int rotate, int kinetic,
                                                             double* partials, unsigned int* ticket, double* result) {
  double k6[6] = {0, 0, 0, 0, 0, 0};
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.nb) {
    BodyState b = A.b[i];
    for (int k = 0; k < 3; k++) b.F[k] = b.tau[k] = 0.0;
    for (int j = 0; j < b.NP; j++) {
      const double* Fj = &F[3 * A.atom[b.first + j]];
      double c[3];
      rb_cross(&A.delta[3 * (b.first + j)], Fj, c);
      for (int k = 0; k < 3; k++) {
        b.F[k] += Fj[k];
        b.tau[k] += c[k];
      }
    }
    if (translate)
      for (int k = 0; k < 3; k++) b.pcm[k] = CP * b.pcm[k] + CF * b.F[k];
    if (rotate) {
      double Ctau = 2.0 * CF, v[3] = {Ctau * b.tau[0], Ctau * b.tau[1], Ctau * b.tau[2]}, c[4], pi[4];
      rb_C(b.q, v, c);
      for (int k = 0; k < 4; k++) pi[k] = CP * b.pi[k] + c[k];
      rb_assign_pi(b, pi);
    }
    if (kinetic)
      for (int k = 0; k < 3; k++) {
        k6[k] = b.invMass * (b.pcm[k] * b.pcm[k]);
        k6[3 + k] = b.MoI[k] * (b.omega[k] * b.omega[k]);
      }
    A.b[i] = b;
  }
  if (kinetic) grid_reduce<6, BODY_THREADS>(k6, partials, ticket, result);
}

// rcm update, rotation, atom positions rcm + delta (rotation branch only, as the reference)
__global__ void __launch_bounds__(BODY_THREADS) k_body_move(BodyArgs A, double* __restrict__ R, double CR, double CP,
                                                            double dt, int translate, int rotate, int mode) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.nb) return;
  BodyState b = A.b[i];
  if (translate)
    for (int k = 0; k < 3; k++) b.rcm[k] = CR * b.rcm[k] + CP * b.invMass * b.pcm[k];
  if (rotate) {
    const double* d = &A.d[3 * b.first];
    double* delta = &A.delta[3 * b.first];
    if (mode == 0) rb_rotate_exact(b, dt, d, delta);
    else rb_rotate_no_squish(b, dt, mode, d, delta);
    for (int j = 0; j < b.NP; j++)
      for (int k = 0; k < 3; k++) R[3 * A.atom[b.first + j] + k] = b.rcm[k] + delta[3 * j + k];
  }
  A.b[i] = b;
}

// W = sum over bodies and their atoms of F . delta (the body virial is -W)
__global__ void __launch_bounds__(BODY_THREADS) k_body_virial(BodyArgs A, const double* __restrict__ F,
                                                              double* partials, unsigned int* ticket, double* result) {
  double w[1] = {0.0};
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.nb) {
    const BodyState& b = A.b[i];
    for (int j = 0; j < b.NP; j++)
      for (int k = 0; k < 3; k++) w[0] += F[3 * A.atom[b.first + j] + k] * A.delta[3 * (b.first + j) + k];
  }
  grid_reduce<1, BODY_THREADS>(w, partials, ticket, result);
}

// momenta of body atoms -> pcm, pi, omega (src/EmDeeData.f90:172-186), with 2KE sums
__global__ void __launch_bounds__(BODY_THREADS) k_body_assign(BodyArgs A, const double* __restrict__ P,
                                                              double* partials, unsigned int* ticket, double* result) {
  double k6[6] = {0, 0, 0, 0, 0, 0};
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.nb) {
    BodyState b = A.b[i];
    double Lm[3] = {0, 0, 0}, v[3], pi[4];
    for (int k = 0; k < 3; k++) b.pcm[k] = 0.0;
    for (int j = 0; j < b.NP; j++) {
      const double* Pj = &P[3 * A.atom[b.first + j]];
      double c[3];
      for (int k = 0; k < 3; k++) b.pcm[k] += Pj[k];
      rb_cross(&A.delta[3 * (b.first + j)], Pj, c);
      for (int k = 0; k < 3; k++) Lm[k] += c[k];
    }
    for (int k = 0; k < 3; k++) {
      k6[k] = b.invMass * (b.pcm[k] * b.pcm[k]);
      v[k] = 2.0 * Lm[k];
    }
    rb_C(b.q, v, pi);
    rb_assign_pi(b, pi);
    for (int k = 0; k < 3; k++) k6[3 + k] = b.MoI[k] * (b.omega[k] * b.omega[k]);
    A.b[i] = b;
  }
  grid_reduce<6, BODY_THREADS>(k6, partials, ticket, result);
}

// particle momenta of body atoms (src/ArBee.f90:328-336) into P
__global__ void __launch_bounds__(BODY_THREADS) k_body_particle_momenta(BodyArgs A, double* P) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.nb) return;
  const BodyState& b = A.b[i];
  double t[4], omega[3];
  rb_B(b.q, b.omega, t);
  rb_Ct(b.q, t, omega);
  for (int j = 0; j < b.NP; j++) {
    double c[3];
    rb_cross(omega, &A.delta[3 * (b.first + j)], c);
    double m = A.M[b.first + j];
    for (int k = 0; k < 3; k++) P[3 * A.atom[b.first + j] + k] = m * (b.invMass * b.pcm[k] + c[k]);
  }
}

// free atoms only: boost and move through the free-atom list
template <bool KIN>
__global__ void __launch_bounds__(BODY_THREADS) k_boost_free(double* __restrict__ P, const double* __restrict__ F,
                                                             const double* __restrict__ invMass, const int* freeList,
                                                             int nfree, double CP, double CF, double* partials,
                                                             unsigned int* ticket, double* result) {
  double k2[3] = {0.0, 0.0, 0.0};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nfree; q += gridDim.x * blockDim.x) {
    int i = freeList[q];
    for (int d = 0; d < 3; d++) {
      double p = CP * P[3 * i + d] + CF * F[3 * i + d];
      P[3 * i + d] = p;
      if (KIN) k2[d] += invMass[i] * (p * p);
    }
  }
  if (KIN) grid_reduce<3, BODY_THREADS>(k2, partials, ticket, result);
}

__global__ void __launch_bounds__(BODY_THREADS) k_move_free(double* __restrict__ R, const double* __restrict__ P,
                                                            const double* __restrict__ invMass, const int* freeList,
                                                            int nfree, double CR, double CP) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nfree) return;
  int i = freeList[q];
  for (int d = 0; d < 3; d++) R[3 * i + d] = CR * R[3 * i + d] + CP * P[3 * i + d] * invMass[i];
}

// ---- host side -------------------------------------------------------------------


static int body_blocks(int n) { return n > 0 ? (n + BODY_THREADS - 1) / BODY_THREADS : 1; }

static void ensure_scratch(System& s, int blocks, int nq) {
  int need = blocks * nq;
  if (s.bodyScratchCap < need) {
    CK(cudaFree(s.dBodyScratch));
    s.bodyScratchCap = need;
    CK(cudaMalloc(&s.dBodyScratch, sizeof(double) * need));
  }
}

// src/EmDeeData.f90:420-439: unwrap every body around its first atom, rebuild its
// frame on the host, and upload the unwrapped coordinates and the bodies
void bodies_update(System& s) {
  if (s.nbodies == 0) return;
  int N = s.natoms;
  std::vector<double> R((size_t)3 * N);
  CK(cudaMemcpyAsync(R.data(), s.dR, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s.stream));
  CK(cudaStreamSynchronize(s.stream));
  double L = *s.Lbox, invL = 1.0 / L;
  for (int bi = 0; bi < s.nbodies; bi++) {
    BodyState& b = s.hBodies[bi];
    std::vector<double> c((size_t)3 * b.NP);
    for (int j = 0; j < b.NP; j++)
      for (int k = 0; k < 3; k++) c[3 * j + k] = R[3 * s.hBodyAtom[b.first + j] + k];
    for (int j = 1; j < b.NP; j++)
      for (int k = 0; k < 3; k++) c[3 * j + k] = c[3 * j + k] - L * std::round(invL * (c[3 * j + k] - c[k]));
    rb_update(b, &s.hBodyM[b.first], c.data(), &s.hBodyD[3 * b.first], &s.hBodyDelta[3 * b.first]);
    for (int j = 0; j < b.NP; j++)
      for (int k = 0; k < 3; k++) R[3 * s.hBodyAtom[b.first + j] + k] = c[3 * j + k];
  }
  // keep the dynamic state (pcm, pi, omega) the device holds
  std::vector<BodyState> dev(s.nbodies);
  CK(cudaMemcpy(dev.data(), s.dBodies, sizeof(BodyState) * s.nbodies, cudaMemcpyDeviceToHost));
  for (int bi = 0; bi < s.nbodies; bi++) {
    BodyState& b = s.hBodies[bi];
    for (int k = 0; k < 3; k++) {
      b.pcm[k] = dev[bi].pcm[k];
      b.omega[k] = dev[bi].omega[k];
      b.F[k] = dev[bi].F[k];
      b.tau[k] = dev[bi].tau[k];
    }
    for (int k = 0; k < 4; k++) b.pi[k] = dev[bi].pi[k];
  }
  size_t na = s.hBodyAtom.size();
  CK(cudaMemcpy(s.dBodies, s.hBodies.data(), sizeof(BodyState) * s.nbodies, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.dBodyD, s.hBodyD.data(), sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.dBodyDelta, s.hBodyDelta.data(), sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.dR, R.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice));
}

// boost of free atoms (through the list) and bodies; 2KE into hResult[10..12]
// (translational) and [13..15] (rotational)
void bodies_boost(System& s, double CP, double CF, bool translate, bool rotate, bool kinetic) {
  double kt[3] = {0, 0, 0};
  int freeBlocks = std::min(body_blocks(s.nfree), 1184);
  ensure_scratch(s, std::max(freeBlocks * 3, body_blocks(s.nbodies) * 6), 1);
  if (translate && s.nfree > 0) {
    int blocks = freeBlocks;
    if (kinetic) {
      k_boost_free<true><<<blocks, BODY_THREADS, 0, s.stream>>>(s.dP, s.F(), s.dInvMass, s.dFree, s.nfree, CP, CF,
                                                                s.dBodyScratch, s.dTicket + 2, s.dResult + 10);
      CK(cudaMemcpyAsync(kt, s.dResult + 10, sizeof(kt), cudaMemcpyDeviceToHost, s.stream));
    } else {
      k_boost_free<false><<<blocks, BODY_THREADS, 0, s.stream>>>(s.dP, s.F(), s.dInvMass, s.dFree, s.nfree, CP, CF,
                                                                 nullptr, nullptr, nullptr);
    }
    CK(cudaGetLastError());
    s.prof.total++;
  }
  int blocks = body_blocks(s.nbodies);
  k_body_boost<<<blocks, BODY_THREADS, 0, s.stream>>>(body_args(s), s.F(), CP, CF, translate, rotate, kinetic,
                                                       s.dBodyScratch + 0, s.dTicket + 3, s.dResult + 16);
  CK(cudaGetLastError());
  s.prof.total++;
  if (kinetic) {
    double k6[6];
    CK(cudaMemcpyAsync(k6, s.dResult + 16, sizeof(k6), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    for (int k = 0; k < 3; k++) {
      s.hResult[10 + k] = (translate && s.nfree > 0 ? kt[k] : 0.0) + k6[k];
      s.hResult[13 + k] = k6[3 + k];
    }
  }
}

void bodies_move(System& s, double CR, double CP, double dt, bool translate, bool rotate, int mode) {
  if (translate && s.nfree > 0) {
    k_move_free<<<body_blocks(s.nfree), BODY_THREADS, 0, s.stream>>>(s.dR, s.dP, s.dInvMass, s.dFree, s.nfree, CR,
                                                                      CP);
    CK(cudaGetLastError());
    s.prof.total++;
  }
  // one warp per block: the exact rotation is a long serial FP64 computation per
  // body, so bodies are spread over as many SMs as possible
  k_body_move<<<(s.nbodies + 31) / 32, 32, 0, s.stream>>>(body_args(s), s.dR, CR, CP, dt, translate, rotate, mode);
  CK(cudaGetLastError());
  s.prof.total++;
}

double bodies_virial(System& s) {
  int blocks = body_blocks(s.nbodies);
  ensure_scratch(s, blocks, 1);
  k_body_virial<<<blocks, BODY_THREADS, 0, s.stream>>>(body_args(s), s.F(), s.dBodyScratch, s.dTicket + 3,
                                                        s.dResult + 6);
  CK(cudaGetLastError());
  s.prof.total++;
  double w = 0.0;
  CK(cudaMemcpyAsync(&w, s.dResult + 6, sizeof(double), cudaMemcpyDeviceToHost, s.stream));
  CK(cudaStreamSynchronize(s.stream));
  return -w;
}

// bodies take their momenta from the particle momenta in dP; 2KE of bodies into k6
void bodies_assign(System& s, double* k6) {
  int blocks = body_blocks(s.nbodies);
  ensure_scratch(s, blocks, 6);
  k_body_assign<<<blocks, BODY_THREADS, 0, s.stream>>>(body_args(s), s.dP, s.dBodyScratch, s.dTicket + 3,
                                                       s.dResult + 16);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(k6, s.dResult + 16, 6 * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
  CK(cudaStreamSynchronize(s.stream));
}

void bodies_particle_momenta(System& s, double* dOut) {
  k_body_particle_momenta<<<body_blocks(s.nbodies), BODY_THREADS, 0, s.stream>>>(body_args(s), dOut);
  CK(cudaGetLastError());
}

void bodies_download(System& s) {
  CK(cudaStreamSynchronize(s.stream));
  CK(cudaMemcpy(s.hBodies.data(), s.dBodies, sizeof(BodyState) * s.nbodies, cudaMemcpyDeviceToHost));
}

void bodies_upload(System& s) {
  CK(cudaMemcpy(s.dBodies, s.hBodies.data(), sizeof(BodyState) * s.nbodies, cudaMemcpyHostToDevice));
}

}  // namespace emdee

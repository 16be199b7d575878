// verlet.cu -- EmDee_verlet_step: one velocity-Verlet step with the
// shadow-Hamiltonian terms of src/EmDeeCode.f90:1107-1211.
//
// pre  (per free atom / per body, fused): the shadow start values s0 / r0, q0
//      (q0 from a virtual rotation by -dt), then boost(1, dt/2) and move(1, dt)
//      with translation and rotation on;
// forces (compute_forces, unconditional);
// post (fused): boost(1, dt/2), then the kinetic energies per dimension,
//      Ks_t = sum rdot . p, Ks_r (quaternion part) and Us = sum F^2/m + tau_b^2/I,
//      in deterministic grid reductions.
// FP64, -fmad=false: every statement rounds like the oracle's.
#include <algorithm>

#include "bodies.cuh"
#include "reduce.cuh"
#include "system.hpp"

namespace emdee {

static const int VV_THREADS = 128;

// list == nullptr: atoms 0..n-1; otherwise the atoms list[0..n-1]
template <bool COMPUTE, bool FMA>
__global__ void __launch_bounds__(VV_THREADS) k_vv_pre_free(double* __restrict__ R, double* __restrict__ P,
                                                            const double* __restrict__ F,
                                                            const double* __restrict__ invMass, const int* list,
                                                            int n, double dt, double dt_2, double* __restrict__ s0) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int j = list ? list[q] : q;
  const double im = invMass[j];
  for (int d = 0; d < 3; d++) {
    const double p = P[3 * j + d], f = F[3 * j + d];
    if (COMPUTE) s0[3 * q + d] = 2.5 * R[3 * j + d] + dt_2 * im * (p - dt_2 * f);
    const double pn = FMA ? fma(dt_2, f, p) : 1.0 * p + dt_2 * f;
    P[3 * j + d] = pn;
    R[3 * j + d] = FMA ? (list == nullptr && im == 1.0 ? fma(dt, pn, R[3 * j + d]) : fma(dt * pn, im, R[3 * j + d]))
                       : 1.0 * R[3 * j + d] + dt * pn * im;
  }
}

// v[0..2] 2KE_t per dimension, v[3] Ks_t, v[4] Us
template <bool COMPUTE, bool FMA>
__global__ void __launch_bounds__(VV_THREADS) k_vv_post_free(const double* __restrict__ R, double* __restrict__ P,
                                                             const double* __restrict__ F,
                                                             const double* __restrict__ invMass, const int* list,
                                                             int n, double dt, double dt_2,
                                                             const double* __restrict__ s0, double* partials,
                                                             unsigned int* ticket, double* result) {
  double v[5] = {0, 0, 0, 0, 0};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int j = list ? list[q] : q;
    const double im = invMass[j];
    double p[3], f[3];
    for (int d = 0; d < 3; d++) {
      f[d] = F[3 * j + d];
      p[d] = FMA ? fma(dt_2, f[d], P[3 * j + d]) : 1.0 * P[3 * j + d] + dt_2 * f[d];
      P[3 * j + d] = p[d];
    }
    if (COMPUTE) {
      for (int d = 0; d < 3; d++) {
        v[d] += im * (p[d] * p[d]);
        const double rdot = 2.5 * R[3 * j + d] + dt * im * (p[d] + dt_2 * f[d]) - s0[3 * q + d];
        v[3] += rdot * p[d];
      }
      v[4] += im * (f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    }
  }
  if (COMPUTE) grid_reduce<5, VV_THREADS>(v, partials, ticket, result);
}

// force and torque, then pcm += CF F, pi += C(q) 2 CF tau (boost with both flags on)
__device__ __forceinline__ void vv_body_boost(BodyState& b, const BodyArgs& A, const double* F, double CF) {
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
  for (int k = 0; k < 3; k++) b.pcm[k] = 1.0 * b.pcm[k] + CF * b.F[k];
  const double Ctau = 2.0 * CF, v[3] = {Ctau * b.tau[0], Ctau * b.tau[1], Ctau * b.tau[2]};
  double c[4], pi[4];
  rb_C(b.q, v, c);
  for (int k = 0; k < 4; k++) pi[k] = 1.0 * b.pi[k] + c[k];
  rb_assign_pi(b, pi);
}

// quaternion of a copy of the body after pi += C(q) dt tau and a free rotation by dt
__device__ __forceinline__ void vv_virtual_rotation(const BodyState& b, double dt, int mode, const double* d,
                                                    double* qout) {
  BodyState c = b;
  const double v[3] = {dt * c.tau[0], dt * c.tau[1], dt * c.tau[2]};
  double t[4], pi[4];
  rb_C(c.q, v, t);
  for (int k = 0; k < 4; k++) pi[k] = c.pi[k] + t[k];
  rb_assign_pi(c, pi);
  if (mode != 0) rb_rotate_no_squish(c, dt, mode, d, nullptr);
  else rb_rotate_exact(c, dt, d, nullptr);
  for (int k = 0; k < 4; k++) qout[k] = c.q[k];
}

template <bool COMPUTE>
__global__ void __launch_bounds__(VV_THREADS) k_vv_pre_body(BodyArgs A, const double* __restrict__ F,
                                                            double* __restrict__ R, double dt, double dt_2, int mode,
                                                            double* __restrict__ r0, double* __restrict__ q0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.nb) return;
  BodyState b = A.b[i];
  const double* d = &A.d[3 * b.first];
  if (COMPUTE) {
    double qv[4];
    for (int k = 0; k < 3; k++) r0[3 * i + k] = 2.5 * b.rcm[k] + dt_2 * b.invMass * (b.pcm[k] - dt_2 * b.F[k]);
    vv_virtual_rotation(b, -dt, mode, d, qv);
    for (int k = 0; k < 4; k++) q0[4 * i + k] = 0.5 * qv[k] - 3.0 * b.q[k];
  }
  vv_body_boost(b, A, F, dt_2);
  for (int k = 0; k < 3; k++) b.rcm[k] = 1.0 * b.rcm[k] + dt * b.invMass * b.pcm[k];
  double* delta = &A.delta[3 * b.first];
  if (mode == 0) rb_rotate_exact(b, dt, d, delta);
  else rb_rotate_no_squish(b, dt, mode, d, delta);
  for (int j = 0; j < b.NP; j++)
    for (int k = 0; k < 3; k++) R[3 * A.atom[b.first + j] + k] = b.rcm[k] + delta[3 * j + k];
  A.b[i] = b;
}

// v[0..2] 2KE_t, v[3..5] 2KE_r, v[6] Ks_t, v[7] Ks_r, v[8] Us
template <bool COMPUTE>
__global__ void __launch_bounds__(VV_THREADS) k_vv_post_body(BodyArgs A, const double* __restrict__ F, double dt,
                                                             double dt_2, int mode, const double* __restrict__ r0,
                                                             const double* __restrict__ q0, double* partials,
                                                             unsigned int* ticket, double* result) {
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.nb) {
    BodyState b = A.b[i];
    vv_body_boost(b, A, F, dt_2);
    if (COMPUTE) {
      for (int k = 0; k < 3; k++) {
        v[k] = b.invMass * (b.pcm[k] * b.pcm[k]);
        v[3 + k] = b.MoI[k] * (b.omega[k] * b.omega[k]);
        const double rdot = 2.5 * b.rcm[k] + dt * b.invMass * (b.pcm[k] + dt_2 * b.F[k]) - r0[3 * i + k];
        v[6] += rdot * b.pcm[k];
      }
      double qv[4], qdot[4], dot = 0.0;
      vv_virtual_rotation(b, dt, mode, &A.d[3 * b.first], qv);
      for (int k = 0; k < 4; k++) {
        qdot[k] = q0[4 * i + k] + 1.5 * b.q[k] + qv[k];
        dot += qdot[k] * b.q[k];
      }
      for (int k = 0; k < 4; k++) v[7] += (qdot[k] - dot * b.q[k]) * b.pi[k];
      double t4[4], tb[3];
      rb_C(b.q, b.tau, t4);
      rb_Bt(b.q, t4, tb);
      v[8] = b.invMass * (b.F[0] * b.F[0] + b.F[1] * b.F[1] + b.F[2] * b.F[2]) +
             (b.invMoI[0] * tb[0] * tb[0] + b.invMoI[1] * tb[1] * tb[1] + b.invMoI[2] * tb[2] * tb[2]);
    }
    A.b[i] = b;
  }
  if (COMPUTE) grid_reduce<9, VV_THREADS>(v, partials, ticket, result);
}

// ---- host -----------------------------------------------------------------------

static void ensure(double*& p, size_t& cap, size_t need) {
  if (cap >= need) return;
  CK(cudaFree(p));
  CK(cudaMalloc(&p, sizeof(double) * (need ? need : 1)));
  cap = need;
}

static int vv_blocks(int n) { return n > 0 ? (n + VV_THREADS - 1) / VV_THREADS : 1; }
// body kernels run one warp per block: their per-body work is long and serial (FP64
// rotations), so bodies are spread over as many SMs as possible
static const int VV_BODY_THREADS = 32;
static int vv_body_blocks(int n) { return n > 0 ? (n + VV_BODY_THREADS - 1) / VV_BODY_THREADS : 1; }

template <bool FMA>
static void verlet_pre(System& s, double dt, bool compute, int mode) {
  VerletScratch& w = s.verlet;
  const double dt_2 = 0.5 * dt;
  const bool all = s.nbodies == 0;
  const int nf = all ? s.natoms : s.nfree;
  ensure(w.s0, w.s0Cap, (size_t)3 * nf);
  if (nf > 0) {
    const int* list = all ? nullptr : s.dFree;
    if (compute)
      k_vv_pre_free<true, FMA><<<vv_blocks(nf), VV_THREADS, 0, s.stream>>>(s.dR, s.dP, s.F(), s.dInvMass, list, nf, dt,
                                                                      dt_2, w.s0);
    else
      k_vv_pre_free<false, FMA><<<vv_blocks(nf), VV_THREADS, 0, s.stream>>>(s.dR, s.dP, s.F(), s.dInvMass, list, nf, dt,
                                                                       dt_2, w.s0);
    CK(cudaGetLastError());
    s.prof.total++;
  }
  if (s.nbodies > 0) {
    ensure(w.r0, w.r0Cap, (size_t)3 * s.nbodies);
    ensure(w.q0, w.q0Cap, (size_t)4 * s.nbodies);
    if (compute)
      k_vv_pre_body<true><<<vv_body_blocks(s.nbodies), VV_BODY_THREADS, 0, s.stream>>>(body_args(s), s.F(), s.dR, dt,
                                                                                        dt_2, mode, w.r0, w.q0);
    else
      k_vv_pre_body<false><<<vv_body_blocks(s.nbodies), VV_BODY_THREADS, 0, s.stream>>>(body_args(s), s.F(), s.dR, dt,
                                                                                         dt_2, mode, w.r0, w.q0);
    CK(cudaGetLastError());
    s.prof.total++;
  }
}

// out[0..2] 2KE_t, [3..5] 2KE_r, [6] Ks_t, [7] Ks_r, [8] Us (bodies first, then free atoms,
// as each thread of the reference sums them)
template <bool FMA>
static void verlet_post(System& s, double dt, bool compute, int mode, double* out) {
  VerletScratch& w = s.verlet;
  const double dt_2 = 0.5 * dt;
  const bool all = s.nbodies == 0;
  const int nf = all ? s.natoms : s.nfree;
  double vb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vf[5] = {0, 0, 0, 0, 0};
  if (s.nbodies > 0) {
    const int blocks = vv_body_blocks(s.nbodies);
    ensure(w.partB, w.partBCap, (size_t)9 * blocks);
    if (compute)
      k_vv_post_body<true><<<blocks, VV_BODY_THREADS, 0, s.stream>>>(body_args(s), s.F(), dt, dt_2, mode, w.r0, w.q0,
                                                                     w.partB, s.dTicket + 5, s.dResult + 24);
    else
      k_vv_post_body<false><<<blocks, VV_BODY_THREADS, 0, s.stream>>>(body_args(s), s.F(), dt, dt_2, mode, w.r0,
                                                                      w.q0, nullptr, nullptr, nullptr);
    CK(cudaGetLastError());
    s.prof.total++;
  }
  if (nf > 0) {
    const int blocks = std::min(vv_blocks(nf), 1184);
    ensure(w.partF, w.partFCap, (size_t)5 * blocks);
    const int* list = all ? nullptr : s.dFree;
    if (compute)
      k_vv_post_free<true, FMA><<<blocks, VV_THREADS, 0, s.stream>>>(s.dR, s.dP, s.F(), s.dInvMass, list, nf, dt, dt_2,
                                                                w.s0, w.partF, s.dTicket + 6, s.dResult + 34);
    else
      k_vv_post_free<false, FMA><<<blocks, VV_THREADS, 0, s.stream>>>(s.dR, s.dP, s.F(), s.dInvMass, list, nf, dt, dt_2,
                                                                 w.s0, nullptr, nullptr, nullptr);
    CK(cudaGetLastError());
    s.prof.total++;
  }
  if (compute) {
    if (s.nbodies > 0) CK(cudaMemcpyAsync(vb, s.dResult + 24, sizeof(vb), cudaMemcpyDeviceToHost, s.stream));
    if (nf > 0) CK(cudaMemcpyAsync(vf, s.dResult + 34, sizeof(vf), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
  }
  for (int d = 0; d < 3; d++) {
    out[d] = vb[d] + vf[d];
    out[3 + d] = vb[3 + d];
  }
  out[6] = vb[6] + vf[3];
  out[7] = vb[7];
  out[8] = vb[8] + vf[4];
}

void device_verlet_pre(System& s, double dt, bool compute, int mode) {
  if (s.precision == 0) verlet_pre<true>(s, dt, compute, mode);
  else verlet_pre<false>(s, dt, compute, mode);
}

void device_verlet_post(System& s, double dt, bool compute, int mode, double* out) {
  if (s.precision == 0) verlet_post<true>(s, dt, compute, mode, out);
  else verlet_post<false>(s, dt, compute, mode, out);
}

}  // namespace emdee

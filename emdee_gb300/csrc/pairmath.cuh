// pairmath.cuh -- non-bonded model arithmetic shared by the host set-up code
// (double), the FP64 force kernel (double, reference operation order) and the
// FP32 force kernel (float, fast intrinsics).
//
// Every expression keeps the operation order of the reference Fortran so that
// the double instantiation, compiled without FMA contraction, rounds exactly
// like the reference:
//   models ........ src/pair_lj_cut.f90:73-118, src/pair_softcore_cut.f90:86-135,
//                   src/coul_*.f90 (compute/energy/virial)
//   modifiers ..... src/apply_modifier.f90:1-60
//   erfc .......... src/math.f90:35-40, 685-691 (Abramowitz & Stegun 7.1.26)
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define EMD_HD __host__ __device__ __forceinline__
#else
#define EMD_HD inline
#endif

namespace emdee {

// model kinds (one code per reference model file)
enum ModelKind : int {
  MK_PAIR_NONE = 0, MK_LJ_CUT = 1, MK_SOFTCORE_CUT = 2,
  MK_COUL_NONE = 10, MK_COUL_CUT, MK_COUL_SF, MK_COUL_DAMPED, MK_COUL_DAMPED_SMOOTHED,
  MK_COUL_DAMPED_SQUARE_SMOOTHED, MK_COUL_SQUARE_SMOOTHED, MK_COUL_SHIFTED_SQUARE_SMOOTHED,
  MK_COUL_LONG,
  MK_BOND_NONE = 30, MK_BOND_HARMONIC, MK_ANGLE_NONE, MK_ANGLE_HARMONIC, MK_DIHEDRAL_NONE,
  MK_KSPACE_EWALD = 40
};

// modifiers, src/modelClass_nonbonded.f90:27-33
enum Modifier : int { NONE = 0, SHIFTED, SHIFTED_FORCE, SMOOTHED, SHIFTED_SMOOTHED, SQUARE_SMOOTHED,
                      SHIFTED_SQUARE_SMOOTHED };

// Set-up result of one non-bonded model, in the arithmetic type T.
template <typename T>
struct NBParams {
  int kind, modifier;
  T eshift, fshift, Rm, Rm2fac, factor;   // modifier / cut-off data (cNonBondedModel)
  T eps4, eps24, sigsq;                   // lj_cut
  T prefactor, prefactor6, invSigSq, shift;   // softcore_cut
  T alpha, beta, Rm2, invRm;              // coul_*
};

// Per (itype, jtype, layer) entry of the pair table.
template <typename T>
struct PairEntry {
  NBParams<T> model;
  int coulomb;
  T kCoul;
};

// Arithmetic helpers: IEEE for double; fast hardware approximations for float
// on the device.
template <typename T> struct Ops;
template <> struct Ops<double> {
  static EMD_HD double div(double a, double b) { return a / b; }
  static EMD_HD double rcp(double a) { return 1.0 / a; }
  static EMD_HD double ex(double a) { return exp(a); }
  static EMD_HD double sq(double a) { return sqrt(a); }
};
template <> struct Ops<float> {
#ifdef __CUDA_ARCH__
  static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ float rcp(float a) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
  }
  static __device__ __forceinline__ float ex(float a) { return __expf(a); }
  static __device__ __forceinline__ float sq(float a) { return sqrtf(a); }
#else
  static inline float div(float a, float b) { return a / b; }
  static inline float rcp(float a) { return 1.0f / a; }
  static inline float ex(float a) { return expf(a); }
  static inline float sq(float a) { return sqrtf(a); }
#endif
};

// Abramowitz & Stegun 7.1.26: erfc(x) ~ t(a1 + t(a2 + t(a3 + t(a4 + t a5)))) exp(-x^2),
// t = 1/(1 + p x).  Published coefficients.
template <typename T>
EMD_HD T uerfc(T x, T expmx2) {
  const T a1 = T(0.254829592), a2 = T(-0.284496736), a3 = T(1.421413741), a4 = T(-1.453152027),
          a5 = T(1.061405429), p = T(0.327591100);
  T t = Ops<T>::rcp(T(1) + p * x);
  return t * (a1 + t * (a2 + t * (a3 + t * (a4 + t * a5)))) * expmx2;
}

// Smoothing polynomial G(u) = 1 + u^3 (15u - 6u^2 - 10) and u^2 (2u - u^2 - 1).
template <typename T>
EMD_HD void switch_G(T u, T& G, T& dG) {
  T u2 = u * u, u3 = u * u2;
  G = T(1) + u3 * (T(15) * u - T(6) * u2 - T(10));
  dG = u2 * (T(2) * u - u2 - T(1));
}

// model%compute(Eij, Wij, invR, invR2)
template <typename T>
EMD_HD void nb_compute(const NBParams<T>& m, T& E, T& W, T invR, T invR2) {
  typedef Ops<T> O;
  switch (m.kind) {
    case MK_LJ_CUT: {
      T sr2 = m.sigsq * invR2, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
      E = m.eps4 * (sr12 - sr6);
      W = m.eps24 * (sr12 + sr12 - sr6);
      return;
    }
    case MK_SOFTCORE_CUT: {
      T rsig2 = O::div(m.invSigSq, invR2), rsig6 = rsig2 * rsig2 * rsig2;
      T sinv = O::rcp(rsig6 + m.shift), sinvSq = sinv * sinv, sinvCb = sinv * sinvSq;
      E = m.prefactor * (sinvSq - sinv);
      W = m.prefactor6 * rsig6 * (sinvCb + sinvCb - sinvSq);
      return;
    }
    case MK_COUL_CUT:
      E = invR;
      W = E;
      return;
    case MK_COUL_SF: {
      T rFc = O::div(m.fshift, invR);
      E = invR + m.eshift + rFc;
      W = invR - rFc;
      return;
    }
    case MK_COUL_DAMPED:
    case MK_COUL_LONG: {
      T x = O::div(m.alpha, invR), expmx2 = O::ex(-x * x);
      E = uerfc(x, expmx2) * invR;
      W = E + m.beta * expmx2;
      return;
    }
    case MK_COUL_DAMPED_SMOOTHED: {
      T r = O::rcp(invR), x = m.alpha * r, expmx2 = O::ex(-x * x), G, dG;
      E = uerfc(x, expmx2) * invR;
      W = E + m.beta * expmx2;
      if (r > m.Rm) {
        switch_G(m.factor * (r - m.Rm), G, dG);
        T WG = T(-30) * dG * m.factor * r;
        W = W * G + E * WG;
        E = E * G;
      }
      return;
    }
    case MK_COUL_DAMPED_SQUARE_SMOOTHED: {
      T x = O::div(m.alpha, invR), expmx2 = O::ex(-x * x), G, dG;
      E = uerfc(x, expmx2) * invR;
      W = E + m.beta * expmx2;
      if (invR < m.invRm) {
        T r2 = O::rcp(invR2);
        switch_G(m.factor * (r2 - m.Rm2), G, dG);
        T WG = T(-60) * dG * m.factor * r2;
        W = W * G + E * WG;
        E = E * G;
      }
      return;
    }
    case MK_COUL_SQUARE_SMOOTHED:
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED: {
      T G, dG;
      W = invR;
      E = (m.kind == MK_COUL_SQUARE_SMOOTHED) ? W : W + m.eshift;
      if (invR < m.invRm) {
        T r2 = O::rcp(invR2);
        switch_G(m.factor * (r2 - m.Rm2), G, dG);
        T WG = T(-60) * dG * m.factor * r2;
        W = W * G + E * WG;
        E = E * G;
      }
      return;
    }
    default:
      E = T(0);
      W = T(0);
      return;
  }
}

// model%energy(Eij, invR, invR2)
template <typename T>
EMD_HD T nb_energy(const NBParams<T>& m, T invR, T invR2) {
  typedef Ops<T> O;
  switch (m.kind) {
    case MK_LJ_CUT: {
      T sr2 = m.sigsq * invR2, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
      return m.eps4 * (sr12 - sr6);
    }
    case MK_SOFTCORE_CUT: {
      T rsig2 = O::div(m.invSigSq, invR2), rsig6 = rsig2 * rsig2 * rsig2;
      T sinv = O::rcp(rsig6 + m.shift);
      return m.prefactor * (sinv * sinv - sinv);
    }
    case MK_COUL_CUT: return invR;
    case MK_COUL_SF: return invR + m.eshift + O::div(m.fshift, invR);
    case MK_COUL_DAMPED:
    case MK_COUL_LONG: {
      T x = O::div(m.alpha, invR);
      return uerfc(x, O::ex(-x * x)) * invR;
    }
    case MK_COUL_DAMPED_SMOOTHED: {
      T r = O::rcp(invR), x = m.alpha * r, G, dG;
      T E = uerfc(x, O::ex(-x * x)) * invR;
      if (r > m.Rm) {
        switch_G(m.factor * (r - m.Rm), G, dG);
        E = E * G;
      }
      return E;
    }
    case MK_COUL_DAMPED_SQUARE_SMOOTHED: {
      T x = O::div(m.alpha, invR), G, dG;
      T E = uerfc(x, O::ex(-x * x)) * invR;
      if (invR < m.invRm) {
        switch_G(m.factor * (O::rcp(invR2) - m.Rm2), G, dG);
        E = E * G;
      }
      return E;
    }
    case MK_COUL_SQUARE_SMOOTHED:
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED: {
      T G, dG;
      T E = (m.kind == MK_COUL_SQUARE_SMOOTHED) ? invR : invR + m.eshift;
      if (invR < m.invRm) {
        switch_G(m.factor * (O::rcp(invR2) - m.Rm2), G, dG);
        E = E * G;
      }
      return E;
    }
    default: return T(0);
  }
}

// model%virial(Wij, invR, invR2)
template <typename T>
EMD_HD T nb_virial(const NBParams<T>& m, T invR, T invR2) {
  typedef Ops<T> O;
  switch (m.kind) {
    case MK_COUL_SQUARE_SMOOTHED: {   // src/coul_square_smoothed.f90:124-143
      T W = invR, G, dG;
      if (invR < m.invRm) {
        T r2 = O::rcp(invR2);
        switch_G(m.factor * (r2 - m.Rm2), G, dG);
        T WG = T(-60) * dG * m.factor * r2;
        W = W * (G + WG);
      }
      return W;
    }
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED: {   // src/coul_shifted_square_smoothed.f90:127-146
      T W = invR, G, dG;
      if (invR < m.invRm) {
        T r2 = O::rcp(invR2);
        switch_G(m.factor * (r2 - m.Rm2), G, dG);
        T WG = T(-60) * dG * m.factor * r2;
        W = W * G + (W + m.eshift) * WG;
      }
      return W;
    }
    case MK_COUL_NONE: return T(0);
    default: {
      T E, W;
      nb_compute(m, E, W, invR, invR2);
      return W;
    }
  }
}

// apply_modifier.f90 with energies
template <typename T>
EMD_HD void modifier_compute(const NBParams<T>& m, T& E, T& W, T invR, T invR2) {
  typedef Ops<T> O;
  T r2fac, G, dG;
  switch (m.modifier) {
    case SHIFTED: E += m.eshift; break;
    case SHIFTED_FORCE: {
      T rFc = O::div(m.fshift, invR);
      W -= rFc;
      E += m.eshift + rFc;
      break;
    }
    case SMOOTHED:
    case SHIFTED_SMOOTHED:
      E += m.eshift;
      r2fac = O::div(m.factor, invR);
      if (r2fac > m.Rm2fac) {
        switch_G(r2fac - m.Rm2fac, G, dG);
        T WG = T(-30) * dG * r2fac;
        W = W * G + E * WG;
        E = E * G;
      }
      break;
    case SQUARE_SMOOTHED:
    case SHIFTED_SQUARE_SMOOTHED:
      E += m.eshift;
      r2fac = O::div(m.factor, invR2);
      if (r2fac > m.Rm2fac) {
        switch_G(r2fac - m.Rm2fac, G, dG);
        T WG = T(-60) * dG * r2fac;
        W = W * G + E * WG;
        E = E * G;
      }
      break;
    default: break;
  }
}

// apply_modifier.f90 without energies
template <typename T>
EMD_HD void modifier_virial(const NBParams<T>& m, T& W, T invR, T invR2) {
  typedef Ops<T> O;
  T r2fac, G, dG, E;
  switch (m.modifier) {
    case SHIFTED_FORCE: W -= O::div(m.fshift, invR); break;
    case SMOOTHED:
    case SHIFTED_SMOOTHED:
      r2fac = O::div(m.factor, invR);
      if (r2fac > m.Rm2fac) {
        E = nb_energy(m, invR, invR2) + m.eshift;
        switch_G(r2fac - m.Rm2fac, G, dG);
        T WG = T(-30) * dG * r2fac;
        W = W * G + E * WG;
      }
      break;
    case SQUARE_SMOOTHED:
    case SHIFTED_SQUARE_SMOOTHED:
      r2fac = O::div(m.factor, invR2);
      if (r2fac > m.Rm2fac) {
        E = nb_energy(m, invR, invR2) + m.eshift;
        switch_G(r2fac - m.Rm2fac, G, dG);
        T WG = T(-60) * dG * r2fac;
        W = W * G + E * WG;
      }
      break;
    default: break;
  }
}

// Full evaluation of one pair (pair model + Coulomb model), as in
// src/compute.f90:44-87.  Returns Wsum; accumulates the energy and virial terms.
template <typename T, bool COMPUTE>
EMD_HD T pair_eval(const PairEntry<T>& pe, const NBParams<T>& coul, bool ijcharged, T Qi, T Qj, T invR,
                   T invR2, T& Epair, T& Ecoul, T& Wpair, T& Wcoul) {
  T Eij = T(0), Wij;
  if (COMPUTE) {
    nb_compute(pe.model, Eij, Wij, invR, invR2);
    modifier_compute(pe.model, Eij, Wij, invR, invR2);
    Epair += Eij;
  } else {
    Wij = nb_virial(pe.model, invR, invR2);
    modifier_virial(pe.model, Wij, invR, invR2);
  }
  Wpair += Wij;
  T Wsum = Wij;
  if (ijcharged && pe.coulomb) {
    if (COMPUTE) {
      nb_compute(coul, Eij, Wij, invR, invR2);
      modifier_compute(coul, Eij, Wij, invR, invR2);
    } else {
      Wij = nb_virial(coul, invR, invR2);
      modifier_virial(coul, Wij, invR, invR2);
    }
    T QiQj = pe.kCoul * Qi * Qj;
    if (COMPUTE) Ecoul += QiQj * Eij;
    Wij = QiQj * Wij;
    Wcoul += Wij;
    Wsum += Wij;
  }
  return Wsum;
}

}  // namespace emdee

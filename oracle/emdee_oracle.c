/*
 * emdee_oracle.c -- CPU restatement of the EmDee hot path, in plain C, FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline ("port") for the GB300 library.  Only the tests, the smoke check
 * and the CPU-baseline leg of the benchmark may load it; the product library
 * (emdee_gb300/) never links, calls or falls back to it.
 *
 * It exports the same C ABI as include/emdee.h (built into its own
 * liboracle_emdee.so) and restates, routine by routine, the reference
 * Fortran (paths relative to the atoms-ufrj/EmDee tree):
 *   - API state machine ............ src/EmDeeCode.f90
 *   - engine, pair driver, motion .. src/EmDeeData.f90
 *   - pair-loop body ................ src/compute.f90, src/apply_modifier.f90
 *   - neighbor lists ................ src/neighbor_lists.f90
 *   - modifiers / mixing / cutoffs .. src/modelClass_nonbonded.f90,
 *                                     src/modelClass_pair.f90, src/modelClass_coul.f90
 *   - models ........................ src/pair_*.f90, src/coul_*.f90
 *   - math and RNG .................. src/math.f90
 * The OpenMP thread decomposition of the reference (contiguous cell ranges per
 * thread, per-thread half neighbor lists, per-thread force arrays summed in
 * thread order) is kept, so the same thread count gives the same summation
 * order.  Compile with -ffp-contract=off so every operation rounds as written.
 *
 * Parity pin: the oracle reproduces the reference's four golden [U, W, U+K]
 * triples (test/test_pair_lj_*.f90) within their 1e-8 tolerance; see
 * tests/test_oracle_golden.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "../include/emdee.h"
#include "rigid_oracle.h"

#define EXTRA 2000      /* src/EmDeeData.f90:31 */
#define NDIV 2          /* src/EmDeeData.f90:33 */
#define NBCELLS 62      /* src/EmDeeData.f90:34 */

/* ======================================================================== */
/* errors (src/global.f90:51-64)                                              */
/* ======================================================================== */

static void error(const char* task, const char* msg) {
  fprintf(stderr, "Error in %s: %s.\n", task, msg);
  exit(1);
}

static void warning(const char* msg) { fprintf(stderr, "WARNING: %s.\n", msg); }

static void* xmalloc(size_t n) {
  void* p = malloc(n ? n : 1);
  if (!p) error("memory allocation", "out of memory");
  return p;
}
static void* xcalloc(size_t n, size_t s) {
  void* p = calloc(n ? n : 1, s ? s : 1);
  if (!p) error("memory allocation", "out of memory");
  return p;
}

/* option strings: at most 256 characters, NUL terminated (src/global.f90:120-128) */
static void option_string(const char* c, char* out) {
  int i;
  for (i = 0; i < 256 && c[i]; i++) out[i] = c[i];
  out[i] = 0;
}

/* ======================================================================== */
/* math (src/math.f90)                                                        */
/* ======================================================================== */

/* A&S 7.1.26 rational approximation of erfc(x)*exp(x^2) times exp(-x^2);
 * src/math.f90:35-40 (coefficients, published in Abramowitz & Stegun) and
 * src/math.f90:685-691 (evaluation order). */
static const double AS_A1 = 0.254829592, AS_A2 = -0.284496736, AS_A3 = 1.421413741,
                    AS_A4 = -1.453152027, AS_A5 = 1.061405429, AS_P = 0.327591100;

static double uerfc(double x, double expmx2) {
  double t = 1.0 / (1.0 + AS_P * x);
  return t * (AS_A1 + t * (AS_A2 + t * (AS_A3 + t * (AS_A4 + t * AS_A5)))) * expmx2;
}

/* phi(x) = (1 - exp(-x))/x with a series below 1e-4; src/math.f90:230-237 */
static double phi(double x) {
  if (fabs(x) > 1e-4) return (1.0 - exp(-x)) / x;
  return 1.0 + 0.5 * x * ((1.0 / 3.0) * x * (1.0 - 0.25 * x) - 1.0);
}

/* Fortran ANINT: round half away from zero */
static inline double anint(double x) { return round(x); }

/* ======================================================================== */
/* KISS generator and Marsaglia-Tsang ziggurat normals (src/math.f90:69-177) */
/* ======================================================================== */

typedef struct {
  int seeding_required;
  int32_t kn[128];
  double wn[128], fn[128];
  uint32_t x, y, z, w;
} okiss;

static uint32_t kiss_m(uint32_t k, int n) { return k ^ (n >= 0 ? (k << n) : (k >> (-n))); }

/* src/math.f90:150-162 */
static void kiss_init(okiss* a, int32_t seed) {
  a->x = kiss_m(kiss_m(kiss_m((uint32_t)seed, 13), -17), 5);
  a->y = kiss_m(kiss_m(kiss_m(a->x, 13), -17), 5);
  a->z = kiss_m(kiss_m(kiss_m(a->y, 13), -17), 5);
  a->w = kiss_m(kiss_m(kiss_m(a->z, 13), -17), 5);
}

/* src/math.f90:166-177, with 32-bit wraparound and logical shifts */
static int32_t kiss_i32(okiss* a) {
  a->x = 69069u * a->x + 1327217885u;
  a->y ^= a->y << 13;
  a->y ^= a->y >> 17;
  a->y ^= a->y << 5;
  a->z = 18000u * (a->z & 65535u) + (a->z >> 16);
  a->w = 30903u * (a->w & 65535u) + (a->w >> 16);
  return (int32_t)(a->x + a->y + (a->z << 16) + a->w);
}

/* src/math.f90:80-105 */
static void rng_setup(okiss* a, int32_t seed) {
  const double m1 = 2147483648.0;
  double q, dn, tn, vn;
  kiss_init(a, seed);
  a->seeding_required = 0;
  dn = 3.442619855899;
  tn = 3.442619855899;
  vn = 0.00991256303526217;
  q = vn * exp(0.5 * dn * dn);
  a->kn[0] = (int32_t)((dn / q) * m1);
  a->kn[1] = 0;
  a->wn[0] = q / m1;
  a->wn[127] = dn / m1;
  a->fn[0] = 1.0;
  a->fn[127] = exp(-0.5 * dn * dn);
  for (int i = 126; i >= 1; i--) {
    dn = sqrt(-2.0 * log(vn / dn + exp(-0.5 * dn * dn)));
    a->kn[i + 1] = (int32_t)((dn / tn) * m1);
    tn = dn;
    a->fn[i] = exp(-0.5 * dn * dn);
    a->wn[i] = dn / m1;
  }
}

static inline int32_t iabs32(int32_t v) { return v == INT32_MIN ? INT32_MIN : (v < 0 ? -v : v); }

/* src/math.f90:109-146 */
static double rng_normal(okiss* a) {
  const double r = 3.442620, s = 0.2328306e-9;
  int32_t hz = kiss_i32(a);
  int32_t iz = hz & 127;
  double x, y;
  if (iabs32(hz) < a->kn[iz]) return (double)hz * a->wn[iz];
  for (;;) {
    if (iz == 0) {
      for (;;) {
        x = -0.2904764 * log(s * (double)kiss_i32(a) + 0.5);
        y = -log(s * (double)kiss_i32(a) + 0.5);
        if (y + y >= x * x) break;
      }
      return hz <= 0 ? -(r + x) : r + x;
    }
    x = (double)hz * a->wn[iz];
    if (a->fn[iz] + (s * (double)kiss_i32(a) + 0.5) * (a->fn[iz - 1] - a->fn[iz]) < exp(-0.5 * x * x))
      return x;
    hz = kiss_i32(a);
    iz = hz & 127;
    if (iabs32(hz) < a->kn[iz]) return (double)hz * a->wn[iz];
  }
}

/* ======================================================================== */
/* models (src/modelClass*.f90, src/pair_*.f90, src/coul_*.f90)              */
/* ======================================================================== */

enum { MC_PAIR = 1, MC_COUL, MC_BOND, MC_ANGLE, MC_DIHEDRAL, MC_KSPACE };
enum {
  MK_PAIR_NONE = 0, MK_LJ_CUT, MK_SOFTCORE_CUT,
  MK_COUL_NONE = 10, MK_COUL_CUT, MK_COUL_SF, MK_COUL_DAMPED, MK_COUL_DAMPED_SMOOTHED,
  MK_COUL_DAMPED_SQUARE_SMOOTHED, MK_COUL_SQUARE_SMOOTHED, MK_COUL_SHIFTED_SQUARE_SMOOTHED,
  MK_COUL_LONG,
  MK_BOND_NONE = 30, MK_BOND_HARMONIC, MK_ANGLE_NONE, MK_ANGLE_HARMONIC, MK_DIHEDRAL_NONE,
  MK_KSPACE_EWALD = 40
};
/* src/modelClass_nonbonded.f90:27-33 */
enum { NONE = 0, SHIFTED, SHIFTED_FORCE, SMOOTHED, SHIFTED_SMOOTHED, SQUARE_SMOOTHED,
       SHIFTED_SQUARE_SMOOTHED };

typedef struct {
  int cls, kind;
  char name[24];
  /* cNonBondedModel (src/modelClass_nonbonded.f90:36-50) */
  int modifier;
  double eshift, fshift, skin, Rm, RmSq, factor, Rm2fac;
  /* pair_lj_cut (src/pair_lj_cut.f90:31-36) */
  double epsilon, sigma, eps4, eps24, sigsq;
  /* pair_softcore_cut (src/pair_softcore_cut.f90:33-39) */
  double lambda, prefactor, prefactor6, invSigSq, shift;
  /* cCoulModel (src/modelClass_coul.f90:28-37) and the coul_* fields */
  int shifted, shifted_force, requires_kspace;
  double alpha, beta, damp, skinWidth, Rm2, invRm;
  /* k-space and bonded parameters */
  double accuracy, k, x0;
} omodel;

static omodel* deliver(const omodel* m) {   /* src/modelClass.f90:51-60 */
  omodel* c = (omodel*)xmalloc(sizeof(omodel));
  *c = *m;
  return c;
}

static omodel new_model(int cls, int kind, const char* name) {
  omodel m;
  memset(&m, 0, sizeof m);
  m.cls = cls;
  m.kind = kind;
  snprintf(m.name, sizeof m.name, "%s", name);
  return m;
}

/* src/pair_lj_cut.f90:52-69 */
static omodel lj_setup(double eps, double sig) {
  omodel m = new_model(MC_PAIR, MK_LJ_CUT, "lj_cut");
  m.epsilon = eps;
  m.sigma = sig;
  m.eps4 = 4.0 * eps;
  m.eps24 = 24.0 * eps;
  m.sigsq = sig * sig;
  return m;
}

/* src/pair_softcore_cut.f90:58-82 (alpha = 1/2, n = p = 1) */
static omodel softcore_setup(double eps, double sig, double lambda) {
  omodel m = new_model(MC_PAIR, MK_SOFTCORE_CUT, "softcore_cut");
  m.epsilon = eps;
  m.sigma = sig;
  m.lambda = lambda;
  if (lambda < 0.0 || lambda > 1.0) error("pair_softcore_cut setup", "out-of-range parameter lambda");
  m.prefactor = 4.0 * eps * pow(lambda, 1.0);
  m.prefactor6 = 6.0 * m.prefactor;
  m.invSigSq = 1.0 / (sig * sig);
  m.shift = 0.5 * pow(1.0 - lambda, 1.0);
  return m;
}

void* EmDee_pair_none(void) { omodel m = new_model(MC_PAIR, MK_PAIR_NONE, "none"); return deliver(&m); }
void* EmDee_coul_none(void) { omodel m = new_model(MC_COUL, MK_COUL_NONE, "none"); return deliver(&m); }
void* EmDee_bond_none(void) { omodel m = new_model(MC_BOND, MK_BOND_NONE, "none"); return deliver(&m); }
void* EmDee_angle_none(void) { omodel m = new_model(MC_ANGLE, MK_ANGLE_NONE, "none"); return deliver(&m); }
void* EmDee_dihedral_none(void) { omodel m = new_model(MC_DIHEDRAL, MK_DIHEDRAL_NONE, "none"); return deliver(&m); }
void* EmDee_pair_lj_cut(double epsilon, double sigma) { omodel m = lj_setup(epsilon, sigma); return deliver(&m); }
void* EmDee_pair_softcore_cut(double epsilon, double sigma, double lambda) {
  omodel m = softcore_setup(epsilon, sigma, lambda);
  return deliver(&m);
}
void* EmDee_coul_cut(void) { omodel m = new_model(MC_COUL, MK_COUL_CUT, "cut"); return deliver(&m); }
void* EmDee_coul_sf(void) {   /* src/coul_sf.f90:37-50 */
  omodel m = new_model(MC_COUL, MK_COUL_SF, "sf");
  m.shifted_force = 1;
  return deliver(&m);
}
void* EmDee_coul_damped(double damp) {   /* src/coul_damped.f90:41-57 */
  omodel m = new_model(MC_COUL, MK_COUL_DAMPED, "damped");
  m.damp = damp;
  m.alpha = damp;
  m.beta = 2.0 * m.alpha / sqrt(3.14159265358979324);
  return deliver(&m);
}
void* EmDee_coul_damped_smoothed(double damp, double skinWidth) {   /* src/coul_damped_smoothed.f90:46-64 */
  omodel m = new_model(MC_COUL, MK_COUL_DAMPED_SMOOTHED, "damped_openmm_smoothed");
  m.damp = damp;
  m.skinWidth = skinWidth;
  m.alpha = damp;
  m.beta = 2.0 * m.alpha / sqrt(3.14159265358979324);
  return deliver(&m);
}
void* EmDee_coul_damped_square_smoothed(double damp, double skinWidth) {
  omodel m = new_model(MC_COUL, MK_COUL_DAMPED_SQUARE_SMOOTHED, "damped_smoothed");
  m.damp = damp;
  m.skinWidth = skinWidth;
  m.alpha = damp;
  m.beta = 2.0 * m.alpha / sqrt(3.14159265358979324);
  return deliver(&m);
}
void* EmDee_coul_square_smoothed(double skinWidth) {
  omodel m = new_model(MC_COUL, MK_COUL_SQUARE_SMOOTHED, "smoothed");
  m.skinWidth = skinWidth;
  return deliver(&m);
}
void* EmDee_coul_shifted_square_smoothed(double skinWidth) {
  omodel m = new_model(MC_COUL, MK_COUL_SHIFTED_SQUARE_SMOOTHED, "shifted_smoothed");
  m.skinWidth = skinWidth;
  m.shifted = 1;
  return deliver(&m);
}
void* EmDee_coul_long(void) {   /* src/coul_long.f90:37-51 */
  omodel m = new_model(MC_COUL, MK_COUL_LONG, "long");
  m.requires_kspace = 1;
  return deliver(&m);
}
void* EmDee_kspace_ewald(double accuracy) {
  omodel m = new_model(MC_KSPACE, MK_KSPACE_EWALD, "ewald");
  m.accuracy = accuracy;
  return deliver(&m);
}
void* EmDee_bond_harmonic(double k, double r0) {
  omodel m = new_model(MC_BOND, MK_BOND_HARMONIC, "harmonic");
  m.k = k;
  m.x0 = r0;
  return deliver(&m);
}
void* EmDee_angle_harmonic(double k, double theta0) {
  omodel m = new_model(MC_ANGLE, MK_ANGLE_HARMONIC, "harmonic");
  m.k = k;
  m.x0 = theta0;
  return deliver(&m);
}

/* modifiers: a new container with the modifier (and skin) set;
 * src/modelClass_nonbonded.f90:83-241 */
static void* modified(void* model, int modifier, double skin, int set_skin, const char* task) {
  if (!model) error(task, "a valid pair model must be provided");
  omodel m = *(omodel*)model;
  if (m.cls != MC_PAIR && m.cls != MC_COUL) error(task, "a valid pair model must be provided");
  m.modifier = modifier;
  if (set_skin) m.skin = skin;
  return deliver(&m);
}
void* EmDee_shifted(void* model) { return modified(model, SHIFTED, 0, 0, "shifted potential assignment"); }
void* EmDee_shifted_force(void* model) {
  return modified(model, SHIFTED_FORCE, 0, 0, "shifted-force potential assignment");
}
void* EmDee_smoothed(void* model, double skin) {
  return modified(model, SMOOTHED, skin, 1, "smoothed potential assignment");
}
void* EmDee_shifted_smoothed(void* model, double skin) {
  return modified(model, SHIFTED_SMOOTHED, skin, 1, "shifted-smoothed potential assignment");
}
void* EmDee_square_smoothed(void* model, double skin) {
  return modified(model, SQUARE_SMOOTHED, skin, 1, "square-smoothed potential assignment");
}
void* EmDee_shifted_square_smoothed(void* model, double skin) {
  return modified(model, SHIFTED_SQUARE_SMOOTHED, skin, 1, "shifted-square-smoothed potential assignment");
}

/* smoothing switch shared by several models: G and the W factor before the
 * r or r^2 scaling (src/apply_modifier.f90:24-33 and the coul_*_smoothed files) */
static inline void switch_G(double u, double* G, double* dG) {
  double u2 = u * u, u3 = u * u2;
  *G = 1.0 + u3 * (15.0 * u - 6.0 * u2 - 10.0);
  *dG = u2 * (2.0 * u - u2 - 1.0);
}

/* model%compute(Eij, Wij, invR, invR2) for every non-bonded model */
static void model_compute(const omodel* m, double* E, double* W, double invR, double invR2) {
  switch (m->kind) {
    case MK_LJ_CUT: {   /* src/pair_lj_cut.f90:73-86 */
      double sr2 = m->sigsq * invR2, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
      *E = m->eps4 * (sr12 - sr6);
      *W = m->eps24 * (sr12 + sr12 - sr6);
      return;
    }
    case MK_SOFTCORE_CUT: {   /* src/pair_softcore_cut.f90:86-101 */
      double rsig2 = m->invSigSq / invR2, rsig6 = rsig2 * rsig2 * rsig2;
      double sinv = 1.0 / (rsig6 + m->shift), sinvSq = sinv * sinv, sinvCb = sinv * sinvSq;
      *E = m->prefactor * (sinvSq - sinv);
      *W = m->prefactor6 * rsig6 * (sinvCb + sinvCb - sinvSq);
      return;
    }
    case MK_COUL_CUT:   /* src/coul_cut.f90:62-72 */
      *E = invR;
      *W = *E;
      return;
    case MK_COUL_SF: {   /* src/coul_sf.f90:54-66 */
      double rFc = m->fshift / invR;
      *E = invR + m->eshift + rFc;
      *W = invR - rFc;
      return;
    }
    case MK_COUL_DAMPED:
    case MK_COUL_LONG: {   /* src/coul_damped.f90:61-72, src/coul_long.f90:69-80 */
      double x = m->alpha / invR, expmx2 = exp(-x * x);
      *E = uerfc(x, expmx2) * invR;
      *W = *E + m->beta * expmx2;
      return;
    }
    case MK_COUL_DAMPED_SMOOTHED: {   /* src/coul_damped_smoothed.f90:84-105 */
      double r = 1.0 / invR, x = m->alpha * r, expmx2 = exp(-x * x), G, dG;
      *E = uerfc(x, expmx2) * invR;
      *W = *E + m->beta * expmx2;
      if (r > m->Rm) {
        switch_G(m->factor * (r - m->Rm), &G, &dG);
        double WG = -30.0 * dG * m->factor * r;
        *W = *W * G + *E * WG;
        *E = *E * G;
      }
      return;
    }
    case MK_COUL_DAMPED_SQUARE_SMOOTHED: {   /* src/coul_damped_square_smoothed.f90:82-103 */
      double x = m->alpha / invR, expmx2 = exp(-x * x), G, dG;
      *E = uerfc(x, expmx2) * invR;
      *W = *E + m->beta * expmx2;
      if (invR < m->invRm) {
        double r2 = 1.0 / invR2;
        switch_G(m->factor * (r2 - m->Rm2), &G, &dG);
        double WG = -60.0 * dG * m->factor * r2;
        *W = *W * G + *E * WG;
        *E = *E * G;
      }
      return;
    }
    case MK_COUL_SQUARE_SMOOTHED:
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED: {   /* src/coul_square_smoothed.f90:76-95, src/coul_shifted_square_smoothed.f90:79-98 */
      double G, dG;
      *W = invR;
      *E = (m->kind == MK_COUL_SQUARE_SMOOTHED) ? *W : *W + m->eshift;
      if (invR < m->invRm) {
        double r2 = 1.0 / invR2;
        switch_G(m->factor * (r2 - m->Rm2), &G, &dG);
        double WG = -60.0 * dG * m->factor * r2;
        *W = *W * G + *E * WG;
        *E = *E * G;
      }
      return;
    }
    default:   /* pair_none, coul_none (src/modelClass_pair.f90:173-179) */
      *E = 0.0;
      *W = 0.0;
      return;
  }
}

/* model%energy(Eij, invR, invR2) */
static double model_energy(const omodel* m, double invR, double invR2) {
  switch (m->kind) {
    case MK_LJ_CUT: {
      double sr2 = m->sigsq * invR2, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
      return m->eps4 * (sr12 - sr6);
    }
    case MK_SOFTCORE_CUT: {
      double rsig2 = m->invSigSq / invR2, rsig6 = rsig2 * rsig2 * rsig2;
      double sinv = 1.0 / (rsig6 + m->shift);
      return m->prefactor * (sinv * sinv - sinv);
    }
    case MK_COUL_CUT: return invR;
    case MK_COUL_SF: return invR + m->eshift + m->fshift / invR;
    case MK_COUL_DAMPED:
    case MK_COUL_LONG: {
      double x = m->alpha / invR;
      return uerfc(x, exp(-x * x)) * invR;
    }
    case MK_COUL_DAMPED_SMOOTHED: {
      double r = 1.0 / invR, x = m->alpha * r, G, dG;
      double E = uerfc(x, exp(-x * x)) * invR;
      if (r > m->Rm) {
        switch_G(m->factor * (r - m->Rm), &G, &dG);
        E = E * G;
      }
      return E;
    }
    case MK_COUL_DAMPED_SQUARE_SMOOTHED: {
      double x = m->alpha / invR, G, dG;
      double E = uerfc(x, exp(-x * x)) * invR;
      if (invR < m->invRm) {
        switch_G(m->factor * (1.0 / invR2 - m->Rm2), &G, &dG);
        E = E * G;
      }
      return E;
    }
    case MK_COUL_SQUARE_SMOOTHED:
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED: {
      double G, dG;
      double E = (m->kind == MK_COUL_SQUARE_SMOOTHED) ? invR : invR + m->eshift;
      if (invR < m->invRm) {
        switch_G(m->factor * (1.0 / invR2 - m->Rm2), &G, &dG);
        E = E * G;
      }
      return E;
    }
    default: return 0.0;
  }
}

/* model%virial(Wij, invR, invR2) */
static double model_virial(const omodel* m, double invR, double invR2) {
  switch (m->kind) {
    case MK_COUL_SQUARE_SMOOTHED: {   /* src/coul_square_smoothed.f90:124-143: W*(G+WG) */
      double W = invR, G, dG;
      if (invR < m->invRm) {
        double r2 = 1.0 / invR2;
        switch_G(m->factor * (r2 - m->Rm2), &G, &dG);
        double WG = -60.0 * dG * m->factor * r2;
        W = W * (G + WG);
      }
      return W;
    }
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED: {   /* src/coul_shifted_square_smoothed.f90:127-146 */
      double W = invR, G, dG;
      if (invR < m->invRm) {
        double r2 = 1.0 / invR2;
        switch_G(m->factor * (r2 - m->Rm2), &G, &dG);
        double WG = -60.0 * dG * m->factor * r2;
        W = W * G + (W + m->eshift) * WG;
      }
      return W;
    }
    case MK_COUL_NONE:
      /* coul_none_virial leaves Wij unset (src/modelClass_coul.f90:175-179);
       * it is never reached on the pair path because coul_none pairs are skipped. */
      return 0.0;
    default: {
      double E, W;
      model_compute(m, &E, &W, invR, invR2);
      return W;
    }
  }
}

/* apply_modifier.f90 with "compute" defined (energies and virials) */
static void apply_modifier_compute(const omodel* m, double* E, double* W, double invR, double invR2) {
  double r2fac, G, dG;
  switch (m->modifier) {
    case SHIFTED: *E += m->eshift; break;
    case SHIFTED_FORCE: {
      double rFc = m->fshift / invR;
      *W -= rFc;
      *E += m->eshift + rFc;
      break;
    }
    case SMOOTHED:
    case SHIFTED_SMOOTHED:
      *E += m->eshift;
      r2fac = m->factor / invR;
      if (r2fac > m->Rm2fac) {
        switch_G(r2fac - m->Rm2fac, &G, &dG);
        double WG = -30.0 * dG * r2fac;
        *W = *W * G + *E * WG;
        *E = *E * G;
      }
      break;
    case SQUARE_SMOOTHED:
    case SHIFTED_SQUARE_SMOOTHED:
      *E += m->eshift;
      r2fac = m->factor / invR2;
      if (r2fac > m->Rm2fac) {
        switch_G(r2fac - m->Rm2fac, &G, &dG);
        double WG = -60.0 * dG * r2fac;
        *W = *W * G + *E * WG;
        *E = *E * G;
      }
      break;
    default: break;
  }
}

/* apply_modifier.f90 without "compute" (virials only; energies evaluated in
 * the switching region only) */
static void apply_modifier_virial(const omodel* m, double* W, double invR, double invR2) {
  double r2fac, G, dG, E;
  switch (m->modifier) {
    case SHIFTED_FORCE: *W -= m->fshift / invR; break;
    case SMOOTHED:
    case SHIFTED_SMOOTHED:
      r2fac = m->factor / invR;
      if (r2fac > m->Rm2fac) {
        E = model_energy(m, invR, invR2) + m->eshift;
        switch_G(r2fac - m->Rm2fac, &G, &dG);
        double WG = -30.0 * dG * r2fac;
        *W = *W * G + E * WG;
      }
      break;
    case SQUARE_SMOOTHED:
    case SHIFTED_SQUARE_SMOOTHED:
      r2fac = m->factor / invR2;
      if (r2fac > m->Rm2fac) {
        E = model_energy(m, invR, invR2) + m->eshift;
        switch_G(r2fac - m->Rm2fac, &G, &dG);
        double WG = -60.0 * dG * r2fac;
        *W = *W * G + E * WG;
      }
      break;
    default: break;
  }
}

/* src/modelClass_nonbonded.f90:245-296 */
static void modifier_setup(omodel* m, double cutoff) {
  double Ec = 0, Wc = 0, Es, Ws;
  int shifting;
  m->fshift = 0.0;
  m->eshift = 0.0;
  m->Rm = cutoff - m->skin;
  m->RmSq = m->Rm * m->Rm;
  shifting = m->modifier == SHIFTED || m->modifier == SHIFTED_FORCE || m->modifier == SHIFTED_SMOOTHED ||
             m->modifier == SHIFTED_SQUARE_SMOOTHED;
  if (shifting) model_compute(m, &Ec, &Wc, 1.0 / cutoff, 1.0 / (cutoff * cutoff));
  switch (m->modifier) {
    case SHIFTED: m->eshift = -Ec; break;
    case SHIFTED_FORCE:
      m->eshift = -(Ec + Wc);
      m->fshift = Wc / cutoff;
      break;
    case SMOOTHED:
    case SHIFTED_SMOOTHED:
      if (shifting) {
        model_compute(m, &Es, &Ws, 1.0 / m->Rm, 1.0 / m->RmSq);
        m->eshift = -0.5 * (Es + Ec);
      }
      m->factor = 1.0 / (cutoff - m->Rm);
      m->Rm2fac = m->factor * m->Rm;
      break;
    case SQUARE_SMOOTHED:
    case SHIFTED_SQUARE_SMOOTHED:
      if (shifting) {
        model_compute(m, &Es, &Ws, 1.0 / m->Rm, 1.0 / m->RmSq);
        m->eshift = -0.5 * (Es + Ec);
      }
      m->factor = 1.0 / (cutoff * cutoff - m->RmSq);
      m->Rm2fac = m->factor * m->RmSq;
      break;
    default: break;
  }
}

/* apply_cutoff of the smoothed Coulomb models (src/coul_*smoothed.f90) */
static void apply_cutoff(omodel* m, double Rc) {
  switch (m->kind) {
    case MK_COUL_DAMPED_SMOOTHED:   /* src/coul_damped_smoothed.f90:70-80 */
      m->Rm = Rc - m->skinWidth;
      m->Rm2 = m->Rm * m->Rm;
      m->invRm = 1.0 / m->Rm;
      m->factor = 1.0 / (Rc - m->Rm);
      break;
    case MK_COUL_DAMPED_SQUARE_SMOOTHED:
    case MK_COUL_SQUARE_SMOOTHED:
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED:
      m->Rm2 = (Rc - m->skinWidth) * (Rc - m->skinWidth);
      m->invRm = 1.0 / (Rc - m->skinWidth);
      m->factor = 1.0 / (Rc * Rc - m->Rm2);
      break;
    default: break;
  }
}

/* src/modelClass_coul.f90:62-93 */
static void cutoff_setup(omodel* m, double cutoff) {
  m->fshift = 0.0;
  m->eshift = 0.0;
  if (m->shifted || m->shifted_force) {
    double invR = 1.0 / cutoff, E, W;
    model_compute(m, &E, &W, invR, invR * invR);
    if (m->shifted_force) {
      m->fshift = W / cutoff;
      m->eshift = -(E + W);
    } else {
      m->fshift = 0.0;
      m->eshift = -E;
    }
  }
  apply_cutoff(m, cutoff);
}

/* src/modelClass_coul.f90:101-106 and src/coul_long.f90:55-64 */
static void coul_kspace_setup(omodel* m, double alpha) {
  if (m->kind == MK_COUL_LONG) {
    m->alpha = alpha;
    m->beta = 2.0 * alpha / sqrt(3.14159265358979324);
  } else if (m->requires_kspace) {
    m->alpha = alpha;
  }
}

typedef struct {
  omodel model;
  int coulomb;
  double kCoul;
} opair;

/* model%mix(other) for pair models; returns 0 when no rule exists
 * (src/pair_lj_cut.f90:122-138, src/pair_softcore_cut.f90:139-163,
 *  src/modelClass_pair.f90:198-208) */
static int model_mix(const omodel* self, const omodel* other, omodel* out) {
  switch (self->kind) {
    case MK_PAIR_NONE: *out = new_model(MC_PAIR, MK_PAIR_NONE, "none"); return 1;
    case MK_LJ_CUT:
      if (other->kind == MK_LJ_CUT) {
        *out = lj_setup(sqrt(self->epsilon * other->epsilon), 0.5 * (self->sigma + other->sigma));
        return 1;
      }
      return 0;
    case MK_SOFTCORE_CUT:
      if (other->kind == MK_SOFTCORE_CUT) {
        *out = softcore_setup(sqrt(self->epsilon * other->epsilon), 0.5 * (self->sigma + other->sigma),
                              self->lambda * other->lambda);
        return 1;
      }
      if (other->kind == MK_LJ_CUT) {
        *out = softcore_setup(sqrt(self->epsilon * other->epsilon), 0.5 * (self->sigma + other->sigma),
                              self->lambda);
        return 1;
      }
      return 0;
    default: return 0;
  }
}

/* src/modelClass_pair.f90:120-140 */
static opair pair_container_mix(const opair* a, const opair* b) {
  opair c;
  memset(&c, 0, sizeof c);
  if (!model_mix(&b->model, &a->model, &c.model) && !model_mix(&a->model, &b->model, &c.model)) {
    char msg[128];
    c.model = new_model(MC_PAIR, MK_PAIR_NONE, "none");
    snprintf(msg, sizeof msg, "no mixing rule found for models %s and %s", a->model.name, b->model.name);
    warning(msg);
  }
  c.coulomb = a->coulomb && b->coulomb;
  if (c.coulomb) c.kCoul = sqrt(a->kCoul * b->kCoul);
  return c;
}

/* ======================================================================== */
/* system data (src/EmDeeData.f90:66-151)                                     */
/* ======================================================================== */

typedef struct {
  int nitems, count;
  int *first, *middle, *last, *item;
  double* value;
} olist;

#include "ewald_oracle.h"

typedef struct {   /* tStruct (src/structs.f90): atoms (1-based) and a copy of the model */
  int i, j, k, l;
  omodel model;
} ostruct;

typedef struct {
  int natoms, mcells, ncells, maxcells, maxatoms, ntypes, nbodies, nfree, nthreads, threadAtoms;
  int threadFreeAtoms, nlayers, layer;
  double* Lbox;
  double Rc, skin, RcSq, xRc, xRcSq, skinSq, InRc, InRcSq, xInRcSq, totalMass, startTime;
  int initialized;
  okiss random;
  /* cellAtom list (1-based items) */
  int *cellFirst, *cellLast, *cellItem;
  int *threadCellFirst, *threadCellLast;
  /* excluded pairs (sorted per atom, 1-based items) */
  int *exFirst, *exLast, *exItem, exCount, exItems;
  int *atomType, *atomCell, *atomBody, *freeAtom, *atomsInCell;
  double *R, *P, *F, *charge, *mass, *invMass, *R0;
  char* charged;
  int* cellNeighbor;   /* ncells x 62, 1-based */
  olist* neighbor;     /* one per thread */
  opair* pair;         /* [layer][jtype][itype] */
  omodel* coul;        /* per layer */
  omodel kspace;
  int kspace_active;
  oewald ewald;
  char *multilayer, *overridable, *interact, *pairs_exist;
  char *bonded, *useInRc, *forcesUpToDate;
  double* layerF;
  tEnergy* layerEnergy;
  tVirial* layerVirial;
  int multilayer_coulomb;
  int ownsR;
  obody* body;
  int threadBodies;
  /* bonded structures (src/structs.f90): bonds, angles, dihedrals in insertion order */
  ostruct *bonds, *angles;
  int nbonds, capbonds, nangles, capangles, ndihedrals;
} odata;

#define PAIR(me, i, j, l) ((me)->pair[((size_t)(l) * (me)->ntypes + (j)) * (me)->ntypes + (i)])
#define T2(me, a, i, j) ((me)->a[(size_t)(j) * (me)->ntypes + (i)])

static odata* get(tEmDee md) {
  if (!md.Data) error("system access", "invalid EmDee system");
  return (odata*)md.Data;
}

/* the 62-cell half stencil: offsets in [-2,2]^3 on one side of the plane z=0
 * (z>0, or z=0 and y>0, or z=y=0 and x>0), ordered by |d|^2 and then
 * lexicographically by (x,y,z); this is the table of src/neighbor_lists.f90:26-35 */
static int NB[NBCELLS][3];
static int nb_ready = 0;
static void make_stencil(void) {
  int n = 0;
  if (nb_ready) return;
  for (int d2 = 1; d2 <= 12; d2++)
    for (int x = -2; x <= 2; x++)
      for (int y = -2; y <= 2; y++)
        for (int z = -2; z <= 2; z++) {
          int half = z > 0 || (z == 0 && (y > 0 || (y == 0 && x > 0)));
          if (half && x * x + y * y + z * z == d2) {
            NB[n][0] = x;
            NB[n][1] = y;
            NB[n][2] = z;
            n++;
          }
        }
  if (n != NBCELLS) error("neighbor stencil", "wrong number of cells");
  nb_ready = 1;
}

/* ======================================================================== */
/* EmDee_system (src/EmDeeCode.f90:69-208)                                    */
/* ======================================================================== */

tEmDee EmDee_system(int threads, int layers, double rc, double skin, int N, int* types, double* masses,
                    int* bodies) {
  tEmDee md;
  odata* me = (odata*)xcalloc(1, sizeof(odata));
  make_stencil();
  memset(&md, 0, sizeof md);
  if (threads < 1) threads = 1;
  if (layers < 1) error("system setup", "wrong number of model layers");
  me->nthreads = threads;
  me->nlayers = layers;
  me->Rc = rc;
  me->skin = skin;
  me->RcSq = rc * rc;
  me->xRc = rc + skin;
  me->xRcSq = me->xRc * me->xRc;
  me->InRc = me->Rc;
  me->InRcSq = me->RcSq;
  me->xInRcSq = me->xRcSq;
  me->skinSq = skin * skin;
  me->natoms = N;
  me->threadAtoms = (N + threads - 1) / threads;
  me->kspace_active = 0;

  me->atomType = (int*)xmalloc(sizeof(int) * N);
  if (types) {
    int mn = types[0], mx = types[0];
    for (int i = 1; i < N; i++) {
      if (types[i] < mn) mn = types[i];
      if (types[i] > mx) mx = types[i];
    }
    if (mn != 1) error("system setup", "wrong specification of atom types");
    me->ntypes = mx;
    memcpy(me->atomType, types, sizeof(int) * N);
  } else {
    me->ntypes = 1;
    for (int i = 0; i < N; i++) me->atomType[i] = 1;
  }
  me->mass = (double*)xmalloc(sizeof(double) * N);
  me->invMass = (double*)xmalloc(sizeof(double) * N);
  me->totalMass = 0.0;
  for (int i = 0; i < N; i++) {
    double m = masses ? masses[me->atomType[i] - 1] : 1.0;
    me->mass[i] = m;
    me->invMass[i] = 1.0 / m;
  }
  if (masses) {
    for (int i = 0; i < N; i++) me->totalMass += masses[me->atomType[i] - 1];
  } else {
    me->totalMass = (double)N;
  }
  me->startTime = omp_get_wtime();
  me->P = (double*)xcalloc((size_t)3 * N, sizeof(double));
  me->R0 = (double*)xcalloc((size_t)3 * N, sizeof(double));
  me->charge = (double*)xcalloc(N, sizeof(double));
  me->charged = (char*)xcalloc(N, 1);
  me->atomCell = (int*)xcalloc(N, sizeof(int));

  /* rigid bodies (src/EmDeeData.f90:268-355) */
  me->atomBody = (int*)xcalloc(N, sizeof(int));
  me->freeAtom = (int*)xmalloc(sizeof(int) * N);
  me->nbodies = 0;
  me->nfree = 0;
  if (bodies) {
    /* clean_body_indices: entries <= 0 or unique are free atoms; other values
     * are renumbered 1..nbodies in order of first appearance */
    int *saved = (int*)xmalloc(sizeof(int) * N), *amount = (int*)xmalloc(sizeof(int) * N);
    int *first = (int*)xmalloc(sizeof(int) * N), n = 0;
    for (int i = 0; i < N; i++) {
      int ib = bodies[i], j = -1;
      me->atomBody[i] = 0;
      if (ib <= 0) continue;
      for (int k = 0; k < n; k++)
        if (saved[k] == ib) { j = k; break; }
      if (j < 0) {
        saved[n] = ib;
        amount[n] = 1;
        first[n] = i;
        n++;
      } else {
        amount[j]++;
        me->atomBody[i] = j + 1;
        me->atomBody[first[j]] = j + 1;
      }
    }
    int k = 0;
    for (int j = 0; j < n; j++)
      if (amount[j] > 1) saved[j] = ++k;
    for (int i = 0; i < N; i++)
      if (me->atomBody[i] > 0) me->atomBody[i] = saved[me->atomBody[i] - 1];
    me->nbodies = k;
    free(saved);
    free(amount);
    free(first);
  }
  for (int i = 0; i < N; i++)
    if (me->atomBody[i] == 0) me->freeAtom[me->nfree++] = i + 1;
  me->body = (obody*)xcalloc(me->nbodies > 0 ? me->nbodies : 1, sizeof(obody));
  if (me->nbodies > 0) {
    int* cnt = (int*)xcalloc(me->nbodies, sizeof(int));
    for (int i = 0; i < N; i++)
      if (me->atomBody[i] > 0) cnt[me->atomBody[i] - 1]++;
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      B->NP = 0;
      B->dof = 6;
      B->index = (int*)xmalloc(sizeof(int) * cnt[b]);
      B->M = (double*)xmalloc(sizeof(double) * cnt[b]);
      B->d = (double*)xcalloc(3 * cnt[b], sizeof(double));
      B->delta = (double*)xcalloc(3 * cnt[b], sizeof(double));
    }
    for (int i = 0; i < N; i++)
      if (me->atomBody[i] > 0) {
        obody* B = &me->body[me->atomBody[i] - 1];
        B->index[B->NP] = i + 1;
        B->M[B->NP] = me->mass[i];
        B->NP++;
      }
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      B->mass = 0.0;
      for (int k = 0; k < B->NP; k++) B->mass += B->M[k];
      B->invMass = 1.0 / B->mass;
    }
    free(cnt);
  }
  {
    int k = me->nbodies;   /* free atoms get distinct body indices */
    for (int i = 0; i < N; i++)
      if (me->atomBody[i] == 0) me->atomBody[i] = ++k;
  }
  me->threadBodies = (me->nbodies + threads - 1) / threads;
  me->threadFreeAtoms = (me->nfree + threads - 1) / threads;

  me->cellItem = (int*)xcalloc(N, sizeof(int));
  me->threadCellFirst = (int*)xcalloc(threads, sizeof(int));
  me->threadCellLast = (int*)xcalloc(threads, sizeof(int));
  me->neighbor = (olist*)xcalloc(threads, sizeof(olist));
  for (int t = 0; t < threads; t++) {
    olist* L = &me->neighbor[t];
    L->nitems = EXTRA;
    L->first = (int*)xcalloc(N, sizeof(int));
    L->middle = (int*)xcalloc(N, sizeof(int));
    L->last = (int*)xcalloc(N, sizeof(int));
    L->item = (int*)xcalloc(EXTRA, sizeof(int));
    L->value = (double*)xcalloc(EXTRA, sizeof(double));
  }
  me->exItems = EXTRA;
  me->exItem = (int*)xcalloc(EXTRA, sizeof(int));
  me->exFirst = (int*)xmalloc(sizeof(int) * (N + 1));
  me->exLast = (int*)xmalloc(sizeof(int) * (N + 1));
  for (int i = 0; i < N; i++) {
    me->exFirst[i] = 1;
    me->exLast[i] = 0;
  }
  me->exCount = 0;

  int nt = me->ntypes;
  me->pair = (opair*)xcalloc((size_t)nt * nt * layers, sizeof(opair));
  for (size_t k = 0; k < (size_t)nt * nt * layers; k++) me->pair[k].model = new_model(MC_PAIR, MK_PAIR_NONE, "none");
  me->multilayer = (char*)xcalloc((size_t)nt * nt, 1);
  me->overridable = (char*)xcalloc((size_t)nt * nt, 1);
  memset(me->overridable, 1, (size_t)nt * nt);
  me->interact = (char*)xcalloc((size_t)nt * nt, 1);
  me->coul = (omodel*)xcalloc(layers, sizeof(omodel));
  for (int l = 0; l < layers; l++) me->coul[l] = new_model(MC_COUL, MK_COUL_NONE, "none");
  me->multilayer_coulomb = 0;
  me->pairs_exist = (char*)xcalloc(layers, 1);
  me->useInRc = (char*)xcalloc(layers, 1);
  me->bonded = (char*)xcalloc(layers, 1);
  memset(me->bonded, 1, layers);
  me->forcesUpToDate = (char*)xcalloc(layers, 1);
  me->layerF = (double*)xcalloc((size_t)3 * N * layers, sizeof(double));
  me->layer = 1;
  me->F = me->layerF;
  me->initialized = 0;
  me->random.seeding_required = 1;

  md.Builds = 0;
  md.Energy.UpToDate = false;
  me->layerEnergy = (tEnergy*)xcalloc(layers, sizeof(tEnergy));
  me->layerVirial = (tVirial*)xcalloc(layers, sizeof(tVirial));
  md.DoF = 3 * (N - 1);
  md.RotDoF = 0;
  md.Data = me;
  md.Options.Translate = true;
  md.Options.Rotate = true;
  md.Options.RotationMode = 0;
  md.Options.AutoForceCompute = true;
  md.Options.AutoBodyUpdate = true;
  md.Options.Compute = true;
  return md;
}

void EmDee_set_precision(tEmDee md, int mode) { (void)get(md); (void)mode; }

void EmDee_destroy(tEmDee* md) { (void)md; }

/* ======================================================================== */
/* model setters (src/EmDeeCode.f90:309-520, src/EmDeeData.f90:193-264)       */
/* ======================================================================== */

static double layer_rc(odata* me, int layer) { return me->useInRc[layer - 1] ? me->InRc : me->Rc; }

/* src/EmDeeData.f90:227-264 */
static void set_pair_type(odata* me, int itype, int jtype, int layer, const omodel* model, double kCoul) {
  double lrc = layer_rc(me, layer);
  if (itype == jtype) {
    opair* p = &PAIR(me, itype - 1, itype - 1, layer - 1);
    p->model = *model;
    p->coulomb = kCoul != 0.0;
    if (p->coulomb) p->kCoul = kCoul;
    modifier_setup(&p->model, lrc);
    for (int k = 1; k <= me->ntypes; k++) {
      if (k != itype && T2(me, overridable, itype - 1, k - 1)) {
        opair c = pair_container_mix(&PAIR(me, k - 1, k - 1, layer - 1), p);
        modifier_setup(&c.model, lrc);
        PAIR(me, itype - 1, k - 1, layer - 1) = c;
        PAIR(me, k - 1, itype - 1, layer - 1) = c;
      }
    }
  } else {
    opair* p = &PAIR(me, itype - 1, jtype - 1, layer - 1);
    p->model = *model;
    p->coulomb = kCoul != 0.0;
    if (p->coulomb) p->kCoul = kCoul;
    modifier_setup(&p->model, lrc);
    PAIR(me, jtype - 1, itype - 1, layer - 1) = *p;
  }
}

static int ranged(int i, int imax) { return i > 0 && i <= imax; }

static void finish_pair_setting(odata* me, int itype, int jtype, int multi) {
  T2(me, multilayer, itype - 1, jtype - 1) = (char)multi;
  T2(me, multilayer, jtype - 1, itype - 1) = (char)multi;
  if (itype == jtype) {
    for (int k = 1; k <= me->ntypes; k++)
      if (k != itype && T2(me, overridable, itype - 1, k - 1)) {
        char v = multi ? 1 : T2(me, multilayer, k - 1, k - 1);
        T2(me, multilayer, itype - 1, k - 1) = v;
        T2(me, multilayer, k - 1, itype - 1) = v;
      }
  } else {
    T2(me, overridable, itype - 1, jtype - 1) = 0;
    T2(me, overridable, jtype - 1, itype - 1) = 0;
  }
}

void EmDee_set_pair_model(tEmDee md, int itype, int jtype, void* model, double kCoul) {
  const char* task = "pair model setup";
  odata* me = get(md);
  if (me->initialized) error(task, "cannot set model after coordinates have been defined");
  if (!ranged(itype, me->ntypes) || !ranged(jtype, me->ntypes)) error(task, "provided type index is out of range");
  if (!model) error(task, "a valid pair model must be provided");
  omodel* m = (omodel*)model;
  if (m->cls != MC_PAIR) error(task, "a valid pair model must be provided");
  for (int l = 1; l <= me->nlayers; l++) set_pair_type(me, itype, jtype, l, m, kCoul);
  finish_pair_setting(me, itype, jtype, 0);
}

void EmDee_set_pair_multimodel(tEmDee md, int itype, int jtype, void* model[], double kCoul[]) {
  const char* task = "pair multimodel setup";
  odata* me = get(md);
  if (me->initialized) error(task, "cannot set model after coordinates have been defined");
  if (!ranged(itype, me->ntypes) || !ranged(jtype, me->ntypes)) error(task, "provided type index is out of range");
  for (int l = 1; l <= me->nlayers; l++) {
    if (!model[l - 1]) {
      char msg[64];
      snprintf(msg, sizeof msg, "%d valid pair models must be provided", me->nlayers);
      error(task, msg);
    }
    omodel* m = (omodel*)model[l - 1];
    if (m->cls != MC_PAIR) error(task, "a valid pair model must be provided");
    set_pair_type(me, itype, jtype, l, m, kCoul[l - 1]);
  }
  finish_pair_setting(me, itype, jtype, 1);
}

void EmDee_set_kspace_model(tEmDee md, void* model) {
  const char* task = "kspace model setup";
  odata* me = get(md);
  if (me->initialized) error(task, "cannot set model after coordinates have been defined");
  if (!model || ((omodel*)model)->cls != MC_KSPACE) error(task, "a valid kspace model must be provided");
  me->kspace = *(omodel*)model;
  me->kspace_active = 1;
}

void EmDee_set_coul_model(tEmDee md, void* model) {
  const char* task = "coulomb model setup";
  odata* me = get(md);
  if (me->initialized) error(task, "cannot set model after coordinates have been defined");
  if (!model) error(task, "a valid coulomb model must be provided");
  omodel* m = (omodel*)model;
  if (m->cls != MC_COUL) error(task, "a valid coulomb model must be provided");
  for (int l = 1; l <= me->nlayers; l++) {
    double lrc = layer_rc(me, l);
    me->coul[l - 1] = *m;
    cutoff_setup(&me->coul[l - 1], lrc);
    modifier_setup(&me->coul[l - 1], lrc);
  }
  me->multilayer_coulomb = 0;
}

void EmDee_set_coul_multimodel(tEmDee md, void* model[]) {
  const char* task = "coulomb multimodel setup";
  odata* me = get(md);
  if (me->initialized) error(task, "cannot set model after coordinates have been defined");
  for (int l = 1; l <= me->nlayers; l++) {
    double lrc = layer_rc(me, l);
    if (!model[l - 1]) {
      char msg[64];
      snprintf(msg, sizeof msg, "%d valid coulomb models must be provided", me->nlayers);
      error(task, msg);
    }
    omodel* m = (omodel*)model[l - 1];
    if (m->cls != MC_COUL) error(task, "a valid coulomb model must be provided");
    me->coul[l - 1] = *m;
    cutoff_setup(&me->coul[l - 1], lrc);
    modifier_setup(&me->coul[l - 1], lrc);
  }
  me->multilayer_coulomb = 1;
}

/* src/EmDeeCode.f90:273-305 */
void EmDee_layer_based_parameters(tEmDee md, double InternalRc, int* Apply, int* Bonded) {
  const char* task = "layer-based parameter setting";
  odata* me = get(md);
  int any = 0;
  if (me->initialized) error(task, "system has already been initialized");
  for (int l = 0; l < me->nlayers; l++) {
    me->useInRc[l] = Apply[l] != 0;
    any |= me->useInRc[l];
  }
  if (any && (InternalRc <= 0.0 || InternalRc > me->Rc)) error(task, "invalid internal cutoff specification");
  me->InRc = InternalRc;
  me->InRcSq = InternalRc * InternalRc;
  me->xInRcSq = (InternalRc + me->skin) * (InternalRc + me->skin);
  for (int l = 0; l < me->nlayers; l++) me->bonded[l] = Bonded[l] != 0;
  for (int l = 1; l <= me->nlayers; l++) cutoff_setup(&me->coul[l - 1], layer_rc(me, l));
}

/* src/EmDeeCode.f90:524-570: sorted, duplicate-free exclusion lists */
void EmDee_ignore_pair(tEmDee md, int i, int j) {
  odata* me = get(md);
  if (i == j || !ranged(i, me->natoms) || !ranged(j, me->natoms)) return;
  for (int pass = 0; pass < 2; pass++) {
    int a = pass ? j : i, b = pass ? i : j;
    int first = me->exFirst[a - 1], last = me->exLast[a - 1], pos;
    int found = 0;
    pos = last + 1;
    for (int k = first; k <= last; k++) {
      if (me->exItem[k - 1] == b) { found = 1; break; }
      if (me->exItem[k - 1] > b) { pos = k; break; }
    }
    if (found) continue;
    if (me->exCount + 1 > me->exItems) {
      me->exItems += EXTRA;
      me->exItem = (int*)realloc(me->exItem, sizeof(int) * me->exItems);
    }
    memmove(&me->exItem[pos], &me->exItem[pos - 1], sizeof(int) * (me->exCount - (pos - 1)));
    me->exItem[pos - 1] = b;
    for (int k = a; k < me->natoms; k++) me->exFirst[k]++;
    for (int k = a - 1; k < me->natoms; k++) me->exLast[k]++;
    me->exCount++;
  }
}

/* src/structs.f90:40-60 (structList_add) */
static void struct_add(ostruct** list, int* n, int* cap, int i, int j, int k, int l, const omodel* model) {
  if (*n == *cap) {
    *cap += EXTRA;
    *list = (ostruct*)realloc(*list, sizeof(ostruct) * (size_t)(*cap));
  }
  ostruct* it = &(*list)[(*n)++];
  it->i = i;
  it->j = j;
  it->k = k;
  it->l = l;
  it->model = *model;
}

/* src/EmDeeCode.f90:574-596 */
void EmDee_add_bond(tEmDee md, int i, int j, void* model) {
  odata* me = get(md);
  if (!ranged(i, me->natoms) || !ranged(j, me->natoms)) error("add_bond", "atom index out of range");
  if (!model) error("add_bond", "a valid model must be provided");
  if (((omodel*)model)->cls != MC_BOND) error("add_bond", "the provided model must be a bond model");
  struct_add(&me->bonds, &me->nbonds, &me->capbonds, i, j, 0, 0, (omodel*)model);
  EmDee_ignore_pair(md, i, j);
}

/* src/EmDeeCode.f90:600-624 */
void EmDee_add_angle(tEmDee md, int i, int j, int k, void* model) {
  odata* me = get(md);
  if (!ranged(i, me->natoms) || !ranged(j, me->natoms) || !ranged(k, me->natoms))
    error("add_angle", "atom index out of range");
  if (!model) error("add_angle", "a valid model must be provided");
  if (((omodel*)model)->cls != MC_ANGLE) error("add_angle", "the provided model must be an angle model");
  struct_add(&me->angles, &me->nangles, &me->capangles, i, j, k, 0, (omodel*)model);
  EmDee_ignore_pair(md, i, j);
  EmDee_ignore_pair(md, i, k);
  EmDee_ignore_pair(md, j, k);
}

/* src/EmDeeCode.f90:628-655; the reference never evaluates dihedrals */
void EmDee_add_dihedral(tEmDee md, int i, int j, int k, int l, void* model) {
  odata* me = get(md);
  if (!ranged(i, me->natoms) || !ranged(j, me->natoms) || !ranged(k, me->natoms) || !ranged(l, me->natoms))
    error("add_dihedral", "atom index out of range");
  if (!model) error("add_dihedral", "a valid model must be provided");
  if (((omodel*)model)->cls != MC_DIHEDRAL) error("add_dihedral", "the provided model must be a dihedral model");
  me->ndihedrals++;
  EmDee_ignore_pair(md, i, j);
  EmDee_ignore_pair(md, i, k);
  EmDee_ignore_pair(md, i, l);
  EmDee_ignore_pair(md, j, k);
  EmDee_ignore_pair(md, j, l);
  EmDee_ignore_pair(md, k, l);
}

/* src/EmDeeData.f90:193-223 */
static void check_actual_interactions(odata* me) {
  int nt = me->ntypes, nl = me->nlayers;
  char* neutral = (char*)xcalloc(nt, 1);
  char* inter = (char*)xcalloc((size_t)nt * nt * nl, 1);
  for (int t = 0; t < nt; t++) {
    int count = 0;
    for (int a = 0; a < me->natoms; a++)
      if (me->atomType[a] == t + 1 && me->charged[a]) count++;
    neutral[t] = count == 0;
  }
  for (int i = 0; i < nt; i++)
    for (int j = 0; j <= i; j++) {
      int any = 0;
      for (int k = 0; k < nl; k++) {
        opair* p = &PAIR(me, i, j, k);
        int no_pair = p->model.kind == MK_PAIR_NONE;
        int no_coul = me->coul[k].kind == MK_COUL_NONE || !p->coulomb;
        int coul_only = no_pair && !no_coul;
        int inert = (no_pair && no_coul) || (coul_only && neutral[i] && neutral[j]);
        inter[((size_t)k * nt + j) * nt + i] = !inert;
        any |= !inert;
      }
      T2(me, interact, i, j) = (char)any;
      T2(me, interact, j, i) = (char)any;
    }
  for (int k = 0; k < nl; k++) {
    int any = 0;
    for (size_t q = 0; q < (size_t)nt * nt; q++) any |= inter[(size_t)k * nt * nt + q];
    me->pairs_exist[k] = (char)any;
  }
  free(neutral);
  free(inter);
}

/* ======================================================================== */
/* neighbor lists (src/neighbor_lists.f90)                                    */
/* ======================================================================== */

/* src/neighbor_lists.f90:41-59 (sum of the largest and of a "next" value that
 * is only refreshed when a new maximum is found) */
static double maximum_approach_sq(odata* me) {
  double maximum, next, dsq;
  const double *R = me->R, *R0 = me->R0;
  double d0 = R[0] - R0[0], d1 = R[1] - R0[1], d2 = R[2] - R0[2];
  maximum = d0 * d0 + d1 * d1 + d2 * d2;
  next = maximum;
  for (int i = 1; i < me->natoms; i++) {
    d0 = R[3 * i] - R0[3 * i];
    d1 = R[3 * i + 1] - R0[3 * i + 1];
    d2 = R[3 * i + 2] - R0[3 * i + 2];
    dsq = d0 * d0 + d1 * d1 + d2 * d2;
    if (dsq > maximum) {
      next = maximum;
      maximum = dsq;
    }
  }
  return maximum + 2 * sqrt(maximum * next) + next;
}

static inline int ipbc(int x, int M) { return x < 0 ? x + M : (x >= M ? x - M : x); }

/* src/neighbor_lists.f90:63-171 */
static void distribute_atoms(odata* me, int M, const double* Rs) {
  int MM = M * M, nt = me->nthreads, make_cells = M != me->mcells, cells_per_thread = 0;
  int* maxNatoms = (int*)xcalloc(nt, sizeof(int));
  int* threadNatoms = (int*)xcalloc(nt, sizeof(int));
  int* next = (int*)xcalloc(me->natoms + 1, sizeof(int));
  if (make_cells) {
    me->mcells = M;
    me->ncells = M * MM;
    if (me->ncells > me->maxcells) {
      free(me->cellNeighbor);
      free(me->cellFirst);
      free(me->cellLast);
      free(me->atomsInCell);
      me->cellNeighbor = (int*)xcalloc((size_t)me->ncells * NBCELLS, sizeof(int));
      me->cellFirst = (int*)xcalloc(me->ncells, sizeof(int));
      me->cellLast = (int*)xcalloc(me->ncells, sizeof(int));
      me->atomsInCell = (int*)xcalloc(me->ncells, sizeof(int));
      me->maxcells = me->ncells;
    }
    cells_per_thread = (me->ncells + nt - 1) / nt;
  }
  omp_set_dynamic(0);
#pragma omp parallel num_threads(nt)
  {
    int thread = omp_get_thread_num() + 1, first, last;
    if (make_cells) {
      first = (thread - 1) * cells_per_thread + 1;
      last = (thread * cells_per_thread < me->ncells) ? thread * cells_per_thread : me->ncells;
      for (int icell = first; icell <= last; icell++) {
        int k = icell - 1, iz = k / MM, j = k - iz * MM, iy = j / M, ix = j - iy * M;
        int* nbr = &me->cellNeighbor[(size_t)(icell - 1) * NBCELLS];
        for (int m = 0; m < NBCELLS; m++)
          nbr[m] = 1 + ipbc(ix + NB[m][0], M) + ipbc(iy + NB[m][1], M) * M + ipbc(iz + NB[m][2], M) * MM;
      }
      me->threadCellFirst[thread - 1] = first;
      me->threadCellLast[thread - 1] = last;
    } else {
      first = me->threadCellFirst[thread - 1];
      last = me->threadCellLast[thread - 1];
    }
    int a1 = (thread - 1) * me->threadAtoms + 1;
    int aN = thread * me->threadAtoms < me->natoms ? thread * me->threadAtoms : me->natoms;
    for (int i = a1; i <= aN; i++) {
      int ic[3];
      for (int d = 0; d < 3; d++) {
        double s = Rs[3 * (i - 1) + d];
        ic[d] = (int)(M * (s - floor(s)));
      }
      me->atomCell[i - 1] = 1 + ic[0] + M * ic[1] + MM * ic[2];
    }
#pragma omp barrier
    int* head = (int*)xcalloc(last >= first ? last - first + 1 : 1, sizeof(int));
    for (int icell = first; icell <= last; icell++) me->atomsInCell[icell - 1] = 0;
    for (int i = 1; i <= me->natoms; i++) {
      int icell = me->atomCell[i - 1];
      if (icell >= first && icell <= last) {
        next[i] = head[icell - first];
        head[icell - first] = i;
        me->atomsInCell[icell - 1]++;
      }
    }
    int tn = 0;
    for (int icell = first; icell <= last; icell++) tn += me->atomsInCell[icell - 1];
    threadNatoms[thread - 1] = tn;
#pragma omp barrier
    int mx = 0, k = 0;
    for (int t = 0; t < thread - 1; t++) k += threadNatoms[t];
    for (int icell = first; icell <= last; icell++) {
      me->cellFirst[icell - 1] = k + 1;
      int i = head[icell - first];
      while (i != 0) {
        me->cellItem[k++] = i;
        i = next[i];
      }
      me->cellLast[icell - 1] = k;
      if (me->atomsInCell[icell - 1] > mx) mx = me->atomsInCell[icell - 1];
    }
    maxNatoms[thread - 1] = mx;
    free(head);
  }
  me->maxatoms = 0;
  for (int t = 0; t < nt; t++)
    if (maxNatoms[t] > me->maxatoms) me->maxatoms = maxNatoms[t];
  free(maxNatoms);
  free(threadNatoms);
  free(next);
}

static inline double pbc(double x) { return x - anint(x); }

/* insertion by r^2 (src/neighbor_lists.f90:283-298) */
static inline void insert_neighbor(int* item, double* value, int* npairs, int j, double r2) {
  int k;
  for (k = *npairs; k >= 1; k--) {
    if (value[k - 1] < r2) break;
    value[k] = value[k - 1];
    item[k] = item[k - 1];
  }
  value[k] = r2;
  item[k] = j;
  (*npairs)++;
}

/* src/neighbor_lists.f90:199-300, one thread's cells */
static void build_neighbor_lists(odata* me, int thread, const double* Rs) {
  olist* nb = &me->neighbor[thread - 1];
  double invL2 = 1.0 / (*me->Lbox * *me->Lbox);
  double xRc2 = me->xRcSq * invL2, xInRc2 = me->xInRcSq * invL2;
  int npairs = 0, cap = (NBCELLS + 1) * (me->maxatoms > 0 ? me->maxatoms : 1);
  char* include = (char*)xmalloc(me->natoms + 1);
  int* atom = (int*)xmalloc(sizeof(int) * cap);
  double* rsq = (double*)xmalloc(sizeof(double) * cap);
  memset(include, 1, me->natoms + 1);
  for (int icell = me->threadCellFirst[thread - 1]; icell <= me->threadCellLast[thread - 1]; icell++) {
    const int* neigh = &me->cellNeighbor[(size_t)(icell - 1) * NBCELLS];
    int nlocal = me->atomsInCell[icell - 1], ntotal = nlocal;
    for (int k = me->cellFirst[icell - 1]; k <= me->cellLast[icell - 1]; k++) atom[k - me->cellFirst[icell - 1]] = me->cellItem[k - 1];
    for (int m = 0; m < NBCELLS; m++) {
      int c = neigh[m];
      for (int k = me->cellFirst[c - 1]; k <= me->cellLast[c - 1]; k++) atom[ntotal++] = me->cellItem[k - 1];
    }
    if (nb->nitems < npairs + nlocal * ntotal) {
      nb->nitems = npairs + nlocal * ntotal + EXTRA;
      nb->item = (int*)realloc(nb->item, sizeof(int) * nb->nitems);
      nb->value = (double*)realloc(nb->value, sizeof(double) * nb->nitems);
    }
    for (int k = 1; k <= nlocal; k++) {
      int i = atom[k - 1], first = npairs + 1, ipairs = 0, middle = 0;
      int itype = me->atomType[i - 1], ibody = me->atomBody[i - 1];
      int* item = &nb->item[first - 1];
      double* value = &nb->value[first - 1];
      nb->first[i - 1] = first;
      for (int x = me->exFirst[i - 1]; x <= me->exLast[i - 1]; x++) include[me->exItem[x - 1]] = 0;
      const double* Ri = &Rs[3 * (i - 1)];
      for (int m = k + 1; m <= ntotal; m++) {
        const double* Rj = &Rs[3 * (atom[m - 1] - 1)];
        double dx = pbc(Ri[0] - Rj[0]), dy = pbc(Ri[1] - Rj[1]), dz = pbc(Ri[2] - Rj[2]);
        rsq[m - k - 1] = dx * dx + dy * dy + dz * dz;
      }
      for (int m = 1; m <= ntotal - k; m++) {
        double r2 = rsq[m - 1];
        if (r2 < xRc2) {
          int j = atom[k + m - 1];
          if (include[j] && me->atomBody[j - 1] != ibody && T2(me, interact, me->atomType[j - 1] - 1, itype - 1)) {
            insert_neighbor(item, value, &ipairs, j, r2);
            if (r2 < xInRc2) middle++;
          }
        }
      }
      for (int x = me->exFirst[i - 1]; x <= me->exLast[i - 1]; x++) include[me->exItem[x - 1]] = 1;
      nb->middle[i - 1] = npairs + middle;
      npairs += ipairs;
      nb->last[i - 1] = npairs;
    }
  }
  nb->count = npairs;
  free(include);
  free(atom);
  free(rsq);
}

/* src/neighbor_lists.f90:175-195 */
static void handle_neighbor_lists(odata* me, int* builds, double* time, const double* Rs) {
  *time -= omp_get_wtime();
  if (maximum_approach_sq(me) > me->skinSq) {
    int M = (int)floor(NDIV * *me->Lbox / me->xRc);
    distribute_atoms(me, M > 2 * NDIV + 1 ? M : 2 * NDIV + 1, Rs);
    memcpy(me->R0, me->R, sizeof(double) * 3 * me->natoms);
    (*builds)++;
#pragma omp parallel num_threads(me->nthreads)
    build_neighbor_lists(me, omp_get_thread_num() + 1, Rs);
  }
  *time += omp_get_wtime();
}

/* ======================================================================== */
/* pair forces (src/EmDeeData.f90:644-685 + src/compute.f90)                  */
/* ======================================================================== */

static void compute_pairs(odata* me, int thread, int compute, const double* Rs, double* F, double* Epair,
                          double* Ecoul, double* Wpair, double* Wcoul) {
  int layer = me->layer;
  memset(F, 0, sizeof(double) * 3 * me->natoms);
  *Wpair = *Wcoul = *Epair = 0.0;
  *Ecoul = 0.0;
  if (!me->pairs_exist[layer - 1]) return;
  double L = *me->Lbox, L2 = L * L, invL2 = 1.0 / L2, Rc2;
  olist* nb = &me->neighbor[thread - 1];
  const int* upper;
  if (me->useInRc[layer - 1]) {
    Rc2 = me->InRcSq * invL2;
    upper = nb->middle;
  } else {
    Rc2 = me->RcSq * invL2;
    upper = nb->last;
  }
  const omodel* coul = &me->coul[layer - 1];
  int firstAtom = me->cellFirst[me->threadCellFirst[thread - 1] - 1];
  int lastAtom = me->cellLast[me->threadCellLast[thread - 1] - 1];
  for (int k = firstAtom; k <= lastAtom; k++) {
    int i = me->cellItem[k - 1], itype = me->atomType[i - 1];
    double Qi = me->charge[i - 1];
    int icharged = me->charged[i - 1];
    const double* Ri = &Rs[3 * (i - 1)];
    double Fi[3] = {0.0, 0.0, 0.0};
    for (int m = nb->first[i - 1]; m <= upper[i - 1]; m++) {
      int j = nb->item[m - 1];
      const double* Rj = &Rs[3 * (j - 1)];
      double Rij[3] = {pbc(Ri[0] - Rj[0]), pbc(Ri[1] - Rj[1]), pbc(Ri[2] - Rj[2])};
      double r2 = Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2];
      if (r2 < Rc2) {
        double invR2 = invL2 / r2, invR = sqrt(invR2), Eij = 0.0, Wij = 0.0, Wsum;
        int jtype = me->atomType[j - 1];
        int ijcharged = icharged && me->charged[j - 1];
        const opair* pr = &PAIR(me, jtype - 1, itype - 1, layer - 1);
        if (compute) {
          model_compute(&pr->model, &Eij, &Wij, invR, invR2);
          apply_modifier_compute(&pr->model, &Eij, &Wij, invR, invR2);
          *Epair += Eij;
        } else {
          Wij = model_virial(&pr->model, invR, invR2);
          apply_modifier_virial(&pr->model, &Wij, invR, invR2);
        }
        *Wpair += Wij;
        Wsum = Wij;
        if (ijcharged && pr->coulomb) {
          if (compute) {
            model_compute(coul, &Eij, &Wij, invR, invR2);
            apply_modifier_compute(coul, &Eij, &Wij, invR, invR2);
          } else {
            Wij = model_virial(coul, invR, invR2);
            apply_modifier_virial(coul, &Wij, invR, invR2);
          }
          double QiQj = pr->kCoul * Qi * me->charge[j - 1];
          if (compute) *Ecoul += QiQj * Eij;
          Wij = QiQj * Wij;
          *Wcoul += Wij;
          Wsum += Wij;
        }
        double s = Wsum * invR2;
        double Fij[3] = {s * Rij[0], s * Rij[1], s * Rij[2]};
        for (int d = 0; d < 3; d++) {
          Fi[d] += Fij[d];
          F[3 * (j - 1) + d] -= Fij[d];
        }
      }
    }
    for (int d = 0; d < 3; d++) F[3 * (i - 1) + d] += Fi[d];
  }
  for (size_t q = 0; q < (size_t)3 * me->natoms; q++) F[q] = L * F[q];
}

/* compute_bonds (src/EmDeeData.f90:443-487) with bond_harmonic (src/bond_harmonic.f90:64-75) */
static void compute_bonds(odata* me, int thread, const double* R, double* F, double* Potential, double* Virial,
                          double* Ecoul) {
  int layer = me->layer, bonded = me->bonded[layer - 1], kspace = me->coul[layer - 1].requires_kspace;
  if (!(me->nbonds > 0 && (bonded || kspace))) return;
  int per = (me->nbonds + me->nthreads - 1) / me->nthreads;
  double L = *me->Lbox, invL2 = 1.0 / (L * L);
  int last = thread * per < me->nbonds ? thread * per : me->nbonds;
  for (int m = (thread - 1) * per + 1; m <= last; m++) {
    const ostruct* b = &me->bonds[m - 1];
    double Rij[3];
    for (int d = 0; d < 3; d++) Rij[d] = pbc(R[3 * (b->i - 1) + d] - R[3 * (b->j - 1) + d]);
    double invR2 = invL2 / (Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2]);
    double E = 0.0, W = 0.0;
    if (bonded) {
      if (b->model.kind == MK_BOND_HARMONIC) {
        double r = 1.0 / sqrt(invR2), delta = r - b->model.x0;
        E = (0.5 * b->model.k) * (delta * delta);
        W = (-b->model.k) * delta * r;
      }
      *Potential += E;
      *Virial += W;
    } else {
      W = 0.0;
    }
    if (kspace) {
      int itype = me->atomType[b->i - 1], jtype = me->atomType[b->j - 1];
      double QiQj = PAIR(me, itype - 1, jtype - 1, layer - 1).kCoul * me->charge[b->i - 1] * me->charge[b->j - 1];
      double EL, WL;
      ewald_discount(&me->ewald, &EL, &WL, 1.0 / invR2, QiQj);
      *Ecoul += EL;
      W = W + WL;
    }
    for (int d = 0; d < 3; d++) {
      double Fij = W * invR2 * L * Rij[d];
      F[3 * (b->i - 1) + d] += Fij;
      F[3 * (b->j - 1) + d] -= Fij;
    }
  }
}

/* compute_angles (src/EmDeeData.f90:491-550) with angle_harmonic (src/angle_harmonic.f90:64-73) */
static void compute_angles(odata* me, int thread, const double* R, double* F, double* Potential, double* Virial,
                           double* Ecoul) {
  int layer = me->layer, bonded = me->bonded[layer - 1], kspace = me->coul[layer - 1].requires_kspace;
  if (!(me->nangles > 0 && (bonded || kspace))) return;
  int per = (me->nangles + me->nthreads - 1) / me->nthreads;
  double L = *me->Lbox;
  int last = thread * per < me->nangles ? thread * per : me->nangles;
  for (int m = (thread - 1) * per + 1; m <= last; m++) {
    const ostruct* g = &me->angles[m - 1];
    int i = g->i, j = g->j, k = g->k;
    double a[3], b[3];
    for (int d = 0; d < 3; d++) {
      a[d] = L * pbc(R[3 * (i - 1) + d] - R[3 * (j - 1) + d]);
      b[d] = L * pbc(R[3 * (k - 1) + d] - R[3 * (j - 1) + d]);
    }
    if (bonded) {
      double aa = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
      double bb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
      double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
      double theta = acos(ab / sqrt(aa * bb)), Ea = 0.0, Fa = 0.0;
      if (g->model.kind == MK_ANGLE_HARMONIC) {
        double delta = theta - g->model.x0;
        Ea = (0.5 * g->model.k) * (delta * delta);
        Fa = (-g->model.k) * delta;
      }
      double factor = Fa / sqrt(aa * bb - ab * ab), Fi[3], Fk[3], v = 0.0;
      for (int d = 0; d < 3; d++) {
        Fi[d] = ((ab / aa) * a[d] - b[d]) * factor;
        Fk[d] = ((ab / bb) * b[d] - a[d]) * factor;
      }
      for (int d = 0; d < 3; d++) {
        F[3 * (i - 1) + d] += Fi[d];
        F[3 * (k - 1) + d] += Fk[d];
        F[3 * (j - 1) + d] -= Fi[d] + Fk[d];
        v += Fi[d] * a[d] + Fk[d] * b[d];
      }
      *Potential += Ea;
      *Virial += v;
    }
    if (kspace) {
      double Rik[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
      double RikSq = Rik[0] * Rik[0] + Rik[1] * Rik[1] + Rik[2] * Rik[2], EL, WL;
      int itype = me->atomType[i - 1], ktype = me->atomType[k - 1];
      double QiQk = PAIR(me, itype - 1, ktype - 1, layer - 1).kCoul * me->charge[i - 1] * me->charge[k - 1];
      ewald_discount(&me->ewald, &EL, &WL, RikSq, QiQk);
      *Ecoul += EL;
      for (int d = 0; d < 3; d++) {
        double Fik = WL * Rik[d] / RikSq;
        F[3 * (i - 1) + d] += Fik;
        F[3 * (k - 1) + d] -= Fik;
      }
    }
  }
}

/* ======================================================================== */
/* EmDee_compute_forces (src/EmDeeCode.f90:1215-1277)                         */
/* ======================================================================== */

void EmDee_compute_forces(tEmDee* md) {
  odata* me = get(*md);
  int N = me->natoms, nt = me->nthreads;
  double L = *me->Lbox, E[5] = {0, 0, 0, 0, 0}, W[5] = {0, 0, 0, 0, 0};
  double* Rs = (double*)xmalloc(sizeof(double) * 3 * N);
  double* Fs = (double*)xmalloc(sizeof(double) * 3 * N * nt);
  double* Et = (double*)xcalloc((size_t)nt * 8, sizeof(double));
  int compute = md->Options.Compute;
  for (size_t q = 0; q < (size_t)3 * N; q++) Rs[q] = me->R[q] / L;
  handle_neighbor_lists(me, &md->Builds, &md->Time.Neighbor, Rs);
  md->Time.Pair -= omp_get_wtime();
#pragma omp parallel num_threads(nt)
  {
    int thread = omp_get_thread_num() + 1;
    double* ev = &Et[8 * (thread - 1)];
    double* Ft = &Fs[(size_t)3 * N * (thread - 1)];
    compute_pairs(me, thread, compute, Rs, Ft, &ev[0], &ev[1], &ev[2], &ev[3]);
    compute_bonds(me, thread, Rs, Ft, &ev[4], &ev[5], &ev[1]);
    compute_angles(me, thread, Rs, Ft, &ev[6], &ev[7], &ev[1]);
  }
  for (int t = 0; t < nt; t++) {   /* OpenMP reduction(+:E,W), taken in thread order */
    E[0] += Et[8 * t];
    E[1] += Et[8 * t + 1];
    W[0] += Et[8 * t + 2];
    W[1] += Et[8 * t + 3];
    E[3] += Et[8 * t + 4];
    W[3] += Et[8 * t + 5];
    E[4] += Et[8 * t + 6];
    W[4] += Et[8 * t + 7];
  }
  for (size_t q = 0; q < (size_t)3 * N; q++) {   /* me%F = sum(Fs,3) */
    double s = Fs[q];
    for (int t = 1; t < nt; t++) s += Fs[(size_t)3 * N * t + q];
    me->F[q] = s;
  }
  if (me->coul[me->layer - 1].requires_kspace) {   /* src/EmDeeCode.f90:1249-1252, src/EmDeeData.f90:689-700 */
    ewald_prepare(&me->ewald, Rs);
    ewald_compute(&me->ewald, me->layer, &E[2], me->F);
    E[2] += ewald_discount_energy(&me->ewald, me->layer);
    W[2] = E[1] + E[2] - W[1];
  }
  md->Virial.Total = W[0] + W[1] + W[2] + W[3] + W[4];
  md->Virial.Body = 0.0;
  if (me->nbodies != 0) {   /* src/EmDeeData.f90:926-953 */
    double Wb = 0.0;
    for (int t = 0; t < nt; t++) {
      double Wt = 0.0;
      int b1 = t * me->threadBodies, bN = (t + 1) * me->threadBodies < me->nbodies ? (t + 1) * me->threadBodies : me->nbodies;
      for (int b = b1; b < bN; b++) {
        obody* B = &me->body[b];
        double s = 0.0;
        for (int k = 0; k < B->NP; k++)
          for (int x = 0; x < 3; x++) s += me->F[3 * (B->index[k] - 1) + x] * B->delta[3 * k + x];
        Wt += s;
      }
      Wb += Wt;
    }
    md->Virial.Body = -Wb;
    md->Virial.Total = md->Virial.Total + md->Virial.Body;
  }
  if (compute) {
    md->Energy.Dispersion = E[0];
    md->Energy.Coulomb = E[1] + E[2];
    md->Energy.Bond = E[3];
    md->Energy.Angle = E[4];
    md->Energy.Potential = E[0] + E[1] + E[2] + E[3] + E[4];
    md->Energy.ShadowPotential = md->Energy.Potential;
  }
  md->Energy.UpToDate = compute;
  me->forcesUpToDate[me->layer - 1] = 1;
  me->layerEnergy[me->layer - 1] = md->Energy;
  me->layerVirial[me->layer - 1] = md->Virial;
  double t = omp_get_wtime();
  md->Time.Pair += t;
  md->Time.Total = t - me->startTime;
  free(Rs);
  free(Fs);
  free(Et);
}

/* ======================================================================== */
/* data exchange, initialization, layers                                      */
/* ======================================================================== */

void EmDee_switch_model_layer(tEmDee* md, int layer) {   /* src/EmDeeCode.f90:929-946 */
  odata* me = get(*md);
  if (layer != me->layer) {
    if (layer < 1 || layer > me->nlayers) error("model layer switch", "selected layer is out of range");
    me->layer = layer;
    md->Energy = me->layerEnergy[layer - 1];
    md->Virial = me->layerVirial[layer - 1];
    me->F = &me->layerF[(size_t)3 * me->natoms * (layer - 1)];
  }
}

/* src/EmDeeData.f90:359-416 (free atoms) */
/* src/EmDeeData.f90:420-439: unwrap each body around its first atom and refresh it */
static void update_rigid_bodies(odata* me) {
  double L = *me->Lbox, invL = 1.0 / L;
  for (int b = 0; b < me->nbodies; b++) {
    obody* B = &me->body[b];
    double* R = (double*)xmalloc(sizeof(double) * 3 * B->NP);
    for (int k = 0; k < B->NP; k++)
      for (int x = 0; x < 3; x++) R[3 * k + x] = me->R[3 * (B->index[k] - 1) + x];
    for (int k = 1; k < B->NP; k++)
      for (int x = 0; x < 3; x++) R[3 * k + x] = R[3 * k + x] - L * anint(invL * (R[3 * k + x] - R[x]));
    body_update(B, R);
    for (int k = 0; k < B->NP; k++)
      for (int x = 0; x < 3; x++) me->R[3 * (B->index[k] - 1) + x] = R[3 * k + x];
    free(R);
  }
}

static double pair_kcoul(void* ctx, int itype, int jtype, int layer) {   /* me%pair%kCoul */
  odata* me = (odata*)ctx;
  return PAIR(me, itype - 1, jtype - 1, layer - 1).kCoul;
}

static void perform_initialization(odata* me, int* DoF, int* RotDoF) {
  update_rigid_bodies(me);
  int bodyDoF = 0;
  for (int b = 0; b < me->nbodies; b++) bodyDoF += me->body[b].dof;
  *RotDoF = bodyDoF - 3 * me->nbodies;
  *DoF = 3 * me->nfree + bodyDoF - 3;
  check_actual_interactions(me);
  int need = 0;
  for (int l = 0; l < me->nlayers; l++) need |= me->coul[l].requires_kspace;
  if (need != me->kspace_active) {
    if (me->kspace_active) me->kspace_active = 0;
    else error("system initialization", "a kspace solver is required, but has not been defined");
  }
  if (me->kspace_active) {   /* src/EmDeeData.f90:384-412 */
    double kspaceRc = 0.0;
    int found = 0;
    for (int l = 1; l <= me->nlayers; l++)
      if (me->coul[l - 1].requires_kspace) {
        double lrc = layer_rc(me, l);
        if (!found) kspaceRc = lrc;
        else if (lrc != kspaceRc)
          error("system initialization", "all layers with ewald-like coulomb models must have the same cutoff");
        found = 1;
      }
    memset(&me->ewald, 0, sizeof(me->ewald));
    me->ewald.accuracy = me->kspace.accuracy;
    ewald_initialize(&me->ewald, kspaceRc, *me->Lbox, me->natoms, me->atomType, me->charge, me->R, me->nbodies,
                     me->body, me->nlayers, pair_kcoul, me);
    for (int l = 0; l < me->nlayers; l++)
      if (me->coul[l].requires_kspace) coul_kspace_setup(&me->coul[l], me->ewald.alpha);
  }
  me->initialized = 1;
}

static void initialize_system(tEmDee* md) {   /* src/EmDeeCode.f90:916-923 */
  odata* me = get(*md);
  perform_initialization(me, &md->DoF, &md->RotDoF);
  for (int layer = me->nlayers; layer >= 1; layer--) {
    EmDee_switch_model_layer(md, layer);
    EmDee_compute_forces(md);
  }
}

static void mark_stale(odata* me, tEmDee* md) {
  for (int l = 0; l < me->nlayers; l++) {
    me->forcesUpToDate[l] = 0;
    me->layerEnergy[l].UpToDate = false;
  }
  md->Energy.UpToDate = false;
}

/* src/EmDeeCode.f90:805-925 */
void EmDee_upload(tEmDee* md, char* option, double* address) {
  odata* me = get(*md);
  char item[257];
  option_string(option, item);
  if (!address) error("upload", "provided address is invalid");
  size_t n3 = (size_t)3 * me->natoms;
  if (!strcmp(item, "box")) {
    if (!me->Lbox) me->Lbox = (double*)xmalloc(sizeof(double));
    *me->Lbox = *address;
    if (me->initialized) mark_stale(me, md);
    else if (me->R) initialize_system(md);
  } else if (!strcmp(item, "coordinates")) {
    if (!me->R) me->R = (double*)xmalloc(sizeof(double) * n3);
    memcpy(me->R, address, sizeof(double) * n3);
    if (me->initialized) {
      mark_stale(me, md);
      if (md->Options.AutoBodyUpdate) update_rigid_bodies(me);
    } else if (me->Lbox) {
      initialize_system(md);
    }
  } else if (!strcmp(item, "momenta")) {
    if (!me->initialized) error("upload", "box and coordinates have not been defined");
    double t2[3] = {0, 0, 0}, r2[3] = {0, 0, 0};   /* src/EmDeeData.f90:157-189 */
    for (int j = 0; j < me->nfree; j++) {
      int i = me->freeAtom[j] - 1;
      for (int d = 0; d < 3; d++) {
        me->P[3 * i + d] = address[3 * i + d];
        t2[d] += me->invMass[i] * (address[3 * i + d] * address[3 * i + d]);
      }
    }
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      double Lm[3] = {0, 0, 0}, v[3], pi[4];
      for (int d = 0; d < 3; d++) B->pcm[d] = 0.0;
      for (int k = 0; k < B->NP; k++) {
        const double* Pj = &address[3 * (B->index[k] - 1)];
        double c[3];
        for (int d = 0; d < 3; d++) B->pcm[d] += Pj[d];
        cross3(&B->delta[3 * k], Pj, c);
        for (int d = 0; d < 3; d++) Lm[d] += c[d];
      }
      for (int d = 0; d < 3; d++) {
        t2[d] += B->invMass * (B->pcm[d] * B->pcm[d]);
        v[d] = 2.0 * Lm[d];
      }
      matC(B->q, v, pi);
      body_assign_pi(B, pi);
      for (int d = 0; d < 3; d++) r2[d] += B->MoI[d] * (B->omega[d] * B->omega[d]);
    }
    for (int d = 0; d < 3; d++) {
      md->Kinetic.RotPart[d] = 0.5 * r2[d];
      md->Kinetic.TransPart[d] = 0.5 * t2[d];
    }
    md->Kinetic.Rotational = md->Kinetic.RotPart[0] + md->Kinetic.RotPart[1] + md->Kinetic.RotPart[2];
    md->Kinetic.Total = md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] +
                        md->Kinetic.Rotational;
    md->Kinetic.ShadowKinetic = md->Kinetic.Total;
    md->Kinetic.ShadowRotational = md->Kinetic.Rotational;
    md->Kinetic.UpToDate = true;
  } else if (!strcmp(item, "forces")) {
    if (!me->initialized) error("upload", "box and coordinates have not been defined");
    memcpy(me->F, address, sizeof(double) * n3);
  } else if (!strcmp(item, "charges")) {
    if (me->initialized) error("upload", "cannot set charges after box and coordinates initialization");
    for (int i = 0; i < me->natoms; i++) {
      me->charge[i] = address[i];
      me->charged[i] = fabs(address[i]) > 2.220446049250313e-16;
    }
    mark_stale(me, md);
  } else {
    error("upload", "invalid option");
  }
}

/* src/EmDeeCode.f90:659-801 (free-atom options) */
void EmDee_download(tEmDee md, char* option, double* address) {
  odata* me = get(md);
  char item[257];
  option_string(option, item);
  if (!address) error("download", "provided address is invalid");
  size_t n3 = (size_t)3 * me->natoms;
  if (!strcmp(item, "box")) {
    *address = *me->Lbox;
  } else if (!strcmp(item, "coordinates")) {
    if (!me->R) error("download", "coordinates have not been allocated");
    memcpy(address, me->R, sizeof(double) * n3);
  } else if (!strcmp(item, "momenta")) {
    for (int j = 0; j < me->nfree; j++)
      for (int d = 0; d < 3; d++) address[3 * (me->freeAtom[j] - 1) + d] = me->P[3 * (me->freeAtom[j] - 1) + d];
    for (int b = 0; b < me->nbodies; b++) particle_momenta(&me->body[b], address);
  } else if (!strcmp(item, "forces")) {
    if (!me->forcesUpToDate[me->layer - 1]) EmDee_compute_forces(&md);
    memcpy(address, me->F, sizeof(double) * n3);
  } else if (!strcmp(item, "centersOfMass")) {
    for (int b = 0; b < me->nbodies; b++)
      for (int d = 0; d < 3; d++) address[3 * b + d] = me->body[b].rcm[d];
    for (int j = 0; j < me->nfree; j++)
      for (int d = 0; d < 3; d++) address[3 * (me->nbodies + j) + d] = me->R[3 * (me->freeAtom[j] - 1) + d];
  } else if (!strcmp(item, "quaternions") || !strcmp(item, "quatmom") || !strcmp(item, "quattau")) {
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      if (!strcmp(item, "quaternions")) for (int d = 0; d < 4; d++) address[4 * b + d] = B->q[d];
      else if (!strcmp(item, "quatmom")) for (int d = 0; d < 4; d++) address[4 * b + d] = B->pi[d];
      else {
        double v[3] = {2.0 * B->tau[0], 2.0 * B->tau[1], 2.0 * B->tau[2]};
        matC(B->q, v, &address[4 * b]);
      }
    }
  } else if (!strcmp(item, "angmom") || !strcmp(item, "bodycoord") || !strcmp(item, "bodymom") ||
             !strcmp(item, "bodyforces") || !strcmp(item, "torques") || !strcmp(item, "inertia")) {
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      const double* v = !strcmp(item, "angmom") ? B->omega : !strcmp(item, "bodycoord") ? B->rcm :
                        !strcmp(item, "bodymom") ? B->pcm : !strcmp(item, "bodyforces") ? B->F :
                        !strcmp(item, "torques") ? B->tau : B->MoI;
      for (int d = 0; d < 3; d++) address[3 * b + d] = v[d];
    }
  } else {
    error("download", "invalid option");
  }
}

void* EmDee_memory_address(tEmDee md, char* option) {   /* src/EmDeeCode.f90:212-235 */
  odata* me = get(md);
  char item[257];
  option_string(option, item);
  if (!strcmp(item, "coordinates")) return me->R;
  if (!strcmp(item, "momenta")) return me->P;
  if (!strcmp(item, "forces")) return me->F;
  if (!strcmp(item, "layerForces")) return me->layerF;
  char msg[300];
  snprintf(msg, sizeof msg, "invalid option %s", item);
  error("memory address retrieving", msg);
  return NULL;
}

void EmDee_share_phase_space(tEmDee mdkeep, tEmDee* mdlose) {   /* src/EmDeeCode.f90:239-269 */
  const char* task = "phase space sharing";
  odata *keep = get(mdkeep), *lose = get(*mdlose);
  if (!(keep->initialized && lose->initialized)) error(task, "EmDee system 1 has not been initialized");
  if (keep->natoms != lose->natoms) error(task, "different numbers of atoms");
  for (int i = 0; i < keep->natoms; i++) {
    if (keep->atomType[i] != lose->atomType[i]) error(task, "atom types do not match");
    if (keep->mass[i] != lose->mass[i]) error(task, "atom masses do not match");
    if (keep->atomBody[i] != lose->atomBody[i]) error(task, "rigid bodies do not match");
  }
  lose->R = keep->R;
  lose->P = keep->P;
  lose->body = keep->body;   /* lose%body => keep%body (src/EmDeeCode.f90:261) */
  lose->Lbox = keep->Lbox;
  mdlose->Kinetic.Total = mdkeep.Kinetic.Total;
  for (int d = 0; d < 3; d++) {
    mdlose->Kinetic.TransPart[d] = mdkeep.Kinetic.TransPart[d];
    mdlose->Kinetic.RotPart[d] = mdkeep.Kinetic.RotPart[d];
  }
  mdlose->Kinetic.Rotational = mdkeep.Kinetic.Rotational;
}

/* ======================================================================== */
/* dynamics (src/EmDeeCode.f90:950-1103, src/EmDeeData.f90:823-922)           */
/* ======================================================================== */

/* src/EmDeeCode.f90:950-1020 */
void EmDee_random_momenta(tEmDee* md, double kT, bool adjust, int seed) {
  odata* me = get(*md);
  double twoKEt[3] = {0, 0, 0}, twoKEr[3] = {0, 0, 0};
  if (me->random.seeding_required) rng_setup(&me->random, seed);
  if (me->nbodies != 0) {
    if (!me->initialized) error("random_momenta", "coordinates have not defined");
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      double f = sqrt(B->mass * kT), w[3];
      double a0 = rng_normal(&me->random), a1 = rng_normal(&me->random), a2 = rng_normal(&me->random);
      B->pcm[0] = f * a0;
      B->pcm[1] = f * a1;
      B->pcm[2] = f * a2;
      double c0 = rng_normal(&me->random), c1 = rng_normal(&me->random), c2 = rng_normal(&me->random);
      w[0] = sqrt(B->invMoI[0] * kT) * c0;
      w[1] = sqrt(B->invMoI[1] * kT) * c1;
      w[2] = sqrt(B->invMoI[2] * kT) * c2;
      body_assign_omega(B, w);
      for (int d = 0; d < 3; d++) {
        twoKEt[d] += B->invMass * (B->pcm[d] * B->pcm[d]);
        twoKEr[d] += B->MoI[d] * (B->omega[d] * B->omega[d]);
      }
    }
  }
  for (int j = 0; j < me->nfree; j++) {
    int i = me->freeAtom[j] - 1;
    double s = sqrt(me->mass[i] * kT);
    double a = rng_normal(&me->random), b = rng_normal(&me->random), c = rng_normal(&me->random);
    me->P[3 * i] = s * a;
    me->P[3 * i + 1] = s * b;
    me->P[3 * i + 2] = s * c;
    for (int d = 0; d < 3; d++) twoKEt[d] += me->invMass[i] * (me->P[3 * i + d] * me->P[3 * i + d]);
  }
  if (adjust) {   /* src/EmDeeCode.f90:994-1018 */
    double vcm[3];
    int bodyDoF = 0;
    for (int b = 0; b < me->nbodies; b++) bodyDoF += me->body[b].dof;
    for (int d = 0; d < 3; d++) {
      double s = 0.0, sb = 0.0;
      for (int j = 0; j < me->nfree; j++) s += me->P[3 * (me->freeAtom[j] - 1) + d];
      for (int b = 0; b < me->nbodies; b++) sb += me->body[b].pcm[d];
      vcm[d] = (s + sb) / me->totalMass;
      twoKEt[d] = 0.0;
    }
    for (int j = 0; j < me->nfree; j++) {
      int i = me->freeAtom[j] - 1;
      for (int d = 0; d < 3; d++) {
        me->P[3 * i + d] = me->P[3 * i + d] - me->mass[i] * vcm[d];
        twoKEt[d] += me->invMass[i] * (me->P[3 * i + d] * me->P[3 * i + d]);
      }
    }
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      for (int d = 0; d < 3; d++) {
        B->pcm[d] = B->pcm[d] - B->mass * vcm[d];
        twoKEt[d] += B->invMass * (B->pcm[d] * B->pcm[d]);
      }
    }
    double sum = (twoKEt[0] + twoKEr[0]) + (twoKEt[1] + twoKEr[1]) + (twoKEt[2] + twoKEr[2]);
    double factor = sqrt((double)(3 * me->nfree + bodyDoF - 3) * kT / sum);
    for (int j = 0; j < me->nfree; j++)
      for (int d = 0; d < 3; d++) me->P[3 * (me->freeAtom[j] - 1) + d] *= factor;
    for (int b = 0; b < me->nbodies; b++) {
      obody* B = &me->body[b];
      double w[3] = {factor * B->omega[0], factor * B->omega[1], factor * B->omega[2]};
      for (int d = 0; d < 3; d++) B->pcm[d] = factor * B->pcm[d];
      body_assign_omega(B, w);
    }
    for (int d = 0; d < 3; d++) {
      twoKEt[d] = factor * factor * twoKEt[d];
      twoKEr[d] = factor * factor * twoKEr[d];
    }
  }
  for (int d = 0; d < 3; d++) {
    md->Kinetic.RotPart[d] = 0.5 * twoKEr[d];
    md->Kinetic.TransPart[d] = 0.5 * twoKEt[d];
  }
  md->Kinetic.Rotational = md->Kinetic.RotPart[0] + md->Kinetic.RotPart[1] + md->Kinetic.RotPart[2];
  md->Kinetic.Total = md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] +
                      md->Kinetic.Rotational;
  md->Kinetic.ShadowKinetic = md->Kinetic.Total;
  md->Kinetic.ShadowRotational = md->Kinetic.Rotational;
  md->Kinetic.UpToDate = true;
}

/* src/EmDeeCode.f90:1024-1065 with src/EmDeeData.f90:864-922 */
void EmDee_boost(tEmDee* md, double lambda, double alpha, double dt) {
  odata* me = get(*md);
  double CF = phi(alpha * dt) * dt, CP = 1.0 - alpha * CF;
  int nt = me->nthreads, compute = md->Options.Compute;
  int translate = md->Options.Translate, rotate = md->Options.Rotate;
  CF = lambda * CF;
  if (lambda != 0.0 && !me->forcesUpToDate[me->layer - 1]) EmDee_compute_forces(md);
  double* t2 = (double*)xcalloc((size_t)6 * nt, sizeof(double));
  const double* F = me->F;
#pragma omp parallel num_threads(nt)
  {
    int thread = omp_get_thread_num() + 1;
    int a1 = (thread - 1) * me->threadFreeAtoms + 1;
    int aN = thread * me->threadFreeAtoms < me->nfree ? thread * me->threadFreeAtoms : me->nfree;
    int b1 = (thread - 1) * me->threadBodies;
    int bN = thread * me->threadBodies < me->nbodies ? thread * me->threadBodies : me->nbodies;
    for (int b = b1; b < bN; b++) force_and_torque(&me->body[b], F);
    if (translate) {
      for (int b = b1; b < bN; b++)
        for (int d = 0; d < 3; d++) me->body[b].pcm[d] = CP * me->body[b].pcm[d] + CF * me->body[b].F[d];
      for (int q = a1; q <= aN; q++) {
        int j = me->freeAtom[q - 1] - 1;
        for (int d = 0; d < 3; d++) me->P[3 * j + d] = CP * me->P[3 * j + d] + CF * F[3 * j + d];
      }
    }
    if (rotate) {
      double Ctau = 2.0 * CF;
      for (int b = b1; b < bN; b++) {
        obody* B = &me->body[b];
        double v[3] = {Ctau * B->tau[0], Ctau * B->tau[1], Ctau * B->tau[2]}, c[4], pi[4];
        matC(B->q, v, c);
        for (int k = 0; k < 4; k++) pi[k] = CP * B->pi[k] + c[k];
        body_assign_pi(B, pi);
      }
    }
    if (compute) {   /* src/EmDeeData.f90:900-922 */
      double* tk = &t2[6 * (thread - 1)];
      if (translate) {
        for (int b = b1; b < bN; b++)
          for (int d = 0; d < 3; d++) tk[d] += me->body[b].invMass * (me->body[b].pcm[d] * me->body[b].pcm[d]);
        for (int q = a1; q <= aN; q++) {
          int j = me->freeAtom[q - 1] - 1;
          for (int d = 0; d < 3; d++) tk[d] += me->invMass[j] * (me->P[3 * j + d] * me->P[3 * j + d]);
        }
      }
      if (rotate)
        for (int b = b1; b < bN; b++)
          for (int d = 0; d < 3; d++) tk[3 + d] += me->body[b].MoI[d] * (me->body[b].omega[d] * me->body[b].omega[d]);
    }
  }
  if (compute) {
    if (translate)
      for (int d = 0; d < 3; d++) {
        double s = t2[d];
        for (int t = 1; t < nt; t++) s += t2[6 * t + d];
        md->Kinetic.TransPart[d] = 0.5 * s;
      }
    if (rotate) {
      for (int d = 0; d < 3; d++) {
        double s = t2[3 + d];
        for (int t = 1; t < nt; t++) s += t2[6 * t + 3 + d];
        md->Kinetic.RotPart[d] = 0.5 * s;
      }
      md->Kinetic.Rotational = md->Kinetic.RotPart[0] + md->Kinetic.RotPart[1] + md->Kinetic.RotPart[2];
    }
    md->Kinetic.Total = md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] +
                        md->Kinetic.Rotational;
  }
  md->Kinetic.UpToDate = compute;
  free(t2);
}

/* src/EmDeeCode.f90:1069-1103 with src/EmDeeData.f90:823-860 */
void EmDee_displace(tEmDee* md, double lambda, double alpha, double dt) {
  odata* me = get(*md);
  double CR, CP;
  int translate = md->Options.Translate, rotate = md->Options.Rotate, mode = md->Options.RotationMode;
  md->Time.Motion -= omp_get_wtime();
  if (alpha != 0.0) {
    CP = phi(alpha * dt) * dt;
    CR = 1.0 - alpha * CP;
    *me->Lbox = CR * *me->Lbox;
  } else {
    CP = dt;
    CR = 1.0;
  }
  CP = lambda * CP;
#pragma omp parallel num_threads(me->nthreads)
  {
    int thread = omp_get_thread_num() + 1;
    int a1 = (thread - 1) * me->threadFreeAtoms + 1;
    int aN = thread * me->threadFreeAtoms < me->nfree ? thread * me->threadFreeAtoms : me->nfree;
    int b1 = (thread - 1) * me->threadBodies;
    int bN = thread * me->threadBodies < me->nbodies ? thread * me->threadBodies : me->nbodies;
    if (translate) {
      for (int b = b1; b < bN; b++) {
        obody* B = &me->body[b];
        for (int d = 0; d < 3; d++) B->rcm[d] = CR * B->rcm[d] + CP * B->invMass * B->pcm[d];
      }
      for (int q = a1; q <= aN; q++) {
        int j = me->freeAtom[q - 1] - 1;
        for (int d = 0; d < 3; d++) me->R[3 * j + d] = CR * me->R[3 * j + d] + CP * me->P[3 * j + d] * me->invMass[j];
      }
    }
    if (rotate)
      for (int b = b1; b < bN; b++) {
        obody* B = &me->body[b];
        if (mode == 0) rotate_exact(B, dt);
        else rotate_no_squish(B, dt, mode);
        for (int k = 0; k < B->NP; k++)
          for (int d = 0; d < 3; d++) me->R[3 * (B->index[k] - 1) + d] = B->rcm[d] + B->delta[3 * k + d];
      }
  }
  mark_stale(me, md);
  md->Time.Motion += omp_get_wtime();
}

void EmDee_move(tEmDee* md, double lambda, double alpha, double dt) { EmDee_displace(md, lambda, alpha, dt); }

/* virtual_rotation of src/EmDeeCode.f90:1150-1163: a copy of the body takes
 * pi + C(q) dt tau and rotates freely for dt; returns the copy's quaternion */
static void virtual_rotation(const obody* b, double dt, int mode, double* qout) {
  obody c = *b;
  c.delta = (double*)xmalloc(sizeof(double) * 3 * (b->NP ? b->NP : 1));
  memcpy(c.delta, b->delta, sizeof(double) * 3 * b->NP);
  double v[3] = {dt * c.tau[0], dt * c.tau[1], dt * c.tau[2]}, t[4], pi[4];
  matC(c.q, v, t);
  for (int k = 0; k < 4; k++) pi[k] = c.pi[k] + t[k];
  body_assign_pi(&c, pi);
  if (mode != 0) rotate_no_squish(&c, dt, mode);
  else rotate_exact(&c, dt);
  for (int k = 0; k < 4; k++) qout[k] = c.q[k];
  free(c.delta);
}

/* boost(me, thread, one, dt_2, me%F, TRUE, TRUE) of src/EmDeeData.f90:864-896 */
static void verlet_boost(odata* me, double CF) {
  const double* F = me->F;
  for (int b = 0; b < me->nbodies; b++) {
    obody* B = &me->body[b];
    force_and_torque(B, F);
    for (int d = 0; d < 3; d++) B->pcm[d] = 1.0 * B->pcm[d] + CF * B->F[d];
    double Ctau = 2.0 * CF, v[3] = {Ctau * B->tau[0], Ctau * B->tau[1], Ctau * B->tau[2]}, c[4], pi[4];
    matC(B->q, v, c);
    for (int k = 0; k < 4; k++) pi[k] = 1.0 * B->pi[k] + c[k];
    body_assign_pi(B, pi);
  }
  for (int q = 0; q < me->nfree; q++) {
    int j = me->freeAtom[q] - 1;
    for (int d = 0; d < 3; d++) me->P[3 * j + d] = 1.0 * me->P[3 * j + d] + CF * F[3 * j + d];
  }
}

/* move(me, thread, one, dt, dt, TRUE, TRUE, mode) of src/EmDeeData.f90:823-860 */
static void verlet_move(odata* me, double dt, int mode) {
  for (int b = 0; b < me->nbodies; b++) {
    obody* B = &me->body[b];
    for (int d = 0; d < 3; d++) B->rcm[d] = 1.0 * B->rcm[d] + dt * B->invMass * B->pcm[d];
  }
  for (int q = 0; q < me->nfree; q++) {
    int j = me->freeAtom[q] - 1;
    for (int d = 0; d < 3; d++) me->R[3 * j + d] = 1.0 * me->R[3 * j + d] + dt * me->P[3 * j + d] * me->invMass[j];
  }
  for (int b = 0; b < me->nbodies; b++) {
    obody* B = &me->body[b];
    if (mode == 0) rotate_exact(B, dt);
    else rotate_no_squish(B, dt, mode);
    for (int k = 0; k < B->NP; k++)
      for (int d = 0; d < 3; d++) me->R[3 * (B->index[k] - 1) + d] = B->rcm[d] + B->delta[3 * k + d];
  }
}

/* src/EmDeeCode.f90:1107-1211 */
void EmDee_verlet_step(tEmDee* md, double dt) {
  odata* me = get(*md);
  const double dt_2 = 0.5 * dt;
  const int compute = md->Options.Compute, mode = md->Options.RotationMode;
  const int nb = me->nbodies, nf = me->nfree;
  double Us = 0.0, Ks_t = 0.0, Ks_r = 0.0;
  double* r0 = (double*)xmalloc(sizeof(double) * 3 * (nb ? nb : 1));
  double* q0 = (double*)xmalloc(sizeof(double) * 4 * (nb ? nb : 1));
  double* s0 = (double*)xmalloc(sizeof(double) * 3 * (nf ? nf : 1));
  /* pre_force */
  if (compute) {
    for (int b = 0; b < nb; b++) {
      obody* B = &me->body[b];
      double qv[4];
      for (int d = 0; d < 3; d++) r0[3 * b + d] = 2.5 * B->rcm[d] + dt_2 * B->invMass * (B->pcm[d] - dt_2 * B->F[d]);
      virtual_rotation(B, -dt, mode, qv);
      for (int k = 0; k < 4; k++) q0[4 * b + k] = 0.5 * qv[k] - 3.0 * B->q[k];
    }
    for (int q = 0; q < nf; q++) {
      int j = me->freeAtom[q] - 1;
      for (int d = 0; d < 3; d++)
        s0[3 * q + d] = 2.5 * me->R[3 * j + d] + dt_2 * me->invMass[j] * (me->P[3 * j + d] - dt_2 * me->F[3 * j + d]);
    }
  }
  verlet_boost(me, dt_2);
  verlet_move(me, dt, mode);
  EmDee_compute_forces(md);   /* unconditional, and other layers keep their flags, as in the reference */
  /* post_force */
  verlet_boost(me, dt_2);
  if (compute) {
    double tk[3] = {0.0, 0.0, 0.0}, rk[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < nb; b++)
      for (int d = 0; d < 3; d++) tk[d] += me->body[b].invMass * (me->body[b].pcm[d] * me->body[b].pcm[d]);
    for (int q = 0; q < nf; q++) {
      int j = me->freeAtom[q] - 1;
      for (int d = 0; d < 3; d++) tk[d] += me->invMass[j] * (me->P[3 * j + d] * me->P[3 * j + d]);
    }
    for (int b = 0; b < nb; b++)
      for (int d = 0; d < 3; d++) rk[d] += me->body[b].MoI[d] * (me->body[b].omega[d] * me->body[b].omega[d]);
    for (int b = 0; b < nb; b++) {
      obody* B = &me->body[b];
      double rdot[3], qdot[4], qv[4], dot = 0.0, t4[4], tb[3];
      for (int d = 0; d < 3; d++) {
        rdot[d] = 2.5 * B->rcm[d] + dt * B->invMass * (B->pcm[d] + dt_2 * B->F[d]) - r0[3 * b + d];
        Ks_t += rdot[d] * B->pcm[d];
      }
      virtual_rotation(B, dt, mode, qv);
      for (int k = 0; k < 4; k++) {
        qdot[k] = q0[4 * b + k] + 1.5 * B->q[k] + qv[k];
        dot += qdot[k] * B->q[k];
      }
      for (int k = 0; k < 4; k++) Ks_r += (qdot[k] - dot * B->q[k]) * B->pi[k];
      matC(B->q, B->tau, t4);   /* tau_b = Bt C tau */
      matBt(B->q, t4, tb);
      Us += B->invMass * (B->F[0] * B->F[0] + B->F[1] * B->F[1] + B->F[2] * B->F[2]) +
            (B->invMoI[0] * tb[0] * tb[0] + B->invMoI[1] * tb[1] * tb[1] + B->invMoI[2] * tb[2] * tb[2]);
    }
    for (int q = 0; q < nf; q++) {
      int j = me->freeAtom[q] - 1;
      const double* P = &me->P[3 * j];
      const double* F = &me->F[3 * j];
      for (int d = 0; d < 3; d++) {
        double rdot = 2.5 * me->R[3 * j + d] + dt * me->invMass[j] * (P[d] + dt_2 * F[d]) - s0[3 * q + d];
        Ks_t += rdot * P[d];
      }
      Us += me->invMass[j] * (F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
    }
    for (int d = 0; d < 3; d++) {
      md->Kinetic.TransPart[d] = 0.5 * tk[d];
      md->Kinetic.RotPart[d] = 0.5 * rk[d];
    }
    md->Kinetic.Rotational = md->Kinetic.RotPart[0] + md->Kinetic.RotPart[1] + md->Kinetic.RotPart[2];
    md->Kinetic.Total = md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] +
                        md->Kinetic.Rotational;
    md->Energy.ShadowPotential = md->Energy.ShadowPotential - dt * dt * Us / 24.0;
    md->Kinetic.ShadowRotational = Ks_r / (6.0 * dt);
    md->Kinetic.ShadowKinetic = (Ks_t + Ks_r) / (6.0 * dt);
  }
  md->Kinetic.UpToDate = compute;
  free(r0);
  free(q0);
  free(s0);
}

/* src/EmDeeCode.f90:1281-1395: pair histograms over the current neighbor lists */
void EmDee_rdf(tEmDee md, int bins, double Rc, int pairs, int itype[], int jtype[], double g[]) {
  const char* task = "radial distribution calculation";
  const double Pi4_3 = 4.188790204786391;
  odata* me = get(md);
  int nt = me->ntypes, maxtype = 0;
  for (int p = 0; p < pairs; p++) {
    if (!ranged(itype[p], nt) || !ranged(jtype[p], nt)) error(task, "at least one provided type index is out of range");
    if (itype[p] > maxtype) maxtype = itype[p];
    if (jtype[p] > maxtype) maxtype = jtype[p];
  }
  char* hasPair = (char*)xcalloc(nt + 1, 1);
  char* pairOn = (char*)xcalloc((size_t)(nt + 1) * (nt + 1), 1);
  for (int p = 0; p < pairs; p++) {
    hasPair[itype[p]] = hasPair[jtype[p]] = 1;
    pairOn[itype[p] * (nt + 1) + jtype[p]] = pairOn[jtype[p] * (nt + 1) + itype[p]] = 1;
  }
  int npt = symm1D(maxtype, maxtype);
  long* count = (long*)xcalloc((size_t)bins * npt, sizeof(long));
  double invL = 1.0 / *me->Lbox, invL2 = invL * invL;
  double* Rs = (double*)xmalloc(sizeof(double) * 3 * me->natoms);
  for (size_t q = 0; q < (size_t)3 * me->natoms; q++) Rs[q] = invL * me->R[q];
  double Rc2 = Rc * Rc * invL2, binsByRc = bins / (Rc * invL);
  for (int t = 0; t < me->nthreads; t++) {
    olist* nb = &me->neighbor[t];
    int* last = Rc < 1.0001 * me->InRc ? nb->middle : nb->last;
    for (int c = me->threadCellFirst[t]; c <= me->threadCellLast[t]; c++)
      for (int k = me->cellFirst[c - 1]; k <= me->cellLast[c - 1]; k++) {
        int i = me->cellItem[k - 1], ti = me->atomType[i - 1];
        if (!hasPair[ti]) continue;
        for (int m = nb->first[i - 1]; m <= last[i - 1]; m++) {
          int j = nb->item[m - 1], tj = me->atomType[j - 1];
          if (!pairOn[ti * (nt + 1) + tj]) continue;
          double r2 = 0.0;
          for (int d = 0; d < 3; d++) {
            double x = Rs[3 * (i - 1) + d] - Rs[3 * (j - 1) + d];
            x = x - anint(x);
            r2 += x * x;
          }
          if (r2 < Rc2) {
            int bin = (int)(sqrt(r2) * binsByRc);
            if (bin > bins - 1) bin = bins - 1;   /* rounding at r -> Rc; the reference would index past the end */
            count[(size_t)(symm1D(ti, tj) - 1) * bins + bin]++;
          }
        }
      }
  }
  for (int p = 0; p < pairs; p++) {
    int i = itype[p], j = jtype[p];
    long Ni = 0, Nj = 0;
    for (int a = 0; a < me->natoms; a++) {
      Ni += me->atomType[a] == i;
      Nj += me->atomType[a] == j;
    }
    for (int b = 1; b <= bins; b++) {
      double w = Rc * invL / bins;
      double rdf = (double)count[(size_t)(symm1D(i, j) - 1) * bins + b - 1] / (Pi4_3 * (w * w * w));
      rdf = rdf / (3 * b * (b - 1) + 1);
      g[(size_t)p * bins + b - 1] = (i == j ? 2.0 * rdf : rdf) / (double)(Ni * Nj);
    }
  }
  free(hasPair);
  free(pairOn);
  free(count);
  free(Rs);
}

/* pairs of the current neighbor lists, (min,max) 1-based, sorted */
static int cmp_pair(const void* a, const void* b) {
  const int *p = (const int*)a, *q = (const int*)b;
  if (p[0] != q[0]) return p[0] < q[0] ? -1 : 1;
  if (p[1] != q[1]) return p[1] < q[1] ? -1 : 1;
  return 0;
}

long EmDee_neighbor_pairs(tEmDee md, int* pairs, long capacity) {
  odata* me = get(md);
  long n = 0;
  for (int t = 0; t < me->nthreads; t++) n += me->neighbor[t].count;
  if (n > capacity) return -n;
  long k = 0;
  for (int t = 0; t < me->nthreads; t++) {
    olist* nb = &me->neighbor[t];
    for (int c = me->threadCellFirst[t]; c <= me->threadCellLast[t]; c++)
      for (int q = me->cellFirst[c - 1]; q <= me->cellLast[c - 1]; q++) {
        int i = me->cellItem[q - 1];
        for (int m = nb->first[i - 1]; m <= nb->last[i - 1]; m++) {
          int j = nb->item[m - 1];
          pairs[2 * k] = i < j ? i : j;
          pairs[2 * k + 1] = i < j ? j : i;
          k++;
        }
      }
  }
  qsort(pairs, (size_t)k, 2 * sizeof(int), cmp_pair);
  return k;
}

/* ------------------------------------------------------------------------ */
/* Oracle-only hook used to pin the shifted-square-smoothed golden triple:   */
/* the triple in test/test_pair_lj_shifted_smoothed.f90 was produced by a    */
/* version whose shift was -E(rc), so the test overrides eshift on the       */
/* (itype,jtype) pair of every layer after the model is set.                  */
/* ------------------------------------------------------------------------ */
void oracle_set_eshift(tEmDee md, int itype, int jtype, double eshift) {
  odata* me = get(md);
  for (int l = 0; l < me->nlayers; l++) {
    PAIR(me, itype - 1, jtype - 1, l).model.eshift = eshift;
    PAIR(me, jtype - 1, itype - 1, l).model.eshift = eshift;
  }
}

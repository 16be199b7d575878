// models.cpp -- model factories, modifiers, cut-off set-up and mixing rules
// (host side), plus the KISS/ziggurat generator.
//
// Follows src/modelClass.f90, src/modelClass_nonbonded.f90,
// src/modelClass_pair.f90, src/modelClass_coul.f90, src/pair_*.f90,
// src/coul_*.f90 and src/math.f90.  The set-up arithmetic evaluates the same
// templated model functions as the kernels (pairmath.cuh) in double.
#include <cmath>
#include <cstring>

#include "system.hpp"

namespace emdee {

static const double PI = 3.14159265358979324;   // src/global.f90:38

Model model_new(int cls, int kind, const char* name) {
  Model m;
  m.cls = cls;
  m.kind = kind;
  m.p.kind = kind;
  m.p.modifier = NONE;
  snprintf(m.name, sizeof m.name, "%s", name);
  return m;
}

Model lj_setup(double eps, double sig) {   // src/pair_lj_cut.f90:52-69
  Model m = model_new(MC_PAIR, MK_LJ_CUT, "lj_cut");
  m.epsilon = eps;
  m.sigma = sig;
  m.p.eps4 = 4.0 * eps;
  m.p.eps24 = 24.0 * eps;
  m.p.sigsq = sig * sig;
  return m;
}

Model softcore_setup(double eps, double sig, double lambda) {   // src/pair_softcore_cut.f90:58-82
  Model m = model_new(MC_PAIR, MK_SOFTCORE_CUT, "softcore_cut");
  m.epsilon = eps;
  m.sigma = sig;
  m.lambda = lambda;
  if (lambda < 0.0 || lambda > 1.0) fatal("pair_softcore_cut setup", "out-of-range parameter lambda");
  m.p.prefactor = 4.0 * eps * std::pow(lambda, 1.0);
  m.p.prefactor6 = 6.0 * m.p.prefactor;
  m.p.invSigSq = 1.0 / (sig * sig);
  m.p.shift = 0.5 * std::pow(1.0 - lambda, 1.0);
  return m;
}

static void* deliver(const Model& m) { return new Model(m); }

// src/modelClass_nonbonded.f90:245-296
void modifier_setup(Model& m, double cutoff) {
  NBParams<double>& p = m.p;
  double Ec = 0, Wc = 0, Es, Ws;
  p.fshift = 0.0;
  p.eshift = 0.0;
  p.Rm = cutoff - m.skin;
  m.RmSq = p.Rm * p.Rm;
  bool shifting = p.modifier == SHIFTED || p.modifier == SHIFTED_FORCE || p.modifier == SHIFTED_SMOOTHED ||
                  p.modifier == SHIFTED_SQUARE_SMOOTHED;
  if (shifting) nb_compute(p, Ec, Wc, 1.0 / cutoff, 1.0 / (cutoff * cutoff));
  switch (p.modifier) {
    case SHIFTED: p.eshift = -Ec; break;
    case SHIFTED_FORCE:
      p.eshift = -(Ec + Wc);
      p.fshift = Wc / cutoff;
      break;
    case SMOOTHED:
    case SHIFTED_SMOOTHED:
      if (shifting) {
        nb_compute(p, Es, Ws, 1.0 / p.Rm, 1.0 / m.RmSq);
        p.eshift = -0.5 * (Es + Ec);
      }
      p.factor = 1.0 / (cutoff - p.Rm);
      p.Rm2fac = p.factor * p.Rm;
      break;
    case SQUARE_SMOOTHED:
    case SHIFTED_SQUARE_SMOOTHED:
      if (shifting) {
        nb_compute(p, Es, Ws, 1.0 / p.Rm, 1.0 / m.RmSq);
        p.eshift = -0.5 * (Es + Ec);
      }
      p.factor = 1.0 / (cutoff * cutoff - m.RmSq);
      p.Rm2fac = p.factor * m.RmSq;
      break;
    default: break;
  }
}

// apply_cutoff of the smoothed Coulomb models
static void apply_cutoff(Model& m, double Rc) {
  NBParams<double>& p = m.p;
  switch (m.kind) {
    case MK_COUL_DAMPED_SMOOTHED:   // src/coul_damped_smoothed.f90:70-80
      p.Rm = Rc - m.skinWidth;
      p.Rm2 = p.Rm * p.Rm;
      p.invRm = 1.0 / p.Rm;
      p.factor = 1.0 / (Rc - p.Rm);
      break;
    case MK_COUL_DAMPED_SQUARE_SMOOTHED:   // src/coul_damped_square_smoothed.f90:70-79
    case MK_COUL_SQUARE_SMOOTHED:
    case MK_COUL_SHIFTED_SQUARE_SMOOTHED:
      p.Rm2 = (Rc - m.skinWidth) * (Rc - m.skinWidth);
      p.invRm = 1.0 / (Rc - m.skinWidth);
      p.factor = 1.0 / (Rc * Rc - p.Rm2);
      break;
    default: break;
  }
}

// src/modelClass_coul.f90:62-93
void cutoff_setup(Model& m, double cutoff) {
  NBParams<double>& p = m.p;
  p.fshift = 0.0;
  p.eshift = 0.0;
  if (m.shifted || m.shifted_force) {
    double invR = 1.0 / cutoff, E, W;
    nb_compute(p, E, W, invR, invR * invR);
    if (m.shifted_force) {
      p.fshift = W / cutoff;
      p.eshift = -(E + W);
    } else {
      p.fshift = 0.0;
      p.eshift = -E;
    }
  }
  apply_cutoff(m, cutoff);
}

// model%mix (src/pair_lj_cut.f90:122-138, src/pair_softcore_cut.f90:139-163,
// src/modelClass_pair.f90:198-208); false when no rule exists
static bool model_mix(const Model& self, const Model& other, Model& out) {
  switch (self.kind) {
    case MK_PAIR_NONE: out = model_new(MC_PAIR, MK_PAIR_NONE, "none"); return true;
    case MK_LJ_CUT:
      if (other.kind == MK_LJ_CUT) {
        out = lj_setup(std::sqrt(self.epsilon * other.epsilon), 0.5 * (self.sigma + other.sigma));
        return true;
      }
      return false;
    case MK_SOFTCORE_CUT:
      if (other.kind == MK_SOFTCORE_CUT) {
        out = softcore_setup(std::sqrt(self.epsilon * other.epsilon), 0.5 * (self.sigma + other.sigma),
                             self.lambda * other.lambda);
        return true;
      }
      if (other.kind == MK_LJ_CUT) {
        out = softcore_setup(std::sqrt(self.epsilon * other.epsilon), 0.5 * (self.sigma + other.sigma),
                             self.lambda);
        return true;
      }
      return false;
    default: return false;
  }
}

// src/modelClass_pair.f90:120-140
PairHost pair_container_mix(const PairHost& a, const PairHost& b) {
  PairHost c;
  if (!model_mix(b.model, a.model, c.model) && !model_mix(a.model, b.model, c.model)) {
    char msg[128];
    c.model = model_new(MC_PAIR, MK_PAIR_NONE, "none");
    snprintf(msg, sizeof msg, "no mixing rule found for models %s and %s", a.model.name, b.model.name);
    warn(msg);
  }
  c.coulomb = a.coulomb && b.coulomb;
  if (c.coulomb) c.kCoul = std::sqrt(a.kCoul * b.kCoul);
  return c;
}

// ---- KISS + ziggurat ----------------------------------------------------------

static uint32_t kiss_m(uint32_t k, int n) { return k ^ (n >= 0 ? (k << n) : (k >> (-n))); }

// src/math.f90:80-105 and 150-162
void Kiss::setup(int32_t seed) {
  const double m1 = 2147483648.0;
  x = kiss_m(kiss_m(kiss_m((uint32_t)seed, 13), -17), 5);
  y = kiss_m(kiss_m(kiss_m(x, 13), -17), 5);
  z = kiss_m(kiss_m(kiss_m(y, 13), -17), 5);
  w = kiss_m(kiss_m(kiss_m(z, 13), -17), 5);
  seeding_required = false;
  double dn = 3.442619855899, tn = dn, vn = 0.00991256303526217;
  double q = vn * std::exp(0.5 * dn * dn);
  kn[0] = (int32_t)((dn / q) * m1);
  kn[1] = 0;
  wn[0] = q / m1;
  wn[127] = dn / m1;
  fn[0] = 1.0;
  fn[127] = std::exp(-0.5 * dn * dn);
  for (int i = 126; i >= 1; i--) {
    dn = std::sqrt(-2.0 * std::log(vn / dn + std::exp(-0.5 * dn * dn)));
    kn[i + 1] = (int32_t)((dn / tn) * m1);
    tn = dn;
    fn[i] = std::exp(-0.5 * dn * dn);
    wn[i] = dn / m1;
  }
}

// src/math.f90:166-177 (32-bit wraparound, logical shifts)
int32_t Kiss::i32() {
  x = 69069u * x + 1327217885u;
  y ^= y << 13;
  y ^= y >> 17;
  y ^= y << 5;
  z = 18000u * (z & 65535u) + (z >> 16);
  w = 30903u * (w & 65535u) + (w >> 16);
  return (int32_t)(x + y + (z << 16) + w);
}

static inline int32_t iabs32(int32_t v) { return v == INT32_MIN ? INT32_MIN : (v < 0 ? -v : v); }

// Marsaglia-Tsang ziggurat, src/math.f90:109-146
double Kiss::normal() {
  const double r = 3.442620, s = 0.2328306e-9;
  int32_t hz = i32(), iz = hz & 127;
  double xx, yy;
  if (iabs32(hz) < kn[iz]) return (double)hz * wn[iz];
  for (;;) {
    if (iz == 0) {
      for (;;) {
        xx = -0.2904764 * std::log(s * (double)i32() + 0.5);
        yy = -std::log(s * (double)i32() + 0.5);
        if (yy + yy >= xx * xx) break;
      }
      return hz <= 0 ? -(r + xx) : r + xx;
    }
    xx = (double)hz * wn[iz];
    if (fn[iz] + (s * (double)i32() + 0.5) * (fn[iz - 1] - fn[iz]) < std::exp(-0.5 * xx * xx)) return xx;
    hz = i32();
    iz = hz & 127;
    if (iabs32(hz) < kn[iz]) return (double)hz * wn[iz];
  }
}

}  // namespace emdee

using namespace emdee;

// ---- C ABI: model factories and modifiers -----------------------------------------

extern "C" {

void* EmDee_pair_none(void) { return deliver(model_new(MC_PAIR, MK_PAIR_NONE, "none")); }
void* EmDee_coul_none(void) { return deliver(model_new(MC_COUL, MK_COUL_NONE, "none")); }
void* EmDee_bond_none(void) { return deliver(model_new(MC_BOND, MK_BOND_NONE, "none")); }
void* EmDee_angle_none(void) { return deliver(model_new(MC_ANGLE, MK_ANGLE_NONE, "none")); }
void* EmDee_dihedral_none(void) { return deliver(model_new(MC_DIHEDRAL, MK_DIHEDRAL_NONE, "none")); }

void* EmDee_pair_lj_cut(double epsilon, double sigma) { return deliver(lj_setup(epsilon, sigma)); }

void* EmDee_pair_softcore_cut(double epsilon, double sigma, double lambda) {
  return deliver(softcore_setup(epsilon, sigma, lambda));
}

void* EmDee_coul_cut(void) { return deliver(model_new(MC_COUL, MK_COUL_CUT, "cut")); }

void* EmDee_coul_sf(void) {   // src/coul_sf.f90:37-50
  Model m = model_new(MC_COUL, MK_COUL_SF, "sf");
  m.shifted_force = 1;
  return deliver(m);
}

static Model damped(int kind, const char* name, double damp, double skinWidth) {
  Model m = model_new(MC_COUL, kind, name);
  m.damp = damp;
  m.skinWidth = skinWidth;
  m.p.alpha = damp;
  m.p.beta = 2.0 * damp / std::sqrt(PI);
  return m;
}

void* EmDee_coul_damped(double damp) { return deliver(damped(MK_COUL_DAMPED, "damped", damp, 0.0)); }

void* EmDee_coul_damped_smoothed(double damp, double skinWidth) {
  return deliver(damped(MK_COUL_DAMPED_SMOOTHED, "damped_openmm_smoothed", damp, skinWidth));
}

void* EmDee_coul_damped_square_smoothed(double damp, double skinWidth) {
  return deliver(damped(MK_COUL_DAMPED_SQUARE_SMOOTHED, "damped_smoothed", damp, skinWidth));
}

void* EmDee_coul_square_smoothed(double skinWidth) {
  Model m = model_new(MC_COUL, MK_COUL_SQUARE_SMOOTHED, "smoothed");
  m.skinWidth = skinWidth;
  return deliver(m);
}

void* EmDee_coul_shifted_square_smoothed(double skinWidth) {
  Model m = model_new(MC_COUL, MK_COUL_SHIFTED_SQUARE_SMOOTHED, "shifted_smoothed");
  m.skinWidth = skinWidth;
  m.shifted = 1;
  return deliver(m);
}

void* EmDee_coul_long(void) {
  Model m = model_new(MC_COUL, MK_COUL_LONG, "long");
  m.requires_kspace = 1;
  return deliver(m);
}

void* EmDee_kspace_ewald(double accuracy) {
  Model m = model_new(MC_KSPACE, MK_KSPACE_EWALD, "ewald");
  m.accuracy = accuracy;
  return deliver(m);
}

void* EmDee_bond_harmonic(double k, double r0) {
  Model m = model_new(MC_BOND, MK_BOND_HARMONIC, "harmonic");
  m.k = k;
  m.x0 = r0;
  return deliver(m);
}

void* EmDee_angle_harmonic(double k, double theta0) {
  Model m = model_new(MC_ANGLE, MK_ANGLE_HARMONIC, "harmonic");
  m.k = k;
  m.x0 = theta0;
  return deliver(m);
}

static void* modified(void* model, int modifier, double skin, bool set_skin, const char* task) {
  if (!model) fatal(task, "a valid pair model must be provided");
  Model m = *(Model*)model;
  if (m.cls != MC_PAIR && m.cls != MC_COUL) fatal(task, "a valid pair model must be provided");
  m.p.modifier = modifier;
  if (set_skin) m.skin = skin;
  return deliver(m);
}

// src/modelClass_nonbonded.f90:83-241
void* EmDee_shifted(void* model) { return modified(model, SHIFTED, 0, false, "shifted potential assignment"); }
void* EmDee_shifted_force(void* model) {
  return modified(model, SHIFTED_FORCE, 0, false, "shifted-force potential assignment");
}
void* EmDee_smoothed(void* model, double skin) {
  return modified(model, SMOOTHED, skin, true, "smoothed potential assignment");
}
void* EmDee_shifted_smoothed(void* model, double skin) {
  return modified(model, SHIFTED_SMOOTHED, skin, true, "shifted-smoothed potential assignment");
}
void* EmDee_square_smoothed(void* model, double skin) {
  return modified(model, SQUARE_SMOOTHED, skin, true, "square-smoothed potential assignment");
}
void* EmDee_shifted_square_smoothed(void* model, double skin) {
  return modified(model, SHIFTED_SQUARE_SMOOTHED, skin, true, "shifted-square-smoothed potential assignment");
}

}  // extern "C"

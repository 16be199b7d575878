// rigid.cuh -- rigid-body (ArBee) arithmetic, FP64, usable on the host (body
// set-up) and on the device (per-body kernels).
//
// Follows src/ArBee.f90: principal frame and quaternion (97-134), quaternion
// matrices B and C (138-176), NO_SQUISH rotation (180-221), exact free rotation
// (225-324, the van Zon-Schofield solution with Carlson's elliptic integrals and
// Jacobi elliptic functions), particle momenta (328-336), force and torque
// (340-352), momentum assignment (356-366).  The symmetric 3x3 eigen-solver is
// cyclic Jacobi rotation with the contract the body code relies on: eigenvalues
// in decreasing order, right-handed frame.  The quaternion of a rotation matrix
// uses Shepperd's method (J. Guidance and Control 1, 223, 1978).
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define RB_HD __host__ __device__ __forceinline__
#define RB_HDN __host__ __device__
#else
#define RB_HD inline
#define RB_HDN
#endif

namespace emdee {

// per-body state; atoms of body b are index[first .. first+NP) (0-based), with
// masses M, body-frame coordinates d and space-frame offsets delta (3 per atom)
struct BodyState {
  int NP, first, dof;
  double mass, invMass;
  double MoI[3], invMoI[3], rcm[3], pcm[3], q[4], pi[4], omega[3], F[3], tau[3];
  double I113, I313, I223, I212, m312;
};

RB_HD void rb_cross(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// B(q) v, C(q) v (4-vectors from 3-vectors) and B(q)^T v, C(q)^T v
RB_HD void rb_B(const double* q, const double* v, double* o) {
  o[0] = -q[1] * v[0] - q[2] * v[1] - q[3] * v[2];
  o[1] = q[0] * v[0] - q[3] * v[1] + q[2] * v[2];
  o[2] = q[3] * v[0] + q[0] * v[1] - q[1] * v[2];
  o[3] = -q[2] * v[0] + q[1] * v[1] + q[0] * v[2];
}
RB_HD void rb_C(const double* q, const double* v, double* o) {
  o[0] = -q[1] * v[0] - q[2] * v[1] - q[3] * v[2];
  o[1] = q[0] * v[0] + q[3] * v[1] - q[2] * v[2];
  o[2] = -q[3] * v[0] + q[0] * v[1] + q[1] * v[2];
  o[3] = q[2] * v[0] - q[1] * v[1] + q[0] * v[2];
}
RB_HD void rb_Bt(const double* q, const double* v, double* o) {
  o[0] = -q[1] * v[0] + q[0] * v[1] + q[3] * v[2] - q[2] * v[3];
  o[1] = -q[2] * v[0] - q[3] * v[1] + q[0] * v[2] + q[1] * v[3];
  o[2] = -q[3] * v[0] + q[2] * v[1] - q[1] * v[2] + q[0] * v[3];
}
RB_HD void rb_Ct(const double* q, const double* v, double* o) {
  o[0] = -q[1] * v[0] + q[0] * v[1] - q[3] * v[2] + q[2] * v[3];
  o[1] = -q[2] * v[0] + q[3] * v[1] + q[0] * v[2] - q[1] * v[3];
  o[2] = -q[3] * v[0] - q[2] * v[1] + q[1] * v[2] + q[0] * v[3];
}

RB_HD void rb_assign_omega(BodyState& b, const double* w) {
  double v[3];
  for (int k = 0; k < 3; k++) {
    b.omega[k] = w[k];
    v[k] = 2.0 * b.MoI[k] * w[k];
  }
  rb_B(b.q, v, b.pi);
}

RB_HD void rb_assign_pi(BodyState& b, const double* pi) {
  double v[3];
  for (int k = 0; k < 4; k++) b.pi[k] = pi[k];
  rb_Bt(b.q, b.pi, v);
  for (int k = 0; k < 3; k++) b.omega[k] = 0.5 * b.invMoI[k] * v[k];
}

// delta = C(q)^T B(q) d for the body's atoms
RB_HD void rb_space_coords(const BodyState& b, const double* d, double* delta) {
  if (!delta) return;   // orientation only (virtual rotations)
  for (int k = 0; k < b.NP; k++) {
    double t[4];
    rb_B(b.q, &d[3 * k], t);
    rb_Ct(b.q, t, &delta[3 * k]);
  }
}

RB_HD void rb_rotate_uniaxial(BodyState& b, int k, double dt) {
  double BkQ[4], BkPi[4];
  const double *q = b.q, *p = b.pi;
  if (k == 1) {
    BkQ[0] = -q[1]; BkQ[1] = q[0]; BkQ[2] = q[3]; BkQ[3] = -q[2];
    BkPi[0] = -p[1]; BkPi[1] = p[0]; BkPi[2] = p[3]; BkPi[3] = -p[2];
  } else if (k == 2) {
    BkQ[0] = -q[2]; BkQ[1] = -q[3]; BkQ[2] = q[0]; BkQ[3] = q[1];
    BkPi[0] = -p[2]; BkPi[1] = -p[3]; BkPi[2] = p[0]; BkPi[3] = p[1];
  } else {
    BkQ[0] = -q[3]; BkQ[1] = q[2]; BkQ[2] = -q[1]; BkQ[3] = q[0];
    BkPi[0] = -p[3]; BkPi[1] = p[2]; BkPi[2] = -p[1]; BkPi[3] = p[0];
  }
  double dot = p[0] * BkQ[0] + p[1] * BkQ[1] + p[2] * BkQ[2] + p[3] * BkQ[3];
  double a = dt * dot / (4.0 * b.MoI[k - 1]);
  double vs = sin(a), vc = cos(a);
  for (int i = 0; i < 4; i++) {
    b.q[i] = vc * b.q[i] + vs * BkQ[i];
    b.pi[i] = vc * b.pi[i] + vs * BkPi[i];
  }
}

RB_HD void rb_rotate_no_squish(BodyState& b, double delta_t, int n, const double* d, double* delta) {
  double dt = delta_t / n, h = 0.5 * dt;
  for (int i = 0; i < n; i++) {
    rb_rotate_uniaxial(b, 3, h);
    rb_rotate_uniaxial(b, 2, h);
    rb_rotate_uniaxial(b, 1, dt);
    rb_rotate_uniaxial(b, 2, h);
    rb_rotate_uniaxial(b, 3, h);
  }
  rb_space_coords(b, d, delta);
}

// Carlson's duplication algorithms for RF, RC and RJ (relative tolerance 1e-3
// on the deviations, as in src/math.f90:505-638)
RB_HDN inline double rb_RF(double x, double y, double z) {
  double xn = x, yn = y, zn = z, mu, xd, yd, zd;
  for (;;) {
    mu = (xn + yn + zn) / 3.0;
    xd = 2.0 - (mu + xn) / mu;
    yd = 2.0 - (mu + yn) / mu;
    zd = 2.0 - (mu + zn) / mu;
    if (fmax(fabs(xd), fmax(fabs(yd), fabs(zd))) < 0.001) break;
    double xr = sqrt(xn), yr = sqrt(yn), zr = sqrt(zn), lam = xr * (yr + zr) + yr * zr;
    xn = (xn + lam) * 0.25;
    yn = (yn + lam) * 0.25;
    zn = (zn + lam) * 0.25;
  }
  const double c1 = 1.0 / 24.0, c2 = 3.0 / 44.0, c3 = 1.0 / 14.0;
  double e2 = xd * yd - zd * zd, e3 = xd * yd * zd;
  return (1.0 + (c1 * e2 - 0.1 - c2 * e3) * e2 + c3 * e3) / sqrt(mu);
}

RB_HDN inline double rb_RC(double x, double y) {
  double xn = x, yn = y, mu, sn;
  for (;;) {
    mu = (xn + yn + yn) / 3.0;
    sn = (yn + mu) / mu - 2.0;
    if (fabs(sn) < 0.001) break;
    double lam = 2.0 * sqrt(xn) * sqrt(yn) + yn;
    xn = (xn + lam) * 0.25;
    yn = (yn + lam) * 0.25;
  }
  const double c1 = 1.0 / 7.0, c2 = 9.0 / 22.0;
  return (1.0 + sn * sn * (0.3 + sn * (c1 + sn * (0.375 + sn * c2)))) / sqrt(mu);
}

RB_HDN inline double rb_RJ(double x, double y, double z, double p) {
  double xn = x, yn = y, zn = z, pn = p, sigma = 0.0, power4 = 1.0, mu, xd, yd, zd, pd;
  for (;;) {
    mu = (xn + yn + zn + pn + pn) * 0.2;
    xd = (mu - xn) / mu;
    yd = (mu - yn) / mu;
    zd = (mu - zn) / mu;
    pd = (mu - pn) / mu;
    if (fmax(fmax(fabs(xd), fabs(yd)), fmax(fabs(zd), fabs(pd))) < 0.001) break;
    double xr = sqrt(xn), yr = sqrt(yn), zr = sqrt(zn), lam = xr * (yr + zr) + yr * zr;
    double al = pn * (xr + yr + zr) + xr * yr * zr;
    al = al * al;
    double be = pn * (pn + lam) * (pn + lam);
    sigma += power4 * rb_RC(al, be);
    power4 *= 0.25;
    xn = (xn + lam) * 0.25;
    yn = (yn + lam) * 0.25;
    zn = (zn + lam) * 0.25;
    pn = (pn + lam) * 0.25;
  }
  const double c1 = 3.0 / 14.0, c2 = 1.0 / 3.0, c3 = 3.0 / 22.0, c4 = 3.0 / 26.0;
  double ea = xd * (yd + zd) + yd * zd, eb = xd * yd * zd, ec = pd * pd;
  double e2 = ea - 3.0 * ec, e3 = eb + 2.0 * pd * (ea - ec);
  double s1 = 1.0 + e2 * (-c1 + 0.75 * c3 * e2 - 1.5 * c4 * e3);
  double s2 = eb * (0.5 * c2 + pd * (-c3 - c3 + pd * c4));
  double s3 = pd * ea * (c2 - pd * c3) - c2 * pd * ec;
  return 3.0 * sigma + power4 * (s1 + s2 + s3) / (mu * sqrt(mu));
}

// Jacobi elliptic functions by the arithmetic-geometric mean (A&S 16.4)
RB_HDN inline void rb_jacobi(double u, double m, double& sn, double& cn, double& dn) {
  const double eps = 2.220446049250313e-16;
  if (fabs(m) < 2 * eps) {
    sn = sin(u); cn = cos(u); dn = 1.0;
    return;
  }
  if (fabs(m - 1.0) < 2 * eps) {
    sn = tanh(u); cn = dn = 1.0 / cosh(u);
    return;
  }
  double mu[16], nu[16], c[16], d[16];
  int n = 0;
  mu[0] = 1.0;
  nu[0] = sqrt(1.0 - m);
  while (fabs(mu[n] - nu[n]) > 4.0 * eps * fabs(mu[n] + nu[n]) && n < 15) {
    mu[n + 1] = 0.5 * (mu[n] + nu[n]);
    nu[n + 1] = sqrt(mu[n] * nu[n]);
    n++;
  }
  double su = sin(u * mu[n]), cu = cos(u * mu[n]);
  bool smallSin = fabs(su) < fabs(cu);
  c[n] = mu[n] * (smallSin ? su / cu : cu / su);
  d[n] = 1.0;
  while (n > 0) {
    c[n - 1] = d[n] * c[n];
    double r = c[n] * c[n] / mu[n];
    n--;
    d[n] = (r + nu[n]) / (r + mu[n]);
  }
  if (smallSin) {
    dn = sqrt(1.0 - m) / d[0];
    cn = dn * (cu < 0 ? -1.0 : 1.0) / hypot(1.0, c[0]);
    sn = cn * c[0] / sqrt(1.0 - m);
  } else {
    dn = d[0];
    sn = (su < 0 ? -1.0 : 1.0) / hypot(1.0, c[0]);
    cn = c[0] * sn;
  }
}

RB_HD int rb_staircase(double x) { return x > 0 ? (int)ceil(x - 0.5) : (int)floor(x + 0.5); }
RB_HD double rb_sign(double a, double b) { return b >= 0 ? fabs(a) : -fabs(a); }

RB_HD double rb_Theta(double x, double n, double m) {
  double x2 = x * x;
  return -(1.0 / 3.0) * n * x * x2 * rb_RJ(1.0 - x2, 1.0 - m * x2, 1.0, 1.0 + n * x2);
}

// exact free rotation over dt (src/ArBee.f90:225-324)
RB_HDN inline void rb_rotate_exact(BodyState& b, double dt, const double* d, double* delta) {
  const double PI = 3.14159265358979324;
  double w0[3] = {b.omega[0], b.omega[1], b.omega[2]}, Iw[3];
  for (int k = 0; k < 3; k++) Iw[k] = b.MoI[k] * w0[k];
  double Lsq = Iw[1] * Iw[1] + Iw[2] * Iw[2];
  if (Lsq < 2.220446049250313e-16) {
    rb_rotate_uniaxial(b, 1, dt);
    return;
  }
  Lsq = Iw[0] * Iw[0] + Lsq;
  double L = sqrt(Lsq);
  double TwoKr = Iw[0] * w0[0] + Iw[1] * w0[1] + Iw[2] * w0[2];
  double r1 = Lsq - TwoKr * b.MoI[2], r3 = TwoKr * b.MoI[0] - Lsq;
  double l1 = b.I223 * r1, l3 = b.I212 * r3, lmin = fmin(l1, l3);
  double a[3] = {rb_sign(1.0, w0[0]) * sqrt(b.I113 * r1), sqrt(lmin), rb_sign(1.0, w0[2]) * sqrt(b.I313 * r3)};
  double m = lmin / fmax(l1, l3);
  double K = rb_RF(0.0, 1.0 - m, 1.0), inv2K = 0.5 / K;
  double s0 = w0[1] / a[1], c0, u0;
  int i0;
  if (fabs(s0) < 1.0) {
    c0 = l1 < l3 ? w0[0] / a[0] : w0[2] / a[2];
    u0 = s0 * rb_RF(1.0 - s0 * s0, 1.0 - m * s0 * s0, 1.0);
    i0 = rb_staircase(u0 * inv2K);
  } else {
    a[1] = fabs(w0[1]);
    s0 = rb_sign(1.0, s0);
    c0 = 0.0;
    u0 = rb_sign(K, s0);
    i0 = 0;
  }
  double wp = b.m312 * a[0] * a[2] / a[1];
  double u = wp * dt + u0;
  int jump = rb_staircase(u * inv2K) - i0;
  double sn, cn, dn, deltaF;
  rb_jacobi(u, m, sn, cn, dn);
  double alpha = b.MoI[0] * a[0] / L;
  // The two cases of src/ArBee.f90 (l1 < l3 or not) differ only in scalar set-up;
  // the elliptic integrals are evaluated by one common code path so that the
  // bodies of a warp do not run them twice (once per case) on the device.
  const double eta = alpha * alpha / (1.0 - alpha * alpha);
  double nTheta, C, y1, y0, extra;
  if (l1 < l3) {
    b.omega[0] = a[0] * cn; b.omega[1] = a[1] * sn; b.omega[2] = a[2] * dn;
    double d0 = w0[2] / a[2];
    nTheta = eta;
    C = sqrt(m + eta);
    y1 = C * sn / dn;
    y0 = C * s0 / d0;
    extra = 0.0;
  } else {
    b.omega[0] = a[0] * dn; b.omega[1] = a[1] * sn; b.omega[2] = a[2] * cn;
    nTheta = m * eta;
    C = sqrt(1.0 + nTheta);
    y1 = C * sn / cn;
    y0 = C * s0 / c0;
    extra = (alpha / C) * PI;
  }
  double r = u - u0 + rb_sign(1.0, cn) * rb_Theta(sn, nTheta, m) - rb_sign(1.0, c0) * rb_Theta(s0, nTheta, m) +
             (alpha / C) * (atan(y1) - atan(y0));
  if (jump != 0) {
    const double T1 = rb_Theta(1.0, nTheta, m);
    r += l1 < l3 ? jump * 2.0 * T1 : jump * (2.0 * T1 + extra);
  }
  deltaF = (eta + 1.0) * r;
  double phi = (Lsq * (u - u0) + r3 * deltaF) / (2.0 * L * b.MoI[0] * wp);
  double z0[4] = {Iw[2], Iw[1], L - Iw[0], 0.0};
  for (int k = 0; k < 3; k++) Iw[k] = b.MoI[k] * b.omega[k];
  double cp = cos(phi), sp = sin(phi), z[4];
  z[0] = Iw[2] * cp - Iw[1] * sp;
  z[1] = Iw[1] * cp + Iw[2] * sp;
  z[2] = (L - Iw[0]) * cp;
  z[3] = (L - Iw[0]) * sp;
  double dotz = z0[0] * b.q[0] + z0[1] * b.q[1] + z0[2] * b.q[2] + z0[3] * b.q[3], t[3], nq[4];
  rb_Ct(z0, b.q, t);
  rb_C(z, t, nq);
  double norm = 0.0;
  for (int k = 0; k < 4; k++) {
    nq[k] = z[k] * dotz + nq[k];
    norm += nq[k] * nq[k];
  }
  norm = sqrt(norm);
  for (int k = 0; k < 4; k++) b.q[k] = nq[k] / norm;
  double v[3] = {2.0 * Iw[0], 2.0 * Iw[1], 2.0 * Iw[2]};
  rb_B(b.q, v, b.pi);
  rb_space_coords(b, d, delta);
}

// ---- host set-up -----------------------------------------------------------------

// symmetric 3x3 eigen-solver (cyclic Jacobi rotations); w decreasing, V columns
// = eigenvectors, right-handed, largest component of the first two positive
inline void rb_eigen_sym3(const double Ain[3][3], double V[3][3], double w[3]) {
  double A[3][3], Q[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = Ain[i][j];
  for (int sweep = 0; sweep < 64; sweep++) {
    if (A[0][1] == 0.0 && A[0][2] == 0.0 && A[1][2] == 0.0) break;
    for (int p = 0; p < 2; p++)
      for (int r = p + 1; r < 3; r++) {
        if (std::fabs(A[p][r]) <= 1e-18 * (std::fabs(A[p][p]) + std::fabs(A[r][r]))) {
          A[p][r] = A[r][p] = 0.0;
          continue;
        }
        double theta = (A[r][r] - A[p][p]) / (2.0 * A[p][r]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {
          double akp = A[k][p], akr = A[k][r];
          A[k][p] = c * akp - s * akr;
          A[k][r] = s * akp + c * akr;
        }
        for (int k = 0; k < 3; k++) {
          double apk = A[p][k], ark = A[r][k];
          A[p][k] = c * apk - s * ark;
          A[r][k] = s * apk + c * ark;
        }
        for (int k = 0; k < 3; k++) {
          double qkp = Q[k][p], qkr = Q[k][r];
          Q[k][p] = c * qkp - s * qkr;
          Q[k][r] = s * qkp + c * qkr;
        }
      }
  }
  int idx[3] = {0, 1, 2};
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (A[idx[j]][idx[j]] > A[idx[i]][idx[i]]) {
        int tmp = idx[i];
        idx[i] = idx[j];
        idx[j] = tmp;
      }
  for (int k = 0; k < 2; k++) {
    double v[3] = {Q[0][idx[k]], Q[1][idx[k]], Q[2][idx[k]]};
    int big = 0;
    for (int i = 1; i < 3; i++)
      if (std::fabs(v[i]) > std::fabs(v[big])) big = i;
    double sg = v[big] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < 3; i++) V[i][k] = sg * v[i];
    w[k] = A[idx[k]][idx[k]];
  }
  w[2] = A[idx[2]][idx[2]];
  double v1[3] = {V[0][0], V[1][0], V[2][0]}, v2[3] = {V[0][1], V[1][1], V[2][1]}, v3[3];
  rb_cross(v1, v2, v3);
  for (int i = 0; i < 3; i++) V[i][2] = v3[i];
}

// Shepperd's quaternion of the rotation matrix A (rows = body axes)
inline void rb_quaternion(const double A[3][3], double* Q) {
  double Q2[4] = {1.0 + A[0][0] + A[1][1] + A[2][2], 1.0 + A[0][0] - A[1][1] - A[2][2],
                  1.0 - A[0][0] + A[1][1] - A[2][2], 1.0 - A[0][0] - A[1][1] + A[2][2]};
  int imax = 0;
  for (int i = 1; i < 4; i++)
    if (Q2[i] > Q2[imax]) imax = i;
  double f = 0.5 * std::sqrt(1.0 / Q2[imax]), m = Q2[imax];
  switch (imax) {
    case 0: Q[0] = m; Q[1] = A[1][2] - A[2][1]; Q[2] = A[2][0] - A[0][2]; Q[3] = A[0][1] - A[1][0]; break;
    case 1: Q[0] = A[1][2] - A[2][1]; Q[1] = m; Q[2] = A[0][1] + A[1][0]; Q[3] = A[0][2] + A[2][0]; break;
    case 2: Q[0] = A[2][0] - A[0][2]; Q[1] = A[0][1] + A[1][0]; Q[2] = m; Q[3] = A[1][2] + A[2][1]; break;
    default: Q[0] = A[0][1] - A[1][0]; Q[1] = A[0][2] + A[2][0]; Q[2] = A[1][2] + A[2][1]; Q[3] = m; break;
  }
  for (int i = 0; i < 4; i++) Q[i] *= f;
}

// src/ArBee.f90:97-134 for one body: coords (3*NP, unwrapped) -> rcm, delta,
// principal moments, quaternion, body-frame coordinates d
inline void rb_update(BodyState& b, const double* M, const double* coords, double* d, double* delta) {
  double I[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, V[3][3], A[3][3];
  for (int x = 0; x < 3; x++) {
    double s = 0.0;
    for (int k = 0; k < b.NP; k++) s += M[k] * coords[3 * k + x];
    b.rcm[x] = s * b.invMass;
  }
  for (int k = 0; k < b.NP; k++)
    for (int x = 0; x < 3; x++) delta[3 * k + x] = coords[3 * k + x] - b.rcm[x];
  for (int k = 0; k < b.NP; k++) {
    const double* e = &delta[3 * k];
    double m = M[k];
    I[0][0] += m * (e[1] * e[1] + e[2] * e[2]);
    I[1][1] += m * (e[0] * e[0] + e[2] * e[2]);
    I[2][2] += m * (e[0] * e[0] + e[1] * e[1]);
    I[0][1] -= m * e[0] * e[1];
    I[0][2] -= m * e[0] * e[2];
    I[1][2] -= m * e[1] * e[2];
  }
  I[1][0] = I[0][1];
  I[2][0] = I[0][2];
  I[2][1] = I[1][2];
  rb_eigen_sym3(I, V, b.MoI);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = V[j][i];
  for (int k = 0; k < 3; k++) b.invMoI[k] = 1.0 / b.MoI[k];
  double I1 = b.MoI[0], I2 = b.MoI[1], I3 = b.MoI[2];
  b.I113 = 1.0 / (I1 * (I1 - I3));
  b.I313 = 1.0 / (I3 * (I1 - I3));
  b.I223 = 1.0 / (I2 * (I2 - I3));
  b.I212 = 1.0 / (I2 * (I1 - I2));
  b.m312 = (I3 - I1) / I2;
  rb_quaternion(A, b.q);
  for (int k = 0; k < b.NP; k++)
    for (int i = 0; i < 3; i++)
      d[3 * k + i] = A[i][0] * delta[3 * k] + A[i][1] * delta[3 * k + 1] + A[i][2] * delta[3 * k + 2];
}

}  // namespace emdee

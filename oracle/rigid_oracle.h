/*
 * rigid_oracle.h -- rigid bodies of the CPU oracle (TEST INFRASTRUCTURE ONLY;
 * included by emdee_oracle.c).  Restates src/ArBee.f90 and the body branches of
 * src/EmDeeData.f90 in FP64.  The symmetric 3x3 eigen-solver is written from
 * the mathematics (cyclic Jacobi rotations), with the output contract the body
 * code relies on: eigenvalues in decreasing order and a right-handed frame.
 * The quaternion of a rotation matrix follows Shepperd's method (S. W.
 * Shepperd, J. Guidance and Control 1, 223, 1978); the exact free rotation
 * follows van Zon and Schofield (J. Comput. Phys. 225, 145, 2007) as
 * src/ArBee.f90:225-324 does, with Carlson's elliptic integrals (B. C. Carlson,
 * Numer. Algorithms 10, 13, 1995) and the AGM evaluation of Jacobi elliptic
 * functions (Abramowitz & Stegun 16.4).
 */
#include <math.h>

typedef struct {
  int NP, dof;
  int* index;      /* 1-based atom indices */
  double* M;       /* particle masses */
  double* d;       /* body-frame coordinates, 3*NP */
  double* delta;   /* space-frame coordinates relative to the centre of mass, 3*NP */
  double mass, invMass;
  double MoI[3], invMoI[3], rcm[3], pcm[3], q[4], pi[4], omega[3], F[3], tau[3];
  double I113, I313, I223, I212, m312;
} obody;

static void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

/* B(q) (4x3), C(q) (4x3) and their transposes applied to vectors
 * (src/ArBee.f90:138-176): columns of B are (-q1,q0,q3,-q2), (-q2,-q3,q0,q1),
 * (-q3,q2,-q1,q0); columns of C are (-q1,q0,-q3,q2), (-q2,q3,q0,-q1),
 * (-q3,-q2,q1,q0). */
static void matB(const double* q, const double* v, double* out) {   /* out = B v */
  out[0] = -q[1] * v[0] - q[2] * v[1] - q[3] * v[2];
  out[1] = q[0] * v[0] - q[3] * v[1] + q[2] * v[2];
  out[2] = q[3] * v[0] + q[0] * v[1] - q[1] * v[2];
  out[3] = -q[2] * v[0] + q[1] * v[1] + q[0] * v[2];
}
static void matC(const double* q, const double* v, double* out) {   /* out = C v */
  out[0] = -q[1] * v[0] - q[2] * v[1] - q[3] * v[2];
  out[1] = q[0] * v[0] + q[3] * v[1] - q[2] * v[2];
  out[2] = -q[3] * v[0] + q[0] * v[1] + q[1] * v[2];
  out[3] = q[2] * v[0] - q[1] * v[1] + q[0] * v[2];
}
static void matBt(const double* q, const double* v, double* out) {   /* out = B^T v */
  out[0] = -q[1] * v[0] + q[0] * v[1] + q[3] * v[2] - q[2] * v[3];
  out[1] = -q[2] * v[0] - q[3] * v[1] + q[0] * v[2] + q[1] * v[3];
  out[2] = -q[3] * v[0] + q[2] * v[1] - q[1] * v[2] + q[0] * v[3];
}
static void matCt(const double* q, const double* v, double* out) {   /* out = C^T v */
  out[0] = -q[1] * v[0] + q[0] * v[1] - q[3] * v[2] + q[2] * v[3];
  out[1] = -q[2] * v[0] + q[3] * v[1] + q[0] * v[2] - q[1] * v[3];
  out[2] = -q[3] * v[0] - q[2] * v[1] + q[1] * v[2] + q[0] * v[3];
}

/* symmetric 3x3 eigen-solver: cyclic Jacobi rotations; w decreasing, V columns
 * = eigenvectors, right-handed (v3 = v1 x v2), largest component of v1, v2 > 0 */
static void eigen_sym3(const double Ain[3][3], double V[3][3], double w[3]) {
  double A[3][3], Q[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = Ain[i][j];
  for (int sweep = 0; sweep < 64; sweep++) {
    if (A[0][1] == 0.0 && A[0][2] == 0.0 && A[1][2] == 0.0) break;
    for (int p = 0; p < 2; p++)
      for (int r = p + 1; r < 3; r++) {
        if (fabs(A[p][r]) <= 1e-18 * (fabs(A[p][p]) + fabs(A[r][r]))) {
          A[p][r] = A[r][p] = 0.0;
          continue;
        }
        double theta = (A[r][r] - A[p][p]) / (2.0 * A[p][r]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {   /* A <- J^T A J */
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
      if (fabs(v[i]) > fabs(v[big])) big = i;
    double sg = v[big] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < 3; i++) V[i][k] = sg * v[i];
    w[k] = A[idx[k]][idx[k]];
  }
  w[2] = A[idx[2]][idx[2]];
  double v1[3] = {V[0][0], V[1][0], V[2][0]}, v2[3] = {V[0][1], V[1][1], V[2][1]}, v3[3];
  cross3(v1, v2, v3);
  for (int i = 0; i < 3; i++) V[i][2] = v3[i];
}

/* unit quaternion of the rotation matrix A (rows = body axes), Shepperd */
static void quaternion_of(const double A[3][3], double* Q) {
  double Q2[4] = {1.0 + A[0][0] + A[1][1] + A[2][2], 1.0 + A[0][0] - A[1][1] - A[2][2],
                  1.0 - A[0][0] + A[1][1] - A[2][2], 1.0 - A[0][0] - A[1][1] + A[2][2]};
  int imax = 0;
  for (int i = 1; i < 4; i++)
    if (Q2[i] > Q2[imax]) imax = i;
  double f = 0.5 * sqrt(1.0 / Q2[imax]), m = Q2[imax];
  switch (imax) {
    case 0: Q[0] = m; Q[1] = A[1][2] - A[2][1]; Q[2] = A[2][0] - A[0][2]; Q[3] = A[0][1] - A[1][0]; break;
    case 1: Q[0] = A[1][2] - A[2][1]; Q[1] = m; Q[2] = A[0][1] + A[1][0]; Q[3] = A[0][2] + A[2][0]; break;
    case 2: Q[0] = A[2][0] - A[0][2]; Q[1] = A[0][1] + A[1][0]; Q[2] = m; Q[3] = A[1][2] + A[2][1]; break;
    default: Q[0] = A[0][1] - A[1][0]; Q[1] = A[0][2] + A[2][0]; Q[2] = A[1][2] + A[2][1]; Q[3] = m; break;
  }
  for (int i = 0; i < 4; i++) Q[i] *= f;
}

/* src/ArBee.f90:97-134: centre of mass, principal frame, quaternion, body-frame coordinates */
static void body_update(obody* b, const double* coords) {
  double I[3][3] = {{0}}, V[3][3], A[3][3];
  for (int x = 0; x < 3; x++) {
    double s = 0.0;
    for (int k = 0; k < b->NP; k++) s += b->M[k] * coords[3 * k + x];
    b->rcm[x] = s * b->invMass;
  }
  for (int k = 0; k < b->NP; k++)
    for (int x = 0; x < 3; x++) b->delta[3 * k + x] = coords[3 * k + x] - b->rcm[x];
  for (int k = 0; k < b->NP; k++) {
    const double* e = &b->delta[3 * k];
    double m = b->M[k];
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
  eigen_sym3(I, V, b->MoI);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = V[j][i];
  for (int k = 0; k < 3; k++) b->invMoI[k] = 1.0 / b->MoI[k];
  double I1 = b->MoI[0], I2 = b->MoI[1], I3 = b->MoI[2];
  b->I113 = 1.0 / (I1 * (I1 - I3));
  b->I313 = 1.0 / (I3 * (I1 - I3));
  b->I223 = 1.0 / (I2 * (I2 - I3));
  b->I212 = 1.0 / (I2 * (I1 - I2));
  b->m312 = (I3 - I1) / I2;
  quaternion_of(A, b->q);
  for (int k = 0; k < b->NP; k++)
    for (int i = 0; i < 3; i++)
      b->d[3 * k + i] = A[i][0] * b->delta[3 * k] + A[i][1] * b->delta[3 * k + 1] + A[i][2] * b->delta[3 * k + 2];
}

/* src/ArBee.f90:356-366 */
static void body_assign_omega(obody* b, const double* omega) {
  double v[3];
  for (int k = 0; k < 3; k++) {
    b->omega[k] = omega[k];
    v[k] = 2.0 * b->MoI[k] * omega[k];
  }
  matB(b->q, v, b->pi);
}
static void body_assign_pi(obody* b, const double* pi) {
  double v[3];
  for (int k = 0; k < 4; k++) b->pi[k] = pi[k];
  matBt(b->q, b->pi, v);
  for (int k = 0; k < 3; k++) b->omega[k] = 0.5 * b->invMoI[k] * v[k];
}

/* delta = C(q)^T B(q) d: body-frame to space-frame coordinates */
static void body_space_coords(obody* b) {
  for (int k = 0; k < b->NP; k++) {
    double t[4];
    matB(b->q, &b->d[3 * k], t);
    matCt(b->q, t, &b->delta[3 * k]);
  }
}

/* src/ArBee.f90:200-221 */
static void rotate_uniaxial(obody* b, int k, double dt) {
  double BkQ[4], BkPi[4], *q = b->q, *p = b->pi;
  switch (k) {
    case 1:
      BkQ[0] = -q[1]; BkQ[1] = q[0]; BkQ[2] = q[3]; BkQ[3] = -q[2];
      BkPi[0] = -p[1]; BkPi[1] = p[0]; BkPi[2] = p[3]; BkPi[3] = -p[2];
      break;
    case 2:
      BkQ[0] = -q[2]; BkQ[1] = -q[3]; BkQ[2] = q[0]; BkQ[3] = q[1];
      BkPi[0] = -p[2]; BkPi[1] = -p[3]; BkPi[2] = p[0]; BkPi[3] = p[1];
      break;
    default:
      BkQ[0] = -q[3]; BkQ[1] = q[2]; BkQ[2] = -q[1]; BkQ[3] = q[0];
      BkPi[0] = -p[3]; BkPi[1] = p[2]; BkPi[2] = -p[1]; BkPi[3] = p[0];
      break;
  }
  double dot = p[0] * BkQ[0] + p[1] * BkQ[1] + p[2] * BkQ[2] + p[3] * BkQ[3];
  double a = dt * dot / (4.0 * b->MoI[k - 1]);
  double vs = sin(a), vc = cos(a);
  for (int i = 0; i < 4; i++) {
    q[i] = vc * q[i] + vs * BkQ[i];
    p[i] = vc * p[i] + vs * BkPi[i];
  }
}

/* src/ArBee.f90:180-196 */
static void rotate_no_squish(obody* b, double delta_t, int n) {
  double dt = delta_t / n, h = 0.5 * dt;
  for (int i = 0; i < n; i++) {
    rotate_uniaxial(b, 3, h);
    rotate_uniaxial(b, 2, h);
    rotate_uniaxial(b, 1, dt);
    rotate_uniaxial(b, 2, h);
    rotate_uniaxial(b, 3, h);
  }
  body_space_coords(b);
}

/* Carlson's symmetric elliptic integrals RF, RC, RJ (duplication algorithm) */
static double carlson_RF(double x, double y, double z) {
  const double errtol = 0.001;
  double xn = x, yn = y, zn = z, mu, xd, yd, zd;
  for (;;) {
    mu = (xn + yn + zn) / 3.0;
    xd = 2.0 - (mu + xn) / mu;
    yd = 2.0 - (mu + yn) / mu;
    zd = 2.0 - (mu + zn) / mu;
    double e = fmax(fabs(xd), fmax(fabs(yd), fabs(zd)));
    if (e < errtol) break;
    double xr = sqrt(xn), yr = sqrt(yn), zr = sqrt(zn);
    double lam = xr * (yr + zr) + yr * zr;
    xn = (xn + lam) * 0.25;
    yn = (yn + lam) * 0.25;
    zn = (zn + lam) * 0.25;
  }
  const double c1 = 1.0 / 24.0, c2 = 3.0 / 44.0, c3 = 1.0 / 14.0;
  double e2 = xd * yd - zd * zd, e3 = xd * yd * zd;
  double s = 1.0 + (c1 * e2 - 0.1 - c2 * e3) * e2 + c3 * e3;
  return s / sqrt(mu);
}

static double carlson_RC(double x, double y) {
  const double errtol = 0.001;
  double xn = x, yn = y, mu, sn;
  for (;;) {
    mu = (xn + yn + yn) / 3.0;
    sn = (yn + mu) / mu - 2.0;
    if (fabs(sn) < errtol) break;
    double lam = 2.0 * sqrt(xn) * sqrt(yn) + yn;
    xn = (xn + lam) * 0.25;
    yn = (yn + lam) * 0.25;
  }
  const double c1 = 1.0 / 7.0, c2 = 9.0 / 22.0;
  double s = sn * sn * (0.3 + sn * (c1 + sn * (0.375 + sn * c2)));
  return (1.0 + s) / sqrt(mu);
}

static double carlson_RJ(double x, double y, double z, double p) {
  const double errtol = 0.001;
  double xn = x, yn = y, zn = z, pn = p, sigma = 0.0, power4 = 1.0, mu, xd, yd, zd, pd;
  for (;;) {
    mu = (xn + yn + zn + pn + pn) * 0.2;
    xd = (mu - xn) / mu;
    yd = (mu - yn) / mu;
    zd = (mu - zn) / mu;
    pd = (mu - pn) / mu;
    double e = fmax(fmax(fabs(xd), fabs(yd)), fmax(fabs(zd), fabs(pd)));
    if (e < errtol) break;
    double xr = sqrt(xn), yr = sqrt(yn), zr = sqrt(zn);
    double lam = xr * (yr + zr) + yr * zr;
    double al = pn * (xr + yr + zr) + xr * yr * zr;
    al = al * al;
    double be = pn * (pn + lam) * (pn + lam);
    sigma += power4 * carlson_RC(al, be);
    power4 *= 0.25;
    xn = (xn + lam) * 0.25;
    yn = (yn + lam) * 0.25;
    zn = (zn + lam) * 0.25;
    pn = (pn + lam) * 0.25;
  }
  double ea = xd * (yd + zd) + yd * zd, eb = xd * yd * zd, ec = pd * pd;
  double e2 = ea - 3.0 * ec, e3 = eb + 2.0 * pd * (ea - ec);
  const double c1 = 3.0 / 14.0, c2 = 1.0 / 3.0, c3 = 3.0 / 22.0, c4 = 3.0 / 26.0;
  double s1 = 1.0 + e2 * (-c1 + 0.75 * c3 * e2 - 1.5 * c4 * e3);
  double s2 = eb * (0.5 * c2 + pd * (-c3 - c3 + pd * c4));
  double s3 = pd * ea * (c2 - pd * c3) - c2 * pd * ec;
  return 3.0 * sigma + power4 * (s1 + s2 + s3) / (mu * sqrt(mu));
}

/* Jacobi elliptic sn, cn, dn by the arithmetic-geometric mean */
static void jacobi_sncndn(double u, double m, double* sn, double* cn, double* dn) {
  const double eps = 2.220446049250313e-16;
  if (fabs(m) < 2 * eps) {
    *sn = sin(u); *cn = cos(u); *dn = 1.0;
    return;
  }
  if (fabs(m - 1.0) < 2 * eps) {
    *sn = tanh(u); *cn = *dn = 1.0 / cosh(u);
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
  if (fabs(su) < fabs(cu)) {
    c[n] = mu[n] * (su / cu);
    d[n] = 1.0;
    while (n > 0) {
      c[n - 1] = d[n] * c[n];
      double r = c[n] * c[n] / mu[n];
      n--;
      d[n] = (r + nu[n]) / (r + mu[n]);
    }
    *dn = sqrt(1.0 - m) / d[0];
    *cn = *dn * (cu < 0 ? -1.0 : 1.0) / hypot(1.0, c[0]);
    *sn = *cn * c[0] / sqrt(1.0 - m);
  } else {
    c[n] = mu[n] * (cu / su);
    d[n] = 1.0;
    while (n > 0) {
      c[n - 1] = d[n] * c[n];
      double r = c[n] * c[n] / mu[n];
      n--;
      d[n] = (r + nu[n]) / (r + mu[n]);
    }
    *dn = d[0];
    *sn = (su < 0 ? -1.0 : 1.0) / hypot(1.0, c[0]);
    *cn = c[0] * *sn;
  }
}

static int staircase(double x) { return x > 0 ? (int)ceil(x - 0.5) : (int)floor(x + 0.5); }
static double sgn(double a, double b) { return b >= 0 ? fabs(a) : -fabs(a); }   /* Fortran SIGN */

static double Theta(double x, double n, double m) {
  double x2 = x * x;
  return -(1.0 / 3.0) * n * x * x2 * carlson_RJ(1.0 - x2, 1.0 - m * x2, 1.0, 1.0 + n * x2);
}

static double deltaFcn(double u0, double c0, double s0, double d0, double u, double cn, double sn, double dn,
                       double m, int jump, double alpha) {
  double eta = alpha * alpha / (1.0 - alpha * alpha), C = sqrt(m + eta);
  double r = u - u0 + sgn(1.0, cn) * Theta(sn, eta, m) - sgn(1.0, c0) * Theta(s0, eta, m) +
             (alpha / C) * (atan(C * sn / dn) - atan(C * s0 / d0));
  if (jump != 0) r += jump * 2.0 * Theta(1.0, eta, m);
  return (eta + 1.0) * r;
}

static double deltaFdn(double u0, double c0, double s0, double u, double cn, double sn, double m, int jump,
                       double alpha) {
  double eta = alpha * alpha;
  eta = eta / (1.0 - eta);
  double k2eta = m * eta, C = sqrt(1.0 + k2eta);
  double r = u - u0 + sgn(1.0, cn) * Theta(sn, k2eta, m) - sgn(1.0, c0) * Theta(s0, k2eta, m) +
             (alpha / C) * (atan(C * sn / cn) - atan(C * s0 / c0));
  if (jump != 0) r += jump * (2.0 * Theta(1.0, k2eta, m) + (alpha / C) * 3.14159265358979324);
  return (eta + 1.0) * r;
}

/* exact free rotation over dt (src/ArBee.f90:225-324) */
static void rotate_exact(obody* b, double dt) {
  double w0[3] = {b->omega[0], b->omega[1], b->omega[2]}, Iw[3];
  for (int k = 0; k < 3; k++) Iw[k] = b->MoI[k] * w0[k];
  double Lsq = Iw[1] * Iw[1] + Iw[2] * Iw[2];
  if (Lsq < 2.220446049250313e-16) {
    rotate_uniaxial(b, 1, dt);
    return;
  }
  Lsq = Iw[0] * Iw[0] + Lsq;
  double L = sqrt(Lsq);
  double TwoKr = Iw[0] * w0[0] + Iw[1] * w0[1] + Iw[2] * w0[2];
  double r1 = Lsq - TwoKr * b->MoI[2], r3 = TwoKr * b->MoI[0] - Lsq;
  double l1 = b->I223 * r1, l3 = b->I212 * r3, lmin = fmin(l1, l3);
  double a[3] = {sgn(1.0, w0[0]) * sqrt(b->I113 * r1), sqrt(lmin), sgn(1.0, w0[2]) * sqrt(b->I313 * r3)};
  double m = lmin / fmax(l1, l3);
  double K = carlson_RF(0.0, 1.0 - m, 1.0), inv2K = 0.5 / K;
  double s0 = w0[1] / a[1], c0, u0;
  int i0;
  if (fabs(s0) < 1.0) {
    c0 = l1 < l3 ? w0[0] / a[0] : w0[2] / a[2];
    u0 = s0 * carlson_RF(1.0 - s0 * s0, 1.0 - m * s0 * s0, 1.0);
    i0 = staircase(u0 * inv2K);
  } else {
    a[1] = fabs(w0[1]);
    s0 = sgn(1.0, s0);
    c0 = 0.0;
    u0 = sgn(K, s0);
    i0 = 0;
  }
  double wp = b->m312 * a[0] * a[2] / a[1];
  double u = wp * dt + u0;
  int jump = staircase(u * inv2K) - i0;
  double sn, cn, dn, deltaF;
  jacobi_sncndn(u, m, &sn, &cn, &dn);
  if (l1 < l3) {
    b->omega[0] = a[0] * cn; b->omega[1] = a[1] * sn; b->omega[2] = a[2] * dn;
    deltaF = deltaFcn(u0, c0, s0, w0[2] / a[2], u, cn, sn, dn, m, jump, b->MoI[0] * a[0] / L);
  } else {
    b->omega[0] = a[0] * dn; b->omega[1] = a[1] * sn; b->omega[2] = a[2] * cn;
    deltaF = deltaFdn(u0, c0, s0, u, cn, sn, m, jump, b->MoI[0] * a[0] / L);
  }
  double phi = (Lsq * (u - u0) + r3 * deltaF) / (2.0 * L * b->MoI[0] * wp);
  double z0[4] = {Iw[2], Iw[1], L - Iw[0], 0.0};
  for (int k = 0; k < 3; k++) Iw[k] = b->MoI[k] * b->omega[k];
  double cp = cos(phi), sp = sin(phi), z[4];
  z[0] = Iw[2] * cp - Iw[1] * sp;
  z[1] = Iw[1] * cp + Iw[2] * sp;
  z[2] = (L - Iw[0]) * cp;
  z[3] = (L - Iw[0]) * sp;
  double dotz = z0[0] * b->q[0] + z0[1] * b->q[1] + z0[2] * b->q[2] + z0[3] * b->q[3], t[3], nq[4];
  matCt(z0, b->q, t);
  matC(z, t, nq);
  double norm = 0.0;
  for (int k = 0; k < 4; k++) {
    nq[k] = z[k] * dotz + nq[k];
    norm += nq[k] * nq[k];
  }
  norm = sqrt(norm);
  for (int k = 0; k < 4; k++) b->q[k] = nq[k] / norm;
  double v[3] = {2.0 * Iw[0], 2.0 * Iw[1], 2.0 * Iw[2]};
  matB(b->q, v, b->pi);
  body_space_coords(b);
}

/* src/ArBee.f90:340-352 */
static void force_and_torque(obody* b, const double* F) {
  for (int k = 0; k < 3; k++) b->F[k] = b->tau[k] = 0.0;
  for (int j = 0; j < b->NP; j++) {
    const double* Fj = &F[3 * (b->index[j] - 1)];
    double c[3];
    cross3(&b->delta[3 * j], Fj, c);
    for (int k = 0; k < 3; k++) {
      b->F[k] += Fj[k];
      b->tau[k] += c[k];
    }
  }
}

/* src/ArBee.f90:328-336 */
static void particle_momenta(const obody* b, double* P) {
  double t[4], omega[3];
  matB(b->q, b->omega, t);
  matCt(b->q, t, omega);
  for (int k = 0; k < b->NP; k++) {
    double c[3];
    cross3(omega, &b->delta[3 * k], c);
    for (int x = 0; x < 3; x++) P[3 * (b->index[k] - 1) + x] = b->M[k] * (b->invMass * b->pcm[x] + c[x]);
  }
}

/*
 * ewald_oracle.h -- Ewald k-space solver of the CPU oracle (TEST INFRASTRUCTURE
 * ONLY; included by emdee_oracle.c).  Restates, in FP64:
 *   - src/modelClass_kspace.f90:111-334 (charged-type lists, rigid-pair and
 *     self-energy discounts, Coulomb constants per type pair and layer),
 *   - src/kspace_ewald.f90:82-314 (alpha and kmax from the accuracy, the half
 *     k-lattice, prefactors, q exp(i k.r) by complex recursion, type structure
 *     factors, energy and forces),
 *   - src/math.f90:642-657 (inverse of x + ln x) and :695-702 (symm1D).
 * The reference's G3 negative-index range uses nmax(2) (src/kspace_ewald.f90:218);
 * boxes are cubic here, so nmax(2) = nmax(3) and the range is the same.
 */
#include <math.h>

typedef struct {
  double accuracy, alpha, beta, kmax, Volume, L;
  int nmax[3], nvecs;
  int* n;           /* nvecs x 3 */
  double* prefac;   /* nvecs */
  double* vec;      /* vec[3 v + d] = 2 prefac k_d */
  double *qre, *qim;   /* q exp(i k.r): [j nvecs + v] */
  double *Sre, *Sim;   /* structure factors per charged type: [t nvecs + v] */
  int ntypes;       /* distinct types of charged atoms */
  int* type;        /* their (1-based) type numbers, ascending */
  int nq;           /* atoms listed (every atom of a charged type) */
  int* item;        /* 1-based atom numbers, grouped by type */
  double* value;    /* their charges */
  int *first, *last;   /* 1-based inclusive ranges of item per local type */
  int nTypePairs;
  double* Erigid;   /* unscaled discount energy per type pair (symm1D order) */
  int nlayers;
  double* lambda;   /* [layer][t2][t1] */
  double* lambda1D; /* [layer][k] */
} oewald;

static int symm1D(int i, int j) {   /* src/math.f90:695-702 */
  int x = (i < j ? i : j) - 1, y = (i > j ? i : j) - 1;
  return x + (y + 1) * y / 2 + 1;
}

static double inverse_of_x_plus_ln_x(double y) {   /* src/math.f90:642-657 */
  const double tol = 1.0e-12;
  double x = y > 0.5671432904097839 ? y - log(y) : exp(y);
  double x0 = x + 1.0;
  while (fabs(x - x0) > tol * x0) {
    x0 = x;
    x = x * (y + 1.0 - log(x)) / (x + 1.0);
  }
  return x;
}

/* src/modelClass_kspace.f90:318-332 */
static void ewald_discount(const oewald* e, double* E, double* W, double rsq, double QiQj) {
  double r = sqrt(rsq), x = e->alpha * r, expmx2 = exp(-x * x);
  *E = -QiQj * (1.0 - uerfc(x, expmx2)) / r;
  *W = *E + QiQj * e->beta * expmx2;
}

/* src/kspace_ewald.f90:82-103 */
static void ewald_set_parameters(oewald* e, double Rc) {
  double s = sqrt(inverse_of_x_plus_ln_x(-log(e->accuracy)));
  e->alpha = s / Rc;
  e->kmax = 2.0 * e->alpha * s;
  printf("KSPACE PARAMETERS: alpha = %10.5f and kmax = %10.5f\n", e->alpha, e->kmax);
  fflush(stdout);
}

/* src/kspace_ewald.f90:107-170 (cubic box) */
static void ewald_update(oewald* e, double L) {
  const double Pi = 3.14159265358979324;
  double unit = 2.0 * Pi / L, unitSq = unit * unit;
  int nmax = (int)ceil(e->kmax / unit);
  if (nmax != e->nmax[0] || nmax != e->nmax[1] || nmax != e->nmax[2]) {
    e->nmax[0] = e->nmax[1] = e->nmax[2] = nmax;
    int M = 2 * nmax + 1;
    long maxnvecs = (long)M * M * M / 2;
    int* n = (int*)xmalloc(sizeof(int) * 3 * (size_t)maxnvecs);
    long M2 = M, M2M3 = (long)M * M;
    int nv = 0;
    double kmaxSq = unitSq * nmax * nmax;   /* maxval(unitSq*nmax**2) */
    for (long i = maxnvecs + 1; i <= 2 * maxnvecs; i++) {
      long n1 = i / M2M3, j = i - n1 * M2M3, n2 = j / M2, n3 = j - n2 * M2;
      int kv[3] = {(int)n1 - nmax, (int)n2 - nmax, (int)n3 - nmax};
      double s = unitSq * kv[0] * kv[0] + unitSq * kv[1] * kv[1] + unitSq * kv[2] * kv[2];
      if (s <= kmaxSq) {
        n[3 * nv] = kv[0];
        n[3 * nv + 1] = kv[1];
        n[3 * nv + 2] = kv[2];
        nv++;
      }
    }
    free(e->n);
    free(e->prefac);
    free(e->vec);
    free(e->qre);
    free(e->qim);
    free(e->Sre);
    free(e->Sim);
    e->nvecs = nv;
    e->n = n;
    e->prefac = (double*)xmalloc(sizeof(double) * (nv ? nv : 1));
    e->vec = (double*)xmalloc(sizeof(double) * 3 * (nv ? nv : 1));
    e->qre = (double*)xmalloc(sizeof(double) * (size_t)(nv ? nv : 1) * e->nq);
    e->qim = (double*)xmalloc(sizeof(double) * (size_t)(nv ? nv : 1) * e->nq);
    e->Sre = (double*)xmalloc(sizeof(double) * (size_t)(nv ? nv : 1) * e->ntypes);
    e->Sim = (double*)xmalloc(sizeof(double) * (size_t)(nv ? nv : 1) * e->ntypes);
    double B = -0.25 / (e->alpha * e->alpha);
    e->Volume = L * L * L;
    double fourPiByV = 4.0 * Pi / e->Volume;
    for (int v = 0; v < nv; v++) {
      double k[3] = {unit * n[3 * v], unit * n[3 * v + 1], unit * n[3 * v + 2]};
      double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
      e->prefac[v] = fourPiByV * exp(ksq * B) / ksq;
      for (int d = 0; d < 3; d++) e->vec[3 * v + d] = 2.0 * e->prefac[v] * k[d];
    }
  } else {
    double factor = e->Volume / (L * L * L);
    for (int v = 0; v < e->nvecs; v++) {
      e->prefac[v] = factor * e->prefac[v];
      for (int d = 0; d < 3; d++) e->vec[3 * v + d] = factor * e->vec[3 * v + d];
    }
    e->Volume = L * L * L;
  }
  e->L = L;
}

/* src/modelClass_kspace.f90:111-243.  kCoul(i, j, layer) gives the Coulomb
 * constant of the type pair (1-based types and layer). */
static void ewald_initialize(oewald* e, double Rc, double L, int N, const int* types, const double* charge,
                             const double* R, int nbodies, const obody* bodies, int nlayers,
                             double (*kCoul)(void*, int, int, int), void* ctx) {
  const char* task = "kspace model initialization";
  const double Pi = 3.14159265358979324, eps = 2.220446049250313e-16;
  char* charged = (char*)xcalloc(N ? N : 1, 1);
  int ncharged = 0, maxType = 0;
  for (int i = 0; i < N; i++) {
    charged[i] = fabs(charge[i]) > eps;
    if (charged[i]) {
      ncharged++;
      if (types[i] > maxType) maxType = types[i];
    }
  }
  if (ncharged == 0) error(task, "system has no charged atoms");
  char* present = (char*)xcalloc(maxType + 1, 1);
  for (int i = 0; i < N; i++)
    if (charged[i]) present[types[i]] = 1;
  e->ntypes = 0;
  for (int t = 1; t <= maxType; t++) e->ntypes += present[t];
  e->type = (int*)xmalloc(sizeof(int) * e->ntypes);
  int* local = (int*)xcalloc(maxType + 1, sizeof(int));
  for (int t = 1, k = 0; t <= maxType; t++)
    if (present[t]) {
      e->type[k] = t;
      local[t] = ++k;
    }
  /* the charge list holds every atom of each charged type, type by type */
  e->nq = 0;
  for (int i = 0; i < N; i++)
    if (types[i] <= maxType && present[types[i]]) e->nq++;
  e->item = (int*)xmalloc(sizeof(int) * e->nq);
  e->value = (double*)xmalloc(sizeof(double) * e->nq);
  e->first = (int*)xmalloc(sizeof(int) * e->ntypes);
  e->last = (int*)xmalloc(sizeof(int) * e->ntypes);
  int lastk = 0;
  for (int t = 0; t < e->ntypes; t++) {
    e->first[t] = lastk + 1;
    for (int i = 0; i < N; i++)
      if (types[i] == e->type[t]) {
        e->item[lastk] = i + 1;
        e->value[lastk] = charge[i];
        lastk++;
      }
    e->last[t] = lastk;
  }
  ewald_set_parameters(e, Rc);
  e->beta = 2.0 * e->alpha / sqrt(Pi);
  /* rigid pairs and self energy */
  e->nTypePairs = e->ntypes * (e->ntypes - 1) / 2 + e->ntypes;
  e->Erigid = (double*)xcalloc(e->nTypePairs, sizeof(double));
  double invL = 1.0 / L;
  for (int b = 0; b < nbodies; b++) {
    const obody* B = &bodies[b];
    for (int ii = 0; ii < B->NP - 1; ii++) {
      int i = B->index[ii] - 1;
      if (!charged[i]) continue;
      for (int jj = ii + 1; jj < B->NP; jj++) {
        int j = B->index[jj] - 1;
        if (!charged[j]) continue;
        double Rij[3], rsq = 0.0, Eij, Wij;
        for (int d = 0; d < 3; d++) {
          Rij[d] = R[3 * i + d] - R[3 * j + d];
          Rij[d] = Rij[d] - L * anint(invL * Rij[d]);
        }
        rsq = Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2];
        ewald_discount(e, &Eij, &Wij, rsq, charge[i] * charge[j]);
        e->Erigid[symm1D(local[types[i]], local[types[j]]) - 1] += Eij;
      }
    }
  }
  for (int t = 1; t <= e->ntypes; t++) {
    double q2 = 0.0;
    for (int k = e->first[t - 1]; k <= e->last[t - 1]; k++) q2 += e->value[k - 1] * e->value[k - 1];
    e->Erigid[symm1D(t, t) - 1] -= e->alpha * q2 / sqrt(Pi);
  }
  /* Coulomb constants */
  e->nlayers = nlayers;
  e->lambda = (double*)xmalloc(sizeof(double) * e->ntypes * e->ntypes * nlayers);
  e->lambda1D = (double*)xmalloc(sizeof(double) * e->nTypePairs * nlayers);
  for (int i = 1; i <= e->ntypes; i++)
    for (int j = i; j <= e->ntypes; j++)
      for (int l = 1; l <= nlayers; l++) {
        double lam = kCoul(ctx, e->type[i - 1], e->type[j - 1], l);
        e->lambda[((l - 1) * e->ntypes + (j - 1)) * e->ntypes + (i - 1)] = lam;
        e->lambda[((l - 1) * e->ntypes + (i - 1)) * e->ntypes + (j - 1)] = lam;
        e->lambda1D[(l - 1) * e->nTypePairs + symm1D(i, j) - 1] = lam;
      }
  e->nmax[0] = e->nmax[1] = e->nmax[2] = -1;
  e->Volume = 0.0;
  ewald_update(e, L);
  free(charged);
  free(present);
  free(local);
}

/* src/kspace_ewald.f90:174-244: q exp(i k.r) and the type structure factors */
static void ewald_prepare(oewald* e, const double* Rs) {
  const double twoPi = 6.28318530717958648;
  int nm = e->nmax[0];
  double* G = (double*)xmalloc(sizeof(double) * 2 * 3 * (2 * nm + 1));
  /* G[d][m + nm] (re, im) for m in [-nm, nm] */
#define GRE(d, m) G[2 * ((d) * (2 * nm + 1) + (m) + nm)]
#define GIM(d, m) G[2 * ((d) * (2 * nm + 1) + (m) + nm) + 1]
  for (int j = 0; j < e->nq; j++) {
    int i = e->item[j] - 1;
    for (int d = 0; d < 3; d++) {
      double theta = twoPi * Rs[3 * i + d], zr = cos(theta), zi = sin(theta);
      GRE(d, 0) = 1.0;
      GIM(d, 0) = 0.0;
      double br = zr, bi = zi;   /* recursion: B = Z; G(1) = B; B = B*Z ... */
      for (int m = 1; m <= nm; m++) {
        GRE(d, m) = br;
        GIM(d, m) = bi;
        double nr = br * zr - bi * zi, ni = br * zi + bi * zr;
        br = nr;
        bi = ni;
      }
      for (int m = 1; m <= nm; m++) {
        GRE(d, -m) = GRE(d, m);
        GIM(d, -m) = -GIM(d, m);
      }
    }
    double q = e->value[j];
    for (int v = 0; v < e->nvecs; v++) {
      const int* nv = &e->n[3 * v];
      double ar = q * GRE(0, nv[0]), ai = q * GIM(0, nv[0]);
      double br = ar * GRE(1, nv[1]) - ai * GIM(1, nv[1]), bi = ar * GIM(1, nv[1]) + ai * GRE(1, nv[1]);
      e->qre[(size_t)j * e->nvecs + v] = br * GRE(2, nv[2]) - bi * GIM(2, nv[2]);
      e->qim[(size_t)j * e->nvecs + v] = br * GIM(2, nv[2]) + bi * GRE(2, nv[2]);
    }
  }
#undef GRE
#undef GIM
  free(G);
  for (int t = 0; t < e->ntypes; t++)
    for (int v = 0; v < e->nvecs; v++) {
      double sr = 0.0, si = 0.0;
      for (int j = e->first[t] - 1; j < e->last[t]; j++) {
        sr += e->qre[(size_t)j * e->nvecs + v];
        si += e->qim[(size_t)j * e->nvecs + v];
      }
      e->Sre[(size_t)t * e->nvecs + v] = sr;
      e->Sim[(size_t)t * e->nvecs + v] = si;
    }
}

/* src/kspace_ewald.f90:248-314: energy into *E, forces added to F (double[N][3]) */
static void ewald_compute(oewald* e, int layer, double* E, double* F) {
  int nv = e->nvecs, nt = e->ntypes;
  const double* lam = &e->lambda[(size_t)(layer - 1) * nt * nt];
  double* sre = (double*)xmalloc(sizeof(double) * (size_t)(nv ? nv : 1) * nt);
  double* sim = (double*)xmalloc(sizeof(double) * (size_t)(nv ? nv : 1) * nt);
  double energy = 0.0;
  for (int v = 0; v < nv; v++) {
    double d = 0.0;
    for (int t = 0; t < nt; t++) {
      double r = 0.0, im = 0.0;   /* sigma(v,t) = sum_t' S(v,t') lambda(t',t) */
      for (int u = 0; u < nt; u++) {
        r += e->Sre[(size_t)u * nv + v] * lam[t * nt + u];
        im += e->Sim[(size_t)u * nv + v] * lam[t * nt + u];
      }
      sre[(size_t)t * nv + v] = r;
      sim[(size_t)t * nv + v] = im;
      d += e->Sre[(size_t)t * nv + v] * r + e->Sim[(size_t)t * nv + v] * im;
    }
    energy += e->prefac[v] * d;
  }
  *E += energy;
  for (int t = 0; t < nt; t++)
    for (int j = e->first[t] - 1; j < e->last[t]; j++) {
      int i = e->item[j] - 1;
      double f[3] = {0.0, 0.0, 0.0};
      for (int v = 0; v < nv; v++) {
        double c = sre[(size_t)t * nv + v] * e->qim[(size_t)j * nv + v] -
                   e->qre[(size_t)j * nv + v] * sim[(size_t)t * nv + v];
        for (int d = 0; d < 3; d++) f[d] += e->vec[3 * v + d] * c;
      }
      for (int d = 0; d < 3; d++) F[3 * i + d] += f[d];
    }
  free(sre);
  free(sim);
}

/* src/modelClass_kspace.f90:247-314 (energy part; the force part is disabled there) */
static double ewald_discount_energy(const oewald* e, int layer) {
  double s = 0.0;
  for (int k = 0; k < e->nTypePairs; k++) s += e->lambda1D[(size_t)(layer - 1) * e->nTypePairs + k] * e->Erigid[k];
  return s;
}

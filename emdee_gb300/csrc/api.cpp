// api.cpp -- the C ABI of include/emdee.h: the reference's API state machine
// (src/EmDeeCode.f90) over device-resident state.
//
// Every call is synchronous at return with respect to what the caller can
// observe: results written into the tEmDee structure are complete, and
// downloads return final data.  Calls that write nothing observable (a boost
// without energies, a displacement) return as soon as their kernels are queued
// on the system's stream; the next call that reads results waits for them.
#include <chrono>
#include <cmath>
#include <cstring>

#include "system.hpp"

namespace emdee {

[[noreturn]] void fatal(const char* task, const char* msg) {   // src/global.f90:51-56
  fprintf(stderr, "Error in %s: %s.\n", task, msg);
  fflush(stderr);
  exit(1);
}

void warn(const char* msg) { fprintf(stderr, "WARNING: %s.\n", msg); }

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    char msg[512];
    snprintf(msg, sizeof msg, "%s failed: %s", what, cudaGetErrorString(e));
    fatal("CUDA", msg);
  }
}

System* sys_of(const tEmDee& md) {
  if (!md.Data) fatal("system access", "invalid EmDee system");
  return (System*)md.Data;
}

static cudaEvent_t prof_event(System& s) {
  if (s.prof.pool.empty()) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    return e;
  }
  cudaEvent_t e = s.prof.pool.back();
  s.prof.pool.pop_back();
  return e;
}

static void prof_resolve(System& s) {
  CK(cudaStreamSynchronize(s.stream));
  for (size_t k = 0; k < s.prof.kind.size(); k++) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, s.prof.ev[2 * k], s.prof.ev[2 * k + 1]));
    s.prof.ms[s.prof.kind[k]] += ms;
    s.prof.launches[s.prof.kind[k]]++;
    s.prof.pool.push_back(s.prof.ev[2 * k]);
    s.prof.pool.push_back(s.prof.ev[2 * k + 1]);
  }
  s.prof.kind.clear();
  s.prof.ev.clear();
}

void prof_begin(System& s, int kind) {
  (void)kind;
  s.prof.total++;
  if (!s.prof.on) return;
  if (s.prof.kind.size() >= 4096) prof_resolve(s);
  cudaEvent_t e = prof_event(s);
  CK(cudaEventRecord(e, s.stream));
  s.prof.ev.push_back(e);
}

void prof_end(System& s, int kind) {
  if (!s.prof.on) return;
  cudaEvent_t e = prof_event(s);
  CK(cudaEventRecord(e, s.stream));
  s.prof.ev.push_back(e);
  s.prof.kind.push_back(kind);
}

// forgets the timing of the last begin/end pair (a launch that returned at once;
// it still counts as a launch)
void prof_drop_last(System& s) {
  if (!s.prof.on || s.prof.kind.empty()) return;
  s.prof.kind.pop_back();
  for (int k = 0; k < 2; k++) {
    s.prof.pool.push_back(s.prof.ev.back());
    s.prof.ev.pop_back();
  }
}

static double wtime() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

static void option_string(const char* c, char* out) {   // src/global.f90:120-128
  int i;
  for (i = 0; i < 256 && c[i]; i++) out[i] = c[i];
  out[i] = 0;
}

static double layer_rc(System& s, int layer) { return s.useInRc[layer - 1] ? s.InRc : s.Rc; }

// Device pair tables of every layer, in double and in float.
static void upload_models(System& s) {
  int nt = s.ntypes, nl = s.nlayers;
  size_t n = (size_t)nt * nt * nl;
  std::vector<PairEntry<double>> t64(n);
  std::vector<PairEntry<float>> t32(n);
  std::vector<NBParams<double>> c64(nl);
  std::vector<NBParams<float>> c32(nl);
  auto to32 = [](const NBParams<double>& a) {
    NBParams<float> b;
    b.kind = a.kind;
    b.modifier = a.modifier;
    b.eshift = (float)a.eshift; b.fshift = (float)a.fshift; b.Rm = (float)a.Rm; b.Rm2fac = (float)a.Rm2fac;
    b.factor = (float)a.factor; b.eps4 = (float)a.eps4; b.eps24 = (float)a.eps24; b.sigsq = (float)a.sigsq;
    b.prefactor = (float)a.prefactor; b.prefactor6 = (float)a.prefactor6; b.invSigSq = (float)a.invSigSq;
    b.shift = (float)a.shift; b.alpha = (float)a.alpha; b.beta = (float)a.beta; b.Rm2 = (float)a.Rm2;
    b.invRm = (float)a.invRm;
    return b;
  };
  for (int l = 0; l < nl; l++) {
    for (int j = 0; j < nt; j++)
      for (int i = 0; i < nt; i++) {
        size_t q = ((size_t)l * nt + j) * nt + i;
        const PairHost& ph = s.P(i, j, l);
        t64[q].model = ph.model.p;
        t64[q].coulomb = ph.coulomb;
        t64[q].kCoul = ph.kCoul;
        t32[q].model = to32(ph.model.p);
        t32[q].coulomb = ph.coulomb;
        t32[q].kCoul = (float)ph.kCoul;
      }
    c64[l] = s.coul[l].p;
    c32[l] = to32(s.coul[l].p);
  }
  std::vector<uint8_t> inter((size_t)nt * nt);
  for (size_t q = 0; q < inter.size(); q++) inter[q] = (uint8_t)s.interact[q];
  DevModels& d = s.models;
  if (!d.d64) {
    CK(cudaMalloc(&d.d64, sizeof(PairEntry<double>) * n));
    CK(cudaMalloc(&d.d32, sizeof(PairEntry<float>) * n));
    CK(cudaMalloc(&d.coul64, sizeof(NBParams<double>) * nl));
    CK(cudaMalloc(&d.coul32, sizeof(NBParams<float>) * nl));
    CK(cudaMalloc(&d.interact, (size_t)nt * nt));
  }
  CK(cudaMemcpy(d.d64, t64.data(), sizeof(PairEntry<double>) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.d32, t32.data(), sizeof(PairEntry<float>) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.coul64, c64.data(), sizeof(NBParams<double>) * nl, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.coul32, c32.data(), sizeof(NBParams<float>) * nl, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.interact, inter.data(), (size_t)nt * nt, cudaMemcpyHostToDevice));
  s.modelsUploaded = true;
}

static void upload_exclusions(System& s) {
  int N = s.natoms;
  std::vector<int> cnt(N);
  s.hasExclusions = false;
  for (int i = 0; i < N; i++) {
    cnt[i] = s.exLast[i] - s.exFirst[i] + 1;
    if (cnt[i] > 0) s.hasExclusions = true;
  }
  if (!s.hasExclusions) return;
  size_t ni = s.exItem.size() ? s.exItem.size() : 1;
  if (!s.dExFirst) {
    CK(cudaMalloc(&s.dExFirst, sizeof(int) * N));
    CK(cudaMalloc(&s.dExCount, sizeof(int) * N));
  }
  CK(cudaFree(s.dExItem));
  CK(cudaMalloc(&s.dExItem, sizeof(int) * ni));
  std::vector<int> first(N);
  for (int i = 0; i < N; i++) first[i] = s.exFirst[i] - 1;
  CK(cudaMemcpy(s.dExFirst, first.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.dExCount, cnt.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.dExItem, s.exItem.data(), sizeof(int) * s.exItem.size(), cudaMemcpyHostToDevice));
}

// src/EmDeeData.f90:193-223
static void check_actual_interactions(System& s) {
  int nt = s.ntypes, nl = s.nlayers;
  std::vector<char> neutral(nt, 1), inter((size_t)nt * nt * nl, 0);
  for (int a = 0; a < s.natoms; a++)
    if (s.charged[a]) neutral[s.atomType[a] - 1] = 0;
  for (int i = 0; i < nt; i++)
    for (int j = 0; j <= i; j++) {
      char any = 0;
      for (int k = 0; k < nl; k++) {
        PairHost& p = s.P(i, j, k);
        bool no_pair = p.model.kind == MK_PAIR_NONE;
        bool no_coul = s.coul[k].kind == MK_COUL_NONE || !p.coulomb;
        bool coul_only = no_pair && !no_coul;
        bool inert = (no_pair && no_coul) || (coul_only && neutral[i] && neutral[j]);
        inter[((size_t)k * nt + j) * nt + i] = !inert;
        any |= !inert;
      }
      s.T2(s.interact, i, j) = any;
      s.T2(s.interact, j, i) = any;
    }
  for (int k = 0; k < nl; k++) {
    char any = 0;
    for (size_t q = 0; q < (size_t)nt * nt; q++) any |= inter[(size_t)k * nt * nt + q];
    s.pairs_exist[k] = any;
  }
}

static void mark_stale(System& s, tEmDee* md) {
  for (int l = 0; l < s.nlayers; l++) {
    s.forcesUpToDate[l] = 0;
    s.layerEnergy[l].UpToDate = false;
  }
  md->Energy.UpToDate = false;
  s.skinReady = s.packReady = false;
}

// ---- host mirrors of EmDee_memory_address ---------------------------------------

static void mirrors_in(System& s) {
  size_t b = sizeof(double) * 3 * s.natoms;
  if (s.hMirrorR && s.hasR) CK(cudaMemcpyAsync(s.dR, s.hMirrorR, b, cudaMemcpyHostToDevice, s.stream));
  if (s.hMirrorP) CK(cudaMemcpyAsync(s.dP, s.hMirrorP, b, cudaMemcpyHostToDevice, s.stream));
  if (s.hMirrorLayerF)
    CK(cudaMemcpyAsync(s.dLayerF, s.hMirrorLayerF, b * s.nlayers, cudaMemcpyHostToDevice, s.stream));
  else if (s.hMirrorF)
    CK(cudaMemcpyAsync(s.F(), s.hMirrorF, b, cudaMemcpyHostToDevice, s.stream));
}

static void mirrors_out(System& s) {
  size_t b = sizeof(double) * 3 * s.natoms;
  bool any = false;
  if (s.hMirrorR && s.hasR) { CK(cudaMemcpyAsync(s.hMirrorR, s.dR, b, cudaMemcpyDeviceToHost, s.stream)); any = true; }
  if (s.hMirrorP) { CK(cudaMemcpyAsync(s.hMirrorP, s.dP, b, cudaMemcpyDeviceToHost, s.stream)); any = true; }
  if (s.hMirrorLayerF) {
    CK(cudaMemcpyAsync(s.hMirrorLayerF, s.dLayerF, b * s.nlayers, cudaMemcpyDeviceToHost, s.stream));
    any = true;
  } else if (s.hMirrorF) {
    CK(cudaMemcpyAsync(s.hMirrorF, s.F(), b, cudaMemcpyDeviceToHost, s.stream));
    any = true;
  }
  if (any) CK(cudaStreamSynchronize(s.stream));
}

struct MirrorScope {   // copies the host mirrors in at entry and out at exit
  System& s;
  bool active;
  explicit MirrorScope(System& sys) : s(sys), active(sys.hMirrorR || sys.hMirrorP || sys.hMirrorF || sys.hMirrorLayerF) {
    if (active) mirrors_in(s);
  }
  ~MirrorScope() {
    if (active) mirrors_out(s);
  }
};

static void compute_forces_impl(tEmDee* md);

static void initialize_system(tEmDee* md) {   // src/EmDeeCode.f90:916-923 and src/EmDeeData.f90:359-416
  System& s = *sys_of(*md);
  bodies_update(s);
  int bodyDoF = 6 * s.nbodies;
  md->RotDoF = bodyDoF - 3 * s.nbodies;
  md->DoF = 3 * s.nfree + bodyDoF - 3;
  check_actual_interactions(s);
  bool need = false;
  for (int l = 0; l < s.nlayers; l++) need |= s.coul[l].requires_kspace != 0;
  if (need != s.kspace_active) {
    if (s.kspace_active) s.kspace_active = false;
    else fatal("system initialization", "a kspace solver is required, but has not been defined");
  }
  if (s.kspace_active) {   // src/EmDeeData.f90:384-412
    double kspaceRc = 0.0;
    bool found = false;
    for (int l = 0; l < s.nlayers; l++)
      if (s.coul[l].requires_kspace) {
        const double lrc = s.useInRc[l] ? s.InRc : s.Rc;
        if (!found) kspaceRc = lrc;
        else if (lrc != kspaceRc)
          fatal("system initialization", "all layers with ewald-like coulomb models must have the same cutoff");
        found = true;
      }
    ewald_initialize(s, kspaceRc);
  }
  s.initialized = true;
  upload_models(s);
  upload_exclusions(s);
  for (int layer = s.nlayers; layer >= 1; layer--) {
    EmDee_switch_model_layer(md, layer);
    compute_forces_impl(md);
  }
}

// src/EmDeeCode.f90:1215-1277
static void compute_forces_impl(tEmDee* md) {
  System& s = *sys_of(*md);
  if (!s.initialized) fatal("compute forces", "system has not been initialized");
  bool compute = md->Options.Compute;
  double t0 = wtime();
  flush_pending(s);   // deferred boosts use the forces they were issued with
  if (!s.r0Valid && !s.tileTuned && s.precision == 0 && s.pairs_exist[s.layer - 1] && !two_level_active(s)) {
    s.tileTuned = true;
    device_tune_tile(s, pair_lj_only(s), [](System& sys) { device_pair_forces(sys, true); });
  }
  bool rebuild = !s.r0Valid, forcesDone = false;
  if (!rebuild && s.skinReady && s.packReady && s.precision == 0 && s.pairs_exist[s.layer - 1]) {
    // the fused step left the skin decision and the packed positions on the device:
    // the pair kernel runs unless a rebuild is due, and one synchronisation returns
    // both the decision and the sums
    forcesDone = device_pair_forces(s, compute, true);
    rebuild = !forcesDone;
  } else if (!rebuild) {
    rebuild = s.skinReady ? device_skin_from_step(s) : device_skin_check(s);
  } else {
    s.hResult[9] = 1.0;
  }
  if (rebuild) {
    if (two_level_active(s) && s.pairs_exist[s.layer - 1]) {
      // the filtering launch computes this step's forces as well
      device_rebuild_two_level(s, compute);
      forcesDone = true;
    } else {
      device_build_lists(s);
    }
    md->Builds++;
  }
  double t1 = wtime();
  md->Time.Neighbor += t1 - t0;
  if (!forcesDone) {
    // the build packs the FP32 positions for its prefilter; a fused step packs them too
    if (!((rebuild || s.packReady) && s.precision == 0)) device_pack(s);
    device_pair_forces(s, compute);
  }
  s.skinReady = s.packReady = false;
  const double* r = s.hResult;   // Epair, Ecoul, Wpair, Wcoul
  double bonded[5];   // Ebond, Wbond, Eangle, Wangle, Coulomb discounts of bonds and angles
  device_bonded(s, bonded);
  const double Ecoul = r[1] + bonded[4];
  double Elong = 0.0, Wlong = 0.0;
  if (s.coul[s.layer - 1].requires_kspace) {   // src/EmDeeCode.f90:1249-1252
    Elong = ewald_compute(s);
    Wlong = Ecoul + Elong - r[3];
  }
  s.forcesF32 = s.precision == 0 && !s.coul[s.layer - 1].requires_kspace && s.bondedTerms.uploaded == 0;
  md->Virial.Total = r[2] + r[3] + Wlong + bonded[1] + bonded[3];
  md->Virial.Body = 0.0;
  if (s.nbodies != 0) {   // src/EmDeeData.f90:926-953
    md->Virial.Body = bodies_virial(s);
    md->Virial.Total = md->Virial.Total + md->Virial.Body;
  }
  if (compute) {
    md->Energy.Dispersion = r[0];
    md->Energy.Coulomb = Ecoul + Elong;
    md->Energy.Bond = bonded[0];
    md->Energy.Angle = bonded[2];
    md->Energy.Potential = r[0] + Ecoul + Elong + bonded[0] + bonded[2];
    md->Energy.ShadowPotential = md->Energy.Potential;
  }
  md->Energy.UpToDate = compute;
  s.forcesUpToDate[s.layer - 1] = 1;
  s.layerEnergy[s.layer - 1] = md->Energy;
  s.layerVirial[s.layer - 1] = md->Virial;
  double t2 = wtime();
  md->Time.Pair += t2 - t1;
  md->Time.Total = t2 - s.startTime;
}

}  // namespace emdee

using namespace emdee;

extern "C" {

// src/EmDeeCode.f90:69-208
tEmDee EmDee_system(int threads, int layers, double rc, double skin, int N, int* types, double* masses,
                    int* bodies) {
  tEmDee md;
  memset(&md, 0, sizeof md);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    fatal("system setup", "no CUDA device is available to the GB300 EmDee library");
  if (layers < 1) fatal("system setup", "wrong number of model layers");
  if (N < 1) fatal("system setup", "wrong number of atoms");
  System* s = new System;
  s->nthreads = threads < 1 ? 1 : threads;
  s->nlayers = layers;
  s->Rc = rc;
  s->skin = skin;
  s->RcSq = rc * rc;
  s->xRc = rc + skin;
  s->xRcSq = s->xRc * s->xRc;
  s->InRc = s->Rc;
  s->InRcSq = s->RcSq;
  s->xInRcSq = s->xRcSq;
  s->skinSq = skin * skin;
  s->natoms = N;
  if (const char* e = getenv("EMDEE_PRECISION")) s->precision = (!strcmp(e, "fp64") || !strcmp(e, "1")) ? 1 : 0;

  s->atomType.assign(N, 1);
  if (types) {
    int mn = types[0], mx = types[0];
    for (int i = 0; i < N; i++) {
      mn = types[i] < mn ? types[i] : mn;
      mx = types[i] > mx ? types[i] : mx;
    }
    if (mn != 1) fatal("system setup", "wrong specification of atom types");
    s->ntypes = mx;
    for (int i = 0; i < N; i++) s->atomType[i] = types[i];
  }
  s->mass.resize(N);
  s->invMass.resize(N);
  for (int i = 0; i < N; i++) {
    double m = masses ? masses[s->atomType[i] - 1] : 1.0;
    s->mass[i] = m;
    s->invMass[i] = 1.0 / m;
    if (m != 1.0) s->unitMass = false;
  }
  s->totalMass = 0.0;
  if (masses)
    for (int i = 0; i < N; i++) s->totalMass += masses[s->atomType[i] - 1];
  else
    s->totalMass = (double)N;
  s->startTime = wtime();
  s->charge.assign(N, 0.0);
  s->charged.assign(N, 0);

  // rigid bodies (src/EmDeeData.f90:268-355): entries <= 0 or unique are free
  // atoms; other values are renumbered 1..nbodies in order of first appearance
  s->atomBody.assign(N, 0);
  if (bodies) {
    std::vector<int> saved, amount, first;
    for (int i = 0; i < N; i++) {
      int ib = bodies[i], j = -1;
      if (ib <= 0) continue;
      for (size_t k = 0; k < saved.size(); k++)
        if (saved[k] == ib) { j = (int)k; break; }
      if (j < 0) {
        saved.push_back(ib);
        amount.push_back(1);
        first.push_back(i);
      } else {
        amount[j]++;
        s->atomBody[i] = j + 1;
        s->atomBody[first[j]] = j + 1;
      }
    }
    int k = 0;
    for (size_t j = 0; j < saved.size(); j++)
      if (amount[j] > 1) saved[j] = ++k;
    for (int i = 0; i < N; i++)
      if (s->atomBody[i] > 0) s->atomBody[i] = saved[s->atomBody[i] - 1];
    s->nbodies = k;
  }
  for (int i = 0; i < N; i++)
    if (s->atomBody[i] == 0) s->freeList.push_back(i);
  s->nfree = (int)s->freeList.size();
  if (s->nbodies > 0) {
    std::vector<int> cnt(s->nbodies, 0);
    for (int i = 0; i < N; i++)
      if (s->atomBody[i] > 0) cnt[s->atomBody[i] - 1]++;
    s->hBodies.assign(s->nbodies, BodyState());
    int off = 0;
    for (int b = 0; b < s->nbodies; b++) {
      BodyState& B = s->hBodies[b];
      memset(&B, 0, sizeof(BodyState));
      B.first = off;
      B.NP = 0;
      B.dof = 6;
      off += cnt[b];
    }
    s->hBodyAtom.assign(off, 0);
    s->hBodyM.assign(off, 0.0);
    s->hBodyD.assign((size_t)3 * off, 0.0);
    s->hBodyDelta.assign((size_t)3 * off, 0.0);
    for (int i = 0; i < N; i++)
      if (s->atomBody[i] > 0) {
        BodyState& B = s->hBodies[s->atomBody[i] - 1];
        s->hBodyAtom[B.first + B.NP] = i;
        s->hBodyM[B.first + B.NP] = s->mass[i];
        B.NP++;
      }
    for (int b = 0; b < s->nbodies; b++) {
      BodyState& B = s->hBodies[b];
      B.mass = 0.0;
      for (int j = 0; j < B.NP; j++) B.mass += s->hBodyM[B.first + j];
      B.invMass = 1.0 / B.mass;
    }
  }
  {
    int k = s->nbodies;   // free atoms get distinct body indices
    for (int i = 0; i < N; i++)
      if (s->atomBody[i] == 0) s->atomBody[i] = ++k;
  }

  s->exFirst.assign(N, 1);
  s->exLast.assign(N, 0);

  int nt = s->ntypes;
  s->pair.assign((size_t)nt * nt * layers, PairHost());
  for (auto& p : s->pair) p.model = model_new(MC_PAIR, MK_PAIR_NONE, "none");
  s->multilayer.assign((size_t)nt * nt, 0);
  s->overridable.assign((size_t)nt * nt, 1);
  s->interact.assign((size_t)nt * nt, 0);
  s->coul.assign(layers, model_new(MC_COUL, MK_COUL_NONE, "none"));
  s->pairs_exist.assign(layers, 0);
  s->useInRc.assign(layers, 0);
  s->bonded.assign(layers, 1);
  s->forcesUpToDate.assign(layers, 0);
  s->layerEnergy.assign(layers, tEnergy());
  s->layerVirial.assign(layers, tVirial());
  s->layer = 1;

  // device state
  CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  size_t b3 = sizeof(double) * 3 * N;
  CK(cudaMalloc(&s->dR, b3));
  CK(cudaMalloc(&s->dP, b3));
  CK(cudaMalloc(&s->dR0, b3));
  CK(cudaMalloc(&s->dLayerF, b3 * layers));
  CK(cudaMemset(s->dR, 0, b3));
  CK(cudaMemset(s->dP, 0, b3));
  CK(cudaMemset(s->dR0, 0, b3));
  CK(cudaMemset(s->dLayerF, 0, b3 * layers));
  CK(cudaMalloc(&s->dInvMass, sizeof(double) * N));
  CK(cudaMalloc(&s->dCharge, sizeof(double) * N));
  CK(cudaMalloc(&s->dType, sizeof(int) * N));
  CK(cudaMalloc(&s->dBody, sizeof(int) * N));
  CK(cudaMemcpy(s->dInvMass, s->invMass.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
  CK(cudaMemset(s->dCharge, 0, sizeof(double) * N));
  CK(cudaMemcpy(s->dType, s->atomType.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s->dBody, s->atomBody.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
  if (s->nbodies > 0) {
    size_t na = s->hBodyAtom.size();
    CK(cudaMalloc(&s->dBodies, sizeof(BodyState) * s->nbodies));
    CK(cudaMalloc(&s->dBodyAtom, sizeof(int) * na));
    CK(cudaMalloc(&s->dBodyM, sizeof(double) * na));
    CK(cudaMalloc(&s->dBodyD, sizeof(double) * 3 * na));
    CK(cudaMalloc(&s->dBodyDelta, sizeof(double) * 3 * na));
    CK(cudaMemcpy(s->dBodies, s->hBodies.data(), sizeof(BodyState) * s->nbodies, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->dBodyAtom, s->hBodyAtom.data(), sizeof(int) * na, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->dBodyM, s->hBodyM.data(), sizeof(double) * na, cudaMemcpyHostToDevice));
    CK(cudaMemset(s->dBodyD, 0, sizeof(double) * 3 * na));
    CK(cudaMemset(s->dBodyDelta, 0, sizeof(double) * 3 * na));
    CK(cudaMalloc(&s->dFree, sizeof(int) * (s->nfree > 0 ? s->nfree : 1)));
    if (s->nfree > 0) CK(cudaMemcpy(s->dFree, s->freeList.data(), sizeof(int) * s->nfree, cudaMemcpyHostToDevice));
  }
  CK(cudaMallocHost(&s->hResult, sizeof(double) * 64));
  CK(cudaMallocHost(&s->hFlags, sizeof(int) * 16));
  CK(cudaMalloc(&s->dResult, sizeof(double) * 64));
  CK(cudaMalloc(&s->dTicket, sizeof(unsigned int) * 16));
  CK(cudaMemset(s->dTicket, 0, sizeof(unsigned int) * 16));
  memset(s->hResult, 0, sizeof(double) * 64);

  md.Builds = 0;
  md.DoF = 3 * (N - 1);
  md.RotDoF = 0;
  md.Data = s;
  md.Options.Translate = true;
  md.Options.Rotate = true;
  md.Options.RotationMode = 0;
  md.Options.AutoForceCompute = true;
  md.Options.AutoBodyUpdate = true;
  md.Options.Compute = true;
  return md;
}

void EmDee_set_precision(tEmDee md, int mode) {
  System& s = *sys_of(md);
  s.keSpecValid = false;
  if (mode != 0 && mode != 1) fatal("precision setting", "mode must be 0 (mixed) or 1 (fp64)");
  s.precision = mode;
}

void EmDee_set_outer_skin(tEmDee md, double delta) {
  System& s = *sys_of(md);
  s.outerSkin = delta < 0.0 ? -1.0 : delta;
}

long EmDee_outer_builds(tEmDee md) { return sys_of(md)->outerBuilds; }

void EmDee_destroy(tEmDee* md) {
  System* s = sys_of(*md);
  cudaStreamSynchronize(s->stream);
  if (s->ownsRP) {
    cudaFree(s->dR);
    cudaFree(s->dP);
  }
  cudaFree(s->dR0);
  cudaFree(s->dLayerF);
  cudaFree(s->dInvMass);
  cudaFree(s->dCharge);
  cudaFree(s->dType);
  cudaFree(s->dBody);
  if (s->ownsBodies) {
    cudaFree(s->dBodies);
    cudaFree(s->dBodyDelta);
  }
  cudaFree(s->dBodyAtom);
  cudaFree(s->dBodyM);
  cudaFree(s->dBodyD);
  cudaFree(s->dFree);
  cudaFree(s->dBodyScratch);
  ewald_free(*s);
  cudaFree(s->verlet.s0);
  cudaFree(s->verlet.r0);
  cudaFree(s->verlet.q0);
  cudaFree(s->verlet.partB);
  cudaFree(s->verlet.partF);
  cudaFree(s->dExFirst);
  cudaFree(s->dExCount);
  cudaFree(s->dExItem);
  bonded_free(*s);
  Grid& g = s->grid;
  cudaFree(g.dCount); cudaFree(g.dStart); cudaFree(g.dScanTmp); cudaFree(g.dOrig);
  cudaFree(g.dSelf); cudaFree(g.dK); cudaFree(g.dAtomK); cudaFree(g.dPos4); cudaFree(g.dType8);
  cudaFree(g.dRs64); cudaFree(g.dNb); cudaFree(g.dHaloTab); cudaFree(g.dNbCount); cudaFree(g.dNbInner); cudaFree(g.dTileInfo);
  cudaFree(g.dSlotOf); cudaFree(g.dPos0); cudaFree(g.dKeyX); cudaFree(g.dLayout);
  cudaFree(g.dNbOuter); cudaFree(g.dNbCountOuter); cudaFree(g.dROuter);
  cudaFree(s->models.d64); cudaFree(s->models.d32); cudaFree(s->models.coul64); cudaFree(s->models.coul32);
  cudaFree(s->models.interact);
  cudaFree(s->dPartials);
  cudaFree(s->dKE);
  cudaFree(s->dTicket);
  cudaFree(s->dResult);
  cudaFreeHost(s->hResult);
  cudaFreeHost(s->hFlags);
  cudaFreeHost(s->hMirrorR); cudaFreeHost(s->hMirrorP); cudaFreeHost(s->hMirrorF); cudaFreeHost(s->hMirrorLayerF);
  if (s->ownsLbox) delete s->Lbox;
  cudaStreamDestroy(s->stream);
  delete s;
  md->Data = nullptr;
}

// src/EmDeeData.f90:227-264
static void set_pair_type(System& s, int itype, int jtype, int layer, const Model& model, double kCoul) {
  double lrc = layer_rc(s, layer);
  int l = layer - 1;
  if (itype == jtype) {
    PairHost& p = s.P(itype - 1, itype - 1, l);
    p.model = model;
    p.coulomb = kCoul != 0.0;
    if (p.coulomb) p.kCoul = kCoul;
    modifier_setup(p.model, lrc);
    for (int k = 1; k <= s.ntypes; k++)
      if (k != itype && s.T2(s.overridable, itype - 1, k - 1)) {
        PairHost c = pair_container_mix(s.P(k - 1, k - 1, l), p);
        modifier_setup(c.model, lrc);
        s.P(itype - 1, k - 1, l) = c;
        s.P(k - 1, itype - 1, l) = c;
      }
  } else {
    PairHost& p = s.P(itype - 1, jtype - 1, l);
    p.model = model;
    p.coulomb = kCoul != 0.0;
    if (p.coulomb) p.kCoul = kCoul;
    modifier_setup(p.model, lrc);
    s.P(jtype - 1, itype - 1, l) = p;
  }
}

static bool ranged(int i, int imax) { return i > 0 && i <= imax; }

static void finish_pair_setting(System& s, int itype, int jtype, bool multi) {
  s.T2(s.multilayer, itype - 1, jtype - 1) = multi;
  s.T2(s.multilayer, jtype - 1, itype - 1) = multi;
  if (itype == jtype) {
    for (int k = 1; k <= s.ntypes; k++)
      if (k != itype && s.T2(s.overridable, itype - 1, k - 1)) {
        char v = multi ? 1 : s.T2(s.multilayer, k - 1, k - 1);
        s.T2(s.multilayer, itype - 1, k - 1) = v;
        s.T2(s.multilayer, k - 1, itype - 1) = v;
      }
  } else {
    s.T2(s.overridable, itype - 1, jtype - 1) = 0;
    s.T2(s.overridable, jtype - 1, itype - 1) = 0;
  }
}

// src/EmDeeCode.f90:309-359
void EmDee_set_pair_model(tEmDee md, int itype, int jtype, void* model, double kCoul) {
  const char* task = "pair model setup";
  System& s = *sys_of(md);
  if (s.initialized) fatal(task, "cannot set model after coordinates have been defined");
  if (!ranged(itype, s.ntypes) || !ranged(jtype, s.ntypes)) fatal(task, "provided type index is out of range");
  if (!model || ((Model*)model)->cls != MC_PAIR) fatal(task, "a valid pair model must be provided");
  for (int l = 1; l <= s.nlayers; l++) set_pair_type(s, itype, jtype, l, *(Model*)model, kCoul);
  finish_pair_setting(s, itype, jtype, false);
}

// src/EmDeeCode.f90:363-412
void EmDee_set_pair_multimodel(tEmDee md, int itype, int jtype, void* model[], double kCoul[]) {
  const char* task = "pair multimodel setup";
  System& s = *sys_of(md);
  if (s.initialized) fatal(task, "cannot set model after coordinates have been defined");
  if (!ranged(itype, s.ntypes) || !ranged(jtype, s.ntypes)) fatal(task, "provided type index is out of range");
  for (int l = 1; l <= s.nlayers; l++) {
    if (!model[l - 1]) {
      char msg[64];
      snprintf(msg, sizeof msg, "%d valid pair models must be provided", s.nlayers);
      fatal(task, msg);
    }
    if (((Model*)model[l - 1])->cls != MC_PAIR) fatal(task, "a valid pair model must be provided");
    set_pair_type(s, itype, jtype, l, *(Model*)model[l - 1], kCoul[l - 1]);
  }
  finish_pair_setting(s, itype, jtype, true);
}

// src/EmDeeCode.f90:416-444
void EmDee_set_kspace_model(tEmDee md, void* model) {
  const char* task = "kspace model setup";
  System& s = *sys_of(md);
  if (s.initialized) fatal(task, "cannot set model after coordinates have been defined");
  if (!model || ((Model*)model)->cls != MC_KSPACE) fatal(task, "a valid kspace model must be provided");
  s.kspace = *(Model*)model;
  s.kspace_active = true;
}

// src/EmDeeCode.f90:448-482: cutoff_setup and then modifier_setup, in this
// order, exactly as the reference (the second zeroes the shifts set by the first)
void EmDee_set_coul_model(tEmDee md, void* model) {
  const char* task = "coulomb model setup";
  System& s = *sys_of(md);
  if (s.initialized) fatal(task, "cannot set model after coordinates have been defined");
  if (!model || ((Model*)model)->cls != MC_COUL) fatal(task, "a valid coulomb model must be provided");
  for (int l = 1; l <= s.nlayers; l++) {
    double lrc = layer_rc(s, l);
    s.coul[l - 1] = *(Model*)model;
    cutoff_setup(s.coul[l - 1], lrc);
    modifier_setup(s.coul[l - 1], lrc);
  }
  s.multilayer_coulomb = false;
}

// src/EmDeeCode.f90:486-520
void EmDee_set_coul_multimodel(tEmDee md, void* model[]) {
  const char* task = "coulomb multimodel setup";
  System& s = *sys_of(md);
  if (s.initialized) fatal(task, "cannot set model after coordinates have been defined");
  for (int l = 1; l <= s.nlayers; l++) {
    double lrc = layer_rc(s, l);
    if (!model[l - 1]) {
      char msg[64];
      snprintf(msg, sizeof msg, "%d valid coulomb models must be provided", s.nlayers);
      fatal(task, msg);
    }
    if (((Model*)model[l - 1])->cls != MC_COUL) fatal(task, "a valid coulomb model must be provided");
    s.coul[l - 1] = *(Model*)model[l - 1];
    cutoff_setup(s.coul[l - 1], lrc);
    modifier_setup(s.coul[l - 1], lrc);
  }
  s.multilayer_coulomb = true;
}

// src/EmDeeCode.f90:273-305
void EmDee_layer_based_parameters(tEmDee md, double InternalRc, int* Apply, int* Bonded) {
  const char* task = "layer-based parameter setting";
  System& s = *sys_of(md);
  if (s.initialized) fatal(task, "system has already been initialized");
  bool any = false;
  for (int l = 0; l < s.nlayers; l++) {
    s.useInRc[l] = Apply[l] != 0;
    any |= s.useInRc[l] != 0;
  }
  if (any && (InternalRc <= 0.0 || InternalRc > s.Rc)) fatal(task, "invalid internal cutoff specification");
  s.InRc = InternalRc;
  s.InRcSq = InternalRc * InternalRc;
  s.xInRcSq = (InternalRc + s.skin) * (InternalRc + s.skin);
  for (int l = 0; l < s.nlayers; l++) s.bonded[l] = Bonded[l] != 0;
  for (int l = 1; l <= s.nlayers; l++) cutoff_setup(s.coul[l - 1], layer_rc(s, l));
}

// src/EmDeeCode.f90:524-570: sorted, duplicate-free exclusion lists
void EmDee_ignore_pair(tEmDee md, int i, int j) {
  System& s = *sys_of(md);
  if (i == j || !ranged(i, s.natoms) || !ranged(j, s.natoms)) return;
  for (int pass = 0; pass < 2; pass++) {
    int a = pass ? j : i, b = pass ? i : j;
    int first = s.exFirst[a - 1], last = s.exLast[a - 1], pos = last + 1;
    bool found = false;
    for (int k = first; k <= last; k++) {
      if (s.exItem[k - 1] == b) { found = true; break; }
      if (s.exItem[k - 1] > b) { pos = k; break; }
    }
    if (found) continue;
    s.exItem.insert(s.exItem.begin() + (pos - 1), b);
    for (int k = a; k < s.natoms; k++) s.exFirst[k]++;
    for (int k = a - 1; k < s.natoms; k++) s.exLast[k]++;
  }
  // the lists change at the next rebuild, as in the reference
  if (s.initialized) upload_exclusions(s);
}

// src/EmDeeCode.f90:574-655: the item is stored and its atom pairs excluded
void EmDee_add_bond(tEmDee md, int i, int j, void* model) {
  System& s = *sys_of(md);
  if (!ranged(i, s.natoms) || !ranged(j, s.natoms)) fatal("add_bond", "atom index out of range");
  if (!model) fatal("add_bond", "a valid model must be provided");
  const Model& m = *(const Model*)model;
  if (m.cls != MC_BOND) fatal("add_bond", "the provided model must be a bond model");
  BondedTerms::Item b;
  b.i = i - 1;
  b.j = j - 1;
  b.kind = m.kind == MK_BOND_HARMONIC ? 1 : 0;
  b.kf = m.k;
  b.x0 = m.x0;
  s.bondedTerms.bonds.push_back(b);
  EmDee_ignore_pair(md, i, j);
}

void EmDee_add_angle(tEmDee md, int i, int j, int k, void* model) {
  System& s = *sys_of(md);
  if (!ranged(i, s.natoms) || !ranged(j, s.natoms) || !ranged(k, s.natoms))
    fatal("add_angle", "atom index out of range");
  if (!model) fatal("add_angle", "a valid model must be provided");
  const Model& m = *(const Model*)model;
  if (m.cls != MC_ANGLE) fatal("add_angle", "the provided model must be an angle model");
  BondedTerms::Item a;
  a.i = i - 1;
  a.j = j - 1;
  a.k = k - 1;
  a.kind = m.kind == MK_ANGLE_HARMONIC ? 1 : 0;
  a.kf = m.k;
  a.x0 = m.x0;
  s.bondedTerms.angles.push_back(a);
  EmDee_ignore_pair(md, i, j);
  EmDee_ignore_pair(md, i, k);
  EmDee_ignore_pair(md, j, k);
}

void EmDee_add_dihedral(tEmDee md, int i, int j, int k, int l, void* model) {
  System& s = *sys_of(md);
  if (!ranged(i, s.natoms) || !ranged(j, s.natoms) || !ranged(k, s.natoms) || !ranged(l, s.natoms))
    fatal("add_dihedral", "atom index out of range");
  if (!model) fatal("add_dihedral", "a valid model must be provided");
  if (((const Model*)model)->cls != MC_DIHEDRAL) fatal("add_dihedral", "the provided model must be a dihedral model");
  s.bondedTerms.ndihedrals++;
  EmDee_ignore_pair(md, i, j);
  EmDee_ignore_pair(md, i, k);
  EmDee_ignore_pair(md, i, l);
  EmDee_ignore_pair(md, j, k);
  EmDee_ignore_pair(md, j, l);
  EmDee_ignore_pair(md, k, l);
}

// The device-side address of a caller buffer in page-locked host memory (registered
// or allocated through CUDA), or null: kernels then read or write the caller's
// array directly over the host link instead of a copy plus a kernel pass.
static double* pinned_device_pointer(double* address) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, address) != cudaSuccess) {
    cudaGetLastError();   // not a CUDA-known pointer: clear the error
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? (double*)at.devicePointer : nullptr;
}

static bool mirrors_active(const System& s) {
  return s.hMirrorR || s.hMirrorP || s.hMirrorF || s.hMirrorLayerF;
}

// src/EmDeeCode.f90:805-925
void EmDee_upload(tEmDee* md, char* option, double* address) {
  System& s = *sys_of(*md);
  s.keSpecValid = false;
  char item[257];
  option_string(option, item);
  if (!strcmp(item, "momenta")) sys_of(*md)->npend = 0;   // replaced: pending kicks are moot
  else flush_pending(*sys_of(*md));
  if (!address) fatal("upload", "provided address is invalid");
  size_t n3 = (size_t)3 * s.natoms;
  MirrorScope scope(s);
  if (!strcmp(item, "box")) {
    if (!s.Lbox) {
      s.Lbox = new double;
      s.ownsLbox = true;
    }
    *s.Lbox = *address;
    if (s.initialized) mark_stale(s, md);
    else if (s.hasR) initialize_system(md);
  } else if (!strcmp(item, "coordinates")) {
    CK(cudaMemcpyAsync(s.dR, address, sizeof(double) * n3, cudaMemcpyHostToDevice, s.stream));
    if (s.hMirrorR) memcpy(s.hMirrorR, address, sizeof(double) * n3);
    s.hasR = true;
    if (s.initialized) {
      mark_stale(s, md);
      if (md->Options.AutoBodyUpdate) bodies_update(s);
    } else if (s.Lbox) {
      initialize_system(md);
    }
  } else if (!strcmp(item, "momenta")) {
    if (!s.initialized) fatal("upload", "box and coordinates have not been defined");
    // every atom free and a pinned caller buffer: one kernel reads it, stores P and
    // sums the kinetic energy; otherwise a copy, then the sum
    const double* src = s.nbodies == 0 ? pinned_device_pointer(address) : nullptr;
    if (!src) CK(cudaMemcpyAsync(s.dP, address, sizeof(double) * n3, cudaMemcpyHostToDevice, s.stream));
    if (s.hMirrorP) memcpy(s.hMirrorP, address, sizeof(double) * n3);
    double t2[3] = {0, 0, 0}, r2[3] = {0, 0, 0};   // src/EmDeeData.f90:157-189
    if (s.nbodies == 0) {
      // every atom is free: sum on the device, and with FP32-exact forces in place the
      // sums of the boost a velocity-Verlet step would do next (its speculative value)
      const bool spec = s.precision == 0 && s.forcesF32 && s.forcesUpToDate[s.layer - 1] && s.haveLastBoostCF &&
                        !s.phaseShared && !mirrors_active(s);
      if (device_kinetic(s, t2, src, spec ? &s.lastBoostCF : nullptr)) {
        for (int d = 0; d < 3; d++) s.keSpec[d] = s.hResult[56 + d];
        s.keSpecCF = s.lastBoostCF;
        s.keSpecValid = true;
      }
    } else {
      for (int i : s.freeList)
        for (int d = 0; d < 3; d++) t2[d] += s.invMass[i] * (address[3 * i + d] * address[3 * i + d]);
    }
    if (s.nbodies > 0) {
      double k6[6];
      bodies_assign(s, k6);
      for (int d = 0; d < 3; d++) {
        t2[d] += k6[d];
        r2[d] = k6[3 + d];
      }
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
    if (!s.initialized) fatal("upload", "box and coordinates have not been defined");
    CK(cudaMemcpyAsync(s.F(), address, sizeof(double) * n3, cudaMemcpyHostToDevice, s.stream));
    if (s.hMirrorF) memcpy(s.hMirrorF, address, sizeof(double) * n3);
    s.forcesF32 = false;
  } else if (!strcmp(item, "charges")) {
    if (s.initialized) fatal("upload", "cannot set charges after box and coordinates initialization");
    for (int i = 0; i < s.natoms; i++) {
      s.charge[i] = address[i];
      s.charged[i] = std::fabs(address[i]) > 2.220446049250313e-16;
    }
    CK(cudaMemcpyAsync(s.dCharge, s.charge.data(), sizeof(double) * s.natoms, cudaMemcpyHostToDevice, s.stream));
    mark_stale(s, md);
  } else {
    fatal("upload", "invalid option");
  }
  CK(cudaStreamSynchronize(s.stream));
}

// src/EmDeeCode.f90:659-801 (free-atom options)
void EmDee_download(tEmDee md, char* option, double* address) {
  System& s = *sys_of(md);
  char item[257];
  option_string(option, item);
  // Pending kicks change only P: the coordinates and the box leave them pending, and a
  // momenta download of free atoms into a pinned buffer applies them in its own pass
  // (k_kick_out).  Everything else, and every download while host mirrors are in use,
  // applies them first.
  const bool isR = !strcmp(item, "coordinates") || !strcmp(item, "box");
  double* kickOut = nullptr;
  if (!strcmp(item, "momenta") && s.npend > 0 && s.nbodies == 0 && !mirrors_active(s) && address)
    kickOut = pinned_device_pointer(address);
  if (mirrors_active(s) || !(isR || kickOut)) flush_pending(s);
  if (!address) fatal("download", "provided address is invalid");
  size_t b = sizeof(double) * 3 * s.natoms;
  MirrorScope scope(s);
  if (!strcmp(item, "box")) {
    *address = *s.Lbox;
  } else if (!strcmp(item, "coordinates")) {
    if (!s.hasR) fatal("download", "coordinates have not been allocated");
    CK(cudaMemcpyAsync(address, s.dR, b, cudaMemcpyDeviceToHost, s.stream));
  } else if (!strcmp(item, "momenta")) {
    if (kickOut) {
      device_kick_out(s, kickOut);
    } else if (s.nbodies == 0) {
      CK(cudaMemcpyAsync(address, s.dP, b, cudaMemcpyDeviceToHost, s.stream));
    } else {   // free atoms: P; body atoms: particle momenta (src/EmDeeCode.f90:729-741)
      double* tmp;
      CK(cudaMalloc(&tmp, b));
      CK(cudaMemcpyAsync(tmp, s.dP, b, cudaMemcpyDeviceToDevice, s.stream));
      bodies_particle_momenta(s, tmp);
      CK(cudaMemcpyAsync(address, tmp, b, cudaMemcpyDeviceToHost, s.stream));
      CK(cudaStreamSynchronize(s.stream));
      CK(cudaFree(tmp));
    }
  } else if (!strcmp(item, "centersOfMass")) {   // bodies first, then free atoms
    std::vector<double> R((size_t)3 * s.natoms);
    CK(cudaMemcpyAsync(R.data(), s.dR, b, cudaMemcpyDeviceToHost, s.stream));
    bodies_download(s);
    for (int k = 0; k < s.nbodies; k++)
      for (int d = 0; d < 3; d++) address[3 * k + d] = s.hBodies[k].rcm[d];
    for (int j = 0; j < s.nfree; j++)
      for (int d = 0; d < 3; d++) address[3 * (s.nbodies + j) + d] = R[3 * s.freeList[j] + d];
  } else if (!strcmp(item, "quaternions") || !strcmp(item, "quatmom") || !strcmp(item, "quattau")) {
    bodies_download(s);
    for (int k = 0; k < s.nbodies; k++) {
      const BodyState& B = s.hBodies[k];
      if (!strcmp(item, "quaternions")) for (int d = 0; d < 4; d++) address[4 * k + d] = B.q[d];
      else if (!strcmp(item, "quatmom")) for (int d = 0; d < 4; d++) address[4 * k + d] = B.pi[d];
      else {
        double v[3] = {2.0 * B.tau[0], 2.0 * B.tau[1], 2.0 * B.tau[2]};
        rb_C(B.q, v, &address[4 * k]);
      }
    }
  } else if (!strcmp(item, "angmom") || !strcmp(item, "bodycoord") || !strcmp(item, "bodymom") ||
             !strcmp(item, "bodyforces") || !strcmp(item, "torques") || !strcmp(item, "inertia")) {
    bodies_download(s);
    for (int k = 0; k < s.nbodies; k++) {
      const BodyState& B = s.hBodies[k];
      const double* v = !strcmp(item, "angmom") ? B.omega : !strcmp(item, "bodycoord") ? B.rcm :
                        !strcmp(item, "bodymom") ? B.pcm : !strcmp(item, "bodyforces") ? B.F :
                        !strcmp(item, "torques") ? B.tau : B.MoI;
      for (int d = 0; d < 3; d++) address[3 * k + d] = v[d];
    }
  } else if (!strcmp(item, "forces")) {
    if (!s.forcesUpToDate[s.layer - 1]) compute_forces_impl(&md);
    CK(cudaMemcpyAsync(address, s.F(), b, cudaMemcpyDeviceToHost, s.stream));
  } else {
    fatal("download", "invalid option");
  }
  CK(cudaStreamSynchronize(s.stream));
}

// src/EmDeeCode.f90:212-235.  Returns a pinned host mirror of the device array;
// the library copies the mirror to the device when a call starts and back when
// it ends, so the caller may read and write it between calls.
void* EmDee_memory_address(tEmDee md, char* option) {
  System& s = *sys_of(md);
  s.keSpecValid = false;
  flush_pending(s);
  char item[257];
  option_string(option, item);
  size_t b = sizeof(double) * 3 * s.natoms;
  double** mirror = nullptr;
  double* src = nullptr;
  size_t bytes = b;
  if (!strcmp(item, "coordinates")) { mirror = &s.hMirrorR; src = s.dR; }
  else if (!strcmp(item, "momenta")) { mirror = &s.hMirrorP; src = s.dP; }
  else if (!strcmp(item, "forces")) { mirror = &s.hMirrorF; src = s.F(); }
  else if (!strcmp(item, "layerForces")) { mirror = &s.hMirrorLayerF; src = s.dLayerF; bytes = b * s.nlayers; }
  else {
    char msg[300];
    snprintf(msg, sizeof msg, "invalid option %s", item);
    fatal("memory address retrieving", msg);
  }
  if (!*mirror) {
    CK(cudaMallocHost(mirror, bytes));
    CK(cudaMemcpyAsync(*mirror, src, bytes, cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
  }
  return *mirror;
}

// src/EmDeeCode.f90:239-269
void EmDee_share_phase_space(tEmDee mdkeep, tEmDee* mdlose) {
  const char* task = "phase space sharing";
  System &keep = *sys_of(mdkeep), &lose = *sys_of(*mdlose);
  keep.keSpecValid = lose.keSpecValid = false;
  flush_pending(keep);
  flush_pending(lose);
  keep.phaseShared = lose.phaseShared = true;
  if (!(keep.initialized && lose.initialized)) fatal(task, "EmDee system 1 has not been initialized");
  if (keep.natoms != lose.natoms) fatal(task, "different numbers of atoms");
  for (int i = 0; i < keep.natoms; i++) {
    if (keep.atomType[i] != lose.atomType[i]) fatal(task, "atom types do not match");
    if (keep.mass[i] != lose.mass[i]) fatal(task, "atom masses do not match");
    if (keep.atomBody[i] != lose.atomBody[i]) fatal(task, "rigid bodies do not match");
  }
  CK(cudaStreamSynchronize(keep.stream));
  CK(cudaStreamSynchronize(lose.stream));
  if (lose.ownsRP) {
    CK(cudaFree(lose.dR));
    CK(cudaFree(lose.dP));
  }
  lose.dR = keep.dR;
  lose.dP = keep.dP;
  lose.ownsRP = false;
  if (lose.nbodies > 0) {   // the reference aliases the body array as well
    if (lose.ownsBodies) {
      CK(cudaFree(lose.dBodies));
      CK(cudaFree(lose.dBodyDelta));
    }
    lose.dBodies = keep.dBodies;
    lose.dBodyDelta = keep.dBodyDelta;
    lose.ownsBodies = false;
  }
  if (lose.ownsLbox) delete lose.Lbox;
  lose.Lbox = keep.Lbox;
  lose.ownsLbox = false;
  lose.r0Valid = false;
  mdlose->Kinetic.Total = mdkeep.Kinetic.Total;
  for (int d = 0; d < 3; d++) {
    mdlose->Kinetic.TransPart[d] = mdkeep.Kinetic.TransPart[d];
    mdlose->Kinetic.RotPart[d] = mdkeep.Kinetic.RotPart[d];
  }
  mdlose->Kinetic.Rotational = mdkeep.Kinetic.Rotational;
}

// src/EmDeeCode.f90:929-946
void EmDee_switch_model_layer(tEmDee* md, int layer) {
  System& s = *sys_of(*md);
  s.keSpecValid = false;
  s.forcesF32 = false;
  flush_pending(s);   // pending kicks belong to the current layer's forces
  if (layer != s.layer) {
    if (layer < 1 || layer > s.nlayers) fatal("model layer switch", "selected layer is out of range");
    s.layer = layer;
    md->Energy = s.layerEnergy[layer - 1];
    md->Virial = s.layerVirial[layer - 1];
  }
}

// src/EmDeeCode.f90:950-1020 (serial KISS/ziggurat draws on the host, as the reference)
void EmDee_random_momenta(tEmDee* md, double kT, bool adjust, int seed) {
  System& s = *sys_of(*md);
  s.keSpecValid = false;
  s.npend = 0;   // the momenta are replaced
  MirrorScope scope(s);
  int N = s.natoms;
  std::vector<double> P((size_t)3 * N, 0.0);
  double twoKEt[3] = {0, 0, 0}, twoKEr[3] = {0, 0, 0};
  if (s.random.seeding_required) s.random.setup(seed);
  if (s.nbodies != 0) {
    if (!s.initialized) fatal("random_momenta", "coordinates have not defined");
    bodies_download(s);
    for (BodyState& b : s.hBodies) {
      double f = std::sqrt(b.mass * kT), w[3];
      double a0 = s.random.normal(), a1 = s.random.normal(), a2 = s.random.normal();
      b.pcm[0] = f * a0;
      b.pcm[1] = f * a1;
      b.pcm[2] = f * a2;
      double c0 = s.random.normal(), c1 = s.random.normal(), c2 = s.random.normal();
      w[0] = std::sqrt(b.invMoI[0] * kT) * c0;
      w[1] = std::sqrt(b.invMoI[1] * kT) * c1;
      w[2] = std::sqrt(b.invMoI[2] * kT) * c2;
      rb_assign_omega(b, w);
      for (int d = 0; d < 3; d++) {
        twoKEt[d] += b.invMass * (b.pcm[d] * b.pcm[d]);
        twoKEr[d] += b.MoI[d] * (b.omega[d] * b.omega[d]);
      }
    }
  }
  for (int i : s.freeList) {
    double f = std::sqrt(s.mass[i] * kT);
    double a = s.random.normal(), b = s.random.normal(), c = s.random.normal();
    P[3 * i] = f * a;
    P[3 * i + 1] = f * b;
    P[3 * i + 2] = f * c;
    for (int d = 0; d < 3; d++) twoKEt[d] += s.invMass[i] * (P[3 * i + d] * P[3 * i + d]);
  }
  if (adjust) {   // src/EmDeeCode.f90:994-1018
    double vcm[3];
    for (int d = 0; d < 3; d++) {
      double sum = 0.0, sb = 0.0;
      for (int i : s.freeList) sum += P[3 * i + d];
      for (const BodyState& b : s.hBodies) sb += b.pcm[d];
      vcm[d] = (sum + sb) / s.totalMass;
      twoKEt[d] = 0.0;
    }
    for (int i : s.freeList)
      for (int d = 0; d < 3; d++) {
        P[3 * i + d] = P[3 * i + d] - s.mass[i] * vcm[d];
        twoKEt[d] += s.invMass[i] * (P[3 * i + d] * P[3 * i + d]);
      }
    for (BodyState& b : s.hBodies)
      for (int d = 0; d < 3; d++) {
        b.pcm[d] = b.pcm[d] - b.mass * vcm[d];
        twoKEt[d] += b.invMass * (b.pcm[d] * b.pcm[d]);
      }
    double sum = (twoKEt[0] + twoKEr[0]) + (twoKEt[1] + twoKEr[1]) + (twoKEt[2] + twoKEr[2]);
    double factor = std::sqrt((double)(3 * s.nfree + 6 * s.nbodies - 3) * kT / sum);
    for (int i : s.freeList)
      for (int d = 0; d < 3; d++) P[3 * i + d] *= factor;
    for (BodyState& b : s.hBodies) {
      double w[3] = {factor * b.omega[0], factor * b.omega[1], factor * b.omega[2]};
      for (int d = 0; d < 3; d++) b.pcm[d] = factor * b.pcm[d];
      rb_assign_omega(b, w);
    }
    for (int d = 0; d < 3; d++) {
      twoKEt[d] = factor * factor * twoKEt[d];
      twoKEr[d] = factor * factor * twoKEr[d];
    }
  }
  CK(cudaMemcpyAsync(s.dP, P.data(), sizeof(double) * P.size(), cudaMemcpyHostToDevice, s.stream));
  CK(cudaStreamSynchronize(s.stream));
  if (s.nbodies != 0) bodies_upload(s);
  if (s.hMirrorP) memcpy(s.hMirrorP, P.data(), sizeof(double) * P.size());
  for (int d = 0; d < 3; d++) {
    md->Kinetic.RotPart[d] = 0.5 * twoKEr[d];
    md->Kinetic.TransPart[d] = 0.5 * twoKEt[d];
  }
  md->Kinetic.Rotational = md->Kinetic.RotPart[0] + md->Kinetic.RotPart[1] + md->Kinetic.RotPart[2];
  md->Kinetic.Total =
      md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] + md->Kinetic.Rotational;
  md->Kinetic.ShadowKinetic = md->Kinetic.Total;
  md->Kinetic.ShadowRotational = md->Kinetic.Rotational;
  md->Kinetic.UpToDate = true;
}

static double phi(double x) {   // src/math.f90:230-237
  if (std::fabs(x) > 1e-4) return (1.0 - std::exp(-x)) / x;
  return 1.0 + 0.5 * x * ((1.0 / 3.0) * x * (1.0 - 0.25 * x) - 1.0);
}

// src/EmDeeCode.f90:1024-1065
void EmDee_boost(tEmDee* md, double lambda, double alpha, double dt) {
  System& s = *sys_of(*md);
  MirrorScope scope(s);
  double CF = phi(alpha * dt) * dt, CP = 1.0 - alpha * CF;
  CF = lambda * CF;
  bool compute = md->Options.Compute;
  bool translate = md->Options.Translate, rotate = md->Options.Rotate;
  const bool deferrable =
      CP == 1.0 && s.nbodies == 0 && translate && !scope.active && s.initialized && !s.phaseShared;
  // With energies in mixed precision the kick is deferred as well and only its kinetic
  // energy is computed now, by a pass that reads P and F and writes nothing.  A boost
  // that needed new forces sums 2KE for this kick and for a second identical one (the
  // next half-kick of a velocity-Verlet loop) in the same pass; that second value
  // serves the next boost if P, F and the layer are unchanged by then.  (Summing them
  // in the pair kernel's epilogue was measured slower twice: in FP64, its work queued
  // on GB300's narrow FP64 pipe at the end of every block; in float-float, the
  // scattered momentum loads and the extra registers cost the pair kernel 31 us at 1M
  // atoms against 23.5 us for this pass.)
  if (compute && deferrable && s.precision == 0) {
    s.lastBoostCF = CF;
    s.haveLastBoostCF = true;
    double twoKE[3];
    const bool stale = lambda != 0.0 && !s.forcesUpToDate[s.layer - 1];
    const bool spec = s.keSpecValid && !stale && s.keSpecCF == CF;
    s.keSpecValid = false;
    bool newSpec = false;
    if (spec) {
      for (int d = 0; d < 3; d++) twoKE[d] = s.keSpec[d];
    } else {
      if (stale) {   // applies the pending kicks first; the pair launch may queue the pass below
        s.keChainReq = true;
        s.keChainCF = CF;
        s.keChained = false;
        compute_forces_impl(md);
        s.keChainReq = false;
      }
      // no kick pending (new forces, or momenta just uploaded): the two-kick pass, whose
      // second sum also serves an identical boost that follows
      if (s.npend == 0) {
        if (!(stale && s.keChained)) device_kinetic_two(s, CF);
        s.keChained = false;
        for (int d = 0; d < 3; d++) {
          twoKE[d] = s.hResult[48 + d];
          s.keSpec[d] = s.hResult[51 + d];
        }
        newSpec = true;
      } else {
        device_kinetic_pending(s, CF);
        for (int d = 0; d < 3; d++) twoKE[d] = s.hResult[10 + d];
      }
    }
    if (s.npend == 2) flush_pending(s);   // keeps P plus its pending kicks unchanged
    s.pendCF[s.npend++] = CF;
    if (newSpec) {
      s.keSpecCF = CF;
      s.keSpecValid = true;
    }
    for (int d = 0; d < 3; d++) md->Kinetic.TransPart[d] = 0.5 * twoKE[d];
    if (rotate) {
      for (int d = 0; d < 3; d++) md->Kinetic.RotPart[d] = 0.0;
      md->Kinetic.Rotational = 0.0;
    }
    md->Kinetic.Total =
        md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] + md->Kinetic.Rotational;
    md->Kinetic.UpToDate = true;
    return;
  }
  s.keSpecValid = false;
  if (lambda != 0.0 && !s.forcesUpToDate[s.layer - 1]) compute_forces_impl(md);
  // Without energies, a plain kick (CP = 1, free atoms) is deferred to the next
  // kernel that touches P: the fused step of EmDee_displace, or a flush.  The
  // arithmetic and its order are unchanged.
  if (!compute && deferrable && s.forcesUpToDate[s.layer - 1]) {
    if (s.npend == 2) flush_pending(s);
    s.pendCF[s.npend++] = CF;
    md->Kinetic.UpToDate = false;
    return;
  }
  flush_pending(s);
  if (s.nbodies > 0) bodies_boost(s, CP, CF, translate, rotate, compute);
  else if (translate) device_boost(s, CP, CF, compute);
  if (compute) {
    if (translate)
      for (int d = 0; d < 3; d++) md->Kinetic.TransPart[d] = 0.5 * s.hResult[10 + d];
    if (rotate) {
      for (int d = 0; d < 3; d++) md->Kinetic.RotPart[d] = s.nbodies > 0 ? 0.5 * s.hResult[13 + d] : 0.0;
      md->Kinetic.Rotational = md->Kinetic.RotPart[0] + md->Kinetic.RotPart[1] + md->Kinetic.RotPart[2];
    }
    md->Kinetic.Total =
        md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] + md->Kinetic.Rotational;
  }
  md->Kinetic.UpToDate = compute;
}

// src/EmDeeCode.f90:1069-1103
void EmDee_displace(tEmDee* md, double lambda, double alpha, double dt) {
  System& s = *sys_of(*md);
  s.keSpecValid = false;
  MirrorScope scope(s);
  double t0 = wtime(), CR, CP;
  if (alpha != 0.0) {
    CP = phi(alpha * dt) * dt;
    CR = 1.0 - alpha * CP;
    *s.Lbox = CR * *s.Lbox;
  } else {
    CP = dt;
    CR = 1.0;
  }
  CP = lambda * CP;
  if (s.nbodies == 0 && md->Options.Translate && CR == 1.0 && s.initialized) {
    // pending boosts, the move, the skin displacement and the FP32 packing in one pass
    mark_stale(s, md);
    device_step_fused(s, CP);
  } else {
    flush_pending(s);
    if (s.nbodies > 0) bodies_move(s, CR, CP, dt, md->Options.Translate, md->Options.Rotate, md->Options.RotationMode);
    else if (md->Options.Translate) device_move(s, CR, CP);
    mark_stale(s, md);
  }
  md->Time.Motion += wtime() - t0;
}

void EmDee_move(tEmDee* md, double lambda, double alpha, double dt) { EmDee_displace(md, lambda, alpha, dt); }

void EmDee_compute_forces(tEmDee* md) {
  System& s = *sys_of(*md);
  s.keSpecValid = false;
  MirrorScope scope(s);
  compute_forces_impl(md);
}

// Device address of the system's coordinates, momenta or forces (double[N][3], API order),
// for zero-copy use by other CUDA code on the library's stream.  Writes through it bypass
// the library's bookkeeping: upload the array afterwards, or use it only through calls
// that treat it as input (the replica batches).
void* EmDee_device_pointer(tEmDee md, const char* item) {
  System& s = *sys_of(md);
  s.keSpecValid = false;
  flush_pending(s);
  if (!strcmp(item, "coordinates")) return s.dR;
  if (!strcmp(item, "momenta")) return s.dP;
  if (!strcmp(item, "forces")) return s.F();
  fatal("device pointer", "unknown item");
}

// src/EmDeeCode.f90:1107-1211
void EmDee_verlet_step(tEmDee* md, double dt) {
  System& s = *sys_of(*md);
  s.keSpecValid = false;
  MirrorScope scope(s);
  if (!s.initialized) fatal("verlet step", "system has not been initialized");
  flush_pending(s);
  s.skinReady = s.packReady = false;
  const bool compute = md->Options.Compute;
  const int mode = md->Options.RotationMode;
  double t0 = wtime();
  device_verlet_pre(s, dt, compute, mode);
  md->Time.Motion += wtime() - t0;
  compute_forces_impl(md);   // unconditional; other layers keep their flags, as in the reference
  double v[9];
  device_verlet_post(s, dt, compute, mode, v);
  if (compute) {
    for (int d = 0; d < 3; d++) {
      md->Kinetic.TransPart[d] = 0.5 * v[d];
      md->Kinetic.RotPart[d] = 0.5 * v[3 + d];
    }
    md->Kinetic.Rotational = md->Kinetic.RotPart[0] + md->Kinetic.RotPart[1] + md->Kinetic.RotPart[2];
    md->Kinetic.Total =
        md->Kinetic.TransPart[0] + md->Kinetic.TransPart[1] + md->Kinetic.TransPart[2] + md->Kinetic.Rotational;
    md->Energy.ShadowPotential = md->Energy.ShadowPotential - dt * dt * v[8] / 24.0;
    md->Kinetic.ShadowRotational = v[7] / (6.0 * dt);
    md->Kinetic.ShadowKinetic = (v[6] + v[7]) / (6.0 * dt);
  }
  md->Kinetic.UpToDate = compute;
}

// src/EmDeeCode.f90:1281-1395: pair histograms over the current neighbor lists,
// normalised by the ideal-gas shell counts in scaled units
void EmDee_rdf(tEmDee md, int bins, double Rc, int pairs, int itype[], int jtype[], double g[]) {
  const char* task = "radial distribution calculation";
  const double Pi4_3 = 4.188790204786391;
  System& s = *sys_of(md);
  MirrorScope scope(s);
  const int nt = s.ntypes;
  int maxtype = 0;
  for (int p = 0; p < pairs; p++) {
    if (itype[p] < 1 || itype[p] > nt || jtype[p] < 1 || jtype[p] > nt)
      fatal(task, "at least one provided type index is out of range");
    maxtype = std::max(maxtype, std::max(itype[p], jtype[p]));
  }
  if (!s.initialized || !s.r0Valid) fatal(task, "system has not been initialized");
  if (bins < 1) fatal(task, "the number of bins must be positive");
  std::vector<uint8_t> hasPair(nt, 0), pairOn((size_t)nt * nt, 0);
  for (int p = 0; p < pairs; p++) {
    hasPair[itype[p] - 1] = hasPair[jtype[p] - 1] = 1;
    pairOn[(size_t)(itype[p] - 1) * nt + (jtype[p] - 1)] = 1;
    pairOn[(size_t)(jtype[p] - 1) * nt + (itype[p] - 1)] = 1;
  }
  const int ntp = maxtype * (maxtype + 1) / 2;
  std::vector<unsigned long long> counts;
  device_rdf_counts(s, bins, Rc, hasPair, pairOn, ntp, counts);
  const double invL = 1.0 / *s.Lbox, w = Rc * invL / bins;
  for (int p = 0; p < pairs; p++) {
    const int i = itype[p], j = jtype[p];
    long long Ni = 0, Nj = 0;
    for (int a = 0; a < s.natoms; a++) {
      Ni += s.atomType[a] == i;
      Nj += s.atomType[a] == j;
    }
    const int k = std::min(i, j) - 1 + std::max(i, j) * (std::max(i, j) - 1) / 2;   // symm1D - 1
    for (int b = 1; b <= bins; b++) {
      double rdf = (double)counts[(size_t)k * bins + b - 1] / (Pi4_3 * (w * w * w));
      rdf = rdf / (3 * b * (b - 1) + 1);
      g[(size_t)p * bins + b - 1] = (i == j ? 2.0 * rdf : rdf) / (double)(Ni * Nj);
    }
  }
}

void* EmDee_cuda_stream(tEmDee md) { return (void*)sys_of(md)->stream; }

void EmDee_profile(tEmDee md, int on) {
  System& s = *sys_of(md);
  if (s.prof.on && !on) prof_resolve(s);
  s.prof.on = on != 0;
}

int EmDee_kernel_times(tEmDee md, double* ms, long* launches, int n) {
  System& s = *sys_of(md);
  prof_resolve(s);
  int m = n < PK_COUNT ? n : PK_COUNT;
  for (int k = 0; k < m; k++) {
    if (ms) ms[k] = s.prof.ms[k];
    if (launches) launches[k] = s.prof.launches[k];
    s.prof.ms[k] = 0.0;
    s.prof.launches[k] = 0;
  }
  return PK_COUNT;
}

void EmDee_pair_statistics(tEmDee md, long* listed, long* within) {
  device_pair_statistics(*sys_of(md), listed, within);
}

long EmDee_launch_count(tEmDee md) { return sys_of(md)->prof.total; }

int EmDee_tile_edge(tEmDee md) { return sys_of(md)->grid.TB; }

int EmDee_tile_threads(tEmDee md, int kernel) {
  const System& s = *sys_of(md);
  if (s.grid.tileStride <= 0) return 0;
  return kernel == 0 ? build_block_threads(s) : pair_block_threads(s);
}

long EmDee_neighbor_pairs(tEmDee md, int* pairs, long capacity) {
  System& s = *sys_of(md);
  return device_neighbor_pairs(s, pairs, capacity);
}

}  // extern "C"

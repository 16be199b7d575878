// system.hpp -- state of one EmDee system: host-side configuration that mirrors
// the reference's tData (src/EmDeeData.f90:66-151) and the device-resident
// arrays of the GB300 implementation.
//
// Layout in HBM
//   per atom, API (original) order:  R, P, R0 (double[N][3]), F per layer
//       (double[nlayers][N][3]), invMass, charge (double), type, body (int)
//   per slot, tile-sorted order:     orig (slot -> atom), K (int4 image-cell of
//       the atom at the last build), pos4 (float4 cell-local position + charge),
//       type8 (uint8), Rs64 (double[3], FP64 mode), neighbor counts
//   neighbor lists: uint16 halo indices, tile-major ELL blocks
//       nb[(tile * cap + k) * tileStride + local]
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/emdee.h"
#include "pairmath.cuh"
#include "rigid.cuh"

namespace emdee {

[[noreturn]] void fatal(const char* task, const char* msg);
void warn(const char* msg);
void cuda_check(cudaError_t e, const char* what);
#define CK(call) ::emdee::cuda_check((call), #call)

// ---- models -------------------------------------------------------------

enum ModelClass : int { MC_PAIR = 1, MC_COUL, MC_BOND, MC_ANGLE, MC_DIHEDRAL, MC_KSPACE };

// A model handle as delivered to the caller (src/modelClass.f90:51-60).
struct Model {
  int cls = 0, kind = 0;
  char name[24] = {0};
  double epsilon = 0, sigma = 0, lambda = 0, damp = 0, skinWidth = 0, accuracy = 0, k = 0, x0 = 0;
  double skin = 0, RmSq = 0;   // cNonBondedModel fields not used by the kernels
  int shifted = 0, shifted_force = 0, requires_kspace = 0;
  NBParams<double> p{};        // set-up result evaluated by the kernels
};

struct PairHost {   // pairContainer (src/modelClass_pair.f90:60-68)
  Model model;
  int coulomb = 0;
  double kCoul = 0;
};

Model model_new(int cls, int kind, const char* name);
Model lj_setup(double eps, double sig);
Model softcore_setup(double eps, double sig, double lambda);
void modifier_setup(Model& m, double cutoff);
void cutoff_setup(Model& m, double cutoff);
PairHost pair_container_mix(const PairHost& a, const PairHost& b);

// ---- KISS + ziggurat generator (src/math.f90:69-177) -----------------------

struct Kiss {
  bool seeding_required = true;
  int32_t kn[128];
  double wn[128], fn[128];
  uint32_t x, y, z, w;
  void setup(int32_t seed);
  int32_t i32();
  double normal();
};

// ---- neighbor machinery ------------------------------------------------------

struct GridCaps {   // allocated capacities of the grid arrays
  size_t ranks = 0, atoms = 0, tiles = 0, nb = 0, scan = 0, nbOuter = 0, outerAtoms = 0;
};

// Ewald k-space solver (src/kspace_ewald.f90, src/modelClass_kspace.f90):
// host set-up and device arrays.  Cubic boxes only, as the reference's Lbox.
struct Ewald {
  double alpha = 0, beta = 0, kmax = 0, Volume = 0, L = 0;
  int nmax = -1, nvecs = 0, ntypes = 0, nq = 0, nTypePairs = 0;
  std::vector<int> type;                   // charged types (1-based), ascending
  std::vector<int> item, qtype;            // charge list: atom (0-based) and local type, type by type
  std::vector<double> value;               // charges of the list
  std::vector<int> first, last;            // per local type: [first, last) in the list
  std::vector<double> Erigid;              // per type pair (symm1D order): rigid-pair and self discounts
  std::vector<double> lambda, lambda1D;    // [layer][t][u] = kCoul(u, t); [layer][k]
  std::vector<int> n;                      // k-vectors (nvecs x 3 integers)
  std::vector<double> prefac, vec;         // nvecs; 3 x nvecs
  // device
  int *dItem = nullptr, *dQType = nullptr, *dFirst = nullptr, *dLast = nullptr;
  double* dValue = nullptr;
  int4* dN = nullptr;
  double *dPrefac = nullptr, *dVec = nullptr, *dLambda = nullptr;
  double2 *dPartial = nullptr, *dSigma = nullptr;
  double* dEnergyPartial = nullptr;
  size_t partialCap = 0;
};

// scratch of EmDee_verlet_step (verlet.cu): shadow start values and reduction partials
struct VerletScratch {
  double *s0 = nullptr, *r0 = nullptr, *q0 = nullptr, *partB = nullptr, *partF = nullptr;
  size_t s0Cap = 0, r0Cap = 0, q0Cap = 0, partBCap = 0, partFCap = 0;
};

// Bonds and angles (src/structs.f90, src/EmDeeData.f90:443-550): host lists in the
// order they were added (0-based atoms) and their device tables.
struct BondedTerms {
  struct Item {
    int i = 0, j = 0, k = -1, kind = 0;   // kind: 0 none, 1 harmonic
    double kf = 0, x0 = 0;                // force constant, equilibrium length or angle
  };
  std::vector<Item> bonds, angles;
  int ndihedrals = 0;   // stored for their exclusions only
  int uploaded = 0;     // items on the device
  int4* dItem = nullptr;
  double2* dParam = nullptr;
  double *dQQ = nullptr, *dVec = nullptr, *dPartials = nullptr;
  int *dFirst = nullptr, *dEntry = nullptr;
};

struct Grid {
  int M = 0;            // cells per dimension (src/neighbor_lists.f90:185-186)
  int TB = 0;           // tile edge in cells
  int nT = 0;           // tiles per dimension
  int nTiles = 0, nRanks = 0, haloCells = 0;
  int cap = 0;          // neighbor capacity per atom
  int tileStride = 0;   // max atoms per tile, padded to a multiple of 32
  int maxHalo = 0;      // max halo atoms over tiles
  size_t nbBytes = 0;
  int *dCount = nullptr, *dStart = nullptr, *dScanTmp = nullptr;
  int* dOrig = nullptr;
  uint16_t* dSelf = nullptr;   // halo index of each slot in its own tile
  int4* dK = nullptr;
  int4* dAtomK = nullptr;
  int* dSlotOf = nullptr;   // atom -> slot of the last build
  float4* dPos0 = nullptr;     // per atom: packed position (u, charge) at the last build
  float* dKeyX = nullptr;      // sort key of each slot (cell-local x) during a build
  float4* dPos4 = nullptr;
  uint8_t* dType8 = nullptr;
  double* dRs64 = nullptr;
  uint16_t* dNb = nullptr;
  int *dNbCount = nullptr, *dNbInner = nullptr;
  // two-level lists: the outer lists (radius rc + skin + outer skin) of the last
  // outer build, from which the force kernel filters the lists above at rebuilds,
  // and the coordinates of that build
  uint16_t* dNbOuter = nullptr;
  int* dNbCountOuter = nullptr;
  int capOuter = 0;
  double* dROuter = nullptr;
  int* dTileInfo = nullptr;   // per tile: atoms, halo atoms
  int2* dHaloTab = nullptr;   // per tile and halo cell: rank, packed halo coordinates
  int* dLayout = nullptr;      // per tile: halo offsets and first slots of the last build
  size_t layoutCap = 0;
  size_t haloTabCap = 0;
  int tabM = 0, tabTB = 0;    // geometry the halo table was written for
  GridCaps caps;
};

struct DevModels {   // per-layer pair tables uploaded for the kernels
  PairEntry<double>* d64 = nullptr;
  PairEntry<float>* d32 = nullptr;
  NBParams<double>* coul64 = nullptr;
  NBParams<float>* coul32 = nullptr;
  uint8_t* interact = nullptr;
};

// Per-kernel CUDA-event timing (EmDee_profile / EmDee_kernel_times).
enum ProfKind : int { PK_SKIN = 0, PK_BUILD, PK_PACK, PK_PAIR, PK_BOOST, PK_MOVE, PK_COUNT };
struct Prof {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  std::vector<int> kind;          // per pending pair of events
  std::vector<cudaEvent_t> ev;    // start, end, start, end, ...
  double ms[PK_COUNT] = {0};
  long launches[PK_COUNT] = {0};
  long total = 0;                 // kernels launched since the system was created
};

struct System {
  // configuration (src/EmDeeData.f90:66-151)
  int natoms = 0, ntypes = 1, nlayers = 1, layer = 1, nthreads = 1;
  double Rc = 0, skin = 0, RcSq = 0, xRc = 0, xRcSq = 0, skinSq = 0, InRc = 0, InRcSq = 0, xInRcSq = 0;
  double totalMass = 0, startTime = 0;
  double* Lbox = nullptr;   // host scalar, shared by EmDee_share_phase_space
  bool ownsLbox = true;
  bool initialized = false;
  int precision = 0;        // 0 mixed (FP32 pair math), 1 FP64
  Kiss random;

  std::vector<int> atomType, atomBody;
  std::vector<double> mass, invMass, charge;
  std::vector<char> charged;
  int nfree = 0, nbodies = 0;
  bool unitMass = true;   // every mass is exactly 1
  // rigid bodies (src/EmDeeData.f90:268-355): host copies and device mirrors
  std::vector<int> freeList;                  // free atoms, 0-based
  std::vector<BodyState> hBodies;
  std::vector<int> hBodyAtom;                 // flat atom indices of every body (0-based)
  std::vector<double> hBodyM, hBodyD, hBodyDelta;
  BodyState* dBodies = nullptr;
  int *dBodyAtom = nullptr, *dFree = nullptr;
  double *dBodyM = nullptr, *dBodyD = nullptr, *dBodyDelta = nullptr, *dBodyScratch = nullptr;
  int bodyScratchCap = 0;
  bool ownsBodies = true;
  std::vector<int> exFirst, exLast, exItem;   // sorted exclusion lists, 1-based items
  std::vector<PairHost> pair;                 // [layer][jtype][itype]
  std::vector<Model> coul;                    // per layer
  Model kspace;
  bool kspace_active = false;
  Ewald ewald;
  VerletScratch verlet;
  BondedTerms bondedTerms;
  std::vector<char> multilayer, overridable, interact, pairs_exist, useInRc, bonded, forcesUpToDate;
  std::vector<tEnergy> layerEnergy;
  std::vector<tVirial> layerVirial;
  bool multilayer_coulomb = false;
  bool hasR = false;

  // device state
  cudaStream_t stream = nullptr;
  double *dR = nullptr, *dP = nullptr, *dR0 = nullptr, *dLayerF = nullptr;
  bool ownsRP = true;
  double *dInvMass = nullptr, *dCharge = nullptr;
  int *dType = nullptr, *dBody = nullptr;
  int *dExFirst = nullptr, *dExCount = nullptr, *dExItem = nullptr;
  bool hasExclusions = false;
  Grid grid;
  DevModels models;
  bool modelsUploaded = false;
  bool r0Valid = false;        // R0 holds the positions of the last build
  // deferred boosts (P += CF F with CP = 1 and no energies), applied by the next kernel
  // that touches P; the fused move also leaves the skin-check value and the packed
  // FP32 positions of the new coordinates (valid until R or the lists change)
  int npend = 0;
  double pendCF[2] = {0.0, 0.0};
  // kinetic energy of deferred kicks with energies (mixed precision, free atoms): a
  // boost that needed new forces also sums 2KE of P + 2 CF F, the momenta after the
  // next identical half-kick of a velocity-Verlet loop, kept as keSpec until P, F
  // or the layer change
  bool keSpecValid = false;
  bool forcesF32 = false;   // the current layer's forces are exact FP32 values (mixed pair forces only)
  int tileOverride = 0;     // tile edge chosen by device_tune_tile (0: the rule)
  // threads per block of the list build and of the single-type pair kernel, chosen by
  // device_tune_tile with the edge (0: the rule of tile_threads)
  int buildThreads = 0, pairThreads = 0;
  bool tileTuned = false;   // device_tune_tile has run for this system
  double keSpecCF = 0.0, keSpec[3] = {0.0, 0.0, 0.0};
  // CF of the last deferred boost with energies: a momenta upload sums 2KE for an
  // identical kick that follows (keSpec) while it reads the caller's array
  bool haveLastBoostCF = false;
  double lastBoostCF = 0.0;
  // a deferred boost with energies that waits for new forces: the speculative pair
  // launch queues the two-kick kinetic pass for kick keChainCF right behind it and
  // sets keChained when that pass ran (no rebuild was due)
  bool keChainReq = false, keChained = false;
  double keChainCF = 0.0;
  bool skinReady = false, packReady = false;
  bool phaseShared = false;   // R/P aliased with another system (no deferral then)
  const double* pairSkip = nullptr;   // device rebuild flag the mixed pair kernel checks first
  double builtL = 0;           // box length at the last build
  // two-level neighbor lists (EmDee_set_outer_skin): outerSkin < 0 not set, 0 off
  double outerSkin = -1.0;
  bool listsOuter = false;     // the grid holds outer lists (the last full build was an outer one)
  double outerDelta = 0, outerL = 0;   // outer skin and box length of that build
  long outerBuilds = 0;
  int* hFlags = nullptr;       // pinned: [0] largest filtered list of the last filtering launch,
                               // [2..3] largest list and tile-size overflow of the last list build

  // reduction scratch
  double* dPartials = nullptr;   // per tile: Epair, Ecoul, Wpair, Wcoul, pairs within rc
  int partialCap = 0;
  double* dKE = nullptr;         // per block: 2KE x, y, z
  int keCap = 0;
  unsigned int* dTicket = nullptr;
  // results (pinned host copy and device): [0..3] Epair, Ecoul, Wpair, Wcoul, [4] pairs within
  // the cut-off, [6] body virial sum, [8] skin value, [9] rebuild flag, [10..12] 2KE
  // (translational) per dimension, [13..15] 2KE (rotational), [16..21] body 2KE sums
  // (translational, rotational) of one body kernel, [22] k-space energy, [24..32] and
  // [34..38] sums of the Verlet step (bodies, free atoms), [40..41] coverage test of
  // the two-level lists, [48..53] 2KE per dimension after one and after two kicks
  double* hResult = nullptr;
  double* dResult = nullptr;

  Prof prof;

  // host mirrors handed out by EmDee_memory_address
  double *hMirrorR = nullptr, *hMirrorP = nullptr, *hMirrorF = nullptr, *hMirrorLayerF = nullptr;

  double* F() const { return dLayerF + (size_t)3 * natoms * (layer - 1); }
  PairHost& P(int itype, int jtype, int l) {   // 0-based
    return pair[((size_t)l * ntypes + jtype) * ntypes + itype];
  }
  char& T2(std::vector<char>& a, int i, int j) { return a[(size_t)j * ntypes + i]; }
};

System* sys_of(const tEmDee& md);
void prof_begin(System& s, int kind);
void prof_end(System& s, int kind);
void prof_drop_last(System& s);

// ---- device entry points (neighbor.cu, pair_*.cu, motion.cu) ---------------------

// Skin-displacement check of src/neighbor_lists.f90:41-59,184; returns true when
// the lists must be rebuilt.  Synchronizes the stream.
bool device_skin_check(System& s);
// Cell binning, tile sort and neighbor-list build (src/neighbor_lists.f90:63-300).
// With two-level lists active it builds the outer lists (radius rc + skin + outer skin).
void device_build_lists(System& s);
// Tile edge and block sizes tuned by timing builds and pair launches on the system
// (first build, mixed precision); pair(s) computes the forces once on the current lists.
void device_tune_tile(System& s, bool ljOnly, void (*pair)(System&));
// Block sizes of the thread-per-atom list build and of the single-type mixed pair
// kernel on the current lists.
int build_block_threads(const System& s);
int pair_block_threads(const System& s);
// Two-level lists: the outer skin in effect for the system (0 = single-level lists),
// and whether the next rebuild goes through them.
double outer_delta(System& s);
bool two_level_active(System& s);
// A rebuild with two-level lists: if the outer lists still cover every pair within
// rc + skin, the force kernel filters them into new lists while computing this
// step's forces; otherwise an outer build comes first.  Leaves the forces, sums and
// lists of a rebuild (hResult[0..3]).
void device_rebuild_two_level(System& s, bool compute);
// the single-type Lennard-Jones variant of the mixed-precision pair kernel applies
bool pair_lj_only(System& s);
// launches the mixed-precision pair kernel that also filters the outer lists into
// the lists (skip: device flag, the launch returns at once if it is non-zero)
void device_pair_refilter(System& s, bool compute, const double* skip);
// Per-step position packing for the force kernels.
void device_pack(System& s);
// Pair forces, energies and virials of the current layer into s.F();
// leaves Epair, Ecoul, Wpair, Wcoul in hResult after synchronizing.
// Forces of the current layer; energies and virials in hResult[0..3].  speculative
// (mixed precision, after a fused step): the kernel runs only if the step's skin
// check found no rebuild due; returns false if it did not run.
bool device_pair_forces(System& s, bool compute, bool speculative = false);
// P <- CP P + CF F (free atoms); optional 2KE per dimension into hResult[10..12].
void device_boost(System& s, double CP, double CF, bool kinetic);
// 2KE per dimension (hResult[10..12]) of the momenta after the pending kicks and one
// more kick of CF, without changing P (free atoms, mixed precision); synchronizes
void device_kinetic_pending(System& s, double CF);
// 2KE per dimension after one (hResult[48..50]) and after two (hResult[51..53]) kicks
// of CF, no pending kicks, P unchanged (free atoms, mixed precision); synchronizes
void device_kinetic_two(System& s, double CF);
// 2KE per dimension of the momenta, free atoms only (no bodies); src: the momenta are
// read from there (a device-accessible pointer to the caller's pinned buffer) and
// stored into P on the way
// 2KE per dimension of the momenta (read from src, a pinned host buffer, and stored
// into P when given).  With specCF (unit masses) it also sums 2KE of P + specCF F
// into hResult[56..58] and returns true.
bool device_kinetic(System& s, double* twoKE, const double* src = nullptr, const double* specCF = nullptr);
// applies the pending kicks (1 or 2) and writes the momenta to P and to out (a
// device-accessible pointer to the caller's pinned buffer); synchronizes
void device_kick_out(System& s, double* out);
// bonds and angles of the current layer: adds their forces to F and returns
// Ebond, Wbond, Eangle, Wangle and the Coulomb discount energy; false if none ran
bool device_bonded(System& s, double out[5]);
void bonded_free(System& s);
// R <- CR R + CP P / m (free atoms).
void device_move(System& s, double CR, double CP);
// pending boosts + move (CR = 1) + skin displacement + FP32 packing in one pass
void device_step_fused(System& s, double CP);
// applies pending boosts (before anything reads P or replaces F)
void flush_pending(System& s);
bool device_skin_from_step(System& s);
void device_pair_statistics(System& s, long* listed, long* within);
// Rigid bodies (bodies.cu).
void bodies_update(System& s);
void bodies_boost(System& s, double CP, double CF, bool translate, bool rotate, bool kinetic);
void bodies_move(System& s, double CR, double CP, double dt, bool translate, bool rotate, int mode);
double bodies_virial(System& s);
void bodies_assign(System& s, double* k6);
void bodies_particle_momenta(System& s, double* dOut);
void bodies_download(System& s);
void bodies_upload(System& s);
// Neighbor pairs (1-based, i<j) of the current lists.
long device_neighbor_pairs(System& s, int* pairs, long capacity);
// Ewald k-space (ewald.cu): set-up at initialization, energy + forces per call
void ewald_initialize(System& s, double kspaceRc);
double ewald_compute(System& s);
void ewald_free(System& s);
// EmDee_rdf histograms over the current lists (neighbor.cu)
void device_rdf_counts(System& s, int bins, double Rc, const std::vector<uint8_t>& hasPair,
                       const std::vector<uint8_t>& pairOn, int ntp, std::vector<unsigned long long>& counts);
// EmDee_verlet_step halves (verlet.cu)
void device_verlet_pre(System& s, double dt, bool compute, int mode);
void device_verlet_post(System& s, double dt, bool compute, int mode, double* out);

}  // namespace emdee

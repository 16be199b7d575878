/*
 * emdee.h -- C ABI of the GB300-native EmDee hot path (libemdee.so).
 *
 * Every entry point keeps the name, argument order and by-value / by-pointer
 * passing of the reference library's bind(C) interface, so C and Fortran
 * (iso_c_binding, include/emdee.f03) host programs link against it unchanged.
 * Each declaration cites the reference routine it replaces
 * (paths relative to the atoms-ufrj/EmDee tree).
 *
 * Conventions kept from the reference:
 *   - atom and type indices are 1-based;
 *   - per-atom arrays are double[N][3] (Fortran (3,N) column-major);
 *   - option names are NUL-terminated strings of at most 256 characters;
 *   - errors print "Error in <task>: <message>." on stderr and exit(1)
 *     (src/global.f90:51-56); there are no return codes.
 *
 * One struct layout is used everywhere: the one of the reference's Fortran
 * header src/emdee_header.f03:28-84 (tOpts carries AutoForceCompute and
 * tKinetic carries UpToDate).  The offsets are pinned by static asserts below.
 */
#ifndef EMDEE_GB300_H
#define EMDEE_GB300_H

#include <stddef.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double Pair;               /* wall time spent in force computations (s) */
  double Motion;             /* wall time spent in EmDee_displace (s) */
  double Neighbor;           /* wall time spent in neighbor-list handling (s) */
  double Total;              /* time since the system was created (s) */
} tTime;

typedef struct {
  double Potential;          /* total potential energy */
  double Dispersion;         /* pair-model (van der Waals) part */
  double Coulomb;            /* electrostatic part (real space + k-space) */
  double Bond;
  double Angle;
  double Dihedral;
  double ShadowPotential;
  bool   UpToDate;           /* energies were computed at the current state */
} tEnergy;

typedef struct {
  double Total;              /* total kinetic energy */
  double TransPart[3];       /* translational kinetic energy per dimension */
  double Rotational;         /* rotational kinetic energy */
  double RotPart[3];         /* rotational kinetic energy per principal axis */
  double ShadowKinetic;
  double ShadowRotational;
  bool   UpToDate;
} tKinetic;

typedef struct {
  double Total;              /* total internal virial */
  double Body;               /* rigid-body contribution */
} tVirial;

typedef struct {
  bool Translate;            /* translate free atoms and body centres */
  bool Rotate;               /* rotate rigid bodies */
  int  RotationMode;         /* 0 = exact free rotation, n>0 = NO_SQUISH with n substeps */
  bool AutoForceCompute;     /* accepted for layout compatibility; stale forces are always recomputed */
  bool AutoBodyUpdate;       /* rebuild rigid bodies when coordinates are uploaded */
  bool Compute;              /* compute energies (false: forces and virial only) */
} tOpts;

typedef struct {
  int      Builds;           /* number of neighbor-list builds */
  tTime    Time;
  tEnergy  Energy;
  tKinetic Kinetic;
  tVirial  Virial;
  int      DoF;              /* total number of degrees of freedom */
  int      RotDoF;           /* rotational degrees of freedom */
  void*    Data;             /* opaque system handle */
  tOpts    Options;
} tEmDee;

#ifdef __cplusplus
#define EMDEE_STATIC_ASSERT static_assert
#else
#define EMDEE_STATIC_ASSERT _Static_assert
#endif
EMDEE_STATIC_ASSERT(offsetof(tEmDee, Time) == 8, "tEmDee.Time offset");
EMDEE_STATIC_ASSERT(offsetof(tEmDee, Energy) == 40, "tEmDee.Energy offset");
EMDEE_STATIC_ASSERT(offsetof(tEmDee, Kinetic) == 104, "tEmDee.Kinetic offset");
EMDEE_STATIC_ASSERT(offsetof(tEmDee, Virial) == 192, "tEmDee.Virial offset");
EMDEE_STATIC_ASSERT(offsetof(tEmDee, DoF) == 208, "tEmDee.DoF offset");
EMDEE_STATIC_ASSERT(offsetof(tEmDee, Data) == 216, "tEmDee.Data offset");
EMDEE_STATIC_ASSERT(offsetof(tEmDee, Options) == 224, "tEmDee.Options offset");
EMDEE_STATIC_ASSERT(sizeof(tOpts) == 12, "tOpts size");
EMDEE_STATIC_ASSERT(sizeof(tEmDee) == 240, "tEmDee size");

/* ---- system life cycle ------------------------------------------------- */

/* src/EmDeeCode.f90:69-208 (EmDee_system) */
tEmDee EmDee_system(int threads, int layers, double rc, double skin, int N,
                    int* types, double* masses, int* bodies);

/* src/EmDeeCode.f90:212-235 (EmDee_memory_address).  Returns a page-locked host
 * mirror of the device array: the library copies it to the device when a call
 * on this system starts and back when the call ends, so reads and writes
 * between calls act on the system's state as with the reference's pointers. */
void* EmDee_memory_address(tEmDee md, char* option);

/* src/EmDeeCode.f90:239-269 (EmDee_share_phase_space) */
void EmDee_share_phase_space(tEmDee mdkeep, tEmDee* mdlose);

/* src/EmDeeCode.f90:273-305 (EmDee_layer_based_parameters) */
void EmDee_layer_based_parameters(tEmDee md, double InternalRc, int* Apply, int* Bonded);

/* ---- interaction models -------------------------------------------------- */

/* src/EmDeeCode.f90:309-359 (EmDee_set_pair_model) */
void EmDee_set_pair_model(tEmDee md, int itype, int jtype, void* model, double kCoul);

/* src/EmDeeCode.f90:363-412 (EmDee_set_pair_multimodel) */
void EmDee_set_pair_multimodel(tEmDee md, int itype, int jtype, void* model[], double kCoul[]);

/* src/EmDeeCode.f90:416-444 (EmDee_set_kspace_model) */
void EmDee_set_kspace_model(tEmDee md, void* model);

/* src/EmDeeCode.f90:448-482 (EmDee_set_coul_model) */
void EmDee_set_coul_model(tEmDee md, void* model);

/* src/EmDeeCode.f90:486-520 (EmDee_set_coul_multimodel) */
void EmDee_set_coul_multimodel(tEmDee md, void* model[]);

/* src/EmDeeCode.f90:524-570 (EmDee_ignore_pair) */
void EmDee_ignore_pair(tEmDee md, int i, int j);

/* src/EmDeeCode.f90:574-596, 600-624, 628-655 (bonded terms: outside the
 * accelerated path; these exit with an error that says so) */
void EmDee_add_bond(tEmDee md, int i, int j, void* model);
void EmDee_add_angle(tEmDee md, int i, int j, int k, void* model);
void EmDee_add_dihedral(tEmDee md, int i, int j, int k, int l, void* model);

/* ---- data exchange --------------------------------------------------------- */

/* src/EmDeeCode.f90:659-801 (EmDee_download) */
void EmDee_download(tEmDee md, char* option, double* address);

/* src/EmDeeCode.f90:805-925 (EmDee_upload) */
void EmDee_upload(tEmDee* md, char* option, double* address);

/* src/EmDeeCode.f90:929-946 (EmDee_switch_model_layer) */
void EmDee_switch_model_layer(tEmDee* md, int layer);

/* ---- dynamics ---------------------------------------------------------------- */

/* src/EmDeeCode.f90:950-1020 (EmDee_random_momenta; KISS + ziggurat, src/math.f90:69-177) */
void EmDee_random_momenta(tEmDee* md, double kT, bool adjust, int seed);

/* src/EmDeeCode.f90:1024-1065 (EmDee_boost) */
void EmDee_boost(tEmDee* md, double lambda, double alpha, double dt);

/* src/EmDeeCode.f90:1069-1103 (EmDee_displace) */
void EmDee_displace(tEmDee* md, double lambda, double alpha, double dt);

/* Alias of EmDee_displace (src/emdee_header.h:79 names the same operation). */
void EmDee_move(tEmDee* md, double lambda, double alpha, double dt);

/* src/EmDeeCode.f90:1107-1211 (EmDee_verlet_step) */
void EmDee_verlet_step(tEmDee* md, double dt);

/* src/EmDeeCode.f90:1215-1277 (EmDee_compute_forces) */
void EmDee_compute_forces(tEmDee* md);

/* src/EmDeeCode.f90:1281-1395 (EmDee_rdf) */
void EmDee_rdf(tEmDee md, int bins, double Rc, int pairs, int itype[], int jtype[], double g[]);

/* ---- model factories and modifiers --------------------------------------------- */

/* src/modelClass_nonbonded.f90:83-241 (modifiers; each returns a new model) */
void* EmDee_shifted(void* model);
void* EmDee_shifted_force(void* model);
void* EmDee_smoothed(void* model, double skin);
void* EmDee_shifted_smoothed(void* model, double skin);
void* EmDee_square_smoothed(void* model, double skin);
void* EmDee_shifted_square_smoothed(void* model, double skin);

/* src/modelClass_pair.f90:154-159, src/modelClass_coul.f90:134-139 and the
 * bonded model classes ("none" models) */
void* EmDee_pair_none(void);
void* EmDee_coul_none(void);
void* EmDee_bond_none(void);
void* EmDee_angle_none(void);
void* EmDee_dihedral_none(void);

/* Generated factories (src/make_models_module.sh:78-135; argument order is the
 * "!<>" declaration order of each model file). */
void* EmDee_pair_lj_cut(double epsilon, double sigma);                       /* src/pair_lj_cut.f90:52-69 */
void* EmDee_pair_softcore_cut(double epsilon, double sigma, double lambda);  /* src/pair_softcore_cut.f90:58-82 */
void* EmDee_coul_cut(void);                                                  /* src/coul_cut.f90:40-47 */
void* EmDee_coul_sf(void);                                                   /* src/coul_sf.f90:37-50 */
void* EmDee_coul_damped(double damp);                                        /* src/coul_damped.f90:41-57 */
void* EmDee_coul_damped_smoothed(double damp, double skinWidth);             /* src/coul_damped_smoothed.f90:46-64 */
void* EmDee_coul_damped_square_smoothed(double damp, double skinWidth);      /* src/coul_damped_square_smoothed.f90:46-64 */
void* EmDee_coul_square_smoothed(double skinWidth);                          /* src/coul_square_smoothed.f90:43-55 */
void* EmDee_coul_shifted_square_smoothed(double skinWidth);                  /* src/coul_shifted_square_smoothed.f90:43-58 */
void* EmDee_coul_long(void);                                                 /* src/coul_long.f90:37-51 */
void* EmDee_kspace_ewald(double accuracy);                                   /* src/kspace_ewald.f90:60-99 */
void* EmDee_bond_harmonic(double k, double r0);                              /* src/bond_harmonic.f90 */
void* EmDee_angle_harmonic(double k, double theta0);                         /* src/angle_harmonic.f90 */

/* ---- extensions (no counterpart in the reference) ------------------------------- */

/* Pair-arithmetic precision of the force kernels: 0 = FP32 pair math with FP64
 * energy/virial accumulation (default), 1 = FP64 throughout (bit-for-bit the
 * reference's per-pair arithmetic).  The EMDEE_PRECISION environment variable
 * ("mixed" or "fp64") sets the default for systems created afterwards. */
void EmDee_set_precision(tEmDee md, int mode);

/* Two-level neighbor lists (mixed precision, single-type Lennard-Jones, one
 * layer): outer lists of radius rc + skin + delta are built only when atoms have
 * moved too far for them; at every other rebuild the force kernel filters them
 * into the lists the reference builds (same rebuild schedule, same pair sets).
 * delta > 0 enables them, 0 disables them, delta < 0 leaves the default (off, or
 * the EMDEE_OUTER_SKIN environment variable).  They pay when many rebuilds fit in
 * one outer skin (slow dynamics); on a hot fluid they do not. */
void EmDee_set_outer_skin(tEmDee md, double delta);
/* Number of outer builds so far (two-level lists). */
long EmDee_outer_builds(tEmDee md);

/* Writes the current neighbor pairs (1-based, i<j, sorted by i then j) to
 * pairs[2*k], pairs[2*k+1]; returns the number of pairs, or -count when
 * capacity is too small.  Used to compare pair sets with the reference. */
long EmDee_neighbor_pairs(tEmDee md, int* pairs, long capacity);

/* The cudaStream_t on which the system's kernels run (for CUDA-event timing
 * by the caller). */
void* EmDee_cuda_stream(tEmDee md);

/* Turns per-kernel CUDA-event timing on (1) or off (0). */
void EmDee_profile(tEmDee md, int on);

/* Accumulated device time (ms) and launch counts per kernel class since the
 * last call: [0] skin check, [1] list build, [2] position packing, [3] pair
 * forces, [4] boost, [5] move.  Writes min(n, 6) entries, resets them and
 * returns 6. */
int EmDee_kernel_times(tEmDee md, double* ms, long* launches, int n);

/* Half-list statistics: pairs in the current neighbor lists and pairs within
 * the cut-off at the last force evaluation. */
void EmDee_pair_statistics(tEmDee md, long* listed, long* within);

/* Number of CUDA kernels the library has launched for this system. */
long EmDee_launch_count(tEmDee md);

/* Edge, in cells, of the tiles the neighbor lists and force kernels work on: tuned
   on the system's first build in mixed precision (timed list builds and force
   launches; EMDEE_TILE fixes it, EMDEE_AUTOTUNE=0 keeps the rule of atoms per cell). */
int EmDee_tile_edge(tEmDee md);

/* Threads per block of the thread-per-atom list build (kernel 0) and of the
   single-type Lennard-Jones force kernel (kernel 1) on the current tiles: tuned with
   the tile edge (every thread takes the same number of a tile's atoms). */
int EmDee_tile_threads(tEmDee md, int kernel);

/* No counterpart in the reference.  EmDee_boost's momentum update and
 * kinetic-energy sums on caller-owned device arrays, allocating nothing: for
 * callers that cannot call cudaMalloc at that point (when another allocator
 * owns the device memory, or in loops that cannot afford the synchronization
 * cudaMalloc/cudaFree may imply).  Call it from ordinary host code, not from a
 * stream's host function (it makes CUDA calls).  P (double[N][3], updated in
 * place), F (double[N][3]), invMass (double[N], or NULL for unit masses) and
 * twoKE (double[3]: 2KE per dimension) are device pointers; stream is a
 * cudaStream_t (NULL: default).  The reduction scratch is a fixed 28 KB device
 * array held by every GPU that loads the library until exit and shared by all
 * calls: calls that overlap on the GPU race.  The first call on a device looks
 * up that array's address; make it before any stream capture.  N must lie in
 * [1, 715827882].  Returns 0, 1 for a size out of range or a NULL P, F or
 * twoKE, 2 for a CUDA error (reason on stderr). */
int EmDee_boost_noalloc(double* P, const double* F, const double* invMass, int N, double CP, double CF,
                        double* twoKE, void* stream);

/* Releases the system and its device memory (the reference has no destroy). */
void EmDee_destroy(tEmDee* md);

/* Replica batches (no counterpart in the reference, which runs one system per
   call).  EmDee_replicas_create takes n initialized systems (one atom type, no
   charges, no rigid bodies, no exclusions, one layer, mixed precision) and
   returns a batch handle; EmDee_replicas_run advances all of them by `steps`
   velocity-Verlet steps of dt -- the reference loop boost(dt/2), displace(dt),
   boost(dt/2) with neighbor-list rebuilds on the skin check -- in one persistent
   kernel launch, with energies at every nprop-th step of the call, and
   writes Builds, Energy, Virial and Kinetic back into each tEmDee.  The first
   run picks the block size and the pair phase's threads per atom by timing
   candidates on copies of the state (kept per batch shape for the process;
   EMDEE_REPLICA_THREADS=threads[,2] fixes them); every (steps, dt, nprop)
   combination is captured once in a CUDA graph.  Systems keep
   their device arrays: they can be downloaded, or stepped alone, between runs. */
void* EmDee_replicas_create(int n, tEmDee** systems);
void EmDee_replicas_run(void* batch, int steps, double dt, int nprop);
int EmDee_replicas_block_size(void* batch);
/* Threads per atom (1 or 2) of the pair phase chosen with the block size. */
int EmDee_replicas_pair_threads(void* batch);
void EmDee_replicas_destroy(void* batch);
/* Forces, potential energy and virial of every replica at its current positions (no step). */
void EmDee_replicas_evaluate(void* batch);
/* Save positions, forces and energies of every replica; restore those with mask[r] != 0
   (the rejections of hybrid Monte Carlo). */
void EmDee_replicas_checkpoint(void* batch);
void EmDee_replicas_restore(void* batch, const int* mask);
/* Copy "coordinates", "momenta" or "forces" of all replicas to / from one contiguous device
   array [n][N][3]. */
void EmDee_replicas_gather(void* batch, const char* item, double* dst);
void EmDee_replicas_scatter(void* batch, const char* item, const double* src);

/* Device address (double[N][3], API order) of "coordinates", "momenta" or "forces", for
   zero-copy access from other CUDA code (no reference counterpart: the reference keeps its
   arrays in host memory, see EmDee_memory_address). */
void* EmDee_device_pointer(tEmDee md, const char* item);

/* Learned surrogate potential for hybrid Monte Carlo proposals (no reference counterpart):
   per-atom radial descriptors (16 Gaussians x 2 species, smooth cut-off), one
   32-64-64-1 SiLU network per species evaluated on the BF16 tensor cores, forces by the
   adjoint of the descriptors, energy+force training with Adam.  Device arrays are FP64
   [chains][N][3] positions/forces and [chains] energies; parameters are FP32, packed per
   species as W1[32][64], b1[64], W2[64][64], b2[64], w3[64], b3. */
int EmDee_surrogate_param_count(void);
void* EmDee_surrogate_create(int chains, int N, double L, const int* types, double rc, double skin, double mu0,
                             double mu15, double width);
void EmDee_surrogate_set_params(void* s, const float* params);
void EmDee_surrogate_get_params(void* s, float* params);
void EmDee_surrogate_descriptors(void* s, const double* dR, float* dG, int rebuild, void* stream);
int EmDee_surrogate_forces(void* s, const double* dR, double* dF, double* dE, int rebuild, void* stream);
void EmDee_surrogate_atom_outputs(void* s, float* dEatom, float* dEdG, void* stream);
void EmDee_surrogate_gradient(void* s, const double* dR, const double* dEtrue, const double* dFtrue, double wE,
                              double wF, float* dGrad, double* loss, void* stream);
void EmDee_surrogate_adam(void* s, const float* dGrad, double lr, int step, void* stream);
void EmDee_surrogate_trajectory(void* s, double* dR, double* dP, double* dF, double* dE, int n, double dt,
                                void* stream);
void EmDee_surrogate_destroy(void* s);

#ifdef __cplusplus
}
#endif

#endif /* EMDEE_GB300_H */

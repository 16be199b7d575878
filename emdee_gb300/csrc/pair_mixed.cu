// pair_mixed.cu -- pair forces, energies and virials with FP32 pair arithmetic
// and FP64 energy/virial accumulation (src/compute.f90:20-100,
// src/EmDeeData.f90:644-685).
//
// One thread block per tile.  The block stages its halo (tile + 2 cells on each
// side) in shared memory as FP32 positions in a tile-local frame, in units of
// the cell edge, so a pair distance is one subtraction per component with no
// periodic image arithmetic (except when M = 5, where a stencil cell can be a
// non-minimum image).  Each thread owns one atom i and walks its full neighbor
// list (16-bit halo indices, coalesced across the warp), accumulating F_i in
// registers: Newton's third law is not used, so no atomics touch the forces.
// Per-thread energy and virial sums are promoted to FP64 for the block and grid
// reductions.
#include <algorithm>
#include <cstdlib>

#include "f32x2.cuh"
#include "reduce.cuh"
#include "system.hpp"
#include "tile.cuh"

namespace emdee {

// Blocks of the single-type variant: at most PAIR_THREADS threads, each taking the
// same number of the tile's atoms (tile_threads); without a tuned count, as few
// rounds as blocks of PAIR_THREADS_RULE threads allow.
static const int PAIR_THREADS = 512;
static const int PAIR_THREADS_RULE = 256;
// The general variant (VAR 1) may run several threads per atom in blocks of up to
// PAIR_THREADS_GENERAL threads.
static const int PAIR_THREADS_GENERAL = 1024;
#define PAIR_MAX_THREADS (VAR == 1 ? PAIR_THREADS_GENERAL : PAIR_THREADS)
// Register budget: the single-type Lennard-Jones variant gets up to PAIR_MAXNREG
// registers (blocks of at most PAIR_THREADS threads), the general variant, in blocks
// of up to 1024 threads, 64, the filtering launches 128.  Under launch bounds alone
// the compiler held the energy variant at 64; 72 measured fastest on the 1M-atom
// workload (157 vs 165 us per launch; 68: 159 us, 80: 178 us).
#ifndef PAIR_MAXNREG
#define PAIR_MAXNREG 72
#endif
#define PAIR_BOUNDS __maxnreg__(VAR == 1 ? 64 : REFILTER ? 128 : PAIR_MAXNREG)

struct PairArgsF {
  TileGeom g;
  const int2* tab;
  const int* layout;   // halo layout saved by the list build
  const float4* pos4;
  const uint8_t* type8;
  const int* start;
  const int* orig;
  const uint16_t* self;
  const uint16_t* nb;
  const int* count;
  int cap, tileStride, haloCap;
  int tpa, tpaShift;   // threads per atom (a power of 2, at most 8) and its log2
  const PairEntry<float>* table;   // this layer: [itype][jtype] -> pair(jtype, itype)
  const NBParams<float>* coul;
  int ntypes;
  float rc2;     // cutoff^2 in cell units^2
  float invw2;   // 1/w^2, w = L/M (cell edge)
  float invw;
  float Mf;
  double* F;     // forces, API order, double[N][3]
  const double* skip;   // if set and *skip != 0 (a rebuild is due), the launch does nothing
  double* partials;
  unsigned int* ticket;
  double* result;
  double* hostResult;   // pinned host copy of the sums, written by the last block
  // filtering launches (nb, count and cap above describe the outer lists): every
  // entry within rc + skin (FP32 distance, FP64 test of the reference inside the
  // band lo2In..hi2In) goes to the lists written here, in the outer lists' order
  uint16_t* nbIn;
  int* countIn;
  int capIn;
  float lo2In, hi2In;   // cell units^2
  double thrIn;         // (rc + skin)^2 / L^2
  const double* R;
  double L;
  int* innerMax;        // largest filtered list
};

// FP64 distance test of the reference (src/neighbor_lists.f90:247-250) for halo
// index q of the tile whose saved layout is lay.
__device__ __noinline__ bool refilter_exact(const PairArgsF& A, const int* lay, int ai, int q) {
  return exact_inside(A.R, A.L, ai, A.orig[saved_slot(A.g, lay, q)], A.thrIn);
}

// VAR 0: one atom type, Lennard-Jones with modifier MOD, no Coulomb term.
// VAR 1: any types, any pair model and modifier, Coulomb term.
// COUNT: also count the pairs within the cut-off (statistics launches only).
// REFILTER (VAR 0, M > 5): walk the outer lists and write the filtered lists.
// Lists are read 8 entries (16 bytes) per lane at a time, one chunk ahead of
// use; padding entries point at a sentinel halo slot far from every atom, so
// the inner loop needs no bounds test (except when M = 5, where the periodic
// wrap would bring the sentinel back).
template <bool COMPUTE, int VAR, int MOD, bool MINIMG, bool COUNT, bool REFILTER>
__global__ void PAIR_BOUNDS k_pair_mixed(PairArgsF A) {
  // plain Lennard-Jones (the benchmark's model): two list entries per step of the
  // inner loop in packed FP32 arithmetic
#ifdef EMDEE_SCALAR_PAIR   // tuning define: the scalar loop for every variant
  constexpr bool PACKED = false;
#else
  constexpr bool PACKED = VAR == 0 && MOD == NONE && !MINIMG && !COUNT && !REFILTER;
#endif
  // the flag is 0.0 or 1.0: tested on its bits (an FP64 compare in every thread of
  // every block would queue on the slow FP64 pipe)
  if (A.skip != nullptr && __double_as_longlong(*A.skip) != 0) return;
  extern __shared__ __align__(16) unsigned char sraw[];
  const TileGeom g = A.g;
  const int t = blockIdx.x, cells = g.TB * g.TB * g.TB;
  // shared memory: the staged halo (and its sentinel), then the general variant's
  // pair table and halo types; the layout stays in global memory
  float4* hpos = (float4*)sraw;
  PairEntry<float>* tbl = (PairEntry<float>*)(hpos + A.haloCap + 1);
  const int ntab = VAR == 1 ? A.ntypes * A.ntypes : 0;
  uint8_t* htype = (uint8_t*)(tbl + ntab);
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) tbl[k] = A.table[k];
  if (threadIdx.x == 0) {
    hpos[A.haloCap] = make_float4(1e9f, 1e9f, 1e9f, 0.f);
    if (VAR == 1) htype[A.haloCap] = 0;
  }
  const int* lay = A.layout + (size_t)t * (2 * g.haloCells + 1);
  stage_frame_saved(g, lay, A.pos4, hpos, VAR == 1 ? htype : (uint8_t*)nullptr, A.type8);
  __syncthreads();

  NBParams<float> m0 = A.table[0].model;
  if (VAR == 0) m0.modifier = MOD;
  const float sigc = m0.sigsq * A.invw2, eps48 = 2.0f * m0.eps24;
  const f32x2 sigc2 = pk2(sigc, sigc), eps48_2 = pk2(eps48, eps48), meps24_2 = pk2(-m0.eps24, -m0.eps24),
              eps4_2 = pk2(m0.eps4, m0.eps4), meps4_2 = pk2(-m0.eps4, -m0.eps4);
  NBParams<float> coul;
  if (VAR == 1) coul = *A.coul;
  const int tb = A.start[t * cells], te = A.start[(t + 1) * cells];
  const int capC = A.cap >> 3;
  float Ep = 0.f, Ec = 0.f, Wp = 0.f, Wc = 0.f, within = 0.f;
  // tpa consecutive threads share an atom: thread sub takes the chunks sub, sub + tpa, ...
  // and the group's partial forces are summed by shuffles in a fixed order
  const int tpa = VAR == 1 ? A.tpa : 1, tpaShift = VAR == 1 ? A.tpaShift : 0, sub = threadIdx.x & (tpa - 1);
  const unsigned gmask = (0xFFFFFFFFu >> (32 - tpa)) << ((threadIdx.x & 31) & ~(tpa - 1));
  int longestIn = 0;   // REFILTER: longest filtered list of this thread
  for (int li = threadIdx.x >> tpaShift; li < te - tb; li += blockDim.x >> tpaShift) {
    const int si = tb + li;
    const int qi = A.self[si];
    const float4 pi = hpos[qi];
    const int n = min(A.count[si], A.cap);
    const int nch = (n + 7) >> 3;
    const uint4* lp = reinterpret_cast<const uint4*>(A.nb) + ((size_t)t * capC * A.tileStride + li);
    const int ti = VAR == 1 ? htype[qi] : 0;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    f32x2 fx2 = 0ull, fy2 = 0ull, fz2 = 0ull, ep2 = 0ull, wp2 = 0ull;   // PACKED accumulators
#ifdef PAIR_KAHAN
    f32x2 ec2 = 0ull, wc2 = 0ull;   // compensations
#endif
    int nIn = 0;
    uint16_t* myIn = REFILTER ? A.nbIn + ((size_t)t * (A.capIn >> 3) * A.tileStride + li) * 8 : nullptr;
    const int ai = REFILTER ? A.orig[si] : 0;
    uint4 cur = sub < nch ? __ldcs(lp + (size_t)sub * A.tileStride) : make_uint4(0u, 0u, 0u, 0u);
    for (int c = sub; c < nch; c += tpa) {
      const uint4 nxt = (c + tpa < nch) ? __ldcs(lp + (size_t)(c + tpa) * A.tileStride) : cur;
      const unsigned w[4] = {cur.x, cur.y, cur.z, cur.w};
      if (PACKED) {
        // entries 2k (low half of word k) and 2k + 1 (high half) side by side;
        // entries beyond the cut-off (and sentinels) get a zero reciprocal, which
        // zeroes their energy, virial and force without a branch
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float4 pa = hpos[w[k] & 0xFFFF], pb = hpos[w[k] >> 16];
          const f32x2 dx = pk2(pi.x - pa.x, pi.x - pb.x), dy = pk2(pi.y - pa.y, pi.y - pb.y),
                      dz = pk2(pi.z - pa.z, pi.z - pb.z);
          const float2 r2 = up2(fma2(dz, dz, fma2(dy, dy, mul2(dx, dx))));
          const f32x2 inv = pk2(r2.x < A.rc2 ? Ops<float>::rcp(r2.x) : 0.f, r2.y < A.rc2 ? Ops<float>::rcp(r2.y) : 0.f);
          const f32x2 sr2 = mul2(sigc2, inv), sr6 = mul2(mul2(sr2, sr2), sr2);
          const f32x2 W = mul2(sr6, fma2(eps48_2, sr6, meps24_2));
#ifdef PAIR_KAHAN   // tuning define: per-thread compensated (Kahan) energy and virial sums
          {
            const f32x2 mone = pk2(-1.f, -1.f);
            if (COMPUTE) {
              const f32x2 y = fma2(mone, ec2, mul2(sr6, fma2(eps4_2, sr6, meps4_2))), t = add2(ep2, y);
              ec2 = fma2(mone, y, fma2(mone, ep2, t));
              ep2 = t;
            }
            const f32x2 y = fma2(mone, wc2, W), t = add2(wp2, y);
            wc2 = fma2(mone, y, fma2(mone, wp2, t));
            wp2 = t;
          }
#else
          if (COMPUTE) ep2 = fma2(sr6, fma2(eps4_2, sr6, meps4_2), ep2);
          wp2 = add2(wp2, W);
#endif
          const f32x2 sc = mul2(W, inv);
          fx2 = fma2(sc, dx, fx2);
          fy2 = fma2(sc, dy, fy2);
          fz2 = fma2(sc, dz, fz2);
        }
        cur = nxt;
        continue;
      }
#pragma unroll
      for (int e = 0; e < 8; e++) {
        if (MINIMG && c * 8 + e >= n) break;
        const int qj = (w[e >> 1] >> ((e & 1) * 16)) & 0xFFFF;
        const float4 pj = hpos[qj];
        float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        if (MINIMG) {
          dx -= A.Mf * rintf(dx / A.Mf);
          dy -= A.Mf * rintf(dy / A.Mf);
          dz -= A.Mf * rintf(dz / A.Mf);
        }
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (REFILTER && (r2 < A.lo2In || (r2 < A.hi2In && refilter_exact(A, lay, ai, qj)))) {
          if (nIn < A.capIn) myIn[(nIn >> 3) * (A.tileStride * 8) + (nIn & 7)] = (uint16_t)qj;
          nIn++;
        }
        if (VAR == 0) {
          // branch-free: every entry runs the same code; entries beyond the
          // cut-off (and sentinels) are zeroed by selects, so the 8 entries of
          // a chunk form one straight-line block the compiler can interleave
          constexpr bool needR = MOD == SHIFTED_FORCE || MOD == SMOOTHED || MOD == SHIFTED_SMOOTHED;
          const bool in = r2 < A.rc2;
          const float invR2c = Ops<float>::rcp(r2);
          const float invR2 = invR2c * A.invw2;
          const float invR = needR ? sqrtf(invR2) : 1.f;
          // sr2 = sigma^2 / r^2 with r in cell units; E = 4 eps sr6 (sr6 - 1),
          // W = 24 eps sr6 (2 sr6 - 1)
          const float sr2 = sigc * invR2c, sr6 = sr2 * sr2 * sr2;
          float E = sr6 * fmaf(m0.eps4, sr6, -m0.eps4), W = sr6 * fmaf(eps48, sr6, -m0.eps24);
          if (MOD != NONE) modifier_compute(m0, E, W, invR, invR2);
          W = in ? W : 0.f;
          if (COUNT) within += in ? 1.f : 0.f;
          if (COMPUTE) Ep += in ? E : 0.f;
          Wp += W;
          const float s = W * invR2c;
          fx += s * dx;
          fy += s * dy;
          fz += s * dz;
        } else if (r2 < A.rc2) {
          if (COUNT) within += 1.f;
          const float invR2c = Ops<float>::rcp(r2);
          const float invR2 = invR2c * A.invw2;
          const int tj = htype[qj];
          const PairEntry<float>& pe = tbl[ti * A.ntypes + tj];
          const float invR = sqrtf(invR2);
          const bool ijch = pi.w != 0.f && pj.w != 0.f;
          const float Wsum = pair_eval<float, COMPUTE>(pe, coul, ijch, pi.w, pj.w, invR, invR2, Ep, Ec, Wp, Wc);
          const float s = Wsum * invR2c;
          fx += s * dx;
          fy += s * dy;
          fz += s * dz;
        }
      }
      cur = nxt;
    }
    if (REFILTER) {   // sentinel padding of the last chunk, count
      for (int k = nIn; k < A.capIn && (k & 7); k++) myIn[(k >> 3) * (A.tileStride * 8) + (k & 7)] = (uint16_t)A.haloCap;
      A.countIn[si] = nIn;
      longestIn = max(longestIn, nIn);
    }
    if (PACKED) {
      const float2 a = up2(fx2), b = up2(fy2), c = up2(fz2), ee = up2(ep2), ww = up2(wp2);
      fx = a.x + a.y;
      fy = b.x + b.y;
      fz = c.x + c.y;
#ifdef PAIR_KAHAN
      const float2 ce = up2(ec2), cw = up2(wc2);
      if (COMPUTE) Ep += (ee.x - ce.x) + (ee.y - ce.y);
      Wp += (ww.x - cw.x) + (ww.y - cw.y);
#else
      if (COMPUTE) Ep += ee.x + ee.y;
      Wp += ww.x + ww.y;
#endif
    }
    for (int o = tpa >> 1; o > 0; o >>= 1) {
      fx += __shfl_xor_sync(gmask, fx, o);
      fy += __shfl_xor_sync(gmask, fy, o);
      fz += __shfl_xor_sync(gmask, fz, o);
    }
    if (!COUNT && sub == 0) {
      double* Fa = A.F + 3 * (size_t)A.orig[si];
      Fa[0] = f2d_exact(fx * A.invw);
      Fa[1] = f2d_exact(fy * A.invw);
      Fa[2] = f2d_exact(fz * A.invw);
    }
  }
  if (REFILTER) {   // one atomic per warp
    longestIn = __reduce_max_sync(0xffffffffu, longestIn);
    if ((threadIdx.x & 31) == 0) atomicMax(A.innerMax, longestIn);
  }
  // each pair is visited from both atoms: halve the sums.  Sums that are zero by
  // construction (energies without COMPUTE, Coulomb terms of VAR 0, the count
  // without COUNT) skip the reduction.
  const float v[5] = {0.5f * Ep, 0.5f * Ec, 0.5f * Wp, 0.5f * Wc, 0.5f * within};
  constexpr unsigned MASK = (COMPUTE ? (VAR == 1 ? 3u : 1u) : 0u) | (VAR == 1 ? 12u : 4u) | (COUNT ? 16u : 0u);
  grid_reduce_ff<5, PAIR_MAX_THREADS, MASK>(v, reinterpret_cast<float2*>(A.partials), A.ticket, A.result,
                                            A.hostResult);
}

template <bool COMPUTE, int VAR, int MOD, bool MINIMG, bool COUNT, bool REFILTER = false>
static void launch(System& s, PairArgsF& A, size_t smem, int nTiles, int threads) {
  auto kern = k_pair_mixed<COMPUTE, VAR, MOD, MINIMG, COUNT, REFILTER>;
  static size_t configured = 0;
  if (smem > configured) {
    CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
#ifdef EMDEE_MAX_CARVEOUT
    CK(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
#endif
    configured = smem;
  }
  kern<<<nTiles, threads, smem, s.stream>>>(A);
}

template <bool COMPUTE, bool MINIMG, bool REFILTER = false>
static void launch_lj(System& s, PairArgsF& A, size_t smem, int nt, int th, int mod) {
  switch (mod) {
    case NONE: launch<COMPUTE, 0, NONE, MINIMG, false, REFILTER>(s, A, smem, nt, th); break;
    case SHIFTED: launch<COMPUTE, 0, SHIFTED, MINIMG, false, REFILTER>(s, A, smem, nt, th); break;
    case SHIFTED_FORCE: launch<COMPUTE, 0, SHIFTED_FORCE, MINIMG, false, REFILTER>(s, A, smem, nt, th); break;
    case SMOOTHED: launch<COMPUTE, 0, SMOOTHED, MINIMG, false, REFILTER>(s, A, smem, nt, th); break;
    case SHIFTED_SMOOTHED: launch<COMPUTE, 0, SHIFTED_SMOOTHED, MINIMG, false, REFILTER>(s, A, smem, nt, th); break;
    case SQUARE_SMOOTHED: launch<COMPUTE, 0, SQUARE_SMOOTHED, MINIMG, false, REFILTER>(s, A, smem, nt, th); break;
    default: launch<COMPUTE, 0, SHIFTED_SQUARE_SMOOTHED, MINIMG, false, REFILTER>(s, A, smem, nt, th); break;
  }
}

// kernel arguments and shared-memory size of a launch on the current lists
static size_t pair_args(System& s, bool useInRc, double rc2scaled, bool general, PairArgsF& A) {
  Grid& g = s.grid;
  const double L = *s.Lbox, w = L / g.M;
  A.g = make_geom(g.M, g.TB);
  A.tab = g.dHaloTab;
  A.layout = g.dLayout;
  A.pos4 = g.dPos4;
  A.type8 = g.dType8;
  A.start = g.dStart;
  A.orig = g.dOrig;
  A.self = g.dSelf;
  A.nb = g.dNb;
  A.count = useInRc ? g.dNbInner : g.dNbCount;
  A.cap = g.cap;
  A.tileStride = g.tileStride;
  A.haloCap = g.maxHalo;
  A.table = s.models.d32 + (size_t)(s.layer - 1) * s.ntypes * s.ntypes;
  A.coul = s.models.coul32 + (s.layer - 1);
  A.ntypes = s.ntypes;
  A.rc2 = (float)(rc2scaled * (double)g.M * g.M);
  A.invw2 = (float)(1.0 / (w * w));
  A.invw = (float)(1.0 / w);
  A.Mf = (float)g.M;
  A.F = s.F();
  A.skip = s.pairSkip;
  A.partials = s.dPartials;
  A.ticket = s.dTicket;
  A.result = s.dResult;
  A.hostResult = s.hResult;
  A.nbIn = nullptr;
  A.countIn = nullptr;
  A.capIn = 0;
  A.lo2In = A.hi2In = 0.f;
  A.thrIn = 0.0;
  A.R = nullptr;
  A.L = L;
  A.innerMax = nullptr;
  size_t smem = (size_t)(g.maxHalo + 1) * sizeof(float4);
  if (general) smem += sizeof(PairEntry<float>) * s.ntypes * s.ntypes + g.maxHalo + 17;
  return smem;
}

int pair_block_threads(const System& s) {
  return s.pairThreads > 0 ? std::min(s.pairThreads, PAIR_THREADS) : tile_threads(s.grid.tileStride, 0, PAIR_THREADS_RULE);
}

// variant: 0 single-type Lennard-Jones without charges, 1 general, 2 pair count only
void device_pair_forces_mixed(System& s, bool compute, bool useInRc, double rc2scaled, int variant) {
  Grid& g = s.grid;
  const double L = *s.Lbox;
  PairArgsF A;
  const size_t smem = pair_args(s, useInRc, rc2scaled, variant != 0, A);
  const bool mi = g.M == 5;
  // Threads per atom: systems too small to fill the GPU with one thread per atom
  // (fewer than ~2048 threads per SM) and with long lists (more than 48 entries per
  // thread) split each list over 2, 4 or 8 threads of a warp (general variant only,
  // blocks of up to 1024 threads).  Threads per block: the tile's largest atom count
  // times that, or fewer with several atoms per thread (EMDEE_PAIR_THREADS), the
  // single-type variant in even rounds (pair_block_threads).
  const int maxTh = variant == 0 ? PAIR_THREADS : PAIR_THREADS_GENERAL;
  const double L3 = L * L * L, expected = s.natoms / L3 * 4.18879020478639 * s.xRcSq * s.xRc;
  int tpa = 1, shift = 0;
  if (variant != 0)
    while (tpa < 8 && g.tileStride * tpa * 2 <= maxTh && (double)s.natoms * tpa * 2 <= 152.0 * 2048 &&
           expected / (tpa * 2) >= 48) {
      tpa *= 2;
      shift++;
    }
  A.tpa = tpa;
  A.tpaShift = shift;
  static const int thEnv = getenv("EMDEE_PAIR_THREADS") ? atoi(getenv("EMDEE_PAIR_THREADS")) : 0;
  const int th = std::max(halo_min_threads(A.g), thEnv >= 32 && thEnv % 32 == 0 ? std::min(thEnv, maxTh)
                                                 : variant == 0 ? pair_block_threads(s)
                                                                : std::min(maxTh, std::max(32, g.tileStride * tpa)));
  const int nt = g.nTiles;
  if (variant == 0) {
    const int mod = s.P(0, 0, s.layer - 1).model.p.modifier;
    if (compute) { if (mi) launch_lj<true, true>(s, A, smem, nt, th, mod); else launch_lj<true, false>(s, A, smem, nt, th, mod); }
    else { if (mi) launch_lj<false, true>(s, A, smem, nt, th, mod); else launch_lj<false, false>(s, A, smem, nt, th, mod); }
  } else if (variant == 1) {
    if (compute) { if (mi) launch<true, 1, -1, true, false>(s, A, smem, nt, th); else launch<true, 1, -1, false, false>(s, A, smem, nt, th); }
    else { if (mi) launch<false, 1, -1, true, false>(s, A, smem, nt, th); else launch<false, 1, -1, false, false>(s, A, smem, nt, th); }
  } else {
    if (mi) launch<false, 1, -1, true, true>(s, A, smem, nt, th); else launch<false, 1, -1, false, true>(s, A, smem, nt, th);
  }
  CK(cudaGetLastError());
}

// The pair kernel over the outer lists (single-type Lennard-Jones, M > 5): forces
// as above, and every outer entry within rc + skin written to the lists (their
// capacity g.cap, largest list into the grid's info array).
void device_pair_refilter(System& s, bool compute, const double* skip) {
  Grid& g = s.grid;
  const double L = *s.Lbox, invL2 = 1.0 / (L * L);
  const bool useInRc = s.useInRc[s.layer - 1] != 0;
  PairArgsF A;
  const size_t smem = pair_args(s, false, (useInRc ? s.InRcSq : s.RcSq) * invL2, false, A);
  A.nb = g.dNbOuter;
  A.count = g.dNbCountOuter;
  A.cap = g.capOuter;
  A.skip = skip;
  A.tpa = 1;
  A.tpaShift = 0;
  A.nbIn = g.dNb;
  A.countIn = g.dNbCount;
  A.capIn = g.cap;
  A.thrIn = s.xRcSq * invL2;   // src/neighbor_lists.f90:213-214
  const double M2 = (double)g.M * g.M;
  A.lo2In = (float)(A.thrIn * M2 * (1.0 - LIST_BAND));
  A.hi2In = (float)(A.thrIn * M2 * (1.0 + LIST_BAND));
  A.R = s.dR;
  A.innerMax = g.dTileInfo + 2 * g.nTiles + 4;
  const int th = std::max(halo_min_threads(A.g), tile_threads(g.tileStride, 0, PAIR_THREADS_RULE));
  const int mod = s.P(0, 0, s.layer - 1).model.p.modifier;
  if (compute) launch_lj<true, false, true>(s, A, smem, g.nTiles, th, mod);
  else launch_lj<false, false, true>(s, A, smem, g.nTiles, th, mod);
  CK(cudaGetLastError());
}

}  // namespace emdee

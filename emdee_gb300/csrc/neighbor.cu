// neighbor.cu -- skin-displacement check, cell binning into tiles and the
// Verlet neighbor-list build (src/neighbor_lists.f90).
//
// The pair set is the reference's: every pair (i, j) whose minimum-image
// distance, computed from scaled FP64 coordinates exactly as in
// src/neighbor_lists.f90:247-250 (Rs = R/L, d = Rs_i - Rs_j, d -= anint(d),
// r2 = dx^2 + dy^2 + dz^2), is below (rc+skin)^2/L^2, that is not excluded
// (EmDee_ignore_pair), not in the same rigid body and whose types interact.
// An FP32 distance in a tile-local frame decides every candidate that is
// clearly inside or outside; candidates within a relative 4e-5 of the
// threshold are decided by the FP64 test.  This file is compiled with
// -fmad=false so the FP64 test rounds like the reference.
//
// Unlike the reference's half lists, the lists are full (each pair appears in
// the lists of both atoms), so the force kernel owns every atom's force and
// needs no atomics.
#include <algorithm>
#include <cmath>
#include <vector>

#include "system.hpp"
#include "tile.cuh"

namespace emdee {

static const int NDIV = 2;   // src/EmDeeData.f90:33
static const double BAND = LIST_BAND;

// ---------------------------------------------------------------------------------
// skin check: maximum_approach_sq (src/neighbor_lists.f90:41-59)
//
// The reference scans atoms in order, refreshing "next" only when a new
// maximum appears.  Its result is max + 2 sqrt(max*next) + next, where
// next = the largest value before the first occurrence of the maximum (or the
// maximum itself when that occurrence is atom 1).  (m, p) pairs over
// contiguous index ranges combine associatively:
//   (mA,pA) . (mB,pB) = mB > mA ? (mB, max(mA, pB)) : (mA, pA)
// ---------------------------------------------------------------------------------

// Values are squared displacements (>= 0), so their IEEE-754 bit patterns order
// like the values: the combine runs on 64-bit integers (-1 = none) instead of
// the slow FP64 pipe.
struct MaxPrev {
  long long m, p;   // bit patterns; p < 0: no element precedes the first maximum
};

__device__ __forceinline__ MaxPrev mp_combine(MaxPrev a, MaxPrev b) {
  if (b.m > a.m) return MaxPrev{b.m, a.m > b.p ? a.m : b.p};
  return a;
}

static const int SKIN_THREADS = 256, SKIN_CHUNKS = 8;   // each warp: 8 x 32 consecutive atoms

__device__ __forceinline__ MaxPrev warp_ordered_combine(MaxPrev acc) {
  // after the loop lane 0 holds the combination of lanes 0..31 in lane order
  const int lane = threadIdx.x & 31;
  for (int o = 1; o < 32; o <<= 1) {
    MaxPrev other{(long long)__shfl_down_sync(0xffffffffu, (unsigned long long)acc.m, o),
                  (long long)__shfl_down_sync(0xffffffffu, (unsigned long long)acc.p, o)};
    if ((lane & (2 * o - 1)) == 0) acc = mp_combine(acc, other);
  }
  return acc;
}

__global__ void __launch_bounds__(SKIN_THREADS) k_skin(const double* __restrict__ R, const double* __restrict__ R0,
                                                       int N, double skinSq, longlong2* partial, unsigned int* ticket,
                                                       double* result) {
  __shared__ MaxPrev wsum[SKIN_THREADS / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int base = (blockIdx.x * (SKIN_THREADS / 32) + warp) * 32 * SKIN_CHUNKS;
  MaxPrev run{-1, -1};
  for (int c = 0; c < SKIN_CHUNKS; c++) {
    const int i = base + c * 32 + lane;
    MaxPrev v{-1, -1};
    if (i < N) {
      double d0 = R[3 * i] - R0[3 * i], d1 = R[3 * i + 1] - R0[3 * i + 1], d2 = R[3 * i + 2] - R0[3 * i + 2];
      v.m = __double_as_longlong(d0 * d0 + d1 * d1 + d2 * d2);
    }
    v = warp_ordered_combine(v);
    run = mp_combine(run, v);   // meaningful in lane 0
  }
  if (lane == 0) wsum[warp] = run;
  __syncthreads();
  if (threadIdx.x == 0) {
    MaxPrev b = wsum[0];
    for (int w = 1; w < SKIN_THREADS / 32; w++) b = mp_combine(b, wsum[w]);
    partial[blockIdx.x] = make_longlong2(b.m, b.p);
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // last block: each warp combines a contiguous range of block partials in
  // order, then warp results are combined in order
  const int nb = gridDim.x, per = (nb + SKIN_THREADS - 1) / SKIN_THREADS;
  MaxPrev acc{-1, -1};
  for (int k = 0; k < per; k++) {
    int b = threadIdx.x * per + k;
    if (b < nb) {
      longlong2 v = __ldcg(&partial[b]);
      acc = mp_combine(acc, MaxPrev{v.x, v.y});
    }
  }
  acc = warp_ordered_combine(acc);
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    MaxPrev b = wsum[0];
    for (int w = 1; w < SKIN_THREADS / 32; w++) b = mp_combine(b, wsum[w]);
    double maximum = __longlong_as_double(b.m), next = __longlong_as_double(b.p < 0 ? b.m : b.p);
    double value = maximum + 2 * sqrt(maximum * next) + next;
    result[8] = value;
    result[9] = value > skinSq ? 1.0 : 0.0;
    *ticket = 0;
  }
}

static void ensure_partials(System& s, int n) {
  if (s.partialCap < n) {
    CK(cudaFree(s.dPartials));
    s.partialCap = std::max(n, 1024);
    CK(cudaMalloc(&s.dPartials, sizeof(double) * 5 * s.partialCap));
  }
}

bool device_skin_check(System& s) {
  int N = s.natoms;
  int blocks = (N + SKIN_THREADS * SKIN_CHUNKS - 1) / (SKIN_THREADS * SKIN_CHUNKS);
  ensure_partials(s, blocks);
  prof_begin(s, PK_SKIN);
  k_skin<<<blocks, SKIN_THREADS, 0, s.stream>>>(s.dR, s.dR0, N, s.skinSq, (longlong2*)s.dPartials, s.dTicket,
                                                 s.dResult);
  CK(cudaGetLastError());
  prof_end(s, PK_SKIN);
  CK(cudaMemcpyAsync(s.hResult + 8, s.dResult + 8, 2 * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
  CK(cudaStreamSynchronize(s.stream));
  return s.hResult[9] != 0.0;
}

// ---------------------------------------------------------------------------------
// binning (src/neighbor_lists.f90:122-128) and tile sort
// ---------------------------------------------------------------------------------

// FP32 rounding of a double (nearest even) on the integer pipes when the result
// is a normal float, else the hardware conversion
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return d2f_normal(b) ? __uint_as_float(d2f_bits(b)) : (float)x;
}

// value of an integer-valued double with |f| < 2^31, from its bits (no FP64 pipe)
__device__ __forceinline__ int dint_exact(double f) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(f);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e < 0) return 0;
  const int v = (int)(((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) >> (52 - e));
  return (b >> 63) ? -v : v;
}

// FP32 copy of a charge, zero below the reference's threshold (|q| > epsilon,
// src/EmDeeCode.f90:879-880), compared and converted on the integer pipes
__device__ __forceinline__ float charge_f32(double q) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(q) & 0x7FFFFFFFFFFFFFFFull;
  return b > 0x3CB0000000000000ull ? d2f(q) : 0.0f;   // 0x3CB0... = 2^-52
}

// Per atom (API order): the image-resolved cell K = floor(M R / L) of each
// coordinate, the cell's rank, the cell-local FP32 position u = M R/L - K with the
// charge (the build-time reference pos0 of the packing), the coordinates R0 of
// this build for the skin check, and the atom's place among its cell's atoms.
// M R/L is one FP64 product per coordinate; its floor and remainder are the only
// other FP64 operations (the remainder is exact), and every later stage of the
// build reads u instead of recomputing it.  A cell index that differs from the
// reference's int(M (R/L - floor(R/L))) by rounding at a cell boundary changes
// only the order of candidates, not the pair set.
__global__ void k_assign(const double* __restrict__ R, const double* __restrict__ charge, int N, double scale,
                         TileGeom g, int4* atomK, int* count, int* inCell, float4* pos0, double* __restrict__ R0) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  int c[3], K[3];
  float u[3];
  for (int d = 0; d < 3; d++) {
    const double r = R[3 * a + d], t = r * scale, fl = floor(t);
    K[d] = dint_exact(fl);
    int ci = K[d] % g.M;
    c[d] = ci < 0 ? ci + g.M : ci;
    u[d] = d2f(t - fl);
    R0[3 * a + d] = r;
  }
  int rank = cell_rank(g, c[0], c[1], c[2]);
  atomK[a] = make_int4(K[0], K[1], K[2], rank);
  pos0[a] = make_float4(u[0], u[1], u[2], charge_f32(charge[a]));
  // one atomic per distinct cell of the warp (neighbouring atoms often share a
  // cell); each atom keeps its place among the cell's atoms for the scatter
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, rank);
  const int leader = __ffs(peers) - 1, lane = threadIdx.x & 31;
  int base = 0;
  if (lane == leader) base = atomicAdd(&count[rank], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  inCell[a] = base + __popc(peers & ((1u << lane) - 1u));
}

// three-phase device-wide exclusive scan (counts -> starts), starts[n] = total
static const int SCAN_THREADS = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void k_scan_local(const int* in, int* out, int n, int* blockSums) {
  __shared__ int buf[SCAN_TILE];
  __shared__ int ws[33];
  int base = blockIdx.x * SCAN_TILE;
  for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS) buf[k] = base + k < n ? in[base + k] : 0;
  __syncthreads();
  int total = block_exclusive_scan<SCAN_ITEMS>(buf, SCAN_TILE, ws);
  for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS)
    if (base + k < n) out[base + k] = buf[k];
  if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int* blockSums, int nb, int* out, int n) {
  __shared__ int ws[33];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += SCAN_TILE) {
    __shared__ int buf[SCAN_TILE];
    for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS) buf[k] = base + k < nb ? blockSums[base + k] : 0;
    __syncthreads();
    int total = block_exclusive_scan<SCAN_ITEMS>(buf, SCAN_TILE, ws);
    for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS)
      if (base + k < nb) blockSums[base + k] = buf[k] + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_scan_add(int* out, int n, const int* blockSums) {
  int base = blockIdx.x * SCAN_TILE, add = blockSums[blockIdx.x];
  for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS)
    if (base + k < n) out[base + k] += add;
}

static void device_scan(System& s, const int* in, int* out, int n) {
  int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_local<<<nb, SCAN_THREADS, 0, s.stream>>>(in, out, n, s.grid.dScanTmp);
  k_scan_sums<<<1, SCAN_THREADS, 0, s.stream>>>(s.grid.dScanTmp, nb, out, n);
  k_scan_add<<<nb, SCAN_THREADS, 0, s.stream>>>(out, n, s.grid.dScanTmp);
  CK(cudaGetLastError());
}

__global__ void k_scatter(const int4* atomK, int N, const int* start, const int* inCell, int* orig) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  orig[start[atomK[a].w] + inCell[a]] = a;
}

// Order inside a cell: ascending cell-local x coordinate u.x (pos0 of k_assign,
// so the build's staged positions are sorted along x within every cell and hence
// along every stencil row), ties by ascending atom index.  Deterministic for
// given coordinates.
__global__ void k_sort_cells(const int* start, int nRanks, int* orig, const float4* __restrict__ pos0, float* key) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nRanks) return;
  int b = start[r], e = start[r + 1];
  for (int i = b; i < e; i++) key[i] = pos0[orig[i]].x;
  for (int i = b + 1; i < e; i++) {
    int v = orig[i], j = i - 1;
    float kv = key[i];
    while (j >= b && (key[j] > kv || (key[j] == kv && orig[j] > v))) {
      orig[j + 1] = orig[j];
      key[j + 1] = key[j];
      j--;
    }
    orig[j + 1] = v;
    key[j + 1] = kv;
  }
}

// The same order for dense cells: one warp per cell; each atom's place is the
// number of atoms of the cell that precede it in (x key, atom index) order.
// Cells of more than 32 atoms are sorted by lane 0 as above.
__global__ void k_sort_cells_warp(const int* start, int nRanks, int* orig, const float4* __restrict__ pos0) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (r >= nRanks) return;
  const int b = start[r], n = start[r + 1] - b;
  if (n <= 1) return;
  if (n > 32) {
    if (lane == 0)
      for (int i = b + 1; i < b + n; i++) {
        const int v = orig[i];
        const float kv = pos0[v].x;
        int j = i - 1;
        while (j >= b) {
          const int u = orig[j];
          const float ku = pos0[u].x;
          if (!(ku > kv || (ku == kv && u > v))) break;
          orig[j + 1] = u;
          j--;
        }
        orig[j + 1] = v;
      }
    return;
  }
  const int a = lane < n ? orig[b + lane] : 0;
  const float k = lane < n ? pos0[a].x : 0.0f;
  int place = 0;
  for (int j = 0; j < n; j++) {
    const int aj = __shfl_sync(0xffffffffu, a, j);
    const float kj = __shfl_sync(0xffffffffu, k, j);
    place += (kj < k || (kj == k && aj < a)) ? 1 : 0;
  }
  __syncwarp();
  if (lane < n) orig[b + place] = a;
}

// per slot: image cell, type, slot of the atom, and the FP32 position and charge
// (pos0 of k_assign)
__global__ void k_fill_slots(const int* orig, int N, const int4* atomK, const int* type, int4* K, uint8_t* type8,
                             int* slotOf, const float4* __restrict__ pos0, float4* pos4) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  int a = orig[s];
  K[s] = atomK[a];
  slotOf[a] = s;
  type8[s] = (uint8_t)(type[a] - 1);
  pos4[s] = pos0[a];
}

__global__ void k_halo_table(TileGeom g, int2* tab) {
  const int t = blockIdx.x;
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x) tab[(size_t)t * g.haloCells + h] = halo_entry(g, t, h);
}

// per tile: number of atoms and of halo atoms; global maxima in maxOut[0..1]
__global__ void k_tile_info(const int* start, TileGeom g, int* info, int* maxOut) {
  __shared__ int sum;
  int t = blockIdx.x;
  if (threadIdx.x == 0) sum = 0;
  __syncthreads();
  int local = 0, hx, hy, hz;
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x) {
    int r = halo_rank(g, t, h, hx, hy, hz);
    local += start[r + 1] - start[r];
  }
  atomicAdd(&sum, local);
  __syncthreads();
  if (threadIdx.x == 0) {
    int cells = g.TB * g.TB * g.TB;
    int n = start[(t + 1) * cells] - start[t * cells];
    info[2 * t] = n;
    info[2 * t + 1] = sum;
    atomicMax(&maxOut[0], n);
    atomicMax(&maxOut[1], sum);
  }
}

// ---------------------------------------------------------------------------------
// per-step packing
// ---------------------------------------------------------------------------------

// cell-local position of each slot in units of the cell edge, u = M R/L - K, and
// the charge, from the coordinates (after a change of the box since the build)
__global__ void k_pack_mixed(const double* __restrict__ R, const double* __restrict__ charge, const int* orig,
                             const int4* K, int N, double scale, float4* pos4) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  int a = orig[s];
  int4 k = K[s];
  float ux = (float)(R[3 * a] * scale - (double)k.x);
  float uy = (float)(R[3 * a + 1] * scale - (double)k.y);
  float uz = (float)(R[3 * a + 2] * scale - (double)k.z);
  double q = charge[a];
  pos4[s] = make_float4(ux, uy, uz, fabs(q) > 2.220446049250313e-16 ? (float)q : 0.0f);
}

// Between builds, with the box of the last build: u = u0 + (R - R0) M/L, the
// displacement since the build rounded to FP32 and scaled in FP32 (one FP64
// subtraction per coordinate instead of the FP64 M R/L - K).  The fused step
// kernel packs with the same arithmetic.
__device__ __forceinline__ float4 pack_delta(float4 p0, double dx, double dy, double dz, float scale) {
  return make_float4(fmaf(d2f(dx), scale, p0.x), fmaf(d2f(dy), scale, p0.y), fmaf(d2f(dz), scale, p0.z), p0.w);
}

__global__ void k_pack_delta(const double* __restrict__ R, const double* __restrict__ R0, const int* orig,
                             const float4* __restrict__ pos0, int N, float scale, float4* pos4) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  int a = orig[s];
  pos4[s] = pack_delta(pos0[a], R[3 * a] - R0[3 * a], R[3 * a + 1] - R0[3 * a + 1], R[3 * a + 2] - R0[3 * a + 2],
                       scale);
}

// scaled FP64 coordinates Rs = R/L (src/EmDeeCode.f90:1228) in slot order
__global__ void k_pack_fp64(const double* __restrict__ R, const int* orig, int N, double L, double* Rs) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  int a = orig[s];
  Rs[3 * s] = R[3 * a] / L;
  Rs[3 * s + 1] = R[3 * a + 1] / L;
  Rs[3 * s + 2] = R[3 * a + 2] / L;
}

void device_pack(System& s) {
  Grid& g = s.grid;
  int N = s.natoms, th = 256, bl = (N + th - 1) / th;
  prof_begin(s, PK_PACK);
  if (s.precision == 1) {
    k_pack_fp64<<<bl, th, 0, s.stream>>>(s.dR, g.dOrig, N, *s.Lbox, g.dRs64);
  } else if (*s.Lbox == s.builtL) {
    k_pack_delta<<<bl, th, 0, s.stream>>>(s.dR, s.dR0, g.dOrig, g.dPos0, N, (float)((double)g.M / *s.Lbox), g.dPos4);
  } else {   // the box changed since the build: from the coordinates
    k_pack_mixed<<<bl, th, 0, s.stream>>>(s.dR, s.dCharge, g.dOrig, g.dK, N, (double)g.M / *s.Lbox, g.dPos4);
  }
  CK(cudaGetLastError());
  prof_end(s, PK_PACK);
}

// ---------------------------------------------------------------------------------
// list build
// ---------------------------------------------------------------------------------


struct BuildArgs {
  TileGeom g;
  const int2* tab;
  const float4* pos4;
  const int* start;
  const int* orig;
  const int4* K;
  const uint8_t* type8;
  const int* body;
  int hasBodies;
  const uint8_t* interact;
  int ntypes;
  const int* exFirst;
  const int* exCount;
  const int* exItem;
  int hasEx;
  const double* R;
  double L;
  float lo2, hi2, loIn2, hiIn2;   // FP32 band limits, cell units^2
  double thr, thrIn;              // FP64 thresholds, scaled units^2
  int layered;                    // inner threshold below the outer one
  int minimg;                     // M == 5: a stencil cell may hold a non-minimum image
  float Mf;
  int haloCap;
  uint16_t* nb;
  int* nbCount;
  int* nbInner;
  uint16_t* selfIdx;
  int cap, tileStride;
  int tpa, tpaShift;   // threads per atom of the split build (a power of 2) and its log2
  int* layout;         // out: per tile off[0..haloCells] and cst[0..haloCells-1] (stage_frame_saved)
  int* maxCount;
};

__device__ __forceinline__ bool excluded(const BuildArgs& A, int a, int b) {
  int f = A.exFirst[a], n = A.exCount[a];
  for (int k = 0; k < n; k++) {
    int v = A.exItem[f + k] - 1;
    if (v == b) return true;
    if (v > b) break;
  }
  return false;
}

// Blocks of the thread-per-atom build: at most BUILD_THREADS threads, each taking
// the same number of the tile's atoms (tile_threads); without a tuned count, as few
// rounds as blocks of BUILD_THREADS_RULE threads allow.
static const int BUILD_THREADS = 512;
static const int BUILD_THREADS_RULE = 256;
static const int BUILD_THREADS_SPLIT = 1024;  // split build: several threads per tile atom

// List layout: for tile t, chunk c (8 entries) and tile-local atom li, the
// entries 8c..8c+7 of atom li are 16 contiguous bytes at
//   nb + ((t * capC + c) * tileStride + li) * 8
// so a warp reads one chunk of 32 consecutive atoms with one 512-byte access.
// Unused entries of the last chunk hold the sentinel halo index haloCap.
__device__ __forceinline__ size_t nb_index(int t, int capC, int tileStride, int li, int n) {
  return (((size_t)t * capC + (n >> 3)) * tileStride + li) * 8 + (n & 7);
}

// GENERAL: several atom types, bodies, exclusions or layered lists; MINIMG: M = 5.
// Register budget: the thread-per-atom variants get up to BUILD_MAXNREG registers
// (blocks of at most BUILD_THREADS threads); the split variant, in blocks of up to
// 1024 threads, 64.  Under launch bounds alone the compiler held this kernel at 64
// registers with spills; 80 (71 used) gave the fastest builds on the 1M-atom
// workload (745 vs 811 us per rebuild with the pair kernel at 72).
#ifndef BUILD_MAXNREG
#define BUILD_MAXNREG 80
#endif
#define BUILD_BOUNDS __maxnreg__(SPLIT ? 64 : BUILD_MAXNREG)
template <bool GENERAL, bool MINIMG, bool SPLIT>
__global__ void BUILD_BOUNDS k_build(BuildArgs A) {
  extern __shared__ __align__(16) unsigned char sraw[];
  __shared__ int ws[33];
  const TileGeom g = A.g;
  const int t = blockIdx.x, cells = g.TB * g.TB * g.TB;
  // shared memory: the staged halo (and a sentinel entry), the halo cell offsets,
  // then for the general variant the halo atoms' slots, the type filter and the
  // halo atoms' types
  float4* hpos = (float4*)sraw;
  int* off = (int*)(hpos + A.haloCap + 1);
  int* hslot = off + g.haloCells + 1;
  const bool single = !GENERAL || A.ntypes == 1;
  uint8_t* sinter = (uint8_t*)(hslot + (GENERAL ? A.haloCap + 1 : 0));
  uint8_t* htype = sinter + A.ntypes * A.ntypes;
  for (int k = threadIdx.x; k < A.ntypes * A.ntypes; k += blockDim.x) sinter[k] = A.interact[k];
  // the layout, saved for the force kernels until the next build: first slots
  // straight to global memory, cell sizes scanned into off
  int* lay = A.layout + (size_t)t * (2 * g.haloCells + 1);
  {
    const int2* tt = A.tab + (size_t)t * g.haloCells;
    for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x) {
      const int r = tt[h].x, b = A.start[r];
      lay[g.haloCells + 1 + h] = b;
      off[h] = A.start[r + 1] - b;
    }
    __syncthreads();
    const int total = block_exclusive_scan<8>(off, g.haloCells, ws);
    if (threadIdx.x == 0) off[g.haloCells] = total;
    __syncthreads();
  }
  const int haloCount = off[g.haloCells];
  {
    // sizes taken from the previous build: a tile or halo that outgrew them is
    // reported (the host re-sizes and builds again) before anything is staged
    const int tileCount = A.start[(t + 1) * g.TB * g.TB * g.TB] - A.start[t * g.TB * g.TB * g.TB];
    if (tileCount > A.tileStride || haloCount > A.haloCap) {
      if (threadIdx.x == 0) atomicOr(A.maxCount + 1, 1);
      return;
    }
  }
  for (int h = threadIdx.x; h <= g.haloCells; h += blockDim.x) lay[h] = off[h];
  // every thread reads back only the first slots it wrote itself
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x)
    mark_halo_cell(hpos, h, off[h], off[h + 1], lay[g.haloCells + 1 + h]);
  __syncthreads();
  stage_marked(g, haloCount, A.pos4, hpos, GENERAL ? hslot : nullptr, single ? (uint8_t*)nullptr : htype, A.type8);
  __syncthreads();
  // slot of halo index q (the general variant keeps them; the band test of the
  // plain one, rare, looks its cell up)
  auto slot_of = [&](int q) {
    if (GENERAL) return hslot[q];
    int lo = 0, hi = g.haloCells - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= q) lo = mid;
      else hi = mid - 1;
    }
    return lay[g.haloCells + 1 + lo] + (q - off[lo]);
  };
  const bool none = A.ntypes == 1 && !sinter[0];   // the only type pair does not interact: empty lists
  const bool filterByAtom = GENERAL && (A.hasBodies || A.hasEx);
  const bool layered = GENERAL && A.layered;
  const int tb = A.start[t * cells], te = A.start[(t + 1) * cells];
  const int HW = g.HW, capC = A.cap >> 3, chunkStride = A.tileStride * 8;
  // SPLIT: tpa threads share an atom, each scanning the stencil rows r = sub,
  // sub + tpa, ...; a first sweep counts the accepted entries (inner and outer),
  // the group's prefix sums give each thread its output positions, and a second
  // sweep writes them.  The list order is then (thread, row, halo index) -- a
  // deterministic function of the coordinates, like the single-thread order.
  const int tpa = SPLIT ? A.tpa : 1, sub = SPLIT ? (int)(threadIdx.x & (tpa - 1)) : 0;
  const int tshift = SPLIT ? A.tpaShift : 0;
  const unsigned gmask = (0xFFFFFFFFu >> (32 - tpa)) << ((threadIdx.x & 31) & ~(tpa - 1));
  for (int li = threadIdx.x >> tshift; li < te - tb; li += blockDim.x >> tshift) {
    const int si = tb + li;
    const int rank = A.K[si].w, lr = rank - t * cells;
    const int hcx = lr % g.TB + 2, hcy = (lr / g.TB) % g.TB + 2, hcz = lr / (g.TB * g.TB) + 2;
    const int myq = off[hcx + HW * (hcy + HW * hcz)] + (si - A.start[rank]);
    if (sub == 0) A.selfIdx[si] = (uint16_t)myq;
    const float4 pi = hpos[myq];
    const int ai = A.orig[si], ti = single ? 0 : A.type8[si];
    const int bi = filterByAtom && A.hasBodies ? A.body[ai] : -1;
    const bool hasEx = filterByAtom && A.hasEx && A.exCount[ai] > 0;
    uint16_t* myList = A.nb + ((size_t)t * capC * A.tileStride + li) * 8;
    // accepted candidates of stencil row (rz, ry) -> f(q, inner); the 5 cells of a
    // row (dx = -2..2) are consecutive in the halo
    auto zdist2 = [&](int rz) {   // squared distance from atom i to the z slab of offset rz
      const float z0 = (float)(hcz + rz - g.C);
      const float dz = fmaxf(fmaxf(z0 - pi.z, pi.z - (z0 + 1.0f)) - 1e-3f, 0.0f);
      return dz * dz;
    };
    auto row = [&](int rz, int ry, float dz2, auto&& f) {
      const int hz = hcz + rz, hy = hcy + ry;
      const int h0 = (hcx - 2) + HW * (hy + HW * hz);
      int q = off[h0];
      const int q1 = off[h0 + 5];
      float xhi = 3.0e38f;
      if (!MINIMG) {
        // Atoms of a row are sorted along x.  With rho the distance from atom i
        // to the row's y-z cross-section, only |x_j - x_i| < sqrt(hi2 - rho^2)
        // can be inside; a 1e-3 cell margin covers the FP32 rounding of the frame.
        const float y0 = (float)(hy - g.C);
        const float dy = fmaxf(fmaxf(y0 - pi.y, pi.y - (y0 + 1.0f)) - 1e-3f, 0.0f);
        const float rem = A.hi2 - (dy * dy + dz2);
        if (rem <= 0.0f) return;
        const float w = rem * rsqrtf(rem) + 1e-3f;   // approximate square root: within the margin
        const float xlo = pi.x - w;
        xhi = pi.x + w;
        // atoms of halo cells left of floor(xlo) lie at x <= floor(xlo) <= xlo (cell
        // hx spans [hx - C, hx - C + 1] in the frame): start at that cell
        const int cs = min(max((int)floorf(xlo) + g.C, hcx - 2), hcx + 2);
        q = off[h0 + cs - (hcx - 2)];
        while (q < q1 && hpos[q].x <= xlo) q++;
      }
      // candidates in groups of CG: the loads and distance tests of a group are
      // independent (predicated, no branch per candidate), then the accepted ones
      // are taken in ascending order; a group that reaches the row's end or the
      // window's end is the last (the row is sorted along x)
      constexpr int CG = 2;   // pairs: measured faster than single candidates or groups of four
      for (; q < q1; q += CG) {
        float4 pj[CG];
#pragma unroll
        for (int u = 0; u < CG; u++) pj[u] = hpos[min(q + u, q1 - 1)];
        float r2s[CG];
        unsigned cand = 0;
        bool last = false;
#pragma unroll
        for (int u = 0; u < CG; u++) {
          const bool valid = q + u < q1 && (MINIMG || pj[u].x < xhi);
          last |= !valid;
          float ex = pi.x - pj[u].x, ey = pi.y - pj[u].y, ez = pi.z - pj[u].z;
          if (MINIMG) {
            ex -= A.Mf * rintf(ex / A.Mf);
            ey -= A.Mf * rintf(ey / A.Mf);
            ez -= A.Mf * rintf(ez / A.Mf);
          }
          r2s[u] = ex * ex + ey * ey + ez * ez;
          cand |= (valid && r2s[u] < A.hi2 && q + u != myq) ? 1u << u : 0u;
        }
#pragma unroll
        for (int u = 0; u < CG; u++) {
          if (!((cand >> u) & 1u)) continue;
          const int qu = q + u;
          const float r2 = r2s[u];
          if (!(r2 < A.lo2 || exact_inside(A.R, A.L, ai, A.orig[slot_of(qu)], A.thr))) continue;
          if (GENERAL && !single && !sinter[ti * A.ntypes + htype[qu]]) continue;
          if (filterByAtom) {
            const int aj = A.orig[hslot[qu]];
            if (A.hasBodies && A.body[aj] == bi) continue;
            if (hasEx && excluded(A, ai, aj)) continue;
          }
          bool inner = true;
          if (layered)
            inner = r2 < A.loIn2 || (r2 < A.hiIn2 && exact_inside(A.R, A.L, ai, A.orig[slot_of(qu)], A.thrIn));
          f(qu, inner);
        }
        if (last) break;
      }
    };
    auto put = [&](int k, int q) {
      if (k < A.cap) myList[(k >> 3) * chunkStride + (k & 7)] = (uint16_t)q;
    };
    int n = 0, nIn = 0;
    if (!SPLIT) {
      // rows in the order dz = -2..2 (outer), dy = -2..2 (inner); layered lists
      // take the inner entries in a first sweep and the outer ones in a second
      for (int pass = 0; pass <= (layered ? 1 : 0) && !none; pass++) {
        for (int rz = -2; rz <= 2; rz++) {
          const float dz2 = MINIMG ? 0.0f : zdist2(rz);
          for (int ry = -2; ry <= 2; ry++)
            row(rz, ry, dz2, [&](int q, bool inner) {
              if (layered && inner == (pass == 1)) return;
              put(n++, q);
            });
        }
        if (pass == 0) nIn = n;
      }
    } else {
      int cIn = 0, cOut = 0;
      if (!none)
        for (int r = sub; r < 25; r += tpa)
          row(r / 5 - 2, r % 5 - 2, MINIMG ? 0.0f : zdist2(r / 5 - 2), [&](int, bool inner) {
            if (inner) cIn++;
            else cOut++;
          });
      // exclusive prefix sums over the group's threads, in sub order
      int pIn = cIn, pOut = cOut;
      for (int o = 1; o < tpa; o <<= 1) {
        const int yIn = __shfl_up_sync(gmask, pIn, o), yOut = __shfl_up_sync(gmask, pOut, o);
        if (sub >= o) {
          pIn += yIn;
          pOut += yOut;
        }
      }
      const int totIn = __shfl_sync(gmask, pIn, tpa - 1, tpa), totOut = __shfl_sync(gmask, pOut, tpa - 1, tpa);
      int kIn = pIn - cIn, kOut = totIn + pOut - cOut;
      if (!none)
        for (int r = sub; r < 25; r += tpa)
          row(r / 5 - 2, r % 5 - 2, MINIMG ? 0.0f : zdist2(r / 5 - 2), [&](int q, bool inner) {
            if (inner) put(kIn++, q);
            else put(kOut++, q);
          });
      n = totIn + totOut;
      nIn = totIn;
      __syncwarp(gmask);
    }
    if (sub == 0) {
      for (int k = n; k < A.cap && (k & 7); k++) myList[(k >> 3) * chunkStride + (k & 7)] = (uint16_t)A.haloCap;
      A.nbCount[si] = n;
      A.nbInner[si] = nIn;
      atomicMax(A.maxCount, n);
    }
  }
}

template <typename T>
static void grow(T*& p, size_t& have, size_t need) {
  if (have >= need) return;
  CK(cudaFree(p));
  CK(cudaMalloc(&p, sizeof(T) * need));
  have = need;
}


int build_block_threads(const System& s) {
  return s.buildThreads > 0 ? std::min(s.buildThreads, BUILD_THREADS)
                            : tile_threads(s.grid.tileStride, 0, BUILD_THREADS_RULE);
}

// the general build variant: several types, bodies, exclusions or layered lists
static bool build_general(const System& s) {
  return s.ntypes > 1 || s.nbodies > 0 || s.hasExclusions || s.xInRcSq < s.xRcSq;
}

static size_t build_smem(const Grid& g, int ntypes, bool general) {
  return (size_t)(g.maxHalo + 1) * (sizeof(float4) + (general ? sizeof(int) + 1 : 0)) +
         sizeof(int) * (g.haloCells + 1) + (size_t)ntypes * ntypes + 16;
}

// Tile edge: EMDEE_TILE, else the system's tuned edge (tileOverride), else a rule on
// the atoms per cell.
static int rule_tile(int M, double perCell) {
  const int tb = perCell <= 4.0 ? 4 : perCell <= 9.0 ? 3 : perCell <= 24.0 ? 2 : 1;
  return std::min(tb, M);
}

static int choose_tile(const System& s, int M, double perCell) {
  if (const char* e = getenv("EMDEE_TILE")) {
    int tb = atoi(e);
    if (tb >= 1 && tb <= 6) return std::min(tb, M);
  }
  if (s.tileOverride > 0) return std::min(s.tileOverride, M);
  return rule_tile(M, perCell);
}

// Tile edge and block sizes tuned on the system itself at its first build (mixed
// precision, M > 5, EMDEE_TILE unset).  For each edge from min(rule - 1, 3) to 6
// cells (the rule's edge always among them) a first build sizes the tiles; then the
// list build and the pair kernel are timed with CUDA events (the faster of two
// launches, after a warm-up launch of the pair kernel), each after a pass that moves
// the memory traffic of an integration step, at the rule's block size and at block
// sizes from 64 to 512 threads (threads loop over the tile's atoms in rounds; the
// best size balances the rounds of typical tiles against residency).  The cost of an
// edge is its fastest pair launch plus a seventh of its fastest build (a rebuild
// every ~7 steps, typical of a liquid with the reference's skin).  The rule's edge
// and block sizes stay unless another choice is more than 5 % cheaper.  The choice
// is kept per (cells per edge, atoms per cell to 1/8, types, model variant) for the
// process, so systems of the same shape use the same tiles and blocks and give
// bit-identical results.
// Reads and rewrites R and P with their own bits and reads F (zero is 0 at run
// time): the memory traffic of an integration step, so that timed tuning launches
// meet the L2 contents a step leaves.
__global__ void k_touch(double* __restrict__ R, double* __restrict__ P, const double* __restrict__ F, long n,
                        long long zero) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long long f = __double_as_longlong(F[i]) & zero;
    R[i] = __longlong_as_double(__double_as_longlong(R[i]) ^ f);
    P[i] = __longlong_as_double(__double_as_longlong(P[i]) ^ f);
  }
}

struct TileChoice {
  int tb, buildThreads, pairThreads;
};
static std::vector<std::pair<std::vector<long>, TileChoice>> g_tileTuned;

void device_tune_tile(System& s, bool ljOnly, void (*pair)(System&)) {
  if (getenv("EMDEE_TILE") || (getenv("EMDEE_AUTOTUNE") && !strcmp(getenv("EMDEE_AUTOTUNE"), "0"))) return;
  const double L = *s.Lbox;
  const int M = std::max((int)std::floor(NDIV * L / s.xRc), 2 * NDIV + 1);
  if (M <= 2 * NDIV + 1) return;
  const double perCell = (double)s.natoms / ((double)M * M * M);
  const std::vector<long> key = {M, (long)std::lround(perCell * 8.0), s.ntypes, ljOnly ? 1 : 0, s.nbodies > 0,
                                 s.hasExclusions ? 1 : 0};
  for (const auto& e : g_tileTuned)
    if (e.first == key) {
      s.tileOverride = e.second.tb;
      s.buildThreads = e.second.buildThreads;
      s.pairThreads = e.second.pairThreads;
      return;
    }
  const int rule = rule_tile(M, perCell);
  const bool chainReq = s.keChainReq;   // no kinetic pass queued behind the timed pair launches
  s.keChainReq = false;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto timed = [&](auto&& f) {
    if (!s.phaseShared) {   // (shared R and P may belong to another system's stream)
      k_touch<<<4 * 152, 256, 0, s.stream>>>(s.dR, s.dP, s.F(), 3L * s.natoms, 0LL);
      CK(cudaGetLastError());
      s.prof.total++;
    }
    CK(cudaEventRecord(e0, s.stream));
    f();
    CK(cudaEventRecord(e1, s.stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    return (double)ms;
  };
  double best = 1e30, ruleCost = 1e30;
  TileChoice choice = {rule, 0, 0};
  for (int tb = std::max(1, std::min(rule - 1, 3)); tb <= std::min(6, M); tb++) {
    s.tileOverride = tb;
    s.buildThreads = s.pairThreads = 0;
    device_build_lists(s);   // sizes the tiles of this edge
    if (s.grid.TB != tb) continue;   // did not fit (halo or shared memory): the build shrank the edge
    // block sizes: 0 (the rule), then 64 to 256 threads in steps of 32 and 320 to 512
    // in steps of 64, from the least the halo scans need up to the largest tile
    const int thMin = halo_min_threads(make_geom(s.grid.M, tb)), thMax = (s.grid.tileStride + 31) / 32 * 32;
    std::vector<int> sizes = {0};
    for (int th = 64; th <= 512; th += th < 256 ? 32 : 64)
      if (th >= thMin && th <= thMax) sizes.push_back(th);
    double msBuild = 1e30, msPair = 1e30, ruleBuild = 0.0, rulePair = 0.0;
    int rb = 0, rp = 0;
    for (int r : sizes) {
      s.buildThreads = r;
      const double ms = std::min(timed([&] { device_build_lists(s); }), timed([&] { device_build_lists(s); }));
      if (getenv("EMDEE_TUNE_LOG"))
        fprintf(stderr, "  edge %d build, %d threads: %.1f us\n", tb, build_block_threads(s), 1e3 * ms);
      if (r == 0) ruleBuild = ms;
      if (ms < msBuild) {
        msBuild = ms;
        rb = r;
      }
    }
    for (int r : sizes) {
      s.pairThreads = r;
      pair(s);   // warm-up
      const double ms = std::min(timed([&] { pair(s); }), timed([&] { pair(s); }));
      if (getenv("EMDEE_TUNE_LOG")) fprintf(stderr, "  edge %d pair, %d threads: %.1f us\n", tb, pair_block_threads(s), 1e3 * ms);
      if (r == 0) rulePair = ms;
      if (ms < msPair) {
        msPair = ms;
        rp = r;
      }
    }
    const double cost = msPair + msBuild / 7.0;
    if (tb == rule) ruleCost = rulePair + ruleBuild / 7.0;
    if (getenv("EMDEE_TUNE_LOG"))
      fprintf(stderr, "tile edge %d (at most %d atoms per tile): cost %.1f us\n", tb, s.grid.tileStride, 1e3 * cost);
    if (cost < best) {
      best = cost;
      choice = {tb, rb, rp};
    }
  }
  if (ruleCost < 1e30 && best > 0.95 * ruleCost) choice = {rule, 0, 0};
  CK(cudaEventDestroy(e0));
  CK(cudaEventDestroy(e1));
  s.tileOverride = choice.tb;
  s.buildThreads = choice.buildThreads;
  s.pairThreads = choice.pairThreads;
  s.r0Valid = false;   // the system's own first build comes next, with the chosen edge
  s.keChainReq = chainReq;
  g_tileTuned.push_back({key, choice});
}

// src/neighbor_lists.f90:175-195 (build part) and 199-300.  reuse: keep the tile
// sizes of the previous build when the cell geometry is unchanged (no per-tile
// count pass and no synchronisation for it); returns false if a tile outgrew them.
static bool build_lists(System& s, bool reuse) {
  Grid& g = s.grid;
  GridCaps& c = g.caps;
  const int N = s.natoms;
  const double L = *s.Lbox;
  // two-level lists: this build writes the outer lists, of radius rc + skin + delta
  const bool outer = two_level_active(s);
  const double delta = outer ? outer_delta(s) : 0.0;
  const double xRc = s.xRc + delta, xRcSq = xRc * xRc;
  uint16_t*& nbList = outer ? g.dNbOuter : g.dNb;
  size_t& nbCap = outer ? c.nbOuter : c.nb;
  int& cap = outer ? g.capOuter : g.cap;
  int M = (int)std::floor(NDIV * L / xRc);
  M = std::max(M, 2 * NDIV + 1);
  double perCell = (double)N / ((double)M * M * M);
  int TB = choose_tile(s, M, perCell);
  reuse = reuse && g.M == M && g.TB == TB && g.maxHalo > 0 && g.tileStride > 0 && c.atoms >= (size_t)N;
  size_t smemLimit = 200 * 1024;
  for (;;) {
    TileGeom geo = make_geom(M, TB);
    g.M = M;
    g.TB = TB;
    g.nT = geo.nT;
    g.nTiles = geo.nT * geo.nT * geo.nT;
    g.nRanks = g.nTiles * TB * TB * TB;
    g.haloCells = geo.haloCells;
    grow(g.dCount, c.ranks, (size_t)g.nRanks + 1);
    if (!g.dStart || c.scan < (size_t)g.nRanks + 1) {
      CK(cudaFree(g.dStart));
      CK(cudaFree(g.dScanTmp));
      CK(cudaMalloc(&g.dStart, sizeof(int) * (g.nRanks + 1)));
      CK(cudaMalloc(&g.dScanTmp, sizeof(int) * ((g.nRanks + SCAN_TILE) / SCAN_TILE + 1)));
      c.scan = (size_t)g.nRanks + 1;
    }
    if (c.atoms < (size_t)N) {
      CK(cudaFree(g.dOrig)); CK(cudaFree(g.dK)); CK(cudaFree(g.dAtomK)); CK(cudaFree(g.dPos4));
      CK(cudaFree(g.dType8)); CK(cudaFree(g.dRs64)); CK(cudaFree(g.dNbCount)); CK(cudaFree(g.dNbInner));
      CK(cudaFree(g.dSelf));
      CK(cudaFree(g.dSlotOf));
      CK(cudaFree(g.dPos0));
      CK(cudaFree(g.dKeyX));
      CK(cudaMalloc(&g.dKeyX, sizeof(float) * N));
      CK(cudaMalloc(&g.dSlotOf, sizeof(int) * N));
      CK(cudaMalloc(&g.dPos0, sizeof(float4) * N));
      CK(cudaMalloc(&g.dOrig, sizeof(int) * N));
      CK(cudaMalloc(&g.dK, sizeof(int4) * N));
      CK(cudaMalloc(&g.dAtomK, sizeof(int4) * N));
      CK(cudaMalloc(&g.dPos4, sizeof(float4) * N));
      CK(cudaMalloc(&g.dType8, N));
      CK(cudaMalloc(&g.dRs64, sizeof(double) * 3 * N));
      CK(cudaMalloc(&g.dNbCount, sizeof(int) * N));
      CK(cudaMalloc(&g.dNbInner, sizeof(int) * N));
      CK(cudaMalloc(&g.dSelf, sizeof(uint16_t) * N));
      c.atoms = N;
    }
    if (c.tiles < (size_t)g.nTiles) {
      CK(cudaFree(g.dTileInfo));
      CK(cudaMalloc(&g.dTileInfo, sizeof(int) * (2 * g.nTiles + 6)));
      c.tiles = g.nTiles;
    }
    int th = 256, bl = (N + th - 1) / th;
    CK(cudaMemsetAsync(g.dCount, 0, sizeof(int) * (g.nRanks + 1), s.stream));
    s.prof.total += reuse ? 7 : 8;   // assign, 3 scan phases, scatter, sort, fill (, tile info)
    // the slot array holds each atom's place in its cell until k_fill_slots
    k_assign<<<bl, th, 0, s.stream>>>(s.dR, s.dCharge, N, (double)M / L, geo, g.dAtomK, g.dCount, g.dSlotOf,
                                      g.dPos0, s.dR0);
    CK(cudaGetLastError());
    device_scan(s, g.dCount, g.dStart, g.nRanks);
    k_scatter<<<bl, th, 0, s.stream>>>(g.dAtomK, N, g.dStart, g.dSlotOf, g.dOrig);
    if (perCell >= 8.0)   // dense cells: a warp per cell
      k_sort_cells_warp<<<(g.nRanks + 7) / 8, 256, 0, s.stream>>>(g.dStart, g.nRanks, g.dOrig, g.dPos0);
    else
      k_sort_cells<<<(g.nRanks + 255) / 256, 256, 0, s.stream>>>(g.dStart, g.nRanks, g.dOrig, g.dPos0, g.dKeyX);
    k_fill_slots<<<bl, th, 0, s.stream>>>(g.dOrig, N, g.dAtomK, s.dType, g.dK, g.dType8, g.dSlotOf, g.dPos0,
                                          g.dPos4);
    int* dMax = g.dTileInfo + 2 * g.nTiles;
    CK(cudaMemsetAsync(dMax, 0, sizeof(int) * 4, s.stream));
    if (reuse) break;
    k_tile_info<<<g.nTiles, 128, 0, s.stream>>>(g.dStart, geo, g.dTileInfo, dMax);
    CK(cudaGetLastError());
    int hmax[2];
    CK(cudaMemcpyAsync(hmax, dMax, sizeof(int) * 2, cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    g.tileStride = std::max(32, (hmax[0] + 31) / 32 * 32);
    g.maxHalo = hmax[1];
    size_t smem = build_smem(g, s.ntypes, build_general(s));
    size_t smem64 = (size_t)(g.maxHalo + 1) * (4 * sizeof(double) + 1) + 2 * sizeof(int) * (g.haloCells + 1) + 64;
    if ((g.maxHalo > 65534 || smem > smemLimit || (s.precision == 1 && smem64 > smemLimit)) && TB > 1) {
      TB--;
      continue;
    }
    if (g.maxHalo > 65534 || smem > smemLimit) fatal("neighbor list build", "too many atoms around a cell");
    break;
  }
  TileGeom geo = make_geom(g.M, g.TB);
  if (g.tabM != g.M || g.tabTB != g.TB) {   // the halo table depends on the geometry only
    size_t need = (size_t)g.nTiles * g.haloCells;
    if (g.haloTabCap < need) {
      CK(cudaFree(g.dHaloTab));
      CK(cudaMalloc(&g.dHaloTab, sizeof(int2) * need));
      g.haloTabCap = need;
    }
    k_halo_table<<<g.nTiles, 128, 0, s.stream>>>(geo, g.dHaloTab);
    CK(cudaGetLastError());
    s.prof.total++;
    g.tabM = g.M;
    g.tabTB = g.TB;
  }
  // neighbor capacity: expected full-list count with margin, grown on overflow
  if (cap == 0) {
    double rho = N / (L * L * L);
    double expected = rho * 4.18879020478639 * xRcSq * xRc;
    cap = (int)std::min(65528.0, expected * 1.35 + 32);
  }
  cap = (cap + 7) / 8 * 8;
  if (outer && c.outerAtoms < (size_t)N) {
    CK(cudaFree(g.dNbCountOuter));
    CK(cudaFree(g.dROuter));
    CK(cudaMalloc(&g.dNbCountOuter, sizeof(int) * N));
    CK(cudaMalloc(&g.dROuter, sizeof(double) * 3 * N));
    c.outerAtoms = N;
  }
  const double invL2 = 1.0 / (L * L);
  BuildArgs A;
  A.g = geo;
  A.tab = g.dHaloTab;
  A.pos4 = g.dPos4;
  A.start = g.dStart;
  A.orig = g.dOrig;
  A.K = g.dK;
  A.type8 = g.dType8;
  A.body = s.dBody;
  A.hasBodies = s.nbodies > 0;
  A.interact = s.models.interact;
  A.ntypes = s.ntypes;
  A.exFirst = s.dExFirst;
  A.exCount = s.dExCount;
  A.exItem = s.dExItem;
  A.hasEx = s.hasExclusions;
  A.R = s.dR;
  A.L = L;
  A.thr = xRcSq * invL2;    // src/neighbor_lists.f90:213-214 (outer lists: rc + skin + delta)
  A.thrIn = s.xInRcSq * invL2;
  double M2 = (double)g.M * g.M;
  A.lo2 = (float)(A.thr * M2 * (1.0 - BAND));
  A.hi2 = (float)(A.thr * M2 * (1.0 + BAND));
  A.loIn2 = (float)(A.thrIn * M2 * (1.0 - BAND));
  A.hiIn2 = (float)(A.thrIn * M2 * (1.0 + BAND));
  A.layered = s.xInRcSq < s.xRcSq ? 1 : 0;
  A.minimg = g.M == 5 ? 1 : 0;
  A.Mf = (float)g.M;
  A.haloCap = g.maxHalo;
  A.nbCount = outer ? g.dNbCountOuter : g.dNbCount;
  A.nbInner = g.dNbInner;
  A.selfIdx = g.dSelf;
  A.tileStride = g.tileStride;
  A.maxCount = g.dTileInfo + 2 * g.nTiles + 2;
  grow(g.dLayout, g.layoutCap, (size_t)g.nTiles * (2 * g.haloCells + 1));
  A.layout = g.dLayout;
  const bool general = build_general(s);
  size_t smem = build_smem(g, s.ntypes, general);
  // Threads per atom: a system too small to fill the GPU with one thread per atom and
  // with long lists (more than 48 entries per thread) splits the stencil rows of each
  // atom over 2, 4 or 8 threads (blocks of up to 1024 threads).
  {
    const double expected = N / (L * L * L) * 4.18879020478639 * xRcSq * xRc;
    int tpa = 1, shift = 0;
    while (tpa < 8 && g.tileStride * tpa * 2 <= BUILD_THREADS_SPLIT && (double)N * tpa * 2 <= 152.0 * 2048 &&
           expected / (tpa * 2) >= 48) {
      tpa *= 2;
      shift++;
    }
    A.tpa = tpa;
    A.tpaShift = shift;
  }
  const bool split = A.tpa > 1;
  auto kb = split ? (general ? (A.minimg ? k_build<true, true, true> : k_build<true, false, true>)
                             : (A.minimg ? k_build<false, true, true> : k_build<false, false, true>))
                  : (general ? (A.minimg ? k_build<true, true, false> : k_build<true, false, false>)
                             : (A.minimg ? k_build<false, true, false> : k_build<false, false, false>));
  const int buildThreads = std::max(halo_min_threads(geo), split ? std::min(BUILD_THREADS_SPLIT, g.tileStride * A.tpa)
                                                                 : build_block_threads(s));
  CK(cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
#ifdef EMDEE_MAX_CARVEOUT
  CK(cudaFuncSetAttribute(kb, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
#endif
  for (int attempt = 0; attempt < 3; attempt++) {
    size_t need = (size_t)g.nTiles * cap * g.tileStride;
    grow(nbList, nbCap, need);
    A.nb = nbList;
    A.cap = cap;
    CK(cudaMemsetAsync(A.maxCount, 0, sizeof(int), s.stream));
    kb<<<g.nTiles, buildThreads, smem, s.stream>>>(A);
    s.prof.total++;
    CK(cudaGetLastError());
    int* mc = s.hFlags + 2;   // pinned: largest list, tile-size overflow
    CK(cudaMemcpyAsync(mc, A.maxCount, 2 * sizeof(int), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    if (mc[1]) return false;
    if (mc[0] <= cap) break;
    if (mc[0] > 65528) fatal("neighbor list build", "more than 65528 neighbors for one atom");
    cap = std::min(65528, (mc[0] + mc[0] / 8 + 16 + 7) / 8 * 8);
  }
  s.r0Valid = true;   // R0 was written by k_assign
  s.builtL = L;
  s.listsOuter = outer;
  if (outer) {   // the reference positions of the coverage test
    CK(cudaMemcpyAsync(g.dROuter, s.dR, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s.stream));
    s.outerDelta = delta;
    s.outerL = L;
  }
  return true;
}

void device_build_lists(System& s) {
  prof_begin(s, PK_BUILD);
  if (!build_lists(s, true)) build_lists(s, false);
  prof_end(s, PK_BUILD);
}

// ---------------------------------------------------------------------------------
// two-level lists
// ---------------------------------------------------------------------------------
//
// An outer build lists every pair within rc + skin + delta; the force kernel of a
// rebuild step filters those lists into the lists the reference would build (every
// pair within rc + skin, the same FP32 + FP64-band test as k_build), as long as
// the outer lists still hold every such pair: with d1 >= d2 the two largest
// displacements since the outer build, a pair now within rc + skin was within
// rc + skin + d1 + d2 then, so d1 + d2 < delta suffices.  The rebuild schedule and
// the pair sets stay those of the reference; only the work per rebuild changes.

// Off unless requested (EmDee_set_outer_skin, or EMDEE_OUTER_SKIN for systems that
// did not set it).  Measured on the 1M-atom Lennard-Jones bench (skin 0.3, T* 1.5):
// the fastest of a million atoms cross any outer skin up to 0.9 within two rebuild
// periods, so outer builds (1.7x a build at rc + skin + 0.45) come every second
// rebuild, and the filtering launch costs about as much as the build it replaces:
// 387 us per step against 350 with single-level lists.  Slower dynamics (more
// rebuilds per outer build) are where the outer lists pay.
double outer_delta(System& s) {
  if (s.outerSkin >= 0.0) return s.outerSkin;
  static const double env = getenv("EMDEE_OUTER_SKIN") ? atof(getenv("EMDEE_OUTER_SKIN")) : 0.0;
  return env > 0.0 ? env : 0.0;
}

bool two_level_active(System& s) {
  const double d = outer_delta(s);
  if (!(d > 0.0) || s.precision != 0 || s.nlayers != 1 || !(s.skin > 0.0) || s.xInRcSq < s.xRcSq) return false;
  if (!pair_lj_only(s)) return false;
  return (int)std::floor(NDIV * *s.Lbox / (s.xRc + d)) > 2 * NDIV + 1;   // outer cells: M > 5
}

// Coverage test of the outer lists and start of a new rebuild period: the largest
// and second largest squared displacement since the outer build (FP64 differences,
// FP32 squares, compared as non-negative bit patterns, an order-independent pair);
// result[40] = 0 if d1 + d2 < delta (with a relative margin for the FP32 squares),
// else 1, result[41] = d1 + d2.  Also R0 = R and pos0 = the current packed position
// of every atom (the reference positions of the skin check and of the packing).
__global__ void __launch_bounds__(SKIN_THREADS) k_cover(const double* __restrict__ R, const double* __restrict__ RO,
                                                        const int* __restrict__ slotOf,
                                                        const float4* __restrict__ pos4, int N, double delta,
                                                        double* __restrict__ R0, float4* __restrict__ pos0,
                                                        int2* partial, unsigned int* ticket, double* result) {
  __shared__ int2 wsum[SKIN_THREADS / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int a = 0, b = 0;   // bits of the largest and second largest d^2 (FP32, >= 0)
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    float d2 = 0.0f;
    for (int k = 0; k < 3; k++) {
      const double r = R[3 * i + k];
      const float d = d2f(r - RO[3 * i + k]);
      d2 = fmaf(d, d, d2);
      R0[3 * i + k] = r;
    }
    pos0[i] = pos4[slotOf[i]];
    const int v = __float_as_int(d2);
    b = max(b, min(a, v));
    a = max(a, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    const int oa = __shfl_down_sync(0xffffffffu, a, o), ob = __shfl_down_sync(0xffffffffu, b, o);
    b = max(max(b, ob), min(a, oa));
    a = max(a, oa);
  }
  if (lane == 0) wsum[warp] = make_int2(a, b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int2 t = wsum[0];
    for (int w = 1; w < SKIN_THREADS / 32; w++) {
      t.y = max(max(t.y, wsum[w].y), min(t.x, wsum[w].x));
      t.x = max(t.x, wsum[w].x);
    }
    partial[blockIdx.x] = t;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  int2 t = make_int2(0, 0);
  for (unsigned int k = 0; k < gridDim.x; k++) {
    const int2 p = __ldcg(&partial[k]);
    t.y = max(max(t.y, p.y), min(t.x, p.x));
    t.x = max(t.x, p.x);
  }
  const double sum = sqrt((double)__int_as_float(t.x)) + sqrt((double)__int_as_float(t.y));
  result[41] = sum;
  result[40] = sum * (1.0 + 1e-5) < delta ? 0.0 : 1.0;
  *ticket = 0;
}

// The filtering pair launch on the current outer lists, with the lists regrown
// until the longest filtered list fits; false if skip was set (nothing ran).
static bool refilter(System& s, bool compute, const double* skip) {
  Grid& g = s.grid;
  ensure_partials(s, g.nTiles);
  for (;;) {
    grow(g.dNb, g.caps.nb, (size_t)g.nTiles * g.cap * g.tileStride);
    int* innerMax = g.dTileInfo + 2 * g.nTiles + 4;
    CK(cudaMemsetAsync(innerMax, 0, sizeof(int), s.stream));
    prof_begin(s, PK_PAIR);
    device_pair_refilter(s, compute, skip);
    prof_end(s, PK_PAIR);
    // the kernel's last block wrote the sums into hResult[0..4]
    if (skip) CK(cudaMemcpyAsync(s.hResult + 40, s.dResult + 40, 2 * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaMemcpyAsync(s.hFlags, innerMax, sizeof(int), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    if (skip && s.hResult[40] != 0.0) {
      prof_drop_last(s);
      return false;
    }
    const int mc = s.hFlags[0];
    if (mc <= g.cap) return true;
    if (mc > 65528) fatal("neighbor list build", "more than 65528 neighbors for one atom");
    g.cap = std::min(65528, (mc + mc / 8 + 16 + 7) / 8 * 8);
    skip = nullptr;   // covered: filter again with room for the longest list
  }
}

void device_rebuild_two_level(System& s, bool compute) {
  Grid& g = s.grid;
  const int N = s.natoms;
  if (s.listsOuter && *s.Lbox == s.outerL && s.outerDelta == outer_delta(s)) {
    if (!s.packReady) device_pack(s);
    const int blocks = std::min((N + SKIN_THREADS - 1) / SKIN_THREADS, 4 * 152);
    ensure_partials(s, blocks);
    prof_begin(s, PK_BUILD);
    k_cover<<<blocks, SKIN_THREADS, 0, s.stream>>>(s.dR, g.dROuter, g.dSlotOf, g.dPos4, N, s.outerDelta, s.dR0,
                                                   g.dPos0, (int2*)s.dPartials, s.dTicket, s.dResult);
    CK(cudaGetLastError());
    prof_end(s, PK_BUILD);
    if (refilter(s, compute, s.dResult + 40)) return;
  }
  device_build_lists(s);
  s.outerBuilds++;
  refilter(s, compute, nullptr);
}

// ---------------------------------------------------------------------------------
// pair-set dump (test support): every full-list entry as (orig_i, orig_j)
// ---------------------------------------------------------------------------------

__global__ void k_dump_pairs(TileGeom g, const int2* tab, const int* start, const int* orig, const uint16_t* nb,
                             const int* nbCount, int cap, int tileStride, const long long* outStart, int2* out) {
  extern __shared__ int hslot[];
  __shared__ int ws[33];
  __shared__ int off[1001], cst[1000];
  const int t = blockIdx.x, cells = g.TB * g.TB * g.TB;
  halo_layout(g, t, tab, start, off, cst, (int*)nullptr, ws);
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x)
    for (int k = off[h]; k < off[h + 1]; k++) hslot[k] = cst[h] + (k - off[h]);
  __syncthreads();
  const int tb = start[t * cells], te = start[(t + 1) * cells];
  for (int li = threadIdx.x; li < te - tb; li += blockDim.x) {
    int si = tb + li, ai = orig[si];
    long long o = outStart[si];
    for (int k = 0; k < nbCount[si]; k++) {
      int q = nb[nb_index(t, cap >> 3, tileStride, li, k)];
      out[o + k] = make_int2(ai + 1, orig[hslot[q]] + 1);
    }
  }
}

long device_neighbor_pairs(System& s, int* pairs, long capacity) {
  Grid& g = s.grid;
  int N = s.natoms;
  if (!s.r0Valid) return 0;
  std::vector<int> cnt(N), orig(N);
  CK(cudaStreamSynchronize(s.stream));
  CK(cudaMemcpy(cnt.data(), g.dNbCount, sizeof(int) * N, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(orig.data(), g.dOrig, sizeof(int) * N, cudaMemcpyDeviceToHost));
  std::vector<long long> st(N + 1, 0);
  for (int i = 0; i < N; i++) st[i + 1] = st[i] + cnt[i];
  long long total = st[N];
  long npairs = (long)(total / 2);
  if (npairs > capacity) return -npairs;
  long long* dSt;
  int2* dOut;
  CK(cudaMalloc(&dSt, sizeof(long long) * (N + 1)));
  CK(cudaMalloc(&dOut, sizeof(int2) * (total + 1)));
  CK(cudaMemcpy(dSt, st.data(), sizeof(long long) * (N + 1), cudaMemcpyHostToDevice));
  TileGeom geo = make_geom(g.M, g.TB);
  k_dump_pairs<<<g.nTiles, 128, sizeof(int) * g.maxHalo, s.stream>>>(geo, g.dHaloTab, g.dStart, g.dOrig, g.dNb,
                                                                      g.dNbCount, g.cap, g.tileStride, dSt, dOut);
  CK(cudaGetLastError());
  std::vector<int2> h(total);
  CK(cudaStreamSynchronize(s.stream));
  CK(cudaMemcpy(h.data(), dOut, sizeof(int2) * total, cudaMemcpyDeviceToHost));
  CK(cudaFree(dSt));
  CK(cudaFree(dOut));
  std::vector<std::pair<int, int>> v;
  v.reserve(npairs);
  for (auto& e : h)
    if (e.x < e.y) v.push_back({e.x, e.y});
  std::sort(v.begin(), v.end());
  long n = (long)v.size();
  if (n > capacity) return -n;
  for (long k = 0; k < n; k++) {
    pairs[2 * k] = v[k].first;
    pairs[2 * k + 1] = v[k].second;
  }
  return n;
}

// ---------------------------------------------------------------------------------
// radial distribution histograms over the current lists (src/EmDeeCode.f90:1281-1395)
// ---------------------------------------------------------------------------------

struct RdfArgs {
  TileGeom g;
  const int2* tab;
  const int* start;
  const int* orig;
  const uint16_t* nb;
  const int* count;   // entries to scan per slot (all, or the inner part)
  const uint8_t* type8;
  const double* R;
  int cap, tileStride, bins, ntp;   // ntp: histogram rows (type pairs, symm1D order)
  double invL, Rc2, binsByRc;
  const uint8_t* hasPair;   // [type] (0-based)
  const uint8_t* pairOn;    // [ti * ntypes + tj]
  int ntypes, haloCap;
  unsigned long long* hist;   // [pair][bin], every pair counted from both of its atoms
  int sharedHist;             // histogram fits in shared memory
};

__global__ void k_rdf(RdfArgs A) {
  extern __shared__ int dyn[];
  __shared__ int ws[33];
  __shared__ int off[1001], cst[1000];
  const TileGeom g = A.g;
  const int t = blockIdx.x, cells = g.TB * g.TB * g.TB;
  int* hslot = dyn;   // halo index -> slot, then the block's histogram
  halo_layout(g, t, A.tab, A.start, off, cst, (int*)nullptr, ws);
  unsigned int* sh = (unsigned int*)(hslot + A.haloCap);
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x)
    for (int k = off[h]; k < off[h + 1]; k++) hslot[k] = cst[h] + (k - off[h]);
  const int hn = A.bins * A.ntp;
  if (A.sharedHist)
    for (int k = threadIdx.x; k < hn; k += blockDim.x) sh[k] = 0u;
  __syncthreads();
  const int tb = A.start[t * cells], te = A.start[(t + 1) * cells];
  for (int li = threadIdx.x; li < te - tb; li += blockDim.x) {
    const int si = tb + li, ai = A.orig[si], ti = A.type8[si];
    if (!A.hasPair[ti]) continue;
    const double xi = A.invL * A.R[3 * ai], yi = A.invL * A.R[3 * ai + 1], zi = A.invL * A.R[3 * ai + 2];
    const int n = A.count[si];
    for (int k = 0; k < n; k++) {
      const int q = A.nb[nb_index(t, A.cap >> 3, A.tileStride, li, k)];
      const int sj = hslot[q], aj = A.orig[sj], tj = A.type8[sj];
      if (!A.pairOn[ti * A.ntypes + tj]) continue;
      double dx = xi - A.invL * A.R[3 * aj], dy = yi - A.invL * A.R[3 * aj + 1], dz = zi - A.invL * A.R[3 * aj + 2];
      dx = dx - round(dx);
      dy = dy - round(dy);
      dz = dz - round(dz);
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < A.Rc2) {
        int bin = (int)(sqrt(r2) * A.binsByRc);
        bin = min(bin, A.bins - 1);
        const int a = min(ti, tj), b = max(ti, tj), p = a + (b + 1) * b / 2;   // symm1D - 1 (0-based types)
        if (A.sharedHist) atomicAdd(&sh[p * A.bins + bin], 1u);
        else atomicAdd(&A.hist[(size_t)p * A.bins + bin], 1ull);
      }
    }
  }
  if (A.sharedHist) {
    __syncthreads();
    for (int k = threadIdx.x; k < hn; k += blockDim.x)
      if (sh[k]) atomicAdd(&A.hist[k], (unsigned long long)sh[k]);
  }
}

// counts[pair][bin] (pairs in symm1D order over types 1..maxtype), each pair once
void device_rdf_counts(System& s, int bins, double Rc, const std::vector<uint8_t>& hasPair,
                       const std::vector<uint8_t>& pairOn, int ntp, std::vector<unsigned long long>& counts) {
  Grid& g = s.grid;
  const int nt = s.ntypes;
  RdfArgs A;
  A.g = make_geom(g.M, g.TB);
  A.tab = g.dHaloTab;
  A.start = g.dStart;
  A.orig = g.dOrig;
  A.nb = g.dNb;
  A.count = Rc < 1.0001 * s.InRc ? g.dNbInner : g.dNbCount;
  A.type8 = g.dType8;
  A.R = s.dR;
  A.cap = g.cap;
  A.tileStride = g.tileStride;
  A.bins = bins;
  A.ntp = ntp;
  const double invL = 1.0 / *s.Lbox;
  A.invL = invL;
  A.Rc2 = Rc * Rc * (invL * invL);
  A.binsByRc = bins / (Rc * invL);
  A.ntypes = nt;
  A.haloCap = g.maxHalo;
  const size_t hn = (size_t)bins * ntp;
  uint8_t *dHas, *dOn;
  unsigned long long* dHist;
  CK(cudaMalloc(&dHas, nt));
  CK(cudaMalloc(&dOn, (size_t)nt * nt));
  CK(cudaMalloc(&dHist, sizeof(unsigned long long) * hn));
  CK(cudaMemcpy(dHas, hasPair.data(), nt, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dOn, pairOn.data(), (size_t)nt * nt, cudaMemcpyHostToDevice));
  CK(cudaMemsetAsync(dHist, 0, sizeof(unsigned long long) * hn, s.stream));
  A.hasPair = dHas;
  A.pairOn = dOn;
  A.hist = dHist;
  size_t smem = sizeof(int) * (size_t)g.maxHalo;
  A.sharedHist = (hn * sizeof(unsigned int) <= 48 * 1024) ? 1 : 0;
  if (A.sharedHist) smem += hn * sizeof(unsigned int);
  CK(cudaFuncSetAttribute(k_rdf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_rdf<<<g.nTiles, 128, smem, s.stream>>>(A);
  CK(cudaGetLastError());
  s.prof.total++;
  counts.assign(hn, 0ull);
  CK(cudaStreamSynchronize(s.stream));
  CK(cudaMemcpy(counts.data(), dHist, sizeof(unsigned long long) * hn, cudaMemcpyDeviceToHost));
  for (auto& c : counts) c /= 2;   // full lists hold every pair twice, at the same distance
  CK(cudaFree(dHas));
  CK(cudaFree(dOn));
  CK(cudaFree(dHist));
}

// ---------------------------------------------------------------------------------
// fused step: pending boosts, move, skin displacement and FP32 packing in one pass
// ---------------------------------------------------------------------------------

// Contiguous atom ranges combined in index order, as in k_skin, so the skin value
// is the same for any range size.  Each
// statement rounds as the separate kernels do (this file uses -fmad=false).
static const int STEP_CHUNKS = 2;   // 64 consecutive atoms per warp: many warps in flight

// FMA (mixed precision only): the updates use fused multiply-adds, which halves the
// work on the FP64 pipe (the limit of this kernel on GB300); FP64 mode keeps the
// reference's separately rounded statements.
template <int NK, bool UNITM, bool PACK, bool FMA>
__global__ void __launch_bounds__(SKIN_THREADS) k_step_fused(double* __restrict__ R, double* __restrict__ P,
                                                             const double* __restrict__ F,
                                                             const double* __restrict__ invMass,
                                                             const double* __restrict__ R0, int N, double cf0,
                                                             double cf1, double CP, double skinSq,
                                                             const int* __restrict__ slotOf,
                                                             const float4* __restrict__ pos0, float scale,
                                                             float4* __restrict__ pos4, longlong2* partial,
                                                             unsigned int* ticket, double* result,
                                                             double* hostResult) {
  __shared__ MaxPrev wsum[SKIN_THREADS / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int base = (blockIdx.x * (SKIN_THREADS / 32) + warp) * 32 * STEP_CHUNKS;
  MaxPrev run{-1, -1};
  for (int c = 0; c < STEP_CHUNKS; c++) {
    const int i = base + c * 32 + lane;
    MaxPrev v{-1, -1};
    if (i < N) {
      const double im = UNITM ? 1.0 : invMass[i];
      double r[3];
      for (int d = 0; d < 3; d++) {
        double p = P[3 * i + d];
        if (FMA) {
          if (NK >= 1) p = fma(cf0, F[3 * i + d], p);
          if (NK >= 2) p = fma(cf1, F[3 * i + d], p);
        } else {
          if (NK >= 1) p = p + cf0 * F[3 * i + d];
          if (NK >= 2) p = p + cf1 * F[3 * i + d];
        }
        if (NK >= 1) P[3 * i + d] = p;
        if (FMA) r[d] = UNITM ? fma(CP, p, R[3 * i + d]) : fma(CP * p, im, R[3 * i + d]);
        else r[d] = R[3 * i + d] + (UNITM ? CP * p : CP * p * im);
        R[3 * i + d] = r[d];
      }
      const double d0 = r[0] - R0[3 * i], d1 = r[1] - R0[3 * i + 1], d2 = r[2] - R0[3 * i + 2];
      v.m = __double_as_longlong(FMA ? fma(d2, d2, fma(d1, d1, d0 * d0)) : d0 * d0 + d1 * d1 + d2 * d2);
      if (PACK) pos4[slotOf[i]] = pack_delta(pos0[i], d0, d1, d2, scale);
    }
    v = warp_ordered_combine(v);
    run = mp_combine(run, v);
  }
  if (lane == 0) wsum[warp] = run;
  __syncthreads();
  if (threadIdx.x == 0) {
    MaxPrev b = wsum[0];
    for (int w = 1; w < SKIN_THREADS / 32; w++) b = mp_combine(b, wsum[w]);
    partial[blockIdx.x] = make_longlong2(b.m, b.p);
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int nb = gridDim.x, per = (nb + SKIN_THREADS - 1) / SKIN_THREADS;
  MaxPrev acc{-1, -1};
  for (int k = 0; k < per; k++) {
    int b = threadIdx.x * per + k;
    if (b < nb) {
      longlong2 v = __ldcg(&partial[b]);
      acc = mp_combine(acc, MaxPrev{v.x, v.y});
    }
  }
  acc = warp_ordered_combine(acc);
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    MaxPrev b = wsum[0];
    for (int w = 1; w < SKIN_THREADS / 32; w++) b = mp_combine(b, wsum[w]);
    double maximum = __longlong_as_double(b.m), next = __longlong_as_double(b.p < 0 ? b.m : b.p);
    double value = maximum + 2 * sqrt(maximum * next) + next;
    result[8] = value;
    result[9] = value > skinSq ? 1.0 : 0.0;
    hostResult[8] = value;   // pinned host memory: read after the next synchronisation
    hostResult[9] = result[9];
    *ticket = 0;
  }
}

void device_step_fused(System& s, double CP) {
  const int N = s.natoms;
  const int blocks = (N + SKIN_THREADS * STEP_CHUNKS - 1) / (SKIN_THREADS * STEP_CHUNKS);
  ensure_partials(s, blocks);
  const bool pack = s.precision == 0 && s.r0Valid && *s.Lbox == s.builtL;
  const Grid& g = s.grid;
  const float scale = g.M > 0 ? (float)((double)g.M / *s.Lbox) : 0.0f;
  prof_begin(s, PK_MOVE);
#define STEP_ARGS s.dR, s.dP, s.F(), s.dInvMass, s.dR0, N, s.pendCF[0], s.pendCF[1], CP, s.skinSq, g.dSlotOf, \
                  g.dPos0, scale, g.dPos4, (longlong2*)s.dPartials, s.dTicket, s.dResult, s.hResult
#define STEP_LAUNCH(NK, UM, PK, FM) k_step_fused<NK, UM, PK, FM><<<blocks, SKIN_THREADS, 0, s.stream>>>(STEP_ARGS)
#define STEP_NK(UM, PK, FM)                 \
  if (s.npend == 0) STEP_LAUNCH(0, UM, PK, FM); \
  else if (s.npend == 1) STEP_LAUNCH(1, UM, PK, FM); \
  else STEP_LAUNCH(2, UM, PK, FM);
  if (pack) {   // mixed precision: fused multiply-adds
    if (s.unitMass) { STEP_NK(true, true, true) } else { STEP_NK(false, true, true) }
  } else if (s.precision == 0) {
    if (s.unitMass) { STEP_NK(true, false, true) } else { STEP_NK(false, false, true) }
  } else {
    if (s.unitMass) { STEP_NK(true, false, false) } else { STEP_NK(false, false, false) }
  }
#undef STEP_NK
#undef STEP_LAUNCH
#undef STEP_ARGS
  CK(cudaGetLastError());
  prof_end(s, PK_MOVE);
  s.npend = 0;
  s.skinReady = s.r0Valid;
  s.packReady = pack;
}

// the skin value left by the fused step (its last block also wrote hResult[8..9])
bool device_skin_from_step(System& s) {
  CK(cudaStreamSynchronize(s.stream));
  return s.hResult[9] != 0.0;
}

}  // namespace emdee

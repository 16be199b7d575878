// tile.cuh -- cell-tile geometry shared by the neighbor-list build and the
// force kernels.
//
// The box is cut into M^3 cells of edge L/M >= (rc+skin)/2 (the cell rule of
// src/neighbor_lists.f90:185-186).  Cells are grouped into tiles of TB^3 cells;
// a thread block owns one tile.  Every atom within rc+skin of a tile atom lies
// in the tile's halo: the (TB+4)^3 cells of the tile grown by two cells on each
// side (the +-2 stencil of src/neighbor_lists.f90:26-35 applied to every cell
// of the tile).  Atoms are stored tile by tile, cell by cell ("rank" order), so
// a halo cell is one contiguous run of slots.
#pragma once

#include <cstdint>

#include "fpconv.h"

namespace emdee {

struct TileGeom {
  int M;      // cells per dimension
  int TB;     // tile edge (cells)
  int nT;     // tiles per dimension
  int HW;     // halo edge = TB + 4
  int C;      // frame origin offset = HW / 2
  int haloCells;   // HW^3
};

__host__ __device__ __forceinline__ TileGeom make_geom(int M, int TB) {
  TileGeom g;
  g.M = M;
  g.TB = TB;
  g.nT = (M + TB - 1) / TB;
  g.HW = TB + 4;
  g.C = g.HW / 2;
  g.haloCells = g.HW * g.HW * g.HW;
  return g;
}

// rank of the cell with coordinates (cx, cy, cz) in [0, M)
__host__ __device__ __forceinline__ int cell_rank(const TileGeom& g, int cx, int cy, int cz) {
  int tx = cx / g.TB, ty = cy / g.TB, tz = cz / g.TB;
  int lx = cx - tx * g.TB, ly = cy - ty * g.TB, lz = cz - tz * g.TB;
  int tile = tx + g.nT * (ty + g.nT * tz);
  return tile * g.TB * g.TB * g.TB + lx + g.TB * (ly + g.TB * lz);
}

__host__ __device__ __forceinline__ int wrap(int x, int M) {
  x %= M;
  return x < 0 ? x + M : x;
}

// rank of halo cell h (h = hx + HW (hy + HW hz)) of tile t
__host__ __device__ __forceinline__ int halo_rank(const TileGeom& g, int t, int h, int& hx, int& hy, int& hz) {
  hx = h % g.HW;
  hy = (h / g.HW) % g.HW;
  hz = h / (g.HW * g.HW);
  int tx = t % g.nT, ty = (t / g.nT) % g.nT, tz = t / (g.nT * g.nT);
  return cell_rank(g, wrap(tx * g.TB + hx - 2, g.M), wrap(ty * g.TB + hy - 2, g.M), wrap(tz * g.TB + hz - 2, g.M));
}

// Relative width of the band around (rc + skin)^2 inside which the list builds
// replace the FP32 distance by the reference's FP64 test.
constexpr double LIST_BAND = 4e-5;

#ifdef __CUDACC__

// FP64 minimum-image distance test of src/neighbor_lists.f90:247-250, with
// explicitly rounded operations (the same result in every file, whatever its
// contraction setting).
static __device__ __noinline__ bool exact_inside(const double* R, double L, int a, int b, double thr) {
  double r2 = 0.0;
  for (int k = 0; k < 3; k++) {
    const double x = __dsub_rn(__ddiv_rn(R[3 * a + k], L), __ddiv_rn(R[3 * b + k], L));
    const double d = __dsub_rn(x, round(x));
    r2 = __dadd_rn(r2, __dmul_rn(d, d));
  }
  return r2 < thr;
}

// Exclusive scan over n <= blockDim.x * ITEMS ints held in shared memory
// (in place); returns the total.  All threads of the block must call it.
template <int ITEMS>
__device__ int block_exclusive_scan(int* data, int n, int* warpSums) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = (blockDim.x + 31) >> 5;
  int base = tid * ITEMS, local[ITEMS], sum = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; k++) {
    int v = (base + k < n) ? data[base + k] : 0;
    local[k] = sum;
    sum += v;
  }
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warpSums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = lane < nwarps ? warpSums[lane] : 0, x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < nwarps) warpSums[lane] = x - v;
    if (lane == 31) warpSums[32] = x;
  }
  __syncthreads();
  int offset = warpSums[warp] + incl - sum;
#pragma unroll
  for (int k = 0; k < ITEMS; k++)
    if (base + k < n) data[base + k] = local[k] + offset;
  int total = warpSums[32];
  __syncthreads();
  return total;
}

// The halo scans below need blockDim.x * 8 >= haloCells: launch sites size their
// blocks with halo_min_threads.
__host__ __device__ __forceinline__ int halo_min_threads(const TileGeom& g) { return (g.haloCells + 255) / 256 * 32; }

// Threads of a block that owns a tile of up to `stride` atoms when each thread
// takes `rounds` of them (rounds <= 0: as few rounds as `cap` threads allow): the
// atoms spread evenly over the warps, so that no warp runs a last round alone
// while the block holds its shared memory and registers.  A multiple of 32, at
// most cap.
__host__ __device__ __forceinline__ int tile_threads(int stride, int rounds, int cap) {
  if (rounds <= 0) rounds = (stride + cap - 1) / cap;
  int th = (stride + rounds - 1) / rounds;
  th = (th + 31) / 32 * 32;
  return th < 32 ? 32 : th > cap ? cap : th;
}

// off[h] = first halo index of halo cell h of tile t; off[haloCells] = halo size.
__device__ __forceinline__ int halo_offsets(const TileGeom& g, int t, const int* start, int* off, int* ws) {
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x) {
    int hx, hy, hz, r = halo_rank(g, t, h, hx, hy, hz);
    off[h] = start[r + 1] - start[r];
  }
  __syncthreads();
  int total = block_exclusive_scan<8>(off, g.haloCells, ws);
  if (threadIdx.x == 0) off[g.haloCells] = total;
  __syncthreads();
  return total;
}

// Per-tile halo table, written once per list build: for halo cell h of tile t,
// tab[t * haloCells + h] = (rank of the cell, hx | hy << 8 | hz << 16).
__device__ __forceinline__ int2 halo_entry(const TileGeom& g, int t, int h) {
  int hx, hy, hz, r = halo_rank(g, t, h, hx, hy, hz);
  return make_int2(r, hx | (hy << 8) | (hz << 16));
}

// Halo layout of tile t: off[h] = first halo index of halo cell h
// (off[haloCells] = halo size), cst[h] = first slot, hxyz[h] = packed cell
// coordinates inside the halo.
__device__ __forceinline__ int halo_layout(const TileGeom& g, int t, const int2* tab, const int* start, int* off,
                                          int* cst, int* hxyz, int* ws) {
  const int2* tt = tab + (size_t)t * g.haloCells;
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x) {
    int2 e = tt[h];
    int b = start[e.x];
    cst[h] = b;
    off[h] = start[e.x + 1] - b;
    if (hxyz) hxyz[h] = e.y;
  }
  __syncthreads();
  int total = block_exclusive_scan<8>(off, g.haloCells, ws);
  if (threadIdx.x == 0) off[g.haloCells] = total;
  __syncthreads();
  return total;
}

// Halo staging in two passes that keep no layout in shared memory.  mark_halo_cell
// (first pass, one thread per halo cell h with first halo index b, end e and first
// slot s0) records for every halo index k its cell (x word of hpos[k]) and its slot
// (y word); after a barrier, stage_marked loads the halo atoms 0..n-1 in the tile
// frame, one thread per halo atom, U loads in flight per thread (a warp's loads
// cover consecutive slots of cell runs); optionally records slots and types.
// Ends without a barrier.
__device__ __forceinline__ void mark_halo_cell(float4* hpos, int h, int b, int e, int s0) {
  int2* mark = reinterpret_cast<int2*>(hpos);
  for (int k = b; k < e; k++) mark[2 * k] = make_int2(h, s0 + k - b);
}

__device__ __forceinline__ void stage_marked(const TileGeom& g, int n, const float4* pos4, float4* hpos, int* hslot,
                                             uint8_t* htype, const uint8_t* type8) {
  const int2* mark = reinterpret_cast<const int2*>(hpos);
  constexpr int U = 4;
  for (int k0 = threadIdx.x; k0 < n; k0 += U * blockDim.x) {
    float4 p[U];
    int hh[U], slot[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = k0 + u * blockDim.x;
      if (k < n) {
        const int2 m = mark[2 * k];
        hh[u] = m.x;
        slot[u] = m.y;
        p[u] = pos4[m.y];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = k0 + u * blockDim.x;
      if (k < n) {
        const int h = hh[u], hy = h / g.HW;
        const float fx = (float)(h - hy * g.HW - g.C), fy = (float)(hy % g.HW - g.C), fz = (float)(hy / g.HW - g.C);
        hpos[k] = make_float4(p[u].x + fx, p[u].y + fy, p[u].z + fz, p[u].w);
        if (hslot) hslot[k] = slot[u];
        if (htype) htype[k] = type8[slot[u]];
      }
    }
  }
}

// Stages the halo of tile t from the layout saved by the list build (global
// memory: off[0..haloCells], then cst[0..haloCells-1]); returns the halo size.
// Ends without a barrier.
__device__ __forceinline__ int stage_frame_saved(const TileGeom& g, const int* __restrict__ lay, const float4* pos4,
                                                 float4* hpos, uint8_t* htype, const uint8_t* type8) {
  for (int h = threadIdx.x; h < g.haloCells; h += blockDim.x)
    mark_halo_cell(hpos, h, lay[h], lay[h + 1], lay[g.haloCells + 1 + h]);
  __syncthreads();
  const int n = lay[g.haloCells];
  stage_marked(g, n, pos4, hpos, nullptr, htype, type8);
  return n;
}

// Slot of halo index q of the tile whose saved layout is lay: its halo cell is the
// last one that starts at or before q.
__device__ __forceinline__ int saved_slot(const TileGeom& g, const int* __restrict__ lay, int q) {
  int lo = 0, hi = g.haloCells - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (lay[mid] <= q) lo = mid;
    else hi = mid - 1;
  }
  return lay[g.haloCells + 1 + lo] + (q - lay[lo]);
}

// Exact float -> double conversion with integer operations (normal numbers and
// zero; denormals were flushed by the FP32 arithmetic).  Keeps the FP64 pipe,
// which is slow on this GPU, out of the force stores.
__device__ __forceinline__ double f2d_exact(float f) {
  unsigned int u = __float_as_uint(f);
  unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  unsigned int e = (u >> 23) & 255u;
  if (e == 0) return __longlong_as_double((long long)sign);
  unsigned long long de = e == 255u ? 2047ull : (unsigned long long)(e + 896u);
  return __longlong_as_double((long long)(sign | (de << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

#endif

}  // namespace emdee

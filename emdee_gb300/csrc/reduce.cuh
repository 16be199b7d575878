// reduce.cuh -- deterministic block and grid reductions of FP64 partial sums.
//
// THREADS is the largest block size the kernel is launched with.  Each block reduces its per-thread values (warp shuffles, then warps in
// order) and writes one partial per quantity; the last block to finish (ticket
// counter) sums the partials in block order with Neumaier compensation.  The
// result does not depend on block scheduling.
#pragma once

namespace emdee {

// Variant whose inputs are already warp sums held by lane 0 of each warp.
template <int NQ, int THREADS>
__device__ __forceinline__ void grid_reduce_lane0(const double (&v)[NQ], double* partials, unsigned int* ticket,
                                                  double* result, double* result2 = nullptr) {
  __shared__ double red[NQ][THREADS / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++) red[q][warp] = v[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < NQ; q++) {
      double x = 0.0;
      for (int w = 0; w < nw; w++) x += red[q][w];
      partials[(size_t)blockIdx.x * NQ + q] = x;
    }
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // last block: thread t sums partials t, t + blockDim, ... (Neumaier), then the
  // per-thread sums are combined by a fixed tree; the order never depends on
  // which block finished last.
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    double s = 0.0, c = 0.0;
    constexpr int U = 8;   // partials in flight per thread, added in increasing block order
    for (unsigned int b0 = threadIdx.x; b0 < gridDim.x; b0 += U * blockDim.x) {
      double xs[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const unsigned int b = b0 + u * blockDim.x;
        xs[u] = b < gridDim.x ? __ldcg(&partials[(size_t)b * NQ + q]) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (b0 + u * blockDim.x >= gridDim.x) break;
        const double x = xs[u], t = s + x;
        c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
      }
    }
    double x = s + c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[q][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    double x = 0.0;
    for (int w = 0; w < nw; w++) x += red[threadIdx.x][w];
    result[threadIdx.x] = x;
    if (result2) result2[threadIdx.x] = x;   // e.g. pinned host memory: no copy back
  }
  if (threadIdx.x == 0) *ticket = 0;
}

// FP64 per-thread values: warp shuffle sums, then as above.
template <int NQ, int THREADS>
__device__ __forceinline__ void grid_reduce(double (&v)[NQ], double* partials, unsigned int* ticket, double* result,
                                            double* result2 = nullptr) {
#pragma unroll
  for (int q = 0; q < NQ; q++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  grid_reduce_lane0<NQ, THREADS>(v, partials, ticket, result, result2);
}

// Warp sums of FP32 values with an error-free two-sum at every level; lane 0
// converts hi + lo to FP64 (other lanes return 0 and touch no FP64 unit).
template <int NQ>
__device__ __forceinline__ void warp_sum_f32(const float (&x)[NQ], double (&out)[NQ]) {
  float hi[NQ], lo[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    hi[q] = x[q];
    lo[q] = 0.f;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      float h2 = __shfl_down_sync(0xffffffffu, hi[q], o), l2 = __shfl_down_sync(0xffffffffu, lo[q], o);
      float s = hi[q] + h2, bp = s - hi[q], err = (hi[q] - (s - bp)) + (h2 - bp);
      hi[q] = s;
      lo[q] = lo[q] + l2 + err;
    }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int q = 0; q < NQ; q++) out[q] = (double)hi[q] + (double)lo[q];
  } else {
#pragma unroll
    for (int q = 0; q < NQ; q++) out[q] = 0.0;
  }
}

// grid_reduce for per-thread FP32 partial sums: compensated warp sums in FP32,
// FP64 from there on.
template <int NQ, int THREADS>
__device__ __forceinline__ void grid_reduce_f32(const float (&v)[NQ], double* partials, unsigned int* ticket,
                                                double* result) {
  double w[NQ];
  warp_sum_f32<NQ>(v, w);
  grid_reduce_lane0<NQ, THREADS>(w, partials, ticket, result);
}

// ---- float-float (FP32 pair) reductions: every level on the FP32 pipe ----------
//
// A value is carried as hi + lo with |lo| << |hi|; additions use Knuth's
// error-free two-sum on the high parts and plain addition of the low parts, so
// the sum keeps about 48 significant bits.  Only the final hi + lo conversion
// per quantity touches FP64.

__device__ __forceinline__ void ff_add(float& hi, float& lo, float bh, float bl) {
  const float s = hi + bh, bp = s - hi, err = (hi - (s - bp)) + (bh - bp);
  hi = s;
  lo = lo + bl + err;
}

// Quantities whose bit is clear in MASK are known to be zero: they skip every
// level and their result is written as 0.
template <int NQ, unsigned MASK = ~0u>
__device__ __forceinline__ void warp_sum_ff(float (&hi)[NQ], float (&lo)[NQ]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      if (!((MASK >> q) & 1u)) continue;
      const float h2 = __shfl_down_sync(0xffffffffu, hi[q], o), l2 = __shfl_down_sync(0xffffffffu, lo[q], o);
      ff_add(hi[q], lo[q], h2, l2);
    }
}

// Per-thread float-float values (hi + lo) -> result[q] (FP64), also into result2 if
// set; partials holds NQ float2 per block.  Every level runs on the FP32 pipe.
template <int NQ, int THREADS>
__device__ __forceinline__ void grid_reduce_ff2(const float (&vh)[NQ], const float (&vl)[NQ], float2* partials,
                                                unsigned int* ticket, double* result, double* result2) {
  __shared__ float2 red2[NQ][THREADS / 32];
  __shared__ bool last2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  float hi[NQ], lo[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    hi[q] = vh[q];
    lo[q] = vl[q];
  }
  warp_sum_ff<NQ>(hi, lo);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++) red2[q][warp] = make_float2(hi[q], lo[q]);
  __syncthreads();
  if (threadIdx.x < NQ) {
    const int q = threadIdx.x;
    float h = 0.f, l = 0.f;
    for (int w = 0; w < nw; w++) ff_add(h, l, red2[q][w].x, red2[q][w].y);
    partials[(size_t)blockIdx.x * NQ + q] = make_float2(h, l);
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last2 = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last2) return;
  __threadfence();
#pragma unroll
  for (int q = 0; q < NQ; q++) hi[q] = lo[q] = 0.f;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x)   // block order per thread
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const float2 x = __ldcg(&partials[(size_t)b * NQ + q]);
      ff_add(hi[q], lo[q], x.x, x.y);
    }
  warp_sum_ff<NQ>(hi, lo);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++) red2[q][warp] = make_float2(hi[q], lo[q]);
  __syncthreads();
  if (threadIdx.x < NQ) {
    const int q = threadIdx.x;
    float h = 0.f, l = 0.f;
    for (int w = 0; w < nw; w++) ff_add(h, l, red2[q][w].x, red2[q][w].y);
    result[q] = (double)h + (double)l;
    if (result2) result2[q] = (double)h + (double)l;
  }
  if (threadIdx.x == 0) *ticket = 0;
}

// Per-thread FP32 values -> result[q] (FP64), also into result2 if set.  partials holds
// NQ float2 per block.
// The last block (ticket) sums the partials in block order; the result does not
// depend on block scheduling.
template <int NQ, int THREADS, unsigned MASK = ~0u>
__device__ __forceinline__ void grid_reduce_ff(const float (&v)[NQ], float2* partials, unsigned int* ticket,
                                               double* result, double* result2 = nullptr) {
  __shared__ float2 red[NQ][THREADS / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  float hi[NQ], lo[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    hi[q] = v[q];
    lo[q] = 0.f;
  }
  warp_sum_ff<NQ, MASK>(hi, lo);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++)
      if ((MASK >> q) & 1u) red[q][warp] = make_float2(hi[q], lo[q]);
  __syncthreads();
  if (threadIdx.x < NQ && ((MASK >> threadIdx.x) & 1u)) {
    const int q = threadIdx.x;
    float h = 0.f, l = 0.f;
    for (int w = 0; w < nw; w++) ff_add(h, l, red[q][w].x, red[q][w].y);
    partials[(size_t)blockIdx.x * NQ + q] = make_float2(h, l);
    __threadfence();   // the partial is visible before the ticket counts this block
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    hi[q] = 0.f;
    lo[q] = 0.f;
  }
  // U partials per quantity in flight per thread, added in increasing block order
  constexpr int U = 8;
  for (unsigned int b0 = threadIdx.x; b0 < gridDim.x; b0 += U * blockDim.x) {
    float2 x[U][NQ];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned int b = b0 + u * blockDim.x;
#pragma unroll
      for (int q = 0; q < NQ; q++)
        if ((MASK >> q) & 1u) x[u][q] = b < gridDim.x ? __ldcg(&partials[(size_t)b * NQ + q]) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < U; u++)
      if (b0 + u * blockDim.x < gridDim.x)
#pragma unroll
        for (int q = 0; q < NQ; q++)
          if ((MASK >> q) & 1u) ff_add(hi[q], lo[q], x[u][q].x, x[u][q].y);
  }
  warp_sum_ff<NQ, MASK>(hi, lo);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++)
      if ((MASK >> q) & 1u) red[q][warp] = make_float2(hi[q], lo[q]);
  __syncthreads();
  if (threadIdx.x < NQ) {
    const int q = threadIdx.x;
    float h = 0.f, l = 0.f;
    if ((MASK >> q) & 1u)
      for (int w = 0; w < nw; w++) ff_add(h, l, red[q][w].x, red[q][w].y);
    result[q] = (double)h + (double)l;
    if (result2) result2[q] = (double)h + (double)l;   // e.g. pinned host memory: no copy back
  }
  if (threadIdx.x == 0) *ticket = 0;
}

}  // namespace emdee

// surrogate.cu -- learned surrogate potential for hybrid Monte Carlo proposals
// (no counterpart in the reference; it serves the surrogate-proposal HMC
// workload: a binary Lennard-Jones mixture, many chains of the same size).
//
// Model (atom-centred, Behler-Parrinello style): for atom i of species s_i,
//   G_i[c, k] = sum_{j != i, s_j = c, r_ij < rc} exp(-(r_ij - mu_k)^2 / (2 w^2)) fc(r_ij),
//   fc(r) = (cos(pi r / rc) + 1) / 2,  mu_k = mu_0 + k (mu_15 - mu_0) / 15,  k = 0..15, c = 0..1,
//   E_i = w3 . silu(W2^T silu(W1^T G_i + b1) + b2) + b3 with one network per species
//   (32 -> 64 -> 64 -> 1), E = sum_i E_i,  F = -dE/dR.
// Kernels (one launch each, over all chains at once):
//   k_sg_pack      FP64 positions -> FP32, wrapped into the box
//   k_sg_list      Verlet lists within rc + skin from a cell list (per chain)
//   k_sg_desc      descriptors, Gaussians by the two-term product recurrence
//   k_sg_mlp       per-species tiles of 64 atoms: forward and backward through the
//                  network on the tensor cores (mma.sync m16n8k16, BF16 operands,
//                  FP32 accumulation): E_i and dE/dG_i
//   k_sg_force     the adjoint: F_i = -sum_j (dE/dG_i[s_j] + dE/dG_j[s_i]) . dh/dr r_hat
//   k_sg_udesc     training: u_i[c, k] = sum_j h'_k(r_ij) (v_i - v_j) . r_hat_ij, the
//                  force residual v pulled back to descriptor space
//   k_sg_train     training: per species, forward, tangent along u, and the
//                  backward pass of O_i = e_c E_i - (dE_i/dG_i . u_i), whose
//                  gradient is the gradient of the energy + force loss; weight
//                  gradients as tensor-core GEMMs over 64-atom tiles, per-block
//                  partials reduced in block order
//   k_sg_adam      Adam update of the FP32 master parameters
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "reduce.cuh"
#include "system.hpp"
#include "tile.cuh"

namespace emdee {

namespace sg {

constexpr int NG = 16, NS = 2, DIN = 32, H = 64;
// packed FP32 parameters per species: W1[32][64], b1[64], W2[64][64], b2[64], w3[64], b3
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + DIN * H, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H, PER_SPECIES = OFF_B3 + 1;
constexpr int NPARAM = NS * PER_SPECIES;
constexpr int TILE = 64;   // atoms per block tile (4 warps x 16)

struct Geometry {
  int chains, N, M;          // M cells per dimension (cell edge >= rc + skin)
  float L, invL, rc, rc2, rlist2, mu0, dmu, a;   // a = 1 / (2 w^2)
};

__device__ __forceinline__ float silu(float x) { return x / (1.f + __expf(-x)); }
__device__ __forceinline__ float dsilu(float x) {
  const float s = 1.f / (1.f + __expf(-x));
  return s * (1.f + x * (1.f - s));
}
__device__ __forceinline__ float d2silu(float x) {
  const float s = 1.f / (1.f + __expf(-x));
  return s * (1.f - s) * (2.f + x * (1.f - 2.f * s));
}

// ---- tensor-core tile GEMM -------------------------------------------------------
// D(16 x 8) += A(16 x 16, row-major) * B(16 x 8, "col": element (k, n) read from
// Bt[n][k]); fragment layouts of mma.sync.m16n8k16 (PTX ISA): lane = 4 g + t,
// A regs (g, 2t..2t+1), (g+8, ..), (g, 2t+8..), (g+8, 2t+8..); B regs (2t..2t+1, g),
// (2t+8.., g); C regs (g, 2t..2t+1), (g+8, 2t..2t+1).
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// acc[nt][4] += A(16 x K) * B(K x 8 NT), A row-major (lda), B given as Bt[n][k] (ldb)
template <int K, int NT>
__device__ __forceinline__ void warp_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Bt, int ldb,
                                          float (&acc)[NT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[4];
    a[0] = ld32(A + g * lda + k0 + 2 * t);
    a[1] = ld32(A + (g + 8) * lda + k0 + 2 * t);
    a[2] = ld32(A + g * lda + k0 + 8 + 2 * t);
    a[3] = ld32(A + (g + 8) * lda + k0 + 8 + 2 * t);
#pragma unroll
    for (int n = 0; n < NT; n++) {
      uint32_t b[2];
      b[0] = ld32(Bt + (n * 8 + g) * ldb + k0 + 2 * t);
      b[1] = ld32(Bt + (n * 8 + g) * ldb + k0 + 8 + 2 * t);
      mma16816(acc[n], a, b);
    }
  }
}

template <int NT>
__device__ __forceinline__ void zero(float (&acc)[NT][4]) {
#pragma unroll
  for (int n = 0; n < NT; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
}

// element (row, col) of fragment tile n, slot q (0..3)
__device__ __forceinline__ int frag_row(int q) { return ((threadIdx.x & 31) >> 2) + (q >= 2 ? 8 : 0); }
__device__ __forceinline__ int frag_col(int n, int q) { return n * 8 + 2 * (threadIdx.x & 3) + (q & 1); }

// shared-memory weights of one species, BF16, in both orientations
struct WeightsSmem {
  __nv_bfloat16 W1[DIN][H + 8];    // W1[k][n]        (B^T for dE/dG = dz1 W1^T)
  __nv_bfloat16 W1t[H][DIN + 8];   // W1^T[n][k]      (B^T for z1 = G W1)
  __nv_bfloat16 W2[H][H + 8];      // W2[k][n]        (B^T for da1 = dz2 W2^T)
  __nv_bfloat16 W2t[H][H + 8];     // W2^T[n][k]      (B^T for z2 = a1 W2)
  float b1[H], b2[H], w3[H], b3;
};

__device__ void load_weights(WeightsSmem& w, const float* p) {
  for (int q = threadIdx.x; q < DIN * H; q += blockDim.x) {
    const int k = q / H, n = q % H;
    const __nv_bfloat16 v = __float2bfloat16(p[OFF_W1 + q]);
    w.W1[k][n] = v;
    w.W1t[n][k] = v;
  }
  for (int q = threadIdx.x; q < H * H; q += blockDim.x) {
    const int k = q / H, n = q % H;
    const __nv_bfloat16 v = __float2bfloat16(p[OFF_W2 + q]);
    w.W2[k][n] = v;
    w.W2t[n][k] = v;
  }
  for (int q = threadIdx.x; q < H; q += blockDim.x) {
    w.b1[q] = p[OFF_B1 + q];
    w.b2[q] = p[OFF_B2 + q];
    w.w3[q] = p[OFF_W3 + q];
  }
  if (threadIdx.x == 0) w.b3 = p[OFF_B3];
}

// ---- geometry kernels ---------------------------------------------------------------

__global__ void k_sg_pack(const double* __restrict__ R, int total, double L, float4* __restrict__ pos) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= total) return;
  float p[3];
  for (int d = 0; d < 3; d++) {
    const double x = R[3 * q + d];
    p[d] = (float)(x - L * floor(x / L));
  }
  pos[q] = make_float4(p[0], p[1], p[2], 0.f);
}

__device__ __forceinline__ int sg_cell(float x, const Geometry& G) {
  int c = (int)(x * G.invL * G.M);
  return c < 0 ? 0 : (c >= G.M ? G.M - 1 : c);
}

// cell counts per chain
__global__ void k_sg_count(const float4* __restrict__ pos, Geometry G, int* __restrict__ cellOf,
                           int* __restrict__ counts) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= G.chains * G.N) return;
  const int c = q / G.N;
  const float4 p = pos[q];
  const int cell = sg_cell(p.x, G) + G.M * (sg_cell(p.y, G) + G.M * sg_cell(p.z, G));
  cellOf[q] = cell;
  atomicAdd(&counts[c * G.M * G.M * G.M + cell], 1);
}

// one block: exclusive scan of all chains' cell counts (chains * M^3 entries)
__global__ void k_sg_scan(const int* counts, int n, int* starts) {
  __shared__ int ws[33];
  __shared__ int carry;
  __shared__ int buf[2048];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 2048) {
    for (int k = threadIdx.x; k < 2048; k += blockDim.x) buf[k] = base + k < n ? counts[base + k] : 0;
    __syncthreads();
    const int total = block_exclusive_scan<8>(buf, 2048, ws);
    for (int k = threadIdx.x; k < 2048; k += blockDim.x)
      if (base + k < n) starts[base + k] = buf[k] + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) starts[n] = carry;
}

__global__ void k_sg_scatter(const int* __restrict__ cellOf, Geometry G, const int* __restrict__ starts,
                             int* __restrict__ cursor, int* __restrict__ sorted) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= G.chains * G.N) return;
  const int c = q / G.N, r = c * G.M * G.M * G.M + cellOf[q];
  sorted[starts[r] + atomicAdd(&cursor[r], 1)] = q;
}

// deterministic order inside a cell
__global__ void k_sg_sort(const int* __restrict__ starts, int n, int* __restrict__ sorted) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int b = starts[r], e = starts[r + 1];
  for (int i = b + 1; i < e; i++) {
    const int v = sorted[i];
    int j = i - 1;
    while (j >= b && sorted[j] > v) {
      sorted[j + 1] = sorted[j];
      j--;
    }
    sorted[j + 1] = v;
  }
}

// Verlet lists (global atom indices), entry k of atom q at list[k * total + q]
__global__ void k_sg_list(const float4* __restrict__ pos, Geometry G, const int* __restrict__ cellOf,
                          const int* __restrict__ starts, const int* __restrict__ sorted, int cap,
                          int* __restrict__ list, int* __restrict__ count, int* __restrict__ overflow) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = G.chains * G.N;
  if (q >= total) return;
  const int c = q / G.N, M = G.M, cell = cellOf[q];
  const int cx = cell % M, cy = (cell / M) % M, cz = cell / (M * M);
  const float4 p = pos[q];
  int n = 0;
  const int span = M >= 3 ? 1 : 0;   // M < 3: every cell is a neighbor cell once
  for (int dz = -span; dz <= span; dz++)
    for (int dy = -span; dy <= span; dy++)
      for (int dx = -span; dx <= span; dx++) {
        if (M < 3 && (dx || dy || dz)) continue;
        const int nc = ((cx + dx + M) % M) + M * (((cy + dy + M) % M) + M * ((cz + dz + M) % M));
        const int r = c * M * M * M + nc;
        const int b0 = M < 3 ? c * M * M * M : r, b1 = M < 3 ? (c + 1) * M * M * M : r + 1;
        for (int k = starts[b0]; k < starts[b1]; k++) {
          const int j = sorted[k];
          if (j == q) continue;
          const float4 pj = pos[j];
          float ex = p.x - pj.x, ey = p.y - pj.y, ez = p.z - pj.z;
          ex -= G.L * rintf(ex * G.invL);
          ey -= G.L * rintf(ey * G.invL);
          ez -= G.L * rintf(ez * G.invL);
          if (ex * ex + ey * ey + ez * ez < G.rlist2) {
            if (n < cap) list[(size_t)n * total + q] = j;
            n++;
          }
        }
      }
  count[q] = n;
  if (n > cap) atomicMax(overflow, n);
}

struct PairGeom {
  float r, ux, uy, uz;   // distance and unit vector (i - j) / r
};

__device__ __forceinline__ bool pair_geom(const float4& pi, const float4& pj, const Geometry& G, PairGeom& pg) {
  float ex = pi.x - pj.x, ey = pi.y - pj.y, ez = pi.z - pj.z;
  ex -= G.L * rintf(ex * G.invL);
  ey -= G.L * rintf(ey * G.invL);
  ez -= G.L * rintf(ez * G.invL);
  const float r2 = ex * ex + ey * ey + ez * ez;
  if (!(r2 < G.rc2)) return false;
  const float r = sqrtf(r2), inv = 1.f / r;
  pg.r = r;
  pg.ux = ex * inv;
  pg.uy = ey * inv;
  pg.uz = ez * inv;
  return true;
}

// h_k = g_k fc and dh_k/dr for the 16 Gaussians (two-term product recurrence:
// g_{k+1} = g_k q_k, q_{k+1} = q_k c, c = exp(-2 a dmu^2))
__device__ __forceinline__ void radial(float r, const Geometry& G, float cdecay, float (&h)[NG], float (&dh)[NG]) {
  float s, co;
  sincospif(r / G.rc, &s, &co);
  const float fc = 0.5f * (co + 1.f), dfc = -0.5f * 3.14159265f / G.rc * s;
  const float x0 = r - G.mu0;
  float gk = __expf(-G.a * x0 * x0);
  float qk = __expf(2.f * G.a * G.dmu * x0 - G.a * G.dmu * G.dmu);
#pragma unroll
  for (int k = 0; k < NG; k++) {
    const float xk = r - (G.mu0 + k * G.dmu);
    h[k] = gk * fc;
    dh[k] = gk * (dfc - 2.f * G.a * xk * fc);
    gk *= qk;
    qk *= cdecay;
  }
}

__global__ void k_sg_desc(const float4* __restrict__ pos, Geometry G, const uint8_t* __restrict__ species,
                          const int* __restrict__ list, const int* __restrict__ count, int cap,
                          float* __restrict__ Gout) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = G.chains * G.N;
  if (q >= total) return;
  const float cdecay = __expf(-2.f * G.a * G.dmu * G.dmu);
  float acc[NS][NG];
#pragma unroll
  for (int c = 0; c < NS; c++)
#pragma unroll
    for (int k = 0; k < NG; k++) acc[c][k] = 0.f;
  const float4 pi = pos[q];
  const int n = min(count[q], cap);
  for (int e = 0; e < n; e++) {
    const int j = list[(size_t)e * total + q];
    PairGeom pg;
    if (!pair_geom(pi, pos[j], G, pg)) continue;
    float h[NG], dh[NG];
    radial(pg.r, G, cdecay, h, dh);
    if (species[j % G.N] == 0) {
#pragma unroll
      for (int k = 0; k < NG; k++) acc[0][k] += h[k];
    } else {
#pragma unroll
      for (int k = 0; k < NG; k++) acc[1][k] += h[k];
    }
  }
  float4* out = reinterpret_cast<float4*>(Gout + (size_t)q * DIN);
#pragma unroll
  for (int c = 0; c < NS; c++)
#pragma unroll
    for (int k = 0; k < NG; k += 4) out[(c * NG + k) / 4] = make_float4(acc[c][k], acc[c][k + 1], acc[c][k + 2], acc[c][k + 3]);
}

// F_i = -sum_j s_ij r_hat_ij, s_ij = sum_k (dEdG_i[s_j, k] + dEdG_j[s_i, k]) dh_k(r_ij)
__global__ void k_sg_force(const float4* __restrict__ pos, Geometry G, const uint8_t* __restrict__ species,
                           const int* __restrict__ list, const int* __restrict__ count, int cap,
                           const float* __restrict__ dEdG, double* __restrict__ F) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = G.chains * G.N;
  if (q >= total) return;
  const float cdecay = __expf(-2.f * G.a * G.dmu * G.dmu);
  const int si = species[q % G.N];
  const float4 pi = pos[q];
  const float* gi = dEdG + (size_t)q * DIN;
  const int n = min(count[q], cap);
  float fx = 0.f, fy = 0.f, fz = 0.f;
  for (int e = 0; e < n; e++) {
    const int j = list[(size_t)e * total + q];
    PairGeom pg;
    if (!pair_geom(pi, pos[j], G, pg)) continue;
    float h[NG], dh[NG];
    radial(pg.r, G, cdecay, h, dh);
    const int sj = species[j % G.N];
    const float4* a = reinterpret_cast<const float4*>(gi + sj * NG);
    const float4* b = reinterpret_cast<const float4*>(dEdG + (size_t)j * DIN + si * NG);
    float s = 0.f;
#pragma unroll
    for (int k4 = 0; k4 < NG / 4; k4++) {
      const float4 x = a[k4], y = __ldg(&b[k4]);
      s += (x.x + y.x) * dh[4 * k4] + (x.y + y.y) * dh[4 * k4 + 1] + (x.z + y.z) * dh[4 * k4 + 2] +
           (x.w + y.w) * dh[4 * k4 + 3];
    }
    fx -= s * pg.ux;
    fy -= s * pg.uy;
    fz -= s * pg.uz;
  }
  F[3 * q] = fx;
  F[3 * q + 1] = fy;
  F[3 * q + 2] = fz;
}

// u_i[s_j, k] = sum_j dh_k(r_ij) (v_i - v_j) . r_hat_ij (force residual in descriptor space)
__global__ void k_sg_udesc(const float4* __restrict__ pos, Geometry G, const uint8_t* __restrict__ species,
                           const int* __restrict__ list, const int* __restrict__ count, int cap,
                           const float* __restrict__ v, float* __restrict__ U) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = G.chains * G.N;
  if (q >= total) return;
  const float cdecay = __expf(-2.f * G.a * G.dmu * G.dmu);
  float acc[NS][NG];
#pragma unroll
  for (int c = 0; c < NS; c++)
#pragma unroll
    for (int k = 0; k < NG; k++) acc[c][k] = 0.f;
  const float4 pi = pos[q];
  const float vix = v[3 * q], viy = v[3 * q + 1], viz = v[3 * q + 2];
  const int n = min(count[q], cap);
  for (int e = 0; e < n; e++) {
    const int j = list[(size_t)e * total + q];
    PairGeom pg;
    if (!pair_geom(pi, pos[j], G, pg)) continue;
    float h[NG], dh[NG];
    radial(pg.r, G, cdecay, h, dh);
    const float w = (vix - v[3 * j]) * pg.ux + (viy - v[3 * j + 1]) * pg.uy + (viz - v[3 * j + 2]) * pg.uz;
    if (species[j % G.N] == 0) {
#pragma unroll
      for (int k = 0; k < NG; k++) acc[0][k] += dh[k] * w;
    } else {
#pragma unroll
      for (int k = 0; k < NG; k++) acc[1][k] += dh[k] * w;
    }
  }
  float* out = U + (size_t)q * DIN;
#pragma unroll
  for (int c = 0; c < NS; c++)
#pragma unroll
    for (int k = 0; k < NG; k++) out[c * NG + k] = acc[c][k];
}

// ---- network: inference -----------------------------------------------------------

// tiles: (first index into the atom list, count <= 64, species)
struct TileArgs {
  const int* atoms;    // atom indices (global), species by species within each chain
  const int3* tiles;   // (start, count, species)
  int ntiles;
};

struct MlpSmem {
  WeightsSmem w[NS];
  __nv_bfloat16 X[4][16][H + 8];   // per warp activations (BF16 GEMM operand)
  __nv_bfloat16 Y[4][16][H + 8];
};

// E_i and dE/dG_i for every atom; one block per tile of <= 64 atoms of one species
__global__ void __launch_bounds__(128) k_sg_mlp(TileArgs T, const float* __restrict__ params,
                                                const float* __restrict__ Gin, float* __restrict__ Eatom,
                                                float* __restrict__ dEdG) {
  extern __shared__ __align__(16) unsigned char raw[];
  MlpSmem& S = *reinterpret_cast<MlpSmem*>(raw);
  const int3 tile = T.tiles[blockIdx.x];
  const int sp = tile.z;
  load_weights(S.w[sp], params + sp * PER_SPECIES);
  __syncthreads();
  const WeightsSmem& W = S.w[sp];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int base = tile.x + warp * 16, nrow = min(16, tile.y - warp * 16);
  if (nrow <= 0) return;
  __nv_bfloat16(*X)[H + 8] = S.X[warp];
  __nv_bfloat16(*Y)[H + 8] = S.Y[warp];
  // G rows -> X (BF16)
  for (int q = lane; q < 16 * DIN; q += 32) {
    const int r = q / DIN, k = q % DIN;
    X[r][k] = __float2bfloat16(r < nrow ? Gin[(size_t)T.atoms[base + r] * DIN + k] : 0.f);
  }
  __syncwarp();
  float z1[8][4], z2[8][4];
  zero(z1);
  warp_gemm<DIN, 8>(&X[0][0], H + 8, &W.W1t[0][0], DIN + 8, z1);
#pragma unroll
  for (int n = 0; n < 8; n++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      z1[n][q] += W.b1[frag_col(n, q)];
      Y[frag_row(q)][frag_col(n, q)] = __float2bfloat16(silu(z1[n][q]));
    }
  __syncwarp();
  zero(z2);
  warp_gemm<H, 8>(&Y[0][0], H + 8, &W.W2t[0][0], H + 8, z2);
  float e[2] = {0.f, 0.f};   // rows g and g + 8
  __syncwarp();
#pragma unroll
  for (int n = 0; n < 8; n++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int col = frag_col(n, q);
      const float z = z2[n][q] + W.b2[col];
      e[q >> 1] += W.w3[col] * silu(z);
      X[frag_row(q)][col] = __float2bfloat16(W.w3[col] * dsilu(z));   // dE/dz2
    }
#pragma unroll
  for (int h = 0; h < 2; h++) {
    e[h] += __shfl_xor_sync(0xffffffffu, e[h], 1);
    e[h] += __shfl_xor_sync(0xffffffffu, e[h], 2);
  }
  if ((lane & 3) == 0) {
    const int g = lane >> 2;
    if (g < nrow) Eatom[T.atoms[base + g]] = e[0] + W.b3;
    if (g + 8 < nrow) Eatom[T.atoms[base + g + 8]] = e[1] + W.b3;
  }
  __syncwarp();
  float d1[8][4];
  zero(d1);
  warp_gemm<H, 8>(&X[0][0], H + 8, &W.W2[0][0], H + 8, d1);   // dE/da1 = dE/dz2 W2^T
  __syncwarp();
#pragma unroll
  for (int n = 0; n < 8; n++)
#pragma unroll
    for (int q = 0; q < 4; q++) Y[frag_row(q)][frag_col(n, q)] = __float2bfloat16(d1[n][q] * dsilu(z1[n][q]));
  __syncwarp();
  float dg[4][4];
  zero(dg);
  warp_gemm<H, 4>(&Y[0][0], H + 8, &W.W1[0][0], H + 8, dg);   // dE/dG = dE/dz1 W1^T
#pragma unroll
  for (int n = 0; n < 4; n++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = frag_row(q);
      if (r < nrow) dEdG[(size_t)T.atoms[base + r] * DIN + frag_col(n, q)] = dg[n][q];
    }
}

// ---- network: inference on the 5th-generation tensor cores (tcgen05) --------------
//
// The same computation as k_sg_mlp (BF16 operands rounded at the same points, FP32
// accumulation) with tcgen05.mma: M = 128 atoms per tile (one species), operands in
// shared memory in the canonical K-major layout without swizzle, accumulators in
// tensor memory.  Persistent blocks of 128 threads hold the BF16 weights of both
// species for their whole life and take 128-atom tiles in turn; thread t owns row t
// of a tile, which is TMEM lane t (warp w reads lanes 32w..32w+31).  Thread 0
// issues each GEMM (one tcgen05.mma per K = 16) and commits it to an mbarrier that
// every thread waits on.  Per tile:
//   Z1 = G W1          TMEM columns   0..63   (K = 32)
//   A1 = silu(Z1 + b1) -> smem X,  Z2 = A1 W2               columns  64..127
//   E = w3 . silu(Z2 + b2) + b3,  dZ2 = w3 silu'(Z2 + b2) -> X
//   dA1 = dZ2 W2^T                                          columns 128..191
//   dZ1 = dA1 silu'(Z1 + b1) -> X,  dE/dG = dZ1 W1^T        columns 192..223 (N = 32)
// Waits are bounded: a wait that runs out sets *err, the block stops taking tiles,
// frees its tensor memory and returns (the host reports the error).

constexpr int TC_M = 128, TC_COLS = 256;

// byte offset of element (r, k) of a K-major operand with K columns: 8 x 16-byte core
// matrices, consecutive along K (leading byte offset 128), row groups of 8 K/8 core
// matrices apart (stride byte offset 16 K)
__host__ __device__ constexpr int tc_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

struct TcWeights {   // one species, BF16 B operands (rows n, K contiguous) and FP32 vectors
  alignas(128) unsigned char B1[64 * 32 * 2];   // Z1:  B1[n][k] = W1[k][n]   (N 64, K 32)
  alignas(128) unsigned char B2[64 * 64 * 2];   // Z2:  B2[n][k] = W2[k][n]   (N 64, K 64)
  alignas(128) unsigned char B3[64 * 64 * 2];   // dA1: B3[n][k] = W2[n][k]   (N 64, K 64)
  alignas(128) unsigned char B4[32 * 64 * 2];   // dG:  B4[n][k] = W1[n][k]   (N 32, K 64)
  float b1[H], b2[H], w3[H], b3;
};

struct TcSmem {
  TcWeights w[NS];
  alignas(128) unsigned char G[TC_M * DIN * 2];   // A operand of Z1 (K 32)
  alignas(128) unsigned char X[TC_M * H * 2];     // A operand of the other GEMMs (K 64)
  alignas(8) unsigned long long bar;
  unsigned int taddr;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading and stride byte offsets,
// descriptor version 1, no swizzle
__device__ __forceinline__ unsigned long long tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[128 x K] B[K x N], issued by one thread, K / 16 instructions
template <int K, int N>
__device__ __forceinline__ void tc_gemm(uint32_t dtmem, const unsigned char* A, const unsigned char* B) {
  const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
  constexpr uint32_t idesc = tc_idesc(TC_M, N);
#pragma unroll
  for (int s = 0; s < K / 16; s++) {
    const unsigned long long ad = tc_sdesc(a0 + 256u * s, 128u, 16u * K), bd = tc_sdesc(b0 + 256u * s, 128u, 16u * K);
    const uint32_t acc = s > 0 ? 1u : 0u;
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
  }
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// bounded wait for the phase; false if it did not complete
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t phase) {
  for (int i = 0; i < (1 << 22); i++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

// 8 BF16 values (from 8 floats) into one 16-byte chunk of a K-major operand
__device__ __forceinline__ void tc_st8(unsigned char* base, int r, int k, int K, const float* v) {
  uint4 w;
  __nv_bfloat162 h[4];
#pragma unroll
  for (int q = 0; q < 4; q++) h[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
  memcpy(&w, h, 16);
  *reinterpret_cast<uint4*>(base + tc_off(r, k, K)) = w;
}

__device__ void tc_load_weights(TcWeights& w, const float* p) {
  for (int q = threadIdx.x; q < DIN * H; q += blockDim.x) {
    const int k = q / H, n = q % H;   // W1[k][n]
    const __nv_bfloat16 v = __float2bfloat16(p[OFF_W1 + q]);
    *reinterpret_cast<__nv_bfloat16*>(w.B1 + tc_off(n, k, DIN)) = v;   // B1[n][k]
    *reinterpret_cast<__nv_bfloat16*>(w.B4 + tc_off(k, n, H)) = v;     // B4[k][n] (rows: input index)
  }
  for (int q = threadIdx.x; q < H * H; q += blockDim.x) {
    const int k = q / H, n = q % H;   // W2[k][n]
    const __nv_bfloat16 v = __float2bfloat16(p[OFF_W2 + q]);
    *reinterpret_cast<__nv_bfloat16*>(w.B2 + tc_off(n, k, H)) = v;   // B2[n][k]
    *reinterpret_cast<__nv_bfloat16*>(w.B3 + tc_off(k, n, H)) = v;   // B3[k][n] (rows: a1 index)
  }
  for (int q = threadIdx.x; q < H; q += blockDim.x) {
    w.b1[q] = p[OFF_B1 + q];
    w.b2[q] = p[OFF_B2 + q];
    w.w3[q] = p[OFF_W3 + q];
  }
  if (threadIdx.x == 0) w.b3 = p[OFF_B3];
}

__global__ void __launch_bounds__(128, 1) k_sg_mlp_tc(TileArgs T, const float* __restrict__ params,
                                                      const float* __restrict__ Gin, float* __restrict__ Eatom,
                                                      float* __restrict__ dEdG, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(raw);
  const int t = threadIdx.x, warp = t >> 5;
  for (int sp = 0; sp < NS; sp++) tc_load_weights(S.w[sp], params + sp * PER_SPECIES);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.taddr)),
                 "r"(TC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = S.taddr, bar = smem_u32(&S.bar);
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;   // this warp's TMEM lanes
  uint32_t phase = 0;
  bool ok = true;
  // one GEMM: operands written by all threads before, accumulator read by all after;
  // ok stays block-uniform (every thread leaves the tile loop together)
  auto run = [&](auto&& issue) {
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    if (t == 0) {
      tc_fence_after();
      issue();
      tc_commit(bar);
    }
    ok = __syncthreads_and(tc_wait(bar, phase) ? 1 : 0) != 0;
    if (ok) phase ^= 1u;
    tc_fence_after();
  };
  for (int ti = blockIdx.x; ti < T.ntiles; ti += gridDim.x) {
    const int3 tile = T.tiles[ti];
    const TcWeights& W = S.w[tile.z];
    const bool have = t < tile.y;
    const int atom = have ? T.atoms[tile.x + t] : 0;
    {   // G row -> BF16 A operand
      float g[DIN];
#pragma unroll
      for (int k = 0; k < DIN; k += 4) {
        const float4 v = have ? *reinterpret_cast<const float4*>(Gin + (size_t)atom * DIN + k) : make_float4(0.f, 0.f, 0.f, 0.f);
        g[k] = v.x;
        g[k + 1] = v.y;
        g[k + 2] = v.z;
        g[k + 3] = v.w;
      }
#pragma unroll
      for (int k = 0; k < DIN; k += 8) tc_st8(S.G, t, k, DIN, g + k);
    }
    run([&] { tc_gemm<DIN, H>(tm + 0, S.G, W.B1); });
    if (!ok) break;
#pragma unroll
    for (int c = 0; c < H; c += 16) {   // A1 = silu(Z1 + b1)
      float z[16];
      tc_ld16(tm + lane_base + c, z);
#pragma unroll
      for (int q = 0; q < 16; q++) z[q] = silu(z[q] + W.b1[c + q]);
      tc_st8(S.X, t, c, H, z);
      tc_st8(S.X, t, c + 8, H, z + 8);
    }
    run([&] { tc_gemm<H, H>(tm + 64, S.X, W.B2); });
    if (!ok) break;
    float e = 0.f;
#pragma unroll
    for (int c = 0; c < H; c += 16) {   // E and dE/dZ2
      float z[16];
      tc_ld16(tm + lane_base + 64 + c, z);
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const float u = z[q] + W.b2[c + q];
        e += W.w3[c + q] * silu(u);
        z[q] = W.w3[c + q] * dsilu(u);
      }
      tc_st8(S.X, t, c, H, z);
      tc_st8(S.X, t, c + 8, H, z + 8);
    }
    if (have) Eatom[atom] = e + W.b3;
    run([&] { tc_gemm<H, H>(tm + 128, S.X, W.B3); });
    if (!ok) break;
#pragma unroll
    for (int c = 0; c < H; c += 16) {   // dE/dZ1 = dE/dA1 silu'(Z1 + b1)
      float d[16], z[16];
      tc_ld16(tm + lane_base + 128 + c, d);
      tc_ld16(tm + lane_base + c, z);
#pragma unroll
      for (int q = 0; q < 16; q++) d[q] *= dsilu(z[q] + W.b1[c + q]);
      tc_st8(S.X, t, c, H, d);
      tc_st8(S.X, t, c + 8, H, d + 8);
    }
    run([&] { tc_gemm<H, DIN>(tm + 192, S.X, W.B4); });
    if (!ok) break;
#pragma unroll
    for (int c = 0; c < DIN; c += 16) {   // dE/dG
      float d[16];
      tc_ld16(tm + lane_base + 192 + c, d);
      if (have)
#pragma unroll
        for (int q = 0; q < 16; q += 4)
          *reinterpret_cast<float4*>(dEdG + (size_t)atom * DIN + c + q) = make_float4(d[q], d[q + 1], d[q + 2], d[q + 3]);
    }
  }
  if (!ok && t == 0) {
    atomicExch(err, 1);
    tc_wait(bar, phase);   // the GEMM in flight, if it completes after all (bounded)
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(TC_COLS) : "memory");
  }
}

// ---- network: training gradient -----------------------------------------------------
//
// Per atom: O_i = e_c(i) E_i - t_i,  t_i = dE_i/dG_i . u_i.  With z1 = G W1 + b1,
// a1 = silu(z1), z2 = a1 W2 + b2, a2 = silu(z2), E = a2 . w3 + b3 and the tangent
// dz1 = u W1, da1 = silu'(z1) dz1, dz2 = da1 W2, da2 = silu'(z2) dz2, t = da2 . w3:
//   dO/dw3 = e a2 - da2,                 dO/db3 = e
//   gz2  = e w3 silu'(z2) - w3 dz2 silu''(z2)        (dO/dz2)
//   gdz2 = -w3 silu'(z2)                               (dO/ddz2)
//   dO/dW2 = a1^T gz2 + da1^T gdz2,       dO/db2 = gz2
//   gz1  = (gz2 W2^T) silu'(z1) + (gdz2 W2^T) dz1 silu''(z1)
//   gdz1 = (gdz2 W2^T) silu'(z1)
//   dO/dW1 = G^T gz1 + u^T gdz1,          dO/db1 = gz1
// The weight gradients are GEMMs over the tile's atoms: [A1; dA1]^T [GZ2; GDZ2] and
// [G; U]^T [GZ1; GDZ1], K = 2 x 64 atoms, on the tensor cores.

struct TrainSmem {
  WeightsSmem w;
  __nv_bfloat16 in[2 * TILE][DIN + 8];       // rows: G (64), U (64)
  __nv_bfloat16 act[2 * TILE][H + 8];        // rows: a1 (64), da1 (64)
  __nv_bfloat16 gz2[2 * TILE][H + 8];        // rows: gz2 (64), gdz2 (64)
  __nv_bfloat16 gz1[2 * TILE][H + 8];        // rows: gz1 (64), gdz1 (64)
  __nv_bfloat16 tA[H][2 * TILE + 8];         // transposed operands of the weight GEMMs
  __nv_bfloat16 tB[H][2 * TILE + 8];
  float vb1[H], vb2[H], vw3[H], vb3;
};

// one launch per species; block b processes tiles b, b + gridDim.x, ... of that species and
// writes its gradient partial (PER_SPECIES floats) to part[b]
__global__ void __launch_bounds__(128) k_sg_train(TileArgs T, int species, const float* __restrict__ params,
                                                  const float* __restrict__ Gin, const float* __restrict__ Uin,
                                                  const float* __restrict__ eAtom, float* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char raw[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(raw);
  load_weights(S.w, params + species * PER_SPECIES);
  for (int q = threadIdx.x; q < H; q += blockDim.x) S.vb1[q] = S.vb2[q] = S.vw3[q] = 0.f;
  if (threadIdx.x == 0) S.vb3 = 0.f;
  __syncthreads();
  const WeightsSmem& W = S.w;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // weight-gradient accumulators: W2 (64 x 64): warp w owns rows 16w..16w+15 (8 n-tiles);
  // W1 (32 x 64): warp w owns rows 16 (w & 1).., columns 32 (w >> 1).. (4 n-tiles)
  float gW2[8][4], gW1[4][4];
  zero(gW2);
  zero(gW1);
  for (int ti = blockIdx.x; ti < T.ntiles; ti += gridDim.x) {
    const int3 tile = T.tiles[ti];
    if (tile.z != species) continue;
    const int r0 = warp * 16;   // this warp's rows in the tile
    const int nrow = max(0, min(16, tile.y - r0));
    // inputs: G and U rows (zero rows beyond the tile)
    for (int q = lane; q < 16 * DIN; q += 32) {
      const int r = q / DIN, k = q % DIN;
      const bool ok = r < nrow;
      const size_t a = ok ? (size_t)T.atoms[tile.x + r0 + r] : 0;
      S.in[r0 + r][k] = __float2bfloat16(ok ? Gin[a * DIN + k] : 0.f);
      S.in[TILE + r0 + r][k] = __float2bfloat16(ok ? Uin[a * DIN + k] : 0.f);
    }
    __syncwarp();
    float z1[8][4], dz1[8][4];
    zero(z1);
    zero(dz1);
    warp_gemm<DIN, 8>(&S.in[r0][0], DIN + 8, &W.W1t[0][0], DIN + 8, z1);
    warp_gemm<DIN, 8>(&S.in[TILE + r0][0], DIN + 8, &W.W1t[0][0], DIN + 8, dz1);
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int r = frag_row(q), c = frag_col(n, q);
        z1[n][q] += W.b1[c];
        const float a = r < nrow ? silu(z1[n][q]) : 0.f, da = r < nrow ? dsilu(z1[n][q]) * dz1[n][q] : 0.f;
        S.act[r0 + r][c] = __float2bfloat16(a);
        S.act[TILE + r0 + r][c] = __float2bfloat16(da);
      }
    __syncwarp();
    float z2[8][4], dz2[8][4];
    zero(z2);
    zero(dz2);
    warp_gemm<H, 8>(&S.act[r0][0], H + 8, &W.W2t[0][0], H + 8, z2);
    warp_gemm<H, 8>(&S.act[TILE + r0][0], H + 8, &W.W2t[0][0], H + 8, dz2);
    float e[2];
    {
      const int g = lane >> 2;
      e[0] = g < nrow ? eAtom[T.atoms[tile.x + r0 + g]] : 0.f;
      e[1] = g + 8 < nrow ? eAtom[T.atoms[tile.x + r0 + g + 8]] : 0.f;
    }
    float lb3 = 0.f;
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int r = frag_row(q), c = frag_col(n, q);
        const float ec = e[q >> 1], z = z2[n][q] + W.b2[c], w3 = W.w3[c];
        const float s1 = dsilu(z), s2 = d2silu(z);
        const float g2 = ec * w3 * s1 - w3 * dz2[n][q] * s2, gd2 = -w3 * s1;
        const bool ok = r < nrow;
        S.gz2[r0 + r][c] = __float2bfloat16(ok ? g2 : 0.f);
        S.gz2[TILE + r0 + r][c] = __float2bfloat16(ok ? gd2 : 0.f);
        if (ok) {
          atomicAdd(&S.vb2[c], g2);
          atomicAdd(&S.vw3[c], ec * silu(z) - s1 * dz2[n][q]);
        }
        if (ok && n == 0 && (q & 1) == 0 && (threadIdx.x & 3) == 0) lb3 += ec;
      }
    if (lb3 != 0.f) atomicAdd(&S.vb3, lb3);
    __syncwarp();
    float p1[8][4], p2[8][4];
    zero(p1);
    zero(p2);
    warp_gemm<H, 8>(&S.gz2[r0][0], H + 8, &W.W2[0][0], H + 8, p1);          // gz2 W2^T
    warp_gemm<H, 8>(&S.gz2[TILE + r0][0], H + 8, &W.W2[0][0], H + 8, p2);   // gdz2 W2^T
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int r = frag_row(q), c = frag_col(n, q);
        const float s1 = dsilu(z1[n][q]), s2 = d2silu(z1[n][q]);
        const bool ok = r < nrow;
        const float g1 = p1[n][q] * s1 + p2[n][q] * dz1[n][q] * s2, gd1 = p2[n][q] * s1;
        S.gz1[r0 + r][c] = __float2bfloat16(ok ? g1 : 0.f);
        S.gz1[TILE + r0 + r][c] = __float2bfloat16(ok ? gd1 : 0.f);
        if (ok) atomicAdd(&S.vb1[c], g1);
      }
    __syncthreads();
    // dW2 += [a1; da1]^T [gz2; gdz2]: A = tA (64 units x 128 atoms), B^T = tB (64 units x 128 atoms)
    for (int q = threadIdx.x; q < 2 * TILE * H; q += blockDim.x) {
      const int r = q / H, c = q % H;
      S.tA[c][r] = S.act[r][c];
      S.tB[c][r] = S.gz2[r][c];
    }
    __syncthreads();
    warp_gemm<2 * TILE, 8>(&S.tA[16 * warp][0], 2 * TILE + 8, &S.tB[0][0], 2 * TILE + 8, gW2);
    __syncthreads();
    // dW1 += [G; U]^T [gz1; gdz1]: A = in^T (32 inputs x 128 atoms), B^T = gz1^T (64 x 128)
    for (int q = threadIdx.x; q < 2 * TILE * H; q += blockDim.x) {
      const int r = q / H, c = q % H;
      if (c < DIN) S.tA[c][r] = S.in[r][c];
      S.tB[c][r] = S.gz1[r][c];
    }
    __syncthreads();
    warp_gemm<2 * TILE, 4>(&S.tA[16 * (warp & 1)][0], 2 * TILE + 8, &S.tB[32 * (warp >> 1)][0], 2 * TILE + 8, gW1);
    __syncthreads();
  }
  // block partial, FP32: layout of the packed parameters of one species
  float* out = part + (size_t)blockIdx.x * PER_SPECIES;
#pragma unroll
  for (int n = 0; n < 8; n++)
#pragma unroll
    for (int q = 0; q < 4; q++) out[OFF_W2 + (16 * warp + frag_row(q)) * H + frag_col(n, q)] = gW2[n][q];
#pragma unroll
  for (int n = 0; n < 4; n++)
#pragma unroll
    for (int q = 0; q < 4; q++)
      out[OFF_W1 + (16 * (warp & 1) + frag_row(q)) * H + 32 * (warp >> 1) + frag_col(n, q)] = gW1[n][q];
  __syncthreads();
  for (int q = threadIdx.x; q < H; q += blockDim.x) {
    out[OFF_B1 + q] = S.vb1[q];
    out[OFF_B2 + q] = S.vb2[q];
    out[OFF_W3 + q] = S.vw3[q];
  }
  if (threadIdx.x == 0) out[OFF_B3] = S.vb3;
}

// grad[p] = sum over blocks (in order) of part[b][p]
__global__ void k_sg_reduce(const float* __restrict__ part, int blocks, int n, float scale, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float s = 0.f;
  for (int b = 0; b < blocks; b++) s += part[(size_t)b * n + p];
  grad[p] = scale * s;
}

__global__ void k_sg_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// per-chain sums of per-atom FP32 values, in atom order within each 256-atom block, blocks in order
__global__ void k_sg_chain_sum(const float* __restrict__ x, int N, double* __restrict__ out) {
  const int c = blockIdx.x;
  __shared__ double ws[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s += (double)x[(size_t)c * N + i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += ws[w];
    out[c] = t;
  }
}

// velocity Verlet pieces for the chains (FP64, unit masses)
__global__ void k_sg_kick_drift(double* __restrict__ R, double* __restrict__ P, const double* __restrict__ F, int n3,
                                double half, double dt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  const double p = P[q] + half * F[q];
  P[q] = p;
  R[q] = R[q] + dt * p;
}
__global__ void k_sg_kick(double* __restrict__ P, const double* __restrict__ F, int n3, double half) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  P[q] = P[q] + half * F[q];
}

}  // namespace sg

// ---- host ---------------------------------------------------------------------------

struct Surrogate {
  sg::Geometry G;
  int total = 0, cap = 0;
  double L = 0, skin = 0;
  uint8_t* dSpecies = nullptr;
  std::vector<int3> tiles, tiles128;   // tiles of <= 64 and of <= 128 atoms of one species
  int* dAtoms = nullptr;
  int3* dTiles = nullptr;
  int3* dTiles128 = nullptr;
  int* dTcError = nullptr;
  float4* dPos = nullptr;
  int *dCellOf = nullptr, *dCounts = nullptr, *dStarts = nullptr, *dCursor = nullptr, *dSorted = nullptr;
  int *dList = nullptr, *dCount = nullptr, *dOverflow = nullptr;
  float *dG = nullptr, *dEatom = nullptr, *dEdG = nullptr, *dU = nullptr, *dV = nullptr, *dEres = nullptr;
  float *dParams = nullptr, *dPart = nullptr, *dGrad = nullptr, *dM = nullptr, *dVar = nullptr;
  int trainBlocks = 0;
  double* dR0 = nullptr;   // positions of the last list build
};

static int sg_blocks(int n) { return (n + 255) / 256; }

static void sg_build_lists(Surrogate& S, const double* dR, cudaStream_t st) {
  using namespace sg;
  const int cells = S.G.chains * S.G.M * S.G.M * S.G.M;
  k_sg_pack<<<sg_blocks(S.total), 256, 0, st>>>(dR, S.total, S.L, S.dPos);
  CK(cudaMemsetAsync(S.dCounts, 0, sizeof(int) * cells, st));
  CK(cudaMemsetAsync(S.dCursor, 0, sizeof(int) * cells, st));
  k_sg_count<<<sg_blocks(S.total), 256, 0, st>>>(S.dPos, S.G, S.dCellOf, S.dCounts);
  k_sg_scan<<<1, 256, 0, st>>>(S.dCounts, cells, S.dStarts);
  k_sg_scatter<<<sg_blocks(S.total), 256, 0, st>>>(S.dCellOf, S.G, S.dStarts, S.dCursor, S.dSorted);
  k_sg_sort<<<sg_blocks(cells), 256, 0, st>>>(S.dStarts, cells, S.dSorted);
  k_sg_list<<<sg_blocks(S.total), 256, 0, st>>>(S.dPos, S.G, S.dCellOf, S.dStarts, S.dSorted, S.cap, S.dList,
                                                 S.dCount, S.dOverflow);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(S.dR0, dR, sizeof(double) * 3 * S.total, cudaMemcpyDeviceToDevice, st));
}

// Dynamic shared memory of k_sg_mlp_tc: at least 100 KB, so that at most two blocks
// (2 x 256 tensor-memory columns of the SM's 512) share an SM.
static size_t tc_smem_bytes() { return std::max(sizeof(sg::TcSmem) + 1024, (size_t)100 * 1024); }

// The network: tcgen05 kernel (default) or the mma.sync one (EMDEE_SG_MMA=sync).
static void sg_network(Surrogate& S, const float* dParams, cudaStream_t st) {
  using namespace sg;
  const char* e = getenv("EMDEE_SG_MMA");
  if (e && !strcmp(e, "sync")) {
    TileArgs T{S.dAtoms, S.dTiles, (int)S.tiles.size()};
    k_sg_mlp<<<T.ntiles, 128, sizeof(MlpSmem), st>>>(T, dParams, S.dG, S.dEatom, S.dEdG);
  } else {
    TileArgs T{S.dAtoms, S.dTiles128, (int)S.tiles128.size()};
    const int blocks = std::min(T.ntiles, 2 * 152);
    k_sg_mlp_tc<<<blocks, 128, tc_smem_bytes(), st>>>(T, dParams, S.dG, S.dEatom, S.dEdG, S.dTcError);
  }
  CK(cudaGetLastError());
}

}  // namespace emdee

using namespace emdee;

extern "C" {

int EmDee_surrogate_param_count(void) { return sg::NPARAM; }

// chains x N atoms (positions chain-major, FP64 [chains][N][3]); types[N] in {1, 2},
// shared by all chains; cubic box L; descriptor cut-off rc; Verlet-list skin; Gaussian
// centres mu0..mu15 (uniform), width w
void* EmDee_surrogate_create(int chains, int N, double L, const int* types, double rc, double skin, double mu0,
                             double mu15, double width) {
  using namespace sg;
  const char* task = "surrogate setup";
  if (chains < 1 || N < 2 || !(L > 0) || !(rc > 0)) fatal(task, "invalid arguments");
  Surrogate* S = new Surrogate;
  S->total = chains * N;
  S->L = L;
  S->skin = skin;
  Geometry& G = S->G;
  G.chains = chains;
  G.N = N;
  G.M = std::max(1, (int)std::floor(L / (rc + skin)));
  G.L = (float)L;
  G.invL = (float)(1.0 / L);
  G.rc = (float)rc;
  G.rc2 = (float)(rc * rc);
  G.rlist2 = (float)((rc + skin) * (rc + skin));
  G.mu0 = (float)mu0;
  G.dmu = (float)((mu15 - mu0) / 15.0);
  G.a = (float)(1.0 / (2.0 * width * width));
  std::vector<uint8_t> sp(N);
  for (int i = 0; i < N; i++) {
    if (types[i] != 1 && types[i] != 2) fatal(task, "species must be 1 or 2");
    sp[i] = (uint8_t)(types[i] - 1);
  }
  CK(cudaMalloc(&S->dSpecies, N));
  CK(cudaMemcpy(S->dSpecies, sp.data(), N, cudaMemcpyHostToDevice));
  // tiles of <= 64 atoms of one species, chain by chain, and over the same atom
  // list tiles of <= 128 (the tensor-memory kernel's M)
  std::vector<int> atoms;
  for (int c = 0; c < chains; c++)
    for (int s = 0; s < NS; s++) {
      std::vector<int> list;
      for (int i = 0; i < N; i++)
        if (sp[i] == s) list.push_back(c * N + i);
      const int first = (int)atoms.size();
      for (size_t b = 0; b < list.size(); b += TILE) {
        const int cnt = (int)std::min<size_t>(TILE, list.size() - b);
        S->tiles.push_back(make_int3((int)atoms.size(), cnt, s));
        atoms.insert(atoms.end(), list.begin() + b, list.begin() + b + cnt);
      }
      for (size_t b = 0; b < list.size(); b += TC_M)
        S->tiles128.push_back(make_int3(first + (int)b, (int)std::min<size_t>(TC_M, list.size() - b), s));
    }
  CK(cudaMalloc(&S->dAtoms, sizeof(int) * atoms.size()));
  CK(cudaMemcpy(S->dAtoms, atoms.data(), sizeof(int) * atoms.size(), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&S->dTiles, sizeof(int3) * S->tiles.size()));
  CK(cudaMemcpy(S->dTiles, S->tiles.data(), sizeof(int3) * S->tiles.size(), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&S->dTiles128, sizeof(int3) * S->tiles128.size()));
  CK(cudaMemcpy(S->dTiles128, S->tiles128.data(), sizeof(int3) * S->tiles128.size(), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&S->dTcError, sizeof(int)));
  CK(cudaMemset(S->dTcError, 0, sizeof(int)));
  const int cells = chains * G.M * G.M * G.M;
  const double rho = N / (L * L * L);
  S->cap = std::max(64, ((int)(2.0 * 4.18879 * std::pow(rc + skin, 3) * rho) + 31) / 32 * 32);
  const size_t T = S->total;
  CK(cudaMalloc(&S->dPos, sizeof(float4) * T));
  CK(cudaMalloc(&S->dCellOf, sizeof(int) * T));
  CK(cudaMalloc(&S->dCounts, sizeof(int) * cells));
  CK(cudaMalloc(&S->dCursor, sizeof(int) * cells));
  CK(cudaMalloc(&S->dStarts, sizeof(int) * (cells + 1)));
  CK(cudaMalloc(&S->dSorted, sizeof(int) * T));
  CK(cudaMalloc(&S->dList, sizeof(int) * T * S->cap));
  CK(cudaMalloc(&S->dCount, sizeof(int) * T));
  CK(cudaMalloc(&S->dOverflow, sizeof(int)));
  CK(cudaMemset(S->dOverflow, 0, sizeof(int)));
  CK(cudaMalloc(&S->dG, sizeof(float) * T * DIN));
  CK(cudaMalloc(&S->dU, sizeof(float) * T * DIN));
  CK(cudaMalloc(&S->dEdG, sizeof(float) * T * DIN));
  CK(cudaMalloc(&S->dEatom, sizeof(float) * T));
  CK(cudaMalloc(&S->dEres, sizeof(float) * T));
  CK(cudaMalloc(&S->dV, sizeof(float) * 3 * T));
  CK(cudaMalloc(&S->dParams, sizeof(float) * NPARAM));
  CK(cudaMemset(S->dParams, 0, sizeof(float) * NPARAM));
  CK(cudaMalloc(&S->dGrad, sizeof(float) * NPARAM));
  CK(cudaMalloc(&S->dM, sizeof(float) * NPARAM));
  CK(cudaMalloc(&S->dVar, sizeof(float) * NPARAM));
  CK(cudaMemset(S->dM, 0, sizeof(float) * NPARAM));
  CK(cudaMemset(S->dVar, 0, sizeof(float) * NPARAM));
  S->trainBlocks = 2 * 152;
  CK(cudaMalloc(&S->dPart, sizeof(float) * (size_t)S->trainBlocks * PER_SPECIES));
  CK(cudaMalloc(&S->dR0, sizeof(double) * 3 * T));
  CK(cudaFuncSetAttribute(k_sg_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpSmem)));
  CK(cudaFuncSetAttribute(k_sg_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
  CK(cudaFuncSetAttribute(k_sg_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem)));
  return S;
}

void EmDee_surrogate_set_params(void* h, const float* params) {
  Surrogate& S = *(Surrogate*)h;
  CK(cudaMemcpy(S.dParams, params, sizeof(float) * sg::NPARAM, cudaMemcpyHostToDevice));
  CK(cudaMemset(S.dM, 0, sizeof(float) * sg::NPARAM));
  CK(cudaMemset(S.dVar, 0, sizeof(float) * sg::NPARAM));
}

void EmDee_surrogate_get_params(void* h, float* params) {
  Surrogate& S = *(Surrogate*)h;
  CK(cudaMemcpy(params, S.dParams, sizeof(float) * sg::NPARAM, cudaMemcpyDeviceToHost));
}

// Rebuilds the Verlet lists (rebuild != 0) and computes descriptors: dGout (optional, device,
// [chains * N][32] FP32)
void EmDee_surrogate_descriptors(void* h, const double* dR, float* dGout, int rebuild, void* stream) {
  using namespace sg;
  Surrogate& S = *(Surrogate*)h;
  cudaStream_t st = (cudaStream_t)stream;
  if (rebuild) sg_build_lists(S, dR, st);
  else k_sg_pack<<<sg_blocks(S.total), 256, 0, st>>>(dR, S.total, S.L, S.dPos);
  k_sg_desc<<<sg_blocks(S.total), 256, 0, st>>>(S.dPos, S.G, S.dSpecies, S.dList, S.dCount, S.cap, S.dG);
  CK(cudaGetLastError());
  if (dGout) CK(cudaMemcpyAsync(dGout, S.dG, sizeof(float) * S.total * DIN, cudaMemcpyDeviceToDevice, st));
}

// Surrogate forces (device FP64 [chains * N][3]) and energies per chain (device FP64 [chains]);
// lists rebuilt when rebuild != 0.  Returns the largest neighbor count seen (list capacity check).
int EmDee_surrogate_forces(void* h, const double* dR, double* dF, double* dE, int rebuild, void* stream) {
  using namespace sg;
  Surrogate& S = *(Surrogate*)h;
  cudaStream_t st = (cudaStream_t)stream;
  EmDee_surrogate_descriptors(h, dR, nullptr, rebuild, stream);
  sg_network(S, S.dParams, st);
  k_sg_force<<<sg_blocks(S.total), 256, 0, st>>>(S.dPos, S.G, S.dSpecies, S.dList, S.dCount, S.cap, S.dEdG, dF);
  CK(cudaGetLastError());
  if (dE) k_sg_chain_sum<<<S.G.chains, 256, 0, st>>>(S.dEatom, S.G.N, dE);
  int ov = 0;
  if (rebuild) {
    int flags[2];
    CK(cudaMemcpyAsync(&flags[0], S.dOverflow, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&flags[1], S.dTcError, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ov = flags[0];
    if (ov > S.cap) fatal("surrogate forces", "a Verlet list outgrew its capacity");
    if (flags[1]) fatal("surrogate forces", "a tensor-core GEMM of the network did not complete");
  }
  return ov;
}

// Per-atom energies, dE/dG (device, FP32) of the last surrogate_forces call
void EmDee_surrogate_atom_outputs(void* h, float* dEatom, float* dEdG, void* stream) {
  Surrogate& S = *(Surrogate*)h;
  cudaStream_t st = (cudaStream_t)stream;
  if (dEatom) CK(cudaMemcpyAsync(dEatom, S.dEatom, sizeof(float) * S.total, cudaMemcpyDeviceToDevice, st));
  if (dEdG) CK(cudaMemcpyAsync(dEdG, S.dEdG, sizeof(float) * S.total * sg::DIN, cudaMemcpyDeviceToDevice, st));
}

// Gradient of the loss  wE sum_c (E_c - Etrue_c)^2 / N^2 / chains + wF sum |F - Ftrue|^2 / (3 N chains)
// for configurations dR (device FP64, chains x N x 3) with reference energies dEtrue (device FP64,
// [chains]) and forces dFtrue (device FP64); lists are rebuilt.  dGrad (device FP32, NPARAM) receives
// the gradient; the loss terms are returned in loss[0] (energy) and loss[1] (force).
void EmDee_surrogate_gradient(void* h, const double* dR, const double* dEtrue, const double* dFtrue, double wE,
                              double wF, float* dGrad, double* loss, void* stream) {
  using namespace sg;
  Surrogate& S = *(Surrogate*)h;
  cudaStream_t st = (cudaStream_t)stream;
  const int C = S.G.chains, N = S.G.N;
  double *dF, *dE;
  CK(cudaMallocAsync(&dF, sizeof(double) * 3 * S.total, st));
  CK(cudaMallocAsync(&dE, sizeof(double) * C, st));
  EmDee_surrogate_forces(h, dR, dF, dE, 1, stream);
  // residuals on the host side of the loss: small arrays per chain, per atom on the device
  std::vector<double> E(C), Et(C);
  CK(cudaMemcpyAsync(E.data(), dE, sizeof(double) * C, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(Et.data(), dEtrue, sizeof(double) * C, cudaMemcpyDeviceToHost, st));
  std::vector<double> F((size_t)3 * S.total), Ft((size_t)3 * S.total);
  CK(cudaMemcpyAsync(F.data(), dF, sizeof(double) * F.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(Ft.data(), dFtrue, sizeof(double) * Ft.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  double lE = 0.0, lF = 0.0;
  std::vector<float> eAtom(S.total), v((size_t)3 * S.total);
  for (int c = 0; c < C; c++) {
    const double d = E[c] - Et[c];
    lE += d * d;
    const float ec = (float)(wE * 2.0 * d / ((double)N * N * C));
    for (int i = 0; i < N; i++) eAtom[(size_t)c * N + i] = ec;
  }
  const double fscale = wF * 2.0 / (3.0 * N * C);
  for (size_t q = 0; q < F.size(); q++) {
    const double d = F[q] - Ft[q];
    lF += d * d;
    v[q] = (float)(fscale * d);
  }
  loss[0] = wE * lE / ((double)N * N * C);
  loss[1] = wF * lF / (3.0 * N * C);
  CK(cudaMemcpyAsync(S.dEres, eAtom.data(), sizeof(float) * S.total, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(S.dV, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice, st));
  k_sg_udesc<<<sg_blocks(S.total), 256, 0, st>>>(S.dPos, S.G, S.dSpecies, S.dList, S.dCount, S.cap, S.dV, S.dU);
  TileArgs T{S.dAtoms, S.dTiles, (int)S.tiles.size()};
  for (int sp = 0; sp < NS; sp++) {
    k_sg_train<<<S.trainBlocks, 128, sizeof(TrainSmem), st>>>(T, sp, S.dParams, S.dG, S.dU, S.dEres, S.dPart);
    k_sg_reduce<<<(PER_SPECIES + 255) / 256, 256, 0, st>>>(S.dPart, S.trainBlocks, PER_SPECIES, 1.f,
                                                           dGrad + sp * PER_SPECIES);
  }
  CK(cudaGetLastError());
  CK(cudaFreeAsync(dF, st));
  CK(cudaFreeAsync(dE, st));
  CK(cudaStreamSynchronize(st));
}

// One Adam step on the device master parameters with gradient dGrad (device)
void EmDee_surrogate_adam(void* h, const float* dGrad, double lr, int step, void* stream) {
  Surrogate& S = *(Surrogate*)h;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  sg::k_sg_adam<<<(sg::NPARAM + 255) / 256, 256, 0, (cudaStream_t)stream>>>(S.dParams, dGrad, S.dM, S.dVar, sg::NPARAM,
                                                                            (float)lr, b1, b2, 1e-8f, c1, c2);
  CK(cudaGetLastError());
}

// n velocity-Verlet steps of the chains (device FP64 R, P [chains * N][3]) on the surrogate
// forces; F holds the forces of the current R on entry and on return.  The lists are rebuilt at
// the start.  Returns the surrogate energies of the final positions in dE (device, [chains]).
void EmDee_surrogate_trajectory(void* h, double* dR, double* dP, double* dF, double* dE, int n, double dt,
                                void* stream) {
  Surrogate& S = *(Surrogate*)h;
  cudaStream_t st = (cudaStream_t)stream;
  const int n3 = 3 * S.total;
  for (int k = 0; k < n; k++) {
    sg::k_sg_kick_drift<<<sg_blocks(n3), 256, 0, st>>>(dR, dP, dF, n3, 0.5 * dt, dt);
    EmDee_surrogate_forces(h, dR, dF, k == n - 1 ? dE : nullptr, 0, stream);
    sg::k_sg_kick<<<sg_blocks(n3), 256, 0, st>>>(dP, dF, n3, 0.5 * dt);
  }
  CK(cudaGetLastError());
}

void EmDee_surrogate_destroy(void* h) {
  Surrogate* S = (Surrogate*)h;
  if (!S) return;
  void* ptrs[] = {S->dSpecies, S->dAtoms, S->dTiles, S->dTiles128, S->dTcError, S->dPos, S->dCellOf, S->dCounts, S->dStarts, S->dCursor,
                  S->dSorted, S->dList, S->dCount, S->dOverflow, S->dG, S->dU, S->dEdG, S->dEatom, S->dEres,
                  S->dV, S->dParams, S->dGrad, S->dM, S->dVar, S->dPart, S->dR0};
  for (void* p : ptrs) cudaFree(p);
  delete S;
}

}  // extern "C"

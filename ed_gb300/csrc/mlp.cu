// mlp.cu -- the learned start vector: a small translation-invariant network
// that maps the gaps between consecutive down spins of a chain
// representative to its k = 0 ground-state amplitude.  No counterpart in the
// reference (whose start vector is random, eigen_solver.f90:92-96).
//
// Network: x (16 inputs) -> 128 -> 128 -> 128 -> 1, tanh hidden activations.
// Parameters are kept in FP32 (master, Adam moments) and used rounded to
// BF16; inputs, hidden activations and back-propagated signals are BF16;
// every product is accumulated in FP32.  Inputs for rotation s of a representative
// with sorted sites n_0 < ... < n_{N-1} (N = NOD <= 4) on a ring of L sites:
//   gaps g_j = n_{j+1} - n_j, g_{N-1} = n_0 + L - n_{N-1};  h_j = g_{(s+j) mod N}
//   x = [h_j / L (j < N), cos(q0 h_j) (j < N), sin(q0 h_j) (j < N), Delta, J2, 0...]
// The network output for a representative is the mean over its N rotations,
// which makes it independent of which down spin is called the first one.
// Its meaning is the amplitude per Ising configuration scaled to O(1):
//   f(r) ~ psi(config r) * sqrt(C(L, N)),  start vector v_r = f(r) * L / list_r(r)
// (for k = 0 the basis state of representative r is sum_t T^t|r> / list_r(r)).
//
// Kernels (hand-written; every matrix product on the tensor cores as
// mma.sync m16n8k16 BF16 x BF16 -> FP32):
//   k_mlp_forward  one tile = 64 rows (16 representatives x 4 rotations); BF16
//                  weights staged transposed in shared memory, activations
//                  row-major BF16 tiles; each warp computes a 16 x 64 block of
//                  a layer's output, bias + tanh in the epilogue.
//   k_mlp_train    the same forward plus the backward pass for a batch of
//                  representatives: weight gradients IN^T DZ and data gradients
//                  DZ W^T on the tensor cores (operands transposed on the fly
//                  by ldmatrix.trans), the back-propagated signals rounded to
//                  BF16 like the activations; gradients accumulated into a
//                  per-block partial (each block owns its slice: no atomics),
//                  loss in FP64.
//   k_mlp_reduce   fixed-order sum of the per-block partials (deterministic).
//   k_mlp_adam     Adam step on the FP32 master copy, refresh of the BF16 copy.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "krylov.h"
#include "qs3g_device.cuh"
#include "qs3g_internal.cuh"
#include "mlp.h"

namespace qs3g {
namespace {

constexpr int kIn = kMlpIn, kHid = kMlpHid;
constexpr int kTile = 64;          // rows per tile (16 representatives x 4 rotations)
constexpr int kThreads = 256;      // 8 warps
constexpr int kXP = kIn + 8;       // BF16 pitch of the input tile and of W1^T (24 elements, 48 bytes)
constexpr int kHP = kHid + 8;      // BF16 pitch of the activation tiles and of W2^T, W3^T (136, 272 bytes)

constexpr int kOffW1 = kMlpOffW1, kOffB1 = kMlpOffB1, kOffW2 = kMlpOffW2, kOffB2 = kMlpOffB2, kOffW3 = kMlpOffW3,
              kOffB3 = kMlpOffB3, kOffW4 = kMlpOffW4, kOffB4 = kMlpOffB4, kNP = kMlpNParams;

// Shared-memory layout (bytes).  Every region and every row starts on a
// 16-byte boundary (ldmatrix rows); the pitches put the 8 rows a fragment
// load touches on 8 different bank quads, so no access conflicts.
constexpr size_t kSmW1 = 0;                                        // W1^T [128][24]  (BF16)
constexpr size_t kSmW2 = kSmW1 + (size_t)kHid * kXP * 2;           // W2^T [128][136]
constexpr size_t kSmW3 = kSmW2 + (size_t)kHid * kHP * 2;           // W3^T [128][136]
constexpr size_t kSmVec = kSmW3 + (size_t)kHid * kHP * 2;          // b1 b2 b3 w4 b4 (FP32)
constexpr size_t kSmX = kSmVec + (size_t)(4 * kHid + 4) * 4;       // X  [64][24]    (BF16)
constexpr size_t kSmH1 = kSmX + (size_t)kTile * kXP * 2;           // H1 [64][136]   (BF16)
constexpr size_t kSmH2 = kSmH1 + (size_t)kTile * kHP * 2;          // H2
constexpr size_t kSmH3 = kSmH2 + (size_t)kTile * kHP * 2;          // H3 (training; inference: out[64])
constexpr size_t kSmG = kSmH3 + (size_t)kTile * kHP * 2;           // dz [64][136]   (BF16)
constexpr size_t kSmRow = kSmG + (size_t)kTile * kHP * 2;          // out[64], dout[64] (FP32)
constexpr size_t kSmTrain = kSmRow + 2 * kTile * 4;
constexpr size_t kSmInfer = kSmH3 + kTile * 4;
static_assert(kSmTrain <= 232448, "training tile exceeds shared memory");
static_assert(kSmX % 16 == 0 && kSmH1 % 16 == 0 && kSmW2 % 16 == 0 && kSmG % 16 == 0, "16-byte regions");

using bf16 = __nv_bfloat16;

struct MlpArgs {
  const uint64_t* conf;       // packed representative per rep
  const int* sample;          // sample id per rep (null: all sample 0)
  const MlpSample* samples;
  const float2* trig;         // (cos, sin)(q0 h) per sample, BF16-rounded
  int NOD, SP;                // spins, rotations per rep padded to a power of two
  int64_t nreps;              // reps addressed by this launch
  const int64_t* index;       // training: rep index per batch entry (null: identity)
  const float* target;        // training: target per rep
  const bf16* params;
  float* out_f;               // inference: f per rep
  float* gpart;               // training: per-block gradient partials
  double* lpart;              // training: per-block loss partials
  float inv_batch;
};

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }
__device__ __forceinline__ uint32_t lds32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // lo in the low half (lower address)
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float2 unpack_bf16(uint32_t u) {
  return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u));
}

// D += A B on the tensor cores: A 16x16 (row), B 16x8 (col), BF16 in, FP32 accumulate.
// Fragments (g = lane / 4, t = lane % 4): a = {A[g][2t..], A[g+8][2t..], A[g][2t+8..],
// A[g+8][2t+8..]}, b = {B[2t..][g], B[2t+8..][g]}, d = {D[g][2t], D[g][2t+1], D[g+8][2t], D[g+8][2t+1]}.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Four transposed 8x8 BF16 tiles: lane l gives the address of row (l % 8) of tile l / 8.
__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], const bf16* p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}

// Stage the BF16 weights transposed (W^T[c][i]) and the FP32 vectors in shared memory.
__device__ void load_params(const bf16* __restrict__ p, unsigned char* sm) {
  bf16* w1 = reinterpret_cast<bf16*>(sm + kSmW1);
  bf16* w2 = reinterpret_cast<bf16*>(sm + kSmW2);
  bf16* w3 = reinterpret_cast<bf16*>(sm + kSmW3);
  float* vec = reinterpret_cast<float*>(sm + kSmVec);
  for (int e = threadIdx.x; e < kIn * kHid; e += blockDim.x) w1[(e % kHid) * kXP + e / kHid] = p[kOffW1 + e];
  for (int e = threadIdx.x; e < kHid * kHid; e += blockDim.x) {
    w2[(e % kHid) * kHP + e / kHid] = p[kOffW2 + e];
    w3[(e % kHid) * kHP + e / kHid] = p[kOffW3 + e];
  }
  for (int e = threadIdx.x; e < kHid; e += blockDim.x) {
    vec[e] = __bfloat162float(p[kOffB1 + e]);
    vec[kHid + e] = __bfloat162float(p[kOffB2 + e]);
    vec[2 * kHid + e] = __bfloat162float(p[kOffB3 + e]);
    vec[3 * kHid + e] = __bfloat162float(p[kOffW4 + e]);
  }
  if (threadIdx.x == 0) vec[4 * kHid] = __bfloat162float(p[kOffB4]);
}

// Inputs of the tile's 64 rows into X[row][f] (BF16); rows past nreps get zeros.
// Row r holds rotation r % SP of representative rep0 + r / SP.
__device__ void tile_features(const MlpArgs& a, int64_t rep0, bf16* X) {
  const int r = threadIdx.x;
  if (r >= kTile) return;
  const int q = r / a.SP, s = r % a.SP;
  const int64_t b = rep0 + q;
  float x[kIn];
#pragma unroll
  for (int f = 0; f < kIn; ++f) x[f] = 0.f;
  if (b < a.nreps && s < a.NOD) {
    const int64_t rep = a.index ? a.index[b] : b;
    const MlpSample sm = a.samples[a.sample ? a.sample[rep] : 0];
    const uint64_t w = a.conf[rep];
    const uint64_t mask = (1ull << sm.bits) - 1ull;
    int n[4];
    for (int j = 0; j < a.NOD; ++j) n[j] = (int)((w >> (sm.bits * j)) & mask);
    int g[4];
    for (int j = 0; j + 1 < a.NOD; ++j) g[j] = n[j + 1] - n[j];
    g[a.NOD - 1] = n[0] + sm.L - n[a.NOD - 1];
    const float invL = 1.0f / (float)sm.L;
    for (int j = 0; j < a.NOD; ++j) {
      const int h = g[(s + j) % a.NOD];
      const float2 cs = a.trig[sm.trig_off + h];
      x[j] = bf16r((float)h * invL);
      x[a.NOD + j] = cs.x;
      x[2 * a.NOD + j] = cs.y;
    }
    x[3 * a.NOD] = bf16r(sm.delta);
    x[3 * a.NOD + 1] = bf16r(sm.j2);
  }
#pragma unroll
  for (int f = 0; f < kIn; f += 2)
    *reinterpret_cast<uint32_t*>(X + r * kXP + f) = pack_bf16(x[f], x[f + 1]);
}

// OUT[r][c] = bf16(tanh(b[c] + sum_k IN[r][k] W[k][c])) for the 64 x 128 tile on
// the tensor cores.  Warp w: rows 16 (w % 4) .. +15, columns 64 (w / 4) .. +63
// (8 n-tiles); K = 16 (layer 1) or 128.  IN has pitch KP, W^T[c][k] too.
template <int K, int KP>
__device__ __forceinline__ void layer_fwd(const bf16* __restrict__ in, const bf16* __restrict__ Wt,
                                          const float* __restrict__ bias, bf16* __restrict__ out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int rb = 16 * (warp & 3), cb = 64 * (warp >> 2);
  float acc[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[4];
    a[0] = lds32(in + (rb + g) * KP + k0 + 2 * t);
    a[1] = lds32(in + (rb + g + 8) * KP + k0 + 2 * t);
    a[2] = lds32(in + (rb + g) * KP + k0 + 2 * t + 8);
    a[3] = lds32(in + (rb + g + 8) * KP + k0 + 2 * t + 8);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const bf16* wr = Wt + (cb + 8 * j + g) * KP + k0 + 2 * t;
      mma_bf16(acc[j], a, lds32(wr), lds32(wr + 8));
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = cb + 8 * j + 2 * t;
    const float b0 = bias[c], b1 = bias[c + 1];
    *reinterpret_cast<uint32_t*>(out + (rb + g) * kHP + c) = pack_bf16(tanhf(acc[j][0] + b0), tanhf(acc[j][1] + b1));
    *reinterpret_cast<uint32_t*>(out + (rb + g + 8) * kHP + c) =
        pack_bf16(tanhf(acc[j][2] + b0), tanhf(acc[j][3] + b1));
  }
}

// out[r] = b4 + sum_c w4[c] H3[r][c] (FP32): 4 threads per row, shuffle reduction.
__device__ __forceinline__ void layer_out(const bf16* __restrict__ h3, const float* __restrict__ w4, float b4,
                                          float* __restrict__ out) {
  const int r = threadIdx.x >> 2, part = threadIdx.x & 3;
  float s = 0.f;
#pragma unroll 4
  for (int c = 2 * part; c < kHid; c += 8) {
    const float2 h = unpack_bf16(lds32(h3 + r * kHP + c));
    s = fmaf(w4[c], h.x, fmaf(w4[c + 1], h.y, s));
  }
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  if (part == 0) out[r] = s + b4;
}

__device__ __forceinline__ void forward_tile(unsigned char* sm, bf16* h3, float* out) {
  const bf16* w1 = reinterpret_cast<const bf16*>(sm + kSmW1);
  const bf16* w2 = reinterpret_cast<const bf16*>(sm + kSmW2);
  const bf16* w3 = reinterpret_cast<const bf16*>(sm + kSmW3);
  const float* vec = reinterpret_cast<const float*>(sm + kSmVec);
  const bf16* X = reinterpret_cast<const bf16*>(sm + kSmX);
  bf16* h1 = reinterpret_cast<bf16*>(sm + kSmH1);
  bf16* h2 = reinterpret_cast<bf16*>(sm + kSmH2);
  layer_fwd<kIn, kXP>(X, w1, vec, h1);
  __syncthreads();
  layer_fwd<kHid, kHP>(h1, w2, vec + kHid, h2);
  __syncthreads();
  layer_fwd<kHid, kHP>(h2, w3, vec + 2 * kHid, h3);
  __syncthreads();
  layer_out(h3, vec + 3 * kHid, vec[4 * kHid], out);
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads) k_mlp_forward(MlpArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  load_params(a.params, sm);
  bf16* X = reinterpret_cast<bf16*>(sm + kSmX);
  bf16* h3 = reinterpret_cast<bf16*>(sm + kSmH1);  // inference reuses H1 for H3
  float* out = reinterpret_cast<float*>(sm + kSmH3);
  const int per = kTile / a.SP;
  const int64_t ntiles = (a.nreps + per - 1) / per;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    __syncthreads();
    tile_features(a, t * per, X);
    __syncthreads();
    forward_tile(sm, h3, out);
    if (threadIdx.x < per) {
      const int64_t b = t * per + threadIdx.x;
      if (b < a.nreps) {
        float f = 0.f;
        for (int s = 0; s < a.NOD; ++s) f += out[threadIdx.x * a.SP + s];
        a.out_f[a.index ? a.index[b] : b] = f / (float)a.NOD;
      }
    }
  }
}

// dW[i][c] (+)= sum_r IN[r][i] DZ[r][c] on the tensor cores (M = KI inputs,
// N = 128, K = 64 rows); both operands come transposed from their row-major
// tiles through ldmatrix.trans.  KI = 128: warp w owns inputs 16 w .. +15 and
// all 16 n-tiles; KI = 16: one m-tile, warp w owns columns 16 w .. +15.
// db[c] (+)= sum_r DZ[r][c].  gW, gb: the block's FP32 partial (no other block
// touches it).
template <int KI, int KP>
__device__ __forceinline__ void grad_w(const bf16* __restrict__ in, const bf16* __restrict__ dz,
                                       float* __restrict__ gW, float* __restrict__ gb) {
  constexpr int NT = (KI == kHid) ? 16 : 2;  // n-tiles per warp
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int i0 = (KI == kHid) ? 16 * warp : 0;
  const int c0w = (KI == kHid) ? 0 : 16 * warp;
  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  const int lr = (lane & 7), lsel = (lane >> 3) & 1, lhi = lane >> 4;
#pragma unroll
  for (int r0 = 0; r0 < kTile; r0 += 16) {
    uint32_t a[4];
    ldsm4t(a, in + (r0 + lr + 8 * lhi) * KP + i0 + 8 * lsel);  // A[i][r] = IN[r][i]
#pragma unroll
    for (int jj = 0; jj < NT / 2; ++jj) {
      uint32_t b[4];
      ldsm4t(b, dz + (r0 + lr + 8 * lsel) * kHP + c0w + 16 * jj + 8 * lhi);  // B[r][c] = DZ[r][c]
      mma_bf16(acc[2 * jj], a, b[0], b[1]);
      mma_bf16(acc[2 * jj + 1], a, b[2], b[3]);
    }
  }
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const int c = c0w + 8 * j + 2 * t;
    gW[(i0 + g) * kHid + c] += acc[j][0];
    gW[(i0 + g) * kHid + c + 1] += acc[j][1];
    gW[(i0 + g + 8) * kHid + c] += acc[j][2];
    gW[(i0 + g + 8) * kHid + c + 1] += acc[j][3];
  }
  if (threadIdx.x < kHid) {
    float s = 0.f;
    for (int r = 0; r < kTile; ++r) s += __bfloat162float(dz[r * kHP + threadIdx.x]);
    gb[threadIdx.x] += s;
  }
}

// DZ_prev[r][i] = bf16((sum_c DZ[r][c] W[i][c]) * (1 - H[r][i]^2)), written over H
// (each element is read and written by the thread that computes it).  M = 64,
// N = 128 inputs, K = 128; warp w: rows 16 (w % 4) .., inputs 64 (w / 4) ..;
// B[c][i] = W[i][c] = W^T[c][i] through ldmatrix.trans.
__device__ __forceinline__ void back_data(const bf16* __restrict__ dz, const bf16* __restrict__ Wt, bf16* h) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int rb = 16 * (warp & 3), ib = 64 * (warp >> 2);
  const int lr = (lane & 7), lsel = (lane >> 3) & 1, lhi = lane >> 4;
  float acc[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll 2
  for (int c0 = 0; c0 < kHid; c0 += 16) {
    uint32_t a[4];
    a[0] = lds32(dz + (rb + g) * kHP + c0 + 2 * t);
    a[1] = lds32(dz + (rb + g + 8) * kHP + c0 + 2 * t);
    a[2] = lds32(dz + (rb + g) * kHP + c0 + 2 * t + 8);
    a[3] = lds32(dz + (rb + g + 8) * kHP + c0 + 2 * t + 8);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      uint32_t b[4];
      ldsm4t(b, Wt + (c0 + lr + 8 * lsel) * kHP + ib + 16 * jj + 8 * lhi);
      mma_bf16(acc[2 * jj], a, b[0], b[1]);
      mma_bf16(acc[2 * jj + 1], a, b[2], b[3]);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int i = ib + 8 * j + 2 * t;
    uint32_t* p0 = reinterpret_cast<uint32_t*>(h + (rb + g) * kHP + i);
    uint32_t* p1 = reinterpret_cast<uint32_t*>(h + (rb + g + 8) * kHP + i);
    const float2 h0 = unpack_bf16(*p0), h1 = unpack_bf16(*p1);
    *p0 = pack_bf16(acc[j][0] * (1.f - h0.x * h0.x), acc[j][1] * (1.f - h0.y * h0.y));
    *p1 = pack_bf16(acc[j][2] * (1.f - h1.x * h1.x), acc[j][3] * (1.f - h1.y * h1.y));
  }
}

__global__ void __launch_bounds__(kThreads) k_mlp_train(MlpArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  load_params(a.params, sm);
  const bf16* w2 = reinterpret_cast<const bf16*>(sm + kSmW2);
  const bf16* w3 = reinterpret_cast<const bf16*>(sm + kSmW3);
  const float* vec = reinterpret_cast<const float*>(sm + kSmVec);
  bf16* X = reinterpret_cast<bf16*>(sm + kSmX);
  bf16* h1 = reinterpret_cast<bf16*>(sm + kSmH1);
  bf16* h2 = reinterpret_cast<bf16*>(sm + kSmH2);
  bf16* h3 = reinterpret_cast<bf16*>(sm + kSmH3);
  bf16* G = reinterpret_cast<bf16*>(sm + kSmG);
  float* out = reinterpret_cast<float*>(sm + kSmRow);
  float* dout = out + kTile;
  float* gp = a.gpart + (size_t)blockIdx.x * kNP;
  const int per = kTile / a.SP;
  const int64_t ntiles = (a.nreps + per - 1) / per;
  double loss = 0.0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    __syncthreads();
    tile_features(a, t * per, X);
    __syncthreads();
    forward_tile(sm, h3, out);
    // per representative: f = mean over rotations; loss and dL/dout
    if (threadIdx.x < kTile) {
      const int r = threadIdx.x, q = r / a.SP, s = r % a.SP;
      const int64_t b = t * per + q;
      float d = 0.f;
      if (b < a.nreps && s < a.NOD) {
        float f = 0.f;
        for (int u = 0; u < a.NOD; ++u) f += out[q * a.SP + u];
        f /= (float)a.NOD;
        const int64_t rep = a.index ? a.index[b] : b;
        const float e = f - a.target[rep];
        d = 2.f * e * a.inv_batch / (float)a.NOD;
        if (s == 0) loss += (double)e * (double)e;
      }
      dout[r] = d;
    }
    __syncthreads();
    // output layer: dw4, db4; dz3 = bf16(dout * w4 * (1 - h3^2)) into G
    if (threadIdx.x < kHid) {
      const int c = threadIdx.x;
      const float w4 = vec[3 * kHid + c];
      float s = 0.f;
      for (int r = 0; r < kTile; ++r) {
        const float h = __bfloat162float(h3[r * kHP + c]);
        s = fmaf(dout[r], h, s);
        G[r * kHP + c] = __float2bfloat16_rn(dout[r] * w4 * (1.f - h * h));
      }
      gp[kOffW4 + c] += s;
    }
    if (threadIdx.x == kHid) {
      float s = 0.f;
      for (int r = 0; r < kTile; ++r) s += dout[r];
      gp[kOffB4] += s;
    }
    __syncthreads();
    grad_w<kHid, kHP>(h2, G, gp + kOffW3, gp + kOffB3);
    __syncthreads();
    back_data(G, w3, h2);   // h2 <- dz2
    __syncthreads();
    grad_w<kHid, kHP>(h1, h2, gp + kOffW2, gp + kOffB2);
    __syncthreads();
    back_data(h2, w2, h1);  // h1 <- dz1
    __syncthreads();
    grad_w<kIn, kXP>(X, h1, gp + kOffW1, gp + kOffB1);
  }
  __shared__ double lsh[kThreads];
  lsh[threadIdx.x] = loss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kTile; ++k) s += lsh[k];
    a.lpart[blockIdx.x] = s;
  }
}

__global__ void k_mlp_reduce(const float* __restrict__ gpart, int nblk, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNP) return;
  float s = 0.f;
  for (int b = 0; b < nblk; ++b) s += gpart[(size_t)b * kNP + p];
  grad[p] = s;
}

__global__ void k_mlp_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ g, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                           float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNP) return;
  const float gi = g[p];
  const float mi = b1 * m[p] + (1.f - b1) * gi;
  const float vi = b2 * v[p] + (1.f - b2) * gi * gi;
  m[p] = mi;
  v[p] = vi;
  const float wi = w[p] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[p] = wi;
  wb[p] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, int n) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) wb[p] = __float2bfloat16_rn(w[p]);
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Batch of representatives drawn with replacement: index[b] = hash(seed, b) mod n.
__global__ void k_batch_index(int64_t* idx, int64_t B, int64_t n, uint64_t seed) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) idx[b] = (int64_t)(mix64(seed + (uint64_t)(b + 1) * 0x9E3779B97F4A7C15ull) % (uint64_t)n);
}

// Targets of one sample: t = v * list_r / L * sqrt(C(L, N)) (real part; the
// k = 0 ground state of the real chain Hamiltonian is real up to a global
// phase, removed on the host).
__global__ void k_targets(const double2* __restrict__ v, const double* __restrict__ r, int64_t D, double scale,
                          double2 phase, float* __restrict__ t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D) return;
  const double2 z = v[i];
  t[i] = (float)((z.x * phase.x - z.y * phase.y) * r[i] * scale);
}

// Start vector from f: v_r = f(r) * L / list_r(r) (complex, imaginary part 0).
__global__ void k_start_from_f(const float* __restrict__ f, const double* __restrict__ r, int64_t D, double L,
                               double2* __restrict__ v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D) return;
  v[i] = make_double2((double)f[i] * L / r[i], 0.0);
}

__global__ void k_set_int(int* p, int64_t n, int v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// sum over the reps of sample s of f * t (fixed grid, per-block partials)
__global__ void k_sample_dots(const float* __restrict__ f, const float* __restrict__ t, const int* __restrict__ sid,
                              int64_t n, int nsamp, double* part) {
  extern __shared__ double acc[];
  for (int s = threadIdx.x; s < nsamp; s += blockDim.x) acc[s] = 0.0;
  __syncthreads();
  // one thread per block walks a contiguous chunk: reps of a sample are contiguous
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = (int64_t)blockIdx.x * per, b1 = min(n, b0 + per);
  if (threadIdx.x == 0) {
    for (int64_t i = b0; i < b1; ++i) acc[sid[i]] += (double)f[i] * (double)t[i];
  }
  __syncthreads();
  for (int s = threadIdx.x; s < nsamp; s += blockDim.x) part[(size_t)blockIdx.x * nsamp + s] = acc[s];
}

__global__ void k_flip_targets(float* t, const int* sid, int64_t n, const int* flip) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flip[sid[i]]) t[i] = -t[i];
}

uint64_t host_mix(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

// ------------------------------------------------------------------ host side
Mlp::Mlp(uint64_t seed) {
  std::vector<float> w(kNP, 0.f);
  auto uni = [&](uint64_t k) { return (double)(host_mix(seed, k) >> 11) * 0x1.0p-53 * 2.0 - 1.0; };
  uint64_t k = 0;
  // uniform(-a, a) with a = sqrt(6 / (fan_in + fan_out)) for the matrices, zero biases
  const double a1 = std::sqrt(6.0 / (kIn + kHid)), a2 = std::sqrt(6.0 / (2 * kHid)), a4 = std::sqrt(6.0 / (kHid + 1));
  for (int e = 0; e < kIn * kHid; ++e) w[kOffW1 + e] = (float)(a1 * uni(k++));
  for (int e = 0; e < kHid * kHid; ++e) w[kOffW2 + e] = (float)(a2 * uni(k++));
  for (int e = 0; e < kHid * kHid; ++e) w[kOffW3 + e] = (float)(a2 * uni(k++));
  for (int e = 0; e < kHid; ++e) w[kOffW4 + e] = (float)(a4 * uni(k++));
  d_w.alloc(kNP); d_m.alloc(kNP); d_v.alloc(kNP); d_g.alloc(kNP); d_wb.alloc(kNP);
  QS3G_CHECK_CUDA(cudaMemcpy(d_w.get(), w.data(), kNP * 4, cudaMemcpyHostToDevice));
  QS3G_CHECK_CUDA(cudaMemset(d_m.get(), 0, kNP * 4));
  QS3G_CHECK_CUDA(cudaMemset(d_v.get(), 0, kNP * 4));
  k_to_bf16<<<(kNP + 255) / 256, 256>>>(d_w.get(), d_wb.get(), kNP);
  check_launch("k_to_bf16");
  QS3G_CHECK_CUDA(cudaDeviceSynchronize());
}

void Mlp::set_params(const double* p, cudaStream_t st) {
  std::vector<float> w(kNP);
  for (int e = 0; e < kNP; ++e) w[e] = (float)p[e];
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_w.get(), w.data(), kNP * 4, cudaMemcpyHostToDevice, st));
  k_to_bf16<<<(kNP + 255) / 256, 256, 0, st>>>(d_w.get(), d_wb.get(), kNP);
  check_launch("k_to_bf16");
  QS3G_CHECK_CUDA(cudaMemsetAsync(d_m.get(), 0, kNP * 4, st));
  QS3G_CHECK_CUDA(cudaMemsetAsync(d_v.get(), 0, kNP * 4, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  adam_t = 0;
}

void Mlp::get_params(double* p, cudaStream_t st) const {
  std::vector<float> w(kNP);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(w.data(), d_w.get(), kNP * 4, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  for (int e = 0; e < kNP; ++e) p[e] = (double)w[e];
}

// (cos, sin)(q0 h) for h = 0..L, rounded to BF16 as the network reads them
static void trig_table(int L, double q0, std::vector<float2>& out) {
  out.resize(L + 1);
  for (int h = 0; h <= L; ++h) {
    const double c = std::cos(q0 * (double)h), s = std::sin(q0 * (double)h);
    out[h] = make_float2(__bfloat162float(__float2bfloat16_rn((float)c)),
                         __bfloat162float(__float2bfloat16_rn((float)s)));
  }
}

static void check_chain_sector(const Model& m, const Sector& s) {
  QS3G_REQUIRE(m.chain && s.anchored, QS3G_ENOTSUP, "the learned start is defined for chain sectors");
  QS3G_REQUIRE(s.NOD >= 1 && s.NOD <= 4, QS3G_ENOTSUP, "the learned start supports NOD <= 4");
  QS3G_REQUIRE(m.NOS < (1 << 15), QS3G_ERANGE, "L too large for the network inputs");
}

void Mlp::add_sample(const Model& m, const Sector& s, const double2* h_psi, const double cond[3], cudaStream_t st) {
  check_chain_sector(m, s);
  QS3G_REQUIRE(s.kzero, QS3G_ENOTSUP, "training samples must be k = 0 ground states");
  QS3G_REQUIRE(nod == 0 || nod == s.NOD, QS3G_EINVAL, "all samples must have the same NOD");
  nod = s.NOD;
  const int64_t D = s.D;
  // global phase: make the largest-modulus amplitude real
  int64_t imax = 0;
  double amax = -1.0;
  for (int64_t i = 0; i < D; ++i) {
    const double a = h_psi[i].x * h_psi[i].x + h_psi[i].y * h_psi[i].y;
    if (a > amax) { amax = a; imax = i; }
  }
  const double ab = std::sqrt(amax);
  QS3G_REQUIRE(ab > 0.0, QS3G_EINVAL, "zero vector");
  double2 ph = make_double2(h_psi[imax].x / ab, -h_psi[imax].y / ab);
  // Global sign: sum_r Re(v_r ph) cos(q0 (g_0 + g_2 + ...)) >= 0, the Marshall
  // sign (-1)^(g_0 + g_2) of the antiferromagnet when q0 = pi and NOD = 4.
  const int L = m.NOS;
  {
    std::vector<uint64_t> hc(D);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(hc.data(), s.d_conf.get(), D * 8, cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    const uint64_t mask = (1ull << m.bits) - 1ull;
    double dot = 0.0;
    for (int64_t i = 0; i < D; ++i) {
      int n[4];
      for (int j = 0; j < s.NOD; ++j) n[j] = (int)((hc[i] >> (m.bits * j)) & mask);
      int ge = 0;
      for (int j = 0; j < s.NOD; j += 2) ge += (j + 1 < s.NOD) ? n[j + 1] - n[j] : n[0] + L - n[j];
      dot += (h_psi[i].x * ph.x - h_psi[i].y * ph.y) * std::cos(cond[2] * (double)ge);
    }
    if (dot < 0.0) ph = make_double2(-ph.x, -ph.y);
  }
  const double scale = std::sqrt((double)binom_u64(L, s.NOD)) / (double)L;
  // grow the device arrays
  const int64_t n0 = nreps, n1 = nreps + D;
  auto grow = [&](auto& buf, size_t elem_count) {
    using T = std::remove_pointer_t<decltype(buf.get())>;
    DevBuf<T> nb(elem_count);
    if (buf.get() && n0 > 0)
      QS3G_CHECK_CUDA(cudaMemcpyAsync(nb.get(), buf.get(), n0 * sizeof(T), cudaMemcpyDeviceToDevice, st));
    buf = std::move(nb);
  };
  grow(d_conf, n1);
  grow(d_target, n1);
  grow(d_sid, n1);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_conf.get() + n0, s.d_conf.get(), D * 8, cudaMemcpyDeviceToDevice, st));
  DevBuf<double2> dv(D);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(dv.get(), h_psi, D * sizeof(double2), cudaMemcpyHostToDevice, st));
  k_targets<<<(unsigned)((D + 255) / 256), 256, 0, st>>>(dv.get(), s.d_list_r.get(), D, scale, ph,
                                                         d_target.get() + n0);
  check_launch("k_targets");
  const int sid = (int)samples.size();
  k_set_int<<<(unsigned)((D + 255) / 256), 256, 0, st>>>(d_sid.get() + n0, D, sid);
  check_launch("k_set_int");
  MlpSample smp{};
  smp.L = L;
  smp.bits = m.bits;
  smp.delta = (float)cond[0];
  smp.j2 = (float)cond[1];
  std::vector<float2> tr;
  trig_table(L, cond[2], tr);
  smp.trig_off = (int64_t)trig.size();
  trig.insert(trig.end(), tr.begin(), tr.end());
  samples.push_back(smp);
  nreps = n1;
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  uploaded = false;
}

void Mlp::clear_samples() {
  samples.clear();
  trig.clear();
  nreps = 0;
  nod = 0;
  d_conf.release(); d_target.release(); d_sid.release();
  uploaded = false;
}

void Mlp::upload(cudaStream_t st) {
  if (uploaded) return;
  d_samples.alloc(std::max<size_t>(1, samples.size()));
  d_trig.alloc(std::max<size_t>(1, trig.size()));
  if (!samples.empty())
    QS3G_CHECK_CUDA(cudaMemcpyAsync(d_samples.get(), samples.data(), samples.size() * sizeof(MlpSample),
                                    cudaMemcpyHostToDevice, st));
  if (!trig.empty())
    QS3G_CHECK_CUDA(cudaMemcpyAsync(d_trig.get(), trig.data(), trig.size() * sizeof(float2), cudaMemcpyHostToDevice,
                                    st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  uploaded = true;
}

static int rotations_padded(int nod) { return nod <= 1 ? 1 : (nod <= 2 ? 2 : 4); }

static int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    QS3G_CHECK_CUDA(cudaGetDevice(&dev));
    QS3G_CHECK_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  }
  return n;
}

// One pass of k_mlp_train over `B` entries (index may be null: all reps in
// order), then the fixed-order reduction.  Returns the mean squared error.
double Mlp::loss_grad(const int64_t* d_index, int64_t B, cudaStream_t st) {
  QS3G_REQUIRE(nreps > 0, QS3G_ESTATE, "no training samples");
  upload(st);
  static bool attr = false;
  if (!attr) {
    QS3G_CHECK_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmTrain));
    attr = true;
  }
  const int SP = rotations_padded(nod);
  const int per = kTile / SP;
  const int64_t ntiles = (B + per - 1) / per;
  const int nblk = (int)std::min<int64_t>(sm_count(), ntiles);
  if (d_gpart.n < (size_t)nblk * kNP) d_gpart.alloc((size_t)nblk * kNP);
  if (d_lpart.n < (size_t)nblk) d_lpart.alloc(nblk);
  QS3G_CHECK_CUDA(cudaMemsetAsync(d_gpart.get(), 0, (size_t)nblk * kNP * 4, st));
  MlpArgs a{};
  a.conf = d_conf.get(); a.sample = d_sid.get(); a.samples = d_samples.get(); a.trig = d_trig.get();
  a.NOD = nod; a.SP = SP; a.nreps = B; a.index = d_index; a.target = d_target.get(); a.params = d_wb.get();
  a.gpart = d_gpart.get(); a.lpart = d_lpart.get(); a.inv_batch = (float)(1.0 / (double)B);
  k_mlp_train<<<nblk, kThreads, kSmTrain, st>>>(a);
  check_launch("k_mlp_train");
  k_mlp_reduce<<<(kNP + 255) / 256, 256, 0, st>>>(d_gpart.get(), nblk, d_g.get());
  check_launch("k_mlp_reduce");
  std::vector<double> lp(nblk);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(lp.data(), d_lpart.get(), nblk * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  double l = 0.0;
  for (double v : lp) l += v;
  return l / (double)B;
}

void Mlp::train(int steps, int64_t B, double lr, uint64_t seed, double* losses, cudaStream_t st) {
  QS3G_REQUIRE(steps >= 0 && B >= 1, QS3G_EINVAL, "steps >= 0 and batch >= 1");
  DevBuf<int64_t> idx(B);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int k = 0; k < steps; ++k) {
    k_batch_index<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(idx.get(), B, nreps,
                                                                host_mix(seed, (uint64_t)(adam_t + k)));
    check_launch("k_batch_index");
    const double l = loss_grad(idx.get(), B, st);
    if (losses) losses[k] = l;
    ++adam_t;
    const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
    k_mlp_adam<<<(kNP + 255) / 256, 256, 0, st>>>(d_w.get(), d_m.get(), d_v.get(), d_g.get(), d_wb.get(),
                                                  (float)lr, b1, b2, eps, c1, c2);
    check_launch("k_mlp_adam");
  }
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

void Mlp::gradient(double* g, cudaStream_t st) const {
  std::vector<float> h(kNP);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(h.data(), d_g.get(), kNP * 4, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  for (int e = 0; e < kNP; ++e) g[e] = (double)h[e];
}

// f for nrep packed configurations of one sample description (device arrays).
void Mlp::forward(const uint64_t* d_c, const int* d_s, const MlpSample* d_smp, const float2* d_tr, int64_t n,
                  float* d_f, cudaStream_t st) const {
  static bool attr = false;
  if (!attr) {
    QS3G_CHECK_CUDA(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmInfer));
    attr = true;
  }
  MlpArgs a{};
  a.conf = d_c; a.sample = d_s; a.samples = d_smp; a.trig = d_tr;
  a.NOD = nod; a.SP = rotations_padded(nod); a.nreps = n; a.params = d_wb.get(); a.out_f = d_f;
  const int per = kTile / a.SP;
  const int64_t ntiles = (n + per - 1) / per;
  const int nblk = (int)std::min<int64_t>((int64_t)sm_count() * 8, ntiles);
  k_mlp_forward<<<nblk, kThreads, kSmInfer, st>>>(a);
  check_launch("k_mlp_forward");
}

// Align every sample's global sign with the current network: flip a
// sample's targets when sum_r f(r) t(r) < 0.
int Mlp::align(cudaStream_t st) {
  QS3G_REQUIRE(nreps > 0, QS3G_ESTATE, "no training samples");
  upload(st);
  DevBuf<float> f(nreps);
  forward(d_conf.get(), d_sid.get(), d_samples.get(), d_trig.get(), nreps, f.get(), st);
  const int ns = (int)samples.size(), nblk = 256;
  DevBuf<double> part((size_t)nblk * ns);
  k_sample_dots<<<nblk, 128, ns * sizeof(double), st>>>(f.get(), d_target.get(), d_sid.get(), nreps, ns, part.get());
  check_launch("k_sample_dots");
  std::vector<double> hp((size_t)nblk * ns);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(hp.data(), part.get(), hp.size() * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  std::vector<int> flip(ns, 0);
  int nflip = 0;
  for (int s = 0; s < ns; ++s) {
    double d = 0.0;
    for (int b = 0; b < nblk; ++b) d += hp[(size_t)b * ns + s];
    flip[s] = d < 0.0 ? 1 : 0;
    nflip += flip[s];
  }
  if (nflip) {
    DevBuf<int> df(ns);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(df.get(), flip.data(), ns * 4, cudaMemcpyHostToDevice, st));
    k_flip_targets<<<(unsigned)((nreps + 255) / 256), 256, 0, st>>>(d_target.get(), d_sid.get(), nreps, df.get());
    check_launch("k_flip_targets");
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return nflip;
}

// Start vector for the sector s (device output, D elements), unnormalised.
void Mlp::predict(const Model& m, const Sector& s, const double cond[3], double2* d_v, cudaStream_t st) {
  check_chain_sector(m, s);
  QS3G_REQUIRE(nod == 0 || nod == s.NOD, QS3G_EINVAL, "network trained for another NOD");
  if (nod == 0) nod = s.NOD;
  MlpSample smp{};
  smp.L = m.NOS; smp.bits = m.bits; smp.delta = (float)cond[0]; smp.j2 = (float)cond[1]; smp.trig_off = 0;
  std::vector<float2> tr;
  trig_table(m.NOS, cond[2], tr);
  DevBuf<MlpSample> dsm(1);
  DevBuf<float2> dtr(tr.size());
  QS3G_CHECK_CUDA(cudaMemcpyAsync(dsm.get(), &smp, sizeof smp, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(dtr.get(), tr.data(), tr.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  DevBuf<float> f(s.D);
  forward(s.d_conf.get(), nullptr, dsm.get(), dtr.get(), s.D, f.get(), st);
  k_start_from_f<<<(unsigned)((s.D + 255) / 256), 256, 0, st>>>(f.get(), s.d_list_r.get(), s.D, (double)m.NOS, d_v);
  check_launch("k_start_from_f");
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

}  // namespace qs3g

// mlp.cu -- the learned start vector: a small translation-invariant network
// that maps the gaps between consecutive down spins of a chain
// representative to its k = 0 ground-state amplitude.  No counterpart in the
// reference (whose start vector is random, eigen_solver.f90:92-96).
//
// Network: x (16 inputs) -> 128 -> 128 -> 128 -> 1, tanh hidden activations.
// Parameters are kept in FP32 (master, Adam moments) and used rounded to
// BF16; inputs are rounded to BF16; every product is accumulated in FP32 and
// hidden activations stay FP32.  Inputs for rotation s of a representative
// with sorted sites n_0 < ... < n_{N-1} (N = NOD <= 4) on a ring of L sites:
//   gaps g_j = n_{j+1} - n_j, g_{N-1} = n_0 + L - n_{N-1};  h_j = g_{(s+j) mod N}
//   x = [h_j / L (j < N), cos(q0 h_j) (j < N), sin(q0 h_j) (j < N), Delta, J2, 0...]
// The network output for a representative is the mean over its N rotations,
// which makes it independent of which down spin is called the first one.
// Its meaning is the amplitude per Ising configuration scaled to O(1):
//   f(r) ~ psi(config r) * sqrt(C(L, N)),  start vector v_r = f(r) * L / list_r(r)
// (for k = 0 the basis state of representative r is sum_t T^t|r> / list_r(r)).
//
// Kernels (hand-written, SIMT, no tensor cores: the network is small and
// this is not the solver's hot path):
//   k_mlp_forward  one tile = 64 rows (16 representatives x 4 rotations); BF16
//                  weights staged in shared memory, activations transposed
//                  [feature][row] in FP32; each thread owns a 4-row x 8-column
//                  register block of every layer's output.
//   k_mlp_train    the same forward plus the backward pass for a batch of
//                  representatives, gradients accumulated into a per-block
//                  partial (each block owns its slice: no atomics), loss in FP64.
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
constexpr int kTile = 64;          // rows per tile
constexpr int kThreads = 256;
constexpr int kWP = 130;           // BF16 weight pitch (65 words: column reads hit 32 banks)
constexpr int kAP = 68;            // FP32 activation pitch [feature][row]

constexpr int kOffW1 = kMlpOffW1, kOffB1 = kMlpOffB1, kOffW2 = kMlpOffW2, kOffB2 = kMlpOffB2, kOffW3 = kMlpOffW3,
              kOffB3 = kMlpOffB3, kOffW4 = kMlpOffW4, kOffB4 = kMlpOffB4, kNP = kMlpNParams;

// shared-memory layout (bytes)
constexpr size_t kSmW1 = 0;
constexpr size_t kSmW2 = kSmW1 + (size_t)kIn * kWP * 2;
constexpr size_t kSmW3 = kSmW2 + (size_t)kHid * kWP * 2;
constexpr size_t kSmVec = kSmW3 + (size_t)kHid * kWP * 2;          // b1 b2 b3 w4 b4 (FP32)
constexpr size_t kSmX = kSmVec + (size_t)(4 * kHid + 4) * 4;
constexpr size_t kSmH1 = kSmX + (size_t)kIn * kAP * 4;
constexpr size_t kSmH2 = kSmH1 + (size_t)kHid * kAP * 4;
constexpr size_t kSmH3 = kSmH2 + (size_t)kHid * kAP * 4;
constexpr size_t kSmG = kSmH3 + (size_t)kHid * kAP * 4;
constexpr size_t kSmRow = kSmG + (size_t)kHid * kAP * 4;             // out[64], dout[64]
constexpr size_t kSmTrain = kSmRow + 2 * kTile * 4;
constexpr size_t kSmInfer = kSmH3;                                   // x, h1, h2 only (+ row)
static_assert(kSmTrain <= 232448, "training tile exceeds shared memory");

struct MlpArgs {
  const uint64_t* conf;       // packed representative per rep
  const int* sample;          // sample id per rep (null: all sample 0)
  const MlpSample* samples;
  const float2* trig;         // (cos, sin)(q0 h) per sample, BF16-rounded
  int NOD, SP;                // spins, rotations per rep padded to a power of two
  int64_t nreps;              // reps addressed by this launch
  const int64_t* index;       // training: rep index per batch entry (null: identity)
  const float* target;        // training: target per rep
  const __nv_bfloat16* params;
  float* out_f;               // inference: f per rep
  float* gpart;               // training: per-block gradient partials
  double* lpart;              // training: per-block loss partials
  float inv_batch;
};

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// Stage the BF16 weights (pitch kWP) and the FP32 vectors in shared memory.
__device__ void load_params(const __nv_bfloat16* __restrict__ p, unsigned char* sm) {
  __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(sm + kSmW1);
  __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(sm + kSmW2);
  __nv_bfloat16* w3 = reinterpret_cast<__nv_bfloat16*>(sm + kSmW3);
  float* vec = reinterpret_cast<float*>(sm + kSmVec);
  for (int e = threadIdx.x; e < kIn * kHid; e += blockDim.x) w1[(e / kHid) * kWP + e % kHid] = p[kOffW1 + e];
  for (int e = threadIdx.x; e < kHid * kHid; e += blockDim.x) {
    w2[(e / kHid) * kWP + e % kHid] = p[kOffW2 + e];
    w3[(e / kHid) * kWP + e % kHid] = p[kOffW3 + e];
  }
  for (int e = threadIdx.x; e < kHid; e += blockDim.x) {
    vec[e] = __bfloat162float(p[kOffB1 + e]);
    vec[kHid + e] = __bfloat162float(p[kOffB2 + e]);
    vec[2 * kHid + e] = __bfloat162float(p[kOffB3 + e]);
    vec[3 * kHid + e] = __bfloat162float(p[kOffW4 + e]);
  }
  if (threadIdx.x == 0) vec[4 * kHid] = __bfloat162float(p[kOffB4]);
}

// Inputs of the tile's 64 rows into xT[f][row]; rows past nrows get zeros.
// Returns (through rep_of) nothing: the row -> rep map is r / SP.
__device__ void tile_features(const MlpArgs& a, int64_t rep0, float* xT) {
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
  for (int f = 0; f < kIn; ++f) xT[f * kAP + r] = x[f];
}

// outT[c][r] = tanh(b[c] + sum_k inT[k][r] W[k][c]) for the 64 x 128 tile.
// Thread t: rows 4*(t/16) .. +3, columns 8*(t%16) .. +7.
template <int K>
__device__ __forceinline__ void layer_fwd(const float* __restrict__ inT, const __nv_bfloat16* __restrict__ W,
                                          const float* __restrict__ bias, float* __restrict__ outT) {
  const int rg = threadIdx.x >> 4, cg = threadIdx.x & 15;
  const int r0 = 4 * rg, c0 = 8 * cg;
  float acc[4][8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b = bias[c0 + j];
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i][j] = b;
  }
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    const float4 a = *reinterpret_cast<const float4*>(inT + k * kAP + r0);
    const __nv_bfloat162* wr = reinterpret_cast<const __nv_bfloat162*>(W + k * kWP + c0);
    float w[8];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float2 f = __bfloat1622float2(wr[u]);
      w[2 * u] = f.x;
      w[2 * u + 1] = f.y;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      acc[0][j] = fmaf(a.x, w[j], acc[0][j]);
      acc[1][j] = fmaf(a.y, w[j], acc[1][j]);
      acc[2][j] = fmaf(a.z, w[j], acc[2][j]);
      acc[3][j] = fmaf(a.w, w[j], acc[3][j]);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float4 o;
    o.x = tanhf(acc[0][j]);
    o.y = tanhf(acc[1][j]);
    o.z = tanhf(acc[2][j]);
    o.w = tanhf(acc[3][j]);
    *reinterpret_cast<float4*>(outT + (c0 + j) * kAP + r0) = o;
  }
}

// out[r] = b4 + sum_c w4[c] h3[c][r]: 4 threads per row, shuffle reduction.
__device__ __forceinline__ void layer_out(const float* __restrict__ h3T, const float* __restrict__ w4, float b4,
                                          float* __restrict__ out) {
  const int r = threadIdx.x >> 2, part = threadIdx.x & 3;
  float s = 0.f;
#pragma unroll 8
  for (int c = part; c < kHid; c += 4) s = fmaf(w4[c], h3T[c * kAP + r], s);
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  if (part == 0) out[r] = s + b4;
}

__device__ __forceinline__ void forward_tile(const MlpArgs& a, unsigned char* sm, float* h3T, float* out) {
  const __nv_bfloat16* w1 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW1);
  const __nv_bfloat16* w2 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW2);
  const __nv_bfloat16* w3 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW3);
  const float* vec = reinterpret_cast<const float*>(sm + kSmVec);
  float* xT = reinterpret_cast<float*>(sm + kSmX);
  float* h1T = reinterpret_cast<float*>(sm + kSmH1);
  float* h2T = reinterpret_cast<float*>(sm + kSmH2);
  layer_fwd<kIn>(xT, w1, vec, h1T);
  __syncthreads();
  layer_fwd<kHid>(h1T, w2, vec + kHid, h2T);
  __syncthreads();
  layer_fwd<kHid>(h2T, w3, vec + 2 * kHid, h3T);
  __syncthreads();
  layer_out(h3T, vec + 3 * kHid, vec[4 * kHid], out);
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads) k_mlp_forward(MlpArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  load_params(a.params, sm);
  float* xT = reinterpret_cast<float*>(sm + kSmX);
  float* h3T = reinterpret_cast<float*>(sm + kSmH1);  // inference reuses h1 for h3
  float* out = reinterpret_cast<float*>(sm + kSmInfer);
  const int per = kTile / a.SP;
  const int64_t ntiles = (a.nreps + per - 1) / per;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    __syncthreads();
    tile_features(a, t * per, xT);
    __syncthreads();
    const __nv_bfloat16* w1 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW1);
    const __nv_bfloat16* w2 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW2);
    const __nv_bfloat16* w3 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW3);
    const float* vec = reinterpret_cast<const float*>(sm + kSmVec);
    float* h1T = reinterpret_cast<float*>(sm + kSmH1);
    float* h2T = reinterpret_cast<float*>(sm + kSmH2);
    layer_fwd<kIn>(xT, w1, vec, h1T);
    __syncthreads();
    layer_fwd<kHid>(h1T, w2, vec + kHid, h2T);
    __syncthreads();
    layer_fwd<kHid>(h2T, w3, vec + 2 * kHid, h3T);
    __syncthreads();
    layer_out(h3T, vec + 3 * kHid, vec[4 * kHid], out);
    __syncthreads();
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

// dW[i][c] (+)= sum_r inT[i][r] gT[c][r] and db[c] (+)= sum_r gT[c][r] into
// the block's partial.  Thread t: i = t/16 + 16u (u < K/16), c = t%16 + 16v.
template <int K>
__device__ __forceinline__ void grad_w(const float* __restrict__ inT, const float* __restrict__ gT,
                                       float* __restrict__ gW, float* __restrict__ gb) {
  constexpr int NU = K / 16;
  const int ig = threadIdx.x >> 4, cg = threadIdx.x & 15;
  float acc[NU][8];
#pragma unroll
  for (int u = 0; u < NU; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
  for (int r = 0; r < kTile; r += 4) {
    float4 gv[8];
#pragma unroll
    for (int v = 0; v < 8; ++v) gv[v] = *reinterpret_cast<const float4*>(gT + (cg + 16 * v) * kAP + r);
#pragma unroll
    for (int u = 0; u < NU; ++u) {
      const float4 x = *reinterpret_cast<const float4*>(inT + (ig + 16 * u) * kAP + r);
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        float s = acc[u][v];
        s = fmaf(x.x, gv[v].x, s);
        s = fmaf(x.y, gv[v].y, s);
        s = fmaf(x.z, gv[v].z, s);
        s = fmaf(x.w, gv[v].w, s);
        acc[u][v] = s;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < NU; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) gW[(ig + 16 * u) * kHid + cg + 16 * v] += acc[u][v];
  if (threadIdx.x < kHid) {
    float s = 0.f;
    for (int r = 0; r < kTile; ++r) s += gT[threadIdx.x * kAP + r];
    gb[threadIdx.x] += s;
  }
}

// dz_prev[i][r] = (sum_c gT[c][r] W[i][c]) * (1 - h[i][r]^2), written over hT.
// Thread t: rows 4*(t/16) .. +3, i = t%16 + 16u.
__device__ __forceinline__ void back_data(const float* __restrict__ gT, const __nv_bfloat16* __restrict__ W,
                                          float* hT) {
  const int rg = threadIdx.x >> 4, ig = threadIdx.x & 15;
  const int r0 = 4 * rg;
  float acc[8][4];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[u][i] = 0.f;
#pragma unroll 2
  for (int c = 0; c < kHid; ++c) {
    const float4 g = *reinterpret_cast<const float4*>(gT + c * kAP + r0);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const float w = __bfloat162float(W[(ig + 16 * u) * kWP + c]);
      acc[u][0] = fmaf(g.x, w, acc[u][0]);
      acc[u][1] = fmaf(g.y, w, acc[u][1]);
      acc[u][2] = fmaf(g.z, w, acc[u][2]);
      acc[u][3] = fmaf(g.w, w, acc[u][3]);
    }
  }
  __syncthreads();  // every thread has read gT; hT is overwritten below (hT != gT)
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    float4* hp = reinterpret_cast<float4*>(hT + (ig + 16 * u) * kAP + r0);
    float4 h = *hp;
    h.x = acc[u][0] * (1.f - h.x * h.x);
    h.y = acc[u][1] * (1.f - h.y * h.y);
    h.z = acc[u][2] * (1.f - h.z * h.z);
    h.w = acc[u][3] * (1.f - h.w * h.w);
    *hp = h;
  }
}

__global__ void __launch_bounds__(kThreads) k_mlp_train(MlpArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  load_params(a.params, sm);
  const __nv_bfloat16* w2 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW2);
  const __nv_bfloat16* w3 = reinterpret_cast<const __nv_bfloat16*>(sm + kSmW3);
  const float* vec = reinterpret_cast<const float*>(sm + kSmVec);
  float* xT = reinterpret_cast<float*>(sm + kSmX);
  float* h1T = reinterpret_cast<float*>(sm + kSmH1);
  float* h2T = reinterpret_cast<float*>(sm + kSmH2);
  float* h3T = reinterpret_cast<float*>(sm + kSmH3);
  float* gT = reinterpret_cast<float*>(sm + kSmG);
  float* out = reinterpret_cast<float*>(sm + kSmRow);
  float* dout = out + kTile;
  float* gp = a.gpart + (size_t)blockIdx.x * kNP;
  const int per = kTile / a.SP;
  const int64_t ntiles = (a.nreps + per - 1) / per;
  double loss = 0.0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    __syncthreads();
    tile_features(a, t * per, xT);
    __syncthreads();
    forward_tile(a, sm, h3T, out);
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
    // output layer: dw4, db4; dz3 = dout * w4 * (1 - h3^2) into gT
    if (threadIdx.x < kHid) {
      const int c = threadIdx.x;
      float s = 0.f;
      for (int r = 0; r < kTile; ++r) s = fmaf(dout[r], h3T[c * kAP + r], s);
      gp[kOffW4 + c] += s;
      const float w4 = vec[3 * kHid + c];
      for (int r = 0; r < kTile; ++r) {
        const float h = h3T[c * kAP + r];
        gT[c * kAP + r] = dout[r] * w4 * (1.f - h * h);
      }
    }
    if (threadIdx.x == kHid) {
      float s = 0.f;
      for (int r = 0; r < kTile; ++r) s += dout[r];
      gp[kOffB4] += s;
    }
    __syncthreads();
    grad_w<kHid>(h2T, gT, gp + kOffW3, gp + kOffB3);
    __syncthreads();
    back_data(gT, w3, h2T);   // h2T <- dz2
    __syncthreads();
    grad_w<kHid>(h1T, h2T, gp + kOffW2, gp + kOffB2);
    __syncthreads();
    back_data(h2T, w2, h1T);  // h1T <- dz1
    __syncthreads();
    // dW1 (16 x 128): i = t/16, c = t%16 + 16v
    {
      const int i = threadIdx.x >> 4, cg = threadIdx.x & 15;
      float acc[8];
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[v] = 0.f;
      for (int r = 0; r < kTile; r += 4) {
        const float4 x = *reinterpret_cast<const float4*>(xT + i * kAP + r);
#pragma unroll
        for (int v = 0; v < 8; ++v) {
          const float4 g = *reinterpret_cast<const float4*>(h1T + (cg + 16 * v) * kAP + r);
          acc[v] = fmaf(x.x, g.x, fmaf(x.y, g.y, fmaf(x.z, g.z, fmaf(x.w, g.w, acc[v]))));
        }
      }
#pragma unroll
      for (int v = 0; v < 8; ++v) gp[kOffW1 + i * kHid + cg + 16 * v] += acc[v];
      if (threadIdx.x < kHid) {
        float s = 0.f;
        for (int r = 0; r < kTile; ++r) s += h1T[threadIdx.x * kAP + r];
        gp[kOffB1 + threadIdx.x] += s;
      }
    }
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
                                         (int)(kSmInfer + 2 * kTile * 4)));
    attr = true;
  }
  MlpArgs a{};
  a.conf = d_c; a.sample = d_s; a.samples = d_smp; a.trig = d_tr;
  a.NOD = nod; a.SP = rotations_padded(nod); a.nreps = n; a.params = d_wb.get(); a.out_f = d_f;
  const int per = kTile / a.SP;
  const int64_t ntiles = (n + per - 1) / per;
  const int nblk = (int)std::min<int64_t>((int64_t)sm_count() * 8, ntiles);
  k_mlp_forward<<<nblk, kThreads, kSmInfer + 2 * kTile * 4, st>>>(a);
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

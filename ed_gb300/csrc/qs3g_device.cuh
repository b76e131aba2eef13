// qs3g_device.cuh -- device helpers shared by the sector, H*v and DSF kernels.
//
// Configurations are the sorted down-spin sites n[0] < ... < n[NOD-1]
// (1-based, as list_fly returns them, state_lists.f90:294-308).  A packed
// configuration stores n[j] in bits [b*j, b*j+b) of a uint64, so the numeric
// order of packed words is the colex order that representative_SQ compares
// (highest site first, state_lists.f90:402-410).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace qs3g {

template <int NOD>
__device__ __forceinline__ void unpack(uint64_t w, int bits, int (&n)[NOD]) {
  const uint64_t mask = (bits >= 64) ? ~0ull : ((1ull << bits) - 1ull);
#pragma unroll
  for (int j = 0; j < NOD; ++j) n[j] = (int)((w >> (bits * j)) & mask);
}

template <int NOD>
__device__ __forceinline__ uint64_t pack(const int (&n)[NOD], int bits) {
  uint64_t w = 0;
#pragma unroll
  for (int j = 0; j < NOD; ++j) w |= (uint64_t)n[j] << (bits * j);
  return w;
}

// Replace n[m] by site e and return the sorted result (j_flip_ni,
// state_lists.f90:333-362, for a bond whose down end n[m] moves to the up end e).
template <int NOD>
__device__ __forceinline__ void move_spin(const int (&n)[NOD], int m, int e, int (&o)[NOD]) {
  // below = number of remaining spins (all but n[m]) on sites < e
  int below = 0;
#pragma unroll
  for (int j = 0; j < NOD; ++j) below += (j != m && n[j] < e) ? 1 : 0;
  // remaining spins r[j] = n[j] for j < m, n[j+1] for j >= m (j = 0..NOD-2);
  // o[j] = r[j] for j < below, e for j == below, r[j-1] for j > below
#pragma unroll
  for (int j = 0; j < NOD; ++j) {
    const int jn = (j + 1 < NOD) ? j + 1 : j;
    const int rj = (j < m) ? n[j] : n[jn];
    const int jp = (j > 0) ? j - 1 : 0;
    const int rjm1 = (jp < m) ? n[jp] : n[j];
    o[j] = (j < below) ? rj : ((j == below) ? e : rjm1);
  }
}

// Directory lookup: candidate index c -> 0-based row, or -1 if c is not a
// row of the sector.  Blocks are 8 x 32-bit words: word 0 = rows before the
// block, words 1..7 = presence bits of 224 consecutive candidates.
__device__ __forceinline__ int64_t dir_lookup(const uint32_t* __restrict__ dir, uint64_t c) {
  const uint64_t blk = c / 224u;
  const unsigned bit = (unsigned)(c - blk * 224u);
  const uint4* bp = reinterpret_cast<const uint4*>(dir) + 2 * blk;
  const uint4 a = __ldg(bp);
  const uint4 b = __ldg(bp + 1);
  const unsigned wi = bit >> 5, bi = bit & 31u;
  const unsigned w0 = a.y, w1 = a.z, w2 = a.w, w3 = b.x, w4 = b.y, w5 = b.z, w6 = b.w;
  unsigned word = w0;
  word = (wi == 1) ? w1 : word;
  word = (wi == 2) ? w2 : word;
  word = (wi == 3) ? w3 : word;
  word = (wi == 4) ? w4 : word;
  word = (wi == 5) ? w5 : word;
  word = (wi == 6) ? w6 : word;
  if (!((word >> bi) & 1u)) return -1;
  unsigned cnt = __popc(word & ((1u << bi) - 1u));
  cnt += (wi > 0) ? __popc(w0) : 0u;
  cnt += (wi > 1) ? __popc(w1) : 0u;
  cnt += (wi > 2) ? __popc(w2) : 0u;
  cnt += (wi > 3) ? __popc(w3) : 0u;
  cnt += (wi > 4) ? __popc(w4) : 0u;
  cnt += (wi > 5) ? __popc(w5) : 0u;
  return (int64_t)a.x + (int64_t)cnt;
}

// Chain representative (LY = LZ = 1).  Among the L translations of a
// configuration, the colex minimum must occupy site 1, so only the NOD
// translations that move one down spin onto site 1 compete.  With cyclic
// gaps g[m] = n[m+1] - n[m] (g[NOD-1] wraps), moving spin m to site 1 gives
// the configuration whose largest site is 1 + L - g[m-1], next 1 + L - g[m-1]
// - g[m-2], ..., so the colex order of candidates is the reverse
// lexicographic order of key_m = (g[m-1], g[m-2], ..., g[m-NOD]).
// The translation recorded as ell follows representative_SQ: the first
// translation i (loop i = 1..L) reaching the minimum, or 0 when n is already
// minimal.  Moving spin m onto site 1 is translation i = L - n[m] + 1, so ties
// go to the candidate with the largest n[m].
// Outputs: p[] = representative (p[0] = 1), ell in [0, L-1].
template <int NOD>
__device__ __forceinline__ void chain_rep(const int (&n)[NOD], int L, int bits, int (&p)[NOD],
                                          int& ell) {
  int g[NOD];
#pragma unroll
  for (int m = 0; m < NOD - 1; ++m) g[m] = n[m + 1] - n[m];
  g[NOD - 1] = n[0] + L - n[NOD - 1];
  uint64_t best = 0, key0 = 0;
  int bm = 0;
#pragma unroll
  for (int m = 0; m < NOD; ++m) {
    uint64_t key = 0;
#pragma unroll
    for (int t = 1; t <= NOD; ++t) key = (key << bits) | (uint64_t)g[(m - t + 2 * NOD) % NOD];
    if (m == 0) key0 = key;
    if (key >= best) { best = key; bm = m; }
  }
  int nb = n[0];
#pragma unroll
  for (int m = 1; m < NOD; ++m) nb = (bm == m) ? n[m] : nb;
  const bool orig = (n[0] == 1) && (key0 == best);
  ell = orig ? 0 : (L - nb + 1);
  // positions of the winning rotation
  p[0] = 1;
#pragma unroll
  for (int j = 1; j < NOD; ++j) {
    int gj = g[0];
#pragma unroll
    for (int m = 1; m < NOD; ++m) gj = (((bm + j - 1) % NOD) == m) ? g[m] : gj;
    p[j] = p[j - 1] + gj;
  }
}

// Anchored candidate index of a configuration with p[0] = 1:
// sum_{j>=1} C(p[j]-2, j), binomA[(j-1)*(L-1) + x] = C(x, j).
template <int NOD>
__device__ __forceinline__ uint64_t anchored_index(const int (&p)[NOD], const uint32_t* __restrict__ binomA,
                                                   int L) {
  uint64_t c = 0;
#pragma unroll
  for (int j = 1; j < NOD; ++j) {
    const int x = p[j] - 2;
    c += (j == 1) ? (uint64_t)x : (uint64_t)__ldg(binomA + (size_t)(j - 1) * (L - 1) + x);
  }
  return c;
}

// Full colex rank minus one: sum_j C(n[j]-1, j+1), binom[k*(NOS+1) + n] = C(n,k).
template <int NOD>
__device__ __forceinline__ uint64_t full_index(const int (&n)[NOD], const uint64_t* __restrict__ binom,
                                               int NOS) {
  uint64_t c = 0;
#pragma unroll
  for (int j = 0; j < NOD; ++j) c += __ldg(binom + (size_t)(j + 1) * (NOS + 1) + (n[j] - 1));
  return c;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

}  // namespace qs3g

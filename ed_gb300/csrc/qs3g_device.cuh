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
// row of the sector.  One 8-byte entry per 32 consecutive candidates:
// .x = rows before the entry, .y = presence bits, so a lookup is one load,
// a mask and a popcount.
__device__ __forceinline__ int dir_lookup(const uint2* __restrict__ dir, uint64_t c) {
  const uint2 w = __ldg(dir + (c >> 5));
  const unsigned b = (unsigned)c & 31u;
  return ((w.y >> b) & 1u) ? (int)(w.x + __popc(w.y & ((1u << b) - 1u))) : -1;
}
__device__ __forceinline__ int dir_lookup32(const uint2* __restrict__ dir, uint32_t c) {
  const uint2 w = __ldg(dir + (c >> 5));
  const unsigned b = c & 31u;
  return ((w.y >> b) & 1u) ? (int)(w.x + __popc(w.y & ((1u << b) - 1u))) : -1;
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
  // The first key component of rotation m is g[m-1]: when the largest gap is
  // unique, its successor wins without comparing whole keys.
  int gmax = g[0], am = 0, ties = 1;
#pragma unroll
  for (int m = 1; m < NOD; ++m) {
    ties = (g[m] == gmax) ? ties + 1 : ((g[m] > gmax) ? 1 : ties);
    am = (g[m] > gmax) ? m : am;
    gmax = max(gmax, g[m]);
  }
  int bm;
  bool orig;
  if (ties == 1) {
    bm = (am + 1 == NOD) ? 0 : am + 1;
    orig = (bm == 0) && (n[0] == 1);
  } else {
    uint64_t best = 0, key0 = 0;
    bm = 0;
#pragma unroll
    for (int m = 0; m < NOD; ++m) {
      uint64_t key = 0;
#pragma unroll
      for (int t = 1; t <= NOD; ++t) key = (key << bits) | (uint64_t)g[(m - t + 2 * NOD) % NOD];
      if (m == 0) key0 = key;
      if (key >= best) { best = key; bm = m; }
    }
    orig = (n[0] == 1) && (key0 == best);
  }
  if (orig) {  // already the representative: ell = 0
    ell = 0;
#pragma unroll
    for (int j = 0; j < NOD; ++j) p[j] = n[j];
    return;
  }
  int nb = n[0];
#pragma unroll
  for (int m = 1; m < NOD; ++m) nb = (bm == m) ? n[m] : nb;
  ell = L - nb + 1;
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

// chain_rep plus the number of self-translations of the representative
// (translations i in 1..L with T^i rep = rep): 1 when the largest gap is
// unique, else the number of rotations whose key equals the winning key.
// The norm of a chain representative depends only on this count.
template <int NOD>
__device__ __forceinline__ void chain_rep_count(const int (&n)[NOD], int L, int bits, int (&p)[NOD], int& ell,
                                                int& cnt) {
  int g[NOD];
#pragma unroll
  for (int m = 0; m < NOD - 1; ++m) g[m] = n[m + 1] - n[m];
  g[NOD - 1] = n[0] + L - n[NOD - 1];
  int gmax = g[0], am = 0, ties = 1;
#pragma unroll
  for (int m = 1; m < NOD; ++m) {
    ties = (g[m] == gmax) ? ties + 1 : ((g[m] > gmax) ? 1 : ties);
    am = (g[m] > gmax) ? m : am;
    gmax = max(gmax, g[m]);
  }
  int bm;
  bool orig;
  if (ties == 1) {
    bm = (am + 1 == NOD) ? 0 : am + 1;
    orig = (bm == 0) && (n[0] == 1);
    cnt = 1;
  } else {
    uint64_t best = 0, key0 = 0;
    uint64_t key[NOD];
    bm = 0;
#pragma unroll
    for (int m = 0; m < NOD; ++m) {
      uint64_t k = 0;
#pragma unroll
      for (int t = 1; t <= NOD; ++t) k = (k << bits) | (uint64_t)g[(m - t + 2 * NOD) % NOD];
      key[m] = k;
      if (m == 0) key0 = k;
      if (k >= best) { best = k; bm = m; }
    }
    cnt = 0;
#pragma unroll
    for (int m = 0; m < NOD; ++m) cnt += (key[m] == best) ? 1 : 0;
    orig = (n[0] == 1) && (key0 == best);
  }
  if (orig) {
    ell = 0;
#pragma unroll
    for (int j = 0; j < NOD; ++j) p[j] = n[j];
    return;
  }
  int nb = n[0];
#pragma unroll
  for (int m = 1; m < NOD; ++m) nb = (bm == m) ? n[m] : nb;
  ell = L - nb + 1;
  p[0] = 1;
#pragma unroll
  for (int j = 1; j < NOD; ++j) {
    int gj = g[0];
#pragma unroll
    for (int m = 1; m < NOD; ++m) gj = (((bm + j - 1) % NOD) == m) ? g[m] : gj;
    p[j] = p[j - 1] + gj;
  }
}

// Number of self-translations of a chain representative p (p[0] = 1, key_0 maximal).
template <int NOD>
__device__ __forceinline__ int chain_self_count(const int (&p)[NOD], int L, int bits) {
  int g[NOD];
#pragma unroll
  for (int m = 0; m < NOD - 1; ++m) g[m] = p[m + 1] - p[m];
  g[NOD - 1] = p[0] + L - p[NOD - 1];
  int gmax = g[0], ties = 1;
#pragma unroll
  for (int m = 1; m < NOD; ++m) {
    ties = (g[m] == gmax) ? ties + 1 : ((g[m] > gmax) ? 1 : ties);
    gmax = max(gmax, g[m]);
  }
  if (ties == 1) return 1;
  uint64_t key0 = 0;
#pragma unroll
  for (int t = 1; t <= NOD; ++t) key0 = (key0 << bits) | (uint64_t)g[(0 - t + 2 * NOD) % NOD];
  int cnt = 1;
#pragma unroll
  for (int m = 1; m < NOD; ++m) {
    uint64_t k = 0;
#pragma unroll
    for (int t = 1; t <= NOD; ++t) k = (k << bits) | (uint64_t)g[(m - t + 2 * NOD) % NOD];
    cnt += (k == key0) ? 1 : 0;
  }
  return cnt;
}

// Anchored candidate index with 32-bit arithmetic: C(x,1) = x and
// C(x,2) = x(x-1)/2 in registers, higher binomials from the table.
template <int NOD>
__device__ __forceinline__ uint32_t anchored_index32(const int (&p)[NOD], const uint32_t* __restrict__ binomA, int L) {
  uint32_t c = 0;
#pragma unroll
  for (int j = 1; j < NOD; ++j) {
    const uint32_t x = (uint32_t)(p[j] - 2);
    if (j == 1) c += x;
    else if (j == 2) c += (x * (x - 1u)) >> 1;
    else c += __ldg(binomA + (size_t)(j - 1) * (L - 1) + x);
  }
  return c;
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

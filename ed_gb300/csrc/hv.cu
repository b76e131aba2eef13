// hv.cu -- matrix-free XXZ H*v over the (NOD, K) representative basis.
//
// Replaces ham_to_vec_wave_vector (ham2vec_v3.f90:37-72).  Gather form: each
// output row is computed by exactly one thread (chains) or one warp (general
// lattices) and written once, with no atomics, so results are deterministic.
//
// Per row the reference loops over all NOxxz bonds; here the loop runs over
// the bonds incident to the row's NOD down spins (site adjacency, both bond
// ends listed), which visits every antiparallel bond exactly once:
//   diagonal  = sum_b sJz_b * (+1 parallel / -1 antiparallel)
//             = Sz_all - 2 * (sum_{d down} Sz_site[d] - sum_{both-down encounters} sJz_b)
//   hop       = sJxy_b * list_r(id) / list_r(i) * explist(ell) * v1(id)
// For chains the representative of each hop comes from chain_rep (O(NOD^2)
// cyclic-gap keys, same ell rule as representative_SQ); general lattices scan
// all translations with the 32 lanes of a warp and reduce with shuffles.
// The row index comes from the sector directory (one 32-byte load) instead of
// findstate's binary search.
#include "eft.cuh"
#include "qs3g_device.cuh"
#include "qs3g_internal.cuh"
#include "krylov.h"

namespace qs3g {
namespace {

template <class F>
void dispatch_nod(int NOD, F&& f) {
  switch (NOD) {
    case 1: f(std::integral_constant<int, 1>{}); break;
    case 2: f(std::integral_constant<int, 2>{}); break;
    case 3: f(std::integral_constant<int, 3>{}); break;
    case 4: f(std::integral_constant<int, 4>{}); break;
    case 5: f(std::integral_constant<int, 5>{}); break;
    case 6: f(std::integral_constant<int, 6>{}); break;
    case 7: f(std::integral_constant<int, 7>{}); break;
    case 8: f(std::integral_constant<int, 8>{}); break;
    default: throw Error(QS3G_ENOTSUP, "NOD > 8 is not instantiated");
  }
}

struct HvArgs {
  int64_t D;
  int L, NOS, bits, LX, LY, LZ, NT;
  const uint64_t* conf;
  const double* list_r;
  const float* list_r32;
  const uint2* dir;
  const uint32_t* binomA;
  const uint64_t* binom;
  const int* adj_off;
  const uint32_t* adj;
  const double* sJxy;
  const double* sJz;
  const double* Sz_site;
  double Sz_all;
  const double2* chainph;
  const float2* chainph32;
  const double2* explist;
  const int16_t* xyz;
  const double* diag;      // H(i,i), precomputed at sector build
  const float* diag32;
  const double* coefR;     // chains: sJxy_b * list_r for a representative with c self-translations
  const float* coefR32;    //         [b * (NOD + 1) + c]
  const double* invR;      // chains: 1 / list_r by self-translation count
  const float* invR32;
  int uno;                 // uniform chains: number of bond distances (0: not uniform)
  int uoff[2];             //   the distances
  int ubond[2];            //   one bond of each distance (their couplings are equal)
};

constexpr int kHvThreads = 256;
static_assert(kSegPartials == kHvThreads / 32, "one alpha partial per warp of a batched product block");
constexpr int kUniBlocks = 5;  // uniform chain rows: 40 resident warps per SM (<= 51 registers)

// ------------------------------------------------------------ chain kernels
// One thread per row.  The row's diagonal is precomputed at sector build
// (diag[i]); every hop costs two FP64 FMAs: the coefficient
// sJxy_b * list_r(id) comes from a (bond, self-translation count) table,
// because a chain representative's norm depends only on that count, which
// chain_rep_count returns with the representative -- so list_r(id) is never
// gathered.  The 1/list_r(i) factor is applied once per row.
//
// V is the vector element: double2 / float2 for complex(8) / complex(4)
// vectors, double / float for the real vectors of sectors whose H is real
// symmetric (k = 0 chains, U(1)); P is the complex type of the phase table.
template <class V>
struct Cplx;
template <>
struct Cplx<double2> {
  using R = double;
  using P = double2;
  static __device__ __forceinline__ double2 mul(double2 a, double2 b) { return cmul(a, b); }
};
template <>
struct Cplx<float2> {
  using R = float;
  using P = float2;
  static __device__ __forceinline__ float2 mul(float2 a, float2 b) { return cmulf(a, b); }
};
template <>
struct Cplx<double> {
  using R = double;
  using P = double2;
};
template <>
struct Cplx<float> {
  using R = float;
  using P = float2;
};

// one hop: (ax, ay) += c * x(id)
__device__ __forceinline__ void hop_acc(double c, double2 v, double& ax, double& ay) {
  ax = fma(c, v.x, ax);
  ay = fma(c, v.y, ay);
}
__device__ __forceinline__ void hop_acc(float c, float2 v, float& ax, float& ay) {
  ax = fmaf(c, v.x, ax);
  ay = fmaf(c, v.y, ay);
}
__device__ __forceinline__ void hop_acc(double c, double v, double& ax, double&) { ax = fma(c, v, ax); }
__device__ __forceinline__ void hop_acc(float c, float v, float& ax, float&) { ax = fmaf(c, v, ax); }
// the row's result di * x(i) + ir * (ax, ay)
__device__ __forceinline__ double2 row_out(double di, double2 xi, double ir, double ax, double ay) {
  return make_double2(fma(di, xi.x, ir * ax), fma(di, xi.y, ir * ay));
}
__device__ __forceinline__ float2 row_out(float di, float2 xi, float ir, float ax, float ay) {
  return make_float2(fmaf(di, xi.x, ir * ax), fmaf(di, xi.y, ir * ay));
}
__device__ __forceinline__ double row_out(double di, double xi, double ir, double ax, double) {
  return fma(di, xi, ir * ax);
}
__device__ __forceinline__ float row_out(float di, float xi, float ir, float ax, float) {
  return fmaf(di, xi, ir * ax);
}
// the same without a row factor (U(1) rows)
__device__ __forceinline__ double2 row_out(double di, double2 xi, double ax, double ay) {
  return make_double2(fma(di, xi.x, ax), fma(di, xi.y, ay));
}
__device__ __forceinline__ float2 row_out(float di, float2 xi, float ax, float ay) {
  return make_float2(fmaf(di, xi.x, ax), fmaf(di, xi.y, ay));
}
__device__ __forceinline__ double row_out(double di, double xi, double ax, double) { return fma(di, xi, ax); }
__device__ __forceinline__ float row_out(float di, float xi, float ax, float) { return fmaf(di, xi, ax); }

// The general hop: j_flip_ni + representative_SQ on the sorted configuration
// (move_spin, then the gap-key search of chain_rep_count).  Returns the row id
// (or -1), the translation ell and the target's self-translation count.
template <int NOD>
__device__ __forceinline__ int chain_hop_general(const HvArgs& a, const int (&n)[NOD], int m, int e, int& ell,
                                                 int& cnt) {
  int o[NOD], p[NOD];
  move_spin<NOD>(n, m, e, o);
  chain_rep_count<NOD>(o, a.L, a.bits, p, ell, cnt);
  return dir_lookup32(a.dir, anchored_index32<NOD>(p, a.binomA, a.L));
}

// The general hop out of line: the uniform rows unroll all their hops, and an
// inlined copy of the general path per hop would crowd the instruction cache.
// The row's configuration comes packed, so the caller's registers stay registers.
template <int NOD>
__device__ __noinline__ int chain_hop_slow(const HvArgs& a, uint64_t conf, int m, int e, int& ell, int& cnt) {
  int n[NOD];
  unpack<NOD>(conf, a.bits, n);
  return chain_hop_general<NOD>(a, n, m, e, ell, cnt);
}

// Chain rows work on the cyclic gaps g[k] = n[k+1] - n[k] (lane k; lane NOD-1
// wraps).  A hop moves spin m by del = e - n[m] (taken the short way round the
// ring); when it neither lands on nor passes another spin (|del| below the gap
// on its side) only lanes m-1 and m change, by +del and -del.  The
// representative is then read off the lanes directly: with a unique largest
// gap at lane c, the spin after it (c+1) goes to site 1, the representative's
// sites are 1, 1 + g[c+1], 1 + g[c+1] + g[c+2], ... (the last one 1 + L -
// g[c]), it has one self-translation, and representative_SQ's ell is
// L - site + 1 of that spin (0 when it already sits on site 1).  The
// anchored index sum_{j>=1} C(p_j - 2, j) and the directory give the row --
// the same (id, ell, count) as the general path, so the products are
// bit-identical.  Moves onto or past another spin, tied largest gaps and a
// single down spin take the general path.
template <int NOD, bool KZERO, class V, bool DEFER = false>
__device__ __forceinline__ void hv_chain_row(const HvArgs& a, const V* __restrict__ x, V* __restrict__ y,
                                             const double* __restrict__ diag,
                                             const typename Cplx<V>::R* __restrict__ coefR,
                                             const typename Cplx<V>::R* __restrict__ invR,
                                             const typename Cplx<V>::P* __restrict__ ph, int64_t i, double shift) {
  using R = typename Cplx<V>::R;
  int n[NOD];
  unpack<NOD>(__ldg(a.conf + i), a.bits, n);
  int g[NOD];
#pragma unroll
  for (int k = 0; k < NOD - 1; ++k) g[k] = n[k + 1] - n[k];
  g[NOD - 1] = n[0] + a.L - n[NOD - 1];
  const V xi = x[i];
  const R di = (R)(__ldg(diag + i) - shift);  // shift applied in FP64 before rounding
  const int L = a.L, half = a.L >> 1;
  R ax = 0, ay = 0;
  uint32_t pend = 0;  // DEFER: general-path hops (spin m, adjacency slot k) as bit 4 m + k
#pragma unroll
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    const int mp = (m + NOD - 1) % NOD;  // lane before spin m
    const int gn = g[m], gp = g[mp];
    // the largest of the other lanes, its lane and how often it occurs
    int omax = -1, oarg = 0, oties = 0;
#pragma unroll
    for (int k = 0; k < NOD; ++k) {
      if (k == m || k == mp) continue;
      oties = (g[k] == omax) ? oties + 1 : ((g[k] > omax) ? 1 : oties);
      oarg = (g[k] > omax) ? k : oarg;
      omax = max(omax, g[k]);
    }
    const int e0 = __ldg(a.adj_off + d), e1 = __ldg(a.adj_off + d + 1);
    for (int t = e0; t < e1; ++t) {
      const uint32_t w = __ldg(a.adj + t);
      const int e = (int)(w & 0xffffu);
      int del = e - d;
      del += (del > half) ? -L : ((del < -half) ? L : 0);
      const int ad = del > 0 ? del : -del;
      int id, ell = 0, cnt = 1;
      int lm = 0, ln = 0, mx = 0, c = 0, nmx = 0;
      if (NOD >= 2) {
        lm = gp + del;  // new lane m-1
        ln = gn - del;  // new lane m
        mx = max(max(lm, ln), omax);
        nmx = (lm == mx) + (ln == mx) + (omax == mx ? oties : 0);
        c = (lm == mx) ? mp : ((ln == mx) ? m : oarg);
      }
      if (NOD >= 2 && ad < (del > 0 ? gn : gp) && nmx == 1) {
        // lanes c+1, c+2, ... of the moved configuration, as sites p_1, p_2, ...;
        // the last site is always 1 + L - (largest gap)
        uint32_t idx = 0;
        if constexpr (NOD == 4) {
          // the four cases of c: lane m-1, lane m, or the larger other lane
          const int m1 = (m + 1) % NOD, m2 = (m + 2) % NOD;
          const bool cA = (lm == mx), cB = (ln == mx), o1 = (oarg == m1);
          const int G1 = cA ? ln : (cB ? g[m1] : (o1 ? g[m2] : lm));
          const int G12 = cA ? ln + g[m1] : (cB ? g[m1] + g[m2] : (o1 ? g[m2] + lm : lm + ln));
          const uint32_t x2 = (uint32_t)(G12 - 1);
          idx = (uint32_t)(G1 - 1) + ((x2 * (x2 - 1u)) >> 1) + __ldg(a.binomA + 2 * (size_t)(L - 1) + (L - 1 - mx));
        } else {
          int pj = 1;
#pragma unroll
          for (int j = 1; j < NOD; ++j) {
            int lane = 0;
            if (j == NOD - 1) {
              lane = L - mx - (pj - 1);
            } else {
#pragma unroll
              for (int k = 0; k < NOD; ++k) {
                const int vk = (k == mp) ? lm : ((k == m) ? ln : g[k]);
                lane = (c == (k - j + NOD) % NOD) ? vk : lane;
              }
            }
            pj += lane;
            const uint32_t xj = (uint32_t)(pj - 2);
            if (j == 1) idx += xj;
            else if (j == 2) idx += (xj * (xj - 1u)) >> 1;
            else idx += __ldg(a.binomA + (size_t)(j - 1) * (L - 1) + xj);
          }
        }
        id = dir_lookup32(a.dir, idx);
        if constexpr (!KZERO) {
          const int sw = (c + 1) % NOD;  // the spin that goes to site 1
          int site = n[0];
#pragma unroll
          for (int k = 1; k < NOD; ++k) site = (sw == k) ? n[k] : site;
          site = (sw == m) ? e : site;
          ell = (site == 1) ? 0 : L - site + 1;
        }
      } else {
        bool edown = false;
#pragma unroll
        for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
        if (edown) continue;  // parallel bond: diagonal only
        if constexpr (DEFER) {
          if (NOD <= 8 && t - e0 < 4) {
            pend |= 1u << (4 * m + (t - e0));
            continue;
          }
        }
        id = chain_hop_general<NOD>(a, n, m, e, ell, cnt);
      }
      if (id < 0) continue;
      V xv = x[id];
      if constexpr (!KZERO) xv = Cplx<V>::mul(__ldg(ph + ell), xv);
      hop_acc(__ldg(coefR + (w >> 16) * (NOD + 1) + cnt), xv, ax, ay);
    }
  }
  if constexpr (DEFER) {
    // Deferred general-path hops: a warp runs this loop as often as its
    // busiest lane has such hops, instead of once for every hop position
    // at which any of its 32 rows needs the general path.
    const uint64_t cw = __ldg(a.conf + i);
    while (pend) {
      const int slot = __ffs(pend) - 1;
      pend &= pend - 1;
      const int m = slot >> 2;
      int d = n[0];
#pragma unroll
      for (int k = 1; k < NOD; ++k) d = (m == k) ? n[k] : d;
      const uint32_t w = __ldg(a.adj + __ldg(a.adj_off + d) + (slot & 3));
      const int e = (int)(w & 0xffffu);
      int ell = 0, cnt = 1;
      const int id = chain_hop_slow<NOD>(a, cw, m, e, ell, cnt);
      if (id < 0) continue;
      V xv = x[id];
      if constexpr (!KZERO) xv = Cplx<V>::mul(__ldg(ph + ell), xv);
      hop_acc(__ldg(coefR + (w >> 16) * (NOD + 1) + cnt), xv, ax, ay);
    }
  }
  const R ir = __ldg(invR + chain_self_count<NOD>(n, a.L, a.bits));
  y[i] = row_out(di, xi, ir, ax, ay);
}


// Uniform chains: every site s carries a bond to s + o (mod L) for each of NO
// distances o < L/2, with one coupling per distance (the chains of the XXZ
// configs).  The hops of spin m are then the moves by +o and -o: no
// adjacency list, no displacement arithmetic, and all NOD * NO * 2 hops are
// unrolled, so their directory and x(id) loads are independent and can be
// in flight together.  Hops that reach another spin or meet a tied largest
// gap take the general path.  The sum runs over the same hops as
// hv_chain_row, in another order.
template <int NOD, int NO, bool KZERO, class V>
__device__ __forceinline__ void hv_uchain_row(const HvArgs& a, const V* __restrict__ x, V* __restrict__ y,
                                              const double* __restrict__ diag,
                                              const typename Cplx<V>::R* __restrict__ coefR,
                                              const typename Cplx<V>::R* __restrict__ invR,
                                              const typename Cplx<V>::P* __restrict__ ph, int64_t i, double shift) {
  using R = typename Cplx<V>::R;
  const uint64_t cw = __ldg(a.conf + i);
  int n[NOD];
  unpack<NOD>(cw, a.bits, n);
  int g[NOD];
#pragma unroll
  for (int k = 0; k < NOD - 1; ++k) g[k] = n[k + 1] - n[k];
  g[NOD - 1] = n[0] + a.L - n[NOD - 1];
  const V xi = x[i];
  const R di = (R)(__ldg(diag + i) - shift);  // shift applied in FP64 before rounding
  const int L = a.L;
  int off[NO];
  R cf[NO];
#pragma unroll
  for (int k = 0; k < NO; ++k) {
    off[k] = a.uoff[k];
    cf[k] = __ldg(coefR + a.ubond[k] * (NOD + 1) + 1);
  }
  R ax = 0, ay = 0;
#pragma unroll
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    const int mp = (m + NOD - 1) % NOD;
    const int gn = g[m], gp = g[mp];
    int omax = -1, oarg = 0, oties = 0;
#pragma unroll
    for (int k = 0; k < NOD; ++k) {
      if (k == m || k == mp) continue;
      oties = (g[k] == omax) ? oties + 1 : ((g[k] > omax) ? 1 : oties);
      oarg = (g[k] > omax) ? k : oarg;
      omax = max(omax, g[k]);
    }
#pragma unroll
    for (int k = 0; k < NO; ++k) {
#pragma unroll
      for (int dir = 0; dir < 2; ++dir) {
        const int o = off[k];
        const int del = dir ? -o : o;
        const int lm = gp + del, ln = gn - del;
        const int mx = max(max(lm, ln), omax);
        const int nmx = (lm == mx) + (ln == mx) + (omax == mx ? oties : 0);
        int id, ell = 0, cnt = 1;
        R cc = cf[k];
        if ((dir ? o < gp : o < gn) && nmx == 1) {
          uint32_t idx = 0;
          const bool cA = (lm == mx), cB = (ln == mx);
          if constexpr (NOD == 4) {
            const int m1 = (m + 1) % NOD, m2 = (m + 2) % NOD;
            const bool o1 = (oarg == m1);
            const int G1 = cA ? ln : (cB ? g[m1] : (o1 ? g[m2] : lm));
            const int G12 = cA ? ln + g[m1] : (cB ? g[m1] + g[m2] : (o1 ? g[m2] + lm : lm + ln));
            const uint32_t x2 = (uint32_t)(G12 - 1);
            idx = (uint32_t)(G1 - 1) + ((x2 * (x2 - 1u)) >> 1) +
                  __ldg(a.binomA + 2 * (size_t)(L - 1) + (L - 1 - mx));
          } else {
            const int c = cA ? mp : (cB ? m : oarg);
            int pj = 1;
#pragma unroll
            for (int j = 1; j < NOD; ++j) {
              int lane = 0;
              if (j == NOD - 1) {
                lane = L - mx - (pj - 1);
              } else {
#pragma unroll
                for (int q = 0; q < NOD; ++q) {
                  const int vq = (q == mp) ? lm : ((q == m) ? ln : g[q]);
                  lane = (c == (q - j + NOD) % NOD) ? vq : lane;
                }
              }
              pj += lane;
              const uint32_t xj = (uint32_t)(pj - 2);
              if (j == 1) idx += xj;
              else if (j == 2) idx += (xj * (xj - 1u)) >> 1;
              else idx += __ldg(a.binomA + (size_t)(j - 1) * (L - 1) + xj);
            }
          }
          id = dir_lookup32(a.dir, idx);
          if constexpr (!KZERO) {
            const int c = cA ? mp : (cB ? m : oarg);
            const int sw = (c + 1) % NOD;  // the spin that goes to site 1
            int e = d + del;
            e = (e > L) ? e - L : ((e < 1) ? e + L : e);
            int site = n[0];
#pragma unroll
            for (int q = 1; q < NOD; ++q) site = (sw == q) ? n[q] : site;
            site = (sw == m) ? e : site;
            ell = (site == 1) ? 0 : L - site + 1;
          }
        } else {
          int e = d + del;
          e = (e > L) ? e - L : ((e < 1) ? e + L : e);
          bool edown = false;
#pragma unroll
          for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
          if (edown) continue;  // parallel bond: diagonal only
          id = chain_hop_slow<NOD>(a, cw, m, e, ell, cnt);
          cc = __ldg(coefR + a.ubond[k] * (NOD + 1) + cnt);
        }
        if (id < 0) continue;
        V xv = x[id];
        if constexpr (!KZERO) xv = Cplx<V>::mul(__ldg(ph + ell), xv);
        hop_acc(cc, xv, ax, ay);
      }
    }
  }
  const R ir = __ldg(invR + chain_self_count<NOD>(n, a.L, a.bits));
  y[i] = row_out(di, xi, ir, ax, ay);
}

template <int NOD, int NO, bool KZERO>
__global__ void __launch_bounds__(kHvThreads, kUniBlocks) k_hv_uchain32(HvArgs a, const float2* __restrict__ x,
                                                            float2* __restrict__ y, float shift) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  hv_uchain_row<NOD, NO, KZERO, float2>(a, x, y, a.diag, a.coefR32, a.invR32, a.chainph32, i, (double)shift);
}


template <int NOD, int NO>
__global__ void __launch_bounds__(kHvThreads, kUniBlocks) k_hv_uchain32r(HvArgs a, const float* __restrict__ x,
                                                             float* __restrict__ y, float shift, int pad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.D) hv_uchain_row<NOD, NO, true, float>(a, x, y, a.diag, a.coefR32, a.invR32, nullptr, i, (double)shift);
  else if (i == a.D && pad) y[i] = 0.f;
}

// f(NOD, NO) for a uniform chain sector with 2 <= NOD <= 6 and 1 <= NO <= 2;
// false when the sector takes the general chain kernels.
template <class F>
bool dispatch_uniform(const Model& m, const Sector& s, F&& f) {
  if (!s.anchored || m.uni_no < 1 || m.uni_no > 2 || s.NOD < 2 || s.NOD > 6) return false;
  auto with_no = [&](auto nod) {
    if (m.uni_no == 1) f(nod, std::integral_constant<int, 1>{});
    else f(nod, std::integral_constant<int, 2>{});
  };
  switch (s.NOD) {
    case 2: with_no(std::integral_constant<int, 2>{}); break;
    case 3: with_no(std::integral_constant<int, 3>{}); break;
    case 4: with_no(std::integral_constant<int, 4>{}); break;
    case 5: with_no(std::integral_constant<int, 5>{}); break;
    default: with_no(std::integral_constant<int, 6>{}); break;
  }
  return true;
}

template <int NOD, bool KZERO>
__global__ void __launch_bounds__(kHvThreads) k_hv_chain64(HvArgs a, const double2* __restrict__ x,
                                                           double2* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  hv_chain_row<NOD, KZERO, double2>(a, x, y, a.diag, a.coefR, a.invR, a.chainph, i, 0.0);
}

template <int NOD, bool KZERO>
__global__ void __launch_bounds__(kHvThreads) k_hv_chain32(HvArgs a, const float2* __restrict__ x,
                                                           float2* __restrict__ y, float shift) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  hv_chain_row<NOD, KZERO, float2>(a, x, y, a.diag, a.coefR32, a.invR32, a.chainph32, i, (double)shift);
}

// Real vectors (k = 0): rows 0..D-1; with pad != 0 also a zero in element D
// (D odd), so that real vectors packed two rows per complex slot keep a zero
// pad.
template <int NOD>
__global__ void __launch_bounds__(kHvThreads) k_hv_chain64r(HvArgs a, const double* __restrict__ x,
                                                            double* __restrict__ y, int pad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.D) hv_chain_row<NOD, true, double>(a, x, y, a.diag, a.coefR, a.invR, nullptr, i, 0.0);
  else if (i == a.D && pad) y[i] = 0.0;
}

template <int NOD>
__global__ void __launch_bounds__(kHvThreads) k_hv_chain32r(HvArgs a, const float* __restrict__ x,
                                                            float* __restrict__ y, float shift, int pad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.D) hv_chain_row<NOD, true, float>(a, x, y, a.diag, a.coefR32, a.invR32, nullptr, i, (double)shift);
  else if (i == a.D && pad) y[i] = 0.f;
}

// ------------------------------------------------------------ batches of chain sectors
// Block b works on segment blk_seg[b], rows (b - blk_first[b]) * 256 + tid of
// it; the segment's tables replace the handle's in the row function.
// ------------------------------------------------------------ cached connection table
// The same products from the table that k_tab_build writes once per sector
// (HvTable): per row the slots in the order the matrix-free row visits its
// hops, each the target row and its coefficient, so the integer work of the
// representative search is done once instead of at every product.  The FP64
// sums take the same terms in the same order as hv_chain_row's, so the
// complex(8) and real FP64 products equal the matrix-free ones bit for bit.
struct TabArgs {
  int64_t D;
  int L, bits, slots;
  const uint64_t* conf;
  const uint32_t* tab;
  const uint32_t* tabc;
  const double* diag;
  const double* coefR;
  const float* coefR32;
  const double* invR;
  const float* invR32;
  const double* tcoef;
  const float* tcoef32;
  const double2* chainph;
  const float2* chainph32;
  const float2* coefS;
  const float4* phS;
};

template <int NOD, bool PACKED, bool KZERO, class V, int SLOTS>
__device__ __forceinline__ V tab_row(const TabArgs& t, const V* __restrict__ x, int64_t i, double shift) {
  using R = typename Cplx<V>::R;
  constexpr bool F64 = sizeof(R) == sizeof(double);
  const R* coefR = [&] { if constexpr (F64) return t.coefR; else return t.coefR32; }();
  const R* tcoef = [&] { if constexpr (F64) return t.tcoef; else return t.tcoef32; }();
  const R* invR = [&] { if constexpr (F64) return t.invR; else return t.invR32; }();
  const auto* ph = [&] { if constexpr (F64) return t.chainph; else return t.chainph32; }();
  int n[NOD];
  unpack<NOD>(__ldg(t.conf + i), t.bits, n);
  const V xi = x[i];
  const R di = (R)(__ldg(t.diag + i) - shift);
  R ax = 0, ay = 0;
  const int ns = SLOTS > 0 ? SLOTS : t.slots;
#pragma unroll
  for (int sl = 0; sl < (SLOTS > 0 ? SLOTS : 64); ++sl) {
    if (SLOTS == 0 && sl >= ns) break;
    const uint32_t e = __ldg(t.tab + (size_t)sl * t.D + i);
    int id, ell = 0;
    R c;
    if constexpr (PACKED) {
      if (e == 0xffffffffu) continue;
      id = (int)(e & 0x7ffffffu);
      c = __ldg(tcoef + (e >> 27));
    } else {
      id = (int)e;
      if (id < 0) continue;
      const uint32_t k = __ldg(t.tabc + (size_t)sl * t.D + i);
      c = __ldg(coefR + (k & 0xffffu));
      ell = (int)(k >> 16);
    }
    V xv = x[id];
    if constexpr (!KZERO) xv = Cplx<V>::mul(__ldg(ph + ell), xv);
    hop_acc(c, xv, ax, ay);
  }
  const R ir = __ldg(invR + chain_self_count<NOD>(n, t.L, t.bits));
  return row_out(di, xi, ir, ax, ay);
}

// The complex(8) table row in double-float arithmetic on the FP32 pipe:
// x(id) split with integer instructions (dsplit), phases and coefficients
// from pre-split tables, sums as unevaluated float pairs; one FP64 subtraction
// (diagonal - shift) and the final joins per row.  GB300 runs FP64 at 1/64 of
// the FP32 rate, and a k != 0 hop costs 6 FP64 operations in FP64.
template <int NOD, bool PACKED, bool KZERO, class V = double2, int SLOTS = 0>
__device__ __forceinline__ V tab_row_df(const TabArgs& t, const V* __restrict__ x, int64_t i, double shift) {
  constexpr bool CPLX = sizeof(V) == sizeof(double2);
  int n[NOD];
  unpack<NOD>(__ldg(t.conf + i), t.bits, n);
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
#pragma unroll
  for (int sl = 0; sl < (SLOTS > 0 ? SLOTS : 64); ++sl) {
    if (SLOTS == 0 && sl >= t.slots) break;
    const uint32_t e = __ldg(t.tab + (size_t)sl * t.D + i);
    int id, ell = 0;
    float2 c;
    if constexpr (PACKED) {
      if (e == 0xffffffffu) continue;
      id = (int)(e & 0x7ffffffu);
      c = __ldg(t.coefS + (e >> 27));
    } else {
      id = (int)e;
      if (id < 0) continue;
      const uint32_t k = __ldg(t.tabc + (size_t)sl * t.D + i);
      c = __ldg(t.coefS + (k & 0xffffu));
      ell = (int)(k >> 16);
    }
    float2 xr, xm = make_float2(0.f, 0.f);
    if constexpr (CPLX) {
      const double2 xv = x[id];
      xr = dsplit(xv.x);
      xm = dsplit(xv.y);
    } else {
      xr = dsplit(x[id]);
    }
    if constexpr (!KZERO && CPLX) {
      const float4 p = __ldg(t.phS + ell);
      const float2 pr = make_float2(p.x, p.y), pm = make_float2(p.z, p.w);
      float zrh = 0.f, zrl = 0.f, zmh = 0.f, zml = 0.f;
      df_fma(zrh, zrl, pr, xr);
      df_fma(zrh, zrl, fneg2(pm), xm);
      df_fma(zmh, zml, pr, xm);
      df_fma(zmh, zml, pm, xr);
      xr = make_float2(zrh, zrl);
      xm = make_float2(zmh, zml);
    }
    df_fma(rh, rl, c, xr);
    if constexpr (CPLX) df_fma(ih, il, c, xm);
  }
  const float2 d = dsplit(__ldg(t.diag + i) - shift);
  const float2 ir = dsplit(__ldg(t.invR + chain_self_count<NOD>(n, t.L, t.bits)));
  float yrh = 0.f, yrl = 0.f, ymh = 0.f, yml = 0.f;
  if constexpr (CPLX) {
    const double2 xi = x[i];
    df_fma(yrh, yrl, d, dsplit(xi.x));
    df_fma(ymh, yml, d, dsplit(xi.y));
    df_fma(yrh, yrl, ir, make_float2(rh, rl));
    df_fma(ymh, yml, ir, make_float2(ih, il));
    return make_double2(djoin(yrh, yrl), djoin(ymh, yml));
  } else {
    df_fma(yrh, yrl, d, dsplit(x[i]));
    df_fma(yrh, yrl, ir, make_float2(rh, rl));
    return djoin(yrh, yrl);
  }
}

template <int NOD, bool PACKED, bool KZERO, class V, int SLOTS>
__global__ void __launch_bounds__(kHvThreads) k_hv_tab_df(TabArgs t, const V* __restrict__ x, V* __restrict__ y,
                                                          int pad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < t.D) y[i] = tab_row_df<NOD, PACKED, KZERO, V, SLOTS>(t, x, i, 0.0);
  else if (i == t.D && pad) y[i] = V{};
}

// split copies of a sector's phases and coefficients for tab_row_df
__global__ void k_split_tables(const double2* __restrict__ ph, int nph, float4* phS, const double* __restrict__ cf,
                               int ncf, float2* cfS) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nph) {
    const float2 r = dsplit(ph[k].x), m = dsplit(ph[k].y);
    phS[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  if (k < ncf) cfS[k] = dsplit(cf[k]);
}

template <int NOD, bool PACKED, bool KZERO, class V, int SLOTS>
__global__ void __launch_bounds__(kHvThreads) k_hv_tab(TabArgs t, const V* __restrict__ x, V* __restrict__ y,
                                                       double shift, int pad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < t.D) y[i] = tab_row<NOD, PACKED, KZERO, V, SLOTS>(t, x, i, shift);
  else if (i == t.D && pad) y[i] = V{};
}

// One thread per row: the table entries of every slot of the row, from the
// general hop (the fast paths of hv_chain_row give the same id, ell and
// count).  bcls: distance index of each bond (packed form only).
template <int NOD>
__global__ void k_tab_build(HvArgs a, int deg, int packed, const uint8_t* __restrict__ bcls, uint32_t* tab,
                            uint32_t* tabc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  int n[NOD];
  unpack<NOD>(__ldg(a.conf + i), a.bits, n);
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    const int e0 = __ldg(a.adj_off + d), e1 = __ldg(a.adj_off + d + 1);
    for (int k = 0; k < deg; ++k) {
      const size_t at = (size_t)(m * deg + k) * a.D + i;
      uint32_t ent = 0xffffffffu, code = 0;
      const int t = e0 + k;
      if (t < e1) {
        const uint32_t w = __ldg(a.adj + t);
        const int e = (int)(w & 0xffffu);
        bool edown = false;
        for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
        if (!edown) {
          int ell = 0, cnt = 1;
          const int id = chain_hop_general<NOD>(a, n, m, e, ell, cnt);
          if (id >= 0) {
            const uint32_t b = w >> 16;
            if (packed) {
              ent = (uint32_t)id | ((uint32_t)(bcls[b] * (NOD + 1) + cnt) << 27);
            } else {
              ent = (uint32_t)id;
              code = ((uint32_t)ell << 16) | (b * (NOD + 1) + (uint32_t)cnt);
            }
          }
        }
      }
      tab[at] = ent;
      if (!packed) tabc[at] = code;
    }
  }
}

TabArgs tab_args(const Model& m, const Sector& s, const HvTable& t) {
  TabArgs a{};
  a.D = s.D; a.L = m.NOS; a.bits = m.bits; a.slots = t.slots;
  a.conf = s.d_conf.get(); a.tab = t.tab.get(); a.tabc = t.tabc.get();
  a.diag = s.d_diag.get(); a.coefR = s.d_coefR.get(); a.coefR32 = s.d_coefR32.get();
  a.invR = s.d_invR.get(); a.invR32 = s.d_invR32.get();
  a.tcoef = t.coef.get(); a.tcoef32 = t.coef32.get();
  a.chainph = s.d_chainph.get(); a.chainph32 = s.d_chainph32.get();
  a.coefS = t.coefS.get(); a.phS = t.phS.get();
  return a;
}

// the complex(8) / real FP64 table product in double-float arithmetic
template <class V>
void launch_tab_df(const Model& m, const Sector& s, const V* x, V* y, int pad, cudaStream_t st) {
  const TabArgs a = tab_args(m, s, s.tab);
  const unsigned grid = (unsigned)((s.D + pad + kHvThreads - 1) / kHvThreads);
  constexpr bool REAL = sizeof(V) == sizeof(double);
  dispatch_nod(s.NOD, [&](auto c) {
    constexpr int N = decltype(c)::value;
    constexpr int S4 = (N == 4 || N == 5) ? 4 * N : 0;  // four bonds per site, unrolled
    const bool unr = S4 > 0 && a.slots == S4;
    if (s.tab.packed) {
      if (unr) k_hv_tab_df<N, true, true, V, S4><<<grid, kHvThreads, 0, st>>>(a, x, y, pad);
      else k_hv_tab_df<N, true, true, V, 0><<<grid, kHvThreads, 0, st>>>(a, x, y, pad);
    } else if (s.kzero) {
      if (unr) k_hv_tab_df<N, false, true, V, S4><<<grid, kHvThreads, 0, st>>>(a, x, y, pad);
      else k_hv_tab_df<N, false, true, V, 0><<<grid, kHvThreads, 0, st>>>(a, x, y, pad);
    } else if constexpr (!REAL) {
      if (unr) k_hv_tab_df<N, false, false, V, S4><<<grid, kHvThreads, 0, st>>>(a, x, y, pad);
      else k_hv_tab_df<N, false, false, V, 0><<<grid, kHvThreads, 0, st>>>(a, x, y, pad);
    }
  });
  check_launch("k_hv_tab_df");
}

// launch k_hv_tab for the sector's NOD, form and slot count (16 and 20 slots
// -- NOD 4 and 5 with four bonds per site -- unrolled, others at run time)
template <class V>
void launch_tab(const Model& m, const Sector& s, const V* x, V* y, double shift, int pad, cudaStream_t st) {
  const TabArgs a = tab_args(m, s, s.tab);
  const unsigned grid = (unsigned)((s.D + pad + kHvThreads - 1) / kHvThreads);
  auto go = [&](auto nod, auto pk, auto kz) {
    constexpr int N = decltype(nod)::value;
    constexpr bool P = decltype(pk)::value, Z = decltype(kz)::value;
    if (a.slots == 4 * N && (N == 4 || N == 5))
      k_hv_tab<N, P, Z, V, 4 * N><<<grid, kHvThreads, 0, st>>>(a, x, y, shift, pad);
    else
      k_hv_tab<N, P, Z, V, 0><<<grid, kHvThreads, 0, st>>>(a, x, y, shift, pad);
  };
  constexpr bool REAL = sizeof(V) == sizeof(typename Cplx<V>::R);
  dispatch_nod(s.NOD, [&](auto c) {
    using T = std::true_type;
    using F = std::false_type;
    if (s.tab.packed) go(c, T{}, T{});  // packed implies k = 0
    else if (s.kzero) go(c, F{}, T{});
    else if constexpr (!REAL) go(c, F{}, F{});  // real vectors only exist at k = 0
  });
  check_launch("k_hv_tab");
}

// Batched chain products, optionally with the Lanczos alpha partials in the
// epilogue: when part is set, block b also writes sum over its rows of
// conj(x_i) y_i (double-float, k_bdot's order) to part[seg_b0[s] + local
// block], the slot the separate dot kernel of batch_trlan.cu would fill.
template <int NOD, int NO, class V>
__device__ __forceinline__ void seg_row(const HvSeg* __restrict__ segs, const int* __restrict__ blk_seg,
                                        const int* __restrict__ blk_first, const V* __restrict__ x, V* __restrict__ y,
                                        double shift, double2* part, const int* __restrict__ seg_b0) {
  const int sg = blk_seg[blockIdx.x];
  const HvSeg& g = segs[sg];
  const int lb = blockIdx.x - blk_first[blockIdx.x];
  const int64_t i = (int64_t)lb * blockDim.x + threadIdx.x;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  if (i < g.D) {
    HvArgs a{};
    a.D = g.D; a.L = g.L; a.NOS = g.L; a.bits = g.bits;
    a.conf = g.conf; a.dir = g.dir; a.binomA = g.binomA; a.adj_off = g.adj_off; a.adj = g.adj;
    const V* xs = x + g.row0;
    V* ys = y + g.row0;
    constexpr bool F64 = sizeof(V) == sizeof(double2);
    const double sh_ = F64 ? shift : g.shift;
    const auto* cR = [&] { if constexpr (F64) return g.coefR; else return g.coefR32; }();
    const auto* iR = [&] { if constexpr (F64) return g.invR; else return g.invR32; }();
    const auto* ph = [&] { if constexpr (F64) return g.chainph; else return g.chainph32; }();
    if constexpr (NO == 4) {
      TabArgs t{};
      t.D = g.D; t.L = g.L; t.bits = g.bits; t.slots = g.tslots;
      t.conf = g.conf; t.tab = g.tab; t.tabc = g.tabc; t.diag = g.diag;
      t.coefR = g.coefR; t.coefR32 = g.coefR32; t.invR = g.invR; t.invR32 = g.invR32;
      t.tcoef = g.tcoef; t.tcoef32 = g.tcoef32; t.chainph = g.chainph; t.chainph32 = g.chainph32;
      t.coefS = g.tcoefS; t.phS = g.tphS;
      if constexpr (F64) {
        constexpr int S4 = (NOD == 4 || NOD == 5) ? 4 * NOD : 0;
        if (S4 > 0 && g.tslots == S4 && !g.tpacked && !g.kzero)  // the common k != 0 chain, unrolled
          ys[i] = tab_row_df<NOD, false, false, V, S4>(t, xs, i, sh_);
        else if (g.tpacked) ys[i] = tab_row_df<NOD, true, true>(t, xs, i, sh_);
        else if (g.kzero) ys[i] = tab_row_df<NOD, false, true>(t, xs, i, sh_);
        else ys[i] = tab_row_df<NOD, false, false>(t, xs, i, sh_);
      } else {
        if (g.tpacked) ys[i] = tab_row<NOD, true, true, V, 0>(t, xs, i, sh_);
        else if (g.kzero) ys[i] = tab_row<NOD, false, true, V, 0>(t, xs, i, sh_);
        else ys[i] = tab_row<NOD, false, false, V, 0>(t, xs, i, sh_);
      }
    } else if constexpr (NO == 0 || NO == 3) {
      if (g.kzero) hv_chain_row<NOD, true, V, NO == 3>(a, xs, ys, g.diag, cR, iR, ph, i, sh_);
      else hv_chain_row<NOD, false, V, NO == 3>(a, xs, ys, g.diag, cR, iR, ph, i, sh_);
    } else {
      a.uno = NO;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        a.uoff[k] = g.uoff[k];
        a.ubond[k] = g.ubond[k];
      }
      if (g.kzero) hv_uchain_row<NOD, NO, true, V>(a, xs, ys, g.diag, cR, iR, ph, i, sh_);
      else hv_uchain_row<NOD, NO, false, V>(a, xs, ys, g.diag, cR, iR, ph, i, sh_);
    }
    if (part) {
      const float4 u = SplitLd<V>::ld(xs[i]), v = SplitLd<V>::ld(ys[i]);
      const float2 ur = make_float2(u.x, u.y), ui = make_float2(u.z, u.w);
      const float2 vr = make_float2(v.x, v.y), vi = make_float2(v.z, v.w);
      df_fma(rh, rl, ur, vr);
      df_fma(rh, rl, ui, vi);
      df_fma(ih, il, ur, vi);
      df_fma(ih, il, fneg2(ui), vr);
    }
  }
  if (part) {  // one partial per warp, reduced in double-float: no barrier, no FP64
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float bh = __shfl_down_sync(0xffffffffu, rh, o), bl = __shfl_down_sync(0xffffffffu, rl, o);
      const float ch = __shfl_down_sync(0xffffffffu, ih, o), cl = __shfl_down_sync(0xffffffffu, il, o);
      df_add(rh, rl, bh);
      rl = __fadd_rn(rl, bl);
      df_add(ih, il, ch);
      il = __fadd_rn(il, cl);
    }
    if ((threadIdx.x & 31) == 0)
      part[(size_t)(seg_b0[sg] + lb) * kSegPartials + (threadIdx.x >> 5)] = make_double2(djoin(rh, rl), djoin(ih, il));
  }
}

template <int NOD, int NO>
__global__ void __launch_bounds__(kHvThreads) k_hv_chain64_seg(const HvSeg* __restrict__ segs,
                                                               const int* __restrict__ blk_seg,
                                                               const int* __restrict__ blk_first,
                                                               const double2* __restrict__ x,
                                                               double2* __restrict__ y, double shift, double2* part,
                                                               const int* __restrict__ seg_b0) {
  seg_row<NOD, NO, double2>(segs, blk_seg, blk_first, x, y, shift, part, seg_b0);
}

template <int NOD, int NO>
__global__ void __launch_bounds__(kHvThreads) k_hv_chain32_seg(const HvSeg* __restrict__ segs,
                                                               const int* __restrict__ blk_seg,
                                                               const int* __restrict__ blk_first,
                                                               const float2* __restrict__ x,
                                                               float2* __restrict__ y, double2* part,
                                                               const int* __restrict__ seg_b0) {
  seg_row<NOD, NO, float2>(segs, blk_seg, blk_first, x, y, 0.0, part, seg_b0);
}

// (NOD, row form) -> f(nod, no) with compile-time constants: no = 0 the
// general row, 1 or 2 the uniform row with that many bond distances (NOD
// 2..6), 3 the general row with its general-path hops deferred, 4 the
// connection table
template <class F>
void dispatch_seg(int NOD, int uni, F&& f) {
  if (uni >= 1 && uni <= 2 && NOD >= 2 && NOD <= 6) {
    auto with_no = [&](auto nod) {
      if (uni == 1) f(nod, std::integral_constant<int, 1>{});
      else f(nod, std::integral_constant<int, 2>{});
    };
    switch (NOD) {
      case 2: with_no(std::integral_constant<int, 2>{}); break;
      case 3: with_no(std::integral_constant<int, 3>{}); break;
      case 4: with_no(std::integral_constant<int, 4>{}); break;
      case 5: with_no(std::integral_constant<int, 5>{}); break;
      default: with_no(std::integral_constant<int, 6>{}); break;
    }
    return;
  }
  if (uni == 3 || uni == kSegTable) {
    dispatch_nod(NOD, [&](auto c) {
      if (uni == 3) f(c, std::integral_constant<int, 3>{});
      else f(c, std::integral_constant<int, kSegTable>{});
    });
    return;
  }
  dispatch_nod(NOD, [&](auto c) { f(c, std::integral_constant<int, 0>{}); });
}

// ------------------------------------------------------------ U(1)-only kernels
// source_only_u1/ham2vec_v3.f90:35-65: no representative search; the hop's
// row is the colex rank of the flipped configuration (inv_list), computed
// from NOD binomial-table loads.  The diagonal is precomputed as for the
// (NOD, K) sectors; coefR holds sJxy_b (R = 1).
template <int NOD, class V>
__device__ __forceinline__ void hv_u1_row(const HvArgs& a, const V* __restrict__ x, V* __restrict__ y,
                                          const typename Cplx<V>::R* __restrict__ coefR, int64_t i, double shift) {
  using R = typename Cplx<V>::R;
  int n[NOD];
  unpack<NOD>(__ldg(a.conf + i), a.bits, n);
  const V xi = x[i];
  const R di = (R)(__ldg(a.diag + i) - shift);
  R ax = 0, ay = 0;
#pragma unroll
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    const int e0 = __ldg(a.adj_off + d), e1 = __ldg(a.adj_off + d + 1);
    for (int t = e0; t < e1; ++t) {
      const uint32_t w = __ldg(a.adj + t);
      const int e = (int)(w & 0xffffu);
      bool edown = false;
#pragma unroll
      for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
      if (edown) continue;
      int o[NOD];
      move_spin<NOD>(n, m, e, o);
      const int64_t id = (int64_t)full_index<NOD>(o, a.binom, a.NOS);
      hop_acc(__ldg(coefR + (w >> 16) * (NOD + 1)), x[id], ax, ay);
    }
  }
  y[i] = row_out(di, xi, ax, ay);
}

template <int NOD>
__global__ void __launch_bounds__(kHvThreads) k_hv_u1_64(HvArgs a, const double2* __restrict__ x,
                                                         double2* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  hv_u1_row<NOD, double2>(a, x, y, a.coefR, i, 0.0);
}

template <int NOD>
__global__ void __launch_bounds__(kHvThreads) k_hv_u1_32(HvArgs a, const float2* __restrict__ x,
                                                         float2* __restrict__ y, float shift) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  hv_u1_row<NOD, float2>(a, x, y, a.coefR32, i, (double)shift);
}

template <int NOD>
__global__ void __launch_bounds__(kHvThreads) k_hv_u1_64r(HvArgs a, const double* __restrict__ x,
                                                          double* __restrict__ y, int pad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.D) hv_u1_row<NOD, double>(a, x, y, a.coefR, i, 0.0);
  else if (i == a.D && pad) y[i] = 0.0;
}

template <int NOD>
__global__ void __launch_bounds__(kHvThreads) k_hv_u1_32r(HvArgs a, const float* __restrict__ x,
                                                          float* __restrict__ y, float shift, int pad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.D) hv_u1_row<NOD, float>(a, x, y, a.coefR32, i, (double)shift);
  else if (i == a.D && pad) y[i] = 0.f;
}

// ------------------------------------------------------------ general lattice helpers
template <int NOD>
__device__ __forceinline__ uint64_t translate_pack(const int (&n)[NOD], int ti, int tj, int tk,
                                                   const HvArgs& a) {
  int t[NOD];
#pragma unroll
  for (int e = 0; e < NOD; ++e) {
    const short4 c = reinterpret_cast<const short4*>(a.xyz)[n[e]];
    int xx = c.x + ti; xx -= (xx >= a.LX) ? a.LX : 0;
    int yy = c.y + tj; yy -= (yy >= a.LY) ? a.LY : 0;
    int zz = c.z + tk; zz -= (zz >= a.LZ) ? a.LZ : 0;
    t[e] = 1 + xx + a.LX * (yy + a.LY * zz);
  }
#pragma unroll
  for (int i = 1; i < NOD; ++i) {
#pragma unroll
    for (int j = i; j > 0; --j) {
      const int lo = min(t[j - 1], t[j]), hi = max(t[j - 1], t[j]);
      t[j - 1] = lo; t[j] = hi;
    }
  }
  return pack<NOD>(t, a.bits);
}

__device__ __forceinline__ void tau_to_ijk(int tau, const HvArgs& a, int& i, int& j, int& k) {
  i = tau % a.LX + 1;
  const int r = tau / a.LX;
  j = r % a.LY + 1;
  k = r / a.LY + 1;
}

// representative_SQ for a general lattice by one thread (used by the connection table).
template <int NOD>
__device__ __forceinline__ uint64_t general_rep_serial(const int (&o)[NOD], const HvArgs& a, int& tau_best) {
  uint64_t best = ~0ull;
  tau_best = 0x7fffffff;
  int tau = 0;
  for (int k = 1; k <= a.LZ; ++k)
    for (int j = 1; j <= a.LY; ++j)
      for (int i = 1; i <= a.LX; ++i, ++tau) {
        const uint64_t w = translate_pack<NOD>(o, i % a.LX, j % a.LY, k % a.LZ, a);
        if (w < best) { best = w; tau_best = tau; }
      }
  return best;
}

// ------------------------------------------------------------ general lattice, complex(8)
// WARP: one warp per row, lanes over the translations, shuffle-min; else one
// thread per row scanning all translations.  Both visit hops in the same
// order and break ties the same way (smallest loop index), so they produce
// identical results; the autotuner below picks the faster per sector.
template <int NOD, bool WARP>
__global__ void __launch_bounds__(kHvThreads) k_hv_general64(HvArgs a, const double2* __restrict__ x,
                                                             double2* __restrict__ y) {
  const int64_t i = WARP ? ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5
                         : (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = WARP ? (threadIdx.x & 31) : 0;
  constexpr int kStep = WARP ? 32 : 1;
  if (i >= a.D) return;
  int n[NOD];
  unpack<NOD>(__ldg(a.conf + i), a.bits, n);
  const double2 xi = x[i];
  const double ri = __ldg(a.list_r + i);
  double sdown = 0.0, both = 0.0;
  double2 acc = make_double2(0.0, 0.0);
  const size_t ex1 = (size_t)a.LX + 1, ex2 = ex1 * ((size_t)a.LY + 1);
#pragma unroll
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    sdown += __ldg(a.Sz_site + d);
    const int e0 = __ldg(a.adj_off + d), e1 = __ldg(a.adj_off + d + 1);
    for (int t = e0; t < e1; ++t) {
      const uint32_t w = __ldg(a.adj + t);
      const int e = (int)(w & 0xffffu), b = (int)(w >> 16);
      bool edown = false;
#pragma unroll
      for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
      if (edown) { both += __ldg(a.sJz + b); continue; }
      int o[NOD];
      move_spin<NOD>(n, m, e, o);
      uint64_t best = ~0ull;
      int bt = 0x7fffffff;
      for (int tau = lane; tau < a.NT; tau += kStep) {
        int ti, tj, tk;
        tau_to_ijk(tau, a, ti, tj, tk);
        const uint64_t v = translate_pack<NOD>(o, ti % a.LX, tj % a.LY, tk % a.LZ, a);
        if (v < best) { best = v; bt = tau; }
      }
      if constexpr (WARP) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, off);
          const int ot = __shfl_xor_sync(0xffffffffu, bt, off);
          if (ob < best || (ob == best && ot < bt)) { best = ob; bt = ot; }
        }
      }
      int rep[NOD];
      unpack<NOD>(best, a.bits, rep);
      const int64_t id = dir_lookup(a.dir, full_index<NOD>(rep, a.binom, a.NOS));
      if (id < 0) continue;
      size_t eidx = 0;
      if (best != pack<NOD>(o, a.bits)) {
        int ti, tj, tk;
        tau_to_ijk(bt, a, ti, tj, tk);
        eidx = (size_t)ti + ex1 * (size_t)tj + ex2 * (size_t)tk;
      }
      const double c = __ldg(a.sJxy + b) * __ldg(a.list_r + id) / ri;
      const double2 ex = __ldg(a.explist + eidx);
      const double2 ce = make_double2(c * ex.x, c * ex.y);
      const double2 tv = cmul(ce, x[id]);
      acc.x += tv.x;
      acc.y += tv.y;
    }
  }
  if (lane == 0) {  // thread-per-row: every thread
    const double diag = fma(-2.0, sdown - both, a.Sz_all);
    y[i] = make_double2(fma(diag, xi.x, acc.x), fma(diag, xi.y, acc.y));
  }
}

template <int NOD, bool WARP>
__global__ void __launch_bounds__(kHvThreads) k_hv_general32(HvArgs a, const float2* __restrict__ x,
                                                             float2* __restrict__ y, float shift) {
  const int64_t i = WARP ? ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5
                         : (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = WARP ? (threadIdx.x & 31) : 0;
  constexpr int kStep = WARP ? 32 : 1;
  if (i >= a.D) return;
  int n[NOD];
  unpack<NOD>(__ldg(a.conf + i), a.bits, n);
  const float2 xi = x[i];
  const float ri = __ldg(a.list_r32 + i);
  float sdown = 0.f, both = 0.f;
  float2 acc = make_float2(0.f, 0.f);
  const size_t ex1 = (size_t)a.LX + 1, ex2 = ex1 * ((size_t)a.LY + 1);
#pragma unroll
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    sdown += (float)__ldg(a.Sz_site + d);
    const int e0 = __ldg(a.adj_off + d), e1 = __ldg(a.adj_off + d + 1);
    for (int t = e0; t < e1; ++t) {
      const uint32_t w = __ldg(a.adj + t);
      const int e = (int)(w & 0xffffu), b = (int)(w >> 16);
      bool edown = false;
#pragma unroll
      for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
      if (edown) { both += (float)__ldg(a.sJz + b); continue; }
      int o[NOD];
      move_spin<NOD>(n, m, e, o);
      uint64_t best = ~0ull;
      int bt = 0x7fffffff;
      for (int tau = lane; tau < a.NT; tau += kStep) {
        int ti, tj, tk;
        tau_to_ijk(tau, a, ti, tj, tk);
        const uint64_t v = translate_pack<NOD>(o, ti % a.LX, tj % a.LY, tk % a.LZ, a);
        if (v < best) { best = v; bt = tau; }
      }
      if constexpr (WARP) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, off);
          const int ot = __shfl_xor_sync(0xffffffffu, bt, off);
          if (ob < best || (ob == best && ot < bt)) { best = ob; bt = ot; }
        }
      }
      int rep[NOD];
      unpack<NOD>(best, a.bits, rep);
      const int64_t id = dir_lookup(a.dir, full_index<NOD>(rep, a.binom, a.NOS));
      if (id < 0) continue;
      size_t eidx = 0;
      if (best != pack<NOD>(o, a.bits)) {
        int ti, tj, tk;
        tau_to_ijk(bt, a, ti, tj, tk);
        eidx = (size_t)ti + ex1 * (size_t)tj + ex2 * (size_t)tk;
      }
      const float c = (float)__ldg(a.sJxy + b) * __ldg(a.list_r32 + id) / ri;
      const double2 ex = __ldg(a.explist + eidx);
      const float2 tv = cmulf(make_float2(c * (float)ex.x, c * (float)ex.y), x[id]);
      acc.x += tv.x;
      acc.y += tv.y;
    }
  }
  if (lane == 0) {
    const float diag = (float)((a.Sz_all - (double)shift) - 2.0 * (double)(sdown - both));
    y[i] = make_float2(fmaf(diag, xi.x, acc.x), fmaf(diag, xi.y, acc.y));
  }
}

// ------------------------------------------------------------ connection table
constexpr int kMaxRowEntries = 64;

// kind: 0 = general lattice, 1 = chain, 2 = U(1) only
template <int NOD>
__global__ void __launch_bounds__(128) k_conn(HvArgs a, int kind, int64_t row0, int64_t row1,
                                              int64_t* counts, const int64_t* offs, int64_t* orow,
                                              int64_t* ocol, int* oell, int* obond, int* overflow) {
  const int64_t i = row0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= row1) return;
  int n[NOD];
  unpack<NOD>(__ldg(a.conf + i), a.bits, n);
  int eb[kMaxRowEntries], ee[kMaxRowEntries];
  int64_t ec[kMaxRowEntries];
  int cnt = 0;
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    const int e0 = a.adj_off[d], e1 = a.adj_off[d + 1];
    for (int t = e0; t < e1; ++t) {
      const uint32_t w = a.adj[t];
      const int e = (int)(w & 0xffffu), b = (int)(w >> 16);
      bool edown = false;
      for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
      if (edown) continue;
      int o[NOD];
      move_spin<NOD>(n, m, e, o);
      int64_t id;
      int ellcode;  // chain: translation i; general: tau+1 (0 = identity / minimal)
      if (kind == 2) {
        id = (int64_t)full_index<NOD>(o, a.binom, a.NOS);
        ellcode = 0;
      } else if (kind == 1) {
        int p[NOD], ell;
        chain_rep<NOD>(o, a.L, a.bits, p, ell);
        id = dir_lookup(a.dir, anchored_index<NOD>(p, a.binomA, a.L));
        ellcode = ell;
      } else {
        int bt;
        const uint64_t best = general_rep_serial<NOD>(o, a, bt);
        int rep[NOD];
        unpack<NOD>(best, a.bits, rep);
        id = dir_lookup(a.dir, full_index<NOD>(rep, a.binom, a.NOS));
        ellcode = (best == pack<NOD>(o, a.bits)) ? 0 : bt + 1;
      }
      if (id < 0) continue;
      if (cnt < kMaxRowEntries) { eb[cnt] = b; ee[cnt] = ellcode; ec[cnt] = id; }
      ++cnt;
    }
  }
  if (cnt > kMaxRowEntries) { atomicExch(overflow, 1); cnt = kMaxRowEntries; }
  if (counts) { counts[i - row0] = cnt; return; }
  // order by bond number (ham2vec_v3.f90:56 loops bonds in list order)
  for (int u = 1; u < cnt; ++u) {
    const int b = eb[u], e = ee[u];
    const int64_t c = ec[u];
    int v = u - 1;
    while (v >= 0 && eb[v] > b) { eb[v + 1] = eb[v]; ee[v + 1] = ee[v]; ec[v + 1] = ec[v]; --v; }
    eb[v + 1] = b; ee[v + 1] = e; ec[v + 1] = c;
  }
  int64_t w = offs[i - row0];
  for (int u = 0; u < cnt; ++u, ++w) {
    orow[w] = i + 1;
    ocol[w] = ec[u] + 1;
    obond[w] = eb[u] + 1;
    int ti = 0, tj = 0, tk = 0;
    if (kind == 1) {
      if (ee[u] != 0) { ti = ee[u]; tj = 1; tk = 1; }
    } else if (ee[u] != 0) {
      tau_to_ijk(ee[u] - 1, a, ti, tj, tk);
    }
    oell[3 * w] = ti; oell[3 * w + 1] = tj; oell[3 * w + 2] = tk;
  }
}

// ------------------------------------------------------------ dense H (ALG = 3)
// make_full_hamiltonian (ham2vec_v3.f90:5-35; source_only_u1/ham2vec_v3.f90:5-33):
// one thread per row i walks all bonds in list order and accumulates into
// H(i, i) and H(i, id) in place, so every entry receives its terms in the
// reference's order.  The thread owns row i, so the read-modify-writes do
// not race.  kind: 0 = general lattice, 1 = chain, 2 = U(1) only.
template <int NOD>
__global__ void __launch_bounds__(128) k_dense(HvArgs a, int kind, const int2* __restrict__ p12, int nbonds,
                                               double2* H, int64_t ld) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  int n[NOD];
  unpack<NOD>(a.conf[i], a.bits, n);
  const size_t ex1 = (size_t)a.LX + 1, ex2 = ex1 * ((size_t)a.LY + 1);
  double2* hii = H + i + i * ld;
  for (int j = 0; j < nbonds; ++j) {
    const int2 p = p12[j];
    int m1 = -1, m2 = -1;
#pragma unroll
    for (int u = 0; u < NOD; ++u) {
      if (n[u] == p.x) m1 = u;
      if (n[u] == p.y) m2 = u;
    }
    const bool f1 = m1 >= 0, f2 = m2 >= 0;
    if (f1 == f2) {
      hii->x = hii->x + a.sJz[j];
      continue;
    }
    hii->x = hii->x - a.sJz[j];
    // j_flip_ni: the down end moves to the up end
    int o[NOD];
    if (f1) move_spin<NOD>(n, m1, p.y, o);
    else move_spin<NOD>(n, m2, p.x, o);
    int64_t id;
    double2 e = make_double2(1.0, 0.0);
    if (kind == 2) {
      id = (int64_t)full_index<NOD>(o, a.binom, a.NOS);
    } else if (kind == 1) {
      int q[NOD], ell;
      chain_rep<NOD>(o, a.L, a.bits, q, ell);
      id = dir_lookup(a.dir, anchored_index<NOD>(q, a.binomA, a.L));
      e = a.chainph[ell];
    } else {
      int bt;
      const uint64_t best = general_rep_serial<NOD>(o, a, bt);
      int rep[NOD];
      unpack<NOD>(best, a.bits, rep);
      id = dir_lookup(a.dir, full_index<NOD>(rep, a.binom, a.NOS));
      size_t eidx = 0;
      if (best != pack<NOD>(o, a.bits)) {
        int ti, tj, tk;
        tau_to_ijk(bt, a, ti, tj, tk);
        eidx = (size_t)ti + ex1 * (size_t)tj + ex2 * (size_t)tk;
      }
      e = a.explist[eidx];
    }
    if (id < 0) continue;
    // sJint(j,2) * list_r(id) / list_r(i) * explist(ell), left to right
    const double c = a.sJxy[j] * a.list_r[id] / a.list_r[i];
    double2* hij = H + i + id * ld;
    hij->x = hij->x + c * e.x;
    hij->y = hij->y + c * e.y;
  }
}

HvArgs make_args(const Model& m, const Sector& s) {
  HvArgs a{};
  a.D = s.D; a.L = m.NOS; a.NOS = m.NOS; a.bits = m.bits;
  a.LX = m.LX; a.LY = m.LY; a.LZ = m.LZ; a.NT = m.LX * m.LY * m.LZ;
  a.conf = s.d_conf.get(); a.list_r = s.d_list_r.get(); a.list_r32 = s.d_list_r32.get();
  a.dir = s.d_dir.get(); a.binomA = s.d_binomA.get(); a.binom = s.d_binom.get();
  a.adj_off = m.d_adj_off.get(); a.adj = m.d_adj.get();
  a.sJxy = m.d_sJxy.get(); a.sJz = m.d_sJz.get(); a.Sz_site = m.d_Sz_site.get(); a.Sz_all = m.Sz_all;
  a.chainph = s.d_chainph.get(); a.chainph32 = s.d_chainph32.get(); a.explist = s.d_explist.get();
  a.xyz = m.d_site_xyz.get();
  a.diag = s.d_diag.get(); a.diag32 = s.d_diag32.get();
  a.coefR = s.d_coefR.get(); a.coefR32 = s.d_coefR32.get();
  a.invR = s.d_invR.get(); a.invR32 = s.d_invR32.get();
  a.uno = m.uni_no;
  for (int k = 0; k < 2; ++k) {
    a.uoff[k] = k < m.uni_no ? m.uni_off[k] : 0;
    a.ubond[k] = k < m.uni_no ? m.uni_bond[k] : 0;
  }
  return a;
}

// Diagonal of H per row: sum_b sJz_b * (+1 parallel / -1 antiparallel)
//   = Sz_all - 2 * (sum_{d down} Sz_site[d] - sum over both-down bond ends of sJz_b)
// (the `f1 .neqv. f2` branches of ham2vec_v3.f90:57-67).
template <int NOD>
__global__ void k_diag(HvArgs a, double* diag, float* diag32) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.D) return;
  int n[NOD];
  unpack<NOD>(a.conf[i], a.bits, n);
  double sdown = 0.0, both = 0.0;
  for (int m = 0; m < NOD; ++m) {
    const int d = n[m];
    sdown += a.Sz_site[d];
    for (int t = a.adj_off[d]; t < a.adj_off[d + 1]; ++t) {
      const uint32_t w = a.adj[t];
      const int e = (int)(w & 0xffffu);
      bool edown = false;
      for (int j = 0; j < NOD; ++j) edown |= (n[j] == e);
      if (edown) both += a.sJz[w >> 16];
    }
  }
  const double dg = a.Sz_all - 2.0 * (sdown - both);
  diag[i] = dg;
  diag32[i] = (float)dg;
}

}  // namespace

HvSeg make_seg(const Model& m, const Sector& s, int64_t row0) {
  QS3G_REQUIRE(s.anchored && !s.u1, QS3G_ENOTSUP, "batched H*v serves chain sectors");
  HvSeg g{};
  g.D = s.D; g.row0 = row0; g.L = m.NOS; g.bits = m.bits; g.kzero = s.kzero ? 1 : 0;
  g.conf = s.d_conf.get(); g.dir = s.d_dir.get(); g.binomA = s.d_binomA.get();
  g.adj_off = m.d_adj_off.get(); g.adj = m.d_adj.get();
  g.diag = s.d_diag.get(); g.coefR = s.d_coefR.get(); g.invR = s.d_invR.get(); g.chainph = s.d_chainph.get();
  g.diag32 = s.d_diag32.get(); g.coefR32 = s.d_coefR32.get(); g.invR32 = s.d_invR32.get();
  g.chainph32 = s.d_chainph32.get();
  g.shift = 0.0;
  g.uno = m.uni_no;
  for (int k = 0; k < 2; ++k) {
    g.uoff[k] = k < m.uni_no ? m.uni_off[k] : 0;
    g.ubond[k] = k < m.uni_no ? m.uni_bond[k] : 0;
  }
  set_seg_table(g, s.tab);
  return g;
}

void set_seg_table(HvSeg& g, const HvTable& t) {
  g.tab = t.built() ? t.tab.get() : nullptr;
  g.tabc = t.built() ? t.tabc.get() : nullptr;
  g.tcoef = t.coef.get();
  g.tcoef32 = t.coef32.get();
  g.tcoefS = t.coefS.get();
  g.tphS = t.phS.get();
  g.tslots = t.slots;
  g.tpacked = t.packed ? 1 : 0;
}

bool seg_uniform_ok(int NOD, int uni) { return uni >= 1 && uni <= 2 && NOD >= 2 && NOD <= 6; }

void hv32_seg(int NOD, const HvSeg* d_segs, const int* d_blk_seg, const int* d_blk_first, int nblk,
              const float2* x, float2* y, cudaStream_t st, double2* part, const int* seg_b0, int uni) {
  if (nblk == 0) return;
  dispatch_seg(NOD, uni, [&](auto c, auto no) {
    k_hv_chain32_seg<decltype(c)::value, decltype(no)::value>
        <<<nblk, kHvThreads, 0, st>>>(d_segs, d_blk_seg, d_blk_first, x, y, part, seg_b0);
  });
  check_launch("k_hv_chain32_seg");
}

void hv64_seg(int NOD, const HvSeg* d_segs, const int* d_blk_seg, const int* d_blk_first, int nblk,
              const double2* x, double2* y, double shift, cudaStream_t st, double2* part, const int* seg_b0,
              int uni) {
  if (nblk == 0) return;
  dispatch_seg(NOD, uni, [&](auto c, auto no) {
    k_hv_chain64_seg<decltype(c)::value, decltype(no)::value>
        <<<nblk, kHvThreads, 0, st>>>(d_segs, d_blk_seg, d_blk_first, x, y, shift, part, seg_b0);
  });
  check_launch("k_hv_chain64_seg");
}

void dense_hamiltonian(const Model& m, const Sector& s, double2* H, int64_t ld, cudaStream_t st) {
  QS3G_REQUIRE(ld >= s.D, QS3G_EINVAL, "leading dimension below D");
  if (s.D == 0) return;
  QS3G_CHECK_CUDA(cudaMemsetAsync(H, 0, (size_t)ld * (size_t)s.D * sizeof(double2), st));
  const HvArgs a = make_args(m, s);
  const int kind = s.u1 ? 2 : (s.anchored ? 1 : 0);
  const unsigned grid = (unsigned)((s.D + 127) / 128);
  dispatch_nod(s.NOD, [&](auto c) {
    k_dense<decltype(c)::value><<<grid, 128, 0, st>>>(a, kind, m.d_p12.get(), m.NOxxz, H, ld);
  });
  check_launch("k_dense");
}

void compute_diag(const Model& m, Sector& s, cudaStream_t st) {
  s.d_diag.alloc(std::max<int64_t>(1, s.D));
  s.d_diag32.alloc(std::max<int64_t>(1, s.D));
  if (s.D == 0) return;
  HvArgs a = make_args(m, s);
  dispatch_nod(s.NOD, [&](auto c) {
    k_diag<decltype(c)::value><<<(unsigned)((s.D + 255) / 256), 256, 0, st>>>(a, s.d_diag.get(), s.d_diag32.get());
  });
  check_launch("k_diag");
}

static bool table_layout(const Model& m, const Sector& s, int& deg, bool& packed) {
  if (!s.anchored || s.u1 || s.D <= 0 || !m.chain) return false;
  deg = 0;
  for (int d = 1; d <= m.NOS; ++d) deg = std::max(deg, m.adj_off[d + 1] - m.adj_off[d]);
  if (deg == 0 || s.NOD * deg > 64) return false;
  packed = s.kzero && m.uni_no >= 1 && s.D < (int64_t(1) << 27) && m.uni_no * (s.NOD + 1) <= 31;
  if (!packed && (s.D >= (int64_t(1) << 31) || (int64_t)m.NOxxz * (s.NOD + 1) >= 65536 || m.NOS >= 65536))
    return false;
  return true;
}

size_t hv_table_bytes(const Model& m, const Sector& s) {
  int deg;
  bool packed;
  if (!table_layout(m, s, deg, packed)) return 0;
  return (size_t)s.NOD * deg * (size_t)s.D * sizeof(uint32_t) * (packed ? 1 : 2);
}

bool build_hv_table(const Model& m, const Sector& s, HvTable& t, size_t keep, cudaStream_t st) {
  t.release();
  int deg;
  bool packed;
  QS3G_REQUIRE(table_layout(m, s, deg, packed), QS3G_ENOTSUP,
               "connection table: chain (NOD, K) sectors with indexable sizes only");
  const size_t bytes = hv_table_bytes(m, s);
  size_t free_b = 0, total_b = 0;
  QS3G_CHECK_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (bytes + keep > free_b) return false;
  const size_t n = (size_t)s.NOD * deg * (size_t)s.D;
  t.tab.alloc(n);
  if (!packed) t.tabc.alloc(n);
  DevBuf<uint8_t> bcls(std::max(1, m.NOxxz));
  const int nc = s.NOD + 1;
  t.coef.alloc(32);
  t.coef32.alloc(32);
  QS3G_CHECK_CUDA(cudaMemsetAsync(t.coef.get(), 0, 32 * sizeof(double), st));
  QS3G_CHECK_CUDA(cudaMemsetAsync(t.coef32.get(), 0, 32 * sizeof(float), st));
  if (packed) {
    std::vector<uint8_t> hb(m.NOxxz, 0);
    for (int b = 0; b < m.NOxxz; ++b) {
      const int o = m.p2[b] - m.p1[b];
      const int dk = std::min(o, m.NOS - o);
      hb[b] = (m.uni_no > 1 && dk == m.uni_off[1]) ? 1 : 0;
    }
    QS3G_CHECK_CUDA(cudaMemcpyAsync(bcls.get(), hb.data(), hb.size(), cudaMemcpyHostToDevice, st));
    // class k * (NOD + 1) + c takes the coefficient of the distance's first bond (all equal)
    for (int k = 0; k < m.uni_no; ++k) {
      QS3G_CHECK_CUDA(cudaMemcpyAsync(t.coef.get() + k * nc, s.d_coefR.get() + (size_t)m.uni_bond[k] * nc,
                                      nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
      QS3G_CHECK_CUDA(cudaMemcpyAsync(t.coef32.get() + k * nc, s.d_coefR32.get() + (size_t)m.uni_bond[k] * nc,
                                      nc * sizeof(float), cudaMemcpyDeviceToDevice, st));
    }
  }
  const HvArgs a = make_args(m, s);
  const unsigned grid = (unsigned)((s.D + 127) / 128);
  dispatch_nod(s.NOD, [&](auto c) {
    k_tab_build<decltype(c)::value><<<grid, 128, 0, st>>>(a, deg, packed ? 1 : 0, bcls.get(), t.tab.get(),
                                                          t.tabc.get());
  });
  check_launch("k_tab_build");
  const int nph = (int)s.d_chainph.n;
  const int ncf = packed ? 32 : (int)s.d_coefR.n;
  t.phS.alloc(std::max(1, nph));
  t.coefS.alloc(std::max(1, ncf));
  k_split_tables<<<(unsigned)((std::max(nph, ncf) + 255) / 256), 256, 0, st>>>(
      s.d_chainph.get(), nph, t.phS.get(), packed ? t.coef.get() : s.d_coefR.get(), ncf, t.coefS.get());
  check_launch("k_split_tables");
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));  // bcls goes out of scope
  t.slots = s.NOD * deg;
  t.deg = deg;
  t.packed = packed;
  return true;
}

void hv64(const Model& m, const Sector& s, const double2* x, double2* y, cudaStream_t st) {
  if (s.D == 0) return;
  if (s.tab.built()) {
    launch_tab<double2>(m, s, x, y, 0.0, 0, st);
    return;
  }
  const HvArgs a = make_args(m, s);
  if (s.u1) {
    const unsigned grid = (unsigned)((s.D + kHvThreads - 1) / kHvThreads);
    dispatch_nod(s.NOD, [&](auto c) { k_hv_u1_64<decltype(c)::value><<<grid, kHvThreads, 0, st>>>(a, x, y); });
    check_launch("k_hv_u1_64");
  } else if (s.anchored) {
    const unsigned grid = (unsigned)((s.D + kHvThreads - 1) / kHvThreads);
    // complex(8): the FP64 pipe (two FMAs per hop) bounds both row forms, and
    // the general one keeps more warps resident (measured 3.04 against 3.12 ms
    // at L = 1000), so the uniform form serves the other three products only
    dispatch_nod(s.NOD, [&](auto c) {
      if (s.kzero) k_hv_chain64<decltype(c)::value, true><<<grid, kHvThreads, 0, st>>>(a, x, y);
      else k_hv_chain64<decltype(c)::value, false><<<grid, kHvThreads, 0, st>>>(a, x, y);
    });
    check_launch("k_hv_chain64");
  } else {
    hv64_general(m, s, x, y, st);
  }
}

bool hv64_df(const Model& m, const Sector& s, const double2* x, double2* y, cudaStream_t st) {
  if (!s.tab.built() || s.D == 0) return false;
  launch_tab_df<double2>(m, s, x, y, 0, st);
  return true;
}

bool hv64r_df(const Model& m, const Sector& s, const double* x, double* y, cudaStream_t st, bool pad) {
  if (!s.tab.built() || s.D == 0 || !s.kzero) return false;
  launch_tab_df<double>(m, s, x, y, (pad && (s.D & 1)) ? 1 : 0, st);
  return true;
}

bool real_sector(const Sector& s) { return s.u1 || (s.anchored && s.kzero); }

// Real vectors of length D; with pad, D odd, also y[D] = 0.
void hv64r(const Model& m, const Sector& s, const double* x, double* y, cudaStream_t st, bool pad) {
  QS3G_REQUIRE(real_sector(s), QS3G_ENOTSUP, "real H*v needs a k = 0 chain sector or a U(1) sector");
  if (s.D == 0) return;
  const HvArgs a = make_args(m, s);
  const int pr = (pad && (s.D & 1)) ? 1 : 0;
  if (s.tab.built()) {
    launch_tab<double>(m, s, x, y, 0.0, pr, st);
    return;
  }
  const unsigned grid = (unsigned)((s.D + pr + kHvThreads - 1) / kHvThreads);
  // the general chain row, as the complex(8) product uses: the real product
  // stays the real part of the complex one bit for bit
  dispatch_nod(s.NOD, [&](auto c) {
    if (s.u1) k_hv_u1_64r<decltype(c)::value><<<grid, kHvThreads, 0, st>>>(a, x, y, pr);
    else k_hv_chain64r<decltype(c)::value><<<grid, kHvThreads, 0, st>>>(a, x, y, pr);
  });
  check_launch("k_hv_real64");
}

void hv32r(const Model& m, const Sector& s, const float* x, float* y, cudaStream_t st, float shift, bool pad) {
  QS3G_REQUIRE(real_sector(s), QS3G_ENOTSUP, "real H*v needs a k = 0 chain sector or a U(1) sector");
  if (s.D == 0) return;
  const HvArgs a = make_args(m, s);
  const int pr = (pad && (s.D & 1)) ? 1 : 0;
  if (s.tab.built()) {
    launch_tab<float>(m, s, x, y, (double)shift, pr, st);
    return;
  }
  const unsigned grid = (unsigned)((s.D + pr + kHvThreads - 1) / kHvThreads);
  const bool uni = !s.u1 && dispatch_uniform(m, s, [&](auto c, auto no) {
    k_hv_uchain32r<decltype(c)::value, decltype(no)::value><<<grid, kHvThreads, 0, st>>>(a, x, y, shift, pr);
  });
  if (!uni) {
    dispatch_nod(s.NOD, [&](auto c) {
      if (s.u1) k_hv_u1_32r<decltype(c)::value><<<grid, kHvThreads, 0, st>>>(a, x, y, shift, pr);
      else k_hv_chain32r<decltype(c)::value><<<grid, kHvThreads, 0, st>>>(a, x, y, shift, pr);
    });
  }
  check_launch("k_hv_real32");
}

// Schedule of the general-lattice H*v: 1 = warp per row, 2 = thread per row.
// With the sector's hv_schedule at 0 (auto), the first product of the sector
// runs both (they give identical results), times them with CUDA events and
// keeps the faster for every later product of that precision.
template <class F1, class F2>
static int autotune(int& slot, F1&& warp, F2&& row, cudaStream_t st) {
  if (slot != 0) {
    if (slot == 1) warp(); else row();
    return slot;
  }
  cudaEvent_t e0, e1, e2;
  QS3G_CHECK_CUDA(cudaEventCreate(&e0));
  QS3G_CHECK_CUDA(cudaEventCreate(&e1));
  QS3G_CHECK_CUDA(cudaEventCreate(&e2));
  QS3G_CHECK_CUDA(cudaEventRecord(e0, st));
  row();
  QS3G_CHECK_CUDA(cudaEventRecord(e1, st));
  warp();
  QS3G_CHECK_CUDA(cudaEventRecord(e2, st));
  QS3G_CHECK_CUDA(cudaEventSynchronize(e2));
  float t_row = 0.f, t_warp = 0.f;
  QS3G_CHECK_CUDA(cudaEventElapsedTime(&t_row, e0, e1));
  QS3G_CHECK_CUDA(cudaEventElapsedTime(&t_warp, e1, e2));
  cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
  slot = (t_row < t_warp) ? 2 : 1;
  return slot;
}

void hv64_general(const Model& m, const Sector& s, const double2* x, double2* y, cudaStream_t st) {
  if (s.D == 0) return;
  const HvArgs a = make_args(m, s);
  const unsigned gw = (unsigned)((s.D * 32 + kHvThreads - 1) / kHvThreads);
  const unsigned gr = (unsigned)((s.D + kHvThreads - 1) / kHvThreads);
  auto warp = [&]() {
    dispatch_nod(s.NOD, [&](auto c) { k_hv_general64<decltype(c)::value, true><<<gw, kHvThreads, 0, st>>>(a, x, y); });
    check_launch("k_hv_general64");
  };
  auto row = [&]() {
    dispatch_nod(s.NOD, [&](auto c) { k_hv_general64<decltype(c)::value, false><<<gr, kHvThreads, 0, st>>>(a, x, y); });
    check_launch("k_hv_general64");
  };
  autotune(s.hv_schedule64, warp, row, st);
}

void hv32(const Model& m, const Sector& s, const float2* x, float2* y, cudaStream_t st, float shift) {
  if (s.D == 0) return;
  if (s.tab.built()) {
    launch_tab<float2>(m, s, x, y, (double)shift, 0, st);
    return;
  }
  const HvArgs a = make_args(m, s);
  if (s.u1) {
    const unsigned grid = (unsigned)((s.D + kHvThreads - 1) / kHvThreads);
    dispatch_nod(s.NOD, [&](auto c) {
      k_hv_u1_32<decltype(c)::value><<<grid, kHvThreads, 0, st>>>(a, x, y, shift);
    });
    check_launch("k_hv_u1_32");
  } else if (s.anchored) {
    const unsigned grid = (unsigned)((s.D + kHvThreads - 1) / kHvThreads);
    const bool uni = dispatch_uniform(m, s, [&](auto c, auto no) {
      constexpr int N = decltype(c)::value, O = decltype(no)::value;
      if (s.kzero) k_hv_uchain32<N, O, true><<<grid, kHvThreads, 0, st>>>(a, x, y, shift);
      else k_hv_uchain32<N, O, false><<<grid, kHvThreads, 0, st>>>(a, x, y, shift);
    });
    if (!uni) {
      dispatch_nod(s.NOD, [&](auto c) {
        if (s.kzero) k_hv_chain32<decltype(c)::value, true><<<grid, kHvThreads, 0, st>>>(a, x, y, shift);
        else k_hv_chain32<decltype(c)::value, false><<<grid, kHvThreads, 0, st>>>(a, x, y, shift);
      });
    }
    check_launch("k_hv_chain32");
  } else {
    const unsigned gw = (unsigned)((s.D * 32 + kHvThreads - 1) / kHvThreads);
    const unsigned gr = (unsigned)((s.D + kHvThreads - 1) / kHvThreads);
    auto warp = [&]() {
      dispatch_nod(s.NOD, [&](auto c) {
        k_hv_general32<decltype(c)::value, true><<<gw, kHvThreads, 0, st>>>(a, x, y, shift);
      });
      check_launch("k_hv_general32");
    };
    auto row = [&]() {
      dispatch_nod(s.NOD, [&](auto c) {
        k_hv_general32<decltype(c)::value, false><<<gr, kHvThreads, 0, st>>>(a, x, y, shift);
      });
      check_launch("k_hv_general32");
    };
    autotune(s.hv_schedule32, warp, row, st);
  }
}

int64_t connection_table_rows(const Model& m, const Sector& s, int64_t row0, int64_t row1, int64_t* row,
                              int64_t* col, int* ell, int* bond, int64_t cap, cudaStream_t st) {
  QS3G_REQUIRE(row0 >= 0 && row1 <= s.D && row0 <= row1, QS3G_EINVAL, "bad row range");
  const int64_t nr = row1 - row0;
  if (nr == 0) return 0;
  const HvArgs a = make_args(m, s);
  const int kind = s.u1 ? 2 : (s.anchored ? 1 : 0);
  DevBuf<int64_t> d_cnt(nr);
  DevBuf<int> d_ovf(1);
  QS3G_CHECK_CUDA(cudaMemsetAsync(d_ovf.get(), 0, sizeof(int), st));
  const unsigned grid = (unsigned)((nr + 127) / 128);
  dispatch_nod(s.NOD, [&](auto c) {
    k_conn<decltype(c)::value><<<grid, 128, 0, st>>>(a, kind, row0, row1, d_cnt.get(), nullptr,
                                                    nullptr, nullptr, nullptr, nullptr, d_ovf.get());
  });
  check_launch("k_conn(count)");
  std::vector<int64_t> h(nr);
  int ovf = 0;
  QS3G_CHECK_CUDA(cudaMemcpyAsync(h.data(), d_cnt.get(), nr * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(&ovf, d_ovf.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  QS3G_REQUIRE(!ovf, QS3G_ERANGE, "a row has more than 64 hops");
  int64_t nnz = 0;
  for (int64_t r = 0; r < nr; ++r) { const int64_t t = h[r]; h[r] = nnz; nnz += t; }
  if (!row) return nnz;
  QS3G_REQUIRE(nnz <= cap, QS3G_ERANGE, "connection table capacity too small");
  if (nnz == 0) return 0;
  DevBuf<int64_t> d_off(nr), d_row(nnz), d_col(nnz);
  DevBuf<int> d_ell(3 * nnz), d_bond(nnz);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_off.get(), h.data(), nr * 8, cudaMemcpyHostToDevice, st));
  dispatch_nod(s.NOD, [&](auto c) {
    k_conn<decltype(c)::value><<<grid, 128, 0, st>>>(a, kind, row0, row1, nullptr, d_off.get(),
                                                    d_row.get(), d_col.get(), d_ell.get(), d_bond.get(),
                                                    d_ovf.get());
  });
  check_launch("k_conn(emit)");
  QS3G_CHECK_CUDA(cudaMemcpyAsync(row, d_row.get(), nnz * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(col, d_col.get(), nnz * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(ell, d_ell.get(), 3 * nnz * 4, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(bond, d_bond.get(), nnz * 4, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  return nnz;
}

int64_t connection_table(const Model& m, const Sector& s, int64_t* row, int64_t* col, int* ell, int* bond,
                         int64_t cap, cudaStream_t st) {
  return connection_table_rows(m, s, 0, s.D, row, col, ell, bond, cap, st);
}

}  // namespace qs3g

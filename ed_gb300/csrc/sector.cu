// sector.cu -- GPU construction of the (NOD, K) representative basis.
//
// Replaces allocate_lists_omp_SQ + checkstate_SQ (state_lists.f90:66-112,
// 225-292).  The reference tests every one of the C(NOS, NOD) ranks with a
// full translation scan, stores the survivors with a critical section and
// quick-sorts them.  Here candidates are enumerated in colex (= rank) order
// by one thread per block of 256 candidates, the survivors are
// marked in a presence bitmap, one exclusive scan turns the bitmap into row
// numbers, and a second pass writes the rows in rank order -- already sorted.
// The bitmap plus its block bases (the "directory") is kept as the O(1)
// rank -> row lookup that replaces findstate's binary search
// (state_lists.f90:364-382) in the H*v kernels.
//
// Chains (LY = LZ = 1) use the anchored space: every representative occupies
// site 1 (a configuration without site 1 is beaten by the translation that
// moves its lowest spin there), so only C(NOS-1, NOD-1) candidates are
// tested, each in O(NOD^2) through the cyclic-gap keys of chain_rep.
#include <cmath>

#include "qs3g_device.cuh"
#include "qs3g_internal.cuh"
#include "krylov.h"

namespace qs3g {

std::atomic<int64_t> g_launches{0};

uint64_t binom_u64(int n, int k) {
  if (n < 0 || k < 0 || n < k) return 0;
  unsigned __int128 v = 1;
  for (int i = 1; i <= k; ++i) {
    v = v * (unsigned)(n - k + i);
    v = v / (unsigned)i;
    if (v > (unsigned __int128)INT64_MAX) return (uint64_t)INT64_MAX;
  }
  return (uint64_t)v;
}

int bits_for(int v) {
  int b = 1;
  while ((1ll << b) <= (long long)v) ++b;
  return b;
}

void wavevector(const int K[3], int LX, int LY, int LZ, double rk[3]) {
  const double PI = std::acos(-1.0);
  rk[0] = 2.0 * PI * (double)K[0] / (double)LX;
  rk[1] = 2.0 * PI * (double)K[1] / (double)LY;
  rk[2] = 2.0 * PI * (double)K[2] / (double)LZ;
}

void host_explist(const double rk[3], int LX, int LY, int LZ, std::vector<double2>& out) {
  out.resize((size_t)(LX + 1) * (LY + 1) * (LZ + 1));
  for (int k = 0; k <= LZ; ++k)
    for (int j = 0; j <= LY; ++j)
      for (int i = 0; i <= LX; ++i) {
        double ph = rk[0] * (double)i + rk[1] * (double)j + rk[2] * (double)k;
        out[(size_t)i + (size_t)(LX + 1) * ((size_t)j + (size_t)(LY + 1) * k)] =
            make_double2(std::cos(ph), std::sin(ph));
      }
}

namespace {

constexpr int kThreads = 128;

// Store the 8 presence words of 256-candidate block b as directory entries
// with their prefix counts inside the block; returns the block's count.
__device__ __forceinline__ uint32_t write_words(uint2* dirw, uint64_t nwords, uint64_t b, const uint32_t (&w)[8]) {
  uint32_t pre = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (b * 8 + k < nwords) dirw[b * 8 + k] = make_uint2(pre, w[k]);
    pre += __popc(w[k]);
  }
  return pre;
}

// ------------------------------------------------------------ chain (anchored space)
struct ChainBuildArgs {
  int L, NOD, bits;
  uint64_t nspace, nblocks;
  const uint32_t* binomA;   // C(x, j), x in [0, L-2], j in [1, NOD-1]
  const uint64_t* binom;    // C(n, k), k in [0, NOD+1]
  const int* keep;          // keep[count] for count in [1, NOD]
  const double* r_by_count; // list_r value for a representative with `count` self-translations
  uint2* dirw;              // one entry per 32 candidates: (rows before, presence bits)
  uint64_t nwords;
  uint32_t* blkcount;
  int64_t* list_s;
  double* list_r;
  float* list_r32;
  uint64_t* conf;
};

// Unrank anchored candidate c -> q[1..NOD-1] (q[j] = p[j] - 2) by the
// combinatorial number system c = sum_j C(q[j], j).
template <int NOD>
__device__ __forceinline__ void anchored_unrank(uint64_t c, const ChainBuildArgs& a, int (&q)[NOD]) {
  q[0] = -1;
#pragma unroll
  for (int j = NOD - 1; j >= 1; --j) {
    int v;
    if (j == 1) {
      v = (int)c;
    } else {
      // largest v in [j-1, L-2] with C(v, j) <= c
      const uint32_t* row = a.binomA + (size_t)(j - 1) * (a.L - 1);
      int lo = j - 1, hi = a.L - 2;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if ((uint64_t)row[mid] <= c) lo = mid; else hi = mid - 1;
      }
      v = lo;
      c -= row[v];
    }
    q[j] = v;
  }
}

// Colex successor of q[1..NOD-1] over values [0, L-2].
template <int NOD>
__device__ __forceinline__ void anchored_next(int (&q)[NOD]) {
  bool done = false;
#pragma unroll
  for (int j = 1; j < NOD; ++j) {
    if (!done) {
      const int lim = (j + 1 < NOD) ? q[(j + 1 < NOD) ? j + 1 : j] : 0x7fffffff;
      if (q[j] + 1 < lim) {
        q[j] += 1;
        done = true;
      } else {
        q[j] = j - 1;
      }
    }
  }
}

// Rep test of an anchored configuration: key_0 >= key_m for all m; returns the
// number of self-translations (m with key_m == key_0) or 0 if not a rep.
template <int NOD>
__device__ __forceinline__ int chain_selfcount(const int (&p)[NOD], int L, int bits) {
  int g[NOD];
#pragma unroll
  for (int m = 0; m < NOD - 1; ++m) g[m] = p[m + 1] - p[m];
  g[NOD - 1] = p[0] + L - p[NOD - 1];
  uint64_t key0 = 0;
#pragma unroll
  for (int t = 1; t <= NOD; ++t) key0 = (key0 << bits) | (uint64_t)g[(0 - t + 2 * NOD) % NOD];
  int count = 1;
  bool rep = true;
#pragma unroll
  for (int m = 1; m < NOD; ++m) {
    uint64_t key = 0;
#pragma unroll
    for (int t = 1; t <= NOD; ++t) key = (key << bits) | (uint64_t)g[(m - t + 2 * NOD) % NOD];
    rep = rep && (key <= key0);
    count += (key == key0) ? 1 : 0;
  }
  return rep ? count : 0;
}

template <int NOD>
__global__ void __launch_bounds__(kThreads) k_chain_mark(ChainBuildArgs a) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const uint64_t c0 = b * 256u;
  int q[NOD];
  anchored_unrank<NOD>(c0, a, q);
  uint32_t words[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int kmax = (int)((a.nspace - c0) < 256u ? (a.nspace - c0) : 256u);
  for (int k = 0; k < kmax; ++k) {
    int p[NOD];
    p[0] = 1;
#pragma unroll
    for (int j = 1; j < NOD; ++j) p[j] = q[j] + 2;
    const int sc = chain_selfcount<NOD>(p, a.L, a.bits);
    if (sc > 0 && a.keep[sc]) words[k >> 5] |= 1u << (k & 31);
    anchored_next<NOD>(q);
  }
  a.blkcount[b] = write_words(a.dirw, a.nwords, b, words);
}

template <int NOD>
__global__ void __launch_bounds__(kThreads) k_chain_emit(ChainBuildArgs a) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const uint64_t c0 = b * 256u;
  const uint2* d = a.dirw + b * 8;
  uint32_t row = d[0].x;
  int q[NOD];
  anchored_unrank<NOD>(c0, a, q);
  const int kmax = (int)((a.nspace - c0) < 256u ? (a.nspace - c0) : 256u);
  for (int k = 0; k < kmax; ++k) {
    if ((d[k >> 5].y >> (k & 31)) & 1u) {
      int p[NOD];
      p[0] = 1;
#pragma unroll
      for (int j = 1; j < NOD; ++j) p[j] = q[j] + 2;
      const int sc = chain_selfcount<NOD>(p, a.L, a.bits);
      int64_t rank = 1;  // inv_list: n(1) + sum_{i>=2} C(n(i)-1, i) with n(1) = 1
#pragma unroll
      for (int j = 1; j < NOD; ++j) rank += (int64_t)a.binom[(size_t)(j + 1) * (a.L + 1) + (p[j] - 1)];
      a.list_s[row] = rank;
      const double r = a.r_by_count[sc];
      a.list_r[row] = r;
      a.list_r32[row] = (float)r;
      a.conf[row] = pack<NOD>(p, a.bits);
      ++row;
    }
    anchored_next<NOD>(q);
  }
}

// ------------------------------------------------------------ general lattice (full space)
struct GenBuildArgs {
  int NOS, NOD, bits, LX, LY, LZ, NT;
  uint64_t nspace, nblocks;
  const uint64_t* binom;     // C(n, k), k in [0, NOD+1]
  const int16_t* xyz;        // (x,y,z,pad) per site, index 1..NOS
  const double2* phase;      // checkstate phase per translation (loop order)
  double NOSd;
  uint2* dirw;
  uint64_t nwords;
  uint32_t* blkcount;
  int64_t* list_s;
  uint64_t* conf;
  double2* coef;             // per row: sum of phases over self-translations
  int* count;                // per row: number of self-translations
};

template <int NOD>
__device__ __forceinline__ void full_unrank(uint64_t c, const GenBuildArgs& a, int (&v)[NOD]) {
#pragma unroll
  for (int j = NOD - 1; j >= 0; --j) {
    const uint64_t* row = a.binom + (size_t)(j + 1) * (a.NOS + 1);
    int lo = j, hi = a.NOS - 1;  // largest x in [j, NOS-1] with C(x, j+1) <= c
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (row[mid] <= c) lo = mid; else hi = mid - 1;
    }
    v[j] = lo;
    c -= row[lo];
  }
}

template <int NOD>
__device__ __forceinline__ void full_next(int (&v)[NOD]) {
  bool done = false;
#pragma unroll
  for (int j = 0; j < NOD; ++j) {
    if (!done) {
      const int lim = (j + 1 < NOD) ? v[(j + 1 < NOD) ? j + 1 : j] : 0x7fffffff;
      if (v[j] + 1 < lim) { v[j] += 1; done = true; } else { v[j] = j; }
    }
  }
}

template <int NOD>
__device__ __forceinline__ uint64_t translate_pack(const int (&n)[NOD], int ti, int tj, int tk,
                                                   const GenBuildArgs& a) {
  int t[NOD];
#pragma unroll
  for (int e = 0; e < NOD; ++e) {
    const short4 c = reinterpret_cast<const short4*>(a.xyz)[n[e]];
    int x = c.x + ti; x -= (x >= a.LX) ? a.LX : 0;
    int y = c.y + tj; y -= (y >= a.LY) ? a.LY : 0;
    int z = c.z + tk; z -= (z >= a.LZ) ? a.LZ : 0;
    t[e] = 1 + x + a.LX * (y + a.LY * z);
  }
  // insertion sort (state_lists.f90:115-129)
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

// checkstate_SQ (state_lists.f90:66-112) for one candidate.
template <int NOD>
__device__ __forceinline__ bool general_check(const int (&n)[NOD], const GenBuildArgs& a, int& count,
                                              double2& coef) {
  const uint64_t self = pack<NOD>(n, a.bits);
  count = 0;
  coef = make_double2(0.0, 0.0);
  int tau = 0;
  for (int k = 1; k <= a.LZ; ++k)
    for (int j = 1; j <= a.LY; ++j)
      for (int i = 1; i <= a.LX; ++i, ++tau) {
        const uint64_t w = translate_pack<NOD>(n, i % a.LX, j % a.LY, k % a.LZ, a);
        if (w < self) return false;
        if (w == self) {
          ++count;
          const double2 ph = a.phase[tau];
          coef.x += ph.x;
          coef.y += ph.y;
        }
      }
  return true;
}

template <int NOD>
__global__ void __launch_bounds__(kThreads) k_gen_mark(GenBuildArgs a) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const uint64_t c0 = b * 256u;
  int v[NOD];
  full_unrank<NOD>(c0, a, v);
  uint32_t words[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int kmax = (int)((a.nspace - c0) < 256u ? (a.nspace - c0) : 256u);
  for (int k = 0; k < kmax; ++k) {
    int n[NOD];
#pragma unroll
    for (int j = 0; j < NOD; ++j) n[j] = v[j] + 1;
    int count;
    double2 coef;
    if (general_check<NOD>(n, a, count, coef)) {
      const double ro = (coef.x * coef.x + coef.y * coef.y) * a.NOSd / (double)count;
      if (ro > 1.0e-15) words[k >> 5] |= 1u << (k & 31);
    }
    full_next<NOD>(v);
  }
  a.blkcount[b] = write_words(a.dirw, a.nwords, b, words);
}

template <int NOD>
__global__ void __launch_bounds__(kThreads) k_gen_emit(GenBuildArgs a) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const uint64_t c0 = b * 256u;
  const uint2* d = a.dirw + b * 8;
  uint32_t row = d[0].x;
  int v[NOD];
  full_unrank<NOD>(c0, a, v);
  const int kmax = (int)((a.nspace - c0) < 256u ? (a.nspace - c0) : 256u);
  for (int k = 0; k < kmax; ++k) {
    if ((d[k >> 5].y >> (k & 31)) & 1u) {
      int n[NOD];
#pragma unroll
      for (int j = 0; j < NOD; ++j) n[j] = v[j] + 1;
      int count;
      double2 coef;
      general_check<NOD>(n, a, count, coef);
      a.list_s[row] = (int64_t)(c0 + k) + 1;
      a.conf[row] = pack<NOD>(n, a.bits);
      a.coef[row] = coef;
      a.count[row] = count;
      ++row;
    }
    full_next<NOD>(v);
  }
}

// ------------------------------------------------------------ scan of block counts
// Exclusive scan of per-block counts: pass 0 sums 1024-block chunks, the host
// scans the chunk sums, pass 1 writes every block's base.
__global__ void k_scan_blocks(const uint32_t* in, uint64_t n, uint64_t* partial, uint64_t* out_base, int pass) {
  __shared__ uint64_t sh[1024];
  const uint64_t base = (uint64_t)blockIdx.x * 1024u;
  const uint64_t i = base + threadIdx.x;
  uint64_t v = (i < n) ? in[i] : 0u;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint64_t t = (threadIdx.x >= (unsigned)off) ? sh[threadIdx.x - off] : 0u;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (pass == 0) {
    if (threadIdx.x == 1023) partial[blockIdx.x] = sh[1023];
  } else {
    if (i < n) out_base[i] = partial[blockIdx.x] + sh[threadIdx.x] - v;
  }
}

// dirw[w].x += base of its 256-candidate block
__global__ void k_dir_fix(uint2* dirw, uint64_t nwords, const uint64_t* base) {
  const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nwords) dirw[w].x += (uint32_t)base[w >> 3];
}

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

// U(1) basis: row i (0-based) is the configuration of colex rank i + 1
// (list_fly, source_only_u1/state_lists.f90:85-99).  Colex unranking: for
// j = NOD..1 the site n_j is the largest n with C(n-1, j) <= remaining rank.
template <int NOD>
__global__ void __launch_bounds__(kThreads) k_u1_emit(int NOS, int bits, int64_t D, const uint64_t* __restrict__ binom,
                                                      int64_t* list_s, double* list_r, float* list_r32,
                                                      uint64_t* conf) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D) return;
  uint64_t r = (uint64_t)i;
  int n[NOD];
  int hi = NOS;
#pragma unroll
  for (int j = NOD; j >= 1; --j) {
    const uint64_t* bj = binom + (size_t)j * (NOS + 1);
    int lo = j, up = hi;  // n in [j, hi]: C(lo-1, j) = 0 <= r always
    while (lo < up) {
      const int mid = (lo + up + 1) >> 1;
      if (bj[mid - 1] <= r) lo = mid; else up = mid - 1;
    }
    n[j - 1] = lo;
    r -= bj[lo - 1];
    hi = lo - 1;
  }
  conf[i] = pack<NOD>(n, bits);
  list_s[i] = i + 1;
  list_r[i] = 1.0;
  list_r32[i] = 1.0f;
}

// Exclusive scan of the block counts, folded into the directory; returns the total.
uint64_t scan_directory(uint32_t* blkcount, uint64_t nblocks, uint2* dirw, uint64_t nwords, cudaStream_t st) {
  const uint64_t nchunks = (nblocks + 1023) / 1024;
  DevBuf<uint64_t> d_partial(nchunks), d_base(nblocks);
  k_scan_blocks<<<(unsigned)nchunks, 1024, 0, st>>>(blkcount, nblocks, d_partial.get(), d_base.get(), 0);
  check_launch("k_scan_blocks");
  std::vector<uint64_t> h(nchunks);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(h.data(), d_partial.get(), nchunks * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  uint64_t run = 0;
  for (uint64_t c = 0; c < nchunks; ++c) { uint64_t t = h[c]; h[c] = run; run += t; }
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_partial.get(), h.data(), nchunks * 8, cudaMemcpyHostToDevice, st));
  k_scan_blocks<<<(unsigned)nchunks, 1024, 0, st>>>(blkcount, nblocks, d_partial.get(), d_base.get(), 1);
  check_launch("k_scan_blocks");
  k_dir_fix<<<(unsigned)((nwords + 255) / 256), 256, 0, st>>>(dirw, nwords, d_base.get());
  check_launch("k_dir_fix");
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  return run;
}

}  // namespace

void build_sector(const Model& m, int NOD, const int K[3], Sector& s, cudaStream_t st) {
  double rk[3];
  wavevector(K, m.LX, m.LY, m.LZ, rk);
  build_sector_rk(m, NOD, rk, s, st);
  for (int d = 0; d < 3; ++d) s.K[d] = K[d];
}

void build_sector_rk(const Model& m, int NOD, const double rk[3], Sector& s, cudaStream_t st) {
  QS3G_REQUIRE(NOD >= 1 && NOD <= kMaxNOD, QS3G_ENOTSUP, "NOD must be in [1, 8]");
  QS3G_REQUIRE(NOD <= m.NOS, QS3G_EINVAL, "NOD > NOS");
  QS3G_REQUIRE(NOD * m.bits <= 64, QS3G_ERANGE, "NOD * bits(NOS) exceeds one 64-bit word");
  s.NOD = NOD;
  for (int d = 0; d < 3; ++d) { s.K[d] = 0; s.rk[d] = rk[d]; }
  std::vector<double2> ex;
  host_explist(s.rk, m.LX, m.LY, m.LZ, ex);
  s.kzero = true;
  for (auto& e : ex) s.kzero = s.kzero && (e.x == 1.0 && e.y == 0.0);
  s.d_explist.alloc(ex.size());
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_explist.get(), ex.data(), ex.size() * sizeof(double2),
                                  cudaMemcpyHostToDevice, st));
  // binomials C(n,k), k in [0, NOD+1]
  const int KB = NOD + 1;
  std::vector<uint64_t> hb((size_t)(KB + 1) * (m.NOS + 1));
  for (int k = 0; k <= KB; ++k)
    for (int n = 0; n <= m.NOS; ++n) hb[(size_t)k * (m.NOS + 1) + n] = binom_u64(n, k);
  s.d_binom.alloc(hb.size());
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_binom.get(), hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, st));
  const uint64_t ths = binom_u64(m.NOS, NOD);
  QS3G_REQUIRE(ths < (uint64_t)INT64_MAX, QS3G_ERANGE, "C(NOS, NOD) overflows 64 bits");

  if (m.chain) {
    const int L = m.NOS;
    s.anchored = true;
    s.nspace = binom_u64(L - 1, NOD - 1);
    QS3G_REQUIRE(s.nspace < (1ull << 32), QS3G_ERANGE, "anchored space exceeds 2^32 candidates");
    // chain phases: explist(i,1,1) for translation i, explist(0,0,0) for ell = 0
    std::vector<double2> cph(L + 1);
    cph[0] = ex[0];
    for (int i = 1; i <= L; ++i)
      cph[i] = ex[(size_t)i + (size_t)(m.LX + 1) * (1 + (size_t)(m.LY + 1) * 1)];
    s.d_chainph.alloc(L + 1);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_chainph.get(), cph.data(), (L + 1) * sizeof(double2),
                                    cudaMemcpyHostToDevice, st));
    std::vector<float2> cph32(L + 1);
    for (int i = 0; i <= L; ++i) cph32[i] = make_float2((float)cph[i].x, (float)cph[i].y);
    s.d_chainph32.alloc(L + 1);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_chainph32.get(), cph32.data(), (L + 1) * sizeof(float2),
                                    cudaMemcpyHostToDevice, st));
    // anchored binomials (u32)
    std::vector<uint32_t> ha((size_t)std::max(1, NOD - 1) * (L - 1 > 0 ? L - 1 : 1), 0);
    for (int j = 1; j < NOD; ++j)
      for (int x = 0; x <= L - 2; ++x) ha[(size_t)(j - 1) * (L - 1) + x] = (uint32_t)binom_u64(x, j);
    s.d_binomA.alloc(ha.size());
    QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_binomA.get(), ha.data(), ha.size() * 4, cudaMemcpyHostToDevice, st));
    // norms by number of self-translations (checkstate_SQ with LY = LZ = 1):
    // self-translations are i = p, 2p, ..., L (p = L / count), summed in loop order.
    std::vector<int> keep(NOD + 1, 0);
    std::vector<double> rbc(NOD + 1, 0.0);
    for (int c = 1; c <= NOD; ++c) {
      if (L % c != 0) continue;
      const int per = L / c;
      double cre = 0.0, cim = 0.0;
      const double p1 = s.rk[2] * 1.0;
      const double p2 = s.rk[1] * 1.0 + p1;
      for (int i = 1; i <= L; ++i) {
        if (i % per != 0) continue;
        const double ph = s.rk[0] * (double)i + p2;
        cre += std::cos(ph);
        cim += -std::sin(ph);
      }
      const double a = std::hypot(cre, cim);
      const double ro = (a * a) * (double)m.NOS / (double)c;
      keep[c] = ro > 1.0e-15 ? 1 : 0;
      rbc[c] = std::sqrt(ro);
    }
    DevBuf<int> d_keep(NOD + 1);
    DevBuf<double> d_rbc(NOD + 1);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(d_keep.get(), keep.data(), (NOD + 1) * 4, cudaMemcpyHostToDevice, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(d_rbc.get(), rbc.data(), (NOD + 1) * 8, cudaMemcpyHostToDevice, st));
    s.nblocks = (s.nspace + 255) / 256;
    s.nwords = (s.nspace + 31) / 32;
    s.d_dir.alloc(s.nwords);
    DevBuf<uint32_t> d_cnt(s.nblocks);
    ChainBuildArgs a{};
    a.L = L; a.NOD = NOD; a.bits = m.bits; a.nspace = s.nspace; a.nblocks = s.nblocks;
    a.binomA = s.d_binomA.get(); a.binom = s.d_binom.get();
    a.keep = d_keep.get(); a.r_by_count = d_rbc.get();
    a.dirw = s.d_dir.get(); a.nwords = s.nwords; a.blkcount = d_cnt.get();
    const unsigned grid = (unsigned)((s.nblocks + kThreads - 1) / kThreads);
    dispatch_nod(NOD, [&](auto c) {
      k_chain_mark<decltype(c)::value><<<grid, kThreads, 0, st>>>(a);
    });
    check_launch("k_chain_mark");
    const uint64_t D = scan_directory(d_cnt.get(), s.nblocks, s.d_dir.get(), s.nwords, st);
    QS3G_REQUIRE(D < (1ull << 31), QS3G_ERANGE, "sector dimension exceeds 2^31");
    s.D = (int64_t)D;
    s.d_list_s.alloc(D); s.d_list_r.alloc(D); s.d_list_r32.alloc(D); s.d_conf.alloc(D);
    a.list_s = s.d_list_s.get(); a.list_r = s.d_list_r.get(); a.list_r32 = s.d_list_r32.get();
    a.conf = s.d_conf.get();
    if (D > 0) {
      dispatch_nod(NOD, [&](auto c) {
        k_chain_emit<decltype(c)::value><<<grid, kThreads, 0, st>>>(a);
      });
      check_launch("k_chain_emit");
    }
    // H*v coefficient tables: sJxy_b * R[c] and 1/R[c] by self-translation count
    std::vector<double> cr((size_t)std::max(1, m.NOxxz) * (NOD + 1), 0.0), ir(NOD + 1, 0.0);
    std::vector<float> cr32(cr.size()), ir32(NOD + 1);
    for (int b = 0; b < m.NOxxz; ++b)
      for (int c = 0; c <= NOD; ++c) cr[(size_t)b * (NOD + 1) + c] = m.sJxy[b] * rbc[c];
    for (int c = 0; c <= NOD; ++c) ir[c] = rbc[c] > 0.0 ? 1.0 / rbc[c] : 0.0;
    for (size_t k = 0; k < cr.size(); ++k) cr32[k] = (float)cr[k];
    for (int c = 0; c <= NOD; ++c) ir32[c] = (float)ir[c];
    s.d_coefR.alloc(cr.size()); s.d_coefR32.alloc(cr.size());
    s.d_invR.alloc(NOD + 1); s.d_invR32.alloc(NOD + 1);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_coefR.get(), cr.data(), cr.size() * 8, cudaMemcpyHostToDevice, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_coefR32.get(), cr32.data(), cr32.size() * 4, cudaMemcpyHostToDevice, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_invR.get(), ir.data(), (NOD + 1) * 8, cudaMemcpyHostToDevice, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_invR32.get(), ir32.data(), (NOD + 1) * 4, cudaMemcpyHostToDevice, st));
    compute_diag(m, s, st);
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    return;
  }

  // general lattice: full colex space with the full translation scan
  s.anchored = false;
  s.nspace = ths;
  QS3G_REQUIRE(s.nspace <= (1ull << 36), QS3G_ERANGE, "C(NOS, NOD) too large for the directory");
  const int NT = m.LX * m.LY * m.LZ;
  std::vector<double2> phase(NT);
  {
    int tau = 0;
    for (int k = 1; k <= m.LZ; ++k) {
      const double p1 = s.rk[2] * (double)k;
      for (int j = 1; j <= m.LY; ++j) {
        const double p2 = s.rk[1] * (double)j + p1;
        for (int i = 1; i <= m.LX; ++i, ++tau) {
          const double ph = s.rk[0] * (double)i + p2;
          phase[tau] = make_double2(std::cos(ph), -std::sin(ph));
        }
      }
    }
  }
  DevBuf<double2> d_phase(NT);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_phase.get(), phase.data(), NT * sizeof(double2), cudaMemcpyHostToDevice, st));
  s.nblocks = (s.nspace + 255) / 256;
  s.nwords = (s.nspace + 31) / 32;
  s.d_dir.alloc(s.nwords);
  DevBuf<uint32_t> d_cnt(s.nblocks);
  GenBuildArgs a{};
  a.NOS = m.NOS; a.NOD = NOD; a.bits = m.bits; a.LX = m.LX; a.LY = m.LY; a.LZ = m.LZ; a.NT = NT;
  a.nspace = s.nspace; a.nblocks = s.nblocks; a.binom = s.d_binom.get();
  a.xyz = m.d_site_xyz.get(); a.phase = d_phase.get(); a.NOSd = (double)m.NOS;
  a.dirw = s.d_dir.get(); a.nwords = s.nwords; a.blkcount = d_cnt.get();
  const unsigned grid = (unsigned)((s.nblocks + kThreads - 1) / kThreads);
  dispatch_nod(NOD, [&](auto c) { k_gen_mark<decltype(c)::value><<<grid, kThreads, 0, st>>>(a); });
  check_launch("k_gen_mark");
  const uint64_t D = scan_directory(d_cnt.get(), s.nblocks, s.d_dir.get(), s.nwords, st);
  QS3G_REQUIRE(D < (1ull << 31), QS3G_ERANGE, "sector dimension exceeds 2^31");
  s.D = (int64_t)D;
  s.d_list_s.alloc(D); s.d_list_r.alloc(D); s.d_list_r32.alloc(D); s.d_conf.alloc(D);
  if (D == 0) { compute_diag(m, s, st); return; }
  DevBuf<double2> d_coef(D);
  DevBuf<int> d_count(D);
  a.list_s = s.d_list_s.get(); a.conf = s.d_conf.get(); a.coef = d_coef.get(); a.count = d_count.get();
  dispatch_nod(NOD, [&](auto c) { k_gen_emit<decltype(c)::value><<<grid, kThreads, 0, st>>>(a); });
  check_launch("k_gen_emit");
  // list_r on the host: sqrt(abs(coef)**2 * NOS / count) with the host libm (state_lists.f90:110,288)
  std::vector<double2> hc(D);
  std::vector<int> hn(D);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(hc.data(), d_coef.get(), D * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(hn.data(), d_count.get(), D * sizeof(int), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  std::vector<double> hr(D);
  std::vector<float> hr32(D);
  for (uint64_t i = 0; i < D; ++i) {
    const double a2 = std::hypot(hc[i].x, hc[i].y);
    hr[i] = std::sqrt((a2 * a2) * (double)m.NOS / (double)hn[i]);
    hr32[i] = (float)hr[i];
  }
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_list_r.get(), hr.data(), D * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_list_r32.get(), hr32.data(), D * 4, cudaMemcpyHostToDevice, st));
  compute_diag(m, s, st);
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

// U(1)-only basis: all C(NOS, NOD) configurations, row = colex rank - 1
// (get_combination + list_fly + inv_list, source_only_u1/state_lists.f90:6-99;
// THS = combination(NOS, NOD) in source_only_u1/main.f90).  No translations:
// list_r = 1 and every hop coefficient is sJxy_b.
void build_sector_u1(const Model& m, int NOD, Sector& s, cudaStream_t st) {
  QS3G_REQUIRE(NOD >= 1 && NOD <= kMaxNOD, QS3G_ENOTSUP, "NOD must be in [1, 8]");
  QS3G_REQUIRE(NOD <= m.NOS, QS3G_EINVAL, "NOD > NOS");
  QS3G_REQUIRE(NOD * m.bits <= 64, QS3G_ERANGE, "NOD * bits(NOS) exceeds one 64-bit word");
  const uint64_t ths = binom_u64(m.NOS, NOD);
  QS3G_REQUIRE(ths < (1ull << 31), QS3G_ERANGE, "C(NOS, NOD) exceeds 2^31 rows");
  s.NOD = NOD;
  s.u1 = true;
  s.anchored = false;
  s.kzero = true;
  for (int d = 0; d < 3; ++d) { s.K[d] = 0; s.rk[d] = 0.0; }
  s.nspace = ths;
  s.D = (int64_t)ths;
  s.nblocks = 0;
  s.nwords = 0;
  const int KB = NOD + 1;
  std::vector<uint64_t> hb((size_t)(KB + 1) * (m.NOS + 1));
  for (int k = 0; k <= KB; ++k)
    for (int n = 0; n <= m.NOS; ++n) hb[(size_t)k * (m.NOS + 1) + n] = binom_u64(n, k);
  s.d_binom.alloc(hb.size());
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_binom.get(), hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, st));
  const int64_t D = s.D;
  s.d_list_s.alloc(D); s.d_list_r.alloc(D); s.d_list_r32.alloc(D); s.d_conf.alloc(D);
  const unsigned grid = (unsigned)((D + kThreads - 1) / kThreads);
  dispatch_nod(NOD, [&](auto c) {
    k_u1_emit<decltype(c)::value><<<grid, kThreads, 0, st>>>(m.NOS, m.bits, D, s.d_binom.get(), s.d_list_s.get(),
                                                              s.d_list_r.get(), s.d_list_r32.get(), s.d_conf.get());
  });
  check_launch("k_u1_emit");
  // hop coefficients sJxy_b (table layout of the chain kernels, R = 1)
  std::vector<double> cr((size_t)std::max(1, m.NOxxz) * (NOD + 1), 0.0), ir(NOD + 1, 1.0);
  std::vector<float> cr32(cr.size()), ir32(NOD + 1, 1.0f);
  for (int b = 0; b < m.NOxxz; ++b)
    for (int c = 0; c <= NOD; ++c) cr[(size_t)b * (NOD + 1) + c] = m.sJxy[b];
  for (size_t k = 0; k < cr.size(); ++k) cr32[k] = (float)cr[k];
  s.d_coefR.alloc(cr.size()); s.d_coefR32.alloc(cr.size());
  s.d_invR.alloc(NOD + 1); s.d_invR32.alloc(NOD + 1);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_coefR.get(), cr.data(), cr.size() * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_coefR32.get(), cr32.data(), cr32.size() * 4, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_invR.get(), ir.data(), (NOD + 1) * 8, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(s.d_invR32.get(), ir32.data(), (NOD + 1) * 4, cudaMemcpyHostToDevice, st));
  compute_diag(m, s, st);
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

}  // namespace qs3g

// batch_trlan.cu -- thick-restart Lanczos for many chain problems in lock step.
//
// lancz_eigen_val_complex (eigen_solver.f90:69-261) for n independent chain
// sectors at once: every Krylov column is one concatenated vector in which
// problem s owns rows [row0_s, row0_s + D_s) (padded to 256-row blocks), so
// one launch of each kernel advances every active problem by one Lanczos
// step.  The launch maps list only the blocks of problems that have not
// converged; a converged problem keeps its Ritz vectors in columns 0..NOE-1
// and drops out of the maps at the next restart.  Per-problem scalars
// (alpha, beta, overlaps, arrow couplings, Ritz coefficients) live in device
// arrays indexed by problem; the small Ritz problems are solved on the host
// for every active problem at each restart.  The steps and the convergence
// rule of each problem are those of trlan_core (krylov.cu); level-1
// arithmetic is double-float on the FP32 pipe (eft.cuh) for both storage
// types, so complex(4) phases keep FP64-accurate reductions.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

#include "eft.cuh"
#include "hosteig.h"
#include "krylov.h"
#include "qs3g_internal.cuh"

namespace qs3g {
namespace {

using zd = std::complex<double>;
constexpr int kB = 256;          // rows per block
constexpr int kChunkTiles = 16;  // overlap chunks: up to 16 blocks of one problem

struct BSeg {
  int64_t row0, D;
};
struct Chunk {
  int64_t row0;
  int n, seg;
};

template <class T>
struct Store;
template <>
struct Store<double2> {
  static __device__ __forceinline__ double2 st(float rh, float rl, float ih, float il) {
    return make_double2(djoin(rh, rl), djoin(ih, il));
  }
};
template <>
struct Store<float2> {
  static __device__ __forceinline__ float2 st(float rh, float rl, float ih, float il) {
    return make_float2(__fadd_rn(rh, rl), __fadd_rn(ih, il));
  }
};

__device__ __forceinline__ bool brow(const BSeg* segs, const int* bs, const int* bf, int64_t& r, int& sg) {
  sg = bs[blockIdx.x];
  const int64_t i = (int64_t)(blockIdx.x - bf[blockIdx.x]) * kB + threadIdx.x;
  r = segs[sg].row0 + i;
  return i < segs[sg].D;
}

// part[b] = sum over the block's rows of conj(x) y (double-float per thread)
template <class T>
__global__ void __launch_bounds__(kB) k_bdot(const BSeg* segs, const int* bs, const int* bf, const T* __restrict__ x,
                                             const T* __restrict__ y, double2* part) {
  __shared__ double2 sh[kB];
  int64_t r;
  int sg;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  if (brow(segs, bs, bf, r, sg)) {
    const float4 a = SplitLd<T>::ld(x[r]), b = SplitLd<T>::ld(y[r]);
    const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
    const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
    df_fma(rh, rl, ar, br);
    df_fma(rh, rl, ai, bi);
    df_fma(ih, il, ar, bi);
    df_fma(ih, il, fneg2(ai), br);
  }
  const double2 s = block_sum2(make_double2(djoin(rh, rl), djoin(ih, il)), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// One block per active problem: fixed-order sum of its blocks' partials.
// mode 0: out[s*ld] = sum; mode 1: out[s*ld] = (sqrt(sum.x), sum.x)
__global__ void __launch_bounds__(kB) k_bfinal(const double2* part, const int* seg_b0, const int* seg_nb,
                                               const int* active, double2* out, int64_t ld, int mode) {
  __shared__ double2 sh[kB];
  const int sg = active[blockIdx.x];
  const int b0 = seg_b0[sg], nb = seg_nb[sg];
  double2 v = make_double2(0.0, 0.0);
  for (int b = threadIdx.x; b < nb; b += kB) {
    v.x += part[b0 + b].x;
    v.y += part[b0 + b].y;
  }
  const double2 s = block_sum2(v, sh);
  if (threadIdx.x == 0)
    out[sg * ld] = (mode == 0) ? s : make_double2(std::sqrt(s.x), s.x);
}

// w = q - a_s v - b_s u (a complex unless real_alpha; b = (sqrt beta2, .), u may be null).
// The FP64 scalars are split once per block (the FP64 pipe is 1/64 rate).
template <class T>
__global__ void __launch_bounds__(kB) k_blanczos_w(const BSeg* segs, const int* bs, const int* bf, T* w,
                                                   const T* q, const T* __restrict__ v, const T* __restrict__ u,
                                                   const double2* a, const double2* b, int64_t ld, int real_alpha) {
  __shared__ float2 sc[3];
  if (threadIdx.x == 0) {
    const int sgb = bs[blockIdx.x];
    const double2 as = a[sgb * ld];
    sc[0] = split(as.x);
    sc[1] = split(real_alpha ? 0.0 : as.y);
    sc[2] = split(u ? b[sgb * ld].x : 0.0);
  }
  __syncthreads();
  int64_t r;
  int sg;
  if (!brow(segs, bs, bf, r, sg)) return;
  const float2 ar = sc[0], ai = sc[1], br = sc[2];
  const float4 qv = SplitLd<T>::ld(q[r]), vv = SplitLd<T>::ld(v[r]);
  float rh = qv.x, rl = qv.y, ih = qv.z, il = qv.w;
  const float2 vr = make_float2(vv.x, vv.y), vi = make_float2(vv.z, vv.w);
  // w -= (ar + i ai)(vr + i vi)
  df_fma(rh, rl, fneg2(ar), vr);
  df_fma(rh, rl, ai, vi);
  df_fma(ih, il, fneg2(ar), vi);
  df_fma(ih, il, fneg2(ai), vr);
  if (u) {
    const float4 uv = SplitLd<T>::ld(u[r]);
    df_fma(rh, rl, fneg2(br), make_float2(uv.x, uv.y));
    df_fma(ih, il, fneg2(br), make_float2(uv.z, uv.w));
  }
  w[r] = Store<T>::st(rh, rl, ih, il);
}

// x *= 1 / s_s.x (the reciprocal and its split once per block)
template <class T>
__global__ void __launch_bounds__(kB) k_bscale(const BSeg* segs, const int* bs, const int* bf, T* x,
                                               const double2* s, int64_t ld) {
  __shared__ float2 sc;
  if (threadIdx.x == 0) sc = split(1.0 / s[bs[blockIdx.x] * ld].x);
  __syncthreads();
  int64_t r;
  int sg;
  if (!brow(segs, bs, bf, r, sg)) return;
  const float2 inv = sc;
  const float4 v = SplitLd<T>::ld(x[r]);
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  df_fma(rh, rl, make_float2(v.x, v.y), inv);
  df_fma(ih, il, make_float2(v.z, v.w), inv);
  x[r] = Store<T>::st(rh, rl, ih, il);
}

// part[b] = sum |x|^2 over the block's rows
template <class T>
__global__ void __launch_bounds__(kB) k_bnrm(const BSeg* segs, const int* bs, const int* bf,
                                             const T* __restrict__ x, double2* part) {
  __shared__ double2 sh[kB];
  int64_t r;
  int sg;
  float rh = 0.f, rl = 0.f;
  if (brow(segs, bs, bf, r, sg)) {
    const float4 a = SplitLd<T>::ld(x[r]);
    df_fma(rh, rl, make_float2(a.x, a.y), make_float2(a.x, a.y));
    df_fma(rh, rl, make_float2(a.z, a.w), make_float2(a.z, a.w));
  }
  const double2 s = block_sum2(make_double2(djoin(rh, rl), 0.0), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Overlaps: grid (column groups of 4, chunks); part[c * nchunk + chunk]
template <class T>
__global__ void __launch_bounds__(kB) k_bgemv_h(const T* __restrict__ V, int64_t ldv, int ncols,
                                                const T* __restrict__ w, const Chunk* chunks, double2* part) {
  __shared__ double2 sh[kB];
  const int c0 = 4 * blockIdx.x;
  const int nc = min(4, ncols - c0);
  const Chunk ch = chunks[blockIdx.y];
  float acc[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k) acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.f;
  for (int t = threadIdx.x; t < ch.n; t += kB) {
    const int64_t i = ch.row0 + t;
    const float4 b = SplitLd<T>::ld(w[i]);
    const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
    T a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < nc) a[k] = V[(int64_t)(c0 + k) * ldv + i];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k < nc) {
        const float4 av = SplitLd<T>::ld(a[k]);
        const float2 ar = make_float2(av.x, av.y), ai = make_float2(av.z, av.w);
        df_fma(acc[k][0], acc[k][1], ar, br);
        df_fma(acc[k][0], acc[k][1], ai, bi);
        df_fma(acc[k][2], acc[k][3], ar, bi);
        df_fma(acc[k][2], acc[k][3], fneg2(ai), br);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (k < nc) {
      const double2 s = block_sum2(make_double2(djoin(acc[k][0], acc[k][1]), djoin(acc[k][2], acc[k][3])), sh);
      if (threadIdx.x == 0) part[(size_t)(c0 + k) * gridDim.y + blockIdx.y] = s;
      __syncthreads();
    }
  }
}

// grid (ncols, active problems): ov[s*ldo + c] = sum over the problem's chunks
__global__ void __launch_bounds__(kB) k_bgemv_final(const double2* part, int nchunk, const int* seg_c0,
                                                    const int* seg_nc, const int* active, double2* ov, int ldo) {
  __shared__ double2 sh[kB];
  const int c = blockIdx.x, sg = active[blockIdx.y];
  const int c0 = seg_c0[sg], n = seg_nc[sg];
  double2 v = make_double2(0.0, 0.0);
  for (int k = threadIdx.x; k < n; k += kB) {
    v.x += part[(size_t)c * nchunk + c0 + k].x;
    v.y += part[(size_t)c * nchunk + c0 + k].y;
  }
  const double2 s = block_sum2(v, sh);
  if (threadIdx.x == 0) ov[(size_t)sg * ldo + c] = s;
}

// w -= V[:, :ncols] * coef_s (coefficients of problem s at coef[s*ldo])
template <class T>
__global__ void __launch_bounds__(kB) k_bgemv_sub(const BSeg* segs, const int* bs, const int* bf,
                                                  const T* __restrict__ V, int64_t ldv, int ncols,
                                                  const double2* __restrict__ coef, int ldo, T* w) {
  __shared__ float4 c[128];
  const int sg = bs[blockIdx.x];
  for (int k = threadIdx.x; k < ncols; k += kB) {
    const double2 ck = coef[(size_t)sg * ldo + k];
    const float2 r = split(ck.x), m = split(ck.y);
    c[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  __syncthreads();
  int64_t r;
  int sg2;
  if (!brow(segs, bs, bf, r, sg2)) return;
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
  for (int k = 0; k < ncols; ++k) {
    const float4 a = SplitLd<T>::ld(V[(int64_t)k * ldv + r]);
    const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
    const float4 ck = c[k];
    const float2 cr = make_float2(ck.x, ck.y), ci = make_float2(ck.z, ck.w);
    df_fma(rh, rl, cr, ar);
    df_fma(rh, rl, fneg2(ci), ai);
    df_fma(ih, il, cr, ai);
    df_fma(ih, il, ci, ar);
  }
  const float4 wv = SplitLd<T>::ld(w[r]);
  float wrh = wv.x, wrl = wv.y, wih = wv.z, wil = wv.w;
  df_add(wrh, wrl, -rh);
  wrl = __fsub_rn(wrl, rl);
  df_add(wih, wil, -ih);
  wil = __fsub_rn(wil, il);
  w[r] = Store<T>::st(wrh, wrl, wih, wil);
}

// In-place restart V[:, :nok] = V[:, :nom] C_s for the block's 256 rows, in
// sub-tiles of 32 rows (C_s: nom x nok column-major at C + s*nom*nok).
template <class T>
__global__ void __launch_bounds__(kB) k_brestart(const BSeg* segs, const int* bs, const int* bf, T* V, int64_t ldv,
                                                 int nom, int nok, const double2* __restrict__ C) {
  extern __shared__ float4 smr[];
  float4* cs = smr;                          // [nok][nom]
  float4* tile = smr + (size_t)nom * nok;    // [nom][32]
  const int sg = bs[blockIdx.x];
  const BSeg g = segs[sg];
  const double2* Cs = C + (size_t)sg * nom * nok;
  for (int k = threadIdx.x; k < nom * nok; k += kB) {
    const float2 r = split(Cs[k].x), m = split(Cs[k].y);
    cs[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  const int64_t base = (int64_t)(blockIdx.x - bf[blockIdx.x]) * kB;
  for (int sub = 0; sub < kB / 32; ++sub) {
    const int64_t l0 = base + sub * 32;
    if (l0 >= g.D) break;
    __syncthreads();
    for (int k = threadIdx.x; k < nom * 32; k += kB) {
      const int col = k / 32, rr = k % 32;
      const int64_t li = l0 + rr;
      tile[k] = (li < g.D) ? SplitLd<T>::ld(V[(int64_t)col * ldv + g.row0 + li]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int rr = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int64_t li = l0 + rr;
    if (li < g.D) {
      for (int oc = grp; oc < nok; oc += kB / 32) {
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        for (int j = 0; j < nom; ++j) {
          const float4 a = tile[j * 32 + rr];
          const float4 c = cs[(size_t)oc * nom + j];
          const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
          const float2 cr = make_float2(c.x, c.y), ci = make_float2(c.z, c.w);
          df_fma(rh, rl, ar, cr);
          df_fma(rh, rl, fneg2(ai), ci);
          df_fma(ih, il, ar, ci);
          df_fma(ih, il, ai, cr);
        }
        V[(int64_t)oc * ldv + g.row0 + li] = Store<T>::st(rh, rl, ih, il);
      }
    }
  }
}

// w = q - e_s v in FP64 (residual check)
__global__ void __launch_bounds__(kB) k_bresid(const BSeg* segs, const int* bs, const int* bf, double2* w,
                                               const double2* q, const double2* v, const double* e) {
  int64_t r;
  int sg;
  if (!brow(segs, bs, bf, r, sg)) return;
  const double es = e[sg];
  w[r] = make_double2(q[r].x - es * v[r].x, q[r].y - es * v[r].y);
}

__global__ void k_bto64(double2* y, const float2* x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = make_double2((double)x[i].x, (double)x[i].y);
}

__device__ __forceinline__ double bsu(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * 0x1.0p-53;
}

// problem-local seeded start: row l of problem s gets the values a single
// qs3g_trlan with the same seed would give its row l
template <class T>
__global__ void k_bstart(const BSeg* segs, const int* bs, const int* bf, T* x, uint64_t seed) {
  int64_t r;
  int sg;
  if (!brow(segs, bs, bf, r, sg)) return;
  const uint64_t l = (uint64_t)(r - segs[sg].row0);
  T o;
  o.x = (decltype(o.x))(bsu(seed, 2 * l) - 0.5);
  o.y = (decltype(o.y))(bsu(seed, 2 * l + 1) - 0.5);
  x[r] = o;
}

unsigned sgrid(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// ------------------------------------------------------------------ launch maps
struct Maps {
  int nseg = 0, nact = 0, nblk = 0, nchunk = 0;
  std::vector<int> active;
  std::vector<int> nod_of;                     // per problem
  std::vector<std::vector<int>> grp_bs, grp_bf;  // per NOD value 1..8: H*v block maps
  DevBuf<int> d_bs, d_bf, d_sb0, d_snb, d_act, d_sc0, d_snc;
  DevBuf<Chunk> d_chunks;
  std::vector<DevBuf<int>> d_gbs, d_gbf;
  std::vector<int> gnblk;

  void build(const std::vector<BSeg>& segs, const std::vector<char>& on, cudaStream_t st) {
    nseg = (int)segs.size();
    active.clear();
    std::vector<int> bs, bf, sb0(nseg, 0), snb(nseg, 0), sc0(nseg, 0), snc(nseg, 0);
    std::vector<Chunk> ch;
    grp_bs.assign(9, {});
    grp_bf.assign(9, {});
    for (int s = 0; s < nseg; ++s) {
      if (!on[s]) continue;
      active.push_back(s);
      const int nb = (int)((segs[s].D + kB - 1) / kB);
      sb0[s] = (int)bs.size();
      snb[s] = nb;
      const int first = (int)bs.size();
      auto& gb = grp_bs[nod_of[s]];
      auto& gf = grp_bf[nod_of[s]];
      const int gfirst = (int)gb.size();
      for (int b = 0; b < nb; ++b) {
        bs.push_back(s);
        bf.push_back(first);
        gb.push_back(s);
        gf.push_back(gfirst);
      }
      sc0[s] = (int)ch.size();
      for (int64_t t = 0; t < segs[s].D; t += (int64_t)kB * kChunkTiles) {
        Chunk c;
        c.row0 = segs[s].row0 + t;
        c.n = (int)std::min<int64_t>((int64_t)kB * kChunkTiles, segs[s].D - t);
        c.seg = s;
        ch.push_back(c);
      }
      snc[s] = (int)ch.size() - sc0[s];
    }
    nact = (int)active.size();
    nblk = (int)bs.size();
    nchunk = (int)ch.size();
    auto up = [&](DevBuf<int>& d, const std::vector<int>& h) {
      d.alloc(std::max<size_t>(1, h.size()));
      if (!h.empty()) QS3G_CHECK_CUDA(cudaMemcpyAsync(d.get(), h.data(), h.size() * 4, cudaMemcpyHostToDevice, st));
    };
    up(d_bs, bs); up(d_bf, bf); up(d_sb0, sb0); up(d_snb, snb); up(d_act, active); up(d_sc0, sc0); up(d_snc, snc);
    d_chunks.alloc(std::max<size_t>(1, ch.size()));
    if (!ch.empty())
      QS3G_CHECK_CUDA(cudaMemcpyAsync(d_chunks.get(), ch.data(), ch.size() * sizeof(Chunk), cudaMemcpyHostToDevice, st));
    d_gbs.clear(); d_gbf.clear();
    d_gbs.resize(9); d_gbf.resize(9);
    gnblk.assign(9, 0);
    for (int g = 1; g <= 8; ++g) {
      gnblk[g] = (int)grp_bs[g].size();
      up(d_gbs[g], grp_bs[g]);
      up(d_gbf[g], grp_bf[g]);
    }
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));  // host vectors go out of scope
  }
};

struct SegState {
  std::vector<double> ene;
  std::vector<zd> Cc, calpha, cbeta, Tm;
  int flag = 0, stall = 0, hv = 0;
  double best = 1e300;
  bool done = false, converged = false;
};

// Lock-step TRLan on the problems marked in `on`, from V[:,0] of each.
// On return each problem's V[:, :NOE] holds its Ritz vectors, ene[s] its
// Ritz values (shifted back), and conv[s] whether it met the test.
template <class T>
void lockstep_core(const std::vector<BSeg>& segs, const DevBuf<HvSeg>& d_hs, const std::vector<int>& nod_of,
                   std::vector<char> on, T* V, int64_t ldv, T* Q, int NOE, int NOK, int NOM, int maxitr,
                   double tol, int conv_mode, const std::vector<double>& shift, std::vector<std::vector<double>>& ene,
                   std::vector<char>& conv, std::vector<int>& hv, cudaStream_t st) {
  const int n = (int)segs.size();
  const int64_t Ls = NOM + 2;  // per-problem stride of the scalar arrays
  DevBuf<BSeg> d_segs(n);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_segs.get(), segs.data(), n * sizeof(BSeg), cudaMemcpyHostToDevice, st));
  DevBuf<double2> alpha((size_t)n * Ls), beta((size_t)n * Ls), ov((size_t)n * Ls), cb((size_t)n * Ls);
  DevBuf<double2> C((size_t)n * NOM * NOK);
  Maps mp;
  mp.nod_of = nod_of;
  mp.build(segs, on, st);
  int64_t maxchunk = 0;
  for (auto& s : segs) maxchunk += (s.D + (int64_t)kB * kChunkTiles - 1) / ((int64_t)kB * kChunkTiles);
  int64_t maxblk = 0;
  for (auto& s : segs) maxblk += (s.D + kB - 1) / kB;
  DevBuf<double2> part((size_t)std::max<int64_t>(maxblk, (int64_t)(NOM + 1) * maxchunk) + 1);
  std::vector<SegState> S(n);
  auto col = [&](int j) { return V + (int64_t)j * ldv; };
  const BSeg* sg = d_segs.get();

  auto hvop = [&](const T* x, T* y) {
    for (int g = 1; g <= 8; ++g) {
      if (mp.gnblk[g] == 0) continue;
      if constexpr (sizeof(T) == sizeof(float2))
        hv32_seg(g, d_hs.get(), mp.d_gbs[g].get(), mp.d_gbf[g].get(), mp.gnblk[g], reinterpret_cast<const float2*>(x),
                 reinterpret_cast<float2*>(y), st);
      else
        hv64_seg(g, d_hs.get(), mp.d_gbs[g].get(), mp.d_gbf[g].get(), mp.gnblk[g], reinterpret_cast<const double2*>(x),
                 reinterpret_cast<double2*>(y), 0.0, st);
    }
    for (int s : mp.active) ++S[s].hv;
  };
  auto final_ = [&](double2* out, int mode) {
    k_bfinal<<<mp.nact, kB, 0, st>>>(part.get(), mp.d_sb0.get(), mp.d_snb.get(), mp.d_act.get(), out, Ls, mode);
    check_launch("k_bfinal");
  };
  auto dot = [&](const T* x, const T* y, double2* out) {
    k_bdot<T><<<mp.nblk, kB, 0, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), x, y, part.get());
    check_launch("k_bdot");
    final_(out, 0);
  };
  auto nrm = [&](const T* x, double2* out) {
    k_bnrm<T><<<mp.nblk, kB, 0, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), x, part.get());
    check_launch("k_bnrm");
    final_(out, 1);
  };
  auto scale = [&](T* x, const double2* s) {
    k_bscale<T><<<mp.nblk, kB, 0, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), x, s, Ls);
    check_launch("k_bscale");
  };
  auto lw = [&](T* w, const T* q, const T* v, const T* u, const double2* a, const double2* b, bool real_alpha) {
    k_blanczos_w<T><<<mp.nblk, kB, 0, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), w, q, v, u, a, b, Ls,
                                             real_alpha ? 1 : 0);
    check_launch("k_blanczos_w");
  };
  auto gsub = [&](int ncols, const double2* coef, T* w) {
    k_bgemv_sub<T><<<mp.nblk, kB, 0, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), V, ldv, ncols, coef, (int)Ls, w);
    check_launch("k_bgemv_sub");
  };
  auto reorth = [&](int i) {  // against columns 0..i-2
    const int ncols = i - 1;
    if (ncols <= 0) return;
    k_bgemv_h<T><<<dim3((unsigned)((ncols + 3) / 4), (unsigned)mp.nchunk), kB, 0, st>>>(V, ldv, ncols, col(i),
                                                                                        mp.d_chunks.get(), part.get());
    check_launch("k_bgemv_h");
    k_bgemv_final<<<dim3((unsigned)ncols, (unsigned)mp.nact), kB, 0, st>>>(part.get(), mp.nchunk, mp.d_sc0.get(),
                                                                         mp.d_snc.get(), mp.d_act.get(), ov.get(),
                                                                         (int)Ls);
    check_launch("k_bgemv_final");
    gsub(ncols, ov.get(), col(i));
  };
  const size_t rsm = ((size_t)NOM * NOK + (size_t)NOM * 32) * sizeof(float4);
  QS3G_CHECK_CUDA(cudaFuncSetAttribute(k_brestart<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
  std::vector<double2> ha((size_t)n * Ls), hb((size_t)n * Ls);
  auto fetch = [&]() {
    QS3G_CHECK_CUDA(cudaMemcpyAsync(ha.data(), alpha.get(), ha.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(hb.data(), beta.get(), hb.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  };

  // ---- initial Lanczos pass
  nrm(col(0), beta.get());
  for (int i = 1; i <= NOM; ++i) {
    scale(col(i - 1), beta.get() + (i - 1));
    hvop(col(i - 1), Q);
    dot(col(i - 1), Q, alpha.get() + i);
    if (i > 1) {
      lw(col(i), Q, col(i - 1), col(i - 2), alpha.get() + i, beta.get() + (i - 1), true);
      reorth(i);
    } else {
      lw(col(i), Q, col(i - 1), nullptr, alpha.get() + i, beta.get(), true);
    }
    nrm(col(i), beta.get() + i);
  }
  scale(col(NOM), beta.get() + NOM);
  fetch();
  for (int s : mp.active) {
    SegState& x = S[s];
    const double2* a = ha.data() + s * Ls;
    const double2* b = hb.data() + s * Ls;
    for (int i = 0; i <= NOM; ++i)
      QS3G_REQUIRE(std::isfinite(b[i].x) && b[i].x > 0.0 && std::isfinite(a[i < 1 ? 1 : i].x), QS3G_EBREAKDOWN,
                   "Lanczos breakdown in the initial pass of a batched problem");
    x.Tm.assign((size_t)NOM * NOM, zd(0.0, 0.0));
    for (int j = 0; j < NOM; ++j) x.Tm[j + (size_t)j * NOM] = a[j + 1].x;
    for (int j = 0; j < NOM - 1; ++j) x.Tm[j + (size_t)(j + 1) * NOM] = b[j + 1].x;
    herm_jacobi(NOM, x.Tm, x.ene, x.Cc);
    x.calpha.assign(NOM + 1, 0.0);
    x.cbeta.assign(NOM + 1, 0.0);
    for (int j = 1; j <= NOM; ++j) x.calpha[j] = a[j].x;
    for (int j = 0; j <= NOM; ++j) x.cbeta[j] = b[j].x;
  }
  std::vector<double2> hC((size_t)n * NOM * NOK), hcb((size_t)n * Ls);
  for (int tritr = 1; tritr <= maxitr; ++tritr) {
    for (int s : mp.active)
      for (int j = 0; j < NOK; ++j)
        for (int i = 0; i < NOM; ++i) {
          const zd c = S[s].Cc[i + (size_t)j * NOM];
          hC[(size_t)s * NOM * NOK + (size_t)j * NOM + i] = make_double2(c.real(), c.imag());
        }
    QS3G_CHECK_CUDA(cudaMemcpyAsync(C.get(), hC.data(), hC.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    k_brestart<T><<<mp.nblk, kB, rsm, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), V, ldv, NOM, NOK, C.get());
    check_launch("k_brestart");
    // convergence per problem (trlan_core's rule)
    bool changed = false;
    for (int s : mp.active) {
      SegState& x = S[s];
      double mc = 0.0;
      if (conv_mode == 0) {
        for (int j = 0; j < NOK; ++j) mc = std::max(mc, std::abs(x.calpha[j + 1] / x.ene[j] - 1.0));
      } else {
        for (int j = 0; j < NOE; ++j) {
          double rj = std::abs(x.cbeta[NOM] * x.Cc[(NOM - 1) + (size_t)j * NOM]);
          if (conv_mode == 2) rj /= std::max(1.0, std::fabs(x.ene[j] + shift[s]));
          mc = std::max(mc, rj);
        }
      }
      x.flag = (mc < tol) ? x.flag + 1 : 0;
      if ((conv_mode == 0 && x.flag == 2) || (conv_mode != 0 && x.flag >= 1)) {
        x.done = x.converged = true;
      } else if (conv_mode == 2) {
        if (mc < 0.95 * x.best) { x.best = mc; x.stall = 0; }
        else if (++x.stall >= 20) x.done = true;
      }
      if (tritr == maxitr) x.done = true;
      if (x.done) { on[s] = 0; changed = true; }
    }
    if (verbose())
      std::printf("batched trlan: restart %d, %d of %d problems active\n", tritr, mp.nact, n);
    if (changed) mp.build(segs, on, st);
    if (mp.nact == 0) break;
    QS3G_CHECK_CUDA(cudaMemcpyAsync(col(NOK), col(NOM), ldv * sizeof(T), cudaMemcpyDeviceToDevice, st));
    for (int s : mp.active) {
      SegState& x = S[s];
      for (int j = 0; j < NOK; ++j) x.calpha[j + 1] = x.ene[j];
      for (int j = 1; j <= NOK; ++j) x.cbeta[j] = x.cbeta[NOM] * x.Cc[(NOM - 1) + (size_t)(j - 1) * NOM];
      for (int j = 0; j < NOK; ++j) hcb[(size_t)s * Ls + j] = make_double2(x.cbeta[j + 1].real(), x.cbeta[j + 1].imag());
    }
    QS3G_CHECK_CUDA(cudaMemcpyAsync(cb.get(), hcb.data(), hcb.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    int i = NOK + 1;
    hvop(col(i - 1), Q);
    dot(col(i - 1), Q, alpha.get() + i);
    gsub(NOK, cb.get(), Q);
    lw(col(i), Q, col(i - 1), nullptr, alpha.get() + i, beta.get(), false);
    reorth(i);
    nrm(col(i), beta.get() + i);
    for (i = NOK + 2; i <= NOM; ++i) {
      scale(col(i - 1), beta.get() + (i - 1));
      hvop(col(i - 1), Q);
      dot(col(i - 1), Q, alpha.get() + i);
      lw(col(i), Q, col(i - 1), col(i - 2), alpha.get() + i, beta.get() + (i - 1), false);
      reorth(i);
      nrm(col(i), beta.get() + i);
    }
    scale(col(NOM), beta.get() + NOM);
    fetch();
    for (int s : mp.active) {
      SegState& x = S[s];
      const double2* a = ha.data() + s * Ls;
      const double2* b = hb.data() + s * Ls;
      for (int j = NOK + 1; j <= NOM; ++j) {
        x.calpha[j] = zd(a[j].x, a[j].y);
        x.cbeta[j] = b[j].x;
        QS3G_REQUIRE(std::isfinite(b[j].x) && b[j].x > 0.0 && std::isfinite(a[j].x), QS3G_EBREAKDOWN,
                     "Lanczos breakdown after a restart of a batched problem");
      }
      std::fill(x.Tm.begin(), x.Tm.end(), zd(0.0, 0.0));
      for (int j = 0; j < NOM; ++j) x.Tm[j + (size_t)j * NOM] = x.calpha[j + 1];
      for (int j = 0; j < NOK; ++j) x.Tm[j + (size_t)NOK * NOM] = x.cbeta[j + 1];
      for (int j = NOK + 1; j <= NOM - 1; ++j) x.Tm[(j - 1) + (size_t)j * NOM] = x.cbeta[j];
      herm_jacobi(NOM, x.Tm, x.ene, x.Cc);
    }
  }
  for (int s = 0; s < n; ++s) {
    if (S[s].ene.empty()) continue;  // not part of this run
    ene[s].assign(S[s].ene.begin(), S[s].ene.begin() + NOE);
    for (double& e : ene[s]) e += shift[s];
    conv[s] = S[s].converged ? 1 : 0;
    hv[s] += S[s].hv;
  }
}

}  // namespace

int trlan_lockstep(const std::vector<const Model*>& models, const std::vector<const Sector*>& secs,
                   const TrlanParams& p, double* ene_out, double* resid_out, int* hv_out, int* status,
                   cudaStream_t st) {
  const int n = (int)secs.size();
  int NOM = p.NOM;
  const int NOE = p.NOE, NOK = p.NOK;
  QS3G_REQUIRE(NOE >= 1 && NOK >= 1 && NOE <= NOK, QS3G_EINVAL, "need 1 <= NOE <= NOK");
  if (NOM < 2 * NOK) NOM = 2 * NOK;
  QS3G_REQUIRE(NOM <= 120 && NOK <= 120, QS3G_EINVAL, "NOM must be <= 120");
  QS3G_REQUIRE(p.precision == 1 || p.precision == 2, QS3G_EINVAL, "the lock-step batch runs precision 1 or 2");
  std::vector<BSeg> segs(n);
  std::vector<int> nod_of(n);
  std::vector<HvSeg> hs(n);
  std::vector<double> shift(n, 0.0), zero(n, 0.0);
  int64_t rows = 0;
  for (int s = 0; s < n; ++s) {
    QS3G_REQUIRE(secs[s]->anchored && !secs[s]->u1, QS3G_ENOTSUP, "the lock-step batch serves chain sectors");
    QS3G_REQUIRE(secs[s]->D >= NOM, QS3G_EINVAL, "sector dimension smaller than NOM (stop 999)");
    segs[s] = BSeg{rows, secs[s]->D};
    hs[s] = make_seg(*models[s], *secs[s], rows);
    hs[s].shift = models[s]->Sz_all;
    shift[s] = models[s]->Sz_all;
    nod_of[s] = secs[s]->NOD;
    rows += (secs[s]->D + kB - 1) / kB * kB;
  }
  const int64_t ldv = (rows + 31) / 32 * 32;
  DevBuf<HvSeg> d_hs(std::max(1, n));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_hs.get(), hs.data(), n * sizeof(HvSeg), cudaMemcpyHostToDevice, st));
  DevBuf<BSeg> d_segs(std::max(1, n));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_segs.get(), segs.data(), n * sizeof(BSeg), cudaMemcpyHostToDevice, st));
  std::vector<char> on(n, 1), conv(n, 0);
  std::vector<std::vector<double>> ene(n);
  std::vector<int> hv(n, 0);
  DevBuf<double2> V64((size_t)ldv * (NOM + 1)), Q64(ldv);
  QS3G_CHECK_CUDA(cudaMemsetAsync(V64.get(), 0, (size_t)ldv * (NOM + 1) * sizeof(double2), st));
  QS3G_CHECK_CUDA(cudaMemsetAsync(Q64.get(), 0, ldv * sizeof(double2), st));
  Maps all;
  all.nod_of = nod_of;
  all.build(segs, on, st);
  if (p.precision == 1) {
    DevBuf<float2> V32((size_t)ldv * (NOM + 1)), Q32(ldv);
    QS3G_CHECK_CUDA(cudaMemsetAsync(V32.get(), 0, (size_t)ldv * (NOM + 1) * sizeof(float2), st));
    QS3G_CHECK_CUDA(cudaMemsetAsync(Q32.get(), 0, ldv * sizeof(float2), st));
    k_bstart<float2><<<all.nblk, kB, 0, st>>>(d_segs.get(), all.d_bs.get(), all.d_bf.get(), V32.get(), p.seed);
    check_launch("k_bstart");
    const double tol1 = phase1_tol(p.tol32);
    lockstep_core<float2>(segs, d_hs, nod_of, on, V32.get(), ldv, Q32.get(), NOE, NOK, NOM, p.maxitr, tol1, 2, shift,
                          ene, conv, hv, st);
    // phase 2 start: the sum of the NOE Ritz vectors, widened to FP64
    k_bto64<<<sgrid(ldv), 256, 0, st>>>(V64.get(), V32.get(), ldv);
    check_launch("k_bto64");
    for (int j = 1; j < NOE; ++j) {
      k_bto64<<<sgrid(ldv), 256, 0, st>>>(Q64.get(), V32.get() + (int64_t)j * ldv, ldv);
      check_launch("k_bto64");
      Ops<double2> o{st, nullptr};
      DevBuf<double2> one(1);
      const double2 h1 = make_double2(1.0, 0.0);
      QS3G_CHECK_CUDA(cudaMemcpyAsync(one.get(), &h1, sizeof h1, cudaMemcpyHostToDevice, st));
      o.axpy(V64.get(), Q64.get(), ldv, one.get(), 1.0);
      QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    }
  } else {
    k_bstart<double2><<<all.nblk, kB, 0, st>>>(d_segs.get(), all.d_bs.get(), all.d_bf.get(), V64.get(), p.seed);
    check_launch("k_bstart");
  }
  // complex(8) phase with double-float arithmetic, then FP64 residual checks;
  // problems whose recomputed residual misses the target continue
  double tol_est = p.conv_mode == 0 ? p.tol : 0.5 * p.tol;
  std::vector<char> todo(n, 1);
  std::vector<double> res((size_t)n * NOE, 0.0);
  DevBuf<double2> W(ldv), part((size_t)all.nblk + 1);
  DevBuf<double> d_e(std::max(1, n));
  DevBuf<double2> d_r((size_t)std::max(1, n) * 1);
  for (int attempt = 0; attempt < 4; ++attempt) {
    std::fill(conv.begin(), conv.end(), 0);
    lockstep_core<double2>(segs, d_hs, nod_of, todo, V64.get(), ldv, Q64.get(), NOE, NOK, NOM, p.maxitr, tol_est,
                           p.conv_mode, zero, ene, conv, hv, st);
    if (p.conv_mode == 0) break;
    // residual of every Ritz pair of the problems just solved
    Maps mp;
    mp.nod_of = nod_of;
    mp.build(segs, todo, st);
    double worst = 0.0;
    std::vector<double> he(n, 0.0);
    for (int j = 0; j < NOE; ++j) {
      for (int s : mp.active) he[s] = ene[s][j];
      QS3G_CHECK_CUDA(cudaMemcpyAsync(d_e.get(), he.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
      const double2* pj = V64.get() + (int64_t)j * ldv;
      for (int g = 1; g <= 8; ++g)
        if (mp.gnblk[g])
          hv64_seg(g, d_hs.get(), mp.d_gbs[g].get(), mp.d_gbf[g].get(), mp.gnblk[g], pj, Q64.get(), 0.0, st);
      k_bresid<<<mp.nblk, kB, 0, st>>>(d_segs.get(), mp.d_bs.get(), mp.d_bf.get(), W.get(), Q64.get(), pj, d_e.get());
      check_launch("k_bresid");
      k_bnrm<double2><<<mp.nblk, kB, 0, st>>>(d_segs.get(), mp.d_bs.get(), mp.d_bf.get(), W.get(), part.get());
      check_launch("k_bnrm");
      DevBuf<double2> rr(std::max(1, n));
      k_bfinal<<<mp.nact, kB, 0, st>>>(part.get(), mp.d_sb0.get(), mp.d_snb.get(), mp.d_act.get(), rr.get(), 1, 1);
      check_launch("k_bfinal");
      std::vector<double2> hr(n);
      QS3G_CHECK_CUDA(cudaMemcpyAsync(hr.data(), rr.get(), n * sizeof(double2), cudaMemcpyDeviceToHost, st));
      QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
      for (int s : mp.active) {
        res[(size_t)s * NOE + j] = hr[s].x;
        hv[s] += 1;
      }
    }
    bool again = false;
    for (int s = 0; s < n; ++s) {
      if (!todo[s]) continue;
      double w = 0.0;
      for (int j = 0; j < NOE; ++j) {
        const double sc = p.conv_mode == 2 ? std::max(1.0, std::fabs(ene[s][j])) : 1.0;
        w = std::max(w, res[(size_t)s * NOE + j] / sc);
      }
      worst = std::max(worst, w);
      if (w <= p.tol || !conv[s]) todo[s] = 0;  // done, or capped by maxitr
      else again = true;
    }
    if (verbose()) std::printf("batched trlan: attempt %d, worst recomputed residual %.3e\n", attempt, worst);
    if (!again) break;
    tol_est *= 0.1;
    // continue the failing problems from the sum of their Ritz vectors
    Maps mp2;
    mp2.nod_of = nod_of;
    mp2.build(segs, todo, st);
    for (int j = 1; j < NOE; ++j) {
      DevBuf<double2> cone((size_t)n * (NOM + 2));
      std::vector<double2> hc((size_t)n * (NOM + 2), make_double2(0.0, 0.0));
      for (int s = 0; s < n; ++s) hc[(size_t)s * (NOM + 2)] = make_double2(-1.0, 0.0);
      QS3G_CHECK_CUDA(cudaMemcpyAsync(cone.get(), hc.data(), hc.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
      // V[:,0] -= (-1) * V[:,j]  (one column through the batched subtraction)
      k_bgemv_sub<double2><<<mp2.nblk, kB, 0, st>>>(d_segs.get(), mp2.d_bs.get(), mp2.d_bf.get(),
                                                    V64.get() + (int64_t)j * ldv, ldv, 1, cone.get(), NOM + 2,
                                                    V64.get());
      check_launch("k_bgemv_sub");
      QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    }
  }
  for (int s = 0; s < n; ++s) {
    for (int j = 0; j < NOE; ++j) {
      ene_out[(size_t)s * NOE + j] = ene[s].empty() ? NAN : ene[s][j];
      if (resid_out) resid_out[(size_t)s * NOE + j] = res[(size_t)s * NOE + j];
    }
    if (hv_out) hv_out[s] = hv[s];
    bool ok = conv[s] != 0;
    if (p.conv_mode != 0) {
      double w = 0.0;
      for (int j = 0; j < NOE; ++j) w = std::max(w, res[(size_t)s * NOE + j]);
      ok = w <= p.tol * (p.conv_mode == 2 ? std::max(1.0, std::fabs(ene[s][0])) : 1.0);
    }
    status[s] = ok ? QS3G_OK : QS3G_ENOTCONV;
  }
  return QS3G_OK;
}

}  // namespace qs3g

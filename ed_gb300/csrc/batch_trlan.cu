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
// arrays indexed by problem; the small Ritz problems are solved on the device
// (k_britz, one block per active problem) and a whole restart cycle is
// replayed as one CUDA graph.  The steps and the convergence
// rule of each problem are those of trlan_core (krylov.cu); level-1
// arithmetic is double-float on the FP32 pipe (eft.cuh) for both storage
// types, so complex(4) phases keep FP64-accurate reductions.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "eft.cuh"
#include "krylov.h"
#include "qs3g_internal.cuh"

namespace qs3g {
namespace {

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

// One block per active problem: fixed-order sum of its blocks' partials
// (per of them for each block).
// mode 0: out[s*ld] = sum; mode 1: out[s*ld] = (sqrt(sum.x), sum.x)
__global__ void __launch_bounds__(kB) k_bfinal(const double2* part, const int* seg_b0, const int* seg_nb,
                                               const int* active, double2* out, int64_t ld, int mode, int per) {
  __shared__ double2 sh[kB];
  const int sg = active[blockIdx.x];
  const int b0 = seg_b0[sg] * per, nb = seg_nb[sg] * per;
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

// w -= V[:, :ncols] * coef_s (coefficients of problem s at coef[s*ldo]);
// with npart set, also part[b] = sum |w|^2 of the stored result (k_bnrm's
// partials, so the norm of the reorthogonalised vector needs no extra pass)
template <class T>
__global__ void __launch_bounds__(kB) k_bgemv_sub(const BSeg* segs, const int* bs, const int* bf,
                                                  const T* __restrict__ V, int64_t ldv, int ncols,
                                                  const double2* __restrict__ coef, int ldo, T* w, double2* npart) {
  __shared__ float4 c[128];
  __shared__ double2 sh[kB];
  const int sg = bs[blockIdx.x];
  for (int k = threadIdx.x; k < ncols; k += kB) {
    const double2 ck = coef[(size_t)sg * ldo + k];
    const float2 r = split(ck.x), m = split(ck.y);
    c[k] = make_float4(r.x, r.y, m.x, m.y);
  }
  __syncthreads();
  int64_t r;
  int sg2;
  float nh = 0.f, nl = 0.f;
  if (brow(segs, bs, bf, r, sg2)) {
    T out;
    if constexpr (sizeof(T) == sizeof(float2)) {
      // complex(4) columns: FP32 FMAs with the coefficients' hi and lo parts
      // summed apart (the single-problem subtraction's arithmetic); the
      // result is stored in FP32 either way
      const float2 wv = reinterpret_cast<const float2*>(w)[r];
      float re = wv.x, im = wv.y, rlo = 0.f, ilo = 0.f;
      for (int k = 0; k < ncols; ++k) {
        const float2 a = reinterpret_cast<const float2*>(V)[(int64_t)k * ldv + r];
        const float4 ck = c[k];
        rlo = fmaf(-ck.y, a.x, rlo);
        ilo = fmaf(-ck.y, a.y, ilo);
        re = fmaf(-ck.x, a.x, re);
        im = fmaf(-ck.x, a.y, im);
        rlo = fmaf(ck.w, a.y, rlo);
        ilo = fmaf(-ck.w, a.x, ilo);
        re = fmaf(ck.z, a.y, re);
        im = fmaf(-ck.z, a.x, im);
      }
      out = Store<T>::st(re, rlo, im, ilo);
    } else {
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
      out = Store<T>::st(wrh, wrl, wih, wil);
    }
    w[r] = out;
    if (npart) {
      const float4 a = SplitLd<T>::ld(out);
      df_fma(nh, nl, make_float2(a.x, a.y), make_float2(a.x, a.y));
      df_fma(nh, nl, make_float2(a.z, a.w), make_float2(a.z, a.w));
    }
  }
  if (npart) {
    const double2 t = block_sum2(make_double2(djoin(nh, nl), 0.0), sh);
    if (threadIdx.x == 0) npart[blockIdx.x] = t;
  }
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
        if constexpr (sizeof(T) == sizeof(float2)) {
          // complex(4) outputs: plain FP32 sums of the hi parts (they are
          // stored in FP32)
          for (int j = 0; j < nom; ++j) {
            const float4 a = tile[j * 32 + rr];
            const float4 c = cs[(size_t)oc * nom + j];
            rh = fmaf(a.x, c.x, rh);
            rh = fmaf(-a.z, c.z, rh);
            ih = fmaf(a.x, c.z, ih);
            ih = fmaf(a.z, c.x, ih);
          }
        } else {
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

// ------------------------------------------------------------------ device Ritz solves
// One block per active problem, at the end of every Lanczos cycle: take the
// cycle's alpha/beta into the problem's projected matrix -- tridiagonal after
// the initial pass, arrowhead plus tridiagonal after a thick restart
// (eigen_solver.f90:196-203) --, diagonalise it with a parallel cyclic Jacobi
// method (round-robin pairs, each rotation herm_jacobi's), sort ascending,
// and do trlan_core's restart bookkeeping on the device: the Ritz
// coefficients C (NOM x NOK) for the next restart, the convergence test
// (eigen_solver.f90:150-159, or the Ritz residual |beta_NOM C(NOM, j)|), the
// retained Ritz values and the arrow couplings of the next cycle.  The host
// only reads the per-problem flags.
constexpr int kMaxRitz = 120;      // NOM limit of the lock-step batch
constexpr int kRitzSmemMax = 80;   // above this the two NOM x NOM matrices live in global scratch

struct RitzState {
  int flag, stall, done, conv, tritr, brk;
  double best;
};

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 zaxpby(double2 a, double2 x, double2 b, double2 y) {
  const double2 p = zmul(a, x), q = zmul(b, y);
  return make_double2(p.x + q.x, p.y + q.y);
}

__global__ void __launch_bounds__(256) k_britz(const int* __restrict__ act, int first, int NOM, int NOK, int NOE,
                                               int maxitr, double tol, int conv_mode, const double* __restrict__ shift,
                                               const double2* __restrict__ alpha, const double2* __restrict__ beta,
                                               double2* calpha, double2* cbeta, double2* C, double2* cb, double* ene,
                                               RitzState* rs, int Ls, double2* scratch) {
  extern __shared__ float4 smr[];  // same declaration as k_brestart's
  const int n = NOM;
  const int s = act[blockIdx.x];
  // A: the projected matrix, Z: its eigenvectors (both n x n column-major)
  double2* A = scratch ? scratch + (size_t)s * 2 * n * n : reinterpret_cast<double2*>(smr);
  double2* Z = A + n * n;
  __shared__ double w[kMaxRitz], red[256];
  __shared__ int ord[kMaxRitz];
  __shared__ int rp[kMaxRitz / 2], rq[kMaxRitz / 2];
  __shared__ double rc[kMaxRitz / 2], rsn[kMaxRitz / 2];
  __shared__ double2 rqp[kMaxRitz / 2], rqq[kMaxRitz / 2];
  __shared__ int brk;
  const int tid = threadIdx.x;
  const double2* a = alpha + (size_t)s * Ls;
  const double2* b = beta + (size_t)s * Ls;
  double2* ca = calpha + (size_t)s * Ls;
  double2* cbt = cbeta + (size_t)s * Ls;
  if (tid == 0) brk = 0;
  __syncthreads();
  // 1. this cycle's scalars
  if (first) {
    for (int j = tid; j <= n; j += blockDim.x) {
      if (j >= 1) ca[j] = make_double2(a[j].x, 0.0);
      cbt[j] = make_double2(b[j].x, 0.0);
      if (!(isfinite(b[j].x) && b[j].x > 0.0) || (j >= 1 && !isfinite(a[j].x))) brk = 1;
    }
  } else {
    for (int j = NOK + 1 + tid; j <= n; j += blockDim.x) {
      ca[j] = a[j];
      cbt[j] = make_double2(b[j].x, 0.0);
      if (!(isfinite(b[j].x) && b[j].x > 0.0) || !isfinite(a[j].x)) brk = 1;
    }
  }
  __syncthreads();
  if (brk) {
    if (tid == 0) { rs[s].brk = 1; rs[s].done = 1; }
    return;
  }
  // 2. the projected matrix (full Hermitian storage)
  for (int e = tid; e < n * n; e += blockDim.x) {
    A[e] = make_double2(0.0, 0.0);
    Z[e] = make_double2((e % n) == (e / n) ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  if (tid == 0) {
    auto setu = [&](int i, int j, double2 v) {  // upper (i < j) and its conjugate
      A[i + (size_t)j * n] = v;
      A[j + (size_t)i * n] = zconj(v);
    };
    for (int j = 0; j < n; ++j) A[j + (size_t)j * n] = make_double2(ca[j + 1].x, 0.0);
    if (first) {
      for (int j = 0; j < n - 1; ++j) setu(j, j + 1, make_double2(b[j + 1].x, 0.0));
    } else {
      for (int j = 0; j < NOK; ++j) setu(j, NOK, cbt[j + 1]);
      for (int j = NOK + 1; j <= n - 1; ++j) setu(j - 1, j, cbt[j]);
    }
  }
  __syncthreads();
  // 3. parallel cyclic Jacobi: m = n rounded up to even, m - 1 rounds of m / 2
  //    disjoint pairs per sweep (circle method)
  const int m = n + (n & 1);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int e = tid; e < n * n; e += blockDim.x) {
      const double a2 = A[e].x * A[e].x + A[e].y * A[e].y;
      tot += a2;
      if ((e % n) != (e / n)) off += a2;
    }
    red[tid] = off;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
      if (tid < h) red[tid] += red[tid + h];
      __syncthreads();
    }
    const double offs = red[0];
    __syncthreads();
    red[tid] = tot;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
      if (tid < h) red[tid] += red[tid + h];
      __syncthreads();
    }
    const double tots = red[0];
    __syncthreads();
    if (offs <= 1e-34 * tots || offs == 0.0) break;
    for (int r = 0; r < m - 1; ++r) {
      if (tid < m / 2) {
        int p = (tid == 0) ? r : (r + tid) % (m - 1);
        int q = (tid == 0) ? m - 1 : (r - tid + (m - 1)) % (m - 1);
        if (p > q) { const int t = p; p = q; q = t; }
        rp[tid] = p;
        rq[tid] = q;
        rc[tid] = 1.0;
        rsn[tid] = 0.0;
        rqp[tid] = make_double2(0.0, 0.0);
        rqq[tid] = make_double2(1.0, 0.0);
        if (q < n) {
          const double2 apq = A[p + (size_t)q * n];
          const double aa = sqrt(apq.x * apq.x + apq.y * apq.y);
          if (aa != 0.0) {
            const double app = A[p + (size_t)p * n].x, aqq = A[q + (size_t)q * n].x;
            const double2 u = make_double2(apq.x / aa, apq.y / aa);
            const double tau = (aqq - app) / (2.0 * aa);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            const double c = 1.0 / sqrt(1.0 + t * t), sn = t * c;
            rc[tid] = c;
            rsn[tid] = sn;
            rqp[tid] = make_double2(-sn * u.x, sn * u.y);  // -s conj(u)
            rqq[tid] = make_double2(c * u.x, -c * u.y);    //  c conj(u)
          } else {
            rq[tid] = n;  // no rotation
          }
        }
      }
      __syncthreads();
      const int np = m / 2;
      // columns: A <- A J, Z <- Z J
      for (int it = tid; it < np * n; it += blockDim.x) {
        const int k = it / n, i = it % n;
        const int p = rp[k], q = rq[k];
        if (q >= n) continue;
        const double2 cc = make_double2(rc[k], 0.0), ss = make_double2(rsn[k], 0.0);
        const double2 aip = A[i + (size_t)p * n], aiq = A[i + (size_t)q * n];
        A[i + (size_t)p * n] = zaxpby(cc, aip, rqp[k], aiq);
        A[i + (size_t)q * n] = zaxpby(ss, aip, rqq[k], aiq);
        const double2 zip = Z[i + (size_t)p * n], ziq = Z[i + (size_t)q * n];
        Z[i + (size_t)p * n] = zaxpby(cc, zip, rqp[k], ziq);
        Z[i + (size_t)q * n] = zaxpby(ss, zip, rqq[k], ziq);
      }
      __syncthreads();
      // rows: A <- J^H A
      for (int it = tid; it < np * n; it += blockDim.x) {
        const int k = it / n, i = it % n;
        const int p = rp[k], q = rq[k];
        if (q >= n) continue;
        const double2 cc = make_double2(rc[k], 0.0), ss = make_double2(rsn[k], 0.0);
        const double2 api = A[p + (size_t)i * n], aqi = A[q + (size_t)i * n];
        A[p + (size_t)i * n] = zaxpby(cc, api, zconj(rqp[k]), aqi);
        A[q + (size_t)i * n] = zaxpby(ss, api, zconj(rqq[k]), aqi);
      }
      __syncthreads();
      if (tid < np) {
        const int p = rp[tid], q = rq[tid];
        if (q < n) {
          A[p + (size_t)q * n] = make_double2(0.0, 0.0);
          A[q + (size_t)p * n] = make_double2(0.0, 0.0);
          A[p + (size_t)p * n].y = 0.0;
          A[q + (size_t)q * n].y = 0.0;
        }
      }
      __syncthreads();
    }
  }
  // 4. ascending order
  if (tid == 0) {
    for (int i = 0; i < n; ++i) { w[i] = A[i + (size_t)i * n].x; ord[i] = i; }
    for (int i = 1; i < n; ++i) {  // stable insertion sort of the indices
      const int oi = ord[i];
      int j = i - 1;
      while (j >= 0 && w[ord[j]] > w[oi]) { ord[j + 1] = ord[j]; --j; }
      ord[j + 1] = oi;
    }
  }
  __syncthreads();
  // 5. convergence (before the retained Ritz values overwrite calpha)
  if (tid == 0) {
    RitzState st = rs[s];
    double mc = 0.0;
    if (conv_mode == 0) {
      for (int j = 0; j < NOK; ++j) mc = fmax(mc, fabs(ca[j + 1].x / w[ord[j]] - 1.0));
    } else {
      const double bN = cbt[n].x;
      for (int j = 0; j < NOE; ++j) {
        const double2 zl = Z[(n - 1) + (size_t)ord[j] * n];
        double rj = fabs(bN) * sqrt(zl.x * zl.x + zl.y * zl.y);
        if (conv_mode == 2) rj /= fmax(1.0, fabs(w[ord[j]] + shift[s]));
        mc = fmax(mc, rj);
      }
    }
    st.tritr += 1;  // one restart follows every Ritz solve
    st.flag = (mc < tol) ? st.flag + 1 : 0;
    if ((conv_mode == 0 && st.flag == 2) || (conv_mode != 0 && st.flag >= 1)) {
      st.done = 1;
      st.conv = 1;
    } else if (conv_mode == 2) {
      if (mc < 0.95 * st.best) { st.best = mc; st.stall = 0; }
      else if (++st.stall >= 20) st.done = 1;
    }
    if (st.tritr >= maxitr) st.done = 1;
    rs[s] = st;
  }
  __syncthreads();
  // 6. Ritz values, coefficients for the restart, next cycle's retained scalars
  for (int j = tid; j < n; j += blockDim.x) ene[(size_t)s * Ls + j] = w[ord[j]];
  for (int e = tid; e < n * NOK; e += blockDim.x) {
    const int j = e / n, i = e % n;
    C[(size_t)s * n * NOK + (size_t)j * n + i] = Z[i + (size_t)ord[j] * n];
  }
  __syncthreads();
  if (tid == 0) {
    const double2 bN = cbt[n];
    for (int j = 0; j < NOK; ++j) ca[j + 1] = make_double2(w[ord[j]], 0.0);
    for (int j = 1; j <= NOK; ++j) {
      const double2 zl = Z[(n - 1) + (size_t)ord[j - 1] * n];
      cbt[j] = zmul(bN, zl);
      cb[(size_t)s * Ls + (j - 1)] = cbt[j];
    }
  }
}

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

// Pinned host copy of the per-problem Ritz states (read once per cycle).
struct PinnedStates {
  RitzState* p = nullptr;
  explicit PinnedStates(size_t n) { QS3G_CHECK_CUDA(cudaMallocHost((void**)&p, std::max<size_t>(1, n) * sizeof(RitzState))); }
  ~PinnedStates() { if (p) cudaFreeHost(p); }
  PinnedStates(const PinnedStates&) = delete;
  PinnedStates& operator=(const PinnedStates&) = delete;
};

// One instantiated restart cycle; re-captured whenever the launch maps change.
struct CycleGraph {
  cudaGraphExec_t exec = nullptr;
  ~CycleGraph() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
};

// Lock-step TRLan on the problems marked in `on`, from V[:,0] of each.
// On return each problem's V[:, :NOE] holds its Ritz vectors, ene[s] its
// Ritz values (shifted back), and conv[s] whether it met the test.
//
// Per cycle everything runs on the device: the Lanczos steps of all active
// problems, k_britz (Ritz solve, convergence test, restart coefficients) and
// k_brestart, followed by one copy of the Ritz states to pinned host memory.
// A cycle is captured once into a CUDA graph and replayed until a problem
// finishes; the host then drops it from the launch maps and captures again.
template <class T>
void lockstep_core(const std::vector<BSeg>& segs, const std::vector<HvSeg>& hs, const DevBuf<HvSeg>& d_hs,
                   const std::vector<int>& nod_of,
                   std::vector<char> on, T* V, int64_t ldv, T* Q, int NOE, int NOK, int NOM, int maxitr,
                   double tol, int conv_mode, const std::vector<double>& shift, std::vector<std::vector<double>>& ene,
                   std::vector<char>& conv, std::vector<int>& hv, cudaStream_t st) {
  const int n = (int)segs.size();
  const int64_t Ls = NOM + 2;  // per-problem stride of the scalar arrays
  QS3G_REQUIRE(NOM <= kMaxRitz, QS3G_EINVAL, "NOM above the lock-step limit");
  DevBuf<BSeg> d_segs(n);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_segs.get(), segs.data(), n * sizeof(BSeg), cudaMemcpyHostToDevice, st));
  DevBuf<double2> alpha((size_t)n * Ls), beta((size_t)n * Ls), ov((size_t)n * Ls), cb((size_t)n * Ls);
  DevBuf<double2> calpha((size_t)n * Ls), cbeta((size_t)n * Ls), C((size_t)n * NOM * NOK);
  DevBuf<double> d_ene((size_t)n * Ls), d_shift(n);
  DevBuf<RitzState> d_rs(n);
  QS3G_CHECK_CUDA(cudaMemsetAsync(C.get(), 0, C.n * sizeof(double2), st));
  QS3G_CHECK_CUDA(cudaMemsetAsync(d_ene.get(), 0, d_ene.n * sizeof(double), st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_shift.get(), shift.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  PinnedStates h_rs(n);
  for (int s = 0; s < n; ++s) h_rs.p[s] = RitzState{0, 0, 0, 0, 0, 0, 1e300};
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_rs.get(), h_rs.p, n * sizeof(RitzState), cudaMemcpyHostToDevice, st));
  const bool ritz_smem = NOM <= kRitzSmemMax;
  DevBuf<double2> ritz_scratch(ritz_smem ? 0 : (size_t)n * 2 * NOM * NOM);
  const size_t ritz_sm = ritz_smem ? (size_t)2 * NOM * NOM * sizeof(double2) : 0;
  if (ritz_smem)
    QS3G_CHECK_CUDA(cudaFuncSetAttribute(k_britz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ritz_sm));
  Maps mp;
  mp.nod_of = nod_of;
  mp.build(segs, on, st);
  int64_t maxchunk = 0;
  for (auto& s : segs) maxchunk += (s.D + (int64_t)kB * kChunkTiles - 1) / ((int64_t)kB * kChunkTiles);
  int64_t maxblk = 0;
  for (auto& s : segs) maxblk += (s.D + kB - 1) / kB;
  DevBuf<double2> part((size_t)std::max<int64_t>(kSegPartials * maxblk, (int64_t)(NOM + 1) * maxchunk) + 1);
  std::vector<int> hv_run(n, 0);
  auto col = [&](int j) { return V + (int64_t)j * ldv; };
  const BSeg* sg = d_segs.get();

  auto final_ = [&](double2* out, int mode, int per) {
    k_bfinal<<<mp.nact, kB, 0, st>>>(part.get(), mp.d_sb0.get(), mp.d_snb.get(), mp.d_act.get(), out, Ls, mode,
                                      per);
    check_launch("k_bfinal");
  };
  // Row form per NOD group: the general chain row, the same with its
  // general-path hops deferred to the end of the row (short chains send many
  // hops there, and a warp otherwise pays for every hop position at which any
  // of its rows does), or -- when every chain of the group is uniform with the
  // same number of bond distances -- the unrolled uniform row.  The fastest
  // on this batch's own data is kept; QS3G_SEG_FORM = general, deferred or
  // uniform pins the choice.
  std::vector<int> seg_uni(9, 0);
  auto hv_group = [&](int g, int uni, const T* x, T* y, double2* pp) {
    if constexpr (sizeof(T) == sizeof(float2))
      hv32_seg(g, d_hs.get(), mp.d_gbs[g].get(), mp.d_gbf[g].get(), mp.gnblk[g], reinterpret_cast<const float2*>(x),
               reinterpret_cast<float2*>(y), st, pp, mp.d_sb0.get(), uni);
    else
      hv64_seg(g, d_hs.get(), mp.d_gbs[g].get(), mp.d_gbf[g].get(), mp.gnblk[g], reinterpret_cast<const double2*>(x),
               reinterpret_cast<double2*>(y), 0.0, st, pp, mp.d_sb0.get(), uni);
  };
  {
    const char* env = std::getenv("QS3G_SEG_FORM");
    const std::string form = env ? env : "auto";
    cudaEvent_t e0, e1;
    QS3G_CHECK_CUDA(cudaEventCreate(&e0));
    QS3G_CHECK_CUDA(cudaEventCreate(&e1));
    for (int g = 1; g <= 8; ++g) {
      if (mp.gnblk[g] == 0) continue;
      int uno = -1;
      for (int s : mp.active)
        if (nod_of[s] == g) uno = (uno == -1 || uno == hs[s].uno) ? hs[s].uno : 0;
      bool tab = true;
      for (int s : mp.active)
        if (nod_of[s] == g) tab = tab && hs[s].tab != nullptr;
      std::vector<int> cand{0, 3};
      if (uno > 0 && seg_uniform_ok(g, uno)) cand.push_back(uno);
      if (tab) cand.push_back(kSegTable);
      if (form == "general") cand = {0};
      else if (form == "deferred") cand = {3};
      else if (form == "uniform") cand = {(uno > 0 && seg_uniform_ok(g, uno)) ? uno : 0};
      else if (form == "table") cand = {tab ? kSegTable : 0};
      std::vector<float> best(cand.size(), 1e30f);
      if (cand.size() > 1)
        for (int rep = 0; rep < 3; ++rep)
          for (size_t f = 0; f < cand.size(); ++f) {
            QS3G_CHECK_CUDA(cudaEventRecord(e0, st));
            hv_group(g, cand[f], col(0), Q, part.get());
            QS3G_CHECK_CUDA(cudaEventRecord(e1, st));
            QS3G_CHECK_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            QS3G_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0) best[f] = std::min(best[f], ms);  // rep 0 warms up
          }
      const size_t k = (size_t)(std::min_element(best.begin(), best.end()) - best.begin());
      seg_uni[g] = cand[k];
      if (verbose()) {
        std::printf("batched trlan: NOD %d group:", g);
        for (size_t f = 0; f < cand.size(); ++f)
          std::printf(" %s %.3f ms",
                      cand[f] == 0 ? "general"
                                   : (cand[f] == 3 ? "deferred" : (cand[f] == kSegTable ? "table" : "uniform")),
                      best[f]);
        std::printf("\n");
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  // y = H x for every active problem, with alpha = <x, y> reduced from the
  // H*v kernels' own block partials
  auto hvdot = [&](const T* x, T* y, double2* out) {
    for (int g = 1; g <= 8; ++g)
      if (mp.gnblk[g]) hv_group(g, seg_uni[g], x, y, part.get());
    final_(out, 0, kSegPartials);
  };
  auto nrm = [&](const T* x, double2* out) {
    k_bnrm<T><<<mp.nblk, kB, 0, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), x, part.get());
    check_launch("k_bnrm");
    final_(out, 1, 1);
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
  auto gsub = [&](int ncols, const double2* coef, T* w, double2* npart) {
    k_bgemv_sub<T><<<mp.nblk, kB, 0, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), V, ldv, ncols, coef, (int)Ls, w, npart);
    check_launch("k_bgemv_sub");
  };
  // column i against columns 0..i-2, then beta_i = ||column i||
  auto reorth_nrm = [&](int i) {
    const int ncols = i - 1;
    if (ncols <= 0) {
      nrm(col(i), beta.get() + i);
      return;
    }
    k_bgemv_h<T><<<dim3((unsigned)((ncols + 3) / 4), (unsigned)mp.nchunk), kB, 0, st>>>(V, ldv, ncols, col(i),
                                                                                        mp.d_chunks.get(), part.get());
    check_launch("k_bgemv_h");
    k_bgemv_final<<<dim3((unsigned)ncols, (unsigned)mp.nact), kB, 0, st>>>(part.get(), mp.nchunk, mp.d_sc0.get(),
                                                                         mp.d_snc.get(), mp.d_act.get(), ov.get(),
                                                                         (int)Ls);
    check_launch("k_bgemv_final");
    gsub(ncols, ov.get(), col(i), part.get());
    final_(beta.get() + i, 1, 1);
  };
  const size_t rsm = ((size_t)NOM * NOK + (size_t)NOM * 32) * sizeof(float4);
  QS3G_CHECK_CUDA(cudaFuncSetAttribute(k_brestart<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
  // Ritz solve + test, restart, the next cycle's first column, states to the host
  auto close_cycle = [&](int first) {
    scale(col(NOM), beta.get() + NOM);
    k_britz<<<mp.nact, 256, ritz_sm, st>>>(mp.d_act.get(), first, NOM, NOK, NOE, maxitr, tol, conv_mode,
                                           d_shift.get(), alpha.get(), beta.get(), calpha.get(), cbeta.get(), C.get(),
                                           cb.get(), d_ene.get(), d_rs.get(), (int)Ls, ritz_scratch.get());
    check_launch("k_britz");
    k_brestart<T><<<mp.nblk, kB, rsm, st>>>(sg, mp.d_bs.get(), mp.d_bf.get(), V, ldv, NOM, NOK, C.get());
    check_launch("k_brestart");
    QS3G_CHECK_CUDA(cudaMemcpyAsync(col(NOK), col(NOM), ldv * sizeof(T), cudaMemcpyDeviceToDevice, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(h_rs.p, d_rs.get(), n * sizeof(RitzState), cudaMemcpyDeviceToHost, st));
  };
  auto restart_cycle = [&]() {
    int i = NOK + 1;
    hvdot(col(i - 1), Q, alpha.get() + i);
    gsub(NOK, cb.get(), Q, nullptr);
    lw(col(i), Q, col(i - 1), nullptr, alpha.get() + i, beta.get(), false);
    reorth_nrm(i);
    for (i = NOK + 2; i <= NOM; ++i) {
      scale(col(i - 1), beta.get() + (i - 1));
      hvdot(col(i - 1), Q, alpha.get() + i);
      lw(col(i), Q, col(i - 1), col(i - 2), alpha.get() + i, beta.get() + (i - 1), false);
      reorth_nrm(i);
    }
    close_cycle(0);
  };
  // read the states of the cycle just run; true when the active set changed
  auto settle = [&](int nhv) {
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    bool changed = false;
    for (int s : mp.active) {
      hv_run[s] += nhv;
      QS3G_REQUIRE(!h_rs.p[s].brk, QS3G_EBREAKDOWN, "Lanczos breakdown in a batched problem");
      if (h_rs.p[s].done) {
        on[s] = 0;
        changed = true;
      }
    }
    return changed;
  };
  const bool can_capture = st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
  CycleGraph graph;
  auto capture = [&]() {
    graph.reset();
    if (!can_capture) return;
    cudaGraph_t g = nullptr;
    QS3G_CHECK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      restart_cycle();
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      throw;
    }
    QS3G_CHECK_CUDA(cudaStreamEndCapture(st, &g));
    const cudaError_t e = cudaGraphInstantiate(&graph.exec, g, 0);
    cudaGraphDestroy(g);
    QS3G_CHECK_CUDA(e);
  };

  const auto t_start = std::chrono::steady_clock::now();
  // ---- initial Lanczos pass
  nrm(col(0), beta.get());
  for (int i = 1; i <= NOM; ++i) {
    scale(col(i - 1), beta.get() + (i - 1));
    hvdot(col(i - 1), Q, alpha.get() + i);
    if (i > 1) lw(col(i), Q, col(i - 1), col(i - 2), alpha.get() + i, beta.get() + (i - 1), true);
    else lw(col(i), Q, col(i - 1), nullptr, alpha.get() + i, beta.get(), true);
    reorth_nrm(i);
  }
  close_cycle(1);
  bool changed = settle(NOM);
  for (int cycle = 0; cycle < maxitr && mp.nact > 0; ++cycle) {
    if (changed) {
      mp.build(segs, on, st);
      if (mp.nact == 0) break;
      graph.reset();
    }
    if (verbose())
      std::printf("batched trlan: cycle %d, %d of %d problems active (%lld rows), %.3f s\n", cycle + 1, mp.nact, n,
                  (long long)mp.nblk * kB,
                  std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count());
    if (can_capture && !graph.exec) capture();
    if (graph.exec) QS3G_CHECK_CUDA(cudaGraphLaunch(graph.exec, st));
    else restart_cycle();
    changed = settle(NOM - NOK);
  }
  std::vector<double> he((size_t)n * Ls);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(he.data(), d_ene.get(), he.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(h_rs.p, d_rs.get(), n * sizeof(RitzState), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  for (int s = 0; s < n; ++s) {
    if (h_rs.p[s].tritr == 0) continue;  // not part of this run
    ene[s].assign(he.begin() + (size_t)s * Ls, he.begin() + (size_t)s * Ls + NOE);
    for (double& e : ene[s]) e += shift[s];
    conv[s] = h_rs.p[s].conv ? 1 : 0;
    hv[s] += hv_run[s];
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
  // Connection tables for the products: the sectors' own cached ones, else
  // temporary ones while the device has room for them next to the Krylov
  // vectors (the row form itself is chosen per NOD group by timing)
  std::vector<HvTable> tmp_tab(n);
  {
    const char* env = std::getenv("QS3G_SEG_FORM");
    const std::string form = env ? env : "auto";
    if (form == "auto" || form == "table") {
      const size_t keep = (p.precision == 1 ? (size_t)ldv * (NOM + 2) * sizeof(float2) : 0) + ((size_t)2 << 30);
      for (int s = 0; s < n; ++s) {
        if (secs[s]->tab.built() || hv_table_bytes(*models[s], *secs[s]) == 0) continue;
        if (!build_hv_table(*models[s], *secs[s], tmp_tab[s], keep, st)) break;
        set_seg_table(hs[s], tmp_tab[s]);
      }
      QS3G_CHECK_CUDA(cudaMemcpyAsync(d_hs.get(), hs.data(), n * sizeof(HvSeg), cudaMemcpyHostToDevice, st));
    }
  }
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
    lockstep_core<float2>(segs, hs, d_hs, nod_of, on, V32.get(), ldv, Q32.get(), NOE, NOK, NOM, p.maxitr, tol1, 2, shift,
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
    lockstep_core<double2>(segs, hs, d_hs, nod_of, todo, V64.get(), ldv, Q64.get(), NOE, NOK, NOM, p.maxitr, tol_est,
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
      k_bfinal<<<mp.nact, kB, 0, st>>>(part.get(), mp.d_sb0.get(), mp.d_snb.get(), mp.d_act.get(), rr.get(), 1, 1,
                                        1);
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
    if (verbose()) std::fflush(stdout);
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
                                                    V64.get(), nullptr);
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

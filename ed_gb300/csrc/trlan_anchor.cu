// trlan_anchor.cu -- thick-restart Lanczos for the lowest eigenpair on FP32
// Krylov vectors anchored on one FP64 vector (qs3g_trlan precision 1, NOE = 1).
//
// The reference (lancz_eigen_val_complex, eigen_solver.f90:69-261) keeps every
// Krylov vector in complex(8).  Here the basis is B = [x, W]: x is the current
// approximation in FP64, W holds NOK-1 retained Ritz vectors and the new
// Lanczos vectors in FP32 (complex(4), or real FP32 two rows per complex
// slot).  Every cycle
//   1. recomputes H x in FP64, the Rayleigh quotient theta and the FP64
//      residual r = H x - theta x (the convergence test is on ||r|| itself);
//   2. starts the extension from r orthogonalised against x and the retained
//      vectors, and runs Lanczos steps on H - sigma (sigma = sum_b Jz_b/4, so
//      the large common diagonal never enters an FP32 rounding) with FP32
//      products and FP64-accurate (double-float) reductions and full
//      reorthogonalisation against W and x;
//   3. assembles the projected matrix G = B^H (H - sigma) B from the
//      reorthogonalisation overlaps themselves (not from an assumed
//      tridiagonal / arrowhead shape), with x's row computed exactly from
//      H x in FP64, and solves the generalized problem G c = theta M c with
//      M = B^H B (the identity except x's row: the FP32 rounding of W leaves
//      overlaps with x that a plain Rayleigh-Ritz turns into a residual floor
//      near 1e-8);
//   4. forms the new x = B c_0 in FP64 and the NOK-1 next Ritz vectors in
//      FP32 in one pass over B.
// The FP32 vectors carry the convergence all the way: they only have to
// represent the correction to x, whose size shrinks with the residual.  One
// FP64 H*v per cycle of NOM - NOK + 1 FP32 ones.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "eft.cuh"
#include "hosteig.h"
#include "krylov.h"
#include "qs3g_device.cuh"

namespace qs3g {
namespace {

constexpr int kT = 256;
constexpr int kChunks = 304;       // row chunks of the overlap kernels (2 per SM) ...
constexpr int kChunksNarrow = 1216;  // ... and for one or two columns (when the occupancy query fails)

__device__ __forceinline__ float4 split2(double2 v) {
  const float2 r = dsplit(v.x), i = dsplit(v.y);
  return make_float4(r.x, r.y, i.x, i.y);
}

// acc (re hi, re lo, im hi, im lo) += conj(a) * b, a exact in FP32, b split
template <bool RE>
__device__ __forceinline__ void acc_cdot(float4& acc, float2 a, float4 b) {
  df_add_prod(acc.x, acc.y, a.x, b.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  df_add_prod(acc.x, acc.y, a.y, b.z);
  acc.y = fmaf(a.y, b.w, acc.y);
  if constexpr (!RE) {
    df_add_prod(acc.z, acc.w, a.x, b.z);
    acc.w = fmaf(a.x, b.w, acc.w);
    df_add_prod(acc.z, acc.w, -a.y, b.x);
    acc.w = fmaf(-a.y, b.y, acc.w);
  }
}

// part[(v * ncols + c) * gridDim.y + chunk] = sum over the chunk's rows of
// conj(W[:, c]) * vec_v, for columns c0 = 2 * blockIdx.x, c0 + 1 and the nv
// (1 or 2) FP64 vectors.  Fixed grid and tree: deterministic.
template <bool RE>
__global__ void __launch_bounds__(kT) k_anchor_ovl(const float2* __restrict__ W, int64_t ldv, int ncols,
                                                   const double2* __restrict__ v0, const double2* __restrict__ v1,
                                                   int64_t n, int64_t rows, double2* part) {
  __shared__ double2 sh[kT];
  const int c0 = 2 * blockIdx.x;
  const int nc = min(2, ncols - c0);
  const int nv = v1 ? 2 : 1;
  const int64_t r0 = (int64_t)blockIdx.y * rows, r1 = min(n, r0 + rows);
  float4 acc[2][2];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) acc[a][b] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t i = r0 + threadIdx.x; i < r1; i += kT) {
    float4 b[2];
    b[0] = split2(v0[i]);
    b[1] = (nv > 1) ? split2(v1[i]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      if (c < nc) {
        const float2 a = W[(int64_t)(c0 + c) * ldv + i];
        acc_cdot<RE>(acc[0][c], a, b[0]);
        if (nv > 1) acc_cdot<RE>(acc[1][c], a, b[1]);
      }
    }
  }
  for (int v = 0; v < nv; ++v)
    for (int c = 0; c < nc; ++c) {
      const float4 a = acc[v][c];
      const double2 s = block_sum2(make_double2(djoin(a.x, a.y), djoin(a.z, a.w)), sh);
      if (threadIdx.x == 0) part[((size_t)v * ncols + c0 + c) * gridDim.y + blockIdx.y] = s;
      __syncthreads();
    }
}

// out[k] = sum of the nb partials of entry k (one block per entry, fixed order)
__global__ void __launch_bounds__(kT) k_anchor_final(const double2* part, int nb, double2* out) {
  __shared__ double2 sh[kT];
  const int k = blockIdx.x;
  double2 a = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < nb; i += kT) {
    a.x += part[(size_t)k * nb + i].x;
    a.y += part[(size_t)k * nb + i].y;
  }
  const double2 s = block_sum2(a, sh);
  if (threadIdx.x == 0) out[k] = s;
}

// w -= s * x with s = conj(*sc) (FP32 w, FP64 x; one rounding to FP32)
__global__ void k_anchor_axpy(float2* __restrict__ w, const double2* __restrict__ x, int64_t n,
                              const double2* __restrict__ sc, int real) {
  const float2 sr = split(sc->x), si = split(real ? 0.0 : -sc->y);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 xv = split2(x[i]);
    const float2 wv = w[i];
    float re = wv.x, im = wv.y;
    // s * x = (sr xr - si xi, sr xi + si xr); low-order terms first
    re = fmaf(-sr.y, xv.x, re); re = fmaf(-sr.x, xv.y, re);
    re = fmaf(si.y, xv.z, re);  re = fmaf(si.x, xv.w, re);
    im = fmaf(-sr.y, xv.z, im); im = fmaf(-sr.x, xv.w, im);
    im = fmaf(-si.y, xv.x, im); im = fmaf(-si.x, xv.y, im);
    re = fmaf(-sr.x, xv.x, re); re = fmaf(si.x, xv.z, re);
    im = fmaf(-sr.x, xv.z, im); im = fmaf(-si.x, xv.x, im);
    w[i] = make_float2(re, im);
  }
}

// u = r - sx * x - W[:, :ncols] * c  (FP64 u, r, x; FP32 W; sx, c complex from
// device memory), the products in double-float, one FP64 subtraction per part
__global__ void k_anchor_start(double2* __restrict__ u, const double2* __restrict__ r,
                               const double2* __restrict__ x, const double2* __restrict__ sx,
                               const float2* __restrict__ W, int64_t ldv, int ncols,
                               const double2* __restrict__ c, int64_t n, int real) {
  __shared__ float4 cs[128];
  for (int k = threadIdx.x; k < ncols; k += blockDim.x) {
    const float2 a = split(c[k].x), b = split(real ? 0.0 : c[k].y);
    cs[k] = make_float4(a.x, a.y, b.x, b.y);
  }
  __syncthreads();
  const float2 sr = split(sx->x), si = split(real ? 0.0 : sx->y);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int k = 0; k < ncols; ++k) {
      const float2 a = W[(int64_t)k * ldv + i];
      const float4 ck = cs[k];
      df_fma(rh, rl, make_float2(ck.x, ck.y), make_float2(a.x, 0.f));
      df_fma(rh, rl, make_float2(-ck.z, -ck.w), make_float2(a.y, 0.f));
      df_fma(ih, il, make_float2(ck.x, ck.y), make_float2(a.y, 0.f));
      df_fma(ih, il, make_float2(ck.z, ck.w), make_float2(a.x, 0.f));
    }
    const float4 xv = split2(x[i]);
    df_fma(rh, rl, sr, make_float2(xv.x, xv.y));
    df_fma(rh, rl, fneg2(si), make_float2(xv.z, xv.w));
    df_fma(ih, il, sr, make_float2(xv.z, xv.w));
    df_fma(ih, il, si, make_float2(xv.x, xv.y));
    const double2 rv = r[i];
    u[i] = make_double2(rv.x - djoin(rh, rl), rv.y - djoin(ih, il));
  }
}

// v = fl32(u / s->x)  (FP64 u, FP32 v)
__global__ void k_anchor_to32(float2* __restrict__ v, const double2* __restrict__ u, int64_t n,
                              const double2* __restrict__ s) {
  const float2 inv = split(1.0 / s->x);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 a = split2(u[i]);
    v[i] = make_float2(fmaf(a.x, inv.x, fmaf(a.x, inv.y, a.y * inv.x)),
                       fmaf(a.z, inv.x, fmaf(a.z, inv.y, a.w * inv.x)));
  }
}

// Restart over B = [x, W[:, :nom]]: xn = B C[:, 0] in FP64 (double-float
// sums of split products) and W[:, k-1] = B C[:, k] for k = 1..nout-1 in
// FP32 (fp32_out: plain FP32 sums of the hi parts; else double-float sums
// rounded once), in place: a block stages its kRestartRows rows of every
// input before writing.  C is (nom + 1) x nout, column-major, already split
// into float pairs (re hi, re lo, im hi, im lo) on the host, so no block
// spends FP64 instructions on it.
constexpr int kRestartRows = 64;

template <bool RE>
__global__ void __launch_bounds__(256) k_anchor_restart(const double2* __restrict__ x, double2* __restrict__ xn,
                                                        float2* W, int64_t ldv, int nom, int nout,
                                                        const float4* __restrict__ C, int64_t n, int fp32_out) {
  extern __shared__ float4 sma[];
  constexpr int R = kRestartRows;
  const int nb = nom + 1;
  float4* cs = sma;                                                   // [nout][nb]
  float4* xt = sma + (size_t)nb * nout;                               // [R]
  float2* tile = reinterpret_cast<float2*>(xt + R);                   // [nom][R]
  const int64_t r0 = (int64_t)blockIdx.x * R;
  for (int k = threadIdx.x; k < nb * nout; k += blockDim.x) cs[k] = C[k];
  for (int k = threadIdx.x; k < R; k += blockDim.x) {
    const int64_t i = r0 + k;
    xt[k] = (i < n) ? split2(x[i]) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int k = threadIdx.x; k < nom * R; k += blockDim.x) {
    const int col = k / R, r = k % R;
    const int64_t i = r0 + r;
    tile[k] = (i < n) ? W[(int64_t)col * ldv + i] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int r = threadIdx.x % R, g = threadIdx.x / R;
  const int64_t i = r0 + r;
  if (i >= n) return;
  for (int oc = g; oc < nout; oc += 256 / R) {
    const float4* cc = cs + (size_t)oc * nb;
    if (oc > 0 && fp32_out) {
      // a retained vector is stored in FP32: plain FP32 sums (the anchor's
      // row with its hi part and c's hi part), rounded once at the store
      float re = 0.f, im = 0.f;
      {
        const float4 a = xt[r], c = cc[0];
        re = fmaf(a.x, c.x, re);
        im = fmaf(a.z, c.x, im);
        if constexpr (!RE) {
          re = fmaf(-a.z, c.z, re);
          im = fmaf(a.x, c.z, im);
        }
      }
      for (int j = 0; j < nom; ++j) {
        const float2 a = tile[j * R + r];
        const float4 c = cc[1 + j];
        re = fmaf(a.x, c.x, re);
        im = fmaf(a.y, c.x, im);
        if constexpr (!RE) {
          re = fmaf(-a.y, c.z, re);
          im = fmaf(a.x, c.z, im);
        }
      }
      W[(int64_t)(oc - 1) * ldv + i] = make_float2(re, im);
      continue;
    }
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    {  // the FP64 anchor's row: (xr_hi + xr_lo, xi_hi + xi_lo) * c_0
      const float4 a = xt[r], c = cc[0];
      df_fma(rh, rl, make_float2(a.x, a.y), make_float2(c.x, c.y));
      df_fma(ih, il, make_float2(a.z, a.w), make_float2(c.x, c.y));
      if constexpr (!RE) {
        df_fma(rh, rl, make_float2(-a.z, -a.w), make_float2(c.z, c.w));
        df_fma(ih, il, make_float2(a.x, a.y), make_float2(c.z, c.w));
      }
    }
    for (int j = 0; j < nom; ++j) {
      const float2 a = tile[j * R + r];
      const float4 c = cc[1 + j];
      df_add_prod(rh, rl, a.x, c.x);
      rl = fmaf(a.x, c.y, rl);
      df_add_prod(ih, il, a.y, c.x);
      il = fmaf(a.y, c.y, il);
      if constexpr (!RE) {
        df_add_prod(rh, rl, -a.y, c.z);
        rl = fmaf(-a.y, c.w, rl);
        df_add_prod(ih, il, a.x, c.z);
        il = fmaf(a.x, c.w, il);
      }
    }
    if (oc == 0) xn[i] = make_double2(djoin(rh, rl), djoin(ih, il));
    else W[(int64_t)(oc - 1) * ldv + i] = make_float2(rh + rl, ih + il);
  }
}

unsigned grid_of(int64_t n) {
  const int64_t g = (n + kT - 1) / kT;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Cholesky M = L L^H of a Hermitian positive definite n x n matrix (column-major,
// lower triangle written to L).
void cholesky(int n, const std::vector<zd>& M, std::vector<zd>& L) {
  L.assign((size_t)n * n, zd(0.0, 0.0));
  for (int j = 0; j < n; ++j) {
    double d = M[j + (size_t)j * n].real();
    for (int k = 0; k < j; ++k) d -= std::norm(L[j + (size_t)k * n]);
    QS3G_REQUIRE(d > 0.0 && std::isfinite(d), QS3G_EBREAKDOWN, "anchored Lanczos: Gram matrix not positive definite");
    const double ljj = std::sqrt(d);
    L[j + (size_t)j * n] = ljj;
    for (int i = j + 1; i < n; ++i) {
      zd s = M[i + (size_t)j * n];
      for (int k = 0; k < j; ++k) s -= L[i + (size_t)k * n] * std::conj(L[j + (size_t)k * n]);
      L[i + (size_t)j * n] = s / ljj;
    }
  }
}

// Generalized Hermitian eigenproblem G c = theta M c (M positive definite):
// theta ascending, C column-major with c^H M c = 1.
void gen_eig(int n, const std::vector<zd>& G, const std::vector<zd>& M, std::vector<double>& theta,
             std::vector<zd>& C) {
  std::vector<zd> L;
  cholesky(n, M, L);
  // A = L^-1 G L^-H: first X = L^-1 G (forward substitution on columns), then A = L^-1 X^H
  auto fwd = [&](std::vector<zd>& B) {  // B <- L^-1 B, column by column
    for (int c = 0; c < n; ++c)
      for (int i = 0; i < n; ++i) {
        zd s = B[i + (size_t)c * n];
        for (int k = 0; k < i; ++k) s -= L[i + (size_t)k * n] * B[k + (size_t)c * n];
        B[i + (size_t)c * n] = s / L[i + (size_t)i * n];
      }
  };
  std::vector<zd> X(G);
  fwd(X);
  std::vector<zd> A((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) A[i + (size_t)j * n] = std::conj(X[j + (size_t)i * n]);
  fwd(A);  // A = L^-1 (L^-1 G)^H = L^-1 G L^-H (G Hermitian)
  std::vector<zd> Z;
  herm_jacobi(n, A, theta, Z);
  // C = L^-H Z: back substitution with L^H
  C = Z;
  for (int c = 0; c < n; ++c)
    for (int i = n - 1; i >= 0; --i) {
      zd s = C[i + (size_t)c * n];
      for (int k = i + 1; k < n; ++k) s -= std::conj(L[k + (size_t)i * n]) * C[k + (size_t)c * n];
      C[i + (size_t)c * n] = s / L[i + (size_t)i * n];
    }
}

}  // namespace

AnchorOut trlan_anchored(const Model& m, const Sector& s, const AnchorParams& p, double2* x, cudaStream_t st) {
  const int NOM = p.NOM, NOK = p.NOK, ky_max = NOK - 1;
  QS3G_REQUIRE(NOK >= 1 && NOM >= NOK + 2 && NOM <= 120, QS3G_EINVAL, "anchored Lanczos needs NOK + 2 <= NOM <= 120");
  const bool real = p.real;
  const int64_t n = p.n, ldv = p.ldv;
  // the FP32 products apply H - fl32(sigma); every FP64 quantity uses the same shift
  const double sigma = (double)(float)m.Sz_all;
  AnchorOut out;
  DevBuf<float2> W((size_t)ldv * (NOM + 1));
  DevBuf<double2> hx(n), hs(n), r(n), xn(n);
  // The restart forms the retained vectors, stored in FP32, as plain FP32
  // sums (the new anchor x' always in double-float).  At L = 1000 this took
  // the same 13,582 H*v as double-float sums rounded once, in 50.2 s against
  // 52.8 s; QS3G_ANCHOR_RESTART=df restores the double-float sums.
  const char* rs_env = std::getenv("QS3G_ANCHOR_RESTART");
  const bool restart_fp32 = !(rs_env && std::string(rs_env) == "df");
  Scratch sc;
  sc.ensure(NOM + 2);
  Ops<double2> o64{st, sc.part.get(), true, real};
  Ops<float2> o32{st, sc.part.get(), false, real};
  DevBuf<double2> part(std::max<size_t>((size_t)kChunks * 2 * (NOM + 2), (size_t)kChunksNarrow * 4));
  // device scalars
  const int NS = NOM + 2;
  DevBuf<double2> dsc((size_t)NS * (NOM + 12));  // the regions below, in this order
  double2* d_theta = dsc.get();            // x^H H x
  double2* d_rn = d_theta + 1;             // ||r||
  double2* d_xr = d_theta + 2;             // x^H r
  double2* d_un = d_theta + 3;             // ||u||
  double2* d_alpha = d_theta + NS;         // [NOM + 1]
  double2* d_beta = d_alpha + NS;          // [NOM + 1]
  double2* d_ov2 = d_beta + NS;            // second-pass overlaps of the first step [NOM + 1]
  double2* d_yrow = d_ov2 + NS;            // conj(y_j) hs, conj(y_j) x: [2][NOM]
  double2* d_yr = d_yrow + 2 * NS;         // y_j^H r [NOM]
  double2* d_row = d_yr + NS;              // per step: conj(v_i) hs, conj(w) hs, conj(v_i) x, conj(w) x: [NOM][4]
  double2* d_ov = d_row + 4 * NS;          // per step overlaps: column i at d_ov + i * NS
  QS3G_REQUIRE((size_t)(d_ov + (size_t)NS * (NOM + 1) - dsc.get()) <= dsc.n, QS3G_EINVAL, "scalar area");
  auto col = [&](int j) { return W.get() + (int64_t)j * ldv; };
  // conj(W[:, c0 .. c0+ncols)) . (v0, v1) into out[v * ncols + c]
  // one or two columns: exactly one wave of resident blocks, so that no
  // second, partly empty wave trails the first
  int narrow = kChunksNarrow;
  {
    int dev = 0, sms = 0, per = 0;
    QS3G_CHECK_CUDA(cudaGetDevice(&dev));
    QS3G_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (real) QS3G_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_anchor_ovl<true>, kT, 0));
    else QS3G_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_anchor_ovl<false>, kT, 0));
    if (sms > 0 && per > 0) narrow = sms * per;
  }
  auto ovl = [&](int c0, int ncols, const double2* v0, const double2* v1, double2* outp) {
    const int64_t tiles = (n + kT - 1) / kT;
    const int nb = (int)std::min<int64_t>(ncols <= 2 ? narrow : kChunks, tiles);
    const int64_t rows = (tiles + nb - 1) / nb * kT;
    const dim3 grid((unsigned)((ncols + 1) / 2), (unsigned)nb);
    if (real) k_anchor_ovl<true><<<grid, kT, 0, st>>>(col(c0), ldv, ncols, v0, v1, n, rows, part.get());
    else k_anchor_ovl<false><<<grid, kT, 0, st>>>(col(c0), ldv, ncols, v0, v1, n, rows, part.get());
    check_launch("k_anchor_ovl");
    k_anchor_final<<<(unsigned)((v1 ? 2 : 1) * ncols), kT, 0, st>>>(part.get(), nb, outp);
    check_launch("k_anchor_final");
  };
  auto hv32op = [&](const float2* a, float2* b) {
    if (real) hv32r(m, s, reinterpret_cast<const float*>(a), reinterpret_cast<float*>(b), st, (float)sigma, true);
    else hv32(m, s, a, b, st, (float)sigma);
  };
  auto hv64op = [&](const double2* a, double2* b) {
    if (real) hv64r(m, s, reinterpret_cast<const double*>(a), reinterpret_cast<double*>(b), st, true);
    else hv64(m, s, a, b, st);
  };
  auto fetch = [&](const double2* d, size_t cnt, std::vector<double2>& h) {
    h.resize(cnt);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(h.data(), d, cnt * sizeof(double2), cudaMemcpyDeviceToHost, st));
  };
  // normalise the start
  o64.nrm(x, n, d_rn);
  o64.scale_inv(x, n, d_rn);
  int ky = 0;
  std::vector<double> thY;  // Ritz values of the retained vectors, on H - sigma
  double best = 1e300, best_theta = 1e300, prev_theta = 0.0;
  int stall = 0, flag = 0;
  const int NB = NOM + 1;
  std::vector<double2> h_all;
  for (int cyc = 1; cyc <= p.maxitr; ++cyc) {
    out.restarts = cyc;
    // 1. anchor: H x in FP64, Rayleigh quotient, residual
    hv64op(x, hx.get());
    ++out.hv64;
    o64.dot(x, hx.get(), n, d_theta);
    std::vector<double2> h2;
    fetch(d_theta, 1, h2);
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    const double theta = h2[0].x;
    residual64(r.get(), hx.get(), x, n, theta, st);
    o64.nrm(r.get(), n, d_rn);
    fetch(d_rn, 1, h2);
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    const double rn = h2[0].x;
    QS3G_REQUIRE(std::isfinite(theta) && std::isfinite(rn), QS3G_EBREAKDOWN, "anchored Lanczos: non-finite residual");
    out.ene = theta;
    out.resid = rn;
    if (verbose())
      std::printf("trlan anchored: cycle %5d  E = %.15e  ||r|| = %.3e  (hv32 %d, hv64 %d)\n", cyc, theta, rn,
                  out.hv32, out.hv64);
    bool done;
    if (p.conv_mode == 0) {
      flag = (cyc > 1 && std::fabs(prev_theta / theta - 1.0) < p.tol) ? flag + 1 : 0;
      done = flag >= 2;
    } else {
      done = rn <= p.tol * (p.conv_mode == 2 ? std::max(1.0, std::fabs(theta)) : 1.0);
    }
    prev_theta = theta;
    if (done || rn == 0.0) {
      out.converged = true;
      break;
    }
    // Progress is a lower Rayleigh quotient or a smaller residual.  Thick-restart
    // Lanczos passes plateaus where the residual rises for many cycles while a
    // near-degenerate competitor is resolved (the energy keeps falling then);
    // only when neither moves is the FP32 basis at its floor.
    const bool lower = theta < best_theta - 1e-15 * std::max(1.0, std::fabs(theta));
    if (rn < 0.9 * best || lower) {
      stall = 0;
      best = std::min(best, rn);
      best_theta = std::min(best_theta, theta);
    } else if (++stall >= p.stall_cycles) {
      out.stalled = true;
      break;
    }
    if (cyc == p.maxitr) break;
    if (p.deadline > 0.0 && now_s() > p.deadline) { out.timed_out = true; break; }
    // 2. x's row of G and M against the retained vectors; the extension start
    residual64(hs.get(), hx.get(), x, n, sigma, st);  // hs = (H - sigma) x
    if (ky > 0) ovl(0, ky, hs.get(), x, d_yrow);      // conj(y) hs | conj(y) x
    o64.dot(x, r.get(), n, d_xr);
    if (ky > 0) ovl(0, ky, r.get(), nullptr, d_yr);   // y^H r
    k_anchor_start<<<grid_of(n), kT, 0, st>>>(xn.get(), r.get(), x, d_xr, W.get(), ldv, ky, d_yr, n, real ? 1 : 0);
    check_launch("k_anchor_start");
    o64.nrm(xn.get(), n, d_un);
    k_anchor_to32<<<grid_of(n), kT, 0, st>>>(col(ky), xn.get(), n, d_un);
    check_launch("k_anchor_to32");
    // 3. Lanczos steps on H - sigma
    for (int i = ky; i < NOM; ++i) {
      float2* w = col(i + 1);
      hv32op(col(i), w);
      ++out.hv32;
      double2* ov = d_ov + (size_t)i * NS;
      if (i == ky) {  // first step: two full passes (its couplings to the retained vectors are not small)
        o32.reorth(W.get(), ldv, i + 1, w, n, ov);
        ovl(i, 2, hs.get(), x, d_row + 4 * (size_t)i);
        k_anchor_axpy<<<grid_of(n), kT, 0, st>>>(w, x, n, d_row + 4 * (size_t)i + 3, real ? 1 : 0);
        check_launch("k_anchor_axpy");
        o32.reorth(W.get(), ldv, i + 1, w, n, d_ov2);
      } else {
        o32.dot(col(i), w, n, d_alpha + i);
        o32.lanczos_w(w, w, col(i), col(i - 1), n, d_alpha + i, d_beta + (i - 1), false);
        o32.reorth(W.get(), ldv, i + 1, w, n, ov);
        ovl(i, 2, hs.get(), x, d_row + 4 * (size_t)i);
        k_anchor_axpy<<<grid_of(n), kT, 0, st>>>(w, x, n, d_row + 4 * (size_t)i + 3, real ? 1 : 0);
        check_launch("k_anchor_axpy");
      }
      o32.nrm(w, n, d_beta + i);
      if (i + 1 < NOM) o32.scale_inv(w, n, d_beta + i);
    }
    // 4. projected problem on the host
    fetch(dsc.get(), dsc.n, h_all);
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    const double2* H = h_all.data();
    auto at = [&](const double2* d) { return H + (d - dsc.get()); };
    auto cz = [&](double2 v) { return real ? zd(v.x, 0.0) : zd(v.x, v.y); };
    bool breakdown = false;
    std::vector<zd> G((size_t)NB * NB, zd(0.0, 0.0)), M((size_t)NB * NB, zd(0.0, 0.0));
    for (int j = 0; j < NB; ++j) M[j + (size_t)j * NB] = 1.0;
    G[0] = theta - sigma;
    for (int j = 0; j < ky; ++j) {
      G[(1 + j) + (size_t)(1 + j) * NB] = thY[j];
      G[0 + (size_t)(1 + j) * NB] = std::conj(cz(at(d_yrow)[j]));            // hs^H y_j
      M[0 + (size_t)(1 + j) * NB] = std::conj(cz(at(d_yrow)[ky + j]));       // x^H y_j
    }
    for (int i = ky; i < NOM; ++i) {
      const double2* rw = at(d_row) + 4 * (size_t)i;
      G[0 + (size_t)(1 + i) * NB] = std::conj(cz(rw[0]));  // hs^H v_i
      M[0 + (size_t)(1 + i) * NB] = std::conj(cz(rw[2]));  // x^H v_i
      const double2* ov = at(d_ov) + (size_t)i * NS;
      for (int j = 0; j <= i; ++j) G[(1 + j) + (size_t)(1 + i) * NB] += cz(ov[j]);
      if (i == ky) {
        for (int j = 0; j <= i; ++j) G[(1 + j) + (size_t)(1 + i) * NB] += cz(at(d_ov2)[j]);
      } else {
        G[(1 + i) + (size_t)(1 + i) * NB] += at(d_alpha)[i].x;
        G[i + (size_t)(1 + i) * NB] += at(d_beta)[i - 1].x;
      }
      if (!(std::isfinite(at(d_beta)[i].x) && at(d_beta)[i].x > 0.0)) breakdown = true;
    }
    for (int jj = 0; jj < NB; ++jj) {  // Hermitian: lower triangle from the upper one
      G[jj + (size_t)jj * NB] = zd(G[jj + (size_t)jj * NB].real(), 0.0);
      for (int ii = jj + 1; ii < NB; ++ii) {
        G[ii + (size_t)jj * NB] = std::conj(G[jj + (size_t)ii * NB]);
        M[ii + (size_t)jj * NB] = std::conj(M[jj + (size_t)ii * NB]);
      }
    }
    std::vector<double> th;
    std::vector<zd> Cg;
    for (const zd& g : G) breakdown = breakdown || !std::isfinite(g.real()) || !std::isfinite(g.imag());
    if (!breakdown) {
      try {
        gen_eig(NB, G, M, th, Cg);
      } catch (const Error&) {
        breakdown = true;
      }
    }
    if (breakdown) {  // an exhausted Krylov space or a non-finite value: x is untouched, hand it back
      out.stalled = true;
      if (verbose()) std::printf("trlan anchored: breakdown in cycle %d, handing over\n", cyc);
      break;
    }
    // 5. new anchor and retained vectors in one pass over B
    // the coefficients split into float pairs here (hi = fl32(c), lo =
    // fl32(c - hi), the device split's arithmetic), 16 bytes each
    static_assert(sizeof(float4) == sizeof(double2), "split coefficients reuse the FP64 coefficient buffer");
    std::vector<float4> hC((size_t)NB * NOK);
    auto sp = [](double v) {
      const float h = (float)v;
      return std::make_pair(h, (float)(v - (double)h));
    };
    for (int k = 0; k < NOK; ++k)
      for (int j = 0; j < NB; ++j) {
        const zd c = Cg[j + (size_t)k * NB];
        const auto a = sp(c.real()), b = sp(real ? 0.0 : c.imag());
        hC[j + (size_t)k * NB] = make_float4(a.first, a.second, b.first, b.second);
      }
    float4* Cs = reinterpret_cast<float4*>(sc.C.get());
    QS3G_CHECK_CUDA(cudaMemcpyAsync(Cs, hC.data(), hC.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
    const size_t sm = (size_t)NB * NOK * sizeof(float4) + kRestartRows * sizeof(float4) +
                      (size_t)NOM * kRestartRows * sizeof(float2);
    auto kern = real ? k_anchor_restart<true> : k_anchor_restart<false>;
    if (sm > 48 * 1024)
      QS3G_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<(unsigned)((n + kRestartRows - 1) / kRestartRows), 256, sm, st>>>(x, xn.get(), W.get(), ldv, NOM, NOK,
                                                                             Cs, n, restart_fp32 ? 1 : 0);
    check_launch("k_anchor_restart");
    QS3G_CHECK_CUDA(cudaMemcpyAsync(x, xn.get(), n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    o64.nrm(x, n, d_rn);
    o64.scale_inv(x, n, d_rn);
    ky = ky_max;
    thY.assign(th.begin() + 1, th.begin() + NOK);
  }
  return out;
}

}  // namespace qs3g

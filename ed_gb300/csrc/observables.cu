// observables.cu -- static correlation functions of a sector eigenvector.
//
// Replaces get_lm_2_wave_vector + calcu_lm_trans_2 and get_cf_2_wave_vector +
// calcu_cf_trans_2 (get_expectation_values.f90:197-279, ham2vec_v3.f90:74-174)
// for the full list of NOS^2 ordered site pairs.
//
// The reference groups the pairs (a, b) into orbits under simultaneous
// translation of both sites (mk_list_ij) and averages over each orbit.  An
// orbit is exactly a displacement class delta = R_b - R_a (periodic), so the
// GPU computes, for every delta, one fixed-order reduction over all rows:
//   SzSz(delta) = 1/4 * sum_i |v_i|^2 * (1 - 4 (N_down - N_dd^(i)(delta)) / NOS)
//     with N_dd^(i)(delta) the number of down spins a of row i whose partner
//     a + delta is also down (delta != 0); SzSz(0) = 1/4;
//   SpSm(delta) = 1/NOS * sum_i sum_{a down, a+delta up} list_r(id)/list_r(i)
//                 * explist(ell) * conj(v_i) v_id            (delta != 0)
//   SpSm(0)     = 1/NOS * sum_i |v_i|^2 * (NOS - N_down)
// where id, ell come from flipping (a, a+delta) and finding the
// representative, as calcu_cf_trans_2 does.  Results are deterministic: a
// fixed grid of blocks, a fixed per-thread row order and fixed tree
// reductions.
#include <algorithm>

#include "qs3g_device.cuh"
#include "qs3g_internal.cuh"
#include "krylov.h"

namespace qs3g {
namespace {

template <class F>
void dispatch_nod3(int NOD, F&& f) {
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

struct CorrArgs {
  int64_t D;
  int NOS, LX, LY, LZ, bits, NT;
  bool chain;
  const uint64_t* conf;
  const double* list_r;
  const uint2* dir;
  const uint32_t* binomA;
  const uint64_t* binom;
  const double2* explist;
  const double2* chainph;
  const int16_t* xyz;
  const double2* v;
};

constexpr int kObsThreads = 256;
constexpr int kObsBlocks = 152 * 2;

__device__ __forceinline__ int shift_site(int a, int dx, int dy, int dz, const CorrArgs& g) {
  const short4 c = reinterpret_cast<const short4*>(g.xyz)[a];
  int x = c.x + dx; x -= (x >= g.LX) ? g.LX : 0;
  int y = c.y + dy; y -= (y >= g.LY) ? g.LY : 0;
  int z = c.z + dz; z -= (z >= g.LZ) ? g.LZ : 0;
  return 1 + x + g.LX * (y + g.LY * z);
}

__device__ __forceinline__ double2 block_sum2(double2 v, double2* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sh[threadIdx.x].x += sh[threadIdx.x + s].x;
      sh[threadIdx.x].y += sh[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  const double2 r = sh[0];
  __syncthreads();
  return r;
}

// Representative search for one flipped configuration (chain or general lattice).
template <int NOD>
__device__ __forceinline__ int find_row(const int (&o)[NOD], const CorrArgs& g, int& ell3) {
  if (g.chain) {
    int p[NOD], ell;
    chain_rep<NOD>(o, g.NOS, g.bits, p, ell);
    ell3 = ell;
    return dir_lookup(g.dir, anchored_index<NOD>(p, g.binomA, g.NOS));
  }
  // general lattice: scan all translations (loop order), first strict minimum
  const uint64_t self = pack<NOD>(o, g.bits);
  uint64_t best = ~0ull;
  int bt = 0, tau = 0;
  for (int k = 1; k <= g.LZ; ++k)
    for (int j = 1; j <= g.LY; ++j)
      for (int i = 1; i <= g.LX; ++i, ++tau) {
        int t[NOD];
#pragma unroll
        for (int e = 0; e < NOD; ++e) t[e] = shift_site(o[e], i % g.LX, j % g.LY, k % g.LZ, g);
#pragma unroll
        for (int u = 1; u < NOD; ++u)
#pragma unroll
          for (int w = u; w > 0; --w) {
            const int lo = min(t[w - 1], t[w]), hi = max(t[w - 1], t[w]);
            t[w - 1] = lo; t[w] = hi;
          }
        const uint64_t pk = pack<NOD>(t, g.bits);
        if (pk < best) { best = pk; bt = tau; }
      }
  ell3 = (best == self) ? -1 : bt;
  int rep[NOD];
  unpack<NOD>(best, g.bits, rep);
  return dir_lookup(g.dir, full_index<NOD>(rep, g.binom, g.NOS));
}

// part[(delta * nblk + block)] = (SzSz numerator partial (x), unused) and SpSm partial
template <int NOD>
__global__ void __launch_bounds__(kObsThreads) k_corr(CorrArgs g, int delta, double2* part_zz, double2* part_pm) {
  __shared__ double2 sh[kObsThreads];
  const int dx = delta % g.LX, dy = (delta / g.LX) % g.LY, dz = delta / (g.LX * g.LY);
  double zz = 0.0;
  double2 pm = make_double2(0.0, 0.0);
  const size_t ex1 = (size_t)g.LX + 1, ex2 = ex1 * ((size_t)g.LY + 1);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.D; i += (int64_t)gridDim.x * blockDim.x) {
    int n[NOD];
    unpack<NOD>(g.conf[i], g.bits, n);
    const double2 vi = g.v[i];
    const double w = vi.x * vi.x + vi.y * vi.y;
    if (delta == 0) {
      zz += w;                                   // SzSz(0) handled on the host
      pm.x += w * (double)(g.NOS - NOD);
      continue;
    }
    int ndd = 0;
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int m = 0; m < NOD; ++m) {
      const int b = shift_site(n[m], dx, dy, dz, g);
      bool bdown = false;
#pragma unroll
      for (int j = 0; j < NOD; ++j) bdown |= (n[j] == b);
      if (bdown) { ++ndd; continue; }
      // flip (a = n[m] down, b up): j_flip_ni(min, max) gives the same sorted list
      int o[NOD];
      move_spin<NOD>(n, m, b, o);
      int ell3;
      const int id = find_row<NOD>(o, g, ell3);
      if (id < 0) continue;
      double2 e;  // explist(ell): chains keep explist(i,1,1) per translation i in chainph
      if (g.chain) {
        e = g.chainph[ell3];
      } else {
        size_t eidx = 0;
        if (ell3 >= 0) {
          const int ti = ell3 % g.LX + 1, r = ell3 / g.LX, tj = r % g.LY + 1, tk = r / g.LY + 1;
          eidx = (size_t)ti + ex1 * (size_t)tj + ex2 * (size_t)tk;
        }
        e = g.explist[eidx];
      }
      // list_r(id)/list_r(i) * explist(ell) * conj(v_i) * v_id  (calcu_cf_trans_2 order)
      const double c = g.list_r[id] / g.list_r[i];
      const double2 ce = make_double2(c * e.x, c * e.y);
      const double2 t1 = cmul(ce, make_double2(vi.x, -vi.y));
      const double2 t2 = cmul(t1, g.v[id]);
      acc.x += t2.x;
      acc.y += t2.y;
    }
    zz += w * (double)ndd;
    pm.x += acc.x;
    pm.y += acc.y;
  }
  const double2 s1 = block_sum2(make_double2(zz, 0.0), sh);
  const double2 s2 = block_sum2(pm, sh);
  if (threadIdx.x == 0) {
    part_zz[(size_t)delta * gridDim.x + blockIdx.x] = s1;
    part_pm[(size_t)delta * gridDim.x + blockIdx.x] = s2;
  }
}

// ------------------------------------------------------------ U(1)-only sectors
// source_only_u1/ham2vec_v3.f90:67-141 (calcu_lm, calcu_cf), one pair at a
// time with no translation average.  For an ordered pair (a, b) the rows
// that matter are enumerated directly: the other down spins form a
// k-subset of the sites outside {a, b}, unranked in colex order, and the
// row is the colex rank of that subset with a and/or b added.
//   a != b:  x = sum_{a, b down} |v_i|^2                     (C(NOS-2, NOD-2) rows)
//            pm = sum_{a down, b up} conj(v_i) v_id           (C(NOS-2, NOD-1) rows)
//            with id the row with a up and b down (j_flip_ni of the pair)
//   a == b:  x = sum_{a down} |v_i|^2                         (C(NOS-1, NOD-1) rows)
// Both cases enumerate C(NOS-1, NOD-1) tasks per pair.

// Sites of the colex-rank-r k-subset of {1..NOS} \ {lo, hi} (hi = 0: only lo
// excluded), merged with the fixed sites f0 <= f1 (nf of them), sorted.
template <int NOD>
__device__ __forceinline__ void u1_config(uint64_t r, int k, int M, int lo, int hi, int nf, int f0, int f1,
                                          const uint64_t* __restrict__ binom, int NOS, int (&out)[NOD]) {
  int q[NOD];
  int top = M;
  for (int j = k; j >= 1; --j) {
    const uint64_t* bj = binom + (size_t)j * (NOS + 1);
    int l = j, u = top;
    while (l < u) {
      const int mid = (l + u + 1) >> 1;
      if (__ldg(bj + mid - 1) <= r) l = mid; else u = mid - 1;
    }
    r -= __ldg(bj + l - 1);
    int s = l;  // position -> site, skipping the excluded sites
    if (s >= lo) ++s;
    if (hi > 0 && s >= hi) ++s;
    q[j - 1] = s;
    top = l - 1;
  }
  // merge q[0..k) with the fixed sites
  int ia = 0, w = 0;
  const int fx[2] = {f0, f1};
  int jf = 0;
  for (; w < k + nf; ++w) {
    if (jf < nf && (ia >= k || fx[jf] < q[ia])) out[w] = fx[jf++];
    else out[w] = q[ia++];
  }
}

template <int NOD>
__global__ void __launch_bounds__(kObsThreads) k_corr_u1(CorrArgs g, int pair0, double2* part_x, double2* part_pm) {
  __shared__ double2 sh[kObsThreads];
  const int pair = pair0 + (int)blockIdx.y;
  const int a = pair % g.NOS + 1, b = pair / g.NOS + 1;
  const int NOS = g.NOS;
  double x = 0.0;
  double2 pm = make_double2(0.0, 0.0);
  if (a == b) {
    const uint64_t nt = (NOD - 1 <= NOS - 1) ? g.binom[(size_t)(NOD - 1) * (NOS + 1) + (NOS - 1)] : 0;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nt; r += (uint64_t)gridDim.x * blockDim.x) {
      int c[NOD];
      u1_config<NOD>(r, NOD - 1, NOS - 1, a, 0, 1, a, 0, g.binom, NOS, c);
      const double2 v = g.v[full_index<NOD>(c, g.binom, NOS)];
      x += v.x * v.x + v.y * v.y;
    }
  } else {
    const int lo = min(a, b), hi = max(a, b);
    const uint64_t nB = (NOD >= 2) ? g.binom[(size_t)(NOD - 2) * (NOS + 1) + (NOS - 2)] : 0;
    const uint64_t nP = g.binom[(size_t)(NOD - 1) * (NOS + 1) + (NOS - 2)];
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nB + nP;
         r += (uint64_t)gridDim.x * blockDim.x) {
      int c[NOD];
      if (r < nB) {
        u1_config<NOD>(r, NOD - 2, NOS - 2, lo, hi, 2, lo, hi, g.binom, NOS, c);
        const double2 v = g.v[full_index<NOD>(c, g.binom, NOS)];
        x += v.x * v.x + v.y * v.y;
      } else {
        u1_config<NOD>(r - nB, NOD - 1, NOS - 2, lo, hi, 1, a, 0, g.binom, NOS, c);
        const double2 vi = g.v[full_index<NOD>(c, g.binom, NOS)];
        u1_config<NOD>(r - nB, NOD - 1, NOS - 2, lo, hi, 1, b, 0, g.binom, NOS, c);
        const double2 vd = g.v[full_index<NOD>(c, g.binom, NOS)];
        const double2 t = cmul(make_double2(vi.x, -vi.y), vd);
        pm.x += t.x;
        pm.y += t.y;
      }
    }
  }
  const double2 s1 = block_sum2(make_double2(x, 0.0), sh);
  const double2 s2 = block_sum2(pm, sh);
  if (threadIdx.x == 0) {
    part_x[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s1;
    part_pm[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s2;
  }
}

int correlations_u1(const Model& m, const Sector& s, const double2* d_v, double* szsz, double2* spsm, double* lm,
                    cudaStream_t st) {
  const int NOS = m.NOS, NOD = s.NOD;
  CorrArgs g{};
  g.D = s.D; g.NOS = NOS; g.bits = m.bits; g.binom = s.d_binom.get(); g.v = d_v;
  const uint64_t tasks = binom_u64(NOS - 1, NOD - 1);
  const int nbx = (int)std::min<uint64_t>(64, std::max<uint64_t>(1, (tasks + kObsThreads - 1) / kObsThreads));
  const int npairs = NOS * NOS;
  const int chunk = std::min(npairs, 16384);
  DevBuf<double2> px((size_t)chunk * nbx), pp((size_t)chunk * nbx);
  std::vector<double> X(npairs);
  std::vector<double2> P(npairs);
  std::vector<double2> hx((size_t)chunk * nbx), hp((size_t)chunk * nbx);
  for (int p0 = 0; p0 < npairs; p0 += chunk) {
    const int np = std::min(chunk, npairs - p0);
    dispatch_nod3(NOD, [&](auto c) {
      k_corr_u1<decltype(c)::value><<<dim3(nbx, np), kObsThreads, 0, st>>>(g, p0, px.get(), pp.get());
    });
    check_launch("k_corr_u1");
    QS3G_CHECK_CUDA(cudaMemcpyAsync(hx.data(), px.get(), (size_t)np * nbx * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(hp.data(), pp.get(), (size_t)np * nbx * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    for (int p = 0; p < np; ++p) {
      double xs = 0.0;
      double2 ps = make_double2(0.0, 0.0);
      for (int k = 0; k < nbx; ++k) {
        xs += hx[(size_t)p * nbx + k].x;
        ps.x += hp[(size_t)p * nbx + k].x;
        ps.y += hp[(size_t)p * nbx + k].y;
      }
      X[p0 + p] = xs;
      P[p0 + p] = ps;
    }
  }
  // N_a = X(a, a); W = sum_a N_a / NOD = sum_i |v_i|^2
  double W = 0.0;
  for (int a = 0; a < NOS; ++a) W += X[(size_t)a + (size_t)a * NOS];
  W /= (double)NOD;
  for (int b = 0; b < NOS; ++b)
    for (int a = 0; a < NOS; ++a) {
      const size_t p = (size_t)a + (size_t)b * NOS;
      const double Na = X[(size_t)a + (size_t)a * NOS], Nb = X[(size_t)b + (size_t)b * NOS];
      if (a == b) {
        szsz[p] = 0.25;
        spsm[p] = make_double2(W - Na, 0.0);
      } else {
        szsz[p] = 0.25 * (W - 2.0 * Na - 2.0 * Nb + 4.0 * X[p]);
        spsm[p] = P[p];
      }
    }
  if (lm)
    for (int a = 0; a < NOS; ++a) lm[a] = 0.5 * (W - 2.0 * X[(size_t)a + (size_t)a * NOS]);
  return QS3G_OK;
}

}  // namespace

int correlations(const Model& m, const Sector& s, const double2* h_v, double* szsz, double2* spsm, double* lm,
                 cudaStream_t st) {
  const int NOS = m.NOS, NOD = s.NOD;
  QS3G_REQUIRE(s.D > 0, QS3G_ESTATE, "empty sector");
  DevBuf<double2> d_v(s.D);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_v.get(), h_v, s.D * sizeof(double2), cudaMemcpyHostToDevice, st));
  if (s.u1) return correlations_u1(m, s, d_v.get(), szsz, spsm, lm, st);
  CorrArgs g{};
  g.D = s.D; g.NOS = NOS; g.LX = m.LX; g.LY = m.LY; g.LZ = m.LZ; g.bits = m.bits; g.NT = NOS; g.chain = s.anchored;
  g.conf = s.d_conf.get(); g.list_r = s.d_list_r.get(); g.dir = s.d_dir.get(); g.binomA = s.d_binomA.get();
  g.binom = s.d_binom.get(); g.explist = s.d_explist.get(); g.chainph = s.d_chainph.get();
  g.xyz = m.d_site_xyz.get(); g.v = d_v.get();
  DevBuf<double2> pz((size_t)NOS * kObsBlocks), pp((size_t)NOS * kObsBlocks);
  for (int delta = 0; delta < NOS; ++delta) {
    dispatch_nod3(NOD, [&](auto c) {
      k_corr<decltype(c)::value><<<kObsBlocks, kObsThreads, 0, st>>>(g, delta, pz.get(), pp.get());
    });
    check_launch("k_corr");
  }
  std::vector<double2> hz((size_t)NOS * kObsBlocks), hp((size_t)NOS * kObsBlocks);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(hz.data(), pz.get(), hz.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(hp.data(), pp.get(), hp.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  // per displacement class, fixed-order sums of the block partials
  std::vector<double> zz(NOS);
  std::vector<double2> pm(NOS);
  for (int d = 0; d < NOS; ++d) {
    double a = 0.0;
    double2 b = make_double2(0.0, 0.0);
    for (int k = 0; k < kObsBlocks; ++k) {
      a += hz[(size_t)d * kObsBlocks + k].x;
      b.x += hp[(size_t)d * kObsBlocks + k].x;
      b.y += hp[(size_t)d * kObsBlocks + k].y;
    }
    zz[d] = a;
    pm[d] = b;
  }
  const double norm = zz[0];  // sum_i |v_i|^2 (the reference assumes 1)
  (void)norm;
  // expe_szsz(ss1 + (ss2-1)*NOS): pair (ss1, ss2), displacement R_ss2 - R_ss1
  for (int b = 1; b <= NOS; ++b)
    for (int a = 1; a <= NOS; ++a) {
      const int ax = (a - 1) % m.LX, ay = ((a - 1) / m.LX) % m.LY, az = (a - 1) / (m.LX * m.LY);
      const int bx = (b - 1) % m.LX, by = ((b - 1) / m.LX) % m.LY, bz = (b - 1) / (m.LX * m.LY);
      const int dx = (bx - ax + m.LX) % m.LX, dy = (by - ay + m.LY) % m.LY, dz = (bz - az + m.LZ) % m.LZ;
      const int d = dx + m.LX * (dy + m.LY * dz);
      const size_t p = (size_t)(a - 1) + (size_t)(b - 1) * NOS;
      if (d == 0) {
        szsz[p] = 0.25;
        spsm[p] = make_double2(pm[0].x / NOS, 0.0);
      } else {
        szsz[p] = 0.25 * (zz[0] - 4.0 * ((double)NOD * zz[0] - zz[d]) / NOS);
        spsm[p] = make_double2(pm[d].x / NOS, pm[d].y / NOS);
      }
    }
  // <Sz_i> (calcu_lm_trans_2): the same for every site of a translation-invariant state
  if (lm)
    for (int i = 0; i < NOS; ++i) lm[i] = 0.5 * zz[0] * (1.0 - 2.0 * (double)NOD / NOS);
  return QS3G_OK;
}

}  // namespace qs3g

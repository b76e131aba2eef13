// dsf.cu -- dynamical structure factor: start vectors S^a(q)|GS> and the
// continued-fraction Lanczos recursion.
//
// Replaces calcu_Sq_a (get_expectation_values.f90:281-377) with
// search_representative_{Spi,Smi,Szi}_state_SQ (state_lists.f90:488-583) and
// calcu_DSF_wavevector (get_expectation_values.f90:379-605).
//
// The reference scatters psi(l) into fn(lp) with OpenMP atomics (and without
// one for S^z, a race).  Here the start vector is built in gather form: one
// thread per row lp of the new (NOD', k+q) sector enumerates every (l, i) whose
// image S^a_i |l> has lp as representative, so each fn(lp) is written once by
// one thread and the result is deterministic.  For chains the enumeration is
// exact and cheap: an image that lands on a ground-state representative must
// occupy site 1, so only the translations of lp that put one of its spins (or,
// for S^+, the removed spin) on site 1 take part.
#include <cmath>

#include "qs3g_device.cuh"
#include "qs3g_internal.cuh"
#include "krylov.h"

namespace qs3g {
namespace {

template <class F>
void dispatch_nod2(int NOD, F&& f) {
  switch (NOD) {
    case 1: f(std::integral_constant<int, 1>{}); break;
    case 2: f(std::integral_constant<int, 2>{}); break;
    case 3: f(std::integral_constant<int, 3>{}); break;
    case 4: f(std::integral_constant<int, 4>{}); break;
    case 5: f(std::integral_constant<int, 5>{}); break;
    case 6: f(std::integral_constant<int, 6>{}); break;
    case 7: f(std::integral_constant<int, 7>{}); break;
    default: throw Error(QS3G_ENOTSUP, "DSF sectors need NOD, NOD' in [1, 7]");
  }
}

struct SqArgs {
  int L, bits, NOD, NODn;
  int64_t Dn;
  const uint64_t* conf_new;
  const double* r_new;
  const uint2* dir_gs;
  const uint32_t* binomA_gs;  // anchored binomials of the ground-state sector (chains)
  const uint64_t* binom_gs;   // full binomials of the ground-state sector (general lattices)
  const double* r_gs;
  const double2* psi;
  const double2* eks;         // exp(-i q.R_i), index 1..NOS
  const double2* ph_new;      // chains: explist_new(i,1,1), [0] = explist_new(0,0,0)
  double2 eks_half_sum;       // 0.5 * sum_i eks_i (S^z)
  double inv_sqrt_nos;
  double2* fn;
};

// fn += ((psi(l) * r'/r) * eks_i) * conj(ph)  in the Fortran evaluation order
__device__ __forceinline__ void sq_term(double2& acc, double2 psi, double rn, double ro, double2 eks, double2 ph) {
  const double2 pv = make_double2((psi.x * rn) / ro, (psi.y * rn) / ro);
  const double2 t = cmul(cmul(pv, eks), make_double2(ph.x, -ph.y));
  acc.x += t.x;
  acc.y += t.y;
}

// S^- (spsmsz = 2): NOD' = NOD + 1.  Chain gather.
template <int NODN>
__global__ void k_sq_minus_chain(SqArgs a) {
  constexpr int NOD = NODN - 1;
  const int64_t lp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (lp >= a.Dn) return;
  int n[NODN];
  unpack<NODN>(a.conf_new[lp], a.bits, n);
  const double rn = a.r_new[lp];
  int g[NODN];
#pragma unroll
  for (int m = 0; m < NODN - 1; ++m) g[m] = n[m + 1] - n[m];
  g[NODN - 1] = n[0] + a.L - n[NODN - 1];
  uint64_t key[NODN];
#pragma unroll
  for (int m = 0; m < NODN; ++m) {
    uint64_t k = 0;
#pragma unroll
    for (int t = 1; t <= NODN; ++t) k = (k << a.bits) | (uint64_t)g[(m - t + 2 * NODN) % NODN];
    key[m] = k;
  }
  double2 acc = make_double2(0.0, 0.0);
#pragma unroll
  for (int m = 0; m < NODN; ++m) {
    bool dup = false;
#pragma unroll
    for (int m2 = 0; m2 < m; ++m2) dup |= (key[m2] == key[m]);
    if (dup) continue;
    // c'' = rotation of n' with spin m on site 1
    int c[NODN];
    c[0] = 1;
#pragma unroll
    for (int j = 1; j < NODN; ++j) c[j] = c[j - 1] + g[(m + j - 1) % NODN];
    int rep[NODN], ell;
    chain_rep<NODN>(c, a.L, a.bits, rep, ell);
    const double2 ph = a.ph_new[ell];
#pragma unroll
    for (int j = 1; j < NODN; ++j) {
      int s[NOD];  // c'' without its spin j (keeps site 1)
#pragma unroll
      for (int u = 0; u < NOD; ++u) s[u] = c[u < j ? u : u + 1];
      const int64_t l = dir_lookup(a.dir_gs, anchored_index<NOD>(s, a.binomA_gs, a.L));
      if (l < 0) continue;
      sq_term(acc, a.psi[l], rn, a.r_gs[l], a.eks[c[j]], ph);
    }
  }
  a.fn[lp] = make_double2(a.inv_sqrt_nos * acc.x, a.inv_sqrt_nos * acc.y);
}

// S^+ (spsmsz = 1): NOD' = NOD - 1.  Chain gather over the translations of lp.
template <int NODN>
__global__ void k_sq_plus_chain(SqArgs a) {
  constexpr int NOD = NODN + 1;
  const int64_t lp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (lp >= a.Dn) return;
  int n[NODN];
  unpack<NODN>(a.conf_new[lp], a.bits, n);
  const double rn = a.r_new[lp];
  // period of n' (smallest t > 0 with T^t n' = n')
  int per = a.L;
  {
    int g[NODN];
#pragma unroll
    for (int m = 0; m < NODN - 1; ++m) g[m] = n[m + 1] - n[m];
    g[NODN - 1] = n[0] + a.L - n[NODN - 1];
    uint64_t k0 = 0;
#pragma unroll
    for (int t = 1; t <= NODN; ++t) k0 = (k0 << a.bits) | (uint64_t)g[(0 - t + 2 * NODN) % NODN];
    int cnt = 1;
#pragma unroll
    for (int m = 1; m < NODN; ++m) {
      uint64_t k = 0;
#pragma unroll
      for (int t = 1; t <= NODN; ++t) k = (k << a.bits) | (uint64_t)g[(m - t + 2 * NODN) % NODN];
      cnt += (k == k0) ? 1 : 0;
    }
    per = a.L / cnt;
  }
  double2 acc = make_double2(0.0, 0.0);
  for (int t = 0; t < per; ++t) {
    // c'' = T^t n' (sites shifted by +t, sorted)
    int c[NODN];
#pragma unroll
    for (int u = 0; u < NODN; ++u) {
      int v = n[u] + t;
      c[u] = (v > a.L) ? v - a.L : v;
    }
#pragma unroll
    for (int u = 1; u < NODN; ++u)
#pragma unroll
      for (int w = u; w > 0; --w) {
        const int lo = min(c[w - 1], c[w]), hi = max(c[w - 1], c[w]);
        c[w - 1] = lo; c[w] = hi;
      }
    int rep[NODN], ell;
    chain_rep<NODN>(c, a.L, a.bits, rep, ell);
    const double2 ph = a.ph_new[ell];
    if (c[0] == 1) {
      // the added site i (the removed spin of S^+_i) is any empty site other than 1
      int nxt = 1;  // index into c of the next occupied site above i
      for (int i = 2; i <= a.L; ++i) {
        while (nxt < NODN && c[nxt] < i) ++nxt;
        if (nxt < NODN && c[nxt] == i) continue;
        int s[NOD];
        // s = c with i inserted (c[0] = 1 stays first)
#pragma unroll
        for (int u = 0; u < NOD; ++u)
          s[u] = (u < nxt) ? c[u < NODN ? u : NODN - 1] : ((u == nxt) ? i : c[u > 0 ? u - 1 : 0]);
        const int64_t l = dir_lookup(a.dir_gs, anchored_index<NOD>(s, a.binomA_gs, a.L));
        if (l < 0) continue;
        sq_term(acc, a.psi[l], rn, a.r_gs[l], a.eks[i], ph);
      }
    } else {
      int s[NOD];
      s[0] = 1;
#pragma unroll
      for (int u = 1; u < NOD; ++u) s[u] = c[u - 1];
      const int64_t l = dir_lookup(a.dir_gs, anchored_index<NOD>(s, a.binomA_gs, a.L));
      if (l >= 0) sq_term(acc, a.psi[l], rn, a.r_gs[l], a.eks[1], ph);
    }
  }
  a.fn[lp] = make_double2(a.inv_sqrt_nos * acc.x, a.inv_sqrt_nos * acc.y);
}

// S^z (spsmsz = 3): NOD' = NOD; the image of l is l itself (ell = 0).
template <int NOD>
__global__ void k_sq_z(SqArgs a, int anchored, int NOS) {
  const int64_t lp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (lp >= a.Dn) return;
  int n[NOD];
  unpack<NOD>(a.conf_new[lp], a.bits, n);
  const uint64_t c = anchored ? anchored_index<NOD>(n, a.binomA_gs, a.L) : full_index<NOD>(n, a.binom_gs, NOS);
  const int64_t l = dir_lookup(a.dir_gs, c);
  double2 out = make_double2(0.0, 0.0);
  if (l >= 0) {
    // sum_i Siz eks_i = 0.5 sum_i eks_i - sum_{i down} eks_i
    double2 s = a.eks_half_sum;
#pragma unroll
    for (int u = 0; u < NOD; ++u) { s.x -= a.eks[n[u]].x; s.y -= a.eks[n[u]].y; }
    double2 acc = make_double2(0.0, 0.0);
    sq_term(acc, a.psi[l], a.r_new[lp], a.r_gs[l], s, a.ph_new[0]);
    out = make_double2(a.inv_sqrt_nos * acc.x, a.inv_sqrt_nos * acc.y);
  }
  a.fn[lp] = out;
}

// U(1)-only start vectors (source_only_u1/get_expectation_values.f90:100-179),
// gather form: row lp of the NOD' sector sums psi(l) * exp(-i q.R_i) over the
// sites i in ascending order, exactly the order in which the reference's
// outer site loop adds into fn(lp).
//   S^+: l = lp's configuration with down spin i added (i up in lp)
//   S^-: l = lp's configuration with down spin i removed (i down in lp)
//   S^z: l = lp, weight Siz = -1/2 (i down) or +1/2 (i up)
template <int NODN, int SPSMSZ>
__global__ void k_sq_u1(SqArgs a, int NOS) {
  const int64_t lp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (lp >= a.Dn) return;
  int n[NODN];
  unpack<NODN>(a.conf_new[lp], a.bits, n);
  double2 acc = make_double2(0.0, 0.0);
  if constexpr (SPSMSZ == 1) {
    constexpr int NOD = NODN + 1;
    int nxt = 0;  // index into n of the first occupied site >= i
    for (int i = 1; i <= NOS; ++i) {
      while (nxt < NODN && n[nxt] < i) ++nxt;
      if (nxt < NODN && n[nxt] == i) continue;
      int s[NOD];
#pragma unroll
      for (int u = 0; u < NOD; ++u)
        s[u] = (u < nxt) ? n[u < NODN ? u : NODN - 1] : ((u == nxt) ? i : n[u > 0 ? u - 1 : 0]);
      const int64_t l = (int64_t)full_index<NOD>(s, a.binom_gs, NOS);
      const double2 t = cmul(a.psi[l], a.eks[i]);
      acc.x += t.x;
      acc.y += t.y;
    }
  } else if constexpr (SPSMSZ == 2) {
    constexpr int NOD = NODN - 1;
#pragma unroll
    for (int j = 0; j < NODN; ++j) {
      int s[NOD > 0 ? NOD : 1];
#pragma unroll
      for (int u = 0; u < NOD; ++u) s[u] = n[u < j ? u : u + 1];
      int64_t l = 0;
      if constexpr (NOD > 0) l = (int64_t)full_index<NOD>(s, a.binom_gs, NOS);
      const double2 t = cmul(a.psi[l], a.eks[n[j]]);
      acc.x += t.x;
      acc.y += t.y;
    }
  } else {
    const double2 pl = a.psi[lp];
    int nxt = 0;
    for (int i = 1; i <= NOS; ++i) {
      while (nxt < NODN && n[nxt] < i) ++nxt;
      const double siz = (nxt < NODN && n[nxt] == i) ? -0.5 : 0.5;
      const double2 t = cmul(make_double2(siz * pl.x, siz * pl.y), a.eks[i]);
      acc.x += t.x;
      acc.y += t.y;
    }
  }
  a.fn[lp] = make_double2(a.inv_sqrt_nos * acc.x, a.inv_sqrt_nos * acc.y);
}

__global__ void k_set_scalar(double2* p, double2 v) { *p = v; }

}  // namespace

// calcu_Sq_a alone for one wave vector: builds the (NOD', k+q) sector in `ns`
// and writes fn = S^a(q)|psi> (before normalisation) to the device buffer fn.
void start_vector(const Model& m, const Sector& gs, const double2* d_psi, int spsmsz, const double* qv,
                  const double* Spos, Sector& ns, DevBuf<double2>& fn, cudaStream_t st) {
  const int NOD = gs.NOD, NOS = m.NOS;
  QS3G_REQUIRE(spsmsz >= 1 && spsmsz <= 3, QS3G_EINVAL, "spsmsz must be 1, 2 or 3");
  QS3G_REQUIRE(!(spsmsz == 1 && NOD <= 1), QS3G_EINVAL, "S+(q,w) needs NOD >= 2");
  QS3G_REQUIRE(gs.u1 || m.chain || spsmsz == 3, QS3G_ENOTSUP, "S+/S- start vectors are implemented for chains");
  const int NODn = (spsmsz == 1) ? NOD - 1 : (spsmsz == 2 ? NOD + 1 : NOD);
  QS3G_REQUIRE(NODn <= NOS, QS3G_EINVAL, "S-(q,w) from the all-down sector");
  double rkn[3] = {gs.rk[0] + qv[0], gs.rk[1] + qv[1], gs.rk[2] + qv[2]};
  if (gs.u1) build_sector_u1(m, NODn, ns, st);
  else build_sector_rk(m, NODn, rkn, ns, st);
  const int64_t Dn = ns.D;
  fn.alloc(std::max<int64_t>(1, Dn));
  if (Dn == 0) return;
  std::vector<double2> eks(NOS + 1, make_double2(0.0, 0.0));
  double2 hsum = make_double2(0.0, 0.0);
  for (int i = 1; i <= NOS; ++i) {
    const double d = qv[0] * Spos[3 * (i - 1)] + qv[1] * Spos[3 * (i - 1) + 1] + qv[2] * Spos[3 * (i - 1) + 2];
    eks[i] = make_double2(std::cos(d), -std::sin(d));
    hsum.x += eks[i].x;
    hsum.y += eks[i].y;
  }
  DevBuf<double2> d_eks(NOS + 1), d_ph;
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_eks.get(), eks.data(), (NOS + 1) * sizeof(double2), cudaMemcpyHostToDevice, st));
  const double2* ph_new = ns.d_chainph.get();
  if (!m.chain) {
    d_ph.alloc(1);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(d_ph.get(), ns.d_explist.get(), sizeof(double2), cudaMemcpyDeviceToDevice, st));
    ph_new = d_ph.get();
  }
  SqArgs a{};
  a.L = NOS; a.bits = m.bits; a.NOD = NOD; a.NODn = NODn; a.Dn = Dn;
  a.conf_new = ns.d_conf.get(); a.r_new = ns.d_list_r.get();
  a.dir_gs = gs.d_dir.get(); a.binomA_gs = gs.d_binomA.get(); a.binom_gs = gs.d_binom.get();
  a.r_gs = gs.d_list_r.get(); a.psi = d_psi; a.eks = d_eks.get(); a.ph_new = ph_new;
  a.eks_half_sum = make_double2(0.5 * hsum.x, 0.5 * hsum.y);
  a.inv_sqrt_nos = 1.0 / std::sqrt((double)NOS);
  a.fn = fn.get();
  const unsigned grid = (unsigned)((Dn + 127) / 128);
  if (gs.u1) {
    dispatch_nod2(NODn, [&](auto c) {
      constexpr int V = decltype(c)::value;
      if (spsmsz == 1) {
        if constexpr (V + 1 <= 8) k_sq_u1<V, 1><<<grid, 128, 0, st>>>(a, NOS);
      } else if (spsmsz == 2) {
        k_sq_u1<V, 2><<<grid, 128, 0, st>>>(a, NOS);
      } else {
        k_sq_u1<V, 3><<<grid, 128, 0, st>>>(a, NOS);
      }
    });
    check_launch("k_sq_u1");
  } else if (spsmsz == 2) {
    dispatch_nod2(NODn, [&](auto c) {
      constexpr int V = decltype(c)::value;
      if constexpr (V >= 2) k_sq_minus_chain<V><<<grid, 128, 0, st>>>(a);
      else throw Error(QS3G_EINVAL, "S- needs NOD >= 1");
    });
    check_launch("k_sq_minus_chain");
  } else if (spsmsz == 1) {
    dispatch_nod2(NODn, [&](auto c) {
      constexpr int V = decltype(c)::value;
      if constexpr (V + 1 <= 7) k_sq_plus_chain<V><<<grid, 128, 0, st>>>(a);
      else throw Error(QS3G_ENOTSUP, "S+ with NOD > 7");
    });
    check_launch("k_sq_plus_chain");
  } else {
    dispatch_nod2(NODn, [&](auto c) {
      k_sq_z<decltype(c)::value><<<grid, 128, 0, st>>>(a, m.chain ? 1 : 0, NOS);
    });
    check_launch("k_sq_z");
  }
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

int sq_a(const Model& m, const Sector& gs, const double2* h_psi, int spsmsz, const double* qv, const double* Spos,
         int64_t* Dn_out, int64_t* list_s_new, double2* h_fn, cudaStream_t st) {
  DevBuf<double2> d_psi(std::max<int64_t>(1, gs.D));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_psi.get(), h_psi, gs.D * sizeof(double2), cudaMemcpyHostToDevice, st));
  Sector ns;
  DevBuf<double2> fn;
  start_vector(m, gs, d_psi.get(), spsmsz, qv, Spos, ns, fn, st);
  *Dn_out = ns.D;
  if (ns.D > 0 && list_s_new)
    QS3G_CHECK_CUDA(cudaMemcpyAsync(list_s_new, ns.d_list_s.get(), ns.D * 8, cudaMemcpyDeviceToHost, st));
  if (ns.D > 0 && h_fn)
    QS3G_CHECK_CUDA(cudaMemcpyAsync(h_fn, fn.get(), ns.D * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  return QS3G_OK;
}

int dsf(const Model& m, const Sector& gs, const double2* h_psi, double ene1, int spsmsz, int nq, const double* qvec,
        const double* Spos, int itr_dsf, double rfield, double* alpha, double* beta2, double* norm1, double* E0,
        int* nlev, cudaStream_t st) {
  QS3G_REQUIRE(spsmsz >= 1 && spsmsz <= 3, QS3G_EINVAL, "spsmsz must be 1, 2 or 3");
  QS3G_REQUIRE(itr_dsf >= 1 && nq >= 1, QS3G_EINVAL, "itr_dsf and nq must be >= 1");
  const int NOD = gs.NOD, NOS = m.NOS;
  QS3G_REQUIRE(!(2 * NOD == NOS && spsmsz == 2), QS3G_EINVAL, "S-(q,w) = S+(q,w) in the sztot = 0 sector");
  QS3G_REQUIRE(!(spsmsz == 1 && NOD <= 1), QS3G_EINVAL, "S+(q,w) needs NOD >= 2");
  QS3G_REQUIRE(gs.u1 || m.chain || spsmsz == 3, QS3G_ENOTSUP, "S+/S- start vectors are implemented for chains");
  const int NODn = (spsmsz == 1) ? NOD - 1 : (spsmsz == 2 ? NOD + 1 : NOD);
  const double sztot = (double)NOS / 2.0 - (double)NOD;
  const double sz_new = (double)NOS / 2.0 - (double)NODn;
  const int64_t D = gs.D;
  DevBuf<double2> d_psi(D);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_psi.get(), h_psi, D * sizeof(double2), cudaMemcpyHostToDevice, st));
  // chains: all q in lock step (batch.cu); other lattices and U(1) sectors: one q at a time
  if (gs.anchored && !gs.u1)
    return dsf_batched(m, gs, d_psi.get(), ene1, spsmsz, nq, qvec, Spos, itr_dsf, rfield, alpha, beta2, norm1, E0,
                       nlev, st);
  Scratch sc;
  sc.ensure(8);
  Ops<double2> ops{st, sc.part.get()};
  DevBuf<double2> d_ab((size_t)2 * (itr_dsf + 3) + 4);
  double2* dal = d_ab.get();                    // alpha(itr) (complex dot)
  double2* dbb = d_ab.get() + (itr_dsf + 3);    // (sqrt(beta2), beta2)
  double2* dk = d_ab.get() + 2 * (itr_dsf + 3); // constants
  for (int q = 0; q < nq; ++q) {
    const double* qv = qvec + 3 * (size_t)q;
    // new sector (N_down', k + q) and fn = S^a(q)|GS> (get_expectation_values.f90:431-491)
    Sector ns;
    DevBuf<double2> f0;
    start_vector(m, gs, d_psi.get(), spsmsz, qv, Spos, ns, f0, st);
    const int64_t Dn = ns.D;
    E0[q] = ene1 - rfield * sztot;
    for (int k = 0; k < itr_dsf; ++k) {
      alpha[(size_t)q * itr_dsf + k] = 1.0e300;
      beta2[(size_t)q * itr_dsf + k] = 0.0;
    }
    if (Dn == 0) { norm1[q] = 0.0; nlev[q] = 0; continue; }
    DevBuf<double2> f1(Dn), f2(Dn);
    // recursion (get_expectation_values.f90:486-592)
    double2* fn = f0.get();
    double2* fnp1 = f1.get();
    double2* fnm1 = f2.get();
    ops.nrm(fn, Dn, dbb + 0);  // (sqrt(norm1), norm1)
    ops.scale_inv(fn, Dn, dbb + 0);
    ops.nrm(fn, Dn, dk + 1);
    k_set_scalar<<<1, 1, 0, st>>>(dk + 0, make_double2(-rfield * sz_new, 0.0));
    check_launch("k_set_scalar");
    hv64(m, ns, fn, fnp1, st);
    ops.axpy(fnp1, fn, Dn, dk + 0, 1.0);
    ops.dot(fn, fnp1, Dn, dal + 1);
    int lev = 1;
    if (Dn > 1) {
      ops.lanczos_w(fnp1, fnp1, fn, nullptr, Dn, dal + 1, dbb, true);
      ops.nrm(fnp1, Dn, dbb + 2);
      ops.scale_inv(fnp1, Dn, dbb + 2);
      for (int itr = 2; itr <= itr_dsf; ++itr) {
        double2* t = fnm1;
        fnm1 = fn;
        fn = fnp1;
        fnp1 = t;
        hv64(m, ns, fn, fnp1, st);
        ops.axpy(fnp1, fn, Dn, dk + 0, 1.0);
        ops.dot(fn, fnp1, Dn, dal + itr);
        lev = itr;
        if (itr == Dn) break;
        ops.lanczos_w(fnp1, fnp1, fn, fnm1, Dn, dal + itr, dbb + itr, true);
        ops.nrm(fnp1, Dn, dbb + itr + 1);
        ops.scale_inv(fnp1, Dn, dbb + itr + 1);
      }
    }
    std::vector<double2> ha(itr_dsf + 3), hb(itr_dsf + 3), hk(4);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(ha.data(), dal, (itr_dsf + 3) * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(hb.data(), dbb, (itr_dsf + 3) * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(hk.data(), dk, 4 * sizeof(double2), cudaMemcpyDeviceToHost, st));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
    norm1[q] = hb[0].y;
    QS3G_REQUIRE(std::isfinite(norm1[q]) && norm1[q] > 0.0, QS3G_EBREAKDOWN, "S^a(q)|GS> vanishes");
    QS3G_REQUIRE(!(hk[1].x - 1.0 > 1.0e-8), QS3G_EBREAKDOWN, "<f1|f1> is not 1");
    nlev[q] = lev;
    for (int k = 1; k <= lev; ++k) {
      alpha[(size_t)q * itr_dsf + (k - 1)] = ha[k].x;
      beta2[(size_t)q * itr_dsf + (k - 1)] = (k == 1) ? 0.0 : hb[k].y;
    }
  }
  return QS3G_OK;
}

}  // namespace qs3g

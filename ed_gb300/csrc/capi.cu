// capi.cu -- the extern "C" boundary of libqs3g.so (declared in include/qs3g.h).
//
// Every entry point catches qs3g::Error and CUDA failures and turns them into
// a status code plus a message retrievable with qs3g_last_error; nothing
// throws across the boundary.  Scalars arrive by pointer (Fortran bind(C)
// by-reference convention).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "krylov.h"
#include "mlp.h"
#include "qs3g_internal.cuh"

using namespace qs3g;

namespace {

std::mutex g_err_mu;
std::string g_last_error;

void set_error(qs3g_ctx* h, const std::string& msg) {
  if (h) h->last_error = msg;
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = msg;
}

}  // namespace

// Message of the last failed handle-free call (file I/O), read back by
// qs3g_last_error(NULL).
void qs3g::set_global_error(const std::string& msg) { set_error(nullptr, msg); }

namespace {

template <class F>
int guarded(qs3g_ctx* h, F&& f) {
  try {
    return f();
  } catch (const Error& e) {
    set_error(h, e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_error(h, "host allocation failed");
    return QS3G_ENOMEM;
  } catch (const std::exception& e) {
    set_error(h, e.what());
    return QS3G_EINVAL;
  }
}

// A chain whose bonds are, for one or two distances o < NOS/2, exactly the
// NOS bonds (s, s + o mod NOS) with one (Jxy, Jz) per distance: the H*v then
// runs its hops as moves by +-o (hv.cu, k_hv_uchain*).
void detect_uniform_chain(Model& m) {
  m.uni_no = 0;
  const int L = m.NOS;
  if (!m.chain || L < 5 || m.NOxxz == 0) return;
  std::vector<int> dist_of(m.NOxxz);
  std::vector<int> offs;
  for (int b = 0; b < m.NOxxz; ++b) {
    const int o = m.p2[b] - m.p1[b];
    const int dk = std::min(o, L - o);
    if (dk <= 0 || 2 * dk >= L) return;  // self or half-ring bonds: general kernels
    dist_of[b] = dk;
    if (std::find(offs.begin(), offs.end(), dk) == offs.end()) offs.push_back(dk);
  }
  if (offs.size() > 2) return;
  std::sort(offs.begin(), offs.end());
  for (size_t k = 0; k < offs.size(); ++k) {
    const int dk = offs[k];
    std::vector<int> seen(L + 1, 0);
    int first = -1;
    for (int b = 0; b < m.NOxxz; ++b) {
      if (dist_of[b] != dk) continue;
      if (first < 0) first = b;
      if (m.sJxy[b] != m.sJxy[first] || m.sJz[b] != m.sJz[first]) return;
      // the site s with (s, s + dk mod L) = this bond
      const int a = m.p1[b], c = m.p2[b];
      const int s0 = (c - a == dk) ? a : c;
      if (seen[s0]++) return;
    }
    for (int s0 = 1; s0 <= L; ++s0)
      if (seen[s0] != 1) return;
    m.uni_off[k] = dk;
    m.uni_bond[k] = first;
  }
  m.uni_no = (int)offs.size();
}

// Site adjacency, per-site Jz sums and device copies of the bond data.
void setup_model(Model& m, int NOS, int LX, int LY, int LZ, int NOxxz, const int* p_xxz, const double* sJint,
                 cudaStream_t st) {
  QS3G_REQUIRE(NOS >= 1 && LX >= 1 && LY >= 1 && LZ >= 1, QS3G_EINVAL, "lattice sizes must be >= 1");
  QS3G_REQUIRE((int64_t)LX * LY * LZ == NOS, QS3G_EINVAL, "NOS must equal LX*LY*LZ");
  QS3G_REQUIRE(NOS < 65535, QS3G_ERANGE, "NOS must be < 65535");
  QS3G_REQUIRE(NOxxz >= 0 && NOxxz < 65535, QS3G_ERANGE, "NOxxz must be < 65535");
  m.NOS = NOS; m.LX = LX; m.LY = LY; m.LZ = LZ; m.NOxxz = NOxxz;
  m.chain = (LY == 1 && LZ == 1);
  m.bits = bits_for(NOS);
  m.p1.resize(NOxxz); m.p2.resize(NOxxz); m.sJxy.resize(NOxxz); m.sJz.resize(NOxxz);
  // Sz_all and the per-site sums enter every diagonal element; they are
  // accumulated with compensation (Neumaier), because a running sum of
  // thousands of equal couplings drifts by up to one rounding per bond
  // (~1e-11 on a 2000-bond chain) -- the rounding the reference's own
  // bond-by-bond diagonal carries.
  m.Sz_all = 0.0;
  m.Sz_site.assign(NOS + 1, 0.0);
  std::vector<double> comp_site(NOS + 1, 0.0);
  double comp_all = 0.0;
  auto nsum = [](double& sum, double& comp, double v) {
    const double t = sum + v;
    comp += (std::fabs(sum) >= std::fabs(v)) ? (sum - t) + v : (v - t) + sum;
    sum = t;
  };
  std::vector<std::vector<uint32_t>> adj(NOS + 1);
  for (int b = 0; b < NOxxz; ++b) {
    int a = p_xxz[2 * b], c = p_xxz[2 * b + 1];
    QS3G_REQUIRE(a >= 1 && a <= NOS && c >= 1 && c <= NOS, QS3G_EINVAL, "bond site out of range");
    if (a > c) std::swap(a, c);  // input_param.f90:97-101
    m.p1[b] = a; m.p2[b] = c;
    m.sJxy[b] = sJint[b];
    m.sJz[b] = sJint[NOxxz + b];
    nsum(m.Sz_all, comp_all, m.sJz[b]);
    if (a != c) {
      adj[a].push_back(((uint32_t)b << 16) | (uint32_t)c);
      adj[c].push_back(((uint32_t)b << 16) | (uint32_t)a);
      nsum(m.Sz_site[a], comp_site[a], m.sJz[b]);
      nsum(m.Sz_site[c], comp_site[c], m.sJz[b]);
    }
  }
  m.Sz_all += comp_all;
  for (int i = 0; i <= NOS; ++i) m.Sz_site[i] += comp_site[i];
  detect_uniform_chain(m);
  m.adj_off.assign(NOS + 2, 0);
  m.adj.clear();
  for (int s = 1; s <= NOS; ++s) {
    m.adj_off[s] = (int)m.adj.size();
    for (uint32_t w : adj[s]) m.adj.push_back(w);
  }
  m.adj_off[NOS + 1] = (int)m.adj.size();
  m.adj_off[0] = 0;
  std::vector<int16_t> xyz(4 * (size_t)(NOS + 1), 0);
  for (int s = 1; s <= NOS; ++s) {
    const int s0 = s - 1;
    xyz[4 * s] = (int16_t)(s0 % LX);
    xyz[4 * s + 1] = (int16_t)((s0 / LX) % LY);
    xyz[4 * s + 2] = (int16_t)(s0 / (LX * LY));
  }
  auto up = [&](auto& dev, const auto& host) {
    using T = typename std::decay_t<decltype(host)>::value_type;
    dev.alloc(std::max<size_t>(1, host.size()));
    if (!host.empty())
      QS3G_CHECK_CUDA(cudaMemcpyAsync(dev.get(), host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  };
  up(m.d_adj_off, m.adj_off);
  up(m.d_adj, m.adj);
  up(m.d_sJxy, m.sJxy);
  up(m.d_sJz, m.sJz);
  up(m.d_Sz_site, m.Sz_site);
  up(m.d_site_xyz, xyz);
  std::vector<int2> p12(NOxxz);
  for (int b = 0; b < NOxxz; ++b) p12[b] = make_int2(m.p1[b], m.p2[b]);
  up(m.d_p12, p12);
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

const Sector& need_sector(qs3g_ctx* h) {
  QS3G_REQUIRE(h && h->sector, QS3G_ESTATE, "no sector: call qs3g_build_sector first");
  return *h->sector;
}

}  // namespace

extern "C" {

int qs3g_create(qs3g_handle* out, const int* NOS, const int* LX, const int* LY, const int* LZ, const int* NOxxz,
                const int* p_xxz, const double* sJint) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(out && NOS && LX && LY && LZ && NOxxz, QS3G_EINVAL, "null argument");
    QS3G_REQUIRE(*NOxxz == 0 || (p_xxz && sJint), QS3G_EINVAL, "null bond arrays");
    *out = nullptr;
    std::unique_ptr<qs3g_ctx> h(new qs3g_ctx());
    QS3G_CHECK_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    try {
      setup_model(h->model, *NOS, *LX, *LY, *LZ, *NOxxz, p_xxz, sJint, h->stream);
    } catch (...) {
      cudaStreamDestroy(h->stream);
      throw;
    }
    *out = h.release();
    return QS3G_OK;
  });
}

int qs3g_destroy(qs3g_handle h) {
  if (!h) return QS3G_OK;
  cudaStream_t st = h->stream;
  const bool own = h->own_stream;
  if (st) cudaStreamSynchronize(st);
  delete h;
  if (st && own) cudaStreamDestroy(st);
  return QS3G_OK;
}

int qs3g_build_sector(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, int64_t* D_out) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h && NOD && KX && KY && KZ, QS3G_EINVAL, "null argument");
    const int K[3] = {*KX, *KY, *KZ};
    std::unique_ptr<Sector> s(new Sector());
    build_sector(h->model, *NOD, K, *s, h->stream);
    h->sector = std::move(s);
    if (D_out) *D_out = h->sector->D;
    return QS3G_OK;
  });
}

int qs3g_build_sector_u1(qs3g_handle h, const int* NOD, int64_t* D_out) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h && NOD, QS3G_EINVAL, "null argument");
    std::unique_ptr<Sector> s(new Sector());
    build_sector_u1(h->model, *NOD, *s, h->stream);
    h->sector = std::move(s);
    if (D_out) *D_out = h->sector->D;
    return QS3G_OK;
  });
}

int qs3g_get_sector(qs3g_handle h, int64_t* list_s, double* list_r) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    if (s.D == 0) return QS3G_OK;
    if (list_s)
      QS3G_CHECK_CUDA(cudaMemcpyAsync(list_s, s.d_list_s.get(), s.D * 8, cudaMemcpyDeviceToHost, h->stream));
    if (list_r)
      QS3G_CHECK_CUDA(cudaMemcpyAsync(list_r, s.d_list_r.get(), s.D * 8, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

// A sector the caller already enumerated (the Fortran's allocate_lists_omp_SQ):
// the (NOD, K) sector is built on the GPU and compared with the caller's
// lists -- D, list_s bit for bit, list_r to 1e-12 relative -- so that the
// handle's rows are the caller's rows; a mismatch is QS3G_EINVAL naming the
// first differing row.
static int load_sector(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, int64_t D,
                       const int64_t* list_s, const double* list_r) {
  QS3G_REQUIRE(h && NOD && KX && KY && KZ && list_s && list_r, QS3G_EINVAL, "null argument");
  QS3G_REQUIRE(D >= 0, QS3G_EINVAL, "D must be >= 0");
  const int K[3] = {*KX, *KY, *KZ};
  std::unique_ptr<Sector> s(new Sector());
  build_sector(h->model, *NOD, K, *s, h->stream);
  QS3G_REQUIRE(s->D == D, QS3G_EINVAL,
               "the caller's sector has " + std::to_string(D) + " rows, the (NOD, K) sector " +
                   std::to_string(s->D));
  if (D > 0) {
    std::vector<int64_t> ls(D);
    std::vector<double> lr(D);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(ls.data(), s->d_list_s.get(), D * 8, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(lr.data(), s->d_list_r.get(), D * 8, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    for (int64_t i = 0; i < D; ++i) {
      QS3G_REQUIRE(list_s[i] == ls[i], QS3G_EINVAL,
                   "list_s(" + std::to_string(i + 1) + ") differs from the (NOD, K) sector's");
      QS3G_REQUIRE(std::fabs(list_r[i] - lr[i]) <= 1e-12 * std::fabs(lr[i]), QS3G_EINVAL,
                   "list_r(" + std::to_string(i + 1) + ") differs from the (NOD, K) sector's");
    }
  }
  h->sector = std::move(s);
  return QS3G_OK;
}

int qs3g_load_sector(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, const int64_t* D,
                     const int64_t* list_s, const double* list_r) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(D, QS3G_EINVAL, "null argument");
    return load_sector(h, NOD, KX, KY, KZ, *D, list_s, list_r);
  });
}

int qs3g_load_sector_i32(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, const int* THS,
                         const int* list_s, const double* list_r) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(THS && list_s && *THS >= 0, QS3G_EINVAL, "null argument or THS < 0");
    const std::vector<int64_t> ls(list_s, list_s + *THS);
    return load_sector(h, NOD, KX, KY, KZ, (int64_t)*THS, ls.data(), list_r);
  });
}

int qs3g_build_sector_i32(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, int* THS) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h && NOD && KX && KY && KZ, QS3G_EINVAL, "null argument");
    const int K[3] = {*KX, *KY, *KZ};
    std::unique_ptr<Sector> s(new Sector());
    build_sector(h->model, *NOD, K, *s, h->stream);
    QS3G_REQUIRE(s->D <= INT32_MAX, QS3G_ERANGE,
                 "the sector has " + std::to_string(s->D) + " rows, more than a default integer holds");
    if (s->D > 0) {  // the largest code is the last row's
      int64_t last = 0;
      QS3G_CHECK_CUDA(cudaMemcpyAsync(&last, s->d_list_s.get() + (s->D - 1), 8, cudaMemcpyDeviceToHost, h->stream));
      QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
      QS3G_REQUIRE(last <= INT32_MAX, QS3G_ERANGE,
                   "list_s codes reach " + std::to_string(last) + ", more than a default integer holds");
    }
    h->sector = std::move(s);
    if (THS) *THS = (int)h->sector->D;
    return QS3G_OK;
  });
}

int qs3g_get_sector_i32(qs3g_handle h, int* list_s, double* list_r) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(s.D <= INT32_MAX, QS3G_ERANGE, "the sector has more rows than a default integer holds");
    if (s.D == 0) return QS3G_OK;
    if (list_s) {
      std::vector<int64_t> ls(s.D);
      QS3G_CHECK_CUDA(cudaMemcpyAsync(ls.data(), s.d_list_s.get(), s.D * 8, cudaMemcpyDeviceToHost, h->stream));
      QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
      QS3G_REQUIRE(ls[s.D - 1] <= INT32_MAX, QS3G_ERANGE, "list_s codes exceed a default integer");
      for (int64_t i = 0; i < s.D; ++i) list_s[i] = (int)ls[i];
    }
    if (list_r)
      QS3G_CHECK_CUDA(cudaMemcpyAsync(list_r, s.d_list_r.get(), s.D * 8, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

// Device staging for the host-pointer forms of H*v: kept in the handle and
// grown on demand, so repeated calls do not allocate.
static void* staging(qs3g_ctx* h, int which, size_t bytes) {
  auto& b = h->stage[which];
  if (b.n < bytes) b.alloc(bytes);
  return b.get();
}

int qs3g_hv(qs3g_handle h, qs3g_cplx* v0, const qs3g_cplx* v1, const int* where) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(v0 && v1 && where, QS3G_EINVAL, "null argument");
    if (*where == QS3G_DEVICE) {  // asynchronous on the handle's stream
      hv64(h->model, s, reinterpret_cast<const double2*>(v1), reinterpret_cast<double2*>(v0), h->stream);
      return QS3G_OK;
    }
    QS3G_REQUIRE(*where == QS3G_HOST, QS3G_EINVAL, "where must be QS3G_HOST or QS3G_DEVICE");
    const size_t bytes = (size_t)s.D * sizeof(double2);
    auto* x = static_cast<double2*>(staging(h, 0, bytes));
    auto* y = static_cast<double2*>(staging(h, 1, bytes));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(x, v1, bytes, cudaMemcpyHostToDevice, h->stream));
    hv64(h->model, s, x, y, h->stream);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v0, y, bytes, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

int qs3g_hv_df(qs3g_handle h, qs3g_cplx* v0, const qs3g_cplx* v1, const int* where) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(v0 && v1 && where, QS3G_EINVAL, "null argument");
    QS3G_REQUIRE(s.tab.built(), QS3G_ESTATE, "no connection table: call qs3g_hv_cache first");
    if (*where == QS3G_DEVICE) {
      hv64_df(h->model, s, reinterpret_cast<const double2*>(v1), reinterpret_cast<double2*>(v0), h->stream);
      return QS3G_OK;
    }
    QS3G_REQUIRE(*where == QS3G_HOST, QS3G_EINVAL, "where must be QS3G_HOST or QS3G_DEVICE");
    const size_t bytes = (size_t)s.D * sizeof(double2);
    auto* x = static_cast<double2*>(staging(h, 0, bytes));
    auto* y = static_cast<double2*>(staging(h, 1, bytes));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(x, v1, bytes, cudaMemcpyHostToDevice, h->stream));
    hv64_df(h->model, s, x, y, h->stream);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v0, y, bytes, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

int qs3g_hv_cache(qs3g_handle h, const int* on, int64_t* bytes) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h && h->sector, QS3G_ESTATE, "no sector: call qs3g_build_sector first");
    Sector& s = *h->sector;
    QS3G_REQUIRE(on && (*on == 0 || *on == 1), QS3G_EINVAL, "on must be 0 or 1");
    if (*on == 0) {
      s.tab.release();
    } else if (!s.tab.built()) {
      QS3G_REQUIRE(hv_table_bytes(h->model, s) > 0, QS3G_ENOTSUP,
                   "connection table: chain (NOD, K) sectors with indexable sizes only");
      QS3G_REQUIRE(build_hv_table(h->model, s, s.tab, (size_t)1 << 30, h->stream), QS3G_ENOMEM,
                   "connection table does not fit in device memory");
    }
    if (bytes) *bytes = (int64_t)s.tab.bytes();
    return QS3G_OK;
  });
}

int qs3g_hv_schedule(qs3g_handle h, const int* mode, int* chosen) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    if (mode) {
      QS3G_REQUIRE(*mode >= 0 && *mode <= 2, QS3G_EINVAL, "schedule must be 0 (auto), 1 (warp) or 2 (thread)");
      s.hv_schedule64 = s.hv_schedule32 = *mode;
    }
    if (chosen) {
      chosen[0] = s.hv_schedule64;
      chosen[1] = s.hv_schedule32;
    }
    return QS3G_OK;
  });
}

int qs3g_hv32(qs3g_handle h, qs3g_cplx32* v0, const qs3g_cplx32* v1, const int* where) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(v0 && v1 && where, QS3G_EINVAL, "null argument");
    if (*where == QS3G_DEVICE) {  // asynchronous on the handle's stream
      hv32(h->model, s, reinterpret_cast<const float2*>(v1), reinterpret_cast<float2*>(v0), h->stream);
      return QS3G_OK;
    }
    QS3G_REQUIRE(*where == QS3G_HOST, QS3G_EINVAL, "where must be QS3G_HOST or QS3G_DEVICE");
    const size_t bytes = (size_t)s.D * sizeof(float2);
    auto* x = static_cast<float2*>(staging(h, 0, bytes));
    auto* y = static_cast<float2*>(staging(h, 1, bytes));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(x, v1, bytes, cudaMemcpyHostToDevice, h->stream));
    hv32(h->model, s, x, y, h->stream);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v0, y, bytes, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

int qs3g_hv_real(qs3g_handle h, double* v0, const double* v1, const int* where) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(v0 && v1 && where, QS3G_EINVAL, "null argument");
    if (*where == QS3G_DEVICE) {  // asynchronous on the handle's stream
      hv64r(h->model, s, v1, v0, h->stream, false);
      return QS3G_OK;
    }
    QS3G_REQUIRE(*where == QS3G_HOST, QS3G_EINVAL, "where must be QS3G_HOST or QS3G_DEVICE");
    QS3G_REQUIRE(real_sector(s), QS3G_ENOTSUP, "real H*v needs a k = 0 chain sector or a U(1) sector");
    const size_t bytes = (size_t)s.D * sizeof(double);
    auto* x = static_cast<double*>(staging(h, 0, bytes));
    auto* y = static_cast<double*>(staging(h, 1, bytes));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(x, v1, bytes, cudaMemcpyHostToDevice, h->stream));
    hv64r(h->model, s, x, y, h->stream, false);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v0, y, bytes, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

int qs3g_hv32_real(qs3g_handle h, float* v0, const float* v1, const float* shift, const int* where) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(v0 && v1 && where, QS3G_EINVAL, "null argument");
    QS3G_REQUIRE(real_sector(s), QS3G_ENOTSUP, "real H*v needs a k = 0 chain sector or a U(1) sector");
    const float sh = shift ? *shift : 0.f;
    if (*where == QS3G_DEVICE) {  // asynchronous on the handle's stream
      hv32r(h->model, s, v1, v0, h->stream, sh, false);
      return QS3G_OK;
    }
    QS3G_REQUIRE(*where == QS3G_HOST, QS3G_EINVAL, "where must be QS3G_HOST or QS3G_DEVICE");
    const size_t bytes = (size_t)s.D * sizeof(float);
    auto* x = static_cast<float*>(staging(h, 0, bytes));
    auto* y = static_cast<float*>(staging(h, 1, bytes));
    QS3G_CHECK_CUDA(cudaMemcpyAsync(x, v1, bytes, cudaMemcpyHostToDevice, h->stream));
    hv32r(h->model, s, x, y, h->stream, sh, false);
    QS3G_CHECK_CUDA(cudaMemcpyAsync(v0, y, bytes, cudaMemcpyDeviceToHost, h->stream));
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

int qs3g_set_stream(qs3g_handle h, void* stream) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h, QS3G_EINVAL, "null handle");
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    if (h->own_stream) {
      QS3G_CHECK_CUDA(cudaStreamDestroy(h->stream));
      h->own_stream = false;
    }
    h->stream = static_cast<cudaStream_t>(stream);
    return QS3G_OK;
  });
}

int qs3g_sync(qs3g_handle h) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h, QS3G_EINVAL, "null handle");
    QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    return QS3G_OK;
  });
}

int qs3g_connection_table(qs3g_handle h, int64_t* row, int64_t* col, int* ell, int* bond, int64_t* nnz) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(nnz, QS3G_EINVAL, "null nnz");
    const int64_t cap = *nnz;
    const int64_t n = connection_table(h->model, s, row, col, ell, bond, row ? cap : 0, h->stream);
    *nnz = n;
    return QS3G_OK;
  });
}

int qs3g_connection_table_rows(qs3g_handle h, const int64_t* row_first, const int64_t* row_last, int64_t* row,
                               int64_t* col, int* ell, int* bond, int64_t* nnz) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(nnz && row_first && row_last, QS3G_EINVAL, "null argument");
    const int64_t cap = *nnz;
    const int64_t n = connection_table_rows(h->model, s, *row_first - 1, *row_last, row, col, ell, bond,
                                            row ? cap : 0, h->stream);
    *nnz = n;
    return QS3G_OK;
  });
}

// precision 0, 1 or 2, plus QS3G_REAL for real Krylov vectors
static void set_precision(TrlanParams& p, int v) {
  p.real = (v & QS3G_REAL) != 0;
  p.precision = v & ~QS3G_REAL;
  QS3G_REQUIRE(p.precision >= 0 && p.precision <= 2, QS3G_EINVAL, "precision must be 0, 1 or 2 (+ QS3G_REAL)");
}

int qs3g_trlan(qs3g_handle h, const int* NOE, const int* NOK, const int* NOM, const int* maxitr, const double* tol,
               const int* precision, const int* conv_mode, const int* start_mode, const uint64_t* seed,
               const qs3g_cplx* start, double* ene, qs3g_cplx* psi, int* iters, double* resid) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(NOE && NOK && NOM && maxitr && tol && ene, QS3G_EINVAL, "null argument");
    TrlanParams p;
    p.NOE = *NOE; p.NOK = *NOK; p.NOM = *NOM; p.maxitr = *maxitr; p.tol = *tol;
    set_precision(p, precision ? *precision : 0);
    p.conv_mode = conv_mode ? *conv_mode : 0;
    p.seed = seed ? *seed : 1;
    QS3G_REQUIRE(p.conv_mode >= 0 && p.conv_mode <= 2, QS3G_EINVAL, "conv_mode must be 0, 1 or 2");
    const int sm = start_mode ? *start_mode : 0;
    QS3G_REQUIRE(sm == 0 || (sm == 1 && start), QS3G_EINVAL, "start_mode 1 needs a start vector");
    p.time_limit = h->time_limit;
    h->last_stats = TrlanStats();
    return trlan(h->model, s, p, sm == 1 ? reinterpret_cast<const double2*>(start) : nullptr, ene,
                 reinterpret_cast<double2*>(psi), iters, resid, h->stream, &h->last_stats);
  });
}

int qs3g_set_time_limit(qs3g_handle h, const double* seconds) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h && seconds && std::isfinite(*seconds) && *seconds >= 0.0, QS3G_EINVAL,
                 "time limit must be finite and >= 0");
    h->time_limit = *seconds;
    return QS3G_OK;
  });
}

int qs3g_trlan_stats(qs3g_handle h, int* hv_fp32, int* hv_fp64, int* restarts, double* seconds, int* timed_out) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(h, QS3G_EINVAL, "null handle");
    const TrlanStats& t = h->last_stats;
    if (hv_fp32) *hv_fp32 = t.hv32;
    if (hv_fp64) *hv_fp64 = t.hv64;
    if (restarts) *restarts = t.restarts;
    if (seconds) *seconds = t.seconds;
    if (timed_out) *timed_out = t.timed_out ? 1 : 0;
    return QS3G_OK;
  });
}

int qs3g_trlan_batch(const int* n, qs3g_handle* hs, const int* NOE, const int* NOK, const int* NOM,
                     const int* maxitr, const double* tol, const int* precision, const int* conv_mode,
                     const uint64_t* seed, const int* nthreads, double* ene, int* iters, double* resid,
                     int* status) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(n && hs && NOE && NOK && NOM && maxitr && tol && ene && status, QS3G_EINVAL, "null argument");
    const int np = *n, noe = *NOE;
    QS3G_REQUIRE(np >= 0 && noe >= 1, QS3G_EINVAL, "n >= 0 and NOE >= 1");
    for (int k = 0; k < np; ++k) QS3G_REQUIRE(hs[k] && hs[k]->sector, QS3G_ESTATE, "every handle needs a sector");
    TrlanParams p;
    p.NOE = noe; p.NOK = *NOK; p.NOM = *NOM; p.maxitr = *maxitr; p.tol = *tol;
    set_precision(p, precision ? *precision : 0);
    p.conv_mode = conv_mode ? *conv_mode : 0;
    p.seed = seed ? *seed : 1;
    // largest sectors first, handed out to the workers from one counter
    std::vector<int> order(np);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hs[a]->sector->D > hs[b]->sector->D; });
    std::atomic<int> next(0);
    int dev = 0;
    QS3G_CHECK_CUDA(cudaGetDevice(&dev));
    auto work = [&]() {
      cudaSetDevice(dev);
      for (;;) {
        const int t = next.fetch_add(1);
        if (t >= np) break;
        const int k = order[t];
        qs3g_ctx* h = hs[k];
        int it = 0;
        int rc;
        try {
          rc = trlan(h->model, *h->sector, p, nullptr, ene + (size_t)k * noe, nullptr, &it,
                     resid ? resid + (size_t)k * noe : nullptr, h->stream);
        } catch (const Error& e) {
          h->last_error = e.what();
          rc = e.code;
        } catch (const std::exception& e) {
          h->last_error = e.what();
          rc = QS3G_ECUDA;
        }
        if (iters) iters[k] = it;
        status[k] = rc;
      }
    };
    const int nt = std::max(1, std::min(np, nthreads && *nthreads > 0 ? *nthreads : 8));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    for (int k = 0; k < np; ++k)
      if (status[k] != QS3G_OK) return (int)status[k];
    return (int)QS3G_OK;
  });
}

int qs3g_trlan_lockstep(const int* n, qs3g_handle* hs, const int* NOE, const int* NOK, const int* NOM,
                        const int* maxitr, const double* tol, const int* precision, const int* conv_mode,
                        const uint64_t* seed, double* ene, int* iters, double* resid, int* status) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(n && hs && NOE && NOK && NOM && maxitr && tol && ene && status, QS3G_EINVAL, "null argument");
    const int np = *n;
    QS3G_REQUIRE(np >= 1, QS3G_EINVAL, "n >= 1");
    std::vector<const Model*> models(np);
    std::vector<const Sector*> secs(np);
    for (int k = 0; k < np; ++k) {
      QS3G_REQUIRE(hs[k] && hs[k]->sector, QS3G_ESTATE, "every handle needs a sector");
      models[k] = &hs[k]->model;
      secs[k] = hs[k]->sector.get();
    }
    TrlanParams p;
    p.NOE = *NOE; p.NOK = *NOK; p.NOM = *NOM; p.maxitr = *maxitr; p.tol = *tol;
    p.precision = precision ? *precision : 1;
    p.conv_mode = conv_mode ? *conv_mode : 1;
    p.seed = seed ? *seed : 1;
    // every handle's stream may hold its sector build; the batch runs on the first handle's stream
    for (int k = 0; k < np; ++k) QS3G_CHECK_CUDA(cudaStreamSynchronize(hs[k]->stream));
    trlan_lockstep(models, secs, p, ene, resid, iters, status, hs[0]->stream);
    for (int k = 0; k < np; ++k)
      if (status[k] != QS3G_OK) return (int)status[k];
    return (int)QS3G_OK;
  });
}

int qs3g_lanczos(qs3g_handle h, const int* maxitr, const int* minitr, const int* itrint, const double* tol,
                 const int* start_mode, const uint64_t* seed, const qs3g_cplx* start, double* ene, qs3g_cplx* psi,
                 int* iters) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(maxitr && minitr && itrint && tol && ene, QS3G_EINVAL, "null argument");
    const int sm = start_mode ? *start_mode : 0;
    QS3G_REQUIRE(sm == 0 || (sm == 1 && start), QS3G_EINVAL, "start_mode 1 needs a start vector");
    return lanczos(h->model, s, *maxitr, *minitr, *itrint, *tol,
                   sm == 1 ? reinterpret_cast<const double2*>(start) : nullptr, seed ? *seed : 1, ene,
                   reinterpret_cast<double2*>(psi), iters, h->stream);
  });
}

int qs3g_dsf(qs3g_handle h, const qs3g_cplx* psi, const double* ene1, const int* spsmsz, const int* nq,
             const double* qvec, const double* Spos, const int* itr_dsf, const double* rfield, double* alpha,
             double* beta2, double* norm1, double* E0, int* nlev) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(psi && ene1 && spsmsz && nq && qvec && Spos && itr_dsf && rfield && alpha && beta2 && norm1 &&
                     E0 && nlev,
                 QS3G_EINVAL, "null argument");
    return dsf(h->model, s, reinterpret_cast<const double2*>(psi), *ene1, *spsmsz, *nq, qvec, Spos, *itr_dsf,
               *rfield, alpha, beta2, norm1, E0, nlev, h->stream);
  });
}

int qs3g_sq_a(qs3g_handle h, const qs3g_cplx* psi, const int* spsmsz, const double* qvec, const double* Spos,
              int64_t* D_new, int64_t* list_s_new, qs3g_cplx* fn) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(psi && spsmsz && qvec && Spos && D_new, QS3G_EINVAL, "null argument");
    return sq_a(h->model, s, reinterpret_cast<const double2*>(psi), *spsmsz, qvec, Spos, D_new, list_s_new,
                reinterpret_cast<double2*>(fn), h->stream);
  });
}

int qs3g_cfrac(const int* nq, const int* ldab, const int* nlev, const double* alpha, const double* beta2,
               const double* norm1, const double* E0, const double* eta, const int* nomega, const double* omega,
               const int* compat, double* S) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(nq && ldab && nlev && alpha && beta2 && norm1 && E0 && eta && nomega && omega && compat && S,
                 QS3G_EINVAL, "null argument");
    QS3G_REQUIRE(*nq >= 1 && *ldab >= 1 && *nomega >= 1, QS3G_EINVAL, "sizes must be >= 1");
    cudaStream_t st;
    QS3G_CHECK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    try {
      cfrac(*nq, *ldab, nlev, alpha, beta2, norm1, E0, *eta, *nomega, omega, *compat, S, st);
    } catch (...) {
      cudaStreamDestroy(st);
      throw;
    }
    cudaStreamDestroy(st);
    return QS3G_OK;
  });
}

int qs3g_correlations(qs3g_handle h, const qs3g_cplx* psi, double* szsz, qs3g_cplx* spsm, double* lm) {
  return guarded(h, [&]() {
    const Sector& s = need_sector(h);
    QS3G_REQUIRE(psi && szsz && spsm, QS3G_EINVAL, "null argument");
    return correlations(h->model, s, reinterpret_cast<const double2*>(psi), szsz, reinterpret_cast<double2*>(spsm),
                        lm, h->stream);
  });
}

int qs3g_cfrac_noalloc(const int* nq, const int* ldab, const int* nlev, const double* alpha, const double* beta2,
                       const double* norm1, const double* E0, const double* eta, const int* nomega,
                       const double* omega, const int* compat, double* S) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(nq && ldab && nlev && alpha && beta2 && norm1 && E0 && eta && nomega && omega && compat && S,
                 QS3G_EINVAL, "null argument");
    QS3G_REQUIRE(*nq >= 1 && *ldab >= 1 && *nomega >= 1, QS3G_EINVAL, "sizes must be >= 1");
    cfrac_noalloc(*nq, *ldab, nlev, alpha, beta2, norm1, E0, *eta, *nomega, omega, *compat, S);
    return QS3G_OK;
  });
}

int qs3g_full_hamiltonian(qs3g_handle h, qs3g_cplx* ham) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(ham, QS3G_EINVAL, "null argument");
    const Sector& s = need_sector(h);
    full_hamiltonian(h->model, s, reinterpret_cast<double2*>(ham), h->stream);
    return QS3G_OK;
  });
}

int qs3g_full_diag(qs3g_handle h, double* ene, qs3g_cplx* psi) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(ene, QS3G_EINVAL, "null argument");
    const Sector& s = need_sector(h);
    full_diag(h->model, s, ene, reinterpret_cast<double2*>(psi), h->stream);
    return QS3G_OK;
  });
}

// ---------------------------------------------------------------- learned start
}  // extern "C"

struct qs3g_mlp_ctx {
  std::unique_ptr<qs3g::Mlp> net;
  cudaStream_t stream = nullptr;
};

extern "C" {

int qs3g_mlp_create(qs3g_mlp* out, const uint64_t* seed) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(out && seed, QS3G_EINVAL, "null argument");
    std::unique_ptr<qs3g_mlp_ctx> c(new qs3g_mlp_ctx());
    QS3G_CHECK_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    try {
      c->net.reset(new Mlp(*seed));
    } catch (...) {
      cudaStreamDestroy(c->stream);
      throw;
    }
    *out = c.release();
    return QS3G_OK;
  });
}

int qs3g_mlp_destroy(qs3g_mlp net) {
  if (!net) return QS3G_OK;
  cudaStreamSynchronize(net->stream);
  cudaStream_t st = net->stream;
  delete net;
  if (st) cudaStreamDestroy(st);
  return QS3G_OK;
}

int qs3g_mlp_params(qs3g_mlp net, double* get, const double* set) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(net, QS3G_EINVAL, "null network");
    if (set) net->net->set_params(set, net->stream);
    if (get) net->net->get_params(get, net->stream);
    return QS3G_OK;
  });
}

int qs3g_mlp_add_sample(qs3g_mlp net, qs3g_handle h, const qs3g_cplx* psi, const double* cond) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(net && psi && cond, QS3G_EINVAL, "null argument");
    const Sector& s = need_sector(h);
    net->net->add_sample(h->model, s, reinterpret_cast<const double2*>(psi), cond, h->stream);
    return QS3G_OK;
  });
}

int qs3g_mlp_clear(qs3g_mlp net) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(net, QS3G_EINVAL, "null network");
    net->net->clear_samples();
    return QS3G_OK;
  });
}

int qs3g_mlp_loss_grad(qs3g_mlp net, double* loss, double* grad) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(net && loss, QS3G_EINVAL, "null argument");
    *loss = net->net->loss_grad(nullptr, net->net->nreps, net->stream);
    if (grad) net->net->gradient(grad, net->stream);
    return QS3G_OK;
  });
}

int qs3g_mlp_train(qs3g_mlp net, const int* steps, const int64_t* batch, const double* lr, const uint64_t* seed,
                   double* losses) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(net && steps && batch && lr && seed, QS3G_EINVAL, "null argument");
    net->net->train(*steps, *batch, *lr, *seed, losses, net->stream);
    return QS3G_OK;
  });
}

int qs3g_mlp_align(qs3g_mlp net, int* nflipped) {
  return guarded(nullptr, [&]() {
    QS3G_REQUIRE(net, QS3G_EINVAL, "null network");
    const int n = net->net->align(net->stream);
    if (nflipped) *nflipped = n;
    return QS3G_OK;
  });
}

int qs3g_mlp_predict(qs3g_mlp net, qs3g_handle h, const double* cond, qs3g_cplx* start, const int* where) {
  return guarded(h, [&]() {
    QS3G_REQUIRE(net && cond && start && where, QS3G_EINVAL, "null argument");
    const Sector& s = need_sector(h);
    if (*where == QS3G_DEVICE) {
      net->net->predict(h->model, s, cond, reinterpret_cast<double2*>(start), h->stream);
    } else {
      DevBuf<double2> v(std::max<int64_t>(1, s.D));
      net->net->predict(h->model, s, cond, v.get(), h->stream);
      QS3G_CHECK_CUDA(cudaMemcpyAsync(start, v.get(), s.D * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
      QS3G_CHECK_CUDA(cudaStreamSynchronize(h->stream));
    }
    return QS3G_OK;
  });
}

const char* qs3g_last_error(qs3g_handle h) {
  if (h) return h->last_error.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_last_error.c_str();
}

int64_t qs3g_kernel_launches(void) { return g_launches.load(); }

}  // extern "C"

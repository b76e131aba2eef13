// qs3g_internal.cuh -- shared declarations of the GB300 QS3 hot-path library.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/qs3g.h"

namespace qs3g {

// ---------------------------------------------------------------- errors
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define QS3G_CHECK_CUDA(call)                                                          \
  do {                                                                                 \
    cudaError_t _e = (call);                                                           \
    if (_e != cudaSuccess)                                                             \
      throw ::qs3g::Error(_e == cudaErrorMemoryAllocation ? QS3G_ENOMEM : QS3G_ECUDA,  \
                          std::string(#call) + ": " + cudaGetErrorString(_e));         \
  } while (0)

#define QS3G_REQUIRE(cond, code, msg)                        \
  do {                                                       \
    if (!(cond)) throw ::qs3g::Error((code), (msg));         \
  } while (0)

extern std::atomic<int64_t> g_launches;
inline void count_launch(int64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }
inline void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(QS3G_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  count_launch();
}

// Record the message of a failed handle-free call for qs3g_last_error(NULL).
void set_global_error(const std::string& msg);

// ---------------------------------------------------------------- device buffers
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    QS3G_CHECK_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  T* get() const { return p; }
  operator T*() const { return p; }
};

// ---------------------------------------------------------------- limits
constexpr int kMaxNOD = 8;          // template instantiations of the row kernels
constexpr int kDirBlock = 256;      // candidates per build thread (8 directory entries)

// ---------------------------------------------------------------- model
// Lattice + bonds as read by read_ip (input_param.f90:58-117).
struct Model {
  int NOS = 0, LX = 0, LY = 0, LZ = 0, NOxxz = 0;
  bool chain = false;               // LY == LZ == 1: one translation axis
  int bits = 0;                     // bits per site in a packed configuration
  std::vector<int> p1, p2;          // bond ends (1-based, p1 <= p2)
  std::vector<double> sJxy, sJz;    // sJint(:,2), sJint(:,3)
  double Sz_all = 0.0;              // sum_b sJz_b
  // per-site adjacency of non-self bonds: entries (neighbour, bond), both ends listed
  std::vector<int> adj_off;         // NOS + 2 (index by site 1..NOS, [NOS+1] end)
  std::vector<uint32_t> adj;        // packed (bond << 16) | neighbour  (NOS < 65536, bonds < 65536)
  std::vector<double> Sz_site;      // sum of sJz over the non-self bonds at a site (index 1..NOS)
  // uniform chain: every site s has one bond to s + uni_off[k] (mod NOS) for
  // k < uni_no, all bonds of a distance with the same couplings (uni_no = 0:
  // not uniform); uni_bond[k] is one bond of distance uni_off[k]
  int uni_no = 0;
  int uni_off[2] = {0, 0};
  int uni_bond[2] = {0, 0};
  // device copies
  DevBuf<int> d_adj_off;
  DevBuf<uint32_t> d_adj;
  DevBuf<double> d_sJxy, d_sJz, d_Sz_site;
  DevBuf<int16_t> d_site_xyz;       // (x, y, z, pad) 0-based per site, index 1..NOS
  DevBuf<int2> d_p12;               // (p1, p2) per bond, bond order (dense H build)
};

// ---------------------------------------------------------------- sector
// A (NOD, K) representative basis (allocate_lists_omp_SQ, state_lists.f90:225-292).
// Cached connection table of a chain sector (qs3g_hv_cache): for every row
// and hop slot (down spin m, adjacency slot k of its site: slot m * deg + k,
// the order in which the matrix-free row visits its hops) the target row and
// what its coefficient needs, stored slot-major (entry [slot * D + row]) so a
// warp's loads of one slot are coalesced.  Packed form (k = 0 uniform chains,
// D < 2^27): id | class << 27 with class = distance index * (NOD + 1) +
// self-translation count, 0xffffffff for no hop; wide form: id (-1 for no
// hop) plus a code plane ell << 16 | (bond * (NOD + 1) + count).
struct HvTable {
  DevBuf<uint32_t> tab, tabc;
  DevBuf<double> coef;   // packed: coefficient per class
  DevBuf<float> coef32;
  DevBuf<float2> coefS;  // coefficients (per class, or per bond * (NOD+1) + count) split hi + lo
  DevBuf<float4> phS;    // chain phases split hi + lo (re, im)
  int slots = 0, deg = 0;
  bool packed = false;
  bool built() const { return slots > 0; }
  size_t bytes() const { return (tab.n + tabc.n) * sizeof(uint32_t); }
  void release() {
    tab.release(); tabc.release(); coef.release(); coef32.release(); coefS.release(); phS.release();
    slots = deg = 0;
    packed = false;
  }
};

struct Sector {
  int NOD = 0;
  int K[3] = {0, 0, 0};
  double rk[3] = {0, 0, 0};
  bool anchored = false;            // chain: reps occupy site 1, directory over C(NOS-1, NOD-1)
  bool u1 = false;                  // U(1) only: every configuration is a row, row = colex rank - 1
  bool kzero = false;               // every phase equals exp(0) = 1 exactly
  uint64_t nspace = 0;              // candidates in the directory space
  int64_t D = 0;
  uint64_t nblocks = 0;             // build blocks of 256 candidates
  uint64_t nwords = 0;              // directory entries (32 candidates each)
  DevBuf<int64_t> d_list_s;         // colex ranks (1-based), ascending
  DevBuf<double> d_list_r;          // sqrt(norm^2)
  DevBuf<float> d_list_r32;         // float copy for the complex(4) kernels
  DevBuf<uint64_t> d_conf;          // packed sorted down-spin sites
  DevBuf<uint2> d_dir;              // per 32 candidates: (rows before, presence bits)
  DevBuf<double2> d_explist;        // explist(0:LX,0:LY,0:LZ), Fortran order
  DevBuf<double2> d_chainph;        // chain: explist(i,1,1) for i = 1..LX, [0] = explist(0,0,0)
  DevBuf<float2> d_chainph32;
  DevBuf<uint64_t> d_binom;         // C(n,k) for n in [0,NOS], k in [0,NOD+1]: [k*(NOS+1)+n]
  DevBuf<uint32_t> d_binomA;        // anchored: C(x,k) for x in [0,NOS-2], k in [1,NOD-1] (u32)
  DevBuf<double> d_diag;            // H(i,i)
  DevBuf<float> d_diag32;
  DevBuf<double> d_coefR, d_invR;   // chains: sJxy_b * R[c] and 1/R[c] by self-translation count c
  DevBuf<float> d_coefR32, d_invR32;
  // general-lattice H*v schedule per precision: 0 = pick on first use,
  // 1 = warp per row, 2 = thread per row (identical results)
  mutable int hv_schedule64 = 0, hv_schedule32 = 0;
  HvTable tab;                      // built by qs3g_hv_cache; every chain H*v then reads it
};

// Host-side explist (input_param.f90:87-89) and checkstate phases
// (state_lists.f90:84-104), computed with the host libm exactly as the
// Fortran expressions are written.
void wavevector(const int K[3], int LX, int LY, int LZ, double rk[3]);
void host_explist(const double rk[3], int LX, int LY, int LZ, std::vector<double2>& out);

// ---------------------------------------------------------------- kernels (host wrappers)
void build_sector(const Model& m, int NOD, const int K[3], Sector& s, cudaStream_t st);

// Bytes the connection table of s would take (0: not a chain sector, or a
// size the table formats cannot index), and its build: false when the device
// lacks the memory (keep = free bytes to leave).
size_t hv_table_bytes(const Model& m, const Sector& s);
bool build_hv_table(const Model& m, const Sector& s, HvTable& t, size_t keep, cudaStream_t st);

void hv64(const Model& m, const Sector& s, const double2* x, double2* y, cudaStream_t st);
// The same from the cached connection table in double-float arithmetic on
// the FP32 pipe (for the solvers' double-float modes); false, launching
// nothing, when no table is cached.
bool hv64_df(const Model& m, const Sector& s, const double2* x, double2* y, cudaStream_t st);
bool hv64r_df(const Model& m, const Sector& s, const double* x, double* y, cudaStream_t st, bool pad);
// complex(4) H*v of H - shift (shift = 0 for the plain product)
void hv32(const Model& m, const Sector& s, const float2* x, float2* y, cudaStream_t st, float shift = 0.f);
void hv64_general(const Model& m, const Sector& s, const double2* x, double2* y, cudaStream_t st);
// Sectors whose H is real symmetric: chains at k = 0 and U(1) sectors.  For
// them hv64r / hv32r multiply real vectors x, y of length D; with pad and D
// odd they also write y[D] = 0, the pad of a real vector stored two rows per
// complex slot.  Other sectors: QS3G_ENOTSUP.
bool real_sector(const Sector& s);
void hv64r(const Model& m, const Sector& s, const double* x, double* y, cudaStream_t st, bool pad);
void hv32r(const Model& m, const Sector& s, const float* x, float* y, cudaStream_t st, float shift, bool pad);

// dense H(i, id) of make_full_hamiltonian, column-major with leading dimension ld
// (zeroed here), accumulated in the reference's bond order
void dense_hamiltonian(const Model& m, const Sector& s, double2* H, int64_t ld, cudaStream_t st);

// connection table: counts per row then entries
int64_t connection_table(const Model& m, const Sector& s, int64_t* row, int64_t* col, int* ell,
                         int* bond, int64_t cap, cudaStream_t st);

// Binomial helper on host (64-bit, saturating at INT64_MAX).
uint64_t binom_u64(int n, int k);
int bits_for(int v);

// What one thick-restart Lanczos call did: H*v products on complex(4) and on
// complex(8) Krylov vectors (FP64 residual checks included), thick restarts,
// wall time, and whether it stopped at its time limit.
struct TrlanStats {
  int hv32 = 0, hv64 = 0, restarts = 0;
  double seconds = 0.0;
  bool timed_out = false;
};

}  // namespace qs3g

// the opaque handle
struct qs3g_ctx {
  qs3g::Model model;
  std::unique_ptr<qs3g::Sector> sector;
  cudaStream_t stream = nullptr;
  bool own_stream = true;
  qs3g::DevBuf<char> stage[2];  // device staging of the host-pointer H*v forms
  std::string last_error;
  double time_limit = 0.0;        // wall-clock limit of qs3g_trlan (qs3g_set_time_limit)
  qs3g::TrlanStats last_stats;    // what the last qs3g_trlan on this handle did
};

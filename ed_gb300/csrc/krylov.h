// krylov.h -- host wrappers of the level-1 kernels and the Krylov drivers.
#pragma once

#include "qs3g_internal.cuh"

namespace qs3g {

constexpr int kRedBlocks = 152 * 4;  // fixed reduction grid: 4 blocks per SM of the GB300

// true when QS3G_VERBOSE is set to a non-zero value (solver progress lines)
bool verbose();
// hand-over residual of the complex(4) phase (see krylov.cu)
double phase1_tol(double tol32);
// first-attempt Ritz-estimate target as a fraction of the residual target
double est_factor();

// Device scratch of one solve: reduction partials, Lanczos scalars, Ritz coefficients.
struct Scratch {
  DevBuf<double2> part;  // kRedBlocks x (up to 128 columns)
  DevBuf<double2> scal;  // alpha, beta, overlaps, arrow couplings
  DevBuf<double2> C;     // NOM x NOK Ritz coefficients
  void ensure(int nom);
};

// Level-1 operations on vectors of T (double2 = complex(8), float2 = complex(4));
// every reduction accumulates in FP64 and writes its result to device memory.
template <class T>
struct Ops {
  cudaStream_t st;
  double2* part;
  bool eft = false;  // complex(8) only: double-float arithmetic on the FP32 pipe for dots, reorth, restart
  // Real vectors stored two rows per complex slot (sectors with a real
  // symmetric H): dots and overlaps keep their real parts, alpha is real.
  bool real = false;
  void dot(const T* x, const T* y, int64_t n, double2* out);              // zdotc
  void nrm(const T* x, int64_t n, double2* out);                          // dznrm2 -> out->x
  void scale_inv(T* x, int64_t n, const double2* s);                      // x *= 1/s->x
  void lanczos_w(T* w, const T* q, const T* v, const T* u, int64_t n, const double2* a, const double2* b,
                 bool real_alpha);                                        // w = q - a v - b u
  void axpy(T* y, const T* x, int64_t n, const double2* a, double sgn);    // y += sgn*a*x
  void reorth(const T* V, int64_t ldv, int ncols, T* w, int64_t n, double2* ov);  // w -= V V^H w
  void overlaps(const T* V, int64_t ldv, int ncols, const T* w, int64_t n, double2* ov);  // ov = V^H w
  void gemv_sub(const T* V, int64_t ldv, int ncols, const double2* coef, T* w, int64_t n);
  void restart(T* V, int64_t ldv, int nom, int nok, const double2* C, int64_t n);
  void random_start(T* x, int64_t n, uint64_t seed);
  void from64(T* y, const double2* x, int64_t n);
};

void f32_to_f64(double2* y, const float2* x, int64_t n, cudaStream_t st);
void residual64(double2* w, const double2* q, const double2* v, int64_t n, double e, cudaStream_t st);

// One chain sector of a batch: everything the chain H*v row needs, with the
// sector's rows stored at x[row0 .. row0 + D) of the batch's vectors.
struct HvSeg {
  int64_t D, row0;
  int L, bits, kzero, pad;
  const uint64_t* conf;
  const uint2* dir;
  const uint32_t* binomA;
  const int* adj_off;
  const uint32_t* adj;
  const double* diag;
  const double* coefR;
  const double* invR;
  const double2* chainph;
  const float* diag32;      // complex(4) tables (batched TRLan)
  const float* coefR32;
  const float* invR32;
  const float2* chainph32;
  double shift;             // per-sector shift of the complex(4) product (H - shift)
  int uno;                  // uniform chain: number of bond distances (0: not uniform)
  int uoff[2], ubond[2];    //   the distances and one bond of each
  const uint32_t* tab;      // connection table (HvTable), or null
  const uint32_t* tabc;
  const double* tcoef;
  const float* tcoef32;
  const float2* tcoefS;     // split coefficients and phases (double-float table rows)
  const float4* tphS;
  int tslots, tpacked;
};

HvSeg make_seg(const Model& m, const Sector& s, int64_t row0);
// point a segment at a connection table (or at none, when t is not built)
void set_seg_table(HvSeg& g, const HvTable& t);

// H*v - shift*v over a batch of chain sectors with the same NOD: one launch,
// block b serves segment blk_seg[b] (blocks of 256 rows, each segment padded
// to whole blocks).  With part set, warp w of block b also stores its rows'
// share of <x, y> at part[8 * (seg_b0[segment] + b - blk_first[b]) + w].
// uni = 1 or 2: every segment of the launch is a uniform chain with that many
// bond distances, and the rows take hv_uchain_row's unrolled form (the same
// hops summed in another order); uni = 0: the general chain row; uni = 3:
// the general row with its general-path hops summed after the others.
constexpr int kSegPartials = 8;  // alpha partials per 256-row block (one per warp)
void hv64_seg(int NOD, const HvSeg* d_segs, const int* d_blk_seg, const int* d_blk_first, int nblk,
              const double2* x, double2* y, double shift, cudaStream_t st, double2* part = nullptr,
              const int* seg_b0 = nullptr, int uni = 0);
// complex(4) form: every segment applies H - its own shift
void hv32_seg(int NOD, const HvSeg* d_segs, const int* d_blk_seg, const int* d_blk_first, int nblk,
              const float2* x, float2* y, cudaStream_t st, double2* part = nullptr, const int* seg_b0 = nullptr,
              int uni = 0);
// true when the uniform form exists for NOD and uni
bool seg_uniform_ok(int NOD, int uni);
// uni = 4: every segment of the launch reads its connection table
// (HvSeg::tab set); complex(8) vectors then take double-float arithmetic on
// the FP32 pipe (the complex(8) phase of the lock-step batch)
constexpr int kSegTable = 4;


struct TrlanParams {
  int NOE = 1, NOK = 2, NOM = 4, maxitr = 1000;
  double tol = 1e-12;
  int precision = 0;      // 0 complex(8) FP64 arithmetic, 1 complex(4) storage + complex(8) refinement,
                          // 2 complex(8) storage with double-float arithmetic on the FP32 pipe
  int conv_mode = 0;      // 0 reference, 1 residual <= tol, 2 residual <= tol*max(1,|E|)
  uint64_t seed = 1;
  double tol32 = 0.0;     // phase-1 relative residual target (0: default 1e-5)
  int reorth_passes = 1;
  bool real = false;      // real Krylov vectors (real_sector(s) only)
  double time_limit = 0;  // wall seconds; > 0: stop (not converged) at the first restart past it
};

// Thick-restart Lanczos on many chain sectors in lock step (batch_trlan.cu).
// ene, resid: n x NOE; hv: n; status: n (host arrays).
int trlan_lockstep(const std::vector<const Model*>& models, const std::vector<const Sector*>& secs,
                   const TrlanParams& p, double* ene, double* resid, int* hv, int* status, cudaStream_t st);

// Thick-restart Lanczos for the lowest eigenpair on FP32 Krylov vectors
// anchored on one FP64 vector (trlan_anchor.cu).  x: the FP64 start vector
// on entry (n slots, leading dimension ldv for the FP32 basis), the
// normalised Ritz vector on return.
struct AnchorParams {
  int NOK = 16, NOM = 48, maxitr = 1000, conv_mode = 1;
  double tol = 1e-10;
  bool real = false;
  int64_t n = 0, ldv = 0;
  double deadline = 0.0;   // steady-clock seconds; 0: none
  int stall_cycles = 30;   // cycles with neither a lower energy nor a 10 % residual drop before handing over
};
struct AnchorOut {
  double ene = 0.0, resid = 0.0;  // Rayleigh quotient and FP64 residual of x
  int hv32 = 0, hv64 = 0, restarts = 0;
  bool converged = false, stalled = false, timed_out = false;
};
AnchorOut trlan_anchored(const Model& m, const Sector& s, const AnchorParams& p, double2* x, cudaStream_t st);

int trlan(const Model& m, const Sector& s, const TrlanParams& p, const double2* h_start, double* ene_out,
          double2* h_psi, int* iters, double* resid, cudaStream_t st, TrlanStats* stats = nullptr);
int lanczos(const Model& m, const Sector& s, int maxitr, int minitr, int itrint, double tol, const double2* h_start,
            uint64_t seed, double* ene_out, double2* h_psi, int* iters, cudaStream_t st);
void cfrac(int nq, int ldab, const int* nlev, const double* alpha, const double* beta2, const double* norm1,
           const double* E0, double eta, int nomega, const double* omega, int compat, double* S, cudaStream_t st);

// The same continued fraction staged in a static device array instead of
// cudaMalloc'd buffers (see krylov.cu); throws QS3G_ERANGE beyond its size.
void cfrac_noalloc(int nq, int ldab, const int* nlev, const double* alpha, const double* beta2, const double* norm1,
                   const double* E0, double eta, int nomega, const double* omega, int compat, double* S);

// DSF (calcu_Sq_a + calcu_DSF_wavevector) for nq wave vectors.
int dsf(const Model& m, const Sector& gs, const double2* h_psi, double ene1, int spsmsz, int nq, const double* qvec,
        const double* Spos, int itr_dsf, double rfield, double* alpha, double* beta2, double* norm1, double* E0,
        int* nlev, cudaStream_t st);

// The same recursion for all nq wave vectors in lock step on chain sectors
// (batch.cu); d_psi is the ground state on the device.
int dsf_batched(const Model& m, const Sector& gs, const double2* d_psi, double ene1, int spsmsz, int nq,
                const double* qvec, const double* Spos, int itr_dsf, double rfield, double* alpha, double* beta2,
                double* norm1, double* E0, int* nlev, cudaStream_t st);

// calcu_Sq_a alone for one wave vector: D' of the new sector, its list_s and
// fn = S^a(q)|psi> before normalisation (host arrays may be null).
int sq_a(const Model& m, const Sector& gs, const double2* h_psi, int spsmsz, const double* qv, const double* Spos,
         int64_t* Dn_out, int64_t* list_s_new, double2* h_fn, cudaStream_t st);

// <Sz_a Sz_b>, <S+_a S-_b> for all NOS^2 ordered pairs and <Sz_i> of the sector
// vector h_v (get_cf_2_wave_vector / get_lm_2_wave_vector); spsm may be null.
int correlations(const Model& m, const Sector& s, const double2* h_v, double* szsz, double2* spsm, double* lm,
                 cudaStream_t st);

// Sector build for an arbitrary wave vector rk (DSF sectors use rk + q).
void build_sector_rk(const Model& m, int NOD, const double rk[3], Sector& s, cudaStream_t st);

// U(1)-only basis: every configuration of NOD down spins, in colex order.
void build_sector_u1(const Model& m, int NOD, Sector& s, cudaStream_t st);

// ALG = 3: dense H to the host, and all eigenpairs via cuSOLVER zheevd.
void full_hamiltonian(const Model& m, const Sector& s, double2* h_H, cudaStream_t st);
void full_diag(const Model& m, const Sector& s, double* h_ene, double2* h_psi, cudaStream_t st);

// H(i,i) for every row of the sector (called by the sector build).
void compute_diag(const Model& m, Sector& s, cudaStream_t st);

int64_t connection_table_rows(const Model& m, const Sector& s, int64_t row0, int64_t row1, int64_t* row,
                              int64_t* col, int* ell, int* bond, int64_t cap, cudaStream_t st);

}  // namespace qs3g

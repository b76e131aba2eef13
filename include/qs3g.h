/* qs3g.h -- C ABI of libqs3g.so, the GB300 (sm_103a) implementation of the
 * QS3 matrix-free Lanczos hot path.
 *
 * Every entry point is extern "C", takes scalars by pointer so that a Fortran
 * `bind(C)` interface can pass them by reference, and returns an int status
 * (QS3G_OK = 0).  No C++ exception crosses this boundary.  Row and site
 * numbers at the boundary are 1-based as in the Fortran; `qs3g_cplx` has the
 * layout of Fortran complex(8); arrays are column-major where they have two
 * dimensions.  One handle belongs to one host thread and owns one CUDA
 * stream; calls on the same handle are not re-entrant.
 *
 * Reference interfaces each entry point replaces are cited as
 * path:line within the QS-Cube/ED source tree.
 */
#ifndef QS3G_H
#define QS3G_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qs3g_ctx* qs3g_handle;
typedef struct { double re, im; } qs3g_cplx;   /* complex(8) */
typedef struct { float re, im; } qs3g_cplx32;  /* complex(4) */

enum {
  QS3G_OK = 0,
  QS3G_EINVAL = 1,     /* bad argument (the Fortran would `stop`) */
  QS3G_ENOMEM = 2,     /* device allocation failed */
  QS3G_ENOTCONV = 3,   /* solver stopped at its iteration cap without converging */
  QS3G_EITERCAP = 4,   /* a device loop hit its iteration cap */
  QS3G_ECUDA = 5,      /* CUDA runtime error */
  QS3G_ESTATE = 6,     /* call out of order (e.g. no sector built) */
  QS3G_ERANGE = 7,     /* sizes beyond what the kernels index (64-bit ranks, packed sites) */
  QS3G_ENOTSUP = 8,    /* option not implemented for this lattice */
  QS3G_EBREAKDOWN = 9  /* Lanczos breakdown (beta = 0) or non-finite value */
};

/* Location of vector arguments. */
enum { QS3G_HOST = 0, QS3G_DEVICE = 1 };

/* Added to qs3g_trlan's precision (0, 1, 2): real Krylov vectors for sectors
 * whose H is real symmetric (chains at k = 0, U(1) sectors), stored two rows
 * per complex slot, with every scalar of the recurrence real -- half the bytes
 * of each vector pass and one FP64 FMA per hop in H*v.  The start vector is
 * the real part of the given one (or a real random vector); psi is returned
 * with zero imaginary parts.  A real start vector has one component in each
 * eigenspace, so a degenerate eigenvalue is found once (a complex start finds
 * its other copies only through rounding); for more than one eigenpair of a
 * sector with degeneracies use the complex modes. */
enum { QS3G_REAL = 8 };

/* Create a handle for the lattice and bonds.
 * Replaces the module state set up by read_ip (source/input_param.f90:58-117),
 * get_combination (source/state_lists.f90:6-15) and mk_shift_{x,y,z}_SQ
 * (source/state_lists.f90:36-64; called at source/main.f90:49-51).
 * p_xxz is p_xxz(1:2,1:NOxxz); sJint is sJint(1:NOxxz,2:3), i.e. Jxy/2 for
 * every bond followed by Jz/4 for every bond.  Bond ends are swapped to i<j
 * as input_param.f90:97-101 does.  NOS must equal LX*LY*LZ. */
int qs3g_create(qs3g_handle* h, const int* NOS, const int* LX, const int* LY, const int* LZ,
                const int* NOxxz, const int* p_xxz, const double* sJint);

/* Release the handle and all device memory it owns. */
int qs3g_destroy(qs3g_handle h);

/* Build the (NOD, K) representative basis on the GPU.
 * Replaces allocate_lists_omp_SQ + checkstate_SQ (source/state_lists.f90:66-112,
 * 225-292; called at source/main.f90:54) and the explist of
 * source/input_param.f90:87-89.  D_out receives THS(k).
 * Limits (QS3G_ERANGE beyond them): NOS < 65535; NOD * bits(NOS) <= 64 (one
 * packed word per row: NOD <= 6 at NOS = 1000); C(NOS, NOD) below 2^63; D
 * below 2^31; chains (LY = LZ = 1) index the C(NOS-1, NOD-1) configurations
 * with a down spin on site 1, which must stay below 2^32 (L = 1000 allows
 * NOD <= 4), other lattices C(NOS, NOD) <= 2^36; the kernels are instantiated
 * for NOD <= 8 (QS3G_ENOTSUP above). */
int qs3g_build_sector(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ,
                      int64_t* D_out);

/* The same with the reference's default-kind integer THS
 * (source/main.f90:28-34): QS3G_ERANGE if the sector has more than
 * 2^31 - 1 rows or a list_s code above 2^31 - 1 (the reference's own
 * combination table overflows there). */
int qs3g_build_sector_i32(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, int* THS);

/* For a caller that already enumerated the sector with allocate_lists_omp_SQ
 * (source/state_lists.f90:225-292): the (NOD, K) sector is built on the GPU
 * and compared with the caller's list_s(1:D) (bit for bit) and list_r(1:D)
 * (1e-12 relative), so the handle's rows are the caller's rows; a mismatch is
 * QS3G_EINVAL naming the first differing row, and the handle keeps its
 * previous sector.  The _i32 form takes default-kind THS and list_s
 * (source/main.f90:28-34, source/ham2vec_v3.f90:45). */
int qs3g_load_sector(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, const int64_t* D,
                     const int64_t* list_s, const double* list_r);
int qs3g_load_sector_i32(qs3g_handle h, const int* NOD, const int* KX, const int* KY, const int* KZ, const int* THS,
                         const int* list_s, const double* list_r);

/* Build the U(1)-only basis of the variant program: all C(NOS, NOD)
 * configurations, row i = the configuration list_fly(i) of colex rank i, no
 * translation symmetry.  Replaces get_combination + list_fly + inv_list
 * (source_only_u1/state_lists.f90:6-99) with THS = combination(NOS, NOD).
 * qs3g_hv / qs3g_hv32 then act as source_only_u1/ham2vec_v3.f90:35-65, and
 * qs3g_trlan, qs3g_lanczos, qs3g_connection_table, qs3g_correlations
 * (source_only_u1/ham2vec_v3.f90:67-141), qs3g_sq_a and qs3g_dsf
 * (source_only_u1/get_expectation_values.f90:100-391) work on it.
 * qs3g_get_sector returns list_s(i) = i and list_r(i) = 1. */
int qs3g_build_sector_u1(qs3g_handle h, const int* NOD, int64_t* D_out);

/* Copy the sector lists to the host: list_s(1:D) (colex ranks, ascending)
 * and list_r(1:D) = sqrt(norm^2), as allocate_lists_omp_SQ leaves them. */
int qs3g_get_sector(qs3g_handle h, int64_t* list_s, double* list_r);

/* The same into default-kind integer list_s (QS3G_ERANGE if a code or D
 * exceeds 2^31 - 1). */
int qs3g_get_sector_i32(qs3g_handle h, int* list_s, double* list_r);

/* Run the handle's work on a caller-owned CUDA stream (a cudaStream_t passed
 * as void*) instead of the handle's own stream.  No counterpart in the
 * reference, which has no device; the analogue of cublasSetStream. */
int qs3g_set_stream(qs3g_handle h, void* stream);

/* Wait for all work queued on the handle's stream. */
int qs3g_sync(qs3g_handle h);

/* Matrix-free H*v in the current sector: v0 = H v1.
 * Replaces ham_to_vec_wave_vector (source/ham2vec_v3.f90:37-72).
 * where = QS3G_HOST copies v1 in and v0 out and returns when v0 is written;
 * QS3G_DEVICE takes device pointers and queues the product on the handle's
 * stream without waiting (call qs3g_sync before reading v0). */
int qs3g_hv(qs3g_handle h, qs3g_cplx* v0, const qs3g_cplx* v1, const int* where);

/* Same product with complex(4) vectors (FP32 Krylov storage). */
int qs3g_hv32(qs3g_handle h, qs3g_cplx32* v0, const qs3g_cplx32* v1, const int* where);

/* The same product on real vectors (D doubles) for sectors whose H is real
 * symmetric: chains at k = 0 and U(1) sectors (QS3G_ENOTSUP otherwise).
 * Equals the real part of qs3g_hv applied to (v1, 0), bit for bit, at one
 * FP64 FMA per hop instead of two.  No counterpart in the reference, whose
 * vectors are complex(8) for every sector. */
int qs3g_hv_real(qs3g_handle h, double* v0, const double* v1, const int* where);

/* The real product in FP32 (D floats): v0 = (H - shift) v1 with the shift
 * subtracted from the diagonal in FP64 before it is rounded (shift may be
 * NULL: 0), for sectors whose H is real symmetric (QS3G_ENOTSUP otherwise).
 * The Krylov vectors of qs3g_trlan precision 1 + QS3G_REAL go through this
 * product.  No counterpart in the reference, whose vectors are complex(8). */
int qs3g_hv32_real(qs3g_handle h, float* v0, const float* v1, const float* shift, const int* where);

/* Schedule of the H*v kernel for the current general-lattice sector (chains
 * and U(1) sectors use one thread per row always): 0 = autotune (the first
 * product of each precision times a warp per row, lanes over the
 * translations, against a thread per row scanning them, and keeps the
 * faster), 1 = warp per row, 2 = thread per row.  Both give identical
 * results.  mode may be NULL (query only); chosen (may be NULL) receives the
 * complex(8) and complex(4) schedules (0 until the first product).  No
 * counterpart in the reference. */
int qs3g_hv_schedule(qs3g_handle h, const int* mode, int* chosen);

/* Cache the current chain sector's connection table in device memory (on =
 * 1) or drop it (on = 0).  The table holds, per row and hop, the target row
 * and its coefficient (4 bytes per hop for k = 0 chains with one coupling per
 * bond distance, 8 otherwise: NOD * (bonds per site) hops per row, e.g.
 * 2.65 GB for L = 1000, N_down = 4 with NN + NNN bonds); while it is cached,
 * every H*v of the sector (qs3g_hv, qs3g_hv_real, qs3g_hv32_real, qs3g_trlan,
 * qs3g_trlan_lockstep) reads it instead of searching representatives per
 * hop.  complex(8) and real FP64 products are bit-identical with and
 * without it; complex(4) and real FP32 ones may differ in rounding (the
 * matrix-free FP32 form sums the hops in another order).  bytes (may be NULL)
 * receives the table's size, 0 when none is cached.  QS3G_ENOTSUP for
 * U(1) sectors and general lattices, QS3G_ENOMEM when it does not fit with
 * 1 GiB to spare.  A new qs3g_build_sector drops it.  No counterpart in the
 * reference (ham_to_vec_wave_vector, source/ham2vec_v3.f90:37-72, searches
 * every hop at every product). */
int qs3g_hv_cache(qs3g_handle h, const int* on, int64_t* bytes);

/* The complex(8) product v0 = H v1 from the cached connection table in
 * double-float arithmetic on the FP32 pipe (the arithmetic of qs3g_trlan's
 * double-float modes): FP64 inputs split into float pairs with integer
 * instructions, products and sums as unevaluated float pairs, about 2^-46
 * relative instead of FP64's rounding.  GB300 executes FP64 at 1/64 of the
 * FP32 rate and the FP64 product needs two FP64 FMAs per hop, so this form is
 * bounded by HBM instead.  Not the reference's arithmetic: qs3g_hv is.
 * QS3G_ESTATE without a cached table; where as for qs3g_hv. */
int qs3g_hv_df(qs3g_handle h, qs3g_cplx* v0, const qs3g_cplx* v1, const int* where);

/* The connection table of ham_to_vec_wave_vector: one entry per antiparallel
 * bond whose hop lands on a row of the sector (the `id > 0` branch of
 * source/ham2vec_v3.f90:61-65): 1-based row and column, the translation
 * ell(1:3) of representative_SQ (source/state_lists.f90:384-416), and the
 * 1-based bond number.  Rows ascend; within a row, bonds ascend.
 * On entry *nnz is the capacity of the arrays; on return it is the number of
 * entries (QS3G_ERANGE if the capacity was too small; pass row == NULL to
 * query the count). */
int qs3g_connection_table(qs3g_handle h, int64_t* row, int64_t* col, int* ell, int* bond,
                          int64_t* nnz);

/* The same table restricted to rows row_first..row_last (1-based, inclusive),
 * for sectors too large to tabulate at once. */
int qs3g_connection_table_rows(qs3g_handle h, const int64_t* row_first, const int64_t* row_last,
                               int64_t* row, int64_t* col, int* ell, int* bond, int64_t* nnz);

/* Thick-restart Lanczos for the lowest NOE eigenpairs.
 * Replaces my_trlanczos_routines_complex + lancz_eigen_val_complex
 * (source/eigen_solver.f90:10-49,69-261; called at source/main.f90:92).
 * precision: 0 = complex(8) Krylov vectors and FP64 arithmetic throughout (the
 *            reference's arithmetic);
 *            1 = complex(4) storage with FP64-accurate reductions,
 *            reorthogonalisation and Ritz solve, followed by a complex(8)
 *            refinement phase run as in precision 2;
 *            2 = complex(8) storage; dots, reorthogonalisation and restarts in
 *            double-float arithmetic on the FP32 pipe (about 2^-47 relative
 *            per operation; GB300 issues FP64 at 1/64 of the FP32 rate).
 *            + QS3G_REAL: real vectors (k = 0 chains, U(1) sectors; else
 *            QS3G_ENOTSUP).
 * conv_mode: 0 = the reference's test (|E_prev/E - 1| < tol on two consecutive
 *            restarts, eigen_solver.f90:150-159);
 *            1 = Ritz residual |beta_NOM C(NOM,j)| <= tol for j = 1..NOE.
 * start_mode: 0 = random start from `seed`; 1 = start vector given in `start`
 *            (host, D elements).
 * ene(1:NOE) receives the eigenvalues; psi (host, D x NOE column-major, may be
 * NULL) the Ritz vectors; iters receives the number of H*v products; resid
 * (may be NULL) receives ||H psi_j - E_j psi_j||_2 recomputed in FP64. */
int qs3g_trlan(qs3g_handle h, const int* NOE, const int* NOK, const int* NOM, const int* maxitr,
               const double* tol, const int* precision, const int* conv_mode,
               const int* start_mode, const uint64_t* seed, const qs3g_cplx* start, double* ene,
               qs3g_cplx* psi, int* iters, double* resid);

/* Wall-clock limit of qs3g_trlan on this handle (seconds; 0 = none, the
 * default): a solve still running at the limit stops at its next thick
 * restart and returns QS3G_ENOTCONV with the Ritz pairs it has (a batch job's
 * time budget; the reference's only limit is maxitr).  No counterpart in the
 * reference. */
int qs3g_set_time_limit(qs3g_handle h, const double* seconds);

/* What the last qs3g_trlan call on this handle did: H*v products on
 * complex(4) and on complex(8) Krylov vectors (the FP64 residual checks
 * counted with the latter), thick restarts, wall seconds, and 1 in timed_out
 * if it stopped at the time limit.  Any pointer may be NULL.  The reference
 * prints its restart count per restart (source/eigen_solver.f90:157-158). */
int qs3g_trlan_stats(qs3g_handle h, int* hv_fp32, int* hv_fp64, int* restarts, double* seconds,
                     int* timed_out);

/* Thick-restart Lanczos on n independent problems at once: hs[0..n-1] are
 * handles with built sectors (any lattices, sizes and couplings); each is
 * solved as qs3g_trlan does with a random start, on its own stream, by a pool
 * of nthreads host workers (NULL or <= 0: 8) taking the largest sectors
 * first, so the GPU runs the problems' kernels concurrently.  ene (n x NOE),
 * iters (n, may be NULL), resid (n x NOE, may be NULL) and status (n, the
 * per-problem return code) are host arrays; the call returns the first
 * non-OK status.  No counterpart in the reference, which solves one sector
 * per run (source/main.f90). */
int qs3g_trlan_batch(const int* n, qs3g_handle* hs, const int* NOE, const int* NOK, const int* NOM,
                     const int* maxitr, const double* tol, const int* precision, const int* conv_mode,
                     const uint64_t* seed, const int* nthreads, double* ene, int* iters, double* resid,
                     int* status);

/* The same n problems solved in lock step: every Krylov column is one
 * concatenated vector over all problems (chain sectors only), so each
 * Lanczos step is one launch sequence for all problems, with per-problem
 * scalars and Ritz solves; converged problems drop out at the next restart.
 * precision 1 (complex(4) phase + complex(8) refinement, the default) or 2;
 * conv_mode 1 (default) or 2 verifies every Ritz pair's FP64 residual.  Runs
 * on the first handle's stream after waiting for every handle's stream.
 * Arguments and results as qs3g_trlan_batch (no thread count).  No
 * counterpart in the reference. */
int qs3g_trlan_lockstep(const int* n, qs3g_handle* hs, const int* NOE, const int* NOK, const int* NOM,
                        const int* maxitr, const double* tol, const int* precision, const int* conv_mode,
                        const uint64_t* seed, double* ene, int* iters, double* resid, int* status);

/* Plain Lanczos (ALG=1) for the lowest eigenpair.
 * Replaces lanczos_routines + lancz_eigen_val (source/lanczos.f90:14-152). */
int qs3g_lanczos(qs3g_handle h, const int* maxitr, const int* minitr, const int* itrint,
                 const double* tol, const int* start_mode, const uint64_t* seed,
                 const qs3g_cplx* start, double* ene, qs3g_cplx* psi, int* iters);

/* Dynamical structure factor recursion for nq momentum transfers at once.
 * Replaces calcu_Sq_a + calcu_DSF_wavevector
 * (source/get_expectation_values.f90:281-605; called at source/main.f90:178).
 * psi: ground state in the current sector (host, D elements); ene1: its energy
 * (ene(1)); spsmsz: 1 = S+, 2 = S-, 3 = Sz; qvec: nq x 3 wave vectors
 * (kvec_calc per q); Spos: site positions Spos(1:3,1:NOS); itr_dsf: number of
 * recursion levels; rfield: Zeeman field.
 * Outputs per q (column-major itr_dsf x nq): alpha(1:itr_dsf) and
 * beta2(1:itr_dsf) exactly as written to alpha_beta_values_*.d (beta2(1) = 0),
 * norm1(1:nq), E0(1:nq) = ene1 - rfield*sztot, nlev(1:nq) = levels computed. */
int qs3g_dsf(qs3g_handle h, const qs3g_cplx* psi, const double* ene1, const int* spsmsz,
             const int* nq, const double* qvec, const double* Spos, const int* itr_dsf,
             const double* rfield, double* alpha, double* beta2, double* norm1, double* E0,
             int* nlev);

/* The start vector alone for one wave vector qvec(1:3): builds the
 * (N_down', k+q) sector and returns its dimension D_new, its list_s (may be
 * NULL) and fn = S^a(q)|psi> before normalisation (may be NULL), as calcu_Sq_a
 * (source/get_expectation_values.f90:281-377) leaves them.  Call with NULL
 * arrays first to learn D_new. */
int qs3g_sq_a(qs3g_handle h, const qs3g_cplx* psi, const int* spsmsz, const double* qvec,
              const double* Spos, int64_t* D_new, int64_t* list_s_new, qs3g_cplx* fn);

/* Static correlations of a sector vector psi (host, D elements, normalised):
 * szsz(1:NOS**2) = <Sz_a Sz_b> and spsm(1:NOS**2) = <S+_a S-_b> at index
 * a + (b-1)*NOS for the pair (list_expe_ss(1), list_expe_ss(2)) = (a, b), and
 * lm(1:NOS) = <Sz_i> (may be NULL).  Replaces get_cf_2_wave_vector +
 * calcu_cf_trans_2 (source/get_expectation_values.f90:234-279,
 * source/ham2vec_v3.f90:111-174) for the full pair list (NOCF = NOS**2) and
 * get_lm_2_wave_vector + calcu_lm_trans_2 (source/get_expectation_values.f90:
 * 197-232, source/ham2vec_v3.f90:74-109). */
int qs3g_correlations(qs3g_handle h, const qs3g_cplx* psi, double* szsz, qs3g_cplx* spsm,
                      double* lm);

/* Continued fraction S(omega) = -Im G / pi of DSFLan
 * (source_DSFLan/main.f90:52-84) for nq spectra at once on an arbitrary omega
 * grid.  alpha/beta2 are column-major (ldab x nq) with nlev(q) levels used;
 * compat = 1 keeps the reference's deepest level (imaginary part not divided
 * by its denominator), compat = 0 evaluates the plain continued fraction.
 * S is column-major (nomega x nq).  Host arrays. */
int qs3g_cfrac(const int* nq, const int* ldab, const int* nlev, const double* alpha,
               const double* beta2, const double* norm1, const double* E0, const double* eta,
               const int* nomega, const double* omega, const int* compat, double* S);

/* The continued fraction of qs3g_cfrac, with the same arguments and results,
 * for callers that cannot call cudaMalloc -- a host code whose own allocator
 * already owns the GPU's memory, or a solver loop that must not trigger the
 * device-wide synchronisation cudaMalloc and cudaFree can cause.  It allocates
 * nothing: inputs and S are staged in one static device array of 4 MiB
 * (524288 doubles) that every GPU loading the library holds until exit, and
 * sizes that do not fit are rejected with QS3G_ERANGE.  The first call on a
 * device looks up that array's device address (make it before any stream
 * capture); calls that overlap on the GPU share the array and race.  Runs on
 * the legacy default stream and returns when S is written.  Has no
 * counterpart in the reference, whose DSFLan runs on the CPU. */
int qs3g_cfrac_noalloc(const int* nq, const int* ldab, const int* nlev, const double* alpha,
                       const double* beta2, const double* norm1, const double* E0, const double* eta,
                       const int* nomega, const double* omega, const int* compat, double* S);

/* ALG = 3, first half: the dense sector Hamiltonian Ham(i, id), D x D
 * column-major complex(8) (host), built on the GPU with the bonds visited in
 * list order as make_full_hamiltonian does (source/ham2vec_v3.f90:5-35;
 * source_only_u1/ham2vec_v3.f90:5-33 for a U(1)-only sector).  D <= 46340. */
int qs3g_full_hamiltonian(qs3g_handle h, qs3g_cplx* ham);

/* ALG = 3: all eigenpairs of the current sector.  Replaces Full_diag_routines +
 * fulldia_routines_with_momentum (source/eigen_solver.f90:51-67, 261-337):
 * the dense H is built on the GPU and diagonalised with cuSOLVER zheevd on its
 * upper triangle (the reference's zheev('V','U')).  ene(1:D) ascending;
 * psi(1:D,1:D) (host, may be NULL) the eigenvectors as columns, unique only up
 * to a phase (and within degenerate levels).  cuSOLVER is loaded at run time;
 * QS3G_ENOTSUP if it is absent. */
int qs3g_full_diag(qs3g_handle h, double* ene, qs3g_cplx* psi);

/* ---- result files in the reference's formats (host only, no GPU needed) ----
 * Byte-compatible with what the Fortran writes, so that a re_wf = 1 restart
 * and the external DSFLan program read files written here and vice versa.
 * Errors are reported through qs3g_last_error(NULL). */

/* wf<i>.bin: psi(1:dim) as one Fortran unformatted sequential record of
 * complex(8) (4-byte record markers; records over 2147483639 bytes split into
 * subrecords as gfortran does).  Replaces write_wf / read_wf
 * (source/input_param.f90:119-184); read takes the first dim values of the
 * record and fails with QS3G_ERANGE if the record is shorter. */
int qs3g_write_wf(const char* path, const int64_t* dim, const qs3g_cplx* psi);
int qs3g_read_wf(const char* path, const int64_t* dim, qs3g_cplx* psi);

/* energy.dat: NOE lines in format (2ES24.15): dble(i), ene(i)
 * (source/input_param.f90:137-142, 170-176). */
int qs3g_write_energy(const char* path, const int* NOE, const double* ene);
int qs3g_read_energy(const char* path, const int* NOE, double* ene);

/* alpha_beta_values_*.d: nlines lines in format (3I6, 8e23.15):
 * ex_i, n, itr, alpha(n), beta2(n), norm1, E0, sztot
 * (source/get_expectation_values.f90:522-525, 570-573, 595-603).  append != 0
 * appends as the reference's position='append' does.  Level 1 of the
 * reference's -tmp.d file is written with an I15 descriptor for the real
 * sztot (rejected at run time by gfortran); here it has the E23.15 field of
 * every other line.  The reader is the list-directed read of DSFLan
 * (source_DSFLan/main.f90:43-48): up to cap levels of alpha and beta2, norm1,
 * E0 and sztot of the last line, nlines = lines read (QS3G_ERANGE if more
 * than cap). */
int qs3g_write_alpha_beta(const char* path, const int* nlines, const int* ex_i, const int* itr,
                          const double* alpha, const double* beta2, const double* norm1, const double* E0,
                          const double* sztot, const int* append);
int qs3g_read_alpha_beta(const char* path, const int* cap, double* alpha, double* beta2, double* norm1,
                         double* E0, double* sztot, int* nlines);

/* One value in a Fortran edit descriptor: kind 0 = Ew.d, 1 = ESw.d
 * (1 <= w <= 64).  out receives w characters and a NUL. */
int qs3g_format_real(const double* x, const int* kind, const int* w, const int* d, char* out);

/* ---- learned start vector (no counterpart in the reference) ----
 * The reference starts thick-restart Lanczos from a random vector
 * (source/eigen_solver.f90:92-96).  This network maps the gaps between
 * consecutive down spins of a chain representative (NOD <= 4) to its k = 0
 * ground-state amplitude; its prediction is passed to qs3g_trlan with
 * start_mode = 1.  Layers 16 -> 128 -> 128 -> 128 -> 1 with tanh; parameters
 * kept in FP32 and used rounded to BF16, products accumulated in FP32; trained
 * on the GPU by the library's own forward and backward kernels on ground
 * states that qs3g_trlan produced.  cond = {Delta, J2, q0}: the anisotropy
 * Jz/Jxy, the next-nearest coupling and the wave number of the magnon band
 * minimum (pi for J2 <= 1/4, acos(-1/(4 J2)) above), which enter the inputs
 * as Delta, J2 and cos/sin(q0 * gap).  Parameters are QS3G_MLP_NPARAMS
 * doubles in the order W1[16][128] b1 W2[128][128] b2 W3[128][128] b3
 * w4[128] b4. */
typedef struct qs3g_mlp_ctx* qs3g_mlp;
#define QS3G_MLP_NPARAMS 35329

/* New network with seeded uniform (Glorot) weights and zero biases. */
int qs3g_mlp_create(qs3g_mlp* net, const uint64_t* seed);
int qs3g_mlp_destroy(qs3g_mlp net);

/* Copy the parameters out (get != NULL) and/or in (set != NULL; resets Adam). */
int qs3g_mlp_params(qs3g_mlp net, double* get, const double* set);

/* Add the k = 0 ground state psi (host, D elements) of the handle's current
 * chain sector to the training set, with its cond.  Targets are
 * psi_r * list_r(r) / L * sqrt(C(L, NOD)) after a global phase fix. */
int qs3g_mlp_add_sample(qs3g_mlp net, qs3g_handle h, const qs3g_cplx* psi, const double* cond);
int qs3g_mlp_clear(qs3g_mlp net);

/* Mean squared error over the whole training set and its gradient
 * (QS3G_MLP_NPARAMS doubles, may be NULL) at the current parameters. */
int qs3g_mlp_loss_grad(qs3g_mlp net, double* loss, double* grad);

/* steps Adam steps on batches of `batch` representatives drawn with
 * replacement from the seed; losses (may be NULL) receives each batch loss. */
int qs3g_mlp_train(qs3g_mlp net, const int* steps, const int64_t* batch, const double* lr, const uint64_t* seed,
                   double* losses);

/* Flip the sign of every training sample whose targets point against the
 * current network output (the ground state's global sign is arbitrary). */
int qs3g_mlp_align(qs3g_mlp net, int* nflipped);

/* Start vector for the handle's current chain sector (k = 0):
 * v_r = f(r) * L / list_r(r), unnormalised, host or device (where). */
int qs3g_mlp_predict(qs3g_mlp net, qs3g_handle h, const double* cond, qs3g_cplx* start, const int* where);

/* Last error message for the handle (or the last global one if h is NULL). */
const char* qs3g_last_error(qs3g_handle h);

/* Number of kernels this library has launched since load (for accounting). */
int64_t qs3g_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* QS3G_H */

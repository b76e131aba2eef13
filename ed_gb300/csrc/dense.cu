// dense.cu -- ALG = 3: the dense sector Hamiltonian and its full
// eigen-decomposition.
//
// Replaces Full_diag_routines + make_full_hamiltonian +
// fulldia_routines_with_momentum (eigen_solver.f90:51-67, 261-337;
// ham2vec_v3.f90:5-35).  H is built on the GPU by k_dense (one thread per
// row, bonds in list order) into a D x D column-major complex(8) array;
// cusolverDnZheevd with the upper triangle then plays the part of
// zheev('V', 'U'): eigenvalues ascending, eigenvectors in the columns.
// Eigenvectors of degenerate levels, and the phase of every eigenvector,
// are not unique and may differ from LAPACK's.
//
// cuSOLVER is resolved at run time with dlopen, so the library loads (and
// every other entry point works) on a system without it; there this path
// returns QS3G_ENOTSUP.
#include <dlfcn.h>

#include <cusolverDn.h>  // types and enums only: the entry points come from dlsym

#include <mutex>

#include "krylov.h"
#include "qs3g_internal.cuh"

namespace qs3g {
namespace {

struct Cusolver {
  bool tried = false;
  void* lib = nullptr;
  cusolverStatus_t (*create)(cusolverDnHandle_t*) = nullptr;
  cusolverStatus_t (*destroy)(cusolverDnHandle_t) = nullptr;
  cusolverStatus_t (*set_stream)(cusolverDnHandle_t, cudaStream_t) = nullptr;
  cusolverStatus_t (*zheevd_buffer)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int,
                                    const cuDoubleComplex*, int, const double*, int*) = nullptr;
  cusolverStatus_t (*zheevd)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int, cuDoubleComplex*, int,
                             double*, cuDoubleComplex*, int, int*) = nullptr;
};

std::mutex g_cs_mu;
Cusolver g_cs;

const Cusolver& cusolver() {
  std::lock_guard<std::mutex> lk(g_cs_mu);
  if (g_cs.tried) return g_cs;
  g_cs.tried = true;
  const char* names[] = {"libcusolver.so", "libcusolver.so.12", "libcusolver.so.11",
                         "/usr/local/cuda/lib64/libcusolver.so"};
  for (const char* nm : names) {
    g_cs.lib = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
    if (g_cs.lib) break;
  }
  if (!g_cs.lib) return g_cs;
  auto sym = [&](auto& fp, const char* name) { fp = reinterpret_cast<std::decay_t<decltype(fp)>>(dlsym(g_cs.lib, name)); };
  sym(g_cs.create, "cusolverDnCreate");
  sym(g_cs.destroy, "cusolverDnDestroy");
  sym(g_cs.set_stream, "cusolverDnSetStream");
  sym(g_cs.zheevd_buffer, "cusolverDnZheevd_bufferSize");
  sym(g_cs.zheevd, "cusolverDnZheevd");
  if (!g_cs.create || !g_cs.destroy || !g_cs.set_stream || !g_cs.zheevd_buffer || !g_cs.zheevd) {
    dlclose(g_cs.lib);
    g_cs = Cusolver{};
    g_cs.tried = true;
  }
  return g_cs;
}

#define QS3G_CHECK_CUSOLVER(call)                                                              \
  do {                                                                                         \
    const cusolverStatus_t _s = (call);                                                        \
    if (_s != CUSOLVER_STATUS_SUCCESS)                                                         \
      throw ::qs3g::Error(QS3G_ECUDA, std::string(#call) + ": cuSOLVER status " + std::to_string((int)_s)); \
  } while (0)

struct SolverHandle {
  const Cusolver& cs;
  cusolverDnHandle_t h = nullptr;
  explicit SolverHandle(const Cusolver& c) : cs(c) { QS3G_CHECK_CUSOLVER(cs.create(&h)); }
  ~SolverHandle() {
    if (h) cs.destroy(h);
  }
};

}  // namespace

// Dense H to the host (make_full_hamiltonian): Ham(i, id), column-major.
void full_hamiltonian(const Model& m, const Sector& s, double2* h_H, cudaStream_t st) {
  const int64_t D = s.D;
  QS3G_REQUIRE(D > 0, QS3G_ESTATE, "empty sector");
  QS3G_REQUIRE(D <= 46340, QS3G_ERANGE, "dense H needs D <= 46340");
  DevBuf<double2> dH((size_t)D * (size_t)D);
  dense_hamiltonian(m, s, dH.get(), D, st);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(h_H, dH.get(), (size_t)D * D * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
}

// All eigenpairs of the sector (Full_diag_routines): ene(1:D) ascending,
// psi(1:D, 1:D) the eigenvectors as columns (skipped when psi is null).
void full_diag(const Model& m, const Sector& s, double* h_ene, double2* h_psi, cudaStream_t st) {
  const int64_t D = s.D;
  QS3G_REQUIRE(D > 0, QS3G_ESTATE, "empty sector");
  QS3G_REQUIRE(D <= 46340, QS3G_ERANGE, "full diagonalisation needs D <= 46340");
  const Cusolver& cs = cusolver();
  QS3G_REQUIRE(cs.lib, QS3G_ENOTSUP, "libcusolver could not be loaded");
  const int n = (int)D;
  DevBuf<double2> dA((size_t)D * (size_t)D);
  DevBuf<double> dW(D);
  DevBuf<int> dInfo(1);
  dense_hamiltonian(m, s, dA.get(), D, st);
  SolverHandle sh(cs);
  QS3G_CHECK_CUSOLVER(cs.set_stream(sh.h, st));
  const cusolverEigMode_t mode = h_psi ? CUSOLVER_EIG_MODE_VECTOR : CUSOLVER_EIG_MODE_NOVECTOR;
  int lwork = 0;
  QS3G_CHECK_CUSOLVER(cs.zheevd_buffer(sh.h, mode, CUBLAS_FILL_MODE_UPPER, n,
                                       reinterpret_cast<const cuDoubleComplex*>(dA.get()), n, dW.get(), &lwork));
  DevBuf<double2> dWork(std::max(1, lwork));
  QS3G_CHECK_CUSOLVER(cs.zheevd(sh.h, mode, CUBLAS_FILL_MODE_UPPER, n, reinterpret_cast<cuDoubleComplex*>(dA.get()),
                                n, dW.get(), reinterpret_cast<cuDoubleComplex*>(dWork.get()), lwork, dInfo.get()));
  int info = 0;
  QS3G_CHECK_CUDA(cudaMemcpyAsync(&info, dInfo.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(h_ene, dW.get(), D * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (h_psi)
    QS3G_CHECK_CUDA(cudaMemcpyAsync(h_psi, dA.get(), (size_t)D * D * sizeof(double2), cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  QS3G_REQUIRE(info == 0, QS3G_ENOTCONV, "zheevd failed, info = " + std::to_string(info));
}

}  // namespace qs3g

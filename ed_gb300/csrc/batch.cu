// batch.cu -- the DSF recursion for every q of a sweep at once.
//
// calcu_DSF_wavevector (get_expectation_values.f90:379-605) runs one
// continued-fraction Lanczos recursion per wave vector q, each in its own
// (NOD', k+q) sector.  Here the nq recursions run in lock step on one set of
// concatenated vectors: sector q owns rows [row0_q, row0_q + D_q).  Every
// step is one batched H*v launch (k_hv_chain64_seg) plus segmented level-1
// kernels whose blocks each serve 256 rows of a single sector, so the
// per-sector scalars (alpha_q, beta_q) are read per block.  Reductions are
// per block, then one block per sector sums its partials in a fixed order,
// so results are deterministic and do not depend on nq.  The whole
// recursion (itr_dsf steps, about six launches each) is captured into one
// CUDA graph and launched once; where capture is not possible (the legacy
// default stream) the same launches run directly.
//
// Steps per sector, as the reference writes them:
//   f1 = f0 / |f0| (norm1 = |f0|^2)
//   f2' = H f1 - h Sz' f1;  alpha_1 = Re <f1|f2'>;  f2' -= alpha_1 f1
//   beta2_2 = |f2'|^2;  f2 = f2' / sqrt(beta2_2)
//   n >= 2: f' = H f_n - h Sz' f_n;  alpha_n = Re <f_n|f'>;
//           f' -= alpha_n f_n + sqrt(beta2_n) f_{n-1};  beta2_{n+1} = |f'|^2;  f_{n+1} = f'/sqrt(beta2_{n+1})
// A sector whose recursion ends early (n = D_q) keeps computing garbage in
// its own rows; those levels are not reported.
#include <cmath>
#include <memory>
#include <vector>

#include "krylov.h"
#include "qs3g_internal.cuh"

namespace qs3g {

// implemented in dsf.cu
void start_vector(const Model& m, const Sector& gs, const double2* d_psi, int spsmsz, const double* qv,
                  const double* Spos, Sector& ns, DevBuf<double2>& fn, cudaStream_t st);

namespace {

constexpr int kRows = 256;  // rows per block of every batched kernel (= H*v block)

__device__ __forceinline__ double2 block_sum(double2 v, double2* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = kRows / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sh[threadIdx.x].x += sh[threadIdx.x + s].x;
      sh[threadIdx.x].y += sh[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  return sh[0];
}

struct SegRows {
  int64_t row0, D;
};

__device__ __forceinline__ bool seg_row(const SegRows* segs, const int* blk_seg, const int* blk_first, int64_t& r,
                                        int& sg) {
  sg = blk_seg[blockIdx.x];
  const int64_t i = (int64_t)(blockIdx.x - blk_first[blockIdx.x]) * kRows + threadIdx.x;
  r = segs[sg].row0 + i;
  return i < segs[sg].D;
}

// part[b] = sum over the block's rows of conj(x) y
__global__ void __launch_bounds__(kRows) k_sdot(const SegRows* segs, const int* blk_seg, const int* blk_first,
                                                const double2* __restrict__ x, const double2* __restrict__ y,
                                                double2* part) {
  __shared__ double2 sh[kRows];
  int64_t r;
  int sg;
  double2 v = make_double2(0.0, 0.0);
  if (seg_row(segs, blk_seg, blk_first, r, sg)) {
    const double2 a = x[r], b = y[r];
    v = make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
  }
  const double2 s = block_sum(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// part[b] = sum |x|^2
__global__ void __launch_bounds__(kRows) k_snrm(const SegRows* segs, const int* blk_seg, const int* blk_first,
                                                const double2* __restrict__ x, double2* part) {
  __shared__ double2 sh[kRows];
  int64_t r;
  int sg;
  double v = 0.0;
  if (seg_row(segs, blk_seg, blk_first, r, sg)) {
    const double2 a = x[r];
    v = a.x * a.x + a.y * a.y;
  }
  const double2 s = block_sum(make_double2(v, 0.0), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// y -= alpha_s x + sqrt(beta2_s) z  (z may be null), then part[b] = sum |y|^2.
// alpha_s = alpha[s * ld], bb_s = bb[s * ld] = (sqrt(beta2), beta2).
__global__ void __launch_bounds__(kRows) k_supdate(const SegRows* segs, const int* blk_seg, const int* blk_first,
                                                   double2* y, const double2* __restrict__ x,
                                                   const double2* __restrict__ z, const double* alpha,
                                                   const double2* bb, int64_t ld, double2* part) {
  __shared__ double2 sh[kRows];
  int64_t r;
  int sg;
  double v = 0.0;
  if (seg_row(segs, blk_seg, blk_first, r, sg)) {
    const double a = alpha[sg * ld];
    double2 w = y[r];
    const double2 xv = x[r];
    w.x -= a * xv.x;
    w.y -= a * xv.y;
    if (z) {
      const double b = bb[sg * ld].x;
      const double2 zv = z[r];
      w.x -= b * zv.x;
      w.y -= b * zv.y;
    }
    y[r] = w;
    v = w.x * w.x + w.y * w.y;
  }
  const double2 s = block_sum(make_double2(v, 0.0), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// x *= 1 / bb_s.x
__global__ void __launch_bounds__(kRows) k_sscale(const SegRows* segs, const int* blk_seg, const int* blk_first,
                                                  double2* x, const double2* bb, int64_t ld) {
  int64_t r;
  int sg;
  if (seg_row(segs, blk_seg, blk_first, r, sg)) {
    const double s = 1.0 / bb[sg * ld].x;
    double2 v = x[r];
    v.x *= s;
    v.y *= s;
    x[r] = v;
  }
}

// One block per sector: fixed-order sum of its blocks' partials.
// mode 0: alpha[s * ld] = Re(sum); mode 1: bb[s * ld] = (sqrt(sum.x), sum.x).
__global__ void __launch_bounds__(kRows) k_sfinal(const double2* part, const int* seg_blk0, const int* seg_nblk,
                                                  int mode, double* alpha, double2* bb, int64_t ld) {
  __shared__ double2 sh[kRows];
  const int sg = blockIdx.x;
  const int b0 = seg_blk0[sg], nb = seg_nblk[sg];
  double2 v = make_double2(0.0, 0.0);
  for (int b = threadIdx.x; b < nb; b += kRows) {
    v.x += part[b0 + b].x;
    v.y += part[b0 + b].y;
  }
  const double2 s = block_sum(v, sh);
  if (threadIdx.x == 0) {
    if (mode == 0) alpha[sg * ld] = s.x;
    else bb[sg * ld] = make_double2(std::sqrt(s.x), s.x);
  }
}

}  // namespace

int dsf_batched(const Model& m, const Sector& gs, const double2* d_psi, double ene1, int spsmsz, int nq,
                const double* qvec, const double* Spos, int itr_dsf, double rfield, double* alpha, double* beta2,
                double* norm1, double* E0, int* nlev, cudaStream_t st) {
  const int NOD = gs.NOD, NOS = m.NOS;
  const int NODn = (spsmsz == 1) ? NOD - 1 : (spsmsz == 2 ? NOD + 1 : NOD);
  const double sztot = (double)NOS / 2.0 - (double)NOD;
  const double sz_new = (double)NOS / 2.0 - (double)NODn;
  // sectors and start vectors, one q at a time
  std::vector<std::unique_ptr<Sector>> secs(nq);
  std::vector<DevBuf<double2>> f0(nq);
  std::vector<int64_t> row0(nq + 1, 0);
  for (int q = 0; q < nq; ++q) {
    secs[q].reset(new Sector());
    start_vector(m, gs, d_psi, spsmsz, qvec + 3 * (size_t)q, Spos, *secs[q], f0[q], st);
    row0[q + 1] = row0[q] + secs[q]->D;
  }
  const int64_t Dtot = row0[nq];
  for (int q = 0; q < nq; ++q) {
    E0[q] = ene1 - rfield * sztot;
    nlev[q] = (int)std::min<int64_t>(itr_dsf, secs[q]->D);
    for (int k = 0; k < itr_dsf; ++k) {
      alpha[(size_t)q * itr_dsf + k] = 1.0e300;
      beta2[(size_t)q * itr_dsf + k] = 0.0;
    }
    norm1[q] = 0.0;
  }
  if (Dtot == 0) return QS3G_OK;
  // block maps: each sector padded to whole 256-row blocks
  std::vector<int> blk_seg, blk_first, seg_blk0(nq), seg_nblk(nq);
  std::vector<HvSeg> hs(nq);
  std::vector<SegRows> sr(nq);
  for (int q = 0; q < nq; ++q) {
    const int nb = (int)((secs[q]->D + kRows - 1) / kRows);
    seg_blk0[q] = (int)blk_seg.size();
    seg_nblk[q] = nb;
    for (int b = 0; b < nb; ++b) {
      blk_seg.push_back(q);
      blk_first.push_back(seg_blk0[q]);
    }
    sr[q] = SegRows{row0[q], secs[q]->D};
    if (secs[q]->D > 0) hs[q] = make_seg(m, *secs[q], row0[q]);
    else hs[q] = HvSeg{};
  }
  const int nblk = (int)blk_seg.size();
  DevBuf<int> d_bs(std::max(1, nblk)), d_bf(std::max(1, nblk)), d_sb0(nq), d_snb(nq);
  DevBuf<HvSeg> d_hs(nq);
  DevBuf<SegRows> d_sr(nq);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_bs.get(), blk_seg.data(), nblk * 4, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_bf.get(), blk_first.data(), nblk * 4, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_sb0.get(), seg_blk0.data(), nq * 4, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_snb.get(), seg_nblk.data(), nq * 4, cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_hs.get(), hs.data(), nq * sizeof(HvSeg), cudaMemcpyHostToDevice, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(d_sr.get(), sr.data(), nq * sizeof(SegRows), cudaMemcpyHostToDevice, st));
  // concatenated vectors
  DevBuf<double2> A(Dtot), B(Dtot), Cv(Dtot), part(nblk);
  for (int q = 0; q < nq; ++q)
    if (secs[q]->D > 0)
      QS3G_CHECK_CUDA(cudaMemcpyAsync(A.get() + row0[q], f0[q].get(), secs[q]->D * sizeof(double2),
                                      cudaMemcpyDeviceToDevice, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  for (auto& f : f0) f.release();
  // per-sector scalars: al[s * ld + n], bbv[s * ld + n] for n = 0..itr_dsf+1
  const int64_t ld = itr_dsf + 2;
  DevBuf<double> al((size_t)nq * ld);
  DevBuf<double2> bbv((size_t)nq * ld);
  QS3G_CHECK_CUDA(cudaMemsetAsync(al.get(), 0, (size_t)nq * ld * 8, st));
  QS3G_CHECK_CUDA(cudaMemsetAsync(bbv.get(), 0, (size_t)nq * ld * 16, st));
  const double shift = rfield * sz_new;
  const SegRows* S = d_sr.get();
  const int *bs = d_bs.get(), *bf = d_bf.get();

  auto record = [&]() {
    double2 *fn = A.get(), *fnp1 = B.get(), *fnm1 = Cv.get();
    // norm1 and f1
    k_snrm<<<nblk, kRows, 0, st>>>(S, bs, bf, fn, part.get());
    check_launch("k_snrm");
    k_sfinal<<<nq, kRows, 0, st>>>(part.get(), d_sb0.get(), d_snb.get(), 1, al.get(), bbv.get() + 0, ld);
    check_launch("k_sfinal");
    k_sscale<<<nblk, kRows, 0, st>>>(S, bs, bf, fn, bbv.get() + 0, ld);
    check_launch("k_sscale");
    // level 1
    hv64_seg(NODn, d_hs.get(), bs, bf, nblk, fn, fnp1, shift, st);
    k_sdot<<<nblk, kRows, 0, st>>>(S, bs, bf, fn, fnp1, part.get());
    check_launch("k_sdot");
    k_sfinal<<<nq, kRows, 0, st>>>(part.get(), d_sb0.get(), d_snb.get(), 0, al.get() + 1, bbv.get(), ld);
    check_launch("k_sfinal");
    k_supdate<<<nblk, kRows, 0, st>>>(S, bs, bf, fnp1, fn, nullptr, al.get() + 1, bbv.get(), ld, part.get());
    check_launch("k_supdate");
    k_sfinal<<<nq, kRows, 0, st>>>(part.get(), d_sb0.get(), d_snb.get(), 1, al.get(), bbv.get() + 2, ld);
    check_launch("k_sfinal");
    k_sscale<<<nblk, kRows, 0, st>>>(S, bs, bf, fnp1, bbv.get() + 2, ld);
    check_launch("k_sscale");
    for (int itr = 2; itr <= itr_dsf; ++itr) {
      double2* t = fnm1;
      fnm1 = fn;
      fn = fnp1;
      fnp1 = t;
      hv64_seg(NODn, d_hs.get(), bs, bf, nblk, fn, fnp1, shift, st);
      k_sdot<<<nblk, kRows, 0, st>>>(S, bs, bf, fn, fnp1, part.get());
      check_launch("k_sdot");
      k_sfinal<<<nq, kRows, 0, st>>>(part.get(), d_sb0.get(), d_snb.get(), 0, al.get() + itr, bbv.get(), ld);
      check_launch("k_sfinal");
      if (itr == itr_dsf) break;  // beta2_{itr+1} is not reported
      k_supdate<<<nblk, kRows, 0, st>>>(S, bs, bf, fnp1, fn, fnm1, al.get() + itr, bbv.get() + itr, ld,
                                        part.get());
      check_launch("k_supdate");
      k_sfinal<<<nq, kRows, 0, st>>>(part.get(), d_sb0.get(), d_snb.get(), 1, al.get(), bbv.get() + itr + 1, ld);
      check_launch("k_sfinal");
      k_sscale<<<nblk, kRows, 0, st>>>(S, bs, bf, fnp1, bbv.get() + itr + 1, ld);
      check_launch("k_sscale");
    }
  };
  bool captured = false;
  if (st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread) {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      record();
      const cudaError_t e = cudaStreamEndCapture(st, &graph);
      if (e == cudaSuccess && graph) {
        cudaGraphExec_t exec = nullptr;
        QS3G_CHECK_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        const cudaError_t le = cudaGraphLaunch(exec, st);
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        QS3G_CHECK_CUDA(le);
        captured = true;
      } else {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
      }
    } else {
      cudaGetLastError();
    }
  }
  if (!captured) record();
  std::vector<double> ha((size_t)nq * ld);
  std::vector<double2> hb((size_t)nq * ld);
  QS3G_CHECK_CUDA(cudaMemcpyAsync(ha.data(), al.get(), ha.size() * 8, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaMemcpyAsync(hb.data(), bbv.get(), hb.size() * 16, cudaMemcpyDeviceToHost, st));
  QS3G_CHECK_CUDA(cudaStreamSynchronize(st));
  QS3G_CHECK_CUDA(cudaGetLastError());
  for (int q = 0; q < nq; ++q) {
    if (secs[q]->D == 0) continue;
    norm1[q] = hb[(size_t)q * ld + 0].y;
    QS3G_REQUIRE(std::isfinite(norm1[q]) && norm1[q] > 0.0, QS3G_EBREAKDOWN, "S^a(q)|GS> vanishes");
    for (int k = 1; k <= nlev[q]; ++k) {
      alpha[(size_t)q * itr_dsf + (k - 1)] = ha[(size_t)q * ld + k];
      beta2[(size_t)q * itr_dsf + (k - 1)] = (k == 1) ? 0.0 : hb[(size_t)q * ld + k].y;
    }
  }
  return QS3G_OK;
}

}  // namespace qs3g

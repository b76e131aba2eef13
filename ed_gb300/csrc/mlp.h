// mlp.h -- the learned start-vector network (see mlp.cu).
#pragma once

#include <cuda_bf16.h>

#include <cstdint>
#include <vector>

#include "qs3g_internal.cuh"

namespace qs3g {

// Parameter layout (FP32 master copy, one contiguous vector):
//   W1[16][128] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] w4[128] b4
// W[i][c] maps input i to output c.
constexpr int kMlpIn = 16, kMlpHid = 128;
constexpr int kMlpOffW1 = 0;
constexpr int kMlpOffB1 = kMlpOffW1 + kMlpIn * kMlpHid;
constexpr int kMlpOffW2 = kMlpOffB1 + kMlpHid;
constexpr int kMlpOffB2 = kMlpOffW2 + kMlpHid * kMlpHid;
constexpr int kMlpOffW3 = kMlpOffB2 + kMlpHid;
constexpr int kMlpOffB3 = kMlpOffW3 + kMlpHid * kMlpHid;
constexpr int kMlpOffW4 = kMlpOffB3 + kMlpHid;
constexpr int kMlpOffB4 = kMlpOffW4 + kMlpHid;
constexpr int kMlpNParams = kMlpOffB4 + 1;

// One training problem (or the problem a start vector is predicted for).
struct MlpSample {
  int L, bits;
  float delta, j2;
  int64_t trig_off;  // offset of its (cos, sin)(q0 h) table, h = 0..L
};

struct Mlp {
  explicit Mlp(uint64_t seed);
  void set_params(const double* p, cudaStream_t st);
  void get_params(double* p, cudaStream_t st) const;
  void add_sample(const Model& m, const Sector& s, const double2* h_psi, const double cond[3], cudaStream_t st);
  void clear_samples();
  double loss_grad(const int64_t* d_index, int64_t B, cudaStream_t st);  // gradient left in d_g
  void gradient(double* g, cudaStream_t st) const;
  void train(int steps, int64_t B, double lr, uint64_t seed, double* losses, cudaStream_t st);
  int align(cudaStream_t st);
  void predict(const Model& m, const Sector& s, const double cond[3], double2* d_v, cudaStream_t st);
  void forward(const uint64_t* d_c, const int* d_s, const MlpSample* d_smp, const float2* d_tr, int64_t n,
               float* d_f, cudaStream_t st) const;
  void upload(cudaStream_t st);

  DevBuf<float> d_w, d_m, d_v, d_g;    // master params, Adam moments, gradient
  DevBuf<__nv_bfloat16> d_wb;          // BF16 params the kernels read
  DevBuf<float> d_gpart;
  DevBuf<double> d_lpart;
  // training set: every representative of every sample, concatenated
  DevBuf<uint64_t> d_conf;
  DevBuf<float> d_target;
  DevBuf<int> d_sid;
  int64_t nreps = 0;
  int nod = 0;
  std::vector<MlpSample> samples;
  std::vector<float2> trig;
  DevBuf<MlpSample> d_samples;
  DevBuf<float2> d_trig;
  bool uploaded = false;
  int64_t adam_t = 0;
};

}  // namespace qs3g

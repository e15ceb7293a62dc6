// Learned vertical-tail closure for q (an extension of the step with no
// reference counterpart).  Per horizontal mode column (compact band) the closure adds
//   C_n = -s * (r_n + i rho_n)(f) * q_n,   n < n_coef (<= 64),
// to the explicit q tendency, where (r, rho) = MLP(f) is a complex
// per-coefficient rate computed from phase-invariant features of the column:
//   f_n      = log1p(|q_n|^2 / sq_n)              n < n_coef (zero-padded to 64)
//   f_64     = |k| / k_max
//   f_65     = log1p(sum_n |k|^2 |psi_n|^2 / se)   (the column's |grad psi|^2)
// The closure multiplies q_n by a complex rate, so it commutes with horizontal
// translations (a phase of the column).  MLP 66 -> 256 -> 128 -> 128 (r_n,
// rho_n) with tanh hidden units, BF16 weights and FP32 accumulation (67 k
// parameters).
//
// Training is a-priori regression on columns of solver-generated data: the
// target is the q tendency a coarse-Nz model misses on a Chebyshev-truncated
// fine-Nz state, loss = mean_c sum_n |C_n - t_n|^2 / tnorm.  The forward and
// backward passes here are hand-written; weight gradients are summed per CTA
// and added to the global FP32 gradient with atomics (order-dependent in the
// last bits; the tests allow for it).
#include <cuda_bf16.h>

#include "engine.h"

namespace nhqg {

namespace {

constexpr int kIn = 66, kH1 = 256, kH2 = 128, kOut = 64, kR = 2 * kOut;
constexpr int kColsPerCta = 16;
constexpr int kThreads = 256;

// parameter offsets (floats / bf16 elements) in one flat buffer
constexpr int oW1 = 0, oB1 = oW1 + kH1 * kIn, oW2 = oB1 + kH1, oB2 = oW2 + kH2 * kH1,
              oW3 = oB2 + kH2, oB3 = oW3 + kR * kH2, kNParams = oB3 + kR;

struct ColIn {
  int M, Mc, ncoef;
  const double2* q;       // [levels][M] Chebyshev coefficients of q
  const double* kx;       // [M]
  const double* ky;       // [M]
  const double* inv_denom;
  const float* sq;        // [64] feature scales
  float se, kmax;
};

// features of column m into x[66]; q_n into qc[64] (FP32)
__device__ __forceinline__ void column_features(const ColIn& c, int m, float* x, float2* qc) {
  const double kx = c.kx[m], ky = c.ky[m];
  const double ksq = kx * kx + ky * ky;
  const double idn = c.inv_denom[m];
  double ke = 0.0;
  for (int n = 0; n < kOut; ++n) {
    float2 v = make_float2(0.f, 0.f);
    float f = 0.f;
    if (n < c.ncoef) {
      const double2 q = c.q[(size_t)n * c.M + m];
      v = make_float2((float)q.x, (float)q.y);
      const double a2 = q.x * q.x + q.y * q.y;
      f = log1pf((float)(a2 / (double)c.sq[n]));
      ke += ksq * idn * idn * a2;
    }
    x[n] = f;
    qc[n] = v;
  }
  x[64] = (float)(sqrt(ksq) / (double)c.kmax);
  x[65] = log1pf((float)(ke / (double)c.se));
}

// one CTA, kColsPerCta columns: forward through the MLP into smem
// activations; fills h1[c][256], h2[c][128], r[c][128] (r_n at n, rho_n at 64 + n)
__device__ __forceinline__ void mlp_forward(const __nv_bfloat16* __restrict__ W, const float (*x)[kIn],
                                            float (*h1)[kH1], float (*h2)[kH2], float (*r)[kR],
                                            int ncols) {
  const int t = threadIdx.x;
  {  // layer 1: thread t = hidden unit t
    const __nv_bfloat16* w = W + oW1 + t * kIn;
    float wr[kIn];
#pragma unroll
    for (int i = 0; i < kIn; ++i) wr[i] = __bfloat162float(w[i]);
    const float b = __bfloat162float(W[oB1 + t]);
    for (int c = 0; c < ncols; ++c) {
      float acc = b;
#pragma unroll
      for (int i = 0; i < kIn; ++i) acc = fmaf(wr[i], x[c][i], acc);
      h1[c][t] = tanhf(acc);
    }
  }
  __syncthreads();
  {  // layer 2: unit j = t % 128, column parity t / 128
    const int j = t % kH2, half = t / kH2;
    const __nv_bfloat16* w = W + oW2 + j * kH1;
    const float b = __bfloat162float(W[oB2 + j]);
    for (int c = half; c < ncols; c += 2) {
      float acc = b;
      for (int i = 0; i < kH1; ++i) acc = fmaf(__bfloat162float(w[i]), h1[c][i], acc);
      h2[c][j] = tanhf(acc);
    }
  }
  __syncthreads();
  {  // layer 3 (linear): unit n = t % 128, column parity t / 128
    const int n = t % kR, half = t / kR;
    const __nv_bfloat16* w = W + oW3 + n * kH2;
    const float b = __bfloat162float(W[oB3 + n]);
    for (int c = half; c < ncols; c += 2) {
      float acc = b;
      for (int i = 0; i < kH2; ++i) acc = fmaf(__bfloat162float(w[i]), h2[c][i], acc);
      r[c][n] = acc;
    }
  }
  __syncthreads();
}

struct SmemFwd {
  float x[kColsPerCta][kIn];
  float2 q[kColsPerCta][kOut];
  float h1[kColsPerCta][kH1];
  float h2[kColsPerCta][kH2];
  float r[kColsPerCta][kR];
};

// Inference in the step: Cq[n][m] = -s r_n q_n for n < ncoef, 0 for the
// other levels (levels = P)
__global__ void __launch_bounds__(kThreads) k_closure_apply(ColIn c, const __nv_bfloat16* __restrict__ W,
                                                            float s, int levels, double2* __restrict__ cq) {
  extern __shared__ __align__(16) unsigned char raw[];
  SmemFwd& sm = *reinterpret_cast<SmemFwd*>(raw);
  const int m0 = blockIdx.x * kColsPerCta;
  const int ncols = min(kColsPerCta, c.M - m0);
  if (threadIdx.x < ncols) column_features(c, m0 + threadIdx.x, sm.x[threadIdx.x], sm.q[threadIdx.x]);
  __syncthreads();
  mlp_forward(W, sm.x, sm.h1, sm.h2, sm.r, ncols);
  for (int i = threadIdx.x; i < levels * kColsPerCta; i += blockDim.x) {
    const int n = i / kColsPerCta, cc = i - n * kColsPerCta;
    if (cc >= ncols) continue;
    double2 v = make_double2(0.0, 0.0);
    if (n < c.ncoef) {
      const float lr = -s * sm.r[cc][n], li = -s * sm.r[cc][kOut + n];
      const float2 q = sm.q[cc][n];
      v = make_double2((double)(lr * q.x - li * q.y), (double)(lr * q.y + li * q.x));
    }
    cq[(size_t)n * c.M + m0 + cc] = v;
  }
}

// Training: forward + loss + backward for a batch of columns given as
// features x [B][66], q [B][64] (FP32 complex) and targets t [B][64].
// Accumulates dL/dtheta into grad (FP32, atomics) and the loss into loss[0].
struct Batch {
  int B;
  const float* x;
  const float2* q;
  const float2* t;
  float s, inv_norm;  // output scale; 1 / (B * tnorm)
};

struct SmemTrain {
  SmemFwd f;
  float g3[kColsPerCta][kR];     // dL/dr, dL/drho
  float d2[kColsPerCta][kH2];    // dL/d(pre-act 2)
  float d1[kColsPerCta][kH1];    // dL/d(pre-act 1)
  float red[kThreads / 32];
};

__global__ void __launch_bounds__(kThreads) k_closure_train(Batch b, const __nv_bfloat16* __restrict__ W,
                                                            float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ __align__(16) unsigned char raw[];
  SmemTrain& sm = *reinterpret_cast<SmemTrain*>(raw);
  const int c0 = blockIdx.x * kColsPerCta;
  const int ncols = min(kColsPerCta, b.B - c0);
  const int t = threadIdx.x;
  for (int i = t; i < ncols * kIn; i += blockDim.x) sm.f.x[i / kIn][i % kIn] = b.x[(size_t)c0 * kIn + i];
  for (int i = t; i < ncols * kOut; i += blockDim.x) sm.f.q[i / kOut][i % kOut] = b.q[(size_t)c0 * kOut + i];
  __syncthreads();
  mlp_forward(W, sm.f.x, sm.f.h1, sm.f.h2, sm.f.r, ncols);
  // output error e = C - t with C_n = -s (r_n + i rho_n) q_n:
  // dL/dr_n = -2 s Re(e conj q_n), dL/drho_n = -2 s Im(e conj q_n) (x inv_norm)
  float lsum = 0.f;
  for (int i = t; i < ncols * kOut; i += blockDim.x) {
    const int c = i / kOut, n = i - c * kOut;
    const float2 q = sm.f.q[c][n], tg = b.t[(size_t)(c0 + c) * kOut + n];
    const float lr = -b.s * sm.f.r[c][n], li = -b.s * sm.f.r[c][kOut + n];
    const float ex = lr * q.x - li * q.y - tg.x, ey = lr * q.y + li * q.x - tg.y;
    lsum += (ex * ex + ey * ey) * b.inv_norm;
    sm.g3[c][n] = -2.f * b.s * (ex * q.x + ey * q.y) * b.inv_norm;
    sm.g3[c][kOut + n] = -2.f * b.s * (ey * q.x - ex * q.y) * b.inv_norm;
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
  if ((t & 31) == 0) sm.red[t >> 5] = lsum;
  __syncthreads();
  if (t == 0) {
    float tot = 0.f;
    for (int w = 0; w < kThreads / 32; ++w) tot += sm.red[w];
    atomicAdd(loss, tot);
  }
  // layer 3 gradients and delta 2
  for (int i = t; i < kR * kH2; i += blockDim.x) {
    const int n = i / kH2, j = i - n * kH2;
    float acc = 0.f;
    for (int c = 0; c < ncols; ++c) acc = fmaf(sm.g3[c][n], sm.f.h2[c][j], acc);
    atomicAdd(grad + oW3 + i, acc);
  }
  if (t < kR) {
    float acc = 0.f;
    for (int c = 0; c < ncols; ++c) acc += sm.g3[c][t];
    atomicAdd(grad + oB3 + t, acc);
  }
  for (int i = t; i < ncols * kH2; i += blockDim.x) {
    const int c = i / kH2, j = i - c * kH2;
    float acc = 0.f;
    for (int n = 0; n < kR; ++n) acc = fmaf(__bfloat162float(W[oW3 + n * kH2 + j]), sm.g3[c][n], acc);
    const float h = sm.f.h2[c][j];
    sm.d2[c][j] = acc * (1.f - h * h);
  }
  __syncthreads();
  // layer 2 gradients and delta 1
  for (int i = t; i < kH2 * kH1; i += blockDim.x) {
    const int j = i / kH1, k = i - j * kH1;
    float acc = 0.f;
    for (int c = 0; c < ncols; ++c) acc = fmaf(sm.d2[c][j], sm.f.h1[c][k], acc);
    atomicAdd(grad + oW2 + i, acc);
  }
  if (t < kH2) {
    float acc = 0.f;
    for (int c = 0; c < ncols; ++c) acc += sm.d2[c][t];
    atomicAdd(grad + oB2 + t, acc);
  }
  for (int i = t; i < ncols * kH1; i += blockDim.x) {
    const int c = i / kH1, k = i - c * kH1;
    float acc = 0.f;
    for (int j = 0; j < kH2; ++j) acc = fmaf(__bfloat162float(W[oW2 + j * kH1 + k]), sm.d2[c][j], acc);
    const float h = sm.f.h1[c][k];
    sm.d1[c][k] = acc * (1.f - h * h);
  }
  __syncthreads();
  // layer 1 gradients
  for (int i = t; i < kH1 * kIn; i += blockDim.x) {
    const int k = i / kIn, f = i - k * kIn;
    float acc = 0.f;
    for (int c = 0; c < ncols; ++c) acc = fmaf(sm.d1[c][k], sm.f.x[c][f], acc);
    atomicAdd(grad + oW1 + i, acc);
  }
  if (t < kH1) {
    float acc = 0.f;
    for (int c = 0; c < ncols; ++c) acc += sm.d1[c][t];
    atomicAdd(grad + oB1 + t, acc);
  }
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; refreshes the BF16
// copy used by the forward/backward kernels
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, __nv_bfloat16* __restrict__ wb, int n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16(wi);
  }
}

// features and FP32 columns of a batch of compact modes (training data)
__global__ void k_closure_features(ColIn c, float* __restrict__ x, float2* __restrict__ qc) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= c.M) return;
  float xf[kIn];
  float2 qq[kOut];
  column_features(c, m, xf, qq);
  for (int i = 0; i < kIn; ++i) x[(size_t)m * kIn + i] = xf[i];
  for (int n = 0; n < kOut; ++n) qc[(size_t)m * kOut + n] = qq[n];
}

}  // namespace

int closure_param_count() { return kNParams; }
size_t closure_apply_smem() { return sizeof(SmemFwd); }

cudaError_t launch_closure_apply(const Params& p, const Tables& t, const ClosureModel& cm,
                                 const double2* q, double2* cq, cudaStream_t st) {
  if (!cm.w) return cudaErrorInvalidValue;
  ColIn c{p.d.M, p.d.Mc, cm.ncoef, q, t.kx, t.ky, t.inv_denom, cm.sq, cm.se, cm.kmax};
  const size_t sm = sizeof(SmemFwd);
  cudaFuncSetAttribute(k_closure_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_closure_apply<<<(p.d.M + kColsPerCta - 1) / kColsPerCta, kThreads, sm, st>>>(
      c, reinterpret_cast<const __nv_bfloat16*>(cm.w), cm.s, p.d.P, cq);
  return cudaGetLastError();
}

cudaError_t launch_closure_features(const Params& p, const Tables& t, const ClosureModel& cm,
                                    const double2* q, float* x, float2* qc, cudaStream_t st) {
  ColIn c{p.d.M, p.d.Mc, cm.ncoef, q, t.kx, t.ky, t.inv_denom, cm.sq, cm.se, cm.kmax};
  k_closure_features<<<(p.d.M + 127) / 128, 128, 0, st>>>(c, x, qc);
  return cudaGetLastError();
}

}  // namespace nhqg

extern "C" {

int nhqg_closure_param_count(void) { return nhqg::kNParams; }

int nhqg_closure_train_step(const void* w_bf16, float* w_master, float* adam_m, float* adam_v,
                            float* grad, float* loss, int batch, const float* x, const float* q,
                            const float* target, float out_scale, float target_norm, float lr, int step,
                            void* stream) {
  using namespace nhqg;
  if (!w_bf16 || !w_master || !adam_m || !adam_v || !grad || !loss || batch <= 0 || !x || !q ||
      !target || step < 1 || !(target_norm > 0.f))
    return NHQG_ERR_BAD_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(grad, 0, kNParams * sizeof(float), st) != cudaSuccess) return NHQG_ERR_CUDA;
  if (cudaMemsetAsync(loss, 0, sizeof(float), st) != cudaSuccess) return NHQG_ERR_CUDA;
  Batch b{batch, x, reinterpret_cast<const float2*>(q), reinterpret_cast<const float2*>(target),
          out_scale, 1.f / ((float)batch * target_norm)};
  const size_t sm = sizeof(SmemTrain);
  cudaFuncSetAttribute(k_closure_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  auto* wb = reinterpret_cast<__nv_bfloat16*>(const_cast<void*>(w_bf16));
  k_closure_train<<<(batch + kColsPerCta - 1) / kColsPerCta, kThreads, sm, st>>>(b, wb, grad, loss);
  if (lr > 0.f) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<(kNParams + 255) / 256, 256, 0, st>>>(w_master, adam_m, adam_v, grad, wb, kNParams, lr,
                                                   b1, b2, 1e-8f, c1, c2);
  }
  return cudaGetLastError() == cudaSuccess ? NHQG_OK : NHQG_ERR_CUDA;
}

}  // extern "C"

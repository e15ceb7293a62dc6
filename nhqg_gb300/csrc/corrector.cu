// Balanced SBP2 thermal corrector and the 1-D mean-temperature kernels.
//
// Reference: _apply_balanced_sbp2_corrector nhqg/solver.py:909-950 with the
// per-substep update :873-906 and the SBP exchange fields :346-358.
//
// Per substep the reference maps theta back to Galerkin coefficients
// (pinv(proj(V^-1 s2c theta_sbp))) and forward again (c2s V S theta_hat).
// S pinv = proj_dir on any coefficient vector, so the round trip is
//   theta_cgl' = y + V[:,N-1] (F0 . y) + V[:,N] (F1 . y),  y = s2c theta_sbp
// with F = (proj_dir - I)[N-1:N+1, :] V^-1 -- a rank-2 correction instead of
// two dense transforms.  Only the last substep returns to coefficients.
// The 1-D system A = I - half (pentadiagonal: D1 diag(<w^2>) D1 and the SBP
// Laplacian) is factored once per corrector without pivoting: it is the
// identity plus a weakly diagonally dominant M-matrix-like term.
#include "column.cuh"
#include "engine.h"

namespace nhqg {

namespace {

using col::TM;
using col::NT;
using col::Prec;
using col::tload;
using col::tstore;
using col::tloadp;
using col::tstorep;
using col::tmat;
using col::tcsr;
using col::tpinv_dir;
using col::tdct;

// offsets inside Work::vec (doubles), each block P long unless noted
struct CV {
  int P;
  __host__ __device__ int w2() const { return 0; }
  __host__ __device__ int flux() const { return P; }
  __host__ __device__ int tb_sbp() const { return 2 * P; }
  __host__ __device__ int g_half() const { return 3 * P; }
  __host__ __device__ int tmp2() const { return 5 * P; }
  __host__ __device__ int Aband() const { return 6 * P; }   // 5P: diag offsets -2..2
  __host__ __device__ int Bband() const { return 11 * P; }  // 5P
  __host__ __device__ int lu32() const { return 16 * P; }   // 3P doubles = 6P floats: FP32 LU band
  __host__ __device__ int total() const { return 19 * P; }
};

struct CK {
  int P, G, N, M;
  bool mixed;
  const double *wa, *wb;
  const double *V, *Vinv;
  col::Dct dct;
  const int *c2s_ptr, *c2s_col, *s2c_ptr, *s2c_col;
  const double *c2s_val, *s2c_val;
  const double *bcF, *bcV, *proj, *D1, *Lsbp;
  const double *c2sV, *tauVinv;  // fused dense 1-D maps (rows applied by many CTAs)
  double mu, kappa;
};

CK make_ck(const Params& p, const Tables& t) {
  CK k;
  k.P = p.d.P; k.G = p.d.G; k.N = p.d.Nz; k.M = p.d.M;
  k.mixed = t.wst_a != nullptr;
  k.wa = t.wst_a; k.wb = t.wst_b;
  k.V = t.V; k.Vinv = t.Vinv;
  k.dct = make_dct(p, t);
  k.c2s_ptr = t.c2s_ptr; k.c2s_col = t.c2s_col; k.c2s_val = t.c2s_val;
  k.s2c_ptr = t.s2c_ptr; k.s2c_col = t.s2c_col; k.s2c_val = t.s2c_val;
  k.bcF = t.bcF; k.bcV = t.bcV; k.proj = t.proj; k.D1 = t.D1; k.Lsbp = t.Lsbp;
  k.c2sV = t.c2sV; k.tauVinv = t.tauVinv;
  k.mu = p.eps_sq;
  k.kappa = 1.0 / p.sigma;
  return k;
}

// Galerkin -> Chebyshev stencil of w (wbasis) or theta on tiles of type C
template <typename C>
__device__ __forceinline__ void tstencil(const CK& k, bool wbasis, C* c, const C* x) {
  const bool mixed = wbasis && k.mixed;
  for (int idx = threadIdx.x; idx < k.P * TM; idx += blockDim.x) {
    const int n = idx / TM, mm = idx - n * TM;
    C v;
    if (!mixed) {
      v = (n < k.G) ? col::gneg(x[n * TM + mm]) : col::gzero<C>();
      if (n >= 2 && n - 2 < k.G) v = gadd(v, x[(n - 2) * TM + mm]);
    } else {
      v = (n < k.G) ? x[n * TM + mm] : col::gzero<C>();
      if (n >= 1 && n - 1 < k.G) v = col::gaxpy(Prec<C>::s(__ldg(k.wa + n - 1)), x[(n - 1) * TM + mm], v);
      if (n >= 2 && n - 2 < k.G) v = col::gaxpy(Prec<C>::s(__ldg(k.wb + n - 2)), x[(n - 2) * TM + mm], v);
    }
    c[idx] = v;
  }
}
// ------------------------------------------------------------ per-mode kernels
// Tiles of type C: double2 in the plain path; cdfl (double-float on the FP32
// pipe, about 48 significant bits) in the mixed-precision path, where these
// transforms carry the state itself and FP32 would be too coarse.  Fields in
// global memory stay FP64 either way.

// out[i] = sum_j Mat[i][j] x[j] for the rows i = blockIdx.x, blockIdx.x +
// gridDim.x, ... < n, one warp per row (lane partial sums over j = lane + 32 q,
// then a fixed shuffle tree): a dense 1-D map spread over the CTAs of a
// multi-CTA kernel instead of one SM's FP64 pipe.
__device__ __forceinline__ void rows_by_ctas(const double* __restrict__ Mat, const double* __restrict__ x,
                                             double* __restrict__ out, int n) {
  if (Mat == nullptr || threadIdx.x >= 32) return;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const double* row = Mat + (size_t)i * n;
    double acc = 0.0;
    for (int j = threadIdx.x; j < n; j += 32) acc = fma(row[j], x[j], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) out[i] = acc;
  }
}

// Predictor w and theta to nodal CGL values and to the SBP grid; the CTAs
// also form tb_sbp = c2s V tbp (the predictor mean temperature on the SBP grid).
template <typename C>
__global__ void __launch_bounds__(NT) k_corr_pre(CK k, const double2* wp, const double2* tp,
                                                 double2* wcgl, double2* wsbp, double2* tsbp,
                                                 const double* tbp, double* vec) {
  rows_by_ctas(k.c2sV, tbp, vec + CV{k.P}.tb_sbp(), k.P);
  extern __shared__ double2 sm_raw[];
  C* sm = reinterpret_cast<C*>(sm_raw);
  const int PT = k.P * TM;
  C *b0 = sm, *b1 = sm + PT;
  const col::DctSharedT<C> ds = col::dct_shared<C>(k.dct, sm + 2 * PT);
  const int m0 = blockIdx.x * TM;
  tloadp(b0, wp, k.G, m0, k.M);
  __syncthreads();
  tstencil(k, true, b1, b0);
  __syncthreads();
  tdct(b0, b1, k.dct, ds, false, k.P);
  __syncthreads();
  tstorep(b0, wcgl, k.P, m0, k.M);
  tcsr(b1, b0, k.c2s_ptr, k.c2s_col, k.c2s_val, k.P);
  __syncthreads();
  tstorep(b1, wsbp, k.P, m0, k.M);
  __syncthreads();
  tloadp(b0, tp, k.G, m0, k.M);
  __syncthreads();
  tstencil(k, false, b1, b0);
  __syncthreads();
  tdct(b0, b1, k.dct, ds, false, k.P);
  __syncthreads();
  tcsr(b1, b0, k.c2s_ptr, k.c2s_col, k.c2s_val, k.P);
  __syncthreads();
  tstorep(b1, tsbp, k.P, m0, k.M);
}

template <typename C>
__global__ void __launch_bounds__(NT) k_corr_sub(CK k, double2* tsbp, const double2* wsbp,
                                                 const double* g_half, double sub_dt, int last,
                                                 double2* t_out, double2* tcgl, const double* y_mean,
                                                 double* tb_out) {
  // last substep: the corrected mean temperature tb_out = P_tau V^-1 y_mean
  if (last) rows_by_ctas(k.tauVinv, y_mean, tb_out, k.P);
  using T = typename Prec<C>::T;
  extern __shared__ double2 sm_raw[];
  C* sm = reinterpret_cast<C*>(sm_raw);
  const int PT = k.P * TM;
  C *b0 = sm, *b1 = sm + PT, *b2 = sm + 2 * PT, *b3 = sm + 3 * PT;
  const col::DctSharedT<C> ds = col::dct_shared<C>(k.dct, sm + 4 * PT);
  __shared__ C delta[2 * TM];
  const int m0 = blockIdx.x * TM;
  const int P = k.P;
  tloadp(b0, tsbp, P, m0, k.M);
  tloadp(b1, wsbp, P, m0, k.M);
  __syncthreads();
  for (int i = threadIdx.x; i < PT; i += blockDim.x) {
    const int l = i / TM;
    b0[i] = (l == 0 || l == P - 1) ? col::gzero<C>()
                                   : col::gaxpy(Prec<C>::s(-sub_dt * g_half[l]), b1[i], b0[i]);
  }
  __syncthreads();
  tcsr(b2, b0, k.s2c_ptr, k.s2c_col, k.s2c_val, P);  // y = s2c theta_sbp_new
  __syncthreads();
  if (!last || tcgl != nullptr) {
    {  // delta_j = F_j . y for j = 0, 1, re/im: 4*TM dot products, one warp each pass
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for (int d = warp; d < 4 * TM; d += blockDim.x >> 5) {
        const int mm = d % TM, j = (d / TM) & 1, im = d / (2 * TM);
        const double* F = k.bcF + j * P;
        T acc = T(0);
        for (int l = lane; l < P; l += 32)
          acc = fma(Prec<C>::s(F[l]), im ? b2[l * TM + mm].y : b2[l * TM + mm].x, acc);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) { if (im) delta[j * TM + mm].y = acc; else delta[j * TM + mm].x = acc; }
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < PT; i += blockDim.x) {
      const int l = i / TM, mm = i - l * TM;
      C v = col::gaxpy(Prec<C>::s(k.bcV[l]), delta[mm], b2[i]);
      b3[i] = col::gaxpy(Prec<C>::s(k.bcV[P + l]), delta[TM + mm], v);
    }
    __syncthreads();
    if (!last) {
      tcsr(b1, b3, k.c2s_ptr, k.c2s_col, k.c2s_val, P);
      __syncthreads();
      tstorep(b1, tsbp, P, m0, k.M);
    } else {
      tstorep(b3, tcgl, P, m0, k.M);
    }
  }
  if (last) {
    __syncthreads();
    tdct(b0, b2, k.dct, ds, true, k.G);  // first G Chebyshev coefficients of V^-1 y
    __syncthreads();
    tpinv_dir(b1, b0, k.G);
    __syncthreads();
    tstorep(b1, t_out, k.G, m0, k.M);
  }
}

// Non-final substep, fused: with x = theta_sbp - sub_dt g_half w_sbp (zero
// at the two end levels), the round trip above is
//   theta_sbp' = R x + u_0 (Fs_0 . x) + u_1 (Fs_1 . x)
// with R = c2s s2c (a few nonzeros per row), Fs_j = s2c^T F_j, u_j = c2s V[:,N-1+j].
// One CTA holds kSM consecutive modes (coalesced 128-byte level rows; the
// 33 KB tile lets six CTAs share an SM); thread (level group lg, mode mm)
// visits levels lg, lg + kLG, ...
constexpr int kSM = 8;
constexpr int kSubThreads = 256;
constexpr int kLG = kSubThreads / kSM;  // level groups

template <typename V>
struct SubK {
  int P, M, rw;
  const int* Rcol;
  const V *Rval, *Fs, *Us;  // V = double, or dfl for double-float tiles
  const double* g_half;
  V sub_dt;
};

template <typename C>
__global__ void __launch_bounds__(kSubThreads) k_corr_sub_mid(SubK<typename Prec<C>::T> k,
                                                              double2* __restrict__ tsbp,
                                                              const double2* __restrict__ wsbp) {
  using T = typename Prec<C>::T;
  extern __shared__ double2 xs_raw[];      // [P][kSM]
  C* xs = reinterpret_cast<C*>(xs_raw);
  __shared__ C part[2][kLG][kSM];          // partial dot products
  const int P = k.P, M = k.M;
  const int mm = threadIdx.x % kSM, lg = threadIdx.x / kSM;
  const int m = blockIdx.x * kSM + mm;
  const bool ok = m < M;
  C d0 = col::gzero<C>(), d1 = col::gzero<C>();
  for (int l = lg; l < P; l += kLG) {
    C x = col::gzero<C>();
    if (ok && l > 0 && l < P - 1) {
      const size_t g = (size_t)l * M + m;
      x = col::gaxpy(-k.sub_dt * Prec<C>::s(k.g_half[l]), Prec<C>::in(wsbp[g]), Prec<C>::in(tsbp[g]));
    }
    xs[l * kSM + mm] = x;
    d0 = col::gaxpy(k.Fs[l], x, d0);
    d1 = col::gaxpy(k.Fs[P + l], x, d1);
  }
  part[0][lg][mm] = d0;
  part[1][lg][mm] = d1;
  __syncthreads();
  if (lg < 2) {  // 2 kSM threads: (j, mm) totals, summed in a fixed order
    C acc = col::gzero<C>();
    for (int q = 0; q < kLG; ++q) acc = gadd(acc, part[lg][q][mm]);
    part[lg][0][mm] = acc;
  }
  __syncthreads();
  d0 = part[0][0][mm];
  d1 = part[1][0][mm];
  if (!ok) return;
  for (int l = lg; l < P; l += kLG) {
    C v = col::gaxpy(k.Us[P + l], d1, gscale(d0, k.Us[l]));
    const int* rc = k.Rcol + (size_t)l * k.rw;
    const T* rv = k.Rval + (size_t)l * k.rw;
    for (int q = 0; q < k.rw; ++q) v = col::gaxpy(rv[q], xs[rc[q] * kSM + mm], v);
    tsbp[(size_t)l * M + m] = Prec<C>::out(v);
  }
}

// ------------------------------------------------------------ 1-D kernels (one CTA)
__device__ void vec_dense(double* out, const double* in, const double* Mat, int n, int ld, int ncol) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double* row = Mat + (size_t)i * ld;
    double acc = 0.0;
    for (int j = 0; j < ncol; ++j) acc = fma(row[j], in[j], acc);
    out[i] = acc;
  }
}
__device__ void vec_csr(double* out, const double* in, const int* ptr, const int* col,
                        const double* val, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double acc = 0.0;
    for (int q = ptr[i]; q < ptr[i + 1]; ++q) acc = fma(val[q], in[col[q]], acc);
    out[i] = acc;
  }
}
// pentadiagonal matrix stored as band[d*P + i] = A[i, i+d-2]
__device__ void band_matvec(double* out, const double* band, const double* x, int P) {
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double acc = 0.0;
    for (int d = 0; d < 5; ++d) {
      const int j = i + d - 2;
      if (j >= 0 && j < P) acc = fma(band[d * P + i], x[j], acc);
    }
    out[i] = acc;
  }
}
// D1 (tridiagonal) product
__device__ void d1_matvec(double* out, const double* D1, const double* x, int P) {
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double acc = 0.0;
    for (int j = max(0, i - 1); j <= min(P - 1, i + 1); ++j) acc = fma(D1[(size_t)i * P + j], x[j], acc);
    out[i] = acc;
  }
}

// The band is built and factored in shared memory: the factorisation is a
// serial recurrence, and shared-memory operands keep each step at on-chip
// latency.  Dynamic shared memory: 10 P doubles.
// Builds the pentadiagonal corrector matrices A = I - h (boundary rows
// identity) and B = I + h in FP64, and factors A in FP32 (LU without
// pivoting: A is the identity plus an M-matrix-like term, diagonally
// dominant, so the factors stay bounded).  The substitutions of
// k_corr_tstep use the FP32 factors inside an FP64 iterative refinement: the
// factorisation and the substitutions are serial recurrences, and on this
// GPU a dependent FP64 operation costs about 14 times a dependent FP32 one
// (a division about 90 times).  Dynamic shared memory: 10 P doubles.
__device__ __forceinline__ void corr_init_body(const CK& k, double* vec, double sub_dt, double* band_sm) {
  const CV cv{k.P};
  const int P = k.P;
  double* w2 = vec + cv.w2();
  double* A = band_sm;
  double* B = band_sm + 5 * P;
  const double c1 = 0.5 * k.mu * k.kappa * sub_dt;
  const double c2 = 0.25 * k.mu * (sub_dt * sub_dt);
  for (int idx = threadIdx.x; idx < 5 * P; idx += blockDim.x) {
    const int d = idx / P, i = idx - d * P;
    const int j = i + d - 2;
    double h = 0.0, a = 0.0, b = 0.0;
    if (j >= 0 && j < P) {
      double dmd = 0.0;  // (D1 diag(w2) D1)[i, j]
      for (int kk = max(0, i - 1); kk <= min(P - 1, i + 1); ++kk) {
        if (abs(kk - j) <= 1) dmd = fma(k.D1[(size_t)i * P + kk] * w2[kk], k.D1[(size_t)kk * P + j], dmd);
      }
      h = fma(c1, k.Lsbp[(size_t)i * P + j], c2 * dmd);
      const double id = (i == j) ? 1.0 : 0.0;
      a = id - h;
      b = id + h;
      if (i == 0 || i == P - 1) a = id;
    }
    A[idx] = a;
    B[idx] = b;
    vec[cv.Aband() + idx] = a;
    vec[cv.Bband() + idx] = b;
  }
  __syncthreads();
  float* L = reinterpret_cast<float*>(band_sm + 5 * P);  // FP32 factors over the B copy
  for (int idx = threadIdx.x; idx < 5 * P; idx += blockDim.x) L[idx] = (float)A[idx];
  __syncthreads();
  if (threadIdx.x == 0) {
    // banded LU: multipliers below the diagonal, 1/pivot in the diagonal
    // slot.  Row i of the band is A[i, i-2 .. i+2]; the running values of
    // the two rows below the current pivot stay in registers.
    float r1_0 = P > 1 ? L[1 * P + 1] : 0.f, r1_1 = P > 1 ? L[2 * P + 1] : 0.f;
    float r1_2 = P > 1 ? L[3 * P + 1] : 0.f;
    float piv = L[2 * P + 0], u1 = L[3 * P + 0], u2 = L[4 * P + 0];
    for (int col = 0; col < P; ++col) {
      const float rp = 1.0f / piv;
      L[2 * P + col] = rp;
      float r2_0 = 0.f, r2_1 = 0.f, r2_2 = 0.f, r2_3 = 0.f;
      if (col + 2 < P) {
        r2_0 = L[0 * P + col + 2];
        r2_1 = L[1 * P + col + 2];
        r2_2 = L[2 * P + col + 2];
        r2_3 = L[3 * P + col + 2];
      }
      float n_piv = 0.f, n_u1 = 0.f, n_u2 = 0.f;
      if (col + 1 < P) {
        const float l = r1_0 * rp;
        L[1 * P + col + 1] = l;
        n_piv = fmaf(-l, u1, r1_1);
        n_u1 = fmaf(-l, u2, r1_2);
        n_u2 = (col + 3 < P) ? L[4 * P + col + 1] : 0.f;
        L[3 * P + col + 1] = n_u1;
      }
      if (col + 2 < P) {
        const float l = r2_0 * rp;
        L[0 * P + col + 2] = l;
        r1_0 = fmaf(-l, u1, r2_1);
        r1_1 = fmaf(-l, u2, r2_2);
        r1_2 = r2_3;
      }
      piv = n_piv; u1 = n_u1; u2 = n_u2;
    }
  }
  __syncthreads();
  float* Lg = reinterpret_cast<float*>(vec + cv.lu32());
  for (int idx = threadIdx.x; idx < 5 * P; idx += blockDim.x) Lg[idx] = L[idx];
  __syncthreads();
}

// d = (LU)^-1 r with the FP32 factors: rf holds r in FP32 on entry and d on
// exit.  Serial, thread 0; FP32 only, so each step costs FP32 latency.
__device__ __forceinline__ void lu32_solve(const float* __restrict__ L, float* __restrict__ rf, int P) {
  // operands are fetched 8 rows ahead of the dependent chain so that the
  // shared-memory latency overlaps the FMAs
  constexpr int U = 8;
  float v1 = rf[0], v2 = 0.f;
  int i = 1;
  for (; i + U <= P; i += U) {
    float a0[U], a1[U], r[U];
#pragma unroll
    for (int q = 0; q < U; ++q) { a0[q] = L[0 * P + i + q]; a1[q] = L[1 * P + i + q]; r[q] = rf[i + q]; }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      float v = fmaf(-a1[q], v1, r[q]);
      if (i + q >= 2) v = fmaf(-a0[q], v2, v);
      rf[i + q] = v;
      v2 = v1;
      v1 = v;
    }
  }
  for (; i < P; ++i) {
    float v = fmaf(-L[1 * P + i], v1, rf[i]);
    if (i >= 2) v = fmaf(-L[0 * P + i], v2, v);
    rf[i] = v;
    v2 = v1;
    v1 = v;
  }
  float x1 = 0.f, x2 = 0.f;
  int j = P - 1;
  for (; j - U + 1 >= 0; j -= U) {
    float d[U], u1[U], u2[U], r[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int ii = j - q;
      d[q] = L[2 * P + ii]; u1[q] = L[3 * P + ii]; u2[q] = L[4 * P + ii]; r[q] = rf[ii];
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int ii = j - q;
      float v = r[q];
      if (ii + 1 < P) v = fmaf(-u1[q], x1, v);
      if (ii + 2 < P) v = fmaf(-u2[q], x2, v);
      v *= d[q];
      rf[ii] = v;
      x2 = x1;
      x1 = v;
    }
  }
  for (; j >= 0; --j) {
    float v = rf[j];
    if (j + 1 < P) v = fmaf(-L[3 * P + j], x1, v);
    if (j + 2 < P) v = fmaf(-L[4 * P + j], x2, v);
    v *= L[2 * P + j];
    rf[j] = v;
    x2 = x1;
    x1 = v;
  }
}

// Solves A tb_new = B tb_sbp - mu sub_dt D1 flux by FP64 iterative
// refinement around the FP32 factors (Wilkinson's mixed-precision iterative
// refinement): x_0 = (LU)^-1 b, x_{k+1} = x_k + (LU)^-1 (b - A x_k) with the
// residual in FP64.  Each sweep divides the error by about
// 1 / (cond(A) eps_32); kRefine sweeps reach FP64 round-off for the
// corrector's well-conditioned A = I + (SPD-like) h.  Dynamic shared memory:
// 5 P doubles (FP64 A band) + 3 P doubles (FP32 factors) + 3 P doubles.
// With init (the first substep) the kernel first builds and factors the
// corrector matrices (corr_init_body); its global writes are visible to the
// rest of the CTA after the barrier that ends the body.
constexpr int kRefine = 2;
__global__ void k_corr_tstep(CK k, double* vec, double sub_dt, int last, int init) {
  const CV cv{k.P};
  const int P = k.P;
  __shared__ double red[64];
  extern __shared__ double band_sm[];
  if (init) corr_init_body(k, vec, sub_dt, band_sm);
  double* flux = vec + cv.flux();
  double* tbs = vec + cv.tb_sbp();
  double* gh = vec + cv.g_half();
  double* A = band_sm;                                  // 5P FP64
  float* L = reinterpret_cast<float*>(band_sm + 5 * P); // 5P FP32 (3P doubles)
  double* b = band_sm + 8 * P;
  double* rhs = band_sm + 9 * P;  // the solution
  double* res = band_sm + 10 * P;
  double* t2 = vec + cv.tmp2();
  const double* B = vec + cv.Bband();
  const float* Lg = reinterpret_cast<const float*>(vec + cv.lu32());
  for (int idx = threadIdx.x; idx < 5 * P; idx += blockDim.x) {
    A[idx] = vec[cv.Aband() + idx];
    L[idx] = Lg[idx];
  }
  // b = B tb_sbp - mu sub_dt D1 flux
  band_matvec(b, B, tbs, P);
  d1_matvec(t2, k.D1, flux, P);
  __syncthreads();
  const double cf = k.mu * sub_dt;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    b[i] = (i == 0 || i == P - 1) ? 0.0 : fma(-cf, t2[i], b[i]);
    res[i] = b[i];
    rhs[i] = 0.0;
  }
  __syncthreads();
  float* rf = reinterpret_cast<float*>(res);  // FP32 view of the residual slot
  for (int it = 0; it <= kRefine; ++it) {
    double rv[4];
    for (int q = 0, i = threadIdx.x; i < P; i += blockDim.x, ++q) rv[q] = res[i];
    __syncthreads();
    for (int q = 0, i = threadIdx.x; i < P; i += blockDim.x, ++q) rf[i] = (float)rv[q];
    __syncthreads();
    if (threadIdx.x == 0) lu32_solve(L, rf, P);
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) rhs[i] += (double)rf[i];
    __syncthreads();
    if (it == kRefine) break;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {  // res = b - A x in FP64
      double acc = b[i];
      for (int d = 0; d < 5; ++d) {
        const int j = i + d - 2;
        if (j >= 0 && j < P) acc = fma(-A[d * P + i], rhs[j], acc);
      }
      res[i] = acc;
    }
    __syncthreads();
  }
  // rhs = tb_new
  for (int i = threadIdx.x; i < P; i += blockDim.x) t2[i] = tbs[i] + rhs[i];
  __syncthreads();
  d1_matvec(gh, k.D1, t2, P);
  __syncthreads();
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    gh[i] *= 0.5;
    if (i == 0 || i == P - 1) rhs[i] = 0.0;
  }
  __syncthreads();
  vec_csr(t2, rhs, k.s2c_ptr, k.s2c_col, k.s2c_val, P);  // y = s2c tb_new
  __syncthreads();
  if (!last) {
    double a0 = 0.0, a1 = 0.0;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      a0 = fma(k.bcF[i], t2[i], a0);
      a1 = fma(k.bcF[P + i], t2[i], a1);
    }
    const double d0 = block_sum(a0, red);
    const double d1 = block_sum(a1, red + 32);
    if (threadIdx.x == 0) { red[0] = d0; red[1] = d1; }
    __syncthreads();
    const double e0 = red[0], e1 = red[1];
    for (int i = threadIdx.x; i < P; i += blockDim.x)
      rhs[i] = fma(k.bcV[P + i], e1, fma(k.bcV[i], e0, t2[i]));
    __syncthreads();
    vec_csr(tbs, rhs, k.c2s_ptr, k.c2s_col, k.c2s_val, P);
  }
  // last substep: y = t2 stays in global memory; the last per-mode kernel of
  // the corrector maps it back to coefficients (k_corr_sub, rows_by_ctas)
}

// ---- mean-temperature stage update: R = combos; out = solve(R)
struct MK {
  int P, N;
  const double *proj, *mean_solve, *GZ2;
  double eps_sq, sigma;
};

__global__ void k_mean_stage(MK k, MeanArgs a) {
  __shared__ double R[1024];
  const int P = k.P, N = k.N;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double r = a.tb0[i];
    if (a.stage == 1) {
      if (a.E1tb) r = fma(a.alpha, a.E1tb[i], r);
    } else {
      if (a.E1tb) r = fma(a.c_E1, a.E1tb[i], r);
      if (a.E2tb) r = fma(a.c_E2, a.E2tb[i], r);
      if (a.itend) {  // omega * (eps^2/sigma) G_Z2 tb1
        const double* row = k.GZ2 + (size_t)i * P;
        double acc = 0.0;
        for (int j = 0; j < P; ++j) acc = fma(row[j], a.tb1[j], acc);
        r = fma(a.omega * (k.eps_sq / k.sigma), acc, r);
      }
      if (a.inv_alpha_c != 0.0) r = fma(a.omega * a.inv_alpha_c, a.tb1[i] - a.tb1p[i], r);
    }
    R[i] = r;
  }
  __syncthreads();
  if (a.closure == NHQG_CLOSURE_EVOLVE_MEAN) {  // legacy implicit 1-D solve with tau rows
    if (threadIdx.x == 0) { R[N - 1] = 0.0; R[N] = 0.0; }
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      const double* row = k.mean_solve + (size_t)i * P;
      double acc = 0.0;
      for (int j = 0; j < P; ++j) acc = fma(row[j], R[j], acc);
      a.out[i] = acc;
    }
  } else {  // Dirichlet tau projection
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      if (i < N - 1) {
        a.out[i] = R[i];
      } else {
        const double* row = k.proj + (size_t)i * P;
        double acc = 0.0;
        for (int j = 0; j < N - 1; ++j) acc = fma(row[j], R[j], acc);
        a.out[i] = acc;
      }
    }
  }
}

// legacy evolve_mean explicit pieces: dtb_nodal = V (G_Z tb);
// E_tb = -eps^2 G_Z (V^-1 flux_nodal); I_tb = (eps^2/sigma) G_Z2 tb
struct LK {
  int P;
  const double *V, *Vinv, *GZ, *GZ2;
  double eps_sq, sigma;
};
__global__ void k_mean_legacy(LK k, const double* tb, const double* flux, double* dtb, double* Etb,
                              double* Itb) {
  __shared__ double t1[1024], t2[1024];
  const int P = k.P;
  if (dtb) {
    vec_dense(t1, tb, k.GZ, P, P, P);
    __syncthreads();
    vec_dense(dtb, t1, k.V, P, P, P);
    __syncthreads();
  }
  if (Etb) {
    vec_dense(t2, flux, k.Vinv, P, P, P);
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      const double* row = k.GZ + (size_t)i * P;
      double acc = 0.0;
      for (int j = 0; j < P; ++j) acc = fma(row[j], t2[j], acc);
      Etb[i] = k.eps_sq * (-acc);
    }
  }
  if (Itb) {
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      const double* row = k.GZ2 + (size_t)i * P;
      double acc = 0.0;
      for (int j = 0; j < P; ++j) acc = fma(row[j], tb[j], acc);
      Itb[i] = (k.eps_sq / k.sigma) * acc;
    }
  }
}

}  // namespace

size_t corrector_vec_doubles(int P) { return (size_t)CV{P}.total(); }

cudaError_t run_corrector(const Params& p, const Tables& t, Work& w, const CorrArgs& a,
                          cudaStream_t st, int* nlaunch) {
  CK k = make_ck(p, t);
  const CV cv{p.d.P};
  const int nsub = p.substeps > 0 ? p.substeps : 1;
  const double sub_dt = a.total_dt / nsub;
  const int grid = (p.d.M + TM - 1) / TM;
  const size_t dsm = col::dct_smem_bytes(k.dct);
  const size_t sm2 = 2 * (size_t)p.d.P * TM * sizeof(double2) + dsm;
  const size_t sm4 = 4 * (size_t)p.d.P * TM * sizeof(double2) + dsm;
  // double-float tiles (same 16-byte complex size) need the fast DCT's tables
  const bool df = a.df && k.dct.fast && k.dct.tw_df != nullptr;
  auto pre = df ? k_corr_pre<cdfl> : k_corr_pre<double2>;
  auto sub = df ? k_corr_sub<cdfl> : k_corr_sub<double2>;
  cudaFuncSetAttribute(pre, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
  cudaFuncSetAttribute(sub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm4);
  const size_t smid = (size_t)p.d.P * kSM * sizeof(double2);
  const bool fused_mid = smid <= 200 * 1024 && t.R_col != nullptr;
  if (fused_mid) {
    cudaFuncSetAttribute(k_corr_sub_mid<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smid);
    cudaFuncSetAttribute(k_corr_sub_mid<cdfl>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smid);
  }
  Profiler& pf = w.prof;
  pf.begin("corr_pre", st);
  pre<<<grid, NT, sm2, st>>>(k, a.wp, a.tp, a.wcgl, a.wsbp, a.tsbp, a.tbp, w.vec);
  pf.end(st);
  pf.begin("parseval", st);
  launch_parseval2(p, a.wsbp, a.wsbp, a.tsbp, p.d.P, w.vec + cv.w2(), w.vec + cv.flux(), w, st, df);
  pf.end(st);
  int n = 2;
  for (int s = 0; s < nsub; ++s) {
    const int last = (s == nsub - 1);
    if (s > 0) {
      pf.begin("parseval", st);
      launch_parseval(p, a.wsbp, a.tsbp, p.d.P, w.vec + cv.flux(), w, st, df);
      pf.end(st);
      ++n;
    }
    pf.begin("corr_step_1d", st);
    k_corr_tstep<<<1, NT, 11 * (size_t)p.d.P * sizeof(double), st>>>(k, w.vec, sub_dt, last, s == 0);
    pf.end(st);
    if (!last && fused_mid) {
      pf.begin("corr_sub_mid", st);
      if (df && t.R_val_df) {
        SubK<dfl> sk{p.d.P, p.d.M, t.R_w, t.R_col, t.R_val_df, t.Fs_df, t.Us_df, w.vec + cv.g_half(),
                     dfl(sub_dt)};
        k_corr_sub_mid<cdfl><<<(p.d.M + kSM - 1) / kSM, kSubThreads, smid, st>>>(sk, a.tsbp, a.wsbp);
      } else {
        SubK<double> sk{p.d.P, p.d.M, t.R_w, t.R_col, t.R_val, t.Fs, t.Us, w.vec + cv.g_half(), sub_dt};
        k_corr_sub_mid<double2><<<(p.d.M + kSM - 1) / kSM, kSubThreads, smid, st>>>(sk, a.tsbp, a.wsbp);
      }
      pf.end(st);
    } else {
      pf.begin(last ? "corr_sub_last" : "corr_sub", st);
      sub<<<grid, NT, sm4, st>>>(k, a.tsbp, a.wsbp, w.vec + cv.g_half(), sub_dt, last, a.t_out,
                                 a.tcgl, w.vec + cv.tmp2(), a.tb_out);
      pf.end(st);
    }
    n += 2;
  }
  if (nlaunch) *nlaunch += n;
  return cudaGetLastError();
}

cudaError_t launch_corr_pre(const Params& p, const Tables& t, const double2* w, const double2* th,
                            double2* wcgl, double2* wsbp, double2* tsbp, cudaStream_t st) {
  CK k = make_ck(p, t);
  const size_t sm2 = 2 * (size_t)p.d.P * TM * sizeof(double2) + col::dct_smem_bytes(k.dct);
  cudaFuncSetAttribute(k_corr_pre<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
  k.c2sV = nullptr;  // no mean-temperature side job here
  k_corr_pre<double2><<<(p.d.M + TM - 1) / TM, NT, sm2, st>>>(k, w, th, wcgl, wsbp, tsbp, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_mean_stage(const Params& p, const Tables& t, const MeanArgs& a, cudaStream_t st) {
  MK k;
  k.P = p.d.P; k.N = p.d.Nz;
  k.proj = t.proj; k.mean_solve = t.mean_solve; k.GZ2 = t.GZ2;
  k.eps_sq = p.eps_sq; k.sigma = p.sigma;
  if (a.closure == NHQG_CLOSURE_EVOLVE_MEAN && t.mean_solve == nullptr) return cudaErrorInvalidValue;
  k_mean_stage<<<1, NT, 0, st>>>(k, a);
  return cudaGetLastError();
}

cudaError_t launch_mean_legacy_rhs(const Params& p, const Tables& t, const double* tb,
                                   const double* flux_nodal, double* dtb_nodal, double* E_tb,
                                   double* I_tb, cudaStream_t st) {
  LK k;
  k.P = p.d.P; k.V = t.V; k.Vinv = t.Vinv; k.GZ = t.GZ; k.GZ2 = t.GZ2;
  k.eps_sq = p.eps_sq; k.sigma = p.sigma;
  k_mean_legacy<<<1, NT, 0, st>>>(k, tb, flux_nodal, dtb_nodal, E_tb, I_tb);
  return cudaGetLastError();
}

}  // namespace nhqg

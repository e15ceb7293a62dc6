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
#include <algorithm>
#include <cmath>

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
  __host__ __device__ int lu_ok() const { return 19 * P; }  // 1: lu32 holds the factors of this A
  __host__ __device__ int win() const { return 19 * P + 2; }  // window factors
  __host__ __device__ int total() const { return 19 * P + 2 + win_doubles(P); }
  // overlapping windows of the 1-D solve: kWinCore core rows, up to
  // kWinOvMax rows of overlap on each side, 5 FP32 band rows each (+1 float
  // of padding per window so that the windows' threads hit distinct banks)
  static constexpr int kWinCore = 32, kWinOvMax = 24, kWinLen = kWinCore + 2 * kWinOvMax;
  static constexpr int kWinStride = 5 * kWinLen + 1;  // floats per window
  __host__ __device__ static constexpr int n_win(int P) { return (P + kWinCore - 1) / kWinCore; }
  __host__ __device__ static constexpr int win_doubles(int P) { return (n_win(P) * kWinStride + 1) / 2; }
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
  const double *D1b, *Lb;  // D1 (3 diagonals) and the SBP Laplacian (5), [d][P]
  int ell_w;               // c2s / s2c as fixed-width rows, [q][P]
  const int *c2s_ecol, *s2c_ecol;
  const double *c2s_eval, *s2c_eval;
  int win_ov;              // overlap of the windowed 1-D solve; 0: one serial LU
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
  k.D1b = t.D1b; k.Lb = t.Lb;
  k.ell_w = t.ell_w;
  k.c2s_ecol = t.c2s_ecol; k.s2c_ecol = t.s2c_ecol; k.c2s_eval = t.c2s_eval; k.s2c_eval = t.s2c_eval;
  k.win_ov = 0;
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
// In the double-float path w runs on FP32 tiles: it enters the corrector only
// through the exchange increment sub_dt g_half w (about 1e-5 of theta, so an
// FP32 w changes theta by ~1e-12 relative), the means <w^2>, <w theta> (an
// FP32-relative error there is again scaled by sub_dt) and the nodal w of the
// next explicit RHS, whose products are FP32.  theta, the state the corrector
// carries, stays double-float.
// The double-float instantiation writes w as FP32 (wcgl_f, wsbp_f; a null
// wcgl_f skips the nodal w), the FP64 one as FP64 (wcgl, wsbp).
template <typename C>
__global__ void __launch_bounds__(NT) k_corr_pre(CK k, const double2* wp, const double2* tp,
                                                 double2* wcgl, double2* wsbp, float2* wcgl_f,
                                                 float2* wsbp_f, double2* tsbp, const double* tbp,
                                                 double* vec) {
  rows_by_ctas(k.c2sV, tbp, vec + CV{k.P}.tb_sbp(), k.P);
  using CW = typename std::conditional<std::is_same<C, cdfl>::value, float2, C>::type;
  extern __shared__ double2 sm_raw[];
  const int PT = k.P * TM;
  void* dct_base = sm_raw + 2 * PT;  // after two tiles of the widest type
  const int m0 = blockIdx.x * TM;
  col::tprefetch(tp, k.G, m0, k.M, sizeof(double2));  // theta, read after w's transform
  {
    CW* sw = reinterpret_cast<CW*>(sm_raw);
    CW *b0 = sw, *b1 = sw + PT;
    const col::DctSharedT<CW> ds = col::dct_shared<CW>(k.dct, dct_base);
    tloadp(b0, wp, k.G, m0, k.M);
    __syncthreads();
    tstencil(k, true, b1, b0);
    __syncthreads();
    tdct(b0, b1, k.dct, ds, false, k.P);
    __syncthreads();
    if constexpr (std::is_same<CW, float2>::value) {
      if (wcgl_f != nullptr) tstorep(b0, wcgl_f, k.P, m0, k.M);
    } else {
      tstorep(b0, wcgl, k.P, m0, k.M);
    }
    tcsr(b1, b0, k.c2s_ptr, k.c2s_col, k.c2s_val, k.P);
    __syncthreads();
    if constexpr (std::is_same<CW, float2>::value) tstorep(b1, wsbp_f, k.P, m0, k.M);
    else tstorep(b1, wsbp, k.P, m0, k.M);
    __syncthreads();
  }
  C* sm = reinterpret_cast<C*>(sm_raw);
  C *b0 = sm, *b1 = sm + PT;
  const col::DctSharedT<C> ds = col::dct_shared<C>(k.dct, dct_base);
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

template <typename C, typename WT>
__global__ void __launch_bounds__(NT) k_corr_sub(CK k, double2* tsbp, const WT* wsbp,
                                                 const double* g_half, double sub_dt, int last,
                                                 double2* t_out,
                                                 typename std::conditional<std::is_same<WT, float2>::value,
                                                                           float2, double2>::type* tcgl,
                                                 const double* y_mean,
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

__device__ __forceinline__ float as_float(dfl v) { return __fadd_rn(v.hi, v.lo); }

template <typename V>
struct SubK {
  int P, M, rw;
  const int* Rcol;
  const V *Rval, *Fs, *Us;  // V = double, or dfl for double-float tiles
  const double* g_half;
  V sub_dt;
};

// With part != nullptr the CTA also forms the per-level sums of
// wt Re(w conj(theta_sbp')) over its kSM modes (the Parseval weights of the
// compact modes, pwt), the next substep's flux <w theta> before its scale;
// part[l * gridDim.x + blockIdx.x] holds them, summed over CTAs in a fixed
// order by k_corr_tstep.  The weights take the ky = 0 column once instead of
// through its Hermitian projection: the corrector's per-mode maps have real
// coefficients, so Hermitian inputs stay Hermitian and the two agree to
// rounding.
template <typename C, typename WT>
__global__ void __launch_bounds__(kSubThreads) k_corr_sub_mid(SubK<typename Prec<C>::T> k,
                                                              double2* __restrict__ tsbp,
                                                              const WT* __restrict__ wsbp,
                                                              double* __restrict__ part,
                                                              const double2* __restrict__ pwt) {
  using T = typename Prec<C>::T;
  extern __shared__ double2 xs_raw[];      // [P][kSM]
  C* xs = reinterpret_cast<C*>(xs_raw);
  __shared__ C sum2[2][kLG][kSM];          // partial dot products
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
  sum2[0][lg][mm] = d0;
  sum2[1][lg][mm] = d1;
  __syncthreads();
  if (lg < 2) {  // 2 kSM threads: (j, mm) totals, summed in a fixed order
    C acc = col::gzero<C>();
    for (int q = 0; q < kLG; ++q) acc = gadd(acc, sum2[lg][q][mm]);
    sum2[lg][0][mm] = acc;
  }
  __syncthreads();
  d0 = sum2[0][0][mm];
  d1 = sum2[1][0][mm];
  float wr = 0.f, wi = 0.f;
  if (part != nullptr && ok) {
    const double2 wt = pwt[m];  // 2, 1, 1/2 or 0: exact in FP32
    wr = (float)wt.x;
    wi = (float)wt.y;
  }
  // the kSM lanes of a level group run the same levels
  const unsigned gmask = 0xFFu << (threadIdx.x & 24);
  for (int l = lg; l < P; l += kLG) {
    C v = col::gaxpy(k.Us[P + l], d1, gscale(d0, k.Us[l]));
    const int* rc = k.Rcol + (size_t)l * k.rw;
    const T* rv = k.Rval + (size_t)l * k.rw;
    for (int q = 0; q < k.rw; ++q) v = col::gaxpy(rv[q], xs[rc[q] * kSM + mm], v);
    const size_t g = (size_t)l * M + m;
    if (ok) tsbp[g] = Prec<C>::out(v);
    if constexpr (std::is_same<WT, float2>::value) {
      // the flux enters th_bar scaled by mu sub_dt D1: FP32 products of the
      // FP32 w with theta rounded to FP32, summed over the kSM modes in FP32,
      // then in FP64 across CTAs
      if (part != nullptr) {
        float f = 0.f;
        if (ok) {
          const float2 w = wsbp[g];
          f = fmaf(wr * w.x, as_float(v.x), (wi * w.y) * as_float(v.y));
        }
        for (int o = 1; o < kSM; o <<= 1) f += __shfl_xor_sync(gmask, f, o);
        if (mm == 0) part[(size_t)l * gridDim.x + blockIdx.x] = f2d_bits(f);
      }
    }
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
// ---- 1-D corrector solve
// A = I - h (boundary rows identity) and B = I + h with the pentadiagonal
// h = (mu kappa sub_dt / 2) L_sbp + (mu sub_dt^2 / 4) D1 diag(<w^2>) D1, per
// corrector.  A = I + (an M-matrix-like term) is diagonally dominant with a
// condition number near 1 (1.7 at 256 levels, dt = 2e-5), and its inverse
// decays geometrically away from the diagonal, like r^|i-j| with r the small
// root of a r^2 - (1 + 2a) r + a = 0, a = mu kappa sub_dt / (2 dz^2)
// (r = 0.125 there).
//
// Solve: FP64 iterative refinement (Wilkinson's mixed-precision scheme)
// around an FP32 approximate inverse, x_0 = M b, x_{k+1} = x_k + M (b - A x_k)
// with the residual in FP64.  M is the restricted additive Schwarz inverse
// over overlapping windows: window w owns the kWinCore core rows
// [32 w, 32 w + 32) and solves the window's own block of A over the core
// widened by win_ov rows on each side (FP32 banded LU, factored per window
// in parallel), keeping its core rows.  The truncated coupling changes the
// core rows by about r^win_ov relative, which the host sets to 1e-7 or
// below, so each sweep divides the error by about 1e7 -- as a global FP32 LU
// would -- while the serial chains are one window long instead of P.  If
// the last correction is not below 1e-10 of the solution (the windows did
// not converge: a far larger <w^2> than the host's estimate assumed), the
// kernel factors the whole band once (one thread) and redoes the solve with
// it.

// Banded LU without pivoting of rows [e0, e0 + n) of the pentadiagonal A
// (band[d P + i] = A[i, i + d - 2]; couplings outside the block dropped):
// F[0][ii], F[1][ii] the multipliers of rows ii-2, ii-1; F[2][ii] = 1 /
// pivot; F[3][ii], F[4][ii] the two superdiagonals of U times 1 / pivot.
// Serial (one thread per block), FP32.
__device__ __forceinline__ void lu32_factor(const float* __restrict__ A, int P, int e0, int n,
                                            float* __restrict__ F, int ld) {
  float d1 = 0.f, d2 = 0.f;    // 1/pivot of rows ii-1, ii-2
  float u11 = 0.f, u21 = 0.f;  // U(ii-1, ii), U(ii-1, ii+1)
  float u12 = 0.f, u22 = 0.f;  // U(ii-2, ii-1), U(ii-2, ii)
  for (int ii = 0; ii < n; ++ii) {
    const int i = e0 + ii;
    const float a0 = ii >= 2 ? A[0 * P + i] : 0.f;
    const float a1 = ii >= 1 ? A[1 * P + i] : 0.f;
    const float a2 = A[2 * P + i];
    const float a3 = ii + 1 < n ? A[3 * P + i] : 0.f;
    const float a4 = ii + 2 < n ? A[4 * P + i] : 0.f;
    const float l2 = a0 * d2;                    // row ii-2 multiplier
    const float l1 = fmaf(-l2, u12, a1) * d1;    // row ii-1 multiplier
    const float piv = fmaf(-l1, u11, fmaf(-l2, u22, a2));
    const float dv = __frcp_rn(piv);
    const float s1 = fmaf(-l1, u21, a3);         // U(ii, ii+1)
    F[0 * ld + ii] = l2;
    F[1 * ld + ii] = l1;
    F[2 * ld + ii] = dv;
    F[3 * ld + ii] = s1 * dv;
    F[4 * ld + ii] = a4 * dv;
    u12 = u11; u22 = u21;
    u11 = s1; u21 = a4;
    d2 = d1; d1 = dv;
  }
}

// x = (LU)^-1 r on a block of n rows with factors F (row stride ld): r is
// read through ridx(ii), x written through xout(ii, v); tmp takes the
// forward sweep (n rounded up to 8 floats).  The sweeps run over whole
// blocks of 8 rows with every operand index clamped into [0, n): the loads
// of a block are unconditional and issue together ahead of its dependent
// chain, rows past n carry zeros into the backward sweep, and each row adds
// the term two rows back first, so the chain through the previous row is
// one FMA in both sweeps.
template <typename RI, typename XO>
__device__ __forceinline__ void lu32_solve(const float* __restrict__ F, int ld, int n, RI ridx,
                                           float* __restrict__ tmp, XO xout) {
  constexpr int U = 8;
  const int npad = (n + U - 1) & ~(U - 1);
  float v1 = 0.f, v2 = 0.f;
  for (int i0 = 0; i0 < npad; i0 += U) {
    float a0[U], a1[U], r[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int i = min(i0 + q, n - 1);
      a0[q] = F[0 * ld + i];
      a1[q] = F[1 * ld + i];
      r[q] = ridx(i);
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const float v = fmaf(-a1[q], v1, fmaf(-a0[q], v2, r[q]));
      tmp[i0 + q] = (i0 + q < n) ? v : 0.f;
      v2 = v1;
      v1 = v;
    }
  }
  float x1 = 0.f, x2 = 0.f;
  for (int j0 = npad - 1; j0 >= 0; j0 -= U) {
    float t[U], u1[U], u2[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int jc = min(j0 - q, n - 1);
      t[q] = tmp[j0 - q] * F[2 * ld + jc];
      u1[q] = F[3 * ld + jc];
      u2[q] = F[4 * ld + jc];
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const float v = fmaf(-u1[q], x1, fmaf(-u2[q], x2, t[q]));
      if (j0 - q < n) xout(j0 - q, v);
      x2 = x1;
      x1 = v;
    }
  }
}

// shared-memory index of level i in the FP32 vectors of the windowed solve:
// one float of padding per 32, so that windows 32 levels apart use distinct
// banks
__device__ __forceinline__ int pz(int i) { return i + (i >> 5); }

// dst[i] = src[i], i < n, eight independent loads in flight per thread
template <typename T>
__device__ __forceinline__ void copy_block(T* __restrict__ dst, const T* __restrict__ src, int n) {
  constexpr int U = 8;
  const int step = blockDim.x * U;
  for (int i0 = threadIdx.x; i0 < n; i0 += step) {
    T v[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int i = i0 + q * blockDim.x;
      v[q] = i < n ? src[i] : T(0);
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int i = i0 + q * blockDim.x;
      if (i < n) dst[i] = v[q];
    }
  }
}

constexpr int kRefine = 2;
// dynamic shared memory of k_corr_tstep, doubles
__host__ __device__ constexpr int kTstepSmem(int P) { return 15 * P + 64 + CV::win_doubles(P); }

// One substep of the 1-D mean-temperature update: solves
//   A tb_new = B tb_sbp - mu sub_dt D1 flux,
// then g_half = D1 (tb_sbp + tb_new) / 2 and, except after the last
// substep, the round trip of tb_new through coefficients to the SBP grid
// (y = s2c tb_new, tb_sbp = c2s (y + V[:,N-1] F_0.y + V[:,N] F_1.y)).
// With init (the first substep of a corrector) the kernel first builds A and
// B and factors the windows.  Every phase issues its global loads together
// (the band tables, the fixed-width c2s / s2c rows), so each costs one
// memory latency.
//
// With part != nullptr (a substep after a fused k_corr_sub_mid) the kernel
// runs on P CTAs: CTA l first sums the nsum per-CTA sums of level l in a
// fixed order into the flux, and the last CTA to finish (arrival counter,
// reset for the next launch) goes on with the 1-D update; the others exit.
__global__ void __launch_bounds__(NT) k_corr_tstep(CK k, double* vec, double sub_dt, int last, int init,
                                                   const double* __restrict__ part, int nsum,
                                                   double scale, unsigned* counter) {
  const CV cv{k.P};
  const int P = k.P;
  const int nw = CV::n_win(P);
  __shared__ double red[64];
  __shared__ float wmax[2][NT / 32];
  __shared__ int fail;
  if (part != nullptr) {
    __shared__ bool is_last;
    const int l = blockIdx.x;
    double acc = 0.0;
    for (int j = threadIdx.x; j < nsum; j += blockDim.x) acc += part[(size_t)l * nsum + j];
    const double tot = block_sum(acc, red);
    if (threadIdx.x == 0) {
      vec[cv.flux() + l] = tot * scale;
      __threadfence();
      is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    if (threadIdx.x == 0) *counter = 0u;
  }
  extern __shared__ double smem[];
  double* A = smem;               // 5P FP64 band
  double* xs = smem + 5 * P;      // tb_sbp
  double* b = smem + 6 * P;
  double* sol = smem + 7 * P;
  double* res = smem + 8 * P;
  double* y = smem + 9 * P;       // s2c tb_new
  double* u = smem + 10 * P;      // tb_sbp + tb_new, then the rank-2 update
  float* rin = reinterpret_cast<float*>(smem + 11 * P);  // FP32 residual (pz index)
  float* xo = reinterpret_cast<float*>(smem + 12 * P);   // FP32 correction (pz index)
  float* fw = reinterpret_cast<float*>(smem + 13 * P);   // forward sweeps, kWinLen + 1 per window
  float* W = reinterpret_cast<float*>(smem + 15 * P + 64);  // window factors, or the global ones
  float* Wg = reinterpret_cast<float*>(vec + cv.win());
  float* Lg = reinterpret_cast<float*>(vec + cv.lu32());
  double* tbs = vec + cv.tb_sbp();
  const double* flux = vec + cv.flux();
  double* gh = vec + cv.g_half();
  double* t2 = vec + cv.tmp2();
  const int ov = k.win_ov;
  auto d1at = [&](int d, int i) { return __ldg(k.D1b + d * P + i); };
  if (init) {
    // A = I - h (identity boundary rows), B = I + h; the FP32 copy of A for
    // the factorisations sits in the not yet used b / sol / res rows
    float* Af = reinterpret_cast<float*>(b);
    const double* w2 = vec + cv.w2();
    const double c1 = 0.5 * k.mu * k.kappa * sub_dt;
    const double c2 = 0.25 * k.mu * (sub_dt * sub_dt);
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      double dl[3][3], wv[3], lb[5];  // D1 rows i-1 .. i+1, <w^2> there, L row i
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int row = i - 1 + c;
        const bool in = row >= 0 && row < P;
        wv[c] = in ? w2[row] : 0.0;
#pragma unroll
        for (int e = 0; e < 3; ++e) dl[c][e] = in ? d1at(e, row) : 0.0;
      }
#pragma unroll
      for (int d = 0; d < 5; ++d) lb[d] = __ldg(k.Lb + d * P + i);
#pragma unroll
      for (int d = 0; d < 5; ++d) {
        const int j = i + d - 2;
        double a = 0.0, bb = 0.0;
        if (j >= 0 && j < P) {
          double dmd = 0.0;  // (D1 diag(w2) D1)[i, j]
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const int kk = i - 1 + c;
            if (kk >= 0 && kk < P && abs(kk - j) <= 1) dmd = fma(dl[1][c] * wv[c], dl[c][j - kk + 1], dmd);
          }
          const double h = fma(c1, lb[d], c2 * dmd);
          const double id = (i == j) ? 1.0 : 0.0;
          a = (i == 0 || i == P - 1) ? id : id - h;
          bb = id + h;
        }
        A[d * P + i] = a;
        Af[d * P + i] = (float)a;
        vec[cv.Aband() + d * P + i] = a;
        vec[cv.Bband() + d * P + i] = bb;
      }
    }
    if (threadIdx.x == 0) vec[cv.lu_ok()] = 0.0;
    __syncthreads();
    if (ov > 0 && threadIdx.x < nw) {  // window factors, one thread each
      const int w = threadIdx.x;
      const int e0 = max(0, w * CV::kWinCore - ov), e1 = min(P, (w + 1) * CV::kWinCore + ov);
      lu32_factor(Af, P, e0, e1 - e0, W + w * CV::kWinStride, CV::kWinLen);
    }
    __syncthreads();
    if (ov > 0) copy_block(Wg, W, nw * CV::kWinStride);
  } else {
    copy_block(A, vec + cv.Aband(), 5 * P);
    if (ov > 0) copy_block(W, Wg, nw * CV::kWinStride);
  }
  copy_block(xs, tbs, P);
  if (threadIdx.x == 0) fail = (ov == 0);
  __syncthreads();
  // b = B tb_sbp - mu sub_dt D1 flux
  const double cf = k.mu * sub_dt;
  const double* Bg = vec + cv.Bband();
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double bv[5], dv[3], fv[3];
#pragma unroll
    for (int d = 0; d < 5; ++d) bv[d] = Bg[d * P + i];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int c = min(max(i - 1 + e, 0), P - 1);
      dv[e] = d1at(e, i);
      fv[e] = __ldcg(flux + c);  // written by other CTAs of this launch
    }
    double acc = 0.0;
#pragma unroll
    for (int d = 0; d < 5; ++d) {
      const int j = i + d - 2;
      if (j >= 0 && j < P) acc = fma(bv[d], xs[j], acc);
    }
    double df = 0.0;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int c = i - 1 + e;
      if (c >= 0 && c < P) df = fma(dv[e], fv[e], df);
    }
    b[i] = (i == 0 || i == P - 1) ? 0.0 : fma(-cf, df, acc);
  }
  __syncthreads();
  // refinement; M = the windows (or, after a failed check, the global LU)
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      if (!fail) break;
      // global factors: factor once per A (lu_ok), else reuse
      if (vec[cv.lu_ok()] == 0.0) {
        float* Af = reinterpret_cast<float*>(res);  // free until the sweeps start
        for (int idx = threadIdx.x; idx < 5 * P; idx += blockDim.x) Af[idx] = (float)A[idx];
        __syncthreads();
        if (threadIdx.x == 0) lu32_factor(Af, P, 0, P, W, P);
        __syncthreads();
        copy_block(Lg, W, 5 * P);
        __syncthreads();
        if (threadIdx.x == 0) vec[cv.lu_ok()] = 1.0;
      } else {
        copy_block(W, Lg, 5 * P);
      }
      __syncthreads();
    } else if (fail) {
      continue;
    }
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      sol[i] = 0.0;
      res[i] = b[i];
    }
    __syncthreads();
    for (int it = 0; it <= kRefine; ++it) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) rin[pz(i)] = (float)res[i];
      __syncthreads();
      if (pass == 0) {
        if (threadIdx.x < nw) {
          const int w = threadIdx.x;
          const int c0 = w * CV::kWinCore, c1 = min(P, c0 + CV::kWinCore);
          const int e0 = max(0, c0 - ov), e1 = min(P, c1 + ov);
          lu32_solve(W + w * CV::kWinStride, CV::kWinLen, e1 - e0,
                     [&](int ii) { return rin[pz(e0 + ii)]; }, fw + w * (CV::kWinLen + 1),
                     [&](int ii, float v) {
                       const int i = e0 + ii;
                       if (i >= c0 && i < c1) xo[pz(i)] = v;
                     });
        }
      } else if (threadIdx.x == 0) {
        lu32_solve(W, P, P, [&](int ii) { return rin[pz(ii)]; }, fw,
                   [&](int ii, float v) { xo[pz(ii)] = v; });
      }
      __syncthreads();
      const bool check = pass == 0 && it == kRefine;
      float cmax = 0.f, smax = 0.f;
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const float c = xo[pz(i)];
        const double v = sol[i] + (double)c;
        sol[i] = v;
        if (check) {
          cmax = fmaxf(cmax, fabsf(c));
          smax = fmaxf(smax, fabsf((float)v));
        }
      }
      if (check) {  // the windows converged: last correction <= 1e-10 max |sol|
        for (int o = 16; o > 0; o >>= 1) {
          cmax = fmaxf(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
          smax = fmaxf(smax, __shfl_xor_sync(0xffffffffu, smax, o));
        }
        if ((threadIdx.x & 31) == 0) {
          wmax[0][threadIdx.x >> 5] = cmax;
          wmax[1][threadIdx.x >> 5] = smax;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          float c = 0.f, sm = 0.f;
          for (int q = 0; q < NT / 32; ++q) { c = fmaxf(c, wmax[0][q]); sm = fmaxf(sm, wmax[1][q]); }
          if (!(c <= 1e-10f * sm)) fail = 1;
        }
      }
      __syncthreads();
      if (it == kRefine) break;
      for (int i = threadIdx.x; i < P; i += blockDim.x) {  // res = b - A sol in FP64
        double acc = b[i];
#pragma unroll
        for (int d = 0; d < 5; ++d) {
          const int j = i + d - 2;
          if (j >= 0 && j < P) acc = fma(-A[d * P + i], sol[j], acc);
        }
        res[i] = acc;
      }
      __syncthreads();
    }
  }
  // sol = tb_new.  u = tb_sbp + tb_new (for g_half) and y = s2c tb_new with
  // the two end values of tb_new taken as zero
  const int ew = k.ell_w;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    u[i] = xs[i] + sol[i];
    double acc = 0.0;
    for (int q = 0; q < ew; ++q) {
      const int c = __ldg(k.s2c_ecol + q * P + i);
      const double v = (c == 0 || c == P - 1) ? 0.0 : sol[c];
      acc = fma(__ldg(k.s2c_eval + q * P + i), v, acc);
    }
    y[i] = acc;
    t2[i] = acc;
  }
  __syncthreads();
  // g_half = D1 u / 2 and the rank-2 dot products F_j . y
  double a0 = 0.0, a1 = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double dv[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) dv[e] = d1at(e, i);
    const double f0 = __ldg(k.bcF + i), f1 = __ldg(k.bcF + P + i);
    double acc = 0.0;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int c = i - 1 + e;
      if (c >= 0 && c < P) acc = fma(dv[e], u[c], acc);
    }
    gh[i] = 0.5 * acc;
    a0 = fma(f0, y[i], a0);
    a1 = fma(f1, y[i], a1);
  }
  if (!last) {
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_down_sync(0xffffffffu, a0, o);
      a1 += __shfl_down_sync(0xffffffffu, a1, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = a0;
      red[32 + (threadIdx.x >> 5)] = a1;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      const int nwp = blockDim.x >> 5;
      double s0 = threadIdx.x < nwp ? red[threadIdx.x] : 0.0;
      double s1 = threadIdx.x < nwp ? red[32 + threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
      }
      __syncwarp();
      if (threadIdx.x == 0) { red[0] = s0; red[1] = s1; }
    }
    __syncthreads();
    const double e0 = red[0], e1 = red[1];
    for (int i = threadIdx.x; i < P; i += blockDim.x)
      u[i] = fma(__ldg(k.bcV + P + i), e1, fma(__ldg(k.bcV + i), e0, y[i]));
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) {  // tb_sbp = c2s u
      double acc = 0.0;
      for (int q = 0; q < ew; ++q)
        acc = fma(__ldg(k.c2s_eval + q * P + i), u[__ldg(k.c2s_ecol + q * P + i)], acc);
      tbs[i] = acc;
    }
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
int corr_mid_ctas(int M) { return (M + kSM - 1) / kSM; }

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
  cudaFuncSetAttribute(pre, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
  cudaFuncSetAttribute(k_corr_sub<cdfl, float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm4);
  cudaFuncSetAttribute(k_corr_sub<double2, double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm4);
  // the double-float path keeps w in FP32 in the wsbp buffer
  float2* wsbp_f = reinterpret_cast<float2*>(a.wsbp);
  const size_t smid = (size_t)p.d.P * kSM * sizeof(double2);
  const bool fused_mid = smid <= 200 * 1024 && t.R_col != nullptr;
  if (fused_mid) {
    cudaFuncSetAttribute(k_corr_sub_mid<double2, double2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smid);
    cudaFuncSetAttribute(k_corr_sub_mid<cdfl, float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smid);
  }
  {  // window overlap: r^ov <= 1e-7 for the decay rate r of A^-1 (two rows of margin)
    const double aa = 0.5 * k.mu * k.kappa * sub_dt * (double)p.d.Nz * (double)p.d.Nz;
    int ov = 2;
    if (aa > 0.0) {
      const double r = 2.0 * aa / ((1.0 + 2.0 * aa) + std::sqrt(1.0 + 4.0 * aa));
      ov = std::max(2, (int)std::ceil(std::log(1e-7) / std::log(r)) + 2);
    }
    k.win_ov = ov <= CV::kWinOvMax ? ov : 0;
    if (p.corr_win_ov >= 0) k.win_ov = p.corr_win_ov <= CV::kWinOvMax ? p.corr_win_ov : 0;
  }
  const size_t tsm = (size_t)kTstepSmem(p.d.P) * sizeof(double);
  cudaFuncSetAttribute(k_corr_tstep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm);
  Profiler& pf = w.prof;
  pf.begin("corr_pre", st);
  pre<<<grid, NT, sm2, st>>>(k, a.wp, a.tp, a.wcgl, a.wsbp, a.wcgl_f, wsbp_f, a.tsbp, a.tbp, w.vec);
  pf.end(st);
  pf.begin("parseval", st);
  if (df)
    launch_parseval2(p, wsbp_f, wsbp_f, a.tsbp, p.d.P, w.vec + cv.w2(), w.vec + cv.flux(), w, st, true);
  else
    launch_parseval2(p, a.wsbp, a.wsbp, a.tsbp, p.d.P, w.vec + cv.w2(), w.vec + cv.flux(), w, st, false);
  pf.end(st);
  int n = 2;
  // the double-float path takes the next substep's flux from the fused
  // substep's per-CTA sums instead of a separate Parseval pass
  const bool mid_flux = df && fused_mid && t.R_val_df && t.pwt && w.mid_part;
  const int nmid = corr_mid_ctas(p.d.M);
  const double n2 = (double)p.d.Nx * (double)p.d.Nx;
  for (int s = 0; s < nsub; ++s) {
    const int last = (s == nsub - 1);
    const bool from_mid = s > 0 && mid_flux;
    if (s > 0 && !from_mid) {
      pf.begin("parseval", st);
      if (df) launch_parseval(p, wsbp_f, a.tsbp, p.d.P, w.vec + cv.flux(), w, st, true);
      else launch_parseval(p, a.wsbp, a.tsbp, p.d.P, w.vec + cv.flux(), w, st, false);
      pf.end(st);
      ++n;
    }
    pf.begin("corr_step_1d", st);
    if (from_mid)
      k_corr_tstep<<<p.d.P, NT, tsm, st>>>(k, w.vec, sub_dt, last, 0, w.mid_part, nmid, 1.0 / (n2 * n2),
                                             w.counters + p.d.P);
    else
      k_corr_tstep<<<1, NT, tsm, st>>>(k, w.vec, sub_dt, last, s == 0, nullptr, 0, 0.0, nullptr);
    pf.end(st);
    if (!last && fused_mid && (!df || t.R_val_df)) {
      pf.begin("corr_sub_mid", st);
      if (df) {
        SubK<dfl> sk{p.d.P, p.d.M, t.R_w, t.R_col, t.R_val_df, t.Fs_df, t.Us_df, w.vec + cv.g_half(),
                     dfl(sub_dt)};
        k_corr_sub_mid<cdfl, float2><<<nmid, kSubThreads, smid, st>>>(sk, a.tsbp, wsbp_f,
                                                                      mid_flux ? w.mid_part : nullptr, t.pwt);
      } else {
        SubK<double> sk{p.d.P, p.d.M, t.R_w, t.R_col, t.R_val, t.Fs, t.Us, w.vec + cv.g_half(), sub_dt};
        k_corr_sub_mid<double2, double2><<<nmid, kSubThreads, smid, st>>>(sk, a.tsbp, a.wsbp, nullptr, nullptr);
      }
      pf.end(st);
    } else {
      pf.begin(last ? "corr_sub_last" : "corr_sub", st);
      if (df)
        k_corr_sub<cdfl, float2><<<grid, NT, sm4, st>>>(k, a.tsbp, wsbp_f, w.vec + cv.g_half(), sub_dt, last,
                                                        a.t_out, a.tcgl_f, w.vec + cv.tmp2(), a.tb_out);
      else
        k_corr_sub<double2, double2><<<grid, NT, sm4, st>>>(k, a.tsbp, a.wsbp, w.vec + cv.g_half(), sub_dt,
                                                            last, a.t_out, a.tcgl, w.vec + cv.tmp2(), a.tb_out);
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
  k_corr_pre<double2><<<(p.d.M + TM - 1) / TM, NT, sm2, st>>>(k, w, th, wcgl, wsbp, nullptr, nullptr, tsbp,
                                                               nullptr, nullptr);
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

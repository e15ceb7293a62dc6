// Column-tile helpers shared by the vertical kernels (FP64).
//
// A CTA owns TM consecutive compact modes and holds their vertical columns in
// shared memory as tiles [level][TM].  The Chebyshev <-> CGL transforms
// V[j,n] = cos(pi j n / N) (nhqg/grid.py:192-201) run as a DCT-I through a
// complex FFT of length 2N of the even extension:
//   (V c)_j = ( DFT_2N(e)_j + c_0 + (-1)^j c_N ) / 2,  e = (c_0..c_N, c_{N-1}..c_1),
// and V^-1 = (2/N) diag(1/w) V diag(1/w), w = (2, 1, .., 1, 2).  That is
// ~5 (2N) log2(2N) flops per complex column instead of 4 (N+1)^2 for the
// dense product; lengths whose 2N is not 2^a 3^b use the dense matrix.
#pragma once
#include "common.cuh"
#include "fft.cuh"

namespace nhqg {
namespace col {

constexpr int TM = 4;    // modes per CTA
constexpr int NT = 256;  // threads per CTA

struct Dct {
  int N, P;
  bool fast;
  FftPlan plan;               // length 2N
  const double2* tw;          // [2N] global
  const int* perm;            // [2N] global
  const double *V, *Vinv;     // dense fallback [P*P]
};

// shared-memory words (double2) the DCT needs: work [TM][2N] + twiddles + perm
__host__ __device__ inline int dct_smem_elems(const Dct& d) {
  return d.fast ? (TM * 2 * d.N + 2 * d.N + (2 * d.N + 1) / 2) : 0;
}

__device__ __forceinline__ void tload(double2* b, const double2* __restrict__ src, int nlev,
                                      int m0, int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    b[i] = (m < M) ? src[(size_t)l * M + m] : czero();
  }
}
__device__ __forceinline__ void tstore(const double2* b, double2* __restrict__ dst, int nlev,
                                       int m0, int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    if (m < M) dst[(size_t)l * M + m] = b[i];
  }
}
// out[i] = sum_{j<nin} Mat[i*ld + j] in[j], i < nout
__device__ __forceinline__ void tmat(double2* out, const double2* in, const double* __restrict__ Mat,
                                     int ld, int nout, int nin) {
  for (int idx = threadIdx.x; idx < nout * TM; idx += blockDim.x) {
    const int i = idx / TM, mm = idx - i * TM;
    const double* row = Mat + (size_t)i * ld;
    double ax = 0.0, ay = 0.0;
    for (int j = 0; j < nin; ++j) {
      const double v = __ldg(row + j);
      const double2 x = in[j * TM + mm];
      ax = fma(v, x.x, ax);
      ay = fma(v, x.y, ay);
    }
    out[idx] = make_double2(ax, ay);
  }
}
__device__ __forceinline__ void tcsr(double2* out, const double2* in, const int* __restrict__ ptr,
                                     const int* __restrict__ colidx, const double* __restrict__ val,
                                     int nrow) {
  for (int idx = threadIdx.x; idx < nrow * TM; idx += blockDim.x) {
    const int i = idx / TM, mm = idx - i * TM;
    double ax = 0.0, ay = 0.0;
    for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
      const double v = val[q];
      const double2 x = in[colidx[q] * TM + mm];
      ax = fma(v, x.x, ax);
      ay = fma(v, x.y, ay);
    }
    out[idx] = make_double2(ax, ay);
  }
}
// Dirichlet stencil c_n = -x_n + x_{n-2} (x: G = N-1 entries; c: P)
__device__ __forceinline__ void tstencil_dir(double2* c, const double2* x, int P, int G) {
  for (int idx = threadIdx.x; idx < P * TM; idx += blockDim.x) {
    const int n = idx / TM, mm = idx - n * TM;
    double2 v = (n < G) ? cneg(x[n * TM + mm]) : czero();
    if (n >= 2 && n - 2 < G) v = cadd(v, x[(n - 2) * TM + mm]);
    c[idx] = v;
  }
}
// open-top basis T_n + a_n T_{n+1} + b_n T_{n+2}
__device__ __forceinline__ void tstencil_mixed(double2* c, const double2* x, int P, int G,
                                               const double* __restrict__ wa,
                                               const double* __restrict__ wb) {
  for (int idx = threadIdx.x; idx < P * TM; idx += blockDim.x) {
    const int n = idx / TM, mm = idx - n * TM;
    double2 v = (n < G) ? x[n * TM + mm] : czero();
    if (n >= 1 && n - 1 < G) v = caxpy(__ldg(wa + n - 1), x[(n - 1) * TM + mm], v);
    if (n >= 2 && n - 2 < G) v = caxpy(__ldg(wb + n - 2), x[(n - 2) * TM + mm], v);
    c[idx] = v;
  }
}
// exact left inverse of the Dirichlet stencil: x_n = x_{n-2} - c_n, n < G
__device__ __forceinline__ void tpinv_dir(double2* x, const double2* c, int G) {
  const int t = threadIdx.x;
  if (t < 2 * TM) {
    const int mm = t >> 1;
    const bool im = t & 1;
    double xm2 = 0.0, xm1 = 0.0;
    for (int n = 0; n < G; ++n) {
      const double cv = im ? c[n * TM + mm].y : c[n * TM + mm].x;
      const double xn = xm2 - cv;
      if (im) x[n * TM + mm].y = xn; else x[n * TM + mm].x = xn;
      xm2 = xm1;
      xm1 = xn;
    }
  }
}
// exact left inverse of the open-top stencil: x_n = c_n - a_{n-1} x_{n-1} - b_{n-2} x_{n-2}
__device__ __forceinline__ void tpinv_mixed(double2* x, const double2* c, int G,
                                            const double* __restrict__ wa,
                                            const double* __restrict__ wb) {
  const int t = threadIdx.x;
  if (t < 2 * TM) {
    const int mm = t >> 1;
    const bool im = t & 1;
    double xm2 = 0.0, xm1 = 0.0;
    for (int n = 0; n < G; ++n) {
      double v = im ? c[n * TM + mm].y : c[n * TM + mm].x;
      if (n >= 1) v = fma(-__ldg(wa + n - 1), xm1, v);
      if (n >= 2) v = fma(-__ldg(wb + n - 2), xm2, v);
      if (im) x[n * TM + mm].y = v; else x[n * TM + mm].x = v;
      xm2 = xm1;
      xm1 = v;
    }
  }
}
// d/dZ on Chebyshev coefficients, G_Z = 2 G_xi: b_{N-1} = 4N a_N,
// b_k = b_{k+2} + 4(k+1) a_{k+1}, b_0 = b_2/2 + 2 a_1 (nhqg/grid.py:148-169)
__device__ __forceinline__ void tgz(double2* b, const double2* a, int N) {
  const int t = threadIdx.x;
  if (t < 2 * TM) {
    const int mm = t >> 1;
    const bool im = t & 1;
    auto A = [&](int n) { return im ? a[n * TM + mm].y : a[n * TM + mm].x; };
    auto S = [&](int n, double v) { if (im) b[n * TM + mm].y = v; else b[n * TM + mm].x = v; };
    S(N, 0.0);
    double bk2 = 0.0;
    double bk1 = 4.0 * N * A(N);
    S(N - 1, bk1);
    for (int kk = N - 2; kk >= 1; --kk) {
      const double bk = fma(4.0 * (kk + 1), A(kk + 1), bk2);
      S(kk, bk);
      bk2 = bk1;
      bk1 = bk;
    }
    S(0, fma(0.5, bk2, 2.0 * A(1)));
  }
}

// Load the DCT twiddle / permutation tables into shared memory.
struct DctShared {
  double2* work;
  double2* tw;
  int* perm;
};
__device__ __forceinline__ DctShared dct_shared(const Dct& d, double2* base) {
  DctShared s;
  s.work = base;
  s.tw = base + TM * 2 * d.N;
  s.perm = reinterpret_cast<int*>(s.tw + 2 * d.N);
  if (d.fast) {
    for (int i = threadIdx.x; i < 2 * d.N; i += blockDim.x) {
      s.tw[i] = d.tw[i];
      s.perm[i] = d.perm[i];
    }
  }
  return s;
}

// out[0:nout] = V in (inverse == false) or V^-1 in (inverse == true), per column.
// Caller syncs before (in ready) and after (out ready).  out != in.
__device__ __forceinline__ void tdct(double2* out, const double2* in, const Dct& d,
                                     const DctShared& s, bool inverse, int nout) {
  const int N = d.N;
  if (!d.fast) {
    tmat(out, in, inverse ? d.Vinv : d.V, d.P, nout, d.P);
    return;
  }
  const int L = 2 * N;
  for (int idx = threadIdx.x; idx < TM * L; idx += blockDim.x) {
    const int mm = idx / L, n = idx - mm * L;
    const int src = n <= N ? n : L - n;
    double2 v = in[src * TM + mm];
    if (inverse && (src == 0 || src == N)) v = cscale(v, 0.5);
    s.work[idx] = v;
  }
  __syncthreads();
  fft_dif_fwd(s.work, TM, L, d.plan, s.tw);
  const double sc = inverse ? (1.0 / N) : 0.5;  // (2/N)/2 after the 1/2 of the DCT-I identity
  for (int idx = threadIdx.x; idx < nout * TM; idx += blockDim.x) {
    const int j = idx / TM, mm = idx - j * TM;
    const double2 Y = s.work[mm * L + s.perm[j]];
    double2 c0 = in[mm], cN = in[N * TM + mm];
    if (inverse) { c0 = cscale(c0, 0.5); cN = cscale(cN, 0.5); }
    double2 y = cadd(Y, c0);
    y = (j & 1) ? csub(y, cN) : cadd(y, cN);
    double f = sc;
    if (inverse && (j == 0 || j == N)) f *= 0.5;
    out[idx] = cscale(y, f);
  }
}

}  // namespace col
}  // namespace nhqg

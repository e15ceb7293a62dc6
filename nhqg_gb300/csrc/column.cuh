// Column-tile helpers shared by the vertical kernels.
//
// A CTA owns TM consecutive compact modes and holds their vertical columns in
// shared memory as tiles [level][TM].  The Chebyshev <-> CGL transforms
// V[j,n] = cos(pi j n / N) (nhqg/grid.py:192-201) run as a DCT-I through one
// complex FFT of length N per complex column (N even, 2^a 3^b):
//   z_j = (c_j + c_{N-j}) / 2 - sin(pi j / N) (c_j - c_{N-j}),   Z = FFT_N(z),
//   (V c)_{2k}   = (Z_k + Z_{N-k}) / 2 + (c_0 + c_N) / 2,
//   (V c)_{2k+1} = F_1 - sum_{m=1..k} D_m + (c_0 - c_N) / 2,
//   D_m = -i (Z_m - Z_{N-m}) / 2,  F_1 = (c_0 - c_N) / 2 + sum_{j=1..N-1} c_j cos(pi j / N)
// (the real-input DCT-I through a half-length FFT, Press et al., Numerical
// Recipes, "cosft1", with the real and imaginary parts of the column carried
// together: every step is real-linear), and V^-1 = (2/N) diag(1/w) V
// diag(1/w), w = (2, 1, .., 1, 2).  That is ~5 N log2 N flops per complex
// column instead of 4 (N+1)^2 for the dense product; other lengths use the
// dense matrix.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "df64.cuh"
#include "fft.cuh"

namespace nhqg {
namespace col {

// modes per CTA: 2 keeps five FP64 tiles of a 257-level column at 41 KB, so
// five CTAs share an SM (4 modes: 82 KB, 2 CTAs, 3% slower mixed step;
// 1 mode: 2% slower)
constexpr int TM = 2;
constexpr int NT = 256;  // threads per CTA

struct Dct {
  int N, P;
  bool fast;
  FftPlan plan;               // length N
  const double2* tw;          // [N] FFT twiddles exp(-2 pi i k / N)
  const float2* tw_f;         // [N] FP32 copy (mixed-precision path)
  const double2* cs;          // [N+1] exp(-i pi j / N) = cos - i sin
  const float2* cs_f;         // [N+1] FP32 copy
  const cdfl* tw_df;          // [N] double-float copies (mixed-precision corrector)
  const cdfl* cs_df;          // [N+1]
  const int* perm;            // [N] position of frequency k in the FFT output
  const double *V, *Vinv;     // dense fallback [P*P]
};

// FFT sequences of the DCT work area carry one padding element every 2^PS
// (fft_pad) where the transform is bound by its shared-memory passes: the
// double-float and FP32 tiles (PS = 2 and 3 for 16- and 8-byte values spread
// the short-span radix-4 passes over the banks); the FP64 tiles, bound by the
// FP64 pipe, stay dense.
template <typename C> __host__ __device__ constexpr int dct_ps() {
  return sizeof(C) == sizeof(float2) ? 3 : (std::is_same<C, double2>::value ? 0 : 2);
}
// stride of one work sequence
template <typename C> __host__ __device__ inline int dct_sx(int N) {
  return dct_ps<C>() > 0 ? N + (N >> dct_ps<C>()) + 1 : N;
}

// shared memory of the fast DCT in units of the complex type C: work
// [TM][sx], FFT twiddles [N], cos/sin table [N+1], permutation [N] ints
template <typename C>
__host__ __device__ inline size_t dct_smem_bytes_t(const Dct& d) {
  if (!d.fast) return 0;
  const size_t n = (size_t)TM * dct_sx<C>(d.N) + d.N + d.N + 1;
  const size_t c = (n * sizeof(C) + 15) / 16 * 16;
  return c + ((size_t)d.N * sizeof(int) + 15) / 16 * 16;
}
// bytes for the FP32 tiles (f32) or the larger of the FP64 and double-float ones
__host__ __device__ inline size_t dct_smem_bytes(const Dct& d, bool f32 = false) {
  if (f32) return dct_smem_bytes_t<float2>(d);
  const size_t a = dct_smem_bytes_t<double2>(d), b = dct_smem_bytes_t<cdfl>(d);
  return a > b ? a : b;
}

// Arithmetic of a tile type: double2 (FP64) or cdfl (double-float, the
// mixed-precision corrector).  s() converts an FP64 table value, in() / out()
// convert FP64 field values on the way into and out of a tile.
template <typename C> struct Prec;
template <> struct Prec<double2> {
  using T = double;
  static __device__ __forceinline__ double s(double v) { return v; }
  static __device__ __forceinline__ double i(int v) { return (double)v; }
  static __device__ __forceinline__ double2 in(double2 v) { return v; }
  static __device__ __forceinline__ double2 in(float2 v) { return make_double2((double)v.x, (double)v.y); }
  static __device__ __forceinline__ double2 out(double2 v) { return v; }
};
template <> struct Prec<cdfl> {
  using T = dfl;
  static __device__ __forceinline__ dfl s(double v) { return df_from_double(v); }
  static __device__ __forceinline__ dfl i(int v) { return dfl((float)v, 0.f); }  // |v| < 2^24
  static __device__ __forceinline__ cdfl in(double2 v) { return cdf_from(v); }
  static __device__ __forceinline__ cdfl in(float2 v) { return cdfl{dfl(v.x, 0.f), dfl(v.y, 0.f)}; }
  static __device__ __forceinline__ double2 out(cdfl v) { return cdf_to(v); }
};
// FP32 tiles (the mixed-precision corrector's w, which enters it only
// through the sub_dt-scaled exchange increment and the FP32 products).  The
// FP64 <-> FP32 conversions go through the integer split of df64.cuh (the
// two-float sum rounded once in FP32) instead of the FP64 pipe.
template <> struct Prec<float2> {
  using T = float;
  static __device__ __forceinline__ float s(double v) {
    const dfl d = df_from_double(v);
    return __fadd_rn(d.hi, d.lo);
  }
  static __device__ __forceinline__ float i(int v) { return (float)v; }
  static __device__ __forceinline__ float2 in(double2 v) { return make_float2(s(v.x), s(v.y)); }
  static __device__ __forceinline__ float2 in(float2 v) { return v; }
  static __device__ __forceinline__ double2 out(float2 v) { return make_double2(f2d_bits(v.x), f2d_bits(v.y)); }
};
template <typename C> __device__ __forceinline__ C gzero() {
  using T = typename Prec<C>::T;
  return gmk<C>(T(0), T(0));
}
template <typename C> __device__ __forceinline__ C gneg(C a) { return gmk<C>(-a.x, -a.y); }
template <typename C, typename T> __device__ __forceinline__ C gaxpy(T s, C a, C acc) {
  return gmk<C>(fma(s, a.x, acc.x), fma(s, a.y, acc.y));
}
// L2 prefetch of a CTA's columns (modes m0 .. m0 + TM - 1) of a [nlev][M]
// field of esize-byte values: one instruction per level, issued a phase ahead
// of the tile load so that the load finds L2 instead of waiting on DRAM
__device__ __forceinline__ void tprefetch(const void* f, int nlev, int m0, int M, size_t esize) {
  if (f == nullptr) return;
  const char* base = static_cast<const char*>(f) + (size_t)m0 * esize;
  for (int l = threadIdx.x; l < nlev; l += blockDim.x)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)l * M * esize));
}
// FP64 field columns <-> tiles of type C
template <typename C>
__device__ __forceinline__ void tloadp(C* b, const double2* __restrict__ src, int nlev, int m0, int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    b[i] = (m < M) ? Prec<C>::in(src[(size_t)l * M + m]) : gzero<C>();
  }
}
template <typename C>
__device__ __forceinline__ void tloadp(C* b, const float2* __restrict__ src, int nlev, int m0, int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    b[i] = (m < M) ? Prec<C>::in(src[(size_t)l * M + m]) : gzero<C>();
  }
}
template <typename C>
__device__ __forceinline__ void tstorep(const C* b, double2* __restrict__ dst, int nlev, int m0, int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    if (m < M) dst[(size_t)l * M + m] = Prec<C>::out(b[i]);
  }
}

// double-float tiles rounded to an FP32 field
__device__ __forceinline__ void tstorep(const cdfl* b, float2* __restrict__ dst, int nlev, int m0, int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    if (m < M) dst[(size_t)l * M + m] = make_float2(__fadd_rn(b[i].x.hi, b[i].x.lo), __fadd_rn(b[i].y.hi, b[i].y.lo));
  }
}
// FP32 tiles straight to an FP32 field
__device__ __forceinline__ void tstorep(const float2* b, float2* __restrict__ dst, int nlev, int m0, int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    if (m < M) dst[(size_t)l * M + m] = b[i];
  }
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
// FP32 tiles of the mixed-precision path: load / store float2 columns and
// convert between the FP64 and FP32 tiles
__device__ __forceinline__ void tload(float2* b, const float2* __restrict__ src, int nlev, int m0,
                                      int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    b[i] = (m < M) ? src[(size_t)l * M + m] : make_float2(0.f, 0.f);
  }
}
__device__ __forceinline__ void tstore(const float2* b, float2* __restrict__ dst, int nlev, int m0,
                                       int M) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x) {
    const int l = i / TM, mm = i - l * TM, m = m0 + mm;
    if (m < M) dst[(size_t)l * M + m] = b[i];
  }
}
__device__ __forceinline__ void tcvt(float2* f, const double2* b, int nlev) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x)
    f[i] = make_float2((float)b[i].x, (float)b[i].y);
}
__device__ __forceinline__ void tcvt(double2* b, const float2* f, int nlev) {
  for (int i = threadIdx.x; i < nlev * TM; i += blockDim.x)
    b[i] = make_double2((double)f[i].x, (double)f[i].y);
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
template <typename C>
__device__ __forceinline__ void tcsr(C* out, const C* in, const int* __restrict__ ptr,
                                     const int* __restrict__ colidx, const double* __restrict__ val,
                                     int nrow) {
  using T = typename Prec<C>::T;
  for (int idx = threadIdx.x; idx < nrow * TM; idx += blockDim.x) {
    const int i = idx / TM, mm = idx - i * TM;
    T ax = T(0), ay = T(0);
    for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
      const T v = Prec<C>::s(val[q]);
      const C x = in[colidx[q] * TM + mm];
      ax = fma(v, x.x, ax);
      ay = fma(v, x.y, ay);
    }
    out[idx] = gmk<C>(ax, ay);
  }
}
// Dirichlet stencil c_n = -x_n + x_{n-2} (x: G = N-1 entries; c: P)
template <typename C>
__device__ __forceinline__ void tstencil_dir(C* c, const C* x, int P, int G) {
  for (int idx = threadIdx.x; idx < P * TM; idx += blockDim.x) {
    const int n = idx / TM, mm = idx - n * TM;
    C v = (n < G) ? gneg(x[n * TM + mm]) : gzero<C>();
    if (n >= 2 && n - 2 < G) v = gadd(v, x[(n - 2) * TM + mm]);
    c[idx] = v;
  }
}
// open-top basis T_n + a_n T_{n+1} + b_n T_{n+2}
template <typename C>
__device__ __forceinline__ void tstencil_mixed(C* c, const C* x, int P, int G,
                                               const double* __restrict__ wa,
                                               const double* __restrict__ wb) {
  for (int idx = threadIdx.x; idx < P * TM; idx += blockDim.x) {
    const int n = idx / TM, mm = idx - n * TM;
    C v = (n < G) ? x[n * TM + mm] : gzero<C>();
    if (n >= 1 && n - 1 < G) v = gaxpy(Prec<C>::s(__ldg(wa + n - 1)), x[(n - 1) * TM + mm], v);
    if (n >= 2 && n - 2 < G) v = gaxpy(Prec<C>::s(__ldg(wb + n - 2)), x[(n - 2) * TM + mm], v);
    c[idx] = v;
  }
}
// Inclusive sums along one parity class of a strided column, one warp per
// (mode, re/im) column; lanes 0-15 take even indices, lanes 16-31 odd ones.
// get(n) reads element n (0 <= n < len), put(n, v) writes result n.  With
// reverse = true the sums run from the top index down (suffix sums).
template <typename Get, typename Put>
__device__ __forceinline__ void warp_parity_scan(int len, bool reverse, Get get, Put put) {
  using T = decltype(get(0));
  const int lane = threadIdx.x & 31;
  const int cls = lane >> 4;               // parity class
  const int sl = lane & 15;                // lane within the class
  const int m = (len - cls + 1) / 2;       // elements in this class
  const int chunk = (m + 15) / 16;
  const int j0 = sl * chunk;
  const int j1 = min(m, j0 + chunk);
  const int top = len - 1 - ((len - 1 - cls) & 1);  // highest index of this class
  auto idx = [&](int j) { return reverse ? top - 2 * j : 2 * j + cls; };
  T run = T(0);
  for (int j = j0; j < j1; ++j) run += get(idx(j));
  // inclusive scan of the 16 chunk totals within each half-warp
  T incl = run;
  for (int o = 1; o < 16; o <<= 1) {
    const T t = __shfl_up_sync(0xffffffffu, incl, o, 16);
    if (sl >= o) incl += t;
  }
  T acc = incl - run;                      // exclusive offset of this chunk
  for (int j = j0; j < j1; ++j) {
    const int n = idx(j);
    acc += get(n);
    put(n, acc);
  }
}

// Inclusive sums along the two parity classes of every (mode, re/im) column
// of a tile, run by the whole CTA (blockDim.x == NT, called by every thread;
// callers synchronise before and after).  Element n < len of mode mm is
// get(n, mm) (a complex C); put(n, mm, v) receives
//   v = sum of get(m, mm) over m = n (mod 2), m <= n      (reverse = false)
//   v = sum of get(m, mm) over m = n (mod 2), m >= n      (reverse = true).
// Thread t takes level t + NT r of round r and all TM modes, so the tile is
// read and written row by row (no shared-memory bank conflicts, where a
// level-strided walk down one column hits one bank); the class scan of a
// warp runs on shuffles at even offsets, warp totals and the running carry
// go through shared memory.
template <typename C, typename Get, typename Put>
__device__ __forceinline__ void tscan(int len, bool reverse, Get get, Put put) {
  constexpr int NW = NT / 32;
  __shared__ double2 red_raw[NW][2][TM];   // warp totals per position class
  __shared__ double2 pref_raw[NW][2][TM];  // exclusive prefix of the warp totals (+ carry)
  __shared__ double2 carry_raw[2][TM];     // totals of the previous rounds
  C (*red)[2][TM] = reinterpret_cast<C (*)[2][TM]>(red_raw);
  C (*pref)[2][TM] = reinterpret_cast<C (*)[2][TM]>(pref_raw);
  C (*carry)[TM] = reinterpret_cast<C (*)[TM]>(carry_raw);
  static_assert(sizeof(C) == sizeof(double2), "16-byte complex tiles");
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t < 2 * TM) carry[t / TM][t % TM] = gzero<C>();
  for (int r0 = 0; r0 < len; r0 += NT) {
    const int pos = r0 + t;                        // position along the scan
    const int n = reverse ? len - 1 - pos : pos;   // level
    const bool in = pos < len;
    // warps of this round that hold at least one position (the others would
    // only add zeros: they skip the shuffles and post zero totals)
    const int nwa = min(NW, (len - r0 + 31) >> 5);
    C v[TM];
#pragma unroll
    for (int mm = 0; mm < TM; ++mm) v[mm] = in ? get(n, mm) : gzero<C>();
    // class scan within the warp: positions of one class are 2 apart
    if (warp < nwa) {
#pragma unroll
      for (int o = 2; o < 32; o <<= 1) {
#pragma unroll
        for (int mm = 0; mm < TM; ++mm) {
          C u;
          u.x = __shfl_up_sync(0xffffffffu, v[mm].x, o);
          u.y = __shfl_up_sync(0xffffffffu, v[mm].y, o);
          if (lane >= o) v[mm] = gadd(v[mm], u);
        }
      }
    }
    // lanes 30 and 31 hold the warp's totals of the two position classes
    if (lane >= 30) {
#pragma unroll
      for (int mm = 0; mm < TM; ++mm) red[warp][lane & 1][mm] = v[mm];
    }
    __syncthreads();
    if (t < 2 * TM) {  // exclusive prefix over the warps, and the carry into the next round
      const int c = t / TM, mm = t % TM;
      C acc = carry[c][mm];
      if (nwa == NW) {  // every warp holds positions: unrolled
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          pref[w][c][mm] = acc;
          acc = gadd(acc, red[w][c][mm]);
        }
      } else {  // a short column or the last round: the warps that hold positions
        for (int w = 0; w < nwa; ++w) {
          pref[w][c][mm] = acc;
          acc = gadd(acc, red[w][c][mm]);
        }
      }
      carry[c][mm] = acc;
    }
    __syncthreads();
    // position class of this thread (pos parity; r0 is a multiple of NT, even)
    const int pc = pos & 1;
    if (in) {
#pragma unroll
      for (int mm = 0; mm < TM; ++mm) put(n, mm, gadd(pref[warp][pc][mm], v[mm]));
    }
    if (r0 + NT < len) __syncthreads();  // red / pref are rewritten by the next round
  }
}

// exact left inverse of the Dirichlet stencil: x_n = x_{n-2} - c_n, i.e.
// x_n = -(sum of c_i over i <= n, i = n mod 2), n < G.  All threads.
template <typename C>
__device__ __forceinline__ void tpinv_dir(C* x, const C* c, int G) {
  tscan<C>(G, false, [&](int n, int mm) { return gneg(c[n * TM + mm]); },
           [&](int n, int mm, C v) { x[n * TM + mm] = v; });
}

// exact left inverse of the open-top stencil: x_n = c_n - a_{n-1} x_{n-1} - b_{n-2} x_{n-2}
template <typename C>
__device__ __forceinline__ void tpinv_mixed(C* x, const C* c, int G,
                                            const double* __restrict__ wa,
                                            const double* __restrict__ wb) {
  using T = typename Prec<C>::T;
  const int t = threadIdx.x;
  if (t < 2 * TM) {
    const int mm = t >> 1;
    const bool im = t & 1;
    T xm2 = T(0), xm1 = T(0);
    for (int n = 0; n < G; ++n) {
      T v = im ? c[n * TM + mm].y : c[n * TM + mm].x;
      if (n >= 1) v = fma(Prec<C>::s(-__ldg(wa + n - 1)), xm1, v);
      if (n >= 2) v = fma(Prec<C>::s(-__ldg(wb + n - 2)), xm2, v);
      if (im) x[n * TM + mm].y = v; else x[n * TM + mm].x = v;
      xm2 = xm1;
      xm1 = v;
    }
  }
}
// d/dZ on Chebyshev coefficients, G_Z = 2 G_xi (nhqg/grid.py:148-169):
// b_k = sum_{j > k, j - k odd} 4 j a_j for 1 <= k <= N-1, b_N = 0,
// b_0 = b_2 / 2 + 2 a_1 -- suffix sums over a parity class.  All threads.
template <typename C>
__device__ __forceinline__ void tgz(C* b, const C* a, int N) {
  using T = typename Prec<C>::T;
  // t_j = 4 j a_j for j = 1..N, summed from the top over j's class:
  // U_j = sum_{i >= j, i = j mod 2} t_i, stored as b_{j-1} (n = j - 1 in [1, N-1])
  tscan<C>(N, true, [&](int n, int mm) { return gscale(a[(n + 1) * TM + mm], Prec<C>::i(4 * (n + 1))); },
           [&](int n, int mm, C v) { if (n >= 1) b[n * TM + mm] = v; });
  __syncthreads();  // b_2 comes from another thread
  if (threadIdx.x < TM) {
    const int mm = threadIdx.x;
    b[N * TM + mm] = gzero<C>();
    const C b2 = N >= 2 ? b[2 * TM + mm] : gzero<C>();
    const C a1 = a[TM + mm];
    b[mm] = gmk<C>(fma(T(0.5), b2.x, T(2.0) * a1.x), fma(T(0.5), b2.y, T(2.0) * a1.y));
  }
}

// Load the DCT twiddle / permutation tables into shared memory.
template <typename C>
struct DctSharedT {
  C* work;
  C* tw;
  C* cs;
  int* perm;
};
using DctShared = DctSharedT<double2>;

template <typename C>
__device__ __forceinline__ const C* dct_tw(const Dct& d);
template <> __device__ __forceinline__ const double2* dct_tw<double2>(const Dct& d) { return d.tw; }
template <> __device__ __forceinline__ const float2* dct_tw<float2>(const Dct& d) { return d.tw_f; }
template <> __device__ __forceinline__ const cdfl* dct_tw<cdfl>(const Dct& d) { return d.tw_df; }
template <typename C>
__device__ __forceinline__ const C* dct_cs(const Dct& d);
template <> __device__ __forceinline__ const double2* dct_cs<double2>(const Dct& d) { return d.cs; }
template <> __device__ __forceinline__ const float2* dct_cs<float2>(const Dct& d) { return d.cs_f; }
template <> __device__ __forceinline__ const cdfl* dct_cs<cdfl>(const Dct& d) { return d.cs_df; }

template <typename C = double2>
__device__ __forceinline__ DctSharedT<C> dct_shared(const Dct& d, void* base) {
  DctSharedT<C> s;
  s.work = reinterpret_cast<C*>(base);
  s.tw = s.work + TM * dct_sx<C>(d.N);
  s.cs = s.tw + d.N;
  const size_t cbytes = ((size_t)(TM * dct_sx<C>(d.N) + d.N + d.N + 1) * sizeof(C) + 15) / 16 * 16;
  s.perm = reinterpret_cast<int*>(reinterpret_cast<char*>(base) + cbytes);
  if (d.fast) {
    const C* tw = dct_tw<C>(d);
    const C* cs = dct_cs<C>(d);
    for (int i = threadIdx.x; i <= d.N; i += blockDim.x) {
      if (i < d.N) {
        s.tw[i] = tw[i];
        s.perm[i] = d.perm[i];
      }
      s.cs[i] = cs[i];
    }
  }
  return s;
}

// out[0:nout] = V in (inverse == false) or V^-1 in (inverse == true), per column,
// in the precision of C.  Caller syncs before (in ready) and after (out
// ready).  out != in.  The FP32 and double-float instantiations require d.fast.  Needs 2 TM
// warps (the odd outputs are a prefix sum per (mode, re/im) column).
template <typename C>
__device__ __forceinline__ void tdct(C* out, const C* in, const Dct& d, const DctSharedT<C>& s,
                                     bool inverse, int nout) {
  using T = decltype(C().x);
  const int N = d.N;
  if constexpr (std::is_same<T, double>::value) {
    if (!d.fast) {
      tmat(out, in, inverse ? d.Vinv : d.V, d.P, nout, d.P);
      return;
    }
  }
  const T half = T(0.5);
  // input with the inverse's endpoint halving: c_n = in_n (x 1/2 at n = 0, N)
  auto cin = [&](int n, int mm) {
    C v = in[n * TM + mm];
    if (inverse && (n == 0 || n == N)) v = gscale(v, half);
    return v;
  };
  constexpr int PS = dct_ps<C>();
  const int SX = dct_sx<C>(N);
  auto W = [&](int mm, int pos) -> C& { return s.work[mm * SX + fft_pad<PS>(pos)]; };
  for (int idx = threadIdx.x; idx < TM * N; idx += blockDim.x) {
    const int mm = idx / N, j = idx - mm * N;
    const C cj = cin(j, mm), cr = cin(N - j, mm);
    const T sn = -s.cs[j].y;  // sin(pi j / N)
    const C sum = gadd(cj, cr), dif = gsub(cj, cr);
    W(mm, j) = gmk<C>(fma(half, sum.x, -sn * dif.x), fma(half, sum.y, -sn * dif.y));
  }
  __syncthreads();
  fft_dif_fwd<C, PS>(s.work, TM, SX, d.plan, s.tw);
  const T sc = inverse ? T(2.0 / N) : T(1);
  // even outputs j = 2k
  for (int idx = threadIdx.x; idx < TM * (N / 2 + 1); idx += blockDim.x) {
    const int k = idx / TM, mm = idx - k * TM;
    const int j = 2 * k;
    if (j >= nout) continue;
    const C Zk = W(mm, s.perm[k % N]);
    const C Zm = W(mm, s.perm[(N - k) % N]);
    const C c0 = cin(0, mm), cN = cin(N, mm);
    C y = gscale(gadd(gadd(Zk, Zm), gadd(c0, cN)), half);
    T f = sc;
    if (inverse && (j == 0 || j == N)) f *= half;
    out[j * TM + mm] = gscale(y, f);
  }
  // odd outputs j = 2k+1: one warp per (mode, re/im) column
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w < 2 * TM) {
    const int mm = w >> 1;
    const bool im = w & 1;
    auto part = [&](const C& v) { return im ? v.y : v.x; };
    const T c0 = part(cin(0, mm)), cN = part(cin(N, mm));
    // F_1 = (c_0 - c_N)/2 + sum_j c_j cos(pi j / N)
    T f1 = T(0);
    for (int j = 1 + lane; j < N; j += 32) f1 = fma(part(in[j * TM + mm]), s.cs[j].x, f1);
    for (int o = 16; o > 0; o >>= 1) f1 += __shfl_xor_sync(0xffffffffu, f1, o);
    f1 = fma(half, c0 - cN, f1);
    // D_m (m = 1 .. N/2-1), re part = Im(Z_m - Z_{N-m})/2, im part = -Re(Z_m - Z_{N-m})/2
    auto dm = [&](int m) {
      const C a = W(mm, s.perm[m]), b = W(mm, s.perm[N - m]);
      return im ? half * (b.x - a.x) : half * (a.y - b.y);
    };
    const int len = N / 2 - 1;
    const int chunk = (len + 31) / 32;
    const int m0 = 1 + lane * chunk, m1 = min(len + 1, m0 + chunk);
    T run = T(0);
    for (int m = m0; m < m1; ++m) run += dm(m);
    T incl = run;
    for (int o = 1; o < 32; o <<= 1) {
      const T t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    T acc = incl - run;
    const T tail = half * (c0 - cN);
    auto put = [&](int k, T F) {
      const int j = 2 * k + 1;
      if (j < nout) {
        const T v = (F + tail) * sc;
        if (im) out[j * TM + mm].y = v; else out[j * TM + mm].x = v;
      }
    };
    if (lane == 0) put(0, f1);
    for (int m = m0; m < m1; ++m) {
      acc += dm(m);
      put(m, f1 - acc);
    }
  }
}

}  // namespace col
}  // namespace nhqg

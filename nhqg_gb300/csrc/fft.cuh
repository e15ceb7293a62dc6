// Batched in-place complex FFTs in shared memory, FP64, lengths 2^a 3^b.
//
// Forward transforms run decimation-in-frequency (natural order in,
// mixed-radix digit-reversed order out); inverse transforms run the exact
// transpose, decimation-in-time (digit-reversed in, natural out, unscaled).
// Keeping the digit-reversed order in shared memory lets every butterfly read
// and write the same R locations, so a pass needs no second buffer; callers
// address the reversed side through the permutation table perm[k] = position
// of frequency k.  Radix-4 passes first, then radix-2, then radix-3: the
// radix-4 butterfly costs 16 DADD + 3 twiddle products (12 FP64 ops) per 4
// points, the cheapest of the three on the FP64 pipe.
#pragma once
#include "common.cuh"

namespace nhqg {

struct FftPlan {
  int n;
  int npass;
  int radix[12];
};

inline FftPlan make_fft_plan(int n) {
  FftPlan p{};
  p.n = n;
  int m = n;
  while (m % 4 == 0 && m > 1) { p.radix[p.npass++] = 4; m /= 4; }
  while (m % 2 == 0 && m > 1) { p.radix[p.npass++] = 2; m /= 2; }
  while (m % 3 == 0 && m > 1) { p.radix[p.npass++] = 3; m /= 3; }
  if (m != 1) p.npass = -1;  // unsupported length
  return p;
}

// position of frequency k in the digit-reversed output of fft_dif_fwd
inline void make_fft_perm(const FftPlan& p, int* perm) {
  for (int k = 0; k < p.n; ++k) {
    int L = p.n, kk = k, pos = 0;
    for (int q = 0; q < p.npass; ++q) {
      const int R = p.radix[q];
      const int Ls = L / R;
      pos += (kk % R) * Ls;
      kk /= R;
      L = Ls;
    }
    perm[k] = pos;
  }
}

constexpr double kSqrt3Half = 0.86602540378443864676;

// complex type per real type
template <typename T> struct CT;
template <> struct CT<double> { using type = double2; };
template <> struct CT<float> { using type = float2; };
template <typename T> using cplx_t = typename CT<T>::type;

template <typename C> __device__ __forceinline__ C gadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C gsub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C, typename T> __device__ __forceinline__ C gscale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename C> __device__ __forceinline__ C gmk(decltype(C().x) x, decltype(C().x) y) { C r; r.x = x; r.y = y; return r; }
// a * b and a * conj(b)
template <typename C> __device__ __forceinline__ C gmul(C a, C b) {
  return gmk<C>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
template <typename C> __device__ __forceinline__ C gmulc(C a, C b) {
  return gmk<C>(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}

// Butterfly index split idx -> (sequence s, block blk, offset j) for nb
// butterflies per sequence and span Ls: shifts and masks when both are powers
// of two (every pass of a 2^a length), integer division otherwise.
struct FftIndex {
  int nb, Ls, lnb, lls;
  bool p2;
  __device__ __forceinline__ FftIndex(int nb_, int Ls_) : nb(nb_), Ls(Ls_) {
    p2 = ((nb & (nb - 1)) == 0) && ((Ls & (Ls - 1)) == 0);
    lnb = __ffs(nb) - 1;
    lls = __ffs(Ls) - 1;
  }
  __device__ __forceinline__ void split(int idx, int& s, int& blk, int& j) const {
    if (p2) {
      s = idx >> lnb;
      const int b = idx & (nb - 1);
      blk = b >> lls;
      j = b & (Ls - 1);
    } else {
      s = idx / nb;
      const int b = idx - s * nb;
      blk = b / Ls;
      j = b - blk * Ls;
    }
  }
};

// Element i of a sequence sits at i + (i >> PS) when PS > 0: one padding
// element every 2^PS breaks the power-of-two strides of the late passes
// across shared-memory banks.
template <int PS>
__device__ __forceinline__ int fft_pad(int i) { return PS > 0 ? i + (i >> PS) : i; }

// Forward DFT (sign -1), natural -> reversed.  tw[k] = exp(-2 pi i k / n).
template <typename C, int PS = 0>
__device__ __forceinline__ void fft_dif_fwd(C* __restrict__ data, int nseq, int stride,
                                            const FftPlan& pl, const C* __restrict__ tw) {
  using T = decltype(C().x);
  int L = pl.n;
  for (int q = 0; q < pl.npass; ++q) {
    const int R = pl.radix[q];
    const int Ls = L / R;
    const int nb = pl.n / R;
    const int tws = pl.n / L;
    const FftIndex ix(nb, Ls);
    for (int idx = threadIdx.x; idx < nseq * nb; idx += blockDim.x) {
      int s, blk, j;
      ix.split(idx, s, blk, j);
      C* const a0 = data + s * stride;
      const int e = blk * L + j;
      auto A = [&](int r) -> C& { return a0[fft_pad<PS>(e + r * Ls)]; };
      if (R == 4) {
        const C x0 = A(0), x1 = A(1), x2 = A(2), x3 = A(3);
        const C t0 = gadd(x0, x2), t1 = gsub(x0, x2), t2 = gadd(x1, x3), t3 = gsub(x1, x3);
        C y1 = gmk<C>(t1.x + t3.y, t1.y - t3.x);  // t1 - i t3
        C y2 = gsub(t0, t2);
        C y3 = gmk<C>(t1.x - t3.y, t1.y + t3.x);  // t1 + i t3
        A(0) = gadd(t0, t2);
        if (j != 0) {
          y1 = gmul(y1, tw[j * tws]);
          y2 = gmul(y2, tw[2 * j * tws]);
          y3 = gmul(y3, tw[3 * j * tws]);
        }
        A(1) = y1;
        A(2) = y2;
        A(3) = y3;
      } else if (R == 2) {
        const C x0 = A(0), x1 = A(1);
        C y1 = gsub(x0, x1);
        A(0) = gadd(x0, x1);
        if (j != 0) y1 = gmul(y1, tw[j * tws]);
        A(1) = y1;
      } else {  // R == 3
        const C x0 = A(0), x1 = A(1), x2 = A(2);
        const C sp = gadd(x1, x2);
        const C d = gscale(gsub(x1, x2), (T)kSqrt3Half);
        const C m = gmk<C>(fma((T)-0.5, sp.x, x0.x), fma((T)-0.5, sp.y, x0.y));
        C y1 = gmk<C>(m.x + d.y, m.y - d.x);  // m - i d
        C y2 = gmk<C>(m.x - d.y, m.y + d.x);  // m + i d
        A(0) = gadd(x0, sp);
        if (j != 0) {
          y1 = gmul(y1, tw[j * tws]);
          y2 = gmul(y2, tw[2 * j * tws]);
        }
        A(1) = y1;
        A(2) = y2;
      }
    }
    __syncthreads();
    L = Ls;
  }
}

// Inverse DFT (sign +1, unscaled), reversed -> natural.
template <typename C, int PS = 0>
__device__ __forceinline__ void fft_dit_inv(C* __restrict__ data, int nseq, int stride,
                                            const FftPlan& pl, const C* __restrict__ tw) {
  using T = decltype(C().x);
  int Ls_of[12];
  {
    int L = pl.n;
    for (int q = 0; q < pl.npass; ++q) { Ls_of[q] = L; L /= pl.radix[q]; }
  }
  for (int q = pl.npass - 1; q >= 0; --q) {
    const int R = pl.radix[q];
    const int L = Ls_of[q];
    const int Ls = L / R;
    const int nb = pl.n / R;
    const int tws = pl.n / L;
    const FftIndex ix(nb, Ls);
    for (int idx = threadIdx.x; idx < nseq * nb; idx += blockDim.x) {
      int s, blk, j;
      ix.split(idx, s, blk, j);
      C* const a0 = data + s * stride;
      const int e = blk * L + j;
      auto A = [&](int r) -> C& { return a0[fft_pad<PS>(e + r * Ls)]; };
      if (R == 4) {
        C x0 = A(0), x1 = A(1), x2 = A(2), x3 = A(3);
        if (j != 0) {
          x1 = gmulc(x1, tw[j * tws]);
          x2 = gmulc(x2, tw[2 * j * tws]);
          x3 = gmulc(x3, tw[3 * j * tws]);
        }
        const C t0 = gadd(x0, x2), t1 = gsub(x0, x2), t2 = gadd(x1, x3), t3 = gsub(x1, x3);
        A(0) = gadd(t0, t2);
        A(1) = gmk<C>(t1.x - t3.y, t1.y + t3.x);      // t1 + i t3
        A(2) = gsub(t0, t2);
        A(3) = gmk<C>(t1.x + t3.y, t1.y - t3.x);  // t1 - i t3
      } else if (R == 2) {
        C x0 = A(0), x1 = A(1);
        if (j != 0) x1 = gmulc(x1, tw[j * tws]);
        A(0) = gadd(x0, x1);
        A(1) = gsub(x0, x1);
      } else {
        C x0 = A(0), x1 = A(1), x2 = A(2);
        if (j != 0) {
          x1 = gmulc(x1, tw[j * tws]);
          x2 = gmulc(x2, tw[2 * j * tws]);
        }
        const C sp = gadd(x1, x2);
        const C d = gscale(gsub(x1, x2), (T)kSqrt3Half);
        const C m = gmk<C>(fma((T)-0.5, sp.x, x0.x), fma((T)-0.5, sp.y, x0.y));
        A(0) = gadd(x0, sp);
        A(1) = gmk<C>(m.x - d.y, m.y + d.x);      // m + i d
        A(2) = gmk<C>(m.x + d.y, m.y - d.x);  // m - i d
      }
    }
    __syncthreads();
  }
}

}  // namespace nhqg

// Shared device helpers for the NHQG GB300 engine (FP64 plain path).
//
// Complex values are double2 (x = re, y = im).  On GB300 the FP64 pipe
// retires ~2 DFMA/clk/SM, ~58x fewer lanes than FP32, so every kernel here
// is written to minimise FP64 instructions; integer/shared-memory work is
// close to free next to it.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nhqg {

__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// i * a
__device__ __forceinline__ double2 cmul_i(double2 a) { return make_double2(-a.y, a.x); }
// a * b
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
// acc + s * a  (s real)
__device__ __forceinline__ double2 caxpy(double s, double2 a, double2 acc) {
  return make_double2(fma(s, a.x, acc.x), fma(s, a.y, acc.y));
}
__device__ __forceinline__ double2 czero() { return make_double2(0.0, 0.0); }

// Sizes of one grid.  Compact mode layout: the stored modes are Mr rows in
// fftfreq order (kx_int = 0..K, then the Mr-K-1 most negative rows) times Mc
// columns ky = 0..Mc-1; mode m = r*Mc + c; a field is [level][m].
//  - 2/3 rule: the keep-rectangle |kx_int| <= K, ky_int <= K with K = Nx/3,
//    Mr = 2K+1, Mc = K+1; products are formed on the Nx grid (Nh = Nx).
//  - 3/2 rule: every rfft2 mode (the state is full band): K = Nx/2 (the
//    Nyquist row counts as a "positive" row), Mr = Nx, Mc = Nk; products are
//    formed on the zero-padded Npad = 3Nx/2 grid (Nh = Npad).
struct Dims {
  int Nx, Nk, Nz, P, G, K, Mr, Mc, M;
  int Nh;    // side of the physical grid the horizontal products use
  bool pad;  // 3/2 rule (full-band layout, padded products)
};

inline Dims make_dims(int Nx, int Nz, bool pad32 = false) {
  Dims d;
  d.Nx = Nx;
  d.Nk = Nx / 2 + 1;
  d.Nz = Nz;
  d.P = Nz + 1;
  d.G = Nz - 1;
  d.pad = pad32;
  if (pad32) {
    d.K = Nx / 2;
    d.Mr = Nx;
    d.Mc = d.Nk;
    d.Nh = 3 * Nx / 2;
  } else {
    d.K = Nx / 3;
    d.Mr = 2 * d.K + 1;
    d.Mc = d.K + 1;
    d.Nh = Nx;
  }
  d.M = d.Mr * d.Mc;
  return d;
}

// full-layout kx row of compact row r
__host__ __device__ __forceinline__ int full_row(int r, int K, int Mr, int Nx) {
  return r <= K ? r : Nx - Mr + r;
}
// compact row of the mirrored wavenumber -kx (ky = 0 column pairing; the
// Nyquist row of the full-band layout is its own mirror)
__host__ __device__ __forceinline__ int mirror_row(int r, int Mr) {
  return r == 0 ? 0 : Mr - r;
}
// row of the zero-padded Nh-point spectrum that holds full-layout row kf
// (nhqg/spectral.py:18-34: rows 0..Nx/2-1 stay, rows Nx/2..Nx-1 move to the
// top, so the Nyquist row becomes kx = -Nx/2); the identity when Nh == Nx
__host__ __device__ __forceinline__ int padded_row(int kf, int Nx, int Nh) {
  return kf < Nx / 2 ? kf : kf + (Nh - Nx);
}

// Block-wide deterministic sum of one double per thread (blockDim <= 1024).
__device__ __forceinline__ double block_sum(double v, double* scratch) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  double t = 0.0;
  if (warp == 0) {
    t = lane < nw ? scratch[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

}  // namespace nhqg

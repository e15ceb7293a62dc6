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

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
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

// Sizes of one grid.  Compact mode layout: the 2/3-rule keep-rectangle
// |kx_int| <= K, ky_int <= K (K = Nx/3) is stored as Mr = 2K+1 rows in
// fftfreq order (kx_int = 0..K, -K..-1) times Mc = K+1 columns; mode
// m = r*Mc + c; a field is [level][m].
struct Dims {
  int Nx, Nk, Nz, P, G, K, Mr, Mc, M;
};

inline Dims make_dims(int Nx, int Nz) {
  Dims d;
  d.Nx = Nx;
  d.Nk = Nx / 2 + 1;
  d.Nz = Nz;
  d.P = Nz + 1;
  d.G = Nz - 1;
  d.K = Nx / 3;
  d.Mr = 2 * d.K + 1;
  d.Mc = d.K + 1;
  d.M = d.Mr * d.Mc;
  return d;
}

// full-layout kx row of compact row r
__host__ __device__ __forceinline__ int full_row(int r, int K, int Nx) {
  return r <= K ? r : Nx - (2 * K + 1) + r;
}
// compact row of the mirrored wavenumber -kx (ky = 0 column pairing)
__host__ __device__ __forceinline__ int mirror_row(int r, int K) {
  return r == 0 ? 0 : (2 * K + 1) - r;
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

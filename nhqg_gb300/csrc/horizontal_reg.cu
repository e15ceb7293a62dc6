// FP32 dealiased horizontal products with register-resident FFTs.
//
// Same products, layouts and reference semantics as the shared-memory
// kernels of horizontal.cu (nhqg/spectral.py:53-60, 281-358 under the 2/3
// rule; the plane API's full-band layout), for transform lengths
// N = R1 * R2 with (R1, R2) in {(8, 8), (8, 16), (16, 16)}: N = 64, 128, 256.
//
// One FFT sequence of length N belongs to R1 lanes of a warp (32 / R1
// sequences per warp), each lane holding R2 complex values in registers:
//   spectral layout  lane l holds X[l + R1 j],            j = 0..R2-1
//   physical layout  lane l holds x[(l + R1 t) + R2 b] at element t R1 + b
// The inverse transform is y[a + R2 b] = sum_l w_R1^{b l} w_N^{a l}
// sum_j w_R2^{a j} X[l + R1 j] (w = exp(+2 pi i / n)): an R2-point DFT in
// registers, the twiddles w_N^{a l}, one transpose through a warp-private
// shared-memory tile, then R2/R1 R1-point DFTs in registers.  The forward
// transform runs the transposed sequence and returns to the spectral layout,
// so pointwise products need no data movement between the two transforms.
// The tile rows are padded to R1 + 1 complex values, which makes both
// transpose directions free of shared-memory bank conflicts; no
// __syncthreads separates the FFT passes (only __syncwarp around the
// transpose).
//
//   H1  column inverse FFTs over kx of the derived spectra; the CTA stages
//       its compact input columns through shared memory (coalesced loads),
//       the output goes to the pair-major intermediate [f][lev][x/2][c][x%2].
//   H2  row pairs (a, b) as one complex sequence Z = Xa + i Xb: inverse FFTs,
//       products in physical space, forward FFTs, the Hermitian split of the
//       paired spectra by one warp shuffle per kept column, i ky / sponge.
//   H3  column forward FFTs, combine i kx G + H, kept rows staged through
//       shared memory for coalesced stores.
#include <utility>

#include "engine.h"

namespace nhqg {

namespace {

// ---------------------------------------------------------------- compile-time helpers
template <typename F, int... I>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// cos and sin of 2 pi k / 16
__host__ __device__ constexpr float cos16(int k) {
  constexpr float C1 = 0.923879532511286756f, H = 0.707106781186547524f, S1 = 0.382683432365089772f;
  switch (k & 15) {
    case 0: return 1.f;   case 1: return C1;  case 2: return H;   case 3: return S1;
    case 4: return 0.f;   case 5: return -S1; case 6: return -H;  case 7: return -C1;
    case 8: return -1.f;  case 9: return -C1; case 10: return -H; case 11: return -S1;
    case 12: return 0.f;  case 13: return S1; case 14: return H;  default: return C1;
  }
}
__host__ __device__ constexpr float sin16(int k) { return cos16(k - 4); }

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * w and a * conj(w)
__device__ __forceinline__ float2 f2mul(float2 a, float2 w) {
  return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ float2 f2mulc(float2 a, float2 w) {
  return make_float2(fmaf(a.x, w.x, a.y * w.y), fmaf(a.y, w.x, -a.x * w.y));
}

// x * exp(SGN 2 pi i K / R), R dividing 16; trivial rotations cost nothing
template <int R, int K, int SGN>
__device__ __forceinline__ float2 rot(float2 x) {
  static_assert(16 % R == 0, "R must divide 16");
  constexpr int k = (((K % R) + R) % R) * (16 / R);
  if constexpr (k == 0) {
    return x;
  } else if constexpr (k == 8) {
    return make_float2(-x.x, -x.y);
  } else if constexpr (k == 4) {  // * SGN i
    return SGN > 0 ? make_float2(-x.y, x.x) : make_float2(x.y, -x.x);
  } else if constexpr (k == 12) {  // * -SGN i
    return SGN > 0 ? make_float2(x.y, -x.x) : make_float2(-x.y, x.x);
  } else {
    constexpr float c = cos16(k), s = SGN * sin16(k);
    return make_float2(fmaf(c, x.x, -s * x.y), fmaf(c, x.y, s * x.x));
  }
}

// In-register DFT of length R over x[O + S i], natural order in and out:
// X[k] = sum_i x_i exp(SGN 2 pi i k i / R).  R = P Q splits as
// y[a + Q b] = sum_p w_P^{b p} w_R^{a p} sum_q w_Q^{a q} x[p + P q].
template <int R, int SGN>
struct RDft {
  static constexpr int P = (R >= 16) ? 4 : 2;
  static constexpr int Q = R / P;
  template <int O, int S>
  __device__ __forceinline__ static void run(float2* x) {
    sfor<P>([&](auto p) { RDft<Q, SGN>::template run<O + S * decltype(p)::value, S * P>(x); });
    sfor<P>([&](auto p) {
      sfor<Q>([&](auto a) {
        constexpr int pp = decltype(p)::value, aa = decltype(a)::value;
        x[O + S * (pp + P * aa)] = rot<R, aa * pp, SGN>(x[O + S * (pp + P * aa)]);
      });
    });
    sfor<Q>([&](auto a) { RDft<P, SGN>::template run<O + S * P * decltype(a)::value, S>(x); });
    float2 t[R];
    sfor<Q>([&](auto a) {
      sfor<P>([&](auto b) {
        constexpr int aa = decltype(a)::value, bb = decltype(b)::value;
        t[aa + Q * bb] = x[O + S * (bb + P * aa)];
      });
    });
    sfor<R>([&](auto i) { x[O + S * decltype(i)::value] = t[decltype(i)::value]; });
  }
};
template <int SGN>
struct RDft<2, SGN> {
  template <int O, int S>
  __device__ __forceinline__ static void run(float2* x) {
    const float2 a = x[O], b = x[O + S];
    x[O] = f2add(a, b);
    x[O + S] = f2sub(a, b);
  }
};
template <int SGN>
struct RDft<4, SGN> {
  template <int O, int S>
  __device__ __forceinline__ static void run(float2* x) {
    const float2 a0 = x[O], a1 = x[O + S], a2 = x[O + 2 * S], a3 = x[O + 3 * S];
    const float2 t0 = f2add(a0, a2), t1 = f2sub(a0, a2), t2 = f2add(a1, a3);
    const float2 t3 = rot<4, 1, SGN>(f2sub(a1, a3));
    x[O] = f2add(t0, t2);
    x[O + 2 * S] = f2sub(t0, t2);
    x[O + S] = f2add(t1, t3);
    x[O + 3 * S] = f2sub(t1, t3);
  }
};

// Length-N transform over the R1 lanes of one sequence group.  T is the
// group's transpose tile (R2 rows of S = R1 + 1), tw the shared table
// tw[a S + l] = exp(+2 pi i a l / N), l the lane within the group.
template <int R1, int R2>
struct LaneFft {
  static_assert(R2 % R1 == 0, "R1 must divide R2");
  static constexpr int S = R1 + 1;
  // groups start 16 banks apart: TILE = 8 (mod 16) complex values
  static constexpr int TILE = R2 * S + ((8 - (R2 * S) % 16) + 16) % 16;

  // spectral -> physical, unscaled, sign +1
  __device__ __forceinline__ static void inv(float2* x, float2* T, const float2* tw, int l) {
    RDft<R2, +1>::template run<0, 1>(x);
    sfor<R2>([&](auto a) {
      constexpr int A = decltype(a)::value;
      if constexpr (A > 0) x[A] = f2mul(x[A], tw[A * S + l]);
    });
    sfor<R2>([&](auto a) { T[decltype(a)::value * S + l] = x[decltype(a)::value]; });
    __syncwarp();
    sfor<R2 / R1>([&](auto t) {
      sfor<R1>([&](auto m) {
        constexpr int tt = decltype(t)::value, mm = decltype(m)::value;
        x[tt * R1 + mm] = T[(l + R1 * tt) * S + mm];
      });
    });
    __syncwarp();
    sfor<R2 / R1>([&](auto t) { RDft<R1, +1>::template run<decltype(t)::value * R1, 1>(x); });
  }

  // physical -> spectral, sign -1
  __device__ __forceinline__ static void fwd(float2* x, float2* T, const float2* tw, int l) {
    sfor<R2 / R1>([&](auto t) { RDft<R1, -1>::template run<decltype(t)::value * R1, 1>(x); });
    sfor<R2 / R1>([&](auto t) {
      sfor<R1>([&](auto m) {
        constexpr int tt = decltype(t)::value, mm = decltype(m)::value;
        if constexpr (mm > 0) x[tt * R1 + mm] = f2mulc(x[tt * R1 + mm], tw[(l + R1 * tt) * S + mm]);
        T[(l + R1 * tt) * S + mm] = x[tt * R1 + mm];
      });
    });
    __syncwarp();
    sfor<R2>([&](auto a) { x[decltype(a)::value] = T[decltype(a)::value * S + l]; });
    __syncwarp();
    RDft<R2, -1>::template run<0, 1>(x);
  }
};

struct HR {
  int Nx, Nk, K, Mr, Mc, M, N, levels;
  int rows_in, cols_in;
  bool full_in, full_out;
  int form, nf1, ng;
  bool sponge, eta, psi_derived;
  float scale;  // 1 / (N Nx)
  const float2 *psi, *q, *w, *th;
  const float *kx_full, *ky_full;
  const double* inv_denom;
  const float2* eta_c;
  const float *sponge_phys, *eta_phys;
  // gradient form of the trap PV: q enters the products without eta and the
  // trap term is u . grad(eta) (flux) or J[psi, eta] (Jacobian), from these
  // tables; FP32 would otherwise cancel a small q against the O(1) eta
  bool eta_grad;
  const float *eta_x, *eta_y;
  const float2* tw;  // exp(-2 pi i k / N), k < N
  float2 *x1, *x2;
  float2 *Aq, *Aw, *Ath;
};

// H1 -> H2 intermediate, pair-major [f][lev][x/2][c][x%2]: H2 reads the row
// pair of a column as one 16-byte value, contiguous across the columns
__device__ __forceinline__ size_t xi(const HR& k, int f, int lev, int pair, int c, int cols) {
  return ((((size_t)f * k.levels + lev) * (k.N / 2) + pair) * cols + c) * 2;
}
// H2 -> H3 intermediate, column-major [g][lev][c][x]: H3's column loads are
// contiguous along x; H2 stores a row pair's two values as one 16-byte value
__device__ __forceinline__ size_t xo(const HR& k, int g, int lev, int c, int x) {
  return (((size_t)g * k.levels + lev) * k.Mc + c) * k.N + x;
}

// twiddle table of the lane transforms: tw_s[a S + l] = conj(tw[a l mod N])
template <int R1, int R2>
__device__ __forceinline__ void load_lane_twiddles(const HR& k, float2* tw_s) {
  constexpr int S = R1 + 1;
  for (int i = threadIdx.x; i < R2 * S; i += blockDim.x) {
    const int a = i / S, l = i - a * S;
    if (l < R1) {
      const float2 t = k.tw[(a * l) % (R1 * R2)];
      tw_s[i] = make_float2(t.x, -t.y);
    }
  }
}

// full-layout row of a compact row
__device__ __forceinline__ int row_full(const HR& k, int r) { return full_row(r, k.K, k.Mr, k.Nx); }
// full-layout row of transform position kpos (-1 in the padding of the 3/2 rule)
__device__ __forceinline__ int pos_row(const HR& k, int kpos) {
  if (kpos < k.Nx / 2) return kpos;
  if (kpos >= k.N - k.Nx / 2) return kpos - (k.N - k.Nx);
  return -1;
}
// compact (kept, 2/3-band) row of full-layout row kf, -1 outside the band
__device__ __forceinline__ int kept_row(const HR& k, int kf) {
  if (kf < 0) return -1;
  if (kf <= k.K) return kf;
  if (kf >= k.Nx - (k.Mr - k.K - 1)) return kf - (k.Nx - k.Mr);
  return -1;
}

// ---------------------------------------------------------------- H1
// One sequence group per column; WARPS warps, 32 / R1 columns per warp.  The
// CTA's columns of psi (unless derived), q, w, theta stage through shared
// memory: tile[field][row][CB + 1].
template <int R1, int R2>
__global__ void __launch_bounds__(128) k_h1r(HR k) {
  using F = LaneFft<R1, R2>;
  constexpr int G = 32 / R1;
  constexpr int CB = 4 * G;  // columns per CTA (4 warps)
  constexpr int TS = CB + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* T = tw_s + R2 * (R1 + 1) + 8;
  float2* tile = T + 4 * G * F::TILE;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / R1, l = lane - g * R1;
  const int lev = blockIdx.y;
  const int c0 = blockIdx.x * CB;
  const int ncb = min(CB, k.cols_in - c0);
  load_lane_twiddles<R1, R2>(k, tw_s);
  // raw fields: 0 psi (read or derived), 1 q (+eta), 2 w, 3 theta; staged two
  // at a time (phase 0: psi, q; phase 1: w, theta) so that the tile stays
  // small enough for five CTAs per SM
  const int nphase = (k.form == HF_SPONGE) ? 1 : 2;
  const size_t plane = (size_t)k.rows_in * k.cols_in;
  const int cc = warp * G + g;
  const int c = c0 + cc;
  const bool live = cc < ncb;
  float2* Tg = T + (size_t)(warp * G + g) * F::TILE;
  const float kys = live ? k.ky_full[c] * k.scale : 0.f;
  const float sc = k.scale;
  if (nphase == 2 && ncb > 0) {
    // L2 prefetch of phase 1's columns (w, theta) while phase 0 runs: one
    // instruction per row and field (the CTA's CB columns share a line or two)
    for (int i = threadIdx.x; i < 2 * k.rows_in; i += blockDim.x) {
      const int r = i >> 1;
      const float2* f = (i & 1) ? k.th : k.w;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(f + (size_t)lev * plane + (size_t)r * k.cols_in + c0));
    }
  }
  for (int phase = 0; phase < nphase; ++phase) {
    if (phase > 0) __syncthreads();  // the previous phase's reads of the tile are done
    for (int i = threadIdx.x; i < k.rows_in * CB; i += blockDim.x) {
      const int r = i / CB, cc2 = i - r * CB, c2 = c0 + cc2;
      float2 v0 = make_float2(0.f, 0.f), v1 = make_float2(0.f, 0.f);
      if (cc2 < ncb) {
        const size_t off = (size_t)lev * plane + (size_t)r * k.cols_in + c2;
        if (k.form == HF_SPONGE) {
          v0 = k.q[off];
        } else if (phase == 0) {
          const float2 qv = k.q[off];
          if (k.psi_derived) {
            const float s = (float)(-k.inv_denom[r * k.Mc + c2]);
            v0 = make_float2(qv.x * s, qv.y * s);
          } else {
            v0 = k.psi[off];
          }
          v1 = qv;
          if (k.eta && !k.eta_grad) v1 = f2add(v1, k.eta_c[r * k.Mc + c2]);
        } else {
          v0 = k.w[off];
          v1 = k.th[off];
        }
      }
      tile[(size_t)r * TS + cc2] = v0;
      tile[((size_t)k.rows_in + r) * TS + cc2] = v1;
    }
    __syncthreads();
    for (int f = 0; f < k.nf1; ++f) {
      // raw field and derivative of output sequence f
      int raw, der;  // der: 0 none (scaled), 1 d/dx, 2 d/dy, 3 u = -d/dy
      if (k.form == HF_FLUX) {
        const int rf[5] = {0, 0, 1, 2, 3}, dv[5] = {3, 1, 0, 0, 0};
        raw = rf[f]; der = dv[f];
      } else if (k.form == HF_JAC) {
        if (f < 8) { raw = f >> 1; der = (f & 1) ? 2 : 1; }
        else { raw = f - 7; der = 0; }
      } else {
        raw = 0; der = 0;
      }
      if ((raw >> 1) != phase) continue;
      const int slot = raw & 1;
      float2 x[R2];
      sfor<R2>([&](auto jj) {
        constexpr int j = decltype(jj)::value;
        const int kpos = l + R1 * j;
        const int kf = live ? pos_row(k, kpos) : -1;
        const int r = k.full_in ? kf : kept_row(k, kf);
        float2 v = make_float2(0.f, 0.f);
        if (r >= 0) {
          const float2 a = tile[((size_t)slot * k.rows_in + r) * TS + cc];
          if (der == 0) {
            v = make_float2(a.x * sc, a.y * sc);
          } else if (der == 2) {  // i ky a
            v = make_float2(-kys * a.y, kys * a.x);
          } else if (der == 3) {  // -i ky a
            v = make_float2(kys * a.y, -kys * a.x);
          } else {  // i kx a
            const float kxs = k.kx_full[k.full_in ? r : row_full(k, r)] * sc;
            v = make_float2(-kxs * a.y, kxs * a.x);
          }
        }
        x[j] = v;
      });
      F::inv(x, Tg, tw_s, l);
      if (live) {
        sfor<R2>([&](auto ee) {
          constexpr int e = decltype(ee)::value;
          const int xx = (l + R1 * (e / R1)) + R2 * (e % R1);
          k.x1[xi(k, f, lev, xx >> 1, c, k.cols_in) + (xx & 1)] = x[e];
        });
      }
    }
  }
}

// ---------------------------------------------------------------- H2
// One sequence group per row pair; per group a transpose tile and the
// own-lane store of the second velocity factor (v, or psi_y).
template <int R1, int R2, int FORM, bool SP>
__global__ void __launch_bounds__(128) k_h2r(HR k) {
  using F = LaneFft<R1, R2>;
  constexpr int N = R1 * R2;
  constexpr int G = 32 / R1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* T = tw_s + R2 * (R1 + 1) + 8;
  float2* Vs = T + 4 * G * F::TILE;
  // output staging: the CTA's 4 G row pairs = 8 G consecutive x of every kept
  // column, stored as one contiguous run per column
  constexpr int OS = 8 * G + 2;  // row stride (complex values) of the staging tile
  float2* Os = Vs + (size_t)4 * G * (N + 8);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / R1, l = lane - g * R1;
  const int lev = blockIdx.y;
  const int pp = (blockIdx.x * 4 + warp) * G + g;  // row pair
  const bool live = pp < N / 2;
  const int pair = live ? pp : 0;
  const int xa = 2 * pair;
  float2* Tg = T + (size_t)(warp * G + g) * F::TILE;
  float2* Vg = Vs + (size_t)(warp * G + g) * (N + 8);
  load_lane_twiddles<R1, R2>(k, tw_s);
  __syncthreads();
  const int cols = k.cols_in;
  const int gbase = g * R1;
  const unsigned full = 0xffffffffu;

  // Hermitian-extended spectrum of the row pair of input field f
  auto load = [&](int f, float2* x) {
    sfor<R2>([&](auto jj) {
      constexpr int j = decltype(jj)::value;
      const int c = l + R1 * j;
      float2 z = make_float2(0.f, 0.f);
      if (c < cols) {
        const float4 ab = *reinterpret_cast<const float4*>(k.x1 + xi(k, f, lev, pair, c, cols));
        z = (c == 0 || c == N / 2) ? make_float2(ab.x, ab.z) : make_float2(ab.x - ab.w, ab.y + ab.z);
      } else if (c > N - cols) {
        const int m = N - c;
        const float4 ab = *reinterpret_cast<const float4*>(k.x1 + xi(k, f, lev, pair, m, cols));
        z = make_float2(ab.x + ab.w, ab.z - ab.y);
      }
      x[j] = z;
    });
  };
  // split the paired spectrum in x (spectral layout) into the rows' spectra
  // at the kept columns c < Mc; emit(j, c, Xa, Xb) for each
  auto split = [&](const float2* x, auto&& emit) {
    const int src = gbase + ((R1 - l) & (R1 - 1));
    sfor<R2 / 2 + 1>([&](auto jj) {
      constexpr int j = decltype(jj)::value;
      if (R1 * j < k.Mc) {  // uniform over the warp
        constexpr int jm = R2 - 1 - j, j0 = (R2 - j) % R2;
        float2 B;
        B.x = __shfl_sync(full, x[jm].x, src);
        B.y = __shfl_sync(full, x[jm].y, src);
        if (l == 0) B = x[j0];
        const float2 A = x[j];
        const int c = l + R1 * j;
        if (c < k.Mc) {
          emit(j, c, make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y)),
               make_float2(0.5f * (A.y + B.y), 0.5f * (B.x - A.x)));
        }
      }
    });
  };
  const int gi = warp * G + g;  // row pair within the CTA
  const int x0 = 2 * blockIdx.x * 4 * G;
  const int nx = min(8 * G, N - x0);
  auto store = [&](int, int c, float2 Ra, float2 Rb) {
    *reinterpret_cast<float4*>(Os + (size_t)c * OS + 2 * gi) = make_float4(Ra.x, Ra.y, Rb.x, Rb.y);
  };
  // after every group has staged output gout: contiguous stores per column
  auto flush = [&](int gout) {
    __syncthreads();
    for (int i = threadIdx.x; i < k.Mc * nx; i += blockDim.x) {
      const int c = i / nx, xx = i - c * nx;
      k.x2[xo(k, gout, lev, c, x0 + xx)] = Os[(size_t)c * OS + xx];
    }
    __syncthreads();
  };
  // sponge and eta at this lane's physical points of rows xa, xa + 1
  auto sig = [&](int e, float& sa, float& sb) {
    const int y = (l + R1 * (e / R1)) + R2 * (e % R1);
    sa = k.sponge_phys[(size_t)xa * N + y];
    sb = k.sponge_phys[(size_t)(xa + 1) * N + y];
  };
  auto eta = [&](int e, float& ea, float& eb) {
    const int y = (l + R1 * (e / R1)) + R2 * (e % R1);
    ea = k.eta_phys[(size_t)xa * N + y];
    eb = k.eta_phys[(size_t)(xa + 1) * N + y];
  };
  // grad(eta) at this lane's physical points of rows xa, xa + 1
  auto geta = [&](int e, float& gxa, float& gxb, float& gya, float& gyb) {
    const int y = (l + R1 * (e / R1)) + R2 * (e % R1);
    gxa = k.eta_x[(size_t)xa * N + y];
    gxb = k.eta_x[(size_t)(xa + 1) * N + y];
    gya = k.eta_y[(size_t)xa * N + y];
    gyb = k.eta_y[(size_t)(xa + 1) * N + y];
  };

  // L2 prefetch of field f's rows of this pair (one instruction per 128-byte
  // line, no registers held): issued one field ahead, so the next load finds
  // its lines in L2 instead of waiting on DRAM behind this field's FFTs
  auto prefetch = [&](int f) {
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(k.x1 + xi(k, f, lev, pair, 0, cols));
    const uintptr_t end = a0 + (uintptr_t)cols * sizeof(float4);
    for (uintptr_t a = (a0 & ~uintptr_t(127)) + 128 * (uintptr_t)l; a < end; a += 128 * R1)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
  };

  float2 x[R2], y[R2], u[R2];
  if constexpr (FORM == HF_FLUX) {
    load(0, u);
    prefetch(1);
    prefetch(2);
    F::inv(u, Tg, tw_s, l);
    load(1, x);
    F::inv(x, Tg, tw_s, l);
    sfor<R2>([&](auto e) { Vg[decltype(e)::value * R1 + l] = x[decltype(e)::value]; });
    for (int f = 0; f < 3; ++f) {
      load(2 + f, x);
      if (f < 2) prefetch(3 + f);
      F::inv(x, Tg, tw_s, l);
      // G = F(u f)
      sfor<R2>([&](auto e) {
        constexpr int ee = decltype(e)::value;
        y[ee] = make_float2(u[ee].x * x[ee].x, u[ee].y * x[ee].y);
      });
      F::fwd(y, Tg, tw_s, l);
      split(y, [&](int, int c, float2 Ra, float2 Rb) { store(2 * f, c, Ra, Rb); });
      flush(2 * f);
      // extra spectrum S = F(sigma (f - eta)) or, in the gradient form,
      // F(sigma q + u . grad(eta)) for q; kept in y
      const bool extra = k.sponge || (f == 0 && k.eta_grad);
      if constexpr (SP) {
        if (extra) {
          sfor<R2>([&](auto e) {
            constexpr int ee = decltype(e)::value;
            float sa = 0.f, sb = 0.f, ea = 0.f, eb = 0.f;
            if (k.sponge) sig(ee, sa, sb);
            if (f == 0 && k.eta && !k.eta_grad) eta(ee, ea, eb);
            float2 v = make_float2(sa * (x[ee].x - ea), sb * (x[ee].y - eb));
            if (f == 0 && k.eta_grad) {
              float gxa, gxb, gya, gyb;
              geta(ee, gxa, gxb, gya, gyb);
              const float2 vv = Vg[ee * R1 + l];
              v.x = fmaf(u[ee].x, gxa, fmaf(vv.x, gya, v.x));
              v.y = fmaf(u[ee].y, gxb, fmaf(vv.y, gyb, v.y));
            }
            y[ee] = v;
          });
          F::fwd(y, Tg, tw_s, l);
        }
      }
      // H = i ky F(v f) (+ S)
      sfor<R2>([&](auto e) {
        constexpr int ee = decltype(e)::value;
        const float2 v = Vg[ee * R1 + l];
        x[ee] = make_float2(v.x * x[ee].x, v.y * x[ee].y);
      });
      F::fwd(x, Tg, tw_s, l);
      if (SP && extra) {
        // y's split values at the same (j, c) are needed beside x's: split both
        float2 Sa[R2 / 2 + 1], Sb[R2 / 2 + 1];
        split(y, [&](int j, int, float2 Ra, float2 Rb) {
          sfor<R2 / 2 + 1>([&](auto q) {
            if (decltype(q)::value == j) { Sa[decltype(q)::value] = Ra; Sb[decltype(q)::value] = Rb; }
          });
        });
        split(x, [&](int j, int c, float2 Va, float2 Vb) {
          const float ky = k.ky_full[c];
          float2 Ra = make_float2(-ky * Va.y, ky * Va.x), Rb = make_float2(-ky * Vb.y, ky * Vb.x);
          sfor<R2 / 2 + 1>([&](auto q) {
            if (decltype(q)::value == j) {
              Ra = f2add(Ra, Sa[decltype(q)::value]);
              Rb = f2add(Rb, Sb[decltype(q)::value]);
            }
          });
          store(2 * f + 1, c, Ra, Rb);
        });
      } else {
        split(x, [&](int, int c, float2 Va, float2 Vb) {
          const float ky = k.ky_full[c];
          store(2 * f + 1, c, make_float2(-ky * Va.y, ky * Va.x), make_float2(-ky * Vb.y, ky * Vb.x));
        });
      }
      flush(2 * f + 1);
    }
  } else if constexpr (FORM == HF_JAC) {
    // J_f = psi_x f_y - psi_y f_x (+ sigma (f - eta)): psi_x in registers, psi_y stored
    load(0, u);
    F::inv(u, Tg, tw_s, l);
    load(1, x);
    F::inv(x, Tg, tw_s, l);
    sfor<R2>([&](auto e) { Vg[decltype(e)::value * R1 + l] = x[decltype(e)::value]; });
    for (int f = 0; f < 3; ++f) {
      load(2 + 2 * f, x);  // f_x
      F::inv(x, Tg, tw_s, l);
      sfor<R2>([&](auto e) {
        constexpr int ee = decltype(e)::value;
        const float2 py = Vg[ee * R1 + l];
        y[ee] = make_float2(-py.x * x[ee].x, -py.y * x[ee].y);
      });
      load(3 + 2 * f, x);  // f_y
      F::inv(x, Tg, tw_s, l);
      sfor<R2>([&](auto e) {
        constexpr int ee = decltype(e)::value;
        y[ee] = make_float2(fmaf(u[ee].x, x[ee].x, y[ee].x), fmaf(u[ee].y, x[ee].y, y[ee].y));
      });
      if constexpr (SP) {
        if (k.sponge) {
          load(8 + f, x);
          F::inv(x, Tg, tw_s, l);
          sfor<R2>([&](auto e) {
            constexpr int ee = decltype(e)::value;
            float sa, sb, ea = 0.f, eb = 0.f;
            sig(ee, sa, sb);
            if (f == 0 && k.eta && !k.eta_grad) eta(ee, ea, eb);
            y[ee] = make_float2(fmaf(sa, x[ee].x - ea, y[ee].x), fmaf(sb, x[ee].y - eb, y[ee].y));
          });
        }
        if (f == 0 && k.eta_grad) {  // J[psi, eta] = psi_x eta_y - psi_y eta_x
          sfor<R2>([&](auto e) {
            constexpr int ee = decltype(e)::value;
            float gxa, gxb, gya, gyb;
            geta(ee, gxa, gxb, gya, gyb);
            const float2 py = Vg[ee * R1 + l];
            y[ee].x = fmaf(u[ee].x, gya, fmaf(-py.x, gxa, y[ee].x));
            y[ee].y = fmaf(u[ee].y, gyb, fmaf(-py.y, gxb, y[ee].y));
          });
        }
      }
      F::fwd(y, Tg, tw_s, l);
      split(y, [&](int, int c, float2 Ra, float2 Rb) { store(f, c, Ra, Rb); });
      flush(f);
    }
  } else {  // sponge-only product
    load(0, x);
    F::inv(x, Tg, tw_s, l);
    sfor<R2>([&](auto e) {
      constexpr int ee = decltype(e)::value;
      float sa, sb;
      sig(ee, sa, sb);
      x[ee] = make_float2(sa * x[ee].x, sb * x[ee].y);
    });
    F::fwd(x, Tg, tw_s, l);
    split(x, [&](int, int c, float2 Ra, float2 Rb) { store(0, c, Ra, Rb); });
    flush(0);
  }
}

// ---------------------------------------------------------------- H3
template <int R1, int R2>
__global__ void __launch_bounds__(128) k_h3r(HR k) {
  using F = LaneFft<R1, R2>;
  constexpr int G = 32 / R1;
  constexpr int CB = 4 * G;
  constexpr int TS = CB + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* T = tw_s + R2 * (R1 + 1) + 8;
  float2* tile = T + 4 * G * F::TILE;  // [Mr][TS]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / R1, l = lane - g * R1;
  const int lev = blockIdx.y;
  const int c0 = blockIdx.x * CB;
  const int ncb = min(CB, k.Mc - c0);
  const int cc = warp * G + g;
  const int c = c0 + cc;
  const bool live = cc < ncb;
  const int cr = live ? c : c0;  // dead groups transform a live column's data and discard it
  float2* Tg = T + (size_t)(warp * G + g) * F::TILE;
  load_lane_twiddles<R1, R2>(k, tw_s);
  __syncthreads();
  const int nout = (k.form == HF_SPONGE) ? 1 : 3;
  auto load = [&](int gi, float2* x) {
    sfor<R2>([&](auto ee) {
      constexpr int e = decltype(ee)::value;
      const int xx = (l + R1 * (e / R1)) + R2 * (e % R1);
      x[e] = k.x2[xo(k, gi, lev, cr, xx)];
    });
  };
  for (int f = 0; f < nout; ++f) {
    float2 x[R2];
    if (k.form == HF_FLUX) {
      float2 h[R2];
      load(2 * f, x);
      F::fwd(x, Tg, tw_s, l);
      load(2 * f + 1, h);
      F::fwd(h, Tg, tw_s, l);
      sfor<R2>([&](auto jj) {
        constexpr int j = decltype(jj)::value;
        const int kf = pos_row(k, l + R1 * j);
        const float kx = (kf >= 0) ? k.kx_full[kf] : 0.f;
        x[j] = make_float2(fmaf(-kx, x[j].y, h[j].x), fmaf(kx, x[j].x, h[j].y));
      });
    } else {
      load(f, x);
      F::fwd(x, Tg, tw_s, l);
    }
    // kept (2/3-band) rows into the staging tile [Mr][TS], then stored row
    // by row (coalesced across the CTA's columns)
    if (f > 0) __syncthreads();  // the previous field's stores have read the tile
    sfor<R2>([&](auto jj) {
      constexpr int j = decltype(jj)::value;
      const int r = kept_row(k, pos_row(k, l + R1 * j));
      if (r >= 0 && live) tile[(size_t)r * TS + cc] = x[j];
    });
    __syncthreads();
    float2* out = (f == 0) ? k.Aq : (f == 1 ? k.Aw : k.Ath);
    for (int i = threadIdx.x; i < k.Mr * CB; i += blockDim.x) {
      const int cc2 = i % CB, r = i / CB;
      if (cc2 >= ncb) continue;
      const int c2 = c0 + cc2;
      const size_t oidx = k.full_out ? ((size_t)lev * k.Nx + row_full(k, r)) * k.Nk + c2
                                     : (size_t)lev * k.M + (size_t)r * k.Mc + c2;
      out[oidx] = tile[(size_t)r * TS + cc2];
    }
  }
}

template <int R1, int R2>
cudaError_t launch_reg(const HR& k, cudaStream_t st, Profiler& prof) {
  using F = LaneFft<R1, R2>;
  constexpr int N = R1 * R2;
  constexpr int G = 32 / R1;
  constexpr int CB = 4 * G;
  const size_t head = ((size_t)R2 * (R1 + 1) + 8 + (size_t)4 * G * F::TILE) * sizeof(float2);
  const size_t sm1 = head + (size_t)2 * k.rows_in * (CB + 1) * sizeof(float2);
  const size_t sm2 = head + ((size_t)4 * G * (N + 8) + (size_t)k.Mc * (8 * G + 2)) * sizeof(float2);
  const int nout = (k.form == HF_SPONGE) ? 1 : 3;
  const size_t sm3 = head + (size_t)k.Mr * (CB + 1) * sizeof(float2);
  const size_t cap = 200 * 1024;
  if (sm1 > cap || sm2 > cap || sm3 > cap) return cudaErrorInvalidConfiguration;
  cudaFuncSetAttribute(k_h1r<R1, R2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  // the SP instantiations carry the sponge and the gradient-form eta terms
  const bool sp = k.sponge || k.eta_grad;
  auto h2 = k_h2r<R1, R2, HF_SPONGE, true>;
  if (k.form == HF_FLUX) h2 = sp ? k_h2r<R1, R2, HF_FLUX, true> : k_h2r<R1, R2, HF_FLUX, false>;
  else if (k.form == HF_JAC) h2 = sp ? k_h2r<R1, R2, HF_JAC, true> : k_h2r<R1, R2, HF_JAC, false>;
  cudaFuncSetAttribute(h2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
  cudaFuncSetAttribute(k_h3r<R1, R2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
  prof.begin("h1_col_ifft_f32", st);
  k_h1r<R1, R2><<<dim3((k.cols_in + CB - 1) / CB, k.levels), 128, sm1, st>>>(k);
  prof.end(st);
  prof.begin("h2_row_products_f32", st);
  h2<<<dim3((N / 2 + 4 * G - 1) / (4 * G), k.levels), 128, sm2, st>>>(k);
  prof.end(st);
  prof.begin("h3_col_fft_f32", st);
  k_h3r<R1, R2><<<dim3((k.Mc + CB - 1) / CB, k.levels), 128, sm3, st>>>(k);
  prof.end(st);
  return cudaGetLastError();
}

}  // namespace

bool horizontal_reg_supported(int N) { return N == 64 || N == 128 || N == 256; }

cudaError_t launch_horizontal_f32_reg(const Params& p, const Tables& t, Work& w,
                                      const HorizArgsT<float2, float2>& a, cudaStream_t st,
                                      int* nlaunch) {
  const Dims& d = p.d;
  if (!horizontal_reg_supported(d.Nh) || d.pad) return cudaErrorNotSupported;
  HR k{};
  k.Nx = d.Nx; k.Nk = d.Nk; k.K = d.K; k.Mr = d.Mr; k.Mc = d.Mc; k.M = d.M;
  k.N = d.Nh;
  k.levels = a.levels;
  k.full_in = a.full_in;
  k.full_out = a.full_out;
  k.rows_in = a.full_in ? d.Nx : d.Mr;
  k.cols_in = a.full_in ? d.Nk : d.Mc;
  k.form = a.form;
  k.sponge = a.sponge || a.form == HF_SPONGE;
  k.eta = a.eta;
  k.psi_derived = a.psi_derived;
  if (a.form == HF_FLUX) { k.nf1 = 5; k.ng = 6; }
  else if (a.form == HF_JAC) { k.nf1 = k.sponge ? 11 : 8; k.ng = 3; }
  else { k.nf1 = 1; k.ng = 1; }
  k.scale = (float)(1.0 / ((double)d.Nh * (double)d.Nx));
  k.psi = a.psi; k.q = a.q; k.w = a.w; k.th = a.th;
  k.kx_full = t.kx_f; k.ky_full = t.ky_f; k.inv_denom = t.inv_denom;
  k.eta_c = t.eta_f; k.sponge_phys = t.sponge_f; k.eta_phys = t.eta_phys_f;
  k.eta_x = t.eta_x_f; k.eta_y = t.eta_y_f;
  k.eta_grad = k.eta && k.eta_x != nullptr && k.eta_y != nullptr;
  k.tw = t.tw_f;
  k.Aq = a.Aq; k.Aw = a.Aw; k.Ath = a.Ath;
  const size_t need1 = (size_t)k.nf1 * a.levels * k.cols_in * d.Nh;
  const size_t need2 = (size_t)k.ng * a.levels * d.Mc * d.Nh;
  const size_t cap1 = w.x1_elems * sizeof(double2) / sizeof(float2);
  const size_t cap2 = w.x2_elems * sizeof(double2) / sizeof(float2);
  if (need1 > cap1 || need2 > cap2) return cudaErrorInvalidValue;
  k.x1 = reinterpret_cast<float2*>(w.x1);
  k.x2 = reinterpret_cast<float2*>(w.x2);
  cudaError_t e;
  if (d.Nh == 256) e = launch_reg<16, 16>(k, st, w.prof);
  else if (d.Nh == 128) e = launch_reg<8, 16>(k, st, w.prof);
  else e = launch_reg<8, 8>(k, st, w.prof);
  if (nlaunch) *nlaunch += 3;
  return e;
}

}  // namespace nhqg

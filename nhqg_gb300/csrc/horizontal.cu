// Dealiased horizontal products (FP64 or FP32), three kernels per call.
//
// Reference semantics, 2/3 rule: nhqg/spectral.py:307-328 (flux form: D =
// i kx F(u f) + i ky F(v f) with u = -psi_y, v = psi_x), :281-304 (Jacobian
// form J = psi_x f_y - psi_y f_x), :53-60 (sponge mask * rfft2(sigma *
// irfft2 f)), each masked to |kx|, ky <= Nx/3, batched over levels
// (:331-358).  3/2 rule: the same products on the zero-padded N = 3Nx/2 grid
// (:18-50 pad / truncate, :63-75 sponge, :147-253 products): the transforms
// below run at length N, the input spectra enter at their padded rows, the
// outputs are read back at the kept rows, and the (N/Nx)^2 of the truncation
// is folded into the input scale (1/(N Nx) per factor).
//
//   H1  per (level, ky column): inverse complex FFT over kx of the derived
//       spectra (u, v, q+eta, w, theta, or the Jacobian's derivatives) -- only
//       the stored ky columns exist, so only Mc columns are transformed.
//   H2  per (level, pair of x rows): two real rows share one complex FFT
//       (c2r via the Hermitian extension, numpy irfft semantics: the imaginary
//       parts of the ky=0 / Nyquist bins are ignored), pointwise products,
//       two products share one forward complex FFT, the i*ky factor and the
//       sponge term are applied to the ky <= K outputs.
//   H3  per (level, ky column): forward complex FFT over x, combine
//       i kx G + H, keep the in-band kx rows.
// Scaling: numpy's irfft2 carries 1/N^2, folded into H1's input spectra
// together with the truncation's (N/Nx)^2.
#include <algorithm>

#include "engine.h"

namespace nhqg {

namespace {

template <typename C, typename CI>
struct HK {
  using T = decltype(C().x);
  // geometry
  int Nx, Nk, K, Mr, Mc, M;
  int N;   // transform length: Nx (2/3 rule) or the padded 3Nx/2 (3/2 rule)
  int sx;  // shared-memory stride of one FFT sequence (N plus FP32 padding)
  int levels;
  int rows_in, cols_in;  // input plane extent (compact Mr x Mc or full Nx x Nk)
  bool full_in, full_out;
  int form, nf1, nprod, ng;
  bool sponge, eta, psi_derived;
  // FP32 products: q enters without eta and the trap term is u . grad(eta)
  // from the tables eta_x, eta_y (added to the q sponge slot's product)
  bool eta_grad;
  const T *eta_x, *eta_y;
  T scale;  // 1/(N Nx)
  FftPlan plan;
  const CI *psi, *q, *w, *th;
  const T *kx_full, *ky_full;
  const double* inv_denom;  // compact [M]
  const C* eta_c;           // compact eta [M]
  const T *sponge_phys, *eta_phys;
  const C* tw;
  const int* perm;
  C *x1, *x2;
  C *Aq, *Aw, *Ath;
};

template <typename C, typename CI>
__device__ __forceinline__ C to_c(CI v) { C r; r.x = v.x; r.y = v.y; return r; }

// FP32 FFT sequences carry one padding element every 8 (fft_pad) so that the
// strided late passes spread over the shared-memory banks; the FP64 kernels,
// bound by the FP64 pipe, keep the dense layout
template <typename C>
__host__ __device__ constexpr int pad_shift() { return sizeof(C) == sizeof(float2) ? 3 : 0; }

// H1 -> H2 -> H3 intermediates, pair-major: [field][level][x/2][column][x%2]
template <typename K>
__device__ __forceinline__ size_t xidx(const K& k, int f, int lev, int pair, int c, int cols) {
  return ((((size_t)f * k.levels + lev) * (k.N / 2) + pair) * cols + c) * 2;
}

template <typename K>
__device__ __forceinline__ int plane_index(const K& k, int r, int c) {
  return r * k.cols_in + c;
}

template <typename K, typename C>
__device__ __forceinline__ void load_tables(const K& k, C* tw_s, int* perm_s) {
  for (int i = threadIdx.x; i < k.N; i += blockDim.x) {
    tw_s[i] = k.tw[i];
    perm_s[i] = k.perm[i];
  }
}

// ---------------------------------------------------------------- H1
template <typename C, typename CI>
__global__ void __launch_bounds__(256) k_h1(HK<C, CI> k, int CB) {
  using T = decltype(C().x);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw_s = reinterpret_cast<C*>(smem_raw);
  int* perm_s = reinterpret_cast<int*>(tw_s + k.N);
  C* seq = reinterpret_cast<C*>(perm_s + ((k.N + 3) / 4) * 4);
  const int lev = blockIdx.y;
  const int c0 = blockIdx.x * CB;
  const int ncb = min(CB, k.cols_in - c0);
  const int nseq = k.nf1 * CB;
  load_tables(k, tw_s, perm_s);
  constexpr int PS = pad_shift<C>();
  for (int i = threadIdx.x; i < nseq * k.sx; i += blockDim.x) seq[i] = gmk<C>(T(0), T(0));
  __syncthreads();

  const size_t plane = (size_t)k.rows_in * k.cols_in;
  for (int i = threadIdx.x; i < k.rows_in * ncb; i += blockDim.x) {
    const int r = i / ncb, cc = i - r * ncb, c = c0 + cc;
    const int kf = k.full_in ? r : full_row(r, k.K, k.Mr, k.Nx);
    const size_t off = (size_t)lev * plane + plane_index(k, r, c);
    const T kxs = k.kx_full[kf] * k.scale;
    const T kys = k.ky_full[c] * k.scale;
    const int pos = perm_s[padded_row(kf, k.Nx, k.N)];
    C* s0 = seq + (size_t)cc * k.sx + fft_pad<PS>(pos);
    const size_t fs = (size_t)CB * k.sx;  // stride between fields
    if (k.form == HF_SPONGE) {
      s0[0] = gscale(to_c<C>(k.q[off]), k.scale);
      continue;
    }
    C qv = to_c<C>(k.q[off]);
    C psi;
    if (k.psi_derived) {
      const int m = r * k.Mc + c;  // compact only
      psi = gscale(qv, (T)(-k.inv_denom[m]));
    } else {
      psi = to_c<C>(k.psi[off]);
    }
    if (k.eta && !k.eta_grad) qv = gadd(qv, k.eta_c[r * k.Mc + c]);
    const C wv = to_c<C>(k.w[off]), tv = to_c<C>(k.th[off]);
    if (k.form == HF_FLUX) {
      // u = -i ky psi, v = i kx psi
      s0[0] = gmk<C>(kys * psi.y, -kys * psi.x);
      s0[fs] = gmk<C>(-kxs * psi.y, kxs * psi.x);
      s0[2 * fs] = gscale(qv, k.scale);
      s0[3 * fs] = gscale(wv, k.scale);
      s0[4 * fs] = gscale(tv, k.scale);
    } else {  // Jacobian: psi_x, psi_y, q_x, q_y, w_x, w_y, t_x, t_y [, q, w, t]
      s0[0] = gmk<C>(-kxs * psi.y, kxs * psi.x);
      s0[fs] = gmk<C>(-kys * psi.y, kys * psi.x);
      s0[2 * fs] = gmk<C>(-kxs * qv.y, kxs * qv.x);
      s0[3 * fs] = gmk<C>(-kys * qv.y, kys * qv.x);
      s0[4 * fs] = gmk<C>(-kxs * wv.y, kxs * wv.x);
      s0[5 * fs] = gmk<C>(-kys * wv.y, kys * wv.x);
      s0[6 * fs] = gmk<C>(-kxs * tv.y, kxs * tv.x);
      s0[7 * fs] = gmk<C>(-kys * tv.y, kys * tv.x);
      if (k.sponge) {
        s0[8 * fs] = gscale(qv, k.scale);
        s0[9 * fs] = gscale(wv, k.scale);
        s0[10 * fs] = gscale(tv, k.scale);
      }
    }
  }
  __syncthreads();
  fft_dit_inv<C, PS>(seq, nseq, k.sx, k.plan, tw_s);
  // pair-major output: consecutive threads take (x parity, column), so the
  // row pairs H2 reads are contiguous
  const int half = k.N / 2;
  for (int i = threadIdx.x; i < k.nf1 * ncb * k.N; i += blockDim.x) {
    const int par = i & 1, r2 = i >> 1;
    const int cc = r2 % ncb, r3 = r2 / ncb;
    const int pp = r3 % half, f = r3 / half;
    const int x = 2 * pp + par;
    k.x1[xidx(k, f, lev, pp, c0 + cc, k.cols_in) + par] = seq[((size_t)f * CB + cc) * k.sx + fft_pad<PS>(x)];
  }
}

// ---------------------------------------------------------------- H2
template <typename C, typename CI>
__global__ void __launch_bounds__(256) k_h2(HK<C, CI> k, int RB) {
  using T = decltype(C().x);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw_s = reinterpret_cast<C*>(smem_raw);
  int* perm_s = reinterpret_cast<int*>(tw_s + k.N);
  C* in = reinterpret_cast<C*>(perm_s + ((k.N + 3) / 4) * 4);
  constexpr int PS = pad_shift<C>();
  const int NPR = RB / 2;
  C* pr = in + (size_t)k.nf1 * NPR * k.sx;
  const int lev = blockIdx.y;
  const int x0 = blockIdx.x * RB;
  load_tables(k, tw_s, perm_s);
  for (int i = threadIdx.x; i < k.nf1 * NPR * k.sx; i += blockDim.x) in[i] = gmk<C>(T(0), T(0));
  __syncthreads();
  const int half = k.N / 2;
  // Hermitian-extended spectra of row pairs (a, b): Z = Xa + i Xb
  for (int i = threadIdx.x; i < k.nf1 * NPR * k.cols_in; i += blockDim.x) {
    const int c = i % k.cols_in;
    const int rest = i / k.cols_in;
    const int p = rest % NPR, f = rest / NPR;
    const int xa = x0 + 2 * p;
    const size_t base = xidx(k, f, lev, xa >> 1, c, k.cols_in);
    const C A = k.x1[base], B = k.x1[base + 1];
    C* s = in + ((size_t)f * NPR + p) * k.sx;
    if (c == 0 || c == half) {
      s[fft_pad<PS>(perm_s[c])] = gmk<C>(A.x, B.x);
    } else {
      s[fft_pad<PS>(perm_s[c])] = gmk<C>(A.x - B.y, A.y + B.x);
      s[fft_pad<PS>(perm_s[k.N - c])] = gmk<C>(A.x + B.y, B.x - A.y);
    }
  }
  __syncthreads();
  fft_dit_inv<C, PS>(in, k.nf1 * NPR, k.sx, k.plan, tw_s);
  // pointwise products, two rows per complex lane
  const size_t fs = (size_t)NPR * k.sx;
  for (int i = threadIdx.x; i < NPR * k.N; i += blockDim.x) {
    const int y = i % k.N, p = i / k.N;
    const int xa = x0 + 2 * p;
    const C* s = in + (size_t)p * k.sx + fft_pad<PS>(y);
    C* o = pr + (size_t)p * k.sx + fft_pad<PS>(y);
    T sa = 0, sb = 0, ea = 0, eb = 0, gxa = 0, gxb = 0, gya = 0, gyb = 0;
    if (k.sponge) {
      sa = k.sponge_phys[(size_t)xa * k.N + y];
      sb = k.sponge_phys[(size_t)(xa + 1) * k.N + y];
      if (k.eta && !k.eta_grad) {
        ea = k.eta_phys[(size_t)xa * k.N + y];
        eb = k.eta_phys[(size_t)(xa + 1) * k.N + y];
      }
    }
    if (k.eta_grad) {
      gxa = k.eta_x[(size_t)xa * k.N + y];
      gxb = k.eta_x[(size_t)(xa + 1) * k.N + y];
      gya = k.eta_y[(size_t)xa * k.N + y];
      gyb = k.eta_y[(size_t)(xa + 1) * k.N + y];
    }
    if (k.form == HF_FLUX) {
      const C u = s[0], v = s[fs], Q = s[2 * fs], W = s[3 * fs], Th = s[4 * fs];
      o[0] = gmk<C>(u.x * Q.x, u.y * Q.y);
      o[fs] = gmk<C>(v.x * Q.x, v.y * Q.y);
      o[2 * fs] = gmk<C>(u.x * W.x, u.y * W.y);
      o[3 * fs] = gmk<C>(v.x * W.x, v.y * W.y);
      o[4 * fs] = gmk<C>(u.x * Th.x, u.y * Th.y);
      o[5 * fs] = gmk<C>(v.x * Th.x, v.y * Th.y);
      if (k.sponge || k.eta_grad) {
        // sigma (q - eta), or with the gradient form sigma q + u . grad(eta)
        T qa = sa * (Q.x - ea), qb = sb * (Q.y - eb);
        if (k.eta_grad) {
          qa = fma(u.x, gxa, fma(v.x, gya, qa));
          qb = fma(u.y, gxb, fma(v.y, gyb, qb));
        }
        o[6 * fs] = gmk<C>(qa, qb);
        o[7 * fs] = gmk<C>(sa * W.x, sb * W.y);
        o[8 * fs] = gmk<C>(sa * Th.x, sb * Th.y);
      }
    } else if (k.form == HF_JAC) {
      const C px = s[0], py = s[fs];
      for (int f = 0; f < 3; ++f) {
        const C fx = s[(2 + 2 * f) * fs], fy = s[(3 + 2 * f) * fs];
        T ja = fma(px.x, fy.x, -py.x * fx.x);
        T jb = fma(px.y, fy.y, -py.y * fx.y);
        if (k.sponge) {
          const C F = s[(8 + f) * fs];
          const T Fa = (f == 0) ? F.x - ea : F.x;
          const T Fb = (f == 0) ? F.y - eb : F.y;
          ja = fma(sa, Fa, ja);
          jb = fma(sb, Fb, jb);
        }
        if (f == 0 && k.eta_grad) {  // J[psi, eta] = psi_x eta_y - psi_y eta_x
          ja = fma(px.x, gya, fma(-py.x, gxa, ja));
          jb = fma(px.y, gyb, fma(-py.y, gxb, jb));
        }
        o[f * fs] = gmk<C>(ja, jb);
      }
    } else {  // sponge-only product
      const C F = s[0];
      o[0] = gmk<C>(sa * F.x, sb * F.y);
    }
  }
  __syncthreads();
  fft_dif_fwd<C, PS>(pr, k.nprod * NPR, k.sx, k.plan, tw_s);
  // split the paired spectra, apply i*ky / sponge, write ky <= K
  for (int i = threadIdx.x; i < k.ng * NPR * k.Mc; i += blockDim.x) {
    const int c = i % k.Mc;
    const int rest = i / k.Mc;
    const int p = rest % NPR, g = rest / NPR;
    const int xa = x0 + 2 * p;
    const int pa = fft_pad<PS>(perm_s[c]), pb = fft_pad<PS>(perm_s[c == 0 ? 0 : k.N - c]);
    auto split = [&](int prod, C& Xa, C& Xb) {
      const C* s = pr + ((size_t)prod * NPR + p) * k.sx;
      const C A = s[pa], B = s[pb];
      Xa = gmk<C>(T(0.5) * (A.x + B.x), T(0.5) * (A.y - B.y));
      Xb = gmk<C>(T(0.5) * (A.y + B.y), T(0.5) * (B.x - A.x));
    };
    C Ra, Rb;
    if (k.form == HF_FLUX) {
      const int f = g >> 1;
      if ((g & 1) == 0) {
        split(2 * f, Ra, Rb);
      } else {
        C Va, Vb;
        split(2 * f + 1, Va, Vb);
        const T ky = k.ky_full[c];
        Ra = gmk<C>(-ky * Va.y, ky * Va.x);
        Rb = gmk<C>(-ky * Vb.y, ky * Vb.x);
        if (k.sponge || k.eta_grad) {
          C Sa, Sb;
          split(6 + f, Sa, Sb);
          Ra = gadd(Ra, Sa);
          Rb = gadd(Rb, Sb);
        }
      }
    } else {
      split(g, Ra, Rb);
    }
    const size_t base = xidx(k, g, lev, xa >> 1, c, k.Mc);
    k.x2[base] = Ra;
    k.x2[base + 1] = Rb;
  }
}

// ---------------------------------------------------------------- H3
template <typename C, typename CI>
__global__ void __launch_bounds__(256) k_h3(HK<C, CI> k, int CB) {
  using T = decltype(C().x);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw_s = reinterpret_cast<C*>(smem_raw);
  int* perm_s = reinterpret_cast<int*>(tw_s + k.N);
  C* seq = reinterpret_cast<C*>(perm_s + ((k.N + 3) / 4) * 4);
  const int lev = blockIdx.y;
  const int c0 = blockIdx.x * CB;
  const int ncb = min(CB, k.Mc - c0);
  constexpr int PS = pad_shift<C>();
  load_tables(k, tw_s, perm_s);
  const int half = k.N / 2;
  for (int i = threadIdx.x; i < k.ng * ncb * k.N; i += blockDim.x) {
    const int par = i & 1, r2 = i >> 1;
    const int cc = r2 % ncb, r3 = r2 / ncb;
    const int pp = r3 % half, g = r3 / half;
    seq[((size_t)g * CB + cc) * k.sx + fft_pad<PS>(2 * pp + par)] = k.x2[xidx(k, g, lev, pp, c0 + cc, k.Mc) + par];
  }
  __syncthreads();
  fft_dif_fwd<C, PS>(seq, k.ng * CB, k.sx, k.plan, tw_s);
  const int nout = (k.form == HF_SPONGE) ? 1 : 3;
  for (int i = threadIdx.x; i < k.Mr * ncb; i += blockDim.x) {
    const int r = i / ncb, cc = i - r * ncb, c = c0 + cc;
    const int kf = full_row(r, k.K, k.Mr, k.Nx);
    const int pos = fft_pad<PS>(perm_s[padded_row(kf, k.Nx, k.N)]);
    const size_t oidx = k.full_out ? ((size_t)lev * k.Nx + kf) * k.Nk + c
                                   : (size_t)lev * k.M + (size_t)r * k.Mc + c;
    for (int f = 0; f < nout; ++f) {
      C val;
      if (k.form == HF_FLUX) {
        const C G = seq[((size_t)(2 * f) * CB + cc) * k.sx + pos];
        const C H = seq[((size_t)(2 * f + 1) * CB + cc) * k.sx + pos];
        const T kx = k.kx_full[kf];
        val = gmk<C>(fma(-kx, G.y, H.x), fma(kx, G.x, H.y));
      } else {
        val = seq[((size_t)f * CB + cc) * k.sx + pos];
      }
      C* out = (f == 0) ? k.Aq : (f == 1 ? k.Aw : k.Ath);
      out[oidx] = val;
    }
  }
}

// ---------------------------------------------------------------- physical maxima
// Row inverse transforms of H1's u, v, w, theta spectra (fields 0, 1, 3, 4 of
// the flux form), then per CTA the maxima of sqrt(u^2 + v^2), |w|, |theta|,
// |w theta| over its rows, merged with atomicMax on the bit patterns (the
// order of non-negative doubles).  FP64 (the reference's diagnostics).
__global__ void __launch_bounds__(256) k_hmax(HK<double2, double2> k, int RB,
                                              unsigned long long* __restrict__ maxima) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tw_s = reinterpret_cast<double2*>(smem_raw);
  int* perm_s = reinterpret_cast<int*>(tw_s + k.N);
  double2* in = reinterpret_cast<double2*>(perm_s + ((k.N + 3) / 4) * 4);
  __shared__ double red[4][8];
  const int NPR = RB / 2;
  const int lev = blockIdx.y;
  const int x0 = blockIdx.x * RB;
  load_tables(k, tw_s, perm_s);
  for (int i = threadIdx.x; i < 4 * NPR * k.N; i += blockDim.x) in[i] = make_double2(0.0, 0.0);
  __syncthreads();
  const int half = k.N / 2;
  const int src[4] = {0, 1, 3, 4};
  for (int i = threadIdx.x; i < 4 * NPR * k.cols_in; i += blockDim.x) {
    const int c = i % k.cols_in;
    const int rest = i / k.cols_in;
    const int p = rest % NPR, f = rest / NPR;
    const int xa = x0 + 2 * p;
    const size_t base = xidx(k, src[f], lev, xa >> 1, c, k.cols_in);
    const double2 A = k.x1[base], B = k.x1[base + 1];
    double2* sq = in + ((size_t)f * NPR + p) * k.N;
    if (c == 0 || c == half) {
      sq[perm_s[c]] = make_double2(A.x, B.x);
    } else {
      sq[perm_s[c]] = make_double2(A.x - B.y, A.y + B.x);
      sq[perm_s[k.N - c]] = make_double2(A.x + B.y, B.x - A.y);
    }
  }
  __syncthreads();
  fft_dit_inv<double2, 0>(in, 4 * NPR, k.N, k.plan, tw_s);
  double mu = 0.0, mw = 0.0, mt = 0.0, mwt = 0.0;
  const size_t fs = (size_t)NPR * k.N;
  for (int i = threadIdx.x; i < NPR * k.N; i += blockDim.x) {
    const double2 u = in[i], v = in[fs + i], w = in[2 * fs + i], t = in[3 * fs + i];
    mu = fmax(mu, fmax(sqrt(fma(u.x, u.x, v.x * v.x)), sqrt(fma(u.y, u.y, v.y * v.y))));
    mw = fmax(mw, fmax(fabs(w.x), fabs(w.y)));
    mt = fmax(mt, fmax(fabs(t.x), fabs(t.y)));
    mwt = fmax(mwt, fmax(fabs(w.x * t.x), fabs(w.y * t.y)));
  }
  double m4[4] = {mu, mw, mt, mwt};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int q = 0; q < 4; ++q) {
    double x = m4[q];
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
    if (lane == 0) red[q][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double x = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) x = fmax(x, red[threadIdx.x][q]);
    atomicMax(maxima + threadIdx.x, (unsigned long long)__double_as_longlong(x));
  }
}

template <typename C>
size_t table_bytes(int Nx) { return (size_t)Nx * sizeof(C) + (size_t)((Nx + 3) / 4) * 4 * sizeof(int); }

template <typename C, typename CI>
cudaError_t launch_horizontal_t(const Params& p, const HTables<C>& t, Work& w, const HorizArgsT<C, CI>& a,
                                cudaStream_t st, int* nlaunch) {
  using T = decltype(C().x);
  HK<C, CI> k;
  const Dims& d = p.d;
  k.Nx = d.Nx; k.Nk = d.Nk; k.K = d.K; k.Mr = d.Mr; k.Mc = d.Mc; k.M = d.M;
  k.N = d.Nh;
  k.sx = pad_shift<C>() > 0 ? k.N + (k.N + 7) / 8 : k.N;
  k.levels = a.levels;
  k.full_in = a.full_in;
  k.full_out = a.full_out;
  k.rows_in = a.full_in ? d.Nx : d.Mr;
  k.cols_in = a.full_in ? d.Nk : d.Mc;
  k.form = a.form;
  k.sponge = a.sponge || a.form == HF_SPONGE;
  k.eta = a.eta;
  k.eta_grad = a.eta && t.eta_x != nullptr && t.eta_y != nullptr;
  k.eta_x = t.eta_x;
  k.eta_y = t.eta_y;
  k.psi_derived = a.psi_derived;
  if (a.form == HF_FLUX) { k.nf1 = 5; k.nprod = (k.sponge || k.eta_grad) ? 9 : 6; k.ng = 6; }
  else if (a.form == HF_JAC) { k.nf1 = k.sponge ? 11 : 8; k.nprod = 3; k.ng = 3; }
  else { k.nf1 = 1; k.nprod = 1; k.ng = 1; }
  k.scale = (T)(1.0 / ((double)d.Nh * (double)d.Nx));
  k.plan = p.plan;
  k.psi = a.psi; k.q = a.q; k.w = a.w; k.th = a.th;
  k.kx_full = t.kx_full; k.ky_full = t.ky_full; k.inv_denom = t.inv_denom;
  k.eta_c = t.eta; k.sponge_phys = t.sponge; k.eta_phys = t.eta_phys;
  k.tw = t.tw; k.perm = t.perm;
  k.Aq = a.Aq; k.Aw = a.Aw; k.Ath = a.Ath;
  const size_t need1 = (size_t)k.nf1 * a.levels * k.cols_in * d.Nh;
  const size_t need2 = (size_t)k.ng * a.levels * d.Mc * d.Nh;
  const size_t cap1 = w.x1_elems * sizeof(double2) / sizeof(C);
  const size_t cap2 = w.x2_elems * sizeof(double2) / sizeof(C);
  if (need1 > cap1 || need2 > cap2) return cudaErrorInvalidValue;
  k.x1 = reinterpret_cast<C*>(w.x1);
  k.x2 = reinterpret_cast<C*>(w.x2);

  const size_t tb = table_bytes<C>(d.Nh);
  const size_t budget = 200 * 1024;
  // FP64: the FP64 pipe is the limit, large tiles amortise the tables; FP32:
  // shared-memory latency is the limit, small tiles keep 4 CTAs per SM
  const int pi = sizeof(T) == 8 ? 0 : 1;
  const size_t tile = (size_t)1024 * (p.h_col_kib[pi] > 0 ? p.h_col_kib[pi] : (pi == 0 ? 96 : 44));
  const size_t budget2 = (size_t)1024 * (p.h_row_kib[pi] > 0 ? p.h_row_kib[pi] : (pi == 0 ? 200 : 52));
  const size_t seqb = (size_t)k.sx * sizeof(C);  // bytes of one FFT sequence
  int CB1 = (int)(tile / ((size_t)k.nf1 * seqb));
  CB1 = max(1, min(CB1, k.cols_in));
  size_t sm1 = tb + (size_t)k.nf1 * CB1 * seqb;
  if (sm1 > budget) return cudaErrorInvalidConfiguration;
  int RB = 2;
  while (RB * 2 <= 16 && d.Nh % (RB * 2) == 0 &&
         tb + (size_t)(k.nf1 + k.nprod) * RB * seqb <= budget2)
    RB *= 2;
  size_t sm2 = tb + (size_t)(k.nf1 + k.nprod) * (RB / 2) * seqb;
  if (sm2 > budget) return cudaErrorInvalidConfiguration;
  int CB3 = (int)(tile / ((size_t)k.ng * seqb));
  CB3 = max(1, min(CB3, d.Mc));
  size_t sm3 = tb + (size_t)k.ng * CB3 * seqb;
  if (sm3 > budget) return cudaErrorInvalidConfiguration;

  cudaFuncSetAttribute(k_h1<C, CI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  cudaFuncSetAttribute(k_h2<C, CI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  cudaFuncSetAttribute(k_h3<C, CI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  dim3 g1((k.cols_in + CB1 - 1) / CB1, a.levels);
  w.prof.begin(sizeof(T) == 4 ? "h1_col_ifft_f32" : "h1_col_ifft", st);
  k_h1<C, CI><<<g1, 256, sm1, st>>>(k, CB1);
  w.prof.end(st);
  dim3 g2(d.Nh / RB, a.levels);
  w.prof.begin(sizeof(T) == 4 ? "h2_row_products_f32" : "h2_row_products", st);
  k_h2<C, CI><<<g2, 256, sm2, st>>>(k, RB);
  w.prof.end(st);
  dim3 g3((d.Mc + CB3 - 1) / CB3, a.levels);
  w.prof.begin(sizeof(T) == 4 ? "h3_col_fft_f32" : "h3_col_fft", st);
  k_h3<C, CI><<<g3, 256, sm3, st>>>(k, CB3);
  w.prof.end(st);
  if (nlaunch) *nlaunch += 3;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_horizontal(const Params& p, const Tables& t, Work& w, const HorizArgs& a,
                              cudaStream_t st, int* nlaunch) {
  HTables<double2> ht{t.kx_full, t.ky_full, t.inv_denom, t.eta, t.sponge, t.eta_phys, t.tw, t.perm};
  HorizArgsT<double2, double2> at{a.form, a.sponge, a.eta, a.full_in, a.full_out, a.psi_derived,
                                  a.levels, a.psi, a.q, a.w, a.th, a.Aq, a.Aw, a.Ath};
  return launch_horizontal_t<double2, double2>(p, ht, w, at, st, nlaunch);
}

cudaError_t launch_phys_maxima(const Params& p0, const Tables& t, Work& w, const double2* qn,
                               const double2* wn, const double2* tn, unsigned long long* maxima,
                               cudaStream_t st) {
  // the context's products may run at Npad (3/2 rule): transforms of length Nx here
  Params p = p0;
  p.d.Nh = p.d.Nx;
  p.plan = p0.plan_nx;
  if (p.plan.npass <= 0) return cudaErrorInvalidValue;
  HTables<double2> ht{t.kx_full, t.ky_full, t.inv_denom, nullptr, nullptr, nullptr, t.tw_nx, t.perm_nx};
  HK<double2, double2> k{};
  const Dims& d = p.d;
  k.Nx = d.Nx; k.Nk = d.Nk; k.K = d.K; k.Mr = d.Mr; k.Mc = d.Mc; k.M = d.M;
  k.N = d.Nx;
  k.sx = k.N;
  k.levels = d.P;
  k.full_in = false;
  k.full_out = false;
  k.rows_in = d.Mr;
  k.cols_in = d.Mc;
  k.form = HF_FLUX;
  k.sponge = false; k.eta = false; k.psi_derived = true;
  k.nf1 = 5; k.nprod = 6; k.ng = 6;
  k.scale = 1.0 / ((double)d.Nx * (double)d.Nx);
  k.plan = p.plan;
  k.psi = nullptr; k.q = qn; k.w = wn; k.th = tn;
  k.kx_full = ht.kx_full; k.ky_full = ht.ky_full; k.inv_denom = ht.inv_denom;
  k.eta_c = nullptr; k.sponge_phys = nullptr; k.eta_phys = nullptr;
  k.tw = ht.tw; k.perm = ht.perm;
  k.Aq = k.Aw = k.Ath = nullptr;
  if ((size_t)k.nf1 * d.P * k.cols_in * k.N > w.x1_elems) return cudaErrorInvalidValue;
  k.x1 = w.x1;
  k.x2 = nullptr;
  cudaError_t e = cudaMemsetAsync(maxima, 0, kDiagMaxima * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  const size_t tb = table_bytes<double2>(k.N);
  const size_t seqb = (size_t)k.N * sizeof(double2);
  const size_t budget = 200 * 1024;
  int CB1 = (int)((size_t)96 * 1024 / ((size_t)k.nf1 * seqb));
  CB1 = std::max(1, std::min(CB1, k.cols_in));
  const size_t sm1 = tb + (size_t)k.nf1 * CB1 * seqb;
  int RB = 2;
  while (RB * 2 <= 16 && k.N % (RB * 2) == 0 && tb + (size_t)4 * (RB * 2 / 2) * seqb <= 96 * 1024) RB *= 2;
  const size_t sm2 = tb + (size_t)4 * (RB / 2) * seqb;
  if (sm1 > budget || sm2 > budget) return cudaErrorInvalidConfiguration;
  cudaFuncSetAttribute(k_h1<double2, double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  cudaFuncSetAttribute(k_hmax, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  w.prof.begin("diag_maxima", st);
  k_h1<double2, double2><<<dim3((k.cols_in + CB1 - 1) / CB1, k.levels), 256, sm1, st>>>(k, CB1);
  k_hmax<<<dim3(k.N / RB, k.levels), 256, sm2, st>>>(k, RB, maxima);
  w.prof.end(st);
  return cudaGetLastError();
}

cudaError_t launch_horizontal_f32(const Params& p, const Tables& t, Work& w,
                                  const HorizArgsT<float2, float2>& a, cudaStream_t st,
                                  int* nlaunch) {
  if (p.reg_fft && !p.d.pad && horizontal_reg_supported(p.d.Nh))
    return launch_horizontal_f32_reg(p, t, w, a, st, nlaunch);
  HTables<float2> ht{t.kx_f, t.ky_f, t.inv_denom, t.eta_f, t.sponge_f, t.eta_phys_f, t.tw_f, t.perm,
                     t.eta_x_f, t.eta_y_f};
  return launch_horizontal_t<float2, float2>(p, ht, w, a, st, nlaunch);
}

}  // namespace nhqg

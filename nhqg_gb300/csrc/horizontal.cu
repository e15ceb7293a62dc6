// 2/3-rule dealiased horizontal products (FP64), three kernels per call.
//
// Reference semantics: nhqg/spectral.py:307-328 (flux form: D = i kx F(u f) +
// i ky F(v f) with u = -psi_y, v = psi_x), :281-304 (Jacobian form
// J = psi_x f_y - psi_y f_x), :53-60 (sponge mask * rfft2(sigma * irfft2 f)),
// each masked to |kx|, ky <= Nx/3, batched over levels (:331-358).
//
//   H1  per (level, ky column): inverse complex FFT over kx of the derived
//       spectra (u, v, q+eta, w, theta, or the Jacobian's derivatives) -- only
//       the in-band ky columns exist, so only Mc of the Nk columns are
//       transformed.
//   H2  per (level, pair of x rows): two real rows share one complex FFT
//       (c2r via the Hermitian extension, numpy irfft semantics: the imaginary
//       parts of the ky=0 / Nyquist bins are ignored), pointwise products,
//       two products share one forward complex FFT, the i*ky factor and the
//       sponge term are applied to the ky <= K outputs.
//   H3  per (level, ky column): forward complex FFT over x, combine
//       i kx G + H, keep the in-band kx rows.
// Scaling: numpy's irfft2 carries 1/Nx^2, folded into H1's input spectra.
#include "engine.h"

namespace nhqg {

namespace {

struct HK {
  // geometry
  int Nx, Nk, K, Mr, Mc, M;
  int levels;
  int rows_in, cols_in;  // input plane extent (compact Mr x Mc or full Nx x Nk)
  bool full_in, full_out;
  int form, nf1, nprod, ng;
  bool sponge, eta, psi_derived;
  double scale;  // 1/Nx^2
  FftPlan plan;
  const double2 *psi, *q, *w, *th;
  const double *kx_full, *ky_full, *inv_denom;  // inv_denom compact [M]
  const double2* eta_c;                          // compact eta [M]
  const double *sponge_phys, *eta_phys;
  const double2* tw;
  const int* perm;
  double2 *x1, *x2;
  double2 *Aq, *Aw, *Ath;
};

__device__ __forceinline__ int plane_index(const HK& k, int r, int c) {
  return r * k.cols_in + c;
}

__device__ __forceinline__ void load_tables(const HK& k, double2* tw_s, int* perm_s) {
  for (int i = threadIdx.x; i < k.Nx; i += blockDim.x) {
    tw_s[i] = k.tw[i];
    perm_s[i] = k.perm[i];
  }
}

// ---------------------------------------------------------------- H1
__global__ void __launch_bounds__(256) k_h1(HK k, int CB) {
  extern __shared__ double2 smem[];
  double2* tw_s = smem;
  int* perm_s = reinterpret_cast<int*>(tw_s + k.Nx);
  double2* seq = tw_s + k.Nx + (k.Nx + 1) / 2;  // after perm (ints packed 2 per double2)
  const int lev = blockIdx.y;
  const int c0 = blockIdx.x * CB;
  const int ncb = min(CB, k.cols_in - c0);
  const int nseq = k.nf1 * CB;
  load_tables(k, tw_s, perm_s);
  for (int i = threadIdx.x; i < nseq * k.Nx; i += blockDim.x) seq[i] = czero();
  __syncthreads();

  const size_t plane = (size_t)k.rows_in * k.cols_in;
  for (int i = threadIdx.x; i < k.rows_in * ncb; i += blockDim.x) {
    const int r = i / ncb, cc = i - r * ncb, c = c0 + cc;
    const int kf = k.full_in ? r : full_row(r, k.K, k.Nx);
    const size_t off = (size_t)lev * plane + plane_index(k, r, c);
    const double kxs = k.kx_full[kf] * k.scale;
    const double kys = k.ky_full[c] * k.scale;
    const int pos = perm_s[kf];
    double2* s0 = seq + (size_t)cc * k.Nx + pos;
    const size_t fs = (size_t)CB * k.Nx;  // stride between fields
    if (k.form == HF_SPONGE) {
      s0[0] = cscale(k.q[off], k.scale);
      continue;
    }
    double2 qv = k.q[off];
    double2 psi;
    if (k.psi_derived) {
      const int m = r * k.Mc + c;  // compact only
      psi = cscale(qv, -k.inv_denom[m]);
    } else {
      psi = k.psi[off];
    }
    if (k.eta) qv = cadd(qv, k.eta_c[r * k.Mc + c]);
    const double2 wv = k.w[off], tv = k.th[off];
    if (k.form == HF_FLUX) {
      // u = -i ky psi, v = i kx psi
      s0[0] = make_double2(kys * psi.y, -kys * psi.x);
      s0[fs] = make_double2(-kxs * psi.y, kxs * psi.x);
      s0[2 * fs] = cscale(qv, k.scale);
      s0[3 * fs] = cscale(wv, k.scale);
      s0[4 * fs] = cscale(tv, k.scale);
    } else {  // Jacobian: psi_x, psi_y, q_x, q_y, w_x, w_y, t_x, t_y [, q, w, t]
      s0[0] = make_double2(-kxs * psi.y, kxs * psi.x);
      s0[fs] = make_double2(-kys * psi.y, kys * psi.x);
      s0[2 * fs] = make_double2(-kxs * qv.y, kxs * qv.x);
      s0[3 * fs] = make_double2(-kys * qv.y, kys * qv.x);
      s0[4 * fs] = make_double2(-kxs * wv.y, kxs * wv.x);
      s0[5 * fs] = make_double2(-kys * wv.y, kys * wv.x);
      s0[6 * fs] = make_double2(-kxs * tv.y, kxs * tv.x);
      s0[7 * fs] = make_double2(-kys * tv.y, kys * tv.x);
      if (k.sponge) {
        s0[8 * fs] = cscale(qv, k.scale);
        s0[9 * fs] = cscale(wv, k.scale);
        s0[10 * fs] = cscale(tv, k.scale);
      }
    }
  }
  __syncthreads();
  fft_dit_inv(seq, nseq, k.Nx, k.plan, tw_s);
  for (int i = threadIdx.x; i < k.nf1 * ncb * k.Nx; i += blockDim.x) {
    const int x = i % k.Nx;
    const int rest = i / k.Nx;
    const int cc = rest % ncb, f = rest / ncb;
    k.x1[(((size_t)f * k.levels + lev) * k.cols_in + (c0 + cc)) * k.Nx + x] =
        seq[((size_t)f * CB + cc) * k.Nx + x];
  }
}

// ---------------------------------------------------------------- H2
__global__ void __launch_bounds__(256) k_h2(HK k, int RB) {
  extern __shared__ double2 smem[];
  double2* tw_s = smem;
  int* perm_s = reinterpret_cast<int*>(tw_s + k.Nx);
  double2* in = tw_s + k.Nx + (k.Nx + 1) / 2;
  const int NPR = RB / 2;
  double2* pr = in + (size_t)k.nf1 * NPR * k.Nx;
  const int lev = blockIdx.y;
  const int x0 = blockIdx.x * RB;
  load_tables(k, tw_s, perm_s);
  for (int i = threadIdx.x; i < k.nf1 * NPR * k.Nx; i += blockDim.x) in[i] = czero();
  __syncthreads();
  const int half = k.Nx / 2;
  // Hermitian-extended spectra of row pairs (a, b): Z = Xa + i Xb
  for (int i = threadIdx.x; i < k.nf1 * NPR * k.cols_in; i += blockDim.x) {
    const int c = i % k.cols_in;
    const int rest = i / k.cols_in;
    const int p = rest % NPR, f = rest / NPR;
    const int xa = x0 + 2 * p;
    const size_t base = (((size_t)f * k.levels + lev) * k.cols_in + c) * k.Nx;
    const double2 A = k.x1[base + xa], B = k.x1[base + xa + 1];
    double2* s = in + ((size_t)f * NPR + p) * k.Nx;
    if (c == 0 || c == half) {
      s[perm_s[c]] = make_double2(A.x, B.x);
    } else {
      s[perm_s[c]] = make_double2(A.x - B.y, A.y + B.x);
      s[perm_s[k.Nx - c]] = make_double2(A.x + B.y, B.x - A.y);
    }
  }
  __syncthreads();
  fft_dit_inv(in, k.nf1 * NPR, k.Nx, k.plan, tw_s);
  // pointwise products, two rows per complex lane
  const size_t fs = (size_t)NPR * k.Nx;
  for (int i = threadIdx.x; i < NPR * k.Nx; i += blockDim.x) {
    const int y = i % k.Nx, p = i / k.Nx;
    const int xa = x0 + 2 * p;
    const double2* s = in + (size_t)p * k.Nx + y;
    double2* o = pr + (size_t)p * k.Nx + y;
    double sa = 0.0, sb = 0.0, ea = 0.0, eb = 0.0;
    if (k.sponge) {
      sa = k.sponge_phys[(size_t)xa * k.Nx + y];
      sb = k.sponge_phys[(size_t)(xa + 1) * k.Nx + y];
      if (k.eta) {
        ea = k.eta_phys[(size_t)xa * k.Nx + y];
        eb = k.eta_phys[(size_t)(xa + 1) * k.Nx + y];
      }
    }
    if (k.form == HF_FLUX) {
      const double2 u = s[0], v = s[fs], Q = s[2 * fs], W = s[3 * fs], T = s[4 * fs];
      o[0] = make_double2(u.x * Q.x, u.y * Q.y);
      o[fs] = make_double2(v.x * Q.x, v.y * Q.y);
      o[2 * fs] = make_double2(u.x * W.x, u.y * W.y);
      o[3 * fs] = make_double2(v.x * W.x, v.y * W.y);
      o[4 * fs] = make_double2(u.x * T.x, u.y * T.y);
      o[5 * fs] = make_double2(v.x * T.x, v.y * T.y);
      if (k.sponge) {
        o[6 * fs] = make_double2(sa * (Q.x - ea), sb * (Q.y - eb));
        o[7 * fs] = make_double2(sa * W.x, sb * W.y);
        o[8 * fs] = make_double2(sa * T.x, sb * T.y);
      }
    } else if (k.form == HF_JAC) {
      const double2 px = s[0], py = s[fs];
      for (int f = 0; f < 3; ++f) {
        const double2 fx = s[(2 + 2 * f) * fs], fy = s[(3 + 2 * f) * fs];
        double ja = fma(px.x, fy.x, -py.x * fx.x);
        double jb = fma(px.y, fy.y, -py.y * fx.y);
        if (k.sponge) {
          const double2 F = s[(8 + f) * fs];
          const double Fa = (f == 0) ? F.x - ea : F.x;
          const double Fb = (f == 0) ? F.y - eb : F.y;
          ja = fma(sa, Fa, ja);
          jb = fma(sb, Fb, jb);
        }
        o[f * fs] = make_double2(ja, jb);
      }
    } else {  // sponge-only product
      const double2 F = s[0];
      o[0] = make_double2(sa * F.x, sb * F.y);
    }
  }
  __syncthreads();
  fft_dif_fwd(pr, k.nprod * NPR, k.Nx, k.plan, tw_s);
  // split the paired spectra, apply i*ky / sponge, write ky <= K
  for (int i = threadIdx.x; i < k.ng * NPR * k.Mc; i += blockDim.x) {
    const int c = i % k.Mc;
    const int rest = i / k.Mc;
    const int p = rest % NPR, g = rest / NPR;
    const int xa = x0 + 2 * p;
    const int pa = perm_s[c], pb = perm_s[c == 0 ? 0 : k.Nx - c];
    auto split = [&](int prod, double2& Xa, double2& Xb) {
      const double2* s = pr + ((size_t)prod * NPR + p) * k.Nx;
      const double2 A = s[pa], B = s[pb];
      Xa = make_double2(0.5 * (A.x + B.x), 0.5 * (A.y - B.y));
      Xb = make_double2(0.5 * (A.y + B.y), 0.5 * (B.x - A.x));
    };
    double2 Ra, Rb;
    if (k.form == HF_FLUX) {
      const int f = g >> 1;
      if ((g & 1) == 0) {
        split(2 * f, Ra, Rb);
      } else {
        double2 Va, Vb;
        split(2 * f + 1, Va, Vb);
        const double ky = k.ky_full[c];
        Ra = make_double2(-ky * Va.y, ky * Va.x);
        Rb = make_double2(-ky * Vb.y, ky * Vb.x);
        if (k.sponge) {
          double2 Sa, Sb;
          split(6 + f, Sa, Sb);
          Ra = cadd(Ra, Sa);
          Rb = cadd(Rb, Sb);
        }
      }
    } else {
      split(g, Ra, Rb);
    }
    const size_t base = (((size_t)g * k.levels + lev) * k.Mc + c) * k.Nx;
    k.x2[base + xa] = Ra;
    k.x2[base + xa + 1] = Rb;
  }
}

// ---------------------------------------------------------------- H3
__global__ void __launch_bounds__(256) k_h3(HK k, int CB) {
  extern __shared__ double2 smem[];
  double2* tw_s = smem;
  int* perm_s = reinterpret_cast<int*>(tw_s + k.Nx);
  double2* seq = tw_s + k.Nx + (k.Nx + 1) / 2;
  const int lev = blockIdx.y;
  const int c0 = blockIdx.x * CB;
  const int ncb = min(CB, k.Mc - c0);
  load_tables(k, tw_s, perm_s);
  for (int i = threadIdx.x; i < k.ng * ncb * k.Nx; i += blockDim.x) {
    const int x = i % k.Nx;
    const int rest = i / k.Nx;
    const int cc = rest % ncb, g = rest / ncb;
    seq[((size_t)g * CB + cc) * k.Nx + x] =
        k.x2[(((size_t)g * k.levels + lev) * k.Mc + (c0 + cc)) * k.Nx + x];
  }
  __syncthreads();
  fft_dif_fwd(seq, k.ng * CB, k.Nx, k.plan, tw_s);
  const int nout = (k.form == HF_SPONGE) ? 1 : 3;
  for (int i = threadIdx.x; i < k.Mr * ncb; i += blockDim.x) {
    const int r = i / ncb, cc = i - r * ncb, c = c0 + cc;
    const int kf = full_row(r, k.K, k.Nx);
    const int pos = perm_s[kf];
    const size_t oidx = k.full_out ? ((size_t)lev * k.Nx + kf) * k.Nk + c
                                   : (size_t)lev * k.M + (size_t)r * k.Mc + c;
    for (int f = 0; f < nout; ++f) {
      double2 val;
      if (k.form == HF_FLUX) {
        const double2 G = seq[((size_t)(2 * f) * CB + cc) * k.Nx + pos];
        const double2 H = seq[((size_t)(2 * f + 1) * CB + cc) * k.Nx + pos];
        const double kx = k.kx_full[kf];
        val = make_double2(fma(-kx, G.y, H.x), fma(kx, G.x, H.y));
      } else {
        val = seq[((size_t)f * CB + cc) * k.Nx + pos];
      }
      double2* out = (f == 0) ? k.Aq : (f == 1 ? k.Aw : k.Ath);
      out[oidx] = val;
    }
  }
}

size_t table_bytes(int Nx) { return (size_t)Nx * sizeof(double2) + (size_t)((Nx + 1) / 2) * sizeof(double2); }

}  // namespace

cudaError_t launch_horizontal(const Params& p, const Tables& t, Work& w, const HorizArgs& a,
                              cudaStream_t st, int* nlaunch) {
  HK k;
  const Dims& d = p.d;
  k.Nx = d.Nx; k.Nk = d.Nk; k.K = d.K; k.Mr = d.Mr; k.Mc = d.Mc; k.M = d.M;
  k.levels = a.levels;
  k.full_in = a.full_in;
  k.full_out = a.full_out;
  k.rows_in = a.full_in ? d.Nx : d.Mr;
  k.cols_in = a.full_in ? d.Nk : d.Mc;
  k.form = a.form;
  k.sponge = a.sponge || a.form == HF_SPONGE;
  k.eta = a.eta;
  k.psi_derived = a.psi_derived;
  if (a.form == HF_FLUX) { k.nf1 = 5; k.nprod = k.sponge ? 9 : 6; k.ng = 6; }
  else if (a.form == HF_JAC) { k.nf1 = k.sponge ? 11 : 8; k.nprod = 3; k.ng = 3; }
  else { k.nf1 = 1; k.nprod = 1; k.ng = 1; }
  k.scale = 1.0 / ((double)d.Nx * (double)d.Nx);
  k.plan = p.plan;
  k.psi = a.psi; k.q = a.q; k.w = a.w; k.th = a.th;
  k.kx_full = t.kx_full; k.ky_full = t.ky_full; k.inv_denom = t.inv_denom;
  k.eta_c = t.eta; k.sponge_phys = t.sponge; k.eta_phys = t.eta_phys;
  k.tw = t.tw; k.perm = t.perm;
  k.Aq = a.Aq; k.Aw = a.Aw; k.Ath = a.Ath;
  const size_t need1 = (size_t)k.nf1 * a.levels * k.cols_in * d.Nx;
  const size_t need2 = (size_t)k.ng * a.levels * d.Mc * d.Nx;
  if (need1 > w.x1_elems || need2 > w.x2_elems) return cudaErrorInvalidValue;
  k.x1 = w.x1; k.x2 = w.x2;

  const size_t tb = table_bytes(d.Nx);
  const size_t budget = 200 * 1024;
  // H1: CB columns per CTA
  int CB1 = (int)((96 * 1024) / ((size_t)k.nf1 * d.Nx * sizeof(double2)));
  CB1 = max(1, min(CB1, k.cols_in));
  size_t sm1 = tb + (size_t)k.nf1 * CB1 * d.Nx * sizeof(double2);
  if (sm1 > budget) return cudaErrorInvalidConfiguration;
  // H2: RB rows per CTA (even, divides Nx)
  int RB = 2;
  while (RB * 2 <= 16 && d.Nx % (RB * 2) == 0 &&
         tb + (size_t)(k.nf1 + k.nprod) * RB * d.Nx * sizeof(double2) <= budget)
    RB *= 2;
  size_t sm2 = tb + (size_t)(k.nf1 + k.nprod) * (RB / 2) * d.Nx * sizeof(double2);
  if (sm2 > budget) return cudaErrorInvalidConfiguration;
  int CB3 = (int)((96 * 1024) / ((size_t)k.ng * d.Nx * sizeof(double2)));
  CB3 = max(1, min(CB3, d.Mc));
  size_t sm3 = tb + (size_t)k.ng * CB3 * d.Nx * sizeof(double2);
  if (sm3 > budget) return cudaErrorInvalidConfiguration;

  cudaFuncSetAttribute(k_h1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  cudaFuncSetAttribute(k_h2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  cudaFuncSetAttribute(k_h3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget);
  dim3 g1((k.cols_in + CB1 - 1) / CB1, a.levels);
  w.prof.begin("h1_col_ifft", st);
  k_h1<<<g1, 256, sm1, st>>>(k, CB1);
  w.prof.end(st);
  dim3 g2(d.Nx / RB, a.levels);
  w.prof.begin("h2_row_products", st);
  k_h2<<<g2, 256, sm2, st>>>(k, RB);
  w.prof.end(st);
  dim3 g3((d.Mc + CB3 - 1) / CB3, a.levels);
  w.prof.begin("h3_col_fft", st);
  k_h3<<<g3, 256, sm3, st>>>(k, CB3);
  w.prof.end(st);
  if (nlaunch) *nlaunch += 3;
  return cudaGetLastError();
}

}  // namespace nhqg

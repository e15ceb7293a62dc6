// Diagnostics of a state.  Scalars (nhqg/diagnostics.py:597-690, the subset
// without the budgets): Clenshaw-Curtis depth integrals of
// |psi|^2, |q|^2, |w|^2, |theta|^2, Re(w theta*) and of the barotropic psi
// per mode, weighted by the half-plane Parseval weights (1 at ky = 0 and, in
// the full-band layout of the 3/2 rule, at ky = Nx/2; 2 elsewhere) and normalised by Nx^4.  Spectra: the shell
// energy spectrum, the q / w / theta shell spectra and the vertical mode
// energies (k_spec_*, k_vspec).  The physical-space maxima come from
// horizontal.cu (launch_phys_maxima).
#include "engine.h"

namespace nhqg {

namespace {

constexpr int kDiagThreads = 256;

// rfft2 half-plane weight of compact mode m (nhqg/diagnostics.py:48-54)
__device__ __forceinline__ double hweight(const Dims& d, int m) {
  const int c = m % d.Mc;
  return (c == 0 || (d.pad && c == d.Nk - 1)) ? 1.0 : 2.0;
}

// one thread per compact mode, levels looped (level-major fields: coalesced)
__global__ void __launch_bounds__(kDiagThreads) k_diag_modes(Dims d, const double* __restrict__ cc,
                                                             const double* __restrict__ kx,
                                                             const double* __restrict__ ky,
                                                             const double* __restrict__ inv_denom,
                                                             const double2* __restrict__ qn,
                                                             const double2* __restrict__ wn,
                                                             const double2* __restrict__ tn,
                                                             double* __restrict__ partials) {
  __shared__ double red[kDiagTerms][kDiagThreads / 32];
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  double v[kDiagTerms] = {0, 0, 0, 0, 0, 0, 0};
  if (m < d.M) {
    const double idn = inv_denom[m];
    double2 pbt = czero();
    double spsi = 0.0, sq = 0.0, sw = 0.0, st = 0.0, swt = 0.0;
    for (int j = 0; j < d.P; ++j) {
      const double c = cc[j];
      const size_t g = (size_t)j * d.M + m;
      const double2 q = qn[g], w = wn[g], t = tn[g];
      const double2 psi = cscale(q, -idn);
      pbt = caxpy(c, psi, pbt);
      spsi = fma(c, fma(psi.x, psi.x, psi.y * psi.y), spsi);
      sq = fma(c, fma(q.x, q.x, q.y * q.y), sq);
      sw = fma(c, fma(w.x, w.x, w.y * w.y), sw);
      st = fma(c, fma(t.x, t.x, t.y * t.y), st);
      swt = fma(c, fma(w.x, t.x, w.y * t.y), swt);
    }
    const double wt = hweight(d, m);
    const double ksq = fma(kx[m], kx[m], ky[m] * ky[m]);
    v[0] = 0.5 * wt * ksq * fma(pbt.x, pbt.x, pbt.y * pbt.y);  // KE_bt
    v[1] = 0.5 * wt * ksq * spsi;                              // KE_tot
    v[2] = wt * sq;
    v[3] = wt * sw;
    v[4] = wt * st;
    v[5] = wt * swt;
    v[6] = 0.0;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < kDiagTerms; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < kDiagTerms) {
    double x = 0.0;
    for (int q = 0; q < kDiagThreads / 32; ++q) x += red[threadIdx.x][q];
    partials[(size_t)blockIdx.x * kDiagTerms + threadIdx.x] = x;
  }
}

// one CTA: sum the block partials in block order, the dealiased flux
// (s2c flux on the SBP grid when flux_on_sbp) against the CC weights, and
// max |th_bar|
__global__ void k_diag_final(int nblocks, int P, double norm, const double* __restrict__ partials,
                             const double* __restrict__ cc, const double* __restrict__ flux,
                             const double* __restrict__ s2c, bool flux_on_sbp,
                             const double* __restrict__ th_bar,
                             const unsigned long long* __restrict__ maxima, double* __restrict__ out) {
  __shared__ double tot[kDiagTerms];
  __shared__ double red[32];
  if (threadIdx.x < kDiagTerms) {
    double x = 0.0;
    for (int b = 0; b < nblocks; ++b) x += partials[(size_t)b * kDiagTerms + threadIdx.x];
    tot[threadIdx.x] = x / norm;
  }
  // sum_j cc_j flux_cgl_j, flux_cgl = s2c flux (SBP) or flux
  double acc = 0.0;
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    double f = flux[j];
    if (flux_on_sbp) {
      f = 0.0;
      for (int i = 0; i < P; ++i) f = fma(s2c[(size_t)j * P + i], flux[i], f);
    }
    acc = fma(cc[j], f, acc);
  }
  const double voltw_d = block_sum(acc, red);
  __syncthreads();
  double mx = 0.0;
  for (int j = threadIdx.x; j < P; j += blockDim.x) mx = fmax(mx, fabs(th_bar[j]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int q = 0; q < (int)(blockDim.x + 31) / 32; ++q) m = fmax(m, red[q]);
    const double ke_bt = tot[0], ke_tot = tot[1], q2 = tot[2], w2 = tot[3], t2 = tot[4], wt = tot[5];
    out[NHQG_DIAG_KE_BT] = ke_bt;
    out[NHQG_DIAG_KE_BC] = ke_tot - ke_bt;
    out[NHQG_DIAG_KE_TOT] = ke_tot;
    out[NHQG_DIAG_ENSTROPHY] = 0.5 * q2;
    out[NHQG_DIAG_NUSSELT] = 1.0 + wt;
    out[NHQG_DIAG_NUSSELT_DEALIASED] = 1.0 + voltw_d;
    out[NHQG_DIAG_VOL_AVG_TW] = wt;
    out[NHQG_DIAG_VOL_AVG_TW_DEALIASED] = voltw_d;
    out[NHQG_DIAG_Q_RMS] = sqrt(q2);
    out[NHQG_DIAG_W_RMS] = sqrt(w2);
    out[NHQG_DIAG_TH_RMS] = sqrt(t2);
    out[NHQG_DIAG_TH_BAR_MAX] = m;
    // physical-space maxima (nhqg/diagnostics.py:631-641) and the heat-flux
    // mismatch between the dealiased and the Parseval volume averages
    out[NHQG_DIAG_MAX_SPEED] = __longlong_as_double((long long)maxima[0]);
    out[NHQG_DIAG_MAX_W] = __longlong_as_double((long long)maxima[1]);
    out[NHQG_DIAG_MAX_THETA] = __longlong_as_double((long long)maxima[2]);
    out[NHQG_DIAG_MAX_TW] = __longlong_as_double((long long)maxima[3]);
    out[NHQG_DIAG_HEAT_FLUX_MISMATCH] = voltw_d - wt;
  }
}

// Shell spectra (nhqg/diagnostics.py:80-111): per compact mode the weighted
// barotropic and depth-integrated psi energies 0.5 w_k |k|^2 |psi_bt|^2 and
// 0.5 w_k |k|^2 sum_j cc_j |psi_j|^2, and the depth-integrated field
// energies w_k sum_j cc_j |f_j|^2 of q, w, theta at the CGL nodes
// (unnormalised, as the reference sums them)
__global__ void __launch_bounds__(kDiagThreads) k_spec_modes(Dims d, const double* __restrict__ cc,
                                                             const double* __restrict__ kx,
                                                             const double* __restrict__ ky,
                                                             const double* __restrict__ inv_denom,
                                                             const double2* __restrict__ qn,
                                                             const double2* __restrict__ wn,
                                                             const double2* __restrict__ tn,
                                                             double* __restrict__ per_mode) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= d.M) return;
  const double idn = inv_denom[m];
  double2 pbt = czero();
  double spsi = 0.0, sq = 0.0, sw = 0.0, st = 0.0;
  for (int j = 0; j < d.P; ++j) {
    const size_t g = (size_t)j * d.M + m;
    const double2 q = qn[g], w = wn[g], t = tn[g];
    const double2 psi = cscale(q, -idn);
    const double c = cc[j];
    pbt = caxpy(c, psi, pbt);
    spsi = fma(c, fma(psi.x, psi.x, psi.y * psi.y), spsi);
    sq = fma(c, fma(q.x, q.x, q.y * q.y), sq);
    sw = fma(c, fma(w.x, w.x, w.y * w.y), sw);
    st = fma(c, fma(t.x, t.x, t.y * t.y), st);
  }
  const double wt = hweight(d, m);
  const double ksq = fma(kx[m], kx[m], ky[m] * ky[m]);
  per_mode[m] = 0.5 * wt * ksq * fma(pbt.x, pbt.x, pbt.y * pbt.y);
  per_mode[d.M + m] = 0.5 * wt * ksq * spsi;
  per_mode[2 * (size_t)d.M + m] = wt * sq;
  per_mode[3 * (size_t)d.M + m] = wt * sw;
  per_mode[4 * (size_t)d.M + m] = wt * st;
}

// one CTA per shell: sum the modes of the shell in a fixed order; E_bt, E_bc,
// E_tot into out[0 .. 3 n_bins), the q, w, theta shell spectra into
// fout[0 .. 3 n_bins)
__global__ void k_spec_bins(int M, const int* __restrict__ bin, const double* __restrict__ per_mode,
                            int n_bins, double* __restrict__ out, double* __restrict__ fout) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  double e[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int m = threadIdx.x; m < M; m += blockDim.x)
    if (bin[m] == b) {
      for (int f = 0; f < 5; ++f) e[f] += per_mode[(size_t)f * M + m];
    }
  for (int f = 0; f < 5; ++f) {
    e[f] = block_sum(e[f], red);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[b] = e[0];
    out[n_bins + b] = e[1] - e[0];
    out[2 * n_bins + b] = e[1];
    fout[b] = e[2];
    fout[n_bins + b] = e[3];
    fout[2 * n_bins + b] = e[4];
  }
}

// vertical spectra (nhqg/diagnostics.py:583-585): CTA (n, f) sums over the
// modes |f_n|^2 for f = q, w, theta (unweighted, as the reference sums the
// whole rfft array) and w_k |k|^2 |psi_n|^2 for f = 3
__global__ void k_vspec(Dims d, const double2* __restrict__ q, const double2* __restrict__ w,
                        const double2* __restrict__ t, const double* __restrict__ kx,
                        const double* __restrict__ ky, const double* __restrict__ inv_denom,
                        double* __restrict__ out) {
  __shared__ double red[32];
  const int n = blockIdx.x, f = blockIdx.y;
  const int levels = (f == 1 || f == 2) ? d.G : d.P;
  if (n >= levels) return;
  const double2* src = (f == 1) ? w : (f == 2) ? t : q;
  double acc = 0.0;
  for (int m = threadIdx.x; m < d.M; m += blockDim.x) {
    const double2 x = src[(size_t)n * d.M + m];
    double a2 = fma(x.x, x.x, x.y * x.y);
    if (f == 3) {
      const double wt = hweight(d, m);
      const double ksq = fma(kx[m], kx[m], ky[m] * ky[m]);
      a2 *= wt * ksq * inv_denom[m] * inv_denom[m];
    }
    acc += a2;
  }
  acc = block_sum(acc, red);
  const int off = (f == 0) ? 0 : (f == 1) ? d.P : (f == 2) ? d.P + d.G : d.P + 2 * d.G;
  if (threadIdx.x == 0) out[off + n] = acc;
}

}  // namespace

int diag_blocks(const Params& p) { return (p.d.M + kDiagThreads - 1) / kDiagThreads; }

cudaError_t launch_spectra(const Params& p, const Tables& t, const double2* qn, const double2* wn,
                           const double2* tn, const double2* q, const double2* w, const double2* th,
                           const int* mode_bin, int n_bins, double* per_mode, double* out,
                           cudaStream_t st) {
  if (!t.cc || n_bins <= 0) return cudaErrorInvalidValue;
  k_spec_modes<<<diag_blocks(p), kDiagThreads, 0, st>>>(p.d, t.cc, t.kx, t.ky, t.inv_denom, qn, wn, tn,
                                                        per_mode);
  double* fout = out + 3 * (size_t)n_bins + 2 * (size_t)p.d.P + 2 * (size_t)p.d.G;
  k_spec_bins<<<n_bins, kDiagThreads, 0, st>>>(p.d.M, mode_bin, per_mode, n_bins, out, fout);
  k_vspec<<<dim3(p.d.P, 4), kDiagThreads, 0, st>>>(p.d, q, w, th, t.kx, t.ky, t.inv_denom,
                                                    out + 3 * (size_t)n_bins);
  return cudaGetLastError();
}

cudaError_t launch_diag_modes(const Params& p, const Tables& t, const double2* qn, const double2* wn,
                              const double2* tn, double* partials, cudaStream_t st) {
  if (!t.cc) return cudaErrorInvalidValue;
  k_diag_modes<<<diag_blocks(p), kDiagThreads, 0, st>>>(p.d, t.cc, t.kx, t.ky, t.inv_denom, qn, wn,
                                                        tn, partials);
  return cudaGetLastError();
}

cudaError_t launch_diag_final(const Params& p, const Tables& t, const double* partials,
                              const double* flux, bool flux_on_sbp, const double* th_bar,
                              const unsigned long long* maxima, double* out, cudaStream_t st) {
  const double nx2 = (double)p.d.Nx * (double)p.d.Nx;
  k_diag_final<<<1, 256, 0, st>>>(diag_blocks(p), p.d.P, nx2 * nx2, partials, t.cc, flux, t.s2c_d,
                                  flux_on_sbp, th_bar, maxima, out);
  return cudaGetLastError();
}

}  // namespace nhqg

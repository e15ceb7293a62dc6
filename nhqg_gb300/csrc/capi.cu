// C ABI of the NHQG GB300 engine: context creation (table upload), the
// ARS(2,2,2) step orchestration and the per-operator entry points.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <new>
#include <vector>

#include "engine.h"
#include "nhqg_gpu.h"

using namespace nhqg;

struct nhqg_ctx {
  Params p{};
  Tables t{};
  Work w{};
  std::vector<void*> allocs;
  int launches = 0;
  // named compact work fields
  double2 *q0, *w0, *t0, *Qn, *Wn, *Tn, *Aq, *Aw, *At, *E1q, *E1w, *E1t, *Rq, *Rt, *rhs;
  double2 *Q1, *W1, *T1p, *T1, *Q2, *W2, *T2p, *T2, *Wcgl, *Wsbp, *Tsbp, *Tcgl;
  // 1-D vectors [P]
  double *tb0, *tb1p, *tb1, *tb2p, *tb2, *E1tb, *E2tb, *Itb, *flux, *dtb;
  double* diag_part = nullptr;  // diagnostics block partials
  unsigned long long* diag_max = nullptr;  // physical-space maxima (bit patterns of doubles >= 0)
  double* spec_mode = nullptr;  // spectra: per-mode energies [5*M], allocated on first use
  // ARS(4,4,3) (scheme RK443, legacy exchange): explicit E_0..E_3 and implicit
  // K_1..K_4 derivatives of (q, w, theta) [P*M] and of th_bar [P]
  double2* rkE[4][3] = {};
  double2* rkK[4][3] = {};
  double* rkEtb[4] = {};
  double* rkKtb[4] = {};
  // mixed-precision path: FP32 nodal inputs and outputs of the horizontal
  // products, allocated by the first nhqg_set_precision(NHQG_PRECISION_MIXED)
  int precision = NHQG_PRECISION_FP64;
  float2 *Qf = nullptr, *Wf = nullptr, *Tf = nullptr, *Aqf = nullptr, *Awf = nullptr, *Atf = nullptr;
  // learned closure (null weights: off) and its tendency buffer [P*M]
  ClosureModel closure{};
  double2* Cq = nullptr;
  // bumped whenever the launch sequence of a step changes (precision, tiles):
  // captured step graphs of a batch compare it
  unsigned version = 0;
};

namespace {

#define PCK(name, call)                      \
  do {                                        \
    c->w.prof.begin(name, st);                \
    cudaError_t e_ = (call);                  \
    c->w.prof.end(st);                        \
    if (e_ != cudaSuccess) return NHQG_ERR_CUDA; \
  } while (0)

#define CK(call)                                  \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return NHQG_ERR_CUDA;  \
  } while (0)

template <typename T>
cudaError_t dalloc(nhqg_ctx* c, T** ptr, size_t n) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T) + 16);
  if (e != cudaSuccess) return e;
  c->allocs.push_back(p);
  *ptr = static_cast<T*>(p);
  return cudaSuccess;
}

template <typename T>
cudaError_t upload(nhqg_ctx* c, T** ptr, const T* host, size_t n) {
  cudaError_t e = dalloc(c, ptr, n);
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*ptr, host, n * sizeof(T), cudaMemcpyHostToDevice);
}

void free_all(nhqg_ctx* c) {
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
}

struct CSR {
  std::vector<int> ptr, col;
  std::vector<double> val;
};
CSR to_csr(const double* A, int n) {
  CSR s;
  s.ptr.push_back(0);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) {
      const double v = A[(size_t)i * n + j];
      if (v != 0.0) { s.col.push_back(j); s.val.push_back(v); }
    }
    s.ptr.push_back((int)s.col.size());
  }
  if (s.col.empty()) { s.col.push_back(0); s.val.push_back(0.0); }
  return s;
}

int full_index(const Dims& d, int r, int c) { return full_row(r, d.K, d.Mr, d.Nx) * d.Nk + c; }

// exp(-2 pi i k / n) with the angle reduced to [0, pi/4] so that each
// component comes from one correctly-rounded-in-practice libm call
double2 twiddle(long k, long n) {
  k %= n;
  if (k < 0) k += n;
  // 8 k / n in [0, 8): octant and reflected fraction
  const long k8 = 8 * k;
  const int oct = (int)(k8 / n);
  long r = k8 - oct * n;                 // remainder in [0, n)
  if (oct & 1) r = n - r;                // reflect inside the octant
  const double a = (M_PI / 4.0) * (double)r / (double)n;  // in [0, pi/4]
  const double c = std::cos(a), s = std::sin(a);
  double cs, sn;                          // cos, sin of 2 pi k / n
  switch (oct) {
    case 0: cs = c;  sn = s;  break;
    case 1: cs = s;  sn = c;  break;
    case 2: cs = -s; sn = c;  break;
    case 3: cs = -c; sn = s;  break;
    case 4: cs = -c; sn = -s; break;
    case 5: cs = -s; sn = -c; break;
    case 6: cs = s;  sn = -c; break;
    default: cs = c; sn = -s; break;
  }
  return make_double2(cs, -sn);
}

}  // namespace

extern "C" {

const char* nhqg_version(void) { return "nhqg_gb300 0.2 (sm_103a, FP64 plain and mixed-precision paths)"; }

int nhqg_ctx_create(const nhqg_grid_desc* g, nhqg_ctx** out) {
  if (!g || !out) return NHQG_ERR_BAD_ARG;
  *out = nullptr;
  if (g->Nx < 8 || g->Nx % 2 != 0 || g->Nz < 4 || g->Nz + 1 > 1024) return NHQG_ERR_UNSUPPORTED;
  if (g->horizontal_dealiasing != NHQG_DEALIAS_23 && g->horizontal_dealiasing != NHQG_DEALIAS_32)
    return NHQG_ERR_BAD_ARG;
  const bool pad32 = g->horizontal_dealiasing == NHQG_DEALIAS_32;
  // the horizontal transforms run on the Nx grid (2/3 rule) or the padded
  // 3Nx/2 grid (3/2 rule): that length must be 2^a 3^b
  FftPlan plan = make_fft_plan(pad32 ? 3 * g->Nx / 2 : g->Nx);
  if (plan.npass <= 0) return NHQG_ERR_UNSUPPORTED;
  if (g->advection != NHQG_ADV_FLUX && g->advection != NHQG_ADV_JACOBIAN) return NHQG_ERR_UNSUPPORTED;
  if (g->exchange < NHQG_EXCHANGE_LEGACY || g->exchange > NHQG_EXCHANGE_BALANCED_SBP2_PC)
    return NHQG_ERR_UNSUPPORTED;
  if (g->thermal_closure == NHQG_CLOSURE_EVOLVE_MEAN && g->exchange == NHQG_EXCHANGE_LEGACY &&
      !g->mean_solve)
    return NHQG_ERR_BAD_ARG;
  if (!g->kx || !g->ky || !g->inv_denom || !g->diss_rate_q || !g->diss_rate_w || !g->diss_rate_th ||
      !g->inv_alpha_q || !g->inv_alpha_th || !g->shell_of_mode || !g->shell_inv || !g->V ||
      !g->V_inv || !g->w_stencil || !g->G_Z || !g->proj_dirichlet || !g->sbp_D1 || !g->sbp_L ||
      !g->cgl_to_sbp || !g->sbp_to_cgl)
    return NHQG_ERR_BAD_ARG;
  if (g->eta_hat && !g->eta_phys) return NHQG_ERR_BAD_ARG;
  if (g->imex_scheme != NHQG_SCHEME_ARS222 && g->imex_scheme != NHQG_SCHEME_RK443)
    return NHQG_ERR_BAD_ARG;

  nhqg_ctx* c = new (std::nothrow) nhqg_ctx();
  if (!c) return NHQG_ERR_BAD_ARG;
  Params& p = c->p;
  p.d = make_dims(g->Nx, g->Nz, pad32);
  p.plan = plan;
  p.plan_v = make_fft_plan(g->Nz);
  p.fast_dct = g->Nz % 2 == 0 && p.plan_v.npass > 0 && getenv("NHQG_DENSE_VERTICAL") == nullptr;
  p.advection = g->advection;
  p.closure = g->thermal_closure;
  p.exchange = g->exchange;
  p.wbc = g->w_bc_top;
  p.substeps = g->substeps > 0 ? g->substeps : 1;
  p.dt = g->dt; p.gamma_imex = g->gamma_imex; p.Ra_sigma = g->Ra_sigma; p.sigma = g->sigma;
  p.beta = g->beta; p.eps_sq = g->eps_sq;
  p.has_eta = g->eta_hat != nullptr;
  p.has_sponge = g->sponge_phys != nullptr;
  p.scheme = g->imex_scheme;
  const Dims& d = p.d;
  const int P = d.P, G = d.G, N = d.Nz, M = d.M;
  int rc = NHQG_OK;
  auto fail = [&](int code) { free_all(c); delete c; return code; };
#define UP(dst, src, n) \
  if (upload(c, &(dst), (src), (n)) != cudaSuccess) return fail(NHQG_ERR_CUDA)

  // ---- w stencil structure ----
  std::vector<double> wa, wb;
  if (g->w_bc_top == NHQG_WBC_DIRICHLET) {
    for (int n = 0; n < G; ++n) {
      if (g->w_stencil[(size_t)n * G + n] != -1.0 || g->w_stencil[(size_t)(n + 2) * G + n] != 1.0)
        return fail(NHQG_ERR_UNSUPPORTED);
    }
  } else if (g->w_bc_top == NHQG_WBC_NEUMANN) {
    wa.resize(G);
    wb.resize(G);
    for (int n = 0; n < G; ++n) {
      if (g->w_stencil[(size_t)n * G + n] != 1.0) return fail(NHQG_ERR_UNSUPPORTED);
      wa[n] = g->w_stencil[(size_t)(n + 1) * G + n];
      wb[n] = g->w_stencil[(size_t)(n + 2) * G + n];
    }
  } else {
    return fail(NHQG_ERR_UNSUPPORTED);
  }

  // ---- per-mode compact tables ----
  std::vector<double> kx(M), ky(M), idn(M), iaq(M), iat(M), drq(M), drw(M), drt(M);
  std::vector<double2> eta;
  if (p.has_eta) eta.resize(M);
  std::vector<int> shell(M);
  for (int r = 0; r < d.Mr; ++r) {
    for (int cc = 0; cc < d.Mc; ++cc) {
      const int m = r * d.Mc + cc;
      const int f = full_index(d, r, cc);
      kx[m] = g->kx[full_row(r, d.K, d.Mr, d.Nx)];
      ky[m] = g->ky[cc];
      idn[m] = g->inv_denom[f];
      iaq[m] = g->inv_alpha_q[f];
      iat[m] = g->inv_alpha_th[f];
      drq[m] = g->diss_rate_q[f];
      drw[m] = g->diss_rate_w[f];
      drt[m] = g->diss_rate_th[f];
      if (p.has_eta) eta[m] = make_double2(g->eta_hat[2 * (size_t)f], g->eta_hat[2 * (size_t)f + 1]);
      shell[m] = g->shell_of_mode[f];
      if (shell[m] < 0 || shell[m] >= g->n_shells) return fail(NHQG_ERR_BAD_ARG);
    }
  }
  Tables& t = c->t;
  UP(t.kx, kx.data(), M); UP(t.ky, ky.data(), M); UP(t.inv_denom, idn.data(), M);
  UP(t.inv_aq, iaq.data(), M); UP(t.inv_at, iat.data(), M);
  UP(t.drq, drq.data(), M); UP(t.drw, drw.data(), M); UP(t.drt, drt.data(), M);
  // physical-space eta and sigma on the Nh grid, in the products' scaling:
  // the horizontal kernels carry each field as (Nh/Nx) irfft2 of its padded
  // spectrum (1 under the 2/3 rule)
  const size_t nh2 = (size_t)d.Nh * d.Nh;
  const double hscale = (double)d.Nh / (double)d.Nx;
  std::vector<double> eta_ph, sponge_ph;
  if (p.has_eta) {
    eta_ph.assign(g->eta_phys, g->eta_phys + nh2);
    for (double& v : eta_ph) v *= hscale;
  }
  if (p.has_sponge) {
    sponge_ph.assign(g->sponge_phys, g->sponge_phys + nh2);
    for (double& v : sponge_ph) v *= hscale;
  }
  if (p.has_eta) {
    UP(t.eta, eta.data(), M);
    UP(t.eta_phys, eta_ph.data(), nh2);
  }
  if (p.has_sponge) UP(t.sponge, sponge_ph.data(), nh2);
  UP(t.kx_full, g->kx, d.Nx);
  UP(t.ky_full, g->ky, d.Nk);
  UP(t.inv_denom_full, g->inv_denom, (size_t)d.Nx * d.Nk);
  if (p.wbc == NHQG_WBC_NEUMANN) { UP(t.wst_a, wa.data(), G); UP(t.wst_b, wb.data(), G); }

  // ---- FFT tables ----
  {
    std::vector<double2> tw(d.Nh);
    for (int k = 0; k < d.Nh; ++k) tw[k] = twiddle(k, d.Nh);
    std::vector<int> perm(d.Nh);
    make_fft_perm(plan, perm.data());
    UP(t.tw, tw.data(), d.Nh);
    UP(t.perm, perm.data(), d.Nh);
  }
  // transforms of length Nx for the physical-space diagnostics (the 3/2 rule's
  // products run at Npad, the reference's maxima are taken on the Nx grid)
  p.plan_nx = make_fft_plan(d.Nx);
  if (d.Nh == d.Nx) {
    t.tw_nx = t.tw;
    t.perm_nx = t.perm;
  } else if (p.plan_nx.npass > 0) {
    std::vector<double2> tw(d.Nx);
    for (int k = 0; k < d.Nx; ++k) tw[k] = twiddle(k, d.Nx);
    std::vector<int> perm(d.Nx);
    make_fft_perm(p.plan_nx, perm.data());
    UP(t.tw_nx, tw.data(), d.Nx);
    UP(t.perm_nx, perm.data(), d.Nx);
  }
  if (p.fast_dct) {
    const int L = d.Nz;
    std::vector<double2> tw(L), cs(L + 1);
    for (int k = 0; k < L; ++k) tw[k] = twiddle(k, L);
    for (int j = 0; j <= L; ++j) cs[j] = twiddle(j, 2 * L);
    std::vector<int> perm(L);
    make_fft_perm(p.plan_v, perm.data());
    UP(t.tw_v, tw.data(), L);
    UP(t.cs_v, cs.data(), L + 1);
    UP(t.perm_v, perm.data(), L);
    // double-float copies: nearest float, then the rounded remainder
    std::vector<cdfl> twd(L), csd(L + 1);
    for (int k = 0; k < L; ++k) twd[k] = cdfl{dfl(tw[k].x), dfl(tw[k].y)};
    for (int j = 0; j <= L; ++j) csd[j] = cdfl{dfl(cs[j].x), dfl(cs[j].y)};
    UP(t.tw_v_df, twd.data(), L);
    UP(t.cs_v_df, csd.data(), L + 1);
  }

  // ---- FP32 copies of the horizontal and DCT tables (mixed-precision path) ----
  {
    auto f32 = [](const double* a, size_t n) {
      std::vector<float> v(n);
      for (size_t i = 0; i < n; ++i) v[i] = (float)a[i];
      return v;
    };
    auto c32 = [](const std::vector<double2>& a) {
      std::vector<float2> v(a.size());
      for (size_t i = 0; i < a.size(); ++i) v[i] = make_float2((float)a[i].x, (float)a[i].y);
      return v;
    };
    std::vector<float> kxf = f32(g->kx, d.Nx), kyf = f32(g->ky, d.Nk);
    UP(t.kx_f, kxf.data(), kxf.size());
    UP(t.ky_f, kyf.data(), kyf.size());
    std::vector<double2> tw(d.Nh);
    for (int k = 0; k < d.Nh; ++k) tw[k] = twiddle(k, d.Nh);
    std::vector<float2> twf = c32(tw);
    UP(t.tw_f, twf.data(), twf.size());
    if (p.fast_dct) {
      std::vector<double2> twv(N), csv(N + 1);
      for (int k = 0; k < N; ++k) twv[k] = twiddle(k, N);
      for (int j = 0; j <= N; ++j) csv[j] = twiddle(j, 2 * N);
      std::vector<float2> twvf = c32(twv), csvf = c32(csv);
      UP(t.tw_v_f, twvf.data(), twvf.size());
      UP(t.cs_v_f, csvf.data(), csvf.size());
    }
    if (p.has_sponge) {
      std::vector<float> v = f32(sponge_ph.data(), nh2);
      UP(t.sponge_f, v.data(), v.size());
    }
    if (p.has_eta) {
      std::vector<float> v = f32(eta_ph.data(), nh2);
      UP(t.eta_phys_f, v.data(), v.size());
      std::vector<float2> e = c32(eta);
      UP(t.eta_f, e.data(), e.size());
      if (g->eta_x_phys && g->eta_y_phys) {  // FP32 products carry u . grad(eta)
        std::vector<double> gx(g->eta_x_phys, g->eta_x_phys + nh2), gy(g->eta_y_phys, g->eta_y_phys + nh2);
        for (double& x : gx) x *= hscale;
        for (double& x : gy) x *= hscale;
        std::vector<float> fx = f32(gx.data(), nh2), fy = f32(gy.data(), nh2);
        UP(t.eta_x_f, fx.data(), fx.size());
        UP(t.eta_y_f, fy.data(), fy.size());
      }
    }
  }

  // ---- vertical tables ----
  UP(t.V, g->V, (size_t)P * P);
  UP(t.Vinv, g->V_inv, (size_t)P * P);
  UP(t.proj, g->proj_dirichlet, (size_t)P * P);
  UP(t.D1, g->sbp_D1, (size_t)P * P);
  UP(t.Lsbp, g->sbp_L, (size_t)P * P);
  {  // Parseval weights of the compact modes
    std::vector<double2> wt(d.M);
    for (int m = 0; m < d.M; ++m) {
      const int r = m / d.Mc, col = m - r * d.Mc;
      double wr = 2.0, wi = 2.0;
      if (col == 0) {
        const int rm = mirror_row(r, d.Mr);
        if (r == 0) { wr = 1.0; wi = 0.0; }
        else if (rm == r) { wr = wi = 0.5; }
        else { wr = wi = 1.0; }
      }
      wt[m] = make_double2(wr, wi);
    }
    UP(t.pwt, wt.data(), wt.size());
  }
  {  // diagonals of D1 and of the SBP Laplacian (the corrector's 1-D kernels)
    std::vector<double> d1b(3 * (size_t)P, 0.0), lb(5 * (size_t)P, 0.0);
    for (int i = 0; i < P; ++i) {
      for (int d = 0; d < 3; ++d) {
        const int j = i - 1 + d;
        if (j >= 0 && j < P) d1b[(size_t)d * P + i] = g->sbp_D1[(size_t)i * P + j];
      }
      for (int d = 0; d < 5; ++d) {
        const int j = i - 2 + d;
        if (j >= 0 && j < P) lb[(size_t)d * P + i] = g->sbp_L[(size_t)i * P + j];
      }
    }
    UP(t.D1b, d1b.data(), d1b.size());
    UP(t.Lb, lb.data(), lb.size());
  }
  UP(t.GZ, g->G_Z, (size_t)P * P);
  {
    std::vector<double> gz2((size_t)P * P, 0.0);
    // G_Z2 = G_Z @ G_Z (nhqg/grid.py:463)
    for (int i = 0; i < P; ++i)
      for (int kk = 0; kk < P; ++kk) {
        const double a = g->G_Z[(size_t)i * P + kk];
        if (a == 0.0) continue;
        for (int j = 0; j < P; ++j) gz2[(size_t)i * P + j] += a * g->G_Z[(size_t)kk * P + j];
      }
    UP(t.GZ2, gz2.data(), (size_t)P * P);
  }
  if (g->mean_solve) UP(t.mean_solve, g->mean_solve, (size_t)P * P);
  if (g->cc_weights) {
    UP(t.cc, g->cc_weights, (size_t)P);
    if (dalloc(c, &c->diag_part, (size_t)diag_blocks(p) * kDiagTerms) != cudaSuccess)
      return fail(NHQG_ERR_CUDA);
    if (dalloc(c, &c->diag_max, (size_t)kDiagMaxima) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  }
  {
    CSR a = to_csr(g->cgl_to_sbp, P), b = to_csr(g->sbp_to_cgl, P);
    UP(t.c2s_ptr, a.ptr.data(), a.ptr.size()); UP(t.c2s_col, a.col.data(), a.col.size());
    UP(t.c2s_val, a.val.data(), a.val.size());
    UP(t.s2c_ptr, b.ptr.data(), b.ptr.size()); UP(t.s2c_col, b.col.data(), b.col.size());
    UP(t.s2c_val, b.val.data(), b.val.size());
    int w = 1;
    for (int i = 0; i < P; ++i)
      w = std::max(w, std::max(a.ptr[i + 1] - a.ptr[i], b.ptr[i + 1] - b.ptr[i]));
    std::vector<int> ac((size_t)w * P), bc((size_t)w * P);
    std::vector<double> av((size_t)w * P, 0.0), bvv((size_t)w * P, 0.0);
    for (int i = 0; i < P; ++i)
      for (int q = 0; q < w; ++q) {
        const int qa = a.ptr[i] + q, qb = b.ptr[i] + q;
        const bool ina = qa < a.ptr[i + 1], inb = qb < b.ptr[i + 1];
        ac[(size_t)q * P + i] = ina ? a.col[qa] : i;
        av[(size_t)q * P + i] = ina ? a.val[qa] : 0.0;
        bc[(size_t)q * P + i] = inb ? b.col[qb] : i;
        bvv[(size_t)q * P + i] = inb ? b.val[qb] : 0.0;
      }
    t.ell_w = w;
    UP(t.c2s_ecol, ac.data(), ac.size()); UP(t.c2s_eval, av.data(), av.size());
    UP(t.s2c_ecol, bc.data(), bc.size()); UP(t.s2c_eval, bvv.data(), bvv.size());
    UP(t.c2s_d, g->cgl_to_sbp, (size_t)P * P);
    UP(t.s2c_d, g->sbp_to_cgl, (size_t)P * P);
  }
  {
    // F = (proj_dir - I)[N-1:N+1, :] @ V_inv ; bcV = V[:, N-1], V[:, N]
    std::vector<double> F(2 * (size_t)P, 0.0), bv(2 * (size_t)P);
    for (int r = 0; r < 2; ++r) {
      const int row = N - 1 + r;
      for (int kk = 0; kk < P; ++kk) {
        const double a = g->proj_dirichlet[(size_t)row * P + kk] - (kk == row ? 1.0 : 0.0);
        if (a == 0.0) continue;
        for (int j = 0; j < P; ++j) F[(size_t)r * P + j] += a * g->V_inv[(size_t)kk * P + j];
      }
    }
    for (int l = 0; l < P; ++l) {
      bv[l] = g->V[(size_t)l * P + (N - 1)];
      bv[P + l] = g->V[(size_t)l * P + N];
    }
    UP(t.bcF, F.data(), F.size());
    UP(t.bcV, bv.data(), bv.size());
    // 1-D corrector maps as single dense rows, applied by many CTAs at once:
    // c2sV = c2s V (predictor th_bar coefficients -> SBP grid) and
    // tauVinv = P_tau V^-1 (CGL values -> coefficients with the Dirichlet tau
    // projection of rows N-1, N)
    std::vector<double> c2sV((size_t)P * P, 0.0), tauVinv((size_t)P * P, 0.0);
    for (int i = 0; i < P; ++i)
      for (int kk = 0; kk < P; ++kk) {
        const double a = g->cgl_to_sbp[(size_t)i * P + kk];
        if (a == 0.0) continue;
        for (int j = 0; j < P; ++j) c2sV[(size_t)i * P + j] += a * g->V[(size_t)kk * P + j];
      }
    for (int i = 0; i < P; ++i) {
      if (i < N - 1) {
        for (int j = 0; j < P; ++j) tauVinv[(size_t)i * P + j] = g->V_inv[(size_t)i * P + j];
      } else {
        for (int kk = 0; kk < N - 1; ++kk) {
          const double a = g->proj_dirichlet[(size_t)i * P + kk];
          if (a == 0.0) continue;
          for (int j = 0; j < P; ++j) tauVinv[(size_t)i * P + j] += a * g->V_inv[(size_t)kk * P + j];
        }
      }
    }
    UP(t.c2sV, c2sV.data(), c2sV.size());
    UP(t.tauVinv, tauVinv.data(), tauVinv.size());
    // fused substep tables: R = c2s s2c, Fs_j = s2c^T F_j, u_j = c2s bcV_j
    const double* c2s = g->cgl_to_sbp;
    const double* s2c = g->sbp_to_cgl;
    std::vector<std::vector<std::pair<int, double>>> rows(P);
    int rw = 1;
    for (int l = 0; l < P; ++l) {
      std::vector<double> acc(P, 0.0);
      std::vector<char> hit(P, 0);
      for (int i = 0; i < P; ++i) {
        const double a = c2s[(size_t)l * P + i];
        if (a == 0.0) continue;
        for (int q = 0; q < P; ++q) {
          const double b = s2c[(size_t)i * P + q];
          if (b == 0.0) continue;
          acc[q] = std::fma(a, b, acc[q]);
          hit[q] = 1;
        }
      }
      for (int q = 0; q < P; ++q)
        if (hit[q]) rows[l].push_back({q, acc[q]});
      rw = std::max(rw, (int)rows[l].size());
    }
    std::vector<int> rcol((size_t)P * rw, 0);
    std::vector<double> rval((size_t)P * rw, 0.0);
    for (int l = 0; l < P; ++l)
      for (size_t q = 0; q < rows[l].size(); ++q) {
        rcol[(size_t)l * rw + q] = rows[l][q].first;
        rval[(size_t)l * rw + q] = rows[l][q].second;
      }
    std::vector<double> Fs(2 * (size_t)P, 0.0), Us(2 * (size_t)P, 0.0);
    for (int j = 0; j < 2; ++j)
      for (int l = 0; l < P; ++l) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < P; ++i) {
          a = std::fma(s2c[(size_t)i * P + l], F[(size_t)j * P + i], a);
          b = std::fma(c2s[(size_t)l * P + i], bv[(size_t)j * P + i], b);
        }
        Fs[(size_t)j * P + l] = a;
        Us[(size_t)j * P + l] = b;
      }
    t.R_w = rw;
    UP(t.R_col, rcol.data(), rcol.size());
    UP(t.R_val, rval.data(), rval.size());
    UP(t.Fs, Fs.data(), Fs.size());
    UP(t.Us, Us.data(), Us.size());
    auto dfv = [](const std::vector<double>& v) {
      std::vector<dfl> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) o[i] = dfl(v[i]);
      return o;
    };
    std::vector<dfl> rvd = dfv(rval), fsd = dfv(Fs), usd = dfv(Us);
    UP(t.R_val_df, rvd.data(), rvd.size());
    UP(t.Fs_df, fsd.data(), fsd.size());
    UP(t.Us_df, usd.data(), usd.size());
  }

  // ---- shells present in the band ----
  {
    std::map<int, std::vector<int>> by_shell;
    for (int m = 0; m < M; ++m) by_shell[shell[m]].push_back(m);
    std::vector<int> start, modes;
    std::vector<int> used;
    for (auto& kv : by_shell) {
      used.push_back(kv.first);
      start.push_back((int)modes.size());
      for (int m : kv.second) modes.push_back(m);
      t.max_shell_modes = std::max(t.max_shell_modes, (int)kv.second.size());
    }
    start.push_back((int)modes.size());
    t.n_shells = (int)used.size();
    if (dalloc(c, &t.shell_inv, (size_t)t.n_shells * G * G) != cudaSuccess) return fail(NHQG_ERR_CUDA);
    for (int s = 0; s < t.n_shells; ++s) {
      if (cudaMemcpy(t.shell_inv + (size_t)s * G * G, g->shell_inv + (size_t)used[s] * G * G,
                     (size_t)G * G * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(NHQG_ERR_CUDA);
    }
    UP(t.shell_start, start.data(), start.size());
    UP(t.shell_modes, modes.data(), modes.size());
    // per-shell tau factors of the mixed-precision w solve
    if (g->shell_coef) {
      std::vector<int> mshell(M);
      std::vector<double> coef(2 * (size_t)t.n_shells);
      for (int sidx = 0; sidx < t.n_shells; ++sidx) {
        coef[2 * sidx] = g->shell_coef[2 * (size_t)used[sidx]];
        coef[2 * sidx + 1] = g->shell_coef[2 * (size_t)used[sidx] + 1];
        for (int q = start[sidx]; q < start[sidx + 1]; ++q) mshell[modes[q]] = sidx;
      }
      std::vector<double> tab, par, uni;
      build_tau_tables(N, p.wbc == NHQG_WBC_NEUMANN, t.n_shells, coef.data(), tab, par, uni);
      UP(t.mode_shell, mshell.data(), mshell.size());
      UP(t.tau_tab, tab.data(), tab.size());
      UP(t.tau_par, par.data(), par.size());
      UP(t.tau_uni, uni.data(), uni.size());
    }
  }

  // ---- tensor-core vertical transforms of the mixed-precision path ----
  if (g->shell_coef) {
    TcHostImage img[TC_IMAGES];
    if (tc_vertical_images(g, img)) {
      for (int i = 0; i < TC_IMAGES; ++i) {
        uint8_t* b = nullptr;
        float* x = nullptr;
        UP(b, img[i].bytes.data(), img[i].bytes.size());
        UP(x, img[i].xrow.data(), img[i].xrow.size());
        t.tc.img[i] = b;
        t.tc.xrow[i] = x;
        t.tc.K[i] = img[i].K;
        t.tc.rows[i] = img[i].rows;
        t.tc.nch[i] = img[i].nch;
      }
      const char* e = getenv("NHQG_TC_VERTICAL");
      p.tc_vertical = !(e && e[0] == '0');
    }
  }
  {
    // FP32 products with register-resident FFTs where the length allows
    // (NHQG_REG_FFT=0 selects the shared-memory FFT kernels)
    const char* e = getenv("NHQG_REG_FFT");
    p.reg_fft = !(e && e[0] == '0');
    // NHQG_CORR_WINDOW_OVERLAP=<rows> overrides the corrector's window overlap
    // (a tuning and test switch: every setting solves to FP64 round-off, small
    // overlaps through the fallback to one global factorisation)
    const char* ov = getenv("NHQG_CORR_WINDOW_OVERLAP");
    p.corr_win_ov = (ov && ov[0]) ? atoi(ov) : -1;
  }

  // ---- work buffers ----
  Work& w = c->w;
  const size_t fe = (size_t)P * M;
  double2** named[] = {&c->q0, &c->w0, &c->t0, &c->Qn, &c->Wn, &c->Tn, &c->Aq, &c->Aw, &c->At,
                       &c->E1q, &c->E1w, &c->E1t, &c->Rq, &c->Rt, &c->rhs, &c->Q1, &c->W1,
                       &c->T1p, &c->T1, &c->Q2, &c->W2, &c->T2p, &c->T2, &c->Wcgl, &c->Wsbp,
                       &c->Tsbp, &c->Tcgl};
  for (double2** f : named) {
    if (dalloc(c, f, fe) != cudaSuccess) return fail(NHQG_ERR_CUDA);
    if (cudaMemset(*f, 0, fe * sizeof(double2)) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  }
  if (p.scheme == NHQG_SCHEME_RK443 && p.exchange == NHQG_EXCHANGE_LEGACY) {
    for (int s = 0; s < 4; ++s) {
      for (int f = 0; f < 3; ++f) {
        if (dalloc(c, &c->rkE[s][f], fe) != cudaSuccess || dalloc(c, &c->rkK[s][f], fe) != cudaSuccess)
          return fail(NHQG_ERR_CUDA);
      }
      if (dalloc(c, &c->rkEtb[s], (size_t)P) != cudaSuccess ||
          dalloc(c, &c->rkKtb[s], (size_t)P) != cudaSuccess)
        return fail(NHQG_ERR_CUDA);
      // th_bar derivatives stay zero unless the legacy mean closure writes them
      if (cudaMemset(c->rkEtb[s], 0, P * sizeof(double)) != cudaSuccess ||
          cudaMemset(c->rkKtb[s], 0, P * sizeof(double)) != cudaSuccess)
        return fail(NHQG_ERR_CUDA);
    }
  }
  double** vecs[] = {&c->tb0, &c->tb1p, &c->tb1, &c->tb2p, &c->tb2, &c->E1tb, &c->E2tb, &c->Itb,
                     &c->flux, &c->dtb};
  for (double** v : vecs) {
    if (dalloc(c, v, (size_t)P) != cudaSuccess) return fail(NHQG_ERR_CUDA);
    cudaMemset(*v, 0, P * sizeof(double));
  }
  if (dalloc(c, &w.vec, corrector_vec_doubles(P)) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  cudaMemset(w.vec, 0, corrector_vec_doubles(P) * sizeof(double));
  if (dalloc(c, &w.partials, parseval_partials(P)) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  if (dalloc(c, &w.counters, (size_t)P + 1) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  if (cudaMemset(w.counters, 0, ((size_t)P + 1) * sizeof(unsigned)) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  if (dalloc(c, &w.mid_part, (size_t)P * corr_mid_ctas(p.d.M)) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  if (dalloc(c, &w.status, 4) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  cudaMemset(w.status, 0, 4 * sizeof(int));
  {
    const int nf1 = (p.advection == NHQG_ADV_JACOBIAN) ? 11 : 5;
    const int ng = (p.advection == NHQG_ADV_JACOBIAN) ? 3 : 6;
    w.x1_elems = (size_t)nf1 * P * d.Mc * d.Nh;
    w.x2_elems = (size_t)ng * P * d.Mc * d.Nh;
    // the plane API (full Nk columns, up to 11 fields) reuses these in level chunks
    const size_t plane_min = (size_t)11 * d.Nk * d.Nh;
    if (w.x1_elems < plane_min) w.x1_elems = plane_min;
    const size_t plane2_min = (size_t)6 * d.Mc * d.Nh;
    if (w.x2_elems < plane2_min) w.x2_elems = plane2_min;
    if (dalloc(c, &w.x1, w.x1_elems) != cudaSuccess) return fail(NHQG_ERR_CUDA);
    if (dalloc(c, &w.x2, w.x2_elems) != cudaSuccess) return fail(NHQG_ERR_CUDA);
  }
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(NHQG_ERR_CUDA);
#undef UP
  (void)rc;
  *out = c;
  return NHQG_OK;
}

int nhqg_ctx_destroy(nhqg_ctx* c) {
  if (!c) return NHQG_ERR_BAD_ARG;
  cudaDeviceSynchronize();
  free_all(c);
  delete c;
  return NHQG_OK;
}

int nhqg_get_device_status(nhqg_ctx* c, int reset) {
  if (!c) return NHQG_ERR_BAD_ARG;
  int s = 0;
  if (cudaMemcpy(&s, c->w.status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (reset) cudaMemset(c->w.status, 0, sizeof(int));
  return s;
}

int nhqg_last_launch_count(const nhqg_ctx* c) { return c ? c->launches : -1; }

int nhqg_profile_enable(nhqg_ctx* c, int on) {
  if (!c) return NHQG_ERR_BAD_ARG;
  c->w.prof.on = on != 0;
  c->w.prof.recs.clear();
  c->w.prof.next = 0;
  return NHQG_OK;
}

int nhqg_profile_report(nhqg_ctx* c, char* buf, int buflen) {
  if (!c || !buf || buflen <= 0) return NHQG_ERR_BAD_ARG;
  Profiler& pf = c->w.prof;
  if (cudaDeviceSynchronize() != cudaSuccess) return NHQG_ERR_CUDA;
  std::vector<std::string> names;
  std::map<std::string, std::pair<int, double>> acc;
  for (const auto& r : pf.recs) {
    if (!r.b) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) return NHQG_ERR_CUDA;
    auto it = acc.find(r.name);
    if (it == acc.end()) { names.push_back(r.name); acc[r.name] = {1, ms}; }
    else { it->second.first += 1; it->second.second += ms; }
  }
  std::string out;
  char line[160];
  for (const auto& n : names) {
    std::snprintf(line, sizeof(line), "%s %d %.6f\n", n.c_str(), acc[n].first, acc[n].second);
    out += line;
  }
  pf.recs.clear();
  pf.next = 0;
  std::snprintf(buf, (size_t)buflen, "%s", out.c_str());
  return (int)out.size() < buflen ? NHQG_OK : NHQG_ERR_BAD_ARG;
}

int nhqg_set_precision(nhqg_ctx* c, int precision) {
  if (!c) return NHQG_ERR_BAD_ARG;
  if (precision == NHQG_PRECISION_FP64) {
    if (c->precision != precision) ++c->version;
    c->precision = precision;
    return NHQG_OK;
  }
  if (precision != NHQG_PRECISION_MIXED) return NHQG_ERR_BAD_ARG;
  const Params& p = c->p;
  if (!p.fast_dct || !c->t.tw_v_f || !c->t.tau_tab) return NHQG_ERR_UNSUPPORTED;
  if (p.closure == NHQG_CLOSURE_EVOLVE_MEAN && p.exchange == NHQG_EXCHANGE_LEGACY)
    return NHQG_ERR_UNSUPPORTED;
  if (p.has_eta && !c->t.eta_x_f) return NHQG_ERR_UNSUPPORTED;  // no eta gradient tables
  if (!c->Qf) {
    const size_t fe = (size_t)p.d.P * p.d.M;
    float2** bufs[] = {&c->Qf, &c->Wf, &c->Tf, &c->Aqf, &c->Awf, &c->Atf};
    for (float2** b : bufs) {
      if (dalloc(c, b, fe) != cudaSuccess) return NHQG_ERR_CUDA;
      if (cudaMemset(*b, 0, fe * sizeof(float2)) != cudaSuccess) return NHQG_ERR_CUDA;
    }
  }
  if (c->precision != precision) ++c->version;
  c->precision = precision;
  return NHQG_OK;
}

int nhqg_set_mixed_vertical(nhqg_ctx* c, int tensor_cores) {
  if (!c) return NHQG_ERR_BAD_ARG;
  const bool on = tensor_cores != 0;
  if (on && !c->t.tc.img[0]) return NHQG_ERR_UNSUPPORTED;
  if (c->p.tc_vertical != on) ++c->version;
  c->p.tc_vertical = on;
  return NHQG_OK;
}

int nhqg_get_mixed_vertical(const nhqg_ctx* c) { return c && c->p.tc_vertical ? 1 : 0; }

int nhqg_tc_to_nodal(nhqg_ctx* c, int field, const void* coef, void* nodal, void* stream) {
  if (!c || !coef || !nodal || field < 0 || field > 2) return NHQG_ERR_BAD_ARG;
  if (!c->t.tc.img[0]) return NHQG_ERR_UNSUPPORTED;
  const double2* in[3] = {nullptr, nullptr, nullptr};
  float2* out[3] = {nullptr, nullptr, nullptr};
  in[field] = static_cast<const double2*>(coef);
  out[field] = static_cast<float2*>(nodal);
  CK(launch_tc_to_nodal(c->p, c->t, c->w, in[0], in[1], in[2], out[0], out[1], out[2],
                        static_cast<cudaStream_t>(stream)));
  return NHQG_OK;
}

int nhqg_tc_to_coef(nhqg_ctx* c, void* nodal_inout, void* stream) {
  if (!c || !nodal_inout) return NHQG_ERR_BAD_ARG;
  if (!c->t.tc.img[0]) return NHQG_ERR_UNSUPPORTED;
  CK(launch_tc_to_coef(c->p, c->t, c->w, static_cast<float2*>(nodal_inout), nullptr, nullptr, false,
                       static_cast<cudaStream_t>(stream)));
  return NHQG_OK;
}

}  // extern "C"

// ============================================================== orchestration
namespace {

cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

int gather_state(nhqg_ctx* c, const nhqg_state* s, cudaStream_t st) {
  const Params& p = c->p;
  if (!s || !s->q_hat || !s->w_hat || !s->th_hat || !s->th_bar) return NHQG_ERR_BAD_ARG;
  PCK("gather", launch_gather(p, (const double2*)s->q_hat, c->q0, p.d.P, c->w.status, st));
  PCK("gather", launch_gather(p, (const double2*)s->w_hat, c->w0, p.d.G, c->w.status, st));
  PCK("gather", launch_gather(p, (const double2*)s->th_hat, c->t0, p.d.G, c->w.status, st));
  CK(cudaMemcpyAsync(c->tb0, s->th_bar, p.d.P * sizeof(double), cudaMemcpyDeviceToDevice, st));
  c->launches += 3;
  return NHQG_OK;
}

int scatter_fields(nhqg_ctx* c, const double2* q, const double2* w, const double2* t,
                   const double* tb, nhqg_state* o, cudaStream_t st) {
  const Params& p = c->p;
  if (!o || !o->q_hat || !o->w_hat || !o->th_hat || !o->th_bar) return NHQG_ERR_BAD_ARG;
  PCK("scatter", launch_scatter(p, q, (double2*)o->q_hat, p.d.P, st));
  PCK("scatter", launch_scatter(p, w, (double2*)o->w_hat, p.d.G, st));
  PCK("scatter", launch_scatter(p, t, (double2*)o->th_hat, p.d.G, st));
  if (tb) {
    CK(cudaMemcpyAsync(o->th_bar, tb, p.d.P * sizeof(double), cudaMemcpyDeviceToDevice, st));
  } else {
    CK(cudaMemsetAsync(o->th_bar, 0, p.d.P * sizeof(double), st));
  }
  c->launches += 3;
  return NHQG_OK;
}

bool mixed(const nhqg_ctx* c) { return c->precision == NHQG_PRECISION_MIXED; }

// FP32 products of the mixed-precision path on the FP32 nodal fields
int horizontal_step_f32(nhqg_ctx* c, const float2* qn, const float2* wn, const float2* tn,
                        cudaStream_t st) {
  const Params& p = c->p;
  HorizArgsT<float2, float2> a{};
  a.form = p.advection == NHQG_ADV_JACOBIAN ? HF_JAC : HF_FLUX;
  a.sponge = p.has_sponge;
  a.eta = p.has_eta;
  a.full_in = false;
  a.full_out = false;
  a.psi_derived = true;
  a.levels = p.d.P;
  a.psi = nullptr; a.q = qn; a.w = wn; a.th = tn;
  a.Aq = c->Aqf; a.Aw = c->Awf; a.Ath = c->Atf;
  CK(launch_horizontal_f32(p, c->t, c->w, a, st, &c->launches));
  if (p.tc_vertical) {  // nodal A -> Chebyshev coefficients on the tensor cores
    PCK("tc_to_coef", launch_tc_to_coef(p, c->t, c->w, c->Aqf, c->Awf, c->Atf, true, st));
    c->launches += 1;
  }
  return NHQG_OK;
}

// FP32 nodal fields of the mixed path from FP64 coefficients (null = skip)
int to_nodal_f32(nhqg_ctx* c, const double2* q, const double2* w, const double2* t, cudaStream_t st) {
  const Params& p = c->p;
  if (p.tc_vertical) {
    PCK("tc_to_nodal", launch_tc_to_nodal(p, c->t, c->w, q, w, t, q ? c->Qf : nullptr,
                                          w ? c->Wf : nullptr, t ? c->Tf : nullptr, st));
  } else {
    PCK("vfwd_f32", launch_vfwd_f32(p, c->t, q, w, t, c->Qf, c->Wf, c->Tf, st));
  }
  c->launches += 1;
  return NHQG_OK;
}

int horizontal_step(nhqg_ctx* c, const double2* qn, const double2* wn, const double2* tn,
                    cudaStream_t st) {
  const Params& p = c->p;
  HorizArgs a{};
  a.form = p.advection == NHQG_ADV_JACOBIAN ? HF_JAC : HF_FLUX;
  a.sponge = p.has_sponge;
  a.eta = p.has_eta;
  a.full_in = false;
  a.full_out = false;
  a.psi_derived = true;
  a.levels = p.d.P;
  a.psi = nullptr; a.q = qn; a.w = wn; a.th = tn;
  a.Aq = c->Aq; a.Aw = c->Aw; a.Ath = c->At;
  CK(launch_horizontal(p, c->t, c->w, a, st, &c->launches));
  return NHQG_OK;
}

// explicit RHS at (q, w, t, tb) -> A in c->Aq/Aw/At (nodal) and, for the
// legacy evolve_mean closure, dtb (nodal dTheta/dZ) and E_tb.
int explicit_front(nhqg_ctx* c, const double2* q, const double2* w, const double2* t,
                   const double* tb, bool legacy_mean, double* Etb, double* Itb, bool need_q,
                   cudaStream_t st) {
  const Params& p = c->p;
  if (mixed(c)) {
    if (legacy_mean) return NHQG_ERR_UNSUPPORTED;
    int rc = to_nodal_f32(c, need_q ? q : nullptr, w, t, st);
    if (rc) return rc;
    return horizontal_step_f32(c, c->Qf, c->Wf, c->Tf, st);
  }
  PCK("vfwd", launch_vfwd(p, c->t, need_q ? q : nullptr, w, t, c->Qn, c->Wn, c->Tn, st));
  c->launches += 1;
  if (legacy_mean) {
    // <w theta>_xy on the padded grid equals the Parseval sum of the band-limited fields
    PCK("parseval", launch_parseval(p, c->Wn, c->Tn, p.d.P, c->flux, c->w, st));
    PCK("mean_1d", launch_mean_legacy_rhs(p, c->t, tb, c->flux, c->dtb, Etb, Itb, st));
    c->launches += 2;
  }
  return horizontal_step(c, c->Qn, c->Wn, c->Tn, st);
}

// the closure tendency of the q state the following vback reads
int closure_front(nhqg_ctx* c, const double2* q, cudaStream_t st) {
  if (!c->closure.w) return NHQG_OK;
  PCK("closure", launch_closure_apply(c->p, c->t, c->closure, q, c->Cq, st));
  c->launches += 1;
  return NHQG_OK;
}

VArgs base_vargs(nhqg_ctx* c) {
  VArgs a{};
  a.Cq = c->closure.w ? c->Cq : nullptr;
  a.Aq = c->Aq; a.Aw = c->Aw; a.At = c->At;
  if (mixed(c)) {
    a.Aqf = c->Aqf; a.Awf = c->Awf; a.Atf = c->Atf;
    a.af_coef = c->p.tc_vertical;
    a.df = true;  // double-float tiles where the operands arrive as coefficients
  }
  a.E1q = c->E1q; a.E1w = c->E1w; a.E1t = c->E1t;
  a.Wn = c->Wn;
  a.Rq = c->Rq; a.Rt = c->Rt; a.rhs_w = c->rhs;
  return a;
}

int solve_back(nhqg_ctx* c, double2* qo, double2* wo, double2* to, bool zero_mean, cudaStream_t st) {
  const Params& p = c->p;
  if (mixed(c)) {
    // scratch: the FP64 explicit operand of the plain path, idle in the mixed step
    PCK("tau_solve", launch_tau_solve(p, c->t, c->rhs, wo, c->Aq, st));
  } else {
    PCK("shell_solve", launch_shell(p, c->t, c->rhs, wo, st));
  }
  PCK("vpost", launch_vpost(p, c->t, c->Rq, c->Rt, wo, qo, to, zero_mean, st, mixed(c)));
  c->launches += 2;
  return NHQG_OK;
}

// ---- ARS(4,4,3) (nhqg/solver.py:1056-1122), gamma = 1/2 in the tables
// Tableau rows: (coefficient, term) with term 0..3 = K_1..K_4, 4..7 = E_0..E_3;
// stage i solves y_n + dt * sum(c X) of row i, the last row is y_{n+1}.
struct RkRow {
  int n;
  double c[8];
  int x[8];
};
const RkRow kRk443[5] = {
    {1, {0.5}, {4}},
    {3, {1.0 / 6.0, 11.0 / 18.0, 1.0 / 18.0}, {0, 4, 5}},
    {5, {-0.5, 0.5, 5.0 / 6.0, -5.0 / 6.0, 0.5}, {0, 1, 4, 5, 6}},
    {7, {1.5, -1.5, 0.5, 0.25, 1.75, 0.75, -1.75}, {0, 1, 2, 4, 5, 6, 7}},
    {8, {1.5, -1.5, 0.5, 0.5, 0.25, 1.75, 0.75, -1.75}, {0, 1, 2, 3, 4, 5, 6, 7}},
};

// y_n + dt * (row terms) -> (Q2, W2, T2p, tb2p)
int rk_combine(nhqg_ctx* c, const RkRow& row, cudaStream_t st) {
  const Params& p = c->p;
  const double2* base[3] = {c->q0, c->w0, c->t0};
  double2* out[3] = {c->Q2, c->W2, c->T2p};
  const int levels[3] = {p.d.P, p.d.G, p.d.G};
  for (int f = 0; f < 3; ++f) {
    LinCombT<double2> a{};
    a.base = base[f];
    a.out = out[f];
    a.n = row.n;
    a.dt = p.dt;
    a.count = (size_t)levels[f] * p.d.M;
    for (int k = 0; k < row.n; ++k) {
      a.c[k] = row.c[k];
      a.x[k] = row.x[k] < 4 ? c->rkK[row.x[k]][f] : c->rkE[row.x[k] - 4][f];
    }
    PCK("rk_combine", launch_lincomb(a, st));
  }
  LinCombT<double> b{};
  b.base = c->tb0;
  b.out = c->tb2p;
  b.n = row.n;
  b.dt = p.dt;
  b.count = (size_t)p.d.P;
  for (int k = 0; k < row.n; ++k) {
    b.c[k] = row.c[k];
    b.x[k] = row.x[k] < 4 ? c->rkKtb[row.x[k]] : c->rkEtb[row.x[k] - 4];
  }
  PCK("rk_combine", launch_lincomb(b, st));
  c->launches += 4;
  return NHQG_OK;
}

// E_s = explicit_rhs_dispatch(Y) into the RK buffers (legacy exchange)
int rk_explicit(nhqg_ctx* c, int s, const double2* q, const double2* w, const double2* t,
                const double* tb, cudaStream_t st) {
  const bool legacy_mean = c->p.closure == NHQG_CLOSURE_EVOLVE_MEAN;
  int rc = explicit_front(c, q, w, t, tb, legacy_mean, c->rkEtb[s], nullptr, true, st);
  if (rc) return rc;
  if ((rc = closure_front(c, q, st))) return rc;
  VArgs a = base_vargs(c);
  a.q0 = q; a.w0 = w; a.t0 = t;
  a.dtb_nodal = legacy_mean ? c->dtb : nullptr;
  a.Eq = c->rkE[s][0]; a.Ew = c->rkE[s][1]; a.Et = c->rkE[s][2];
  PCK("vback_rhs", launch_vback(c->p, c->t, VB_RHS, a, st));
  c->launches += 1;
  return NHQG_OK;
}

int one_step_rk443(nhqg_ctx* c, cudaStream_t st) {
  const Params& p = c->p;
  if (mixed(c) || !c->rkE[0][0]) return NHQG_ERR_UNSUPPORTED;
  const bool evolve = p.closure == NHQG_CLOSURE_EVOLVE_MEAN;
  int rc = rk_explicit(c, 0, c->q0, c->w0, c->t0, c->tb0, st);
  if (rc) return rc;
  for (int i = 1; i <= 4; ++i) {
    if ((rc = rk_combine(c, kRk443[i - 1], st))) return rc;
    // Y_i = implicit solve of the combination (imex_implicit_solve, imex_mean_temp_solve)
    VArgs a = base_vargs(c);
    a.q0 = c->Q2; a.w0 = c->W2; a.t0 = c->T2p;
    PCK("vback_solve", launch_vback(p, c->t, VB_SOLVE, a, st));
    MeanArgs m{};
    m.tb0 = c->tb2p; m.out = c->tb1; m.stage = 1; m.closure = p.closure;
    PCK("mean_1d", launch_mean_stage(p, c->t, m, st));
    c->launches += 2;
    if ((rc = solve_back(c, c->Q1, c->W1, c->T1, false, st))) return rc;
    // K_i = implicit_tendency(Y_i) - dissipation (nhqg/solver.py:1002-1009)
    double2* const* K = c->rkK[i - 1];
    PCK("itend", launch_itend(p, c->t, c->Q1, c->W1, c->T1, K[0], K[1], K[2], st));
    PCK("itend", launch_sub_diss(p, K[0], c->Q1, c->t.drq, p.d.P, st));
    PCK("itend", launch_sub_diss(p, K[1], c->W1, c->t.drw, p.d.G, st));
    PCK("itend", launch_sub_diss(p, K[2], c->T1, c->t.drt, p.d.G, st));
    c->launches += 4;
    if (evolve) {
      PCK("mean_1d", launch_mean_legacy_rhs(p, c->t, c->tb1, nullptr, nullptr, nullptr, c->rkKtb[i - 1], st));
      c->launches += 1;
    }
    if (i < 4 && (rc = rk_explicit(c, i, c->Q1, c->W1, c->T1, c->tb1, st))) return rc;
  }
  if ((rc = rk_combine(c, kRk443[4], st))) return rc;
  PCK("finalize", launch_finalize(p, c->Q2, c->W2, c->T2p, c->q0, c->w0, c->t0, st));
  CK(cudaMemcpyAsync(c->tb0, c->tb2p, p.d.P * sizeof(double), cudaMemcpyDeviceToDevice, st));
  c->launches += 1;
  return NHQG_OK;
}

// one step from (q0,w0,t0,tb0); result left in (q0,w0,t0,tb0).  ARS(2,2,2)
// unless the scheme is RK443 with the legacy exchange (nhqg/solver.py:1228-1242)
int one_step(nhqg_ctx* c, cudaStream_t st) {
  const Params& p = c->p;
  if (p.scheme == NHQG_SCHEME_RK443 && p.exchange == NHQG_EXCHANGE_LEGACY) return one_step_rk443(c, st);
  const double dt = p.dt, g = p.gamma_imex;
  const double alpha = g * dt;
  const double delta = -std::sqrt(2.0) / 2.0;
  const double omega = dt * (1.0 - g);
  const bool split = p.exchange != NHQG_EXCHANGE_LEGACY;
  const bool evolve = p.closure == NHQG_CLOSURE_EVOLVE_MEAN;
  const bool legacy_mean = evolve && !split;
  const bool pc = p.exchange == NHQG_EXCHANGE_BALANCED_SBP2_PC;
  const int base_closure = split ? NHQG_CLOSURE_FIXED_CONDUCTION : p.closure;
  int rc;

  // ---------------- stage 1
  rc = explicit_front(c, c->q0, c->w0, c->t0, c->tb0, legacy_mean, c->E1tb, nullptr, true, st);
  if (rc) return rc;
  if ((rc = closure_front(c, c->q0, st))) return rc;
  VArgs a = base_vargs(c);
  a.q0 = c->q0; a.w0 = c->w0; a.t0 = c->t0;
  a.dtb_nodal = legacy_mean ? c->dtb : nullptr;
  a.alpha = alpha;
  PCK("vback_stage1", launch_vback(p, c->t, VB_STAGE1, a, st));
  MeanArgs m1{};
  m1.tb0 = c->tb0; m1.E1tb = legacy_mean ? c->E1tb : nullptr; m1.out = c->tb1p;
  m1.alpha = alpha; m1.stage = 1; m1.closure = base_closure;
  PCK("mean_1d", launch_mean_stage(p, c->t, m1, st));
  c->launches += 2;
  if ((rc = solve_back(c, c->Q1, c->W1, c->T1p, false, st))) return rc;

  // stage-1 corrector (pc only)
  const double2* t1 = c->T1p;
  const double* tb1 = c->tb1p;
  bool have_nodal_wt = false;
  if (pc && evolve) {
    CorrArgs ca{};
    ca.wp = c->W1; ca.tp = c->T1p; ca.tbp = c->tb1p;
    ca.t_out = c->T1; ca.tb_out = c->tb1;
    ca.wcgl = c->Wcgl; ca.wsbp = c->Wsbp; ca.tsbp = c->Tsbp; ca.tcgl = c->Tcgl;
    ca.total_dt = alpha;
    ca.df = mixed(c);
    // nodal w and theta of state1 straight to the FP32 products
    ca.wcgl_f = mixed(c) ? c->Wf : nullptr;
    ca.tcgl_f = mixed(c) ? c->Tf : nullptr;
    CK(run_corrector(p, c->t, c->w, ca, st, &c->launches));
    t1 = c->T1;
    tb1 = c->tb1;
    have_nodal_wt = true;
  }

  // ---------------- stage 2
  if (have_nodal_wt) {
    // nodal w and theta of state1 come out of the corrector
    if (mixed(c)) {
      if ((rc = to_nodal_f32(c, c->Q1, nullptr, nullptr, st))) return rc;
      if ((rc = horizontal_step_f32(c, c->Qf, c->Wf, c->Tf, st))) return rc;
    } else {
      PCK("vfwd", launch_vfwd(p, c->t, c->Q1, nullptr, nullptr, c->Qn, nullptr, nullptr, st));
      c->launches += 1;
      if ((rc = horizontal_step(c, c->Qn, c->Wcgl, c->Tcgl, st))) return rc;
    }
  } else {
    rc = explicit_front(c, c->Q1, c->W1, t1, tb1, legacy_mean, c->E2tb, c->Itb, true, st);
    if (rc) return rc;
  }
  if ((rc = closure_front(c, c->Q1, st))) return rc;
  a = base_vargs(c);
  a.q0 = c->q0; a.w0 = c->w0; a.t0 = c->t0;
  a.q1 = c->Q1; a.w1 = c->W1; a.t1 = t1; a.t1p = c->T1p;
  a.Wn = have_nodal_wt ? c->Wcgl : c->Wn;
  a.dtb_nodal = legacy_mean ? c->dtb : nullptr;
  a.c_E1 = dt * delta;
  a.c_E2 = dt * (1.0 - delta);
  a.omega = omega;
  a.inv_alpha_c = (pc && evolve) ? 1.0 / alpha : 0.0;
  PCK("vback_stage2", launch_vback(p, c->t, VB_STAGE2, a, st));
  MeanArgs m2{};
  m2.tb0 = c->tb0; m2.E1tb = legacy_mean ? c->E1tb : nullptr; m2.E2tb = legacy_mean ? c->E2tb : nullptr;
  m2.tb1 = tb1; m2.tb1p = c->tb1p; m2.out = c->tb2p;
  m2.c_E1 = dt * delta; m2.c_E2 = dt * (1.0 - delta); m2.omega = omega;
  m2.inv_alpha_c = (pc && evolve) ? 1.0 / alpha : 0.0;
  m2.stage = 2; m2.closure = base_closure; m2.itend = legacy_mean ? 1 : 0;
  PCK("mean_1d", launch_mean_stage(p, c->t, m2, st));
  c->launches += 2;
  // balanced_sbp2 (split, not pc) finalizes the base step before its corrector
  const bool split_plain = split && !pc && evolve;
  if ((rc = solve_back(c, c->Q2, c->W2, c->T2p, split_plain, st))) return rc;

  const double2* t2 = c->T2p;
  const double* tb2 = c->tb2p;
  if (split && evolve) {
    CorrArgs ca{};
    ca.wp = c->W2; ca.tp = c->T2p; ca.tbp = c->tb2p;
    ca.t_out = c->T2; ca.tb_out = c->tb2;
    ca.wcgl = c->Wcgl; ca.wsbp = c->Wsbp; ca.tsbp = c->Tsbp; ca.tcgl = nullptr;
    ca.total_dt = pc ? alpha : dt;
    ca.df = mixed(c);
    if (split_plain) {  // the base step's finalize zeroed the k=0 mode of w
      PCK("finalize", launch_zero_mode0(p, c->W2, p.d.G, st));
      c->launches += 1;
    }
    CK(run_corrector(p, c->t, c->w, ca, st, &c->launches));
    t2 = c->T2;
    tb2 = c->tb2;
  }
  PCK("finalize", launch_finalize(p, c->Q2, c->W2, t2, c->q0, c->w0, c->t0, st));
  CK(cudaMemcpyAsync(c->tb0, tb2, p.d.P * sizeof(double), cudaMemcpyDeviceToDevice, st));
  c->launches += 1;
  return NHQG_OK;
}

}  // namespace

extern "C" {

int nhqg_step(nhqg_ctx* c, nhqg_state* s, int n_steps, void* stream) {
  if (!c || !s || n_steps < 0) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  c->launches = 0;
  int rc = gather_state(c, s, st);
  if (rc) return rc;
  for (int i = 0; i < n_steps; ++i)
    if ((rc = one_step(c, st))) return rc;
  return scatter_fields(c, c->q0, c->w0, c->t0, c->tb0, s, st);
}

int nhqg_explicit_rhs(nhqg_ctx* c, const nhqg_state* in, nhqg_state* out, int closure,
                      int exchange, void* stream) {
  if (!c) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  c->launches = 0;
  int rc = gather_state(c, in, st);
  if (rc) return rc;
  const bool legacy_mean = closure == NHQG_CLOSURE_EVOLVE_MEAN && exchange == NHQG_EXCHANGE_LEGACY;
  if (legacy_mean && !c->t.mean_solve) return NHQG_ERR_UNSUPPORTED;
  rc = explicit_front(c, c->q0, c->w0, c->t0, c->tb0, legacy_mean, c->E1tb, nullptr, true, st);
  if (rc) return rc;
  if ((rc = closure_front(c, c->q0, st))) return rc;
  VArgs a = base_vargs(c);
  a.q0 = c->q0; a.w0 = c->w0; a.t0 = c->t0;
  a.dtb_nodal = legacy_mean ? c->dtb : nullptr;
  a.Eq = c->E1q; a.Ew = c->E1w; a.Et = c->E1t;
  CK(launch_vback(c->p, c->t, VB_RHS, a, st));
  c->launches += 1;
  return scatter_fields(c, c->E1q, c->E1w, c->E1t, legacy_mean ? c->E1tb : nullptr, out, st);
}

int nhqg_implicit_tendency(nhqg_ctx* c, const nhqg_state* in, nhqg_state* out, int closure,
                           void* stream) {
  if (!c) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  c->launches = 0;
  int rc = gather_state(c, in, st);
  if (rc) return rc;
  CK(launch_itend(c->p, c->t, c->q0, c->w0, c->t0, c->Aq, c->Aw, c->At, st));
  c->launches += 1;
  const bool evolve = closure == NHQG_CLOSURE_EVOLVE_MEAN;
  if (evolve) {
    CK(launch_mean_legacy_rhs(c->p, c->t, c->tb0, nullptr, nullptr, nullptr, c->Itb, st));
    c->launches += 1;
  }
  return scatter_fields(c, c->Aq, c->Aw, c->At, evolve ? c->Itb : nullptr, out, st);
}

int nhqg_implicit_solve(nhqg_ctx* c, const nhqg_state* rhs, nhqg_state* out, int closure,
                        void* stream) {
  if (!c) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  c->launches = 0;
  if (closure == NHQG_CLOSURE_EVOLVE_MEAN && !c->t.mean_solve) return NHQG_ERR_UNSUPPORTED;
  int rc = gather_state(c, rhs, st);
  if (rc) return rc;
  VArgs a = base_vargs(c);
  a.q0 = c->q0; a.w0 = c->w0; a.t0 = c->t0;
  CK(launch_vback(c->p, c->t, VB_SOLVE, a, st));
  MeanArgs m{};
  m.tb0 = c->tb0; m.out = c->tb1p; m.stage = 1; m.closure = closure;
  CK(launch_mean_stage(c->p, c->t, m, st));
  c->launches += 2;
  if ((rc = solve_back(c, c->Q1, c->W1, c->T1p, false, st))) return rc;
  return scatter_fields(c, c->Q1, c->W1, c->T1p, c->tb1p, out, st);
}

int nhqg_sbp2_corrector(nhqg_ctx* c, const nhqg_state* in, nhqg_state* out, double total_dt,
                        void* stream) {
  if (!c) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  c->launches = 0;
  int rc = gather_state(c, in, st);
  if (rc) return rc;
  if (c->p.closure != NHQG_CLOSURE_EVOLVE_MEAN)
    return scatter_fields(c, c->q0, c->w0, c->t0, c->tb0, out, st);
  CorrArgs ca{};
  ca.wp = c->w0; ca.tp = c->t0; ca.tbp = c->tb0;
  ca.t_out = c->T1; ca.tb_out = c->tb1;
  ca.wcgl = c->Wcgl; ca.wsbp = c->Wsbp; ca.tsbp = c->Tsbp; ca.tcgl = nullptr;
  ca.total_dt = total_dt;
  CK(run_corrector(c->p, c->t, c->w, ca, st, &c->launches));
  return scatter_fields(c, c->q0, c->w0, c->T1, c->tb1, out, st);
}

int nhqg_diagnostics(nhqg_ctx* c, const nhqg_state* s, double* out, void* stream) {
  if (!c || !out) return NHQG_ERR_BAD_ARG;
  if (!c->t.cc) return NHQG_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  c->launches = 0;
  int rc = gather_state(c, s, st);
  if (rc) return rc;
  const Params& p = c->p;
  CK(launch_vfwd(p, c->t, c->q0, c->w0, c->t0, c->Qn, c->Wn, c->Tn, st));
  CK(launch_diag_modes(p, c->t, c->Qn, c->Wn, c->Tn, c->diag_part, st));
  const bool sbp = p.exchange == NHQG_EXCHANGE_BALANCED_SBP2 || p.exchange == NHQG_EXCHANGE_BALANCED_SBP2_PC;
  if (sbp) {
    CK(launch_corr_pre(p, c->t, c->w0, c->t0, c->Wcgl, c->Wsbp, c->Tsbp, st));
    CK(launch_parseval(p, c->Wsbp, c->Tsbp, p.d.P, c->flux, c->w, st));
  } else {
    CK(launch_parseval(p, c->Wn, c->Tn, p.d.P, c->flux, c->w, st));
  }
  if (p.plan_nx.npass > 0) {
    CK(launch_phys_maxima(p, c->t, c->w, c->Qn, c->Wn, c->Tn, c->diag_max, st));
    c->launches += 3;
  } else {
    CK(cudaMemsetAsync(c->diag_max, 0xff, kDiagMaxima * sizeof(unsigned long long), st));  // NaN
  }
  CK(launch_diag_final(p, c->t, c->diag_part, c->flux, sbp, c->tb0, c->diag_max, out, st));
  c->launches += sbp ? 5 : 4;
  return NHQG_OK;
}

int nhqg_spectra(nhqg_ctx* c, const nhqg_state* s, const int* mode_bin, int n_bins, double* out,
                 void* stream) {
  if (!c || !out || !mode_bin || n_bins <= 0) return NHQG_ERR_BAD_ARG;
  if (!c->t.cc) return NHQG_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  c->launches = 0;
  if (!c->spec_mode && dalloc(c, &c->spec_mode, 5 * (size_t)c->p.d.M) != cudaSuccess)
    return NHQG_ERR_CUDA;
  int rc = gather_state(c, s, st);
  if (rc) return rc;
  const Params& p = c->p;
  CK(launch_vfwd(p, c->t, c->q0, c->w0, c->t0, c->Qn, c->Wn, c->Tn, st));
  CK(launch_spectra(p, c->t, c->Qn, c->Wn, c->Tn, c->q0, c->w0, c->t0, mode_bin, n_bins, c->spec_mode,
                    out, st));
  c->launches += 4;
  return NHQG_OK;
}

int nhqg_sanitize(nhqg_ctx* c, nhqg_state* s, void* stream) {
  if (!c) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  c->launches = 0;
  int rc = gather_state(c, s, st);
  if (rc) return rc;
  CK(launch_hermitian(c->p, c->q0, c->w0, c->t0, st));
  c->launches += 1;
  return scatter_fields(c, c->q0, c->w0, c->t0, c->tb0, s, st);
}

int nhqg_mean_temp_solve(nhqg_ctx* c, const double* R, double* out, int closure, void* stream) {
  if (!c || !R || !out) return NHQG_ERR_BAD_ARG;
  if (closure == NHQG_CLOSURE_EVOLVE_MEAN && !c->t.mean_solve) return NHQG_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  c->launches = 0;
  MeanArgs m{};
  m.tb0 = R; m.out = out; m.stage = 1; m.closure = closure;
  CK(launch_mean_stage(c->p, c->t, m, st));
  c->launches = 1;
  return NHQG_OK;
}

}  // extern "C"

namespace {

// Plane APIs: products of caller-supplied nodal planes in the full rfft2
// layout, in level chunks that fit the step's workspace.  The context's
// dealiasing rule (pad32) selects the 2/3 or the 3/2 products.
int plane_advection(nhqg_ctx* c, bool pad32, int advection, int levels, const void* psi,
                    const void* q, const void* w, const void* th, void* Aq, void* Aw, void* Ath,
                    void* stream) {
  if (!c || levels <= 0 || !psi || !q || !w || !th || !Aq || !Aw || !Ath) return NHQG_ERR_BAD_ARG;
  if (advection != NHQG_ADV_FLUX && advection != NHQG_ADV_JACOBIAN) return NHQG_ERR_UNSUPPORTED;
  if (c->p.d.pad != pad32) return NHQG_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  c->launches = 0;
  const Dims& d = c->p.d;
  const size_t plane = (size_t)d.Nx * d.Nk;
  const int nf1 = advection == NHQG_ADV_JACOBIAN ? 8 : 5;
  const int ng = advection == NHQG_ADV_JACOBIAN ? 3 : 6;
  int chunk = (int)std::min(c->w.x1_elems / ((size_t)nf1 * d.Nk * d.Nh),
                            c->w.x2_elems / ((size_t)ng * d.Mc * d.Nh));
  if (chunk < 1) return NHQG_ERR_UNSUPPORTED;
  CK(cudaMemsetAsync(Aq, 0, (size_t)levels * plane * sizeof(double2), st));
  CK(cudaMemsetAsync(Aw, 0, (size_t)levels * plane * sizeof(double2), st));
  CK(cudaMemsetAsync(Ath, 0, (size_t)levels * plane * sizeof(double2), st));
  for (int l0 = 0; l0 < levels; l0 += chunk) {
    const int nl = std::min(chunk, levels - l0);
    HorizArgs a{};
    a.form = advection == NHQG_ADV_JACOBIAN ? HF_JAC : HF_FLUX;
    a.sponge = false; a.eta = false; a.full_in = true; a.full_out = true; a.psi_derived = false;
    a.levels = nl;
    const size_t off = (size_t)l0 * plane;
    a.psi = (const double2*)psi + off; a.q = (const double2*)q + off;
    a.w = (const double2*)w + off; a.th = (const double2*)th + off;
    a.Aq = (double2*)Aq + off; a.Aw = (double2*)Aw + off; a.Ath = (double2*)Ath + off;
    CK(launch_horizontal(c->p, c->t, c->w, a, st, &c->launches));
  }
  return NHQG_OK;
}

int plane_sponge(nhqg_ctx* c, bool pad32, int levels, const void* f, void* out, void* stream) {
  if (!c || levels <= 0 || !f || !out) return NHQG_ERR_BAD_ARG;
  if (!c->p.has_sponge || c->p.d.pad != pad32) return NHQG_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  c->launches = 0;
  const Dims& d = c->p.d;
  const size_t plane = (size_t)d.Nx * d.Nk;
  int chunk = (int)std::min(c->w.x1_elems / ((size_t)d.Nk * d.Nh), c->w.x2_elems / ((size_t)d.Mc * d.Nh));
  if (chunk < 1) return NHQG_ERR_UNSUPPORTED;
  CK(cudaMemsetAsync(out, 0, (size_t)levels * plane * sizeof(double2), st));
  for (int l0 = 0; l0 < levels; l0 += chunk) {
    const int nl = std::min(chunk, levels - l0);
    HorizArgs a{};
    a.form = HF_SPONGE;
    a.sponge = true; a.eta = false; a.full_in = true; a.full_out = true; a.psi_derived = false;
    a.levels = nl;
    const size_t off = (size_t)l0 * plane;
    a.q = (const double2*)f + off;
    a.Aq = (double2*)out + off; a.Aw = nullptr; a.Ath = nullptr;
    CK(launch_horizontal(c->p, c->t, c->w, a, st, &c->launches));
  }
  return NHQG_OK;
}

}  // namespace

extern "C" {

int nhqg_triple_advection_23(nhqg_ctx* c, int advection, int levels, const void* psi,
                             const void* q, const void* w, const void* th, void* Aq, void* Aw,
                             void* Ath, void* stream) {
  return plane_advection(c, false, advection, levels, psi, q, w, th, Aq, Aw, Ath, stream);
}

int nhqg_triple_advection_32(nhqg_ctx* c, int advection, int levels, const void* psi,
                             const void* q, const void* w, const void* th, void* Aq, void* Aw,
                             void* Ath, void* stream) {
  return plane_advection(c, true, advection, levels, psi, q, w, th, Aq, Aw, Ath, stream);
}

int nhqg_sponge_product_23(nhqg_ctx* c, int levels, const void* f, void* out, void* stream) {
  return plane_sponge(c, false, levels, f, out, stream);
}

int nhqg_sponge_product_32(nhqg_ctx* c, int levels, const void* f, void* out, void* stream) {
  return plane_sponge(c, true, levels, f, out, stream);
}

}  // extern "C"

// ============================================================== batches and tiles
struct nhqg_batch {
  std::vector<nhqg_ctx*> members;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr;
  int spl = 1;  // steps per graph launch
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    int steps = 0;
    std::vector<unsigned> versions;
  } g_many, g_one;
};

namespace {

void drop_graph(nhqg_batch::Graph& g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  g.exec = nullptr;
  g.versions.clear();
}

bool graph_current(const nhqg_batch* b, const nhqg_batch::Graph& g) {
  if (!g.exec || g.versions.size() != b->members.size()) return false;
  for (size_t i = 0; i < b->members.size(); ++i)
    if (g.versions[i] != b->members[i]->version) return false;
  return true;
}

// Capture `steps` steps of every member, each on its own stream forked from
// and joined into the origin stream, into one executable graph.
int capture(nhqg_batch* b, nhqg_batch::Graph& g, int steps) {
  drop_graph(g);
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed));
  int rc = NHQG_OK;
  if (cudaEventRecord(b->fork, b->origin) != cudaSuccess) rc = NHQG_ERR_CUDA;
  for (size_t i = 0; i < b->members.size() && rc == NHQG_OK; ++i) {
    nhqg_ctx* c = b->members[i];
    cudaStream_t st = b->streams[i];
    const bool prof = c->w.prof.on;
    c->w.prof.on = false;  // no event records inside a graph
    if (cudaStreamWaitEvent(st, b->fork, 0) != cudaSuccess) rc = NHQG_ERR_CUDA;
    for (int k = 0; k < steps && rc == NHQG_OK; ++k) rc = one_step(c, st);
    if (rc == NHQG_OK && cudaEventRecord(b->joins[i], st) != cudaSuccess) rc = NHQG_ERR_CUDA;
    if (rc == NHQG_OK && cudaStreamWaitEvent(b->origin, b->joins[i], 0) != cudaSuccess) rc = NHQG_ERR_CUDA;
    c->w.prof.on = prof;
  }
  const cudaError_t e = cudaStreamEndCapture(b->origin, &graph);
  if (rc != NHQG_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc != NHQG_OK ? rc : NHQG_ERR_CUDA;
  }
  const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return NHQG_ERR_CUDA;
  g.steps = steps;
  for (nhqg_ctx* c : b->members) g.versions.push_back(c->version);
  return NHQG_OK;
}

// time one horizontal-product evaluation (ms, median of 3) with the current tiles
float time_products(nhqg_ctx* c, bool f32, cudaStream_t st) {
  cudaEvent_t a, z;
  cudaEventCreate(&a);
  cudaEventCreate(&z);
  float best = -1.f;
  std::vector<float> t;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, st);
    const int rc = f32 ? horizontal_step_f32(c, c->Qf, c->Wf, c->Tf, st)
                       : horizontal_step(c, c->Qn, c->Wn, c->Tn, st);
    cudaEventRecord(z, st);
    if (rc != NHQG_OK || cudaEventSynchronize(z) != cudaSuccess) {
      cudaGetLastError();
      t.clear();
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, z);
    if (rep > 0) t.push_back(ms);  // the first run warms up
  }
  if (t.size() == 3) {
    std::sort(t.begin(), t.end());
    best = t[1];
  }
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  return best;
}

}  // namespace

extern "C" {

int nhqg_get_tiles(const nhqg_ctx* c, int* tiles) {
  if (!c || !tiles) return NHQG_ERR_BAD_ARG;
  tiles[0] = c->p.h_col_kib[0]; tiles[1] = c->p.h_row_kib[0];
  tiles[2] = c->p.h_col_kib[1]; tiles[3] = c->p.h_row_kib[1];
  return NHQG_OK;
}

int nhqg_set_tiles(nhqg_ctx* c, const int* tiles) {
  if (!c || !tiles) return NHQG_ERR_BAD_ARG;
  for (int i = 0; i < 4; ++i)
    if (tiles[i] < 0 || tiles[i] > 200) return NHQG_ERR_BAD_ARG;
  c->p.h_col_kib[0] = tiles[0]; c->p.h_row_kib[0] = tiles[1];
  c->p.h_col_kib[1] = tiles[2]; c->p.h_row_kib[1] = tiles[3];
  ++c->version;
  return NHQG_OK;
}

int nhqg_autotune(nhqg_ctx* c, void* stream) {
  if (!c) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  const bool prof = c->w.prof.on;
  c->w.prof.on = false;
  static const int col64[] = {24, 48, 96, 144}, row64[] = {25, 50, 100, 200};
  static const int col32[] = {6, 12, 24, 44, 64}, row32[] = {13, 26, 52, 104};
  for (int pi = 0; pi < 2; ++pi) {
    const bool f32 = pi == 1;
    if (f32 && !c->Qf) continue;  // FP32 buffers exist once the mixed path is enabled
    const int* cols = f32 ? col32 : col64;
    const int* rows = f32 ? row32 : row64;
    const int nc = f32 ? 5 : 4, nr = 4;
    int best_c = 0, best_r = 0;
    float best = -1.f;
    for (int i = 0; i < nc; ++i)
      for (int j = 0; j < nr; ++j) {
        c->p.h_col_kib[pi] = cols[i];
        c->p.h_row_kib[pi] = rows[j];
        const float ms = time_products(c, f32, st);
        if (ms > 0.f && (best < 0.f || ms < best)) { best = ms; best_c = cols[i]; best_r = rows[j]; }
      }
    c->p.h_col_kib[pi] = best_c;  // 0 (built-in default) if nothing ran
    c->p.h_row_kib[pi] = best_r;
  }
  c->w.prof.on = prof;
  ++c->version;
  return cudaGetLastError() == cudaSuccess ? NHQG_OK : NHQG_ERR_CUDA;
}

int nhqg_batch_create(nhqg_ctx* const* members, int n, int steps_per_launch, nhqg_batch** out) {
  if (!members || n <= 0 || steps_per_launch <= 0 || !out) return NHQG_ERR_BAD_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (!members[i] || members[i] == members[j]) return NHQG_ERR_BAD_ARG;
  nhqg_batch* b = new (std::nothrow) nhqg_batch();
  if (!b) return NHQG_ERR_BAD_ARG;
  b->members.assign(members, members + n);
  b->spl = steps_per_launch;
  bool ok = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; i < n && ok; ++i) {
    cudaStream_t st;
    cudaEvent_t ev;
    ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
    if (ok) { b->streams.push_back(st); b->joins.push_back(ev); }
  }
  if (!ok) { nhqg_batch_destroy(b); return NHQG_ERR_CUDA; }
  *out = b;
  return NHQG_OK;
}

int nhqg_batch_destroy(nhqg_batch* b) {
  if (!b) return NHQG_ERR_BAD_ARG;
  if (b->origin) cudaStreamSynchronize(b->origin);
  drop_graph(b->g_many);
  drop_graph(b->g_one);
  for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
  for (cudaEvent_t ev : b->joins) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
  return NHQG_OK;
}

int nhqg_batch_load(nhqg_batch* b, int member, const nhqg_state* s, void* stream) {
  if (!b || member < 0 || member >= (int)b->members.size()) return NHQG_ERR_BAD_ARG;
  nhqg_ctx* c = b->members[member];
  c->launches = 0;
  return gather_state(c, s, S(stream));
}

int nhqg_batch_store(nhqg_batch* b, int member, nhqg_state* s, void* stream) {
  if (!b || member < 0 || member >= (int)b->members.size()) return NHQG_ERR_BAD_ARG;
  nhqg_ctx* c = b->members[member];
  return scatter_fields(c, c->q0, c->w0, c->t0, c->tb0, s, S(stream));
}

int nhqg_batch_step(nhqg_batch* b, int n_steps, void* stream) {
  if (!b || n_steps < 0) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  const int q = n_steps / b->spl, r = n_steps % b->spl;
  int rc;
  if (q > 0 && !graph_current(b, b->g_many) && (rc = capture(b, b->g_many, b->spl))) return rc;
  if (r > 0 && !graph_current(b, b->g_one) && (rc = capture(b, b->g_one, 1))) return rc;
  for (int i = 0; i < q; ++i) CK(cudaGraphLaunch(b->g_many.exec, st));
  for (int i = 0; i < r; ++i) CK(cudaGraphLaunch(b->g_one.exec, st));
  return NHQG_OK;
}

int nhqg_batch_size(const nhqg_batch* b) { return b ? (int)b->members.size() : -1; }

}  // extern "C"

// ============================================================== learned closure
extern "C" {

int nhqg_mode_count(const nhqg_ctx* c) { return c ? c->p.d.M : -1; }

int nhqg_closure_set(nhqg_ctx* c, const void* w_bf16, const float* sq, int ncoef, float se,
                     float kmax, float out_scale) {
  if (!c) return NHQG_ERR_BAD_ARG;
  if (!w_bf16) {
    if (c->closure.w) ++c->version;
    c->closure = ClosureModel{};
    return NHQG_OK;
  }
  if (!sq || ncoef < 1 || ncoef > 64 || ncoef > c->p.d.P || !(se > 0.f) || !(kmax > 0.f))
    return NHQG_ERR_BAD_ARG;
  if (!c->Cq && dalloc(c, &c->Cq, (size_t)c->p.d.P * c->p.d.M) != cudaSuccess) return NHQG_ERR_CUDA;
  c->closure.w = w_bf16;
  c->closure.sq = sq;
  c->closure.ncoef = ncoef;
  c->closure.se = se;
  c->closure.kmax = kmax;
  c->closure.s = out_scale;
  ++c->version;
  return NHQG_OK;
}

int nhqg_closure_apply(nhqg_ctx* c, const nhqg_state* s, void* out_q, void* stream) {
  if (!c || !s || !out_q) return NHQG_ERR_BAD_ARG;
  if (!c->closure.w) return NHQG_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  c->launches = 0;
  int rc = gather_state(c, s, st);
  if (rc) return rc;
  CK(launch_closure_apply(c->p, c->t, c->closure, c->q0, c->Cq, st));
  CK(launch_scatter(c->p, c->Cq, (double2*)out_q, c->p.d.P, st));
  c->launches += 2;
  return NHQG_OK;
}

int nhqg_closure_features(nhqg_ctx* c, const nhqg_state* s, const float* sq, int ncoef, float se,
                          float kmax, float* x, float* qcols, void* stream) {
  if (!c || !s || !sq || !x || !qcols || ncoef < 1 || ncoef > 64 || ncoef > c->p.d.P)
    return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  int rc = gather_state(c, s, st);
  if (rc) return rc;
  ClosureModel cm{};
  cm.sq = sq; cm.ncoef = ncoef; cm.se = se; cm.kmax = kmax;
  CK(launch_closure_features(c->p, c->t, cm, c->q0, x, reinterpret_cast<float2*>(qcols), st));
  return NHQG_OK;
}

int nhqg_gather_q(nhqg_ctx* c, const nhqg_state* s, void* out_compact, void* stream) {
  if (!c || !s || !out_compact) return NHQG_ERR_BAD_ARG;
  cudaStream_t st = S(stream);
  int rc = gather_state(c, s, st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out_compact, c->q0, (size_t)c->p.d.P * c->p.d.M * sizeof(double2),
                     cudaMemcpyDeviceToDevice, st));
  return NHQG_OK;
}

}  // extern "C"

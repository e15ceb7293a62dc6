// Internal engine interface: device tables, work buffers, kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "df64.cuh"
#include "fft.cuh"
#include "nhqg_gpu.h"

namespace nhqg {

// bits of the device status word
constexpr int NHQG_STATUS_BIT_OOB = 0;      // input content outside the 2/3 band
constexpr int NHQG_STATUS_BIT_TIMEOUT = 1;  // a bounded device wait ran out

// Tensor-core vertical transforms (csrc/tc_vertical.cu): per transform the
// parity-folded TF32 hi/lo matrix image in shared-memory order, the CUDA-core
// row, the input rows K, the output rows and the number of k-chunks.
enum TcImage {
  TC_FWD_Q = 0,  // V: Chebyshev q -> nodal
  TC_FWD_W = 1,  // V S_w: Galerkin w -> nodal
  TC_FWD_T = 2,  // V S: Galerkin theta -> nodal
  TC_INV = 3,    // V^-1: nodal -> Chebyshev
  TC_E_Q = 4,    // -V^-1: nodal A_q -> E_q (Chebyshev)
  TC_E_G = 5,    // -pinv V^-1: nodal A_w, A_theta -> E_w, E_theta (Galerkin, Dirichlet basis)
  TC_IMAGES = 6
};
struct TcHostImage {
  std::vector<uint8_t> bytes;
  std::vector<float> xrow;
  int K = 0, rows = 0, nch = 0;
};
struct TcTables {
  const uint8_t* img[TC_IMAGES] = {};
  const float* xrow[TC_IMAGES] = {};
  int K[TC_IMAGES] = {}, rows[TC_IMAGES] = {}, nch[TC_IMAGES] = {};
};

// Device-resident tables, uploaded once by nhqg_ctx_create.
struct Tables {
  // per compact mode [M]
  double *kx = nullptr, *ky = nullptr, *inv_denom = nullptr;
  double *inv_aq = nullptr, *inv_at = nullptr, *drq = nullptr, *drw = nullptr, *drt = nullptr;
  double2* eta = nullptr;  // [M] or null
  // full-layout wavenumbers for the plane API
  double *kx_full = nullptr, *ky_full = nullptr;  // [Nx], [Nk]
  double *inv_denom_full = nullptr;               // [Nx*Nk]
  // physical-space fields [Nx*Nx]
  double *sponge = nullptr, *eta_phys = nullptr;
  // FFT over Nx
  double2* tw = nullptr;  // [Nh]
  int* perm = nullptr;    // [Nh]
  // FFT over Nx (the physical-space diagnostics; the same tables as tw/perm
  // unless the 3/2 rule's products run at Npad)
  double2* tw_nx = nullptr;
  int* perm_nx = nullptr;
  // FP32 copies for the mixed-precision path (kx_f [Nx], ky_f [Nk] full layout)
  float *kx_f = nullptr, *ky_f = nullptr, *sponge_f = nullptr, *eta_phys_f = nullptr;
  float2 *eta_f = nullptr, *tw_f = nullptr, *tw_v_f = nullptr, *cs_v_f = nullptr;
  // d eta / dx, d eta / dy on the products' grid (FP32): the mixed path's
  // products take q itself and add u . grad(eta), which keeps FP32 from
  // cancelling a small q against the O(1) trap PV
  float *eta_x_f = nullptr, *eta_y_f = nullptr;
  // FFT over Nz (DCT-I of the vertical columns)
  double2* tw_v = nullptr;  // [Nz]   exp(-2 pi i k / Nz)
  double2* cs_v = nullptr;  // [Nz+1] exp(-i pi j / Nz)
  int* perm_v = nullptr;    // [Nz]
  cdfl *tw_v_df = nullptr, *cs_v_df = nullptr;  // double-float copies (mixed-path corrector)
  // vertical operators
  double *V = nullptr, *Vinv = nullptr;        // [P*P]
  double *wst_a = nullptr, *wst_b = nullptr;   // mixed w stencil a_n, b_n [G]; null = Dirichlet
  int *c2s_ptr = nullptr, *c2s_col = nullptr;
  double* c2s_val = nullptr;
  int *s2c_ptr = nullptr, *s2c_col = nullptr;
  double* s2c_val = nullptr;
  // the same two maps as fixed-width rows (ELL, [q][P], zero-padded, in the
  // CSR order) for the 1-D kernels: every entry's position is known up front
  int ell_w = 0;
  int *c2s_ecol = nullptr, *s2c_ecol = nullptr;
  double *c2s_eval = nullptr, *s2c_eval = nullptr;
  double* bcF = nullptr;    // [2*P] rows N-1, N of (proj_dir - I) V_inv
  double* bcV = nullptr;    // [2*P] columns N-1, N of V
  double* c2sV = nullptr;     // [P*P] cgl_to_sbp V (th_bar coefficients -> SBP grid)
  double* tauVinv = nullptr;  // [P*P] P_tau V^-1 (CGL values -> tau-projected coefficients)
  // fused SBP2 substep: R = c2s s2c (rw nonzeros per row, padded), Fs =
  // s2c^T bcF (2 rows), u = c2s bcV (2 columns)
  int* R_col = nullptr;     // [P*rw]
  double* R_val = nullptr;  // [P*rw]
  int R_w = 0;
  double* Fs = nullptr;     // [2*P]
  double* Us = nullptr;     // [2*P]
  dfl *R_val_df = nullptr, *Fs_df = nullptr, *Us_df = nullptr;  // double-float copies
  double* proj = nullptr;   // [P*P] proj_dirichlet
  double* D1 = nullptr;     // [P*P] SBP first derivative
  double* Lsbp = nullptr;   // [P*P] SBP Laplacian
  double* D1b = nullptr;    // [3*P] D1[i][i-1+d] at d*P + i
  double* Lb = nullptr;     // [5*P] Lsbp[i][i-2+d] at d*P + i
  // Parseval weights of the compact modes for a horizontal mean (re, im
  // parts): 2 for ky > 0, 1 on the ky = 0 column (its Hermitian projection
  // for Hermitian fields), 1/2 at the padded kx Nyquist, (1, 0) at k = 0
  double2* pwt = nullptr;   // [M]
  double* GZ = nullptr;     // [P*P]
  double* GZ2 = nullptr;    // [P*P]
  double* mean_solve = nullptr;  // [P*P] or null
  double* c2s_d = nullptr;  // [P*P] dense (1-D vectors)
  double* s2c_d = nullptr;  // [P*P]
  // Clenshaw-Curtis weights [P] (diagnostics) or null
  double* cc = nullptr;
  // shells
  double* shell_inv = nullptr;  // [n_shells*G*G]
  int* shell_start = nullptr;   // [n_shells+1]
  int* shell_modes = nullptr;   // [M]
  int n_shells = 0;
  int max_shell_modes = 0;
  // O(N) tau solve of the mixed-precision path (null: not available)
  int* mode_shell = nullptr;  // [M] shell of each compact mode (order of shell_inv)
  double *tau_tab = nullptr, *tau_par = nullptr, *tau_uni = nullptr;
  // tensor-core vertical transforms of the mixed-precision path (img null: absent)
  TcTables tc;
};

struct Params {
  Dims d;
  FftPlan plan;
  FftPlan plan_v;  // length Nz (DCT-I); npass <= 0 -> dense vertical transforms
  FftPlan plan_nx; // length Nx (physical-space diagnostics)
  bool fast_dct;
  int advection, closure, exchange, wbc, substeps;
  double dt, gamma_imex, Ra_sigma, sigma, beta, eps_sq;
  bool has_eta, has_sponge;
  // horizontal-product tile budgets in KiB per precision [0] FP64, [1] FP32:
  // column tiles of H1/H3 and the row tile of H2 (0 = built-in default);
  // set by nhqg_autotune
  int h_col_kib[2], h_row_kib[2];
  // mixed-precision vertical transforms on the tensor cores (else FP32 DCT)
  bool tc_vertical;
  // FP32 horizontal products with register-resident FFTs (horizontal_reg.cu)
  // where the transform length allows, else the shared-memory FFT kernels
  bool reg_fft;
  // overlap rows of the corrector's windowed 1-D solve; -1: set from the decay
  // of A^-1 (the default), 0: one global FP32 LU, > 24: windows off
  int corr_win_ov;
  int scheme;  // NHQG_SCHEME_*
};

}  // namespace nhqg
#include "column.cuh"
namespace nhqg {

inline col::Dct make_dct(const Params& p, const Tables& t) {
  col::Dct d;
  d.N = p.d.Nz;
  d.P = p.d.P;
  d.fast = p.fast_dct;
  d.plan = p.plan_v;
  d.tw = t.tw_v;
  d.tw_f = t.tw_v_f;
  d.cs = t.cs_v;
  d.cs_f = t.cs_v_f;
  d.tw_df = t.tw_v_df;
  d.cs_df = t.cs_v_df;
  d.perm = t.perm_v;
  d.V = t.V;
  d.Vinv = t.Vinv;
  return d;
}

// Horizontal product launch description.
enum HForm { HF_FLUX = 0, HF_JAC = 1, HF_SPONGE = 2 };

struct HorizArgs {
  int form;            // HForm
  bool sponge;         // add sigma*f terms (flux/jac forms)
  bool eta;            // q_adv = q + eta (step engine)
  bool full_in;        // inputs are full (Nx, Nk) planes, else compact
  bool full_out;       // outputs are full planes (in-band written), else compact
  bool psi_derived;    // psi = -inv_denom * q (step engine) else read psi
  int levels;
  const double2 *psi, *q, *w, *th;  // planes [level][plane]
  double2 *Aq, *Aw, *Ath;
};

// Optional per-kernel CUDA-event timing (stream-ordered, read after a sync).
struct Profiler {
  bool on = false;
  struct Rec { const char* name; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  size_t next = 0;
  cudaEvent_t get() {
    if (next == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[next++];
  }
  void begin(const char* name, cudaStream_t st) {
    if (!on) return;
    Rec r{name, get(), nullptr};
    cudaEventRecord(r.a, st);
    recs.push_back(r);
  }
  void end(cudaStream_t st) {
    if (!on || recs.empty()) return;
    recs.back().b = get();
    cudaEventRecord(recs.back().b, st);
  }
};

// Horizontal-kernel tables in the compute precision (T = real of C).
template <typename C>
struct HTables {
  using T = decltype(C().x);
  const T *kx_full, *ky_full;  // [Nx], [Nk]
  const double* inv_denom;     // compact [M] (psi derivation)
  const C* eta;                // compact [M] or null
  const T *sponge, *eta_phys;  // [Nx*Nx] or null
  const C* tw;                 // [Nx]
  const int* perm;             // [Nx]
  // gradient form of the trap PV (FP32 products): d eta/dx, d eta/dy or null
  const T *eta_x = nullptr, *eta_y = nullptr;
};

template <typename C, typename CI>
struct HorizArgsT {
  int form;
  bool sponge, eta, full_in, full_out, psi_derived;
  int levels;
  const CI *psi, *q, *w, *th;
  C *Aq, *Aw, *Ath;
};

struct Work {
  Profiler prof;
  // H1 / H2 intermediates
  double2* x1 = nullptr;  size_t x1_elems = 0;
  double2* x2 = nullptr;  size_t x2_elems = 0;
  // compact fields [P*M] each
  std::vector<double2*> f;
  // small vectors
  double* vec = nullptr;       // assorted 1-D vectors (see corrector.cu)
  double* partials = nullptr;    // per-segment reduction sums [P * parseval segments]
  unsigned* counters = nullptr;  // arrival counters of the reductions [P + 1], kept at 0
  // per-CTA level sums of <w theta> from the fused corrector substeps
  // [P * corr_mid_ctas(M)]
  double* mid_part = nullptr;
  int* status = nullptr;       // device status word
};

// ---- launchers (return cudaError_t of the last launch) ----
cudaError_t launch_horizontal(const Params& p, const Tables& t, Work& w, const HorizArgs& a,
                              cudaStream_t st, int* nlaunch);

cudaError_t launch_horizontal_f32(const Params& p, const Tables& t, Work& w,
                                  const HorizArgsT<float2, float2>& a, cudaStream_t st, int* nlaunch);
// register-resident FFT variant (transform lengths 64, 128, 256 of the 2/3
// rule); cudaErrorNotSupported for other lengths
bool horizontal_reg_supported(int N);
cudaError_t launch_horizontal_f32_reg(const Params& p, const Tables& t, Work& w,
                                      const HorizArgsT<float2, float2>& a, cudaStream_t st,
                                      int* nlaunch);

// learned vertical-tail closure for q (csrc/closure.cu)
struct ClosureModel {
  const void* w = nullptr;    // BF16 parameters, nhqg_closure_param_count() values
  const float* sq = nullptr;  // [64] feature scales of |q_n|^2
  int ncoef = 0;              // coefficients the closure acts on (<= 64)
  float se = 1.f, kmax = 1.f, s = 0.f;
};
int closure_param_count();
cudaError_t launch_closure_apply(const Params& p, const Tables& t, const ClosureModel& cm,
                                 const double2* q, double2* cq, cudaStream_t st);
cudaError_t launch_closure_features(const Params& p, const Tables& t, const ClosureModel& cm,
                                    const double2* q, float* x, float2* qc, cudaStream_t st);

// vertical / column engine
enum VBackMode { VB_RHS = 0, VB_STAGE1 = 1, VB_STAGE2 = 2, VB_SOLVE = 3 };
struct VArgs {
  // state the step started from (y_n) and stage-1 state (s1); predictor theta
  const double2 *q0, *w0, *t0;
  const double2 *q1, *w1, *t1, *t1p;
  // explicit operands (nodal A) and stored E1; the mixed-precision path
  // passes A in FP32 (Aqf, Awf, Atf non-null) instead
  const double2 *Aq, *Aw, *At;
  const float2 *Aqf, *Awf, *Atf;
  bool af_coef;  // Aqf/Awf/Atf already hold Chebyshev coefficients (tensor-core inverse)
  double2 *E1q, *E1w, *E1t;
  // learned closure tendency of q (added to E_q) or null
  const double2* Cq;
  // nodal w (legacy exchange product), dtb nodal vector
  const double2* Wn;
  const double* dtb_nodal;  // [P] or null
  // outputs
  double2 *Rq, *Rt, *rhs_w;
  // RHS-only outputs
  double2 *Eq, *Ew, *Et;
  double alpha;       // gamma*dt (stage 1)
  double c_E1, c_E2;  // dt*delta, dt*(1-delta)
  double omega;       // dt*(1-gamma)
  double inv_alpha_c; // 1/alpha for the corrector tendency (0 = none)
  bool df;            // double-float tiles (mixed path with coefficient operands)
};
cudaError_t launch_vfwd(const Params& p, const Tables& t, const double2* q, const double2* w,
                        const double2* th, double2* qn, double2* wn, double2* tn, cudaStream_t st);
cudaError_t launch_vfwd_f32(const Params& p, const Tables& t, const double2* q, const double2* w,
                            const double2* th, float2* qn, float2* wn, float2* tn, cudaStream_t st);
cudaError_t launch_vback(const Params& p, const Tables& t, int mode, const VArgs& a, cudaStream_t st);
// stage combination out = base + dt * sum_k c_k x_k over count elements
constexpr int kLinCombMax = 8;
template <typename T>
struct LinCombT {
  const T* base;
  T* out;
  const T* x[kLinCombMax];
  double c[kLinCombMax];
  int n;
  double dt;
  size_t count;
};
template <typename T>
cudaError_t launch_lincomb(const LinCombT<T>& a, cudaStream_t st);
// K -= rate[m] * Y over levels x M compact elements
cudaError_t launch_sub_diss(const Params& p, double2* K, const double2* Y, const double* rate,
                            int levels, cudaStream_t st);
// tensor-core vertical transforms (csrc/tc_vertical.cu).  Host images: false
// when Nz is odd or above 256, or a matrix lacks the mirror parity.
bool tc_vertical_images(const nhqg_grid_desc* g, TcHostImage img[TC_IMAGES]);
// FP64 Chebyshev (q) / Galerkin (w, theta) coefficients -> FP32 nodal values
cudaError_t launch_tc_to_nodal(const Params& p, const Tables& t, const Work& w, const double2* q,
                               const double2* wf, const double2* th, float2* qn, float2* wn,
                               float2* tn, cudaStream_t st);
// FP32 nodal values -> FP32 Chebyshev coefficients, in place (TC_INV), or
// with explicit = true the explicit tendencies E_q (Chebyshev, P rows) and
// E_w, E_theta (Galerkin, G rows) of nodal A_q, A_w, A_theta (TC_E_Q, TC_E_G)
cudaError_t launch_tc_to_coef(const Params& p, const Tables& t, const Work& w, float2* aq,
                              float2* aw, float2* at, bool explicit_form, cudaStream_t st);
// O(N) tau solve of the per-shell w system (the mixed-precision path's
// replacement for the dense shell inverses)
cudaError_t launch_tau_solve(const Params& p, const Tables& t, const double2* rhs_w, double2* w_out,
                             double2* scratch, cudaStream_t st);  // scratch: P*M
// host factorisation of the per-shell tau systems; coef = [n_shells][2] (a, s)
void build_tau_tables(int Nz, bool open_top, int n_shells, const double* coef,
                      std::vector<double>& tab, std::vector<double>& par, std::vector<double>& uni);
cudaError_t launch_shell(const Params& p, const Tables& t, const double2* rhs_w, double2* w_out,
                         cudaStream_t st);
cudaError_t launch_vpost(const Params& p, const Tables& t, const double2* Rq, const double2* Rt,
                         const double2* w_new, double2* q_out, double2* t_out, bool zero_mean,
                         cudaStream_t st, bool df = false);
size_t corrector_vec_doubles(int P);
cudaError_t launch_itend(const Params& p, const Tables& t, const double2* q, const double2* w,
                         const double2* th, double2* Iq, double2* Iw, double2* It, cudaStream_t st);
cudaError_t launch_gather(const Params& p, const double2* full, double2* compact, int levels,
                          int* status, cudaStream_t st);
cudaError_t launch_scatter(const Params& p, const double2* compact, double2* full, int levels,
                           cudaStream_t st);
cudaError_t launch_finalize(const Params& p, const double2* q, const double2* w, const double2* th,
                            double2* qo, double2* wo, double2* to, cudaStream_t st);
cudaError_t launch_parseval(const Params& p, const double2* a, const double2* b, int levels,
                            double* out, Work& w, cudaStream_t st, bool df = false);
cudaError_t launch_parseval(const Params& p, const float2* a, const double2* b, int levels,
                            double* out, Work& w, cudaStream_t st, bool df = false);
size_t parseval_partials(int levels);
// CTAs of the fused corrector substep (one level sum each per level)
int corr_mid_ctas(int M);
// <a b> and <a c> per level in one pass over a
cudaError_t launch_parseval2(const Params& p, const double2* a, const double2* b, const double2* c,
                             int levels, double* out_ab, double* out_ac, Work& w, cudaStream_t st,
                             bool df = false);
cudaError_t launch_parseval2(const Params& p, const float2* a, const float2* b, const double2* c,
                             int levels, double* out_ab, double* out_ac, Work& w, cudaStream_t st,
                             bool df = false);
cudaError_t launch_hermitian(const Params& p, double2* q, double2* w, double2* th, cudaStream_t st);
cudaError_t launch_zero_mode0(const Params& p, double2* f, int levels, cudaStream_t st);

// 1-D mean-temperature kernels (single CTA)
struct MeanArgs {
  const double *tb0, *E1tb, *E2tb, *tb1, *tb1p;
  double* out;
  double alpha, c_E1, c_E2, omega, inv_alpha_c;
  int stage;     // 1 or 2
  int closure;   // solve flavour
  int itend;     // add omega * I(tb1) (stage 2)
};
cudaError_t launch_mean_stage(const Params& p, const Tables& t, const MeanArgs& a, cudaStream_t st);
cudaError_t launch_mean_legacy_rhs(const Params& p, const Tables& t, const double* tb,
                                   const double* flux_nodal, double* dtb_nodal, double* E_tb,
                                   double* I_tb, cudaStream_t st);

// SBP2 corrector
struct CorrArgs {
  const double2 *wp, *tp;  // predictor w, theta (Galerkin)
  const double* tbp;       // predictor th_bar
  double2* t_out;          // corrected theta
  double* tb_out;          // corrected th_bar
  double2 *wcgl, *wsbp, *tsbp, *tcgl;  // work; tcgl may be null
  double total_dt;
  bool df;  // double-float column tiles (the mixed-precision path)
  // double-float path: w stays FP32 (it enters the corrector only through the
  // sub_dt-scaled exchange increment, the means and the FP32 products); the
  // SBP-grid w lives in the wsbp buffer as float2, the nodal w goes to
  // wcgl_f (the FP32 products' input) or nowhere (null)
  float2* wcgl_f = nullptr;
  float2* tcgl_f = nullptr;  // double-float path: nodal theta rounded to FP32 (or null)
};
cudaError_t run_corrector(const Params& p, const Tables& t, Work& w, const CorrArgs& a,
                          cudaStream_t st, int* nlaunch);
// w and theta (Galerkin) to nodal CGL (w only) and to the SBP grid
cudaError_t launch_corr_pre(const Params& p, const Tables& t, const double2* w, const double2* th,
                            double2* wcgl, double2* wsbp, double2* tsbp, cudaStream_t st);

// diagnostics: per-block partial sums over modes of the depth integrals
// (kDiagTerms doubles per block), then one CTA for the scalars
constexpr int kDiagTerms = 7;
constexpr int kDiagMaxima = 4;  // max |u|, |w|, |theta|, |w theta| over the CGL nodes
int diag_blocks(const Params& p);
cudaError_t launch_diag_modes(const Params& p, const Tables& t, const double2* qn, const double2* wn,
                              const double2* tn, double* partials, cudaStream_t st);
cudaError_t launch_diag_final(const Params& p, const Tables& t, const double* partials,
                              const double* flux, bool flux_on_sbp, const double* th_bar,
                              const unsigned long long* maxima, double* out, cudaStream_t st);
// physical-space maxima over the Nx grid at every CGL level of the FP64
// nodal compact fields (q, w, theta): max sqrt(u^2+v^2), |w|, |theta|,
// |w theta| as bit patterns of non-negative doubles in maxima[0..3]
cudaError_t launch_phys_maxima(const Params& p, const Tables& t, Work& w, const double2* qn,
                               const double2* wn, const double2* tn, unsigned long long* maxima,
                               cudaStream_t st);
// shell energy spectrum (3 n_bins), vertical spectra (P, G, G, P), then the
// shell spectra of q, w, theta (3 n_bins) into out; qn, wn, tn: FP64 nodal
// fields; per_mode: 5 M doubles of scratch
cudaError_t launch_spectra(const Params& p, const Tables& t, const double2* qn, const double2* wn,
                           const double2* tn, const double2* q, const double2* w, const double2* th,
                           const int* mode_bin, int n_bins, double* per_mode, double* out,
                           cudaStream_t st);

}  // namespace nhqg

/*
 * nhqg_gpu.h -- C ABI of the GB300 (sm_103a) NHQG time-step engine.
 *
 * The engine advances the nonhydrostatic quasi-geostrophic state of
 * ksr-ocean/NHQG with the ARS(2,2,2) IMEX step: 2/3-rule dealiased
 * horizontal products (flux or Jacobian form), Chebyshev / Dirichlet-Galerkin
 * vertical transforms, per-|k|^2-shell implicit solves with buoyancy
 * elimination, and the balanced SBP2 mean-temperature corrector.
 *
 * Conventions
 *   - Spectral fields are complex128 stored as interleaved (re, im) doubles in
 *     the reference layout (levels, Nx, Nx/2+1), ky contiguous, kx in fftfreq
 *     order; q_hat has Nz+1 levels (Chebyshev), w_hat / th_hat have Nz-1
 *     (Galerkin), th_bar is Nz+1 doubles.  Pointers passed to the compute
 *     entry points are DEVICE pointers; the caller owns them.
 *   - Every call is ordered on the given CUDA stream (passed as void*, NULL =
 *     legacy default stream) and never synchronises the host.
 *   - Every entry point returns an nhqg_status; device-side conditions (a
 *     state that is not band-limited, a bounded wait that ran out) are latched
 *     in the context and read with nhqg_get_device_status after the stream
 *     has been synchronised.
 *   - A context is used by one host thread at a time; separate contexts may
 *     run concurrently on separate streams.
 */
#ifndef NHQG_GPU_H
#define NHQG_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nhqg_status {
  NHQG_OK = 0,
  NHQG_ERR_BAD_ARG = 1,          /* null pointer, inconsistent sizes */
  NHQG_ERR_UNSUPPORTED = 2,      /* configuration outside the GPU path */
  NHQG_ERR_CUDA = 3,             /* a CUDA runtime call failed */
  NHQG_ERR_DEVICE_TIMEOUT = 4,   /* a bounded device wait ran out */
  NHQG_ERR_NOT_BAND_LIMITED = 5, /* input had content outside the 2/3 band */
  NHQG_ERR_SCRATCH_TOO_SMALL = 6 /* one level does not fit the static scratch */
} nhqg_status;

enum { NHQG_ADV_FLUX = 0, NHQG_ADV_JACOBIAN = 1 };
enum { NHQG_CLOSURE_FIXED_CONDUCTION = 0, NHQG_CLOSURE_EVOLVE_MEAN = 1 };
enum { NHQG_EXCHANGE_LEGACY = 0, NHQG_EXCHANGE_BALANCED_SBP2 = 1,
       NHQG_EXCHANGE_BALANCED_SBP2_PC = 2 };
enum { NHQG_WBC_DIRICHLET = 0, NHQG_WBC_NEUMANN = 1 };
enum { NHQG_PRECISION_FP64 = 0, NHQG_PRECISION_MIXED = 1 };
/* imex_scheme (nhqg/config.py:45).  As in the reference's dispatch
 * (nhqg/solver.py:1228-1242) the scheme selects the stepper only with the
 * legacy exchange; the balanced SBP2 exchanges run their own stage-wise
 * stepper with the grid's gamma.  RK443 runs in FP64 (NHQG_PRECISION_MIXED
 * steps return NHQG_ERR_UNSUPPORTED). */
enum { NHQG_SCHEME_ARS222 = 0, NHQG_SCHEME_RK443 = 1 };
/* horizontal_dealiasing (nhqg/config.py:62).  NHQG_DEALIAS_23 ("23_rule"):
 * products on the Nx grid masked to |kx|, ky <= Nx/3, states band-limited to
 * that rectangle.  NHQG_DEALIAS_32 ("32_rule", the reference's default):
 * products on the zero-padded 3Nx/2 grid and truncated back
 * (nhqg/spectral.py:18-50, 147-253); states are full band and the horizontal
 * means <a b> are those of the padded fields (nhqg/solver.py:204-245).
 * 3Nx/2 must factor as 2^a 3^b. */
enum { NHQG_DEALIAS_23 = 0, NHQG_DEALIAS_32 = 1 };

/*
 * Host-side description of a Grid (nhqg/grid.py:29-141 Grid fields, built by
 * make_grid, nhqg/grid.py:439-789).  All arrays are HOST float64 row-major in
 * the reference's shapes; they are copied to the device by nhqg_ctx_create
 * and may be freed afterwards.  P = Nz+1, G = Nz-1, Nk = Nx/2+1.
 */
typedef struct nhqg_grid_desc {
  int Nx, Nz;
  int advection;          /* NHQG_ADV_* (nonlinear_advection) */
  int thermal_closure;    /* NHQG_CLOSURE_* */
  int exchange;           /* NHQG_EXCHANGE_* (mean_exchange_discretization) */
  int w_bc_top;           /* NHQG_WBC_* */
  int substeps;           /* sbp_corrector_substeps */
  int n_shells;           /* number of matrices in shell_inv */
  double dt, gamma_imex, Ra_sigma, sigma, beta, eps_sq;
  const double *kx, *ky;                       /* (Nx,), (Nk,) */
  const double *inv_denom;                     /* (Nx,Nk) */
  const double *diss_rate_q, *diss_rate_w, *diss_rate_th;  /* (Nx,Nk) */
  const double *inv_alpha_q, *inv_alpha_th;    /* (Nx,Nk) */
  const int *shell_of_mode;                    /* (Nx,Nk) row of shell_inv, or -1 */
  const double *shell_inv;                     /* (n_shells,G,G) imex_inv rows */
  const double *eta_hat;                       /* (Nx,Nk) complex or NULL */
  const double *eta_phys;                      /* (Nh,Nh) physical eta, or NULL:
                                                  irfft2(eta_hat) on the Nx grid
                                                  (2/3 rule); irfft2 of the
                                                  zero-padded eta_hat on the
                                                  Npad grid, no rescale (3/2
                                                  rule) */
  const double *sponge_phys;                   /* (Nh,Nh) or NULL: the Grid's
                                                  sponge_phys (2/3 rule) or
                                                  sponge_phys_pad (3/2 rule,
                                                  nhqg/grid.py:663-667) */
  const double *V, *V_inv;                     /* (P,P) */
  const double *w_stencil;                     /* (P,G) */
  const double *G_Z;                           /* (P,P) */
  const double *proj_dirichlet;                /* (P,P) */
  const double *sbp_D1, *sbp_L;                /* (P,P) */
  const double *cgl_to_sbp, *sbp_to_cgl;       /* (P,P) */
  const double *mean_solve;                    /* (P,P) inverse of the tau'd
                                                  1-D mean operator (legacy
                                                  evolve_mean), else NULL */
  const double *shell_coef;                    /* (n_shells,2) per shell_inv row:
                                                  alpha_w_eff and
                                                  (gamma dt)^2 c_k / alpha_q at the
                                                  shell's rounded |k|^2
                                                  (nhqg/grid.py:398-430); NULL
                                                  disables NHQG_PRECISION_MIXED */
  const double *cc_weights;                    /* (P,) Clenshaw-Curtis weights on
                                                  [0,1]; NULL disables
                                                  nhqg_diagnostics */
  int imex_scheme;                             /* NHQG_SCHEME_*; gamma_imex and the
                                                  shell tables must be the
                                                  scheme's (1 - 1/sqrt 2 for
                                                  ARS222, 1/2 for RK443) */
  int horizontal_dealiasing;                   /* NHQG_DEALIAS_*; Nh = Nx for the
                                                  2/3 rule, Npad = 3Nx/2 for the
                                                  3/2 rule */
  const double *eta_x_phys, *eta_y_phys;       /* (Nh,Nh) d eta/dx, d eta/dy on
                                                  the grid of eta_phys, or NULL.
                                                  The mixed path carries the trap
                                                  PV as u . grad(eta) beside the
                                                  products of q itself (no FP32
                                                  cancellation of q against
                                                  eta); NULL with eta_hat set
                                                  disables NHQG_PRECISION_MIXED */
} nhqg_grid_desc;

typedef struct nhqg_ctx nhqg_ctx;

/* Device-resident state in the reference layout (nhqg/solver.py:33-38). */
typedef struct nhqg_state {
  void *q_hat;     /* (Nz+1, Nx, Nk) complex128 */
  void *w_hat;     /* (Nz-1, Nx, Nk) complex128 */
  void *th_hat;    /* (Nz-1, Nx, Nk) complex128 */
  double *th_bar;  /* (Nz+1,) float64 */
} nhqg_state;

/* Create a context: validates the configuration, uploads the tables.
 * Replaces the jit closure over the Grid in the reference drivers
 * (scripts/benchmark.py:39-45: jax.jit(lambda s: imex_step(s, grid))). */
int nhqg_ctx_create(const nhqg_grid_desc *desc, nhqg_ctx **out);
int nhqg_ctx_destroy(nhqg_ctx *ctx);

/* n_steps applications of imex_step (nhqg/solver.py:1228-1242, including
 * sanitize_state), in place.  Under the 2/3 rule the input must be
 * band-limited (every state that sanitize_state, make_initial_state, run or
 * imex_step produced is); under the 3/2 rule every mode is stored. */
int nhqg_step(nhqg_ctx *ctx, nhqg_state *state, int n_steps, void *stream);

/* Arithmetic of the following nhqg_step / nhqg_explicit_rhs /
 * nhqg_implicit_solve calls.  It has no counterpart in the reference, whose
 * only precision switch is float_dtype (nhqg/config.py:59), which changes
 * every array.
 *   NHQG_PRECISION_FP64 (default): the plain path, all FP64, the reference's
 *     dense per-shell inverses.
 *   NHQG_PRECISION_MIXED: the horizontal products and the Chebyshev <-> nodal
 *     transforms that feed them and read them back run in FP32 (TF32 split
 *     products on the tensor cores for the transforms); the Galerkin
 *     stencils, stage combinations and the SBP2 corrector's column transforms
 *     run in double-float (an FP32 pair, about 48 significant bits, on the
 *     FP32 pipe; fields stay FP64 in memory); the 1-D mean-temperature solves
 *     and the implicit w solve stay FP64, the latter as an O(Nz)
 *     Chebyshev-tau solve per mode instead of the dense shell inverse.  Not
 *     supported
 *     (NHQG_ERR_UNSUPPORTED): legacy evolve_mean (its nodal exchange
 *     product), Nz whose 2*Nz is not 2^a 3^b, and a descriptor
 *     without shell_coef.
 * The first switch to MIXED allocates 6 FP32 fields of (Nz+1) x (stored
 * modes) each. */
int nhqg_set_precision(nhqg_ctx *ctx, int precision);

/* Engine of the mixed path's Chebyshev <-> nodal transforms (the FP32 part of
 * _to_nodal / _to_coeffs, nhqg/solver.py:45-52).  tensor_cores = 1: dense
 * parity-folded products on the tcgen05 tensor cores, TF32 hi/lo split
 * operands with FP32 accumulation (the default where available); 0: FP32
 * fast DCT-I on the CUDA cores.  NHQG_ERR_UNSUPPORTED for 1 when Nz is odd or
 * above 256, the w basis is the open-top one, or the descriptor has no
 * shell_coef.  The environment variable NHQG_TC_VERTICAL=0 makes 0 the
 * context's default. */
int nhqg_set_mixed_vertical(nhqg_ctx *ctx, int tensor_cores);
/* 1 if the mixed path's vertical transforms run on the tensor cores. */
int nhqg_get_mixed_vertical(const nhqg_ctx *ctx);
/* The tensor-core transforms alone, on M = nhqg_mode_count() columns.
 * nhqg_tc_to_nodal: field 0 (q, Chebyshev coefficients, (Nz+1) x M), 1 (w) or
 * 2 (theta) (Galerkin coefficients, (Nz-1) x M), complex128, to the
 * (Nz+1) x M complex64 nodal values of _to_nodal(_dirichlet_to_cheb(.)).
 * nhqg_tc_to_coef: (Nz+1) x M complex64 nodal values to Chebyshev
 * coefficients (_to_coeffs), in place.  NHQG_ERR_UNSUPPORTED where
 * nhqg_set_mixed_vertical(ctx, 1) is. */
int nhqg_tc_to_nodal(nhqg_ctx *ctx, int field, const void *coef, void *nodal, void *stream);
int nhqg_tc_to_coef(nhqg_ctx *ctx, void *nodal_inout, void *stream);

/* explicit_rhs (nhqg/solver.py:510-599) at `in`, written to `out`.
 * closure/exchange select the Grid flavour the reference call would see
 * (the split steppers evaluate it on the fixed_conduction/legacy base grid,
 * nhqg/solver.py:1172-1175). */
int nhqg_explicit_rhs(nhqg_ctx *ctx, const nhqg_state *in, nhqg_state *out,
                      int thermal_closure, int exchange, void *stream);

/* implicit_tendency (nhqg/solver.py:615-641). */
int nhqg_implicit_tendency(nhqg_ctx *ctx, const nhqg_state *in, nhqg_state *out,
                           int thermal_closure, void *stream);

/* imex_implicit_solve (nhqg/solver.py:691-738) of (R.q_hat, R.w_hat,
 * R.th_hat) and imex_mean_temp_solve (nhqg/solver.py:741-758) of R.th_bar. */
int nhqg_implicit_solve(nhqg_ctx *ctx, const nhqg_state *rhs, nhqg_state *out,
                        int thermal_closure, void *stream);

/* _apply_balanced_sbp2_corrector (nhqg/solver.py:909-950) with total_dt. */
int nhqg_sbp2_corrector(nhqg_ctx *ctx, const nhqg_state *in, nhqg_state *out,
                        double total_dt, void *stream);

/* triple_conservative_flux_divergence_23 / triple_jacobian_23
 * (nhqg/spectral.py:331-358) on `levels` planes (Nx, Nk) complex128 each:
 * inputs psi, q, w, th; outputs Aq, Aw, Ath (masked). advection = NHQG_ADV_*.
 * The outputs are written while inputs are still being read: no output may
 * overlap an input. */
int nhqg_triple_advection_23(nhqg_ctx *ctx, int advection, int levels,
                             const void *psi, const void *q, const void *w,
                             const void *th, void *Aq, void *Aw, void *Ath,
                             void *stream);

/* Allocation-free variant of nhqg_triple_advection_23.  It has no
 * counterpart in the reference.  It is for callers that must not allocate
 * device memory themselves: XLA FFI handlers (all buffers come from XLA's
 * allocator) and hosts that run on a fixed device-memory pool.  No context is
 * needed and nothing is allocated: the FFT tables and the H1/H2
 * intermediates live in one static __device__ array of
 * NHQG_NOALLOC_SCRATCH_BYTES per GPU, held from library load until process
 * exit.  kx (Nx doubles) and ky (Nx/2+1 doubles) are device pointers with the
 * reference's wavenumbers; planes as in nhqg_triple_advection_23, and no
 * output may overlap an input (NHQG_ERR_BAD_ARG).  Levels are processed in
 * chunks that fit the array.  One level must fit: with the 32 MiB array that
 * holds up to Nx = 648 (flux) and Nx = 576 (Jacobian); a larger Nx returns
 * NHQG_ERR_SCRATCH_TOO_SMALL, and Nx above 2048 NHQG_ERR_UNSUPPORTED.
 * The first call on each device sets up the array's address with that device
 * current (make it before any stream capture); a device reset makes that
 * address stale, so do not call this again in a process that reset the
 * device.  All calls share the array, so calls that overlap on the GPU race
 * on it. */
#define NHQG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int nhqg_triple_advection_23_noalloc(int advection, int Nx, int levels,
                                     const double *kx, const double *ky,
                                     const void *psi, const void *q, const void *w,
                                     const void *th, void *Aq, void *Aw, void *Ath,
                                     void *stream);

/* sponge_product_23 (nhqg/spectral.py:53-60) with the context's sponge. */
int nhqg_sponge_product_23(nhqg_ctx *ctx, int levels, const void *f, void *out,
                           void *stream);

/* 3/2-rule planes, on a context built with NHQG_DEALIAS_32 (a 2/3-rule
 * context returns NHQG_ERR_UNSUPPORTED, and the _23 calls refuse a 3/2-rule
 * context): triple_jacobian / triple_conservative_flux_divergence
 * (nhqg/spectral.py:147-253) on `levels` planes (Nx, Nk) complex128 each,
 * zero-padded to the context's Npad = 3Nx/2 grid and truncated back; and
 * sponge_product_32 (nhqg/spectral.py:63-75) with the context's padded
 * sponge. */
int nhqg_triple_advection_32(nhqg_ctx *ctx, int advection, int levels,
                             const void *psi, const void *q, const void *w,
                             const void *th, void *Aq, void *Aw, void *Ath,
                             void *stream);
int nhqg_sponge_product_32(nhqg_ctx *ctx, int levels, const void *f, void *out,
                           void *stream);

/* sanitize_state (nhqg/solver.py:128-146), in place: Hermitian projection
 * of the ky=0 column and the 2/3 band limit (2/3 rule), or of the ky=0 and
 * ky=Nx/2 columns (3/2 rule, no band limit). */
int nhqg_sanitize(nhqg_ctx *ctx, nhqg_state *state, void *stream);

/* imex_mean_temp_solve (nhqg/solver.py:741-758) of R_th_bar (Nz+1 doubles,
 * device) into out. */
int nhqg_mean_temp_solve(nhqg_ctx *ctx, const double *R_th_bar, double *out,
                         int thermal_closure, void *stream);

/* Scalar diagnostics of a state: the depth-integrated energies, rms values
 * and Nusselt numbers of compute_diagnostics (nhqg/diagnostics.py:597-690),
 * the physical-space maxima over the Nx grid at every CGL node
 * (max_speed = max sqrt(u^2 + v^2), max_w, max_theta, max_tw = max |w theta|;
 * nhqg/diagnostics.py:631-641) and the heat-flux mismatch
 * vol_avg_tw_dealiased - vol_avg_tw (its budgets are not computed).  out:
 * NHQG_DIAG_COUNT doubles in DEVICE memory, written stream-ordered in the
 * NHQG_DIAG_* order.  The dealiased heat flux follows the mean equation's
 * path (SBP grid for the balanced SBP2 exchange).  Needs cc_weights in the
 * descriptor. */
enum {
  NHQG_DIAG_KE_BT = 0, NHQG_DIAG_KE_BC, NHQG_DIAG_KE_TOT, NHQG_DIAG_ENSTROPHY,
  NHQG_DIAG_NUSSELT, NHQG_DIAG_NUSSELT_DEALIASED, NHQG_DIAG_VOL_AVG_TW,
  NHQG_DIAG_VOL_AVG_TW_DEALIASED, NHQG_DIAG_Q_RMS, NHQG_DIAG_W_RMS, NHQG_DIAG_TH_RMS,
  NHQG_DIAG_TH_BAR_MAX, NHQG_DIAG_MAX_SPEED, NHQG_DIAG_MAX_W, NHQG_DIAG_MAX_THETA,
  NHQG_DIAG_MAX_TW, NHQG_DIAG_HEAT_FLUX_MISMATCH, NHQG_DIAG_COUNT
};
int nhqg_diagnostics(nhqg_ctx *ctx, const nhqg_state *state, double *out, void *stream);

/* Spectra of a state, unnormalised like the reference's:
 *   out[0 : 3 n_bins]   energy_spectrum (nhqg/diagnostics.py:80-101) of psi:
 *                       E_bt, E_bc, E_tot per horizontal shell;
 *   then (Nz+1) + (Nz-1) + (Nz-1) values: vertical_mode_energy (:583-585)
 *                       of q_hat, w_hat, th_hat per Chebyshev index;
 *   then (Nz+1) values: the psi kinetic energy per Chebyshev index,
 *                       sum_k w_k |k|^2 |psi_n(k)|^2 (w_k the rfft weights);
 *   then 3 n_bins:      the horizontal shell spectra of q, w, theta at the
 *                       CGL nodes (compute_diagnostics, nhqg/diagnostics.py:
 *                       104-111, 667-669): per shell sum w_k sum_j cc_j |f_j|^2.
 * mode_bin: DEVICE int array of nhqg_mode_count() entries, the shell of each
 * compact mode (row r = kx index 0..2K with K = Nx/3, rows above K holding
 * kx = r - (2K+1); column c = ky index 0..K; m = r (K+1) + c) under the
 * reference's test i dk <= |k| < (i+1) dk, or -1.  out in DEVICE memory,
 * written stream-ordered.  Needs cc_weights in the descriptor. */
int nhqg_spectra(nhqg_ctx *ctx, const nhqg_state *state, const int *mode_bin, int n_bins,
                 double *out, void *stream);

/* Latched device-side status of the last calls (after a stream sync);
 * reset = 1 clears it. */
int nhqg_get_device_status(nhqg_ctx *ctx, int reset);

/* Number of kernel launches the last compute call issued (bench accounting). */
int nhqg_last_launch_count(const nhqg_ctx *ctx);

/* Per-kernel CUDA-event timing of subsequent calls (stream-ordered).
 * nhqg_profile_report synchronises the device and writes one line per kernel
 * class, "name launches total_ms", into buf, then clears the record. */
int nhqg_profile_enable(nhqg_ctx *ctx, int on);
int nhqg_profile_report(nhqg_ctx *ctx, char *buf, int buflen);

/* ---- Tiles and autotuning (no reference counterpart) ----
 * The horizontal-product kernels size their tiles from shared-memory budgets:
 * tiles[0], tiles[1] = FP64 column / row budget in KiB, tiles[2], tiles[3] =
 * the FP32 ones; 0 selects the built-in default.  nhqg_autotune times
 * candidate budgets on the context's own buffers (both precisions once the
 * mixed path is enabled) and keeps the fastest; it synchronises the stream. */
int nhqg_get_tiles(const nhqg_ctx *ctx, int *tiles);
int nhqg_set_tiles(nhqg_ctx *ctx, const int *tiles);
int nhqg_autotune(nhqg_ctx *ctx, void *stream);

/* ---- Batched ensemble (no reference counterpart) ----
 * Independent contexts (any sizes, parameters and precisions) stepped
 * together.  The steps of all members are captured once into a CUDA graph,
 * each member on its own stream forked from and joined into the graph's
 * origin, and one graph launch advances every member by steps_per_launch
 * steps (a second, single-step graph takes the remainder).  A member keeps
 * its state inside its context between calls: nhqg_batch_load copies a state
 * in (the band check of nhqg_step applies), nhqg_batch_store copies it out.
 * Changing a member's precision or tiles recaptures the graphs at the next
 * nhqg_batch_step.  The contexts must outlive the batch and must not be
 * stepped through other entry points while the batch is in use. */
typedef struct nhqg_batch nhqg_batch;
int nhqg_batch_create(nhqg_ctx *const *members, int n, int steps_per_launch, nhqg_batch **out);
int nhqg_batch_destroy(nhqg_batch *batch);
int nhqg_batch_load(nhqg_batch *batch, int member, const nhqg_state *state, void *stream);
int nhqg_batch_store(nhqg_batch *batch, int member, nhqg_state *state, void *stream);
int nhqg_batch_step(nhqg_batch *batch, int n_steps, void *stream);
int nhqg_batch_size(const nhqg_batch *batch);

/* ---- Learned vertical-tail closure for q (no reference counterpart) ----
 * An opt-in extra q tendency C_n = -s (r_n + i rho_n) q_n on the first ncoef
 * (<= 64) Chebyshev coefficients of every horizontal mode, with (r, rho) =
 * MLP(features of the column): features log1p(|q_n|^2 / sq_n) (n < 64),
 * |k| / kmax and log1p(sum_n |k|^2 |psi_n|^2 / se).  MLP 66 -> 256 -> 128 ->
 * 128 (r_n at n, rho_n at 64 + n), tanh hidden units,
 * nhqg_closure_param_count() BF16 parameters (layer-major: W1 [256][66], b1,
 * W2 [128][256], b2, W3 [128][128], b3), FP32 accumulation.
 * nhqg_closure_set attaches DEVICE pointers owned by the caller (weights and
 * sq [64]) to a context: every later explicit RHS and step adds C to E_q;
 * w_bf16 = NULL detaches.  nhqg_closure_apply writes C for a state as a
 * (Nz+1, Nx, Nk) complex128 plane set.  nhqg_closure_features writes the
 * features (x [M][66] FP32) and columns (q [M][64] complex FP32) of a state's
 * M = nhqg_mode_count() in-band modes.  nhqg_closure_train_step runs one
 * forward/backward pass over a batch (x [B][66], q and target [B][64] complex
 * FP32), writes the mean loss sum_n |C_n - t_n|^2 / target_norm and the FP32
 * gradient, and (lr > 0) one Adam step on the FP32 master weights that also
 * refreshes the BF16 copy (step counts from 1).  nhqg_gather_q copies a
 * state's q to the compact (Nz+1) x M layout of the context. */
int nhqg_mode_count(const nhqg_ctx *ctx);
int nhqg_closure_param_count(void);
int nhqg_closure_set(nhqg_ctx *ctx, const void *w_bf16, const float *sq, int ncoef, float se,
                     float kmax, float out_scale);
int nhqg_closure_apply(nhqg_ctx *ctx, const nhqg_state *state, void *out_q, void *stream);
int nhqg_closure_features(nhqg_ctx *ctx, const nhqg_state *state, const float *sq, int ncoef,
                          float se, float kmax, float *x, float *qcols, void *stream);
int nhqg_closure_train_step(const void *w_bf16, float *w_master, float *adam_m, float *adam_v,
                            float *grad, float *loss, int batch, const float *x, const float *q,
                            const float *target, float out_scale, float target_norm, float lr,
                            int step, void *stream);
int nhqg_gather_q(nhqg_ctx *ctx, const nhqg_state *state, void *out_compact, void *stream);

/* Engine build identification string (static storage). */
const char *nhqg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* NHQG_GPU_H */

// Column engine: everything that acts on one horizontal mode's vertical
// column (FP64).  Each CTA owns TM consecutive compact modes and stages their
// columns (all levels) in shared memory as tiles [level][TM].
//
// Reference operations (nhqg/solver.py):
//   Chebyshev <-> CGL nodal transforms V, V^-1           :45-52
//   Galerkin stencil S and its exact left inverse pinv   :65-72 (grid.py:497-506, 322-342)
//   d/dZ on Chebyshev coefficients G_Z                    grid.py:148-169
//   explicit-RHS assembly                                 :541-549
//   implicit tendency                                     :615-641
//   implicit solve (block elimination)                    :691-738
//   stage combinations of ARS(2,2,2) / SBP2-PC            :1023-1048, :1205-1217
//   finalize + sanitize                                   :993-999, :128-146
// pinv_w(proj_w(x)) == pinv_w(x) because pinv reads only the first Nz-1
// Chebyshev coefficients and the tau projection rewrites only the last two,
// so the tau projections that feed a pinv are not applied.
#include <algorithm>
#include <type_traits>

#include "column.cuh"
#include "engine.h"

namespace nhqg {

namespace {

using col::TM;
using col::NT;
using col::tload;
using col::tstore;
using col::tcvt;
using col::tmat;
using col::tstencil_dir;
using col::tpinv_dir;
using col::tgz;
using col::tdct;

struct VK {
  int P, G, N, M, Mr, Mc, K, Nx, Nk;
  bool mixed;                 // open-top (Neumann) w basis
  const double *wa, *wb;      // mixed stencil coefficients
  col::Dct dct;
  const double *kx, *inv_denom, *inv_aq, *inv_at, *drq, *drw, *drt;
  double beta, Ra, gdt;
};

VK make_vk(const Params& p, const Tables& t) {
  VK k;
  k.P = p.d.P; k.G = p.d.G; k.N = p.d.Nz; k.M = p.d.M; k.Mr = p.d.Mr; k.Mc = p.d.Mc;
  k.K = p.d.K; k.Nx = p.d.Nx; k.Nk = p.d.Nk;
  k.mixed = t.wst_a != nullptr;
  k.wa = t.wst_a; k.wb = t.wst_b;
  k.dct = make_dct(p, t);
  k.kx = t.kx; k.inv_denom = t.inv_denom; k.inv_aq = t.inv_aq; k.inv_at = t.inv_at;
  k.drq = t.drq; k.drw = t.drw; k.drt = t.drt;
  k.beta = p.beta; k.Ra = p.Ra_sigma; k.gdt = p.gamma_imex * p.dt;
  return k;
}

template <typename C>
__device__ __forceinline__ void tstencil_w(const VK& k, C* c, const C* x) {
  if (!k.mixed) tstencil_dir(c, x, k.P, k.G);
  else col::tstencil_mixed(c, x, k.P, k.G, k.wa, k.wb);
}
template <typename C>
__device__ __forceinline__ void tpinv_w(const VK& k, C* x, const C* c) {
  if (!k.mixed) tpinv_dir(x, c, k.G);
  else col::tpinv_mixed(x, c, k.G, k.wa, k.wb);
}

__device__ __forceinline__ int mode_of(int idx, int m0) { return m0 + (idx % TM); }

// =========================================================== forward: to nodal
// DCT of the FP64 tile src (ready) to nodal values in the precision of CO,
// stored to out; spare is a free FP64 tile used as scratch.
template <typename CO>
__device__ __forceinline__ void to_nodal(const VK& k, const col::DctSharedT<CO>& ds,
                                         const double2* src, double2* spare, CO* out, int m0) {
  if constexpr (sizeof(CO) == sizeof(double2)) {
    tdct(spare, src, k.dct, ds, false, k.P);
    __syncthreads();
    tstore(spare, out, k.P, m0, k.M);
  } else {
    float2* fs = reinterpret_cast<float2*>(spare);
    float2* fo = fs + k.P * TM;
    tcvt(fs, src, k.P);
    __syncthreads();
    tdct(fo, fs, k.dct, ds, false, k.P);
    __syncthreads();
    tstore(fo, out, k.P, m0, k.M);
  }
}

// CO = double2: plain FP64 path; CO = float2: the mixed-precision path keeps
// the Galerkin stencils in FP64 and runs the DCT in FP32.
template <typename CO>
__global__ void __launch_bounds__(NT) k_vfwd(VK k, const double2* q, const double2* w,
                                             const double2* th, CO* qn, CO* wn, CO* tn) {
  extern __shared__ double2 sm[];
  double2* b0 = sm;
  double2* b1 = sm + k.P * TM;
  const col::DctSharedT<CO> ds = col::dct_shared<CO>(k.dct, sm + 2 * k.P * TM);
  const int m0 = blockIdx.x * TM;
  if (q) {
    tload(b0, q, k.P, m0, k.M);
    __syncthreads();
    to_nodal(k, ds, b0, b1, qn, m0);
    __syncthreads();
  }
  if (w) {
    tload(b0, w, k.G, m0, k.M);
    __syncthreads();
    tstencil_w(k, b1, b0);
    __syncthreads();
    to_nodal(k, ds, b1, b0, wn, m0);
    __syncthreads();
  }
  if (th) {
    tload(b0, th, k.G, m0, k.M);
    __syncthreads();
    tstencil_dir(b1, b0, k.P, k.G);
    __syncthreads();
    to_nodal(k, ds, b1, b0, tn, m0);
  }
}

// form of the explicit operand A that k_vback reads
enum AKind {
  AK_F64 = 0,       // FP64 nodal values (plain path)
  AK_F32_NODAL = 1, // FP32 nodal values, inverse DCT in FP32
  AK_F32_COEF = 2,  // FP32 explicit tendencies from the tensor-core inverse:
                    // E_q (Chebyshev), E_w and E_theta (Galerkin, pinv applied)
};

// Chebyshev coefficients (FP64 tile out) of the explicit operand A, read in
// the form AK; tmp is a free tile.
template <int AK, typename DS, typename C>
__device__ __forceinline__ void a_to_coef(const VK& k, const DS& ds, const double2* Ad,
                                          const float2* Af, C* tmp, C* out, int m0) {
  if constexpr (AK == AK_F32_COEF) {
    col::tloadp(out, Af, k.P, m0, k.M);
  } else if constexpr (AK == AK_F64) {
    tload(tmp, Ad, k.P, m0, k.M);
    __syncthreads();
    tdct(out, tmp, k.dct, ds, true, k.P);
  } else {
    float2* fi = reinterpret_cast<float2*>(tmp);
    float2* fo = fi + k.P * TM;
    tload(fi, Af, k.P, m0, k.M);
    __syncthreads();
    tdct(fo, fi, k.dct, ds, true, k.P);
    __syncthreads();
    tcvt(out, fo, k.P);
  }
}

// =========================================================== back + stage + solve-pre
// Tiles of type C: double2, or cdfl (double-float, the mixed path with the
// tensor-core inverse, AK_F32_COEF) -- fields in global memory stay FP64.
template <int MODE, int AK, typename C = double2>
__global__ void __launch_bounds__(NT) k_vback(VK k, VArgs a) {
  static_assert(std::is_same<C, double2>::value || AK == AK_F32_COEF,
                "double-float tiles read the explicit operand as coefficients");
  using T = typename col::Prec<C>::T;
  using Pr = col::Prec<C>;
  extern __shared__ double2 sm_raw[];
  C* sm = reinterpret_cast<C*>(sm_raw);
  const int PT = k.P * TM;
  C *b0 = sm, *b1 = sm + PT, *b2 = sm + 2 * PT, *b3 = sm + 3 * PT, *b4 = sm + 4 * PT;
  using CA = typename std::conditional<AK == AK_F32_NODAL, float2, double2>::type;
  col::DctSharedT<CA> ds{};
  if constexpr (AK != AK_F32_COEF) ds = col::dct_shared<CA>(k.dct, sm_raw + 5 * PT);
  const int m0 = blockIdx.x * TM;
  const int P = k.P, G = k.G, M = k.M;
  const size_t Ms = (size_t)M;
  const T alpha = Pr::s(a.alpha), cE1 = Pr::s(a.c_E1), cE2 = Pr::s(a.c_E2);
  const T omega = Pr::s(a.omega), gdt = Pr::s(k.gdt), Ra = Pr::s(k.Ra);
  // L2 prefetch of the CTA's columns of a field (the line holding modes m0,
  // m0 + 1 at every level), one field group ahead of the phase that reads it,
  // so that the phase's loads find L2 instead of waiting on DRAM
  auto pf = [&](const void* f, int nlev, size_t esize) {
    if (f == nullptr) return;
    const char* base = static_cast<const char*>(f) + (size_t)m0 * esize;
    for (int l = threadIdx.x; l < nlev; l += blockDim.x)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)l * Ms * esize));
  };
  if constexpr (MODE == VB_STAGE2) {
    pf(a.w1, G, 16); pf(a.q0, P, 16); pf(a.E1q, P, 16); pf(a.q1, P, 16);
  } else if constexpr (MODE == VB_STAGE1) {
    pf(a.q0, P, 16); pf(AK == AK_F32_COEF ? (const void*)a.Awf : (const void*)nullptr, G, 8);
  }

  // ------------------------------------------------------------- q
  if (MODE != VB_SOLVE) {
    a_to_coef<AK>(k, ds, a.Aq, a.Aqf, b0, b1, m0);
    __syncthreads();
    // E_q = -Aq - i beta kx psi, psi = -inv_denom * q_state
    const double2* qs = (MODE == VB_STAGE2) ? a.q1 : a.q0;
    for (int i = threadIdx.x; i < PT; i += blockDim.x) {
      const int l = i / TM, m = mode_of(i, m0);
      if (m >= M) continue;
      C e = (AK == AK_F32_COEF) ? b1[i] : col::gneg(b1[i]);
      if (k.beta != 0.0) {
        const T sb = Pr::s(k.beta * k.kx[m] * k.inv_denom[m]);
        const C qv = Pr::in(qs[(size_t)l * Ms + m]);
        e = gmk<C>(fma(-sb, qv.y, e.x), fma(sb, qv.x, e.y));
      }
      if (a.Cq) e = gadd(e, Pr::in(a.Cq[(size_t)l * Ms + m]));  // learned closure
      b1[i] = e;
    }
    __syncthreads();
    if (MODE == VB_RHS) {
      col::tstorep(b1, a.Eq, P, m0, M);
    } else if (MODE == VB_STAGE1) {
      col::tstorep(b1, a.E1q, P, m0, M);
      for (int i = threadIdx.x; i < PT; i += blockDim.x) {
        const int l = i / TM, m = mode_of(i, m0);
        if (m < M) b1[i] = col::gaxpy(alpha, b1[i], Pr::in(a.q0[(size_t)l * Ms + m]));
      }
    } else {  // STAGE2: I_q = G_Z S_w w1
      col::tloadp(b2, a.w1, G, m0, M);
      __syncthreads();
      tstencil_w(k, b3, b2);
      __syncthreads();
      tgz(b2, b3, k.N);
      __syncthreads();
      for (int i = threadIdx.x; i < PT; i += blockDim.x) {
        const int l = i / TM, m = mode_of(i, m0);
        if (m >= M) continue;
        const size_t g = (size_t)l * Ms + m;
        C r = Pr::in(a.q0[g]);
        r = col::gaxpy(cE1, Pr::in(a.E1q[g]), r);
        r = col::gaxpy(cE2, b1[i], r);
        r = col::gaxpy(omega, b2[i], r);
        r = col::gaxpy((-omega) * Pr::s(k.drq[m]), Pr::in(a.q1[g]), r);
        b1[i] = r;
      }
    }
    __syncthreads();
  } else {
    col::tloadp(b1, a.q0, P, m0, M);  // R_q given
    __syncthreads();
  }
  if (MODE != VB_RHS) {
    col::tstorep(b1, a.Rq, P, m0, M);
    // temp = R_q / alpha_q ; d_gal = pinv_w(inv_denom * G_Z temp)
    for (int i = threadIdx.x; i < PT; i += blockDim.x) {
      const int m = mode_of(i, m0);
      b2[i] = (m < M) ? gscale(b1[i], Pr::s(k.inv_aq[m])) : col::gzero<C>();
    }
    __syncthreads();
    tgz(b3, b2, k.N);
    __syncthreads();
    for (int i = threadIdx.x; i < PT; i += blockDim.x) {
      const int m = mode_of(i, m0);
      b3[i] = (m < M) ? gscale(b3[i], Pr::s(k.inv_denom[m])) : col::gzero<C>();
    }
    __syncthreads();
    tpinv_w(k, b4, b3);
    __syncthreads();
  }

  // ------------------------------------------------------------- w
  if constexpr (MODE == VB_STAGE2) {
    if constexpr (AK == AK_F32_COEF) pf(a.Awf, G, 8);
    pf(a.t1, G, 16); pf(a.w0, G, 16); pf(a.E1w, G, 16);
  } else if constexpr (MODE == VB_STAGE1) {
    pf(a.w0, G, 16);
    if constexpr (AK == AK_F32_COEF) pf(a.Atf, G, 8);
  }
  if (MODE != VB_SOLVE) {
    if constexpr (AK == AK_F32_COEF) {  // E_w in the Galerkin basis
      col::tloadp(b2, a.Awf, G, m0, M);
    } else {
      a_to_coef<AK>(k, ds, a.Aw, a.Awf, b0, b1, m0);
      __syncthreads();
      for (int i = threadIdx.x; i < PT; i += blockDim.x) b1[i] = col::gneg(b1[i]);
      __syncthreads();
      tpinv_w(k, b2, b1);
    }
    __syncthreads();
    if (MODE == VB_RHS) {
      col::tstorep(b2, a.Ew, G, m0, M);
    } else if (MODE == VB_STAGE1) {
      col::tstorep(b2, a.E1w, G, m0, M);
      for (int i = threadIdx.x; i < G * TM; i += blockDim.x) {
        const int l = i / TM, m = mode_of(i, m0);
        if (m < M) b2[i] = col::gaxpy(alpha, b2[i], Pr::in(a.w0[(size_t)l * Ms + m]));
      }
    } else {  // I_w = pinv_w(inv_denom G_Z q1 + Ra S_dir t1)
      col::tloadp(b0, a.q1, P, m0, M);
      __syncthreads();
      tgz(b1, b0, k.N);
      __syncthreads();
      col::tloadp(b0, a.t1, G, m0, M);
      __syncthreads();
      tstencil_dir(b3, b0, P, G);
      __syncthreads();
      for (int i = threadIdx.x; i < PT; i += blockDim.x) {
        const int m = mode_of(i, m0);
        b1[i] = (m < M) ? col::gaxpy(Ra, b3[i], gscale(b1[i], Pr::s(k.inv_denom[m]))) : col::gzero<C>();
      }
      __syncthreads();
      tpinv_w(k, b0, b1);
      __syncthreads();
      for (int i = threadIdx.x; i < G * TM; i += blockDim.x) {
        const int l = i / TM, m = mode_of(i, m0);
        if (m >= M) continue;
        const size_t g = (size_t)l * Ms + m;
        C r = Pr::in(a.w0[g]);
        r = col::gaxpy(cE1, Pr::in(a.E1w[g]), r);
        r = col::gaxpy(cE2, b2[i], r);
        r = col::gaxpy(omega, b0[i], r);
        r = col::gaxpy((-omega) * Pr::s(k.drw[m]), Pr::in(a.w1[g]), r);
        b2[i] = r;
      }
    }
    __syncthreads();
  } else {
    col::tloadp(b2, a.w0, G, m0, M);  // R_w given
    __syncthreads();
  }
  if (MODE != VB_RHS) {
    for (int i = threadIdx.x; i < G * TM; i += blockDim.x) b4[i] = col::gaxpy(gdt, b4[i], b2[i]);
    __syncthreads();
  }

  // ------------------------------------------------------------- theta
  if constexpr (MODE == VB_STAGE2) {
    if constexpr (AK == AK_F32_COEF) pf(a.Atf, G, 8);
    pf(a.t0, G, 16); pf(a.E1t, G, 16); pf(a.t1p, G, 16);
  } else if constexpr (MODE == VB_STAGE1) {
    pf(a.t0, G, 16);
  }
  if (MODE != VB_SOLVE) {
    if constexpr (AK == AK_F64) {
      tload(b0, a.At, P, m0, M);
      __syncthreads();
      if (a.dtb_nodal != nullptr) {  // legacy evolve_mean: + (dTheta/dZ)_nodal * w_nodal
        for (int i = threadIdx.x; i < PT; i += blockDim.x) {
          const int l = i / TM, m = mode_of(i, m0);
          if (m < M) b0[i] = caxpy(a.dtb_nodal[l], a.Wn[(size_t)l * Ms + m], b0[i]);
        }
        __syncthreads();
      }
      tdct(b1, b0, k.dct, ds, true, P);
    } else if constexpr (AK == AK_F32_NODAL) {  // the mixed path has no legacy evolve_mean term
      a_to_coef<AK>(k, ds, nullptr, a.Atf, b0, b1, m0);
    }
    if constexpr (AK == AK_F32_COEF) {  // E_theta in the Galerkin basis
      col::tloadp(b2, a.Atf, G, m0, M);
    } else {
      __syncthreads();
      for (int i = threadIdx.x; i < PT; i += blockDim.x) b1[i] = col::gneg(b1[i]);
      __syncthreads();
      tpinv_dir(b2, b1, G);
    }
    __syncthreads();
    if (MODE == VB_RHS) {
      col::tstorep(b2, a.Et, G, m0, M);
    } else if (MODE == VB_STAGE1) {
      col::tstorep(b2, a.E1t, G, m0, M);
      for (int i = threadIdx.x; i < G * TM; i += blockDim.x) {
        const int l = i / TM, m = mode_of(i, m0);
        if (m < M) b2[i] = col::gaxpy(alpha, b2[i], Pr::in(a.t0[(size_t)l * Ms + m]));
      }
    } else {  // I_t = w1 (shared basis) or pinv_dir(S_w w1)
      col::tloadp(b0, a.w1, G, m0, M);
      __syncthreads();
      if (k.mixed) {
        tstencil_w(k, b1, b0);
        __syncthreads();
        tpinv_dir(b0, b1, G);
        __syncthreads();
      }
      const T iac = Pr::s(a.inv_alpha_c);
      for (int i = threadIdx.x; i < G * TM; i += blockDim.x) {
        const int l = i / TM, m = mode_of(i, m0);
        if (m >= M) continue;
        const size_t g = (size_t)l * Ms + m;
        C r = Pr::in(a.t0[g]);
        r = col::gaxpy(cE1, Pr::in(a.E1t[g]), r);
        r = col::gaxpy(cE2, b2[i], r);
        r = col::gaxpy(omega, b0[i], r);
        const C t1v = Pr::in(a.t1[g]);
        r = col::gaxpy((-omega) * Pr::s(k.drt[m]), t1v, r);
        if (a.inv_alpha_c != 0.0) {
          const C c = gscale(gsub(t1v, Pr::in(a.t1p[g])), iac);
          r = col::gaxpy(omega, c, r);
        }
        b2[i] = r;
      }
    }
    __syncthreads();
  } else {
    col::tloadp(b2, a.t0, G, m0, M);  // R_th given
    __syncthreads();
  }
  if (MODE != VB_RHS) {
    col::tstorep(b2, a.Rt, G, m0, M);
    for (int i = threadIdx.x; i < G * TM; i += blockDim.x) {
      const int m = mode_of(i, m0);
      b0[i] = (m < M) ? gscale(b2[i], Pr::s(k.inv_at[m])) : col::gzero<C>();
    }
    __syncthreads();
    if (k.mixed) {  // theta basis -> w basis
      tstencil_dir(b1, b0, P, G);
      __syncthreads();
      tpinv_w(k, b0, b1);
      __syncthreads();
    }
    const T c = Pr::s(k.gdt * k.Ra);
    for (int i = threadIdx.x; i < G * TM; i += blockDim.x) b4[i] = col::gaxpy(c, b0[i], b4[i]);
    __syncthreads();
    col::tstorep(b4, a.rhs_w, G, m0, M);
  }
}

// =========================================================== back-substitution
template <typename C = double2>
__global__ void __launch_bounds__(NT) k_vpost(VK k, const double2* Rq, const double2* Rt,
                                              const double2* wn, double2* qo, double2* to,
                                              bool zero_mean) {
  using Pr = col::Prec<C>;
  extern __shared__ double2 sm_raw[];
  C* sm = reinterpret_cast<C*>(sm_raw);
  const int PT = k.P * TM;
  C *b0 = sm, *b1 = sm + PT, *b2 = sm + 2 * PT;
  const int m0 = blockIdx.x * TM;
  const int M = k.M;
  const typename Pr::T gdt = Pr::s(k.gdt);
  col::tprefetch(Rq, k.P, m0, M, sizeof(double2));
  col::tprefetch(Rt, k.G, m0, M, sizeof(double2));
  col::tloadp(b0, wn, k.G, m0, M);
  __syncthreads();
  tstencil_w(k, b1, b0);  // w Chebyshev coefficients
  __syncthreads();
  tgz(b2, b1, k.N);
  __syncthreads();
  for (int i = threadIdx.x; i < PT; i += blockDim.x) {
    const int l = i / TM, m = mode_of(i, m0);
    if (m >= M) continue;
    const size_t g = (size_t)l * M + m;
    qo[g] = (zero_mean && m == 0) ? czero()
                                  : Pr::out(gscale(col::gaxpy(gdt, b2[i], Pr::in(Rq[g])), Pr::s(k.inv_aq[m])));
  }
  if (k.mixed) {  // w basis -> theta basis
    __syncthreads();
    tpinv_dir(b0, b1, k.G);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < k.G * TM; i += blockDim.x) {
    const int l = i / TM, m = mode_of(i, m0);
    if (m >= M) continue;
    const size_t g = (size_t)l * M + m;
    to[g] = (zero_mean && m == 0) ? czero()
                                  : Pr::out(gscale(col::gaxpy(gdt, b0[i], Pr::in(Rt[g])), Pr::s(k.inv_at[m])));
  }
}

// =========================================================== implicit tendency
__global__ void __launch_bounds__(NT) k_itend(VK k, const double2* q, const double2* w,
                                              const double2* th, double2* Iq, double2* Iw,
                                              double2* It) {
  extern __shared__ double2 sm[];
  const int PT = k.P * TM;
  double2 *b0 = sm, *b1 = sm + PT, *b2 = sm + 2 * PT, *b3 = sm + 3 * PT;
  const int m0 = blockIdx.x * TM;
  const int M = k.M;
  tload(b0, w, k.G, m0, M);
  __syncthreads();
  tstencil_w(k, b1, b0);
  __syncthreads();
  tgz(b2, b1, k.N);
  __syncthreads();
  tstore(b2, Iq, k.P, m0, M);
  if (k.mixed) {
    tpinv_dir(b3, b1, k.G);
    __syncthreads();
    tstore(b3, It, k.G, m0, M);
  } else {
    tstore(b0, It, k.G, m0, M);
  }
  __syncthreads();
  tload(b0, q, k.P, m0, M);
  __syncthreads();
  tgz(b1, b0, k.N);
  tload(b2, th, k.G, m0, M);
  __syncthreads();
  tstencil_dir(b3, b2, k.P, k.G);
  __syncthreads();
  for (int i = threadIdx.x; i < PT; i += blockDim.x) {
    const int m = mode_of(i, m0);
    b1[i] = (m < M) ? caxpy(k.Ra, b3[i], cscale(b1[i], k.inv_denom[m])) : czero();
  }
  __syncthreads();
  tpinv_w(k, b0, b1);
  __syncthreads();
  tstore(b0, Iw, k.G, m0, M);
}

// =========================================================== per-shell dense solve
// w = imex_inv[shell(k)] @ rhs_w for every mode; one CTA per shell, the
// shell's matrix streams once through L1 while its modes' columns sit in
// shared memory.  NC modes per pass (compile-time, so no FMA is wasted).
template <int NC>
__device__ __forceinline__ void shell_rows(const double* __restrict__ A, const double2* xs, int G,
                                           int ld_x, double2* out, const int* modes, int M) {
  for (int i = threadIdx.x; i < G; i += blockDim.x) {
    double2 acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = czero();
    const double* row = A + (size_t)i * G;
    for (int j = 0; j < G; ++j) {
      const double v = __ldg(row + j);
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = caxpy(v, xs[j * ld_x + c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) out[(size_t)i * M + modes[c]] = acc[c];
  }
}

constexpr int SHELL_NC = 8;

__global__ void __launch_bounds__(NT) k_shell(const double* mats, const int* start, const int* list,
                                              const double2* rhs, double2* out, int G, int M) {
  extern __shared__ double2 xs[];  // [G][SHELL_NC]
  __shared__ int modes[SHELL_NC];
  const int s = blockIdx.x;
  const int b = start[s], e = start[s + 1];
  const double* A = mats + (size_t)s * G * G;
  for (int c0 = b; c0 < e; c0 += SHELL_NC) {
    const int nc = min(SHELL_NC, e - c0);
    if (threadIdx.x < nc) modes[threadIdx.x] = list[c0 + threadIdx.x];
    __syncthreads();
    for (int i = threadIdx.x; i < G * nc; i += blockDim.x) {
      const int j = i / nc, c = i - j * nc;
      xs[j * SHELL_NC + c] = rhs[(size_t)j * M + modes[c]];
    }
    __syncthreads();
    switch (nc) {
      case 1: shell_rows<1>(A, xs, G, SHELL_NC, out, modes, M); break;
      case 2: shell_rows<2>(A, xs, G, SHELL_NC, out, modes, M); break;
      case 3: shell_rows<3>(A, xs, G, SHELL_NC, out, modes, M); break;
      case 4: shell_rows<4>(A, xs, G, SHELL_NC, out, modes, M); break;
      case 5: shell_rows<5>(A, xs, G, SHELL_NC, out, modes, M); break;
      case 6: shell_rows<6>(A, xs, G, SHELL_NC, out, modes, M); break;
      case 7: shell_rows<7>(A, xs, G, SHELL_NC, out, modes, M); break;
      default: shell_rows<8>(A, xs, G, SHELL_NC, out, modes, M); break;
    }
    __syncthreads();
  }
}

// =========================================================== layout kernels
__global__ void k_gather(Dims d, const double2* full, double2* cmp, int levels, int* status) {
  const size_t total = (size_t)levels * d.Nx * d.Nk;
  bool outside_nonzero = false;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % d.Nk);
    const size_t rest = i / d.Nk;
    const int row = (int)(rest % d.Nx);
    const int l = (int)(rest / d.Nx);
    const int kxi = row <= d.Nx / 2 ? row : row - d.Nx;
    const double2 v = full[i];
    if (abs(kxi) <= d.K && c <= d.K) {
      const int r = kxi >= 0 ? kxi : kxi + d.Mr;
      cmp[(size_t)l * d.M + r * d.Mc + c] = v;
    } else if (v.x != 0.0 || v.y != 0.0) {
      outside_nonzero = true;
    }
  }
  if (outside_nonzero && status) atomicOr(status, 1 << NHQG_STATUS_BIT_OOB);
}

__global__ void k_scatter(Dims d, const double2* cmp, double2* full, int levels) {
  const size_t total = (size_t)levels * d.Nx * d.Nk;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % d.Nk);
    const size_t rest = i / d.Nk;
    const int row = (int)(rest % d.Nx);
    const int l = (int)(rest / d.Nx);
    const int kxi = row <= d.Nx / 2 ? row : row - d.Nx;
    double2 v = czero();
    if (abs(kxi) <= d.K && c <= d.K) {
      const int r = kxi >= 0 ? kxi : kxi + d.Mr;
      v = cmp[(size_t)l * d.M + r * d.Mc + c];
    }
    full[i] = v;
  }
}

// zero the k=0 mode, Hermitian-project the ky=0 column and, in the
// full-band layout of the 3/2 rule, the ky = Nx/2 column
// (nhqg/solver.py:107-146, 993-999)
__global__ void k_finalize(Dims d, const double2* q, const double2* w, const double2* th,
                           double2* qo, double2* wo, double2* to) {
  const int nlev[3] = {d.P, d.G, d.G};
  const double2* src[3] = {q, w, th};
  double2* dst[3] = {qo, wo, to};
  const size_t per = (size_t)d.M;
  const size_t total = (size_t)(d.P + 2 * d.G) * per;
  const int cnyq = d.pad ? d.Nk - 1 : -1;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int f = 0;
    size_t j = i;
    while (j >= (size_t)nlev[f] * per) { j -= (size_t)nlev[f] * per; ++f; }
    const int m = (int)(j % per);
    const size_t lbase = j - m;
    const int r = m / d.Mc, c = m - r * d.Mc;
    double2 v;
    if (c != 0 && c != cnyq) {
      v = src[f][j];
    } else {
      const int rm = mirror_row(r, d.Mr);
      const bool z0 = c == 0;  // the zeroed k = 0 mode sits in the ky = 0 column
      double2 a = (z0 && r == 0) ? czero() : src[f][lbase + (size_t)r * d.Mc + c];
      double2 b = (z0 && rm == 0) ? czero() : src[f][lbase + (size_t)rm * d.Mc + c];
      v = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
    }
    dst[f][j] = v;
  }
}

// Hermitian projection of the ky=0 column (and of the ky = Nx/2 column in the
// full-band layout), in place (no k=0 zeroing)
__global__ void k_hermitian(Dims d, double2* q, double2* w, double2* th) {
  const int nlev[3] = {d.P, d.G, d.G};
  double2* f3[3] = {q, w, th};
  const int half = d.Mr / 2;  // rows 1..half pair with Mr-1..Mr-half
  const int ncol = d.pad ? 2 : 1;
  const int per = ncol * (half + 1);
  const int total = (d.P + 2 * d.G) * per;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    int f = 0, j = i;
    while (j >= nlev[f] * per) { j -= nlev[f] * per; ++f; }
    const int l = j / per, rc = j - l * per;
    const int ci = rc / (half + 1), r = rc - ci * (half + 1);
    double2* col = f3[f] + (size_t)l * d.M + (ci == 0 ? 0 : d.Nk - 1);  // entries at row*Mc
    if (r == 0) {
      col[0] = make_double2(col[0].x, 0.0);
    } else {
      const int rm = mirror_row(r, d.Mr);
      const double2 a = col[(size_t)r * d.Mc], b = col[(size_t)rm * d.Mc];
      const double2 h = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
      col[(size_t)r * d.Mc] = h;
      col[(size_t)rm * d.Mc] = cconj(h);
    }
  }
}

// Horizontal mean of irfft2(a) irfft2(b) per level by Parseval: every mode of
// the half plane counts twice except the ky = 0 column, which enters through
// its Hermitian projection.  In the full-band layout of the 3/2 rule the
// means are those of the zero-padded fields (nhqg/solver.py:204-245): the
// ky = Nx/2 column is an ordinary column of the padded grid (weight 2), and
// the kx Nyquist entry of the ky = 0 column sits at kx = -Nx/2 alone, so its
// Hermitian part contributes Re(a b*)/2.  Each level is split into kParSeg segments, one CTA
// each; the last CTA of a level to finish adds the segment sums in segment
// order (deterministic) and resets the level's counter for the next launch.
// C = cdfl accumulates the per-thread sums in double-float (the mixed path;
// the FP64 pipe bounds the FP64 form on GB300); CTA totals are FP64.
constexpr int kParSeg = 4;  // 4 P CTAs: one wave on 152 SMs for P <= 257
__device__ __forceinline__ double2 as_d2(double2 v) { return v; }
__device__ __forceinline__ double2 as_d2(float2 v) { return make_double2(f2d_bits(v.x), f2d_bits(v.y)); }

template <typename C, typename TA>
__global__ void __launch_bounds__(NT) k_parseval(Dims d, const TA* a, const double2* b,
                                                 double* out, double scale, double* partials,
                                                 unsigned* counters) {
  using T = typename col::Prec<C>::T;
  __shared__ double scratch[32];
  __shared__ bool is_last;
  const int l = blockIdx.y, seg = blockIdx.x;
  const TA* al = a + (size_t)l * d.M;
  const double2* bl = b + (size_t)l * d.M;
  const int chunk = (d.M + kParSeg - 1) / kParSeg;
  const int m0 = seg * chunk, m1 = min(d.M, m0 + chunk);
  // two FMAs per element on two accumulators; the half-plane weight 2 is
  // applied once
  T accr = T(0), acci = T(0);
#pragma unroll 8
  for (int m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
    const C x = col::Prec<C>::in(al[m]), y = col::Prec<C>::in(bl[m]);
    accr = fma(x.x, y.x, accr);
    acci = fma(x.y, y.y, acci);
  }
  double acc;
  if constexpr (std::is_same<C, double2>::value) acc = 2.0 * (accr + acci);
  else acc = 2.0 * df_to_double(accr + acci);
  // the ky = 0 column: replace the doubled term by the Hermitian projection
  for (int r = threadIdx.x; r < d.Mr; r += blockDim.x) {
    const int m = r * d.Mc;
    if (m < m0 || m >= m1) continue;
    const int rm = mirror_row(r, d.Mr);
    const double2 x = as_d2(al[m]), xm = as_d2(al[rm * d.Mc]);
    const double2 y = bl[m], ym = bl[rm * d.Mc];
    const double xy = fma(x.x, y.x, x.y * y.y);
    if (rm == r && r != 0) {  // padded kx Nyquist (full-band layout only)
      acc += 0.5 * xy - 2.0 * xy;
      continue;
    }
    const double hx_re = 0.5 * (x.x + xm.x), hx_im = 0.5 * (x.y - xm.y);
    const double hy_re = 0.5 * (y.x + ym.x), hy_im = 0.5 * (y.y - ym.y);
    acc += fma(hx_re, hy_re, hx_im * hy_im) - 2.0 * xy;
  }
  const double tot = block_sum(acc, scratch);
  if (threadIdx.x == 0) {
    partials[(size_t)l * kParSeg + seg] = tot;
    __threadfence();
    is_last = atomicAdd(&counters[l], 1u) == kParSeg - 1;
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    double sum = 0.0;
    for (int q = 0; q < kParSeg; ++q) sum += __ldcg(partials + (size_t)l * kParSeg + q);
    out[l] = sum * scale;
    counters[l] = 0u;
  }
}

// Two horizontal means in one pass over a: out_ab[l] = <a b>, out_ac[l] =
// <a c> (the corrector's <w^2> and <w theta>), same weights, order and
// arithmetic as k_parseval; partials hold two sums per (level, segment).
template <typename C, typename TA>
__global__ void __launch_bounds__(NT) k_parseval2(Dims d, const TA* a, const TA* b,
                                                  const double2* c, double* out_ab, double* out_ac,
                                                  double scale, double* partials, unsigned* counters) {
  using T = typename col::Prec<C>::T;
  __shared__ double scratch[32];
  __shared__ bool is_last;
  const int l = blockIdx.y, seg = blockIdx.x;
  const TA* al = a + (size_t)l * d.M;
  const TA* bl = b + (size_t)l * d.M;
  const double2* cl = c + (size_t)l * d.M;
  const int chunk = (d.M + kParSeg - 1) / kParSeg;
  const int m0 = seg * chunk, m1 = min(d.M, m0 + chunk);
  T br = T(0), bi = T(0), cr = T(0), ci = T(0);
#pragma unroll 8
  for (int m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
    const C x = col::Prec<C>::in(al[m]), y = col::Prec<C>::in(bl[m]), z = col::Prec<C>::in(cl[m]);
    br = fma(x.x, y.x, br);
    bi = fma(x.y, y.y, bi);
    cr = fma(x.x, z.x, cr);
    ci = fma(x.y, z.y, ci);
  }
  double ab, ac;
  if constexpr (std::is_same<C, double2>::value) {
    ab = 2.0 * (br + bi);
    ac = 2.0 * (cr + ci);
  } else {
    ab = 2.0 * df_to_double(br + bi);
    ac = 2.0 * df_to_double(cr + ci);
  }
  for (int r = threadIdx.x; r < d.Mr; r += blockDim.x) {
    const int m = r * d.Mc;
    if (m < m0 || m >= m1) continue;
    const int rm = mirror_row(r, d.Mr);
    const double2 x = as_d2(al[m]), xm = as_d2(al[rm * d.Mc]);
    const double2 y = as_d2(bl[m]), ym = as_d2(bl[rm * d.Mc]);
    const double2 z = cl[m], zm = cl[rm * d.Mc];
    const double xy = fma(x.x, y.x, x.y * y.y), xz = fma(x.x, z.x, x.y * z.y);
    if (rm == r && r != 0) {
      ab += 0.5 * xy - 2.0 * xy;
      ac += 0.5 * xz - 2.0 * xz;
      continue;
    }
    const double hx_re = 0.5 * (x.x + xm.x), hx_im = 0.5 * (x.y - xm.y);
    const double hy_re = 0.5 * (y.x + ym.x), hy_im = 0.5 * (y.y - ym.y);
    const double hz_re = 0.5 * (z.x + zm.x), hz_im = 0.5 * (z.y - zm.y);
    ab += fma(hx_re, hy_re, hx_im * hy_im) - 2.0 * xy;
    ac += fma(hx_re, hz_re, hx_im * hz_im) - 2.0 * xz;
  }
  const double tab = block_sum(ab, scratch);
  __syncthreads();
  const double tac = block_sum(ac, scratch);
  if (threadIdx.x == 0) {
    partials[((size_t)l * kParSeg + seg) * 2] = tab;
    partials[((size_t)l * kParSeg + seg) * 2 + 1] = tac;
    __threadfence();
    is_last = atomicAdd(&counters[l], 1u) == kParSeg - 1;
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    double s1 = 0.0, s2 = 0.0;
    for (int q = 0; q < kParSeg; ++q) {
      s1 += __ldcg(partials + ((size_t)l * kParSeg + q) * 2);
      s2 += __ldcg(partials + ((size_t)l * kParSeg + q) * 2 + 1);
    }
    out_ab[l] = s1 * scale;
    out_ac[l] = s2 * scale;
    counters[l] = 0u;
  }
}

__global__ void k_zero_mode0(double2* f, int levels, int M) {
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < levels; l += gridDim.x * blockDim.x)
    f[(size_t)l * M] = czero();
}

// dynamic shared memory of a column kernel: nbuf FP64 tiles plus the DCT
// work area in FP64 or (f32_dct) FP32
inline size_t vsmem(const Params& p, int nbuf, bool dct = false, bool f32_dct = false) {
  size_t b = (size_t)nbuf * p.d.P * TM * sizeof(double2);
  if (dct) b += col::dct_smem_bytes(make_dct(p, Tables{}), f32_dct);
  return b;
}
inline int vgrid(const Params& p) { return (p.d.M + TM - 1) / TM; }

template <typename CO>
cudaError_t vfwd_t(const Params& p, const Tables& t, const double2* q, const double2* w,
                   const double2* th, CO* qn, CO* wn, CO* tn, cudaStream_t st) {
  VK k = make_vk(p, t);
  const size_t sm = vsmem(p, 2, true, sizeof(CO) == sizeof(float2));
  cudaFuncSetAttribute(k_vfwd<CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_vfwd<CO><<<vgrid(p), NT, sm, st>>>(k, q, w, th, qn, wn, tn);
  return cudaGetLastError();
}

template <int MODE, int AK, typename C = double2>
void vback_t(const VK& k, const VArgs& a, size_t sm, int grid, cudaStream_t st) {
  cudaFuncSetAttribute(k_vback<MODE, AK, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_vback<MODE, AK, C><<<grid, NT, sm, st>>>(k, a);
}
template <int MODE>
void vback_ak(int ak, const VK& k, const VArgs& a, size_t sm, int grid, cudaStream_t st) {
  if (ak == AK_F64) vback_t<MODE, AK_F64>(k, a, sm, grid, st);
  else if (ak == AK_F32_NODAL) vback_t<MODE, AK_F32_NODAL>(k, a, sm, grid, st);
  else if (a.df) vback_t<MODE, AK_F32_COEF, cdfl>(k, a, sm, grid, st);
  else vback_t<MODE, AK_F32_COEF>(k, a, sm, grid, st);
}

}  // namespace

cudaError_t launch_vfwd(const Params& p, const Tables& t, const double2* q, const double2* w,
                        const double2* th, double2* qn, double2* wn, double2* tn, cudaStream_t st) {
  return vfwd_t<double2>(p, t, q, w, th, qn, wn, tn, st);
}

cudaError_t launch_vfwd_f32(const Params& p, const Tables& t, const double2* q, const double2* w,
                            const double2* th, float2* qn, float2* wn, float2* tn, cudaStream_t st) {
  if (!p.fast_dct || !t.tw_v_f) return cudaErrorInvalidValue;
  return vfwd_t<float2>(p, t, q, w, th, qn, wn, tn, st);
}

cudaError_t launch_vback(const Params& p, const Tables& t, int mode, const VArgs& a, cudaStream_t st) {
  VK k = make_vk(p, t);
  const bool f32 = a.Aqf != nullptr;
  const int ak = (!f32 || mode == VB_SOLVE) ? AK_F64 : (a.af_coef ? AK_F32_COEF : AK_F32_NODAL);
  const size_t sm = ak == AK_F32_COEF ? vsmem(p, 5) : vsmem(p, 5, true, ak == AK_F32_NODAL);
  const int g = vgrid(p);
  if (f32 && (a.dtb_nodal || !a.Awf || !a.Atf)) return cudaErrorInvalidValue;
  if (ak == AK_F32_NODAL && (!p.fast_dct || !t.tw_v_f)) return cudaErrorInvalidValue;
  switch (mode) {
    case VB_RHS: vback_ak<VB_RHS>(ak, k, a, sm, g, st); break;
    case VB_STAGE1: vback_ak<VB_STAGE1>(ak, k, a, sm, g, st); break;
    case VB_STAGE2: vback_ak<VB_STAGE2>(ak, k, a, sm, g, st); break;
    default: vback_t<VB_SOLVE, AK_F64>(k, a, sm, g, st); break;
  }
  return cudaGetLastError();
}

namespace {

__device__ __forceinline__ double2 operator*(double a, double2 b) { return make_double2(a * b.x, a * b.y); }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// out = base + dt * (sum_k c_k x_k), the sum taken left to right (the stage
// combinations of nhqg/solver.py:1066-1119)
template <typename T>
__global__ void k_lincomb(LinCombT<T> a) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += stride) {
    T s = a.c[0] * a.x[0][i];
    for (int k = 1; k < a.n; ++k) s = s + a.c[k] * a.x[k][i];
    a.out[i] = a.base[i] + a.dt * s;
  }
}

// K -= rate * Y per compact mode (nhqg/solver.py:1002-1009)
__global__ void k_sub_diss(double2* __restrict__ K, const double2* __restrict__ Y,
                           const double* __restrict__ rate, int levels, int M) {
  const size_t n = (size_t)levels * M;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double r = rate[i % M];
    K[i] = make_double2(K[i].x - r * Y[i].x, K[i].y - r * Y[i].y);
  }
}

}  // namespace

template <typename T>
cudaError_t launch_lincomb(const LinCombT<T>& a, cudaStream_t st) {
  if (a.n < 1 || a.n > kLinCombMax) return cudaErrorInvalidValue;
  if (a.count == 0) return cudaSuccess;
  const int blocks = (int)std::min<size_t>((a.count + 255) / 256, 152 * 8);
  k_lincomb<T><<<blocks, 256, 0, st>>>(a);
  return cudaGetLastError();
}
template cudaError_t launch_lincomb<double>(const LinCombT<double>&, cudaStream_t);
template cudaError_t launch_lincomb<double2>(const LinCombT<double2>&, cudaStream_t);

cudaError_t launch_sub_diss(const Params& p, double2* K, const double2* Y, const double* rate,
                            int levels, cudaStream_t st) {
  const size_t n = (size_t)levels * p.d.M;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_sub_diss<<<blocks, 256, 0, st>>>(K, Y, rate, levels, p.d.M);
  return cudaGetLastError();
}

cudaError_t launch_shell(const Params& p, const Tables& t, const double2* rhs_w, double2* w_out,
                         cudaStream_t st) {
  const size_t sm = (size_t)p.d.G * SHELL_NC * sizeof(double2);
  cudaFuncSetAttribute(k_shell, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_shell<<<t.n_shells, NT, sm, st>>>(t.shell_inv, t.shell_start, t.shell_modes, rhs_w, w_out,
                                      p.d.G, p.d.M);
  return cudaGetLastError();
}

cudaError_t launch_vpost(const Params& p, const Tables& t, const double2* Rq, const double2* Rt,
                         const double2* w_new, double2* q_out, double2* t_out, bool zero_mean,
                         cudaStream_t st, bool df) {
  VK k = make_vk(p, t);
  const size_t sm = vsmem(p, 3);
  auto kern = df ? k_vpost<cdfl> : k_vpost<double2>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  kern<<<vgrid(p), NT, sm, st>>>(k, Rq, Rt, w_new, q_out, t_out, zero_mean);
  return cudaGetLastError();
}

cudaError_t launch_itend(const Params& p, const Tables& t, const double2* q, const double2* w,
                         const double2* th, double2* Iq, double2* Iw, double2* It, cudaStream_t st) {
  VK k = make_vk(p, t);
  const size_t sm = vsmem(p, 4);
  cudaFuncSetAttribute(k_itend, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_itend<<<vgrid(p), NT, sm, st>>>(k, q, w, th, Iq, Iw, It);
  return cudaGetLastError();
}

cudaError_t launch_gather(const Params& p, const double2* full, double2* compact, int levels,
                          int* status, cudaStream_t st) {
  k_gather<<<4 * 152, 256, 0, st>>>(p.d, full, compact, levels, status);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const Params& p, const double2* compact, double2* full, int levels,
                           cudaStream_t st) {
  k_scatter<<<4 * 152, 256, 0, st>>>(p.d, compact, full, levels);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const Params& p, const double2* q, const double2* w, const double2* th,
                            double2* qo, double2* wo, double2* to, cudaStream_t st) {
  k_finalize<<<4 * 152, 256, 0, st>>>(p.d, q, w, th, qo, wo, to);
  return cudaGetLastError();
}

cudaError_t launch_hermitian(const Params& p, double2* q, double2* w, double2* th, cudaStream_t st) {
  k_hermitian<<<4 * 152, 256, 0, st>>>(p.d, q, w, th);
  return cudaGetLastError();
}

cudaError_t launch_zero_mode0(const Params& p, double2* f, int levels, cudaStream_t st) {
  k_zero_mode0<<<1, 256, 0, st>>>(f, levels, p.d.M);
  return cudaGetLastError();
}

size_t parseval_partials(int levels) { return 2 * (size_t)levels * kParSeg; }

template <typename TA>
cudaError_t parseval2_t(const Params& p, const TA* a, const TA* b, const double2* c,
                        int levels, double* out_ab, double* out_ac, Work& w, cudaStream_t st,
                        bool df) {
  const double n2 = (double)p.d.Nx * (double)p.d.Nx;
  auto kern = df ? k_parseval2<cdfl, TA> : k_parseval2<double2, TA>;
  kern<<<dim3(kParSeg, levels), NT, 0, st>>>(p.d, a, b, c, out_ab, out_ac, 1.0 / (n2 * n2), w.partials,
                                             w.counters);
  return cudaGetLastError();
}

template <typename TA>
cudaError_t parseval_t(const Params& p, const TA* a, const double2* b, int levels,
                       double* out, Work& w, cudaStream_t st, bool df) {
  const double n2 = (double)p.d.Nx * (double)p.d.Nx;
  auto kern = df ? k_parseval<cdfl, TA> : k_parseval<double2, TA>;
  kern<<<dim3(kParSeg, levels), NT, 0, st>>>(p.d, a, b, out, 1.0 / (n2 * n2), w.partials,
                                             w.counters);
  return cudaGetLastError();
}

cudaError_t launch_parseval(const Params& p, const double2* a, const double2* b, int levels,
                            double* out, Work& w, cudaStream_t st, bool df) {
  return parseval_t(p, a, b, levels, out, w, st, df);
}
cudaError_t launch_parseval(const Params& p, const float2* a, const double2* b, int levels,
                            double* out, Work& w, cudaStream_t st, bool df) {
  return parseval_t(p, a, b, levels, out, w, st, df);
}
cudaError_t launch_parseval2(const Params& p, const double2* a, const double2* b, const double2* c,
                             int levels, double* out_ab, double* out_ac, Work& w, cudaStream_t st,
                             bool df) {
  return parseval2_t(p, a, b, c, levels, out_ab, out_ac, w, st, df);
}
cudaError_t launch_parseval2(const Params& p, const float2* a, const float2* b, const double2* c,
                             int levels, double* out_ab, double* out_ac, Work& w, cudaStream_t st,
                             bool df) {
  return parseval2_t(p, a, b, c, levels, out_ab, out_ac, w, st, df);
}

}  // namespace nhqg

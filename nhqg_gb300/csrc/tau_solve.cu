// O(N) implicit w solve of the mixed-precision path (FP64).
//
// The per-shell operator of the reference (nhqg/grid.py:398-430, q_boundary
// 'none') is A' = a I - s pinv_w G_Z^2 S_w with, at the shell's rounded |k|^2,
//   a = alpha_w - (gamma dt)^2 Ra_sigma / alpha_th,  s = (gamma dt)^2 c_k / alpha_q.
// (With the open-top w basis the reference subtracts (gamma dt)^2 Ra/alpha_th K
// with K = map_th_to_w map_w_to_th, which is the identity up to rounding.)
// Multiplying A' w = r by the top block of S_w gives the Chebyshev-tau
// Helmholtz problem for c = S_w w:
//   a c_n - 4 s e_n = f_n  (n <= N-2),   f = (S_w r)[0:N-1],
// with e = G_xi^2 c and the two w boundary rows.  In the unknowns e (the
// second-derivative coefficients) plus c_0, c_1, the relation
//   c_n = A_n e_{n-2} + B_n e_n + C_n e_{n+2},
//   A_n = k_{n-2} / (4n(n-1)), B_n = -1 / (2(n^2-1)), C_n = 1 / (4n(n+1))
// (e_j = 0 for j > N-2) makes each parity class tridiagonal (weakly
// diagonally dominant, so the Thomas sweep needs no pivoting) with one free
// unknown e_p, and the boundary rows close a 2x2 system for e_0, e_1.
//
// Everything that depends only on the shell -- the Thomas pivots, the
// homogeneous column z of the free unknown, the inverse 2x2 boundary matrix
// -- is factored once on the host (build_tau_tables).  Per mode the solve is
// then two first-order recurrences per parity class plus dot products, ~12 N
// FP64 operations instead of 2 (N-1)^2 for the dense inverse, and it never
// forms G_Z^2 (entries up to N^4), so it is also more accurate than the
// reference's dense table: the two differ by that table's rounding, 1e-12 at
// Nz=16 to 1e-8 at Nz=256 for the lowest |k|.
#include <cmath>

#include "engine.h"

namespace nhqg {

namespace {

// universal coefficients of c_n(e), n >= 2 (zero where e would leave 0..N-2)
inline double coefA(int n) { return (n == 2 ? 2.0 : 1.0) / (4.0 * n * (n - 1)); }
inline double coefB(int n, int N) { return n <= N - 2 ? -1.0 / (2.0 * (n * (double)n - 1.0)) : 0.0; }
inline double coefC(int n, int N) { return n + 2 <= N - 2 ? 1.0 / (4.0 * n * (n + 1)) : 0.0; }

}  // namespace

// Host factorisation of the tau systems of all shells.  Layout:
//   tab [shell][4][P]: rm (Thomas pivot reciprocals), Lrm (L_n rm_n, 0 on
//                      the first row of a class), cp (U_n rm_n), z (free-
//                      unknown column, z_p = 1)
//   par [shell][8]:    1/a, 4 s / a, Minv (4, row-major), s == 0 flag, 0
//   uni [5][P]:        A_n, B_n, C_n, W1_n, W2_n (boundary-row weights on e)
// g1 is the first boundary functional (1 for Dirichlet, n^2 for the open
// top); the second is (-1)^n.
void build_tau_tables(int N, bool open_top, int n_shells, const double* coef,
                      std::vector<double>& tab, std::vector<double>& par, std::vector<double>& uni) {
  const int P = N + 1;
  uni.assign(5 * (size_t)P, 0.0);
  double* A = uni.data();
  double* B = A + P;
  double* C = B + P;
  double* W1 = C + P;
  double* W2 = W1 + P;
  auto g1 = [&](int n) { return open_top ? (double)n * n : 1.0; };
  auto g2 = [&](int n) { return (n & 1) ? -1.0 : 1.0; };
  for (int n = 2; n <= N; ++n) { A[n] = coefA(n); B[n] = coefB(n, N); C[n] = coefC(n, N); }
  // c_n(v) for n >= 2 involves v_{n-2}, v_n, v_{n+2}: W_i[j] = sum_n g_i(n) dc_n/dv_j
  for (int j = 2; j <= N - 2; ++j) {
    double w1 = 0.0, w2 = 0.0;
    if (j + 2 <= N) { w1 += g1(j + 2) * A[j + 2]; w2 += g2(j + 2) * A[j + 2]; }
    w1 += g1(j) * B[j];
    w2 += g2(j) * B[j];
    if (j - 2 >= 2) { w1 += g1(j - 2) * C[j - 2]; w2 += g2(j - 2) * C[j - 2]; }
    W1[j] = w1;
    W2[j] = w2;
  }
  tab.assign((size_t)n_shells * 4 * P, 0.0);
  par.assign((size_t)n_shells * 8, 0.0);
  std::vector<double> zf(P), zeta(P);
  for (int sh = 0; sh < n_shells; ++sh) {
    const double a = coef[2 * sh], s = coef[2 * sh + 1];
    double* rm = tab.data() + (size_t)sh * 4 * P;
    double* Lrm = rm + P;
    double* cp = Lrm + P;
    double* z = cp + P;
    double* pr = par.data() + (size_t)sh * 8;
    pr[0] = 1.0 / a;
    pr[1] = 4.0 * s / a;
    pr[6] = (s == 0.0) ? 1.0 : 0.0;
    if (s == 0.0) continue;
    for (int p = 0; p < 2; ++p) {
      int last = -1;
      for (int n = p + 2; n <= N - 2; n += 2) {
        const double L = a * A[n], D = a * B[n] - 4.0 * s, U = a * C[n];
        const bool first = (n == p + 2);
        const double r = 1.0 / (first ? D : D - L * cp[n - 2]);
        rm[n] = r;
        Lrm[n] = first ? 0.0 : L * r;
        cp[n] = U * r;
        zf[n] = first ? L * r : -L * r * zf[n - 2];
        last = n;
      }
      for (int n = last; n >= p + 2; n -= 2) zeta[n] = (n == last) ? zf[n] : zf[n] - cp[n] * zeta[n + 2];
      for (int n = p + 2; n <= N - 2; n += 2) z[n] = -zeta[n];
      z[p] = 1.0;
    }
    // boundary matrix M_ij = sum_n g_i(n) c_n(z^(j))
    double M[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    for (int j = 0; j < 2; ++j) {
      auto zj = [&](int n) { return (n >= 0 && n <= N - 2 && (n & 1) == j) ? z[n] : 0.0; };
      for (int n = 0; n <= N; ++n) {
        double c;
        if (n < 2) c = (n == j) ? 4.0 * s / a : 0.0;
        else c = A[n] * zj(n - 2) + B[n] * zj(n) + C[n] * zj(n + 2);
        M[0][j] += g1(n) * c;
        M[1][j] += g2(n) * c;
      }
    }
    const double rdet = 1.0 / (M[0][0] * M[1][1] - M[0][1] * M[1][0]);
    pr[2] = M[1][1] * rdet;
    pr[3] = -M[0][1] * rdet;
    pr[4] = -M[1][0] * rdet;
    pr[5] = M[0][0] * rdet;
  }
}

namespace {

constexpr int kTauThreads = 64;  // 16 modes per CTA, 4 chains (re/im x parity) per mode: small CTAs
                                  // spread the chains evenly over the SMs
constexpr int kPF = 8;            // rows per operand prefetch block

struct TK {
  int N, G, M;
  bool open_top;
  double g1_0, g1_1;  // first boundary functional at n = 0, 1
  const int* mode_shell;
  const double *tab, *par, *uni;
  const double *wa, *wb;
};

// Thread t owns chain (compact mode t/4, re/im, parity).  The columns stay in
// global memory (the per-launch working set, a few tens of MB, lives in L2):
// element n of a [level][M] complex field viewed as doubles is
// (n M + m) 2 + re/im.  Without shared-memory columns the occupancy is set by
// registers, and many chains in flight hide the 64-cycle FP64 latency of the
// serial recurrences.  y is scratch for the particular solution and then c.
__global__ void __launch_bounds__(kTauThreads) k_tau_solve(TK k, const double* __restrict__ r,
                                                           double* __restrict__ y,
                                                           double* __restrict__ wout) {
  const int N = k.N, G = k.G, M = k.M, P = N + 1;
  const int t = blockIdx.x * kTauThreads + threadIdx.x;
  const int m = t >> 2, ri = (t >> 1) & 1, p = t & 1;
  // lanes past M run the same warp collectives on zeros and store nothing
  const bool live = m < M;
  const int mc = live ? m : 0;
  auto at = [&](int n) { return ((size_t)n * M + mc) * 2 + ri; };
  auto rv = [&](int n) { return live ? r[at(n)] : 0.0; };
  auto f = [&](int n) {  // (S_w r)_n
    if (!k.open_top) {
      double v = -rv(n);
      if (n >= 2) v += rv(n - 2);
      return v;
    }
    double v = rv(n);
    if (n >= 1) v = fma(k.wa[n - 1], rv(n - 1), v);
    if (n >= 2) v = fma(k.wb[n - 2], rv(n - 2), v);
    return v;
  };
  const double* uA = k.uni;
  const double* uB = uA + P;
  const double* uC = uB + P;
  const double* uW1 = uC + P;
  const double* uW2 = uW1 + P;
  const int sh = live ? k.mode_shell[m] : 0;
  const double* rm = k.tab + (size_t)sh * 4 * P;
  const double* Lrm = rm + P;
  const double* cp = Lrm + P;
  const double* z = cp + P;
  const double* pr = k.par + (size_t)sh * 8;
  const double ra = pr[0], s4ra = pr[1];
  const bool s_zero = pr[6] != 0.0;
  const double f0 = f(0), f1 = f(1);
  const double fp = p ? f1 : f0;
  // Thomas forward and back substitution in the class, then the boundary-row
  // dot products of the particular solution.  Each block of kPF rows loads
  // its operands before its dependent chain runs.
  double b0 = 0.0, b1 = 0.0;
  if (!s_zero) {
    const int cnt = (N - 2 - p) / 2;  // rows n = p+2, p+4, .., last
    const int last = p + 2 * cnt;
    double d = 0.0;
    double rprev = rv(p);  // Dirichlet f_n = r_{n-2} - r_n: r_{n-2} carried from the row before
    for (int r0 = 0; r0 < cnt; r0 += kPF) {
      double lr[kPF], ty[kPF];
      if (!k.open_top) {
        double rr[kPF], rmv[kPF];
#pragma unroll
        for (int q = 0; q < kPF; ++q) {
          const int n = p + 2 + 2 * (r0 + q);
          const bool in = r0 + q < cnt;
          lr[q] = in ? __ldg(Lrm + n) : 0.0;
          rmv[q] = in ? __ldg(rm + n) : 0.0;
          rr[q] = in ? rv(n) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < kPF; ++q) {
          ty[q] = (rprev - rr[q]) * rmv[q];
          rprev = rr[q];
        }
      } else {
#pragma unroll
        for (int q = 0; q < kPF; ++q) {
          const int n = p + 2 + 2 * (r0 + q);
          const bool in = r0 + q < cnt;
          lr[q] = in ? __ldg(Lrm + n) : 0.0;
          ty[q] = in ? f(n) * __ldg(rm + n) : 0.0;
        }
      }
#pragma unroll
      for (int q = 0; q < kPF; ++q) {
        if (r0 + q < cnt) {
          d = fma(-lr[q], d, ty[q]);
          if (live) y[at(p + 2 + 2 * (r0 + q))] = d;
        }
      }
    }
    double nxt = 0.0;
    for (int r0 = cnt - 1; r0 >= 0; r0 -= kPF) {
      double cc[kPF], yy[kPF], w1[kPF], w2[kPF];
#pragma unroll
      for (int q = 0; q < kPF; ++q) {
        const int n = p + 2 + 2 * (r0 - q);
        const bool in = r0 - q >= 0;
        cc[q] = in ? __ldg(cp + n) : 0.0;
        yy[q] = (in && live) ? y[at(n)] : 0.0;
        w1[q] = in ? __ldg(uW1 + n) : 0.0;
        w2[q] = in ? __ldg(uW2 + n) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < kPF; ++q) {
        if (r0 - q >= 0) {
          const int n = p + 2 + 2 * (r0 - q);
          const double v = (n == last) ? yy[q] : fma(-cc[q], nxt, yy[q]);
          if (live) y[at(n)] = v;
          nxt = v;
          b0 = fma(w1[q], v, b0);
          b1 = fma(w2[q], v, b1);
        }
      }
    }
  }
  b0 += __shfl_xor_sync(0xffffffffu, b0, 1);  // partner lane: same column, other parity
  b1 += __shfl_xor_sync(0xffffffffu, b1, 1);
  // Dirichlet w basis: the pseudo-inverse w_n = -sum_{j <= n} c_j (same
  // parity, n < G = N-1) runs inside the pass that forms c; the open top's
  // w recurrence couples the two classes and reads c back from y
  const bool fold = !k.open_top;
  double acc = 0.0;
  if (s_zero) {
    // A' = a I: c_n = f_n / a for n <= N-2 (the rows the pseudo-inverse reads)
    for (int n = p; n <= N - 2; n += 2) {
      const double cv = f(n) * ra;
      if (fold) {
        acc -= cv;
        if (live) wout[at(n)] = acc;
      } else if (live) {
        y[at(n)] = cv;
      }
    }
  } else {
    b0 = fma(ra, fma(k.g1_0, f0, k.g1_1 * f1), b0);
    b1 = fma(ra, f0 - f1, b1);
    const double x = -fma(pr[2 + 2 * p], b0, pr[3 + 2 * p] * b1);
    // e = v + x z on the class (e_p = x, z_p = 1), then c in place with a
    // sliding window over e_{n-2}, e_n, e_{n+2}; e_{n+2} is formed from v_{n+2}
    // before row n+2 is overwritten
    double em2 = 0.0, e0 = x;
#pragma unroll 4
    for (int n = p; n <= N - 2; n += 2) {
      double ep2 = 0.0;
      if (n + 2 <= N - 2) ep2 = fma(x, __ldg(z + n + 2), live ? y[at(n + 2)] : 0.0);
      double c;
      if (n < 2) c = fma(s4ra, e0, fp * ra);
      else c = fma(__ldg(uA + n), em2, fma(__ldg(uB + n), e0, __ldg(uC + n) * ep2));
      if (fold) {
        acc -= c;
        if (live) wout[at(n)] = acc;
      } else if (live) {
        y[at(n)] = c;
      }
      em2 = e0;
      e0 = ep2;
    }
  }
  if (fold) return;
  __syncwarp();
  // open top: w = pinv_w c over n < G (the pseudo-inverse reads c_0 .. c_{N-2})
  if (!live) return;
  if (p == 0) {
    double w1 = 0.0, w2 = 0.0;
    for (int n = 0; n < G; ++n) {
      double w = y[at(n)];
      if (n >= 1) w = fma(-k.wa[n - 1], w1, w);
      if (n >= 2) w = fma(-k.wb[n - 2], w2, w);
      wout[at(n)] = w;
      w2 = w1;
      w1 = w;
    }
  }
}

}  // namespace

cudaError_t launch_tau_solve(const Params& p, const Tables& t, const double2* rhs_w, double2* w_out,
                             double2* scratch, cudaStream_t st) {
  if (!t.tau_tab || !scratch) return cudaErrorInvalidValue;
  TK k;
  k.N = p.d.Nz; k.G = p.d.G; k.M = p.d.M;
  k.open_top = t.wst_a != nullptr;
  k.g1_0 = k.open_top ? 0.0 : 1.0;
  k.g1_1 = 1.0;
  k.mode_shell = t.mode_shell;
  k.tab = t.tau_tab; k.par = t.tau_par; k.uni = t.tau_uni;
  k.wa = t.wst_a; k.wb = t.wst_b;
  const size_t threads = 4 * (size_t)k.M;
  const int blocks = (int)((threads + kTauThreads - 1) / kTauThreads);
  k_tau_solve<<<blocks, kTauThreads, 0, st>>>(k, reinterpret_cast<const double*>(rhs_w),
                                               reinterpret_cast<double*>(scratch),
                                               reinterpret_cast<double*>(w_out));
  return cudaGetLastError();
}

}  // namespace nhqg

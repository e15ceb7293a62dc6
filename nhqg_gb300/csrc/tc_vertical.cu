// Chebyshev <-> CGL vertical transforms of the mixed-precision path on the
// 5th-generation tensor cores: tcgen05.mma kind::tf32, FP32 accumulators in
// tensor memory, the matrix operand streamed by the bulk-copy (TMA) engine.
//
// Reference operations: _to_nodal / _to_coeffs (nhqg/solver.py:45-52) with
// V[j,n] = cos(pi j n / N) and V^-1 the DCT-I inverse (nhqg/grid.py:192-201).
// The forward transforms of the Galerkin fields fold their stencil into the
// matrix, V S (nhqg/grid.py:499-502; nhqg/solver.py:65-72).
//
// Parity folding.  CGL row j and its mirror N-j see the same |cos|,
// A[N-j,n] = (-1)^n A[j,n] (also for V S: S maps index g to g and g+2).  With
//   E_j = sum_{n even} A[j,n] c_n,   O_j = sum_{n odd} A[j,n] c_n   (j < N/2)
// the nodal values are x_j = E_j + O_j and x_{N-j} = E_j - O_j; the middle row
// x_{N/2} is a dot product on the CUDA cores.  The inverse folds its input:
// s_j = x_j + x_{N-j} feeds the even coefficients, d_j = x_j - x_{N-j} the odd
// ones, and coefficient N is the CUDA-core row.  Each fold is a GEMM with
// M = 128 rows (N/2 <= 128), which halves the tensor work of the dense
// product.  The host checks the mirror property of every matrix before it
// enables this path.
//
// Precision: every operand is split into two TF32 terms a = a_hi + a_lo
// (22 significant bits) and D = A_hi B_hi + A_hi B_lo + A_lo B_hi accumulates
// in FP32 (the dropped A_lo B_lo term is 2^-22 relative).
//
// Work decomposition.  One CTA owns 128 real columns (64 complex modes; the
// matrices are real, so real and imaginary parts are independent columns)
// and every level.  The fold index (K) runs in chunks of 8 (one MMA k-step)
// through a 3-stage shared-memory ring (two CTAs per SM); per stage
//   A chunk: E_hi, E_lo, O_hi, O_lo (4 tiles of 128 x 8 TF32), laid out by the
//     host in the canonical no-swizzle K-major core-matrix order and fetched
//     by one cp.async.bulk on the stage's "full" mbarrier;
//   B chunk: 16 converter warps (4 groups x 128 columns) fold, split and
//     store their input rows in the same order, then arrive on the stage's
//     "ready" mbarrier.  Each converter streams its own input elements into
//     registers 3 chunks ahead (coalesced across the warp).
// A control warp owns TMEM; its lane 0 issues the bulk copies and six MMAs
// per chunk (E and O accumulators, 128 TMEM columns each) and commits them to
// the stage's "empty" mbarrier, which releases the stage.  The epilogue reads
// the accumulators with tcgen05.ld (warp w owns TMEM lanes 32(w%4)..+31) and
// writes FP32 rows through a shared-memory transpose.  Every mbarrier wait is
// bounded (one second); a wait that runs out sets the timeout bit of the
// status word, drains the copies and MMAs in flight, frees TMEM and returns.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "engine.h"

namespace nhqg {

namespace {

constexpr int kCols = 128;                 // real columns per CTA = MMA N
constexpr int kFold = 128;                 // MMA M
constexpr int kKc = 8;                     // fold indices per chunk (TF32 k-step)
constexpr int kStages = 3;
constexpr int kThreads = 512;
constexpr int kGroups = kThreads / 128;    // thread groups per column (2 fold indices each)
static_assert(2 * kGroups == 8, "each group converts two fold indices of a chunk");
constexpr int kTile = kFold * kKc * 4;     // one 128 x 8 TF32 operand tile, bytes
constexpr int kAB = 4 * kTile;             // hi/lo x even/odd tiles of one chunk
constexpr int kAhead = 3;                  // chunks of input prefetched into registers
static_assert(kAhead == kStages, "the register ring and the stage ring share their index");
constexpr uint32_t kTmemCols = 256;        // E accumulator [0,128), O [128,256)
constexpr uint64_t kWaitNs = 1000000000ull;
constexpr int kXrow = 512;                 // CUDA-core row table (zero-padded)

// canonical no-swizzle K-major layout: 8-row x 16-byte core matrices, the two
// core matrices of a k-step 128 B apart (leading byte offset), consecutive
// 8-row groups 256 B apart (stride byte offset)
constexpr uint32_t kLBO = 128, kSBO = 256;
__host__ __device__ constexpr int tile_off(int row, int k) {
  return (row >> 3) * kSBO + (k >> 2) * kLBO + (row & 7) * 16 + (k & 3) * 4;
}

// instruction descriptor: D FP32, A and B TF32, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kCols >> 3) << 17) |
                            ((uint32_t)(kFold >> 4) << 24);

template <bool INV>
__host__ __device__ constexpr int stage_bytes() { return 2 * kAB; }
template <bool INV>
constexpr size_t tc_smem() {
  return 1024 + (size_t)kStages * stage_bytes<INV>() + 128 + (kGroups * 128 + kXrow) * sizeof(float);
}

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t saddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// wait for the phase of the given parity to complete, at most kWaitNs
__device__ bool mbar_wait(uint32_t a, uint32_t parity) {
  if (mbar_try(a, parity)) return true;
  const uint64_t t0 = gtimer();
  while (!mbar_try(a, parity))
    if (gtimer() - t0 > kWaitNs) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ uint64_t sdesc(uint32_t a) {
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)(kLBO >> 4) << 16) |
         ((uint64_t)(kSBO >> 4) << 32) | (1ull << 46);
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t ad, uint64_t bd, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   mbar)
               : "memory");
}
// 32 consecutive TMEM columns of this thread's lane, waited for
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// round to the nearest TF32 value (10 explicit mantissa bits), ties away
__host__ __device__ inline float tf32_round(float x) {
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(x);
  u = (u + 0x1000u) & 0xFFFFE000u;
  return __uint_as_float(u);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u = (u + 0x1000u) & 0xFFFFE000u;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
__host__ __device__ inline void tf32_split(double v, float& hi, float& lo) {
  hi = tf32_round((float)v);
  lo = tf32_round((float)(v - (double)hi));
}
// FP32 split (the device's conversion of its inputs): no FP64 arithmetic,
// which GB300 retires at 1/64 of the FP32 rate
__device__ __forceinline__ void tf32_split_f(float v, float& hi, float& lo) {
  hi = tf32_round(v);
  lo = tf32_round(v - hi);
}
// FP64 -> FP32 by truncating the significand to 23 bits, in integer
// arithmetic (magnitudes below 2^-126 flush to zero; the operands of these
// transforms stay far below the FP32 overflow)
__device__ __forceinline__ float f64_to_f32_trunc(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const uint32_t hw = static_cast<uint32_t>(b >> 32);
  const int e = static_cast<int>((hw >> 20) & 0x7FFu) - 1023 + 127;
  const uint32_t m = ((hw & 0xFFFFFu) << 3) | static_cast<uint32_t>((b >> 29) & 7u);
  const uint32_t sgn = hw & 0x80000000u;
  return __uint_as_float(e > 0 ? (sgn | (static_cast<uint32_t>(e) << 23) | m) : sgn);
}

struct TcField {
  const void* in;      // forward: FP64 [K][ncols]; inverse: FP32 [P][ncols]
  float* out;          // FP32 [P][ncols] (the inverse writes over its input)
  const uint8_t* img;  // nch * kAB bytes
  const float* xrow;   // CUDA-core row: forward A[N/2][0:K], inverse A[N][0:P]
  int K, rows, nch;    // input rows, output rows (inverse: P or G), k-chunks
};
struct TcArgs {
  TcField f[3];
  int ncols, N, H;
  int* status;
};

template <bool INV>
__global__ void __launch_bounds__(kThreads + 64, 2) k_tc_vertical(const __grid_constant__ TcArgs a) {
  using In = typename std::conditional<INV, float, double>::type;
  constexpr int SB = stage_bytes<INV>();
  extern __shared__ uint8_t tc_smem_raw[];
  uint8_t* sm = tc_smem_raw + ((1024 - (saddr(tc_smem_raw) & 1023)) & 1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kStages * SB);  // full, ready, empty
  uint32_t* slot = reinterpret_cast<uint32_t*>(bars + 3 * kStages);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(slot + 1);
  volatile int* progress = abort_flag + 1;  // [0] chunks committed, [1] matrix copies issued
  float* red = reinterpret_cast<float*>(sm + kStages * SB + 128);   // [kGroups][kCols]
  float* xr = red + kGroups * kCols;                                 // [kXrow]

  const TcField& F = a.f[blockIdx.y];
  const int tid = threadIdx.x;
  const bool control = tid >= kThreads;  // warp 16: TMEM and MMAs; warp 17: matrix copies
  const int t = tid & (kCols - 1);       // converters: column of the tile
  const int grp = (tid / kCols) & (kGroups - 1);  // fold indices 2 grp, 2 grp + 1 of a chunk
  const int col0 = blockIdx.x * kCols;
  const int col = col0 + t;
  const bool cval = !control && col < a.ncols;
  const int N = a.N, H = a.H, K = F.K, nch = F.nch;
  const size_t ld = (size_t)a.ncols;
  const uint32_t sbase = saddr(sm);
  const uint32_t full0 = saddr(bars), ready0 = full0 + 8 * kStages, empty0 = ready0 + 8 * kStages;
  const In* src = static_cast<const In*>(F.in) + (cval ? col : 0);

  if (tid == kThreads) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(ready0 + 8 * s, kThreads);
      mbar_init(empty0 + 8 * s, 1);
    }
    *abort_flag = 0;
    progress[0] = progress[1] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid >= kThreads && tid < kThreads + 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int i = tid; i < kXrow; i += blockDim.x) xr[i] = F.xrow[i];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;

  float xacc = 0.f;   // converters: CUDA-core row, this thread's share of column t
  if (!control) {
    // Input rows of chunk c that this thread converts (column t), loaded
    // straight into registers kAhead chunks ahead: forward rows 16c + 4grp + q
    // (q = 0..3: even, odd, even, odd), inverse rows j = 8c + 2grp + h and
    // N - j (h = 0, 1).  Rows outside the matrix read as zero.
    In pre[kAhead][4];
    auto load = [&](int c, In (&v)[4]) {
      if constexpr (!INV) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int n = 16 * c + 4 * grp + q;
          v[q] = (cval && n < K) ? __ldcs(src + (size_t)n * ld) : In(0);
        }
      } else {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int j = 8 * c + 2 * grp + h;
          v[2 * h] = (cval && j <= H) ? __ldcs(src + (size_t)j * ld) : In(0);
          v[2 * h + 1] = (cval && j < H) ? __ldcs(src + (size_t)(N - j) * ld) : In(0);
        }
      }
    };
#pragma unroll
    for (int d = 0; d < kAhead; ++d)
      if (d < nch) load(d, pre[d]);
    for (int c0 = 0; c0 < nch; c0 += kAhead) {
#pragma unroll
      for (int d = 0; d < kAhead; ++d) {
        const int c = c0 + d;  // stage d
        if (c >= nch || *abort_flag) break;
        // the stage's previous MMAs (chunk c - kStages) must be done before B is rewritten
        if (c >= kStages && !mbar_wait(empty0 + 8 * d, ((c / kStages) - 1) & 1)) {
          *abort_flag = 1;
          break;
        }
        float ve[2], vo[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if constexpr (!INV) {
            const int n = 16 * c + 4 * grp + 2 * h;
            ve[h] = f64_to_f32_trunc(pre[d][2 * h]);
            vo[h] = f64_to_f32_trunc(pre[d][2 * h + 1]);
            const float2 x = *reinterpret_cast<const float2*>(xr + n);
            xacc = fmaf(x.x, ve[h], fmaf(x.y, vo[h], xacc));
          } else {
            const int j = 8 * c + 2 * grp + h;
            const float top = pre[d][2 * h], bot = pre[d][2 * h + 1];
            ve[h] = top + bot;  // j == H: bot reads zero; beyond H both do
            vo[h] = top - bot;  // (the odd matrix is zero at and beyond column H)
            xacc = fmaf(xr[j], top, fmaf(xr[N - j], bot, xacc));
          }
        }
        if (c + kAhead < nch) load(c + kAhead, pre[d]);
        float eh[2], el[2], oh[2], ol[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          tf32_split_f(ve[h], eh[h], el[h]);
          tf32_split_f(vo[h], oh[h], ol[h]);
        }
        uint8_t* bst = sm + d * SB + kAB + tile_off(t, 2 * grp);
        *reinterpret_cast<float2*>(bst + 0 * kTile) = make_float2(eh[0], eh[1]);
        *reinterpret_cast<float2*>(bst + 1 * kTile) = make_float2(el[0], el[1]);
        *reinterpret_cast<float2*>(bst + 2 * kTile) = make_float2(oh[0], oh[1]);
        *reinterpret_cast<float2*>(bst + 3 * kTile) = make_float2(ol[0], ol[1]);
        fence_async_smem();
        mbar_arrive(ready0 + 8 * d);
      }
    }
    red[grp * kCols + t] = xacc;
  } else if (tid == kThreads) {
    // MMA issuer: both operands of chunk c present -> six MMAs -> release the stage
    for (int c = 0; c < nch; ++c) {
      const int s = c % kStages;
      const uint32_t ph = (c / kStages) & 1;
      if (*abort_flag || !mbar_wait(full0 + 8 * s, ph) || !mbar_wait(ready0 + 8 * s, ph)) {
        *abort_flag = 1;
        break;
      }
      tc_fence_after();
      const uint32_t a0 = sbase + s * SB, b0 = a0 + kAB;
      const uint32_t acc = c > 0 ? 1u : 0u;
      tc_mma(tmem, sdesc(a0), sdesc(b0), acc);                                  // E_hi B_hi
      tc_mma(tmem, sdesc(a0), sdesc(b0 + kTile), 1u);                           // E_hi B_lo
      tc_mma(tmem, sdesc(a0 + kTile), sdesc(b0), 1u);                           // E_lo B_hi
      tc_mma(tmem + 128, sdesc(a0 + 2 * kTile), sdesc(b0 + 2 * kTile), acc);    // O_hi B_hi
      tc_mma(tmem + 128, sdesc(a0 + 2 * kTile), sdesc(b0 + 3 * kTile), 1u);     // O_hi B_lo
      tc_mma(tmem + 128, sdesc(a0 + 3 * kTile), sdesc(b0 + 2 * kTile), 1u);     // O_lo B_hi
      tc_commit(empty0 + 8 * s);
      progress[0] = c + 1;
    }
    if (progress[0] == nch && !*abort_flag &&
        !mbar_wait(empty0 + 8 * ((nch - 1) % kStages), ((nch - 1) / kStages) & 1))
      *abort_flag = 1;
  } else if (tid == kThreads + 32) {
    // matrix producer: chunk c's A into its stage once the stage's previous MMAs are done
    for (int c = 0; c < nch; ++c) {
      const int s = c % kStages;
      if (*abort_flag) break;
      if (c >= kStages && !mbar_wait(empty0 + 8 * s, ((c / kStages) - 1) & 1)) {
        *abort_flag = 1;
        break;
      }
      const uint32_t fb = full0 + 8 * s;
      mbar_expect_tx(fb, kAB);
      bulk_g2s(sbase + s * SB, F.img + (size_t)c * kAB, kAB, fb);
      progress[1] = c + 1;
    }
  }
  __syncthreads();
  const bool ok = !*abort_flag;
  if (ok && !control) {
    // Warp w reads TMEM lanes 32 (w % 4) .. + 31 (its lane quarter) for the
    // 32 columns 32 (w / 4) ..; the 32 x 32 block goes through shared memory
    // (the idle ring) so that every global store writes 32 consecutive
    // columns of one row.
    tc_fence_after();
    const int warp = tid >> 5, lane = tid & 31;
    const int lq = warp & 3, cc = 32 * (warp >> 2);
    const uint32_t tl = tmem + ((uint32_t)(lq * 32) << 16);
    float* tt = reinterpret_cast<float*>(sm) + warp * (32 * 33);
    const int nrow = min(32, H - lq * 32);  // valid fold rows of this lane quarter
    const int cg = col0 + cc + lane;
    // one 32-column accumulator block in registers at a time: E goes to the
    // transpose tile first, then O is combined with it (forward: E + O and
    // E - O from the same two values) or written after it (inverse)
    auto store_rows = [&](int pass) {  // rows 2i / i (pass 0), 2i+1 / N-i (pass 1)
      __syncwarp();
      if (cg < a.ncols) {
        for (int r = 0; r < nrow; ++r) {
          const int i = lq * 32 + r;
          const int row = INV ? 2 * i + pass : (pass ? N - i : i);
          if (INV && row >= F.rows) break;
          F.out[(size_t)row * ld + cg] = tt[r * 33 + lane];
        }
      }
      __syncwarp();
    };
    float v[32];
    tc_ld32(tl + cc, v);
#pragma unroll
    for (int q = 0; q < 32; ++q) tt[lane * 33 + q] = v[q];
    if (INV) store_rows(0);
    tc_ld32(tl + 128 + cc, v);
    if (INV) {
#pragma unroll
      for (int q = 0; q < 32; ++q) tt[lane * 33 + q] = v[q];
      store_rows(1);
    } else {
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const float e = tt[lane * 33 + q];
        tt[lane * 33 + q] = e + v[q];
        v[q] = e - v[q];
      }
      store_rows(0);
#pragma unroll
      for (int q = 0; q < 32; ++q) tt[lane * 33 + q] = v[q];
      store_rows(1);
    }
    if (grp == 0 && cval && (!INV || F.rows > N)) {
      const float x = ((red[t] + red[kCols + t]) + red[2 * kCols + t]) + red[3 * kCols + t];
      F.out[(size_t)(INV ? N : H) * ld + col] = x;
    }
  } else if (!ok && tid == kThreads) {
    atomicOr(a.status, 1 << NHQG_STATUS_BIT_TIMEOUT);
    // drain the bulk copies and MMAs still in flight (bounded)
    const int committed = progress[0], issued = progress[1];
    for (int cc = committed; cc < issued; ++cc)
      mbar_wait(full0 + 8 * (cc % kStages), (cc / kStages) & 1);
    if (committed > 0)
      mbar_wait(empty0 + 8 * ((committed - 1) % kStages), ((committed - 1) / kStages) & 1);
  }
  tc_fence_before();
  __syncthreads();
  if (tid >= kThreads && tid < kThreads + 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// ------------------------------------------------------------ host: images
struct Dense {
  int rows, cols;
  std::vector<double> a;
  double at(int r, int c) const { return a[(size_t)r * cols + c]; }
};

// mirror property of the forward (rows) or inverse (columns) fold
bool mirror_ok(const Dense& A, int N, bool inverse) {
  double amax = 0.0, dmax = 0.0;
  for (double v : A.a) amax = std::max(amax, std::fabs(v));
  for (int r = 0; r < A.rows; ++r)
    for (int k = 0; k < A.cols; ++k) {
      double d;
      if (!inverse) {
        if (r > N / 2) continue;
        const double sg = (k & 1) ? -1.0 : 1.0;
        d = A.at(N - r, k) - sg * A.at(r, k);
      } else {
        if (k > N / 2) continue;
        const double sg = (r & 1) ? -1.0 : 1.0;
        d = A.at(r, N - k) - sg * A.at(r, k);
      }
      dmax = std::max(dmax, std::fabs(d));
    }
  return dmax <= 1e-12 * amax;
}

// A image of one transform: nch chunks of [E_hi, E_lo, O_hi, O_lo]
void fold_image(const Dense& A, int N, bool inverse, TcHostImage& out) {
  const int H = N / 2;
  const int KE = inverse ? H + 1 : (A.cols + 1) / 2;
  out.nch = (KE + kKc - 1) / kKc;
  out.K = inverse ? A.rows : A.cols;
  out.bytes.assign((size_t)out.nch * kAB, 0);
  auto put = [&](int chunk, int tile, int row, int kk, float v) {
    std::memcpy(&out.bytes[(size_t)chunk * kAB + tile * kTile + tile_off(row, kk)], &v, 4);
  };
  for (int i = 0; i < H; ++i)
    for (int f = 0; f < out.nch * kKc; ++f) {
      double e = 0.0, o = 0.0;
      if (!inverse) {
        if (2 * f < A.cols) e = A.at(i, 2 * f);
        if (2 * f + 1 < A.cols) o = A.at(i, 2 * f + 1);
      } else {
        if (f <= H && 2 * i < A.rows) e = A.at(2 * i, f);
        if (f < H && 2 * i + 1 < A.rows) o = A.at(2 * i + 1, f);
      }
      float hi, lo;
      const int chunk = f / kKc, kk = f % kKc;
      tf32_split(e, hi, lo);
      put(chunk, 0, i, kk, hi);
      put(chunk, 1, i, kk, lo);
      tf32_split(o, hi, lo);
      put(chunk, 2, i, kk, hi);
      put(chunk, 3, i, kk, lo);
    }
  const int xr = inverse ? N : H;  // no CUDA-core row for G-row inverse matrices
  out.rows = inverse ? A.rows : N + 1;
  out.xrow.assign(kXrow, 0.f);
  if (xr < A.rows)
    for (int k = 0; k < A.cols; ++k) out.xrow[k] = (float)A.at(xr, k);
}

}  // namespace

bool tc_vertical_images(const nhqg_grid_desc* g, TcHostImage img[TC_IMAGES]) {
  const int N = g->Nz, P = N + 1, G = N - 1;
  // N >= 16 keeps every fold index of the last chunk (< N/2 + 8) inside [0, N]
  if (N % 2 != 0 || N / 2 > kFold || N < 16) return false;
  Dense V{P, P, std::vector<double>(g->V, g->V + (size_t)P * P)};
  Dense Vi{P, P, std::vector<double>(g->V_inv, g->V_inv + (size_t)P * P)};
  auto times = [&](const std::vector<double>& S) {  // V (P x P) times S (P x G)
    Dense R{P, G, std::vector<double>((size_t)P * G, 0.0)};
    for (int j = 0; j < P; ++j)
      for (int n = 0; n < P; ++n) {
        const double v = V.at(j, n);
        if (v == 0.0) continue;
        for (int k = 0; k < G; ++k) R.a[(size_t)j * G + k] += v * S[(size_t)n * G + k];
      }
    return R;
  };
  std::vector<double> Sd((size_t)P * G, 0.0);  // -T_g + T_{g+2}
  for (int k = 0; k < G; ++k) {
    Sd[(size_t)k * G + k] = -1.0;
    Sd[(size_t)(k + 2) * G + k] = 1.0;
  }
  // explicit-tendency forms: E_q = -V^-1 A_q; E_g = pinv_dir(-V^-1 A_g) with
  // pinv_dir[g][n] = -1 for n <= g, n = g mod 2 (x_n = x_{n-2} - c_n), so
  // -pinv_dir V^-1 sums the rows of V^-1 of g's parity up to g
  Dense Eq{P, P, std::vector<double>((size_t)P * P)};
  for (size_t i = 0; i < Eq.a.size(); ++i) Eq.a[i] = -Vi.a[i];
  Dense Eg{G, P, std::vector<double>((size_t)G * P, 0.0)};
  for (int gg = 0; gg < G; ++gg)
    for (int n = gg & 1; n <= gg; n += 2)
      for (int j = 0; j < P; ++j) Eg.a[(size_t)gg * P + j] += Vi.at(n, j);
  const Dense mats[TC_IMAGES] = {
      V, times(std::vector<double>(g->w_stencil, g->w_stencil + (size_t)P * G)), times(Sd), Vi, Eq, Eg};
  for (int i = 0; i < TC_IMAGES; ++i) {
    const bool inv = i >= TC_INV;
    if (!mirror_ok(mats[i], N, inv)) return false;
    fold_image(mats[i], N, inv, img[i]);
  }
  return true;
}

size_t tc_vertical_smem(bool inverse) { return inverse ? tc_smem<true>() : tc_smem<false>(); }

namespace {
template <bool INV>
cudaError_t tc_launch(const TcArgs& a, int nf, cudaStream_t st) {
  const size_t sm = tc_smem<INV>();
  cudaError_t e = cudaFuncSetAttribute(k_tc_vertical<INV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sm);
  if (e != cudaSuccess) return e;
  dim3 grid((a.ncols + kCols - 1) / kCols, nf);
  k_tc_vertical<INV><<<grid, kThreads + 64, sm, st>>>(a);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_tc_to_nodal(const Params& p, const Tables& t, const Work& w, const double2* q,
                               const double2* wf, const double2* th, float2* qn, float2* wn,
                               float2* tn, cudaStream_t st) {
  if (!t.tc.img[0]) return cudaErrorInvalidValue;
  TcArgs a{};
  a.ncols = 2 * p.d.M;
  a.N = p.d.Nz;
  a.H = p.d.Nz / 2;
  a.status = w.status;
  const double2* in[3] = {q, wf, th};
  float2* out[3] = {qn, wn, tn};
  int nf = 0;
  for (int i = 0; i < 3; ++i) {
    if (!in[i]) continue;
    TcField& f = a.f[nf++];
    f.in = in[i];
    f.out = reinterpret_cast<float*>(out[i]);
    f.img = t.tc.img[i];
    f.xrow = t.tc.xrow[i];
    f.K = t.tc.K[i];
    f.rows = t.tc.rows[i];
    f.nch = t.tc.nch[i];
  }
  if (nf == 0) return cudaSuccess;
  return tc_launch<false>(a, nf, st);
}

cudaError_t launch_tc_to_coef(const Params& p, const Tables& t, const Work& w, float2* aq,
                              float2* aw, float2* at, bool explicit_form, cudaStream_t st) {
  if (!t.tc.img[TC_INV]) return cudaErrorInvalidValue;
  TcArgs a{};
  a.ncols = 2 * p.d.M;
  a.N = p.d.Nz;
  a.H = p.d.Nz / 2;
  a.status = w.status;
  float2* io[3] = {aq, aw, at};
  int nf = 0;
  for (int i = 0; i < 3; ++i) {
    if (!io[i]) continue;
    TcField& f = a.f[nf++];
    f.in = io[i];
    f.out = reinterpret_cast<float*>(io[i]);
    const int im = !explicit_form ? TC_INV : (i == 0 ? TC_E_Q : TC_E_G);
    f.img = t.tc.img[im];
    f.xrow = t.tc.xrow[im];
    f.K = t.tc.K[im];
    f.rows = t.tc.rows[im];
    f.nch = t.tc.nch[im];
  }
  if (nf == 0) return cudaSuccess;
  return tc_launch<true>(a, nf, st);
}

}  // namespace nhqg

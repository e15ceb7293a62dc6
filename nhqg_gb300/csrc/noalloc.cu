// Allocation-free variant of the 2/3-rule triple advection.
//
// Some callers cannot allocate device memory themselves: an XLA FFI custom
// call must take every buffer from XLA's allocator, and hosts that run on a
// fixed device-memory pool forbid allocations outside it.
// nhqg_triple_advection_23_noalloc serves them: it creates no context and
// allocates nothing.  Its working storage (the FFT twiddle/permutation tables
// and the H1/H2 intermediates) lives in one file-scope __device__ array of
// NHQG_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds
// from module load until process exit.
//
// The host reaches that array only through the address that
// cudaGetSymbolAddress returns (the symbol's name in host code is a host-side
// stand-in, not a device address).  The first call on each device looks it up
// with that device current and keeps it for later calls; make that first call
// before any stream capture.  cudaDeviceReset destroys the context that holds
// the array, so after a reset the cached address is stale: do not call this
// entry point again in a process that reset the device.
// All calls share the array and it keeps the last call's contents, so calls
// that overlap on the GPU (other streams, other host threads on the same
// device) race on it and must be serialised by the caller.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "engine.h"
#include "nhqg_gpu.h"

using namespace nhqg;

namespace {

constexpr size_t kTableBytes = 64 * 1024;  // twiddles + permutation, Nx <= 2048
static __device__ __align__(256) unsigned char g_scratch[NHQG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// twiddles exp(-2 pi i k / n) and the digit-reversal permutation of the
// radix-4/2/3 decimation-in-frequency FFT, computed on the device
__global__ void k_noalloc_tables(FftPlan plan, double2* tw, int* perm) {
  const int n = plan.n;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)k / (double)n, &s, &c);
    tw[k] = make_double2(c, -s);
    int L = n, kk = k, pos = 0;
    for (int q = 0; q < plan.npass; ++q) {
      const int R = plan.radix[q];
      const int Ls = L / R;
      pos += (kk % R) * Ls;
      kk /= R;
      L = Ls;
    }
    perm[k] = pos;
  }
}

int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return NHQG_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return NHQG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_addr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || p == nullptr) return NHQG_ERR_CUDA;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return NHQG_OK;
}

}  // namespace

extern "C" int nhqg_triple_advection_23_noalloc(int advection, int Nx, int levels,
                                                const double* kx, const double* ky,
                                                const void* psi, const void* q, const void* w,
                                                const void* th, void* Aq, void* Aw, void* Ath,
                                                void* stream) {
  if (levels <= 0 || !kx || !ky || !psi || !q || !w || !th || !Aq || !Aw || !Ath)
    return NHQG_ERR_BAD_ARG;
  if (advection != NHQG_ADV_FLUX && advection != NHQG_ADV_JACOBIAN) return NHQG_ERR_UNSUPPORTED;
  if (Nx < 8 || Nx % 2 != 0 || Nx > 2048) return NHQG_ERR_UNSUPPORTED;
  const FftPlan plan = make_fft_plan(Nx);
  if (plan.npass <= 0) return NHQG_ERR_UNSUPPORTED;

  Params p{};
  p.d = make_dims(Nx, 4);
  p.plan = plan;
  const Dims& d = p.d;
  const int nf1 = advection == NHQG_ADV_JACOBIAN ? 8 : 5;
  const int ng = advection == NHQG_ADV_JACOBIAN ? 3 : 6;
  const size_t per_level =
      ((size_t)nf1 * d.Nk * d.Nx + (size_t)ng * d.Mc * d.Nx) * sizeof(double2);
  const size_t work_bytes = NHQG_NOALLOC_SCRATCH_BYTES - kTableBytes;
  const int chunk = (int)std::min<size_t>((size_t)levels, work_bytes / per_level);
  if (chunk < 1) return NHQG_ERR_SCRATCH_TOO_SMALL;
  {
    // the outputs are zeroed before any input is read: no output may overlap an input
    const size_t bytes = (size_t)levels * Nx * (Nx / 2 + 1) * 16;
    const char* ins[4] = {(const char*)psi, (const char*)q, (const char*)w, (const char*)th};
    const char* outs[3] = {(const char*)Aq, (const char*)Aw, (const char*)Ath};
    for (const char* o : outs)
      for (const char* i : ins)
        if (o < i + bytes && i < o + bytes) return NHQG_ERR_BAD_ARG;
  }

  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc != NHQG_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* b = static_cast<unsigned char*>(base);
  Tables t{};
  t.tw = reinterpret_cast<double2*>(b);
  t.perm = reinterpret_cast<int*>(b + (size_t)2048 * sizeof(double2));
  t.kx_full = const_cast<double*>(kx);
  t.ky_full = const_cast<double*>(ky);
  Work wk{};
  wk.x1 = reinterpret_cast<double2*>(b + kTableBytes);
  wk.x1_elems = (size_t)nf1 * chunk * d.Nk * d.Nx;
  wk.x2 = wk.x1 + wk.x1_elems;
  wk.x2_elems = (size_t)ng * chunk * d.Mc * d.Nx;

  // an error left pending by other code on this thread stays for its owner to read
  if (cudaPeekAtLastError() != cudaSuccess) return NHQG_ERR_CUDA;
  k_noalloc_tables<<<(Nx + 255) / 256, 256, 0, st>>>(plan, t.tw, t.perm);
  if (cudaGetLastError() != cudaSuccess) return NHQG_ERR_CUDA;
  const size_t plane = (size_t)d.Nx * d.Nk;
  const size_t bytes = (size_t)levels * plane * sizeof(double2);
  if (cudaMemsetAsync(Aq, 0, bytes, st) != cudaSuccess || cudaMemsetAsync(Aw, 0, bytes, st) != cudaSuccess ||
      cudaMemsetAsync(Ath, 0, bytes, st) != cudaSuccess)
    return NHQG_ERR_CUDA;
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
    if (launch_horizontal(p, t, wk, a, st, nullptr) != cudaSuccess) return NHQG_ERR_CUDA;
  }
  return NHQG_OK;
}

// Allocation-free spectral diagnostics: tg_diagnostics_noalloc (include/tgdns.h).
//
// Why: some callers cannot allocate device memory at the point where they want
// the energies -- a host framework that owns every device buffer and forbids
// cudaMalloc inside its custom-call / operator execution (an XLA FFI handler, a
// PyTorch operator under a caching allocator it must not bypass), or a real-time
// loop that runs with a fixed memory footprint.  tg_diagnostics needs a plan,
// and creating a plan allocates.  This entry point needs no plan: the only
// scratch is the block partial sums, held in the file-scope device array below.
//
// The array is part of the library image: every GPU that loads the library
// holds it (TG_NOALLOC_MAX_RUNS * 96 * 5 doubles = 240 KiB) until the process
// exits.  All calls share it and it keeps the previous call's contents; each
// call overwrites every slot it reads, so nothing needs clearing.  Calls that
// overlap on the GPU (different streams, or host threads racing on one device)
// race on the array and must be ordered by the caller.
//
// The array's device address is looked up (cudaGetSymbolAddress) on the first
// call in each CUDA context, with that context current, and cached under the
// context's unique id: a device reset, or a context other than the primary one,
// loads the module again at a new address, and the next call then looks it up
// again instead of handing a stale address to the kernels.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/tgdns.h"
#include "tg_common.cuh"

namespace tg {
void set_last_error(const std::string& message);  // tg_api.cu
bool size_built(int n, int prec);                  // tg_api.cu
}

namespace {

constexpr int kBlocks = 96;   // partial sums per run
constexpr int kThreads = 256;
constexpr int kQ = 5;         // E_k, enstrophy, sum w k^2 |u|^2, E_m, H_c
constexpr int kMaxContexts = 64;

static __device__ __align__(256) double g_partials[TG_NOALLOC_MAX_RUNS * kBlocks * kQ];

// host copies of the array's device address, one per CUDA context (keyed by the
// context's unique id), most recent first
std::mutex g_mu;
struct CtxAddr {
  unsigned long long id = 0;
  double* addr = nullptr;
};
CtxAddr g_addr[kMaxContexts];
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;


struct Comp {
  double s = 0.0, c = 0.0;
  __device__ void add(double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ double value() const { return s + c; }
};

template <typename R>
__global__ void __launch_bounds__(kThreads) partial_kernel(const tg::cplx<R>* S, tg::Geo g, int F, double* part) {
  using C = tg::cplx<R>;
  const int run = blockIdx.y;
  const C* base = S + (long long)run * F * g.sS;
  // the per-mode terms of tg_diagnostics (diag_terms), one (kx, ky) row per warp and pass
  double q[kQ] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const int lane = threadIdx.x & 31, nw = kThreads / 32;
  for (int r = blockIdx.x * nw + (threadIdx.x >> 5); r < g.M * g.M; r += gridDim.x * nw) {
    const int ix = r / g.M, iy = r - ix * g.M;
    const int kx = tg::ksigned(ix, g.K), ky = tg::ksigned(iy, g.K);
    for (int kz = lane; kz < g.Hk; kz += 32) {
      double t[kQ];
      tg::diag_terms(base, g.sS, (long long)r * g.Hz + kz, kx, ky, kz, F, t);
      for (int i = 0; i < kQ; ++i) q[i] += t[i];
    }
  }
  __shared__ double sh[kQ][kThreads];
  for (int i = 0; i < kQ; ++i) sh[i][threadIdx.x] = q[i];
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int i = 0; i < kQ; ++i) sh[i][threadIdx.x] += sh[i][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kQ) part[((long long)run * kBlocks + blockIdx.x) * kQ + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void final_kernel(const double* part, double nu, int F, double* out) {
  const int run = blockIdx.x;
  __shared__ double v[kQ];
  if (threadIdx.x < kQ) {
    Comp s;
    for (int b = 0; b < kBlocks; ++b) s.add(part[((long long)run * kBlocks + b) * kQ + threadIdx.x]);
    v[threadIdx.x] = s.value();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double* o = out + (long long)run * TG_DIAG_WIDTH;
    o[TG_D_KINETIC] = v[0];
    o[TG_D_ENSTROPHY] = v[1];
    o[TG_D_DISSIPATION] = nu * v[2];
    o[TG_D_MAGNETIC] = (F == 6) ? v[3] : 0.0;
    o[TG_D_CROSS_HELICITY] = (F == 6) ? v[4] : 0.0;
    o[TG_D_TOTAL] = v[0] + ((F == 6) ? v[3] : 0.0);
    o[TG_D_DIVU_MAX] = -1.0;  // not computed here (needs transform scratch)
    o[TG_D_DIVB_MAX] = -1.0;
  }
}

int fail(int code, const std::string& m) {
  tg::set_last_error(m);  // reported by tg_last_error()
  return code;
}

// the device address of g_partials in the current context (looked up once per context)
int partials_address(double** out) {
  cudaError_t e;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_ctx_current || !g_ctx_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void* f1 = nullptr;
    void* f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return fail(TG_E_CUDA, "tg_diagnostics_noalloc: the driver does not provide cuCtxGetCurrent / cuCtxGetId");
    g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_current(&ctx) != CUDA_SUCCESS)
    return fail(TG_E_CUDA, "tg_diagnostics_noalloc: cuCtxGetCurrent failed");
  if (!ctx) {  // no context yet: the runtime binds the device's primary context on this call
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess)
      return fail(TG_E_CUDA, std::string("tg_diagnostics_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx)
      return fail(TG_E_CUDA, "tg_diagnostics_noalloc: no current CUDA context");
  }
  if (g_ctx_id(ctx, &id) != CUDA_SUCCESS)
    return fail(TG_E_CUDA, "tg_diagnostics_noalloc: cuCtxGetId failed");
  for (int i = 0; i < kMaxContexts; ++i) {
    if (g_addr[i].addr && g_addr[i].id == id) {
      *out = g_addr[i].addr;
      return TG_OK;
    }
  }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_partials);
  if (e != cudaSuccess || !p)
    return fail(TG_E_CUDA, std::string("tg_diagnostics_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  for (int i = kMaxContexts - 1; i > 0; --i) g_addr[i] = g_addr[i - 1];  // oldest entry drops out
  g_addr[0].id = id;
  g_addr[0].addr = static_cast<double*>(p);
  *out = g_addr[0].addr;
  return TG_OK;
}

}  // namespace

extern "C" int tg_diagnostics_noalloc(const void* state, int n, int batch, int physics, int precision, double nu,
                                      double eta, double* out, void* stream) {
  (void)eta;
  if (!state || !out) return fail(TG_E_INVALID, "tg_diagnostics_noalloc: null argument");
  if (physics != TG_PHYS_HYDRO && physics != TG_PHYS_MHD)
    return fail(TG_E_INVALID, "tg_diagnostics_noalloc: physics must be TG_PHYS_HYDRO or TG_PHYS_MHD");
  if (precision != TG_PREC_F32 && precision != TG_PREC_F64)
    return fail(TG_E_INVALID, "tg_diagnostics_noalloc: precision must be TG_PREC_F32 or TG_PREC_F64");
  // only the sizes tg_plan_create accepts: their states are the only buffers laid out this way
  if (!tg::size_built(n, precision))
    return fail(TG_E_UNSUPPORTED, "tg_diagnostics_noalloc: grid size " + std::to_string(n) +
                                      " is not built for this precision");
  // there is no plan whose nu a negative value could select: nu is used as given
  if (!(nu >= 0.0)) return fail(TG_E_INVALID, "tg_diagnostics_noalloc: nu must be nonnegative");
  if (batch < 1 || batch > TG_NOALLOC_MAX_RUNS)
    return fail(TG_E_INVALID, "tg_diagnostics_noalloc: batch " + std::to_string(batch) +
                                  " is outside 1.." + std::to_string(TG_NOALLOC_MAX_RUNS) +
                                  " (the fixed size of its static scratch)");
  double* part = nullptr;
  int rc = partials_address(&part);
  if (rc) return rc;
  tg::Geo g{};
  g.n = n;
  g.K = n / 3;
  g.M = 2 * g.K + 1;
  g.Hk = g.K + 1;
  g.Hz = (g.Hk + 3) / 4 * 4;
  g.sS = (long long)g.M * g.M * g.Hz;
  const int F = physics == TG_PHYS_MHD ? 6 : 3;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  dim3 grid(kBlocks, batch);
  if (precision == TG_PREC_F64)
    partial_kernel<double><<<grid, kThreads, 0, st>>>(static_cast<const tg::cplx<double>*>(state), g, F, part);
  else
    partial_kernel<float><<<grid, kThreads, 0, st>>>(static_cast<const tg::cplx<float>*>(state), g, F, part);
  final_kernel<<<batch, 32, 0, st>>>(part, nu, F, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(TG_E_CUDA, std::string("tg_diagnostics_noalloc: launch: ") + cudaGetErrorString(e));
  return TG_OK;
}

// One (real type, grid size) instantiation of the pass kernels.  The build
// compiles this file once per supported pair with -DTG_REAL=float|double and
// -DTG_N=<n>, so the translation units compile in parallel.
#include "tg_kernels.cuh"

#ifndef TG_REAL
#error "define TG_REAL (float or double)"
#endif
#ifndef TG_N
#error "define TG_N"
#endif

#define TG_CAT2(a, b, c) a##_##b##_##c
#define TG_CAT(a, b, c) TG_CAT2(a, b, c)

namespace tg {
cudaError_t TG_CAT(launch, TG_REAL, TG_N)(int op, const PassArgs<TG_REAL>& a, int runs, cudaStream_t st) {
  return launch_pass<TG_REAL, TG_N>(op, a, runs, st);
}
}  // namespace tg

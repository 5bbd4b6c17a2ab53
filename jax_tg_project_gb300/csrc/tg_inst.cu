// One (real type, grid size) instantiation of the pass kernels.  The build
// compiles this file once per supported pair with -DTG_REAL=float|double and
// -DTG_N=<n>, so the translation units compile in parallel.
#include <type_traits>

#include "tg_kernels_reg.cuh"

#ifndef TG_REAL
#error "define TG_REAL (float or double)"
#endif
#ifndef TG_N
#error "define TG_N"
#endif

#define TG_CAT2(a, b, c) a##_##b##_##c
#define TG_CAT(a, b, c) TG_CAT2(a, b, c)

namespace tg {
// number of y-pass configurations the autotuner may choose among (FP32 plans)
int TG_CAT(yconfs, TG_REAL, TG_N)() { return std::is_same<TG_REAL, float>::value ? YConfCount<TG_N>::value : 1; }

cudaError_t TG_CAT(launch, TG_REAL, TG_N)(int op, const PassArgs<TG_REAL>& a, int runs, cudaStream_t st) {
  // a.variant: bit 0 selects the shared-memory z passes, bit 1 the shared-memory x passes
  const bool reg_z = (a.variant & 1) == 0, reg_x = (a.variant & 2) == 0;
  (void)reg_z;
  (void)reg_x;
  if constexpr (std::is_same<TG_REAL, float>::value && HasRegZHydro<TG_N>::value) {
    if (reg_z && op == OP_KZ_PROD_HD) return launch_kz_reg<TG_REAL, TG_N>(a, runs, st);
  }
  if constexpr (std::is_same<TG_REAL, float>::value && HasRegZ<TG_N>::value) {
    if (reg_z && op == OP_KZ_PROD_MHD) return launch_kz_reg_mhd<TG_REAL, TG_N>(a, runs, st);
    if (reg_z && op == OP_KZ_ADJ) return launch_kz_reg_adj<TG_REAL, TG_N>(a, runs, st);
    const bool tape = (a.flags & FLAG_TAPE) != 0;
    if (op == OP_KX_ADJ_LOAD)
      return tape ? launch_kx_reg_adj<TG_REAL, TG_N, KX_ADJ_LOAD_T>(a, runs, st)
                  : launch_kx_reg_adj<TG_REAL, TG_N, KX_ADJ_LOAD>(a, runs, st);
    if (op == OP_KX_ADJ_FWD)
      return tape ? launch_kx_reg_adj<TG_REAL, TG_N, KX_ADJ_FWD_T>(a, runs, st)
                  : launch_kx_reg_adj<TG_REAL, TG_N, KX_ADJ_FWD>(a, runs, st);
    if (op == OP_KX_NL_FWD) return launch_kx_reg_adj<TG_REAL, TG_N, KX_NL_FWD>(a, runs, st);
  }
  if constexpr (std::is_same<TG_REAL, float>::value && HasStashX<TG_N>::value) {
    // bit 2: the x stage with the state stashed in shared memory (unless bit 1 asks for the
    // shared-memory x pass)
    if (reg_x && (a.variant & 4) && op == OP_KX_STAGE3) return launch_kx_stash<TG_REAL, TG_N>(a, runs, st);
  }
  if constexpr (std::is_same<TG_REAL, float>::value && HasRegX<TG_N>::value) {
    if (reg_x) {
      if (op == OP_KX_STAGE3) return launch_kx_reg<TG_REAL, TG_N, KX_STAGE>(a, runs, st);
      if (op == OP_KX_LOAD3 && a.map == MAP_UW && a.nin == 3 && a.nout == 6)
        return launch_kx_reg<TG_REAL, TG_N, KX_LOAD>(a, runs, st);
    }
  }
  return launch_pass<TG_REAL, TG_N>(op, a, runs, st);
}
}  // namespace tg

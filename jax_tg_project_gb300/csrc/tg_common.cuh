// Shared definitions of the Taylor-Green pseudo-spectral kernels: geometry of
// the pruned half-spectrum layouts, per-size FFT plans and kernel arguments.
//
// Layouts (complex, kz innermost with a padded row stride Hz):
//   state S, accumulator A   [run][F][M][M][Hz]   kept modes only (compact)
//   X  (after inverse-x)     [run][G][N][M][Hz]   x physical, ky kept
//   Y  (after inverse-y)     [run][G][N][N][Hz]   x, y physical
//   Z  (forward-z output)    [run][F][N][N][Hz]
//   W  (after forward-y)     [run][F][N][M][Hz]   (aliases Y)
// with K the 2/3 cutoff, M = 2K+1 kept modes on a full axis (ordered
// 0..K, -K..-1), Hk = K+1 kept kz modes, F = 3 (hydro) or 6 (MHD) state
// fields and G = 2F transformed fields (u, curl u [, b, curl b]).
// Spectral values are Fourier coefficients: u(x) = sum_k c_k exp(i k.x).
#pragma once

#include <cstdint>

#include "tg_fft.cuh"

namespace tg {

struct Geo {
  int n, K, M, Hk, Hz;
  long long sS;  // complex elements per field, compact state: M*M*Hz
  long long sX;  // per field of X / W: N*M*Hz
  long long sY;  // per field of Y / Z: N*N*Hz
  long long sP;  // real elements per physical field: N^3
};

struct RunCoef {
  double nu, eta, dt;
  double lorentz;  // sign of j x b in the momentum equation (+1 physical)
};

// per-size FFT plan (radix sequence and threads per transform)
template <int N> struct PlanFor;
template <> struct PlanFor<8> { using T = FftPlan<8, 2, 4, 2>; };
template <> struct PlanFor<12> { using T = FftPlan<12, 1, 4, 3>; };
template <> struct PlanFor<16> { using T = FftPlan<16, 4, 4, 4>; };
template <> struct PlanFor<24> { using T = FftPlan<24, 2, 2, 12>; };
template <> struct PlanFor<32> { using T = FftPlan<32, 4, 8, 4>; };
template <> struct PlanFor<48> { using T = FftPlan<48, 4, 4, 12>; };
template <> struct PlanFor<64> { using T = FftPlan<64, 8, 8, 8>; };
template <> struct PlanFor<96> { using T = FftPlan<96, 8, 4, 4, 6>; };
template <> struct PlanFor<128> { using T = FftPlan<128, 8, 16, 8>; };
template <> struct PlanFor<256> { using T = FftPlan<256, 16, 16, 16>; };
template <> struct PlanFor<512> { using T = FftPlan<512, 64, 8, 8, 8>; };  // 64 threads a column (E = 8): occupancy
// the y pass keeps 16 threads a column at 512: its CTAs hold 16 columns, and 64 threads a
// column would make them 1024 threads wide (measured 1.15 ms against 0.78 ms at 512^3)
template <int N> struct YPlanFor { using T = typename PlanFor<N>::T; };
template <> struct YPlanFor<512> { using T = FftPlan<512, 16, 16, 32>; };

// y-pass configurations (radix plan, kz columns per CTA) that plan creation with
// TG_FLAG_AUTOTUNE times on the plan's own shape; configuration 0 is the default.  The
// column count sets the width of each CTA's row segments (8 bytes a column) and how many
// padding columns the last tile of a row carries.
template <int N> constexpr int ytile_default() { return (N >= 128) ? 16 : ((N >= 12) ? 8 : 4); }
template <int N, int I> struct YConf { using Plan = typename YPlanFor<N>::T; static constexpr int TZ = ytile_default<N>(); };
template <int N> struct YConfCount { static constexpr int value = 1; };
template <> struct YConfCount<32> { static constexpr int value = 4; };
template <> struct YConf<32, 1> { using Plan = PlanFor<32>::T; static constexpr int TZ = 4; };
template <> struct YConf<32, 2> { using Plan = PlanFor<32>::T; static constexpr int TZ = 12; };
template <> struct YConf<32, 3> { using Plan = FftPlan<32, 8, 4, 2, 4>; static constexpr int TZ = 8; };
template <> struct YConfCount<64> { static constexpr int value = 4; };
template <> struct YConf<64, 1> { using Plan = PlanFor<64>::T; static constexpr int TZ = 12; };
template <> struct YConf<64, 2> { using Plan = PlanFor<64>::T; static constexpr int TZ = 16; };
template <> struct YConf<64, 3> { using Plan = FftPlan<64, 16, 4, 4, 4>; static constexpr int TZ = 8; };
template <> struct YConfCount<96> { static constexpr int value = 4; };
template <> struct YConf<96, 1> { using Plan = PlanFor<96>::T; static constexpr int TZ = 12; };
template <> struct YConf<96, 2> { using Plan = PlanFor<96>::T; static constexpr int TZ = 16; };
template <> struct YConf<96, 3> { using Plan = FftPlan<96, 4, 8, 12>; static constexpr int TZ = 12; };
template <> struct YConfCount<128> { static constexpr int value = 3; };
template <> struct YConf<128, 1> { using Plan = PlanFor<128>::T; static constexpr int TZ = 12; };
template <> struct YConf<128, 2> { using Plan = FftPlan<128, 16, 8, 2, 8>; static constexpr int TZ = 16; };
template <> struct YConfCount<256> { static constexpr int value = 2; };
template <> struct YConf<256, 1> { using Plan = FftPlan<256, 32, 8, 4, 8>; static constexpr int TZ = 8; };
// the shared-memory x pass at 128 (the MHD stage, FP64 plans): 16 threads a column (E = 8),
// two 256-thread CTAs per SM in FP32.  Its grid is 85 x 3 CTAs at 128^3, so 8 threads a
// column left 7 warps per SM
template <int N> struct XPlanFor { using T = typename PlanFor<N>::T; static constexpr int MINB = 1; };
template <> struct XPlanFor<128> { using T = FftPlan<128, 16, 8, 2, 8>; static constexpr int MINB = 2; };

__host__ __device__ constexpr int kept_of(int n) { return n / 3; }

// columns (consecutive kz) per CTA of the x and y passes
template <typename R, int N, int F> struct TileZ {
  static constexpr int base = (N >= 128) ? 16 : ((N >= 12) ? 8 : 4);
  static constexpr int CS = ColLayout<N>::CS;
  static constexpr long long smem(int tz) {
    // twiddles + exchange columns + spectral column buffer (F fields, M <= 2*(N/3)+1 rows)
    return (long long)sizeof(cplx<R>) * (N + tz * CS + (long long)F * (2 * (N / 3) + 1) * tz);
  }
  static constexpr int value = (smem(base) <= 200 * 1024) ? base : base / 2;
};

// line pairs per CTA of the z pass: the largest power of two <= pref that divides
// the number of line pairs and keeps the CTA's shared memory (BUFS buffers of CS
// complex values per pair, plus the twiddles) under 200 KiB
template <typename R, int N, int BUFS = 7> struct LinesZ {
  static constexpr int P = PlanFor<N>::T::P;
  static constexpr int pref = (P >= 16) ? 8 : ((P >= 8) ? 16 : 32);
  static constexpr int pairs = N * N / 2;
  static constexpr long long bytes(int lp) {
    return (long long)sizeof(cplx<R>) * (N + (long long)lp * BUFS * ColLayout<N>::CS);
  }
  static constexpr int fit(int lp) {
    return (lp <= 1) ? 1 : ((pairs % lp == 0 && bytes(lp) <= 200 * 1024) ? lp : fit(lp / 2));
  }
  static constexpr int value = fit(pref);
};

enum KxMode { KX_STAGE = 0, KX_LOAD = 1, KX_FWD = 2, KX_ADJ_LOAD = 3, KX_ADJ_FWD = 4, KX_NL_FWD = 5,
              KX_ADJ_LOAD_T = 6, KX_ADJ_FWD_T = 7 };  // _T: the stage-tape forms (FLAG_TAPE)
enum FieldMap { MAP_ID = 0, MAP_UW = 1, MAP_UWBJ = 2, MAP_DIV = 3, MAP_DIVB = 4, MAP_CURL = 5, MAP_ADJ = 6 };
enum KzMode { KZ_PROD_HD = 0, KZ_PROD_MHD = 1, KZ_C2R = 2, KZ_R2C = 3, KZ_ADJ = 4 };
enum Flags { FLAG_EXPLICIT = 1, FLAG_RHS = 2, FLAG_AMAX = 4, FLAG_NONLIN = 8, FLAG_ADJ = 16,
             FLAG_TAPE = 32 };  // FLAG_TAPE: adjoint stage kernels read the step tape

template <typename R> struct PassArgs {
  Geo g;
  const cplx<R>* in;     // pass input (X, Y, Z or W)
  cplx<R>* out;          // pass output
  cplx<R>* S;            // state (KX_STAGE)
  cplx<R>* acc;          // RK4 accumulator
  cplx<R>* vs;           // stage state (explicit-viscosity RK4 only)
  const cplx<R>* spec_in;
  cplx<R>* spec_out;
  const R* phys_in;
  R* phys_out;
  const cplx<R>* tw;     // W_N^m, forward sign
  const RunCoef* coef;   // per run
  unsigned long long* amax;  // per (run, field) abs-max bit patterns
  int stage;             // 1..4
  int flags;
  int map;               // FieldMap for KX_LOAD
  int nin, nout;         // fields read / written by this pass
  int variant;           // 0: register-resident x/z passes where built, 1: shared-memory passes
  int yconf;             // y-pass configuration (YConf index, 0 = default)
  cplx<R>* tape;         // KX_STAGE (batch 1): the step tape [V, n1, n2, n3], or null
  const cplx<R>* tp[4];  // FLAG_TAPE adjoint stage kernels: the step tape V, n1, n2, n3
  cplx<R>* out2;         // KX_ADJ_LOAD_T with nout = 9: the three a = P mu fields (x-pass layout)
  double* part;          // KX_ADJ_FWD_T: per-CTA partial sums of d(loss)/d(nu) of the stage
  int tiles;             // tiles of a persistent or tile-indexed kernel (set by its launcher)
};

// The geometry a kernel works with: the plan's (runtime) or, for DEFK, that of the default
// 2/3 cutoff K = N/3 as compile-time constants, so that index and stride arithmetic and the
// kept / removed tests of mode slots fold (the launchers pick DEFK when the plan's K is N/3).
template <int N, bool DEFK>
__device__ __forceinline__ Geo geo_of(const Geo& g0) {
  if constexpr (!DEFK) {
    return g0;
  } else {
    constexpr int K = N / 3, M = 2 * K + 1, Hk = K + 1, Hz = (Hk + 3) / 4 * 4;
    Geo g;
    g.n = N;
    g.K = K;
    g.M = M;
    g.Hk = Hk;
    g.Hz = Hz;
    g.sS = (long long)M * M * Hz;
    g.sX = (long long)N * M * Hz;
    g.sY = (long long)N * N * Hz;
    g.sP = (long long)N * N * N;
    return g;
  }
}

// signed wavenumber of compact index i (0..M-1)
__device__ __forceinline__ int ksigned(int i, int K) { return i <= K ? i : i - (2 * K + 1); }
// compact index of full-axis frequency row k, or -1 when k is dealiased away
__device__ __forceinline__ int kcompact(int k, int N, int K) {
  return k <= K ? k : (k >= N - K ? k - N + 2 * K + 1 : -1);
}
// full-axis frequency row of compact index i
__device__ __forceinline__ int kfull(int i, int N, int K) { return i <= K ? i : i + N - (2 * K + 1); }

// Per-mode terms of the scalar diagnostics and the energy spectrum.  For FP32 states the
// products and their six-term sums are formed in FP32 (the precision the state itself
// carries, ~1e-7 relative per term) and widened to FP64 for accumulation; FP64 states use
// FP64 throughout.  The diagnostics, the allocation-free diagnostics and the spectrum share
// these, so that their per-mode terms agree bit for bit.
__device__ __forceinline__ float mode_sq(float2 a, float2 b, float2 c) {  // |a|^2 + |b|^2 + |c|^2
  float s = a.x * a.x;
  s = fmaf(a.y, a.y, s);
  s = fmaf(b.x, b.x, s);
  s = fmaf(b.y, b.y, s);
  s = fmaf(c.x, c.x, s);
  return fmaf(c.y, c.y, s);
}
__device__ __forceinline__ double mode_sq(double2 a, double2 b, double2 c) {
  return a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y;
}
__device__ __forceinline__ float mode_dot(float2 a, float2 b, float2 c, float2 p, float2 q, float2 r) {
  float s = a.x * p.x;  // Re(a conj p + b conj q + c conj r)
  s = fmaf(a.y, p.y, s);
  s = fmaf(b.x, q.x, s);
  s = fmaf(b.y, q.y, s);
  s = fmaf(c.x, r.x, s);
  return fmaf(c.y, r.y, s);
}
__device__ __forceinline__ double mode_dot(double2 a, double2 b, double2 c, double2 p, double2 q, double2 r) {
  return a.x * p.x + a.y * p.y + b.x * q.x + b.y * q.y + c.x * r.x + c.y * r.y;
}
// |k x u|^2 with complex components (k integer-valued, exact in either precision)
template <typename R, typename C>
__device__ __forceinline__ R mode_curl_sq(R kx, R ky, R kz, C ux, C uy, C uz) {
  const C cx = {ky * uz.x - kz * uy.x, ky * uz.y - kz * uy.y};
  const C cy = {kz * ux.x - kx * uz.x, kz * ux.y - kx * uz.y};
  const C cz = {kx * uy.x - ky * ux.x, kx * uy.y - ky * ux.y};
  return mode_sq(cx, cy, cz);
}
// the five diagnostic terms of compact mode o (weight w = 1 at kz = 0, else 2):
//   w/2 |u|^2, w/2 |k x u|^2, w |k|^2 |u|^2, and for F = 6 w/2 |b|^2, w Re(u . conj b)
template <typename C>
__device__ __forceinline__ void diag_terms(const C* base, long long sS, long long o, int kx, int ky, int kz,
                                           int F, double t[5]) {
  using R = decltype(C{}.x);
  const R hw = (kz == 0) ? R(0.5) : R(1);  // w / 2
  const R fx = R(kx), fy = R(ky), fz = R(kz);
  const C ux = base[o], uy = base[sS + o], uz = base[2 * sS + o];
  const R e2 = mode_sq(ux, uy, uz);
  t[0] = double(hw * e2);  // exact scalings by powers of two
  t[1] = double(hw * mode_curl_sq(fx, fy, fz, ux, uy, uz));
  t[2] = double((R(2) * hw * R(kx * kx + ky * ky + kz * kz)) * e2);
  if (F == 6) {
    const C bx = base[3 * sS + o], by = base[4 * sS + o], bz = base[5 * sS + o];
    t[3] = double(hw * mode_sq(bx, by, bz));
    t[4] = double(R(2) * hw * mode_dot(ux, uy, uz, bx, by, bz));
  } else {
    t[3] = t[4] = 0.0;
  }
}

// Slot q of a thread holds the modes k = t + P q (0 <= t < P).  Every dealiasing cutoff
// satisfies K <= N/3, so a slot lying wholly inside (N/3, N - N/3) only ever holds removed
// modes, and a slot with P q > N/3 never holds a kept non-negative kz: both tests are
// compile-time constants once the slot loops are unrolled.
template <int N, int P> __host__ __device__ constexpr bool slot_cut(int q) {
  return P * q > N / 3 && P * q + P - 1 < N - N / 3;
}
template <int N, int P> __host__ __device__ constexpr bool slot_past_k(int q) { return P * q > N / 3; }
// compact index of the mode of slot q of thread t (-1: removed), constant for cut slots
template <int N, int P> __device__ __forceinline__ int kcompact_slot(int t, int q, int K) {
  return slot_cut<N, P>(q) ? -1 : kcompact(t + P * q, N, K);
}


}  // namespace tg

// Pass kernels of the pseudo-spectral Taylor-Green step (templated on the
// real type R and the grid size N; instantiated per (R, N) in tg_inst_*.cu).
//
//   kx_kernel  x-direction column pass over one (ky, kz-tile): optional
//              forward-x of the nonlinear fields, the fused spectral pointwise
//              stage (1/N^3, 2/3 mask, Leray projection, curl for the
//              induction term, integrating factor, RK4 combine), and the
//              inverse-x of u, curl u (and b, curl b) for the next stage.
//   ky_kernel  y-direction column pass (inverse: kept ky rows -> all y;
//              forward: all y -> kept ky rows).
//   kz_kernel  z lines, two at a time packed as one complex transform:
//              C2R -> u x omega (+ j x b, u x b) -> R2C, or plain C2R / R2C.
#pragma once

#include <algorithm>
#include <initializer_list>
#include <type_traits>

#include "tg_common.cuh"

namespace tg {

// L2 eviction-priority hints (createpolicy + .L2::cache_hint): data read once and dead after it
// (evict_first), data the next pass reads back (evict_last).  The forward y pass reads Z with the
// first and writes W, which the x stage reads next, with the second (256^3 step 1.371 -> 1.358 ms,
// MHD 128^3 0.413 -> 0.403 ms).  The same evict_first loads for the x stage's inputs measured
// slower (x stage 118 -> 125 us), as L1::no_allocate loads had
__device__ __forceinline__ unsigned long long l2_policy_first() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long l2_policy_last() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float2 ld_l2hint(const float2* ptr, unsigned long long pol) {
  float2 v;
  asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(ptr), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ld_l2hint(const double2* ptr, unsigned long long) { return *ptr; }
__device__ __forceinline__ void st_l2hint(float2* ptr, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(ptr), "f"(v.x), "f"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_l2hint(double2* ptr, double2 v, unsigned long long) { *ptr = v; }

// ------------------------------------------------------------------ x pass
template <typename C>
__device__ __forceinline__ C curl_comp(int c, C vx, C vy, C vz, float kx, float ky, float kz) {
  using Re = decltype(C::x);
  C r;
  if (c == 0) r = mk<C>(Re(ky) * vz.x - Re(kz) * vy.x, Re(ky) * vz.y - Re(kz) * vy.y);
  else if (c == 1) r = mk<C>(Re(kz) * vx.x - Re(kx) * vz.x, Re(kz) * vx.y - Re(kx) * vz.y);
  else r = mk<C>(Re(kx) * vy.x - Re(ky) * vx.x, Re(kx) * vy.y - Re(ky) * vx.y);
  return cmul_i(r);  // i (k x v)_c
}

// value of transformed field gi at one kept mode from the spectral column buffer
template <typename C>
__device__ __forceinline__ C field_value(int map, int gi, const C* sb, int ic, int col, int M, int TZ,
                                         float kx, float ky, float kz) {
  using Re = decltype(C::x);
  auto V = [&](int f) -> C { return sb[(f * M + ic) * TZ + col]; };
  switch (map) {
    case MAP_ID:
      return V(gi);
    case MAP_UW:
    case MAP_UWBJ: {
      const int grp = gi / 3, c = gi % 3, base = (grp >= 2) ? 3 : 0;
      if ((grp & 1) == 0) return V(base + c);
      return curl_comp(c, V(base), V(base + 1), V(base + 2), kx, ky, kz);
    }
    case MAP_DIV: {  // gi = 0: div u, gi = 1: div b
      const int base = 3 * gi;
      C a = V(base), b = V(base + 1), c = V(base + 2);
      return cmul_i(mk<C>(Re(kx) * a.x + Re(ky) * b.x + Re(kz) * c.x,
                          Re(kx) * a.y + Re(ky) * b.y + Re(kz) * c.y));
    }
    case MAP_CURL:
      return curl_comp(gi % 3, V(3 * (gi / 3)), V(3 * (gi / 3) + 1), V(3 * (gi / 3) + 2), kx, ky, kz);
    case MAP_ADJ: {  // u, curl u of the state (fields 0..2) and the projected adjoint field (3..5)
      if (gi < 3) return V(gi);
      if (gi < 6) return curl_comp(gi - 3, V(0), V(1), V(2), kx, ky, kz);
      C a = V(3), b = V(4), c = V(5);
      const float k2 = kx * kx + ky * ky + kz * kz;
      if (k2 > 0.f) {
        const Re ik2 = Re(1) / Re(k2);
        const Re dx = (Re(kx) * a.x + Re(ky) * b.x + Re(kz) * c.x) * ik2;
        const Re dy = (Re(kx) * a.y + Re(ky) * b.y + Re(kz) * c.y) * ik2;
        const Re kc = (gi == 6) ? Re(kx) : ((gi == 7) ? Re(ky) : Re(kz));
        const C v = (gi == 6) ? a : ((gi == 7) ? b : c);
        return mk<C>(v.x - kc * dx, v.y - kc * dy);
      }
      return (gi == 6) ? a : ((gi == 7) ? b : c);
    }
    default:
      return czero<C>();
  }
}

template <typename C>
__device__ __forceinline__ void leray(C& a, C& b, C& c, float kx, float ky, float kz, float k2) {
  using Re = decltype(C::x);
  if (k2 > 0.f) {
    const Re ik2 = Re(1) / Re(k2);
    const Re dx = (Re(kx) * a.x + Re(ky) * b.x + Re(kz) * c.x) * ik2;
    const Re dy = (Re(kx) * a.y + Re(ky) * b.y + Re(kz) * c.y) * ik2;
    a = mk<C>(a.x - Re(kx) * dx, a.y - Re(kx) * dy);
    b = mk<C>(b.x - Re(ky) * dx, b.y - Re(ky) * dy);
    c = mk<C>(c.x - Re(kz) * dx, c.y - Re(kz) * dy);
  }
}

template <typename R> __device__ __forceinline__ R rexpm1(R x);
template <> __device__ __forceinline__ float rexpm1<float>(float x) { return expm1f(x); }
template <> __device__ __forceinline__ double rexpm1<double>(double x) { return expm1(x); }
// expm1(a + b) from x = expm1(a) and y = expm1(b): x + y + x y, an exact identity (the terms
// share a sign, so the two roundings stay within a few ulps of the result)
template <typename R> __device__ __forceinline__ R expm1_add(R x, R y) { return fma(x, y, x + y); }

// One RK4 stage for one component: n is the (projected) nonlinear tendency,
// s the state at the start of the step, lin = nu k^2, h the step.  Returns the
// next stage state (the new state after stage 4).
//
// The integrating factors E(t) = exp(-lin t) are applied to the state in delta
// form s + expm1(-lin t) s: for the small lin*h of a DNS step, E rounded to the
// working precision would bias the viscous decay (e.g. 1 - 1.9e-6 in FP32 is
// only 31 ulps below 1), while expm1 keeps the decrement to full precision.
// Lawson (integrating-factor) RK4 stage with the factors given as m1 = expm1(-lin h) and
// mh = expm1(-lin h / 2)
template <typename C>
__device__ __forceinline__ C lawson_combine(int stage, C n, C s, C& acc, decltype(C::x) h, decltype(C::x) m1,
                                            decltype(C::x) mh) {
  using Re = decltype(C::x);
  const Re e1 = Re(1) + m1, eh = Re(1) + mh;
  if (stage == 1) {  // acc = E1 n;  v = E(h/2)(s + h/2 n)
    acc = mk<C>(e1 * n.x, e1 * n.y);
    return mk<C>(s.x + (mh * s.x + eh * Re(0.5) * h * n.x), s.y + (mh * s.y + eh * Re(0.5) * h * n.y));
  }
  if (stage == 2) {  // acc += 2 E(h/2) n;  v = E(h/2) s + h/2 n
    acc = mk<C>(acc.x + Re(2) * eh * n.x, acc.y + Re(2) * eh * n.y);
    return mk<C>(s.x + (mh * s.x + Re(0.5) * h * n.x), s.y + (mh * s.y + Re(0.5) * h * n.y));
  }
  if (stage == 3) {  // acc += 2 E(h/2) n;  v = E(h) s + h E(h/2) n
    acc = mk<C>(acc.x + Re(2) * eh * n.x, acc.y + Re(2) * eh * n.y);
    return mk<C>(s.x + (m1 * s.x + h * eh * n.x), s.y + (m1 * s.y + h * eh * n.y));
  }
  const Re h6 = h / Re(6);  // s' = E(h) s + h/6 (acc + n)
  return mk<C>(s.x + (m1 * s.x + h6 * (acc.x + n.x)), s.y + (m1 * s.y + h6 * (acc.y + n.y)));
}

template <typename C>
__device__ __forceinline__ C rk4_combine(int stage, bool expl, C n, C s, C& acc, C vs, decltype(C::x) h,
                                         decltype(C::x) lin) {
  using Re = decltype(C::x);
  if (expl) {  // classical RK4 with explicit viscosity: k = N - nu k^2 v_stage
    const C k = mk<C>(n.x - lin * vs.x, n.y - lin * vs.y);
    if (stage == 1) { acc = k; return mk<C>(s.x + Re(0.5) * h * k.x, s.y + Re(0.5) * h * k.y); }
    if (stage == 2) { acc = mk<C>(acc.x + Re(2) * k.x, acc.y + Re(2) * k.y);
                      return mk<C>(s.x + Re(0.5) * h * k.x, s.y + Re(0.5) * h * k.y); }
    if (stage == 3) { acc = mk<C>(acc.x + Re(2) * k.x, acc.y + Re(2) * k.y);
                      return mk<C>(s.x + h * k.x, s.y + h * k.y); }
    const Re h6 = h / Re(6);
    return mk<C>(s.x + h6 * (acc.x + k.x), s.y + h6 * (acc.y + k.y));
  }
  return lawson_combine<C>(stage, n, s, acc, h, rexpm1<Re>(-lin * h), rexpm1<Re>(Re(-0.5) * lin * h));
}

template <typename R, int N, int F, int MODE, bool DEFK = false>
__global__ void __launch_bounds__(XPlanFor<N>::T::P * TileZ<R, N, F>::value, (sizeof(R) == 4) ? XPlanFor<N>::MINB : 1)
kx_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Plan = typename XPlanFor<N>::T;
  constexpr int P = Plan::P, TZ = TileZ<R, N, F>::value, CS = ColLayout<N>::CS, NT = P * TZ;
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, M = g.M, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* xb = tw + N;
  C* sb = xb + TZ * CS;  // [F][M][TZ]
  const int col = threadIdx.x % TZ, t = threadIdx.x / TZ;
  const int iyc = blockIdx.x, z0 = blockIdx.y * TZ, run = blockIdx.z;
  const int kz = z0 + col;
  const bool zok = kz < g.Hk;
  C* xcol = xb + col * CS;
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, NT);
  const float kyf = float(ksigned(iyc, K)), kzf = float(kz);

  if constexpr (MODE == KX_LOAD) {
    const C* sin_ = a.spec_in + (long long)run * a.nin * g.sS;
    for (int idx = threadIdx.x; idx < a.nin * M * TZ; idx += NT) {
      const int c = idx % TZ, ic = (idx / TZ) % M, f = idx / (TZ * M);
      C v = czero<C>();
      if (z0 + c < g.Hk) v = sin_[f * g.sS + ((long long)ic * M + iyc) * Hz + z0 + c];
      sb[(f * M + ic) * TZ + c] = v;
    }
    __syncthreads();
  } else {
    __syncthreads();  // twiddles
    const R inv_n3 = R(1) / (R(N) * R(N) * R(N));
    const C* win = a.in + (long long)run * a.nin * g.sX + (long long)iyc * Hz + kz;
    for (int f = 0; f < a.nin; ++f) {
      const C* wf = win + f * g.sX;
      auto src = [&](int x, int) -> C { return zok ? wf[(long long)x * M * Hz] : czero<C>(); };
      auto dst = [&](int b, int r, int k, C v) {
        if (slot_cut<N, P>(out_slot<Plan>(b, r))) return;  // always-removed modes
        const int ic = kcompact(k, N, K);
        if (ic >= 0) sb[(f * M + ic) * TZ + col] = cscale(v, inv_n3);
      };
      fft_column<Plan, -1>(t, src, dst, xcol, tw);
    }
    __syncthreads();

    // ---- fused spectral pointwise stage
    const RunCoef cf = a.coef[run];
    const long long soff = (long long)run * F * g.sS;
    for (int idx = threadIdx.x; idx < M * TZ; idx += NT) {
      const int c = idx % TZ, ic = idx / TZ;
      if (z0 + c >= g.Hk) continue;
      const float kx = float(ksigned(ic, K));
      const float k2 = kx * kx + kyf * kyf + kzf * kzf;
      const long long m0 = ((long long)ic * M + iyc) * Hz + z0 + c;
      C n[F];
#pragma unroll
      for (int f = 0; f < F; ++f) n[f] = sb[(f * M + ic) * TZ + c];
      if constexpr (MODE == KX_FWD && F == 6) {
        if (a.flags & FLAG_ADJ) {  // adjoint nonlinear term: F(omega x a) + i k x F(a x u)
          C* so = a.spec_out + (long long)run * 3 * g.sS;
#pragma unroll
          for (int f = 0; f < 3; ++f) {
            const C cq = curl_comp(f, n[3], n[4], n[5], kx, kyf, kzf);
            so[f * g.sS + m0] = mk<C>(n[f].x + cq.x, n[f].y + cq.y);
          }
          continue;
        }
      }
      if constexpr (F == 6) {  // induction: i k x F(u x b), then projection (as the reference)
        C ex = n[3], ey = n[4], ez = n[5];
        n[3] = curl_comp(0, ex, ey, ez, kx, kyf, kzf);
        n[4] = curl_comp(1, ex, ey, ez, kx, kyf, kzf);
        n[5] = curl_comp(2, ex, ey, ez, kx, kyf, kzf);
        leray(n[3], n[4], n[5], kx, kyf, kzf, k2);
      }
      leray(n[0], n[1], n[2], kx, kyf, kzf, k2);
      if constexpr (MODE == KX_FWD) {
        C* so = a.spec_out + soff;
        if (a.flags & (FLAG_RHS | FLAG_NONLIN)) {  // RHS = P N - nu k^2 v (v from spec_in); P N alone
          const C* vi = a.spec_in + soff;
          const bool visc = (a.flags & FLAG_NONLIN) == 0;
#pragma unroll
          for (int f = 0; f < F; ++f) {
            if (!visc) {
              so[f * g.sS + m0] = n[f];
              continue;
            }
            const R lin = R((f < 3 ? cf.nu : cf.eta) * double(k2));
            const C v = vi[f * g.sS + m0];
            so[f * g.sS + m0] = mk<C>(n[f].x - lin * v.x, n[f].y - lin * v.y);
          }
        } else {
          // plain forward transform: masked coefficients (no projection)
#pragma unroll
          for (int f = 0; f < F; ++f) so[f * g.sS + m0] = sb[(f * M + ic) * TZ + c];
        }
      } else {  // KX_STAGE
        const bool expl = (a.flags & FLAG_EXPLICIT) != 0;
        const R h = R(cf.dt);
        // the state, accumulator (and stage-state) arrays are distinct, and all loads of the
        // mode are issued before its arithmetic and stores
        C* __restrict__ Sp = a.S;
        C* __restrict__ Ap = a.acc;
        C* __restrict__ Vp = a.vs;
        C sv[F], av[F];
#pragma unroll
        for (int f = 0; f < F; ++f) {
          const long long o = soff + f * g.sS + m0;
          sv[f] = Sp[o];
          av[f] = (a.stage > 1) ? Ap[o] : czero<C>();
        }
#pragma unroll
        for (int f = 0; f < F; ++f) {
          const double visc = (f < 3) ? cf.nu : cf.eta;
          const R lin = R(visc * double(k2));
          const long long o = soff + f * g.sS + m0;
          const C s = sv[f];
          C acc = av[f];
          const C vs = (expl && a.stage > 1) ? Vp[o] : s;
          const C v = rk4_combine<C>(a.stage, expl, n[f], s, acc, vs, h, lin);
          if (a.stage < 4) {
            Ap[o] = acc;
            if (expl) Vp[o] = v;
          } else {
            Sp[o] = v;
          }
          sb[(f * M + ic) * TZ + c] = v;
        }
      }
    }
    __syncthreads();
  }

  if constexpr (MODE != KX_FWD) {
    // ---- inverse-x of the fields the next pass needs
    const int map = (MODE == KX_STAGE) ? (F == 6 ? MAP_UWBJ : MAP_UW) : a.map;
    C* xo = a.out + (long long)run * a.nout * g.sX + (long long)iyc * Hz + kz;
    for (int gi = 0; gi < a.nout; ++gi) {
      auto src = [&](int k, int q) -> C {
        if (slot_cut<N, P>(q)) return czero<C>();  // always-removed modes
        const int ic = kcompact(k, N, K);
        if (!zok || ic < 0) return czero<C>();
        return field_value<C>(map, gi, sb, ic, col, M, TZ, float(ksigned(ic, K)), kyf, kzf);
      };
      C* xg = xo + gi * g.sX;
      auto dst = [&](int, int, int x, C v) {  // padding columns (kz >= Hk) get the zeros they hold
        if (kz < Hz) xg[(long long)x * M * Hz] = v;
      };
      fft_column<Plan, +1>(t, src, dst, xcol, tw);
    }
  }
}

// ------------------------------------------------------------------ y pass
template <typename R, int N, int DIR, int YC, bool DEFK = false>
__global__ void __launch_bounds__(YConf<N, YC>::Plan::P * YConf<N, YC>::TZ)
ky_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Plan = typename YConf<N, YC>::Plan;
  constexpr int P = Plan::P, TZ = YConf<N, YC>::TZ, CS = ColLayout<N>::CS, NT = P * TZ, E = Plan::E;
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, M = g.M, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* xb = tw + N;
  const int col = threadIdx.x % TZ, t = threadIdx.x / TZ;
  const int z0 = blockIdx.x * TZ, x = blockIdx.y;
  const int f = blockIdx.z % a.nin, run = blockIdx.z / a.nin;
  const int kz = z0 + col;
  const bool zok = kz < g.Hk;
  C* xcol = xb + col * CS;
  // the column's inputs (first pass of thread t: index t + P q into slot q) are loaded before
  // the twiddle table is built, so that the two global round trips overlap
  C pre[E];
  if constexpr (DIR > 0) {
    const C* in = a.in + ((long long)run * a.nin + f) * g.sX + (long long)x * M * Hz + kz;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      const int ic = slot_cut<N, P>(q) ? -1 : kcompact(t + P * q, N, K);  // always-removed rows
      pre[q] = (zok && ic >= 0) ? in[(long long)ic * Hz] : czero<C>();
    }
  } else {
    const C* in = a.in + ((long long)run * a.nin + f) * g.sY + (long long)x * N * Hz + kz;
    const unsigned long long pf = l2_policy_first();
#pragma unroll
    for (int q = 0; q < E; ++q) pre[q] = zok ? ld_l2hint(in + (long long)(t + P * q) * Hz, pf) : czero<C>();
  }
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, NT);
  __syncthreads();
  auto src = [&](int, int q) -> C { return pre[q]; };
  if constexpr (DIR > 0) {
    C* out = a.out + ((long long)run * a.nin + f) * g.sY + (long long)x * N * Hz + kz;
    auto dst = [&](int, int, int y, C v) {  // padding columns (kz >= Hk) get the zeros they hold
      if (kz < Hz) out[(long long)y * Hz] = v;
    };
    fft_column<Plan, +1, 4, true, 0, true>(t, src, dst, xcol, tw);  // twiddle powers in registers
  } else {
    C* out = a.out + ((long long)run * a.nin + f) * g.sX + (long long)x * M * Hz + kz;
    const unsigned long long pl = l2_policy_last();
    auto dst = [&](int b, int r, int k, C v) {
      if (slot_cut<N, P>(out_slot<Plan>(b, r))) return;  // always-removed rows
      const int ic = kcompact(k, N, K);
      if (kz < Hz && ic >= 0) st_l2hint(out + (long long)ic * Hz, v, pl);  // zeros in the padding columns
    };
    fft_column<Plan, -1, 4, true, 0, true>(t, src, dst, xcol, tw);
  }
}

// ------------------------------------------------------------------ z pass
template <typename R, int N, int MODE>
struct KzShape {
  using Plan = typename PlanFor<N>::T;
  static constexpr int P = Plan::P;
  static constexpr int CS = ColLayout<N>::CS;
  // accumulate the cross products in registers (float) or shared memory (double)
  static constexpr bool ACC_REG = sizeof(R) == 4;
  static constexpr int NPH = (MODE == KZ_PROD_HD) ? 3 : ((MODE == KZ_PROD_MHD || MODE == KZ_ADJ) ? 6 : 0);
  static constexpr int NACC = (MODE == KZ_C2R || MODE == KZ_R2C || ACC_REG) ? 0 : 3;
  static constexpr int BUFS = NPH + NACC + 1;  // + exchange column
  static constexpr int LP = LinesZ<R, N, BUFS>::value;
  static constexpr long long smem = (long long)sizeof(cplx<R>) * (N + (long long)LP * BUFS * CS);
};

template <typename R, int N, int MODE, bool DEFK = false>
__global__ void __launch_bounds__(KzShape<R, N, MODE>::P * KzShape<R, N, MODE>::LP)
kz_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Sh = KzShape<R, N, MODE>;
  using Plan = typename Sh::Plan;
  constexpr int P = Sh::P, LP = Sh::LP, CS = Sh::CS, NT = P * LP, E = Plan::E;
  constexpr int RL = Plan::template radix<Plan::NPASS - 1>();
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  const int t = threadIdx.x % P, lp = threadIdx.x / P;
  C* pbuf = tw + N + (long long)lp * Sh::BUFS * CS;
  C* xcol = pbuf + (Sh::BUFS - 1) * CS;
  const int pair = blockIdx.x * LP + lp, run = blockIdx.y;
  const int x = pair / (N / 2), y0 = 2 * (pair % (N / 2));
  const long long row0 = ((long long)x * N + y0) * Hz;  // row (x, y0); row (x, y0+1) is + Hz
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, NT);
  __syncthreads();
  // after the twiddles, a pair's buffers are private to its P threads: when they lie in one
  // warp (P divides 32) the exchanges and buffer hand-overs need only a warp barrier
  using ZSync = typename std::conditional<(P <= 32 && 32 % P == 0), WarpSync, CtaSync>::type;
  const ZSync zsync;

  // Hermitian packing of rows (x,y0) and (x,y0+1) of one spectral field: Z = A + iB
  auto packed = [&](const C* fld) {
    return [=](int k, int q) -> C {
      if (slot_cut<N, Plan::P>(q)) return czero<C>();  // always-removed modes
      if (k <= K) {
        C A = fld[row0 + k], B = fld[row0 + Hz + k];
        if (k == 0) { A.y = 0; B.y = 0; }
        return mk<C>(A.x - B.y, A.y + B.x);
      }
      if (k >= N - K) {
        const C A = fld[row0 + (N - k)], B = fld[row0 + Hz + (N - k)];
        return mk<C>(A.x + B.y, B.x - A.y);
      }
      return czero<C>();
    };
  };
  // unpack Z (in shared memory, natural order) into rows (x,y0) and (x,y0+1), kz <= K
  auto unpack_store = [&](const C* zb, C* outf) {
    for (int k = t; k < Hz; k += P) {
      if (k > K) {  // the rows' padding: whole 32-byte sectors written, no read-modify-write
        outf[row0 + k] = czero<C>();
        outf[row0 + Hz + k] = czero<C>();
        continue;
      }
      const C zk = zb[padx(k)];
      const C zm = zb[padx((N - k) % N)];
      const C A = mk<C>((zk.x + zm.x) * R(0.5), (zk.y - zm.y) * R(0.5));
      const C B = mk<C>((zk.y + zm.y) * R(0.5), (zm.x - zk.x) * R(0.5));
      outf[row0 + k] = A;
      outf[row0 + Hz + k] = B;
    }
  };

  if constexpr (MODE == KZ_ADJ) {
    // adjoint of u x omega: inputs u (0..2), omega (3..5), a (6..8); outputs
    // p = omega x a (0..2) and q = a x u (3..5)
    const C* yin = a.in + (long long)run * 9 * g.sY;
    C* zout = a.out + (long long)run * 6 * g.sY;
    C* ph = pbuf;  // u (0..2), a (3..5)
    C zr[E];
    C mr[Sh::ACC_REG ? 3 : 1][Sh::ACC_REG ? E : 1];
    auto dst_reg = [&](int b, int r, int, C v) { zr[b * RL + r] = v; };
    auto pt = [&](int e) { return out_index<Plan>(t, e / RL, e % RL); };
    auto macc = [&](int c, int e) -> C& {
      if constexpr (Sh::ACC_REG) return mr[c][e];
      else return pbuf[(Sh::NPH + c) * CS + padx(pt(e))];
    };
    for (int c = 0; c < 6; ++c) {
      const int fi = (c < 3) ? c : 3 + c;  // u -> 0..2, a -> 6..8
      auto src = packed(yin + fi * g.sY);
      fft_column<Plan, +1>(t, src, dst_reg, xcol, tw, zsync);
#pragma unroll
      for (int e = 0; e < E; ++e) ph[c * CS + padx(pt(e))] = zr[e];
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
#pragma unroll
      for (int c = 0; c < 3; ++c) macc(c, e) = czero<C>();
    }
#pragma unroll
    for (int w = 0; w < 3; ++w) {  // (omega x a)_{w+1} -= omega_w a_{w+2};  (omega x a)_{w+2} += omega_w a_{w+1}
      auto src = packed(yin + (3 + w) * g.sY);
      fft_column<Plan, +1>(t, src, dst_reg, xcol, tw, zsync);
      const int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = padx(pt(e));
        const C a1 = ph[(3 + c1) * CS + n], a2 = ph[(3 + c2) * CS + n];
        const C om = zr[e];
        C& p1 = macc(c1, e);
        C& p2 = macc(c2, e);
        p1 = mk<C>(p1.x - om.x * a2.x, p1.y - om.y * a2.y);
        p2 = mk<C>(p2.x + om.x * a1.x, p2.y + om.y * a1.y);
      }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {  // q = a x u into 3..5, p into 0..2
      const int n = padx(pt(e));
      const C ux = ph[n], uy = ph[CS + n], uz = ph[2 * CS + n];
      const C ax = ph[3 * CS + n], ay = ph[4 * CS + n], az = ph[5 * CS + n];
      ph[3 * CS + n] = mk<C>(ay.x * uz.x - az.x * uy.x, ay.y * uz.y - az.y * uy.y);
      ph[4 * CS + n] = mk<C>(az.x * ux.x - ax.x * uz.x, az.y * ux.y - ax.y * uz.y);
      ph[5 * CS + n] = mk<C>(ax.x * uy.x - ay.x * ux.x, ax.y * uy.y - ay.y * ux.y);
#pragma unroll
      for (int c = 0; c < 3; ++c) ph[c * CS + n] = macc(c, e);
    }
    zsync();
    for (int c = 0; c < 6; ++c) {
      C* pc = ph + c * CS;
      auto src = [&](int n, int) -> C { return pc[padx(n)]; };
      fft_column<Plan, -1>(t, src, dst_reg, xcol, tw, zsync);
      zsync();
#pragma unroll
      for (int e = 0; e < E; ++e) pc[padx(pt(e))] = zr[e];
      zsync();
      unpack_store(pc, zout + c * g.sY);
    }
  } else if constexpr (MODE == KZ_PROD_HD || MODE == KZ_PROD_MHD) {
    constexpr int F = (MODE == KZ_PROD_HD) ? 3 : 6;  // output fields
    const C* yin = a.in + (long long)run * (2 * F) * g.sY;
    C* zout = a.out + (long long)run * F * g.sY;
    C* ph = pbuf;  // [NPH][CS]: u (and b)
    C zr[E];
    C mr[Sh::ACC_REG ? 3 : 1][Sh::ACC_REG ? E : 1];
    auto dst_reg = [&](int b, int r, int, C v) { zr[b * RL + r] = v; };
    auto pt = [&](int e) { return out_index<Plan>(t, e / RL, e % RL); };
    auto macc = [&](int c, int e) -> C& {
      if constexpr (Sh::ACC_REG) return mr[c][e];
      else return pbuf[(Sh::NPH + c) * CS + padx(pt(e))];
    };
    // u (fields 0..2) and b (fields 6..8) to shared memory
    for (int c = 0; c < Sh::NPH; ++c) {
      const int fi = (c < 3) ? c : 3 + c;  // G order: u, omega, b, j
      auto src = packed(yin + fi * g.sY);
      fft_column<Plan, +1>(t, src, dst_reg, xcol, tw, zsync);
#pragma unroll
      for (int e = 0; e < E; ++e) ph[c * CS + padx(pt(e))] = zr[e];
    }
    // omega (fields 3..5): m = u x omega, one component at a time
#pragma unroll
    for (int e = 0; e < E; ++e) {
#pragma unroll
      for (int c = 0; c < 3; ++c) macc(c, e) = czero<C>();
    }
#pragma unroll
    for (int w = 0; w < 3; ++w) {
      auto src = packed(yin + (3 + w) * g.sY);
      fft_column<Plan, +1>(t, src, dst_reg, xcol, tw, zsync);
      // (u x omega): omega_x -> m_y += u_z w_x, m_z -= u_y w_x; cyclic
      const int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = padx(pt(e));
        const C u1 = ph[c1 * CS + n], u2 = ph[c2 * CS + n];  // u_{w+1}, u_{w+2}
        const C om = zr[e];
        // line 0 in .x, line 1 in .y (real lines packed)
        C& m1 = macc(c1, e);
        C& m2 = macc(c2, e);
        m1 = mk<C>(m1.x + u2.x * om.x, m1.y + u2.y * om.y);  // m_{w+1} += u_{w+2} w_w
        m2 = mk<C>(m2.x - u1.x * om.x, m2.y - u1.y * om.y);  // m_{w+2} -= u_{w+1} w_w
      }
    }
    if constexpr (MODE == KZ_PROD_MHD) {
      const R sl = R(a.coef[run].lorentz);
#pragma unroll
      for (int w = 0; w < 3; ++w) {  // j (fields 9..11): m += s (j x b)
        auto src = packed(yin + (9 + w) * g.sY);
        fft_column<Plan, +1>(t, src, dst_reg, xcol, tw, zsync);
        const int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int n = padx(pt(e));
          const C b1 = ph[(3 + c1) * CS + n], b2 = ph[(3 + c2) * CS + n];
          const C jw = zr[e];
          C& m1 = macc(c1, e);
          C& m2 = macc(c2, e);
          // (j x b)_{w+1} = j_{w+2} b_w - j_w b_{w+2};  (j x b)_{w+2} = j_w b_{w+1} - j_{w+1} b_w
          m1 = mk<C>(m1.x - sl * jw.x * b2.x, m1.y - sl * jw.y * b2.y);
          m2 = mk<C>(m2.x + sl * jw.x * b1.x, m2.y + sl * jw.y * b1.y);
        }
      }
      // e = u x b into fields 3..5, m into 0..2 (each thread owns its points)
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = padx(pt(e));
        const C ux = ph[n], uy = ph[CS + n], uz = ph[2 * CS + n];
        const C bx = ph[3 * CS + n], by = ph[4 * CS + n], bz = ph[5 * CS + n];
        ph[3 * CS + n] = mk<C>(uy.x * bz.x - uz.x * by.x, uy.y * bz.y - uz.y * by.y);
        ph[4 * CS + n] = mk<C>(uz.x * bx.x - ux.x * bz.x, uz.y * bx.y - ux.y * bz.y);
        ph[5 * CS + n] = mk<C>(ux.x * by.x - uy.x * bx.x, ux.y * by.y - uy.y * bx.y);
#pragma unroll
        for (int c = 0; c < 3; ++c) ph[c * CS + n] = macc(c, e);
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int n = padx(pt(e));
#pragma unroll
        for (int c = 0; c < 3; ++c) ph[c * CS + n] = macc(c, e);
      }
    }
    zsync();
    // forward transforms of the products
    for (int c = 0; c < F; ++c) {
      C* pc = ph + c * CS;
      auto src = [&](int n, int) -> C { return pc[padx(n)]; };
      fft_column<Plan, -1>(t, src, dst_reg, xcol, tw, zsync);
      zsync();
#pragma unroll
      for (int e = 0; e < E; ++e) pc[padx(pt(e))] = zr[e];
      zsync();
      unpack_store(pc, zout + c * g.sY);
    }
  } else if constexpr (MODE == KZ_C2R) {
    // spectral rows -> physical lines (optional output and/or abs-max per field)
    C zr[E];
    auto dst_reg = [&](int b, int r, int, C v) { zr[b * RL + r] = v; };
    for (int f = 0; f < a.nin; ++f) {
      auto src = packed(a.in + ((long long)run * a.nin + f) * g.sY);
      fft_column<Plan, +1>(t, src, dst_reg, xcol, tw, zsync);
      R m = 0;
      if (a.phys_out) {
        R* po = a.phys_out + ((long long)run * a.nin + f) * g.sP + ((long long)x * N + y0) * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int n = out_index<Plan>(t, e / RL, e % RL);
          po[n] = zr[e].x;
          po[N + n] = zr[e].y;
        }
      }
      if (a.flags & FLAG_AMAX) {
#pragma unroll
        for (int e = 0; e < E; ++e) m = fmax(m, fmax(fabs(zr[e].x), fabs(zr[e].y)));
        // warp max, then one atomic per warp (values are >= 0: bit order = value order)
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) {
          const unsigned long long bits = (sizeof(R) == 8)
              ? (unsigned long long)__double_as_longlong(double(m))
              : (unsigned long long)__double_as_longlong(double(m));
          atomicMax(a.amax + run * a.nin + f, bits);
        }
      }
    }
  } else {  // KZ_R2C: physical lines -> spectral rows kz <= K
    C zr[E];
    auto dst_reg = [&](int b, int r, int, C v) { zr[b * RL + r] = v; };
    for (int f = 0; f < a.nin; ++f) {
      const R* pi = a.phys_in + ((long long)run * a.nin + f) * g.sP + ((long long)x * N + y0) * N;
      auto src = [&](int n, int) -> C { return mk<C>(pi[n], pi[N + n]); };
      fft_column<Plan, -1>(t, src, dst_reg, xcol, tw, zsync);
      zsync();
#pragma unroll
      for (int e = 0; e < E; ++e) xcol[padx(out_index<Plan>(t, e / RL, e % RL))] = zr[e];
      zsync();
      unpack_store(xcol, a.out + ((long long)run * a.nin + f) * g.sY);
      zsync();
    }
  }
}

// ------------------------------------------------------------------ launcher
enum PassOp {
  OP_KX_STAGE3 = 0, OP_KX_STAGE6, OP_KX_LOAD3, OP_KX_LOAD6, OP_KX_FWD3, OP_KX_FWD6,
  OP_KY_INV, OP_KY_FWD, OP_KZ_PROD_HD, OP_KZ_PROD_MHD, OP_KZ_C2R, OP_KZ_R2C, OP_KZ_ADJ,
  OP_KX_ADJ_LOAD, OP_KX_ADJ_FWD, OP_KX_NL_FWD, OP_COUNT  // the last three: register-resident only
};

// the first of several CUDA results that is an error, else cudaSuccess
static inline cudaError_t first_error(std::initializer_list<cudaError_t> es) {
  for (cudaError_t e : es)
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

template <typename K>
static cudaError_t set_smem(K kernel, long long bytes) {
  if (bytes > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) (void)cudaGetLastError();  // report through the return code only
    return e;
  }
  return cudaSuccess;
}

template <typename R, int N, int F, int MODE>
static cudaError_t launch_kx(const PassArgs<R>& a, int runs, cudaStream_t st) {
  constexpr int TZ = TileZ<R, N, F>::value;
  constexpr int NT = XPlanFor<N>::T::P * TZ;
  const long long smem = TileZ<R, N, F>::smem(TZ);
  static cudaError_t attr = set_smem(kx_kernel<R, N, F, MODE>, smem);
  if (attr != cudaSuccess) return attr;
  dim3 grid(a.g.M, (a.g.Hk + TZ - 1) / TZ, runs);
  if constexpr (sizeof(R) == 4) {  // FP32 plans: the default cutoff's geometry at compile time
    static cudaError_t attr_d = set_smem(kx_kernel<R, N, F, MODE, true>, smem);
    if (attr_d != cudaSuccess) return attr_d;
    if (a.g.K == N / 3) {
      kx_kernel<R, N, F, MODE, true><<<grid, NT, smem, st>>>(a);
      return cudaGetLastError();
    }
  }
  kx_kernel<R, N, F, MODE><<<grid, NT, smem, st>>>(a);
  return cudaGetLastError();  // also clears a launch-configuration error
}

// resident CTAs of a kernel on the whole GPU (occupancy per SM times the SMs; once per
// process, on the device current at the first launch), or 0 if unknown
template <typename Kern>
static int resident_ctas(Kern kernel, int threads, long long smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, (size_t)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return sms * per_sm;
}

template <typename R, int N, int DIR, int YC>
static cudaError_t launch_ky_conf(const PassArgs<R>& a, int runs, cudaStream_t st) {
  constexpr int TZ = YConf<N, YC>::TZ;
  constexpr int NT = YConf<N, YC>::Plan::P * TZ;
  const long long smem = (long long)sizeof(cplx<R>) * (N + TZ * ColLayout<N>::CS);
  static cudaError_t attr = set_smem(ky_kernel<R, N, DIR, YC>, smem);
  if (attr != cudaSuccess) return attr;
  dim3 grid((a.g.Hk + TZ - 1) / TZ, N, runs * a.nin);
  if constexpr (sizeof(R) == 4) {  // FP32 plans: the default cutoff's geometry at compile time
    static cudaError_t attr_d = set_smem(ky_kernel<R, N, DIR, YC, true>, smem);
    if (attr_d != cudaSuccess) return attr_d;
    // a shared-memory carveout of 58 % (132 KB): fewer y CTAs per SM than the default and a
    // larger L1, which the columns' global loads need in flight (256^3 y 76.0 / 41.3 -> 74.7 /
    // 39.3 us, MHD 128^3 step 0.404 -> 0.380 ms; 100 % or 6 CTAs a SM: y 98 / 56 us)
    static cudaError_t attr_c = first_error(
        {cudaFuncSetAttribute(ky_kernel<R, N, DIR, YC, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 58),
         cudaFuncSetAttribute(ky_kernel<R, N, DIR, YC>, cudaFuncAttributePreferredSharedMemoryCarveout, 58)});
    if (attr_c != cudaSuccess) return attr_c;
    if (a.g.K == N / 3) {
      ky_kernel<R, N, DIR, YC, true><<<grid, NT, smem, st>>>(a);
      return cudaGetLastError();
    }
  }
  ky_kernel<R, N, DIR, YC><<<grid, NT, smem, st>>>(a);
  return cudaGetLastError();
}

// the y pass in configuration a.yconf (FP32 plans; FP64 plans use the default)
template <typename R, int N, int DIR, int YC = 0>
static cudaError_t launch_ky(const PassArgs<R>& a, int runs, cudaStream_t st) {
  if constexpr (YC + 1 < YConfCount<N>::value && sizeof(R) == 4) {
    if (a.yconf > YC) return launch_ky<R, N, DIR, YC + 1>(a, runs, st);
  }
  return launch_ky_conf<R, N, DIR, YC>(a, runs, st);
}

template <typename R, int N, int MODE>
static cudaError_t launch_kz(const PassArgs<R>& a, int runs, cudaStream_t st) {
  using Sh = KzShape<R, N, MODE>;
  static cudaError_t attr = set_smem(kz_kernel<R, N, MODE>, Sh::smem);
  if (attr != cudaSuccess) return attr;
  const int pairs = N * N / 2;
  dim3 grid((pairs + Sh::LP - 1) / Sh::LP, runs);
  if constexpr (sizeof(R) == 4) {  // FP32 plans: the default cutoff's geometry at compile time
    static cudaError_t attr_d = set_smem(kz_kernel<R, N, MODE, true>, Sh::smem);
    if (attr_d != cudaSuccess) return attr_d;
    if (a.g.K == N / 3) {
      kz_kernel<R, N, MODE, true><<<grid, Sh::P * Sh::LP, Sh::smem, st>>>(a);
      return cudaGetLastError();
    }
  }
  kz_kernel<R, N, MODE><<<grid, Sh::P * Sh::LP, Sh::smem, st>>>(a);
  return cudaGetLastError();
}

template <typename R, int N>
cudaError_t launch_pass(int op, const PassArgs<R>& a, int runs, cudaStream_t st) {
  switch (op) {
    case OP_KX_STAGE3: return launch_kx<R, N, 3, KX_STAGE>(a, runs, st);
    case OP_KX_STAGE6: return launch_kx<R, N, 6, KX_STAGE>(a, runs, st);
    case OP_KX_LOAD3: return launch_kx<R, N, 3, KX_LOAD>(a, runs, st);
    case OP_KX_LOAD6: return launch_kx<R, N, 6, KX_LOAD>(a, runs, st);
    case OP_KX_FWD3: return launch_kx<R, N, 3, KX_FWD>(a, runs, st);
    case OP_KX_FWD6: return launch_kx<R, N, 6, KX_FWD>(a, runs, st);
    case OP_KY_INV: return launch_ky<R, N, +1>(a, runs, st);
    case OP_KY_FWD: return launch_ky<R, N, -1>(a, runs, st);
    case OP_KZ_PROD_HD: return launch_kz<R, N, KZ_PROD_HD>(a, runs, st);
    case OP_KZ_PROD_MHD: return launch_kz<R, N, KZ_PROD_MHD>(a, runs, st);
    case OP_KZ_C2R: return launch_kz<R, N, KZ_C2R>(a, runs, st);
    case OP_KZ_R2C: return launch_kz<R, N, KZ_R2C>(a, runs, st);
    case OP_KZ_ADJ: return launch_kz<R, N, KZ_ADJ>(a, runs, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace tg

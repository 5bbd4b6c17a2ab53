// Register-resident x and z passes of the hydro step (FP32, N = 8 ... 256).
//
// With P = N/8 threads per transform (E = 8 values each), thread t of a column
// reads the inputs n = t (mod P) in the first pass and ends with the outputs
// k = t (mod P) after the last pass (see fft_pass).  Everything that is
// pointwise along the transformed axis therefore stays in the registers of the
// thread that owns those indices:
//
//   kz_reg_kernel  one z line pair per P threads: six inverse transforms of the
//                  Hermitian-packed rows (u, omega), u x omega in registers, three
//                  forward transforms read straight from those registers, and the
//                  Hermitian unpack Z(N-k) fetched from the partner lane by shuffle.
//   kx_reg_kernel  four consecutive kz columns per group of 4P threads: the three
//                  forward transforms, the fused 1/N^3 / Leray / RK4 stage and the
//                  six inverse transforms all keep the column in registers.
//
// Shared memory holds only the twiddle table and one exchange column per
// transform, so barriers are per warp (z) or per 4-column group (x, a named
// barrier), never CTA-wide inside the loops.  The z passes at N >= 128 use the
// XOR-swizzled exchange layout (no bank conflicts); the x and z passes form the twiddle
// powers in registers from one table read per butterfly (the x pass, whose four columns share
// each read, waits on the shared-memory queue more than on its arithmetic).
#pragma once

#include <algorithm>
#include <type_traits>

#include "tg_kernels.cuh"

namespace tg {

template <int N> struct RegPlan;
template <> struct RegPlan<8> { using T = FftPlan<8, 1, 8>; };
template <> struct RegPlan<16> { using T = FftPlan<16, 2, 8, 2>; };
template <> struct RegPlan<32> { using T = FftPlan<32, 4, 8, 4>; };
template <> struct RegPlan<64> { using T = FftPlan<64, 8, 8, 8>; };
template <> struct RegPlan<128> { using T = FftPlan<128, 16, 8, 2, 8>; };
template <> struct RegPlan<256> { using T = FftPlan<256, 32, 8, 4, 8>; };
template <> struct RegPlan<96> { using T = FftPlan<96, 8, 4, 4, 6>; };  // E = 12: x and hydro z passes

// sizes with a register-resident z pass (E = 8; N = 8 has fewer line pairs than one
// CTA holds) and with a register-resident x pass
template <int N> struct HasRegZ { static constexpr bool value = (N == 16 || N == 32 || N == 64 || N == 128 || N == 256); };
template <int N> struct HasRegX { static constexpr bool value = HasRegZ<N>::value || N == 96; };
// the hydro z pass also at N = 96 (E = 12, two CTAs per SM)
template <int N> struct HasRegZHydro { static constexpr bool value = HasRegZ<N>::value || N == 96; };

// 16-byte asynchronous global -> shared copy (L1 bypass) and its completion wait
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory"); }

// ------------------------------------------------------------------ z pass
template <typename R, int N>
struct KzRegShape {
  using Plan = typename RegPlan<N>::T;
  static constexpr int P = Plan::P, E = Plan::E;
  static constexpr int NT = 128;
  static constexpr int LP = NT / P;  // line pairs per CTA
  // exchange layout: XOR swizzle at N >= 128, padding below (bank-conflict model)
  static constexpr int PSH = (N >= 128) ? kSwizzle : (N >= 64) ? 4 : 3;
  static constexpr int CS = ColLayout<N, PSH, (N == 16) ? 2 : 4>::CS;
  static constexpr int HZMAX = ((N / 3 + 1) + 3) / 4 * 4;
  // per pair: exchange column + the two spectral rows of the six input fields
  static constexpr long long per_pair = CS + 6LL * 2 * HZMAX;
  static constexpr long long smem = (long long)sizeof(cplx<R>) * (N + (long long)LP * per_pair);
  // resident CTAs per SM the registers must allow: E = 12 holds 84 complex values a thread
  static constexpr int MINB = (E > 8) ? 2 : 3;
};

template <typename R, int N, bool DEFK = false>
__global__ void __launch_bounds__(128, KzRegShape<R, N>::MINB) kz_reg_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Sh = KzRegShape<R, N>;
  using Plan = typename Sh::Plan;
  constexpr int P = Sh::P, E = Sh::E, LP = Sh::LP, CS = Sh::CS;
  constexpr int NBL = N / (Plan::template radix<Plan::NPASS - 1>() * P);
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  const int t = threadIdx.x % P, lp = threadIdx.x / P;
  C* xcol = tw + N + lp * Sh::per_pair;
  C* stg = xcol + CS;  // [6][2][Hz]: rows (x, y0), (x, y0+1) of each input field
  const int pair = blockIdx.x * LP + lp, run = blockIdx.y;
  const int x = pair / (N / 2), y0 = 2 * (pair % (N / 2));
  const long long row0 = ((long long)x * N + y0) * Hz;
  const C* yin = a.in + (long long)run * 6 * g.sY;
  C* zout = a.out + (long long)run * 3 * g.sY;
  // stage the 2 x Hz contiguous values of every field (16-byte aligned: Hz % 4 == 0),
  // one commit group per field so that transform f waits only for its own rows
  {
    const int chunks = Hz;  // 2 * Hz complex = Hz 16-byte chunks
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const C* src = yin + f * g.sY + row0;
      C* dst = stg + f * 2 * Hz;
      for (int c = t; c < chunks; c += P) cp_async16(dst + 2 * c, src + 2 * c);
      cp_async_commit();
    }
  }
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, Sh::NT);
  __syncthreads();
  const WarpSync ws;
  // this thread's twiddles of passes 1.. in registers, shared by the nine transforms (where
  // every pass's butterflies of a thread share them), else formed per pass from the table
  constexpr bool TWR = twr_ok<Plan>();
  C wr[TWR ? TwrCount<Plan>::value : 1];
  if constexpr (TWR) load_twiddle_regs<Plan>(wr, tw, t);
  auto fftz = [&](auto& src, auto& dst, auto dir_tag) {
    constexpr int DIR = decltype(dir_tag)::value;
    if constexpr (TWR) fft_column_wr<Plan, DIR, Sh::PSH>(t, src, dst, xcol, wr, ws);
    else fft_column<Plan, DIR, Sh::PSH, true>(t, src, dst, xcol, tw, ws);
  };

  // Z = A + iB for rows (x, y0), (x, y0+1); kz > K is zero, kz < 0 by Hermitian symmetry
  auto packed = [&](const C* fld) {
    return [=](int k, int q) -> C {
      if (slot_cut<N, P>(q)) return czero<C>();
      if (k <= K) {
        C A = fld[k], B = fld[Hz + k];
        if (k == 0) { A.y = 0; B.y = 0; }
        return mk<C>(A.x - B.y, A.y + B.x);
      }
      if (k >= N - K) {
        const C A = fld[N - k], B = fld[Hz + (N - k)];
        return mk<C>(A.x + B.y, B.x - A.y);
      }
      return czero<C>();
    };
  };
  C u[3][E], m[3][E], z[E];
  auto inverse = [&](int f) {  // staged field f -> z (after waiting for its rows)
    switch (f) {  // 5 - f later commit groups may still be in flight
      case 0: cp_async_wait<5>(); break;
      case 1: cp_async_wait<4>(); break;
      case 2: cp_async_wait<3>(); break;
      case 3: cp_async_wait<2>(); break;
      case 4: cp_async_wait<1>(); break;
      default: cp_async_wait<0>(); break;
    }
    __syncwarp();
    auto src = packed(stg + f * 2 * Hz);
    auto dst = [&](int b, int r, int, C v) { z[b + r * NBL] = v; };
    fftz(src, dst, std::integral_constant<int, +1>());
  };
  auto inv_u = [&](auto c_tag) {
    constexpr int c = decltype(c_tag)::value;
    inverse(c);
#pragma unroll
    for (int q = 0; q < E; ++q) u[c][q] = z[q];
  };
  inv_u(std::integral_constant<int, 0>());
  inv_u(std::integral_constant<int, 1>());
  inv_u(std::integral_constant<int, 2>());
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < E; ++q) m[c][q] = czero<C>();
  // m = u x omega, one vorticity component at a time (lines packed in .x / .y); the three
  // transforms share one FFT body, the accumulation is selected by a switch
  auto accumulate = [&](auto w_tag) {
    constexpr int w = decltype(w_tag)::value;
    constexpr int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      m[c1][q] = lane_fma(u[c2][q], z[q], m[c1][q]);
      m[c2][q] = lane_fma(u[c1][q], lane_neg(z[q]), m[c2][q]);
    }
  };
#pragma unroll 1
  for (int w = 0; w < 3; ++w) {
    inverse(3 + w);
    switch (w) {
      case 0: accumulate(std::integral_constant<int, 0>()); break;
      case 1: accumulate(std::integral_constant<int, 1>()); break;
      default: accumulate(std::integral_constant<int, 2>()); break;
    }
  }
  // forward transforms straight from the registers, Hermitian unpack by shuffle; the three
  // share one FFT body (a loop over a uniform component, the input selected by a switch
  // with compile-time register indices), which keeps the code small for the instruction cache
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
    C in[E];
    switch (c) {
      case 0:
#pragma unroll
        for (int q = 0; q < E; ++q) in[q] = m[0][q];
        break;
      case 1:
#pragma unroll
        for (int q = 0; q < E; ++q) in[q] = m[1][q];
        break;
      default:
#pragma unroll
        for (int q = 0; q < E; ++q) in[q] = m[2][q];
        break;
    }
    auto src = [&](int, int q) -> C { return in[q]; };
    auto dst = [&](int b, int r, int, C v) { z[b + r * NBL] = v; };
    fftz(src, dst, std::integral_constant<int, -1>());
    // partner value Z(N-k) for k = t + P q: lane (P-t) mod P, slot E-1-q (t != 0) or
    // this lane, slot (E-q) mod E (t == 0)
    C zm[E];
    const int src_lane = (P - t) % P;
#pragma unroll
    for (int qq = 0; qq < E; ++qq) {
      if (slot_past_k<N, P>(E - 1 - qq)) continue;  // zm of a slot that is never stored
      C v;
      v.x = __shfl_sync(0xffffffffu, z[qq].x, src_lane, P);
      v.y = __shfl_sync(0xffffffffu, z[qq].y, src_lane, P);
      zm[E - 1 - qq] = (t != 0) ? v : z[(qq + 1) % E];
    }
    C* outf = zout + c * g.sY + row0;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      if (slot_past_k<N, P>(q)) continue;
      const int k = t + P * q;
      if (k <= K) {
        outf[k] = mk<C>((z[q].x + zm[q].x) * R(0.5), (z[q].y - zm[q].y) * R(0.5));
        outf[Hz + k] = mk<C>((z[q].y + zm[q].y) * R(0.5), (zm[q].x - z[q].x) * R(0.5));
      } else if (k < Hz) {  // the rows' padding: whole 32-byte sectors written, no read-modify-write
        outf[k] = czero<C>();
        outf[Hz + k] = czero<C>();
      }
    }
  }
}

// ------------------------------------------------------------------ z pass, MHD
// Twelve inverse transforms (u, omega, b, j) and six forward ones (m = u x omega +
// s j x b, e = u x b) per line pair, products in registers:
//   u, b -> registers; e = u x b transformed straight from them; b parked in shared
//   memory; omega accumulates m += u x omega; b back; j accumulates m += s j x b.
// Inputs u, b, omega are staged by cp.async; j is read directly.
template <typename R, int N>
struct KzRegMhdShape {
  using Plan = typename RegPlan<N>::T;
  static constexpr int P = Plan::P, E = Plan::E;
  static constexpr int NT = 128;
  static constexpr int LP = NT / P;
  static constexpr int PSH = (N >= 128) ? kSwizzle : (N >= 64) ? 4 : 3;
  static constexpr int CS = ColLayout<N, PSH, (N == 16) ? 2 : 4>::CS;
  static constexpr int HZMAX = ((N / 3 + 1) + 3) / 4 * 4;
  static constexpr int NSTAGE = 9;        // staging slots, in order of use: u (0..2), b (3..5), omega (6..8)
  static constexpr int SS = 2 * HZMAX;     // complex values per slot (two rows of up to HZMAX)
  // exchange column + staged rows; b parks in slots 0..5 once u and b are transformed
  static constexpr long long per_pair = CS + (long long)NSTAGE * SS;
  static constexpr long long smem = (long long)sizeof(cplx<R>) * (N + (long long)LP * per_pair);
  static_assert(3 * E * P <= 6 * SS, "parked b must fit in the slots of u and b");
};

template <typename R, int N, bool DEFK = false>
__global__ void __launch_bounds__(128, 3) kz_reg_mhd_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Sh = KzRegMhdShape<R, N>;
  using Plan = typename Sh::Plan;
  constexpr int P = Sh::P, E = Sh::E, LP = Sh::LP, CS = Sh::CS;
  constexpr int NBL = N / (Plan::template radix<Plan::NPASS - 1>() * P);
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  const int t = threadIdx.x % P, lp = threadIdx.x / P;
  C* xcol = tw + N + lp * Sh::per_pair;
  C* stg = xcol + CS;  // slot i at stg + i * SS
  const int pair = blockIdx.x * LP + lp, run = blockIdx.y;
  const int x = pair / (N / 2), y0 = 2 * (pair % (N / 2));
  const long long row0 = ((long long)x * N + y0) * Hz;
  const C* yin = a.in + (long long)run * 12 * g.sY;
  C* zout = a.out + (long long)run * 6 * g.sY;
  // stage in the order of use, slot i <- field 0,1,2 (u), 6,7,8 (b), 3,4,5 (omega);
  // one commit group per slot
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int f = (i < 3) ? i : ((i < 6) ? i + 3 : i - 3);
    const C* src = yin + f * g.sY + row0;
    C* dst = stg + i * Sh::SS;
    for (int c = t; c < Hz; c += P) cp_async16(dst + 2 * c, src + 2 * c);
    cp_async_commit();
  }
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, Sh::NT);
  __syncthreads();
  const WarpSync ws;
  const R sl = R(a.coef[run].lorentz);

  auto packed = [&](const C* fld) {
    return [=](int k, int q) -> C {
      if (slot_cut<N, P>(q)) return czero<C>();
      if (k <= K) {
        C A = fld[k], B = fld[Hz + k];
        if (k == 0) { A.y = 0; B.y = 0; }
        return mk<C>(A.x - B.y, A.y + B.x);
      }
      if (k >= N - K) {
        const C A = fld[N - k], B = fld[Hz + (N - k)];
        return mk<C>(A.x + B.y, B.x - A.y);
      }
      return czero<C>();
    };
  };
  auto packed_g = [&](const C* fld) {  // j: straight from global memory
    return [=](int k, int q) -> C {
      if (slot_cut<N, P>(q)) return czero<C>();
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
  C z[E];
  // forward transform of a register field given by src(q), Hermitian unpack, store field c
  auto forward_store = [&](auto& src, int c) {
    auto dst = [&](int b, int r, int, C v) { z[b + r * NBL] = v; };
    fft_column<Plan, -1, Sh::PSH, true>(t, src, dst, xcol, tw, ws);
    C zm[E];
    const int src_lane = (P - t) % P;
#pragma unroll
    for (int qq = 0; qq < E; ++qq) {
      if (slot_past_k<N, P>(E - 1 - qq)) continue;  // zm of a slot that is never stored
      C v;
      v.x = __shfl_sync(0xffffffffu, z[qq].x, src_lane, P);
      v.y = __shfl_sync(0xffffffffu, z[qq].y, src_lane, P);
      zm[E - 1 - qq] = (t != 0) ? v : z[(qq + 1) % E];
    }
    C* outf = zout + c * g.sY + row0;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      if (slot_past_k<N, P>(q)) continue;
      const int k = t + P * q;
      if (k <= K) {
        outf[k] = mk<C>((z[q].x + zm[q].x) * R(0.5), (z[q].y - zm[q].y) * R(0.5));
        outf[Hz + k] = mk<C>((z[q].y + zm[q].y) * R(0.5), (zm[q].x - z[q].x) * R(0.5));
      } else if (k < Hz) {  // the rows' padding: whole 32-byte sectors written, no read-modify-write
        outf[k] = czero<C>();
        outf[Hz + k] = czero<C>();
      }
    }
  };

  C u[3][E], b[3][E];
  auto inv_to = [&](auto slot_tag, auto wait_tag, auto* dstarr) {
    constexpr int SLOT = decltype(slot_tag)::value;
    cp_async_wait<decltype(wait_tag)::value>();
    __syncwarp();
    auto src = packed(stg + SLOT * Sh::SS);
    auto dst = [&](int bb, int r, int, C v) { dstarr[bb + r * NBL] = v; };
    fft_column<Plan, +1, Sh::PSH, true>(t, src, dst, xcol, tw, ws);
  };
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  inv_to(I0(), std::integral_constant<int, 8>(), u[0]);
  inv_to(I1(), std::integral_constant<int, 7>(), u[1]);
  inv_to(I2(), std::integral_constant<int, 6>(), u[2]);
  inv_to(std::integral_constant<int, 3>(), std::integral_constant<int, 5>(), b[0]);
  inv_to(std::integral_constant<int, 4>(), std::integral_constant<int, 4>(), b[1]);
  inv_to(std::integral_constant<int, 5>(), std::integral_constant<int, 3>(), b[2]);
  // e = u x b (output fields 3..5)
  {
    auto e0 = [&](int, int q) -> C { return mk<C>(u[1][q].x * b[2][q].x - u[2][q].x * b[1][q].x,
                                                  u[1][q].y * b[2][q].y - u[2][q].y * b[1][q].y); };
    auto e1 = [&](int, int q) -> C { return mk<C>(u[2][q].x * b[0][q].x - u[0][q].x * b[2][q].x,
                                                  u[2][q].y * b[0][q].y - u[0][q].y * b[2][q].y); };
    auto e2 = [&](int, int q) -> C { return mk<C>(u[0][q].x * b[1][q].x - u[1][q].x * b[0][q].x,
                                                  u[0][q].y * b[1][q].y - u[1][q].y * b[0][q].y); };
    forward_store(e0, 3);
    forward_store(e1, 4);
    forward_store(e2, 5);
  }
  // park b in slots 0..5 (every thread of the warp is past the reads of u and b)
  __syncwarp();
  C* park = stg;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < E; ++q) park[(c * E + q) * P + t] = b[c][q];
  C m[3][E];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < E; ++q) m[c][q] = czero<C>();
  auto add_uw = [&](auto w_tag, auto wait_tag) {
    constexpr int w = decltype(w_tag)::value;
    inv_to(std::integral_constant<int, 6 + w>(), wait_tag, z);
    constexpr int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      m[c1][q] = lane_fma(u[c2][q], z[q], m[c1][q]);
      m[c2][q] = lane_fma(u[c1][q], lane_neg(z[q]), m[c2][q]);
    }
  };
  add_uw(I0(), std::integral_constant<int, 2>());
  add_uw(I1(), std::integral_constant<int, 1>());
  add_uw(I2(), std::integral_constant<int, 0>());
  __syncwarp();
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < E; ++q) b[c][q] = park[(c * E + q) * P + t];
  // m += s (j x b):  (j x b)_{w+1} -= j_w b_{w+2};  (j x b)_{w+2} += j_w b_{w+1}
  auto add_jb = [&](auto w_tag) {
    constexpr int w = decltype(w_tag)::value;
    auto src = packed_g(yin + (9 + w) * g.sY);
    auto dst = [&](int bb, int r, int, C v) { z[bb + r * NBL] = v; };
    fft_column<Plan, +1, Sh::PSH, true>(t, src, dst, xcol, tw, ws);
    constexpr int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      m[c1][q] = mk<C>(m[c1][q].x - sl * z[q].x * b[c2][q].x, m[c1][q].y - sl * z[q].y * b[c2][q].y);
      m[c2][q] = mk<C>(m[c2][q].x + sl * z[q].x * b[c1][q].x, m[c2][q].y + sl * z[q].y * b[c1][q].y);
    }
  };
  add_jb(I0());
  add_jb(I1());
  add_jb(I2());
  auto m0 = [&](int, int q) -> C { return m[0][q]; };
  auto m1 = [&](int, int q) -> C { return m[1][q]; };
  auto m2 = [&](int, int q) -> C { return m[2][q]; };
  forward_store(m0, 0);
  forward_store(m1, 1);
  forward_store(m2, 2);
}

template <typename R, int N>
static cudaError_t launch_kz_reg_mhd(const PassArgs<R>& a, int runs, cudaStream_t st) {
  using Sh = KzRegMhdShape<R, N>;
  static cudaError_t attr = set_smem(kz_reg_mhd_kernel<R, N>, Sh::smem);
  if (attr != cudaSuccess) return attr;
  static cudaError_t attr_d = set_smem(kz_reg_mhd_kernel<R, N, true>, Sh::smem);
  if (attr_d != cudaSuccess) return attr_d;
  const int pairs = N * N / 2;
  dim3 grid(pairs / Sh::LP, runs);
  if (a.g.K == N / 3) kz_reg_mhd_kernel<R, N, true><<<grid, Sh::NT, Sh::smem, st>>>(a);
  else kz_reg_mhd_kernel<R, N><<<grid, Sh::NT, Sh::smem, st>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ z pass, adjoint
// Adjoint of u x omega for one line pair: inverse transforms of u, omega (state) and
// a (projected adjoint field); outputs p = omega x a (fields 0..2) and q = a x u (3..5).
// Order: a -> registers; each u component accumulates q, which is then transformed
// from the registers; each omega component accumulates p in the same registers.
// At most a, one accumulator and one transform are live: three CTAs per SM.
template <typename R, int N, bool DEFK = false>
__global__ void __launch_bounds__(128, 3) kz_reg_adj_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Sh = KzRegMhdShape<R, N>;  // same footprint: 9 staged fields per pair
  using Plan = typename Sh::Plan;
  constexpr int P = Sh::P, E = Sh::E, LP = Sh::LP, CS = Sh::CS;
  constexpr int NBL = N / (Plan::template radix<Plan::NPASS - 1>() * P);
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  const int t = threadIdx.x % P, lp = threadIdx.x / P;
  C* xcol = tw + N + lp * Sh::per_pair;
  C* stg = xcol + CS;  // slot i at stg + i * SS
  const int pair = blockIdx.x * LP + lp, run = blockIdx.y;
  const int x = pair / (N / 2), y0 = 2 * (pair % (N / 2));
  const long long row0 = ((long long)x * N + y0) * Hz;
  const C* yin = a.in + (long long)run * 9 * g.sY;
  C* zout = a.out + (long long)run * 6 * g.sY;
  // slots in order of use: a (fields 6,7,8), u (0,1,2), omega (3,4,5)
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int f = (i < 3) ? i + 6 : i - 3;
    const C* src = yin + f * g.sY + row0;
    C* dst = stg + i * Sh::SS;
    for (int c = t; c < Hz; c += P) cp_async16(dst + 2 * c, src + 2 * c);
    cp_async_commit();
  }
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, Sh::NT);
  __syncthreads();
  const WarpSync ws;
  auto packed = [&](const C* fld) {
    return [=](int k, int q) -> C {
      if (slot_cut<N, P>(q)) return czero<C>();
      if (k <= K) {
        C A = fld[k], B = fld[Hz + k];
        if (k == 0) { A.y = 0; B.y = 0; }
        return mk<C>(A.x - B.y, A.y + B.x);
      }
      if (k >= N - K) {
        const C A = fld[N - k], B = fld[Hz + (N - k)];
        return mk<C>(A.x + B.y, B.x - A.y);
      }
      return czero<C>();
    };
  };
  C z[E];
  auto forward_store = [&](auto& src, int c) {
    auto dst = [&](int b, int r, int, C v) { z[b + r * NBL] = v; };
    fft_column<Plan, -1, Sh::PSH, true>(t, src, dst, xcol, tw, ws);
    C zm[E];
    const int src_lane = (P - t) % P;
#pragma unroll
    for (int qq = 0; qq < E; ++qq) {
      if (slot_past_k<N, P>(E - 1 - qq)) continue;  // zm of a slot that is never stored
      C v;
      v.x = __shfl_sync(0xffffffffu, z[qq].x, src_lane, P);
      v.y = __shfl_sync(0xffffffffu, z[qq].y, src_lane, P);
      zm[E - 1 - qq] = (t != 0) ? v : z[(qq + 1) % E];
    }
    C* outf = zout + c * g.sY + row0;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      if (slot_past_k<N, P>(q)) continue;
      const int k = t + P * q;
      if (k <= K) {
        outf[k] = mk<C>((z[q].x + zm[q].x) * R(0.5), (z[q].y - zm[q].y) * R(0.5));
        outf[Hz + k] = mk<C>((z[q].y + zm[q].y) * R(0.5), (zm[q].x - z[q].x) * R(0.5));
      } else if (k < Hz) {  // the rows' padding: whole 32-byte sectors written, no read-modify-write
        outf[k] = czero<C>();
        outf[Hz + k] = czero<C>();
      }
    }
  };
  C av[3][E], pm[3][E];
  auto inv_to = [&](auto slot_tag, auto wait_tag, auto* dstarr) {
    constexpr int SLOT = decltype(slot_tag)::value;
    cp_async_wait<decltype(wait_tag)::value>();
    __syncwarp();
    auto src = packed(stg + SLOT * Sh::SS);
    auto dst = [&](int bb, int r, int, C v) { dstarr[bb + r * NBL] = v; };
    fft_column<Plan, +1, Sh::PSH, true>(t, src, dst, xcol, tw, ws);
  };
  inv_to(std::integral_constant<int, 0>(), std::integral_constant<int, 8>(), av[0]);
  inv_to(std::integral_constant<int, 1>(), std::integral_constant<int, 7>(), av[1]);
  inv_to(std::integral_constant<int, 2>(), std::integral_constant<int, 6>(), av[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < E; ++q) pm[c][q] = czero<C>();
  // q = a x u:  q_{w+1} += a_{w+2} u_w;  q_{w+2} -= a_{w+1} u_w
  auto add_u = [&](auto w_tag, auto wait_tag) {
    constexpr int w = decltype(w_tag)::value;
    inv_to(std::integral_constant<int, 3 + w>(), wait_tag, z);
    constexpr int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      pm[c1][q] = mk<C>(pm[c1][q].x + av[c2][q].x * z[q].x, pm[c1][q].y + av[c2][q].y * z[q].y);
      pm[c2][q] = mk<C>(pm[c2][q].x - av[c1][q].x * z[q].x, pm[c2][q].y - av[c1][q].y * z[q].y);
    }
  };
  add_u(std::integral_constant<int, 0>(), std::integral_constant<int, 5>());
  add_u(std::integral_constant<int, 1>(), std::integral_constant<int, 4>());
  add_u(std::integral_constant<int, 2>(), std::integral_constant<int, 3>());
  // every input row of this pair is in shared memory before the first output store, so
  // the outputs may overwrite the inputs (out == in: the pass runs in place)
  cp_async_wait_all();
  __syncwarp();
  {
    auto q0 = [&](int, int q) -> C { return pm[0][q]; };
    auto q1 = [&](int, int q) -> C { return pm[1][q]; };
    auto q2 = [&](int, int q) -> C { return pm[2][q]; };
    forward_store(q0, 3);
    forward_store(q1, 4);
    forward_store(q2, 5);
  }
  // p = omega x a:  (omega x a)_{w+1} -= omega_w a_{w+2};  (omega x a)_{w+2} += omega_w a_{w+1}
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < E; ++q) pm[c][q] = czero<C>();
  auto add_w = [&](auto w_tag, auto wait_tag) {
    constexpr int w = decltype(w_tag)::value;
    inv_to(std::integral_constant<int, 6 + w>(), wait_tag, z);
    constexpr int c1 = (w + 1) % 3, c2 = (w + 2) % 3;
#pragma unroll
    for (int q = 0; q < E; ++q) {
      pm[c1][q] = mk<C>(pm[c1][q].x - z[q].x * av[c2][q].x, pm[c1][q].y - z[q].y * av[c2][q].y);
      pm[c2][q] = mk<C>(pm[c2][q].x + z[q].x * av[c1][q].x, pm[c2][q].y + z[q].y * av[c1][q].y);
    }
  };
  add_w(std::integral_constant<int, 0>(), std::integral_constant<int, 2>());
  add_w(std::integral_constant<int, 1>(), std::integral_constant<int, 1>());
  add_w(std::integral_constant<int, 2>(), std::integral_constant<int, 0>());
  auto p0 = [&](int, int q) -> C { return pm[0][q]; };
  auto p1 = [&](int, int q) -> C { return pm[1][q]; };
  auto p2 = [&](int, int q) -> C { return pm[2][q]; };
  forward_store(p0, 0);
  forward_store(p1, 1);
  forward_store(p2, 2);
}

template <typename R, int N>
static cudaError_t launch_kz_reg_adj(const PassArgs<R>& a, int runs, cudaStream_t st) {
  using Sh = KzRegMhdShape<R, N>;
  static cudaError_t attr = set_smem(kz_reg_adj_kernel<R, N>, Sh::smem);
  if (attr != cudaSuccess) return attr;
  static cudaError_t attr_d = set_smem(kz_reg_adj_kernel<R, N, true>, Sh::smem);
  if (attr_d != cudaSuccess) return attr_d;
  const int pairs = N * N / 2;
  dim3 grid(pairs / Sh::LP, runs);
  if (a.g.K == N / 3) kz_reg_adj_kernel<R, N, true><<<grid, Sh::NT, Sh::smem, st>>>(a);
  else kz_reg_adj_kernel<R, N><<<grid, Sh::NT, Sh::smem, st>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ x pass
template <typename R, int N>
struct KxRegShape {
  using Plan = typename RegPlan<N>::T;
  static constexpr int P = Plan::P, E = Plan::E;
  // kz columns per group (one 32-byte sector; 8-column groups at 256, with a conflict-free
  // exchange stride = 2 (mod 16), measured no faster).  The staging loops copy 16-byte chunks
  // and skip any past the padded row (Hz is a multiple of 4), whose columns are never used.
  static constexpr int QW = 4;
  static constexpr int CPR = QW / 2;                // 16-byte cp.async chunks per row segment
  static constexpr int GT = QW * P;                 // threads per group
  static constexpr int TARGET = (P >= 16) ? 256 : 128;  // threads per CTA
  static constexpr int NG0 = (GT >= TARGET) ? 1 : TARGET / GT;
  // kz column groups of the default cutoff (K = N/3), and groups per CTA: NG0, or down to
  // half of it when that leaves fewer idle groups in the last kz block of a row (96: 9
  // groups, 3 per CTA instead of 4, which had transformed 48 columns for 33; 64: 6, 3)
  static constexpr int QUADS = (N / 3 + 1 + QW - 1) / QW;
  static constexpr int idle(int ng) { return (QUADS + ng - 1) / ng * ng - QUADS; }
  static constexpr int best_ng(int ng, int best) {
    return (2 * ng < NG0) ? best : best_ng(ng - 1, (idle(ng) < idle(best)) ? ng : best);
  }
  static constexpr int NG = best_ng(NG0, NG0);
  static constexpr int NT = NG * GT;
  // resident CTAs per SM the registers must allow (E = 12 at N = 96 needs ~168 registers)
  static constexpr int MINB = (NT >= 256) ? 2 : ((E > 8) ? 3 : 4);
  // the x stage runs persistent CTAs with its tiles in kz-fastest order at N >= 256 (256^3:
  // 156 -> 149 us); at smaller N one tile per CTA in ky-fastest order measured faster (the
  // per-tile set-up is small there, and the batched 96^3 group ran 260 -> 313 us persistent)
  static constexpr bool PERSIST = (N >= 256);
  static constexpr int PSH = 3;
  // exchange column stride: = 4 (mod 16) for 4-column groups, = 2 for 8 (bank-conflict model)
  static constexpr int CS = ColLayout<N, PSH, (QW == 8) ? 2 : 4>::CS;
  // at 96 the register x stage alternates between two exchange columns per kz column (one group
  // barrier per exchange instead of two; batched 96^3 x stage 173.5 -> 161.4 us).  At 128 and 256
  // the larger shared-memory footprint measured slower (20.9 -> 22.3 and 122.0 -> 136.2 us).
  // XOFF is the distance between the two columns
  static constexpr int XCOLS = (Plan::NPASS == 3 && N == 96) ? 2 : 1;
  static constexpr int XOFF = (XCOLS == 2) ? NG * QW * CS : 0;
  static constexpr int MMAX = 2 * (N / 3) + 1;
  // per group: state and accumulator tiles [2][3][M][QW], staged by cp.async
  static constexpr long long stage_elems = 2LL * 3 * MMAX * QW;
  // + the integrating-factor tables: (expm1(-c kx^2) for c = nu h, nu h / 2) over kx, and
  // the same of ky^2 + kz^2 for the CTA's columns
  // (two copies of the factor tables: the persistent x stage writes a tile's while the previous
  // tile's may still be read)
  static constexpr long long smem =
      (long long)sizeof(cplx<R>) * (N + (long long)XCOLS * NG * QW * CS + (long long)NG * stage_elems + 2 * (MMAX + NG * QW));
  // RK4 stage 1 stages the state only (no accumulator yet): its kernel lays out and requests
  // half the staging area
  static constexpr long long smem1 = smem - (long long)sizeof(cplx<R>) * NG * (stage_elems / 2);
  // adjoint kernels, per group: a ring of four [N][QW] input tiles of the forward transforms,
  // or up to two [3][M][QW] spectral tiles, both staged by cp.async
  static constexpr long long ring_elems = 4LL * N * QW;
  static constexpr long long adj_area = (ring_elems > stage_elems) ? ring_elems : stage_elems;
  // + the integrating-factor tables of the x stage (the tape forms)
  static constexpr long long smem_adj =
      (long long)sizeof(cplx<R>) * (N + (long long)NG * QW * CS + (long long)NG * adj_area + MMAX + NG * QW);
};




// one of the six inverse-transformed fields u, curl u from the column's state
template <int GI, typename A>
__device__ __forceinline__ auto uw_field(const A& v, int q, float kx, float ky, float kz) {
  if constexpr (GI < 3) {
    return v[GI][q];
  } else {
    return curl_comp(GI - 3, v[0][q], v[1][q], v[2][q], kx, ky, kz);
  }
}

// The x stage is tiled by (ky row, NG * QW kz columns, run): a.tiles tiles, taken by each CTA
// in the order blockIdx.x, + gridDim.x, ...  With Sh::PERSIST (KX_STAGE), persistent CTAs
// take the tiles in kz-fastest order: the twiddles are built once per CTA, and while a
// tile's inverse transforms run, the state / accumulator tiles of the CTA's next tile are
// staged into shared memory (cp.async), so that a tile starts with its operands at hand.  Its
// forward inputs W are mostly still in L2 (the forward y pass writes them with an evict_last
// policy); an explicit L2 prefetch of them, issued here before that, measured 1 % slower once
// they were (118.1 -> 116.7 us without it).  Otherwise one tile per CTA, ky fastest.
template <typename R, int N, int MODE, bool DEFK = false, int STG = 0>
__global__ void __launch_bounds__(KxRegShape<R, N>::NT, KxRegShape<R, N>::MINB) kx_reg_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Sh = KxRegShape<R, N>;
  using Plan = typename Sh::Plan;
  constexpr int P = Sh::P, E = Sh::E, QW = Sh::QW, GT = Sh::GT, CS = Sh::CS;
  constexpr int NBL = N / (Plan::template radix<Plan::NPASS - 1>() * P);
  const Geo g = geo_of<N, DEFK>(a.g);
  const int stage = STG ? STG : a.stage;  // the RK4 stage (KX_STAGE), compile-time for STG > 0
  const int K = g.K, M = g.M, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  const int grp = threadIdx.x / GT, lt = threadIdx.x % GT;
  const int col = lt % QW, t = lt / QW;
  const int kzb = ((g.Hk + QW - 1) / QW + Sh::NG - 1) / Sh::NG;  // kz blocks per ky row
  constexpr bool KZF = (MODE == KX_STAGE) && Sh::PERSIST;
  // tile -> (kz block, ky row, run)
  auto tile_bkz = [&](int tl) { return KZF ? tl % kzb : (tl / M) % kzb; };
  auto tile_iyc = [&](int tl) { return KZF ? (tl / kzb) % M : tl % M; };
  C* xcol = tw + N + (grp * QW + col) * CS;
  // [0] state, [1] accumulator: [3][M][QW] each
  constexpr long long SE = (STG == 1) ? Sh::stage_elems / 2 : Sh::stage_elems;  // staging area per group
  C* stg = tw + N + Sh::XCOLS * Sh::NG * QW * CS + grp * SE;
  // integrating factors of the Lawson stages: expm1(-c (kx^2 + q)) with c = nu h (or nu h / 2)
  // and q = ky^2 + kz^2 is expm1(a) + expm1(b) + expm1(a) expm1(b), a = -c kx^2, b = -c q, an
  // exact identity; the kx terms (M entries) and the (ky, kz) terms of the tile's columns are
  // tabulated per tile, so that no mode evaluates expm1 (the factors stay in delta form).
  // Two copies, by tile parity: a tile's table is written while the previous tile's may
  // still be read
  C* ftab0 = tw + N + Sh::XCOLS * Sh::NG * QW * CS + Sh::NG * SE;
  constexpr int FT = Sh::MMAX + Sh::NG * QW;
  // stage the state (and accumulator) tiles of this group's columns of tile (iyc, bkz, run):
  // rows of QW consecutive kz are 32-byte aligned (Hz % 4 == 0, kz0 a multiple of QW); chunks
  // past the padded row (kz0 + 2h >= Hz) are skipped; one commit group per call
  auto stage_state = [&](int iyc_, int bkz_, int run_) {
    const int kz0_ = (bkz_ * Sh::NG + grp) * QW;
    if (kz0_ < g.Hk) {
      const int narr = (stage > 1) ? 2 : 1;
      const long long base = (long long)run_ * 3 * g.sS + (long long)iyc_ * Hz + kz0_;
      constexpr int CPR = Sh::CPR;
      const int chunks = narr * 3 * M * CPR;  // 16-byte chunks of each row segment
      for (int c = lt; c < chunks; c += GT) {
        const int h = c % CPR, row = c / CPR;  // row = (arr * 3 + f) * M + ic
        if (kz0_ + 2 * h >= Hz) continue;
        const int arr = row / (3 * M), fi = row % (3 * M);
        const C* src = (arr == 0 ? a.S : a.acc) + base + (long long)fi * M * Hz + 2 * h;
        cp_async16(stg + (long long)row * QW + 2 * h, src);
      }
    }
    cp_async_commit();
  };
  int tile = blockIdx.x;
  if constexpr (MODE == KX_STAGE) {
    if (tile < a.tiles) stage_state(tile_iyc(tile), tile_bkz(tile), tile / (kzb * M));
  }
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, Sh::NT);
  if constexpr (MODE != KX_STAGE) __syncthreads();

  C v[3][E];
  auto run_fft = [&](auto& src, auto& dst, auto dir_tag) {
    constexpr int DIR = decltype(dir_tag)::value;
    if constexpr (GT > 32) {
      const NamedSync ns{1 + grp, GT};
      fft_column<Plan, DIR, Sh::PSH, true, Sh::XOFF>(t, src, dst, xcol, tw, ns);
    } else {
      const WarpSync ws;
      fft_column<Plan, DIR, Sh::PSH, true, Sh::XOFF>(t, src, dst, xcol, tw, ws);
    }
  };
  auto gsync = [&]() {
    if constexpr (GT > 32) {
      const NamedSync ns{1 + grp, GT};
      ns();
    } else {
      __syncwarp();
    }
  };
  using Fwd = std::integral_constant<int, -1>;
  using Inv = std::integral_constant<int, +1>;

  for (int it = 0; tile < a.tiles; tile += gridDim.x, ++it) {
    const int bkz = tile_bkz(tile), iyc = tile_iyc(tile), run = tile / (kzb * M);
    const int kz0 = (bkz * Sh::NG + grp) * QW;
    const int kz = kz0 + col;
    const bool zok = kz < g.Hk;
    const float kyf = float(ksigned(iyc, K)), kzf = float(kz);
    const long long soff = (long long)run * 3 * g.sS + (long long)iyc * Hz + kz;  // + (f*M + ic)*M*Hz
    C* ftab = ftab0 + (it & 1) * FT;

    if constexpr (MODE == KX_LOAD) {
      const C* sin_ = a.spec_in + soff;
#pragma unroll
      for (int f = 0; f < 3; ++f)
#pragma unroll
        for (int q = 0; q < E; ++q) {
          const int ic = kcompact_slot<N, P>(t, q, K);
          v[f][q] = (zok && ic >= 0) ? sin_[((long long)f * M + ic) * M * Hz] : czero<C>();
        }
    } else {
      const R inv_n3 = R(1) / (R(N) * R(N) * R(N));
      const C* win = a.in + (long long)run * 3 * g.sX + (long long)iyc * Hz + kz;
      // issue the global loads of all three fields before the first transform (the
      // first pass of thread t reads x = t + P q into slot q), so that their latency
      // is paid once; the slots are consumed field by field
      C pre[3][E];
#pragma unroll
      for (int f = 0; f < 3; ++f)
#pragma unroll
        for (int q = 0; q < E; ++q)
          pre[f][q] = zok ? win[f * g.sX + (long long)(t + P * q) * M * Hz] : czero<C>();
      {  // this tile's factor tables (and, on the first tile, the twiddles) before any use
        const RunCoef cf0 = a.coef[run];
        const R c1 = R(cf0.nu * cf0.dt), ch = R(0.5) * c1;
        for (int i = threadIdx.x; i < M + Sh::NG * QW; i += Sh::NT) {
          R k2;
          if (i < M) {
            const R kx = R(ksigned(i, K));
            k2 = kx * kx;
          } else {
            const R kc = R(bkz * Sh::NG * QW + (i - M));  // kz of column i - M
            k2 = R(kyf * kyf) + kc * kc;
          }
          ftab[i] = mk<C>(rexpm1<R>(-c1 * k2), rexpm1<R>(-ch * k2));
        }
      }
      __syncthreads();
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        auto src = [&](int, int q) -> C { return pre[f][q]; };
        auto dst = [&](int b, int r, int, C val) { v[f][b + r * NBL] = cscale(val, inv_n3); };
        run_fft(src, dst, Fwd());
      }
      // fused spectral pointwise stage on the modes k = t (mod P) of this column
      cp_async_wait_all();
      gsync();
      const RunCoef cf = a.coef[run];
      const bool expl = (a.flags & FLAG_EXPLICIT) != 0;
      const R h = R(cf.dt);
      const C fyz = ftab[M + grp * QW + col];  // the (ky, kz) terms of this column
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int ic = kcompact_slot<N, P>(t, q, K);
        if (zok && ic >= 0) {
          const float kx = float(ksigned(ic, K));
          const float k2 = kx * kx + kyf * kyf + kzf * kzf;
          leray(v[0][q], v[1][q], v[2][q], kx, kyf, kzf, k2);
          const R lin = expl ? R(cf.nu * double(k2)) : R(0);  // explicit viscosity only
          const C fx = ftab[ic];
          const R m1 = expm1_add(fx.x, fyz.x), mh = expm1_add(fx.y, fyz.y);
#pragma unroll
          for (int f = 0; f < 3; ++f) {
            const long long o = soff + ((long long)f * M + ic) * M * Hz;
            const C s = stg[((long long)f * M + ic) * QW + col];
            if (a.tape != nullptr) {  // adjoint tape (batch 1): n_stage for stages 1..3, V at stage 1
              if (stage <= 3) a.tape[(long long)stage * 3 * g.sS + o] = v[f][q];
              if (stage == 1) a.tape[o] = s;
            }
            C acc = (stage > 1) ? stg[((long long)(3 + f) * M + ic) * QW + col] : czero<C>();
            const C vs = (expl && stage > 1) ? a.vs[o] : s;
            const C nv = expl ? rk4_combine<C>(stage, true, v[f][q], s, acc, vs, h, lin)
                              : lawson_combine<C>(stage, v[f][q], s, acc, h, m1, mh);
            if (stage < 4) {
              a.acc[o] = acc;
              if (expl) a.vs[o] = nv;
            } else {
              a.S[o] = nv;
            }
            v[f][q] = nv;
          }
        } else {
#pragma unroll
          for (int f = 0; f < 3; ++f) v[f][q] = czero<C>();
          // padding columns: zeros, so that every 32-byte sector of a row is written whole
          // (no read-modify-write of partly written sectors in the L2)
          if (!zok && kz < Hz && ic >= 0) {
#pragma unroll
            for (int f = 0; f < 3; ++f) {
              const long long o = soff + ((long long)f * M + ic) * M * Hz;
              if (stage < 4) {
                a.acc[o] = czero<C>();
                if (expl) a.vs[o] = czero<C>();
              } else {
                a.S[o] = czero<C>();
              }
            }
          }
        }
      }
      // the next tile: its state / accumulator tiles into the staging area (every thread of
      // the group is past its reads of this tile's)
      const int next = tile + gridDim.x;
      if (next < a.tiles) {
        const int nbkz = tile_bkz(next), niyc = tile_iyc(next), nrun = next / (kzb * M);
        gsync();
        stage_state(niyc, nbkz, nrun);
      }
    }

    // inverse-x of u and curl u straight from the registers.  At N >= 128 the six transforms
    // share one FFT body (a loop over a uniform field index; the values of this thread's modes
    // are formed first by a switch whose cases index the registers at compile time), which
    // keeps the kernel's code small enough for the instruction cache; smaller transforms are
    // unrolled (the loop would raise their register count and lower occupancy).
    C* xo = a.out + (long long)run * 6 * g.sX + (long long)iyc * Hz + kz;
    auto values = [&](auto gi_tag, C* in) {
      constexpr int GI = decltype(gi_tag)::value;
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int ic = kcompact_slot<N, P>(t, q, K);
        in[q] = (ic < 0) ? czero<C>() : uw_field<GI>(v, q, float(ksigned(ic, K)), kyf, kzf);
      }
    };
    auto inverse_of = [&](const C* in, int gi) {
      auto src = [&](int, int q) -> C { return in[q]; };
      C* xg = xo + gi * g.sX;
      auto dst = [&](int, int, int x, C val) {  // padding columns (kz >= Hk) get the zeros they hold
        if (kz < Hz) xg[(long long)x * M * Hz] = val;
      };
      run_fft(src, dst, Inv());
    };
    if constexpr (N >= 128) {
#pragma unroll 1
      for (int gi = 0; gi < 6; ++gi) {
        C in[E];
        switch (gi) {
          case 0: values(std::integral_constant<int, 0>(), in); break;
          case 1: values(std::integral_constant<int, 1>(), in); break;
          case 2: values(std::integral_constant<int, 2>(), in); break;
          case 3: values(std::integral_constant<int, 3>(), in); break;
          case 4: values(std::integral_constant<int, 4>(), in); break;
          default: values(std::integral_constant<int, 5>(), in); break;
        }
        inverse_of(in, gi);
      }
    } else {
      auto inverse = [&](auto gi_tag) {
        C in[E];
        values(gi_tag, in);
        inverse_of(in, decltype(gi_tag)::value);
      };
      inverse(std::integral_constant<int, 0>());
      inverse(std::integral_constant<int, 1>());
      inverse(std::integral_constant<int, 2>());
      inverse(std::integral_constant<int, 3>());
      inverse(std::integral_constant<int, 4>());
      inverse(std::integral_constant<int, 5>());
    }
  }
}

// ------------------------------------------------------------------ x stage, stashed state
// The fused x stage (KX_STAGE, hydro) with the column's spectral values parked between its
// phases in a thread-private shared-memory stash instead of in registers, so that a thread
// holds at most one field's values (and the next field's inputs) at a time: fewer registers,
// three CTAs (24 warps) per SM instead of two.  Each thread stashes only the mode slots it
// owns (and only those no 2/3 cutoff removes), so the stash needs no barriers.  The state and
// accumulator are read straight from global memory (prefetched into L2 with the next tile's
// forward inputs while the current tile's inverse transforms run); persistent CTAs take the
// tiles of (ky row, NG x QW kz columns, run) in kz-fastest order.
template <int N, int P, int E> __host__ __device__ constexpr int kept_slot_count() {
  int c = 0;
  for (int q = 0; q < E; ++q)
    if (!slot_cut<N, P>(q)) ++c;
  return c;
}
template <int N, int P> __host__ __device__ constexpr int kept_slot_rank(int q) {
  int c = 0;
  for (int i = 0; i < q; ++i)
    if (!slot_cut<N, P>(i)) ++c;
  return c;
}

template <typename R, int N>
struct KxStashShape {
  using Reg = KxRegShape<R, N>;
  using Plan = typename Reg::Plan;
  static constexpr int P = Reg::P, E = Reg::E, QW = Reg::QW, GT = Reg::GT, NG = Reg::NG, NT = Reg::NT;
  static constexpr int CS = Reg::CS, MMAX = Reg::MMAX;
  static constexpr int NK = kept_slot_count<N, P, E>();  // stashed slots per field and thread
  static constexpr int MINB = (NT >= 256) ? 3 : 5;
  static constexpr long long stash_elems = 3LL * NK * GT;  // per group
  static constexpr long long smem =
      (long long)sizeof(cplx<R>) * (N + (long long)NG * QW * CS + (long long)NG * stash_elems + 2 * (MMAX + NG * QW));
};
// sizes with the stashed x stage (FP32)
template <int N> struct HasStashX { static constexpr bool value = (N == 64 || N == 96 || N == 128 || N == 256); };

template <typename R, int N, bool DEFK = false, int STG = 0>
__global__ void __launch_bounds__(KxStashShape<R, N>::NT, KxStashShape<R, N>::MINB) kx_stash_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Sh = KxStashShape<R, N>;
  using Plan = typename Sh::Plan;
  constexpr int P = Sh::P, E = Sh::E, QW = Sh::QW, GT = Sh::GT, CS = Sh::CS, NK = Sh::NK;
  constexpr int NBL = N / (Plan::template radix<Plan::NPASS - 1>() * P);
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, M = g.M, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  const int grp = threadIdx.x / GT, lt = threadIdx.x % GT;
  const int col = lt % QW, t = lt / QW;
  const int kzb = ((g.Hk + QW - 1) / QW + Sh::NG - 1) / Sh::NG;  // kz blocks per ky row
  C* xcol = tw + N + (grp * QW + col) * CS;
  // this thread's stash: element (field f, kept slot rank qi) at st[(f * NK + qi) * GT]
  C* st = tw + N + Sh::NG * QW * CS + grp * Sh::stash_elems + lt;
  // integrating-factor tables (as in kx_reg_kernel), two copies by tile parity
  C* ftab0 = tw + N + Sh::NG * QW * CS + Sh::NG * Sh::stash_elems;
  constexpr int FT = Sh::MMAX + Sh::NG * QW;
  auto run_fft = [&](auto& src, auto& dst, auto dir_tag) {
    constexpr int DIR = decltype(dir_tag)::value;
    if constexpr (GT > 32) {
      const NamedSync ns{1 + grp, GT};
      fft_column<Plan, DIR, Sh::Reg::PSH, false>(t, src, dst, xcol, tw, ns);
    } else {
      const WarpSync ws;
      fft_column<Plan, DIR, Sh::Reg::PSH, false>(t, src, dst, xcol, tw, ws);
    }
  };
  using Fwd = std::integral_constant<int, -1>;
  using Inv = std::integral_constant<int, +1>;
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, Sh::NT);
  const R inv_n3 = R(1) / (R(N) * R(N) * R(N));
  const bool expl = (a.flags & FLAG_EXPLICIT) != 0;
  const int stage = STG ? STG : a.stage;  // compile-time for STG > 0

  for (int tile = blockIdx.x, it = 0; tile < a.tiles; tile += gridDim.x, ++it) {
    const int bkz = tile % kzb, iyc = (tile / kzb) % M, run = tile / (kzb * M);
    const int kz0 = (bkz * Sh::NG + grp) * QW;
    const int kz = kz0 + col;
    const bool zok = kz < g.Hk;
    const float kyf = float(ksigned(iyc, K)), kzf = float(kz);
    const long long soff = (long long)run * 3 * g.sS + (long long)iyc * Hz + kz;  // + (f*M + ic)*M*Hz
    C* ftab = ftab0 + (it & 1) * FT;
    const C* win = a.in + (long long)run * 3 * g.sX + (long long)iyc * Hz + kz;
    // forward inputs of field 0 (thread t reads x = t + P q into slot q)
    C cur[E];
#pragma unroll
    for (int q = 0; q < E; ++q) cur[q] = zok ? win[(long long)(t + P * q) * M * Hz] : czero<C>();
    {  // this tile's factor tables (and, on the first tile, the twiddles) before any use
      const RunCoef cf0 = a.coef[run];
      const R c1 = R(cf0.nu * cf0.dt), ch = R(0.5) * c1;
      for (int i = threadIdx.x; i < M + Sh::NG * QW; i += Sh::NT) {
        R k2;
        if (i < M) {
          const R kx = R(ksigned(i, K));
          k2 = kx * kx;
        } else {
          const R kc = R(bkz * Sh::NG * QW + (i - M));  // kz of column i - M
          k2 = R(kyf * kyf) + kc * kc;
        }
        ftab[i] = mk<C>(rexpm1<R>(-c1 * k2), rexpm1<R>(-ch * k2));
      }
    }
    __syncthreads();
    // forward transforms, field by field through one FFT body (instruction cache; the next
    // field's inputs are loaded before the current transform), the kept slots of the result
    // (x 1/N^3) into the stash
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
      C nxt[E];
      if (f < 2) {
#pragma unroll
        for (int q = 0; q < E; ++q)
          nxt[q] = zok ? win[(f + 1) * g.sX + (long long)(t + P * q) * M * Hz] : czero<C>();
      }
      C* sf = st + f * NK * GT;
      auto src = [&](int, int q) -> C { return cur[q]; };
      auto dst = [&](int b, int r, int, C val) {
        const int q = b + r * NBL;
        if (!slot_cut<N, P>(q)) sf[kept_slot_rank<N, P>(q) * GT] = cscale(val, inv_n3);
      };
      run_fft(src, dst, Fwd());
      if (f < 2) {
#pragma unroll
        for (int q = 0; q < E; ++q) cur[q] = nxt[q];
      }
    }
    // Leray projection in the stash (removed modes of partly cut slots set to zero)
#pragma unroll
    for (int q = 0; q < E; ++q) {
      if (slot_cut<N, P>(q)) continue;
      const int qi = kept_slot_rank<N, P>(q);
      const int ic = kcompact_slot<N, P>(t, q, K);
      C v0 = czero<C>(), v1 = czero<C>(), v2 = czero<C>();
      if (zok && ic >= 0) {
        v0 = st[(0 * NK + qi) * GT];
        v1 = st[(1 * NK + qi) * GT];
        v2 = st[(2 * NK + qi) * GT];
        const float kx = float(ksigned(ic, K));
        leray(v0, v1, v2, kx, kyf, kzf, kx * kx + kyf * kyf + kzf * kzf);
      }
      st[(0 * NK + qi) * GT] = v0;
      st[(1 * NK + qi) * GT] = v1;
      st[(2 * NK + qi) * GT] = v2;
    }
    // RK4 stage combine, field by field: the state / accumulator loads of all slots first
    {
      const RunCoef cf = a.coef[run];
      const R h = R(cf.dt);
      const C fyz = ftab[M + grp * QW + col];  // the (ky, kz) terms of this column
      const C* __restrict__ Sp = a.S;
      const C* __restrict__ Ap = a.acc;
#pragma unroll 1
      for (int f = 0; f < 3; ++f) {
        C sv[NK], av[NK];
#pragma unroll
        for (int q = 0; q < E; ++q) {
          if (slot_cut<N, P>(q)) continue;
          const int qi = kept_slot_rank<N, P>(q);
          const int ic = kcompact_slot<N, P>(t, q, K);
          const bool ok = zok && ic >= 0;
          const long long o = soff + ((long long)f * M + (ok ? ic : 0)) * M * Hz;
          sv[qi] = ok ? Sp[o] : czero<C>();
          av[qi] = (ok && stage > 1) ? Ap[o] : czero<C>();
        }
#pragma unroll
        for (int q = 0; q < E; ++q) {
          if (slot_cut<N, P>(q)) continue;
          const int qi = kept_slot_rank<N, P>(q);
          const int ic = kcompact_slot<N, P>(t, q, K);
          if (!(zok && ic >= 0)) {  // stash entry already zero
            if (!zok && kz < Hz && ic >= 0) {  // padding columns: zeros, whole sectors written
              const long long o = soff + ((long long)f * M + ic) * M * Hz;
              if (stage < 4) {
                a.acc[o] = czero<C>();
                if (expl) a.vs[o] = czero<C>();
              } else {
                a.S[o] = czero<C>();
              }
            }
            continue;
          }
          const long long o = soff + ((long long)f * M + ic) * M * Hz;
          const C n = st[(f * NK + qi) * GT];
          const C s = sv[qi];
          if (a.tape != nullptr) {  // adjoint tape (batch 1): n_stage for stages 1..3, V at stage 1
            if (stage <= 3) a.tape[(long long)stage * 3 * g.sS + o] = n;
            if (stage == 1) a.tape[o] = s;
          }
          C acc = av[qi];
          C nv;
          if (expl) {
            const float kx = float(ksigned(ic, K));
            const R lin = R(cf.nu * double(kx * kx + kyf * kyf + kzf * kzf));
            const C vs = (stage > 1) ? a.vs[o] : s;
            nv = rk4_combine<C>(stage, true, n, s, acc, vs, h, lin);
            if (stage < 4) a.vs[o] = nv;
          } else {
            const C fx = ftab[ic];
            nv = lawson_combine<C>(stage, n, s, acc, h, expm1_add(fx.x, fyz.x), expm1_add(fx.y, fyz.y));
          }
          if (stage < 4) a.acc[o] = acc;
          else a.S[o] = nv;
          st[(f * NK + qi) * GT] = nv;
        }
      }
    }
    // the next tile's forward inputs and state / accumulator rows into L2 (32-byte segments)
    const int next = tile + gridDim.x;
    if (next < a.tiles) {
      const int nbkz = next % kzb, niyc = (next / kzb) % M, nrun = next / (kzb * M);
      const int nkz0 = (nbkz * Sh::NG + grp) * QW;
      if (nkz0 < g.Hk) {
        const C* nw = a.in + (long long)nrun * 3 * g.sX + (long long)niyc * Hz + nkz0;
        for (int r = lt; r < 3 * N; r += GT)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(nw + (long long)(r / N) * g.sX + (long long)(r % N) * M * Hz));
        const long long nbase = (long long)nrun * 3 * g.sS + (long long)niyc * Hz + nkz0;
        const int narr = (stage > 1) ? 2 : 1;
        for (int r = lt; r < narr * 3 * M; r += GT) {
          const C* arr = (r < 3 * M) ? a.S : a.acc;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(arr + nbase + (long long)(r % (3 * M)) * M * Hz));
        }
      }
    }
    // inverse-x of u and curl u from the stash (one FFT body for the six fields at N >= 128)
    C* xo = a.out + (long long)run * 6 * g.sX + (long long)iyc * Hz + kz;
    auto values = [&](auto gi_tag, C* in) {
      constexpr int GI = decltype(gi_tag)::value;
#pragma unroll
      for (int q = 0; q < E; ++q) {
        if (slot_cut<N, P>(q)) {
          in[q] = czero<C>();
          continue;
        }
        const int qi = kept_slot_rank<N, P>(q);
        if constexpr (GI < 3) {
          in[q] = st[(GI * NK + qi) * GT];
        } else {
          const int ic = kcompact_slot<N, P>(t, q, K);
          const float kx = float(ksigned(ic < 0 ? 0 : ic, K));
          in[q] = curl_comp(GI - 3, st[(0 * NK + qi) * GT], st[(1 * NK + qi) * GT], st[(2 * NK + qi) * GT], kx,
                            kyf, kzf);
        }
      }
    };
    auto inverse_of = [&](const C* in, int gi) {
      auto src = [&](int, int q) -> C { return in[q]; };
      C* xg = xo + gi * g.sX;
      auto dst = [&](int, int, int x, C val) {  // padding columns (kz >= Hk) get the zeros they hold
        if (kz < Hz) xg[(long long)x * M * Hz] = val;
      };
      run_fft(src, dst, Inv());
    };
#pragma unroll 1
    for (int gi = 0; gi < 6; ++gi) {
      C in[E];
      switch (gi) {
        case 0: values(std::integral_constant<int, 0>(), in); break;
        case 1: values(std::integral_constant<int, 1>(), in); break;
        case 2: values(std::integral_constant<int, 2>(), in); break;
        case 3: values(std::integral_constant<int, 3>(), in); break;
        case 4: values(std::integral_constant<int, 4>(), in); break;
        default: values(std::integral_constant<int, 5>(), in); break;
      }
      inverse_of(in, gi);
    }
  }
}

template <typename R, int N>
static cudaError_t launch_kx_stash(const PassArgs<R>& a0, int runs, cudaStream_t st) {
  using Sh = KxStashShape<R, N>;
  static cudaError_t attr = set_smem(kx_stash_kernel<R, N>, Sh::smem);
  if (attr != cudaSuccess) return attr;
  static cudaError_t attr_d = first_error({set_smem(kx_stash_kernel<R, N, true, 1>, Sh::smem),
                                           set_smem(kx_stash_kernel<R, N, true, 2>, Sh::smem),
                                           set_smem(kx_stash_kernel<R, N, true, 3>, Sh::smem),
                                           set_smem(kx_stash_kernel<R, N, true, 4>, Sh::smem)});
  if (attr_d != cudaSuccess) return attr_d;
  static const int resident = resident_ctas(kx_stash_kernel<R, N>, Sh::NT, Sh::smem);
  PassArgs<R> a = a0;
  const int kzb = ((a.g.Hk + Sh::QW - 1) / Sh::QW + Sh::NG - 1) / Sh::NG;
  a.tiles = kzb * a.g.M * runs;
  const int ctas = resident > 0 ? std::min(a.tiles, resident) : a.tiles;
  if (a.g.K == N / 3) {  // default cutoff: geometry and RK4 stage at compile time
    switch (a.stage) {
      case 1: kx_stash_kernel<R, N, true, 1><<<ctas, Sh::NT, Sh::smem, st>>>(a); break;
      case 2: kx_stash_kernel<R, N, true, 2><<<ctas, Sh::NT, Sh::smem, st>>>(a); break;
      case 3: kx_stash_kernel<R, N, true, 3><<<ctas, Sh::NT, Sh::smem, st>>>(a); break;
      default: kx_stash_kernel<R, N, true, 4><<<ctas, Sh::NT, Sh::smem, st>>>(a); break;
    }
  } else {
    kx_stash_kernel<R, N><<<ctas, Sh::NT, Sh::smem, st>>>(a);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------ x pass, adjoint
// KX_ADJ_LOAD:   inverse-x of u, curl u of the state W (spec_in) and of a = P mu (mu in S)
//                -> 9 fields (u 0..2, omega 3..5, a 6..8); nout = 3 / 6: only a / only u, omega
// KX_ADJ_FWD:    forward-x of p (0..2), q (3..5) -> spec_out = F p + i k x F q (1/N^3 applied)
// KX_NL_FWD:     spec_out = P F(u x omega) / N^3 (the nonlinear term alone)
// Stage-tape forms (tp = the step tape V, n1, n2, n3; S = L, the adjoint of the step output):
// KX_ADJ_LOAD_T: stage s = a.stage: mu_s = cl L + cg g_{s+1} (g_{s+1} in acc), a = P mu_s
//                -> out2 (3 fields); u, curl u of the stage state a_s (from V, n_{s-1}) -> out
// KX_ADJ_FWD_T:  stage s: g_s as KX_ADJ_FWD (-> spec_out unless null); lam (vs) accumulated:
//                s = 4: lam = E(h) (L + g4);  s = 3, 2: lam += E(h/2) g_s;  s = 1: lam += g1;
//                d(loss)/d(nu) terms of the stage (w = 1 at kz = 0, else 2) -> part[CTA]:
//                s = 4: <g4, -k^2 h E(h) V - k^2 h^2/2 E(h/2) n3>
//                       + <L, -k^2 h E(h) V - k^2 h^2/6 (E(h) n1 + E(h/2) (n2 + n3))>
//                s = 3: <g3, -k^2 h/2 E(h/2) V>;  s = 2: <g2, -k^2 h/2 a2>, a2 = E(h/2)(V + h/2 n1)
template <typename R, int N, int MODE, bool DEFK = false>
__global__ void __launch_bounds__(KxRegShape<R, N>::NT, KxRegShape<R, N>::MINB) kx_reg_adj_kernel(const PassArgs<R> a) {
  using C = cplx<R>;
  using Sh = KxRegShape<R, N>;
  using Plan = typename Sh::Plan;
  constexpr int P = Sh::P, E = Sh::E, QW = Sh::QW, GT = Sh::GT, CS = Sh::CS;
  constexpr int NBL = N / (Plan::template radix<Plan::NPASS - 1>() * P);
  constexpr bool TAPE = (MODE == KX_ADJ_LOAD_T || MODE == KX_ADJ_FWD_T);
  constexpr bool HAS_FWD = (MODE == KX_ADJ_FWD || MODE == KX_ADJ_FWD_T);
  constexpr bool HAS_INV = (MODE == KX_ADJ_LOAD || MODE == KX_ADJ_LOAD_T);
  const Geo g = geo_of<N, DEFK>(a.g);
  const int K = g.K, M = g.M, Hz = g.Hz;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  const int grp = threadIdx.x / GT, lt = threadIdx.x % GT;
  const int col = lt % QW, t = lt / QW;
  const int iyc = blockIdx.x, run = blockIdx.z;
  const int kz0 = (blockIdx.y * Sh::NG + grp) * QW;
  const int kz = kz0 + col;
  const bool zok = kz < g.Hk;
  C* xcol = tw + N + (grp * QW + col) * CS;
  C* stg = tw + N + Sh::NG * QW * CS + grp * Sh::adj_area;  // this group's staging area
  // a group's barrier (its named barrier, or the warp when the group fits in one)
  auto gsync = [&]() {
    if constexpr (GT > 32) {
      const NamedSync ns{1 + grp, GT};
      ns();
    } else {
      __syncwarp();
    }
  };
  // cp.async staging: rows of QW consecutive kz are 32-byte aligned (Hz % 4 == 0); chunks
  // past the padded row (kz0 + 2h >= Hz) are skipped; a group without a valid
  // column copies nothing but still commits, so that the group counts stay uniform
  const bool gok = kz0 < g.Hk;
  // forward input f (rows x = 0..N-1 of the X-layout field at src) -> ring slot f % 4
  auto stage_x = [&](int f, const C* src) {
    C* d = stg + (f & 3) * N * QW;
    if (gok) {
      for (int c = lt; c < Sh::CPR * N; c += GT) {
        const int h = c % Sh::CPR, row = c / Sh::CPR;
        if (kz0 + 2 * h < Hz) cp_async16(d + row * QW + 2 * h, src + (long long)row * M * Hz + 2 * h);
      }
    }
    cp_async_commit();
  };
  // three spectral fields (rows (f, ic) of the compact layout at src) -> dst [3][M][QW]
  auto stage_spec = [&](C* dst, const C* src) {
    if (gok) {
      for (int c = lt; c < 3 * M * Sh::CPR; c += GT) {
        const int h = c % Sh::CPR, row = c / Sh::CPR;  // row = f * M + ic
        if (kz0 + 2 * h < Hz) cp_async16(dst + row * QW + 2 * h, src + (long long)row * M * Hz + 2 * h);
      }
    }
  };
  const long long soff0 = (long long)run * 3 * g.sS + (long long)iyc * Hz + kz0;
  const int st = a.stage;
  const C* const* tape = a.tp;
  // the state whose u, curl u the load part transforms: spec_in, or the tape's stage state
  // a_st, formed from V (tp[0]) and n_{st-1}
  auto stage_state = [&]() {
    if constexpr (TAPE) {
      stage_spec(stg, tape[0] + soff0);
      if (st > 1) stage_spec(stg + 3 * M * QW, tape[st - 1] + soff0);
    } else {
      stage_spec(stg, a.spec_in + soff0);
    }
    cp_async_commit();
  };
  // the first copies are issued before the twiddles are built
  if constexpr (MODE == KX_NL_FWD) {
    const C* win = a.in + (long long)run * 3 * g.sX + (long long)iyc * Hz + kz0;
    for (int f = 0; f < 3; ++f) stage_x(f, win + f * g.sX);
  } else if constexpr (HAS_FWD) {
    const C* win = a.in + (long long)run * 6 * g.sX + (long long)iyc * Hz + kz0;
    for (int f = 0; f < 4; ++f) stage_x(f, win + f * g.sX);
  } else {
    if (a.nout != 6) {  // mu = cl L + cg g_{st+1}: L (S) and, below stage 4, g (acc)
      stage_spec(stg, a.S + soff0);
      if (TAPE && st != 4) stage_spec(stg + 3 * M * QW, a.acc + soff0);
      cp_async_commit();
    } else {
      stage_state();
    }
  }
  build_twiddles<Plan>(tw, a.tw, threadIdx.x, Sh::NT);
  const float kyf = float(ksigned(iyc, K)), kzf = float(kz);
  // the integrating factors exactly as the forward x stage forms them (its per-CTA tables of
  // expm1 over kx^2 and over ky^2 + kz^2 of the columns, combined by expm1_add)
  C* ftab = tw + N + Sh::NG * QW * CS + Sh::NG * Sh::adj_area;
  if constexpr (TAPE) {
    const RunCoef cf0 = a.coef[run];
    const R c1 = R(cf0.nu * cf0.dt), ch = R(0.5) * c1;
    for (int i = threadIdx.x; i < M + Sh::NG * QW; i += Sh::NT) {
      R k2;
      if (i < M) {
        const R kx = R(ksigned(i, K));
        k2 = kx * kx;
      } else {
        const R kc = R(blockIdx.y * Sh::NG * QW + (i - M));
        k2 = R(kyf * kyf) + kc * kc;
      }
      ftab[i] = mk<C>(rexpm1<R>(-c1 * k2), rexpm1<R>(-ch * k2));
    }
  }
  __syncthreads();
  const long long soff = soff0 + col;
  const RunCoef cf = a.coef[run];
  const R h = R(cf.dt);
  auto run_fft = [&](auto& src, auto& dst, auto dir_tag) {
    constexpr int DIR = decltype(dir_tag)::value;
    if constexpr (GT > 32) {
      const NamedSync ns{1 + grp, GT};
      fft_column<Plan, DIR, Sh::PSH, false>(t, src, dst, xcol, tw, ns);
    } else {
      const WarpSync ws;
      fft_column<Plan, DIR, Sh::PSH, false>(t, src, dst, xcol, tw, ws);
    }
  };
  using Fwd = std::integral_constant<int, -1>;
  using Inv = std::integral_constant<int, +1>;
  const R inv_n3 = R(1) / (R(N) * R(N) * R(N));
  // k^2 and the Lawson factors expm1(-nu k^2 h), expm1(-nu k^2 h / 2) of mode (ic, iyc, kz)
  // (tape forms: from the tables above)
  auto factors = [&](int ic, R& kk, R& m1, R& mh) {
    const float kx = float(ksigned(ic, K));
    kk = R(kx * kx + kyf * kyf + kzf * kzf);
    const C fx = ftab[ic], fyz = ftab[M + grp * QW + col];
    m1 = expm1_add(fx.x, fyz.x);
    mh = expm1_add(fx.y, fyz.y);
  };
  // adjoint seeds of the stage nonlinear terms: mu_s = cl L + cg g_{s+1}
  auto seeds = [&](int s, R e1, R eh, R& cl, R& cg) {
    if (s == 4) { cl = h / R(6); cg = R(0); }
    else if (s == 3) { cl = h / R(3) * eh; cg = h * eh; }
    else if (s == 2) { cl = h / R(3) * eh; cg = R(0.5) * h; }
    else { cl = h / R(6) * e1; cg = R(0.5) * h * eh; }
  };

  if constexpr (MODE == KX_NL_FWD) {  // spec_out = P F(u x omega) / N^3 (nonlinear term alone)
    C nv[3][E];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      if (f == 0) cp_async_wait<2>();
      else if (f == 1) cp_async_wait<1>();
      else cp_async_wait_all();
      gsync();
      const C* sl = stg + f * N * QW + col;
      auto src = [&](int xx, int) -> C { return zok ? sl[xx * QW] : czero<C>(); };
      auto dst = [&](int b, int r, int, C val) { nv[f][b + r * NBL] = cscale(val, inv_n3); };
      run_fft(src, dst, Fwd());
    }
#pragma unroll
    for (int q = 0; q < E; ++q) {
      const int ic = kcompact_slot<N, P>(t, q, K);
      if (zok && ic >= 0) {
        const float kx = float(ksigned(ic, K));
        leray(nv[0][q], nv[1][q], nv[2][q], kx, kyf, kzf, kx * kx + kyf * kyf + kzf * kzf);
#pragma unroll
        for (int f = 0; f < 3; ++f) a.spec_out[soff + ((long long)f * M + ic) * M * Hz] = nv[f][q];
      }
    }
    return;
  }

  C acc[3][E];  // g_s (forward part) or mu (projected, load part)
  if constexpr (HAS_FWD) {
    C z[E];
    const C* win = a.in + (long long)run * 6 * g.sX + (long long)iyc * Hz + kz0;
    // inputs 0..3 were issued at entry; 4 and 5 reuse the ring slots of 0 and 1 once their
    // transforms are done.  Commit order 0 1 2 3 4 5, so before transform f the copies of
    // f + 1 .. min(f + 3, 5) may still be in flight.
    auto fwd_to = [&](int f, auto* dstarr) {
      if (f <= 2) cp_async_wait<3>();
      else if (f == 3) cp_async_wait<2>();
      else if (f == 4) cp_async_wait<1>();
      else cp_async_wait_all();
      gsync();
      const C* sl = stg + (f & 3) * N * QW + col;
      auto src = [&](int xx, int) -> C { return zok ? sl[xx * QW] : czero<C>(); };
      auto dst = [&](int b, int r, int, C val) { dstarr[b + r * NBL] = cscale(val, inv_n3); };
      run_fft(src, dst, Fwd());
      if (f <= 1) {  // slot f is free once every thread of the group is past the transform
        gsync();
        stage_x(f + 4, win + (f + 4) * g.sX);
      }
    };
    fwd_to(0, acc[0]);
    fwd_to(1, acc[1]);
    fwd_to(2, acc[2]);
    // + i k x F q, one component of q at a time
    auto add_curl = [&](auto c_tag) {
      constexpr int c = decltype(c_tag)::value;
      fwd_to(3 + c, z);
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int ic = kcompact_slot<N, P>(t, q, K);
        const float kx = float(ksigned(ic < 0 ? 0 : ic, K));
        const float kk[3] = {kx, kyf, kzf};
        // (k x e_c q)_{c+1} = k_{c+2} q,  (k x e_c q)_{c+2} = -k_{c+1} q; then times i
        constexpr int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
        const C iz = cmul_i(z[q]);
        acc[c1][q] = mk<C>(acc[c1][q].x + R(kk[c2]) * iz.x, acc[c1][q].y + R(kk[c2]) * iz.y);
        acc[c2][q] = mk<C>(acc[c2][q].x - R(kk[c1]) * iz.x, acc[c2][q].y - R(kk[c1]) * iz.y);
      }
    };
    if constexpr (N >= 128) {  // one FFT body for the three q components (instruction cache)
#pragma unroll 1
      for (int c = 0; c < 3; ++c) {
        switch (c) {
          case 0: add_curl(std::integral_constant<int, 0>()); break;
          case 1: add_curl(std::integral_constant<int, 1>()); break;
          default: add_curl(std::integral_constant<int, 2>()); break;
        }
      }
    } else {
      add_curl(std::integral_constant<int, 0>());
      add_curl(std::integral_constant<int, 1>());
      add_curl(std::integral_constant<int, 2>());
    }
    double dsum = 0.0;
    if constexpr (!TAPE) {
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int ic = kcompact_slot<N, P>(t, q, K);
        if (zok && ic >= 0) {
#pragma unroll
          for (int f = 0; f < 3; ++f) a.spec_out[soff + ((long long)f * M + ic) * M * Hz] = acc[f][q];
        }
      }
    } else {
      // the stage is a compile-time constant inside (no branches between the loads), the
      // buffers are distinct (restrict), and each mode's loads are issued before its
      // arithmetic, so that the loads of several modes are in flight together
      auto epilogue = [&](auto st_tag) {
        constexpr int S = decltype(st_tag)::value;
        const C* __restrict__ Lp = a.S;
        const C* __restrict__ t0 = a.tp[0];
        const C* __restrict__ t1 = a.tp[1];
        const C* __restrict__ t2 = a.tp[2];
        const C* __restrict__ t3 = a.tp[3];
        C* __restrict__ lamp = a.vs;
        C* __restrict__ gout = a.spec_out;
#pragma unroll
        for (int q = 0; q < E; ++q) {
          const int ic = kcompact_slot<N, P>(t, q, K);
          if (zok && ic >= 0) {
            long long o[3];
            C l[3], v[3], y1[3], y2[3], y3[3];
#pragma unroll
            for (int f = 0; f < 3; ++f) {
              o[f] = soff + ((long long)f * M + ic) * M * Hz;
              l[f] = (S == 4) ? Lp[o[f]] : lamp[o[f]];  // L at stage 4, else the lam so far
              if constexpr (S >= 2) v[f] = t0[o[f]];
              if constexpr (S == 4 || S == 2) y1[f] = t1[o[f]];
              if constexpr (S == 4) {
                y2[f] = t2[o[f]];
                y3[f] = t3[o[f]];
              }
            }
            R kk, m1, mh;
            factors(ic, kk, m1, mh);
            const R e1 = R(1) + m1, eh = R(1) + mh;
            R dn = R(0);
#pragma unroll
            for (int f = 0; f < 3; ++f) {
              const C gs = acc[f][q];
              if (gout != nullptr) gout[o[f]] = gs;
              C lam;
              if constexpr (S == 4) {
                lam = mk<C>(e1 * (l[f].x + gs.x), e1 * (l[f].y + gs.y));
              } else {
                const R c = (S == 1) ? R(1) : eh;
                lam = mk<C>(l[f].x + c * gs.x, l[f].y + c * gs.y);
              }
              lamp[o[f]] = lam;
              if constexpr (S == 4) {
                const C vv = v[f], a1 = y1[f], a2 = y2[f], a3 = y3[f], ll = l[f];
                const R b4x = -kk * h * e1 * vv.x - kk * R(0.5) * h * h * eh * a3.x;
                const R b4y = -kk * h * e1 * vv.y - kk * R(0.5) * h * h * eh * a3.y;
                const R bLx = -kk * h * e1 * vv.x - kk * h * h / R(6) * (e1 * a1.x + eh * (a2.x + a3.x));
                const R bLy = -kk * h * e1 * vv.y - kk * h * h / R(6) * (e1 * a1.y + eh * (a2.y + a3.y));
                dn += gs.x * b4x + gs.y * b4y + ll.x * bLx + ll.y * bLy;
              } else if constexpr (S == 3) {
                const R c3 = -kk * R(0.5) * h * eh;
                dn += c3 * (gs.x * v[f].x + gs.y * v[f].y);
              } else if constexpr (S == 2) {
                const C vv = v[f], a1 = y1[f];
                const R a2x = vv.x + (mh * vv.x + eh * R(0.5) * h * a1.x);
                const R a2y = vv.y + (mh * vv.y + eh * R(0.5) * h * a1.y);
                dn += -kk * R(0.5) * h * (gs.x * a2x + gs.y * a2y);
              }
            }
            dsum += (kz == 0 ? 1.0 : 2.0) * double(dn);
          }
        }
      };
      switch (st) {
        case 4: epilogue(std::integral_constant<int, 4>()); break;
        case 3: epilogue(std::integral_constant<int, 3>()); break;
        case 2: epilogue(std::integral_constant<int, 2>()); break;
        default: epilogue(std::integral_constant<int, 1>()); break;
      }
    }
    if constexpr (TAPE) {
      // the host allocates M x ceil(Hk / 4) partial-sum slots per stage
      static_assert(QW % 4 == 0, "partial-sum slots assume at least four kz columns per group");
      if (st >= 2 && a.part != nullptr) {  // CTA sum in a fixed order: warp tree, then the warps
        __shared__ double wsum[Sh::NT / 32];
        for (int o = 16; o > 0; o >>= 1) dsum += __shfl_down_sync(0xffffffffu, dsum, o);
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = dsum;
        __syncthreads();
        if (threadIdx.x == 0) {
          double tot = 0.0;
          for (int w = 0; w < Sh::NT / 32; ++w) tot += wsum[w];
          a.part[blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z)] = tot;
        }
      }
    }
  }

  if constexpr (HAS_INV) {
    // a = P mu first (its three transforms retire the mu registers), then u, curl u of the
    // state: one three-field array live at a time.  nout = 9 writes u, omega into out and a
    // into out2 (tape forms) or into out's fields 6..8; nout = 3 only a, nout = 6 only u, omega.
    const int sl = st;  // load stage
    C* xo = a.out + (long long)run * a.nout * g.sX + (long long)iyc * Hz + kz;
    const int gi0 = (a.nout == 3) ? 6 : 0;  // output field of GI = gi0 + slot
    C* xa = (TAPE && a.nout == 9) ? a.out2 + (long long)iyc * Hz + kz - 6 * g.sX : xo - gi0 * g.sX;
    // field gi of (u, omega, a) -> its inverse-x transform.  The values of this thread's
    // modes are formed by a switch with compile-time register indices; at N >= 128 the
    // fields loop over one FFT body (instruction cache), smaller transforms are unrolled.
    auto field = [&](int gi, auto* arr) {
      C in[E];
      auto fill = [&](auto gi_tag) {
        constexpr int GI = decltype(gi_tag)::value;
#pragma unroll
        for (int q = 0; q < E; ++q) {
          const int ic = kcompact_slot<N, P>(t, q, K);
          if constexpr (GI < 6) in[q] = (ic < 0) ? czero<C>() : uw_field<GI>(arr, q, float(ksigned(ic, K)), kyf, kzf);
          else in[q] = (ic < 0) ? czero<C>() : arr[GI - 6][q];
        }
      };
      switch (gi) {
        case 0: fill(std::integral_constant<int, 0>()); break;
        case 1: fill(std::integral_constant<int, 1>()); break;
        case 2: fill(std::integral_constant<int, 2>()); break;
        case 3: fill(std::integral_constant<int, 3>()); break;
        case 4: fill(std::integral_constant<int, 4>()); break;
        case 5: fill(std::integral_constant<int, 5>()); break;
        case 6: fill(std::integral_constant<int, 6>()); break;
        case 7: fill(std::integral_constant<int, 7>()); break;
        default: fill(std::integral_constant<int, 8>()); break;
      }
      C* xg = (gi >= 6) ? xa + gi * g.sX : xo + (gi - gi0) * g.sX;
      auto src = [&](int, int q) -> C { return in[q]; };
      auto dst = [&](int, int, int xx, C val) {
        if (zok) xg[(long long)xx * M * Hz] = val;
      };
      run_fft(src, dst, Inv());
    };
    if (a.nout != 6) {  // the staged L (and g) tiles
      cp_async_wait_all();
      gsync();
    }
    {  // mu (projected) into acc: plain S, or the tape seeds
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int ic = kcompact_slot<N, P>(t, q, K);
        const bool ok = zok && ic >= 0;
        R cl = R(1), cg = R(0);
        if (TAPE && ok) {
          R kk, m1, mh;
          factors(ic, kk, m1, mh);
          seeds(sl, R(1) + m1, R(1) + mh, cl, cg);
        }
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          C m = czero<C>();
          if (ok && a.nout != 6) {
            const C l = stg[((long long)f * M + ic) * QW + col];
            m = mk<C>(cl * l.x, cl * l.y);
            if (TAPE && sl != 4) {
              const C gp = stg[((long long)(3 + f) * M + ic) * QW + col];
              m = mk<C>(m.x + cg * gp.x, m.y + cg * gp.y);
            }
          }
          acc[f][q] = m;
        }
        if (ok && a.nout != 6) {
          const float kx = float(ksigned(ic, K));
          leray(acc[0][q], acc[1][q], acc[2][q], kx, kyf, kzf, kx * kx + kyf * kyf + kzf * kzf);
        }
      }
    }
    if (a.nout != 6) {
      if (a.nout != 3) {  // the tiles of mu are consumed: stage the state during a's transforms
        gsync();
        stage_state();
      }
      if constexpr (N >= 128) {
#pragma unroll 1
        for (int gi = 6; gi < 9; ++gi) field(gi, acc);
      } else {
#pragma unroll
        for (int gi = 6; gi < 9; ++gi) field(gi, acc);
      }
    }
    if (a.nout != 3) {
      // the state whose u, curl u are transformed: spec_in, or the tape's stage state a_sl
      cp_async_wait_all();
      gsync();
      C v[3][E];
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int ic = kcompact_slot<N, P>(t, q, K);
        const bool ok = zok && ic >= 0;
        R kk = R(0), m1 = R(0), mh = R(0);
        if (TAPE && ok && sl > 1) factors(ic, kk, m1, mh);
        const R eh = R(1) + mh;
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          C x = czero<C>();
          if (ok) {
            x = stg[((long long)f * M + ic) * QW + col];
            if (TAPE && sl > 1) {
              const C nn = stg[((long long)(3 + f) * M + ic) * QW + col];
              R dx, dy;
              if (sl == 2) { dx = mh * x.x + eh * R(0.5) * h * nn.x; dy = mh * x.y + eh * R(0.5) * h * nn.y; }
              else if (sl == 3) { dx = mh * x.x + R(0.5) * h * nn.x; dy = mh * x.y + R(0.5) * h * nn.y; }
              else { dx = m1 * x.x + h * eh * nn.x; dy = m1 * x.y + h * eh * nn.y; }
              x = mk<C>(x.x + dx, x.y + dy);
            }
          }
          v[f][q] = x;
        }
      }
      if constexpr (N >= 128) {
#pragma unroll 1
        for (int gi = 0; gi < 6; ++gi) field(gi, v);
      } else {
#pragma unroll
        for (int gi = 0; gi < 6; ++gi) field(gi, v);
      }
    }
  }
}

template <typename R, int N, int MODE>
static cudaError_t launch_kx_reg_adj(const PassArgs<R>& a, int runs, cudaStream_t st) {
  using Sh = KxRegShape<R, N>;
  static cudaError_t attr = set_smem(kx_reg_adj_kernel<R, N, MODE>, Sh::smem_adj);
  if (attr != cudaSuccess) return attr;
  static cudaError_t attr_d = set_smem(kx_reg_adj_kernel<R, N, MODE, true>, Sh::smem_adj);
  if (attr_d != cudaSuccess) return attr_d;
  const int quads = (a.g.Hk + Sh::QW - 1) / Sh::QW;
  dim3 grid(a.g.M, (quads + Sh::NG - 1) / Sh::NG, runs);
  if (a.g.K == N / 3) kx_reg_adj_kernel<R, N, MODE, true><<<grid, Sh::NT, Sh::smem_adj, st>>>(a);
  else kx_reg_adj_kernel<R, N, MODE><<<grid, Sh::NT, Sh::smem_adj, st>>>(a);
  return cudaGetLastError();
}

template <typename R, int N>
static cudaError_t launch_kz_reg(const PassArgs<R>& a, int runs, cudaStream_t st) {
  using Sh = KzRegShape<R, N>;
  static cudaError_t attr = set_smem(kz_reg_kernel<R, N>, Sh::smem);
  if (attr != cudaSuccess) return attr;
  static cudaError_t attr_d = set_smem(kz_reg_kernel<R, N, true>, Sh::smem);
  if (attr_d != cudaSuccess) return attr_d;
  const int pairs = N * N / 2;
  dim3 grid(pairs / Sh::LP, runs);
  if (a.g.K == N / 3) kz_reg_kernel<R, N, true><<<grid, Sh::NT, Sh::smem, st>>>(a);
  else kz_reg_kernel<R, N><<<grid, Sh::NT, Sh::smem, st>>>(a);
  return cudaGetLastError();
}

template <typename R, int N, int MODE>
static cudaError_t launch_kx_reg(const PassArgs<R>& a0, int runs, cudaStream_t st) {
  using Sh = KxRegShape<R, N>;
  static cudaError_t attr = set_smem(kx_reg_kernel<R, N, MODE>, Sh::smem);
  if (attr != cudaSuccess) return attr;
  static cudaError_t attr_d = set_smem(kx_reg_kernel<R, N, MODE, true>, Sh::smem);
  if (attr_d != cudaSuccess) return attr_d;
  if constexpr (MODE == KX_STAGE) {
    static cudaError_t attr_s = first_error({set_smem(kx_reg_kernel<R, N, MODE, true, 1>, Sh::smem1),
                                             set_smem(kx_reg_kernel<R, N, MODE, true, 2>, Sh::smem),
                                             set_smem(kx_reg_kernel<R, N, MODE, true, 3>, Sh::smem),
                                             set_smem(kx_reg_kernel<R, N, MODE, true, 4>, Sh::smem)});
    if (attr_s != cudaSuccess) return attr_s;
  }
  static const int resident = resident_ctas(kx_reg_kernel<R, N, MODE>, Sh::NT, Sh::smem);
  PassArgs<R> a = a0;
  const int kzb = ((a.g.Hk + Sh::QW - 1) / Sh::QW + Sh::NG - 1) / Sh::NG;
  a.tiles = kzb * a.g.M * runs;
  int ctas = a.tiles;  // one tile per CTA
  if (MODE == KX_STAGE && Sh::PERSIST && resident > 0) ctas = std::min(a.tiles, resident);
  if (MODE == KX_STAGE && a.g.K == N / 3) {  // default cutoff: geometry and RK4 stage at compile time
    switch (a.stage) {
      case 1: kx_reg_kernel<R, N, MODE, true, 1><<<ctas, Sh::NT, Sh::smem1, st>>>(a); break;
      case 2: kx_reg_kernel<R, N, MODE, true, 2><<<ctas, Sh::NT, Sh::smem, st>>>(a); break;
      case 3: kx_reg_kernel<R, N, MODE, true, 3><<<ctas, Sh::NT, Sh::smem, st>>>(a); break;
      default: kx_reg_kernel<R, N, MODE, true, 4><<<ctas, Sh::NT, Sh::smem, st>>>(a); break;
    }
  } else if (a.g.K == N / 3) {
    kx_reg_kernel<R, N, MODE, true><<<ctas, Sh::NT, Sh::smem, st>>>(a);
  } else {
    kx_reg_kernel<R, N, MODE><<<ctas, Sh::NT, Sh::smem, st>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace tg

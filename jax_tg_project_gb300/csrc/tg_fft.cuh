// In-register DFT codelets and the shared-memory Stockham pass engine used by
// every transform pass of the Taylor-Green time step.
//
// A length-N transform is executed by P cooperating threads ("one column").
// It is a sequence of radix-R passes (N = R_0 * R_1 * ...), each thread doing
// N/(R*P) radix-R butterflies per pass, in the self-sorting Stockham order of
// Govindaraju et al. (SC 2008): pass with sub-length Ns reads
// x[j + r*N/R], multiplies by W_{Ns*R}^{(j mod Ns) r}, does a radix-R DFT and
// writes y[(j/Ns)*Ns*R + (j mod Ns) + r*Ns].  The first pass reads through a
// caller functor (global memory, Hermitian packing, a spectral formula ...),
// the last pass hands each result to a caller functor; intermediate data sit
// in a padded shared-memory column.  Twiddles come from a table generated in
// FP64 on the host, rearranged per pass in shared memory (build_twiddles).
#pragma once

#include <cuda_runtime.h>

#include "tg_consts.cuh"

namespace tg {

// ------------------------------------------------------------------ complex
template <typename R> struct CplxT;
template <> struct CplxT<float> { using T = float2; };
template <> struct CplxT<double> { using T = double2; };
template <typename R> using cplx = typename CplxT<R>::T;

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) a, decltype(C::x) b) {
  C c; c.x = a; c.y = b; return c;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
  return mk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C> __device__ __forceinline__ C cscale(C a, decltype(C::x) s) { return mk<C>(a.x * s, a.y * s); }

// FP32: the two lanes of a complex add, subtract or real scaling in one packed
// instruction (add/sub/mul.rn.f32x2, sm_100 family); each lane rounds exactly like
// the scalar instruction, so results are unchanged
__device__ __forceinline__ unsigned long long pack2(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
  return unpack2(r);
}
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
  return unpack2(r);
}
template <> __device__ __forceinline__ float2 cscale<float2>(float2 a, float s) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(make_float2(s, s))));
  return unpack2(r);
}
// lane-wise a * b + c (one rounding per lane) and -a (exact): the two lines of a packed pair
template <typename C> __device__ __forceinline__ C lane_fma(C a, C b, C c) {
  return mk<C>(a.x * b.x + c.x, a.y * b.y + c.y);
}
template <> __device__ __forceinline__ float2 lane_fma<float2>(float2 a, float2 b, float2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)), "l"(pack2(c)));
  return unpack2(r);
}
template <typename C> __device__ __forceinline__ C lane_neg(C a) { return cscale(a, decltype(C::x)(-1)); }
template <typename C> __device__ __forceinline__ C cconj(C a) { return mk<C>(a.x, -a.y); }
// multiply by i*s (s = +1 or -1 at compile time, or any real)
template <typename C> __device__ __forceinline__ C cmul_i(C a) { return mk<C>(-a.y, a.x); }
template <typename C> __device__ __forceinline__ C czero() { return mk<C>(0, 0); }

// W_R^m with sign DIR (-1 forward, +1 inverse), R | 96, folded at compile time
template <typename C, int R, int DIR>
__device__ __forceinline__ C wconst(int m) {
  using Re = decltype(C::x);
  const int q = (m % R) * (96 / R);
  return mk<C>(Re(kCos96(q)), Re(DIR * kSin96(q)));
}

// a * W_R^m (m a constant after unrolling): quarter turns are exact rotations, the
// others a complex multiply by the tabulated constant
template <typename C, int R, int DIR>
__device__ __forceinline__ C cmul_w(C a, int m) {
  const int q = (m % R) * (96 / R);
  if (q == 0) return a;
  if (q == 48) return mk<C>(-a.x, -a.y);
  if (q == 24) return (DIR > 0) ? mk<C>(-a.y, a.x) : mk<C>(a.y, -a.x);  // * i DIR
  if (q == 72) return (DIR > 0) ? mk<C>(a.y, -a.x) : mk<C>(-a.y, a.x);  // * -i DIR
  return cmul(a, wconst<C, R, DIR>(m));
}

// ------------------------------------------------------------------ codelets
template <int R> struct Split {
  static constexpr int A = (R % 4 == 0 && R > 4) ? 4 : ((R % 2 == 0 && R > 2) ? 2 : ((R % 3 == 0 && R > 3) ? 3 : R));
  static constexpr int B = R / A;
};

// In-place DFT of R values held in registers: X[k] = sum_n x[n] W_R^{nk},
// W_R = exp(DIR * 2 pi i / R).
template <int R, int DIR, typename C>
__device__ __forceinline__ void dft(C* v) {
  using Re = decltype(C::x);
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 3) {
    const Re h = Re(0.5), s = Re(DIR * 0.8660254037844386);  // sin(2 pi / 3)
    C a = v[0], b = v[1], c = v[2];
    C t1 = cadd(b, c);
    C t2 = mk<C>(a.x - h * t1.x, a.y - h * t1.y);
    C d = csub(b, c);
    C t3 = mk<C>(-s * d.y, s * d.x);  // i * s * (b - c)
    v[0] = cadd(a, t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  } else if constexpr (R == 4) {
    C a = v[0], b = v[1], c = v[2], d = v[3];
    C s0 = cadd(a, c), s1 = csub(a, c), s2 = cadd(b, d), s3 = csub(b, d);
    // i*DIR*(b-d)
    C r3 = (DIR > 0) ? mk<C>(-s3.y, s3.x) : mk<C>(s3.y, -s3.x);
    v[0] = cadd(s0, s2);
    v[1] = cadd(s1, r3);
    v[2] = csub(s0, s2);
    v[3] = csub(s1, r3);
  } else {
    constexpr int A = Split<R>::A, B = Split<R>::B;
    C t[R];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      C a[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) a[n1] = v[B * n1 + n2];
      dft<A, DIR>(a);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) {
        if (n2 * k1 == 0) {
          t[n2 * A + k1] = a[k1];
        } else {
          t[n2 * A + k1] = cmul_w<C, R, DIR>(a[k1], n2 * k1);
        }
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      C b[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) b[n2] = t[n2 * A + k1];
      dft<B, DIR>(b);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = b[k2];
    }
  }
}

// ------------------------------------------------------------------ plans
// N = product of the radices; P threads per transform.
template <int N_, int P_, int R0_, int R1_ = 1, int R2_ = 1>
struct FftPlan {
  static constexpr int N = N_, P = P_;
  static constexpr int NPASS = (R1_ == 1) ? 1 : ((R2_ == 1) ? 2 : 3);
  template <int I> __host__ __device__ static constexpr int radix() { return I == 0 ? R0_ : (I == 1 ? R1_ : R2_); }
  static_assert(R0_ * R1_ * R2_ == N_, "radices must multiply to N");
  static_assert((N_ / R0_) % P_ == 0 && (N_ / R1_) % P_ == 0 && (N_ / R2_) % P_ == 0,
                "P must divide N/R for every pass");
  static constexpr int E = N_ / P_;  // elements held per thread per pass
};

// Exchange-buffer index.  PSH >= 0: one spare slot every 2^PSH complex values.
// PSH == kSwizzle: no spare slots; the low four index bits (the 16 eight-byte
// bank pairs) are XORed with (n4, n5, n6, n4 ^ n5).  For the register plans
// (8,2,8) / (8,4,8) with P = 16 / 32 threads per transform (N = 128 / 256) every
// exchange store and load of a half warp then touches 16 distinct bank pairs.
constexpr int kSwizzle = -1;
template <int PSH = 4>
__device__ __forceinline__ int padx(int n) {
  if constexpr (PSH == kSwizzle) {
    const int h = n >> 4;
    return n ^ ((h & 7) | (((h ^ (h >> 1)) & 1) << 3));
  } else {
    return n + (n >> PSH);
  }
}
// per-column stride in complex elements, congruent to CSMOD modulo 16 (the 16
// eight-byte bank pairs), so that the columns of a CTA interleave banks
template <int N, int PSH = 4, int CSMOD = 1> struct ColLayout {
  static constexpr int PADN = (PSH == kSwizzle) ? N : N + (N >> PSH);
  static constexpr int CS = PADN + (((CSMOD - PADN) % 16) + 16) % 16;
};

// Per-pass twiddle tables: pass I (sub-length NS, radix R) uses W_{NS R}^{jm r}
// for jm < NS, 1 <= r < R, stored at offset (NS - R0) + (r - 1) NS + jm, so the
// threads of a warp (consecutive jm) read consecutive slots.  The blocks add up
// to N - R0 < N entries.  Values are copied from the FP64-generated W_N table.
template <class Plan, int I = 0, int NS = 1, typename C>
__device__ __forceinline__ void build_twiddles(C* dst, const C* wn, int tid, int nthr) {
  if constexpr (I < Plan::NPASS) {
    constexpr int R = Plan::template radix<I>();
    if constexpr (I > 0) {
      constexpr int OFF = NS - Plan::template radix<0>();
      for (int e = tid; e < (R - 1) * NS; e += nthr) {
        const int r = 1 + e / NS, jm = e % NS;
        dst[OFF + e] = wn[jm * r * (Plan::N / (NS * R))];
      }
    }
    build_twiddles<Plan, I + 1, NS * R>(dst, wn, tid, nthr);
  }
}

// j mod NS for j >= 0 (a mask for powers of two, so that jm of the butterflies
// b and b + 1 of a thread is seen to be equal when P is a multiple of NS)
template <int NS>
__device__ __forceinline__ int jmod(int j) {
  if constexpr ((NS & (NS - 1)) == 0) return j & (NS - 1);
  else return j % NS;
}

// Barriers between passes: the threads that share exchange columns.
struct CtaSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct WarpSync {
  __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
struct NamedSync {  // bar.sync on a named barrier shared by `count` threads (whole warps)
  int id, count;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
};

// Execute pass I of Plan for one column.
//   src(n, q)         -> value at input index n (pass 0 only); q = (n - t) / P
//   dst(b, r, k, v)   <- output v at index k (last pass); b, r compile-time
//   xb                -> this column's padded shared-memory buffer
//   tw                -> per-pass twiddle tables (build_twiddles), forward sign
//   sync()            -> barrier over every thread using the exchange columns
// Thread t reads exactly the inputs n = t (mod P) in pass 0 and holds exactly the
// outputs k = t (mod P) after the last pass (q = b + r*N/(R*P) in both), so a
// transform can take its input from, and leave its output in, registers.
// Twiddles held in registers (TWR): one thread's factors W_{NS R}^{jm r} of every pass after
// the first, read once from the per-pass tables and kept across all transforms the thread runs.
// Pass I occupies entries twr_offset<Plan, I>() + r - 1 (1 <= r < R); jm = t mod NS is the same
// for all butterflies of a thread when P is a multiple of NS (checked).
template <class Plan, int I>
__host__ __device__ constexpr int twr_offset() {
  if constexpr (I <= 1) return 0;
  else return twr_offset<Plan, I - 1>() + Plan::template radix<I - 1>() - 1;
}
template <class Plan> struct TwrCount {
  static constexpr int value = twr_offset<Plan, Plan::NPASS>();
};
template <class Plan, int I = 1, int NS = Plan::template radix<0>()>
__host__ __device__ constexpr bool twr_ok() {
  if constexpr (I >= Plan::NPASS) return true;
  else return (Plan::P % NS == 0) && twr_ok<Plan, I + 1, NS * Plan::template radix<I>()>();
}
template <class Plan, int I = 1, int NS = Plan::template radix<0>(), typename C>
__device__ __forceinline__ void load_twiddle_regs(C* wr, const C* tw, int t) {
  if constexpr (I < Plan::NPASS) {
    constexpr int R = Plan::template radix<I>();
    static_assert(Plan::P % NS == 0, "register twiddles need P to be a multiple of every pass's NS");
    constexpr int OFF = NS - Plan::template radix<0>();
    constexpr int OR = twr_offset<Plan, I>();
    const int jm = jmod<NS>(t);
#pragma unroll
    for (int r = 1; r < R; ++r) wr[OR + r - 1] = tw[OFF + (r - 1) * NS + jm];
    load_twiddle_regs<Plan, I + 1, NS * R>(wr, tw, t);
  }
}

template <class Plan, int DIR, int I, int NS, int PSH = 4, bool TWC = false, bool TWR = false, int XOFF = 0,
          bool FRESH = false, typename C, class Src, class Dst, class Sync = CtaSync>
__device__ __forceinline__ void fft_pass(int t, Src& src, Dst& dst, C* xb, const C* tw,
                                         const Sync& sync = Sync(), const C* wr = nullptr) {
  constexpr int N = Plan::N, P = Plan::P;
  constexpr int R = Plan::template radix<I>();
  constexpr int NB = N / (R * P);
  constexpr bool LAST = (I == Plan::NPASS - 1);
  // XOFF > 0: two exchange columns XOFF apart, pass I writing column I % 2.  With three passes
  // every transform writes the first, then the second, so a write to a column always follows a
  // barrier that every thread passed after its reads of that column: one barrier per exchange
  static_assert(XOFF == 0 || Plan::NPASS == 3, "double exchange columns need three passes");
  constexpr int ROFF = (XOFF > 0 && I > 0 && ((I - 1) & 1)) ? XOFF : 0;  // column read by pass I
  constexpr int WOFF = (XOFF > 0 && (I & 1)) ? XOFF : 0;                 // column written by pass I
  C v[NB][R];
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int j = t + P * b;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if constexpr (I == 0) {
        v[b][r] = src(j + r * (N / R), b + r * NB);
      } else {
        v[b][r] = xb[ROFF + padx<PSH>(j + r * (N / R))];
      }
    }
    if constexpr (I > 0) {
      const int jm = jmod<NS>(j);
      constexpr int OFF = NS - Plan::template radix<0>();
      C w[R];
      if constexpr (TWR) {
        constexpr int OR = twr_offset<Plan, I>();
#pragma unroll
        for (int r = 1; r < R; ++r) w[r] = wr[OR + r - 1];
      } else if constexpr (TWC && sizeof(w[0].x) == 4) {
        // read W^jm only and form W^(jm r) = W^(jm r/2) W^(jm (r - r/2)) in registers
        // (at most log2(R) products deep): fewer table reads on the shared-memory pipe
        w[1] = tw[OFF + jm];
        if constexpr (DIR > 0) w[1].y = -w[1].y;
#pragma unroll
        for (int r = 2; r < R; ++r) w[r] = cmul(w[r / 2], w[r - r / 2]);
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          w[r] = tw[OFF + (r - 1) * NS + jm];
          if constexpr (DIR > 0) w[r].y = -w[r].y;
        }
      }
#pragma unroll
      for (int r = 1; r < R; ++r) v[b][r] = (TWR && DIR > 0) ? cmulc(v[b][r], w[r]) : cmul(v[b][r], w[r]);
    }
    dft<R, DIR>(v[b]);
  }
  if constexpr (!LAST) {
    // every reader of xb (this or a previous transform) is done; FRESH: the column's only
    // transform, whose first exchange follows a barrier already (nobody has read xb yet)
    if constexpr (XOFF == 0 && !(FRESH && I == 0)) sync();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + P * b;
      const int jm = jmod<NS>(j);
      const int base = (j - jm) * R + jm;
#pragma unroll
      for (int r = 0; r < R; ++r) xb[WOFF + padx<PSH>(base + r * NS)] = v[b][r];
    }
    sync();
    fft_pass<Plan, DIR, I + 1, NS * R, PSH, TWC, TWR, XOFF>(t, src, dst, xb, tw, sync, wr);
  } else {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + P * b;
#pragma unroll
      for (int r = 0; r < R; ++r) dst(b, r, j + r * NS, v[b][r]);
    }
  }
}

template <class Plan, int DIR, int PSH = 4, bool TWC = false, int XOFF = 0, bool FRESH = false, typename C,
          class Src, class Dst, class Sync = CtaSync>
__device__ __forceinline__ void fft_column(int t, Src& src, Dst& dst, C* xb, const C* tw,
                                           const Sync& sync = Sync()) {
  fft_pass<Plan, DIR, 0, 1, PSH, TWC, false, XOFF, FRESH>(t, src, dst, xb, tw, sync);
}

// the same with the twiddles of every pass in registers (load_twiddle_regs)
template <class Plan, int DIR, int PSH = 4, typename C, class Src, class Dst, class Sync>
__device__ __forceinline__ void fft_column_wr(int t, Src& src, Dst& dst, C* xb, const C* wr, const Sync& sync) {
  fft_pass<Plan, DIR, 0, 1, PSH, false, true>(t, src, dst, xb, wr, sync, wr);
}

// register slot q of the output (b, r) of the last pass
template <class Plan>
__host__ __device__ constexpr int out_slot(int b, int r) {
  return b + r * (Plan::N / (Plan::template radix<Plan::NPASS - 1>() * Plan::P));
}

// index of output element (b, r) held by thread t after the last pass
template <class Plan>
__device__ __forceinline__ int out_index(int t, int b, int r) {
  constexpr int R = Plan::template radix<Plan::NPASS - 1>();
  constexpr int NS = Plan::N / R;
  return t + Plan::P * b + r * NS;
}

}  // namespace tg

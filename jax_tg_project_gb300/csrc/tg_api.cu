// Plan, run loop, diagnostics / initial-condition kernels and the C ABI
// (include/tgdns.h) of the GB300-native Taylor-Green time step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <new>
#include <string>
#include <vector>

#include "../../include/tgdns.h"
#include "tg_common.cuh"

namespace tg {

// pass-kernel launchers, one per instantiated (real type, size): tg_inst.cu
#define TG_SIZES_F32(X) X(float, 8) X(float, 12) X(float, 16) X(float, 24) X(float, 32) X(float, 48) \
  X(float, 64) X(float, 96) X(float, 128) X(float, 256) X(float, 512)
#define TG_SIZES_F64(X) X(double, 8) X(double, 16) X(double, 32) X(double, 64) X(double, 96) \
  X(double, 128) X(double, 256)
#define TG_DECL(R, N) cudaError_t launch_##R##_##N(int, const PassArgs<R>&, int, cudaStream_t); \
  int yconfs_##R##_##N();
TG_SIZES_F32(TG_DECL)
TG_SIZES_F64(TG_DECL)
#undef TG_DECL

enum PassOpHost {
  OP_KX_STAGE3 = 0, OP_KX_STAGE6, OP_KX_LOAD3, OP_KX_LOAD6, OP_KX_FWD3, OP_KX_FWD6,
  OP_KY_INV, OP_KY_FWD, OP_KZ_PROD_HD, OP_KZ_PROD_MHD, OP_KZ_C2R, OP_KZ_R2C, OP_KZ_ADJ,
  OP_KX_ADJ_LOAD, OP_KX_ADJ_FWD, OP_KX_NL_FWD
};

// sizes whose FP32 build has the register-resident adjoint x / z passes
static bool has_reg_adjoint(int n) { return n == 16 || n == 32 || n == 64 || n == 128 || n == 256; }

template <typename R> using LaunchFn = cudaError_t (*)(int, const PassArgs<R>&, int, cudaStream_t);

static LaunchFn<float> find_f32(int n) {
  switch (n) {
#define TG_CASE(R, N) case N: return &launch_##R##_##N;
    TG_SIZES_F32(TG_CASE)
#undef TG_CASE
    default: return nullptr;
  }
}
static LaunchFn<double> find_f64(int n) {
  switch (n) {
#define TG_CASE(R, N) case N: return &launch_##R##_##N;
    TG_SIZES_F64(TG_CASE)
#undef TG_CASE
    default: return nullptr;
  }
}
// y-pass configurations built for a size (1 where the autotuner has no alternatives)
static int yconf_count(int n, int prec) {
  switch (prec == TG_PREC_F64 ? -n : n) {
#define TG_CASE(R, N) case N: return yconfs_##R##_##N();
    TG_SIZES_F32(TG_CASE)
#undef TG_CASE
#define TG_CASE(R, N) case -N: return yconfs_##R##_##N();
    TG_SIZES_F64(TG_CASE)
#undef TG_CASE
    default: return 1;
  }
}

// ------------------------------------------------------------------ generic kernels
constexpr int kDiagBlocks = 304;  // at most two CTAs per SM
constexpr int kDiagThreads = 256;
constexpr int kNQ = 5;  // E_k, enstrophy, sum w k^2 |u|^2, E_m, H_c

// CTAs of diag_partial for a grid: one (kx, ky) row of the compact spectrum per warp and
// pass, at most kDiagBlocks
static int diag_blocks(const Geo& g) {
  const long long rows = (long long)g.M * g.M;
  return (int)std::min<long long>(kDiagBlocks, (rows + kDiagThreads / 32 - 1) / (kDiagThreads / 32));
}

struct Neumaier {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

// per-CTA partial sums of the five diagnostic terms: each warp takes whole (kx, ky) rows
// (lanes along kz), each thread sums its own modes in FP64 in a fixed order, then a fixed
// tree over the CTA
template <typename R>
__global__ void __launch_bounds__(kDiagThreads) diag_partial(const cplx<R>* S, Geo g, int F, double* part) {
  using C = cplx<R>;
  const int run = blockIdx.y;
  const C* base = S + (long long)run * F * g.sS;
  const int lane = threadIdx.x & 31;
  const int nw = kDiagThreads / 32;
  double q[kNQ] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int r = blockIdx.x * nw + (threadIdx.x >> 5); r < g.M * g.M; r += gridDim.x * nw) {
    const int ic = r / g.M, iyc = r - ic * g.M;
    const int kx = ksigned(ic, g.K), ky = ksigned(iyc, g.K);
    for (int kz = lane; kz < g.Hk; kz += 32) {
      double t[kNQ];
      diag_terms(base, g.sS, (long long)r * g.Hz + kz, kx, ky, kz, F, t);
#pragma unroll
      for (int i = 0; i < kNQ; ++i) q[i] += t[i];
    }
  }
  __shared__ double sh[kNQ][kDiagThreads];
  for (int i = 0; i < kNQ; ++i) sh[i][threadIdx.x] = q[i];
  __syncthreads();
  for (int s = kDiagThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int i = 0; i < kNQ; ++i) sh[i][threadIdx.x] += sh[i][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kNQ) part[((long long)run * gridDim.x + blockIdx.x) * kNQ + threadIdx.x] = sh[threadIdx.x][0];
}

// one CTA of kNQ warps per run: warp i sums quantity i over the nblk partials (lane l takes
// partials l, l + 32, ... with compensation, then a fixed shuffle tree), one record
__global__ void __launch_bounds__(32 * kNQ) diag_final(const double* part, int nblk, const RunCoef* coef,
                                                       const unsigned long long* amax, int namax, int F,
                                                       double* out) {
  const int run = blockIdx.x;
  const int i = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ double v[kNQ];
  Neumaier s;
  for (int b = lane; b < nblk; b += 32) s.add(part[((long long)run * nblk + b) * kNQ + i]);
  double x = s.value();
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if (lane == 0) v[i] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double* o = out + (long long)run * TG_DIAG_WIDTH;
    o[TG_D_KINETIC] = v[0];
    o[TG_D_ENSTROPHY] = v[1];
    o[TG_D_DISSIPATION] = coef[run].nu * v[2];
    o[TG_D_MAGNETIC] = (F == 6) ? v[3] : 0.0;
    o[TG_D_CROSS_HELICITY] = (F == 6) ? v[4] : 0.0;
    o[TG_D_TOTAL] = v[0] + ((F == 6) ? v[3] : 0.0);
    o[TG_D_DIVU_MAX] = (namax > 0) ? __longlong_as_double((long long)amax[run * namax]) : 0.0;
    o[TG_D_DIVB_MAX] = (namax > 1) ? __longlong_as_double((long long)amax[run * namax + 1]) : 0.0;
  }
}

__global__ void amax_to_double(const unsigned long long* amax, int count, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = __longlong_as_double((long long)amax[i]);
}

// analytic Fourier coefficients of the Taylor-Green fields (modes |k_i| = 1)
template <typename R>
__global__ void ic_kernel(cplx<R>* S, Geo g, int F, int batch, int kind, double b_amp) {
  using C = cplx<R>;
  const long long per_run = (long long)F * g.sS;
  const long long total = per_run * batch;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long r = idx % per_run;
    const int f = int(r / g.sS);
    const long long m = r % g.sS;
    const int kz = int(m % g.Hz);
    const int iyc = int((m / g.Hz) % g.M), ic = int(m / ((long long)g.Hz * g.M));
    const int kx = ksigned(ic, g.K), ky = ksigned(iyc, g.K);
    double re = 0.0, im = 0.0;
    if (kz == 1 && (kx == 1 || kx == -1) && (ky == 1 || ky == -1) && kind != TG_IC_ZERO) {
      const double sx = kx, sy = ky, sz = 1.0;
      const int c = f % 3;
      if (f < 3) {  // u = (sin x cos y cos z, -cos x sin y cos z, 0)
        if (c == 0) im = -sx / 8.0;
        if (c == 1) im = sy / 8.0;
      } else if (kind == TG_IC_MHD_REFERENCE) {
        if (c == 0) im = -b_amp * sx / 8.0;
        if (c == 1) im = b_amp * sy / 8.0;
      } else if (kind == TG_IC_MHD_EQUAL_ENERGY) {
        const double s = 1.0 / sqrt(3.0);
        if (c == 0) re = -s * sy * sz / 8.0;
        if (c == 1) re = -s * sx * sz / 8.0;
        if (c == 2) re = s * sx * sy / 4.0;
      }
    }
    C v;
    v.x = R(re);
    v.y = R(im);
    S[idx] = v;
  }
}

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  unsigned long long z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform53(unsigned long long h) {
  return (double(h >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

// Seeded divergence-free perturbation (unnormalised) of the velocity, written to
// P[run][3][M][M][Hz]; the definition is the one documented in include/tgdns.h.
template <typename R>
__global__ void pert_kernel(cplx<R>* P, Geo g, int batch, unsigned long long seed, double k0) {
  using C = cplx<R>;
  const long long per_run = (long long)g.M * g.M * g.Hk;
  const long long total = per_run * batch;
  const int N = g.n, H = g.n / 2 + 1;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int run = int(idx / per_run);
    const long long m = idx % per_run;
    const int kz = int(m % g.Hk);
    const int iyc = int((m / g.Hk) % g.M), ic = int(m / ((long long)g.Hk * g.M));
    int kx = ksigned(ic, g.K), ky = ksigned(iyc, g.K);
    // kz = 0 plane: the lower half takes the conjugate of its mirror mode
    const bool lower = (kz == 0) && (ky < 0 || (ky == 0 && kx < 0));
    const int gx = lower ? -kx : kx, gy = lower ? -ky : ky;
    const unsigned long long key = splitmix64(seed + (unsigned long long)run);
    const unsigned long long ix = (unsigned long long)((gx + N) % N), iy = (unsigned long long)((gy + N) % N);
    double gr[3], gi[3];
    for (int c = 0; c < 3; ++c) {
      const unsigned long long cnt = ((((unsigned long long)c * N + ix) * N + iy) * H + kz) * 2ull;
      const double u1 = uniform53(splitmix64(key ^ cnt));
      const double u2 = uniform53(splitmix64(key ^ (cnt + 1ull)));
      const double rr = sqrt(-2.0 * log(u1));
      const double th = 2.0 * 3.141592653589793 * u2;
      gr[c] = rr * cos(th);
      gi[c] = rr * sin(th);
    }
    const double fx = gx, fy = gy, fz = kz;
    const double k2 = fx * fx + fy * fy + fz * fz;
    const double k2s = (k2 == 0.0) ? 1.0 : k2;
    const double kdr = fx * gr[0] + fy * gr[1] + fz * gr[2];
    const double kdi = fx * gi[0] + fy * gi[1] + fz * gi[2];
    const double kk[3] = {fx, fy, fz};
    const double amp = (k2 == 0.0) ? 0.0 : sqrt(k2) * exp(-k2 / (k0 * k0));
    const long long base = (long long)run * 3 * g.sS + ((long long)ic * g.M + iyc) * g.Hz + kz;
    for (int c = 0; c < 3; ++c) {
      double vr = (gr[c] - kk[c] * kdr / k2s) * amp;
      double vi = (gi[c] - kk[c] * kdi / k2s) * amp;
      if (lower) vi = -vi;
      C v;
      v.x = R(vr);
      v.y = R(vi);
      P[base + c * g.sS] = v;
    }
  }
}

template <typename R>
__global__ void axpy_pert(cplx<R>* S, const cplx<R>* P, Geo g, int F, int batch, const double* scale) {
  const long long per = 3 * g.sS;
  const long long total = per * batch;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int run = int(idx / per);
    const long long o = (long long)run * F * g.sS + idx % per;
    const double s = scale[run];
    cplx<R> v = S[o];
    const cplx<R> p = P[idx];
    v.x = R(double(v.x) + s * double(p.x));
    v.y = R(double(v.y) + s * double(p.y));
    S[o] = v;
  }
}


// compact state -> full fftn layout (x N^3, Hermitian completion for kz > N/2)
template <typename R>
__global__ void to_full_kernel(const cplx<R>* S, cplx<R>* out, Geo g, int F, int batch) {
  using C = cplx<R>;
  const int N = g.n;
  const long long n3 = (long long)N * N * N;
  const long long total = n3 * F * batch;
  const double scale = double(N) * N * N;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long rf = idx / n3;  // run * F + f
    const long long m = idx % n3;
    const int kzr = int(m % N), kyr = int((m / N) % N), kxr = int(m / ((long long)N * N));
    double re = 0.0, im = 0.0;
    int ic, iyc, kz;
    bool conj = false, ok = false;
    if (kzr <= g.K) {
      ic = kcompact(kxr, N, g.K); iyc = kcompact(kyr, N, g.K); kz = kzr; ok = ic >= 0 && iyc >= 0;
    } else if (kzr >= N - g.K) {
      ic = kcompact((N - kxr) % N, N, g.K); iyc = kcompact((N - kyr) % N, N, g.K); kz = N - kzr;
      ok = ic >= 0 && iyc >= 0; conj = true;
    }
    if (ok) {
      const C v = S[rf * g.sS + ((long long)ic * g.M + iyc) * g.Hz + kz];
      re = double(v.x) * scale;
      im = (conj ? -double(v.y) : double(v.y)) * scale;
    }
    C o;
    o.x = R(re);
    o.y = R(im);
    out[idx] = o;
  }
}

// full fftn layout -> compact state (kept modes, / N^3); padding rows zeroed
template <typename R>
__global__ void from_full_kernel(const cplx<R>* full, cplx<R>* S, Geo g, int F, int batch) {
  using C = cplx<R>;
  const int N = g.n;
  const long long n3 = (long long)N * N * N;
  const long long total = g.sS * F * batch;
  const double inv = 1.0 / (double(N) * N * N);
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long rf = idx / g.sS;
    const long long m = idx % g.sS;
    const int kz = int(m % g.Hz), iyc = int((m / g.Hz) % g.M), ic = int(m / ((long long)g.Hz * g.M));
    C o;
    o.x = R(0);
    o.y = R(0);
    if (kz <= g.K) {
      const C v = full[rf * n3 + ((long long)kfull(ic, N, g.K) * N + kfull(iyc, N, g.K)) * N + kz];
      o.x = R(double(v.x) * inv);
      o.y = R(double(v.y) * inv);
    }
    S[idx] = o;
  }
}

// 0.5 <sum_c u_c^2> of physical fields, groups of 3 components: partial sums
template <typename R>
__global__ void __launch_bounds__(kDiagThreads) phys_energy_partial(const R* u, long long n3, double* part) {
  const int grp = blockIdx.y;  // (run * F + 3 * j) / 3
  const R* base = u + (long long)grp * 3 * n3;
  Neumaier q;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x) {
    const double a = base[i], b = base[n3 + i], c = base[2 * n3 + i];
    q.add(a * a + b * b + c * c);
  }
  __shared__ double sh[kDiagThreads];
  sh[threadIdx.x] = q.value();
  __syncthreads();
  for (int s = kDiagThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(long long)grp * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void phys_energy_final(const double* part, int nblk, int groups, long long n3, double* out) {
  const int grp = blockIdx.x * blockDim.x + threadIdx.x;
  if (grp >= groups) return;
  Neumaier s;
  for (int b = 0; b < nblk; ++b) s.add(part[(long long)grp * nblk + b]);
  out[grp] = 0.5 * s.value() / double(n3);
}

// ------------------------------------------------------------------ adjoint pointwise kernels
// All act on one run's compact fields [3][M][M][Hz]; k^2 from the mode index.
struct ModeIdx {
  int ic, iy, kz;
  long long o;
  double kx, ky, kzd, k2, w;
};
__device__ __forceinline__ bool mode_of(long long idx, const Geo& g, ModeIdx& m) {
  const long long total = (long long)g.M * g.M * g.Hk;
  if (idx >= total) return false;
  m.kz = int(idx % g.Hk);
  const long long r = idx / g.Hk;
  m.iy = int(r % g.M);
  m.ic = int(r / g.M);
  m.o = ((long long)m.ic * g.M + m.iy) * g.Hz + m.kz;
  m.kx = ksigned(m.ic, g.K);
  m.ky = ksigned(m.iy, g.K);
  m.kzd = m.kz;
  m.k2 = m.kx * m.kx + m.ky * m.ky + m.kzd * m.kzd;
  m.w = (m.kz == 0) ? 1.0 : 2.0;
  return true;
}

// Lawson stage states: s = 2: E(h/2)(V + h/2 n); s = 3: E(h/2) V + h/2 n; s = 4: E(h) V + h E(h/2) n
// (working precision; factors applied in the expm1 delta form like the forward kernels)
template <typename R> __device__ __forceinline__ R wexpm1(R x);
template <> __device__ __forceinline__ float wexpm1<float>(float x) { return expm1f(x); }
template <> __device__ __forceinline__ double wexpm1<double>(double x) { return expm1(x); }

template <typename R>
__global__ void lawson_stage_kernel(int s, const cplx<R>* V, const cplx<R>* n, cplx<R>* out, Geo g, double nu,
                                    double hd) {
  ModeIdx m;
  const R h = R(hd);
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; mode_of(idx, g, m);
       idx += (long long)gridDim.x * blockDim.x) {
    const R lin = R(nu * m.k2);
    const R m1 = wexpm1<R>(-lin * h), mh = wexpm1<R>(R(-0.5) * lin * h), eh = R(1) + mh;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const long long o = f * g.sS + m.o;
      const cplx<R> v = V[o], nn = n[o];
      R dx, dy;
      if (s == 2) { dx = mh * v.x + eh * R(0.5) * h * nn.x; dy = mh * v.y + eh * R(0.5) * h * nn.y; }
      else if (s == 3) { dx = mh * v.x + R(0.5) * h * nn.x; dy = mh * v.y + R(0.5) * h * nn.y; }
      else { dx = m1 * v.x + h * eh * nn.x; dy = m1 * v.y + h * eh * nn.y; }
      cplx<R> r;
      r.x = v.x + dx;
      r.y = v.y + dy;
      out[o] = r;
    }
  }
}

// adjoint seeds of the stage nonlinear terms
//   s = 4: mu = h/6 L;  s = 3: mu = h/3 E(h/2) L + h E(h/2) gp;  s = 2: mu = h/3 E(h/2) L + h/2 gp;
//   s = 1: mu = h/6 E(h) L + h/2 E(h/2) gp   (L = adjoint of the step output, gp = previous stage adjoint)
template <typename R>
__global__ void adj_mu_kernel(int s, const cplx<R>* L, const cplx<R>* gp, cplx<R>* mu, Geo g, double nu, double hd) {
  ModeIdx m;
  const R h = R(hd);
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; mode_of(idx, g, m);
       idx += (long long)gridDim.x * blockDim.x) {
    const R lin = R(nu * m.k2);
    const R e1 = R(1) + wexpm1<R>(-lin * h), eh = R(1) + wexpm1<R>(R(-0.5) * lin * h);
    R cl, cg;
    if (s == 4) { cl = h / R(6); cg = R(0); }
    else if (s == 3) { cl = h / R(3) * eh; cg = h * eh; }
    else if (s == 2) { cl = h / R(3) * eh; cg = R(0.5) * h; }
    else { cl = h / R(6) * e1; cg = R(0.5) * h * eh; }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const long long o = f * g.sS + m.o;
      cplx<R> r;
      r.x = cl * L[o].x;
      r.y = cl * L[o].y;
      if (s != 4) { r.x += cg * gp[o].x; r.y += cg * gp[o].y; }
      mu[o] = r;
    }
  }
}

// adjoint of the state at the start of the step:
//   lam = E(h) L + E(h/2) (g2 + g3) + E(h) g4 + g1
template <typename R>
__global__ void adj_lambda_kernel(const cplx<R>* L, const cplx<R>* g1, const cplx<R>* g2, const cplx<R>* g3,
                                  const cplx<R>* g4, cplx<R>* lam, Geo g, double nu, double hd) {
  ModeIdx m;
  const R h = R(hd);
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; mode_of(idx, g, m);
       idx += (long long)gridDim.x * blockDim.x) {
    const R lin = R(nu * m.k2);
    const R e1 = R(1) + wexpm1<R>(-lin * h), eh = R(1) + wexpm1<R>(R(-0.5) * lin * h);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const long long o = f * g.sS + m.o;
      cplx<R> r;
      r.x = e1 * (L[o].x + g4[o].x) + eh * (g2[o].x + g3[o].x) + g1[o].x;
      r.y = e1 * (L[o].y + g4[o].y) + eh * (g2[o].y + g3[o].y) + g1[o].y;
      lam[o] = r;
    }
  }
}

// d(loss)/d(nu) contribution of one step (block partial sums, FP64):
//   <g2, -k^2 h/2 a2> + <g3, -k^2 h/2 E(h/2) V> + <g4, -k^2 h E(h) V - k^2 h^2/2 E(h/2) n3>
//   + <L, -k^2 h E(h) V - k^2 h^2/6 (E(h) n1 + E(h/2) (n2 + n3))>,  <A,B> = sum_half w Re(A . conj B)
template <typename R>
__global__ void __launch_bounds__(kDiagThreads) adj_dnu_partial(const cplx<R>* L, const cplx<R>* V,
                                                                const cplx<R>* a2, const cplx<R>* n1,
                                                                const cplx<R>* n2, const cplx<R>* n3,
                                                                const cplx<R>* g2, const cplx<R>* g3,
                                                                const cplx<R>* g4, Geo g, double nu, double hd,
                                                                double* part) {
  // per mode in working precision, accumulated in FP64 (plain sum per thread, fixed tree per block)
  double acc_t = 0.0;
  ModeIdx m;
  const R h = R(hd);
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; mode_of(idx, g, m);
       idx += (long long)gridDim.x * blockDim.x) {
    const R kk = R(m.k2);
    const R lin = R(nu) * kk;
    const R e1 = R(1) + wexpm1<R>(-lin * h), eh = R(1) + wexpm1<R>(R(-0.5) * lin * h);
    R acc = R(0);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const long long o = f * g.sS + m.o;
      const cplx<R> v = V[o], x2 = a2[o], y1 = n1[o], y2 = n2[o], y3 = n3[o];
      const cplx<R> G2 = g2[o], G3 = g3[o], G4 = g4[o], LL = L[o];
      const R c2 = -kk * R(0.5) * h, c3 = -kk * R(0.5) * h * eh;
      acc += G2.x * c2 * x2.x + G2.y * c2 * x2.y;
      acc += G3.x * c3 * v.x + G3.y * c3 * v.y;
      const R b4x = -kk * h * e1 * v.x - kk * R(0.5) * h * h * eh * y3.x;
      const R b4y = -kk * h * e1 * v.y - kk * R(0.5) * h * h * eh * y3.y;
      acc += G4.x * b4x + G4.y * b4y;
      const R bLx = -kk * h * e1 * v.x - kk * h * h / R(6) * (e1 * y1.x + eh * (y2.x + y3.x));
      const R bLy = -kk * h * e1 * v.y - kk * h * h / R(6) * (e1 * y1.y + eh * (y2.y + y3.y));
      acc += LL.x * bLx + LL.y * bLy;
    }
    acc_t += m.w * double(acc);
  }
  __shared__ double sh[kDiagThreads];
  sh[threadIdx.x] = acc_t;
  __syncthreads();
  for (int s = kDiagThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// acc += fixed-order sum of n partials with one block of 256 threads: strided thread
// sums, a shuffle tree per warp, then the eight warp sums in turn
__global__ void __launch_bounds__(256) accumulate_partials_wide(const double* part, int n, double* acc) {
  __shared__ double ws[8];
  double v = 0.0;
  for (int b = threadIdx.x; b < n; b += 256) v += part[b];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += ws[w];
    *acc += t;
  }
}

// acc += fixed-order sum of nblk partials (one warp: strided lane sums, then a fixed
// shuffle tree, so the result does not depend on scheduling)
__global__ void accumulate_partials(const double* part, int nblk, double* acc) {
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += 32) v += part[b];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) *acc += v;
}

// gradient of the enstrophy 0.5 sum_half w |k x V|^2:  lam = k^2 V - k (k . V)
template <typename R>
__global__ void enstrophy_grad_kernel(const cplx<R>* V, cplx<R>* lam, Geo g) {
  ModeIdx m;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; mode_of(idx, g, m);
       idx += (long long)gridDim.x * blockDim.x) {
    const double kv[3] = {m.kx, m.ky, m.kzd};
    double dr = 0.0, di = 0.0;
    for (int f = 0; f < 3; ++f) {
      dr += kv[f] * double(V[f * g.sS + m.o].x);
      di += kv[f] * double(V[f * g.sS + m.o].y);
    }
    for (int f = 0; f < 3; ++f) {
      const long long o = f * g.sS + m.o;
      cplx<R> r;
      r.x = R(m.k2 * double(V[o].x) - kv[f] * dr);
      r.y = R(m.k2 * double(V[o].y) - kv[f] * di);
      lam[o] = r;
    }
  }
}

__global__ void copy_double(const double* src, double* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = *src;
}

// shell-summed energy spectrum E(k) = 0.5 sum_{round|k| = k} w |u_k|^2: per-block partial
// histograms in shared memory (fixed order inside a block), then a fixed-order sum over blocks
constexpr int kSpecBlocks = 64;
template <typename R>
__global__ void __launch_bounds__(256) spectrum_partial(const cplx<R>* S, Geo g, int F, int nbins, double* part) {
  extern __shared__ double hist[];
  const int run = blockIdx.y;
  const cplx<R>* base = S + (long long)run * F * g.sS;
  for (int i = threadIdx.x; i < 2 * nbins; i += blockDim.x) hist[i] = 0.0;
  __syncthreads();
  const long long total = (long long)g.M * g.M * g.Hk;
  // each thread owns a contiguous chunk; bins accumulate thread by thread in order
  const long long per_block = (total + gridDim.x - 1) / gridDim.x;
  const long long b0 = (long long)blockIdx.x * per_block, b1 = min(total, b0 + per_block);
  for (int tt = 0; tt < blockDim.x; ++tt) {
    // serialise the threads of a block so that the per-bin order is fixed
    if (threadIdx.x == tt) {
      for (long long idx = b0 + tt; idx < b1; idx += blockDim.x) {
        const int kz = int(idx % g.Hk);
        const long long r = idx / g.Hk;
        const int iyc = int(r % g.M), ic = int(r / g.M);
        const double kx = ksigned(ic, g.K), ky = ksigned(iyc, g.K);
        const int bin = int(floor(sqrt(kx * kx + ky * ky + double(kz) * kz) + 0.5));
        const double w = (kz == 0) ? 1.0 : 2.0;
        const long long o = ((long long)ic * g.M + iyc) * g.Hz + kz;
        // the per-mode squares of the scalar diagnostics (mode_sq), so that the bins sum
        // to their energies
        const double eu = double(mode_sq(base[o], base[g.sS + o], base[2 * g.sS + o]));
        const double eb = (F == 6) ? double(mode_sq(base[3 * g.sS + o], base[4 * g.sS + o], base[5 * g.sS + o])) : 0.0;
        if (bin < nbins) {
          hist[bin] += 0.5 * w * eu;
          hist[nbins + bin] += 0.5 * w * eb;
        }
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < 2 * nbins; i += blockDim.x)
    part[((long long)run * gridDim.x + blockIdx.x) * 2 * nbins + i] = hist[i];
}

__global__ void spectrum_final(const double* part, int nblk, int nbins, int F, double* out) {
  const int run = blockIdx.x;
  for (int i = threadIdx.x; i < nbins * (F == 6 ? 2 : 1); i += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += part[((long long)run * nblk + b) * 2 * nbins + i];
    out[(long long)run * nbins * (F == 6 ? 2 : 1) + i] = s;
  }
}
}  // namespace tg

// ====================================================================== plan
using namespace tg;

static thread_local std::string g_last_error;

namespace tg {
// lets other translation units of the library report through tg_last_error()
void set_last_error(const std::string& message) { g_last_error = message; }
// whether the pass kernels of an n^3 grid are built for a precision (TG_PREC_*)
bool size_built(int n, int prec) {
  return prec == TG_PREC_F64 ? (find_f64(n) != nullptr) : (find_f32(n) != nullptr);
}
}  // namespace tg

static int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
static int cuda_fail(cudaError_t e, const char* where) {
  return fail(TG_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define TG_CUDA(call, where)                      \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

struct ProfEvent {
  int op;
  cudaEvent_t start, stop;
};

struct tg_plan {
  Geo g{};
  int n = 0, K = 0, batch = 1, F = 3, G = 6, physics = 0, prec = 0, flags = 0;
  cudaStream_t st = nullptr;
  cudaStream_t cap = nullptr;  // private non-blocking stream used only to capture the step graph
  void* X = nullptr;    // [batch][G][N][M][Hz]
  void* Y = nullptr;    // [batch][G][N][N][Hz]; W aliases it
  void* Z = nullptr;    // [batch][F][N][N][Hz], right after Y in the same allocation
  void* tape = nullptr; // adjoint step tape written by the x stage kernels (batch 1), or null
  void* htape = nullptr;   // pinned host memory of the adjoint tape, kept for later calls
  size_t htape_bytes = 0;
  void* ACC = nullptr;  // [batch][F][M][M][Hz]
  void* VS = nullptr;   // explicit-viscosity stage state
  void* TW = nullptr;   // W_N^m
  double* part = nullptr;
  double* dtmp = nullptr;  // [batch][TG_DIAG_WIDTH] scratch record
  unsigned long long* amax = nullptr;
  RunCoef* coef = nullptr;
  std::vector<RunCoef> hcoef;
  LaunchFn<float> l32 = nullptr;
  LaunchFn<double> l64 = nullptr;
  cudaGraphExec_t step_exec = nullptr;
  cudaGraph_t step_graph = nullptr;
  const void* step_state = nullptr;
  int64_t launches = 0;
  int64_t scratch = 0;
  int variant = 0;  // pass variant: bit 0 shared-memory z passes, bit 1 shared-memory x passes
  int yconf = 0;    // y-pass configuration (radix plan, kz columns per CTA), 0 = default
  int nyconf = 1;   // configurations built for this size and precision
  // per-launch CUDA events (op, start, stop) while tg_profile_passes runs
  std::vector<ProfEvent>* prof = nullptr;
  // phases of the last stage-tape adjoint (tg_adjoint_profile): forward run, tape recording
  // sweeps of the segments, backward sweeps (ms, CUDA events on the plan's stream)
  double adj_ms[3] = {0.0, 0.0, 0.0};
};

namespace {

size_t csize(const tg_plan* p) { return p->prec == TG_PREC_F64 ? 16 : 8; }

template <typename R> LaunchFn<R> launcher(const tg_plan* p);
template <> LaunchFn<float> launcher<float>(const tg_plan* p) { return p->l32; }
template <> LaunchFn<double> launcher<double>(const tg_plan* p) { return p->l64; }

template <typename R>
struct Ops {
  using C = cplx<R>;

  static PassArgs<R> base(tg_plan* p) {
    PassArgs<R> a;
    std::memset(&a, 0, sizeof(a));
    a.g = p->g;
    a.tw = static_cast<const C*>(p->TW);
    a.coef = p->coef;
    a.amax = p->amax;
    a.variant = p->variant;
    a.yconf = p->yconf;
    if (p->flags & TG_FLAG_EXPLICIT_VISC) a.flags |= FLAG_EXPLICIT;
    return a;
  }
  static int go(tg_plan* p, int op, const PassArgs<R>& a, const char* what) {
    ProfEvent pe{op, nullptr, nullptr};
    if (p->prof) {
      TG_CUDA(cudaEventCreate(&pe.start), "event");
      TG_CUDA(cudaEventCreate(&pe.stop), "event");
      TG_CUDA(cudaEventRecord(pe.start, p->st), "event record");
    }
    cudaError_t e = launcher<R>(p)(op, a, p->batch, p->st);
    ++p->launches;
    if (p->prof) {
      cudaEventRecord(pe.stop, p->st);
      p->prof->push_back(pe);
    }
    if (e != cudaSuccess) return cuda_fail(e, what);
    return TG_OK;
  }
  // spectral state -> inverse-x of nout fields (map) into X
  static int load_inv(tg_plan* p, const void* S, int map, int nin, int nout, void* out = nullptr) {
    PassArgs<R> a = base(p);
    a.spec_in = static_cast<const C*>(S);
    a.out = static_cast<C*>(out ? out : p->X);
    a.map = map;
    a.nin = nin;
    a.nout = nout;
    return go(p, p->F == 6 ? OP_KX_LOAD6 : OP_KX_LOAD3, a, "kx load");
  }
  static int y_inv(tg_plan* p, int nf, const void* in = nullptr) {
    PassArgs<R> a = base(p);
    a.in = static_cast<const C*>(in ? in : p->X);
    a.out = static_cast<C*>(p->Y);
    a.nin = a.nout = nf;
    return go(p, OP_KY_INV, a, "ky inverse");
  }
  static int z_prod(tg_plan* p) {
    PassArgs<R> a = base(p);
    a.in = static_cast<const C*>(p->Y);
    a.out = static_cast<C*>(p->Z);
    a.nin = p->G;
    a.nout = p->F;
    return go(p, p->F == 6 ? OP_KZ_PROD_MHD : OP_KZ_PROD_HD, a, "kz product");
  }
  static int y_fwd(tg_plan* p, int nf) {
    PassArgs<R> a = base(p);
    a.in = static_cast<const C*>(p->Z);
    a.out = static_cast<C*>(p->Y);  // W aliases Y
    a.nin = a.nout = nf;
    return go(p, OP_KY_FWD, a, "ky forward");
  }
  static int x_stage(tg_plan* p, void* S, int stage) {
    PassArgs<R> a = base(p);
    a.in = static_cast<const C*>(p->Y);
    a.out = static_cast<C*>(p->X);
    a.S = static_cast<C*>(S);
    a.acc = static_cast<C*>(p->ACC);
    a.vs = static_cast<C*>(p->VS);
    a.tape = static_cast<C*>(p->tape);
    a.stage = stage;
    a.nin = p->F;
    a.nout = p->G;
    return go(p, p->F == 6 ? OP_KX_STAGE6 : OP_KX_STAGE3, a, "kx stage");
  }
  static int x_fwd(tg_plan* p, void* out, const void* spec_in, bool rhs) {
    PassArgs<R> a = base(p);
    a.in = static_cast<const C*>(p->Y);
    a.spec_out = static_cast<C*>(out);
    a.spec_in = static_cast<const C*>(spec_in);
    a.nin = p->F;
    if (rhs) a.flags |= FLAG_RHS;
    return go(p, p->F == 6 ? OP_KX_FWD6 : OP_KX_FWD3, a, "kx forward");
  }
  static int z_c2r(tg_plan* p, void* phys, int nf, bool amax) {
    PassArgs<R> a = base(p);
    a.in = static_cast<const C*>(p->Y);
    a.phys_out = static_cast<R*>(phys);
    a.nin = nf;
    if (amax) a.flags |= FLAG_AMAX;
    return go(p, OP_KZ_C2R, a, "kz c2r");
  }
  static int z_r2c(tg_plan* p, const void* phys, int nf) {
    PassArgs<R> a = base(p);
    a.phys_in = static_cast<const R*>(phys);
    a.out = static_cast<C*>(p->Z);
    a.nin = nf;
    return go(p, OP_KZ_R2C, a, "kz r2c");
  }
  static int stages(tg_plan* p, void* S) {
    for (int s = 1; s <= 4; ++s) {
      int rc;
      if ((rc = y_inv(p, p->G))) return rc;
      if ((rc = z_prod(p))) return rc;
      if ((rc = y_fwd(p, p->F))) return rc;
      if ((rc = x_stage(p, S, s))) return rc;
    }
    return TG_OK;
  }
  static int start(tg_plan* p, const void* S) {
    return load_inv(p, S, p->F == 6 ? MAP_UWBJ : MAP_UW, p->F, p->G);
  }
  static int diagnostics(tg_plan* p, const void* S, double* out) {
    int rc;
    const int nd = p->F / 3;
    TG_CUDA(cudaMemsetAsync(p->amax, 0, sizeof(unsigned long long) * p->batch * 2, p->st), "memset");
    // the divergence goes through Z (x-pass layout, nd <= F fields) and Y, so that X keeps
    // the inverse-x fields of a state being advanced (tg_run loads the state once)
    if ((rc = load_inv(p, S, MAP_DIV, p->F, nd, p->Z))) return rc;
    if ((rc = y_inv(p, nd, p->Z))) return rc;
    {
      PassArgs<R> a = base(p);
      a.in = static_cast<const C*>(p->Y);
      a.phys_out = nullptr;
      a.nin = nd;
      a.amax = p->amax;
      a.flags |= FLAG_AMAX;
      if ((rc = go(p, OP_KZ_C2R, a, "kz divergence"))) return rc;
    }
    const int nblk = diag_blocks(p->g);
    dim3 grid(nblk, p->batch);
    diag_partial<R><<<grid, kDiagThreads, 0, p->st>>>(static_cast<const C*>(S), p->g, p->F, p->part);
    TG_CUDA(cudaGetLastError(), "diag_partial");
    diag_final<<<p->batch, 32 * kNQ, 0, p->st>>>(p->part, nblk, p->coef, p->amax, nd, p->F, out);
    TG_CUDA(cudaGetLastError(), "diag_final");
    p->launches += 2;
    return TG_OK;
  }
  static int absmax(tg_plan* p, const void* S, int which, double* out) {
    int rc;
    const int nf = (which == TG_ABSMAX_DIVERGENCE) ? p->F / 3 : p->F;
    TG_CUDA(cudaMemsetAsync(p->amax, 0, sizeof(unsigned long long) * p->batch * nf, p->st), "memset");
    if ((rc = load_inv(p, S, which == TG_ABSMAX_DIVERGENCE ? MAP_DIV : MAP_ID, p->F, nf))) return rc;
    if ((rc = y_inv(p, nf))) return rc;
    PassArgs<R> a = base(p);
    a.in = static_cast<const C*>(p->Y);
    a.nin = nf;
    a.flags |= FLAG_AMAX;
    if ((rc = go(p, OP_KZ_C2R, a, "kz absmax"))) return rc;
    const int cnt = p->batch * nf;
    amax_to_double<<<(cnt + 127) / 128, 128, 0, p->st>>>(p->amax, cnt, out);
    TG_CUDA(cudaGetLastError(), "amax_to_double");
    return TG_OK;
  }

  static int derived(tg_plan* p, const void* S, int which, void* phys) {
    int rc;
    const int nf = (which == TG_DERIVED_DIVERGENCE) ? p->F / 3 : p->F;
    if ((rc = load_inv(p, S, which == TG_DERIVED_DIVERGENCE ? MAP_DIV : MAP_CURL, p->F, nf))) return rc;
    if ((rc = y_inv(p, nf))) return rc;
    return z_c2r(p, phys, nf, false);
  }
  static int full(tg_plan* p, const void* S, void* out, bool to_full) {
    const long long total = to_full ? (long long)p->g.sP * p->F * p->batch : p->g.sS * p->F * p->batch;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 8192);
    if (to_full)
      to_full_kernel<R><<<blocks, 256, 0, p->st>>>(static_cast<const C*>(S), static_cast<C*>(out), p->g, p->F, p->batch);
    else
      from_full_kernel<R><<<blocks, 256, 0, p->st>>>(static_cast<const C*>(S), static_cast<C*>(out), p->g, p->F, p->batch);
    TG_CUDA(cudaGetLastError(), "full spectrum conversion");
    ++p->launches;
    return TG_OK;
  }
  static int energy(tg_plan* p, const void* phys, double* out) {
    const int groups = p->batch * (p->F / 3);
    dim3 grid(kDiagBlocks, groups);
    // the partial buffer holds batch * kDiagBlocks * kNQ doubles >= groups * kDiagBlocks
    phys_energy_partial<R><<<grid, kDiagThreads, 0, p->st>>>(static_cast<const R*>(phys), p->g.sP, p->part);
    TG_CUDA(cudaGetLastError(), "phys_energy_partial");
    phys_energy_final<<<(groups + 63) / 64, 64, 0, p->st>>>(p->part, kDiagBlocks, groups, p->g.sP, out);
    TG_CUDA(cudaGetLastError(), "phys_energy_final");
    p->launches += 2;
    return TG_OK;
  }
  static int initial(tg_plan* p, int kind, uint64_t seed, double amp, double k0, double b_amp, void* S) {
    const long long total = (long long)p->batch * p->F * p->g.sS;
    ic_kernel<R><<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, p->st>>>(
        static_cast<C*>(S), p->g, p->F, p->batch, kind, b_amp);
    TG_CUDA(cudaGetLastError(), "ic_kernel");
    if (amp > 0.0) {
      const long long modes = (long long)p->batch * p->g.M * p->g.M * p->g.Hk;
      C* P = static_cast<C*>(p->ACC);  // scratch: [batch][3][M][M][Hz]
      TG_CUDA(cudaMemsetAsync(P, 0, csize(p) * 3 * p->g.sS * p->batch, p->st), "memset");
      pert_kernel<R><<<(int)std::min<long long>((modes + 255) / 256, 4096), 256, 0, p->st>>>(
          P, p->g, p->batch, (unsigned long long)seed, k0);
      TG_CUDA(cudaGetLastError(), "pert_kernel");
      const int nblk = diag_blocks(p->g);
      dim3 grid(nblk, p->batch);
      diag_partial<R><<<grid, kDiagThreads, 0, p->st>>>(P, p->g, 3, p->part);
      diag_final<<<p->batch, 32 * kNQ, 0, p->st>>>(p->part, nblk, p->coef, p->amax, 0, 3, p->dtmp);
      TG_CUDA(cudaGetLastError(), "perturbation energy");
      std::vector<double> rec((size_t)p->batch * TG_DIAG_WIDTH), scale(p->batch);
      TG_CUDA(cudaMemcpyAsync(rec.data(), p->dtmp, rec.size() * sizeof(double), cudaMemcpyDeviceToHost, p->st),
              "memcpy");
      TG_CUDA(cudaStreamSynchronize(p->st), "sync");
      for (int r = 0; r < p->batch; ++r) {
        const double e = rec[(size_t)r * TG_DIAG_WIDTH + TG_D_KINETIC];  // 0.5 <|v|^2>
        scale[r] = (e > 0.0) ? amp / std::sqrt(2.0 * e / 3.0) : 0.0;
      }
      TG_CUDA(cudaMemcpyAsync(p->dtmp, scale.data(), scale.size() * sizeof(double), cudaMemcpyHostToDevice, p->st),
              "memcpy");
      axpy_pert<R><<<(int)std::min<long long>((3 * p->g.sS * p->batch + 255) / 256, 4096), 256, 0, p->st>>>(
          static_cast<C*>(S), P, p->g, p->F, p->batch, p->dtmp);
      TG_CUDA(cudaGetLastError(), "axpy_pert");
    }
    TG_CUDA(cudaStreamSynchronize(p->st), "sync");
    return TG_OK;
  }
};

template <typename Fn>
int dispatch(tg_plan* p, Fn&& fn) {
  if (p->prec == TG_PREC_F64) return fn(Ops<double>());
  return fn(Ops<float>());
}

// each coefficient given (dt > 0, nu >= 0, eta >= 0) replaces the per-run values; the others
// keep theirs (the per-run table of tg_set_run_params)
int set_coefs(tg_plan* p, double dt, double nu, double eta) {
  for (auto& c : p->hcoef) {
    if (dt > 0.0) c.dt = dt;
    if (nu >= 0.0) c.nu = nu;
    if (eta >= 0.0) c.eta = eta;
  }
  TG_CUDA(cudaMemcpyAsync(p->coef, p->hcoef.data(), sizeof(RunCoef) * p->hcoef.size(), cudaMemcpyHostToDevice,
                          p->st),
          "coef upload");
  return TG_OK;
}

void drop_graph(tg_plan* p) {
  if (p->step_exec) cudaGraphExecDestroy(p->step_exec);
  if (p->step_graph) cudaGraphDestroy(p->step_graph);
  p->step_exec = nullptr;
  p->step_graph = nullptr;
  p->step_state = nullptr;
}

// advance nsteps RK4 steps; X must already hold the inverse-x fields of S
int advance(tg_plan* p, void* S, int nsteps) {
  if (nsteps <= 0) return TG_OK;
  int rc;
  int done = 0;
  if (p->step_state != S || !p->step_exec) {
    drop_graph(p);
    // one eager step first: it also sets every kernel attribute outside capture
    rc = dispatch(p, [&](auto ops) { return decltype(ops)::stages(p, S); });
    if (rc) return rc;
    done = 1;
    // capture on the plan's private stream (the caller's may be the legacy default
    // stream, which cannot be captured); the graph is then launched on the caller's
    if (!p->cap) TG_CUDA(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking), "capture stream");
    cudaStream_t user = p->st;
    TG_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    const int64_t before = p->launches;
    p->st = p->cap;
    rc = dispatch(p, [&](auto ops) { return decltype(ops)::stages(p, S); });
    p->st = user;
    p->launches = before;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(p->cap, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "end capture");
    e = cudaGraphInstantiate(&p->step_exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      return cuda_fail(e, "graph instantiate");
    }
    p->step_graph = graph;
    p->step_state = S;
  }
  for (int s = done; s < nsteps; ++s) {
    TG_CUDA(cudaGraphLaunch(p->step_exec, p->st), "graph launch");
    p->launches += 16;
  }
  return TG_OK;
}

bool size_supported(int n, int prec) { return tg::size_built(n, prec); }

}  // namespace

// ====================================================================== C ABI
extern "C" {

const char* tg_last_error(void) { return g_last_error.c_str(); }
int tg_version(void) { return 100; }

// ---------------------------------------------------------------- autotuning
// TG_FLAG_AUTOTUNE times, on this plan's own shape and batch (graph-launched steps of a
// perturbed Taylor-Green state), first the pass variants (register-resident or
// shared-memory x and z passes), then with the fastest variant the y-pass configurations
// (radix plan and kz columns per CTA, YConf in tg_common.cuh), and keeps the fastest of
// each.  TG_PASS_VARIANT / TG_Y_CONF force a choice and skip its timing.  With
// TG_AUTOTUNE_CACHE naming a file, choices are looked up there first (keyed by device,
// grid size, batch, physics, precision, cutoff and scheme) and new ones are appended.

// best of two timings of three graph-launched steps (after the eager step and capture)
static int time_steps(tg_plan* p, void* S, cudaEvent_t e0, cudaEvent_t e1, float* best) {
  drop_graph(p);
  int rc;
  if ((rc = tg_step(p, S, 1e-4, 1e-2, 1e-2, 2))) return rc;  // eager step, capture, one replay
  *best = 1e30f;
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(e0, p->st);
    if ((rc = tg_step(p, S, 1e-4, 1e-2, 1e-2, 3))) return rc;
    cudaEventRecord(e1, p->st);
    float ms = 0.0f;
    cudaError_t e;
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess || (e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess)
      return cuda_fail(e, "autotune timing");
    *best = std::min(*best, ms);
  }
  return TG_OK;
}

static std::string tune_key(const tg_plan* p) {
  int dev = 0;
  cudaDeviceProp prop;
  std::string name = "unknown";
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
    name = prop.name;
    name += "_sm" + std::to_string(prop.major) + std::to_string(prop.minor);
  }
  for (char& c : name)
    if (c == ' ' || c == '\t') c = '_';
  const int scheme = p->flags & (TG_FLAG_EXPLICIT_VISC | TG_FLAG_LORENTZ_REF);
  return "tg-autotune-v1 " + name + " n=" + std::to_string(p->n) + " batch=" + std::to_string(p->batch) +
         " F=" + std::to_string(p->F) + " prec=" + std::to_string(p->prec) + " K=" + std::to_string(p->K) +
         " scheme=" + std::to_string(scheme);
}

// the cached (variant, yconf) of this plan's key, if any (the last matching line wins)
static bool cache_lookup(const char* path, const std::string& key, int* variant, int* yconf) {
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof(line), f)) {
    std::string l(line);
    const size_t at = l.find(" variant=");
    if (at == std::string::npos || l.compare(0, at, key) != 0 || at != key.size()) continue;
    int v = -1, y = -1;
    if (std::sscanf(l.c_str() + at, " variant=%d yconf=%d", &v, &y) == 2) {
      *variant = v;
      *yconf = y;
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

static void cache_store(const char* path, const std::string& key, int variant, int yconf) {
  FILE* f = std::fopen(path, "a");  // one short line per append
  if (!f) return;                   // a cache that cannot be written only costs a re-tune
  std::fprintf(f, "%s variant=%d yconf=%d\n", key.c_str(), variant, yconf);
  std::fclose(f);
}

static int autotune(tg_plan* p) {
  const bool f32 = p->prec == TG_PREC_F32;
  const bool reg_z = f32 && (has_reg_adjoint(p->n) || (p->F == 3 && p->n == 96));  // z: 16 ... 256, hydro 96
  const bool reg_x = f32 && p->F == 3 && (has_reg_adjoint(p->n) || p->n == 96);  // x: hydro
  const bool stash_x = f32 && p->F == 3 && (p->n == 64 || p->n == 96 || p->n == 128 || p->n == 256);
  const bool tune_variant = !std::getenv("TG_PASS_VARIANT");
  const bool tune_y = !std::getenv("TG_Y_CONF") && p->nyconf > 1;
  std::vector<int> cands = {0};
  if (tune_variant) {
    if (reg_z) cands.push_back(1);
    if (reg_x) cands.push_back(2);
    if (reg_z && reg_x) cands.push_back(3);
    if (stash_x) cands.push_back(4);
    if (stash_x && reg_z) cands.push_back(5);
  }
  if (cands.size() == 1 && !tune_y) return TG_OK;
  const char* cache = std::getenv("TG_AUTOTUNE_CACHE");
  const std::string key = cache ? tune_key(p) : std::string();
  if (cache) {
    int v = -1, y = -1;
    if (cache_lookup(cache, key, &v, &y) && v >= 0 && v <= 7 && y >= 0 && y < p->nyconf) {
      if (tune_variant) p->variant = v;
      if (tune_y) p->yconf = y;
      return TG_OK;
    }
  }
  void* S = nullptr;
  const size_t bytes = csize(p) * (size_t)p->batch * p->F * p->g.sS;
  cudaError_t e = cudaMalloc(&S, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "autotune state");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = TG_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = TG_E_CUDA;
  if (!rc) rc = tg_initial_condition(p, p->F == 6 ? TG_IC_MHD_EQUAL_ENERGY : TG_IC_TAYLOR_GREEN, 1, 1e-3, 4.0,
                                     0.0, S);
  if (!rc && cands.size() > 1) {
    int best = p->variant;
    float best_ms = 1e30f;
    for (int v : cands) {
      p->variant = v;
      float ms = 0.0f;
      if ((rc = time_steps(p, S, e0, e1, &ms))) break;
      if (ms < best_ms) {
        best_ms = ms;
        best = v;
      }
    }
    p->variant = best;
  }
  if (!rc && tune_y) {
    int best = 0;
    float best_ms = 1e30f;
    for (int y = 0; y < p->nyconf; ++y) {
      p->yconf = y;
      float ms = 0.0f;
      if ((rc = time_steps(p, S, e0, e1, &ms))) break;
      if (ms < best_ms) {
        best_ms = ms;
        best = y;
      }
    }
    p->yconf = best;
  }
  drop_graph(p);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(S);
  p->launches = 0;
  if (!rc && cache) cache_store(cache, key, p->variant, p->yconf);
  return rc;
}

int tg_plan_create(tg_plan** out, const tg_desc* d) {
  if (!out || !d) return fail(TG_E_INVALID, "tg_plan_create: null argument");
  *out = nullptr;
  if (d->physics != TG_PHYS_HYDRO && d->physics != TG_PHYS_MHD)
    return fail(TG_E_INVALID, "tg_plan_create: physics must be TG_PHYS_HYDRO or TG_PHYS_MHD");
  if (d->precision != TG_PREC_F32 && d->precision != TG_PREC_F64)
    return fail(TG_E_INVALID, "tg_plan_create: precision must be TG_PREC_F32 or TG_PREC_F64");
  if (d->batch < 1) return fail(TG_E_INVALID, "tg_plan_create: batch must be >= 1");
  if (!size_supported(d->n, d->precision))
    return fail(TG_E_UNSUPPORTED, "tg_plan_create: grid size " + std::to_string(d->n) +
                                      " is not built for this precision");
  const int n = d->n;
  const int K = d->cutoff > 0 ? d->cutoff : n / 3;
  if (K < 1 || K > n / 3)
    return fail(TG_E_INVALID, "tg_plan_create: cutoff must satisfy 1 <= cutoff <= n/3 (2/3 rule)");
  tg_plan* p = new (std::nothrow) tg_plan();
  if (!p) return fail(TG_E_NOMEM, "tg_plan_create: host allocation failed");
  p->n = n;
  p->K = K;
  p->batch = d->batch;
  p->physics = d->physics;
  p->prec = d->precision;
  p->flags = d->flags;
  p->F = d->physics == TG_PHYS_MHD ? 6 : 3;
  p->G = 2 * p->F;
  if (const char* v = std::getenv("TG_PASS_VARIANT")) p->variant = std::atoi(v);
  p->nyconf = yconf_count(d->n, d->precision);
  if (const char* v = std::getenv("TG_Y_CONF")) p->yconf = std::max(0, std::min(std::atoi(v), p->nyconf - 1));
  Geo& g = p->g;
  g.n = n;
  g.K = K;
  g.M = 2 * K + 1;
  g.Hk = K + 1;
  g.Hz = (g.Hk + 3) / 4 * 4;
  g.sS = (long long)g.M * g.M * g.Hz;
  g.sX = (long long)n * g.M * g.Hz;
  g.sY = (long long)n * n * g.Hz;
  g.sP = (long long)n * n * n;
  if (p->prec == TG_PREC_F64) p->l64 = find_f64(n);
  else p->l32 = find_f32(n);
  const size_t cs = csize(p);
  const size_t B = (size_t)p->batch;
  struct Alloc { void** ptr; size_t bytes; } allocs[] = {
      {&p->X, cs * B * p->G * g.sX},
      // Y and Z in one block, Z right after Y: with batch 1 the block is also the
      // contiguous nine-field buffer of the adjoint's in-place z pass
      {&p->Y, cs * B * (p->G + p->F) * g.sY},
      {&p->ACC, cs * B * p->F * g.sS},
      {&p->VS, (p->flags & TG_FLAG_EXPLICIT_VISC) ? cs * B * p->F * g.sS : 0},
      {&p->TW, cs * n},
      {(void**)&p->part, sizeof(double) * B * kDiagBlocks * kNQ},
      {(void**)&p->dtmp, sizeof(double) * B * TG_DIAG_WIDTH},
      {(void**)&p->amax, sizeof(unsigned long long) * B * 6},
      {(void**)&p->coef, sizeof(RunCoef) * B},
  };
  for (auto& a : allocs) {
    if (a.bytes == 0) continue;
    cudaError_t e = cudaMalloc(a.ptr, a.bytes);
    if (e != cudaSuccess) {
      tg_plan_destroy(p);
      return fail(TG_E_NOMEM, std::string("tg_plan_create: cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    p->scratch += (int64_t)a.bytes;
  }
  p->Z = static_cast<char*>(p->Y) + cs * B * p->G * g.sY;
  // twiddles W_N^m = exp(-2 pi i m / N), generated in FP64
  std::vector<double> tw(2 * (size_t)n);
  for (int m = 0; m < n; ++m) {
    // exact quarter-turn values; cos/sin of a reduced angle elsewhere
    const double ang = 2.0 * M_PI * (double)m / (double)n;
    double c = std::cos(ang), s = std::sin(ang);
    if ((4 * m) % n == 0) {
      const int q = (4 * m) / n;
      c = (q == 0) ? 1.0 : (q == 2 ? -1.0 : 0.0);
      s = (q == 1) ? 1.0 : (q == 3 ? -1.0 : 0.0);
    }
    tw[2 * m] = c;
    tw[2 * m + 1] = -s;
  }
  cudaError_t e;
  if (p->prec == TG_PREC_F64) {
    e = cudaMemcpy(p->TW, tw.data(), sizeof(double) * 2 * n, cudaMemcpyHostToDevice);
  } else {
    std::vector<float> tf(tw.begin(), tw.end());
    e = cudaMemcpy(p->TW, tf.data(), sizeof(float) * 2 * n, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    tg_plan_destroy(p);
    return cuda_fail(e, "tg_plan_create: twiddle upload");
  }
  p->hcoef.assign(p->batch, RunCoef{0.0, 0.0, 0.0, (p->flags & TG_FLAG_LORENTZ_REF) ? -1.0 : 1.0});
  e = cudaMemcpy(p->coef, p->hcoef.data(), sizeof(RunCoef) * p->batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->amax, 0, sizeof(unsigned long long) * B * 6);
  if (e != cudaSuccess) {
    tg_plan_destroy(p);
    return cuda_fail(e, "tg_plan_create: init");
  }
  if (p->flags & TG_FLAG_AUTOTUNE) {
    const int rc = autotune(p);
    if (rc) {
      tg_plan_destroy(p);
      return rc;
    }
  }
  *out = p;
  return TG_OK;
}

int tg_pass_variant(const tg_plan* p) { return p ? p->variant : 0; }

int tg_adjoint_profile(const tg_plan* p, double ms[3]) {
  if (!p || !ms) return fail(TG_E_INVALID, "tg_adjoint_profile: null argument");
  for (int i = 0; i < 3; ++i) ms[i] = p->adj_ms[i];
  return TG_OK;
}

int tg_y_config(const tg_plan* p, int* count) {
  if (count) *count = p ? p->nyconf : 0;
  return p ? p->yconf : 0;
}

int tg_release_host_tape(tg_plan* p) {
  if (!p) return fail(TG_E_INVALID, "tg_release_host_tape: null plan");
  if (p->htape) {
    const cudaError_t e = cudaFreeHost(p->htape);
    p->htape = nullptr;
    p->htape_bytes = 0;
    if (e != cudaSuccess) return cuda_fail(e, "tg_release_host_tape");
  }
  return TG_OK;
}

int tg_plan_destroy(tg_plan* p) {
  if (!p) return TG_OK;
  drop_graph(p);
  if (p->cap) cudaStreamDestroy(p->cap);
  if (p->htape) cudaFreeHost(p->htape);
  void* bufs[] = {p->X, p->Y, p->ACC, p->VS, p->TW, p->part, p->dtmp, p->amax, p->coef};  // Z lies in Y's block
  for (void* b : bufs)
    if (b) cudaFree(b);
  delete p;
  return TG_OK;
}

int tg_set_stream(tg_plan* p, void* stream) {
  if (!p) return fail(TG_E_INVALID, "tg_set_stream: null plan");
  if (p->st != static_cast<cudaStream_t>(stream)) drop_graph(p);
  p->st = static_cast<cudaStream_t>(stream);
  return TG_OK;
}

int64_t tg_state_layout(const tg_plan* p, int dims[7]) {
  if (!p) return 0;
  if (dims) {
    dims[0] = p->batch;
    dims[1] = p->F;
    dims[2] = p->g.M;
    dims[3] = p->g.M;
    dims[4] = p->g.Hz;
    dims[5] = p->K;
    dims[6] = p->n;
  }
  return (int64_t)p->batch * p->F * p->g.sS;
}

int64_t tg_plan_scratch_bytes(const tg_plan* p) { return p ? p->scratch : 0; }
int64_t tg_last_launch_count(const tg_plan* p) { return p ? p->launches : 0; }

int tg_set_run_params(tg_plan* p, const double* nu, const double* eta, const double* dt, int count) {
  if (!p) return fail(TG_E_INVALID, "tg_set_run_params: null plan");
  if (count != 1 && count != p->batch) return fail(TG_E_INVALID, "tg_set_run_params: count must be 1 or batch");
  for (int r = 0; r < p->batch; ++r) {
    const int i = (count == 1) ? 0 : r;
    if (nu) {
      if (!(nu[i] >= 0.0)) return fail(TG_E_INVALID, "tg_set_run_params: nu must be nonnegative");
      p->hcoef[r].nu = nu[i];
    }
    if (eta) {
      if (!(eta[i] >= 0.0)) return fail(TG_E_INVALID, "tg_set_run_params: eta must be nonnegative");
      p->hcoef[r].eta = eta[i];
    }
    if (dt) {
      if (!(dt[i] > 0.0)) return fail(TG_E_INVALID, "tg_set_run_params: dt must be positive");
      p->hcoef[r].dt = dt[i];
    }
  }
  return set_coefs(p, -1.0, -1.0, -1.0);
}

int tg_initial_condition(tg_plan* p, int kind, uint64_t seed, double pert_amp, double k0, double b_amp,
                         void* state) {
  if (!p || !state) return fail(TG_E_INVALID, "tg_initial_condition: null argument");
  if (kind < TG_IC_TAYLOR_GREEN || kind > TG_IC_ZERO) return fail(TG_E_INVALID, "tg_initial_condition: bad kind");
  if ((kind == TG_IC_MHD_REFERENCE || kind == TG_IC_MHD_EQUAL_ENERGY) && p->F != 6)
    return fail(TG_E_INVALID, "tg_initial_condition: MHD initial condition needs an MHD plan");
  if (pert_amp < 0.0 || (pert_amp > 0.0 && !(k0 > 0.0)))
    return fail(TG_E_INVALID, "tg_initial_condition: need pert_amp >= 0 and k0 > 0");
  p->launches = 0;
  return dispatch(p, [&](auto ops) { return decltype(ops)::initial(p, kind, seed, pert_amp, k0, b_amp, state); });
}

int tg_forward(tg_plan* p, const void* phys, void* state) {
  if (!p || !phys || !state) return fail(TG_E_INVALID, "tg_forward: null argument");
  p->launches = 0;
  return dispatch(p, [&](auto ops) {
    using O = decltype(ops);
    int rc;
    if ((rc = O::z_r2c(p, phys, p->F))) return rc;
    if ((rc = O::y_fwd(p, p->F))) return rc;
    return O::x_fwd(p, state, nullptr, false);
  });
}

int tg_inverse(tg_plan* p, const void* state, void* phys) {
  if (!p || !phys || !state) return fail(TG_E_INVALID, "tg_inverse: null argument");
  p->launches = 0;
  return dispatch(p, [&](auto ops) {
    using O = decltype(ops);
    int rc;
    if ((rc = O::load_inv(p, state, MAP_ID, p->F, p->F))) return rc;
    if ((rc = O::y_inv(p, p->F))) return rc;
    return O::z_c2r(p, phys, p->F, false);
  });
}

int tg_rhs(tg_plan* p, const void* state, double nu, double eta, void* rhs_out) {
  if (!p || !state || !rhs_out) return fail(TG_E_INVALID, "tg_rhs: null argument");
  int rc = set_coefs(p, -1.0, nu, eta);
  if (rc) return rc;
  p->launches = 0;
  return dispatch(p, [&](auto ops) {
    using O = decltype(ops);
    int r;
    if ((r = O::start(p, state))) return r;
    if ((r = O::y_inv(p, p->G))) return r;
    if ((r = O::z_prod(p))) return r;
    if ((r = O::y_fwd(p, p->F))) return r;
    return O::x_fwd(p, rhs_out, state, true);
  });
}

int tg_step(tg_plan* p, void* state, double dt, double nu, double eta, int nsteps) {
  if (!p || !state) return fail(TG_E_INVALID, "tg_step: null argument");
  if (nsteps < 0) return fail(TG_E_INVALID, "tg_step: nsteps must be >= 0");
  if (dt > 0.0 && nu < 0.0) return fail(TG_E_INVALID, "tg_step: nu must be nonnegative");
  int rc = set_coefs(p, dt, nu, eta);
  if (rc) return rc;
  for (const auto& c : p->hcoef)
    if (!(c.dt > 0.0)) return fail(TG_E_INVALID, "tg_step: dt must be positive");
  p->launches = 0;
  if (nsteps == 0) return TG_OK;
  rc = dispatch(p, [&](auto ops) { return decltype(ops)::start(p, state); });
  if (rc) return rc;
  return advance(p, state, nsteps);
}

int tg_run(tg_plan* p, void* state, double dt, double nu, double eta, int nsteps, int save_every,
           double* series) {
  if (!p || !state || !series) return fail(TG_E_INVALID, "tg_run: null argument");
  if (nsteps < 0 || save_every < 1) return fail(TG_E_INVALID, "tg_run: need nsteps >= 0 and save_every >= 1");
  int rc = set_coefs(p, dt, nu, eta);
  if (rc) return rc;
  for (const auto& c : p->hcoef)
    if (!(c.dt > 0.0)) return fail(TG_E_INVALID, "tg_run: dt must be positive");
  p->launches = 0;
  const long long stride = (long long)p->batch * TG_DIAG_WIDTH;
  int64_t total = 0;
  rc = dispatch(p, [&](auto ops) { return decltype(ops)::diagnostics(p, state, series); });
  if (rc) return rc;
  total += p->launches;
  int rec = 1;
  int step = 0;
  // X holds the inverse-x fields of the state from here on: the steps leave those of their
  // result, and the diagnostics between chunks do not use X
  if (nsteps > 0) {
    p->launches = 0;
    rc = dispatch(p, [&](auto ops) { return decltype(ops)::start(p, state); });
    if (rc) return rc;
    total += p->launches;
  }
  while (step < nsteps) {
    const int chunk = std::min(save_every - (step % save_every), nsteps - step);
    p->launches = 0;
    rc = advance(p, state, chunk);
    if (rc) return rc;
    step += chunk;
    rc = dispatch(p, [&](auto ops) { return decltype(ops)::diagnostics(p, state, series + rec * stride); });
    if (rc) return rc;
    total += p->launches;
    ++rec;
  }
  p->launches = total;
  // failure detection: a non-finite diagnostic means the run blew up (e.g. dt above the
  // stability limit, or a NaN in the initial state); report the first such record
  std::vector<double> h((size_t)rec * stride);
  TG_CUDA(cudaMemcpyAsync(h.data(), series, h.size() * sizeof(double), cudaMemcpyDeviceToHost, p->st),
          "series readback");
  TG_CUDA(cudaStreamSynchronize(p->st), "tg_run sync");
  for (int r = 0; r < rec; ++r)
    for (long long i = 0; i < stride; ++i)
      if (!std::isfinite(h[(size_t)r * stride + i]))
        return fail(TG_E_NONFINITE, "tg_run: non-finite diagnostics at record " + std::to_string(r) +
                                        " (run " + std::to_string(i / TG_DIAG_WIDTH) + ")");
  return TG_OK;
}

int tg_diagnostics(tg_plan* p, const void* state, double nu, double eta, double* out) {
  if (!p || !state || !out) return fail(TG_E_INVALID, "tg_diagnostics: null argument");
  int rc = set_coefs(p, -1.0, nu, eta);
  if (rc) return rc;
  p->launches = 0;
  return dispatch(p, [&](auto ops) { return decltype(ops)::diagnostics(p, state, out); });
}

int tg_field_absmax(tg_plan* p, const void* state, int which, double* out) {
  if (!p || !state || !out) return fail(TG_E_INVALID, "tg_field_absmax: null argument");
  if (which != TG_ABSMAX_VELOCITY && which != TG_ABSMAX_DIVERGENCE)
    return fail(TG_E_INVALID, "tg_field_absmax: bad selector");
  p->launches = 0;
  return dispatch(p, [&](auto ops) { return decltype(ops)::absmax(p, state, which, out); });
}

int tg_derived(tg_plan* p, const void* state, int which, void* phys) {
  if (!p || !state || !phys) return fail(TG_E_INVALID, "tg_derived: null argument");
  if (which != TG_DERIVED_VORTICITY && which != TG_DERIVED_DIVERGENCE)
    return fail(TG_E_INVALID, "tg_derived: bad selector");
  p->launches = 0;
  return dispatch(p, [&](auto ops) { return decltype(ops)::derived(p, state, which, phys); });
}

int tg_to_full_spectrum(tg_plan* p, const void* state, void* full) {
  if (!p || !state || !full) return fail(TG_E_INVALID, "tg_to_full_spectrum: null argument");
  p->launches = 0;
  return dispatch(p, [&](auto ops) { return decltype(ops)::full(p, state, full, true); });
}

int tg_from_full_spectrum(tg_plan* p, const void* full, void* state) {
  if (!p || !state || !full) return fail(TG_E_INVALID, "tg_from_full_spectrum: null argument");
  p->launches = 0;
  return dispatch(p, [&](auto ops) { return decltype(ops)::full(p, full, state, false); });
}

int tg_physical_energy(tg_plan* p, const void* phys, double* out) {
  if (!p || !phys || !out) return fail(TG_E_INVALID, "tg_physical_energy: null argument");
  p->launches = 0;
  return dispatch(p, [&](auto ops) { return decltype(ops)::energy(p, phys, out); });
}

int tg_profile_passes(tg_plan* p, void* state, double dt, double nu, double eta, int nsteps, double* ms,
                      int64_t* count) {
  if (!p || !state || !ms || !count) return fail(TG_E_INVALID, "tg_profile_passes: null argument");
  if (nsteps < 1) return fail(TG_E_INVALID, "tg_profile_passes: nsteps must be >= 1");
  int rc = set_coefs(p, dt, nu, eta);
  if (rc) return rc;
  for (int i = 0; i < TG_PROF_SLOTS; ++i) {
    ms[i] = 0.0;
    count[i] = 0;
  }
  std::vector<ProfEvent> ev;
  p->prof = &ev;
  p->launches = 0;
  rc = dispatch(p, [&](auto ops) {
    using O = decltype(ops);
    int r = O::start(p, state);
    for (int s = 0; s < nsteps && !r; ++s) r = O::stages(p, state);
    return r;
  });
  p->prof = nullptr;
  cudaError_t e = cudaStreamSynchronize(p->st);
  for (auto& pe : ev) {
    float t = 0.f;
    if (!rc && e == cudaSuccess && cudaEventElapsedTime(&t, pe.start, pe.stop) == cudaSuccess &&
        pe.op >= 0 && pe.op < TG_PROF_SLOTS) {
      ms[pe.op] += t;
      count[pe.op] += 1;
    }
    cudaEventDestroy(pe.start);
    cudaEventDestroy(pe.stop);
  }
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "tg_profile_passes");
  for (int i = 0; i < TG_PROF_SLOTS; ++i)
    if (count[i]) ms[i] /= (double)count[i];
  return TG_OK;
}

}  // extern "C"

// ====================================================================== adjoint
namespace {

template <typename R>
struct Adjoint {
  using C = cplx<R>;
  tg_plan* p;
  std::vector<void*> bufs;
  size_t fbytes = 0;  // one 3-field compact array
  C *X9 = nullptr, *Y9 = nullptr, *Z6 = nullptr, *WMU = nullptr;
  C *cur = nullptr, *lam = nullptr, *lamn = nullptr, *mu = nullptr;
  C *n1 = nullptr, *n2 = nullptr, *n3 = nullptr, *a2 = nullptr, *a3 = nullptr, *a4 = nullptr;
  C *g1 = nullptr, *g2 = nullptr, *g3 = nullptr, *g4 = nullptr;
  C *seg = nullptr, *ck = nullptr;
  double* dnu = nullptr;
  double* dpart = nullptr;  // per-block partial sums of d(loss)/d(nu)
  int blocks = 0;
  static constexpr int kDnuBlocks = 1024;

  ~Adjoint() {
    release_tape();
    for (void* b : bufs) cudaFree(b);
  }
  int alloc(void** ptr, size_t bytes) {
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(TG_E_NOMEM, std::string("tg_adjoint: cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    bufs.push_back(*ptr);
    return TG_OK;
  }
  int setup(int seglen, int nck) {
    const Geo& g = p->g;
    fbytes = sizeof(C) * 3 * (size_t)g.sS;
    int rc;
    struct { void** ptr; size_t bytes; } list[] = {
        {(void**)&X9, sizeof(C) * 9 * (size_t)g.sX}, {(void**)&Y9, sizeof(C) * 9 * (size_t)g.sY},
        {(void**)&Z6, sizeof(C) * 6 * (size_t)g.sY}, {(void**)&WMU, 2 * fbytes},
        {(void**)&cur, fbytes}, {(void**)&lam, fbytes}, {(void**)&lamn, fbytes}, {(void**)&mu, fbytes},
        {(void**)&n1, fbytes}, {(void**)&n2, fbytes}, {(void**)&n3, fbytes}, {(void**)&a2, fbytes},
        {(void**)&a3, fbytes}, {(void**)&a4, fbytes}, {(void**)&g1, fbytes}, {(void**)&g2, fbytes},
        {(void**)&g3, fbytes}, {(void**)&g4, fbytes}, {(void**)&seg, fbytes * (size_t)seglen},
        {(void**)&ck, fbytes * (size_t)nck}, {(void**)&dnu, sizeof(double)},
        {(void**)&dpart, sizeof(double) * kDnuBlocks}};
    for (auto& b : list)
      if ((rc = alloc(b.ptr, b.bytes))) return rc;
    const long long modes = (long long)g.M * g.M * g.Hk;
    blocks = (int)std::min<long long>((modes + 255) / 256, 2048);
    return TG_OK;
  }
  int copy(C* dst, const C* src) {
    TG_CUDA(cudaMemcpyAsync(dst, src, fbytes, cudaMemcpyDeviceToDevice, p->st), "adjoint copy");
    return TG_OK;
  }
  // one RK4 step of X in place (eager launches, no graph)
  int step(C* X) {
    int rc;
    if ((rc = Ops<R>::start(p, X))) return rc;
    return Ops<R>::stages(p, X);
  }
  // out = P F[u x omega] of state X (no viscous term)
  int nonlin(const C* X, C* out) {
    int rc;
    if ((rc = Ops<R>::start(p, X))) return rc;
    if ((rc = Ops<R>::y_inv(p, p->G))) return rc;
    if ((rc = Ops<R>::z_prod(p))) return rc;
    if ((rc = Ops<R>::y_fwd(p, p->F))) return rc;
    PassArgs<R> a = Ops<R>::base(p);
    a.in = static_cast<const C*>(p->Y);
    a.spec_out = out;
    a.spec_in = X;
    a.nin = 3;
    if (sizeof(R) == 4 && has_reg_adjoint(p->n) && (p->variant & ~4) == 0)
      return Ops<R>::go(p, OP_KX_NL_FWD, a, "kx nonlinear");
    a.flags |= FLAG_NONLIN;
    return Ops<R>::go(p, OP_KX_FWD3, a, "kx nonlinear");
  }
  // out = N'(W)^T mu = F[omega x a] + i k x F[a x u],  a = F^-1 (P mu), (u, omega) of W
  int nonlin_adj(const C* W, const C* m, C* out) {
    int rc;
    if (sizeof(R) == 4 && has_reg_adjoint(p->n) && (p->variant & ~4) == 0) {
      PassArgs<R> a = Ops<R>::base(p);
      a.spec_in = W;
      a.S = const_cast<C*>(m);
      a.out = X9;
      a.nin = 6;
      a.nout = 9;
      if ((rc = Ops<R>::go(p, OP_KX_ADJ_LOAD, a, "kx adjoint load"))) return rc;
      a = Ops<R>::base(p);
      a.in = X9;
      a.out = Y9;
      a.nin = a.nout = 9;
      if ((rc = Ops<R>::go(p, OP_KY_INV, a, "ky adjoint inverse"))) return rc;
      a = Ops<R>::base(p);
      a.in = Y9;
      a.out = Z6;
      a.nin = 9;
      a.nout = 6;
      if ((rc = Ops<R>::go(p, OP_KZ_ADJ, a, "kz adjoint"))) return rc;
      a = Ops<R>::base(p);
      a.in = Z6;
      a.out = Y9;
      a.nin = a.nout = 6;
      if ((rc = Ops<R>::go(p, OP_KY_FWD, a, "ky adjoint forward"))) return rc;
      a = Ops<R>::base(p);
      a.in = Y9;
      a.spec_out = out;
      a.nin = 6;
      return Ops<R>::go(p, OP_KX_ADJ_FWD, a, "kx adjoint forward");
    }
    if ((rc = copy(WMU, W))) return rc;
    if ((rc = copy(WMU + 3 * p->g.sS, m))) return rc;
    PassArgs<R> a = Ops<R>::base(p);
    a.spec_in = WMU;
    a.out = X9;
    a.map = MAP_ADJ;
    a.nin = 6;
    a.nout = 9;
    if ((rc = Ops<R>::go(p, OP_KX_LOAD6, a, "kx adjoint load"))) return rc;
    a = Ops<R>::base(p);
    a.in = X9;
    a.out = Y9;
    a.nin = a.nout = 9;
    if ((rc = Ops<R>::go(p, OP_KY_INV, a, "ky adjoint inverse"))) return rc;
    a = Ops<R>::base(p);
    a.in = Y9;
    a.out = Z6;
    a.nin = 9;
    a.nout = 6;
    if ((rc = Ops<R>::go(p, OP_KZ_ADJ, a, "kz adjoint"))) return rc;
    a = Ops<R>::base(p);
    a.in = Z6;
    a.out = Y9;
    a.nin = a.nout = 6;
    if ((rc = Ops<R>::go(p, OP_KY_FWD, a, "ky adjoint forward"))) return rc;
    a = Ops<R>::base(p);
    a.in = Y9;
    a.spec_out = out;
    a.nin = 6;
    a.flags |= FLAG_ADJ;
    return Ops<R>::go(p, OP_KX_FWD6, a, "kx adjoint forward");
  }
  int launch_check(const char* what) {
    TG_CUDA(cudaGetLastError(), what);
    return TG_OK;
  }
  // lam_out = (d step / d V)^T lam_in at V; dnu += d(step)/d(nu) . lam_in
  int step_adjoint(const C* V, const C* L, C* lam_out, double nu, double h) {
    int rc;
    const Geo& g = p->g;
    cudaStream_t st = p->st;
    if ((rc = nonlin(V, n1))) return rc;
    lawson_stage_kernel<R><<<blocks, 256, 0, st>>>(2, V, n1, a2, g, nu, h);
    if ((rc = launch_check("lawson stage"))) return rc;
    if ((rc = nonlin(a2, n2))) return rc;
    lawson_stage_kernel<R><<<blocks, 256, 0, st>>>(3, V, n2, a3, g, nu, h);
    if ((rc = nonlin(a3, n3))) return rc;
    lawson_stage_kernel<R><<<blocks, 256, 0, st>>>(4, V, n3, a4, g, nu, h);
    adj_mu_kernel<R><<<blocks, 256, 0, st>>>(4, L, nullptr, mu, g, nu, h);
    if ((rc = launch_check("adjoint seeds"))) return rc;
    if ((rc = nonlin_adj(a4, mu, g4))) return rc;
    adj_mu_kernel<R><<<blocks, 256, 0, st>>>(3, L, g4, mu, g, nu, h);
    if ((rc = nonlin_adj(a3, mu, g3))) return rc;
    adj_mu_kernel<R><<<blocks, 256, 0, st>>>(2, L, g3, mu, g, nu, h);
    if ((rc = nonlin_adj(a2, mu, g2))) return rc;
    adj_mu_kernel<R><<<blocks, 256, 0, st>>>(1, L, g2, mu, g, nu, h);
    if ((rc = nonlin_adj(V, mu, g1))) return rc;
    adj_lambda_kernel<R><<<blocks, 256, 0, st>>>(L, g1, g2, g3, g4, lam_out, g, nu, h);
    adj_dnu_partial<R><<<kDnuBlocks, kDiagThreads, 0, st>>>(L, V, a2, n1, n2, n3, g2, g3, g4, g, nu, h, dpart);
    accumulate_partials<<<1, 32, 0, st>>>(dpart, kDnuBlocks, dnu);
    p->launches += 10;
    return launch_check("adjoint combine");
  }

  // ---------------------------------------------------------------- stage tape
  // One graph-launched forward sweep in which the x stage kernels also write, per step,
  // the input state V and the stage nonlinear terms n1, n2, n3 into one of two device
  // slots; a copy stream moves every slot to pinned host memory.  The backward sweep
  // streams the tape back (each buffer refilled as soon as its last reader has run)
  // and runs the four adjoint stages of each step with no state recomputed:
  //   stage s:  x (mu_s = seeds of L, g_{s+1}; a = P mu_s) -> y -> x (u, omega of the
  //             stage state a_s, formed from V and n_{s-1}) -> y -> z (in place, nine
  //             fields in the plan's Y|Z block) -> y -> x (g_s; lam accumulated)
  //             -> d/dnu partial sums
  // Device memory beyond the plan: the two slots (eight states, reused by the backward
  // sweep as V[2], n1, n2, n3, L, lam, g), the working state and the partial sums.
  std::vector<cudaEvent_t> evs;
  cudaStream_t cs = nullptr;
  cudaGraphExec_t gx[2] = {nullptr, nullptr};
  cudaGraph_t gg[2] = {nullptr, nullptr};
  cudaEvent_t event() {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) evs.push_back(e);
    return e;
  }
  void release_tape() {
    for (int k = 0; k < 2; ++k) {
      if (gx[k]) cudaGraphExecDestroy(gx[k]);
      if (gg[k]) cudaGraphDestroy(gg[k]);
      gx[k] = nullptr;
      gg[k] = nullptr;
    }
    if (cs) cudaStreamSynchronize(cs);
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    evs.clear();
    if (cs) cudaStreamDestroy(cs);
    cs = nullptr;
  }
  // capture stages(S) with the tape pointer set (the step graph of one tape slot)
  int capture(int k, C* S, C* tape) {
    if (!p->cap) TG_CUDA(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking), "capture stream");
    cudaStream_t user = p->st;
    TG_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    const int64_t before = p->launches;
    p->st = p->cap;
    p->tape = tape;
    int rc = Ops<R>::stages(p, S);
    p->tape = nullptr;
    p->st = user;
    p->launches = before;
    cudaError_t e = cudaStreamEndCapture(p->cap, &gg[k]);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "tape end capture");
    TG_CUDA(cudaGraphInstantiate(&gx[k], gg[k], 0), "tape graph instantiate");
    return TG_OK;
  }
  // y and z passes of one adjoint stage: a (x-pass layout, first three field slots of Y)
  // and u, omega (X) -> Y (nine fields) -> in-place z (p, q) -> forward y -> X (six fields)
  int tape_yz() {
    int rc;
    const Geo& g = p->g;
    C* X = static_cast<C*>(p->X);
    C* Y = static_cast<C*>(p->Y);
    PassArgs<R> b = Ops<R>::base(p);
    b.in = Y;  // x-pass layout (field stride sX)
    b.out = Y + 6 * g.sY;
    b.nin = b.nout = 3;
    if ((rc = Ops<R>::go(p, OP_KY_INV, b, "ky adjoint inverse (a)"))) return rc;
    b = Ops<R>::base(p);
    b.in = X;
    b.out = Y;
    b.nin = b.nout = 6;
    if ((rc = Ops<R>::go(p, OP_KY_INV, b, "ky adjoint inverse (u, omega)"))) return rc;
    b = Ops<R>::base(p);
    b.in = Y;
    b.out = Y;  // in place: p, q over u, omega
    b.nin = 9;
    b.nout = 6;
    if ((rc = Ops<R>::go(p, OP_KZ_ADJ, b, "kz adjoint"))) return rc;
    b = Ops<R>::base(p);
    b.in = Y;
    b.out = X;
    b.nin = b.nout = 6;
    return Ops<R>::go(p, OP_KY_FWD, b, "ky adjoint forward");
  }
  // adjoint x pass of stage s: OP_KX_ADJ_LOAD (mu_s from L and g_{s+1} in G; a, u, omega)
  // or OP_KX_ADJ_FWD (g_s into G unless null; lam accumulated in LA; nu partials into part)
  int tape_x(int op, int s, const C* const tp[4], const C* L, C* LA, C* G, double* part) {
    PassArgs<R> a = Ops<R>::base(p);
    a.flags |= FLAG_TAPE;
    a.stage = s;
    for (int i = 0; i < 4; ++i) a.tp[i] = tp[i];
    a.in = static_cast<C*>(p->X);
    a.out = static_cast<C*>(p->X);
    a.out2 = static_cast<C*>(p->Y);
    a.S = const_cast<C*>(L);
    a.acc = G;
    a.spec_out = G;
    a.vs = LA;
    a.part = part;
    a.nin = 6;
    a.nout = 9;
    return Ops<R>::go(p, op, a, "kx adjoint");
  }
  // The stage-tape adjoint.  seglen >= nsteps: one forward sweep records the tape of every
  // step in pinned host memory, and the backward sweep reads it back.  seglen < nsteps
  // (sqrt(n) checkpointing): a forward sweep keeps the state at the start of every segment
  // of seglen steps (pinned host memory) and records the last segment's tape; the segments
  // are then taken last to first, each (but the last) recomputed from its checkpoint with its
  // tape recorded (seglen steps of tape in host memory) and swept backwards.  While a segment is recomputed, lam (whose device buffer
  // is a tape slot then) is parked in host memory.  Device memory beyond the plan is the
  // same in both schedules: the two tape slots (eight states, the backward buffers V x 2,
  // n1, n2, n3, lam x 2, g), the working state and the partial sums.
  int run_tape(const void* state0, double dt, double nu, int nsteps, int seglen, void* grad, double* grad_nu,
               double* loss) {
    int rc;
    const Geo& g = p->g;
    cudaStream_t st = p->st;
    fbytes = sizeof(C) * 3 * (size_t)g.sS;
    const size_t sN = 3 * (size_t)g.sS;  // elements of one state
    seglen = std::max(1, std::min(seglen, nsteps));
    const int nseg = (nsteps + seglen - 1) / seglen;
    const size_t tape_states = (size_t)seglen * 4;
    const size_t extra_states = (nseg > 1) ? (size_t)nseg + 1 : 0;  // checkpoints, parked lam
    const size_t need = (tape_states + extra_states) * fbytes;
    if (p->htape_bytes < need) {
      if (p->htape) cudaFreeHost(p->htape);
      p->htape = nullptr;
      p->htape_bytes = 0;
      cudaError_t e = cudaHostAlloc(&p->htape, need, cudaHostAllocDefault);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        p->htape = nullptr;
        return TG_E_NOMEM;  // the caller falls back to recomputing the stage terms
      }
      p->htape_bytes = need;
    }
    C* host = static_cast<C*>(p->htape);
    C* hck = host + tape_states * sN;    // segment checkpoints
    C* hlam = hck + (size_t)nseg * sN;   // lam while a segment is recomputed
    C *slot = nullptr, *cur0 = nullptr;
    if ((rc = alloc((void**)&slot, 8 * fbytes))) return rc;
    if ((rc = alloc((void**)&cur0, fbytes))) return rc;
    if ((rc = alloc((void**)&dnu, sizeof(double)))) return rc;
    // partial sums: stages 4, 3, 2, one slot per CTA of the x pass (its CTAs hold groups of
    // four consecutive kz, so there are at most M x ceil(Hk / 4)); slots a grid with several
    // groups per CTA leaves unwritten stay zero
    const size_t pslots = (size_t)g.M * ((g.Hk + 3) / 4);
    if ((rc = alloc((void**)&dpart, sizeof(double) * 3 * pslots))) return rc;
    TG_CUDA(cudaMemsetAsync(dpart, 0, sizeof(double) * 3 * pslots, st), "memset");
    TG_CUDA(cudaMemsetAsync(dnu, 0, sizeof(double), st), "memset");
    blocks = (int)std::min<long long>(((long long)g.M * g.M * g.Hk + 255) / 256, 2048);
    TG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "copy stream");
    cudaEvent_t written[2] = {event(), event()}, copied[2] = {event(), event()};
    // refill events: a tape buffer is reloaded as soon as its last reader has run
    //   n3 (stage-4 nu terms), n2 (stage-3 state), n1 (stage-2 nu terms), V (stage-1 state)
    cudaEvent_t n3_free = event(), n2_free = event(), n1_free = event(), v_free[2] = {event(), event()};
    cudaEvent_t n3_ready = event(), n2_ready = event(), n1_ready = event(), v_ready[2] = {event(), event()};
    for (cudaEvent_t e : evs)
      if (!e) return fail(TG_E_CUDA, "tg_adjoint: event creation failed");
    C* tslot[2] = {slot, slot + 4 * sN};
    // backward buffers (the tape slots once offloaded)
    C* Vb[2] = {slot, slot + sN};
    C* N1 = slot + 2 * sN;
    C* N2 = slot + 3 * sN;
    C* N3 = slot + 4 * sN;
    C* Lb[2] = {slot + 5 * sN, slot + 6 * sN};
    C* Gb = slot + 7 * sN;

    auto offload = [&](int j, int k) -> int {
      TG_CUDA(cudaEventRecord(written[k], st), "event record");
      TG_CUDA(cudaStreamWaitEvent(cs, written[k], 0), "stream wait");
      TG_CUDA(cudaMemcpyAsync(host + (size_t)j * 4 * sN, tslot[k], 4 * fbytes, cudaMemcpyDeviceToHost, cs),
              "tape offload");
      TG_CUDA(cudaEventRecord(copied[k], cs), "event record");
      return TG_OK;
    };
    // len steps of cur0 (X holding its inverse-x fields) with the x stage kernels writing
    // V, n1, n2, n3 of step j into tape slot j % 2, each slot offloaded to host step j; the
    // first sweep runs its first step eagerly (kernel attributes are set outside capture)
    auto tape_forward = [&](int len) -> int {
      int r;
      int j0 = 0;
      if (!gx[0]) {
        p->tape = tslot[0];
        r = Ops<R>::stages(p, cur0);
        p->tape = nullptr;
        if (r) return r;
        if ((r = offload(0, 0))) return r;
        j0 = 1;
      }
      for (int j = j0; j < len; ++j) {
        const int k = j & 1;
        if (!gx[0]) {
          if ((r = capture(0, cur0, tslot[0]))) return r;
          if ((r = capture(1, cur0, tslot[1]))) return r;
        }
        TG_CUDA(cudaStreamWaitEvent(st, copied[k], 0), "stream wait");  // slot k offloaded
        TG_CUDA(cudaGraphLaunch(gx[k], st), "tape graph launch");
        p->launches += 16;
        if ((r = offload(j, k))) return r;
      }
      // the slots become the backward buffers once offloaded
      TG_CUDA(cudaStreamWaitEvent(st, copied[0], 0), "stream wait");
      TG_CUDA(cudaStreamWaitEvent(st, copied[1], 0), "stream wait");
      return TG_OK;
    };
    auto fetch = [&](int j, C* dst, int item, cudaEvent_t free_, cudaEvent_t ready) -> int {
      TG_CUDA(cudaStreamWaitEvent(cs, free_, 0), "stream wait");
      TG_CUDA(cudaMemcpyAsync(dst, host + ((size_t)j * 4 + item) * sN, fbytes, cudaMemcpyHostToDevice, cs),
              "tape fetch");
      TG_CUDA(cudaEventRecord(ready, cs), "event record");
      return TG_OK;
    };
    auto wait = [&](std::initializer_list<cudaEvent_t> es) -> int {
      for (cudaEvent_t e : es) TG_CUDA(cudaStreamWaitEvent(st, e, 0), "stream wait");
      return TG_OK;
    };
    // one backward step with buffer parity q (the q-th step of a segment's sweep, modulo 2:
    // V in Vb[q], lam read from Lb[q] and written to Lb[q ^ 1]), enqueued on p->st; inside a
    // capture the buffer-free events become external record nodes
    int kernels = 0;
    auto step_work = [&](int q, bool capturing) -> int {
      int r;
      const int64_t before = p->launches;
      const C* tp[4] = {Vb[q], N1, N2, N3};
      const C* Lq = Lb[q];
      C* LAq = Lb[q ^ 1];
      auto record = [&](cudaEvent_t e) -> int {
        TG_CUDA(cudaEventRecordWithFlags(e, p->st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault),
                "event record");
        return TG_OK;
      };
      for (int s = 4; s >= 1; --s) {
        if ((r = tape_x(OP_KX_ADJ_LOAD, s, tp, Lq, LAq, Gb, nullptr))) return r;
        if (s == 3 && (r = record(n2_free))) return r;
        if (s == 1 && (r = record(v_free[q]))) return r;
        if ((r = tape_yz())) return r;
        double* part = (s >= 2) ? dpart + (size_t)(4 - s) * pslots : nullptr;
        if ((r = tape_x(OP_KX_ADJ_FWD, s, tp, Lq, LAq, s > 1 ? Gb : nullptr, part))) return r;
        if (s == 4 && (r = record(n3_free))) return r;
        if (s == 2 && (r = record(n1_free))) return r;
      }
      accumulate_partials_wide<<<1, 256, 0, p->st>>>(dpart, (int)(3 * pslots), dnu);
      ++p->launches;
      if ((r = launch_check("adjoint nu sum"))) return r;
      kernels = (int)(p->launches - before);
      return TG_OK;
    };
    cudaGraphExec_t bx[2] = {nullptr, nullptr};
    cudaGraph_t bg[2] = {nullptr, nullptr};
    struct GraphGuard {  // the backward step graphs are released on every return path
      cudaGraphExec_t* x;
      cudaGraph_t* g;
      ~GraphGuard() {
        for (int k = 0; k < 2; ++k) {
          if (x[k]) cudaGraphExecDestroy(x[k]);
          if (g[k]) cudaGraphDestroy(g[k]);
        }
      }
    } guard{bx, bg};
    // backward over the len steps of the tape in host memory; lam enters in Lb[0] and is
    // left in Lb[0]
    auto backward = [&](int len) -> int {
      int r;
      for (cudaEvent_t e : {v_free[0], v_free[1], n1_free, n2_free, n3_free})  // the slots are free
        TG_CUDA(cudaEventRecord(e, st), "event record");
      for (int k = 0; k < len; ++k) {
        const int j = len - 1 - k, q = k & 1;
        if (k == 0) {
          if ((r = fetch(j, Vb[0], 0, v_free[0], v_ready[0]))) return r;
          if ((r = fetch(j, N3, 3, n3_free, n3_ready))) return r;
          if ((r = fetch(j, N2, 2, n2_free, n2_ready))) return r;
          if ((r = fetch(j, N1, 1, n1_free, n1_ready))) return r;
        }
        if ((r = wait({v_ready[q], n1_ready, n2_ready, n3_ready}))) return r;
        if (!bx[0]) {  // eagerly (sets the kernels' attributes outside capture), then one graph per parity
          if ((r = step_work(q, false))) return r;
          if (!p->cap) TG_CUDA(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking), "capture stream");
          for (int b = 0; b < 2; ++b) {
            cudaStream_t user = p->st;
            TG_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
            const int64_t before = p->launches;
            p->st = p->cap;
            r = step_work(b, true);
            p->st = user;
            p->launches = before;
            cudaError_t e = cudaStreamEndCapture(p->cap, &bg[b]);
            if (r) return r;
            if (e != cudaSuccess) return cuda_fail(e, "adjoint end capture");
            TG_CUDA(cudaGraphInstantiate(&bx[b], bg[b], 0), "adjoint graph instantiate");
          }
        } else {
          TG_CUDA(cudaGraphLaunch(bx[q], st), "adjoint graph launch");
          p->launches += kernels;
        }
        if (j > 0) {  // refill with step j - 1 once step j's readers are done (V: the other buffer)
          const int qn = (k + 1) & 1;
          if ((r = fetch(j - 1, Vb[qn], 0, v_free[qn], v_ready[qn]))) return r;
          if ((r = fetch(j - 1, N3, 3, n3_free, n3_ready))) return r;
          if ((r = fetch(j - 1, N2, 2, n2_free, n2_ready))) return r;
          if ((r = fetch(j - 1, N1, 1, n1_free, n1_ready))) return r;
        }
      }
      if (len & 1) TG_CUDA(cudaMemcpyAsync(Lb[0], Lb[1], fbytes, cudaMemcpyDeviceToDevice, st), "lam copy");
      return TG_OK;
    };

    // phase timing: a timing event before the work and after every phase
    std::vector<cudaEvent_t> tev;
    std::vector<int> tphase;  // phase that ends at tev[i] (i >= 1)
    struct TevGuard {
      std::vector<cudaEvent_t>* v;
      ~TevGuard() {
        for (cudaEvent_t e : *v) cudaEventDestroy(e);
      }
    } tev_guard{&tev};
    auto mark = [&](int phase) -> int {
      cudaEvent_t e = nullptr;
      TG_CUDA(cudaEventCreate(&e), "event");
      tev.push_back(e);
      tphase.push_back(phase);
      TG_CUDA(cudaEventRecord(e, st), "event record");
      return TG_OK;
    };
    if ((rc = mark(-1))) return rc;
    TG_CUDA(cudaMemcpyAsync(cur0, state0, fbytes, cudaMemcpyDeviceToDevice, st), "state copy");
    if (nseg == 1) {  // the tape sweep is the forward run
      if ((rc = Ops<R>::start(p, cur0))) return rc;
      if ((rc = tape_forward(nsteps))) return rc;
    } else {  // the forward run keeps the segment checkpoints and records the last segment's tape
      for (int c = 0; c < nseg; ++c) {
        const int len = std::min(seglen, nsteps - c * seglen);
        if ((rc = Ops<R>::start(p, cur0))) return rc;
        if (c == nseg - 1) {
          if ((rc = tape_forward(len))) return rc;
        } else {
          TG_CUDA(cudaMemcpyAsync(hck + (size_t)c * sN, cur0, fbytes, cudaMemcpyDeviceToHost, st), "checkpoint");
          if ((rc = advance(p, cur0, len))) return rc;
        }
      }
    }
    // loss = enstrophy of the final state, lam = its gradient
    if ((rc = Ops<R>::diagnostics(p, cur0, p->dtmp))) return rc;
    copy_double<<<1, 32, 0, st>>>(p->dtmp + TG_D_ENSTROPHY, loss);
    enstrophy_grad_kernel<R><<<blocks, 256, 0, st>>>(cur0, Lb[0], g);
    if ((rc = launch_check("loss gradient"))) return rc;
    if ((rc = mark(0))) return rc;
    if (nseg == 1) {
      if ((rc = backward(nsteps))) return rc;
      if ((rc = mark(2))) return rc;
    } else {
      for (int c = nseg - 1; c >= 0; --c) {
        const int len = std::min(seglen, nsteps - c * seglen);
        if (c < nseg - 1) {  // recompute the segment from its checkpoint, recording its tape
          TG_CUDA(cudaMemcpyAsync(hlam, Lb[0], fbytes, cudaMemcpyDeviceToHost, st), "lam park");
          TG_CUDA(cudaMemcpyAsync(cur0, hck + (size_t)c * sN, fbytes, cudaMemcpyHostToDevice, st), "checkpoint");
          if ((rc = Ops<R>::start(p, cur0))) return rc;
          if ((rc = tape_forward(len))) return rc;
          TG_CUDA(cudaMemcpyAsync(Lb[0], hlam, fbytes, cudaMemcpyHostToDevice, st), "lam unpark");
        }
        if ((rc = mark(1))) return rc;
        if ((rc = backward(len))) return rc;
        if ((rc = mark(2))) return rc;
      }
    }
    TG_CUDA(cudaMemcpyAsync(grad, Lb[0], fbytes, cudaMemcpyDeviceToDevice, st), "grad copy");
    TG_CUDA(cudaMemcpyAsync(grad_nu, dnu, sizeof(double), cudaMemcpyDeviceToDevice, st), "grad_nu copy");
    TG_CUDA(cudaStreamSynchronize(st), "adjoint sync");
    for (int i = 0; i < 3; ++i) p->adj_ms[i] = 0.0;
    for (size_t i = 1; i < tev.size(); ++i) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, tev[i - 1], tev[i]) == cudaSuccess) p->adj_ms[tphase[i]] += ms;
    }
    drop_graph(p);  // the plan's step graph of the checkpoint sweep refers to cur0
    return TG_OK;
  }

  int run(const void* state0, double dt, double nu, int nsteps, int seglen, void* grad, double* grad_nu,
          double* loss) {
    int rc;
    const int nck = (nsteps + seglen - 1) / seglen;
    if ((rc = setup(seglen, nck))) return rc;
    cudaStream_t st = p->st;
    const Geo& g = p->g;
    // forward sweep, keeping the state at the start of every segment
    if ((rc = copy(cur, static_cast<const C*>(state0)))) return rc;
    for (int c = 0; c < nck; ++c) {
      if ((rc = copy(ck + (size_t)c * 3 * g.sS, cur))) return rc;
      const int len = std::min(seglen, nsteps - c * seglen);
      if ((rc = Ops<R>::start(p, cur))) return rc;
      if ((rc = advance(p, cur, len))) return rc;  // graph-launched steps
    }
    // loss = enstrophy of the final state, and its gradient
    if ((rc = Ops<R>::diagnostics(p, cur, p->dtmp))) return rc;
    copy_double<<<1, 32, 0, st>>>(p->dtmp + TG_D_ENSTROPHY, loss);
    enstrophy_grad_kernel<R><<<blocks, 256, 0, st>>>(cur, lam, g);
    TG_CUDA(cudaMemsetAsync(dnu, 0, sizeof(double), st), "memset");
    if ((rc = launch_check("loss gradient"))) return rc;
    // backward sweep over the segments, recomputing each segment's states
    for (int c = nck - 1; c >= 0; --c) {
      const int len = std::min(seglen, nsteps - c * seglen);
      if ((rc = copy(seg, ck + (size_t)c * 3 * g.sS))) return rc;
      for (int j = 1; j < len; ++j) {
        C* sj = seg + (size_t)j * 3 * g.sS;
        if ((rc = copy(sj, sj - 3 * g.sS))) return rc;
        if ((rc = step(sj))) return rc;
      }
      for (int j = len - 1; j >= 0; --j) {
        if ((rc = step_adjoint(seg + (size_t)j * 3 * g.sS, lam, lamn, nu, dt))) return rc;
        std::swap(lam, lamn);
      }
    }
    TG_CUDA(cudaMemcpyAsync(grad, lam, fbytes, cudaMemcpyDeviceToDevice, st), "grad copy");
    TG_CUDA(cudaMemcpyAsync(grad_nu, dnu, sizeof(double), cudaMemcpyDeviceToDevice, st), "grad_nu copy");
    // the work buffers are freed on return: finish first
    TG_CUDA(cudaStreamSynchronize(st), "adjoint sync");
    return TG_OK;
  }
};

}  // namespace

extern "C" int tg_adjoint(tg_plan* p, const void* state0, double dt, double nu, int nsteps, int checkpoint_every,
                          void* grad_state, double* grad_nu, double* loss) {
  if (!p || !state0 || !grad_state || !grad_nu || !loss) return fail(TG_E_INVALID, "tg_adjoint: null argument");
  if (p->F != 3 || p->batch != 1) return fail(TG_E_UNSUPPORTED, "tg_adjoint: hydro plans with batch 1 only");
  if (!(dt > 0.0) || !(nu >= 0.0) || nsteps < 1)
    return fail(TG_E_INVALID, "tg_adjoint: need dt > 0, nu >= 0 and nsteps >= 1");
  if (p->flags & TG_FLAG_EXPLICIT_VISC)
    return fail(TG_E_UNSUPPORTED, "tg_adjoint: differentiates the integrating-factor RK4 only");
  // segment length: the whole run for the host tape, else the checkpoint spacing
  const int sqrt_len = (int)std::ceil(std::sqrt((double)nsteps));
  const int tape_len = (checkpoint_every == TG_ADJ_HOST_TAPE) ? nsteps
                       : (checkpoint_every > 0 ? checkpoint_every : sqrt_len);
  if (p->prec == TG_PREC_F32 && has_reg_adjoint(p->n) && (p->variant & ~4) == 0) {
    // the stage-tape kernels: the tape of one segment (or of the whole run) in host memory
    int rc = set_coefs(p, dt, nu, 0.0);
    if (rc) return rc;
    p->launches = 0;
    Adjoint<float> A{p};
    rc = A.run_tape(state0, dt, nu, nsteps, tape_len, grad_state, grad_nu, loss);
    if (rc != TG_E_NOMEM) return rc;
    (void)cudaGetLastError();  // no pinned host memory for the tape: recompute instead
  }
  if (checkpoint_every == TG_ADJ_HOST_TAPE) checkpoint_every = 0;
  int seglen = checkpoint_every > 0 ? checkpoint_every : (int)std::ceil(std::sqrt((double)nsteps));
  seglen = std::max(1, std::min(seglen, nsteps));
  int rc = set_coefs(p, dt, nu, 0.0);
  if (rc) return rc;
  p->launches = 0;
  if (p->prec == TG_PREC_F64) {
    Adjoint<double> A{p};
    return A.run(state0, dt, nu, nsteps, seglen, grad_state, grad_nu, loss);
  }
  Adjoint<float> A{p};
  return A.run(state0, dt, nu, nsteps, seglen, grad_state, grad_nu, loss);
}

extern "C" int tg_spectrum_bins(const tg_plan* p) {
  return p ? (int)std::floor(std::sqrt(3.0) * p->K + 0.5) + 1 : 0;
}

extern "C" int tg_energy_spectrum(tg_plan* p, const void* state, double* out) {
  if (!p || !state || !out) return fail(TG_E_INVALID, "tg_energy_spectrum: null argument");
  const int nbins = tg_spectrum_bins(p);
  double* part = nullptr;
  const size_t pbytes = sizeof(double) * (size_t)p->batch * kSpecBlocks * 2 * nbins;
  cudaError_t e = cudaMallocAsync((void**)&part, pbytes, p->st);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(TG_E_NOMEM, std::string("tg_energy_spectrum: ") + cudaGetErrorString(e));
  }
  dim3 grid(kSpecBlocks, p->batch);
  const size_t shm = sizeof(double) * 2 * nbins;
  if (p->prec == TG_PREC_F64)
    spectrum_partial<double><<<grid, 256, shm, p->st>>>(static_cast<const cplx<double>*>(state), p->g, p->F, nbins, part);
  else
    spectrum_partial<float><<<grid, 256, shm, p->st>>>(static_cast<const cplx<float>*>(state), p->g, p->F, nbins, part);
  spectrum_final<<<p->batch, 128, 0, p->st>>>(part, kSpecBlocks, nbins, p->F, out);
  e = cudaGetLastError();
  cudaFreeAsync(part, p->st);
  if (e != cudaSuccess) return cuda_fail(e, "tg_energy_spectrum");
  return TG_OK;
}

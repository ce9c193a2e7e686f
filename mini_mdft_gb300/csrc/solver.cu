// solver.cu -- the caller of the energy/gradient path: a solute's external
// potential on the grid and an L-BFGS minimisation of the MDFT functional in
// xi = sqrt(rho / rho0) (the loop around Solver::energy_cproj_mrso,
// src/mini-mdft.hpp:130-183).
//
// The reference defines the data these terms use -- solvent and solute sites
// (charge, sigma, epsilon, position: common/MDFT_Solvent.hpp:410-494,
// common/MDFT_Solute.hpp:150-200), the rotation matrix of each orientation
// (common/MDFT_Grid.hpp:283-310), qfact and kT (common/MDFT_Constants.hpp:
// 46-47, common/MDFT_Thermo.hpp:60) -- but computes neither the external
// potential, nor the ideal and external energies, nor a minimiser step.  The
// formulas here are the standard MDFT functional in the xi parameterisation,
// with no reference result to match:
//
//   vext(r, o) = sum_a sum_s 4 eps_as [(sig_as/d)^12 - (sig_as/d)^6] + qfact q_a q_s / d
//       d = |r + R(o) x_a - x_s| under the minimum-image convention (d^2 >= 1e-12),
//       eps_as = sqrt(eps_a eps_s), sig_as = (sig_a + sig_s) / 2 (Lorentz-Berthelot),
//       clamped to [-vmax, vmax] (vmax where the sum is not finite);
//   E_id  = kT rho0 dv sum_{r,o} w_o (xi^2 ln xi^2 - xi^2 + 1)
//   E_ext =    rho0 dv sum_{r,o} w_o xi^2 vext
//   E_exc = ff of get_delta_f = prefactor rho0 sum_{r,o} w_o vexc (xi^2 - 1)
//   dE/dxi = 2 rho0 dv w_o xi (kT ln xi^2 + vext) + 2 prefactor w_o df,  df = 2 rho0 xi vexc
//
// The last term is the exact gradient of ff when the direct correlation
// function is symmetric, c(1,2) = c(2,1) (the weighted convolution is then
// self-adjoint); for a table without that symmetry it is the reference's df
// scaled the same way, not a gradient.
//
// The minimiser is L-BFGS (Nocedal 1980; the two-loop recursion of Liu and
// Nocedal 1989) with an Armijo backtracking line search.  Every vector pass
// over the field is one kernel that updates one vector and forms the next
// dot product the recursion needs (2h + 1 passes per direction for h stored
// pairs); the dot products' scalars stay on the device, so the host only
// reads the energies and the curvature of each accepted step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "handles.hpp"
#include "solver.hpp"

using mdft::DevBuf;
using mdft::Error;
using mdft::throw_if;

namespace mdft {
namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 152 * 8;  // largest grid of the streaming reductions
constexpr int kMaxHistory = 32;

// ---- deterministic grid-wide sums -----------------------------------------
// Each thread accumulates its elements (FP64 multiply-adds, or double-float
// sums; the FP64 pipe of this GPU is 1/64 as wide as the FP32 one, so a
// compensated FP64 sum per element would bound the streaming kernels); the
// threads' sums are combined as double-double values: a CTA adds its warps in
// a fixed order and writes its partials, the last CTA to finish adds all
// partials in CTA order.  With the fixed grid of kRedBlocks CTAs the result
// does not depend on scheduling.
struct Dd {
  double hi, lo;
};
__device__ __forceinline__ Dd dd_plus(Dd a, Dd b) {
  const double s = a.hi + b.hi;
  const double bb = s - a.hi;
  const double e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
  const double h = s + e;
  return Dd{h, e - (h - s)};
}
__device__ __forceinline__ Dd dd_plus(Dd a, double b) { return dd_plus(a, Dd{b, 0.0}); }

template <int K>
struct Red {
  Dd s[K];
  double mx;
};
template <int K>
__device__ __forceinline__ Red<K> red_zero() {
  Red<K> r;
#pragma unroll
  for (int k = 0; k < K; ++k) r.s[k] = Dd{0.0, 0.0};
  r.mx = 0.0;
  return r;
}
template <int K>
__device__ __forceinline__ void red_add(Red<K>& a, const Red<K>& b) {
#pragma unroll
  for (int k = 0; k < K; ++k) a.s[k] = dd_plus(a.s[k], b.s[k]);
  a.mx = fmax(a.mx, b.mx);
}
// part: (gridDim.x, 2K + 1) doubles; counter: zero on entry, left zero
template <int K, typename Fin>
__device__ void grid_reduce(Red<K> r, double* __restrict__ part, unsigned* __restrict__ counter, Fin fin) {
  constexpr int W = 2 * K + 1;
  __shared__ double sh[kRedThreads / 32][W];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    Red<K> o;
#pragma unroll
    for (int k = 0; k < K; ++k)
      o.s[k] = Dd{__shfl_down_sync(0xffffffffu, r.s[k].hi, off), __shfl_down_sync(0xffffffffu, r.s[k].lo, off)};
    o.mx = __shfl_down_sync(0xffffffffu, r.mx, off);
    red_add(r, o);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      sh[wid][2 * k] = r.s[k].hi;
      sh[wid][2 * k + 1] = r.s[k].lo;
    }
    sh[wid][2 * K] = r.mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Red<K> t = red_zero<K>();
    for (int w = 0; w < kRedThreads / 32; ++w) {
      Red<K> o;
      for (int k = 0; k < K; ++k) o.s[k] = Dd{sh[w][2 * k], sh[w][2 * k + 1]};
      o.mx = sh[w][2 * K];
      red_add(t, o);
    }
    double* q = part + (size_t)blockIdx.x * W;
    for (int k = 0; k < K; ++k) {
      q[2 * k] = t.s[k].hi;
      q[2 * k + 1] = t.s[k].lo;
    }
    q[2 * K] = t.mx;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return;
  // the last CTA's first warp: lane l adds partials l, l + 32, ..., then the
  // lanes combine in the fixed shuffle order
  __threadfence();
  Red<K> t = red_zero<K>();
  for (unsigned b = lane; b < gridDim.x; b += 32) {
    const double* q = part + (size_t)b * W;
    Red<K> o;
#pragma unroll
    for (int k = 0; k < K; ++k) o.s[k] = Dd{__ldcg(q + 2 * k), __ldcg(q + 2 * k + 1)};
    o.mx = __ldcg(q + 2 * K);
    red_add(t, o);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    Red<K> o;
#pragma unroll
    for (int k = 0; k < K; ++k)
      o.s[k] = Dd{__shfl_down_sync(0xffffffffu, t.s[k].hi, off), __shfl_down_sync(0xffffffffu, t.s[k].lo, off)};
    o.mx = __shfl_down_sync(0xffffffffu, t.mx, off);
    red_add(t, o);
  }
  if (lane == 0) {
    fin(t);
    *counter = 0u;
  }
}

// Warp sums of per-thread double-float values on the FP32 pipes (shuffles
// in a fixed order): the L-BFGS dot products are double-float Dot2 sums per
// thread, so double-float combining keeps their precision, where combining
// them as double-doubles would spend tens of microseconds per launch on the
// narrow FP64 pipe.
template <int K>
__device__ __forceinline__ void df_warp_sum(DF (&v)[K]) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k)
      v[k] = v[k] + DF(__shfl_down_sync(0xffffffffu, v[k].hi, off), __shfl_down_sync(0xffffffffu, v[k].lo, off));
}

// grid of a streaming reduction: at most `cap` CTAs (the energy kernel
// passes 4 per SM, the CTAs its registers allow)
unsigned red_blocks(long long n, int cap = kRedBlocks) {
  const long long b = (n + kRedThreads - 1) / kRedThreads;
  return (unsigned)std::max(1LL, std::min<long long>(b, cap));
}

// ---- external potential ----------------------------------------------------
// Double-float arithmetic on the FP32 pipes; the host supplies every
// coordinate and pair constant as a double-float pair: grid coordinates
// (i L / n), the rotated site offsets R(o) x_a, solute positions, and per
// (solvent site, solute site) 4 eps_as, sig_as^2 and qfact q_a q_s.  1/d is
// a float rsqrt seed and one Newton step in double-float; the minimum-image
// shift is decided on the float part (near half a box the two images are
// equally far, so the choice does not change d).  Solvent sites at the
// molecular origin (the water oxygen) do not depend on the orientation: a
// first pass evaluates them once per grid point.
struct VextPlan {
  int nx, ny, nz, no, nof, n0, nsu;  // offset sites, origin sites, solute sites
  float2 L[3];                       // box lengths
  float il[3];                       // 1 / L (image shift only)
  double vmax;
  const float2* cx;
  const float2* cy;
  const float2* cz;
  const float2* off;  // (no, nof, 3) R(o) x_a
  const float2* su;   // (nsu, 3)
  const float2* pof;  // (nof, nsu, 3) pair constants of the offset sites
  const float2* p0;   // (n0, nsu, 3) pair constants of the origin sites
  float2* v0;         // (N) origin-site potential
};

__device__ __forceinline__ DF f2df(float2 v) { return DF(v.x, v.y); }

// LJ + Coulomb between one solvent site at p and every solute site
__device__ __forceinline__ DF site_potential(const DF (&p)[3], const float2* __restrict__ pc, const VextPlan& P) {
  DF v(0.f, 0.f);
  for (int s = 0; s < P.nsu; ++s) {
    Acc<DF> d2a;
    acc_zero(d2a);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      DF d = p[k] - f2df(P.su[3 * s + k]);
      const float f = rintf(d.hi * P.il[k]);
      if (f != 0.f) d = d - DF(f, 0.f) * f2df(P.L[k]);
      acc_mac(d2a, d, d);
    }
    DF d2 = acc_get(d2a);
    if (!(d2.hi >= 1e-12f)) d2 = DF(1e-12f, 0.f);
    const float y0 = rsqrtf(d2.hi);
    const DF yy0 = DF(y0, 0.f) * DF(y0, 0.f);
    const DF e = DF(1.f, 0.f) - d2 * yy0;
    const DF y = DF(y0, 0.f) + DF(0.5f * y0, 0.f) * e;  // 1/d
    const float2* c = pc + 3 * s;
    if (c[0].x != 0.f) {
      const DF s2 = f2df(c[1]) * (y * y);
      const DF s6 = s2 * s2 * s2;
      v = v + f2df(c[0]) * (s6 * s6 - s6);
    }
    if (c[2].x != 0.f) v = v + f2df(c[2]) * y;
  }
  return v;
}

__global__ void __launch_bounds__(256) vext_origin_kernel(const VextPlan P) {
  const long long n = (long long)P.nx * P.ny * P.nz;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    const int iz = (int)(r % P.nz);
    const long long rxy = r / P.nz;
    const int iy = (int)(rxy % P.ny), ix = (int)(rxy / P.ny);
    const DF p[3] = {f2df(P.cx[ix]), f2df(P.cy[iy]), f2df(P.cz[iz])};
    DF v(0.f, 0.f);
    for (int a = 0; a < P.n0; ++a) v = v + site_potential(p, P.p0 + (size_t)3 * P.nsu * a, P);
    P.v0[r] = make_float2(v.hi, v.lo);
  }
}

__global__ void __launch_bounds__(256) vext_kernel(const VextPlan P, double* __restrict__ vext) {
  const long long n = (long long)P.nx * P.ny * P.nz * P.no;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / P.no;
    const int o = (int)(i - r * P.no);
    const int iz = (int)(r % P.nz);
    const long long rxy = r / P.nz;
    const int iy = (int)(rxy % P.ny), ix = (int)(rxy / P.ny);
    const DF px = f2df(P.cx[ix]), py = f2df(P.cy[iy]), pz = f2df(P.cz[iz]);
    DF v = f2df(P.v0[r]);
    for (int a = 0; a < P.nof; ++a) {
      const float2* q = P.off + 3 * ((size_t)o * P.nof + a);
      const DF p[3] = {px + f2df(q[0]), py + f2df(q[1]), pz + f2df(q[2])};
      v = v + site_potential(p, P.pof + (size_t)3 * P.nsu * a, P);
    }
    const double vd = df_to_double(v);
    vext[i] = isfinite(vd) ? fmin(fmax(vd, -P.vmax), P.vmax) : P.vmax;
  }
}

// ---- energy and gradient ---------------------------------------------------
// Double-float arithmetic on the FP32 pipes (this GPU's FP64 pipe is 1/64 of
// them): per element one FMA forms t = xi^2 - 1 in FP64 (no cancellation near
// the bulk value xi = 1), the rest runs on double-float pairs, and only
// elements with |xi| outside [2^-20, 2^20] (solute cores, where xi^2 leaves
// the float exponent range) take the FP64 formulas.
//
// ln(xi^2) = e ln 2 + 2 atanh(s), s = (m - 1)/(m + 1), xi^2 = m 2^e with m in
// [1/sqrt 2, sqrt 2) (m - 1 exact; for e = 0 the FMA value of xi^2 - 1), and
// atanh(s) = s sum_k s^2k / (2k + 1) (the classical series; |s| <= 0.1716,
// so ten terms leave a truncation below 2^-55; the terms from k = 5 on, below
// 2e-9 of the sum, are added in float).
}  // namespace
struct EgArgs {
  const double* xi;
  const void* vexc;    // double (FP64 fields) or float (MDFT_F32)
  const double* vext;  // null: no external potential
  const double* w;
  double* g;
  long long n;
  int no;
  double kT, rho0, dv, prefactor;
  float kh, kl, ch, cl, xh, xl;  // kT, rho0 dv, 2 prefactor rho0 as double-float pairs
  float ln2h, ln2l;
  float ah[10], al[10];          // 1 / (2k + 1), k = 0..9
  double* out;  // [E_total, E_id, E_ext, E_exc, max |g|]
  // reduction scratch of field 0: (CTAs, 9) doubles, then at counter_off
  // the completion counter; field f's at f scratch_stride bytes further
  void* scratch;
  size_t counter_off, scratch_stride;
  long long out_stride;  // doubles between the fields' out blocks
  const float* dir;      // search direction (may be null): out[5] = g . dir
  // 1 / D with D = 2 rho0 dv w kT max(ln xi^2 + 2 + vext/kT, 1): the local
  // terms' curvature d^2/dxi^2 (E_id + E_ext), floored at half its value at
  // their minimum -- the minimiser's diagonal preconditioner (may be null)
  float* hinv;
};
namespace {

// Dekker's division (1971): the quotient of the leading floats, corrected once
// from the remainder formed with an exact product.
// The correction r / b.hi (about 2^-24 of the quotient) only has to be good
// to a few ulps of its own: the approximate division (error 2^-46 of the
// quotient at most) instead of a correctly rounded one.
__device__ __forceinline__ DF df_div(DF a, DF b) {
  const float q1 = a.hi / b.hi;
  const float p = q1 * b.hi;
  const float pe = fmaf(q1, b.hi, -p);  // q1 b.hi = p + pe exactly
  const float r = (((a.hi - p) - pe) + a.lo) - q1 * b.lo;
  return df_fast_two_sum(q1, __fdividef(r, b.hi));
}

// a field value as a double-float pair: exact for both storage types
__device__ __forceinline__ DF eg_df(float a) { return DF(a, 0.f); }
__device__ __forceinline__ DF eg_df(double a) { return df_from_double_bits(a); }

// ln(x^2) and x^2 - 1 for 2^-20 <= |x| < 2^21 from one FMA: |x| = mx 2^ex with
// mx in [1, 2); u = mx^2 = m 2^k with m in [1/sqrt 2, sqrt 2) (k = 0, 1, 2 by mx
// against 2^(1/4) and 2^(3/4)); m - 1 = fma(mx, mx, -2^k) / 2^k (one
// rounding); x^2 = m 2^e with e = 2 ex + k, so x^2 - 1 is m - 1 itself for
// e = 0 and (1 + (m - 1)) 2^e - 1 otherwise (then |x^2 - 1| >= 0.29: no
// cancellation).
struct LnSq {
  DF L, t;
};
__device__ __forceinline__ LnSq df_ln_sq(double x, const EgArgs& A) {
  const unsigned long long b = bits_of(x) & 0x7fffffffffffffffull;
  const unsigned long long f = b & 0x000fffffffffffffull;
  const int ex = (int)(b >> 52) - 1023;
  const double mx = double_of(f | 0x3ff0000000000000ull);
  const int k = f < 0x306fe0a31b715ull ? 0 : (f < 0xae89f995ad3adull ? 1 : 2);  // 2^(1/4), 2^(3/4)
  const double r = fma(mx, mx, k == 0 ? -1.0 : (k == 1 ? -2.0 : -4.0));
  const DF rd = df_from_double_bits(r);
  const float sk = k == 0 ? 1.f : (k == 1 ? 0.5f : 0.25f);
  const DF tm(rd.hi * sk, rd.lo * sk);
  const int e = 2 * ex + k;
  const DF s = df_div(tm, tm + DF(2.f, 0.f));
  const DF z = s * s;
  // terms k >= 5 (at most z^5/11 < 2e-9 of the sum) in float, the rest in double-float
  float tail = A.ah[9];
#pragma unroll
  for (int j = 8; j >= 5; --j) tail = fmaf(tail, z.hi, A.ah[j]);
  DF P = DF(tail * z.hi, 0.f) + DF(A.ah[4], A.al[4]);
#pragma unroll
  for (int j = 3; j >= 0; --j) P = P * z + DF(A.ah[j], A.al[j]);
  LnSq o;
  o.L = twice(s * P);
  o.t = tm;
  if (e != 0) {
    o.L = o.L + DF((float)e, 0.f) * DF(A.ln2h, A.ln2l);
    const float p2 = __int_as_float((127 + e) << 23);  // 2^e, |e| <= 42
    const DF u = tm + DF(1.f, 0.f);
    o.t = DF(u.hi * p2, u.lo * p2) - DF(1.f, 0.f);
  }
  return o;
}

// The FP64 formulas, for elements outside the double-float range (x = 0,
// |x| < 2^-20, |x| >= 2^21): a call, so that the common path does not carry
// its FP64 instructions predicated.
struct Terms64 {
  double id, ext, exc, g;
  float hinv;
};
__device__ __noinline__ Terms64 terms_f64(double x, double wo, double v, double ve, const EgArgs A) {
  const double x2 = x * x;
  const double l = x2 > 0.0 ? log(x2) : 0.0;
  const double c_ext = A.rho0 * A.dv, c_exc = A.prefactor * A.rho0;
  return Terms64{wo * (x2 * l - x2 + 1.0), wo * x2 * ve, wo * v * fma(x, x, -1.0),
                 2.0 * x * wo * (c_ext * (A.kT * l + ve) + 2.0 * c_exc * v),
                 (float)(1.0 / (2.0 * wo * c_ext * A.kT * fmax(l + 2.0 + ve / A.kT, 1.0)))};
}

template <typename TV>
__global__ void __launch_bounds__(kRedThreads, 4) eg_kernel(const EgArgs A) {
  extern __shared__ double ws[];  // w as double (no), then as double-float pairs (no)
  float2* wf = reinterpret_cast<float2*>(ws + A.no);
  for (int i = threadIdx.x; i < A.no; i += blockDim.x) {
    const double wv = A.w[i];
    const DF d = df_from_double_bits(wv);
    ws[i] = wv;
    wf[i] = make_float2(d.hi, d.lo);
  }
  __syncthreads();
  // field blockIdx.y of a batch: its arrays start at y n, its outputs and
  // scratch at their strides
  const long long fo = (long long)blockIdx.y * A.n;
  const double* __restrict__ xi = A.xi + fo;
  const TV* __restrict__ vx = static_cast<const TV*>(A.vexc) + fo;
  const double* __restrict__ vext = A.vext ? A.vext + fo : nullptr;
  double* __restrict__ gout = A.g + fo;
  float* __restrict__ hinv = A.hinv ? A.hinv + fo : nullptr;
  const double c_id = A.kT * A.rho0 * A.dv, c_ext = A.rho0 * A.dv, c_exc = A.prefactor * A.rho0;
  const DF kT(A.kh, A.kl), cext(A.ch, A.cl), cexc2(A.xh, A.xl), one(1.f, 0.f);
  // preconditioner constants (the preconditioner only scales search
  // directions: float precision and approximate division are enough)
  const float ikT = 1.f / A.kh, c2k = 2.f * A.ch * A.kh;
  // sums of w (xi^2 ln xi^2 - xi^2 + 1), w xi^2 vext and w vexc (xi^2 - 1):
  // double-float Dot2 accumulators, and plain FP64 sums for the FP64 elements
  Acc<DF> a_id, a_ext, a_exc, a_gd;
  acc_zero(a_id);
  acc_zero(a_ext);
  acc_zero(a_exc);
  acc_zero(a_gd);  // g . dir (with a direction only)
  const float* __restrict__ dir = A.dir ? A.dir + fo : nullptr;
  double d_id = 0.0, d_ext = 0.0, d_exc = 0.0;
  unsigned long long gmax = 0;  // bits of max |g| (non-negative doubles order as integers)
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int o = (int)(i % A.no);
  const int ostep = (int)(stride % A.no);
  for (; i < A.n; i += stride) {
    const double x = xi[i], ve = vext ? vext[i] : 0.0;
    const TV vv = vx[i];
    const unsigned ebits = (unsigned)(bits_of(x) >> 52) & 0x7ffu;
    double gi;
    if constexpr (std::is_same<TV, float>::value) {
      // the mixed form: FP32 arithmetic per element (its vexc is FP32), the
      // sums still Dot2 double-float accumulators; 2^-120 <= |x| < 2^60
      if (ebits - 903u < 180u) {
        const float2 w2 = wf[o];
        const float xf = df_from_double_bits(x).hi;                     // nearest float
        const float tf = df_from_double_bits(fma(x, x, -1.0)).hi;       // xi^2 - 1, no cancellation
        const float vef = df_from_double_bits(ve).hi, xsq = xf * xf;
        float L, fid;  // ln xi^2 and (1 + t) ln(1 + t) - t
        if (tf > -0.5f && tf < 1.f) {
          // f = 2 s^2 Q(s) / (1 - s), s = t / (2 + t), Q = 1 + s/3 + s^2/3
          // + s^3/5 + s^4/5 + ... (from ln(1 + t) = 2 atanh s): no
          // cancellation near xi = 1; |s| < 1/3, the terms to s^14 leave a
          // truncation below 4e-9 of f
          L = log1pf(tf);
          const float sv = __fdividef(tf, 2.f + tf);
          float Q = 1.f / 15.f;
          Q = fmaf(Q, sv, 1.f / 15.f);
          Q = fmaf(Q, sv, 1.f / 13.f);
          Q = fmaf(Q, sv, 1.f / 13.f);
          Q = fmaf(Q, sv, 1.f / 11.f);
          Q = fmaf(Q, sv, 1.f / 11.f);
          Q = fmaf(Q, sv, 1.f / 9.f);
          Q = fmaf(Q, sv, 1.f / 9.f);
          Q = fmaf(Q, sv, 1.f / 7.f);
          Q = fmaf(Q, sv, 1.f / 7.f);
          Q = fmaf(Q, sv, 1.f / 5.f);
          Q = fmaf(Q, sv, 1.f / 5.f);
          Q = fmaf(Q, sv, 1.f / 3.f);
          Q = fmaf(Q, sv, 1.f / 3.f);
          Q = fmaf(Q, sv, 1.f);
          fid = __fdividef(2.f * sv * sv * Q, 1.f - sv);
        } else {
          L = 2.f * logf(fabsf(xf));
          fid = fmaf(xsq, L, -tf);
        }
        const DF wd(w2.x, w2.y);
        acc_mac(a_id, wd, DF(fid, 0.f));
        acc_mac(a_ext, wd, DF(xsq * vef, 0.f));
        acc_mac(a_exc, wd, DF(vv * tf, 0.f));
        const float gf = 2.f * xf * w2.x * (A.ch * fmaf(A.kh, L, vef) + A.xh * vv);
        gi = f2d_bits(gf);
        if (dir) acc_mac(a_gd, DF(gf, 0.f), DF(dir[i], 0.f));
        if (hinv) hinv[i] = __fdividef(1.f, w2.x * c2k * fmaxf(L + 2.f + vef * ikT, 1.f));
      } else {
        const Terms64 tt = terms_f64(x, ws[o], (double)vv, ve, A);
        d_id += tt.id;
        d_ext += tt.ext;
        d_exc += tt.exc;
        gi = tt.g;
        if (hinv) hinv[i] = tt.hinv;
        if (dir) acc_mac(a_gd, df_from_double_bits(gi), DF(dir[i], 0.f));
      }
    } else if (ebits - 1003u <= 40u) {  // 2^-20 <= |x| < 2^21
      const LnSq q = df_ln_sq(x, A);
      const float2 w2 = wf[o];
      const DF wd(w2.x, w2.y), vd = eg_df(vv), ved = df_from_double_bits(ve);
      acc_mac(a_id, wd, q.L + q.t * (q.L - one));  // (1 + t) L - t
      acc_mac(a_ext, wd, (q.t + one) * ved);
      acc_mac(a_exc, wd, vd * q.t);
      const DF inner = cext * (kT * q.L + ved) + cexc2 * vd;
      const DF gdf = twice(df_from_double_bits(x) * wd) * inner;
      gi = df_to_double(gdf);
      if (dir) acc_mac(a_gd, gdf, DF(dir[i], 0.f));
      if (hinv) hinv[i] = __fdividef(1.f, wd.hi * c2k * fmaxf(q.L.hi + 2.f + ved.hi * ikT, 1.f));
    } else {
      const Terms64 tt = terms_f64(x, ws[o], (double)vv, ve, A);
      d_id += tt.id;
      d_ext += tt.ext;
      d_exc += tt.exc;
      gi = tt.g;
      if (hinv) hinv[i] = tt.hinv;
      if (dir) acc_mac(a_gd, df_from_double_bits(gi), DF(dir[i], 0.f));
    }
    gout[i] = gi;
    const unsigned long long gb = bits_of(gi) & 0x7fffffffffffffffull;
    gmax = gb > gmax ? gb : gmax;
    o += ostep;
    if (o >= A.no) o -= A.no;
  }
  Red<4> r;
  r.s[0] = dd_plus(Dd{c_id * df_to_double(acc_get(a_id)), 0.0}, c_id * d_id);
  r.s[1] = dd_plus(Dd{c_ext * df_to_double(acc_get(a_ext)), 0.0}, c_ext * d_ext);
  r.s[2] = dd_plus(Dd{c_exc * df_to_double(acc_get(a_exc)), 0.0}, c_exc * d_exc);
  r.s[3] = Dd{df_to_double(acc_get(a_gd)), 0.0};
  r.mx = double_of(gmax);
  double* out = A.out + (long long)blockIdx.y * A.out_stride;
  unsigned char* scr = static_cast<unsigned char*>(A.scratch) + (size_t)blockIdx.y * A.scratch_stride;
  const bool want_gd = dir != nullptr;
  grid_reduce<4>(r, reinterpret_cast<double*>(scr), reinterpret_cast<unsigned*>(scr + A.counter_off), [out, want_gd](const Red<4>& tt) {
    const double id = tt.s[0].hi + tt.s[0].lo, ext = tt.s[1].hi + tt.s[1].lo, exc = tt.s[2].hi + tt.s[2].lo;
    const Dd tot = dd_plus(dd_plus(tt.s[0], tt.s[1]), tt.s[2]);
    out[0] = tot.hi + tot.lo;
    out[1] = id;
    out[2] = ext;
    out[3] = exc;
    out[4] = tt.mx;
    if (want_gd) out[5] = tt.s[3].hi + tt.s[3].lo;
  });
}

// ---- batched L-BFGS step: one persistent kernel over every field's ops ------
// The search direction and the stored pairs (s, y) are FP32 vectors: the
// two-loop recursion only forms a preconditioned direction, whose rounding
// the line search absorbs, while the iterate and the gradient stay FP64.
// Every dot product is a double-float Dot2 sum on the FP32 pipe (products
// exact by FMA, compensated additions), so no pass leans on the narrow FP64
// pipe.  Each field's elements are cut into kLbChunks fixed chunks; a chunk
// is always handled by one CTA (the same in every round), its threads' sums
// combined in a fixed order, and a field's chunk sums added in chunk order:
// the result depends on neither the grid nor the other fields of the batch.
constexpr int kLbChunks = 1024;  // per field: enough items to keep every CTA of the grid busy
constexpr int kLbPerThread = kLbChunks / kRedThreads;  // chunks each thread adds in the final sum
static_assert(kLbChunks % kRedThreads == 0, "the final sum gives each thread whole chunks");
constexpr int kLbMaxSlots = 16;
constexpr int kLbMaxOps = 192;
constexpr long long kLbSpin = 1LL << 24;  // polls of the grid barrier (x 64 ns sleep): ~1 s

struct LbSlot {
  double *x, *xt, *g, *gt;
  float* d;
  double* S;
  long long n;
  int op0, nops;
};
struct LbBatch {
  int nslots, maxops;
  LbSlot slot[kLbMaxSlots];
  LbOp op[kLbMaxOps];
};

// elements per chunk: a multiple of 4, so that every chunk starts 16-byte
// aligned in FP32 and FP64 arrays whose base is
__host__ __device__ __forceinline__ long long lb_chunk_len(long long n) {
  return ((n + kLbChunks - 1) / kLbChunks + 3) & ~3LL;
}

__device__ __forceinline__ DF as_df(float a) { return DF(a, 0.f); }
__device__ __forceinline__ DF as_df(double a) { return df_from_double_bits(a); }
__device__ __forceinline__ float as_f(double a) { return df_from_double_bits(a).hi; }  // nearest float
__device__ __forceinline__ float ldu(const void* p, int is64, long long i) {
  return is64 ? as_f(static_cast<const double*>(p)[i]) : static_cast<const float*>(p)[i];
}
__device__ __forceinline__ DF ldv(const void* p, int is64, long long i) {
  return is64 ? as_df(static_cast<const double*>(p)[i]) : as_df(static_cast<const float*>(p)[i]);
}

// Grid barrier of a cooperative launch: bar[0] arrivals, bar[1] generation,
// bar[2] abort.  The last of `expected` arrivals resets the count and
// advances the generation; the others poll it with a bounded wait.  A wait
// that runs out (or finds abort raised) raises abort and returns false.
__device__ bool lb_grid_sync(unsigned* bar, unsigned expected) {
  __shared__ int okb;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vb = bar;
    int ok = vb[2] == 0u;
    if (ok) {
      const unsigned g0 = vb[1];
      __threadfence();
      if (atomicAdd(&bar[0], 1u) == expected - 1u) {
        vb[0] = 0u;
        __threadfence();
        atomicAdd(&bar[1], 1u);
      } else {
        for (long long i = 0; vb[1] == g0; ++i) {
          if (vb[2] != 0u || i > kLbSpin) {
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
    if (!ok) vb[2] = 1u;
    okb = ok;
  }
  __syncthreads();
  return okb != 0;
}

// block sum of K double-float values (warps by shuffles, warp 0 over the
// warps), valid in thread 0
template <int K>
__device__ __forceinline__ void lb_block_sum(DF (&v)[K]) {
  __shared__ float2 sh[K][kRedThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  df_warp_sum<K>(v);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][wid] = make_float2(v[k].hi, v[k].lo);
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const float2 q = lane < kRedThreads / 32 ? sh[k][lane] : make_float2(0.f, 0.f);
      v[k] = DF(q.x, q.y);
    }
    df_warp_sum<K>(v);
  }
}

__device__ __forceinline__ int lb_dots(const LbOp& op) {
  return op.type == kOpPair ? 2 : (op.type == kOpPass && op.out >= 0 ? 1 : 0);
}

// ---- vector access: 4 consecutive elements from 16-byte aligned storage ----
__device__ __forceinline__ void ld4(const float* p, long long i, float (&o)[4]) {
  const float4 v = *reinterpret_cast<const float4*>(p + i);
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
}
__device__ __forceinline__ void ld4(const double* p, long long i, double (&o)[4]) {
  const double2 a = *reinterpret_cast<const double2*>(p + i), b = *reinterpret_cast<const double2*>(p + i + 2);
  o[0] = a.x;
  o[1] = a.y;
  o[2] = b.x;
  o[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, long long i, const float (&o)[4]) {
  *reinterpret_cast<float4*>(p + i) = make_float4(o[0], o[1], o[2], o[3]);
}
__device__ __forceinline__ void st4(double* p, long long i, const double (&o)[4]) {
  *reinterpret_cast<double2*>(p + i) = make_double2(o[0], o[1]);
  *reinterpret_cast<double2*>(p + i + 2) = make_double2(o[2], o[3]);
}
// a float or double vector as floats (doubles rounded to nearest)
__device__ __forceinline__ void ldu4(const void* p, int is64, long long i, float (&o)[4]) {
  if (is64) {
    double t[4];
    ld4(static_cast<const double*>(p), i, t);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = as_f(t[q]);
  } else {
    ld4(static_cast<const float*>(p), i, o);
  }
}
// a float or double vector as double-float values (doubles split exactly)
__device__ __forceinline__ void ldv4(const void* p, int is64, long long i, DF (&o)[4]) {
  if (is64) {
    double t[4];
    ld4(static_cast<const double*>(p), i, t);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = as_df(t[q]);
  } else {
    float t[4];
    ld4(static_cast<const float*>(p), i, t);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = as_df(t[q]);
  }
}
__device__ __forceinline__ bool al16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// The element work of one op over elements [i0, i1) of one field, the CTA's
// threads striding by kRedThreads: with every array 16-byte aligned and i0 a
// multiple of 4, thread t takes the 4-element groups t, t + 256, ... (two
// groups' loads in flight per step), the elements past the last whole group
// one by one; otherwise every element one by one.  The op's fields are read
// into registers first (the kernel's parameter space would otherwise be
// re-read around every store).  Dots accumulate into a0 (and a1).
__device__ void lb_elements(const LbOp& opr, const LbSlot& slr, long long i0, long long i1, Acc<DF>& a0,
                            Acc<DF>& a1) {
  const int tid = threadIdx.x;
  const int type = opr.type;
  if (type == kOpPass) {
    const double* S = slr.S;
    double cc = opr.c0;
    if (opr.i1 >= 0) cc += opr.c1 * __ldcg(S + opr.i1);
    if (opr.i2 >= 0) cc += opr.c2 * __ldcg(S + opr.i2);
    const double a = opr.ja >= 0 ? __ldcg(S + opr.ja) : opr.a0;
    const float cf = (float)cc, af = (float)a, hf = opr.jh >= 0 ? (float)__ldcg(S + opr.jh) : 1.f;
    const bool rx = a != 0.0, dot = opr.out >= 0;
    float* __restrict__ x = opr.f0;
    const void* u = opr.u;
    const void* v = opr.v;
    const float* __restrict__ h = opr.h;
    const int u64 = opr.u64, v64 = opr.v64;
    long long i = i0 + tid;
    if (al16(x) && al16(u) && al16(v) && al16(h)) {
      const long long g1 = i1 >> 2;  // whole groups end
      long long g = (i0 >> 2) + tid;
      for (; g < g1; g += 2 * kRedThreads) {
        const bool two = g + kRedThreads < g1;
        float xo[2][4], uo[2][4], ho[2][4];
        DF vo[2][4];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if (k == 1 && !two) break;
          const long long e = (g + k * kRedThreads) << 2;
          if (rx) {
            ld4(x, e, xo[k]);
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) xo[k][q] = 0.f;
          }
          ldu4(u, u64, e, uo[k]);
          if (h) {
            ld4(h, e, ho[k]);
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) ho[k][q] = 1.f;
          }
          if (dot) ldv4(v, v64, e, vo[k]);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if (k == 1 && !two) break;
          float xv[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            xv[q] = (h ? hf * ho[k][q] : 1.f) * fmaf(cf, uo[k][q], af * xo[k][q]);
            if (dot) acc_mac(a0, vo[k][q], as_df(xv[q]));
          }
          st4(x, (g + k * kRedThreads) << 2, xv);
        }
      }
      i = max(i0, g1 << 2) + tid;  // the tail past the last whole group (none in an empty chunk)
    }
    for (; i < i1; i += kRedThreads) {
      const float xv = (h ? hf * h[i] : 1.f) * fmaf(cf, ldu(u, u64, i), rx ? af * x[i] : 0.f);
      x[i] = xv;
      if (dot) acc_mac(a0, ldv(v, v64, i), as_df(xv));
    }
  } else if (type == kOpPair) {
    const float tf = (float)opr.t;
    float* __restrict__ hs = opr.f0;
    float* __restrict__ hy = opr.f1;
    const float* __restrict__ h = opr.h;
    double* __restrict__ gg = slr.g;
    double* __restrict__ xx = slr.x;
    const double* __restrict__ gt = slr.gt;
    const double* __restrict__ xt = slr.xt;
    const float* __restrict__ d = slr.d;
    long long i = i0 + tid;
    if (al16(hs) && al16(hy) && al16(h) && al16(gg) && al16(xx) && al16(gt) && al16(xt) && al16(d)) {
      const long long g1 = i1 >> 2;
      long long g = (i0 >> 2) + tid;
      for (; g < g1; g += kRedThreads) {
        const long long e = g << 2;
        double gn[4], go[4], xn[4];
        float dv[4], hv[4];
        ld4(gt, e, gn);
        ld4(gg, e, go);
        ld4(d, e, dv);
        ld4(xt, e, xn);
        if (h) ld4(h, e, hv);
        float sv[4], yv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          sv[q] = tf * dv[q];
          yv[q] = (df_from_double_bits(gn[q]) - df_from_double_bits(go[q])).hi;
          acc_mac(a0, as_df(sv[q]), as_df(yv[q]));
          acc_mac(a1, as_df(h ? hv[q] * yv[q] : yv[q]), as_df(yv[q]));
        }
        st4(hs, e, sv);
        st4(hy, e, yv);
        st4(gg, e, gn);  // the accepted point
        st4(xx, e, xn);
      }
      i = max(i0, g1 << 2) + tid;
    }
    for (; i < i1; i += kRedThreads) {
      const double gn = gt[i], go = gg[i];
      const float sv = tf * d[i];
      const float yv = (df_from_double_bits(gn) - df_from_double_bits(go)).hi;
      hs[i] = sv;
      hy[i] = yv;
      acc_mac(a0, as_df(sv), as_df(yv));
      acc_mac(a1, as_df(h ? h[i] * yv : yv), as_df(yv));
      gg[i] = gn;
      xx[i] = xt[i];
    }
  } else if (type == kOpCopy) {
    double* __restrict__ gg = slr.g;
    double* __restrict__ xx = slr.x;
    const double* __restrict__ gt = slr.gt;
    const double* __restrict__ xt = slr.xt;
    long long i = i0 + tid;
    if (al16(gg) && al16(xx) && al16(gt) && al16(xt)) {
      const long long g1 = i1 >> 2;
      long long g = (i0 >> 2) + tid;
      for (; g < g1; g += kRedThreads) {
        const long long e = g << 2;
        double a[4], b[4];
        ld4(gt, e, a);
        ld4(xt, e, b);
        st4(gg, e, a);
        st4(xx, e, b);
      }
      i = max(i0, g1 << 2) + tid;
    }
    for (; i < i1; i += kRedThreads) {
      gg[i] = gt[i];
      xx[i] = xt[i];
    }
  } else {  // kOpStep: one FP64 FMA per element, d widened exactly from its bits
    const double t = opr.t;
    double* __restrict__ xt = slr.xt;
    const double* __restrict__ xx = slr.x;
    const float* __restrict__ d = slr.d;
    long long i = i0 + tid;
    if (al16(xt) && al16(xx) && al16(d)) {
      const long long g1 = i1 >> 2;
      long long g = (i0 >> 2) + tid;
      for (; g < g1; g += 2 * kRedThreads) {
        const bool two = g + kRedThreads < g1;
        double xo[2][4];
        float dv[2][4];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if (k == 1 && !two) break;
          ld4(xx, (g + k * kRedThreads) << 2, xo[k]);
          ld4(d, (g + k * kRedThreads) << 2, dv[k]);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if (k == 1 && !two) break;
          double o[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) o[q] = fma(t, f2d_bits(dv[k][q]), xo[k][q]);
          st4(xt, (g + k * kRedThreads) << 2, o);
        }
      }
      i = max(i0, g1 << 2) + tid;
    }
    for (; i < i1; i += kRedThreads) xt[i] = fma(t, f2d_bits(d[i]), xx[i]);
  }
}

// element work of item `it` (chunk c of field j) in round r; its chunk sums
// go to part[it]
__device__ __forceinline__ void lb_item(const LbBatch& B, int r, long long it, float2* __restrict__ part) {
  const int j = (int)(it / kLbChunks), c = (int)(it % kLbChunks);
  const LbSlot& sl = B.slot[j];
  if (r >= sl.nops) return;
  const LbOp& op = B.op[sl.op0 + r];
  const long long len = lb_chunk_len(sl.n);
  const long long i0 = min(sl.n, (long long)c * len), i1 = min(sl.n, i0 + len);
  Acc<DF> a0, a1;
  acc_zero(a0);
  acc_zero(a1);
  lb_elements(op, sl, i0, i1, a0, a1);
  if (lb_dots(op)) {
    DF v[2] = {acc_get(a0), acc_get(a1)};
    lb_block_sum<2>(v);
    if (threadIdx.x == 0) {
      part[it * 2] = make_float2(v[0].hi, v[0].lo);
      part[it * 2 + 1] = make_float2(v[1].hi, v[1].lo);
    }
  }
}

// field j's sums of round r from its chunk sums, in chunk order (thread t
// adds chunks kLbPerThread t .. kLbPerThread (t + 1) - 1, then the block sum),
// and the scalars they set
__device__ __forceinline__ void lb_field_sums(const LbBatch& B, int r, int j, const float2* __restrict__ part) {
  const int tid = threadIdx.x;
  const LbSlot& sl = B.slot[j];
  if (r >= sl.nops) return;
  const LbOp& op = B.op[sl.op0 + r];
  if (!lb_dots(op)) return;
  DF v[2] = {DF(0.f, 0.f), DF(0.f, 0.f)};
#pragma unroll
  for (int q = 0; q < kLbPerThread; ++q) {
    const long long c = (long long)j * kLbChunks + tid * kLbPerThread + q;
    const float2 q0 = __ldcg(&part[c * 2]), q1 = __ldcg(&part[c * 2 + 1]);
    v[0] = v[0] + DF(q0.x, q0.y);
    v[1] = v[1] + DF(q1.x, q1.y);
  }
  lb_block_sum<2>(v);
  if (tid == 0) {
    double* S = sl.S;
    const double t0 = df_to_double(v[0]), t1 = df_to_double(v[1]);
    if (op.type == kOpPass) {
      const double scale = (op.js1 >= 0 ? S[op.js1] : op.sc0) * (op.js2 >= 0 ? S[op.js2] : 1.0);
      S[op.out] = scale * t0;
    } else {
      S[op.out] = t0;
      S[op.out + 1] = t1;
      const bool good = t1 > 0.0 && t0 > 1e-12 * t1;
      S[op.i1] = good ? 1.0 / t0 : 0.0;
      if (good) S[op.i2] = t0 / t1;
    }
    __threadfence();
  }
}

__device__ __forceinline__ bool lb_round_dots(const LbBatch& B, int r) {
  for (int j = 0; j < B.nslots; ++j)
    if (r < B.slot[j].nops && lb_dots(B.op[B.slot[j].op0 + r])) return true;
  return false;
}

// Persistent form: every round of every field in one cooperative launch, the
// rounds and their sums separated by the bounded grid barrier.
__global__ void __launch_bounds__(kRedThreads) lbfgs_batch_kernel(const __grid_constant__ LbBatch B,
                                                                   float2* __restrict__ part, unsigned* bar,
                                                                   int* err, int* flag) {
  const long long items = (long long)B.nslots * kLbChunks;
  bool ok = true;
  for (int r = 0; r < B.maxops && ok; ++r) {
    for (long long it = blockIdx.x; it < items; it += gridDim.x) lb_item(B, r, it, part);
    if (!lb_grid_sync(bar, gridDim.x)) {
      ok = false;
      break;
    }
    if (!lb_round_dots(B, r)) continue;
    for (int j = blockIdx.x; j < B.nslots; j += gridDim.x) lb_field_sums(B, r, j, part);
    if (!lb_grid_sync(bar, gridDim.x)) {
      ok = false;
      break;
    }
  }
  if (!ok && blockIdx.x == 0 && threadIdx.x == 0) note_wait_timeout(err, flag);
}

// Round form: one ordinary launch per round, the op program in device memory.
// The last CTA to finish the round's element work (completion counter) adds
// every field's sums, exactly as the persistent form does, and clears the
// counter; the next round's launch then reads them.  No CTA waits for
// another, so the launch needs no co-residency and shares the GPU with other
// streams' kernels.
__global__ void __launch_bounds__(kRedThreads) lbfgs_round_kernel(const LbBatch* __restrict__ Bp, int r,
                                                                   float2* __restrict__ part,
                                                                   unsigned* __restrict__ counter) {
  const LbBatch& B = *Bp;
  const long long items = (long long)B.nslots * kLbChunks;
  for (long long it = blockIdx.x; it < items; it += gridDim.x) lb_item(B, r, it, part);
  if (!lb_round_dots(B, r)) return;
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int j = 0; j < B.nslots; ++j) lb_field_sums(B, r, j, part);
  if (threadIdx.x == 0) *counter = 0u;
}

__global__ void __launch_bounds__(kRedThreads) grid_barrier_selftest_kernel(unsigned* bar, unsigned missing,
                                                                            int* err, int* flag) {
  if (!lb_grid_sync(bar, gridDim.x + missing) && blockIdx.x == 0 && threadIdx.x == 0) note_wait_timeout(err, flag);
}

// a field's scalar block at the start of a run: zero, gamma = 1
__global__ void lb_init_kernel(double* S, int n, int ogam) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) S[i] = i == ogam ? 1.0 : 0.0;
}

__global__ void __launch_bounds__(256) to_float_kernel(float* __restrict__ y, const double* __restrict__ x,
                                                       long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

unsigned stream_blocks(long long n) {
  const long long b = (n + 255) / 256;
  return (unsigned)std::max(1LL, std::min<long long>(b, 152LL * 16));
}

// qfact of common/MDFT_Constants.hpp:46-47: q_i q_j / r in kJ/mol for charges
// in e and r in Angstrom
double qfact() {
  const double pi = 3.14159265358979323846;
  const double eps0 = 8.854187817e-12, qunit = 1.602176565e-19, navo = 6.02214129e23;
  return qunit * qunit * 1.0e-3 * navo / (4.0 * pi * eps0 * 1.0e-10);
}

// Rotation matrix of every orientation, common/MDFT_Grid.hpp:283-310 (theta
// the Gauss-Legendre nodes, phi = i 2 pi / nphi, psi = k 2 pi / (mrso npsi),
// orientation index (theta, phi, psi) with psi fastest).
std::vector<double> orientation_rotations(const Grid& g) {
  const double pi = 3.14159265358979323846;
  std::vector<double> rot((size_t)g.no * 9);
  const double dphi = 2.0 * pi / g.nphi, dpsi = 2.0 * pi / g.mrso / g.npsi;
  int io = 0;
  for (int it = 0; it < g.ntheta; ++it)
    for (int ip = 0; ip < g.nphi; ++ip)
      for (int is = 0; is < g.npsi; ++is, ++io) {
        const double ct = std::cos(g.theta[it]), st = std::sin(g.theta[it]);
        const double cp = std::cos(ip * dphi), sp = std::sin(ip * dphi);
        const double cs = std::cos(is * dpsi), ss = std::sin(is * dpsi);
        double* R = rot.data() + 9 * (size_t)io;
        R[0] = ct * cp * cs - sp * ss;
        R[1] = -ct * cp * ss - sp * cs;
        R[2] = st * cp;
        R[3] = ct * sp * cs + cp * ss;
        R[4] = -ct * sp * ss + cp * cs;
        R[5] = st * sp;
        R[6] = -st * cs;
        R[7] = st * ss;
        R[8] = ct;
      }
  return rot;
}

}  // namespace
}  // namespace mdft

// ---- host side ---------------------------------------------------------------
namespace mdft {

namespace {
void launch_ok(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(MDFT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace

size_t reduction_scratch_bytes() { return sizeof(double) * kRedBlocks * 9 + 256; }

void to_float(float* y, const double* x, long long n, cudaStream_t s) {
  to_float_kernel<<<stream_blocks(n), 256, 0, s>>>(y, x, n);
  launch_ok("xi conversion launch");
}

void vext_compute(const Grid& g, const double* sv_sites, int n_solvent, const double* su_sites, int n_solute,
                  double vmax, double* vext, cudaStream_t s) {
  throw_if(!vext || !sv_sites || (n_solute > 0 && !su_sites), "NULL argument");
  throw_if(n_solvent < 1 || n_solute < 0, "site counts must be >= 1 (solvent) and >= 0 (solute)");
  throw_if(!(vmax > 0), "vmax must be positive");
  const int nsv = n_solvent, nsu = n_solute;
  const long double qf = qfact();
  auto df2 = [](long double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (long double)h));
  };
  std::vector<int> origin, offset;  // solvent sites at the molecular origin, the others
  for (int a = 0; a < nsv; ++a) {
    const double* A = sv_sites + 6 * a;
    throw_if(A[1] < 0 || A[2] < 0, "sigma and epsilon must be >= 0");
    (A[3] == 0.0 && A[4] == 0.0 && A[5] == 0.0 ? origin : offset).push_back(a);
  }
  for (int t = 0; t < nsu; ++t)
    throw_if(su_sites[6 * t + 1] < 0 || su_sites[6 * t + 2] < 0, "sigma and epsilon must be >= 0");
  auto pairs = [&](const std::vector<int>& sites) {
    std::vector<float2> pc((size_t)3 * std::max<size_t>(sites.size(), 1) * std::max(nsu, 1));
    for (size_t j = 0; j < sites.size(); ++j)
      for (int t = 0; t < nsu; ++t) {
        const double* A = sv_sites + 6 * sites[j];
        const double* B = su_sites + 6 * t;
        const long double eps = std::sqrt((long double)A[2] * B[2]), sig = 0.5L * ((long double)A[1] + B[1]);
        float2* c = pc.data() + 3 * (j * nsu + t);
        c[0] = df2(4.0L * eps);
        c[1] = df2(sig * sig);
        c[2] = df2(qf * A[0] * B[0]);
      }
    return pc;
  };
  const std::vector<float2> pof = pairs(offset), p0 = pairs(origin);
  const std::vector<double> rot = orientation_rotations(g);
  std::vector<float2> off((size_t)3 * g.no * std::max<size_t>(offset.size(), 1));
  for (int o = 0; o < g.no; ++o)
    for (size_t j = 0; j < offset.size(); ++j) {
      const double* R = rot.data() + 9 * (size_t)o;
      const double* x = sv_sites + 6 * offset[j] + 3;
      for (int k = 0; k < 3; ++k)
        off[3 * (o * offset.size() + j) + k] =
            df2((long double)R[3 * k] * x[0] + (long double)R[3 * k + 1] * x[1] + (long double)R[3 * k + 2] * x[2]);
    }
  std::vector<float2> su((size_t)3 * std::max(nsu, 1));
  for (int t = 0; t < nsu; ++t)
    for (int k = 0; k < 3; ++k) su[3 * t + k] = df2(su_sites[6 * t + 3 + k]);
  const int nn[3] = {g.nx, g.ny, g.nz};
  const double ll[3] = {g.lx, g.ly, g.lz};
  std::vector<float2> coord[3];
  for (int k = 0; k < 3; ++k) {
    coord[k].resize(nn[k]);
    for (int i = 0; i < nn[k]; ++i) coord[k][i] = df2((long double)i * ll[k] / nn[k]);
  }
  DevBuf dcx, dcy, dcz, doff, dsu, dpof, dp0, dv0;
  dcx.upload(coord[0].data(), sizeof(float2) * coord[0].size());
  dcy.upload(coord[1].data(), sizeof(float2) * coord[1].size());
  dcz.upload(coord[2].data(), sizeof(float2) * coord[2].size());
  doff.upload(off.data(), sizeof(float2) * off.size());
  dsu.upload(su.data(), sizeof(float2) * su.size());
  dpof.upload(pof.data(), sizeof(float2) * pof.size());
  dp0.upload(p0.data(), sizeof(float2) * p0.size());
  dv0.alloc(sizeof(float2) * (size_t)g.N());
  VextPlan P{};
  P.nx = g.nx;
  P.ny = g.ny;
  P.nz = g.nz;
  P.no = g.no;
  P.nof = (int)offset.size();
  P.n0 = (int)origin.size();
  P.nsu = nsu;
  for (int k = 0; k < 3; ++k) {
    P.L[k] = df2(ll[k]);
    P.il[k] = (float)(1.0 / ll[k]);
  }
  P.vmax = vmax;
  P.cx = dcx.as<float2>();
  P.cy = dcy.as<float2>();
  P.cz = dcz.as<float2>();
  P.off = doff.as<float2>();
  P.su = dsu.as<float2>();
  P.pof = dpof.as<float2>();
  P.p0 = dp0.as<float2>();
  P.v0 = dv0.as<float2>();
  vext_origin_kernel<<<stream_blocks(g.N()), 256, 0, s>>>(P);
  launch_ok("vext kernel launch");
  const long long n = g.N() * (long long)g.no;
  vext_kernel<<<stream_blocks(n), 256, 0, s>>>(P, vext);
  launch_ok("vext kernel launch");
  // the tables are freed on return: finish first
  cuda_check(cudaStreamSynchronize(s), "vext kernel");
}

void energy_grad(const EgConst& c, const double* xi, const void* vexc, bool vexc_f32, const double* vext,
                 const double* w, double* grad, long long n, int no, double* out, void* scratch, float* hinv,
                 cudaStream_t s, int nf, long long out_stride, const float* dir) {
  throw_if(nf < 1 || nf > 65535, "internal: energy batch size", 4);
  EgArgs A{};
  A.hinv = hinv;
  A.dir = dir;
  A.xi = xi;
  A.vexc = vexc;
  A.vext = vext;
  A.w = w;
  A.g = grad;
  A.n = n;
  A.no = no;
  A.kT = c.kT;
  A.rho0 = c.rho0;
  A.dv = c.dv;
  A.prefactor = c.prefactor;
  auto split = [](long double v, float& hi, float& lo) {
    hi = (float)v;
    lo = (float)(v - (long double)hi);
  };
  split(c.kT, A.kh, A.kl);
  split((long double)c.rho0 * c.dv, A.ch, A.cl);
  split(2.0L * c.prefactor * c.rho0, A.xh, A.xl);
  split(0.693147180559945309417232121458176568L, A.ln2h, A.ln2l);
  for (int k = 0; k < 10; ++k) split(1.0L / (2 * k + 1), A.ah[k], A.al[k]);
  A.out = out;
  A.out_stride = out_stride;
  A.scratch = scratch;
  A.counter_off = sizeof(double) * kRedBlocks * 9;  // the (CTAs, 2 x 4 + 1) partials of grid_reduce<4>
  A.scratch_stride = reduction_scratch_bytes();
  const size_t smem = (sizeof(double) + sizeof(float2)) * (size_t)no;
  throw_if(smem > 48 * 1024, "too many orientations for the energy kernel", MDFT_ERR_UNSUPPORTED);
  // the grid of each field depends on n only: a field's sums are the same
  // alone and in a batch
  const dim3 grid(red_blocks(n, 152 * 4), nf);
  if (vexc_f32)
    eg_kernel<float><<<grid, kRedThreads, smem, s>>>(A);
  else
    eg_kernel<double><<<grid, kRedThreads, smem, s>>>(A);
  launch_ok("energy kernel launch");
}

// ---- L-BFGS state machine ------------------------------------------------------
void Lbfgs::bind(const Bufs& b, long long n, int m) {
  b_ = b;
  n_ = n;
  m_ = m;
}

void Lbfgs::pass(float* x, const void* u, int u64, const void* v, int v64, double a0, int ja, double c0, double c1,
                 int i1, double c2, int i2, double sc0, int js1, int js2, int out, const float* h, int jh) {
  LbOp o{};
  o.type = kOpPass;
  o.f0 = x;
  o.u = u;
  o.u64 = u64;
  o.v = v;
  o.v64 = v64;
  o.a0 = a0;
  o.ja = ja;
  o.c0 = c0;
  o.c1 = c1;
  o.i1 = i1;
  o.c2 = c2;
  o.i2 = i2;
  o.sc0 = sc0;
  o.js1 = js1;
  o.js2 = js2;
  o.out = out;
  o.h = h;
  o.jh = jh;
  ops_.push_back(o);
}

// d = -H g by the two-loop recursion over the nh_ stored pairs, with the
// initial inverse Hessian gamma P, P = 1/D the diagonal of the inverse local
// curvature (written by the last evaluation, at x) and gamma = (s . y) /
// (y . P y) of the newest pair (P alone before the first pair); S[gd] = g . d.  Every coefficient
// comes from the device scalars: alpha_i = rho_i (s_i . q), beta_i =
// rho_i (y_i . r).
void Lbfgs::direction() {
  float* d = b_.d;
  const double* g = b_.g;
  const float* h0 = b_.hinv;
  auto hs = [&](int i) { return b_.hs + (size_t)i * n_; };
  auto hy = [&](int i) { return b_.hy + (size_t)i * n_; };
  if (nh_ == 0) {  // d = h0 (-g); S[gd] = g . d
    pass(d, g, 1, g, 1, 0.0, -1, -1.0, 0.0, -1, 0.0, -1, 1.0, -1, -1, gd(), h0);
    return;
  }
  auto idx = [&](int j) { return ((head_ - 1 - j) % m_ + m_) % m_; };  // j = 0: newest
  // q = -g; alpha_newest = rho (s . q)
  pass(d, g, 1, hs(idx(0)), 0, 0.0, -1, -1.0, 0.0, -1, 0.0, -1, 0.0, rho(idx(0)), -1, alpha(idx(0)));
  for (int j = 0; j < nh_; ++j) {
    const int i = idx(j);
    if (j + 1 < nh_) {  // q -= alpha_i y_i; alpha_next = rho_next (s_next . q)
      const int nx = idx(j + 1);
      pass(d, hy(i), 0, hs(nx), 0, 1.0, -1, 0.0, -1.0, alpha(i), 0.0, -1, 0.0, rho(nx), -1, alpha(nx));
    } else {  // last: r = gamma h0 (q - alpha y); beta_oldest = rho_oldest (y_oldest . r)
      pass(d, hy(i), 0, hy(i), 0, 1.0, -1, 0.0, -1.0, alpha(i), 0.0, -1, 0.0, rho(i), -1, beta(0), h0, gamma());
    }
  }
  for (int j = 0; j < nh_; ++j) {  // oldest first: r += (alpha_i - beta_i) s_i
    const int i = idx(nh_ - 1 - j);
    if (j + 1 < nh_) {
      const int nx = idx(nh_ - 2 - j);
      pass(d, hs(i), 0, hy(nx), 0, 1.0, -1, 0.0, 1.0, alpha(i), -1.0, beta(j), 0.0, rho(nx), -1, beta(j + 1));
    } else {
      pass(d, hs(i), 0, g, 1, 1.0, -1, 0.0, 1.0, alpha(i), -1.0, beta(j), 1.0, -1, -1, gd());
    }
  }
}

void Lbfgs::step() {
  LbOp o{};
  o.type = kOpStep;
  o.t = t_;
  o.out = -1;
  ops_.push_back(o);
}

void Lbfgs::start(double gtol, double ftol, int max_iter, cudaStream_t s, double e_noise) {
  gtol_ = gtol;
  ftol_ = ftol;
  e_noise_ = e_noise;
  max_iter_ = max_iter;
  nh_ = head_ = ls_ = iter_ = 0;
  first_ = true;
  status_ = kRunning;
  trace_.clear();
  lb_init_kernel<<<1, 128, 0, s>>>(b_.S, nscalars(m_), gamma());
  launch_ok("L-BFGS init launch");
}

bool Lbfgs::on_eval(const double* tail) {
  const double c1 = 1e-4;
  const int max_ls = 40;
  const double gdv = tail[0];
  const double* Et = tail + 3;
  ops_.clear();
  if (!first_) {
    if (!(gdv < 0.0)) {  // not a descent direction (rounding): restart from -H0 g
      nh_ = 0;
      direction();
      t_ = 1.0;
      ls_ = 0;
      step();
      return false;
    }
    // Armijo; or, with noisy energies, approximate Wolfe: E within the noise
    // of the current value and the slope at the trial point risen to at most
    // (1 - 2 delta) |g.d| (for a quadratic along d this is Armijo with
    // c1 = delta, told by the slope, which the noise of E does not reach)
    const double delta = 0.1, slope_t = tail[8];
    const bool armijo = std::isfinite(Et[0]) && Et[0] <= E_[0] + c1 * t_ * gdv;
    const bool approx = e_noise_ > 0.0 && std::isfinite(Et[0]) && std::isfinite(slope_t) &&
                        Et[0] <= E_[0] + e_noise_ * std::fabs(E_[0]) && slope_t <= (1.0 - 2.0 * delta) * -gdv;
    if (!(armijo || approx)) {
      t_ *= 0.5;
      if (++ls_ > max_ls) {  // no decrease along the direction: end at x
        status_ = kStalled;
        return true;
      }
      step();
      return false;
    }
  }
  const double Eprev = E_[0];
  std::copy(Et, Et + 5, E_);
  trace_.insert(trace_.end(), Et, Et + 5);
  if (!first_) {
    // accepted: curvature pair into the ring slot head_, the point kept
    LbOp o{};
    o.type = kOpPair;
    o.f0 = b_.hs + (size_t)head_ * n_;
    o.f1 = b_.hy + (size_t)head_ * n_;
    o.h = b_.hinv;
    o.t = t_;
    o.out = gd() + 1;
    o.i1 = rho(head_);
    o.i2 = gamma();
    ops_.push_back(o);
    head_ = (head_ + 1) % m_;
    nh_ = std::min(nh_ + 1, m_);
    ++iter_;
  } else {
    LbOp o{};
    o.type = kOpCopy;
    o.out = -1;
    ops_.push_back(o);
  }
  bool done = false;
  if (E_[4] <= gtol_) {
    status_ = kConverged;
    done = true;
  } else if (!first_ && std::fabs(Eprev - E_[0]) <= ftol_ * std::max(1.0, std::fabs(E_[0]))) {
    status_ = kFlat;
    done = true;
  } else if (iter_ >= max_iter_) {
    status_ = kMaxIter;
    done = true;
  }
  if (done) return true;  // the accepted point still has to be kept: the caller runs ops()
  direction();
  t_ = 1.0;  // the diagonal preconditioner scales even the first step
  first_ = false;
  ls_ = 0;
  step();
  return false;
}

void LbRunner::init() {
  const size_t part = sizeof(float2) * 2 * (size_t)kLbMaxSlots * kLbChunks;
  buf.alloc(part + 64);
  cuda_check(cudaMemset(buf.ptr, 0, part + 64), "L-BFGS batch state reset");
  int dev = 0, nsm = 0, per = 0, coop = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (rounds) {
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lbfgs_round_kernel, kRedThreads, 0),
               "L-BFGS round occupancy");
    throw_if(per < 1, "internal: the L-BFGS round kernel does not fit an SM", 4);
    prog.alloc(sizeof(LbBatch));
    blocks = nsm * per;  // one wave
    return;
  }
  cuda_check(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev), "cooperative launch attribute");
  throw_if(!coop, "the device does not support cooperative launches", 4);
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lbfgs_batch_kernel, kRedThreads, 0),
             "L-BFGS batch occupancy");
  throw_if(per < 1, "internal: the L-BFGS batch kernel does not fit an SM", 4);
  // two CTAs per SM at most: enough loads in flight with the vector loads
  blocks = nsm * std::min(per, 2);
}

namespace {
void lb_launch(LbBatch& B, int nop, LbRunner& r, cudaStream_t s) {
  const size_t part = sizeof(float2) * 2 * (size_t)kLbMaxSlots * kLbChunks;
  unsigned* bar = reinterpret_cast<unsigned*>(static_cast<unsigned char*>(r.buf.ptr) + part);
  if (r.rounds) {
    // the program's used part; from pageable memory, so B may change as soon
    // as the call returns
    const size_t bytes = offsetof(LbBatch, op) + sizeof(LbOp) * (size_t)nop;
    cuda_check(cudaMemcpyAsync(r.prog.ptr, &B, bytes, cudaMemcpyHostToDevice, s), "L-BFGS program upload");
    const long long items = (long long)B.nslots * kLbChunks;
    const unsigned grid = (unsigned)std::min<long long>(items, r.blocks);
    float2* pp = static_cast<float2*>(r.buf.ptr);
    clear_stale_error();
    for (int k = 0; k < B.maxops; ++k)
      lbfgs_round_kernel<<<grid, kRedThreads, 0, s>>>(static_cast<const LbBatch*>(r.prog.ptr), k, pp, bar);
    launch_ok("L-BFGS round launch");
    return;
  }
  cuda_check(cudaMemsetAsync(bar, 0, 16, s), "grid barrier reset");
  const WaitStatus& w = device_wait_status();
  float2* pp = static_cast<float2*>(r.buf.ptr);
  int* err = w.count;
  int* flag = w.flag_dev;
  void* args[] = {const_cast<LbBatch*>(&B), &pp, &bar, &err, &flag};
  clear_stale_error();
  cuda_check(cudaLaunchCooperativeKernel((const void*)lbfgs_batch_kernel, dim3(r.blocks), dim3(kRedThreads), args,
                                         0, s),
             "L-BFGS batch launch");
}
}  // namespace

void lbfgs_run(Lbfgs* const* lbs, int k, LbRunner& r, cudaStream_t s) {
  if (!r.buf.ptr) r.init();
  LbBatch B;
  B.nslots = 0;
  B.maxops = 0;
  int nop = 0;
  auto flush = [&] {
    if (B.nslots) lb_launch(B, nop, r, s);
    B.nslots = 0;
    B.maxops = 0;
    nop = 0;
  };
  for (int i = 0; i < k; ++i) {
    std::vector<LbOp>& ops = lbs[i]->ops();
    if (ops.empty()) continue;
    throw_if((int)ops.size() > kLbMaxOps, "internal: L-BFGS program too long", 4);
    if (B.nslots == kLbMaxSlots || nop + (int)ops.size() > kLbMaxOps) flush();
    const Lbfgs::Bufs& b = lbs[i]->bufs();
    LbSlot& sl = B.slot[B.nslots++];
    sl.x = b.x;
    sl.xt = b.xt;
    sl.g = b.g;
    sl.gt = b.gt;
    sl.d = b.d;
    sl.S = b.S;
    sl.n = lbs[i]->size();
    sl.op0 = nop;
    sl.nops = (int)ops.size();
    for (const LbOp& o : ops) B.op[nop++] = o;
    B.maxops = std::max(B.maxops, sl.nops);
    ops.clear();
  }
  flush();
}

void grid_barrier_selftest(int missing, LbRunner& r, cudaStream_t s) {
  throw_if(missing < 0 || missing > 1024, "missing arrivals must be in [0, 1024]");
  if (!r.buf.ptr) r.init();
  const size_t part = sizeof(float2) * 2 * (size_t)kLbMaxSlots * kLbChunks;
  unsigned* bar = reinterpret_cast<unsigned*>(static_cast<unsigned char*>(r.buf.ptr) + part);
  cuda_check(cudaMemsetAsync(bar, 0, 16, s), "grid barrier reset");
  const WaitStatus& w = device_wait_status();
  unsigned miss = (unsigned)missing;
  int* err = w.count;
  int* flag = w.flag_dev;
  void* args[] = {&bar, &miss, &err, &flag};
  clear_stale_error();
  cuda_check(cudaLaunchCooperativeKernel((const void*)grid_barrier_selftest_kernel, dim3(r.blocks),
                                         dim3(kRedThreads), args, 0, s),
             "grid barrier self-test launch");
}

}  // namespace mdft

// ---- solver handle -----------------------------------------------------------
struct mdft_solver_s {
  mdft_opt_s* opt = nullptr;
  mdft_conv_s* conv = nullptr;
  int prec = 0, device = 0, m = 5;
  long long N = 0, n = 0;
  int no = 0, np = 0;
  mdft::EgConst c{};
  bool has_vext = false;
  DevBuf vext, w, p, vexc, xf, x, xt, g, gt, d, hs, hy, hinv, S, scratch;
  mdft::Lbfgs lb;
  mdft::LbRunner lbr;
};

namespace {

using mdft::cuda_check;

template <typename F>
int solver_guard(F&& f) {
  try {
    f();
    return MDFT_OK;
  } catch (const Error& e) {
    return mdft::record_error(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return mdft::record_error(MDFT_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return mdft::record_error(MDFT_ERR_INVALID, e.what());
  }
}

// E(x) and its gradient into g; the 5 terms to out (device), and with_slope
// g . d (the minimiser's direction) to out[5]
void evaluate(mdft_solver_s* h, const double* x, double* g, double* out, cudaStream_t s, bool with_slope = false) {
  const void* xin = x;
  if (h->prec == MDFT_F32) {
    mdft::to_float(h->xf.as<float>(), x, h->n, s);
    xin = h->xf.ptr;
  }
  mdft::detail::angl2proj_fields(h->opt, xin, true, h->c.rho0, h->p.ptr, 1, s);
  mdft::detail::execute_fields(h->conv, h->p.ptr, 1, s);
  mdft::detail::proj2angl_fields(h->opt, h->p.ptr, h->vexc.ptr, 1, s);
  mdft::energy_grad(h->c, x, h->vexc.ptr, h->prec == MDFT_F32, h->has_vext ? h->vext.as<double>() : nullptr,
                    h->w.as<double>(), g, h->n, h->no, out, h->scratch.ptr, h->hinv.as<float>(), s, 1, 0,
                    with_slope ? h->d.as<float>() : nullptr);
}

}  // namespace

extern "C" {

int mdft_vext_lj_coulomb(mdft_grid_t grid, const double* solvent_sites, int n_solvent_sites,
                         const double* solute_sites, int n_solute_sites, double vmax, double* vext, void* stream) {
  return solver_guard([&] {
    throw_if(!grid, "NULL argument");
    mdft::vext_compute(grid->g, solvent_sites, n_solvent_sites, solute_sites, n_solute_sites, vmax, vext,
                       static_cast<cudaStream_t>(stream));
  });
}

int mdft_solver_create(mdft_solver_t* out, mdft_opt_t opt, mdft_conv_t conv, const double* vext, double kT,
                       double rho0, double prefactor, int history) {
  return solver_guard([&] {
    throw_if(!out || !opt || !conv, "NULL argument");
    *out = nullptr;
    throw_if(opt->prec != conv->prec, "the OPT and Convolution handles must have the same precision");
    throw_if(opt->batch != 1 || conv->batch != 1, "the solver takes single-field (batch 1) plans");
    const mdft::Grid &go = opt->g, &gc = conv->g;
    throw_if(go.nx != gc.nx || go.ny != gc.ny || go.nz != gc.nz || go.mmax != gc.mmax || go.mrso != gc.mrso,
             "the OPT and Convolution handles must share one grid");
    throw_if(history < 1 || history > mdft::kMaxHistory, "history must be 1..32");
    throw_if(!(kT > 0) || !(rho0 > 0), "kT and rho0 must be positive");
    throw_if(mdft::detail::current_device() != opt->device || opt->device != conv->device,
             "the handles belong to another device");
    auto h = std::make_unique<mdft_solver_s>();
    h->opt = opt;
    h->conv = conv;
    h->prec = opt->prec;
    h->device = opt->device;
    h->m = history;
    h->N = go.N();
    h->no = go.no;
    h->np = go.np;
    h->n = h->N * h->no;
    h->c = mdft::EgConst{kT, rho0, (go.lx / go.nx) * (go.ly / go.ny) * (go.lz / go.nz), prefactor};
    const size_t fb = sizeof(double) * (size_t)h->n;
    const size_t eb = h->prec == MDFT_F32 ? 4 : 8;
    h->w.upload(go.w.data(), sizeof(double) * go.no);
    h->p.alloc(2 * eb * (size_t)h->np * h->N);
    h->vexc.alloc(eb * (size_t)h->n);
    if (h->prec == MDFT_F32) h->xf.alloc(sizeof(float) * (size_t)h->n);
    h->x.alloc(fb);
    h->xt.alloc(fb);
    h->g.alloc(fb);
    h->gt.alloc(fb);
    h->d.alloc(fb / 2);  // FP32 direction, curvature pairs and diagonal preconditioner
    h->hinv.alloc(fb / 2);
    h->hs.alloc(fb / 2 * h->m);
    h->hy.alloc(fb / 2 * h->m);
    h->S.alloc(sizeof(double) * mdft::Lbfgs::nscalars(h->m));
    h->scratch.alloc(mdft::reduction_scratch_bytes());
    cuda_check(cudaMemset(h->scratch.ptr, 0, mdft::reduction_scratch_bytes()), "scratch reset");
    cuda_check(cudaMemset(h->S.ptr, 0, sizeof(double) * mdft::Lbfgs::nscalars(h->m)), "scalar reset");
    if (vext) {
      h->vext.alloc(fb);
      cuda_check(cudaMemcpy(h->vext.ptr, vext, fb, cudaMemcpyDeviceToDevice), "vext copy");
      h->has_vext = true;
    }
    h->lb.bind(mdft::Lbfgs::Bufs{h->x.as<double>(), h->xt.as<double>(), h->g.as<double>(), h->gt.as<double>(),
                                 h->d.as<float>(), h->hs.as<float>(), h->hy.as<float>(), h->hinv.as<float>(),
                                 h->S.as<double>(), h->scratch.ptr},
               h->n, h->m);
    *out = h.release();
  });
}

int mdft_solver_energy(mdft_solver_t h, const double* xi, double* grad, double* terms, void* stream) {
  return solver_guard([&] {
    throw_if(!h || !xi || !terms, "NULL argument");
    throw_if(mdft::detail::current_device() != h->device, "the solver belongs to another device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* out = h->S.as<double>() + mdft::Lbfgs::energy_at(h->m);
    evaluate(h, xi, grad ? grad : h->gt.as<double>(), out, s);
    cuda_check(cudaMemcpyAsync(terms, out, 5 * sizeof(double), cudaMemcpyDeviceToHost, s), "energy read-back");
    cuda_check(cudaStreamSynchronize(s), "solver stream");
  });
}

int mdft_solver_minimize(mdft_solver_t h, double* xi, int max_iter, double gtol, double ftol, double* trace,
                         int* iterations, void* stream) {
  return solver_guard([&] {
    throw_if(!h || !xi, "NULL argument");
    throw_if(max_iter < 0, "max_iter must be >= 0");
    throw_if(mdft::detail::current_device() != h->device, "the solver belongs to another device");
    mdft::check_device_waits();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t fb = sizeof(double) * (size_t)h->n;
    cuda_check(cudaMemcpyAsync(h->xt.ptr, xi, fb, cudaMemcpyDeviceToDevice, s), "start copy");
    // the FP32 form's energies carry ~1e-7 relative noise (its transforms
    // run in FP32): the line search then also accepts by the slope
    const double e_noise = h->prec == MDFT_F32 ? 1e-6 : 0.0;
    h->lb.start(gtol, ftol, max_iter, s, e_noise);
    const int m = h->m;
    double* Sd = h->S.as<double>();
    double tail[mdft::Lbfgs::kTail];
    for (;;) {
      evaluate(h, h->xt.as<double>(), h->gt.as<double>(), Sd + mdft::Lbfgs::energy_at(m), s, e_noise > 0.0);
      cuda_check(cudaMemcpyAsync(tail, Sd + mdft::Lbfgs::tail_at(m), sizeof tail, cudaMemcpyDeviceToHost, s),
                 "tail read-back");
      cuda_check(cudaStreamSynchronize(s), "solver stream");
      const bool done = h->lb.on_eval(tail);
      mdft::Lbfgs* one = &h->lb;
      mdft::lbfgs_run(&one, 1, h->lbr, s);
      if (done) break;
    }
    cuda_check(cudaMemcpyAsync(xi, h->x.ptr, fb, cudaMemcpyDeviceToDevice, s), "final iterate copy");
    cuda_check(cudaStreamSynchronize(s), "solver stream");
    const std::vector<double>& tr = h->lb.trace();
    if (trace) std::memcpy(trace, tr.data(), sizeof(double) * std::min(tr.size(), (size_t)5 * (max_iter + 1)));
    if (iterations) *iterations = h->lb.iterations();
  });
}

int mdft_solver_status(mdft_solver_t h, int* status) {
  return solver_guard([&] {
    throw_if(!h || !status, "NULL argument");
    *status = (int)h->lb.status();
  });
}

int mdft_solver_destroy(mdft_solver_t h) {
  delete h;
  return MDFT_OK;
}

int mdft_grid_barrier_selftest(int missing, void* stream) {
  return solver_guard([&] {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<mdft::LbRunner>> runners;
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(mu);
    auto& r = runners[dev];
    if (!r) r = std::make_unique<mdft::LbRunner>();
    mdft::grid_barrier_selftest(missing, *r, static_cast<cudaStream_t>(stream));
  });
}

}  // extern "C"

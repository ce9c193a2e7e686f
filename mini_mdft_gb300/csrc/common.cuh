// common.cuh -- complex type, launch checks and the device-side plan
// structures shared by the hot-path kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "host_setup.hpp"

namespace mdft {

// Interleaved complex (re, im): the layout of Kokkos::complex<T>.
template <typename T>
struct __align__(2 * sizeof(T)) Cx {
  T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ Cx<T> mkc(T r, T i) {
  Cx<T> z;
  z.re = r;
  z.im = i;
  return z;
}
template <typename T>
__host__ __device__ __forceinline__ Cx<T> operator+(Cx<T> a, Cx<T> b) {
  return mkc<T>(a.re + b.re, a.im + b.im);
}
template <typename T>
__host__ __device__ __forceinline__ Cx<T> operator-(Cx<T> a, Cx<T> b) {
  return mkc<T>(a.re - b.re, a.im - b.im);
}
template <typename T>
__host__ __device__ __forceinline__ Cx<T> operator*(Cx<T> a, Cx<T> b) {
  return mkc<T>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T>
__host__ __device__ __forceinline__ Cx<T> operator*(Cx<T> a, T s) {
  return mkc<T>(a.re * s, a.im * s);
}
template <typename T>
__host__ __device__ __forceinline__ Cx<T> conj(Cx<T> a) {
  return mkc<T>(a.re, -a.im);
}
// a + b * c (complex multiply-accumulate)
template <typename T>
__host__ __device__ __forceinline__ Cx<T> cmac(Cx<T> a, Cx<T> b, Cx<T> c) {
  return mkc<T>(a.re + b.re * c.re - b.im * c.im, a.im + b.re * c.im + b.im * c.re);
}

// ---------------------------------------------------------------------------
// Double-float: a value hi + lo held as two floats with |lo| <= ulp(hi)/2,
// about 48 significand bits.  Sums use Knuth's TwoSum and products Dekker's
// TwoProd through FMA, then a fast renormalisation (Dekker 1971; the
// "sloppy" pair addition of Joldes, Muller and Popescu 2017, whose error is
// bounded relative to |a| + |b|, the norm-wise bound FFT and matrix-vector
// error analyses need).  It lets the FP64 form run on the FP32 pipes, which
// are 64x wider than the FP64 pipe of this GPU.
// ---------------------------------------------------------------------------
struct DF {
  float hi, lo;
  DF() = default;
  __host__ __device__ constexpr DF(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr DF(int v) : hi((float)v), lo(0.f) {}
  __host__ __device__ explicit DF(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ explicit DF(long double x)
      : hi((float)x), lo((float)(x - (long double)(float)x)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__host__ __device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return DF(s, e);
}
__host__ __device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
  const float s = a + b;
  return DF(s, b - (s - a));
}
__host__ __device__ __forceinline__ DF operator+(DF a, DF b) {
  const DF s = df_two_sum(a.hi, b.hi);
  const float t = a.lo + b.lo;
  return df_fast_two_sum(s.hi, s.lo + t);
}
__host__ __device__ __forceinline__ DF operator-(DF a) { return DF(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__host__ __device__ __forceinline__ DF operator*(DF a, DF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ DF& operator+=(DF& a, DF b) { return a = a + b; }
// |x| < e for e a power of two representable in float (exact on normalised pairs)
__host__ __device__ __forceinline__ bool df_abs_lt(DF x, float e) {
  const float h = fabsf(x.hi);
  return h < e || (h == e && (x.hi > 0.f ? x.lo < 0.f : x.lo > 0.f));
}

// double <-> double-float conversions built from the IEEE bit fields with
// integer and FP32 instructions: the hardware double<->float conversions run
// on this GPU's narrow FP64 pipe, and even an untaken fallback branch costs
// FP64 issue slots once the compiler predicates it.  Host and device run the
// same code.
__host__ __device__ __forceinline__ unsigned long long bits_of(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
__host__ __device__ __forceinline__ double double_of(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}
__host__ __device__ __forceinline__ unsigned bits_of(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
__host__ __device__ __forceinline__ float float_of(unsigned b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}
// leading zeros of a non-zero word
__host__ __device__ __forceinline__ int clz32(unsigned x) {
#ifdef __CUDA_ARCH__
  return __clz(x);
#else
  return __builtin_clz(x);
#endif
}
__host__ __device__ __forceinline__ int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// x -> (hi, lo): hi is x rounded to 24 significant bits (to nearest, ties
// up), lo the signed remainder rounded to 24 bits by the integer-to-float
// conversion, so |x - (hi + lo)| <= 2^-48 |x| without bias for
// 2^-73 <= |x| < 2^127 (2^127 <= |x| < 2^128: hi truncated, lo the next 24
// bits truncated, 2^-47).  Smaller |x| keep hi only (x truncated to float,
// subnormal or zero), larger ones become +-inf; NaN stays NaN.
__host__ __device__ __forceinline__ DF df_from_double_bits(double x) {
  const unsigned long long b = bits_of(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const unsigned e = (hi32 >> 20) & 0x7ffu;  // biased exponent
  const unsigned sign = hi32 & 0x80000000u;
  const unsigned m23 = ((hi32 & 0x000fffffu) << 3) | (lo32 >> 29);  // top 23 fraction bits
  if (e >= 950u && e <= 1149u) {
    // the low 29 fraction bits decide the rounding of hi; a carry out of the
    // fraction moves into the exponent field by itself
    const unsigned low = lo32 & 0x1fffffffu;
    const unsigned up = low >= 0x10000000u ? 1u : 0u;
    const float h = float_of(sign | (((e - 896u) << 23) + m23 + up));
    const int r = (int)low - (int)(up << 29);        // |r| <= 2^28, units 2^(e - 1075)
    const float scale = float_of((e - 948u) << 23);  // 2^(e - 1075), a normal float
    const float l = (float)r * scale;
    return DF(h, sign ? -l : l);
  }
  if (e == 1150u) {
    const float h = float_of(sign | ((e - 896u) << 23) | m23);
    const unsigned r = lo32 & 0x1fffffffu;  // remaining 29 fraction bits
    float l = 0.f;
    if (r) {
      const int top = 31 - clz32(r);  // leading bit, 0..28
      const unsigned mr = top >= 23 ? (r >> (top - 23)) : (r << (23 - top));
      const unsigned lexp = e - 948u + (unsigned)top;  // biased exponent of lo, 2..230
      l = float_of(sign | (lexp << 23) | (mr & 0x7fffffu));
    }
    return df_fast_two_sum(h, l);
  }
  if (e > 1150u) {  // |x| >= 2^128, inf, NaN
    const bool nan = e == 0x7ffu && (b & 0x000fffffffffffffull) != 0;
    return DF(float_of(sign | (nan ? 0x7fc00000u : 0x7f800000u)), 0.f);
  }
  if (e >= 897u) return DF(float_of(sign | ((e - 896u) << 23) | m23), 0.f);  // normal float
  if (e < 874u) return DF(float_of(sign), 0.f);  // below the smallest subnormal float
  // subnormal float: m 2^-149 with m = significand >> (926 - e), 1 <= m < 2^23
  const unsigned long long full = (b & 0x000fffffffffffffull) | (1ull << 52);
  return DF(float_of(sign | (unsigned)(full >> (926u - e))), 0.f);
}

// float -> double, exact for every float (zero, subnormal, inf, NaN too)
__host__ __device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = bits_of(f);
  const unsigned ex = (u >> 23) & 0xffu;
  const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long fr = u & 0x7fffffu;
  if (ex == 0xffu) return double_of(s | 0x7ff0000000000000ull | (fr << 29));
  if (ex == 0u) {
    if (fr == 0) return double_of(s);
    const int top = 31 - clz32((unsigned)fr);  // value = 1.x 2^(top - 149)
    return double_of(s | ((unsigned long long)(top + 874) << 52) |
                     ((fr << (52 - top)) & 0x000fffffffffffffull));
  }
  return double_of(s | ((unsigned long long)(ex + 896u) << 52) | (fr << 29));
}

// (hi, lo) -> double: both halves widened exactly from their bits, then one
// FP64 add, which rounds hi + lo correctly.  One FP64 instruction per value
// (the narrow pipe is otherwise idle in the double-float kernels) costs far
// less issue time than aligning and rounding the pair in 64-bit integers.
__host__ __device__ __forceinline__ double df_to_double(DF a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

// Sums of products.  For float and double a plain multiply-add chain (the
// order of the scalar code it replaces).  For double-float a compensated dot
// product (Ogita, Rump and Oishi 2005, "Dot2", with double-float operands):
// each product hi*hi is split exactly by FMA, the cross terms hi*lo and
// lo*hi join its error term, the running sum of the high parts is carried
// through TwoSum and every error lands in one float, normalised once at
// the end.  12 FP32 instructions per real product instead of the 18 of a
// double-float multiply followed by a double-float add, with an error of
// order n 2^-48 of the sum of |terms|, as for the chained operations.
template <typename C>
struct Acc {
  C s;
};
template <>
struct Acc<DF> {
  float hi, lo;
};
template <typename C>
__host__ __device__ __forceinline__ void acc_zero(Acc<C>& a) {
  a.s = C(0);
}
__host__ __device__ __forceinline__ void acc_zero(Acc<DF>& a) {
  a.hi = 0.f;
  a.lo = 0.f;
}
template <typename C>
__host__ __device__ __forceinline__ void acc_set(Acc<C>& a, C v) {
  a.s = v;
}
__host__ __device__ __forceinline__ void acc_set(Acc<DF>& a, DF v) {
  a.hi = v.hi;
  a.lo = v.lo;
}
// 2 x, exact
template <typename C>
__host__ __device__ __forceinline__ C twice(C x) {
  return x + x;
}
template <>
__host__ __device__ __forceinline__ DF twice<DF>(DF x) {
  return DF(2.f * x.hi, 2.f * x.lo);
}
template <typename C>
__host__ __device__ __forceinline__ void acc_mac(Acc<C>& a, C x, C y) {
  a.s = a.s + x * y;
}
__host__ __device__ __forceinline__ void acc_mac(Acc<DF>& a, DF x, DF y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  const float t = a.hi + p;
  const float bb = t - a.hi;
  const float err = (a.hi - (t - bb)) + (p - bb);
  a.hi = t;
  a.lo = a.lo + (err + e);
}
template <typename C>
__host__ __device__ __forceinline__ C acc_get(const Acc<C>& a) {
  return a.s;
}
__host__ __device__ __forceinline__ DF acc_get(const Acc<DF>& a) { return df_two_sum(a.hi, a.lo); }

// complex sums of products: s += x y and s += x conj(y)
template <typename C>
struct CAcc {
  Acc<C> re, im;
};
template <typename C>
__host__ __device__ __forceinline__ void cacc_zero(CAcc<C>& s) {
  acc_zero(s.re);
  acc_zero(s.im);
}
template <typename C>
__host__ __device__ __forceinline__ void cacc_mac(CAcc<C>& s, Cx<C> x, Cx<C> y) {
  acc_mac(s.re, x.re, y.re);
  acc_mac(s.re, -x.im, y.im);
  acc_mac(s.im, x.re, y.im);
  acc_mac(s.im, x.im, y.re);
}
template <typename C>
__host__ __device__ __forceinline__ void cacc_macc(CAcc<C>& s, Cx<C> x, Cx<C> y) {
  acc_mac(s.re, x.re, y.re);
  acc_mac(s.re, x.im, y.im);
  acc_mac(s.im, -x.re, y.im);
  acc_mac(s.im, x.im, y.re);
}
// s += x y for a real y: half the products of a complex y
template <typename C>
__host__ __device__ __forceinline__ void cacc_mac_r(CAcc<C>& s, Cx<C> x, C y) {
  acc_mac(s.re, x.re, y);
  acc_mac(s.im, x.im, y);
}
template <typename C>
__host__ __device__ __forceinline__ Cx<C> cacc_get(const CAcc<C>& s) {
  return mkc<C>(acc_get(s.re), acc_get(s.im));
}
// x y as one two-term sum per component
template <typename C>
__host__ __device__ __forceinline__ Cx<C> cx_mul(Cx<C> x, Cx<C> y) {
  CAcc<C> s;
  cacc_zero(s);
  cacc_mac(s, x, y);
  return cacc_get(s);
}

// xi^2 - 1 of get_delta_rho in the storage type by one fused multiply-add:
// for xi near 1 the difference cancels, so it is formed before any
// conversion to the arithmetic type (double-float keeps 48 bits of the
// small result instead of 48 bits of xi^2).
__host__ __device__ __forceinline__ double xi_sq_minus_one(double x) { return fma(x, x, -1.0); }
__host__ __device__ __forceinline__ float xi_sq_minus_one(float x) { return fmaf(x, x, -1.0f); }

// Storage <-> compute conversions (identity unless the compute type is DF).
template <typename C, typename S>
__host__ __device__ __forceinline__ C to_compute(S x) {
  return (C)x;
}
template <>
__host__ __device__ __forceinline__ DF to_compute<DF, double>(double x) {
#ifdef __CUDA_ARCH__
  return df_from_double_bits(x);
#else
  return DF(x);
#endif
}
template <typename S, typename C>
__host__ __device__ __forceinline__ S to_storage(C x) {
  return (S)x;
}
template <>
__host__ __device__ __forceinline__ double to_storage<double, DF>(DF x) {
#ifdef __CUDA_ARCH__
  return df_to_double(x);
#else
  return (double)x;
#endif
}

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();  // a non-sticky error must not resurface at a later check
    throw Error(2, std::string(what) + ": " + cudaGetErrorString(e));
  }
}
inline void launch_check(const char* what) { cuda_check(cudaGetLastError(), what); }
// Clears a non-sticky error left by an earlier, unrelated runtime call so that
// the launch_check after our launch reports our launch only.
inline void clear_stale_error() { (void)cudaGetLastError(); }

// Opts a kernel in to the device's full dynamic shared-memory size.  The
// attribute is per function, so it is never lowered to one plan's size (a
// later, smaller plan would otherwise make earlier plans' launches fail).
template <typename K>
inline void allow_max_smem(K* func, size_t needed, const char* what) {
  int dev = 0, optin = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
             "cudaDeviceGetAttribute");
  cudaFuncAttributes fa;
  cuda_check(cudaFuncGetAttributes(&fa, func), what);
  const int maxdyn = optin - (int)fa.sharedSizeBytes;  // static smem counts against the opt-in
  if (needed > (size_t)maxdyn)
    throw Error(4, std::string(what) + ": needs more shared memory than the device offers");
  cuda_check(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn), what);
}

// Owning device buffer.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() {
    if (ptr) cudaFree(ptr);
  }
  void alloc(size_t n) {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = n;
    if (n == 0) return;
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
      ptr = nullptr;
      throw Error(5, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
  }
  void upload(const void* src, size_t n) {
    alloc(n);
    if (n) cuda_check(cudaMemcpy(ptr, src, n, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(ptr);
  }
};

// ---------------------------------------------------------------------------
// Orientation <-> projection transform plan (device tables).
// ---------------------------------------------------------------------------
// One direction of the tensor-core angular transform (angular_tc.cu): the
// dense per-point matrix of ang_matrix_a2p / ang_matrix_p2a applied to all
// grid points as one GEMM, both operands as exact BF16 digit slices.
struct AngTcDir {
  int K, nkc;            // real inputs per point; 16-wide K chunks
  int NOUT, NC, nnc;     // real outputs per point; N-chunk width; N-chunks
  int tcols;             // tensor-memory columns per CTA
  int nsm;               // persistent grid: one CTA per SM
  size_t raw_bytes;      // shared-memory bytes of one raw input tile
  size_t smem;           // dynamic shared memory per CTA
  const uint16_t* bsl;   // (nnc, nkc, digits, 2, NC/8, 8, 8) BF16 digits of the matrix
  const int* fexp;       // (nnc NC) exponent of each output column's digits
};

struct AngPlan {
  long long N;  // grid points
  int ntheta, nphi, npsi, K, mmax, mrso, np, no;
  int tile_a2p, tile_p2a;           // points per CTA
  int tc;                           // bit 0 / 1: angl2proj / proj2angl on the tensor cores
  AngTcDir tc_a2p, tc_p2a;
  int fast;                         // 1: compile-time-shape kernels (angular_fast.cu)
  size_t smem_a2p, smem_p2a;        // dynamic shared memory bytes
  const void* coef_a2p;             // (ntheta, np) T : d * wtheta * fm / (nphi*npsi)
  const void* coef_p2a;             // (ntheta, np) T : d * fm
  const void* tw_phi;               // (nphi) Cx<T> : exp(-2 pi i t / nphi)
  const void* tw_psi;               // (npsi) Cx<T>
  const int* ip_m;                  // (np)
  const int* ip_mup;                // (np)
  const int* ip_mu2;                // (np)
  const int* pmap;                  // (mmax+1, 2mmax+1, K+1)
};

// S: storage type of the fields (double/float); C: arithmetic type
// (double, float, or DF for the FP64 form on the FP32 pipes).
template <typename S, typename C>
void launch_angl2proj(const AngPlan& P, const S* o, Cx<S>* p, bool from_xi,
                      double rho0, cudaStream_t s);
template <typename S, typename C>
void launch_proj2angl(const AngPlan& P, const Cx<S>* p, S* o, cudaStream_t s);
template <typename S, typename C>
void ang_plan_finish(AngPlan& P);
// Tensor-core path: digit slices of the dense matrices (host), launches.
// S = double (FP64 fields, the double-float form) or float (mixed form).
// ang_tc_setup returns false (and leaves D unused) when the shape does not fit
// the kernel: K above the exact-sum limit, or the tiles beyond shared memory.
template <typename S>
bool ang_tc_setup(AngTcDir& D, const std::vector<double>& T, int nout, int k, int dir, DevBuf& bsl,
                  DevBuf& fexp);
template <typename S>
void ang_tc_launch(const AngPlan& P, int dir, const S* in, S* out, cudaStream_t s);
// Compile-time-shape kernels for (mmax, mrso) in {1..5} x {2}.
bool ang_fast_supported(int mmax, int mrso);
template <typename S, typename C>
void ang_fast_setup(const AngPlan& P);
template <typename S, typename C>
void ang_fast_a2p(const AngPlan& P, const S* o, Cx<S>* p, bool from_xi, double rho0, cudaStream_t s);
template <typename S, typename C>
void ang_fast_p2a(const AngPlan& P, const Cx<S>* p, S* o, cudaStream_t s);  // picks tiles / smem sizes, sets attributes

// ---------------------------------------------------------------------------
// Batched 1-D FFT along one axis of a (B, n, S) complex array.
// ---------------------------------------------------------------------------
constexpr int kMaxRadices = 16;
struct FftAxis {
  int n;          // transform length
  long long S;    // stride between consecutive elements of one transform
  long long ncols;  // number of transforms (B * S)
  int nr;         // number of radix stages
  int radix[kMaxRadices];
  int cols;       // transforms per CTA
  size_t smem;
  int fixed;      // 1: compile-time-length kernel for n, 0: runtime-radix kernel
  int tma;        // 1: S > 1 tiles may move by tensor-memory-access copies
  int* err;       // device counter of timed-out copy waits (this device's)
  int* flag;      // host-mapped word set to 1 by a timed-out wait (this device's)
  const void* tw;  // (n) Cx<T> : exp(-2 pi i t / n)
};
// The current device's record of bounded device waits that ran out: a
// device counter (exact count, read by mdft_wait_timeouts) and a word of
// mapped page-locked host memory that the timed-out kernel sets, so the host
// sees it without a synchronisation.  Created on first use (call outside
// stream capture).
struct WaitStatus {
  int* count;                // device memory
  int* flag_dev;             // device address of the mapped host word
  volatile int* flag_host;   // host address of the same word
};
const WaitStatus& device_wait_status();
int* fft_wait_error_counter();
// Throws Error(MDFT_ERR_TIMEOUT) if a kernel launched earlier on the current
// device reported a timed-out wait since the last check, and clears the
// report: a kernel that gives up on a wait leaves its output wrong, and the
// next call that launches work on the device says so.
void check_device_waits();
// Launches a one-CTA kernel whose bounded wait runs out (nothing arrives).
void launch_wait_selftest(long long spins, cudaStream_t s);
// Device side of a timed-out wait: count it and raise the host-visible word.
__device__ __forceinline__ void note_wait_timeout(int* count, int* flag) {
  atomicAdd(count, 1);
  *reinterpret_cast<volatile int*>(flag) = 1;
  __threadfence_system();
}
bool fft_factor(int n, FftAxis& a);  // false if n has a prime factor > 13
// Si / So: storage type of the tile on load / store (the same size, in
// place); the double-float form keeps the projections as packed DF pairs
// between the passes of one convolution.
template <typename Si, typename So, typename C>
void fft_axis_finish(FftAxis& a);
template <typename Si, typename So, typename C>
void launch_fft_axis(const FftAxis& a, void* data, int sign, cudaStream_t s);

// ---------------------------------------------------------------------------
// Fused (q,-q) rotation + Ornstein-Zernike + rotation back.
// ---------------------------------------------------------------------------
// projections from which the split forms' k-space step runs one warp per
// pair (oz_warp_kernel) instead of one lane per pair side, by measurement on
// one GB300: double-float from mmax 4 (np 55 at mrso 2: 5.64 -> 5.08 ms at
// 96^3; mmax 5, 39.9 -> 21.9 ms at 128^3), FP32 from mmax 5 (10.1 -> 9.0 ms
// at 128^3; at mmax 4 the lane kernel is faster, 1.46 against 2.18 ms)
template <typename C>
constexpr int oz_warp_min_np() {
  return sizeof(C) == 4 ? 80 : 50;
}

struct OzPlan {
  int nx, ny, nz, np, mmax, mrso, K, np_new, nq, npairs;
  long long N;
  // batched plans: nbatch same-shape fields, p laid out (np, nbatch, N), so
  // the projection stride is pstride = nbatch N and field b starts at b N
  int nbatch;
  long long pstride;
  double dq;
  const int4* pairs;       // (npairs) ix, iy, iz, 0 -- sorted by q's linear index
  const double* kx;        // (nx)
  const double* ky;
  const double* kz;
  const double* rot;       // a (5,13,13) | b (5,13,13) | c (5,13) | d (5,13)
  const int* pmap;         // (mmax+1, 2mmax+1, K+1)
  const int* ip_m;
  const int* ip_mup;
  const int* ip_mu2;
  const int* ia_map;       // (np, mmax+1, 2mmax/mrso+1)
  const void* ctab;        // (nq, np_new) Cx<T>, transposed mnmunukhi_q
  // (nu, np_new) Cx<C>: c(|q|) already interpolated for each distinct |q| of
  // the pair list (lane path; pinfo.z then indexes its rows), or null
  const void* ceff;
  // split lane kernel on a pair list sorted by |q| (ceff rows in increasing
  // |q|): up to crow_stage consecutive ceff rows, from the row of the CTA's
  // first pair, are staged in shared memory at byte offset cstage_off
  int crow_stage;
  size_t cstage_off;
  int warps_per_cta;
  size_t smem;
  // Lane-per-pair path: per-pair geometry computed once at plan creation.
  int lane_path;           // 1: oz_lane_kernel, 0: warp-per-pair fallback
  // lane path of the split forms on large angular grids: one warp per pair
  // (oz_warp_kernel) over the same tables, instead of a lane per pair side
  int warp_pairs;
  long long npairs_pad;    // npairs rounded up to a multiple of 32
  int nR;                  // entries per pair in rtab (see oz_build_rtab)
  const int4* pinfo;       // (npairs_pad) lq, lmq, iq, singular (padding: zeros)
  const void* palpha;      // (npairs_pad) T interpolation weight of row iq+1
  const int* ia_start;     // (np) first OZ coefficient of each projection
  // (npairs_pad/32, nR, 32), lane fastest: R(q) of 32 pairs as Cx<double>
  // (FP64 arithmetic), or the real factor and phase powers of R as T
  const void* rtab;
};
template <typename S, typename C>
void oz_plan_finish(OzPlan& P);
// Fills the R(q) table of the lane path (FP64 recursion, stored as T).
template <typename C>
void oz_build_rtab(const OzPlan& P, DevBuf& rtab);
template <typename S, typename C>
void launch_oz(const OzPlan& P, Cx<S>* p, cudaStream_t s);
// Shared-memory attributes of the lane kernels for storage S (used for the
// packed double-float storage inside one convolution).
template <typename S, typename C>
void oz_lane_attr(const OzPlan& P);

// ---------------------------------------------------------------------------
// Energy / gradient.
// ---------------------------------------------------------------------------
template <typename T>
void launch_delta_rho(const T* xi, T* dr, size_t n, double rho0, cudaStream_t s);
// partials: >= delta_f_partials(nxyz) double2 entries + one uint counter
// (zeroed by the caller before the first use; the kernel leaves it zero).
size_t delta_f_partials(size_t nxyz, int no);
// Stores `msg` as the calling thread's mdft_last_error() text and returns
// `code` (for extern "C" entry points defined outside capi.cu).
int record_error(int code, const std::string& msg);

// fp64: FP64 arithmetic (the MDFT_F64 form); otherwise double-float on the
// FP32 pipes (double fields) or float (float fields)
template <typename T>
void launch_delta_f(const T* xi, const T* vexc, const double* w, T* df,
                    double* ff, size_t nxyz, int no, double rho0,
                    double prefactor, void* work, cudaStream_t s, bool fp64);

}  // namespace mdft

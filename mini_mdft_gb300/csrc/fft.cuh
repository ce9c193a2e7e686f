// fft.cuh -- batched in-place complex 1-D FFTs along one axis of the
// projection array, the building block of the 3-D transforms of
// Convolution::execute (common/MDFT_Convolution.hpp:198-208, :328, :546).
//
// The array is viewed as (B, n, S): n is the transform length and S the
// distance between consecutive elements of one transform (S = 1 for the
// contiguous z axis, S = nz for y, S = ny*nz for x).  One CTA owns `cols`
// transforms: it stages them in shared memory (for S > 1 the `cols`
// transforms are adjacent in memory, so every row of the tile is one
// contiguous run), runs a mixed-radix Stockham autosort FFT in shared memory
// (natural order in and out, no bit reversal) and writes the tile back.
// Forward uses exp(-2 pi i jk/n), backward exp(+2 pi i jk/n); neither is
// normalised (KokkosFFT::Normalization::none).
//
// S is the storage type of the array (double or float), C the arithmetic
// type (the same, or double-float DF for the FP64 form on the FP32 pipes).
#pragma once
#include <type_traits>

#include <cuda.h>

#include <cstdint>

#include "common.cuh"

namespace mdft {

inline bool fft_factor_impl(int n, FftAxis& a) {
  a.n = n;
  a.nr = 0;
  int m = n;
  while (m % 4 == 0 && m > 4 && m != 8) {
    a.radix[a.nr++] = 4;
    m /= 4;
  }
  const int rs[] = {4, 2, 3, 5, 7, 11, 13};
  for (int r : rs) {
    while (m % r == 0) {
      if (a.nr >= kMaxRadices) return false;
      a.radix[a.nr++] = r;
      m /= r;
    }
  }
  return m == 1;
}

namespace {

constexpr int kFftThreads = 256;

template <typename C, typename S>
__device__ __forceinline__ Cx<C> ld_c(const Cx<S>& z) {
  return mkc<C>(to_compute<C>(z.re), to_compute<C>(z.im));
}
template <typename S, typename C>
__device__ __forceinline__ Cx<S> st_c(const Cx<C>& z) {
  return mkc<S>(to_storage<S>(z.re), to_storage<S>(z.im));
}

template <typename T>
__device__ __forceinline__ Cx<T> twiddle(const Cx<T>* tw, int idx, int sign) {
  Cx<T> t = tw[idx];
  if (sign > 0) t.im = -t.im;
  return t;
}

// In-register DFT of length R on v[0..R-1] (R <= 13), runtime radix.
template <typename T>
__device__ __forceinline__ void small_dft(Cx<T>* v, int R, int sign, const Cx<T>* tw, int n) {
  if (R == 2) {
    Cx<T> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  } else if (R == 4) {
    Cx<T> a0 = v[0] + v[2], a1 = v[0] - v[2];
    Cx<T> b0 = v[1] + v[3], b1 = v[1] - v[3];
    // forward: b1 * (-i); backward: b1 * (+i)
    Cx<T> jb = sign < 0 ? mkc<T>(b1.im, -b1.re) : mkc<T>(-b1.im, b1.re);
    v[0] = a0 + b0;
    v[1] = a1 + jb;
    v[2] = a0 - b0;
    v[3] = a1 - jb;
  } else if (R == 3) {
    const T s3 = T(0.86602540378443864676372317075293618);
    Cx<T> a = v[0], b = v[1], c = v[2];
    Cx<T> bc = b + c;
    Cx<T> t = mkc<T>(a.re - T(0.5) * bc.re, a.im - T(0.5) * bc.im);
    Cx<T> u = mkc<T>(s3 * (b.re - c.re), s3 * (b.im - c.im));
    v[0] = a + bc;
    if (sign < 0) {
      v[1] = mkc<T>(t.re + u.im, t.im - u.re);
      v[2] = mkc<T>(t.re - u.im, t.im + u.re);
    } else {
      v[1] = mkc<T>(t.re - u.im, t.im + u.re);
      v[2] = mkc<T>(t.re + u.im, t.im - u.re);
    }
  } else {
    Cx<T> out[13];
    const int step = n / R;
    for (int s = 0; s < R; ++s) {
      Cx<T> acc = v[0];
      for (int q = 1; q < R; ++q) acc = cmac(acc, v[q], twiddle(tw, ((q * s) % R) * step, sign));
      out[s] = acc;
    }
    for (int s = 0; s < R; ++s) v[s] = out[s];
  }
}

// Runtime-radix kernel: any length whose prime factors are <= 13.  The tile
// is loaded as Si and stored as So (same size; in place).
template <typename Si, typename So, typename C>
__global__ void __launch_bounds__(kFftThreads)
fft_axis_kernel(const FftAxis A, void* __restrict__ vdata, int sign) {
  const Cx<Si>* din = static_cast<const Cx<Si>*>(vdata);
  Cx<So>* dout = static_cast<Cx<So>*>(vdata);
  extern __shared__ __align__(16) unsigned char sm[];
  const int n = A.n, CL = A.cols;
  Cx<C>* buf0 = reinterpret_cast<Cx<C>*>(sm);
  Cx<C>* buf1 = buf0 + (size_t)n * CL;
  Cx<C>* tw = buf1 + (size_t)n * CL;
  const int tid = threadIdx.x, bd = blockDim.x;
  const long long c0 = (long long)blockIdx.x * CL;
  const int cc = (int)min((long long)CL, A.ncols - c0);
  const long long S_ = A.S;

  for (int i = tid; i < n; i += bd) tw[i] = static_cast<const Cx<C>*>(A.tw)[i];
  if (S_ == 1) {
    const Cx<Si>* src = din + c0 * n;
    for (int i = tid; i < n * cc; i += bd) {
      const int c = i / n, j = i % n;
      buf0[j * CL + c] = ld_c<C>(src[i]);
    }
  } else {
    for (int i = tid; i < n * cc; i += bd) {
      const int j = i / cc, c = i % cc;
      const long long col = c0 + c;
      const long long b = col / S_, s = col % S_;
      buf0[j * CL + c] = ld_c<C>(din[(b * n + j) * S_ + s]);
    }
  }
  Cx<C>* in = buf0;
  Cx<C>* out = buf1;
  int Ns = 1;
  for (int st = 0; st < A.nr; ++st) {
    const int R = A.radix[st];
    const int nR = n / R;
    const int twstep = n / (Ns * R);
    __syncthreads();
    for (int w = tid; w < nR * cc; w += bd) {
      const int c = w % cc, j = w / cc;
      const int k = j % Ns;
      Cx<C> v[13];
      v[0] = in[j * CL + c];
      for (int r = 1; r < R; ++r) {
        const Cx<C> x = in[(j + r * nR) * CL + c];
        v[r] = (k == 0) ? x : x * twiddle(tw, k * r * twstep, sign);
      }
      small_dft(v, R, sign, tw, n);
      const int d = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; ++r) out[(d + r * Ns) * CL + c] = v[r];
    }
    Cx<C>* t = in;
    in = out;
    out = t;
    Ns *= R;
  }
  __syncthreads();
  if (S_ == 1) {
    Cx<So>* dst = dout + c0 * n;
    for (int i = tid; i < n * cc; i += bd) {
      const int c = i / n, j = i % n;
      dst[i] = st_c<So>(in[j * CL + c]);
    }
  } else {
    for (int i = tid; i < n * cc; i += bd) {
      const int j = i / cc, c = i % cc;
      const long long col = c0 + c;
      const long long b = col / S_, s = col % S_;
      dout[(b * n + j) * S_ + s] = st_c<So>(in[j * CL + c]);
    }
  }
}

// ---------------------------------------------------------------------------
// Compile-time-length kernels for the grid sizes of the workloads
// (16..256 with radices 4, 2, 3, 5).  The radix schedule, the tile width and
// every index stride are compile-time constants, so the butterflies stay in
// registers and no runtime division is left in the loops.  Tiles are stored
// [element][column] with one column of padding, which keeps both the
// contiguous z-axis load and the column-wise butterflies bank-conflict-free.
// ---------------------------------------------------------------------------
template <int... Rs>
struct RList {};
template <int N>
struct FftRadices;
template <> struct FftRadices<16> { using type = RList<4, 4>; };
template <> struct FftRadices<32> { using type = RList<8, 4>; };
template <> struct FftRadices<64> { using type = RList<8, 8>; };
template <> struct FftRadices<128> { using type = RList<8, 4, 4>; };
template <> struct FftRadices<256> { using type = RList<8, 8, 4>; };
template <> struct FftRadices<48> { using type = RList<4, 4, 3>; };
template <> struct FftRadices<96> { using type = RList<8, 4, 3>; };
template <> struct FftRadices<192> { using type = RList<8, 8, 3>; };
template <> struct FftRadices<80> { using type = RList<4, 4, 5>; };
template <> struct FftRadices<160> { using type = RList<8, 4, 5>; };

// x * w for a twiddle w: the plain complex product, and for double-float
// each component a.b + c.d as two exact FMA products whose high parts meet
// in one TwoSum (19 FP32 instructions a component instead of 25)
template <typename T>
__device__ __forceinline__ Cx<T> cmul_tw(Cx<T> x, Cx<T> w) {
  return x * w;
}
__device__ __forceinline__ DF df_dot2_pair(DF a, DF b, DF c, DF d) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float q = c.hi * d.hi;
  float f = fmaf(c.hi, d.hi, -q);
  f = fmaf(c.hi, d.lo, f);
  f = fmaf(c.lo, d.hi, f);
  const DF s = df_two_sum(p, q);
  return df_fast_two_sum(s.hi, s.lo + (e + f));
}
template <>
__device__ __forceinline__ Cx<DF> cmul_tw<DF>(Cx<DF> x, Cx<DF> w) {
  return mkc<DF>(df_dot2_pair(x.re, w.re, -x.im, w.im), df_dot2_pair(x.re, w.im, x.im, w.re));
}
// Sums inside a butterfly: for double-float the pair is left unnormalised
// (hi = fl(a.hi + b.hi), lo = its rounding error + a.lo + b.lo, still the
// exact sum up to the lo additions); the butterfly's outputs are normalised.
// The error stays bounded relative to the operands, the norm-wise bound of
// FFT error analysis.
template <typename T>
__device__ __forceinline__ Cx<T> lz_add(Cx<T> a, Cx<T> b) {
  return a + b;
}
template <typename T>
__device__ __forceinline__ Cx<T> lz_sub(Cx<T> a, Cx<T> b) {
  return a - b;
}
__device__ __forceinline__ DF df_add_lazy(DF a, DF b) {
  const DF s = df_two_sum(a.hi, b.hi);
  return DF(s.hi, s.lo + (a.lo + b.lo));
}
template <>
__device__ __forceinline__ Cx<DF> lz_add<DF>(Cx<DF> a, Cx<DF> b) {
  return mkc<DF>(df_add_lazy(a.re, b.re), df_add_lazy(a.im, b.im));
}
template <>
__device__ __forceinline__ Cx<DF> lz_sub<DF>(Cx<DF> a, Cx<DF> b) {
  return mkc<DF>(df_add_lazy(a.re, -b.re), df_add_lazy(a.im, -b.im));
}

// the length-4 DFT on registers (forward: e^{-2 pi i nk/4}); LAZY leaves
// the outputs unnormalised too (they feed another layer of sums)
template <typename T, bool FWD, bool LAZY = false>
__device__ __forceinline__ void dft4(Cx<T>& v0, Cx<T>& v1, Cx<T>& v2, Cx<T>& v3) {
  const Cx<T> a0 = lz_add(v0, v2), a1 = lz_sub(v0, v2);
  const Cx<T> b0 = lz_add(v1, v3), b1 = lz_sub(v1, v3);
  const Cx<T> jb = FWD ? mkc<T>(b1.im, -b1.re) : mkc<T>(-b1.im, b1.re);
  if (LAZY) {
    v0 = lz_add(a0, b0);
    v1 = lz_add(a1, jb);
    v2 = lz_sub(a0, b0);
    v3 = lz_sub(a1, jb);
  } else {
    v0 = a0 + b0;
    v1 = a1 + jb;
    v2 = a0 - b0;
    v3 = a1 - jb;
  }
}

template <typename T, bool FWD>
__device__ __forceinline__ Cx<T> tw_at(const Cx<T>* tw, int idx) {
  Cx<T> t = tw[idx];
  if (!FWD) t.im = -t.im;
  return t;
}

// DFT of length R (2, 3, 4, 5) on registers.
template <typename T, int R, bool FWD>
__device__ __forceinline__ void dft_small(Cx<T>* v, const Cx<T>* tw, int n) {
  if constexpr (R == 2) {
    const Cx<T> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  } else if constexpr (R == 4) {
    dft4<T, FWD>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    // two length-4 DFTs (even and odd inputs) and the e^{-+2 pi i k/8}
    // twiddles between them; 1/sqrt(2) from the twiddle table, tw[n/8]
    Cx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    Cx<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<T, FWD, true>(e0, e1, e2, e3);
    dft4<T, FWD, true>(o0, o1, o2, o3);
    const T h = tw[n / 8].re;
    // forward: o1 (1 - i) h, o2 (-i), o3 (-1 - i) h; inverse: conjugates
    const Cx<T> o1s = lz_add(o1, mkc<T>(o1.im, -o1.re)), o3s = lz_add(o3, mkc<T>(-o3.im, o3.re));
    if (FWD) {
      o1 = mkc<T>(o1s.re * h, o1s.im * h);  // (re + im, im - re) h
      o2 = mkc<T>(o2.im, -o2.re);
      o3 = mkc<T>(-o3s.re * h, -o3s.im * h);  // (im - re, -(re + im)) h
    } else {
      const Cx<T> o1c = lz_add(o1, mkc<T>(-o1.im, o1.re)), o3c = lz_add(o3, mkc<T>(o3.im, -o3.re));
      o1 = mkc<T>(o1c.re * h, o1c.im * h);  // (re - im, im + re) h
      o2 = mkc<T>(-o2.im, o2.re);
      o3 = mkc<T>(-o3c.re * h, -o3c.im * h);  // (-(re + im), re - im) h
    }
    v[0] = e0 + o0;
    v[4] = e0 - o0;
    v[1] = e1 + o1;
    v[5] = e1 - o1;
    v[2] = e2 + o2;
    v[6] = e2 - o2;
    v[3] = e3 + o3;
    v[7] = e3 - o3;
  } else if constexpr (R == 3) {
    // sin(2 pi / 3) from the twiddle table, tw[n/3] = (-1/2, -sin(2 pi/3))
    const T s3 = -tw[n / 3].im;
    const Cx<T> a = v[0], b = v[1], c = v[2];
    const Cx<T> bc = b + c;
    const Cx<T> hb = mkc<T>(bc.re * tw[n / 3].re, bc.im * tw[n / 3].re);  // -bc/2
    const Cx<T> t = mkc<T>(a.re + hb.re, a.im + hb.im);
    const Cx<T> u = mkc<T>(s3 * (b.re - c.re), s3 * (b.im - c.im));
    v[0] = a + bc;
    if (FWD) {
      v[1] = mkc<T>(t.re + u.im, t.im - u.re);
      v[2] = mkc<T>(t.re - u.im, t.im + u.re);
    } else {
      v[1] = mkc<T>(t.re - u.im, t.im + u.re);
      v[2] = mkc<T>(t.re + u.im, t.im - u.re);
    }
  } else {
    static_assert(R == 5, "radix");
    Cx<T> out[5];
    const int step = n / 5;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      Cx<T> acc = v[0];
#pragma unroll
      for (int q = 1; q < 5; ++q) acc = cmac(acc, v[q], tw_at<T, FWD>(tw, ((q * s) % 5) * step));
      out[s] = acc;
    }
#pragma unroll
    for (int s = 0; s < 5; ++s) v[s] = out[s];
  }
}

template <typename T, int N, int LD, bool FWD, int Ns>
__device__ __forceinline__ Cx<T>* stages(Cx<T>* in, Cx<T>*, const Cx<T>*, int, int, RList<>) {
  return in;
}

template <typename T, int N, int LD, bool FWD, int Ns, int R, int... Rest>
__device__ __forceinline__ Cx<T>* stages(Cx<T>* in, Cx<T>* out, const Cx<T>* tw, int cols, int cc,
                                         RList<R, Rest...>) {
  constexpr int NR = N / R;
  constexpr int TWS = N / (Ns * R);
  __syncthreads();
  for (int w = threadIdx.x; w < NR * cols; w += blockDim.x) {
    const int c = w % cols, j = w / cols;
    if (c < cc) {
      const int k = j % Ns;
      Cx<T> v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const Cx<T> x = in[(j + r * NR) * LD + c];
        // the first stage (Ns = 1) has unit twiddles
        v[r] = (r == 0 || Ns == 1) ? x : cmul_tw(x, tw_at<T, FWD>(tw, k * r * TWS));
      }
      dft_small<T, R, FWD>(v, tw, N);
      const int d = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) out[(d + r * Ns) * LD + c] = v[r];
    }
  }
  return stages<T, N, LD, FWD, Ns * R>(out, in, tw, cols, cc, RList<Rest...>{});
}

template <typename Si, typename So, typename C, int N, int COLS, bool FWD, int THREADS>
__global__ void __launch_bounds__(THREADS)
fft_fixed_kernel(const FftAxis A, void* __restrict__ vdata) {
  const Cx<Si>* din = static_cast<const Cx<Si>*>(vdata);
  Cx<So>* dout = static_cast<Cx<So>*>(vdata);
  extern __shared__ __align__(16) unsigned char sm[];
  constexpr int LD = COLS + 1;  // padded column stride of the tile
  Cx<C>* buf0 = reinterpret_cast<Cx<C>*>(sm);
  Cx<C>* buf1 = buf0 + N * LD;
  Cx<C>* tw = buf1 + N * LD;
  const int tid = threadIdx.x, bd = blockDim.x;
  const long long c0 = (long long)blockIdx.x * COLS;
  const int cc = (int)min((long long)COLS, A.ncols - c0);
  const long long S_ = A.S;
  for (int i = tid; i < N; i += bd) tw[i] = static_cast<const Cx<C>*>(A.tw)[i];
  // full tiles: every load of a thread issued before its shared stores (one
  // memory round trip per tile); THREADS is the launch's block size
  constexpr int IT = N * COLS / THREADS;
  static_assert(N * COLS % THREADS == 0, "tile and block size");
  if (S_ == 1) {
    const Cx<Si>* src = din + c0 * N;
    if (cc == COLS) {
      Cx<Si> v[IT];
#pragma unroll
      for (int r = 0; r < IT; ++r) v[r] = src[tid + r * THREADS];
#pragma unroll
      for (int r = 0; r < IT; ++r) {
        const int i = tid + r * THREADS, c = i / N, j = i % N;
        buf0[j * LD + c] = ld_c<C>(v[r]);
      }
    } else {
      for (int i = tid; i < N * cc; i += bd) {
        const int c = i / N, j = i % N;
        buf0[j * LD + c] = ld_c<C>(src[i]);
      }
    }
  } else {
    const long long b = c0 / S_, s0 = c0 % S_;
    if (s0 + cc <= S_) {  // the tile's columns are one contiguous run per row
      const Cx<Si>* base = din + b * N * S_ + s0;
      if (cc == COLS) {
        Cx<Si> v[IT];
#pragma unroll
        for (int r = 0; r < IT; ++r) {
          const int i = tid + r * THREADS, j = i / COLS, c = i % COLS;
          v[r] = base[(long long)j * S_ + c];
        }
#pragma unroll
        for (int r = 0; r < IT; ++r) {
          const int i = tid + r * THREADS, j = i / COLS, c = i % COLS;
          buf0[j * LD + c] = ld_c<C>(v[r]);
        }
      } else {
        for (int i = tid; i < N * COLS; i += bd) {
          const int j = i / COLS, c = i % COLS;
          if (c < cc) buf0[j * LD + c] = ld_c<C>(base[(long long)j * S_ + c]);
        }
      }
    } else {
      for (int i = tid; i < N * COLS; i += bd) {
        const int j = i / COLS, c = i % COLS;
        if (c < cc) {
          const long long col = c0 + c, bb = col / S_, ss = col % S_;
          buf0[j * LD + c] = ld_c<C>(din[(bb * N + j) * S_ + ss]);
        }
      }
    }
  }
  Cx<C>* res = stages<C, N, LD, FWD, 1>(buf0, buf1, tw, COLS, cc, typename FftRadices<N>::type{});
  __syncthreads();
  if (S_ == 1) {
    Cx<So>* dst = dout + c0 * N;
    for (int i = tid; i < N * cc; i += bd) {
      const int c = i / N, j = i % N;
      dst[i] = st_c<So>(res[j * LD + c]);
    }
  } else {
    const long long b = c0 / S_, s0 = c0 % S_;
    if (s0 + cc <= S_) {
      Cx<So>* base = dout + b * N * S_ + s0;
      for (int i = tid; i < N * COLS; i += bd) {
        const int j = i / COLS, c = i % COLS;
        if (c < cc) base[(long long)j * S_ + c] = st_c<So>(res[j * LD + c]);
      }
    } else {
      for (int i = tid; i < N * COLS; i += bd) {
        const int j = i / COLS, c = i % COLS;
        if (c < cc) {
          const long long col = c0 + c, bb = col / S_, ss = col % S_;
          dout[(bb * N + j) * S_ + ss] = st_c<So>(res[j * LD + c]);
        }
      }
    }
  }
}

template <typename C>
constexpr int fixed_cols() {
  return sizeof(Cx<C>) == 16 ? 16 : 32;
}

// threads per CTA: one per butterfly of the widest stage (N / smallest radix
// butterflies per column), at most 256
template <int R, int... Rest>
constexpr int min_radix(RList<R, Rest...>) {
  if constexpr (sizeof...(Rest) == 0)
    return R;
  else
    return R < min_radix(RList<Rest...>{}) ? R : min_radix(RList<Rest...>{});
}
template <typename C, int N>
constexpr int fixed_threads() {
  constexpr int w = N / min_radix(typename FftRadices<N>::type{}) * fixed_cols<C>();
  return w < 256 ? w : 256;
}

template <typename C, int N>
size_t fixed_smem() {
  constexpr int LD = fixed_cols<C>() + 1;
  return sizeof(Cx<C>) * ((size_t)2 * N * LD + N);
}

template <typename Si, typename So, typename C, int N>
void fixed_attr() {
  constexpr int T = fixed_threads<C, N>();
  allow_max_smem(fft_fixed_kernel<Si, So, C, N, fixed_cols<C>(), true, T>, fixed_smem<C, N>(),
                 "fft smem attribute");
  allow_max_smem(fft_fixed_kernel<Si, So, C, N, fixed_cols<C>(), false, T>, fixed_smem<C, N>(),
                 "fft smem attribute");
}

template <typename Si, typename So, typename C, int N>
void fixed_launch(const FftAxis& a, void* data, int sign, cudaStream_t s) {
  constexpr int COLS = fixed_cols<C>();
  const long long nb = (a.ncols + COLS - 1) / COLS;
  throw_if(nb > 0x7fffffffLL, "FFT batch too large", 4);
  constexpr int T = fixed_threads<C, N>();
  if (sign < 0)
    fft_fixed_kernel<Si, So, C, N, COLS, true, T><<<(unsigned)nb, T, fixed_smem<C, N>(), s>>>(a, data);
  else
    fft_fixed_kernel<Si, So, C, N, COLS, false, T><<<(unsigned)nb, T, fixed_smem<C, N>(), s>>>(a, data);
}

#define MDFT_FIXED_SIZES(X) X(16) X(32) X(64) X(128) X(256) X(48) X(96) X(192) X(80) X(160)

bool fixed_supported(int n) {
  switch (n) {
#define X(N) case N:
    MDFT_FIXED_SIZES(X)
#undef X
    return true;
  }
  return false;
}

template <typename Si, typename So, typename C>
void fixed_setup(int n, size_t& smem) {
  switch (n) {
#define X(N)                      \
  case N:                         \
    fixed_attr<Si, So, C, N>();   \
    smem = fixed_smem<C, N>();    \
    return;
    MDFT_FIXED_SIZES(X)
#undef X
  }
}

template <typename Si, typename So, typename C>
void fixed_dispatch(const FftAxis& a, void* data, int sign, cudaStream_t s) {
  switch (a.n) {
#define X(N)                                       \
  case N:                                          \
    fixed_launch<Si, So, C, N>(a, data, sign, s);  \
    return;
    MDFT_FIXED_SIZES(X)
#undef X
  }
  throw Error(4, "no fixed-length FFT kernel for this length");
}

}  // namespace

// ---------------------------------------------------------------------------
// Tensor-memory-access (TMA) tiles for the strided axes (S > 1).  A CTA's
// tile is COLS adjacent columns of one run of S columns: as a 3-D tensor
// (S, n, ncols / S) of 8-byte words it is the box (COLS w, n, 1), w words
// per complex value, which lands in shared memory as the dense [n][COLS]
// tile the Stockham stages read row by row (conflict-free without padding).
// One thread issues the load, completing on an mbarrier, and, after every
// thread has fenced its writes to the async proxy, the store of the result.
// Columns past the end of a run are filled with zeros on load and clipped on
// store by the copy engine.  The wait is bounded: a copy that does not land
// in time is counted in A.err, waited for once more (bounded), and the CTA
// returns without touching its tile.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned phase, long long limit) {
  for (long long i = 0; i < limit; ++i) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}
constexpr long long kTmaWaitLimit = 1LL << 22;

template <typename Si, typename So, typename C, int N, int COLS, bool FWD, int THREADS>
__global__ void __launch_bounds__(THREADS)
fft_tma_kernel(const __grid_constant__ CUtensorMap tm, const FftAxis A, long long tiles_per_run) {
  static_assert(sizeof(Cx<Si>) == sizeof(Cx<C>) && sizeof(Cx<So>) == sizeof(Cx<C>), "in-place tile");
  constexpr int W = (int)(sizeof(Cx<Si>) / 8);  // 8-byte words per complex value
  constexpr int TILE = N * COLS;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  unsigned char* sm = sm_raw + ((128u - (smem_u32(sm_raw) & 127u)) & 127u);  // 128-byte aligned tile
  Cx<C>* buf0 = reinterpret_cast<Cx<C>*>(sm);
  Cx<C>* buf1 = buf0 + TILE;
  Cx<C>* tw = buf1 + TILE;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(tw + N);
  const int tid = threadIdx.x;
  const long long run = (long long)blockIdx.x / tiles_per_run;
  const int x0 = (int)((long long)blockIdx.x - run * tiles_per_run) * COLS * W;
  const unsigned bar_a = smem_u32(bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a),
                 "r"((unsigned)(TILE * sizeof(Cx<Si>)))
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(buf0)),
        "l"(reinterpret_cast<unsigned long long>(&tm)), "r"(x0), "r"(0), "r"((int)run), "r"(bar_a)
        : "memory");
  }
  for (int i = tid; i < N; i += THREADS) tw[i] = static_cast<const Cx<C>*>(A.tw)[i];
  const bool late = !mbar_wait(bar_a, 0, kTmaWaitLimit);
  if (__syncthreads_or(late)) {
    if (tid == 0) {
      note_wait_timeout(A.err, A.flag);
      mbar_wait(bar_a, 0, kTmaWaitLimit);  // the copy may still be writing the tile
    }
    return;
  }
  if constexpr (!std::is_same<Si, C>::value) {
#pragma unroll
    for (int r = 0; r < TILE / THREADS; ++r) {
      const int i = tid + r * THREADS;
      const Cx<Si> v = reinterpret_cast<const Cx<Si>*>(buf0)[i];
      buf0[i] = ld_c<C>(v);
    }
  }
  Cx<C>* res = stages<C, N, COLS, FWD, 1>(buf0, buf1, tw, COLS, COLS, typename FftRadices<N>::type{});
  __syncthreads();
  if constexpr (!std::is_same<So, C>::value) {
#pragma unroll
    for (int r = 0; r < TILE / THREADS; ++r) {
      const int i = tid + r * THREADS;
      const Cx<C> v = res[i];
      reinterpret_cast<Cx<So>*>(res)[i] = st_c<So>(v);
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (tid == 0) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     reinterpret_cast<unsigned long long>(&tm)),
                 "r"(x0), "r"(0), "r"((int)run), "r"(smem_u32(res))
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
  }
}

template <typename C, int N>
size_t tma_smem() {
  return sizeof(Cx<C>) * ((size_t)2 * N * fixed_cols<C>() + N) + 16 + 128;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      f = nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

// Launches the TMA kernel for this axis and data pointer; false when the
// tile rules do not hold here (the caller then uses the plain kernel).
template <typename Si, typename So, typename C, int N>
bool tma_launch(const FftAxis& a, void* data, int sign, cudaStream_t s) {
  constexpr int COLS = fixed_cols<C>();
  constexpr int T = fixed_threads<C, N>();
  const size_t csize = sizeof(Cx<Si>), W = csize / 8;
  if (!a.tma || a.S <= 1 || a.ncols % a.S != 0) return false;
  if (reinterpret_cast<uintptr_t>(data) % 16 != 0 || (a.S * csize) % 16 != 0) return false;
  const long long runs = a.ncols / a.S, tiles_per_run = (a.S + COLS - 1) / COLS;
  // grid and tile coordinates are 32-bit signed
  if (runs > 0x7fffffffLL || tiles_per_run * runs > 0x7fffffffLL || a.S * (long long)W > 0x7fffffffLL) return false;
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  CUtensorMap tm;
  const cuuint64_t dim[3] = {(cuuint64_t)(a.S * W), (cuuint64_t)N, (cuuint64_t)runs};
  const cuuint64_t stride[2] = {(cuuint64_t)(a.S * csize), (cuuint64_t)(a.S * csize * N)};
  const cuuint32_t box[3] = {(cuuint32_t)(COLS * W), (cuuint32_t)N, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, data, dim, stride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  const unsigned grid = (unsigned)(tiles_per_run * runs);
  if (sign < 0)
    fft_tma_kernel<Si, So, C, N, COLS, true, T><<<grid, T, tma_smem<C, N>(), s>>>(tm, a, tiles_per_run);
  else
    fft_tma_kernel<Si, So, C, N, COLS, false, T><<<grid, T, tma_smem<C, N>(), s>>>(tm, a, tiles_per_run);
  return true;
}

template <typename Si, typename So, typename C>
bool tma_dispatch(const FftAxis& a, void* data, int sign, cudaStream_t s) {
  switch (a.n) {
#define X(N) \
  case N:    \
    return tma_launch<Si, So, C, N>(a, data, sign, s);
    MDFT_FIXED_SIZES(X)
#undef X
  }
  return false;
}

template <typename Si, typename So, typename C>
void tma_setup(int n) {
  switch (n) {
#define X(N)                                                                                                    \
  case N:                                                                                                       \
    allow_max_smem(fft_tma_kernel<Si, So, C, N, fixed_cols<C>(), true, fixed_threads<C, N>()>, tma_smem<C, N>(), \
                   "fft smem attribute");                                                                       \
    allow_max_smem(fft_tma_kernel<Si, So, C, N, fixed_cols<C>(), false, fixed_threads<C, N>()>,                 \
                   tma_smem<C, N>(), "fft smem attribute");                                                     \
    return;
    MDFT_FIXED_SIZES(X)
#undef X
  }
}

template <typename Si, typename So, typename C>
void fft_axis_finish(FftAxis& a) {
  a.tma = 0;
  a.err = nullptr;
  a.flag = nullptr;
  if (fixed_supported(a.n)) {
    a.fixed = 1;
    a.cols = fixed_cols<C>();
    fixed_setup<Si, So, C>(a.n, a.smem);
    if (a.S > 1) {
      a.err = device_wait_status().count;
      a.flag = device_wait_status().flag_dev;
      tma_setup<Si, So, C>(a.n);
      a.tma = 1;
    }
    return;
  }
  a.fixed = 0;
  // transforms per CTA: keep the two ping-pong tiles near 32-64 KB
  int cols = 16;
  if (a.n <= 16) cols = 64;
  else if (a.n <= 32) cols = 32;
  if (a.S > 1 && a.S < cols) {
    // adjacent columns are only contiguous within one S-run
    cols = (int)a.S;
  }
  if (cols < 1) cols = 1;
  a.cols = cols;
  a.smem = sizeof(Cx<C>) * ((size_t)2 * a.n * cols + a.n);
  throw_if(a.smem > 200 * 1024, "FFT length too large for the shared-memory tile", 4);
  allow_max_smem(fft_axis_kernel<Si, So, C>, a.smem, "fft smem attribute");
}

template <typename Si, typename So, typename C>
void launch_fft_axis(const FftAxis& a, void* data, int sign, cudaStream_t s) {
  if (a.n <= 1 || a.ncols == 0) {
    // a length-1 axis is the identity, but the storage format may change
    throw_if(!std::is_same<Si, So>::value, "internal: format change on a length-1 axis", 4);
    return;
  }
  clear_stale_error();
  if (a.fixed) {
    if (!tma_dispatch<Si, So, C>(a, data, sign, s)) fixed_dispatch<Si, So, C>(a, data, sign, s);
    launch_check("fft kernel launch");
    return;
  }
  const long long nb = (a.ncols + a.cols - 1) / a.cols;
  throw_if(nb > 0x7fffffffLL, "FFT batch too large", 4);
  fft_axis_kernel<Si, So, C><<<(unsigned)nb, kFftThreads, a.smem, s>>>(a, data, sign);
  launch_check("fft kernel launch");
}

}  // namespace mdft

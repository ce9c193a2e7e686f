// fft.cu -- batched in-place complex 1-D FFTs along one axis of the
// projection array, the building block of the 3-D transforms of
// Convolution::execute (common/MDFT_Convolution.hpp:198-208, :328, :546).
//
// The array is viewed as (B, n, S): n is the transform length and S the
// distance between consecutive elements of one transform (S = 1 for the
// contiguous z axis, S = nz for y, S = ny*nz for x).  One CTA owns `cols`
// transforms: it stages them in shared memory (for S > 1 the `cols`
// transforms are adjacent in memory, so every row of the tile is one
// contiguous run), runs a mixed-radix Stockham autosort FFT in shared memory
// (radices 4, 2, 3, 5, 7, 11, 13; natural order in and out, no bit reversal)
// and writes the tile back.  Forward uses exp(-2 pi i jk/n), backward
// exp(+2 pi i jk/n); neither is normalised (KokkosFFT::Normalization::none).
#include "common.cuh"

namespace mdft {

bool fft_factor(int n, FftAxis& a) {
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

template <typename T>
__device__ __forceinline__ Cx<T> twiddle(const Cx<T>* tw, int idx, int sign) {
  Cx<T> t = tw[idx];
  if (sign > 0) t.im = -t.im;
  return t;
}

// In-register DFT of length R on v[0..R-1] (R <= 13).
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

template <typename T>
__global__ void __launch_bounds__(kFftThreads)
fft_axis_kernel(const FftAxis A, Cx<T>* __restrict__ data, int sign) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int n = A.n, C = A.cols;
  Cx<T>* buf0 = reinterpret_cast<Cx<T>*>(sm);
  Cx<T>* buf1 = buf0 + (size_t)n * C;
  Cx<T>* tw = buf1 + (size_t)n * C;
  const int tid = threadIdx.x, bd = blockDim.x;
  const long long c0 = (long long)blockIdx.x * C;
  const int cc = (int)min((long long)C, A.ncols - c0);
  const long long S = A.S;

  for (int i = tid; i < n; i += bd) tw[i] = static_cast<const Cx<T>*>(A.tw)[i];
  if (S == 1) {
    const Cx<T>* src = data + c0 * n;
    for (int i = tid; i < n * cc; i += bd) {
      const int c = i / n, j = i % n;
      buf0[j * C + c] = src[i];
    }
  } else {
    for (int i = tid; i < n * cc; i += bd) {
      const int j = i / cc, c = i % cc;
      const long long col = c0 + c;
      const long long b = col / S, s = col % S;
      buf0[j * C + c] = data[(b * n + j) * S + s];
    }
  }
  Cx<T>* in = buf0;
  Cx<T>* out = buf1;
  int Ns = 1;
  for (int st = 0; st < A.nr; ++st) {
    const int R = A.radix[st];
    const int nR = n / R;
    const int twstep = n / (Ns * R);
    __syncthreads();
    for (int w = tid; w < nR * cc; w += bd) {
      const int c = w % cc, j = w / cc;
      const int k = j % Ns;
      Cx<T> v[13];
      v[0] = in[j * C + c];
      for (int r = 1; r < R; ++r) {
        const Cx<T> x = in[(j + r * nR) * C + c];
        v[r] = (k == 0) ? x : x * twiddle(tw, k * r * twstep, sign);
      }
      small_dft(v, R, sign, tw, n);
      const int d = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; ++r) out[(d + r * Ns) * C + c] = v[r];
    }
    Cx<T>* t = in;
    in = out;
    out = t;
    Ns *= R;
  }
  __syncthreads();
  if (S == 1) {
    Cx<T>* dst = data + c0 * n;
    for (int i = tid; i < n * cc; i += bd) {
      const int c = i / n, j = i % n;
      dst[i] = in[j * C + c];
    }
  } else {
    for (int i = tid; i < n * cc; i += bd) {
      const int j = i / cc, c = i % cc;
      const long long col = c0 + c;
      const long long b = col / S, s = col % S;
      data[(b * n + j) * S + s] = in[j * C + c];
    }
  }
}

}  // namespace

template <typename T>
void fft_axis_finish(FftAxis& a) {
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
  a.smem = sizeof(Cx<T>) * ((size_t)2 * a.n * cols + a.n);
  throw_if(a.smem > 200 * 1024, "FFT length too large for the shared-memory tile", 4);
  allow_max_smem(fft_axis_kernel<T>, a.smem, "fft smem attribute");
}

template <typename T>
void launch_fft_axis(const FftAxis& a, Cx<T>* data, int sign, cudaStream_t s) {
  if (a.n <= 1 || a.ncols == 0) return;
  const long long nb = (a.ncols + a.cols - 1) / a.cols;
  throw_if(nb > 0x7fffffffLL, "FFT batch too large", 4);
  clear_stale_error();
  fft_axis_kernel<T><<<(unsigned)nb, kFftThreads, a.smem, s>>>(a, data, sign);
  launch_check("fft kernel launch");
}

template void fft_axis_finish<double>(FftAxis&);
template void fft_axis_finish<float>(FftAxis&);
template void launch_fft_axis<double>(const FftAxis&, Cx<double>*, int, cudaStream_t);
template void launch_fft_axis<float>(const FftAxis&, Cx<float>*, int, cudaStream_t);

}  // namespace mdft

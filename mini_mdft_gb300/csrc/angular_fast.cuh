// angular_fast.cuh -- orientation <-> projection transforms specialised at
// compile time for the angular grids of the workloads (mrso = 2, mmax 1..5).
//
// Same mathematics as angular.cu (angl2proj:
// common/MDFT_OrientationProjectionTransform.hpp:270-380, proj2angl:
// :391-484), restructured so that every loop bound and table index is a
// compile-time constant:
//   * one thread per (grid point, theta) runs the psi and phi DFTs in
//     registers, using the input symmetries: the psi DFT has real input, so
//     only kpsi = 0..K is formed with the (x_j +- x_{n-j}) pairing; the phi
//     DFT of the real kpsi = 0 column forms half the outputs and conjugates
//     the rest; the complex columns pair k with n - k;
//   * one thread per (grid point, projection) forms the theta contraction,
//     writing p in (np, N) layout with consecutive threads on consecutive
//     points;
//   * the point-major orientation tile is staged with one word of padding
//     per point so that the per-thread rows are read bank-conflict-free.
// S is the storage type of the fields, C the arithmetic type.
#pragma once
#include <type_traits>

#include "common.cuh"

namespace mdft {

namespace {

constexpr int np_of(int mmax, int mrso) {
  int n = 0;
  for (int m = 0; m <= mmax; ++m) n += (2 * m + 1) * (m / mrso + 1);
  return n;
}

template <int MMAX, int MRSO>
struct Shape {
  static constexpr int NT = MMAX + 1;
  static constexpr int NPHI = 2 * MMAX + 1;
  static constexpr int K = MMAX / MRSO;
  static constexpr int NPSI = 2 * K + 1;
  static constexpr int ROW = NPHI * NPSI;  // values per (point, theta)
  static constexpr int NO = NT * ROW;
  static constexpr int NP = np_of(MMAX, MRSO);
  static constexpr int LDO = NO + 1;  // padded point stride of the o tile
  // projection index of (m, mup, mu2) in OrientationProjectionMap order
  static constexpr int ip(int m, int mup, int mu2) {
    return np_of(m - 1, MRSO) + (mup + m) * (m / MRSO + 1) + mu2;
  }
};

// Double-float at mmax >= 4: the per-(point, theta) DFT stages would keep a
// whole (phi, psi) row of complex double-float values in registers (up to
// 255 per thread, one CTA per SM); they are split instead into a psi stage
// and a phi stage, one thread per row or column, passing the values through
// shared memory in place.  Every output is formed by the same operations in
// the same order, so results do not change.  These kernels run one CTA of
// 512 threads per SM over twice the points of a 256-thread CTA: the stages'
// work items (a few hundred per tile) then fill the threads' rounds.
template <typename C, int MMAX>
constexpr bool split_dft() {
  return std::is_same<C, DF>::value && MMAX >= 4;
}
// threads per CTA of both kernels (the launches and the staging loops)
template <typename C, int MMAX>
constexpr int ang_threads() {
  return split_dft<C, MMAX>() ? 512 : 256;
}
// CTAs per SM the kernels are compiled for (launch bounds): 128 registers a
// thread for FP32 (two 256-thread CTAs) and for the split stages (one
// 512-thread CTA); the other double-float and FP64 kernels take what they need
template <typename C, int MMAX>
constexpr int ang_min_blocks() {
  return sizeof(C) == 4 ? 2 : 1;
}

// points per CTA: keep the CTA's shared memory near 100 KB (two CTAs per SM),
// or 200 KB for the one 512-thread CTA of the split stages
template <typename C, int MMAX, int MRSO>
constexpr int pts_per_cta() {
  using Sh = Shape<MMAX, MRSO>;
  const long long budget = split_dft<C, MMAX>() ? 200 * 1024 : 104 * 1024;
  int pts = 128;
  while (pts > 16) {
    const long long bytes = (long long)pts * Sh::LDO * sizeof(C) +
                            (long long)Sh::NT * (Sh::K + 1) * Sh::NPHI * pts * sizeof(Cx<C>);
    if (bytes <= budget) break;
    pts /= 2;
  }
  return pts;
}

// bytes of the contraction tables at the end of angl2proj's shared memory:
// coef (NT x NP) and the packed (mup + mmax, mu2) of each projection
template <typename C, int MMAX, int MRSO>
constexpr size_t tab_bytes() {
  using Sh = Shape<MMAX, MRSO>;
  return (size_t)Sh::NT * Sh::NP * sizeof(C) + (size_t)Sh::NP * sizeof(int);
}

template <typename C, int MMAX, int MRSO>
constexpr size_t fast_smem() {
  using Sh = Shape<MMAX, MRSO>;
  constexpr int PTS = pts_per_cta<C, MMAX, MRSO>();
  const size_t a = ((size_t)PTS * Sh::LDO * sizeof(C) + 15) & ~size_t(15);
  const size_t z = (size_t)Sh::NT * (Sh::K + 1) * Sh::NPHI * PTS * sizeof(Cx<C>);
  return a + z + tab_bytes<C, MMAX, MRSO>();
}

template <typename C>
__device__ __forceinline__ Cx<C> ldtw(const void* t, int i) {
  return static_cast<const Cx<C>*>(t)[i];
}


template <typename S, typename C, int MMAX, int MRSO, bool FROM_XI>
__global__ void __launch_bounds__((ang_threads<C, MMAX>()), (ang_min_blocks<C, MMAX>()))
angl2proj_fast_kernel(const AngPlan P, const S* __restrict__ o, Cx<S>* __restrict__ p, C rho0) {
  using Sh = Shape<MMAX, MRSO>;
  constexpr int PTS = pts_per_cta<C, MMAX, MRSO>();
  constexpr int NT = Sh::NT, NPHI = Sh::NPHI, NPSI = Sh::NPSI, K = Sh::K, NO = Sh::NO;
  constexpr int LDO = Sh::LDO, NP = Sh::NP;
  constexpr int HPHI = (NPHI - 1) / 2, HPSI = (NPSI - 1) / 2;
  extern __shared__ __align__(16) unsigned char sm[];
  C* ot = reinterpret_cast<C*>(sm);
  Cx<C>* Zs = reinterpret_cast<Cx<C>*>(sm + (((size_t)PTS * LDO * sizeof(C) + 15) & ~size_t(15)));
  C* coef_s = reinterpret_cast<C*>(Zs + (size_t)NT * (K + 1) * NPHI * PTS);
  int* idx_s = reinterpret_cast<int*>(coef_s + NT * NP);
  const int tid = threadIdx.x;
  const long long pt0 = (long long)blockIdx.x * PTS;
  const int cnt = (int)min((long long)PTS, P.N - pt0);
  for (int i = tid; i < NT * NP; i += blockDim.x) coef_s[i] = static_cast<const C*>(P.coef_a2p)[i];
  for (int i = tid; i < NP; i += blockDim.x) idx_s[i] = (P.ip_mup[i] + MMAX) | (P.ip_mu2[i] << 16);

  // stage the contiguous o tile (and fold in get_delta_rho if asked); all of
  // a thread's loads are issued before the first shared store, so the tile
  // costs one memory round trip instead of one per element
  {
    constexpr int NTH = ang_threads<C, MMAX>();
    constexpr int IT = (PTS * NO + NTH - 1) / NTH;
    const S* src = o + pt0 * NO;
    const int n = cnt * NO;
    S v[IT];
#pragma unroll
    for (int r = 0; r < IT; ++r) {
      const int i = tid + r * NTH;
      if (i < n) v[r] = src[i];
    }
#pragma unroll
    for (int r = 0; r < IT; ++r) {
      const int i = tid + r * NTH;
      if (i < n) {
        const int q = i / NO, j = i - q * NO;
        ot[q * LDO + j] = FROM_XI ? rho0 * to_compute<C>(xi_sq_minus_one(v[r])) : to_compute<C>(v[r]);
      }
    }
  }
  __syncthreads();

  if constexpr (split_dft<C, MMAX>()) {
    // psi DFT, one thread per (point, theta, phi row): Y(f, kpsi) into the
    // Z tile at [theta][kpsi][f][point]
    for (int w = tid; w < NT * NPHI * PTS; w += blockDim.x) {
      const int tf = w / PTS, q = w - tf * PTS;
      if (q >= cnt) continue;
      const int th = tf / NPHI, f = tf - th * NPHI;
      const C* r = ot + q * LDO + th * NPHI * NPSI + f * NPSI;
      Cx<C>* zy = Zs + ((size_t)th * (K + 1) * NPHI + f) * PTS + q;
      C s0 = r[0];
#pragma unroll
      for (int j = 1; j < NPSI; ++j) s0 = s0 + r[j];
      zy[0] = mkc<C>(s0, C(0));
#pragma unroll
      for (int k = 1; k <= K; ++k) {
        Acc<C> re, im;
        acc_set(re, r[0]);
        acc_zero(im);
#pragma unroll
        for (int j = 1; j <= HPSI; ++j) {
          const Cx<C> t = ldtw<C>(P.tw_psi, (k * j) % NPSI);
          acc_mac(re, r[j] + r[NPSI - j], t.re);
          acc_mac(im, r[j] - r[NPSI - j], t.im);
        }
        zy[(size_t)k * NPHI * PTS] = mkc<C>(acc_get(re), acc_get(im));
      }
    }
    __syncthreads();
    // phi DFT, one thread per (point, theta, kpsi): reads its column Y(., kpsi)
    // and writes the outputs over the same slots
    for (int w = tid; w < NT * (K + 1) * PTS; w += blockDim.x) {
      const int tk = w / PTS, q = w - tk * PTS;
      if (q >= cnt) continue;
      const int th = tk / (K + 1), kp = tk - th * (K + 1);
      Cx<C>* zk = Zs + (size_t)(th * (K + 1) + kp) * NPHI * PTS + q;
      Cx<C> Yc[NPHI];
#pragma unroll
      for (int f = 0; f < NPHI; ++f) Yc[f] = zk[(size_t)f * PTS];
      if (kp == 0) {  // real input, X(n-k) = conj(X(k))
        C s0 = Yc[0].re;
#pragma unroll
        for (int j = 1; j < NPHI; ++j) s0 = s0 + Yc[j].re;
        zk[(0 + MMAX) * PTS] = mkc<C>(s0, C(0));
#pragma unroll
        for (int k = 1; k <= HPHI; ++k) {
          Acc<C> are, aim;
          acc_set(are, Yc[0].re);
          acc_zero(aim);
#pragma unroll
          for (int j = 1; j <= HPHI; ++j) {
            const Cx<C> t = ldtw<C>(P.tw_phi, (k * j) % NPHI);
            acc_mac(are, Yc[j].re + Yc[NPHI - j].re, t.re);
            acc_mac(aim, Yc[j].re - Yc[NPHI - j].re, t.im);
          }
          const C re = acc_get(are), im = acc_get(aim);
          zk[(k + MMAX) * PTS] = mkc<C>(re, -im);
          zk[(-k + MMAX) * PTS] = mkc<C>(re, im);
        }
      } else {  // complex input, pair k with n - k
        Cx<C> s0 = Yc[0];
#pragma unroll
        for (int j = 1; j < NPHI; ++j) s0 = s0 + Yc[j];
        zk[(0 + MMAX) * PTS] = conj(s0);
#pragma unroll
        for (int k = 1; k <= HPHI; ++k) {
          Acc<C> pr, pi, qr, qi;
          acc_set(pr, Yc[0].re);
          acc_set(pi, Yc[0].im);
          acc_zero(qr);
          acc_zero(qi);
#pragma unroll
          for (int j = 1; j <= HPHI; ++j) {
            const Cx<C> t = ldtw<C>(P.tw_phi, (k * j) % NPHI);
            const Cx<C> A = Yc[j] + Yc[NPHI - j], B = Yc[j] - Yc[NPHI - j];
            acc_mac(pr, A.re, t.re);
            acc_mac(pi, A.im, t.re);
            acc_mac(qr, B.re, t.im);
            acc_mac(qi, B.im, t.im);
          }
          const Cx<C> Pk = mkc<C>(acc_get(pr), acc_get(pi)), Qk = mkc<C>(acc_get(qr), acc_get(qi));
          zk[(k + MMAX) * PTS] = conj(mkc<C>(Pk.re - Qk.im, Pk.im + Qk.re));
          zk[(-k + MMAX) * PTS] = conj(mkc<C>(Pk.re + Qk.im, Pk.im - Qk.re));
        }
      }
    }
  } else {
  // psi and phi DFTs, one thread per (point, theta)
  for (int w = tid; w < NT * PTS; w += blockDim.x) {
    const int th = w / PTS, q = w - th * PTS;
    if (q >= cnt) continue;
    const C* x = ot + q * LDO + th * NPHI * NPSI;
    Cx<C> Y[NPHI][K + 1];
#pragma unroll
    for (int f = 0; f < NPHI; ++f) {
      const C* r = x + f * NPSI;
      C s0 = r[0];
#pragma unroll
      for (int j = 1; j < NPSI; ++j) s0 = s0 + r[j];
      Y[f][0] = mkc<C>(s0, C(0));
#pragma unroll
      for (int k = 1; k <= K; ++k) {
        Acc<C> re, im;
        acc_set(re, r[0]);
        acc_zero(im);
#pragma unroll
        for (int j = 1; j <= HPSI; ++j) {
          const Cx<C> t = ldtw<C>(P.tw_psi, (k * j) % NPSI);
          acc_mac(re, r[j] + r[NPSI - j], t.re);
          acc_mac(im, r[j] - r[NPSI - j], t.im);
        }
        Y[f][k] = mkc<C>(acc_get(re), acc_get(im));
      }
    }
    Cx<C>* zt = Zs + (size_t)th * (K + 1) * NPHI * PTS + q;
    // kpsi = 0: real input, X(n-k) = conj(X(k))
    {
      C s0 = Y[0][0].re;
#pragma unroll
      for (int j = 1; j < NPHI; ++j) s0 = s0 + Y[j][0].re;
      zt[(0 + MMAX) * PTS] = mkc<C>(s0, C(0));
#pragma unroll
      for (int k = 1; k <= HPHI; ++k) {
        Acc<C> are, aim;
        acc_set(are, Y[0][0].re);
        acc_zero(aim);
#pragma unroll
        for (int j = 1; j <= HPHI; ++j) {
          const Cx<C> t = ldtw<C>(P.tw_phi, (k * j) % NPHI);
          acc_mac(are, Y[j][0].re + Y[NPHI - j][0].re, t.re);
          acc_mac(aim, Y[j][0].re - Y[NPHI - j][0].re, t.im);
        }
        const C re = acc_get(are), im = acc_get(aim);
        // s_f(mup) = conj(o_hat(mup mod nphi)); mup = k and mup = -k
        zt[(k + MMAX) * PTS] = mkc<C>(re, -im);
        zt[(-k + MMAX) * PTS] = mkc<C>(re, im);
      }
    }
    // kpsi >= 1: complex input, pair k with n - k
#pragma unroll
    for (int kp = 1; kp <= K; ++kp) {
      Cx<C>* zk = zt + (size_t)kp * NPHI * PTS;
      Cx<C> s0 = Y[0][kp];
#pragma unroll
      for (int j = 1; j < NPHI; ++j) s0 = s0 + Y[j][kp];
      zk[(0 + MMAX) * PTS] = conj(s0);
#pragma unroll
      for (int k = 1; k <= HPHI; ++k) {
        Acc<C> pr, pi, qr, qi;
        acc_set(pr, Y[0][kp].re);
        acc_set(pi, Y[0][kp].im);
        acc_zero(qr);
        acc_zero(qi);
#pragma unroll
        for (int j = 1; j <= HPHI; ++j) {
          const Cx<C> t = ldtw<C>(P.tw_phi, (k * j) % NPHI);  // (cos, -sin)
          const Cx<C> A = Y[j][kp] + Y[NPHI - j][kp], B = Y[j][kp] - Y[NPHI - j][kp];
          acc_mac(pr, A.re, t.re);
          acc_mac(pi, A.im, t.re);
          acc_mac(qr, B.re, t.im);
          acc_mac(qi, B.im, t.im);
        }
        const Cx<C> Pk = mkc<C>(acc_get(pr), acc_get(pi)), Qk = mkc<C>(acc_get(qr), acc_get(qi));
        // X(k) = P + i Q', X(n-k) = P - i Q' with Q' = sum B (-sin) = Qk
        const Cx<C> Xk = mkc<C>(Pk.re - Qk.im, Pk.im + Qk.re);
        const Cx<C> Xn = mkc<C>(Pk.re + Qk.im, Pk.im - Qk.re);
        zk[(k + MMAX) * PTS] = conj(Xk);
        zk[(-k + MMAX) * PTS] = conj(Xn);
      }
    }
  }
  }
  __syncthreads();

  // theta contraction, one thread per (point, projection)
  for (int w = tid; w < NP * PTS; w += blockDim.x) {
    const int ip = w / PTS, q = w - ip * PTS;
    if (q >= cnt) continue;
    const int mm = idx_s[ip], mupi = mm & 0xffff, mu2 = mm >> 16;
    const Cx<C>* z = Zs + ((size_t)mu2 * NPHI + mupi) * PTS + q;
    Acc<C> sre, sim;
    acc_zero(sre);
    acc_zero(sim);
#pragma unroll
    for (int th = 0; th < NT; ++th) {
      const Cx<C> v = z[(size_t)th * (K + 1) * NPHI * PTS];
      const C c = coef_s[th * NP + ip];
      acc_mac(sre, v.re, c);
      acc_mac(sim, v.im, c);
    }
    const Cx<C> sum = mkc<C>(acc_get(sre), acc_get(sim));
    p[(long long)ip * P.N + pt0 + q] = mkc<S>(to_storage<S>(sum.re), to_storage<S>(sum.im));
  }
}

template <typename S, typename C, int MMAX, int MRSO>
__global__ void __launch_bounds__((ang_threads<C, MMAX>()), (ang_min_blocks<C, MMAX>()))
proj2angl_fast_kernel(const AngPlan P, const Cx<S>* __restrict__ p, S* __restrict__ o) {
  using Sh = Shape<MMAX, MRSO>;
  constexpr int PTS = pts_per_cta<C, MMAX, MRSO>();
  constexpr int NT = Sh::NT, NPHI = Sh::NPHI, NPSI = Sh::NPSI, K = Sh::K, NO = Sh::NO;
  constexpr int LDO = Sh::LDO, NP = Sh::NP;
  constexpr int HPHI = (NPHI - 1) / 2;
  extern __shared__ __align__(16) unsigned char sm[];
  C* ot = reinterpret_cast<C*>(sm);
  Cx<C>* Ps = reinterpret_cast<Cx<C>*>(sm + (((size_t)PTS * LDO * sizeof(C) + 15) & ~size_t(15)));
  const int tid = threadIdx.x;
  const long long pt0 = (long long)blockIdx.x * PTS;
  const int cnt = (int)min((long long)PTS, P.N - pt0);

  // stage p(ip, pt0 .. pt0 + cnt) as Ps[ip][point], loads batched as above
  {
    constexpr int NTH = ang_threads<C, MMAX>();
    constexpr int IT = (NP * PTS + NTH - 1) / NTH;
    Cx<S> v[IT];
#pragma unroll
    for (int r = 0; r < IT; ++r) {
      const int w = tid + r * NTH;
      const int ip = w / PTS, q = w - ip * PTS;
      if (w < NP * PTS && q < cnt) v[r] = p[(long long)ip * P.N + pt0 + q];
    }
#pragma unroll
    for (int r = 0; r < IT; ++r) {
      const int w = tid + r * NTH;
      const int q = w - (w / PTS) * PTS;
      if (w < NP * PTS && q < cnt) Ps[w] = mkc<C>(to_compute<C>(v[r].re), to_compute<C>(v[r].im));
    }
  }
  __syncthreads();

  const C* coef = static_cast<const C*>(P.coef_p2a);
  if constexpr (split_dft<C, MMAX>()) {
    constexpr int HPHI2 = (NPHI - 1) / 2;
    // synthesis over m and inverse phi DFT, one thread per (point, theta,
    // kpsi); U(f, kpsi) goes into the o tile at the slots its psi row will
    // occupy: (f, j = 0) holds the real U(f, 0), (f, 2 kpsi - 1) and
    // (f, 2 kpsi) the real and imaginary parts of U(f, kpsi)
    for (int w = tid; w < NT * (K + 1) * PTS; w += blockDim.x) {
      const int tk = w / PTS, q = w - tk * PTS;
      if (q >= cnt) continue;
      const int th = tk / (K + 1), kp = tk - th * (K + 1);
      Cx<C> oh[NPHI];
#pragma unroll
      for (int mup = -MMAX; mup <= MMAX; ++mup) {
        Acc<C> sre, sim;
        acc_zero(sre);
        acc_zero(sim);
        const int a = mup < 0 ? -mup : mup, b = MRSO * kp;
        const int m0 = a > b ? a : b;
#pragma unroll
        for (int m = m0; m <= MMAX; ++m) {
          const int ip = Sh::ip(m, mup, kp);
          const Cx<C> v = Ps[ip * PTS + q];
          const C c = coef[th * NP + ip];
          acc_mac(sre, v.re, c);
          acc_mac(sim, v.im, c);
        }
        const int kf = mup >= 0 ? mup : mup + NPHI;
        oh[kf] = conj(mkc<C>(acc_get(sre), acc_get(sim)));
      }
      C* row = ot + q * LDO + th * NPHI * NPSI;
      if (kp == 0) {  // only the real part is used (C2R)
        C s0 = oh[0].re;
#pragma unroll
        for (int k = 1; k < NPHI; ++k) s0 = s0 + oh[k].re;
        row[0] = s0;
#pragma unroll
        for (int f = 1; f <= HPHI2; ++f) {
          Acc<C> aa, ab;
          acc_set(aa, oh[0].re);
          acc_zero(ab);
#pragma unroll
          for (int k = 1; k <= HPHI2; ++k) {
            const Cx<C> t = ldtw<C>(P.tw_phi, (k * f) % NPHI);
            acc_mac(aa, oh[k].re + oh[NPHI - k].re, t.re);
            acc_mac(ab, oh[k].im - oh[NPHI - k].im, t.im);
          }
          const C ca = acc_get(aa), cb = acc_get(ab);
          row[f * NPSI] = ca + cb;
          row[(NPHI - f) * NPSI] = ca - cb;
        }
      } else {
        Cx<C> s0 = oh[0];
#pragma unroll
        for (int k = 1; k < NPHI; ++k) s0 = s0 + oh[k];
        row[2 * kp - 1] = s0.re;
        row[2 * kp] = s0.im;
#pragma unroll
        for (int f = 1; f <= HPHI2; ++f) {
          Acc<C> pr, pi, qr, qi;
          acc_set(pr, oh[0].re);
          acc_set(pi, oh[0].im);
          acc_zero(qr);
          acc_zero(qi);
#pragma unroll
          for (int k = 1; k <= HPHI2; ++k) {
            const Cx<C> t = ldtw<C>(P.tw_phi, (k * f) % NPHI);
            const Cx<C> A = oh[k] + oh[NPHI - k], B = oh[k] - oh[NPHI - k];
            acc_mac(pr, A.re, t.re);
            acc_mac(pi, A.im, t.re);
            acc_mac(qr, B.re, t.im);
            acc_mac(qi, B.im, t.im);
          }
          const Cx<C> Pf = mkc<C>(acc_get(pr), acc_get(pi)), Qf = mkc<C>(acc_get(qr), acc_get(qi));
          row[f * NPSI + 2 * kp - 1] = Pf.re + Qf.im;
          row[f * NPSI + 2 * kp] = Pf.im - Qf.re;
          row[(NPHI - f) * NPSI + 2 * kp - 1] = Pf.re - Qf.im;
          row[(NPHI - f) * NPSI + 2 * kp] = Pf.im + Qf.re;
        }
      }
    }
    __syncthreads();
    // C2R along psi, one thread per (point, theta, phi row): reads its row's
    // U values and writes the orientations over the same slots
    for (int w = tid; w < NT * NPHI * PTS; w += blockDim.x) {
      const int tf = w / PTS, q = w - tf * PTS;
      if (q >= cnt) continue;
      C* r = ot + q * LDO + tf * NPSI;  // (theta, f) = tf: row tf of the point
      C u[NPSI];
#pragma unroll
      for (int j = 0; j < NPSI; ++j) u[j] = r[j];
#pragma unroll
      for (int j = 0; j < NPSI; ++j) {
        Acc<C> v;
        acc_set(v, u[0]);
#pragma unroll
        for (int kp = 1; kp <= K; ++kp) {
          const Cx<C> e = ldtw<C>(P.tw_psi, (kp * j) % NPSI);
          acc_mac(v, twice(u[2 * kp - 1]), e.re);
          acc_mac(v, twice(u[2 * kp]), e.im);
        }
        r[j] = acc_get(v);
      }
    }
  } else {
  for (int w = tid; w < NT * PTS; w += blockDim.x) {
    const int th = w / PTS, q = w - th * PTS;
    if (q >= cnt) continue;
    // synthesis over m (OPT:435-449) into FFT order: oh[kf][kp]
    Cx<C> oh[NPHI][K + 1];
#pragma unroll
    for (int mup = -MMAX; mup <= MMAX; ++mup) {
#pragma unroll
      for (int kp = 0; kp <= K; ++kp) {
        Acc<C> sre, sim;
        acc_zero(sre);
        acc_zero(sim);
        const int a = mup < 0 ? -mup : mup, b = MRSO * kp;
        const int m0 = a > b ? a : b;
#pragma unroll
        for (int m = m0; m <= MMAX; ++m) {
          const int ip = Sh::ip(m, mup, kp);
          const Cx<C> v = Ps[ip * PTS + q];
          const C c = coef[th * NP + ip];
          acc_mac(sre, v.re, c);
          acc_mac(sim, v.im, c);
        }
        const Cx<C> s = mkc<C>(acc_get(sre), acc_get(sim));
        const int kf = mup >= 0 ? mup : mup + NPHI;
        oh[kf][kp] = conj(s);
      }
    }
    // inverse phi DFT; for kpsi = 0 only the real part is used (C2R)
    C u0[NPHI];
    {
      C s0 = oh[0][0].re;
#pragma unroll
      for (int k = 1; k < NPHI; ++k) s0 = s0 + oh[k][0].re;
      u0[0] = s0;
#pragma unroll
      for (int f = 1; f <= HPHI; ++f) {
        // Re sum_k oh(k) e^{+i 2 pi k f / n}, pairing k with n - k
        Acc<C> aa, ab;
        acc_set(aa, oh[0][0].re);
        acc_zero(ab);
#pragma unroll
        for (int k = 1; k <= HPHI; ++k) {
          const Cx<C> t = ldtw<C>(P.tw_phi, (k * f) % NPHI);  // (cos, -sin)
          acc_mac(aa, oh[k][0].re + oh[NPHI - k][0].re, t.re);
          acc_mac(ab, oh[k][0].im - oh[NPHI - k][0].im, t.im);
        }
        const C ca = acc_get(aa), cb = acc_get(ab);
        // Re(f) = ca + sum (im_k - im_{n-k}) sin = ca - cb ; Re(n-f) = ca + cb
        u0[f] = ca + cb;
        u0[NPHI - f] = ca - cb;
      }
    }
    Cx<C> u[NPHI][K + 1 > 1 ? K + 1 : 2];
#pragma unroll
    for (int kp = 1; kp <= K; ++kp) {
      Cx<C> s0 = oh[0][kp];
#pragma unroll
      for (int k = 1; k < NPHI; ++k) s0 = s0 + oh[k][kp];
      u[0][kp] = s0;
#pragma unroll
      for (int f = 1; f <= HPHI; ++f) {
        Acc<C> pr, pi, qr, qi;
        acc_set(pr, oh[0][kp].re);
        acc_set(pi, oh[0][kp].im);
        acc_zero(qr);
        acc_zero(qi);
#pragma unroll
        for (int k = 1; k <= HPHI; ++k) {
          const Cx<C> t = ldtw<C>(P.tw_phi, (k * f) % NPHI);
          const Cx<C> A = oh[k][kp] + oh[NPHI - k][kp], B = oh[k][kp] - oh[NPHI - k][kp];
          acc_mac(pr, A.re, t.re);
          acc_mac(pi, A.im, t.re);
          acc_mac(qr, B.re, t.im);
          acc_mac(qi, B.im, t.im);
        }
        const Cx<C> Pf = mkc<C>(acc_get(pr), acc_get(pi)), Qf = mkc<C>(acc_get(qr), acc_get(qi));
        // backward: X(f) = P - i Q', X(n-f) = P + i Q', Q' = sum B (-sin) = Qf
        u[f][kp] = mkc<C>(Pf.re + Qf.im, Pf.im - Qf.re);
        u[NPHI - f][kp] = mkc<C>(Pf.re - Qf.im, Pf.im + Qf.re);
      }
    }
    // C2R along psi: o = Re U0 + 2 sum_k Re(U_k e^{+2 pi i k psi/npsi})
    C* out = ot + q * LDO + th * NPHI * NPSI;
#pragma unroll
    for (int f = 0; f < NPHI; ++f) {
#pragma unroll
      for (int j = 0; j < NPSI; ++j) {
        Acc<C> v;
        acc_set(v, u0[f]);
#pragma unroll
        for (int kp = 1; kp <= K; ++kp) {
          const Cx<C> e = ldtw<C>(P.tw_psi, (kp * j) % NPSI);  // (cos, -sin)
          acc_mac(v, twice(u[f][kp].re), e.re);
          acc_mac(v, twice(u[f][kp].im), e.im);
        }
        out[f * NPSI + j] = acc_get(v);
      }
    }
  }
  }
  __syncthreads();
  S* dst = o + pt0 * NO;
  for (int i = tid; i < cnt * NO; i += blockDim.x) {
    const int q = i / NO, j = i - q * NO;
    dst[i] = to_storage<S>(ot[q * LDO + j]);
  }
}

template <typename S, typename C, int MMAX, int MRSO>
void fast_attr() {
  constexpr size_t sm = fast_smem<C, MMAX, MRSO>();
  allow_max_smem(angl2proj_fast_kernel<S, C, MMAX, MRSO, false>, sm, "angl2proj smem attribute");
  allow_max_smem(angl2proj_fast_kernel<S, C, MMAX, MRSO, true>, sm, "angl2proj smem attribute");
  // proj2angl's second buffer holds NP complex per point instead of the Z tile
  using Sh = Shape<MMAX, MRSO>;
  constexpr int PTS = pts_per_cta<C, MMAX, MRSO>();
  constexpr size_t sm2 = (((size_t)PTS * Sh::LDO * sizeof(C) + 15) & ~size_t(15)) +
                         (size_t)Sh::NP * PTS * sizeof(Cx<C>);
  allow_max_smem(proj2angl_fast_kernel<S, C, MMAX, MRSO>, sm2, "proj2angl smem attribute");
}

template <typename S, typename C, int MMAX, int MRSO>
void fast_a2p(const AngPlan& P, const S* o, Cx<S>* p, bool from_xi, double rho0, cudaStream_t s) {
  constexpr int PTS = pts_per_cta<C, MMAX, MRSO>();
  constexpr size_t sm = fast_smem<C, MMAX, MRSO>();
  const long long nb = (P.N + PTS - 1) / PTS;
  throw_if(nb > 0x7fffffffLL, "grid too large", 4);
  if (from_xi)
    angl2proj_fast_kernel<S, C, MMAX, MRSO, true><<<(unsigned)nb, ang_threads<C, MMAX>(), sm, s>>>(P, o, p, C(rho0));
  else
    angl2proj_fast_kernel<S, C, MMAX, MRSO, false><<<(unsigned)nb, ang_threads<C, MMAX>(), sm, s>>>(P, o, p, C(rho0));
}

template <typename S, typename C, int MMAX, int MRSO>
void fast_p2a(const AngPlan& P, const Cx<S>* p, S* o, cudaStream_t s) {
  using Sh = Shape<MMAX, MRSO>;
  constexpr int PTS = pts_per_cta<C, MMAX, MRSO>();
  constexpr size_t sm2 = (((size_t)PTS * Sh::LDO * sizeof(C) + 15) & ~size_t(15)) +
                         (size_t)Sh::NP * PTS * sizeof(Cx<C>);
  const long long nb = (P.N + PTS - 1) / PTS;
  throw_if(nb > 0x7fffffffLL, "grid too large", 4);
  proj2angl_fast_kernel<S, C, MMAX, MRSO><<<(unsigned)nb, ang_threads<C, MMAX>(), sm2, s>>>(P, p, o);
}

}  // namespace

#define MDFT_ANG_FAST_CASES(X) X(1, 2) X(2, 2) X(3, 2) X(4, 2) X(5, 2)

inline bool ang_fast_supported_impl(int mmax, int mrso) {
#define X(M, R) \
  if (mmax == M && mrso == R) return true;
  MDFT_ANG_FAST_CASES(X)
#undef X
  return false;
}

template <typename S, typename C>
void ang_fast_setup(const AngPlan& P) {
#define X(M, R)                            \
  if (P.mmax == M && P.mrso == R) {        \
    fast_attr<S, C, M, R>();               \
    return;                                \
  }
  MDFT_ANG_FAST_CASES(X)
#undef X
  throw Error(4, "no specialised angular kernel for this grid");
}

template <typename S, typename C>
void ang_fast_a2p(const AngPlan& P, const S* o, Cx<S>* p, bool from_xi, double rho0, cudaStream_t s) {
#define X(M, R)                                          \
  if (P.mmax == M && P.mrso == R) {                      \
    fast_a2p<S, C, M, R>(P, o, p, from_xi, rho0, s);     \
    return;                                              \
  }
  MDFT_ANG_FAST_CASES(X)
#undef X
  throw Error(4, "no specialised angular kernel for this grid");
}

template <typename S, typename C>
void ang_fast_p2a(const AngPlan& P, const Cx<S>* p, S* o, cudaStream_t s) {
#define X(M, R)                             \
  if (P.mmax == M && P.mrso == R) {         \
    fast_p2a<S, C, M, R>(P, p, o, s);       \
    return;                                 \
  }
  MDFT_ANG_FAST_CASES(X)
#undef X
  throw Error(4, "no specialised angular kernel for this grid");
}

}  // namespace mdft

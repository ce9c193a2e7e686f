// angular.cu -- orientation <-> projection transforms.
//
// angl2proj (common/MDFT_OrientationProjectionTransform.hpp:270-380) is, per
// grid point, a real 2-D DFT over (phi, psi) restricted to the frequencies
// the projections use, followed by a contraction over theta with the Wigner-d
// table.  proj2angl (:391-484) is the synthesis over m, the scatter to FFT
// order and an unnormalised 2-D C2R transform.  The reference runs these as
// a batched kokkos-fft call that writes an (N, ntheta, nphi, npsi/2+1)
// complex o_hat buffer to memory, then a team-per-point kernel.  Here one CTA
// owns a tile of consecutive grid points: the tile of o (contiguous in the
// (N, ntheta, nphi, npsi) layout) is staged in shared memory, both DFT
// directions and the theta contraction run out of shared memory, and p is
// written (or read) in (np, N) layout with consecutive threads on
// consecutive points, so no o_hat round trip to HBM exists.
#include <type_traits>

#include "common.cuh"

namespace mdft {

namespace {

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

template <typename C>
struct A2PSmem {
  // byte offsets inside the dynamic shared memory block
  size_t coef, twphi, twpsi, ipm, otile, ybuf, sbuf, total;
  __host__ __device__ A2PSmem(const AngPlan& P, int tp) {
    size_t o = 0;
    coef = o;
    o = align16(o + sizeof(C) * P.ntheta * P.np);
    twphi = o;
    o = align16(o + sizeof(Cx<C>) * P.nphi);
    twpsi = o;
    o = align16(o + sizeof(Cx<C>) * P.npsi);
    ipm = o;
    o = align16(o + sizeof(int) * 3 * P.np);
    otile = o;
    o = align16(o + sizeof(C) * (size_t)tp * P.no);
    ybuf = o;
    o = align16(o + sizeof(Cx<C>) * (size_t)tp * P.ntheta * P.nphi * (P.K + 1));
    sbuf = o;
    o = align16(o + sizeof(Cx<C>) * (size_t)tp * P.ntheta * P.nphi * (P.K + 1));
    total = o;
  }
};

template <typename C>
struct P2ASmem {
  size_t coef, twphi, twpsi, pmap, ptile, ohat, ubuf, otile, total;
  __host__ __device__ P2ASmem(const AngPlan& P, int tp) {
    size_t o = 0;
    coef = o;
    o = align16(o + sizeof(C) * P.ntheta * P.np);
    twphi = o;
    o = align16(o + sizeof(Cx<C>) * P.nphi);
    twpsi = o;
    o = align16(o + sizeof(Cx<C>) * P.npsi);
    pmap = o;
    o = align16(o + sizeof(int) * (P.mmax + 1) * P.nphi * (P.K + 1));
    ptile = o;
    o = align16(o + sizeof(Cx<C>) * (size_t)tp * P.np);
    ohat = o;
    o = align16(o + sizeof(Cx<C>) * (size_t)tp * P.ntheta * P.nphi * (P.K + 1));
    ubuf = o;
    o = align16(o + sizeof(Cx<C>) * (size_t)tp * P.ntheta * P.nphi * (P.K + 1));
    otile = o;
    o = align16(o + sizeof(C) * (size_t)tp * P.no);
    total = o;
  }
};

constexpr int kAngThreads = 256;

template <typename S, typename C, bool FROM_XI>
__global__ void __launch_bounds__(kAngThreads)
angl2proj_kernel(const AngPlan P, const S* __restrict__ o, Cx<S>* __restrict__ p,
                 C rho0) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int tp = P.tile_a2p;
  const A2PSmem<C> L(P, tp);
  C* coef = reinterpret_cast<C*>(sm + L.coef);
  Cx<C>* twphi = reinterpret_cast<Cx<C>*>(sm + L.twphi);
  Cx<C>* twpsi = reinterpret_cast<Cx<C>*>(sm + L.twpsi);
  int* ipm = reinterpret_cast<int*>(sm + L.ipm);
  C* ot = reinterpret_cast<C*>(sm + L.otile);
  Cx<C>* Y = reinterpret_cast<Cx<C>*>(sm + L.ybuf);
  Cx<C>* Sf = reinterpret_cast<Cx<C>*>(sm + L.sbuf);

  const int tid = threadIdx.x, bd = blockDim.x;
  const int nt = P.ntheta, nphi = P.nphi, npsi = P.npsi, K1 = P.K + 1;
  const int np = P.np, no = P.no, mmax = P.mmax;
  const long long pt0 = (long long)blockIdx.x * tp;
  const int cnt = (int)min((long long)tp, P.N - pt0);

  for (int i = tid; i < nt * np; i += bd) coef[i] = static_cast<const C*>(P.coef_a2p)[i];
  for (int i = tid; i < nphi; i += bd) twphi[i] = static_cast<const Cx<C>*>(P.tw_phi)[i];
  for (int i = tid; i < npsi; i += bd) twpsi[i] = static_cast<const Cx<C>*>(P.tw_psi)[i];
  for (int i = tid; i < np; i += bd) {
    ipm[i] = P.ip_m[i];
    ipm[np + i] = P.ip_mup[i];
    ipm[2 * np + i] = P.ip_mu2[i];
  }
  // Stage the contiguous tile of o (and fold in get_delta_rho if asked).
  const S* src = o + pt0 * no;
  for (int i = tid; i < cnt * no; i += bd) {
    ot[i] = FROM_XI ? rho0 * to_compute<C>(xi_sq_minus_one(src[i])) : to_compute<C>(src[i]);
  }
  __syncthreads();

  // psi-direction real DFT: Y(pt,theta,iphi,kpsi), kpsi = 0..K.
  const int nrow = cnt * nt * nphi;
  for (int w = tid; w < nrow * K1; w += bd) {
    const int kp = w % K1, row = w / K1;
    const C* x = ot + row * npsi;
    Cx<C> acc = mkc<C>(x[0], C(0));
    for (int j = 1; j < npsi; ++j) {
      Cx<C> t = twpsi[(kp * j) % npsi];
      acc.re += x[j] * t.re;
      acc.im += x[j] * t.im;
    }
    Y[w] = acc;
  }
  __syncthreads();
  // phi-direction complex DFT; S(pt,theta,mup+mmax,kpsi) = conj(o_hat).
  for (int w = tid; w < nrow * K1; w += bd) {
    const int kp = w % K1, t = w / K1;
    const int kf = t % nphi, row2 = t / nphi;
    const Cx<C>* y = Y + (size_t)row2 * nphi * K1 + kp;
    Cx<C> acc = y[0];
    for (int j = 1; j < nphi; ++j) acc = cmac(acc, y[j * K1], twphi[(kf * j) % nphi]);
    const int mup = kf <= mmax ? kf : kf - nphi;
    Sf[((size_t)row2 * nphi + (mup + mmax)) * K1 + kp] = conj(acc);
  }
  __syncthreads();
  // theta contraction; p(ip, pt0 + pt), consecutive threads on consecutive pt.
  for (int w = tid; w < np * cnt; w += bd) {
    const int ip = w / cnt, pt = w % cnt;
    const int mupi = ipm[np + ip] + mmax, mu2 = ipm[2 * np + ip];
    Cx<C> sum = mkc<C>(C(0), C(0));
    for (int it = 0; it < nt; ++it) {
      const Cx<C> s = Sf[(((size_t)pt * nt + it) * nphi + mupi) * K1 + mu2];
      const C c = coef[it * np + ip];
      sum.re += s.re * c;
      sum.im += s.im * c;
    }
    p[(long long)ip * P.N + pt0 + pt] = mkc<S>(to_storage<S>(sum.re), to_storage<S>(sum.im));
  }
}

template <typename S, typename C>
__global__ void __launch_bounds__(kAngThreads)
proj2angl_kernel(const AngPlan P, const Cx<S>* __restrict__ p, S* __restrict__ o) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int tp = P.tile_p2a;
  const P2ASmem<C> L(P, tp);
  C* coef = reinterpret_cast<C*>(sm + L.coef);
  Cx<C>* twphi = reinterpret_cast<Cx<C>*>(sm + L.twphi);
  Cx<C>* twpsi = reinterpret_cast<Cx<C>*>(sm + L.twpsi);
  int* pmap = reinterpret_cast<int*>(sm + L.pmap);
  Cx<C>* Ps = reinterpret_cast<Cx<C>*>(sm + L.ptile);
  Cx<C>* Oh = reinterpret_cast<Cx<C>*>(sm + L.ohat);
  Cx<C>* U = reinterpret_cast<Cx<C>*>(sm + L.ubuf);
  C* ot = reinterpret_cast<C*>(sm + L.otile);

  const int tid = threadIdx.x, bd = blockDim.x;
  const int nt = P.ntheta, nphi = P.nphi, npsi = P.npsi, K1 = P.K + 1;
  const int np = P.np, no = P.no, mmax = P.mmax, mrso = P.mrso;
  const long long pt0 = (long long)blockIdx.x * tp;
  const int cnt = (int)min((long long)tp, P.N - pt0);

  for (int i = tid; i < nt * np; i += bd) coef[i] = static_cast<const C*>(P.coef_p2a)[i];
  for (int i = tid; i < nphi; i += bd) twphi[i] = static_cast<const Cx<C>*>(P.tw_phi)[i];
  for (int i = tid; i < npsi; i += bd) twpsi[i] = static_cast<const Cx<C>*>(P.tw_psi)[i];
  for (int i = tid; i < (mmax + 1) * nphi * K1; i += bd) pmap[i] = P.pmap[i];
  for (int w = tid; w < np * cnt; w += bd) {
    const int ip = w / cnt, pt = w % cnt;
    const Cx<S> v = p[(long long)ip * P.N + pt0 + pt];
    Ps[pt * np + ip] = mkc<C>(to_compute<C>(v.re), to_compute<C>(v.im));
  }
  __syncthreads();

  // Synthesis over m (MDFT_OrientationProjectionTransform.hpp:435-449) and
  // the scatter to FFT order (:454-477): o_hat(kphi) = conj(sum) where
  // kphi = (imup - mmax) mod nphi.
  const int nrow2 = cnt * nt;
  for (int w = tid; w < nrow2 * nphi * K1; w += bd) {
    const int kp = w % K1, t = w / K1;
    const int imup = t % nphi, row2 = t / nphi;
    const int pt = row2 / nt, it = row2 % nt;
    const int a = abs(imup - mmax), b = mrso * kp;
    const int m0 = a > b ? a : b;
    Cx<C> sum = mkc<C>(C(0), C(0));
    for (int m = m0; m <= mmax; ++m) {
      const int ip = pmap[(m * nphi + imup) * K1 + kp];
      const Cx<C> v = Ps[pt * np + ip];
      const C c = coef[it * np + ip];
      sum.re += v.re * c;
      sum.im += v.im * c;
    }
    int kf = imup - mmax;
    if (kf < 0) kf += nphi;
    Oh[((size_t)row2 * nphi + kf) * K1 + kp] = conj(sum);
  }
  __syncthreads();
  // Inverse DFT along phi: U(row2, iphi, kpsi).
  for (int w = tid; w < nrow2 * nphi * K1; w += bd) {
    const int kp = w % K1, t = w / K1;
    const int iphi = t % nphi, row2 = t / nphi;
    const Cx<C>* x = Oh + (size_t)row2 * nphi * K1 + kp;
    Cx<C> acc = x[0];
    for (int j = 1; j < nphi; ++j) acc = cmac(acc, x[j * K1], conj(twphi[(j * iphi) % nphi]));
    U[w] = acc;
  }
  __syncthreads();
  // C2R along psi (npsi odd): o = Re U0 + 2 sum_k Re(U_k e^{+2 pi i k ipsi/npsi}).
  for (int w = tid; w < cnt * no; w += bd) {
    const int ipsi = w % npsi, t = w / npsi;
    const Cx<C>* u = U + (size_t)t * K1;
    C v = u[0].re;
    for (int k = 1; k < K1; ++k) {
      const Cx<C> e = twpsi[(k * ipsi) % npsi];  // exp(-i..): use conj
      v += C(2) * (u[k].re * e.re + u[k].im * e.im);
    }
    ot[w] = v;
  }
  __syncthreads();
  S* dst = o + pt0 * no;
  for (int i = tid; i < cnt * no; i += bd) dst[i] = to_storage<S>(ot[i]);
}

}  // namespace

template <typename S, typename C>
void ang_plan_finish(AngPlan& P) {
  P.fast = ang_fast_supported(P.mmax, P.mrso) ? 1 : 0;
  if (P.fast) ang_fast_setup<S, C>(P);
  const size_t budget = 100 * 1024;
  int tp = 64;
  while (tp > 1 && A2PSmem<C>(P, tp).total > budget) tp /= 2;
  P.tile_a2p = tp;
  P.smem_a2p = A2PSmem<C>(P, tp).total;
  tp = 64;
  while (tp > 1 && P2ASmem<C>(P, tp).total > budget) tp /= 2;
  P.tile_p2a = tp;
  P.smem_p2a = P2ASmem<C>(P, tp).total;
  throw_if(P.smem_a2p > 200 * 1024 || P.smem_p2a > 200 * 1024,
           "angular grid too large for the shared-memory tile", 4);
  allow_max_smem(angl2proj_kernel<S, C, false>, P.smem_a2p, "angl2proj smem attribute");
  allow_max_smem(angl2proj_kernel<S, C, true>, P.smem_a2p, "angl2proj smem attribute");
  allow_max_smem(proj2angl_kernel<S, C>, P.smem_p2a, "proj2angl smem attribute");
}

template <typename S, typename C>
void launch_angl2proj(const AngPlan& P, const S* o, Cx<S>* p, bool from_xi,
                      double rho0, cudaStream_t s) {
  if (P.N == 0) return;
  if constexpr (!std::is_same<C, double>::value) {
    if ((P.tc & 1) && !from_xi) {
      ang_tc_launch<S>(P, 0, o, reinterpret_cast<S*>(p), s);
      return;
    }
  }
  if (P.fast) {
    clear_stale_error();
    ang_fast_a2p<S, C>(P, o, p, from_xi, rho0, s);
    launch_check("angl2proj kernel launch");
    return;
  }
  const long long nb = (P.N + P.tile_a2p - 1) / P.tile_a2p;
  throw_if(nb > 0x7fffffffLL, "grid too large", 4);
  clear_stale_error();
  if (from_xi)
    angl2proj_kernel<S, C, true><<<(unsigned)nb, kAngThreads, P.smem_a2p, s>>>(P, o, p, C(rho0));
  else
    angl2proj_kernel<S, C, false><<<(unsigned)nb, kAngThreads, P.smem_a2p, s>>>(P, o, p, C(rho0));
  launch_check("angl2proj kernel launch");
}

template <typename S, typename C>
void launch_proj2angl(const AngPlan& P, const Cx<S>* p, S* o, cudaStream_t s) {
  if (P.N == 0) return;
  if constexpr (!std::is_same<C, double>::value) {
    if (P.tc & 2) {
      ang_tc_launch<S>(P, 1, reinterpret_cast<const S*>(p), o, s);
      return;
    }
  }
  if (P.fast) {
    clear_stale_error();
    ang_fast_p2a<S, C>(P, p, o, s);
    launch_check("proj2angl kernel launch");
    return;
  }
  const long long nb = (P.N + P.tile_p2a - 1) / P.tile_p2a;
  throw_if(nb > 0x7fffffffLL, "grid too large", 4);
  clear_stale_error();
  proj2angl_kernel<S, C><<<(unsigned)nb, kAngThreads, P.smem_p2a, s>>>(P, p, o);
  launch_check("proj2angl kernel launch");
}

template void ang_plan_finish<double, double>(AngPlan&);
template void ang_plan_finish<float, float>(AngPlan&);
template void ang_plan_finish<double, DF>(AngPlan&);
template void launch_angl2proj<double, double>(const AngPlan&, const double*, Cx<double>*, bool, double,
                                               cudaStream_t);
template void launch_angl2proj<float, float>(const AngPlan&, const float*, Cx<float>*, bool, double,
                                             cudaStream_t);
template void launch_angl2proj<double, DF>(const AngPlan&, const double*, Cx<double>*, bool, double,
                                           cudaStream_t);
template void launch_proj2angl<double, double>(const AngPlan&, const Cx<double>*, double*, cudaStream_t);
template void launch_proj2angl<float, float>(const AngPlan&, const Cx<float>*, float*, cudaStream_t);
template void launch_proj2angl<double, DF>(const AngPlan&, const Cx<double>*, double*, cudaStream_t);

}  // namespace mdft

// oz.cuh -- the k-space step of Convolution::execute
// (common/MDFT_Convolution.hpp:376-543), fused into one kernel.
//
// For each (q, -q) pair of the half-space pair list (:129-176) one warp:
//   1. builds R(q), the rotation matrix between complex spherical harmonics
//      of degree <= mmax, by the l-recursion of
//      common/MDFT_Rotation.hpp:103-283 in FP64 (level 1 by one lane, then
//      the entries of each level l >= 2 spread over the lanes);
//   2. reads the np projections at q and at -q once (:420-425);
//   3. rotates them to the q frame (:427-443);
//   4. forms the OZ product with c(|q|) linearly interpolated between the
//      two bracketing table rows (:449-496); the interpolation is done on the
//      fly because every OZ coefficient is used exactly once per pair;
//   5. chops |gamma| < epsilon to zero (:514-517), rotates back with conj(R)
//      (:518-536) and stores q then -q, conjugating -q at the singular
//      mid-k points (:538-541).
// Pairs are visited sorted by the linear index of q, so neighbouring warps
// touch neighbouring addresses of each projection plane.
#include <cfloat>
#include <type_traits>

#pragma once
#include "common.cuh"

namespace mdft {

// The split lane kernel specialised for mrso = 2 on packed storage (S = C):
// defined in oz_r2.cuh and instantiated in its own translation units.
template <typename C, int MMAX>
void oz_lane_r2_attr(size_t smem);
template <typename C, int MMAX>
void oz_lane_r2_launch(const OzPlan& P, Cx<C>* p, dim3 grid, dim3 block, cudaStream_t s);

namespace {

constexpr int kRotL5 = 5, kRotM13 = 13;  // RotationCoeffs extents (l-2, m+6)

__host__ __device__ constexpr int roff(int l) { return l * (2 * l - 1) * (2 * l + 1) / 3; }
__host__ __device__ constexpr int nrot(int mmax) { return roff(mmax + 1); }
// offset of block l in the half table (entries with m1 >= 0):
// sum_{l' < l} (2l'+1)(l'+1) = l(l+1)(4l-1)/6 (closed forms throughout: a
// recursive constexpr function becomes a real call when an argument is not
// a constant)
__host__ __device__ constexpr int hoff(int l) { return l * (l + 1) * (4 * l - 1) / 6; }

template <typename T>
struct OzSmem {
  size_t R, gq, gmq, dq, dmq, per_warp;
  __host__ __device__ OzSmem(int mmax, int np) {
    size_t o = 0;
    R = o;
    o += sizeof(Cx<double>) * nrot(mmax);
    gq = o;
    o += sizeof(Cx<T>) * np;
    gmq = o;
    o += sizeof(Cx<T>) * np;
    dq = o;
    o += sizeof(Cx<T>) * np;
    dmq = o;
    o += sizeof(Cx<T>) * np;
    per_warp = (o + 15) & ~size_t(15);
  }
};

// prevent_underflow (common/MDFT_Math_Utils.hpp:102-113) with the FP64
// threshold in both forms.  The reference's float instantiation chops at
// FLT_EPSILON (1.2e-7, absolute), which at the field magnitudes of this path
// (|gamma| ~ 1e-4 .. 1e-1) zeroes real signal; the mixed form keeps the FP64
// semantics and only its arithmetic is FP32.
template <typename T>
__device__ __forceinline__ Cx<T> chop(Cx<T> x) {
  const T e = (T)DBL_EPSILON;
  if (fabs(x.re) < e) x.re = T(0);
  if (fabs(x.im) < e) x.im = T(0);
  return x;
}

__device__ __forceinline__ Cx<DF> chop(Cx<DF> x) {
  const float e = 2.220446049250313e-16f;  // DBL_EPSILON = 2^-52, exact in float
  if (df_abs_lt(x.re, e)) x.re = DF(0);
  if (df_abs_lt(x.im, e)) x.im = DF(0);
  return x;
}

template <typename T>
__device__ __forceinline__ Cx<T> to(Cx<double> z) {
  return mkc<T>((T)z.re, (T)z.im);
}

template <typename T>
__global__ void __launch_bounds__(256)
oz_kernel(const OzPlan P, Cx<T>* __restrict__ p) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long pair = (long long)blockIdx.x * P.warps_per_cta + wib;
  if (pair >= P.npairs) return;  // whole warp exits together
  const OzSmem<T> L(P.mmax, P.np);
  unsigned char* base = sm + (size_t)wib * L.per_warp;
  Cx<double>* R = reinterpret_cast<Cx<double>*>(base + L.R);
  Cx<T>* gq = reinterpret_cast<Cx<T>*>(base + L.gq);
  Cx<T>* gmq = reinterpret_cast<Cx<T>*>(base + L.gmq);
  Cx<T>* dq = reinterpret_cast<Cx<T>*>(base + L.dq);
  Cx<T>* dmq = reinterpret_cast<Cx<T>*>(base + L.dmq);

  const int mmax = P.mmax, mrso = P.mrso, K1 = P.K + 1, np = P.np;
  const int nphi = 2 * mmax + 1, n2 = 2 * mmax / mrso + 1;
  const int4 pr = P.pairs[pair];
  const int ix = pr.x, iy = pr.y, iz = pr.z;
  const int ixm = ix == 0 ? 0 : P.nx - ix;
  const int iym = iy == 0 ? 0 : P.ny - iy;
  const int izm = iz == 0 ? 0 : P.nz - iz;
  const double q0 = P.kx[ix], q1 = P.ky[iy], q2 = P.kz[iz];
  const double* A = P.rot;
  const double* B = A + kRotL5 * kRotM13 * kRotM13;
  const double* Cc = B + kRotL5 * kRotM13 * kRotM13;
  const double* D = Cc + kRotL5 * kRotM13;
  constexpr int mm = 6;
#define RI(l, m, m1) (roff(l) + ((m) + (l)) * (2 * (l) + 1) + ((m1) + (l)))
#define AA(l, i, j) A[((l)*kRotM13 + (i)) * kRotM13 + (j)]
#define BB(l, i, j) B[((l)*kRotM13 + (i)) * kRotM13 + (j)]
#define CC(l, i) Cc[(l)*kRotM13 + (i)]
#define DD(l, i) D[(l)*kRotM13 + (i)]

  // ---- 1. R(q) -----------------------------------------------------------
  if (lane == 0) {
    R[0] = mkc<double>(1.0, 0.0);
    double r2[3], r1[3], r0[3];
    if (q0 == 0.0 && q1 == 0.0 && q2 == 0.0) {
      r2[0] = 0.0;
      r2[1] = 0.0;
      r2[2] = 1.0;
    } else {
      r2[0] = q0;
      r2[1] = q1;
      r2[2] = q2;
    }
    if (r2[0] != 0.0 || r2[1] != 0.0) {  // cross((0,0,1), r2)
      r1[0] = 0.0 * r2[2] - 1.0 * r2[1];
      r1[1] = 1.0 * r2[0] - 0.0 * r2[2];
      r1[2] = 0.0 * r2[1] - 0.0 * r2[0];
    } else {  // cross(r2, (1,0,0))
      r1[0] = r2[1] * 0.0 - r2[2] * 0.0;
      r1[1] = r2[2] * 1.0 - r2[0] * 0.0;
      r1[2] = r2[0] * 0.0 - r2[1] * 1.0;
    }
    double n2v = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
    for (int i = 0; i < 3; ++i) r2[i] = r2[i] / n2v;
    double n1v = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
    for (int i = 0; i < 3; ++i) r1[i] = r1[i] / n1v;
    r0[0] = r1[1] * r2[2] - r1[2] * r2[1];
    r0[1] = r1[2] * r2[0] - r1[0] * r2[2];
    r0[2] = r1[0] * r2[1] - r1[1] * r2[0];
    const double is2 = 1.0 / sqrt(2.0);
    R[RI(1, -1, -1)] = mkc<double>((r1[1] + r0[0]) * 0.5, (r0[1] - r1[0]) * 0.5);
    R[RI(1, -1, 0)] = mkc<double>(r2[0] * is2, r2[1] * is2);
    R[RI(1, -1, 1)] = mkc<double>((r1[1] - r0[0]) * 0.5, (-r0[1] - r1[0]) * 0.5);
    R[RI(1, 0, -1)] = mkc<double>(r0[2] * is2, -r1[2] * is2);
    R[RI(1, 0, 0)] = mkc<double>(r2[2], 0.0);
    R[RI(1, 0, 1)] = mkc<double>(-r0[2] * is2, -r1[2] * is2);
    R[RI(1, 1, -1)] = mkc<double>((r1[1] - r0[0]) * 0.5, (r0[1] + r1[0]) * 0.5);
    R[RI(1, 1, 0)] = mkc<double>(-r2[0] * is2, r2[1] * is2);
    R[RI(1, 1, 1)] = mkc<double>((r1[1] + r0[0]) * 0.5, (r1[0] - r0[1]) * 0.5);
  }
  __syncwarp();
  for (int l = 2; l <= mmax; ++l) {
    // entries (m, m1): m in [-l, l], m1 in [m>0 ? 1 : 0, l]
    const int cnt = (2 * l + 1) * (l + 1) - l;  // l rows (m>0) lack m1 = 0
    const Cx<double> R1m0 = R[RI(1, -1, 0)], R1z0 = R[RI(1, 0, 0)], R1p0 = R[RI(1, 1, 0)];
    const Cx<double> R1m1 = R[RI(1, -1, 1)], R1z1 = R[RI(1, 0, 1)], R1p1 = R[RI(1, 1, 1)];
    for (int e = lane; e < cnt; e += 32) {
      // decode: rows m = -l..0 have l+1 entries (m1 = 0..l), rows m = 1..l have l
      int m, m1;
      const int first = (l + 1) * (l + 1);
      if (e < first) {
        m = -l + e / (l + 1);
        m1 = e % (l + 1);
      } else {
        const int e2 = e - first;
        m = 1 + e2 / l;
        m1 = 1 + e2 % l;
      }
      const int l1 = l - 1;
      double f, g;
      if (m1 <= l - 1) {
        if (m == -l) {
          const double bt = BB(l - 2, mm - m, mm + m1);
          const Cx<double> a = R1m0, b = R[RI(l1, m + 1, m1)];
          f = bt * (a.re * b.re - a.im * b.im);
          g = bt * (a.re * b.im + a.im * b.re);
        } else if (m == l) {
          const double bt = BB(l - 2, mm + m, mm + m1);
          const Cx<double> a = R1p0, b = R[RI(l1, m - 1, m1)];
          f = bt * (a.re * b.re - a.im * b.im);
          g = bt * (a.re * b.im + a.im * b.re);
        } else {
          const double at = AA(l - 2, mm + m, mm + m1);
          const double bp = BB(l - 2, mm + m, mm + m1);
          const double bn = BB(l - 2, mm - m, mm + m1);
          const Cx<double> R0 = R1z0, Ra = R1p0, Rb = R1m0;
          const Cx<double> Rm0 = R[RI(l1, m, m1)];
          const Cx<double> Rm1 = (m + 1 <= l1) ? R[RI(l1, m + 1, m1)] : mkc<double>(0, 0);
          const Cx<double> Rm2 = (m - 1 >= -l1) ? R[RI(l1, m - 1, m1)] : mkc<double>(0, 0);
          f = at * (R0.re * Rm0.re) + bp * (Ra.re * Rm2.re - Ra.im * Rm2.im) +
              bn * (Rb.re * Rm1.re - Rb.im * Rm1.im);
          g = at * (R0.re * Rm0.im) + bp * (Ra.re * Rm2.im + Ra.im * Rm2.re) +
              bn * (Rb.re * Rm1.im + Rb.im * Rm1.re);
        }
      } else {  // m1 == l
        if (m == -l) {
          const double dt = DD(l - 2, mm - m);
          const Cx<double> a = R1m1, b = R[RI(l1, m + 1, m1 - 1)];
          f = dt * (a.re * b.re - a.im * b.im);
          g = dt * (a.re * b.im + a.im * b.re);
        } else if (m == l) {
          const double dt = DD(l - 2, mm + m);
          const Cx<double> a = R1p1, b = R[RI(l1, m - 1, m1 - 1)];
          f = dt * (a.re * b.re - a.im * b.im);
          g = dt * (a.re * b.im + a.im * b.re);
        } else {
          const double ct = CC(l - 2, mm + m);
          const double dp = DD(l - 2, mm + m);
          const double dn = DD(l - 2, mm - m);
          const Cx<double> R0 = R1z1, Ra = R1p1, Rb = R1m1;
          const Cx<double> Rm0 = R[RI(l1, m, m1 - 1)];
          const Cx<double> Rm1 = (m + 1 <= l1) ? R[RI(l1, m + 1, m1 - 1)] : mkc<double>(0, 0);
          const Cx<double> Rm2 = (m - 1 >= -l1) ? R[RI(l1, m - 1, m1 - 1)] : mkc<double>(0, 0);
          f = ct * (R0.re * Rm0.re - R0.im * Rm0.im) + dp * (Ra.re * Rm2.re - Ra.im * Rm2.im) +
              dn * (Rb.re * Rm1.re - Rb.im * Rm1.im);
          g = ct * (R0.re * Rm0.im + R0.im * Rm0.re) + dp * (Ra.re * Rm2.im + Ra.im * Rm2.re) +
              dn * (Rb.re * Rm1.im + Rb.im * Rm1.re);
        }
      }
      R[RI(l, m, m1)] = mkc<double>(f, g);
      const double pw = ((m + m1) & 1) ? -1.0 : 1.0;
      R[RI(l, -m, -m1)] = mkc<double>(pw * f, -pw * g);
    }
    __syncwarp();
  }

  // ---- 2. load gamma(q), gamma(-q) ------------------------------------------
  // projection stride; field blockIdx.y of a batched plan starts at y N
  const long long N = P.pstride, f0 = (long long)blockIdx.y * P.N;
  const long long lq = ((long long)ix * P.ny + iy) * P.nz + iz + f0;
  const long long lmq = ((long long)ixm * P.ny + iym) * P.nz + izm + f0;
  for (int ip = lane; ip < np; ip += 32) {
    gq[ip] = p[(long long)ip * N + lq];
    gmq[ip] = p[(long long)ip * N + lmq];
  }
  __syncwarp();
  // ---- 3. rotation to the q frame ---------------------------------------------
  for (int ip = lane; ip < np; ip += 32) {
    const int im = P.ip_m[ip], ikhi = P.ip_mup[ip], imu2 = P.ip_mu2[ip];
    Cx<T> a = mkc<T>(0, 0), b = mkc<T>(0, 0);
    for (int imup = -im; imup <= im; ++imup) {
      const int ipm = P.pmap[(im * nphi + imup + mmax) * K1 + imu2];
      a = cmac(a, gq[ipm], to<T>(R[RI(im, imup, ikhi)]));
      b = cmac(b, gmq[ipm], to<T>(R[RI(im, imup, -ikhi)]));
    }
    dq[ip] = a;
    dmq[ip] = (im & 1) ? mkc<T>(-b.re, -b.im) : b;
  }
  __syncwarp();
  // ---- 4. OZ with interpolated c(|q|) -------------------------------------
  const double qn = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
  const double eiq = qn / P.dq;
  // |q| <= q_max and nq = int(q_max/dq + 0.5) + 2 keep iq + 1 < nq; the
  // clamp only guards the table bounds against rounding at that edge.
  const int iq = min((int)eiq, P.nq - 2);
  const T alpha = (T)(eiq - (double)iq);
  const T beta = T(1) - alpha;
  const Cx<T>* ctab = static_cast<const Cx<T>*>(P.ctab);
  const Cx<T>* clo = ctab + (size_t)iq * P.np_new;
  const Cx<T>* chi = ctab + (size_t)(iq + 1) * P.np_new;
  for (int ip = lane; ip < np; ip += 32) {
    const int ikhi = P.ip_mup[ip];
    Cx<T> sq = mkc<T>(0, 0), smq = mkc<T>(0, 0);
    for (int in = abs(ikhi); in <= mmax; ++in) {
      for (int inu2 = -in / mrso; inu2 <= in / mrso; ++inu2) {
        const int ia = P.ia_map[((size_t)ip * (mmax + 1) + in) * n2 + inu2 + mmax / mrso];
        const Cx<T> h = chi[ia], lo = clo[ia];
        const Cx<T> c = mkc<T>(alpha * h.re + beta * lo.re, alpha * h.im + beta * lo.im);
        if (inu2 < 0) {
          const int ipm = P.pmap[(in * nphi + ikhi + mmax) * K1 + (-inu2)];
          sq = cmac(sq, c, dq[ipm]);
          smq = cmac(smq, c, dmq[ipm]);
        } else {
          const int ipm = P.pmap[(in * nphi + ikhi + mmax) * K1 + inu2];
          sq = cmac(sq, c, conj(dmq[ipm]));
          smq = cmac(smq, c, conj(dq[ipm]));
        }
      }
    }
    gq[ip] = sq;
    gmq[ip] = smq;
  }
  __syncwarp();
  // ---- 5. chop, rotate back, store -----------------------------------------
  const bool qeq = (ixm == ix && iym == iy && izm == iz);
  const bool singular = qeq && (ix == P.nx / 2 || iy == P.ny / 2 || iz == P.nz / 2);
  for (int ip = lane; ip < np; ip += 32) {
    const int im = P.ip_m[ip], imup = P.ip_mup[ip], imu2 = P.ip_mu2[ip];
    Cx<T> a = mkc<T>(0, 0), b = mkc<T>(0, 0);
    for (int ikhi = -im; ikhi <= im; ++ikhi) {
      const int ipm = P.pmap[(im * nphi + ikhi + mmax) * K1 + imu2];
      a = cmac(a, chop(gq[ipm]), conj(to<T>(R[RI(im, imup, ikhi)])));
      b = cmac(b, chop(gmq[ipm]), conj(to<T>(R[RI(im, imup, -ikhi)])));
    }
    if (im & 1) b = mkc<T>(-b.re, -b.im);
    p[(long long)ip * N + lq] = a;
    p[(long long)ip * N + lmq] = singular ? conj(b) : b;
  }
#undef RI
#undef AA
#undef BB
#undef CC
#undef DD
}

// ---------------------------------------------------------------------------
// Lane-per-pair path.
//
// R(q) depends only on the grid, so it is computed once per plan by
// rot_table_kernel (the same FP64 l-recursion, one thread per pair) into a
// resident table laid out (pair block of 32, entry, lane): 32 consecutive
// pairs read each entry as one coalesced 32-wide access.  oz_lane_kernel then
// gives every lane its own pair.  All pairs run the identical instruction
// stream (same mmax, same maps), so no lane idles or diverges; each lane
// keeps its rotated projections in its own column of shared memory
// ([projection][lane], conflict-free), and the OZ output of each (m, mu2)
// block is rotated back from registers and stored straight to HBM.
// ---------------------------------------------------------------------------

// Strided view of one pair's compact R entries.
struct RView {
  Cx<double>* base;
  long long stride;
  __device__ Cx<double>& operator[](int e) const { return base[(long long)e * stride]; }
};

// rotation_matrix_between_complex_spherical_harmonics_lu
// (common/MDFT_Rotation.hpp:103-283), sequential, FP64.
__device__ void rot_recursion(double q0, double q1, double q2, int mmax, const double* A,
                              const double* B, const double* Cc, const double* D, const RView& R) {
  constexpr int mm = 6;
#define RI(l, m, m1) (roff(l) + ((m) + (l)) * (2 * (l) + 1) + ((m1) + (l)))
#define AA(l, i, j) A[((l)*kRotM13 + (i)) * kRotM13 + (j)]
#define BB(l, i, j) B[((l)*kRotM13 + (i)) * kRotM13 + (j)]
#define CC(l, i) Cc[(l)*kRotM13 + (i)]
#define DD(l, i) D[(l)*kRotM13 + (i)]
  R[0] = mkc<double>(1.0, 0.0);
  double r2[3], r1[3], r0[3];
  if (q0 == 0.0 && q1 == 0.0 && q2 == 0.0) {
    r2[0] = 0.0;
    r2[1] = 0.0;
    r2[2] = 1.0;
  } else {
    r2[0] = q0;
    r2[1] = q1;
    r2[2] = q2;
  }
  if (r2[0] != 0.0 || r2[1] != 0.0) {
    r1[0] = 0.0 * r2[2] - 1.0 * r2[1];
    r1[1] = 1.0 * r2[0] - 0.0 * r2[2];
    r1[2] = 0.0 * r2[1] - 0.0 * r2[0];
  } else {
    r1[0] = r2[1] * 0.0 - r2[2] * 0.0;
    r1[1] = r2[2] * 1.0 - r2[0] * 0.0;
    r1[2] = r2[0] * 0.0 - r2[1] * 1.0;
  }
  const double n2v = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
  for (int i = 0; i < 3; ++i) r2[i] = r2[i] / n2v;
  const double n1v = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
  for (int i = 0; i < 3; ++i) r1[i] = r1[i] / n1v;
  r0[0] = r1[1] * r2[2] - r1[2] * r2[1];
  r0[1] = r1[2] * r2[0] - r1[0] * r2[2];
  r0[2] = r1[0] * r2[1] - r1[1] * r2[0];
  const double is2 = 1.0 / sqrt(2.0);
  R[RI(1, -1, -1)] = mkc<double>((r1[1] + r0[0]) * 0.5, (r0[1] - r1[0]) * 0.5);
  R[RI(1, -1, 0)] = mkc<double>(r2[0] * is2, r2[1] * is2);
  R[RI(1, -1, 1)] = mkc<double>((r1[1] - r0[0]) * 0.5, (-r0[1] - r1[0]) * 0.5);
  R[RI(1, 0, -1)] = mkc<double>(r0[2] * is2, -r1[2] * is2);
  R[RI(1, 0, 0)] = mkc<double>(r2[2], 0.0);
  R[RI(1, 0, 1)] = mkc<double>(-r0[2] * is2, -r1[2] * is2);
  R[RI(1, 1, -1)] = mkc<double>((r1[1] - r0[0]) * 0.5, (r0[1] + r1[0]) * 0.5);
  R[RI(1, 1, 0)] = mkc<double>(-r2[0] * is2, r2[1] * is2);
  R[RI(1, 1, 1)] = mkc<double>((r1[1] + r0[0]) * 0.5, (r1[0] - r0[1]) * 0.5);
  const Cx<double> R1m0 = R[RI(1, -1, 0)], R1z0 = R[RI(1, 0, 0)], R1p0 = R[RI(1, 1, 0)];
  const Cx<double> R1m1 = R[RI(1, -1, 1)], R1z1 = R[RI(1, 0, 1)], R1p1 = R[RI(1, 1, 1)];
  for (int l = 2; l <= mmax; ++l) {
    const int l1 = l - 1;
    for (int m = -l; m <= l; ++m) {
      const int m1min = m > 0 ? 1 : 0;
      for (int m1 = m1min; m1 <= l; ++m1) {
        double f, g;
        if (m1 <= l - 1) {
          if (m == -l) {
            const double bt = BB(l - 2, mm - m, mm + m1);
            const Cx<double> a = R1m0, b = R[RI(l1, m + 1, m1)];
            f = bt * (a.re * b.re - a.im * b.im);
            g = bt * (a.re * b.im + a.im * b.re);
          } else if (m == l) {
            const double bt = BB(l - 2, mm + m, mm + m1);
            const Cx<double> a = R1p0, b = R[RI(l1, m - 1, m1)];
            f = bt * (a.re * b.re - a.im * b.im);
            g = bt * (a.re * b.im + a.im * b.re);
          } else {
            const double at = AA(l - 2, mm + m, mm + m1);
            const double bp = BB(l - 2, mm + m, mm + m1);
            const double bn = BB(l - 2, mm - m, mm + m1);
            const Cx<double> Rm0 = R[RI(l1, m, m1)];
            const Cx<double> Rm1 = (m + 1 <= l1) ? R[RI(l1, m + 1, m1)] : mkc<double>(0, 0);
            const Cx<double> Rm2 = (m - 1 >= -l1) ? R[RI(l1, m - 1, m1)] : mkc<double>(0, 0);
            f = at * (R1z0.re * Rm0.re) + bp * (R1p0.re * Rm2.re - R1p0.im * Rm2.im) +
                bn * (R1m0.re * Rm1.re - R1m0.im * Rm1.im);
            g = at * (R1z0.re * Rm0.im) + bp * (R1p0.re * Rm2.im + R1p0.im * Rm2.re) +
                bn * (R1m0.re * Rm1.im + R1m0.im * Rm1.re);
          }
        } else {
          if (m == -l) {
            const double dt = DD(l - 2, mm - m);
            const Cx<double> a = R1m1, b = R[RI(l1, m + 1, m1 - 1)];
            f = dt * (a.re * b.re - a.im * b.im);
            g = dt * (a.re * b.im + a.im * b.re);
          } else if (m == l) {
            const double dt = DD(l - 2, mm + m);
            const Cx<double> a = R1p1, b = R[RI(l1, m - 1, m1 - 1)];
            f = dt * (a.re * b.re - a.im * b.im);
            g = dt * (a.re * b.im + a.im * b.re);
          } else {
            const double ct = CC(l - 2, mm + m);
            const double dp = DD(l - 2, mm + m);
            const double dn = DD(l - 2, mm - m);
            const Cx<double> Rm0 = R[RI(l1, m, m1 - 1)];
            const Cx<double> Rm1 = (m + 1 <= l1) ? R[RI(l1, m + 1, m1 - 1)] : mkc<double>(0, 0);
            const Cx<double> Rm2 = (m - 1 >= -l1) ? R[RI(l1, m - 1, m1 - 1)] : mkc<double>(0, 0);
            f = ct * (R1z1.re * Rm0.re - R1z1.im * Rm0.im) + dp * (R1p1.re * Rm2.re - R1p1.im * Rm2.im) +
                dn * (R1m1.re * Rm1.re - R1m1.im * Rm1.im);
            g = ct * (R1z1.re * Rm0.im + R1z1.im * Rm0.re) + dp * (R1p1.re * Rm2.im + R1p1.im * Rm2.re) +
                dn * (R1m1.re * Rm1.im + R1m1.im * Rm1.re);
          }
        }
        R[RI(l, m, m1)] = mkc<double>(f, g);
        const double pw = ((m + m1) & 1) ? -1.0 : 1.0;
        R[RI(l, -m, -m1)] = mkc<double>(pw * f, -pw * g);
      }
    }
  }
#undef RI
#undef AA
#undef BB
#undef CC
#undef DD
}

// One thread per (padded) pair: R(q) in FP64 straight into the table layout.
__global__ void rot_table_kernel(const OzPlan P, Cx<double>* __restrict__ rt64) {
  const long long pair = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pair >= P.npairs_pad) return;
  double q0 = 0, q1 = 0, q2 = 0;
  if (pair < P.npairs) {
    const int4 pr = P.pairs[pair];
    q0 = P.kx[pr.x];
    q1 = P.ky[pr.y];
    q2 = P.kz[pr.z];
  }
  const double* A = P.rot;
  const double* B = A + kRotL5 * kRotM13 * kRotM13;
  const double* Cc = B + kRotL5 * kRotM13 * kRotM13;
  const double* D = Cc + kRotL5 * kRotM13;
  const long long blk = pair >> 5, lane = pair & 31;
  RView R{rt64 + blk * (long long)P.nR * 32 + lane, 32};
  rot_recursion(q0, q1, q2, P.mmax, A, B, Cc, D, R);
}

// e^{-i phi} of the frame of rot_recursion: r1_y + i r1_x with r1 = z x q
// normalised, (0, sign qz, 0) on the z axis and (0, 1, 0) at q = 0.  In that
// frame R(l, m, m1) = w^m d(l, m, m1) with d real (the Euler factorisation
// R = e^{-i m phi} d(theta); the third angle is zero).
__device__ __forceinline__ Cx<double> frame_phase(double q0, double q1, double q2) {
  double x, y;  // r1 before normalisation
  if (q0 != 0.0 || q1 != 0.0) {
    x = -q1;
    y = q0;
  } else {
    x = 0.0;
    y = q2 == 0.0 ? 1.0 : q2;
  }
  const double n = sqrt(x * x + y * y);
  return mkc<double>(y / n, x / n);
}

// Table of the split lane kernel from the FP64 table, one thread per padded
// pair: per block of 32 pairs the real entries d(l, m, j) = Re(w^-m R(l, m, j)),
// j = 0..l, at hoff(l) + (m + l)(l + 1) + j (the m1 < 0 half follows from
// d(l, -m, -m1) = (-1)^(m+m1) d(l, m, m1)), then w^k, k = 1..mmax, as
// (re, im) at hoff(mmax + 1) + 2 (k - 1); all converted to C.
template <typename C>
__global__ void rot_table_real(const OzPlan P, const Cx<double>* __restrict__ full, C* __restrict__ tab,
                               int nfull) {
  const long long pair = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pair >= P.npairs_pad) return;
  double q0 = 0, q1 = 0, q2 = 0;
  if (pair < P.npairs) {
    const int4 pr = P.pairs[pair];
    q0 = P.kx[pr.x];
    q1 = P.ky[pr.y];
    q2 = P.kz[pr.z];
  }
  const Cx<double> w = frame_phase(q0, q1, q2);
  Cx<double> wp[7];  // w^k, k = 0..mmax (mmax <= 6 on the lane path)
  wp[0] = mkc<double>(1.0, 0.0);
  for (int k = 1; k <= P.mmax; ++k)
    wp[k] = mkc<double>(wp[k - 1].re * w.re - wp[k - 1].im * w.im, wp[k - 1].re * w.im + wp[k - 1].im * w.re);
  const long long blk = pair >> 5;
  const int lane = (int)(pair & 31);
  const Cx<double>* R = full + blk * (long long)nfull * 32 + lane;
  C* T = tab + blk * (long long)P.nR * 32 + lane;
  for (int l = 0; l <= P.mmax; ++l)
    for (int m = -l; m <= l; ++m) {
      const Cx<double> e = m >= 0 ? conj(wp[m]) : wp[-m];  // w^-m
      for (int j = 0; j <= l; ++j) {
        const Cx<double> r = R[(long long)(roff(l) + (m + l) * (2 * l + 1) + (j + l)) * 32];
        T[(long long)(hoff(l) + (m + l) * (l + 1) + j) * 32] = to_compute<C>(r.re * e.re - r.im * e.im);
      }
    }
  const int nh = hoff(P.mmax + 1);
  for (int k = 1; k <= P.mmax; ++k) {
    T[(long long)(nh + 2 * (k - 1)) * 32] = to_compute<C>(wp[k].re);
    T[(long long)(nh + 2 * (k - 1) + 1) * 32] = to_compute<C>(wp[k].im);
  }
}

// Projection index of (m, mup, mu2) in OrientationProjectionMap order
// (m outer, mup, mu2 inner).
struct PIndex {
  int base[8];
  int mrso;
  __device__ __forceinline__ int operator()(int m, int mup, int mu2) const {
    return base[m] + (mup + m) * (m / mrso + 1) + mu2;
  }
};

// coefficient slots of the OZ sum of one projection, terms n' < n:
// sum_{n' < n} (2 (n' / mrso) + 1) = n + mrso q (q - 1) + 2 q (n mod mrso),
// q = n / mrso
__host__ __device__ constexpr int oz_coff(int n, int mrso) {
  return n + mrso * (n / mrso) * (n / mrso - 1) + 2 * (n / mrso) * (n % mrso);
}
// projections of an angular grid: sum_m (2m+1)(m/mrso+1)
__host__ __device__ constexpr int oz_np(int mmax, int mrso) {
  return mmax < 0 ? 0 : oz_np(mmax - 1, mrso) + (2 * mmax + 1) * (mmax / mrso + 1);
}
// warps per CTA of the lane kernels: one warp's shared columns take
// per_warp bytes; the split kernel keeps a CTA near 100 KB so that two share
// an SM, the unsplit one near 200 KB
__host__ __device__ constexpr int lane_warps(size_t per_warp, bool split) {
  return (int)((split ? 100 : 200) * 1024 / per_warp) < 1   ? 1
         : (int)((split ? 100 : 200) * 1024 / per_warp) > 8 ? 8
                                                              : (int)((split ? 100 : 200) * 1024 / per_warp);
}
// threads per CTA the split kernel is compiled for: exact when mrso is a
// compile-time constant, 256 (the most) otherwise
template <typename C, int MMAX, int MRSO>
constexpr int oz_split_threads() {
  return MRSO > 0 ? 32 * lane_warps((size_t)oz_np(MMAX, MRSO) * 32 * sizeof(Cx<C>), true) : 256;
}
// registers per thread that keep two such CTAs on one SM (at most 255):
// the warps spread over the SM's four schedulers, each with a quarter of the
// register file (16384), so the busiest scheduler holds ceil(2 W / 4) warps
template <typename C, int MMAX, int MRSO>
constexpr int oz_split_regs() {
  return 16384 / (32 * ((2 * (oz_split_threads<C, MMAX, MRSO>() / 32) + 3) / 4)) / 8 * 8 > 255
             ? 255
             : 16384 / (32 * ((2 * (oz_split_threads<C, MMAX, MRSO>() / 32) + 3) / 4)) / 8 * 8;
}

// Loops over the rows of one rotation block: fully unrolled for FP32 up to
// mmax 3, where one iteration holds little arithmetic and unrolling lets the
// loads of later rows overlap the current one (larger blocks would spill);
// rolled for double-float, whose arithmetic per row already covers the load
// latency and whose unrolled code would crowd the instruction cache.
template <typename C, int MMAX>
constexpr int kOzUnroll = (sizeof(C) == 4 && MMAX <= 3) ? 2 * MMAX + 1 : 1;

// MRSO > 0: the molecule's rotational symmetry order fixed at compile time
// (every loop over nu unrolled, so the c(|q|) loads of a projection can be
// issued together); MRSO = 0: read from the plan.
template <typename S, typename C, int MMAX, int MRSO>
__global__ void __maxnreg__((oz_split_regs<C, MMAX, MRSO>()))
oz_lane_kernel(const OzPlan P, Cx<S>* __restrict__ p) {
  extern __shared__ __align__(16) unsigned char sm[];
  // Two lanes per pair: lane i (< 16) carries the q side of pair i of the
  // warp's 16, lane i + 16 its -q side.  Each lane keeps its rotated
  // projections in its own shared column; the OZ product reads the partner's
  // column for the conjugated terms.
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int side = lane >> 4;
  // c(|q|) rows of the CTA's pairs: the list is sorted by |q|, so the CTA's
  // pairs use a short run of consecutive rows from the row of its first
  // pair; up to P.crow_stage of them are copied to shared memory by all
  // threads (before any warp leaves), later rows are read from global memory
  int r0 = 0, nst = 0;
  Cx<C>* cst = nullptr;
  if (P.crow_stage > 0) {
    const long long first = (long long)blockIdx.x * P.warps_per_cta * 16;
    const long long last = min(first + (long long)P.warps_per_cta * 16, (long long)P.npairs) - 1;
    r0 = P.pinfo[first].z;
    nst = min(P.crow_stage, P.pinfo[last].z - r0 + 1);
    cst = reinterpret_cast<Cx<C>*>(sm + P.cstage_off);
    const Cx<C>* src = static_cast<const Cx<C>*>(P.ceff) + (size_t)r0 * P.np_new;
    const int cnt = nst * P.np_new;
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) cst[i] = src[i];
    __syncthreads();
  }
  const long long grp = (long long)blockIdx.x * P.warps_per_cta + wib;
  if (grp * 16 >= P.npairs) return;  // whole warp exits together
  const long long pair = grp * 16 + (lane & 15);
  const bool valid = pair < P.npairs;
  const int np = P.np;
  const int mrso = MRSO > 0 ? MRSO : P.mrso;
  Cx<C>* D = reinterpret_cast<Cx<C>*>(sm + (size_t)wib * np * 32 * sizeof(Cx<C>));
  PIndex ipx;
  ipx.mrso = mrso;
  {
    int b = 0;
#pragma unroll
    for (int m = 0; m <= MMAX; ++m) {
      ipx.base[m] = b;
      b += (2 * m + 1) * (m / mrso + 1);
    }
  }
  const int4 info = P.pinfo[pair];
  // projection stride; field blockIdx.y of a batched plan starts at y N
  const long long N = P.pstride;
  const long long lown = (side ? info.y : info.x) + (long long)blockIdx.y * P.N;
  // the q side does not store at self-paired k-points: the -q store wins
  const bool store = valid && (side == 1 || info.x != info.y);
  // R(l, m, m1) = w^m d(l, m, m1) with w = e^{-i phi} and d real; the table
  // holds Rh(l, m, j) = d(l, m, j) for j >= 0 (for m1 < 0, d(l, m, m1) =
  // (-1)^(m+m1) Rh(l, -m, -m1)) and the powers WPOW(k) = w^k.  Both lanes of a
  // pair read the same entries, so every load serves the two half-warps.
  const C* Rt = static_cast<const C*>(P.rtab) + (pair >> 5) * (long long)P.nR * 32 + (pair & 31);
#define RH(l, m, j) Rt[(hoff(l) + ((m) + (l)) * ((l) + 1) + (j)) * 32]
#define WPOW(k) mkc<C>(Rt[(hoff(MMAX + 1) + 2 * ((k)-1)) * 32], Rt[(hoff(MMAX + 1) + 2 * ((k)-1) + 1) * 32])

  // rotation to the q frame (MDFT_Convolution.hpp:427-443), block by block:
  // D(m, k) = sum_a g_a R(m, a - m, ks k) = sum_a (g_a w^(a-m)) d(m, a - m, ks k)
  // with ks = +1 on the q side and -1 on the -q side.  For j = |k| > 0 one
  // side needs column +j (direct) and the other column -j (mirrored), both
  // from the row Rh(m, ., j).
#pragma unroll
  for (int m = 0; m <= MMAX; ++m) {
    const bool flip = side && (m & 1);  // (-1)^m of R(-q) = (-1)^l R(q)
#pragma unroll 1
    for (int mu2 = 0; mu2 <= m / mrso; ++mu2) {
      Cx<C> g[2 * MMAX + 1];
#pragma unroll
      for (int a = 0; a <= 2 * m; ++a) {
        const Cx<S> u = p[(long long)ipx(m, a - m, mu2) * N + lown];
        g[a] = mkc<C>(to_compute<C>(u.re), to_compute<C>(u.im));
      }
#pragma unroll
      for (int t = 1; t <= m; ++t) {
        const Cx<C> wt = WPOW(t);
        g[m + t] = cx_mul(g[m + t], wt);
        g[m - t] = cx_mul(g[m - t], conj(wt));
      }
      {  // k = 0: column 0 on both sides
        CAcc<C> x;
        cacc_zero(x);
#pragma unroll
        for (int b = 0; b <= 2 * m; ++b) cacc_mac_r(x, g[b], RH(m, b - m, 0));
        Cx<C> v = cacc_get(x);
        if (flip) v = mkc<C>(-v.re, -v.im);
        D[ipx(m, 0, mu2) * 32 + lane] = v;
      }
#pragma unroll(kOzUnroll<C, MMAX>)
      for (int j = 1; j <= m; ++j) {
        // direct: sum_b g_b h_b; mirrored: sum_b (-1)^(m+b+j) g_{2m-b} h_b
        CAcc<C> xd, xm;
        cacc_zero(xd);
        cacc_zero(xm);
#pragma unroll
        for (int b = 0; b <= 2 * m; ++b) {
          const C h = RH(m, b - m, j);
          cacc_mac_r(xd, g[b], h);
          cacc_mac_r(xm, g[2 * m - b], ((m + b) & 1) ? -h : h);
        }
        Cx<C> vd = cacc_get(xd), vm = cacc_get(xm);
        if (j & 1) vm = mkc<C>(-vm.re, -vm.im);
        // q side: k = +j direct, k = -j mirrored; -q side the other way round
        Cx<C> kp = side ? vm : vd, kn = side ? vd : vm;
        if (flip) {
          kp = mkc<C>(-kp.re, -kp.im);
          kn = mkc<C>(-kn.re, -kn.im);
        }
        D[ipx(m, j, mu2) * 32 + lane] = kp;
        D[ipx(m, -j, mu2) * 32 + lane] = kn;
      }
    }
  }
  __syncwarp();
  // OZ with c(|q|) interpolated on the fly (:449-496), chop (:514-517),
  // rotation back (:518-536) and the stores (:538-541)
  const int iq = info.z;
  const bool singular = info.w != 0;
  const C alpha = static_cast<const C*>(P.palpha)[pair];
  const C beta = C(1) - alpha;
  const bool pre = P.ceff != nullptr;
  const int slot = iq - r0;  // staged row of this pair (padding pairs may fall outside)
  const Cx<C>* clo = (slot >= 0 && slot < nst)
                         ? cst + (size_t)slot * P.np_new
                         : static_cast<const Cx<C>*>(pre ? P.ceff : P.ctab) + (size_t)iq * P.np_new;
  const Cx<C>* chi = clo + P.np_new;
  const int other = lane ^ 16;
  // c(|q|) of coefficient ia, and term (n, nu2) of the OZ sum of projection
  // (m, k, mu2): c times the own column at -nu2 (nu2 < 0) or the partner's,
  // conjugated, at nu2
#define OZ_COEF(ia)                                                                        \
  (pre ? clo[ia]                                                                           \
       : mkc<C>(alpha * chi[ia].re + beta * clo[ia].re, alpha * chi[ia].im + beta * clo[ia].im))
#define OZ_TERM(s, c, n, k, nu2)                         \
  do {                                                   \
    if ((nu2) < 0)                                       \
      cacc_mac(s, c, D[ipx(n, k, -(nu2)) * 32 + lane]);  \
    else                                                 \
      cacc_macc(s, c, D[ipx(n, k, (nu2)) * 32 + other]); \
  } while (0)
#pragma unroll
  for (int m = 0; m <= MMAX; ++m) {
    const bool flip = side && (m & 1);
#pragma unroll 1
    for (int mu2 = 0; mu2 <= m / mrso; ++mu2) {
      // rotation back as the OZ outputs appear: conj R(m, a', kk) =
      // w^-a' d(m, a', kk), so acc_a += g_k d(m, a', ks k) and out_a = w^-a' acc_a
      CAcc<C> acc[2 * MMAX + 1];
#pragma unroll
      for (int a = 0; a <= 2 * m; ++a) cacc_zero(acc[a]);
#pragma unroll(kOzUnroll<C, MMAX>)
      for (int k = -m; k <= m; ++k) {
        const int ak = k < 0 ? -k : k;
        CAcc<C> sacc;
        cacc_zero(sacc);
        const int ia_k = P.ia_start[ipx(m, k, mu2)];
        if constexpr (MRSO > 0) {
          // slot t of term (n, u) at ia0 + t; every loop below unrolls
          const int ia0 = ia_k - oz_coff(ak, MRSO);
#pragma unroll
          for (int n = 0; n <= MMAX; ++n) {
            if (n < ak) continue;
            const int nn = n / MRSO;
#pragma unroll
            for (int u = 0; u <= 2 * nn; ++u) {
              const Cx<C> c = OZ_COEF(ia0 + oz_coff(n, MRSO) + u);
              OZ_TERM(sacc, c, n, k, u - nn);
            }
          }
        } else {
          int ia = ia_k;
#pragma unroll
          for (int n = 0; n <= MMAX; ++n) {
            if (n < ak) continue;
            const int nn = n / mrso;
            for (int nu2 = -nn; nu2 <= nn; ++nu2, ++ia) {
              const Cx<C> c = OZ_COEF(ia);
              OZ_TERM(sacc, c, n, k, nu2);
            }
          }
        }
        const Cx<C> gk = chop(cacc_get(sacc));
        // d(m, a', kk), kk = ks k: Rh(m, a', |k|) when kk >= 0, else
        // (-1)^(a'+k) Rh(m, -a', |k|); the row Rh(m, ., |k|) serves both sides
        const bool direct = side ? (k <= 0) : (k >= 0);
        const bool kodd = (k & 1) != 0;
        C h[2 * MMAX + 1];
#pragma unroll
        for (int b = 0; b <= 2 * m; ++b) h[b] = RH(m, b - m, ak);
#pragma unroll
        for (int a = 0; a <= 2 * m; ++a) {
          const C hm = h[2 * m - a];
          const bool neg = (((a - m) & 1) != 0) != kodd;
          cacc_mac_r(acc[a], gk, direct ? h[a] : (neg ? -hm : hm));
        }
      }
#pragma unroll
      for (int a = 0; a <= 2 * m; ++a) {
        Cx<C> v = cacc_get(acc[a]);
        if (a > m) v = cx_mul(v, conj(WPOW(a - m)));
        if (a < m) v = cx_mul(v, WPOW(m - a));
        if (flip) v = mkc<C>(-v.re, -v.im);
        if (side && singular) v = conj(v);
        if (store) p[(long long)ipx(m, a - m, mu2) * N + lown] = mkc<S>(to_storage<S>(v.re), to_storage<S>(v.im));
      }
    }
  }
#undef OZ_COEF
#undef OZ_TERM
#undef RH
#undef WPOW
}

// One lane per pair (both sides in one thread): used for FP64 arithmetic,
// where the FP64 pipe, not latency, bounds the kernel and splitting the pair
// would repeat the interpolation of c(|q|) on both lanes.
template <typename S, typename C, int MMAX>
__global__ void __launch_bounds__(256)
oz_lane1_kernel(const OzPlan P, Cx<S>* __restrict__ p) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long blk = (long long)blockIdx.x * P.warps_per_cta + wib;
  if (blk * 32 >= P.npairs) return;  // whole warp exits together
  const long long pair = blk * 32 + lane;
  const bool valid = pair < P.npairs;
  const int np = P.np, mrso = P.mrso;
  Cx<C>* Dq = reinterpret_cast<Cx<C>*>(sm + (size_t)wib * 2 * np * 32 * sizeof(Cx<C>));
  Cx<C>* Dmq = Dq + (size_t)np * 32;
  PIndex ipx;
  ipx.mrso = mrso;
  {
    int b = 0;
#pragma unroll
    for (int m = 0; m <= MMAX; ++m) {
      ipx.base[m] = b;
      b += (2 * m + 1) * (m / mrso + 1);
    }
  }
  const int4 info = P.pinfo[pair];
  // projection stride; field blockIdx.y of a batched plan starts at y N
  const long long N = P.pstride, lq = info.x + (long long)blockIdx.y * P.N,
                  lmq = info.y + (long long)blockIdx.y * P.N;
  const Cx<C>* Rt = static_cast<const Cx<C>*>(P.rtab) + blk * (long long)P.nR * 32 + lane;
#define RT(l, m, m1) Rt[(roff(l) + ((m) + (l)) * (2 * (l) + 1) + ((m1) + (l))) * 32]

  // rotation to the q frame (MDFT_Convolution.hpp:427-443), block by block
#pragma unroll
  for (int m = 0; m <= MMAX; ++m) {
    for (int mu2 = 0; mu2 <= m / mrso; ++mu2) {
      Cx<C> gq[2 * MMAX + 1], gmq[2 * MMAX + 1];
#pragma unroll
      for (int a = 0; a <= 2 * m; ++a) {
        const long long off = (long long)ipx(m, a - m, mu2) * N;
        const Cx<S> u = p[off + lq], v = p[off + lmq];
        gq[a] = mkc<C>(to_compute<C>(u.re), to_compute<C>(u.im));
        gmq[a] = mkc<C>(to_compute<C>(v.re), to_compute<C>(v.im));
      }
#pragma unroll 1
      for (int k = -m; k <= m; ++k) {
        Cx<C> x = mkc<C>(C(0), C(0)), y = mkc<C>(C(0), C(0));
#pragma unroll
        for (int a = 0; a <= 2 * m; ++a) {
          x = cmac(x, gq[a], RT(m, a - m, k));
          y = cmac(y, gmq[a], RT(m, a - m, -k));
        }
        const int j = ipx(m, k, mu2) * 32 + lane;
        Dq[j] = x;
        Dmq[j] = (m & 1) ? mkc<C>(-y.re, -y.im) : y;
      }
    }
  }
  // OZ with c(|q|) interpolated on the fly (:449-496), chop (:514-517),
  // rotation back (:518-536) and the stores (:538-541)
  const int iq = info.z;
  const bool singular = info.w != 0;
  const C alpha = static_cast<const C*>(P.palpha)[pair];
  const C beta = C(1) - alpha;
  const bool pre = P.ceff != nullptr;
  const Cx<C>* clo = static_cast<const Cx<C>*>(pre ? P.ceff : P.ctab) + (size_t)iq * P.np_new;
  const Cx<C>* chi = clo + P.np_new;
#pragma unroll
  for (int m = 0; m <= MMAX; ++m) {
    for (int mu2 = 0; mu2 <= m / mrso; ++mu2) {
      Cx<C> gq[2 * MMAX + 1], gmq[2 * MMAX + 1];
#pragma unroll
      for (int k = -m; k <= m; ++k) {
        int ia = P.ia_start[ipx(m, k, mu2)];
        Cx<C> sq = mkc<C>(C(0), C(0)), smq = mkc<C>(C(0), C(0));
#pragma unroll
        for (int n = (k < 0 ? -k : k); n <= MMAX; ++n) {
          const int nn = n / mrso;
          for (int nu2 = -nn; nu2 <= nn; ++nu2, ++ia) {
            Cx<C> c;
            if (pre) {
              c = clo[ia];
            } else {
              const Cx<C> h = chi[ia], lo = clo[ia];
              c = mkc<C>(alpha * h.re + beta * lo.re, alpha * h.im + beta * lo.im);
            }
            if (nu2 < 0) {
              const int j = ipx(n, k, -nu2) * 32 + lane;
              sq = cmac(sq, c, Dq[j]);
              smq = cmac(smq, c, Dmq[j]);
            } else {
              const int j = ipx(n, k, nu2) * 32 + lane;
              sq = cmac(sq, c, conj(Dmq[j]));
              smq = cmac(smq, c, conj(Dq[j]));
            }
          }
        }
        gq[k + m] = chop(sq);
        gmq[k + m] = chop(smq);
      }
#pragma unroll 1
      for (int a = -m; a <= m; ++a) {
        Cx<C> x = mkc<C>(C(0), C(0)), y = mkc<C>(C(0), C(0));
#pragma unroll
        for (int k = -m; k <= m; ++k) {
          x = cmac(x, gq[k + m], conj(RT(m, a, k)));
          y = cmac(y, gmq[k + m], conj(RT(m, a, -k)));
        }
        if (m & 1) y = mkc<C>(-y.re, -y.im);
        if (valid) {
          const long long off = (long long)ipx(m, a, mu2) * N;
          const Cx<C> yy = singular ? conj(y) : y;
          p[off + lq] = mkc<S>(to_storage<S>(x.re), to_storage<S>(x.im));
          p[off + lmq] = mkc<S>(to_storage<S>(yy.re), to_storage<S>(yy.im));
        }
      }
    }
  }
#undef RT
}


// ---------------------------------------------------------------------------
// Warp-per-pair path for large angular grids (split forms, np >=
// oz_warp_min_np).
//
// The lane kernel keeps every lane's np rotated projections in its own
// shared column, np x 16 bytes per thread in double-float: at mmax 5 (np 88)
// an SM then holds 4 warps (double-float) or 8 (FP32).  Here one warp owns
// one (q, -q) pair and spreads its projections over the lanes, so the
// shared state is per warp (the pair's inputs, rotated projections and
// R(q) entries, ~7 KB in double-float at mmax 5) and an SM holds 32 warps.
// Each output is the same sum, in the same order, as in the lane kernel:
// lane t takes projections t, t + 32, ... of both sides in every stage,
// sharing the R(q) entries (rotations) and the c(|q|) coefficients (OZ)
// between the two sides.
// ---------------------------------------------------------------------------
template <typename C>
__host__ __device__ constexpr size_t warp_pair_smem(int np, int nR) {
  return ((size_t)4 * np * sizeof(Cx<C>) + (size_t)nR * sizeof(C) + 15) & ~size_t(15);
}

template <typename S, typename C, int MMAX>
__global__ void __launch_bounds__(256)
oz_warp_kernel(const OzPlan P, Cx<S>* __restrict__ p) {
  extern __shared__ __align__(16) unsigned char sm[];
  // the OZ stage's order of the projections: by |k| from MMAX down, so that
  // the lanes of one round have sums of similar length
  __shared__ short oz_order[256];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int np = P.np, mrso = P.mrso;
  for (int ip = threadIdx.x; ip < np; ip += blockDim.x) {  // rank of ip in that order
    const int a = abs(__ldg(P.ip_mup + ip));
    int r = 0;
    for (int q = 0; q < np; ++q) {
      const int b = abs(__ldg(P.ip_mup + q));
      r += (b > a || (b == a && q < ip)) ? 1 : 0;
    }
    oz_order[r] = (short)ip;
  }
  __syncthreads();
  const long long pair = (long long)blockIdx.x * P.warps_per_cta + wib;
  if (pair >= P.npairs) return;  // whole warp exits together
  unsigned char* base = sm + (size_t)wib * warp_pair_smem<C>(np, P.nR);
  Cx<C>* G0 = reinterpret_cast<Cx<C>*>(base);  // q side: inputs, then OZ outputs
  Cx<C>* G1 = G0 + np;                          // -q side
  Cx<C>* D0 = G1 + np;                          // rotated to the q frame
  Cx<C>* D1 = D0 + np;
  C* rt = reinterpret_cast<C*>(D1 + np);  // the pair's R(q) entries
  // projection index arithmetic in registers (no per-thread array that a
  // runtime m would index through local memory): byte m of bpack is the
  // first projection of degree m (< 256 for mmax <= 6), nibble m of wpack
  // the count m / mrso + 1 of its mu2 values
  unsigned long long bpack = 0, wpack = 0;
  {
    int b = 0;
#pragma unroll
    for (int m = 0; m <= MMAX; ++m) {
      bpack |= (unsigned long long)b << (8 * m);
      wpack |= (unsigned long long)(m / mrso + 1) << (4 * m);
      b += (2 * m + 1) * (m / mrso + 1);
    }
  }
  auto pbase = [&](int m) { return (int)((bpack >> (8 * m)) & 0xffu); };
  auto pw = [&](int m) { return (int)((wpack >> (4 * m)) & 0xfu); };
  auto ipx = [&](int m, int mup, int mu2) { return pbase(m) + (mup + m) * pw(m) + mu2; };
  // (m, mup, mu2) of projection ip
  auto decode = [&](int ip, int& m, int& mup, int& mu2) {
    m = 0;
#pragma unroll
    for (int l = 1; l <= MMAX; ++l)
      if (ip >= pbase(l)) m = l;
    const int w = pw(m), r = ip - pbase(m);
    mup = r / w - m;
    mu2 = r - (r / w) * w;
  };
  const int4 info = P.pinfo[pair];
  const long long N = P.pstride;
  const long long lq = info.x + (long long)blockIdx.y * P.N, lmq = info.y + (long long)blockIdx.y * P.N;
  {
    const C* Rt = static_cast<const C*>(P.rtab) + (pair >> 5) * (long long)P.nR * 32 + (pair & 31);
    for (int e = lane; e < P.nR; e += 32) rt[e] = Rt[(long long)e * 32];
  }
#define RH(l, m, j) rt[hoff(l) + ((m) + (l)) * ((l) + 1) + (j)]
#define WPOW(k) mkc<C>(rt[hoff(MMAX + 1) + 2 * ((k)-1)], rt[hoff(MMAX + 1) + 2 * ((k)-1) + 1])
  __syncwarp();
  // inputs of both sides, times w^(a - m) as the lane kernel applies it
  for (int ip = lane; ip < np; ip += 32) {
    int m, mup, mu2;
    decode(ip, m, mup, mu2);
    const Cx<S> u = p[(long long)ip * N + lq], v = p[(long long)ip * N + lmq];
    Cx<C> a = mkc<C>(to_compute<C>(u.re), to_compute<C>(u.im));
    Cx<C> b = mkc<C>(to_compute<C>(v.re), to_compute<C>(v.im));
    if (mup != 0) {
      const int t = mup > 0 ? mup : -mup;
      const Cx<C> wt = mup > 0 ? WPOW(t) : conj(WPOW(t));
      a = cx_mul(a, wt);
      b = cx_mul(b, wt);
    }
    G0[ip] = a;
    G1[ip] = b;
  }
  __syncwarp();
  // rotation to the q frame (MDFT_Convolution.hpp:427-443)
  for (int ip = lane; ip < np; ip += 32) {
    int m, k, mu2;
    decode(ip, m, k, mu2);
    const int j = k < 0 ? -k : k;
    const int b0 = ipx(m, -m, mu2), bs = pw(m);  // g_b at b0 + b bs
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const Cx<C>* g = s ? G1 : G0;
      const bool direct = k == 0 || (s == 0 ? k > 0 : k < 0);
      CAcc<C> x;
      cacc_zero(x);
      // direct: sum_b g_b h_b; mirrored: sum_b (-1)^(m+b) g_{2m-b} h_b (selects,
      // not branches: neighbouring lanes take either)
      for (int b = 0; b <= 2 * m; ++b) {
        const C h = RH(m, b - m, j);
        const int bb = direct ? b : 2 * m - b;
        cacc_mac_r(x, g[b0 + bb * bs], (!direct && ((m + b) & 1)) ? -h : h);
      }
      Cx<C> v = cacc_get(x);
      if (!direct && (j & 1)) v = mkc<C>(-v.re, -v.im);
      if (s == 1 && (m & 1)) v = mkc<C>(-v.re, -v.im);
      (s ? D1 : D0)[ip] = v;
    }
  }
  __syncwarp();
  // OZ with c(|q|) (:449-496) and the chop (:514-517); outputs over G
  const bool singular = info.w != 0;
  const C alpha = static_cast<const C*>(P.palpha)[pair];
  const C beta = C(1) - alpha;
  const bool pre = P.ceff != nullptr;
  const Cx<C>* clo = static_cast<const Cx<C>*>(pre ? P.ceff : P.ctab) + (size_t)info.z * P.np_new;
  const Cx<C>* chi = clo + P.np_new;
  for (int r = lane; r < np; r += 32) {
    const int ip = oz_order[r];
    int m, k, mu2;
    decode(ip, m, k, mu2);
    const int ak = k < 0 ? -k : k;
    CAcc<C> s0, s1;
    cacc_zero(s0);
    cacc_zero(s1);
    int ia = P.ia_start[ip];
    for (int n = ak; n <= MMAX; ++n) {
      const int nn = pw(n) - 1;
      for (int u = 0; u <= 2 * nn; ++u, ++ia) {
        const Cx<C> c = pre ? clo[ia]
                            : mkc<C>(alpha * chi[ia].re + beta * clo[ia].re, alpha * chi[ia].im + beta * clo[ia].im);
        // nu2 < 0: own column at -nu2; nu2 >= 0: the other side's at nu2,
        // conjugated (c conj(D) = the same products as cacc_macc)
        const int nu2 = u - nn;
        const bool own = nu2 < 0;
        const int jj = ipx(n, k, own ? -nu2 : nu2);
        const Cx<C> d0 = own ? D0[jj] : conj(D1[jj]), d1 = own ? D1[jj] : conj(D0[jj]);
        cacc_mac(s0, c, d0);
        cacc_mac(s1, c, d1);
      }
    }
    G0[ip] = chop(cacc_get(s0));
    G1[ip] = chop(cacc_get(s1));
  }
  __syncwarp();
  // rotation back with conj R (:518-536) and the stores (:538-541): the -q
  // store wins at self-paired points, -q conjugated at singular mid-k points
  const bool store0 = info.x != info.y;
  for (int ip = lane; ip < np; ip += 32) {
    int m, a, mu2;
    decode(ip, m, a, mu2);
    a += m;  // 0 .. 2m
    const int k0 = ipx(m, -m, mu2), ks = pw(m);  // G(m, k) at k0 + (k + m) ks
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const Cx<C>* g = s ? G1 : G0;
      CAcc<C> acc;
      cacc_zero(acc);
      for (int k = -m; k <= m; ++k) {
        const int ak = k < 0 ? -k : k;
        const bool direct = s ? (k <= 0) : (k >= 0);
        const bool neg = (((a - m) & 1) != 0) != ((k & 1) != 0);
        const C hd = RH(m, a - m, ak), hm = RH(m, m - a, ak);
        cacc_mac_r(acc, g[k0 + (k + m) * ks], direct ? hd : (neg ? -hm : hm));
      }
      Cx<C> v = cacc_get(acc);
      if (a > m) v = cx_mul(v, conj(WPOW(a - m)));
      if (a < m) v = cx_mul(v, WPOW(m - a));
      if (s == 1 && (m & 1)) v = mkc<C>(-v.re, -v.im);
      if (s == 1 && singular) v = conj(v);
      if (s == 1 || store0) p[(long long)ip * N + (s ? lmq : lq)] = mkc<S>(to_storage<S>(v.re), to_storage<S>(v.im));
    }
  }
#undef RH
#undef WPOW
}

constexpr int kLaneMaxMmax = 6;

template <typename C>
constexpr bool split_pairs() {
  return !std::is_same<C, double>::value;
}

template <typename C>
size_t lane_smem_per_warp(int np) {
  // split: 16 pairs x 2 sides per warp; unsplit: 32 pairs x (q, -q)
  return (size_t)np * 32 * sizeof(Cx<C>) * (split_pairs<C>() ? 1 : 2);
}

// Shared-memory attribute and launch of the lane kernel for one mmax: the
// split kernel specialised for mrso = 2 (packed storage) comes from its own
// translation unit, every other case from the generic instantiations here.
template <typename S, typename C, int K>
void lane_attr_one(const OzPlan& P) {
  if constexpr (split_pairs<C>()) {
    if (P.warp_pairs) {
      allow_max_smem(oz_warp_kernel<S, C, K>, P.smem, "oz smem attribute");
      return;
    }
    if constexpr (std::is_same<S, C>::value) {
      if (P.mrso == 2) {
        oz_lane_r2_attr<C, K>(P.smem);
        return;
      }
    }
    allow_max_smem(oz_lane_kernel<S, C, K, 0>, P.smem, "oz smem attribute");
  } else {
    allow_max_smem(oz_lane1_kernel<S, C, K>, P.smem, "oz smem attribute");
  }
}

template <typename S, typename C>
void lane_attr_all(const OzPlan& P) {
  switch (P.mmax) {
    case 1: lane_attr_one<S, C, 1>(P); break;
    case 2: lane_attr_one<S, C, 2>(P); break;
    case 3: lane_attr_one<S, C, 3>(P); break;
    case 4: lane_attr_one<S, C, 4>(P); break;
    case 5: lane_attr_one<S, C, 5>(P); break;
    case 6: lane_attr_one<S, C, 6>(P); break;
  }
}

template <typename S, typename C, int K>
void lane_launch_one(const OzPlan& P, Cx<S>* p, dim3 grid, dim3 block, cudaStream_t s) {
  if constexpr (split_pairs<C>()) {
    if (P.warp_pairs) {
      oz_warp_kernel<S, C, K><<<grid, block, P.smem, s>>>(P, p);
      return;
    }
    if constexpr (std::is_same<S, C>::value) {
      if (P.mrso == 2) {
        oz_lane_r2_launch<C, K>(P, p, grid, block, s);
        return;
      }
    }
    oz_lane_kernel<S, C, K, 0><<<grid, block, P.smem, s>>>(P, p);
  } else {
    oz_lane1_kernel<S, C, K><<<grid, block, P.smem, s>>>(P, p);
  }
}

}  // namespace

template <typename S, typename C>
void oz_plan_finish(OzPlan& P) {
  // Lane path when one warp's shared columns fit with room for a few warps
  // per SM; otherwise the warp-per-pair kernel (R computed on the fly).
  const size_t per_warp = lane_smem_per_warp<C>(P.np);
  P.warp_pairs = 0;
  if (split_pairs<C>() && P.np >= oz_warp_min_np<C>() && P.mmax <= kLaneMaxMmax && P.N < (1LL << 31)) {
    // the lane kernel's per-thread columns would leave few warps per SM:
    // one warp per pair, 8 pairs per CTA, over the same tables
    P.lane_path = 1;
    P.warp_pairs = 1;
    P.warps_per_cta = 8;
    P.smem = warp_pair_smem<C>(P.np, hoff(P.mmax + 1) + 2 * P.mmax) * P.warps_per_cta;
    lane_attr_all<S, C>(P);
    return;
  }
  P.lane_path = (P.mmax <= kLaneMaxMmax && per_warp <= 64 * 1024 && P.N < (1LL << 31)) ? 1 : 0;
  if (P.lane_path) {
    P.warps_per_cta = lane_warps(per_warp, split_pairs<C>());
    P.smem = per_warp * P.warps_per_cta;
    lane_attr_all<S, C>(P);
    return;
  }
  const OzSmem<S> L(P.mmax, P.np);
  P.warps_per_cta = 8;
  P.smem = L.per_warp * P.warps_per_cta;
  throw_if(P.smem > 200 * 1024, "mmax too large for the OZ kernel", 4);
  allow_max_smem(oz_kernel<S>, P.smem, "oz smem attribute");
}

template <typename S, typename C>
void oz_lane_attr(const OzPlan& P) {
  throw_if(!P.lane_path, "internal: lane attributes without the lane path", 4);
  lane_attr_all<S, C>(P);
}

template <typename C>
void oz_build_rtab(const OzPlan& P, DevBuf& rtab) {
  // the unsplit kernel (FP64) reads the full complex table; the split kernels
  // the real factor d for m1 >= 0 and the powers of the phase w (entries per
  // pair: sum_l (2l+1)(l+1) + 2 mmax)
  constexpr bool split = split_pairs<C>();
  const int nfull = nrot(P.mmax), nsplit = hoff(P.mmax + 1) + 2 * P.mmax;
  throw_if(P.nR != (split ? nsplit : nfull), "internal: R table size", 4);
  throw_if(P.mmax > 6, "internal: R table mmax", 4);
  OzPlan F = P;
  F.nR = nfull;
  DevBuf rt64;
  DevBuf& target64 = split ? rt64 : rtab;
  target64.alloc(sizeof(Cx<double>) * (size_t)(P.npairs_pad * (long long)nfull));
  const long long nb = (P.npairs_pad + 127) / 128;
  clear_stale_error();
  rot_table_kernel<<<(unsigned)nb, 128>>>(F, target64.as<Cx<double>>());
  launch_check("R(q) table kernel launch");
  if (split) {
    rtab.alloc(sizeof(C) * (size_t)(P.npairs_pad * (long long)nsplit));
    rot_table_real<C><<<(unsigned)nb, 128>>>(P, rt64.as<Cx<double>>(), rtab.as<C>(), nfull);
    launch_check("R(q) table conversion launch");
  }
  cuda_check(cudaDeviceSynchronize(), "R(q) table build");
}

template <typename S, typename C>
void launch_oz(const OzPlan& P, Cx<S>* p, cudaStream_t s) {
  if (P.npairs == 0) return;
  clear_stale_error();
  if (P.lane_path) {
    const int per_warp_pairs = P.warp_pairs ? 1 : (split_pairs<C>() ? 16 : 32);
    const long long ngrp = (P.npairs + per_warp_pairs - 1) / per_warp_pairs;
    const long long nb = (ngrp + P.warps_per_cta - 1) / P.warps_per_cta;
    throw_if(nb > 0x7fffffffLL, "too many k-space pairs", 4);
    throw_if(P.nbatch < 1 || P.nbatch > 65535, "batch must be 1..65535", 4);
    const dim3 grid((unsigned)nb, (unsigned)P.nbatch), block(32 * P.warps_per_cta);
    switch (P.mmax) {
      case 1: lane_launch_one<S, C, 1>(P, p, grid, block, s); break;
      case 2: lane_launch_one<S, C, 2>(P, p, grid, block, s); break;
      case 3: lane_launch_one<S, C, 3>(P, p, grid, block, s); break;
      case 4: lane_launch_one<S, C, 4>(P, p, grid, block, s); break;
      case 5: lane_launch_one<S, C, 5>(P, p, grid, block, s); break;
      case 6: lane_launch_one<S, C, 6>(P, p, grid, block, s); break;
      default: throw Error(4, "mmax outside the lane kernel's range");
    }
    launch_check("oz lane kernel launch");
    return;
  }
  if constexpr (std::is_same<S, DF>::value) {
    throw Error(4, "internal: packed storage needs the lane path");
  } else {
    const long long nb = (P.npairs + P.warps_per_cta - 1) / P.warps_per_cta;
    throw_if(P.nbatch < 1 || P.nbatch > 65535, "batch must be 1..65535", 4);
    oz_kernel<S><<<dim3((unsigned)nb, (unsigned)P.nbatch), 32 * P.warps_per_cta, P.smem, s>>>(P, p);
    launch_check("oz kernel launch");
  }
}

}  // namespace mdft

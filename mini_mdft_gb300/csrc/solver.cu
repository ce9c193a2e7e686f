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
//       d = |r + R(o) x_a - x_s| under the minimum-image convention,
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
#include <memory>
#include <string>
#include <vector>

#include "handles.hpp"

using mdft::DevBuf;
using mdft::Error;
using mdft::throw_if;

namespace mdft {
namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 152 * 4;  // fixed grid of the streaming reductions
constexpr int kMaxHistory = 32;

// ---- deterministic grid-wide sums -----------------------------------------
// Each thread accumulates compensated (double-double) sums; a CTA adds its
// warps in a fixed order and writes its partials; the last CTA to finish adds
// all partials in CTA order.  With the fixed grid of kRedBlocks CTAs the
// result does not depend on scheduling.
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
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  Red<K> t = red_zero<K>();
  for (unsigned b = 0; b < gridDim.x; ++b) {
    const double* q = part + (size_t)b * W;
    Red<K> o;
    for (int k = 0; k < K; ++k) o.s[k] = Dd{__ldcg(q + 2 * k), __ldcg(q + 2 * k + 1)};
    o.mx = __ldcg(q + 2 * K);
    red_add(t, o);
  }
  fin(t);
  *counter = 0u;
}

unsigned red_blocks(long long n) {
  const long long b = (n + kRedThreads - 1) / kRedThreads;
  return (unsigned)std::max(1LL, std::min<long long>(b, kRedBlocks));
}

// ---- external potential ----------------------------------------------------
struct VextPlan {
  int nx, ny, nz, no, nsv, nsu;
  double dx, dy, dz, lx, ly, lz, ilx, ily, ilz;
  double vmax;
  const double* rot;   // (no, 9): rows xx xy xz yx yy yz zx zy zz
  const double* site;  // solvent (nsv, 3) then solute (nsu, 3) positions
  const double* pair;  // (nsv, nsu, 3): 4 eps_as, sig_as^2, qfact q_a q_s
};

__device__ __forceinline__ double min_image(double d, double l, double il) { return d - l * rint(d * il); }

__global__ void __launch_bounds__(256) vext_kernel(const VextPlan P, double* __restrict__ vext) {
  const long long n = (long long)P.nx * P.ny * P.nz * P.no;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / P.no;
    const int o = (int)(i - r * P.no);
    const int iz = (int)(r % P.nz);
    const long long rxy = r / P.nz;
    const int iy = (int)(rxy % P.ny), ix = (int)(rxy / P.ny);
    const double px = ix * P.dx, py = iy * P.dy, pz = iz * P.dz;
    const double* R = P.rot + 9 * (size_t)o;
    double v = 0.0;
    for (int a = 0; a < P.nsv; ++a) {
      const double xa = P.site[3 * a], ya = P.site[3 * a + 1], za = P.site[3 * a + 2];
      const double sx = px + (R[0] * xa + R[1] * ya + R[2] * za);
      const double sy = py + (R[3] * xa + R[4] * ya + R[5] * za);
      const double sz = pz + (R[6] * xa + R[7] * ya + R[8] * za);
      for (int s = 0; s < P.nsu; ++s) {
        const double* us = P.site + 3 * (P.nsv + s);
        const double ddx = min_image(sx - us[0], P.lx, P.ilx);
        const double ddy = min_image(sy - us[1], P.ly, P.ily);
        const double ddz = min_image(sz - us[2], P.lz, P.ilz);
        const double d2 = fmax(ddx * ddx + ddy * ddy + ddz * ddz, 1e-12);
        const double* c = P.pair + 3 * ((size_t)a * P.nsu + s);
        if (c[0] != 0.0) {
          const double s2 = c[1] / d2;
          const double s6 = s2 * s2 * s2;
          v += c[0] * (s6 * s6 - s6);
        }
        if (c[2] != 0.0) v += c[2] / sqrt(d2);
      }
    }
    vext[i] = isfinite(v) ? fmin(fmax(v, -P.vmax), P.vmax) : P.vmax;
  }
}

// ---- energy and gradient ---------------------------------------------------
struct EgArgs {
  const double* xi;
  const void* vexc;    // double (FP64 fields) or float (MDFT_F32)
  const double* vext;  // null: no external potential
  const double* w;
  double* g;
  long long n;
  int no;
  double kT, rho0, dv, prefactor;
  double* out;  // [E_total, E_id, E_ext, E_exc, max |g|]
  double* part;
  unsigned* counter;
};

template <typename TV>
__global__ void __launch_bounds__(kRedThreads) eg_kernel(const EgArgs A) {
  extern __shared__ double ws[];
  for (int i = threadIdx.x; i < A.no; i += blockDim.x) ws[i] = A.w[i];
  __syncthreads();
  const TV* vx = static_cast<const TV*>(A.vexc);
  const double c_id = A.kT * A.rho0 * A.dv, c_ext = A.rho0 * A.dv, c_exc = A.prefactor * A.rho0;
  Red<3> r = red_zero<3>();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n;
       i += (long long)gridDim.x * blockDim.x) {
    const double wo = ws[(int)(i % A.no)];
    const double x = A.xi[i], x2 = x * x, v = (double)vx[i];
    const double ve = A.vext ? A.vext[i] : 0.0;
    const double l = x2 > 0.0 ? log(x2) : 0.0;
    r.s[0] = dd_plus(r.s[0], c_id * wo * (x2 * l - x2 + 1.0));
    r.s[1] = dd_plus(r.s[1], c_ext * wo * x2 * ve);
    r.s[2] = dd_plus(r.s[2], c_exc * wo * v * (x2 - 1.0));
    const double gi = 2.0 * x * wo * (c_ext * (A.kT * l + ve) + 2.0 * c_exc * v);
    A.g[i] = gi;
    r.mx = fmax(r.mx, fabs(gi));
  }
  double* out = A.out;
  grid_reduce<3>(r, A.part, A.counter, [out](const Red<3>& t) {
    const double id = t.s[0].hi + t.s[0].lo, ext = t.s[1].hi + t.s[1].lo, exc = t.s[2].hi + t.s[2].lo;
    const Dd tot = dd_plus(dd_plus(t.s[0], t.s[1]), t.s[2]);
    out[0] = tot.hi + tot.lo;
    out[1] = id;
    out[2] = ext;
    out[3] = exc;
    out[4] = t.mx;
  });
}

// ---- L-BFGS vector passes --------------------------------------------------
// x <- a0 x + c u with c = c0 + c1 S[i1] + c2 S[i2] (slots < 0 left out; a0 = 0
// does not read x; u null adds nothing), then S[out] = scale (v . x) when
// out >= 0.
struct PassArgs {
  double* x;
  const double* u;
  const double* v;
  long long n;
  double a0, c0, c1, c2;
  int i1, i2;
  double scale;
  int out;
  double* S;
  double* part;
  unsigned* counter;
};

__global__ void __launch_bounds__(kRedThreads) lbfgs_pass_kernel(const PassArgs A) {
  double c = A.c0;
  if (A.i1 >= 0) c += A.c1 * A.S[A.i1];
  if (A.i2 >= 0) c += A.c2 * A.S[A.i2];
  Red<1> r = red_zero<1>();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < A.n;
       i += (long long)gridDim.x * blockDim.x) {
    double xv = A.a0 == 0.0 ? 0.0 : A.a0 * A.x[i];
    if (A.u) xv += c * A.u[i];
    A.x[i] = xv;
    if (A.out >= 0) r.s[0] = dd_plus(r.s[0], A.v[i] * xv);
  }
  if (A.out < 0) return;
  double* S = A.S;
  const int out = A.out;
  const double scale = A.scale;
  grid_reduce<1>(r, A.part, A.counter, [S, out, scale](const Red<1>& t) { S[out] = scale * (t.s[0].hi + t.s[0].lo); });
}

// xn = x + t d
__global__ void __launch_bounds__(256) step_kernel(double* __restrict__ xn, const double* __restrict__ x,
                                                   const double* __restrict__ d, double t, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    xn[i] = x[i] + t * d[i];
}

// s = t d, y = gn - g; S[o] = s . y, S[o + 1] = y . y
__global__ void __launch_bounds__(kRedThreads)
pair_kernel(double* __restrict__ s, double* __restrict__ y, const double* __restrict__ d,
            const double* __restrict__ gn, const double* __restrict__ g, double t, long long n, double* S, int o,
            double* part, unsigned* counter) {
  Red<2> r = red_zero<2>();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double sv = t * d[i], yv = gn[i] - g[i];
    s[i] = sv;
    y[i] = yv;
    r.s[0] = dd_plus(r.s[0], sv * yv);
    r.s[1] = dd_plus(r.s[1], yv * yv);
  }
  grid_reduce<2>(r, part, counter, [S, o](const Red<2>& t2) {
    S[o] = t2.s[0].hi + t2.s[0].lo;
    S[o + 1] = t2.s[1].hi + t2.s[1].lo;
  });
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

// ---- solver handle -----------------------------------------------------------
struct mdft_solver_s {
  mdft_opt_s* opt = nullptr;
  mdft_conv_s* conv = nullptr;
  int prec = 0, device = 0, m = 5;
  long long N = 0, n = 0;
  int no = 0, np = 0;
  double kT = 0, rho0 = 0, prefactor = 0, dv = 0;
  bool has_vext = false;
  DevBuf vext, w, p, vexc, xf, ga, gb, xa, d, hs, hy, scal, energy, part, counter;
  // L-BFGS history (ring of m pairs): rho_i = 1 / (s_i . y_i), gamma of the newest
  std::vector<double> rho;
  int nh = 0, head = 0;
  double gamma = 1.0;
  double* hs_at(int i) const { return hs.as<double>() + (size_t)i * n; }
  double* hy_at(int i) const { return hy.as<double>() + (size_t)i * n; }
  // scalar slots: alpha_i at i < m, then two beta slots, g.d, s.y, y.y
  int ALPHA(int i) const { return i; }
  int BETA(int j) const { return m + (j & 1); }
  int GD() const { return m + 2; }
  int SY() const { return m + 3; }
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

void launch_ok(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(MDFT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void pass(mdft_solver_s* h, double* x, const double* u, const double* v, double a0, double c0, double c1, int i1,
          double c2, int i2, double scale, int out, cudaStream_t s) {
  mdft::PassArgs A{x, u, v, h->n, a0, c0, c1, c2, i1, i2, scale, out, h->scal.as<double>(),
                   h->part.as<double>(), h->counter.as<unsigned>()};
  mdft::lbfgs_pass_kernel<<<mdft::red_blocks(h->n), mdft::kRedThreads, 0, s>>>(A);
  launch_ok("L-BFGS pass launch");
}

// E(x) and its gradient into g; the energies land in h->energy on the device
void evaluate(mdft_solver_s* h, const double* x, double* g, cudaStream_t s) {
  const void* xin = x;
  if (h->prec == MDFT_F32) {
    mdft::to_float_kernel<<<mdft::stream_blocks(h->n), 256, 0, s>>>(h->xf.as<float>(), x, h->n);
    launch_ok("xi conversion launch");
    xin = h->xf.ptr;
  }
  mdft::detail::angl2proj_fields(h->opt, xin, true, h->rho0, h->p.ptr, 1, s);
  mdft::detail::execute_fields(h->conv, h->p.ptr, 1, s);
  mdft::detail::proj2angl_fields(h->opt, h->p.ptr, h->vexc.ptr, 1, s);
  mdft::EgArgs A{x,          h->vexc.ptr, h->has_vext ? h->vext.as<double>() : nullptr,
                 h->w.as<double>(),       g,
                 h->n,       h->no,       h->kT,
                 h->rho0,    h->dv,       h->prefactor,
                 h->energy.as<double>(),  h->part.as<double>(),
                 h->counter.as<unsigned>()};
  const size_t smem = sizeof(double) * (size_t)h->no;
  if (h->prec == MDFT_F32)
    mdft::eg_kernel<float><<<mdft::red_blocks(h->n), mdft::kRedThreads, smem, s>>>(A);
  else
    mdft::eg_kernel<double><<<mdft::red_blocks(h->n), mdft::kRedThreads, smem, s>>>(A);
  launch_ok("energy kernel launch");
}

void read_energy(mdft_solver_s* h, double* terms, cudaStream_t s) {
  cuda_check(cudaMemcpyAsync(terms, h->energy.ptr, 5 * sizeof(double), cudaMemcpyDeviceToHost, s),
             "energy read-back");
  cuda_check(cudaStreamSynchronize(s), "solver stream");
}

double read_scalar(mdft_solver_s* h, int slot, cudaStream_t s) {
  double v = 0;
  cuda_check(cudaMemcpyAsync(&v, h->scal.as<double>() + slot, sizeof(double), cudaMemcpyDeviceToHost, s),
             "scalar read-back");
  cuda_check(cudaStreamSynchronize(s), "solver stream");
  return v;
}

// d = -H g by the two-loop recursion over the h->nh stored pairs; returns g . d
double direction(mdft_solver_s* h, const double* g, cudaStream_t s) {
  double* d = h->d.as<double>();
  const int m = h->m, nh = h->nh;
  if (nh == 0) {
    pass(h, d, g, g, 0.0, -1.0, 0, -1, 0, -1, 1.0, h->GD(), s);
    return read_scalar(h, h->GD(), s);
  }
  auto idx = [&](int j) { return ((h->head - 1 - j) % m + m) % m; };  // j = 0: newest
  // q = -g; alpha_newest = rho (s . q)
  pass(h, d, g, h->hs_at(idx(0)), 0.0, -1.0, 0, -1, 0, -1, h->rho[idx(0)], h->ALPHA(idx(0)), s);
  for (int j = 0; j < nh; ++j) {
    const int i = idx(j);
    if (j + 1 < nh) {  // q -= alpha_i y_i; alpha_next = rho_next (s_next . q)
      const int nx = idx(j + 1);
      pass(h, d, h->hy_at(i), h->hs_at(nx), 1.0, 0.0, -1.0, h->ALPHA(i), 0, -1, h->rho[nx], h->ALPHA(nx), s);
    } else {  // last: beta_oldest = rho_oldest gamma (y_oldest . q)
      pass(h, d, h->hy_at(i), h->hy_at(i), 1.0, 0.0, -1.0, h->ALPHA(i), 0, -1, h->rho[i] * h->gamma, h->BETA(0),
           s);
    }
  }
  for (int j = 0; j < nh; ++j) {  // oldest first: r = (gamma) r + (alpha_i - beta_i) s_i
    const int i = idx(nh - 1 - j);
    const double a0 = j == 0 ? h->gamma : 1.0;
    if (j + 1 < nh) {
      const int nx = idx(nh - 2 - j);
      pass(h, d, h->hs_at(i), h->hy_at(nx), a0, 0.0, 1.0, h->ALPHA(i), -1.0, h->BETA(j), h->rho[nx],
           h->BETA(j + 1), s);
    } else {
      pass(h, d, h->hs_at(i), g, a0, 0.0, 1.0, h->ALPHA(i), -1.0, h->BETA(j), 1.0, h->GD(), s);
    }
  }
  return read_scalar(h, h->GD(), s);
}

}  // namespace

extern "C" {

int mdft_vext_lj_coulomb(mdft_grid_t grid, const double* solvent_sites, int n_solvent_sites,
                         const double* solute_sites, int n_solute_sites, double vmax, double* vext, void* stream) {
  return solver_guard([&] {
    throw_if(!grid || !vext, "NULL argument");
    throw_if(n_solvent_sites < 1 || n_solute_sites < 0, "site counts must be >= 1 (solvent) and >= 0 (solute)");
    throw_if(!solvent_sites || (n_solute_sites > 0 && !solute_sites), "NULL argument");
    throw_if(!(vmax > 0), "vmax must be positive");
    const mdft::Grid& g = grid->g;
    const int nsv = n_solvent_sites, nsu = n_solute_sites;
    const double qf = mdft::qfact();
    std::vector<double> site((size_t)3 * (nsv + nsu)), pr((size_t)3 * nsv * std::max(nsu, 1), 0.0);
    for (int a = 0; a < nsv; ++a)
      for (int k = 0; k < 3; ++k) site[3 * a + k] = solvent_sites[6 * a + 3 + k];
    for (int s = 0; s < nsu; ++s)
      for (int k = 0; k < 3; ++k) site[3 * (nsv + s) + k] = solute_sites[6 * s + 3 + k];
    for (int a = 0; a < nsv; ++a)
      for (int s = 0; s < nsu; ++s) {
        const double* A = solvent_sites + 6 * a;
        const double* B = solute_sites + 6 * s;
        throw_if(A[1] < 0 || A[2] < 0 || B[1] < 0 || B[2] < 0, "sigma and epsilon must be >= 0");
        const double eps = std::sqrt(A[2] * B[2]), sig = 0.5 * (A[1] + B[1]);
        double* c = pr.data() + 3 * ((size_t)a * nsu + s);
        c[0] = 4.0 * eps;
        c[1] = sig * sig;
        c[2] = qf * A[0] * B[0];
      }
    const std::vector<double> rot = mdft::orientation_rotations(g);
    DevBuf drot, dsite, dpair;
    drot.upload(rot.data(), sizeof(double) * rot.size());
    dsite.upload(site.data(), sizeof(double) * site.size());
    dpair.upload(pr.data(), sizeof(double) * pr.size());
    mdft::VextPlan P{};
    P.nx = g.nx;
    P.ny = g.ny;
    P.nz = g.nz;
    P.no = g.no;
    P.nsv = nsv;
    P.nsu = nsu;
    P.lx = g.lx;
    P.ly = g.ly;
    P.lz = g.lz;
    P.dx = g.lx / g.nx;
    P.dy = g.ly / g.ny;
    P.dz = g.lz / g.nz;
    P.ilx = 1.0 / g.lx;
    P.ily = 1.0 / g.ly;
    P.ilz = 1.0 / g.lz;
    P.vmax = vmax;
    P.rot = drot.as<double>();
    P.site = dsite.as<double>();
    P.pair = dpair.as<double>();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long n = g.N() * (long long)g.no;
    mdft::vext_kernel<<<mdft::stream_blocks(n), 256, 0, s>>>(P, vext);
    launch_ok("vext kernel launch");
    // the tables are freed on return: finish first
    cuda_check(cudaStreamSynchronize(s), "vext kernel");
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
    h->kT = kT;
    h->rho0 = rho0;
    h->prefactor = prefactor;
    h->dv = (go.lx / go.nx) * (go.ly / go.ny) * (go.lz / go.nz);
    const size_t fb = sizeof(double) * (size_t)h->n;
    const size_t eb = h->prec == MDFT_F32 ? 4 : 8;
    h->w.upload(go.w.data(), sizeof(double) * go.no);
    h->p.alloc(2 * eb * (size_t)h->np * h->N);
    h->vexc.alloc(eb * (size_t)h->n);
    if (h->prec == MDFT_F32) h->xf.alloc(sizeof(float) * (size_t)h->n);
    h->ga.alloc(fb);
    h->gb.alloc(fb);
    h->xa.alloc(fb);
    h->d.alloc(fb);
    h->hs.alloc(fb * h->m);
    h->hy.alloc(fb * h->m);
    h->scal.alloc(sizeof(double) * (h->m + 5));
    h->energy.alloc(sizeof(double) * 5);
    h->part.alloc(sizeof(double) * mdft::kRedBlocks * 7);
    h->counter.alloc(256);
    cuda_check(cudaMemset(h->counter.ptr, 0, 256), "counter reset");
    cuda_check(cudaMemset(h->scal.ptr, 0, sizeof(double) * (h->m + 5)), "scalar reset");
    if (vext) {
      h->vext.alloc(fb);
      cuda_check(cudaMemcpy(h->vext.ptr, vext, fb, cudaMemcpyDeviceToDevice), "vext copy");
      h->has_vext = true;
    }
    h->rho.assign(h->m, 0.0);
    *out = h.release();
  });
}

int mdft_solver_energy(mdft_solver_t h, const double* xi, double* grad, double* terms, void* stream) {
  return solver_guard([&] {
    throw_if(!h || !xi || !terms, "NULL argument");
    throw_if(mdft::detail::current_device() != h->device, "the solver belongs to another device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    evaluate(h, xi, grad ? grad : h->ga.as<double>(), s);
    read_energy(h, terms, s);
  });
}

int mdft_solver_minimize(mdft_solver_t h, double* xi, int max_iter, double gtol, double ftol, double* trace,
                         int* iterations, void* stream) {
  return solver_guard([&] {
    throw_if(!h || !xi, "NULL argument");
    throw_if(max_iter < 0, "max_iter must be >= 0");
    throw_if(mdft::detail::current_device() != h->device, "the solver belongs to another device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const double c1 = 1e-4, max_first_step = 0.1;
    const int max_ls = 40;
    h->nh = 0;
    h->head = 0;
    double* x = xi;                  // current iterate
    double* xn = h->xa.as<double>();  // trial iterate
    double* g = h->ga.as<double>();
    double* gn = h->gb.as<double>();
    double E[5], En[5];
    evaluate(h, x, g, s);
    read_energy(h, E, s);
    if (trace) std::memcpy(trace, E, sizeof E);
    int it = 0;
    while (it < max_iter && E[4] > gtol) {
      double gd = direction(h, g, s);
      double t = 1.0;
      if (!(gd < 0.0) || h->nh == 0) {  // first step, or no descent: steepest descent
        h->nh = 0;
        if (!(gd < 0.0)) gd = direction(h, g, s);
        t = std::min(1.0, max_first_step / E[4]);
      }
      bool ok = false;
      for (int ls = 0; ls < max_ls; ++ls) {
        mdft::step_kernel<<<mdft::stream_blocks(h->n), 256, 0, s>>>(xn, x, h->d.as<double>(), t, h->n);
        launch_ok("step kernel launch");
        evaluate(h, xn, gn, s);
        read_energy(h, En, s);
        if (std::isfinite(En[0]) && En[0] <= E[0] + c1 * t * gd) {
          ok = true;
          break;
        }
        t *= 0.5;
      }
      if (!ok) break;  // no decrease along the direction: stop at the current iterate
      // curvature pair of the accepted step into the ring slot `head`
      mdft::pair_kernel<<<mdft::red_blocks(h->n), mdft::kRedThreads, 0, s>>>(
          h->hs_at(h->head), h->hy_at(h->head), h->d.as<double>(), gn, g, t, h->n, h->scal.as<double>(), h->SY(),
          h->part.as<double>(), h->counter.as<unsigned>());
      launch_ok("pair kernel launch");
      double sy_yy[2];
      cuda_check(cudaMemcpyAsync(sy_yy, h->scal.as<double>() + h->SY(), sizeof sy_yy, cudaMemcpyDeviceToHost, s),
                 "curvature read-back");
      cuda_check(cudaStreamSynchronize(s), "solver stream");
      if (sy_yy[0] > 1e-12 * sy_yy[1] && sy_yy[1] > 0) {
        h->rho[h->head] = 1.0 / sy_yy[0];
        h->gamma = sy_yy[0] / sy_yy[1];
        h->head = (h->head + 1) % h->m;
        h->nh = std::min(h->nh + 1, h->m);
      } else {
        h->nh = 0;  // the slot was overwritten: restart the history
      }
      std::swap(x, xn);
      std::swap(g, gn);
      const double Eprev = E[0];
      std::memcpy(E, En, sizeof E);
      ++it;
      if (trace) std::memcpy(trace + 5 * (size_t)it, E, sizeof E);
      if (std::fabs(Eprev - E[0]) <= ftol * std::max(1.0, std::fabs(E[0]))) break;
    }
    if (x != xi)
      cuda_check(cudaMemcpyAsync(xi, x, sizeof(double) * (size_t)h->n, cudaMemcpyDeviceToDevice, s),
                 "final iterate copy");
    cuda_check(cudaStreamSynchronize(s), "solver stream");
    if (iterations) *iterations = it;
  });
}

int mdft_solver_destroy(mdft_solver_t h) {
  delete h;
  return MDFT_OK;
}

}  // extern "C"

// capi.cu -- the extern "C" boundary declared in include/mdft_gb300.h.
//
// Handles own the host set-up (grids, maps, tables) and the device copies of
// the tables; the hot-path stages are enqueued on the caller's stream.  No
// exception leaves this file: every entry point returns an mdft_status and
// records the message for mdft_last_error().
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include <cstdlib>

#include "../../include/mdft_gb300.h"
#include "common.cuh"
#include "handles.hpp"

using mdft::Cx;
using mdft::DevBuf;
using mdft::Error;
using mdft::throw_if;

namespace {

thread_local std::string g_last_error;

template <typename F>
int guarded(F&& f) {
  try {
    f();
    return MDFT_OK;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return MDFT_ERR_NOMEM;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return MDFT_ERR_INVALID;
  } catch (...) {
    g_last_error = "unknown error";
    return MDFT_ERR_INVALID;
  }
}

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

void check_prec(int precision) {
  throw_if(precision != MDFT_F64 && precision != MDFT_F32 && precision != MDFT_F64_DF,
           "precision must be MDFT_F64, MDFT_F32 or MDFT_F64_DF");
}

// Calls f(S{}, C{}) with the storage and arithmetic types of a precision:
// MDFT_F64 (double, double), MDFT_F32 (float, float), MDFT_F64_DF (double,
// double-float).
template <typename F>
void with_types(int precision, F&& f) {
  switch (precision) {
    case MDFT_F64: f(double{}, double{}); return;
    case MDFT_F32: f(float{}, float{}); return;
    case MDFT_F64_DF: f(double{}, mdft::DF{}); return;
  }
  throw Error(MDFT_ERR_INVALID, "precision must be MDFT_F64, MDFT_F32 or MDFT_F64_DF");
}

constexpr long double kPiL = 3.141592653589793238462643383279502884L;

// exp(-2 pi i t / n), t = 0..n-1, rounded from long double.
template <typename T>
T from_ld(long double x) {
  return (T)x;
}
template <>
mdft::DF from_ld<mdft::DF>(long double x) {
  return mdft::DF(x);
}

template <typename T>
std::vector<Cx<T>> twiddles(int n) {
  std::vector<Cx<T>> tw(n > 0 ? n : 1);
  for (int t = 0; t < n; ++t) {
    const long double a = 2.0L * kPiL * (long double)t / (long double)n;
    tw[t] = mdft::mkc<T>(from_ld<T>(std::cos(a)), from_ld<T>(-std::sin(a)));
  }
  return tw;
}

template <typename T>
std::vector<T> cast_vec(const std::vector<double>& v) {
  return std::vector<T>(v.begin(), v.end());
}

}  // namespace

int mdft::record_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

namespace {

template <typename S, typename T>
void opt_build(mdft_opt_s* h) {
  const mdft::Grid& g = h->g;
  const int nt = g.ntheta, np = g.np;
  std::vector<T> ca((size_t)nt * np), cp((size_t)nt * np);
  const double inv = 1.0 / (double)(g.nphi * g.npsi);
  for (int it = 0; it < nt; ++it)
    for (int ip = 0; ip < np; ++ip) {
      const double d = g.wigner[(size_t)it * np + ip];
      const double f = g.fm[g.m[ip]];
      ca[(size_t)it * np + ip] = from_ld<T>((long double)d * g.wtheta[it] * f * inv);
      cp[(size_t)it * np + ip] = from_ld<T>((long double)d * f);
    }
  h->coef_a2p.upload(ca.data(), sizeof(T) * ca.size());
  h->coef_p2a.upload(cp.data(), sizeof(T) * cp.size());
  auto tp = twiddles<T>(g.nphi);
  auto ts = twiddles<T>(g.npsi);
  h->tw_phi.upload(tp.data(), sizeof(Cx<T>) * g.nphi);
  h->tw_psi.upload(ts.data(), sizeof(Cx<T>) * g.npsi);
  h->ip_m.upload(g.m.data(), sizeof(int) * np);
  h->ip_mup.upload(g.mup.data(), sizeof(int) * np);
  h->ip_mu2.upload(g.mu2.data(), sizeof(int) * np);
  h->pmap.upload(g.p.data(), sizeof(int) * g.p.size());
  mdft::AngPlan& P = h->plan;
  P.N = g.N() * h->batch;
  P.ntheta = g.ntheta;
  P.nphi = g.nphi;
  P.npsi = g.npsi;
  P.K = g.K;
  P.mmax = g.mmax;
  P.mrso = g.mrso;
  P.np = g.np;
  P.no = g.no;
  P.coef_a2p = h->coef_a2p.ptr;
  P.coef_p2a = h->coef_p2a.ptr;
  P.tw_phi = h->tw_phi.ptr;
  P.tw_psi = h->tw_psi.ptr;
  P.ip_m = h->ip_m.as<int>();
  P.ip_mup = h->ip_mup.as<int>();
  P.ip_mu2 = h->ip_mu2.as<int>();
  P.pmap = h->pmap.as<int>();
  mdft::ang_plan_finish<S, T>(P);
  // MDFT_ANG_TC=1 at create time: the double-float and FP32 forms run the
  // transforms as tensor-core GEMMs with exact digit slicing, where the
  // shape fits that kernel.  Off by default: on one GB300 at 64^3 / mmax 3
  // the CUDA-core kernels are faster (angl2proj / proj2angl: FP32 85 / 47 us
  // against 137 / 174; double-float 217 / 189 against 252 / 312).
  if constexpr (!std::is_same<T, double>::value) {
    const char* env = std::getenv("MDFT_ANG_TC");
    const bool use = env && env[0] == '1';
    if (use && mdft::ang_tc_setup<S>(P.tc_a2p, mdft::ang_matrix_a2p(g), 2 * np, g.no, 0, h->tc_bsl_a2p,
                                     h->tc_fexp_a2p))
      P.tc |= 1;
    if (use && mdft::ang_tc_setup<S>(P.tc_p2a, mdft::ang_matrix_p2a(g), g.no, 2 * np, 1, h->tc_bsl_p2a,
                                     h->tc_fexp_p2a))
      P.tc |= 2;
  }
}

template <typename ST, typename T>
void fft_axis_build(mdft::FftAxis& a, DevBuf& twbuf, int n, long long S, long long ncols) {
  throw_if(!mdft::fft_factor(n, a), "FFT length " + std::to_string(n) +
                                        " has a prime factor above 13", MDFT_ERR_UNSUPPORTED);
  a.S = S;
  a.ncols = ncols;
  auto tw = twiddles<T>(n);
  twbuf.upload(tw.data(), sizeof(Cx<T>) * n);
  a.tw = twbuf.ptr;
  if constexpr (std::is_same<T, mdft::DF>::value) {
    // double-float: every load/store format the pass chains use
    mdft::fft_axis_finish<double, double, T>(a);
    mdft::fft_axis_finish<double, mdft::DF, T>(a);
    mdft::fft_axis_finish<mdft::DF, mdft::DF, T>(a);
    mdft::fft_axis_finish<mdft::DF, double, T>(a);
  } else {
    mdft::fft_axis_finish<ST, ST, T>(a);
  }
}

template <typename S, typename T>
void conv_build(mdft_conv_s* h, const mdft::LucTable& t) {
  const mdft::Grid& g = h->g;
  throw_if(g.mmax > mdft::kRotMmaxMax, "Convolution supports mmax <= 6 (RotationCoeffs)",
           MDFT_ERR_UNSUPPORTED);
  const int need = (int)(g.qmax() / t.dq + 0.5) + 2;
  throw_if(t.nq < need, "c(q) table has " + std::to_string(t.nq) + " rows, the grid needs " +
                            std::to_string(need));
  h->nq = need;
  h->dq = t.dq;
  h->mnq = mdft::reorder_luc(g, t, need);
  // pair list: reference order kept for the getter, device copy sorted by
  // the linear index of q (each pair is independent; roles are unchanged).
  // FP32 arithmetic sorts by |q| first: the pairs of a warp then share their
  // c(|q|) row, which that latency-bound kernel gains more from than it
  // loses to scattered field accesses (the issue-bound double-float and FP64
  // kernels lose more than they gain).
  h->pair_list = mdft::gamma_p_map(g.nx, g.ny, g.nz);
  h->npairs = (int)(h->pair_list.size() / 3);
  std::vector<int4> pr(h->npairs);
  for (int i = 0; i < h->npairs; ++i)
    pr[i] = make_int4(h->pair_list[3 * i], h->pair_list[3 * i + 1], h->pair_list[3 * i + 2], 0);
  // (the warp-per-pair kernel of large angular grids reads a pair's
  // projections across the lanes, so it keeps the linear order, in which
  // neighbouring warps share the sectors of the field they read)
  const bool by_q = std::is_same<T, float>::value && g.np < mdft::oz_warp_min_np<T>();
  auto q2 = [&](const int4& a) { return g.kx[a.x] * g.kx[a.x] + g.ky[a.y] * g.ky[a.y] + g.kz[a.z] * g.kz[a.z]; };
  std::sort(pr.begin(), pr.end(), [&](const int4& a, const int4& b) {
    if (by_q) {
      const double qa = q2(a), qb = q2(b);
      if (qa != qb) return qa < qb;
    }
    const long long la = ((long long)a.x * g.ny + a.y) * g.nz + a.z;
    const long long lb = ((long long)b.x * g.ny + b.y) * g.nz + b.z;
    return la < lb;
  });
  h->pairs.upload(pr.data(), sizeof(int4) * pr.size());
  h->kx.upload(g.kx.data(), sizeof(double) * g.nx);
  h->ky.upload(g.ky.data(), sizeof(double) * g.ny);
  h->kz.upload(g.kz.data(), sizeof(double) * g.nz);
  mdft::RotationCoeffs rc;
  std::vector<double> rot;
  rot.insert(rot.end(), rc.a, rc.a + mdft::kRotL * mdft::kRotM * mdft::kRotM);
  rot.insert(rot.end(), rc.b, rc.b + mdft::kRotL * mdft::kRotM * mdft::kRotM);
  rot.insert(rot.end(), rc.c, rc.c + mdft::kRotL * mdft::kRotM);
  rot.insert(rot.end(), rc.d, rc.d + mdft::kRotL * mdft::kRotM);
  h->rot.upload(rot.data(), sizeof(double) * rot.size());
  h->pmap.upload(g.p.data(), sizeof(int) * g.p.size());
  h->ip_m.upload(g.m.data(), sizeof(int) * g.np);
  h->ip_mup.upload(g.mup.data(), sizeof(int) * g.np);
  h->ip_mu2.upload(g.mu2.data(), sizeof(int) * g.np);
  h->ia_map.upload(g.ia_map.data(), sizeof(int) * g.ia_map.size());
  mdft::OzPlan& O = h->oz;
  O.nx = g.nx;
  O.ny = g.ny;
  O.nz = g.nz;
  O.np = g.np;
  O.mmax = g.mmax;
  O.mrso = g.mrso;
  O.K = g.K;
  O.np_new = g.np_new;
  O.nq = need;
  O.npairs = h->npairs;
  O.N = g.N();
  O.nbatch = h->batch;
  O.pstride = g.N() * h->batch;
  O.dq = t.dq;
  O.pairs = h->pairs.as<int4>();
  O.kx = h->kx.as<double>();
  O.ky = h->ky.as<double>();
  O.kz = h->kz.as<double>();
  O.rot = h->rot.as<double>();
  O.pmap = h->pmap.as<int>();
  O.ip_m = h->ip_m.as<int>();
  O.ip_mup = h->ip_mup.as<int>();
  O.ip_mu2 = h->ip_mu2.as<int>();
  O.ia_map = h->ia_map.as<int>();
  mdft::oz_plan_finish<S, T>(O);
  // c(q) table transposed to (nq, np_new) so a pair's two rows are
  // contiguous, in the arithmetic type of the kernel that reads it
  auto upload_ctab = [&](auto tag) {
    using U = decltype(tag);
    std::vector<Cx<U>> ct((size_t)need * g.np_new);
    for (int i = 0; i < g.np_new; ++i)
      for (int iq = 0; iq < need; ++iq) {
        const auto z = h->mnq[(size_t)i * need + iq];
        ct[(size_t)iq * g.np_new + i] =
            mdft::mkc<U>(from_ld<U>((long double)z.real()), from_ld<U>((long double)z.imag()));
      }
    h->ctab.upload(ct.data(), sizeof(Cx<U>) * ct.size());
  };
  if (O.lane_path)
    upload_ctab(T{});
  else
    upload_ctab(S{});
  O.ctab = h->ctab.ptr;
  if (O.lane_path) {
    // Per-pair geometry of the lane path, in the sorted pair order: linear
    // indices of q and -q, the c(q) row iq and weight alpha of
    // MDFT_Convolution.hpp:449-455 (FP64, host, no contraction), and the
    // singular mid-k flag of :507-509.
    O.npairs_pad = ((long long)h->npairs + 31) / 32 * 32;
    // R entries per pair: all sum_l (2l+1)^2 complex ones for the unsplit
    // FP64 kernel; for the split FP32 / double-float one the real factor of
    // the m1 >= 0 half, sum_l (2l+1)(l+1), and the mmax phase powers (re, im)
    O.nR = std::is_same<T, double>::value ? (g.mmax + 1) * (2 * g.mmax + 1) * (2 * g.mmax + 3) / 3
                                          : (g.mmax + 1) * (g.mmax + 2) * (4 * g.mmax + 3) / 6 + 2 * g.mmax;
    std::vector<int4> info((size_t)O.npairs_pad, make_int4(0, 0, 0, 0));
    std::vector<T> alpha((size_t)O.npairs_pad, T(0));
    std::vector<double> alpha_d((size_t)O.npairs_pad, 0.0);
    for (int i = 0; i < h->npairs; ++i) {
      const int ix = pr[i].x, iy = pr[i].y, iz = pr[i].z;
      const int ixm = ix == 0 ? 0 : g.nx - ix, iym = iy == 0 ? 0 : g.ny - iy, izm = iz == 0 ? 0 : g.nz - iz;
      const double q[3] = {g.kx[ix], g.ky[iy], g.kz[iz]};
      double s2 = 0;
      for (int k = 0; k < 3; ++k) s2 += q[k] * q[k];
      const double eiq = std::sqrt(s2) / t.dq;
      const int iq = std::min((int)eiq, need - 2);
      const bool qeq = (ixm == ix && iym == iy && izm == iz);
      const bool sing = qeq && (ix == g.nx / 2 || iy == g.ny / 2 || iz == g.nz / 2);
      info[i] = make_int4((int)(((long long)ix * g.ny + iy) * g.nz + iz),
                          (int)(((long long)ixm * g.ny + iym) * g.nz + izm), iq, sing ? 1 : 0);
      alpha_d[i] = eiq - (double)iq;
      alpha[i] = from_ld<T>((long double)alpha_d[i]);
    }
    // c(|q|) interpolated once per distinct (iq, alpha) of the pair list
    // (MDFT_Convolution.hpp:449-463): on a cubic box the pairs share a few
    // thousand |q| values, so the per-pair interpolation becomes a row read.
    {
      std::map<std::pair<int, double>, int> rows;
      std::vector<std::pair<int, double>> keys;
      std::vector<int> row_of(h->npairs);
      for (int i = 0; i < h->npairs; ++i) {
        const std::pair<int, double> key(info[i].z, alpha_d[i]);
        auto it = rows.find(key);
        if (it == rows.end()) {
          it = rows.emplace(key, (int)keys.size()).first;
          keys.push_back(key);
        }
        row_of[i] = it->second;
      }
      const size_t bytes = keys.size() * (size_t)g.np_new * sizeof(Cx<T>);
      if (bytes <= (size_t)256 << 20) {
        std::vector<Cx<T>> ce(keys.size() * (size_t)g.np_new);
        for (size_t r = 0; r < keys.size(); ++r) {
          const int iq = keys[r].first;
          const long double a = keys[r].second, b = 1.0L - a;
          for (int ia = 0; ia < g.np_new; ++ia) {
            const auto lo = h->mnq[(size_t)ia * need + iq], hi = h->mnq[(size_t)ia * need + iq + 1];
            ce[r * g.np_new + ia] = mdft::mkc<T>(from_ld<T>(a * hi.real() + b * lo.real()),
                                                 from_ld<T>(a * hi.imag() + b * lo.imag()));
          }
        }
        h->ceff.upload(ce.data(), sizeof(Cx<T>) * ce.size());
        for (int i = 0; i < h->npairs; ++i) info[i].z = row_of[i];
        O.ceff = h->ceff.ptr;
        // The FP32 split kernel stages its CTA's rows in shared memory (the
        // pairs run in |q| order, so rows increase along the list): at mmax
        // <= 3 that took the 64^3 k-space step from 134 to 123 us on one
        // GB300; at mmax 4 (96^3) the larger rows cost more than they saved
        // (1.46 -> 1.96 ms), and the double-float kernel, issue-bound on a
        // list in linear order, gained nothing from a |q| order with staged
        // rows (331 -> 379 us).
        if (by_q && g.mmax <= 3) {
          const int budget = 16 << 10;
          const size_t row_bytes = sizeof(Cx<T>) * (size_t)g.np_new;
          O.crow_stage = (int)std::min<size_t>(16, (size_t)budget / row_bytes);
          if (O.crow_stage > 0) {
            O.cstage_off = (O.smem + 15) & ~size_t(15);
            O.smem = O.cstage_off + row_bytes * O.crow_stage;
            mdft::oz_lane_attr<S, T>(O);
            if constexpr (!std::is_same<S, T>::value) mdft::oz_lane_attr<T, T>(O);
          }
        }
      }
    }
    h->pinfo.upload(info.data(), sizeof(int4) * info.size());
    h->palpha.upload(alpha.data(), sizeof(T) * alpha.size());
    // first OZ coefficient of each projection (the ia_map enumeration order,
    // MDFT_Convolution.hpp:186-195)
    std::vector<int> ia0(g.np);
    {
      int ia = 0;
      for (int ip = 0; ip < g.np; ++ip) {
        ia0[ip] = ia;
        for (int in = std::abs(g.mup[ip]); in <= g.mmax; ++in) ia += 2 * (in / g.mrso) + 1;
      }
    }
    h->ia_start.upload(ia0.data(), sizeof(int) * ia0.size());
    O.pinfo = h->pinfo.as<int4>();
    O.palpha = h->palpha.ptr;
    O.ia_start = h->ia_start.as<int>();
    mdft::oz_build_rtab<T>(O, h->rtab);
    O.rtab = h->rtab.ptr;
  }
  const long long N = g.N(), np = (long long)g.np * h->batch;  // transforms per axis scale with the batch
  fft_axis_build<S, T>(h->az, h->tw_z, g.nz, 1, np * g.nx * g.ny);
  fft_axis_build<S, T>(h->ay, h->tw_y, g.ny, g.nz, np * g.nx * (long long)g.nz);
  fft_axis_build<S, T>(h->ax, h->tw_x, g.nx, (long long)g.ny * g.nz, np * (long long)g.ny * g.nz);
  if constexpr (std::is_same<T, mdft::DF>::value) {
    h->df_packed = O.lane_path && (g.nx > 1 || g.ny > 1 || g.nz > 1);
    if (h->df_packed) mdft::oz_lane_attr<mdft::DF, mdft::DF>(O);
  }
  (void)N;
}

// One 3-D transform as three axis passes (z, y, x forward; x, y, z
// backward).  In the double-float form the passes of one chain keep the data
// as packed DF pairs: the first pass converts from `in_packed` storage, the
// last converts to `out_packed` storage.
// The launch descriptors of a convolution plan restricted to its first k
// fields: the FFT passes cover k of the batch's transforms and the k-space
// kernel k fields, with p laid out (np, k, N).
struct ConvLaunch {
  mdft::FftAxis ax, ay, az;
  mdft::OzPlan oz;
};
ConvLaunch conv_launch(const mdft_conv_s* h, int k) {
  throw_if(k < 1 || k > h->batch, "active fields must be 1.." + std::to_string(h->batch));
  ConvLaunch L{h->ax, h->ay, h->az, h->oz};
  if (k != h->batch) {
    for (mdft::FftAxis* a : {&L.ax, &L.ay, &L.az}) a->ncols = a->ncols / h->batch * k;
    L.oz.nbatch = k;
    L.oz.pstride = h->oz.N * k;
  }
  return L;
}

// One 3-D transform as three axis passes (z, y, x forward; x, y, z
// inverse).  after (optional): three events, each recorded once its pass has
// been enqueued (a length-1 axis records at once).
template <typename S, typename T>
void conv_fft(ConvLaunch& L, void* p, int sign, cudaStream_t s, bool in_packed = false,
              bool out_packed = false, cudaEvent_t const* after = nullptr) {
  mdft::FftAxis* order[3];
  if (sign < 0) {
    order[0] = &L.az;
    order[1] = &L.ay;
    order[2] = &L.ax;
  } else {
    order[0] = &L.ax;
    order[1] = &L.ay;
    order[2] = &L.az;
  }
  auto mark = [&](int i) {
    if (after) mdft::cuda_check(cudaEventRecord(after[i], s), "pass event record");
  };
  if constexpr (std::is_same<T, mdft::DF>::value) {
    int nl = 0;
    for (auto* a : order)
      if (a->n > 1) ++nl;
    throw_if(nl == 0 && in_packed != out_packed, "internal: no FFT pass to change the format", 4);
    int li = 0;
    for (int k = 0; k < 3; ++k) {
      mdft::FftAxis* a = order[k];
      if (a->n > 1) {
        const bool src = li == 0 ? in_packed : true;
        const bool dst = li == nl - 1 ? out_packed : true;
        if (!src && !dst)
          mdft::launch_fft_axis<double, double, T>(*a, p, sign, s);
        else if (!src && dst)
          mdft::launch_fft_axis<double, mdft::DF, T>(*a, p, sign, s);
        else if (src && dst)
          mdft::launch_fft_axis<mdft::DF, mdft::DF, T>(*a, p, sign, s);
        else
          mdft::launch_fft_axis<mdft::DF, double, T>(*a, p, sign, s);
        ++li;
      }
      mark(k);
    }
  } else {
    for (int k = 0; k < 3; ++k) {
      mdft::launch_fft_axis<S, S, T>(*order[k], p, sign, s);
      mark(k);
    }
  }
}

int current_device() {
  int d = 0;
  mdft::cuda_check(cudaGetDevice(&d), "cudaGetDevice");
  return d;
}

void check_device(int dev) {
  throw_if(current_device() != dev, "handle was created on another CUDA device");
}

// Stream-ordered scratch for the energy partials.
// The library's own stream-ordered memory pool on the current device, for
// the temporaries of its allocating entry points.  It keeps up to
// kScratchKeep bytes mapped between calls: the device's default pool hands
// its memory back to the driver at every synchronisation (unless its owner
// raised the release threshold), so each call made after a synchronize --
// a solver reads its energy back every iteration -- would map its scratch
// afresh, about 100 us of host time per call.  A handle found invalid (the
// context torn down and created again) is replaced.
constexpr uint64_t kScratchKeep = uint64_t(64) << 20;
std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pools;

cudaMemPool_t scratch_pool() {
  int dev = 0;
  mdft::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_pool_mu);
  auto it = g_pools.find(dev);
  if (it != g_pools.end()) {
    uint64_t v = 0;
    if (cudaMemPoolGetAttribute(it->second, cudaMemPoolAttrReleaseThreshold, &v) == cudaSuccess) return it->second;
    cudaGetLastError();
    g_pools.erase(it);
  }
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  mdft::cuda_check(cudaMemPoolCreate(&pool, &props), "cudaMemPoolCreate");
  uint64_t keep = kScratchKeep;
  mdft::cuda_check(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep),
                   "cudaMemPoolSetAttribute");
  g_pools[dev] = pool;
  return pool;
}

struct Scratch {
  void* p = nullptr;
  cudaStream_t s;
  Scratch(size_t bytes, cudaStream_t st) : s(st) {
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, scratch_pool(), s);
    if (e != cudaSuccess)
      throw Error(MDFT_ERR_NOMEM, std::string("cudaMallocFromPoolAsync: ") + cudaGetErrorString(e));
  }
  ~Scratch() {
    if (p) cudaFreeAsync(p, s);
  }
};

}  // namespace

extern "C" {

int mdft_abi_version(void) { return MDFT_GB300_ABI_VERSION; }

int mdft_scratch_pool(void** pool) {
  return guarded([&] {
    throw_if(!pool, "NULL argument");
    *pool = scratch_pool();
  });
}

const char* mdft_last_error(void) { return g_last_error.c_str(); }

int mdft_grid_create(mdft_grid_t* out, int nx, int ny, int nz, double lx, double ly, double lz,
                     int mmax, int molrotsymorder) {
  return guarded([&] {
    throw_if(!out, "out is NULL");
    *out = nullptr;
    mdft::Grid g(nx, ny, nz, lx, ly, lz, mmax, molrotsymorder);
    *out = new mdft_grid_s(g);
  });
}

int mdft_grid_destroy(mdft_grid_t g) {
  delete g;
  return MDFT_OK;
}

int mdft_grid_info(mdft_grid_t h, int* v) {
  return guarded([&] {
    throw_if(!h || !v, "NULL argument");
    const mdft::Grid& g = h->g;
    const int vals[11] = {g.nx, g.ny, g.nz, g.mmax, g.mrso, g.ntheta, g.nphi, g.npsi, g.no, g.np, g.np_new};
    std::memcpy(v, vals, sizeof(vals));
  });
}

int mdft_grid_kvectors(mdft_grid_t h, double* kx, double* ky, double* kz) {
  return guarded([&] {
    throw_if(!h || !kx || !ky || !kz, "NULL argument");
    std::memcpy(kx, h->g.kx.data(), sizeof(double) * h->g.nx);
    std::memcpy(ky, h->g.ky.data(), sizeof(double) * h->g.ny);
    std::memcpy(kz, h->g.kz.data(), sizeof(double) * h->g.nz);
  });
}

int mdft_grid_angular(mdft_grid_t h, double* theta, double* wtheta, double* w) {
  return guarded([&] {
    throw_if(!h || !theta || !wtheta || !w, "NULL argument");
    std::memcpy(theta, h->g.theta.data(), sizeof(double) * h->g.ntheta);
    std::memcpy(wtheta, h->g.wtheta.data(), sizeof(double) * h->g.ntheta);
    std::memcpy(w, h->g.w.data(), sizeof(double) * h->g.no);
  });
}

int mdft_grid_opmap(mdft_grid_t h, int* p, int* m, int* mup, int* mu, int* mu2, double* wigner) {
  return guarded([&] {
    throw_if(!h || !p || !m || !mup || !mu || !mu2 || !wigner, "NULL argument");
    const mdft::Grid& g = h->g;
    std::memcpy(p, g.p.data(), sizeof(int) * g.p.size());
    std::memcpy(m, g.m.data(), sizeof(int) * g.np);
    std::memcpy(mup, g.mup.data(), sizeof(int) * g.np);
    std::memcpy(mu, g.mu.data(), sizeof(int) * g.np);
    std::memcpy(mu2, g.mu2.data(), sizeof(int) * g.np);
    std::memcpy(wigner, g.wigner.data(), sizeof(double) * g.wigner.size());
  });
}

int mdft_grid_ang_matrices(mdft_grid_t h, double* a2p, double* p2a) {
  return guarded([&] {
    throw_if(!h || !a2p || !p2a, "NULL argument");
    const auto A = mdft::ang_matrix_a2p(h->g), B = mdft::ang_matrix_p2a(h->g);
    std::memcpy(a2p, A.data(), sizeof(double) * A.size());
    std::memcpy(p2a, B.data(), sizeof(double) * B.size());
  });
}

int mdft_opt_create(mdft_opt_t* out, mdft_grid_t g, int precision) {
  return mdft_opt_create_batched(out, g, precision, 1);
}

int mdft_opt_create_batched(mdft_opt_t* out, mdft_grid_t g, int precision, int batch) {
  return guarded([&] {
    throw_if(!out || !g, "NULL argument");
    *out = nullptr;
    check_prec(precision);
    throw_if(batch < 1 || batch > 65535, "batch must be 1..65535");
    throw_if((long long)batch * g->g.N() >= (1LL << 31), "batch times grid points must stay below 2^31", 4);
    auto h = std::make_unique<mdft_opt_s>(g->g);
    h->batch = batch;
    h->prec = precision;
    h->device = current_device();
    with_types(precision, [&](auto st, auto ct) { opt_build<decltype(st), decltype(ct)>(h.get()); });
    *out = h.release();
  });
}

int mdft_opt_destroy(mdft_opt_t h) {
  delete h;
  return MDFT_OK;
}

int mdft_opt_angl2proj(mdft_opt_t h, const void* o, void* p, void* stream) {
  return guarded([&] {
    throw_if(!h || !o || !p, "NULL argument");
    check_device(h->device);
    with_types(h->prec, [&](auto st, auto ct) {
      using S = decltype(st);
      mdft::launch_angl2proj<S, decltype(ct)>(h->plan, static_cast<const S*>(o), static_cast<Cx<S>*>(p),
                                               false, 0.0, as_stream(stream));
    });
  });
}

int mdft_opt_angl2proj_from_xi(mdft_opt_t h, const void* xi, double rho0, void* p, void* stream) {
  return guarded([&] {
    throw_if(!h || !xi || !p, "NULL argument");
    check_device(h->device);
    with_types(h->prec, [&](auto st, auto ct) {
      using S = decltype(st);
      mdft::launch_angl2proj<S, decltype(ct)>(h->plan, static_cast<const S*>(xi), static_cast<Cx<S>*>(p),
                                               true, rho0, as_stream(stream));
    });
  });
}

int mdft_opt_proj2angl(mdft_opt_t h, const void* p, void* o, void* stream) {
  return guarded([&] {
    throw_if(!h || !o || !p, "NULL argument");
    check_device(h->device);
    with_types(h->prec, [&](auto st, auto ct) {
      using S = decltype(st);
      mdft::launch_proj2angl<S, decltype(ct)>(h->plan, static_cast<const Cx<S>*>(p), static_cast<S*>(o),
                                               as_stream(stream));
    });
  });
}

static int conv_create_impl(mdft_conv_t* out, mdft_grid_t g, const mdft::LucTable& t, int precision,
                            int batch = 1) {
  return guarded([&] {
    throw_if(!out || !g, "NULL argument");
    *out = nullptr;
    check_prec(precision);
    throw_if(batch < 1 || batch > 65535, "batch must be 1..65535");
    throw_if((long long)batch * g->g.N() >= (1LL << 31), "batch times grid points must stay below 2^31", 4);
    auto h = std::make_unique<mdft_conv_s>(g->g);
    h->batch = batch;
    h->prec = precision;
    h->device = current_device();
    with_types(precision, [&](auto st, auto ct) { conv_build<decltype(st), decltype(ct)>(h.get(), t); });
    *out = h.release();
  });
}

int mdft_conv_create(mdft_conv_t* out, mdft_grid_t g, const int* luc_index, const double* luc,
                     int np_luc, int nq, double dq, int precision) {
  return mdft_conv_create_batched(out, g, luc_index, luc, np_luc, nq, dq, precision, 1);
}

int mdft_conv_create_batched(mdft_conv_t* out, mdft_grid_t g, const int* luc_index, const double* luc,
                             int np_luc, int nq, double dq, int precision, int batch) {
  mdft::LucTable t;
  int rc = guarded([&] {
    throw_if(!luc_index || !luc, "NULL argument");
    throw_if(np_luc <= 0 || nq <= 1 || !(dq > 0), "invalid c(q) table extents");
    t.np_luc = np_luc;
    t.nq = nq;
    t.dq = dq;
    t.index.assign(luc_index, luc_index + 5 * (size_t)np_luc);
    t.tab.resize((size_t)np_luc * nq);
    std::memcpy(t.tab.data(), luc, sizeof(double) * 2 * t.tab.size());
  });
  if (rc != MDFT_OK) {
    if (out) *out = nullptr;
    return rc;
  }
  return conv_create_impl(out, g, t, precision, batch);
}

int mdft_conv_create_from_file(mdft_conv_t* out, mdft_grid_t g, const char* path, int np_luc,
                               int precision) {
  mdft::LucTable t;
  int rc = guarded([&] {
    throw_if(!path || !g, "NULL argument");
    t = mdft::read_luc_file(path, np_luc, g->g.qmax());
  });
  if (rc != MDFT_OK) {
    if (out) *out = nullptr;
    return rc;
  }
  return conv_create_impl(out, g, t, precision);
}

int mdft_conv_destroy(mdft_conv_t h) {
  delete h;
  return MDFT_OK;
}

int mdft_conv_fft(mdft_conv_t h, void* p, int sign, void* stream) {
  return guarded([&] {
    throw_if(!h || !p, "NULL argument");
    throw_if(sign != -1 && sign != 1, "sign must be -1 or +1");
    check_device(h->device);
    mdft::check_device_waits();
    with_types(h->prec, [&](auto st, auto ct) {
      ConvLaunch L = conv_launch(h, h->batch);
      conv_fft<decltype(st), decltype(ct)>(L, p, sign, as_stream(stream));
    });
  });
}

int mdft_conv_kspace(mdft_conv_t h, void* p, void* stream) {
  return guarded([&] {
    throw_if(!h || !p, "NULL argument");
    check_device(h->device);
    mdft::check_device_waits();
    with_types(h->prec, [&](auto st, auto ct) {
      using S = decltype(st);
      mdft::launch_oz<S, decltype(ct)>(h->oz, static_cast<Cx<S>*>(p), as_stream(stream));
    });
  });
}

namespace {
// execute(): forward FFT, k-space step, inverse FFT.  ev (optional) receives
// an event record before the forward FFT and after each of the three stages;
// pev (optional) eight records: before the forward FFT, after each of its
// three axis passes, after the k-space step and after each inverse pass.
void conv_execute(mdft_conv_s* h, void* p, cudaStream_t s, cudaEvent_t const* ev, int k = 0,
                  cudaEvent_t const* pev = nullptr) {
  auto mark = [&](int i) {
    if (ev) mdft::cuda_check(cudaEventRecord(ev[i], s), "stage event record");
  };
  auto pmark = [&](int i) {
    if (pev) mdft::cuda_check(cudaEventRecord(pev[i], s), "pass event record");
  };
  const cudaEvent_t* fwd = pev ? pev + 1 : nullptr;
  const cudaEvent_t* inv = pev ? pev + 5 : nullptr;
  ConvLaunch L = conv_launch(h, k > 0 ? k : h->batch);
  with_types(h->prec, [&](auto st, auto ct) {
    using S = decltype(st);
    using C = decltype(ct);
    if constexpr (std::is_same<C, mdft::DF>::value) {
      if (h->df_packed) {
        mark(0);
        pmark(0);
        conv_fft<S, C>(L, p, -1, s, false, true, fwd);
        mark(1);
        mdft::launch_oz<mdft::DF, C>(L.oz, static_cast<Cx<mdft::DF>*>(p), s);
        mark(2);
        pmark(4);
        conv_fft<S, C>(L, p, +1, s, true, false, inv);
        mark(3);
        return;
      }
    }
    mark(0);
    pmark(0);
    conv_fft<S, C>(L, p, -1, s, false, false, fwd);
    mark(1);
    mdft::launch_oz<S, C>(L.oz, static_cast<Cx<S>*>(p), s);
    mark(2);
    pmark(4);
    conv_fft<S, C>(L, p, +1, s, false, false, inv);
    mark(3);
  });
}
}  // namespace

int mdft_conv_execute(mdft_conv_t h, void* p, void* stream) {
  return guarded([&] {
    throw_if(!h || !p, "NULL argument");
    check_device(h->device);
    mdft::check_device_waits();
    conv_execute(h, p, as_stream(stream), nullptr);
  });
}

int mdft_conv_execute_timed(mdft_conv_t h, void* p, void* stream, void* const* events) {
  return guarded([&] {
    throw_if(!h || !p || !events, "NULL argument");
    for (int i = 0; i < 4; ++i) throw_if(!events[i], "NULL event");
    check_device(h->device);
    mdft::check_device_waits();
    conv_execute(h, p, as_stream(stream), reinterpret_cast<cudaEvent_t const*>(events));
  });
}

int mdft_conv_execute_timed_passes(mdft_conv_t h, void* p, void* stream, void* const* events) {
  return guarded([&] {
    throw_if(!h || !p || !events, "NULL argument");
    for (int i = 0; i < 8; ++i) throw_if(!events[i], "NULL event");
    check_device(h->device);
    mdft::check_device_waits();
    conv_execute(h, p, as_stream(stream), nullptr, 0, reinterpret_cast<cudaEvent_t const*>(events));
  });
}

int mdft_conv_info(mdft_conv_t h, int* ints, double* dq) {
  return guarded([&] {
    throw_if(!h || !ints || !dq, "NULL argument");
    ints[0] = h->npairs;
    ints[1] = h->g.np_new;
    ints[2] = h->nq;
    *dq = h->dq;
  });
}

int mdft_conv_gamma_p_map(mdft_conv_t h, int* map) {
  return guarded([&] {
    throw_if(!h || !map, "NULL argument");
    std::memcpy(map, h->pair_list.data(), sizeof(int) * h->pair_list.size());
  });
}

int mdft_conv_mnmunukhi_q(mdft_conv_t h, double* tab) {
  return guarded([&] {
    throw_if(!h || !tab, "NULL argument");
    std::memcpy(tab, h->mnq.data(), sizeof(double) * 2 * h->mnq.size());
  });
}

int mdft_get_delta_rho(const void* xi, void* delta_rho, size_t n, double rho0, int precision,
                       void* stream) {
  return guarded([&] {
    check_prec(precision);
    throw_if(n > 0 && (!xi || !delta_rho), "NULL argument");
    if (precision != MDFT_F32)  // MDFT_F64 and MDFT_F64_DF fields are double
      mdft::launch_delta_rho<double>(static_cast<const double*>(xi), static_cast<double*>(delta_rho), n,
                                     rho0, as_stream(stream));
    else
      mdft::launch_delta_rho<float>(static_cast<const float*>(xi), static_cast<float*>(delta_rho), n, rho0,
                                    as_stream(stream));
  });
}

int mdft_get_delta_f(const void* xi, const void* vexc, const double* w, void* delta_f, double* ff_dev,
                     size_t nxyz, int no, double rho0, double prefactor, int precision, void* stream) {
  return guarded([&] {
    check_prec(precision);
    throw_if(no <= 0, "angular grid size must be positive");
    throw_if(!ff_dev, "NULL argument");
    throw_if(nxyz > 0 && (!xi || !vexc || !w || !delta_f), "NULL argument");
    cudaStream_t s = as_stream(stream);
    const size_t nb = mdft::delta_f_partials(nxyz, no);
    const size_t bytes = sizeof(double2) * nb + 16;
    Scratch scratch(bytes, s);
    mdft::cuda_check(cudaMemsetAsync(static_cast<char*>(scratch.p) + sizeof(double2) * nb, 0, 16, s),
                     "cudaMemsetAsync");
    if (precision != MDFT_F32)  // MDFT_F64 and MDFT_F64_DF fields are double
      mdft::launch_delta_f<double>(static_cast<const double*>(xi), static_cast<const double*>(vexc), w,
                                   static_cast<double*>(delta_f), ff_dev, nxyz, no, rho0, prefactor,
                                   scratch.p, s, precision == MDFT_F64);
    else
      mdft::launch_delta_f<float>(static_cast<const float*>(xi), static_cast<const float*>(vexc), w,
                                  static_cast<float*>(delta_f), ff_dev, nxyz, no, rho0, prefactor,
                                  scratch.p, s, false);
  });
}

}  // extern "C"

// ---- stages on the first k fields of a batched plan (the job server) -------
namespace mdft {
namespace detail {

void angl2proj_fields(mdft_opt_s* h, const void* o, bool from_xi, double rho0, void* p, int k,
                      cudaStream_t s) {
  throw_if(k < 1 || k > h->batch, "active fields must be 1.." + std::to_string(h->batch));
  AngPlan P = h->plan;
  P.N = h->g.N() * k;
  with_types(h->prec, [&](auto st, auto ct) {
    using S = decltype(st);
    launch_angl2proj<S, decltype(ct)>(P, static_cast<const S*>(o), static_cast<Cx<S>*>(p), from_xi, rho0, s);
  });
}

void proj2angl_fields(mdft_opt_s* h, const void* p, void* o, int k, cudaStream_t s) {
  throw_if(k < 1 || k > h->batch, "active fields must be 1.." + std::to_string(h->batch));
  AngPlan P = h->plan;
  P.N = h->g.N() * k;
  with_types(h->prec, [&](auto st, auto ct) {
    using S = decltype(st);
    launch_proj2angl<S, decltype(ct)>(P, static_cast<const Cx<S>*>(p), static_cast<S*>(o), s);
  });
}

void execute_fields(mdft_conv_s* h, void* p, int k, cudaStream_t s) { conv_execute(h, p, s, nullptr, k); }

int current_device() { return ::current_device(); }

}  // namespace detail
}  // namespace mdft

// ---- c(q) files ------------------------------------------------------------------
int mdft_luc_read(const char* path, int np_luc, double qmax, int* luc_index, double* luc, int* nq,
                  double* dq) {
  return guarded([&] {
    throw_if(!path || !nq || !dq, "NULL argument");
    throw_if(!(qmax > 0), "qmax must be positive");
    const mdft::LucTable t = mdft::read_luc_file(path, np_luc, qmax);
    *nq = t.nq;
    *dq = t.dq;
    if (luc_index && luc) {
      std::memcpy(luc_index, t.index.data(), sizeof(int) * t.index.size());
      std::memcpy(luc, t.tab.data(), sizeof(double) * 2 * t.tab.size());
    }
  });
}

int mdft_luc_write(const char* path, const int* luc_index, const double* luc, int np_luc, int nq, double dq,
                   const char* header) {
  return guarded([&] {
    throw_if(!path || !luc_index || !luc, "NULL argument");
    throw_if(np_luc <= 0 || nq <= 0 || !(dq > 0), "invalid c(q) table extents");
    mdft::LucTable t;
    t.np_luc = np_luc;
    t.nq = nq;
    t.dq = dq;
    t.index.assign(luc_index, luc_index + 5 * (size_t)np_luc);
    t.tab.resize((size_t)np_luc * nq);
    std::memcpy(t.tab.data(), luc, sizeof(double) * 2 * t.tab.size());
    mdft::write_luc_file(path, t, header ? header : "c(q) table");
  });
}

int mdft_wait_selftest(int spins, void* stream) {
  return guarded([&] { mdft::launch_wait_selftest(spins, static_cast<cudaStream_t>(stream)); });
}

int mdft_wait_timeouts(int* count) {
  return guarded([&] {
    throw_if(!count, "NULL argument");
    mdft::cuda_check(cudaMemcpy(count, mdft::fft_wait_error_counter(), sizeof(int), cudaMemcpyDeviceToHost),
                     "read wait counter");
  });
}

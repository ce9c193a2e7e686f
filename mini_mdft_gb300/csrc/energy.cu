// energy.cu -- get_delta_rho and get_delta_f (common/MDFT_Solvent.hpp:578-660).
//
// get_delta_f streams xi and vexc once: each CTA takes tiles of grid points
// in turn (the (nxyz, no) rows are contiguous, so a tile is one contiguous
// run), writes delta_f = 2 rho0 xi vexc on the way, and sums each tile's
// energy terms in double-float (compensated) arithmetic.  The tile sums go to a
// small partials array; the last CTA to finish adds them in a fixed order,
// so ff is deterministic and independent of scheduling.
#include <algorithm>
#include <mutex>
#include <string>

#include "common.cuh"

namespace mdft {

namespace {

constexpr int kEnergyThreads = 256;
constexpr int kEnergyPoints = 32;  // grid points per CTA

template <typename T>
__global__ void delta_rho_kernel(const T* __restrict__ xi, T* __restrict__ dr, size_t n, T rho0) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const T x = xi[i];
    dr[i] = rho0 * (x * x - T(1));
  }
}

struct DD {
  double hi, lo;
};
__device__ __forceinline__ DD two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  const double e = (a - (s - bb)) + (b - bb);
  return DD{s, e};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  const double e = s.lo + (a.lo + b.lo);
  const double hi = s.hi + e;
  return DD{hi, e - (hi - s.hi)};
}
__device__ __forceinline__ DD dd_shfl_down(DD v, int off) {
  return DD{__shfl_down_sync(0xffffffffu, v.hi, off), __shfl_down_sync(0xffffffffu, v.lo, off)};
}
__device__ __forceinline__ DD warp_dd_sum(DD v) {
  for (int off = 16; off > 0; off >>= 1) v = dd_add(v, dd_shfl_down(v, off));
  return v;
}

// df = 2 rho0 xi vexc in the field type: double-float arithmetic and one FP64
// add to store (FP64 fields), plain float (FP32 fields, as the reference's
// float instantiation computes it)
__device__ __forceinline__ double df_value(double x, double v, DF two_rho0) {
  return df_to_double((two_rho0 * df_from_double_bits(x)) * df_from_double_bits(v));
}
__device__ __forceinline__ float df_value(float x, float v, DF two_rho0) { return two_rho0.hi * x * v; }
__device__ __forceinline__ DF as_pair(double x) { return df_from_double_bits(x); }
__device__ __forceinline__ DF as_pair(float x) { return DF(x, 0.f); }

// Tiles of kEnergyPoints grid points (contiguous runs of the (nxyz, no)
// fields).  Every element's energy term vexc w (xi^2 - 1) is formed in
// double-float on the FP32 pipes (the FP64 pipe of this GPU is 1/64 as
// wide; in FP64 this kernel is bound by it at ~5 FP64 operations per
// element) and accumulated in a Dot2 sum per thread -- or, for the FP64
// form (F64), in FP64 as the reference does; the threads' sums are combined
// as double-double values in a fixed order (warps, then the CTA's warps,
// then the CTAs' partials in the last CTA), so ff is deterministic.
template <typename T, bool F64>
__global__ void __launch_bounds__(kEnergyThreads)
delta_f_kernel(const T* __restrict__ xi, const T* __restrict__ vexc, const double* __restrict__ w,
               T* __restrict__ df, double* __restrict__ ff, size_t nxyz, int no, double rho0,
               double prefactor, double2* __restrict__ partials, unsigned* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char sm[];
  float2* ws = reinterpret_cast<float2*>(sm);  // w as double-float pairs (no)
  // per-warp sums of a tile, double-buffered by tile parity (one barrier per
  // tile): double-float pairs, or doubles for the FP64 form
  __shared__ float2 wsf[2][kEnergyThreads / 32];
  __shared__ double wsd[2][kEnergyThreads / 32];
  __shared__ bool last;
  const int tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = bd / 32;
  int buf = 0;
  for (int i = tid; i < no; i += bd) {
    const DF wd = df_from_double_bits(w[i]);
    ws[i] = make_float2(wd.hi, wd.lo);
  }
  __syncthreads();
  const float tr_h = (float)(2.0 * rho0);
  const DF two_rho0(tr_h, (float)(2.0 * rho0 - (double)tr_h)), one(1.f, 0.f);
  const double sc = rho0 * prefactor;
  const size_t ntiles = (nxyz + kEnergyPoints - 1) / kEnergyPoints;
  const int ostep = bd % no;
  // the CTA takes tiles blockIdx.x, blockIdx.x + gridDim.x, ...; each tile's
  // sum goes to its own partial
  for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const size_t pt0 = tile * kEnergyPoints;
    const int cnt = (int)min((size_t)kEnergyPoints, nxyz - pt0);
    const size_t g0 = pt0 * (size_t)no;
    const int n = cnt * no;
    Acc<DF> acc;
    acc_zero(acc);
    double acc64 = 0.0;
    int o = tid % no;
    auto one_elem = [&](int i, T x, T v) {
      if constexpr (F64) {
        df[g0 + i] = (T)(2.0 * rho0) * x * v;
        acc64 = fma((double)v * w[o], fma((double)x, (double)x, -1.0), acc64);
      } else {
        df[g0 + i] = df_value(x, v, two_rho0);
        const DF xd = as_pair(x);
        const float2 w2 = ws[o];
        acc_mac(acc, as_pair(v) * DF(w2.x, w2.y), xd * xd - one);
      }
      o += ostep;
      if (o >= no) o -= no;
    };
    int i = tid;
    for (; i + 3 * bd < n; i += 4 * bd) {  // four elements' loads in flight
      T x[4], v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        x[j] = xi[g0 + i + j * bd];
        v[j] = vexc[g0 + i + j * bd];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) one_elem(i + j * bd, x[j], v[j]);
    }
    for (; i < n; i += bd) one_elem(i, xi[g0 + i], vexc[g0 + i]);
    // the tile's sum: warps by shuffles, then warp 0 over the warps --
    // double-float additions on the FP32 pipe (plain FP64 adds for the FP64
    // form); the tile's share of ff = rho0 prefactor sum becomes a
    // double-double partial
    if constexpr (F64) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc64 += __shfl_down_sync(0xffffffffu, acc64, off);
      if (lane == 0) wsd[buf][wid] = acc64;
    } else {
      DF a = acc_get(acc);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        a = a + DF(__shfl_down_sync(0xffffffffu, a.hi, off), __shfl_down_sync(0xffffffffu, a.lo, off));
      if (lane == 0) wsf[buf][wid] = make_float2(a.hi, a.lo);
    }
    __syncthreads();
    if (wid == 0) {
      if constexpr (F64) {
        double t = lane < nw ? wsd[buf][lane] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
        if (lane == 0) partials[tile] = make_double2(t * sc, 0.0);
      } else {
        const float2 q = lane < nw ? wsf[buf][lane] : make_float2(0.f, 0.f);
        DF t(q.x, q.y);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
          t = t + DF(__shfl_down_sync(0xffffffffu, t.hi, off), __shfl_down_sync(0xffffffffu, t.lo, off));
        if (lane == 0) {
          const DD u = two_sum((double)t.hi * sc, (double)t.lo * sc);
          partials[tile] = make_double2(u.hi, u.lo);
        }
      }
    }
    buf ^= 1;
  }
  if (tid == 0) {
    __threadfence();
    const unsigned done = atomicAdd(counter, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || tid >= 32) return;
  __threadfence();
  DD acc2{0.0, 0.0};
  for (size_t b = tid; b < ntiles; b += 32) {
    const double2 q = __ldcg(&partials[b]);
    acc2 = dd_add(acc2, DD{q.x, q.y});
  }
  acc2 = warp_dd_sum(acc2);
  if (tid == 0) {
    *ff = acc2.hi + acc2.lo;
    *counter = 0u;  // leave the counter ready for the next call
  }
}

}  // namespace

size_t delta_f_partials(size_t nxyz, int) {
  return (nxyz + kEnergyPoints - 1) / kEnergyPoints;
}

template <typename T>
void launch_delta_rho(const T* xi, T* dr, size_t n, double rho0, cudaStream_t s) {
  if (n == 0) return;
  size_t nb = (n + kEnergyThreads - 1) / kEnergyThreads;
  if (nb > 152 * 64) nb = 152 * 64;
  clear_stale_error();
  delta_rho_kernel<T><<<(unsigned)nb, kEnergyThreads, 0, s>>>(xi, dr, n, (T)rho0);
  launch_check("delta_rho kernel launch");
}

template <typename T>
void launch_delta_f(const T* xi, const T* vexc, const double* w, T* df, double* ff, size_t nxyz,
                    int no, double rho0, double prefactor, void* work, cudaStream_t s, bool fp64) {
  const size_t nb = delta_f_partials(nxyz, no);
  throw_if(nb > 0x7fffffffULL, "grid too large", 4);
  const size_t smem = sizeof(float2) * (size_t)no;
  throw_if(smem > 48 * 1024, "too many orientations for the energy kernel", 4);
  double2* partials = static_cast<double2*>(work);
  unsigned* counter = reinterpret_cast<unsigned*>(partials + nb);
  if (nb == 0) {
    cuda_check(cudaMemsetAsync(ff, 0, sizeof(double), s), "cudaMemsetAsync(ff)");
    return;
  }
  clear_stale_error();
  // at most 8 CTAs per SM, each looping over tiles (one partial per tile)
  const unsigned grid = (unsigned)std::min<size_t>(nb, 152 * 8);
  if (fp64 && sizeof(T) == 8)
    delta_f_kernel<T, true><<<grid, kEnergyThreads, smem, s>>>(xi, vexc, w, df, ff, nxyz, no, rho0, prefactor,
                                                               partials, counter);
  else
    delta_f_kernel<T, false><<<grid, kEnergyThreads, smem, s>>>(xi, vexc, w, df, ff, nxyz, no, rho0, prefactor,
                                                                partials, counter);
  launch_check("delta_f kernel launch");
}

template void launch_delta_rho<double>(const double*, double*, size_t, double, cudaStream_t);
template void launch_delta_rho<float>(const float*, float*, size_t, double, cudaStream_t);
template void launch_delta_f<double>(const double*, const double*, const double*, double*, double*,
                                     size_t, int, double, double, void*, cudaStream_t, bool);
template void launch_delta_f<float>(const float*, const float*, const double*, float*, double*,
                                    size_t, int, double, double, void*, cudaStream_t, bool);


// ---------------------------------------------------------------------------
// get_delta_f without any device allocation.
//
// Some callers of this library cannot allocate device memory while they run
// the solve: an application that hands the whole GPU to its own pool
// allocator up front (as Kokkos-based codes often do) and treats any
// cudaMalloc behind its back as a budget violation, or a time-critical loop
// that must not pay for, or serialise on, an allocation call.  For them
// mdft_get_delta_f_noalloc runs the same reduction as mdft_get_delta_f with
// its per-CTA partial sums kept in one fixed array in the library's own
// device memory instead of a stream-ordered temporary.
//
// The array holds kNoAllocMaxPartials partials (one per 32 grid points), so
// grids of up to 2,097,152 points (128^3) are accepted and larger ones are
// rejected with an error; it costs 1 MiB of device memory on every GPU that
// loads the library, held until the process exits.  All calls share it and
// it keeps the last call's contents, so calls that overlap on the GPU (on
// different streams, or from different threads) race and must be ordered by
// the caller.  The completion counter is cleared on the caller's stream at
// the start of every call.  The first call on a device looks up the array's
// device address (cudaGetSymbolAddress) for that device and caches it; make
// that first call before any stream capture.
// ---------------------------------------------------------------------------
namespace {
constexpr size_t kNoAllocMaxPartials = size_t(1) << 16;
constexpr size_t kNoAllocBytes = kNoAllocMaxPartials * sizeof(double2) + 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device, looked up once
// per device with that device current.
void* noalloc_scratch_for_current_device() {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  throw_if(dev < 0 || dev >= kMaxDevices, "device index out of range for the fixed scratch table");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    cuda_check(cudaGetSymbolAddress(&ptr, g_noalloc_scratch), "cudaGetSymbolAddress(fixed scratch)");
    throw_if(ptr == nullptr, "cudaGetSymbolAddress returned a null scratch address", 2);
    g_noalloc_ptr[dev] = ptr;
  }
  return g_noalloc_ptr[dev];
}
}  // namespace

}  // namespace mdft

extern "C" int mdft_get_delta_f_noalloc(const void* xi, const void* vexc, const double* w,
                                        void* delta_f, double* ff_dev, size_t nxyz, int no,
                                        double rho0, double prefactor, int precision,
                                        void* stream) {
  using namespace mdft;
  try {
    throw_if(precision < 0 || precision > 2, "precision must be MDFT_F64, MDFT_F32 or MDFT_F64_DF");
    throw_if(no <= 0, "angular grid size must be positive");
    throw_if(!ff_dev, "NULL argument");
    throw_if(nxyz > 0 && (!xi || !vexc || !w || !delta_f), "NULL argument");
    const size_t nb = delta_f_partials(nxyz, no);
    throw_if(nb > kNoAllocMaxPartials,
             "mdft_get_delta_f_noalloc: " + std::to_string(nxyz) +
                 " grid points exceed the fixed scratch limit of " +
                 std::to_string(kNoAllocMaxPartials * 32) + " points",
             4);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char* scratch = static_cast<unsigned char*>(noalloc_scratch_for_current_device());
    // partials first, then the completion counter, which must start at zero
    unsigned char* counter = scratch + sizeof(double2) * nb;
    cuda_check(cudaMemsetAsync(counter, 0, sizeof(unsigned), s), "cudaMemsetAsync(fixed scratch counter)");
    if (precision != 1)  // MDFT_F64 and MDFT_F64_DF fields are double
      launch_delta_f<double>(static_cast<const double*>(xi), static_cast<const double*>(vexc), w,
                             static_cast<double*>(delta_f), ff_dev, nxyz, no, rho0, prefactor, scratch, s,
                             precision == 0);
    else
      launch_delta_f<float>(static_cast<const float*>(xi), static_cast<const float*>(vexc), w,
                            static_cast<float*>(delta_f), ff_dev, nxyz, no, rho0, prefactor, scratch, s, false);
    return 0;
  } catch (const Error& e) {
    return record_error(e.code, e.what());
  } catch (const std::exception& e) {
    return record_error(1, e.what());
  }
}

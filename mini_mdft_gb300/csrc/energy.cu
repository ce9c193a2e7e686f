// energy.cu -- get_delta_rho and get_delta_f (common/MDFT_Solvent.hpp:578-660).
//
// get_delta_f streams xi and vexc once: each CTA takes one contiguous run of
// grid points (the (nxyz, no) rows are contiguous), writes
// delta_f = 2 rho0 xi vexc on the way, and sums its energy terms in
// double-float (compensated) arithmetic.  The grid is one wave of CTAs of
// equal runs; each CTA leaves one partial sum and the last CTA to finish adds
// them in a fixed order, so ff is deterministic and independent of
// scheduling.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <string>

#include "common.cuh"

namespace mdft {

namespace {

constexpr int kEnergyThreads = 256;
constexpr int kEnergyPoints = 32;  // grid points per partial slot of the scratch (sizing unit)

template <typename T>
__global__ void delta_rho_kernel(const T* __restrict__ xi, T* __restrict__ dr, size_t n, T rho0) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const T x = xi[i];
    dr[i] = rho0 * (x * x - T(1));
  }
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

// One contiguous run of `chunk` grid points per CTA (the last CTA's run may
// be shorter).  Every element's energy term vexc w (xi^2 - 1) is formed in
// double-float on the FP32 pipes (the FP64 pipe of this GPU is 1/64 as wide;
// in FP64 this kernel is bound by it at ~5 FP64 operations per element) and
// accumulated in a Dot2 sum per thread -- or, for the FP64 form (F64), in
// FP64 as the reference does.  The threads' sums are combined in a fixed
// order (warps by shuffles, then warp 0 over the CTA's warps) into one
// partial per CTA; the last CTA to finish adds the partials with all its
// threads in the same fixed order.  The combining runs in double-float on
// the FP32 pipes (plain FP64 adds for the FP64 form): a double-double sum of
// ~1000 partials by one warp spends hundreds of microseconds on the FP64
// pipe while every other SM idles.
template <typename T, bool F64>
__global__ void __launch_bounds__(kEnergyThreads)
delta_f_kernel(const T* __restrict__ xi, const T* __restrict__ vexc, const double* __restrict__ w,
               T* __restrict__ df, double* __restrict__ ff, size_t nxyz, int no, size_t chunk, double rho0,
               double prefactor, void* __restrict__ partials, unsigned* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char sm[];
  float2* ws = reinterpret_cast<float2*>(sm);  // w as double-float pairs (no)
  __shared__ float2 wsf[kEnergyThreads / 32];  // per-warp sums (double-float)
  __shared__ double wsd[kEnergyThreads / 32];  // per-warp sums (FP64 form)
  __shared__ bool last;
  float2* pf = static_cast<float2*>(partials);
  double* pd = static_cast<double*>(partials);
  const int tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = bd / 32;
  if constexpr (!F64) {
    for (int i = tid; i < no; i += bd) {
      const DF wd = df_from_double_bits(w[i]);
      ws[i] = make_float2(wd.hi, wd.lo);
    }
    __syncthreads();
  }
  const float tr_h = (float)(2.0 * rho0);
  const DF two_rho0(tr_h, (float)(2.0 * rho0 - (double)tr_h)), one(1.f, 0.f);
  const double sc = rho0 * prefactor;
  const size_t pt0 = (size_t)blockIdx.x * chunk;
  const int n = pt0 < nxyz ? (int)((min(chunk, nxyz - pt0)) * (size_t)no) : 0;
  const T* __restrict__ xs = xi + pt0 * (size_t)no;
  const T* __restrict__ vs = vexc + pt0 * (size_t)no;
  T* __restrict__ ds = df + pt0 * (size_t)no;
  Acc<DF> acc;
  acc_zero(acc);
  double acc64 = 0.0;
  // the run starts on a grid point, so element i has orientation i mod no
  int o = tid % no;
  const int ostep = bd % no;
  auto one_elem = [&](int i, T x, T v) {
    if constexpr (F64) {
      ds[i] = (T)(2.0 * rho0) * x * v;
      acc64 = fma((double)v * w[o], fma((double)x, (double)x, -1.0), acc64);
    } else {
      ds[i] = df_value(x, v, two_rho0);
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
      x[j] = xs[i + j * bd];
      v[j] = vs[i + j * bd];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) one_elem(i + j * bd, x[j], v[j]);
  }
  for (; i < n; i += bd) one_elem(i, xs[i], vs[i]);

  // the CTA's sum: warps by shuffles, then warp 0 over the warps; the
  // partial is the unscaled sum (double-float pair, or a double)
  if constexpr (F64) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc64 += __shfl_down_sync(0xffffffffu, acc64, off);
    if (lane == 0) wsd[wid] = acc64;
  } else {
    DF a = acc_get(acc);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      a = a + DF(__shfl_down_sync(0xffffffffu, a.hi, off), __shfl_down_sync(0xffffffffu, a.lo, off));
    if (lane == 0) wsf[wid] = make_float2(a.hi, a.lo);
  }
  __syncthreads();
  if (wid == 0) {
    if constexpr (F64) {
      double t = lane < nw ? wsd[lane] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
      if (lane == 0) pd[blockIdx.x] = t;
    } else {
      const float2 q = lane < nw ? wsf[lane] : make_float2(0.f, 0.f);
      DF t(q.x, q.y);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        t = t + DF(__shfl_down_sync(0xffffffffu, t.hi, off), __shfl_down_sync(0xffffffffu, t.lo, off));
      if (lane == 0) pf[blockIdx.x] = make_float2(t.hi, t.lo);
    }
    if (tid == 0) {
      __threadfence();
      last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
  }
  __syncthreads();  // also ends warp 0's reads of wsf / wsd
  if (!last) return;
  __threadfence();
  // the last CTA: thread t adds partials t, t + bd, ...; then the warps by
  // shuffles and warp 0 over the warps, as above
  if constexpr (F64) {
    double t = 0.0;
    for (unsigned b = tid; b < gridDim.x; b += bd) t += __ldcg(&pd[b]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
    if (lane == 0) wsd[wid] = t;
    __syncthreads();
    if (wid == 0) {
      t = lane < nw ? wsd[lane] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
      if (lane == 0) {
        *ff = t * sc;
        *counter = 0u;  // leave the counter ready for the next call
      }
    }
  } else {
    DF t(0.f, 0.f);
    for (unsigned b = tid; b < gridDim.x; b += bd) {
      const float2 q = __ldcg(&pf[b]);
      t = t + DF(q.x, q.y);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      t = t + DF(__shfl_down_sync(0xffffffffu, t.hi, off), __shfl_down_sync(0xffffffffu, t.lo, off));
    if (lane == 0) wsf[wid] = make_float2(t.hi, t.lo);
    __syncthreads();
    if (wid == 0) {
      const float2 q = lane < nw ? wsf[lane] : make_float2(0.f, 0.f);
      t = DF(q.x, q.y);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        t = t + DF(__shfl_down_sync(0xffffffffu, t.hi, off), __shfl_down_sync(0xffffffffu, t.lo, off));
      if (lane == 0) {
        *ff = fma(sc, f2d_bits(t.hi), sc * f2d_bits(t.lo));
        *counter = 0u;  // leave the counter ready for the next call
      }
    }
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

// One wave: as many CTAs as the device holds at once (SMs x resident CTAs of
// this kernel), each with an equal run of grid points, and no more CTAs than
// the scratch has partial slots (one per kEnergyPoints points).  The grid
// depends only on the device and the problem, so ff does too.
// SMs x resident CTAs of one delta_f kernel instance at a shared-memory size,
// per device: queried once and cached (a query per call costs microseconds
// of host time on every get_delta_f)
template <typename T, bool F64>
size_t delta_f_wave(size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<int, size_t>, size_t> cache;
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({dev, smem});
  if (it != cache.end()) return it->second;
  int sms = 0, per_sm = 0;
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, delta_f_kernel<T, F64>, kEnergyThreads, smem),
             "cudaOccupancyMaxActiveBlocksPerMultiprocessor(delta_f)");
  const size_t wave = (size_t)std::max(1, sms) * (size_t)std::max(1, per_sm);
  cache[{dev, smem}] = wave;
  return wave;
}

template <typename T, bool F64>
unsigned delta_f_grid(size_t nxyz, size_t nb, size_t smem, size_t* chunk) {
  const size_t wave = delta_f_wave<T, F64>(smem);
  const size_t want = std::min(nb, wave);
  *chunk = (nxyz + want - 1) / want;
  return (unsigned)((nxyz + *chunk - 1) / *chunk);  // CTAs with a non-empty run
}

template <typename T>
void launch_delta_f(const T* xi, const T* vexc, const double* w, T* df, double* ff, size_t nxyz,
                    int no, double rho0, double prefactor, void* work, cudaStream_t s, bool fp64) {
  const size_t nb = delta_f_partials(nxyz, no);
  throw_if(nb > 0x7fffffffULL, "grid too large", 4);
  const size_t smem = sizeof(float2) * (size_t)no;
  throw_if(smem > 48 * 1024, "too many orientations for the energy kernel", 4);
  unsigned* counter = reinterpret_cast<unsigned*>(static_cast<double2*>(work) + nb);
  if (nb == 0) {
    cuda_check(cudaMemsetAsync(ff, 0, sizeof(double), s), "cudaMemsetAsync(ff)");
    return;
  }
  const bool f64 = fp64 && sizeof(T) == 8;
  size_t chunk = 0;
  const unsigned grid = f64 ? delta_f_grid<T, true>(nxyz, nb, smem, &chunk)
                            : delta_f_grid<T, false>(nxyz, nb, smem, &chunk);
  // a CTA's run indexes its elements with int
  throw_if(chunk * (size_t)no > (size_t)0x7fffffff - 4 * kEnergyThreads, "grid too large", 4);
  clear_stale_error();
  if (f64)
    delta_f_kernel<T, true><<<grid, kEnergyThreads, smem, s>>>(xi, vexc, w, df, ff, nxyz, no, chunk, rho0,
                                                               prefactor, work, counter);
  else
    delta_f_kernel<T, false><<<grid, kEnergyThreads, smem, s>>>(xi, vexc, w, df, ff, nxyz, no, chunk, rho0,
                                                                prefactor, work, counter);
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
// The array holds kNoAllocMaxPartials partial slots (one per 32 grid points,
// the scratch sizing of every get_delta_f call; a call fills one per CTA), so
// grids of up to 2,097,152 points (128^3) are accepted and larger ones are
// rejected with an error; it costs 1 MiB of device memory on every GPU that
// loads the library, held until the process exits.  All calls share it and
// it keeps the last call's contents, so calls that overlap on the GPU (on
// different streams, or from different threads) race and must be ordered by
// the caller.  The completion counter is cleared on the caller's stream at
// the start of every call.  Every call made outside stream capture looks up
// the array's device address (cudaGetSymbolAddress) on the current device
// and caches it, so a context torn down and created again (cudaDeviceReset)
// is seen at the next such call; a call on a capturing stream uses the
// cached address, so the first call on a device must come before any stream
// capture.
// ---------------------------------------------------------------------------
namespace {
constexpr size_t kNoAllocMaxPartials = size_t(1) << 16;
constexpr size_t kNoAllocBytes = kNoAllocMaxPartials * sizeof(double2) + 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device.  Looked up with
// that device current whenever `stream` is not capturing (a reset context
// loads the module again, possibly at another address); a capturing stream
// takes the address cached by an earlier call.
void* noalloc_scratch_for_current_device(cudaStream_t stream) {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  throw_if(dev < 0 || dev >= kMaxDevices, "device index out of range for the fixed scratch table");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cuda_check(cudaStreamIsCapturing(stream, &cap), "cudaStreamIsCapturing");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* ptr = nullptr;
    cuda_check(cudaGetSymbolAddress(&ptr, g_noalloc_scratch), "cudaGetSymbolAddress(fixed scratch)");
    throw_if(ptr == nullptr, "cudaGetSymbolAddress returned a null scratch address", 2);
    g_noalloc_ptr[dev] = ptr;
  }
  throw_if(!g_noalloc_ptr[dev],
           "mdft_get_delta_f_noalloc: the first call on a device must come before any stream capture", 2);
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
    unsigned char* scratch = static_cast<unsigned char*>(noalloc_scratch_for_current_device(s));
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

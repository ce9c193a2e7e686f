// energy.cu -- get_delta_rho and get_delta_f (common/MDFT_Solvent.hpp:578-660).
//
// get_delta_f streams xi and vexc once: each CTA stages a tile of grid points
// (the (nxyz, no) rows are contiguous, so the tile is one contiguous run),
// writes delta_f = 2 rho0 xi vexc on the way, sums each point's orientations
// in index order, and reduces the per-point energies of the tile with
// compensated (two-sum) arithmetic.  The tile sums go to a small partials
// array; the last CTA to finish adds them in a fixed order, so ff is
// deterministic and independent of scheduling.
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

template <typename T>
__global__ void __launch_bounds__(kEnergyThreads)
delta_f_kernel(const T* __restrict__ xi, const T* __restrict__ vexc, const double* __restrict__ w,
               T* __restrict__ df, double* __restrict__ ff, size_t nxyz, int no, double rho0,
               double prefactor, double2* __restrict__ partials, unsigned* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char sm[];
  double* ws = reinterpret_cast<double*>(sm);            // (no)
  double* term = ws + no;                                // (kEnergyPoints * no)
  __shared__ double ppt[kEnergyPoints];
  __shared__ bool last;
  const int tid = threadIdx.x, bd = blockDim.x;
  const size_t pt0 = (size_t)blockIdx.x * kEnergyPoints;
  const int cnt = (int)min((size_t)kEnergyPoints, nxyz - pt0);
  for (int i = tid; i < no; i += bd) ws[i] = w[i];
  __syncthreads();
  const size_t g0 = pt0 * (size_t)no;
  const T two_rho0 = (T)(2.0 * rho0);
  for (int i = tid; i < cnt * no; i += bd) {
    const T x = xi[g0 + i], v = vexc[g0 + i];
    df[g0 + i] = two_rho0 * x * v;
    term[i] = (double)v * ws[i % no] * ((double)x * (double)x - 1.0);
  }
  __syncthreads();
  if (tid < kEnergyPoints) {
    double s = 0.0;
    if (tid < cnt)
      for (int io = 0; io < no; ++io) s += term[tid * no + io];
    ppt[tid] = tid < cnt ? rho0 * s * prefactor : 0.0;
  }
  __syncthreads();
  if (tid < 32) {
    DD v = warp_dd_sum(DD{ppt[tid], 0.0});
    if (tid == 0) {
      partials[blockIdx.x] = make_double2(v.hi, v.lo);
      __threadfence();
      const unsigned done = atomicAdd(counter, 1u);
      last = (done == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last || tid >= 32) return;
  __threadfence();
  DD acc{0.0, 0.0};
  for (unsigned b = tid; b < gridDim.x; b += 32) {
    const double2 q = __ldcg(&partials[b]);
    acc = dd_add(acc, DD{q.x, q.y});
  }
  acc = warp_dd_sum(acc);
  if (tid == 0) {
    *ff = acc.hi + acc.lo;
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
                    int no, double rho0, double prefactor, void* work, cudaStream_t s) {
  const size_t nb = delta_f_partials(nxyz, no);
  throw_if(nb > 0x7fffffffULL, "grid too large", 4);
  const size_t smem = sizeof(double) * ((size_t)no + (size_t)kEnergyPoints * no);
  throw_if(smem > 200 * 1024, "too many orientations for the energy kernel", 4);
  if (smem > 48 * 1024) allow_max_smem(delta_f_kernel<T>, smem, "delta_f smem attribute");
  double2* partials = static_cast<double2*>(work);
  unsigned* counter = reinterpret_cast<unsigned*>(partials + nb);
  if (nb == 0) {
    cuda_check(cudaMemsetAsync(ff, 0, sizeof(double), s), "cudaMemsetAsync(ff)");
    return;
  }
  clear_stale_error();
  delta_f_kernel<T><<<(unsigned)nb, kEnergyThreads, smem, s>>>(xi, vexc, w, df, ff, nxyz, no, rho0,
                                                               prefactor, partials, counter);
  launch_check("delta_f kernel launch");
}

template void launch_delta_rho<double>(const double*, double*, size_t, double, cudaStream_t);
template void launch_delta_rho<float>(const float*, float*, size_t, double, cudaStream_t);
template void launch_delta_f<double>(const double*, const double*, const double*, double*, double*,
                                     size_t, int, double, double, void*, cudaStream_t);
template void launch_delta_f<float>(const float*, const float*, const double*, float*, double*,
                                    size_t, int, double, double, void*, cudaStream_t);


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
                             static_cast<double*>(delta_f), ff_dev, nxyz, no, rho0, prefactor, scratch, s);
    else
      launch_delta_f<float>(static_cast<const float*>(xi), static_cast<const float*>(vexc), w,
                            static_cast<float*>(delta_f), ff_dev, nxyz, no, rho0, prefactor, scratch, s);
    return 0;
  } catch (const Error& e) {
    return record_error(e.code, e.what());
  } catch (const std::exception& e) {
    return record_error(1, e.what());
  }
}

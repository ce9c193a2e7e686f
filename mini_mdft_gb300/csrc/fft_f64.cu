// fft_f64.cu -- instantiates the axis FFTs of fft.cuh for the f64
// precision (one translation unit per precision so the builds run in
// parallel).
#include <map>
#include <mutex>

#include "fft.cuh"
#include "../../include/mdft_gb300.h"

namespace mdft {

bool fft_factor(int n, FftAxis& a) { return fft_factor_impl(n, a); }

namespace {
std::mutex g_wait_mu;
std::map<int, WaitStatus> g_wait_status;
}  // namespace

const WaitStatus& device_wait_status() {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_wait_mu);
  WaitStatus& w = g_wait_status[dev];
  if (!w.count) {
    void* h = nullptr;
    cuda_check(cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable),
               "cudaHostAlloc(wait flag)");
    *static_cast<volatile int*>(h) = 0;
    void* d = nullptr;
    cuda_check(cudaHostGetDevicePointer(&d, h, 0), "cudaHostGetDevicePointer(wait flag)");
    int* c = nullptr;
    cuda_check(cudaMalloc(&c, sizeof(int)), "cudaMalloc(wait error counter)");
    cuda_check(cudaMemset(c, 0, sizeof(int)), "cudaMemset(wait error counter)");
    w.flag_host = static_cast<volatile int*>(h);
    w.flag_dev = static_cast<int*>(d);
    w.count = c;
  }
  return w;
}

int* fft_wait_error_counter() { return device_wait_status().count; }

void check_device_waits() {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_wait_mu);
  auto it = g_wait_status.find(dev);
  // no record yet: no kernel with a bounded wait was set up on this device
  if (it == g_wait_status.end() || !it->second.flag_host) return;
  if (*it->second.flag_host) {
    *it->second.flag_host = 0;
    throw Error(MDFT_ERR_TIMEOUT,
                "a bounded device wait ran out in a kernel launched earlier on this device "
                "(an asynchronous tile copy or a persistent kernel's flag did not arrive in time); "
                "the results of that launch are wrong (mdft_wait_timeouts gives the count)");
  }
}

// One CTA whose wait on an mbarrier that nothing arrives on runs out after
// `spins` polls and is recorded like a timed-out tile copy (the error path of
// the bounded waits, exercised without a fault or a hang).
__global__ void wait_selftest_kernel(int* count, int* flag, long long spins) {
  __shared__ __align__(8) unsigned long long bar;
  const unsigned b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool late = !mbar_wait(b, 0, spins);
  if (__syncthreads_or(late) && threadIdx.x == 0) note_wait_timeout(count, flag);
}

void launch_wait_selftest(long long spins, cudaStream_t s) {
  throw_if(spins < 1 || spins > (1LL << 20), "spins must be in [1, 2^20]");
  const WaitStatus& w = device_wait_status();
  clear_stale_error();
  wait_selftest_kernel<<<1, 32, 0, s>>>(w.count, w.flag_dev, spins);
  launch_check("wait self-test launch");
}

template void fft_axis_finish<double, double, double>(FftAxis&);
template void launch_fft_axis<double, double, double>(const FftAxis&, void*, int, cudaStream_t);

}  // namespace mdft

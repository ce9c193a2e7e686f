// fft_f64.cu -- instantiates the axis FFTs of fft.cuh for the f64
// precision (one translation unit per precision so the builds run in
// parallel).
#include <map>
#include <mutex>

#include "fft.cuh"

namespace mdft {

bool fft_factor(int n, FftAxis& a) { return fft_factor_impl(n, a); }

int* fft_wait_error_counter() {
  static std::mutex mu;
  static std::map<int, int*> per_device;
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  int*& p = per_device[dev];
  if (!p) {
    cuda_check(cudaMalloc(&p, sizeof(int)), "cudaMalloc(wait error counter)");
    cuda_check(cudaMemset(p, 0, sizeof(int)), "cudaMemset(wait error counter)");
  }
  return p;
}

template void fft_axis_finish<double, double, double>(FftAxis&);
template void launch_fft_axis<double, double, double>(const FftAxis&, void*, int, cudaStream_t);

}  // namespace mdft

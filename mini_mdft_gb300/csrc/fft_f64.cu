// fft_f64.cu -- instantiates the axis FFTs of fft.cuh for the f64
// precision (one translation unit per precision so the builds run in
// parallel).
#include "fft.cuh"

namespace mdft {

bool fft_factor(int n, FftAxis& a) { return fft_factor_impl(n, a); }

template void fft_axis_finish<double, double, double>(FftAxis&);
template void launch_fft_axis<double, double, double>(const FftAxis&, void*, int, cudaStream_t);

}  // namespace mdft

// fft_f32.cu -- instantiates the axis FFTs of fft.cuh for the f32
// precision (one translation unit per precision so the builds run in
// parallel).
#include "fft.cuh"

namespace mdft {

template void fft_axis_finish<float, float, float>(FftAxis&);
template void launch_fft_axis<float, float, float>(const FftAxis&, void*, int, cudaStream_t);

}  // namespace mdft

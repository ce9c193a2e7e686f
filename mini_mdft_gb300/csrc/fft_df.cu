// fft_df.cu -- instantiates the axis FFTs of fft.cuh for the df
// precision (one translation unit per precision so the builds run in
// parallel).
#include "fft.cuh"

namespace mdft {

template void fft_axis_finish<double, double, DF>(FftAxis&);
template void launch_fft_axis<double, double, DF>(const FftAxis&, void*, int, cudaStream_t);
template void fft_axis_finish<double, DF, DF>(FftAxis&);
template void launch_fft_axis<double, DF, DF>(const FftAxis&, void*, int, cudaStream_t);
template void fft_axis_finish<DF, DF, DF>(FftAxis&);
template void launch_fft_axis<DF, DF, DF>(const FftAxis&, void*, int, cudaStream_t);
template void fft_axis_finish<DF, double, DF>(FftAxis&);
template void launch_fft_axis<DF, double, DF>(const FftAxis&, void*, int, cudaStream_t);

}  // namespace mdft

// oz_r2.cuh -- the split lane kernel of oz.cuh specialised for mrso = 2
// (the water-like molecules of the benchmark workloads) on packed storage;
// included by oz_r2_f32.cu and oz_r2_df.cu, which instantiate it.
#pragma once
#include "oz.cuh"

namespace mdft {

template <typename C, int MMAX>
void oz_lane_r2_attr(size_t smem) {
  allow_max_smem(oz_lane_kernel<C, C, MMAX, 2>, smem, "oz smem attribute");
}

template <typename C, int MMAX>
void oz_lane_r2_launch(const OzPlan& P, Cx<C>* p, dim3 grid, dim3 block, cudaStream_t s) {
  oz_lane_kernel<C, C, MMAX, 2><<<grid, block, P.smem, s>>>(P, p);
}

}  // namespace mdft

#define MDFT_OZ_R2_INSTANTIATE(C, K)                                                      \
  template void mdft::oz_lane_r2_attr<C, K>(size_t);                                      \
  template void mdft::oz_lane_r2_launch<C, K>(const mdft::OzPlan&, mdft::Cx<C>*, dim3, dim3, \
                                              cudaStream_t);

// oz_f32.cu -- instantiates the k-space step of oz.cuh for storage float,
// arithmetic float (one translation unit per precision so the builds run in
// parallel).
#include "oz.cuh"

namespace mdft {

template void oz_plan_finish<float, float>(OzPlan&);
template void oz_build_rtab<float>(const OzPlan&, DevBuf&);
template void launch_oz<float, float>(const OzPlan&, Cx<float>*, cudaStream_t);
template void oz_lane_attr<float, float>(const OzPlan&);

}  // namespace mdft

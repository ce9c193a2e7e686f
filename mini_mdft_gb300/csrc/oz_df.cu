// oz_df.cu -- instantiates the k-space step of oz.cuh for storage double,
// arithmetic DF (one translation unit per precision so the builds run in
// parallel).
#include "oz.cuh"

namespace mdft {

template void oz_plan_finish<double, DF>(OzPlan&);
template void oz_build_rtab<DF>(const OzPlan&, DevBuf&);
template void launch_oz<double, DF>(const OzPlan&, Cx<double>*, cudaStream_t);
template void launch_oz<DF, DF>(const OzPlan&, Cx<DF>*, cudaStream_t);
template void oz_lane_attr<DF, DF>(const OzPlan&);
template void oz_lane_attr<double, DF>(const OzPlan&);

}  // namespace mdft

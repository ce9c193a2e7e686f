// oz_f64.cu -- instantiates the k-space step of oz.cuh for storage double,
// arithmetic double (one translation unit per precision so the builds run in
// parallel).
#include "oz.cuh"

namespace mdft {

template void oz_plan_finish<double, double>(OzPlan&);
template void oz_build_rtab<double>(const OzPlan&, DevBuf&);
template void launch_oz<double, double>(const OzPlan&, Cx<double>*, cudaStream_t);

}  // namespace mdft

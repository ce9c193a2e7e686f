// angular_fast_f64.cu -- instantiates the compile-time-shape angular
// kernels of angular_fast.cuh for storage double, arithmetic double (one
// translation unit per precision so the builds run in parallel).
#include "angular_fast.cuh"

namespace mdft {

bool ang_fast_supported(int mmax, int mrso) { return ang_fast_supported_impl(mmax, mrso); }

template void ang_fast_setup<double, double>(const AngPlan&);
template void ang_fast_a2p<double, double>(const AngPlan&, const double*, Cx<double>*, bool, double, cudaStream_t);
template void ang_fast_p2a<double, double>(const AngPlan&, const Cx<double>*, double*, cudaStream_t);

}  // namespace mdft

// Instantiations of the photon kernel on the counter-based Philox stream (production mode).
#include "photon_kernel.cuh"

namespace clr {
cudaError_t launch_philox(const LaunchArgs& a) {
    return a.records ? launch_t<PhiloxMode, true, false>(a) : launch_t<PhiloxMode, false, false>(a);
}
int occupancy_philox(bool records) {
    return records ? occupancy_t<PhiloxMode, true, false>() : occupancy_t<PhiloxMode, false, false>();
}
}  // namespace clr

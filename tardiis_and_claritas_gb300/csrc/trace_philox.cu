// Instantiations of the persistent photon kernel on the counter-based Philox stream (production mode).
#include "wavefront.cuh"

namespace clr {
cudaError_t launch_philox(const LaunchArgs& a) {
    return a.records ? launch_t<PhiloxMode, true, false>(a) : launch_t<PhiloxMode, false, false>(a);
}
int occupancy_philox(bool records) {
    return records ? occupancy_t<PhiloxMode, true, false>() : occupancy_t<PhiloxMode, false, false>();
}
}  // namespace clr

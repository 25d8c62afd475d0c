// Instantiations of the photon kernel on the counter-based Philox stream (production mode).
#include "wavefront.cuh"

namespace clr {
cudaError_t launch_philox(const LaunchArgs& a) {
    return a.records ? launch_t<PhiloxMode, true, false>(a) : launch_t<PhiloxMode, false, false>(a);
}
int occupancy_philox(bool records) {
    return records ? occupancy_t<PhiloxMode, true, false>() : occupancy_t<PhiloxMode, false, false>();
}
cudaError_t wave_run_philox(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes, int* passes) {
    return w.records ? wave_run_t<PhiloxMode, true>(w, num_sms, st, max_passes, passes)
                     : wave_run_t<PhiloxMode, false>(w, num_sms, st, max_passes, passes);
}
}  // namespace clr

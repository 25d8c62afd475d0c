// Instantiations of the wavefront engine on the counter-based Philox stream (production mode); a unit of
// its own so that it compiles in parallel with the persistent kernel's.
#include "wavefront.cuh"

namespace clr {
cudaError_t wave_run_philox(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes, WaveRunInfo* info) {
    return w.records ? wave_run_t<PhiloxMode, true>(w, num_sms, st, max_passes, info)
                     : wave_run_t<PhiloxMode, false>(w, num_sms, st, max_passes, info);
}
}  // namespace clr

// Instantiations of the photon kernel on the reference's xorshift streams (parity mode).
#include "wavefront.cuh"

namespace clr {
cudaError_t launch_xor(const LaunchArgs& a) {
    return a.records ? launch_t<XorMode, true, false>(a) : launch_t<XorMode, false, false>(a);
}
int occupancy_xor(bool records) { return records ? occupancy_t<XorMode, true, false>() : occupancy_t<XorMode, false, false>(); }
cudaError_t wave_run_xor(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes, int* passes) {
    return w.records ? wave_run_t<XorMode, true>(w, num_sms, st, max_passes, passes)
                     : wave_run_t<XorMode, false>(w, num_sms, st, max_passes, passes);
}
size_t wave_ray_bytes() { return sizeof(Ray); }
size_t wave_lane_bytes(int rng_mode) {
    return rng_mode == CLR_RNG_PHILOX ? sizeof(PhiloxMode::Lane) : sizeof(XorMode::Lane);
}
}  // namespace clr

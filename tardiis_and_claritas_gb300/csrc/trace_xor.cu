// Instantiations of the persistent photon kernel on the reference's xorshift streams (parity mode).
#include "wavefront.cuh"

namespace clr {
cudaError_t launch_xor(const LaunchArgs& a) {
    return a.records ? launch_t<XorMode, true, false>(a) : launch_t<XorMode, false, false>(a);
}
int occupancy_xor(bool records) { return records ? occupancy_t<XorMode, true, false>() : occupancy_t<XorMode, false, false>(); }
size_t wave_ray_bytes() { return sizeof(Ray); }
size_t wave_lane_bytes(int rng_mode) {
    return rng_mode == CLR_RNG_PHILOX ? sizeof(PhiloxMode::Lane) : sizeof(XorMode::Lane);
}
}  // namespace clr

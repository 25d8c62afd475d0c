// Instantiations of the photon kernel on the reference's xorshift streams (parity mode).
#include "photon_kernel.cuh"

namespace clr {
cudaError_t launch_xor(const LaunchArgs& a) {
    return a.records ? launch_t<XorMode, true, false>(a) : launch_t<XorMode, false, false>(a);
}
int occupancy_xor(bool records) { return records ? occupancy_t<XorMode, true, false>() : occupancy_t<XorMode, false, false>(); }
}  // namespace clr

// Instantiations of the wavefront engine on the reference's xorshift streams (parity mode); a unit of its
// own so that it compiles in parallel with the persistent kernel's.
#include "wavefront.cuh"

namespace clr {
cudaError_t wave_run_xor(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes, WaveRunInfo* info) {
    return w.records ? wave_run_t<XorMode, true>(w, num_sms, st, max_passes, info)
                     : wave_run_t<XorMode, false>(w, num_sms, st, max_passes, info);
}
}  // namespace clr

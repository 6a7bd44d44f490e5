// pass_inst.cu — one kernel family of pass.cuh per object file.
//
// The build compiles this file once per family, with
//   TCG_PASS_MODE = MODE_FWD / MODE_BWD / MODE_MEAS / MODE_PACC and
//   TCG_PASS_KIND = 0 (pass_kernel), 1 (batch_kernel, full body),
//                   2 (batch_kernel, light body),
// so the twelve kernel bodies compile in parallel instead of in one unit.
#include "pass.cuh"

#if !defined(TCG_PASS_MODE) || !defined(TCG_PASS_KIND)
#error "pass_inst.cu is compiled with -DTCG_PASS_MODE=<0..3> -DTCG_PASS_KIND=<0..2>"
#endif

namespace tcg {

#if TCG_PASS_KIND == 0
template cudaError_t launch_pass_mode<TCG_PASS_MODE>(const PassArgs&, int, int64_t, cudaStream_t);
#elif TCG_PASS_KIND == 1
template cudaError_t launch_batch_mode<TCG_PASS_MODE, false>(const BatchLaunch&, int, int, cudaStream_t);
#elif TCG_PASS_KIND == 2
template cudaError_t launch_batch_mode<TCG_PASS_MODE, true>(const BatchLaunch&, int, int, cudaStream_t);
#else
#error "TCG_PASS_KIND must be 0, 1 or 2"
#endif

}  // namespace tcg

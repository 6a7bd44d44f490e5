// pass.cu — dispatch to the tile-pass kernel families.
//
// The kernels themselves are templates in pass.cuh; pass_inst.cu instantiates
// one family per object file.  This unit only maps a runtime mode (and, for
// persistent batches, the kernel body) to the family's launcher.
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.h"
#include "kernels.h"

namespace tcg {

cudaError_t launch_batch(int mode, const BatchLaunch& bl, int L, int max_slots, bool lite, cudaStream_t st) {
  if (max_slots < 1) max_slots = 1;
  if (lite) {
    if (mode == MODE_FWD) return launch_batch_mode<MODE_FWD, true>(bl, L, max_slots, st);
    if (mode == MODE_BWD) return launch_batch_mode<MODE_BWD, true>(bl, L, max_slots, st);
    if (mode == MODE_MEAS) return launch_batch_mode<MODE_MEAS, true>(bl, L, max_slots, st);
    if (mode == MODE_PACC) return launch_batch_mode<MODE_PACC, true>(bl, L, max_slots, st);
    return cudaErrorInvalidValue;
  }
  if (mode == MODE_FWD) return launch_batch_mode<MODE_FWD, false>(bl, L, max_slots, st);
  if (mode == MODE_BWD) return launch_batch_mode<MODE_BWD, false>(bl, L, max_slots, st);
  if (mode == MODE_MEAS) return launch_batch_mode<MODE_MEAS, false>(bl, L, max_slots, st);
  if (mode == MODE_PACC) return launch_batch_mode<MODE_PACC, false>(bl, L, max_slots, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_pass(int mode, int R, const PassArgs& a, int L, int64_t batch, cudaStream_t st) {
  if (R != 4) return cudaErrorInvalidValue;
  if (mode == MODE_FWD) return launch_pass_mode<MODE_FWD>(a, L, batch, st);
  if (mode == MODE_BWD) return launch_pass_mode<MODE_BWD>(a, L, batch, st);
  if (mode == MODE_MEAS) return launch_pass_mode<MODE_MEAS>(a, L, batch, st);
  if (mode == MODE_PACC) return launch_pass_mode<MODE_PACC>(a, L, batch, st);
  return cudaErrorInvalidValue;
}

}  // namespace tcg

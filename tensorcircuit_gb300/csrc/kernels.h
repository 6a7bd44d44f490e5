// kernels.h — launch interface between the C ABI (api.cu) and the kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.h"
#include "../../include/tcgb300.h"

namespace tcg {

enum { MODE_FWD = 0, MODE_BWD = 1, MODE_MEAS = 2, MODE_PACC = 3 };

constexpr int kRFwd = 4;   // register bits of forward / measure kernels
constexpr int kRBwd = 4;   // register bits of the adjoint kernel (psi + mu live)
constexpr int kMaxThreads = 256;

struct PassArgs {
  ProgramView prog;
  int pass;
  int n;
  float2* psi;              // [B][2^n]
  float2* mu;               // [B][2^n] (BWD, PACC)
  const float2* mats;       // [B][mat_stride]
  int64_t mat_stride;
  float2* partial;          // [B][part_stride][ntiles] accumulator partials
  int64_t part_stride;
  const float* coef;        // PACC: [B][coef_stride]
  int64_t coef_stride;
  int max_slots;
  // the first pass of a sweep may read its input elsewhere: psi_in
  // ([B][in_stride], in_stride 0 = one state for every circuit) instead of
  // psi, and (mu_zero) zeros instead of mu; every pass writes psi / mu
  const float2* psi_in;
  int64_t in_stride;
  int mu_zero;
};

// Argument block of the specialised (generated) pass kernels; the same
// layout as KParams in jit_device.cuh.
struct KParams_Host {
  float2* psi;
  float2* mu;
  const float2* mats;
  long long mat_stride;
  float2* partial;
  long long part_stride;
  const float* coef;
  long long coef_stride;
  const float2* psi_in;   // see PassArgs
  long long in_stride;
  int mu_zero;
  int pad;
};

// ---- uneven batches: many circuits, one persistent launch per sweep.
// Work item = one tile of one pass of one circuit; items are dequeued in
// order from a global counter, and an item of pass p waits (bounded) until
// every tile of pass p-1 of its circuit is complete.
struct BatchCirc {
  ProgramView prog;     // this launch's program (FWD / MEAS / PACC / BWD)
  int32_t n;
  int32_t max_slots;
  int64_t state_off;    // complex entries into the ragged state buffers
  int64_t mat_off;      // complex entries into the ragged matrix buffer
  int64_t part_off;     // complex entries into the partial buffer
  int64_t part_stride;  // accumulator outputs per tile slice
  int64_t coef_off;     // PACC coefficients
};
struct BatchSeg {
  int64_t item0;        // first work item of this (circuit, pass)
  int32_t circ;
  int32_t pass;
  uint32_t ntiles;
  uint32_t need;        // completed tiles of the circuit this segment waits for
};
constexpr int kBatchCoarse = 256;  // items per coarse segment-index entry
constexpr int kBatchChunk = 4;     // items a CTA dequeues at once

struct BatchLaunch {
  const BatchCirc* circ;
  const BatchSeg* segs;
  const int32_t* coarse; // segment of item k * kBatchCoarse, k = 0 .. nitems / kBatchCoarse
  int32_t nsegs;
  int32_t pad;
  int64_t nitems;
  float2* psi;
  float2* mu;
  const float2* mats;
  float2* partial;
  const float* coef;
  unsigned int* queue;  // work-item counter, zero at launch
  unsigned int* done;   // per-circuit completed tiles, zero at launch
  unsigned int* err;    // this call: a dependency wait ran out of time (zero at launch)
  unsigned int* sticky; // set with err; cleared only by the caller's check
  unsigned long long wait_ns;  // limit of one dependency wait
};
// L: tile bits shared by every program of the launch; max_slots: largest
// stage slot count over the circuits.
// lite: every program holds only 1-qubit dense gates, Pauli rotations,
// Z-rotation runs and Pauli terms (no shared-memory stages, 2-qubit dense or
// diagonal ops), which selects the smaller kernel body (two CTAs per SM).
cudaError_t launch_batch(int mode, const BatchLaunch& bl, int L, int max_slots, bool lite, cudaStream_t st);

// every kernel launch of the library increments this counter
void count_launch(int64_t n = 1);
int64_t launch_count();

cudaError_t launch_pass(int mode, int R, const PassArgs& a, int L, int64_t batch, cudaStream_t st);

// The per-family launchers behind launch_pass (one per MODE) and
// launch_batch (one per MODE and body).  Defined in pass.cuh; each is
// explicitly instantiated in its own translation unit (pass_inst.cu, compiled
// once per family) so the large kernel bodies compile in parallel.
template <int MODE>
cudaError_t launch_pass_mode(const PassArgs& a, int L, int64_t batch, cudaStream_t st);
template <int MODE, bool LITE>
cudaError_t launch_batch_mode(const BatchLaunch& bl, int L, int max_slots, cudaStream_t st);

// partial[b][e][t] (complex64) summed over t in fp64 for the listed entries.
// out_c64 (complex64) or out_c128 (complex128), one of them non-null.
cudaError_t launch_reduce_partials(const float2* partial, int64_t part_stride, uint32_t ntiles,
                                   const int64_t* entries_dev, int64_t nentries, int64_t batch,
                                   float2* out_c64, int64_t out_stride_c64, double* out_c128,
                                   int64_t out_stride_c128, cudaStream_t st);

// Pauli terms with many X/Y bits, one global pass per term.
cudaError_t launch_direct_expect(const float2* psi, int n, int64_t batch, const tcg_pauli* terms_dev,
                                 const int* term_ids_dev, int nterms_direct, int64_t nterms_total,
                                 float2* partial, uint32_t nblocks, cudaStream_t st);
cudaError_t launch_direct_pacc(const float2* psi, float2* mu, int n, int64_t batch,
                               const tcg_pauli* terms, const int* term_ids, int nterms_direct,
                               const float* coef, int64_t coef_stride, cudaStream_t st);

cudaError_t launch_probability(const float2* psi, int64_t len, float* p, cudaStream_t st);
cudaError_t launch_inner(const float2* a, const float2* b, int64_t len, int64_t batch, double* out,
                         void* scratch, cudaStream_t st);
size_t inner_scratch_bytes(int64_t len, int64_t batch);

// tensor-core passes (tcpass.cu)
cudaError_t launch_tc_fuse(const TcBlock* blocks, int nblocks, const TcGate* gates, const float2* mats,
                           int64_t mat_stride, int64_t batch, uint8_t* fused, float2* scales, int slots,
                           cudaStream_t st);
cudaError_t launch_tc_pass(const DevPass& pass, const TcPassDesc& desc, const uint32_t* runs_dev,
                           const TcBlock* blocks_dev, float2* psi, const float2* psi_in, int64_t in_stride, int n,
                           int64_t batch, const uint8_t* fused, const float2* scales, int slots, unsigned int* err,
                           cudaStream_t st);
cudaError_t launch_tc_mma_probe(const void* A, const void* B, float* D, int K, int N, unsigned int* err,
                                cudaStream_t st);

// sampling
size_t sample_scratch_bytes(int n, int64_t batch);
cudaError_t launch_sample(const float2* psi, int n, int64_t batch, const float* u, int64_t u_stride,
                          int64_t nshots, int64_t* out, void* scratch, cudaStream_t st);

// Monte-Carlo Kraus pick and its backward
cudaError_t launch_kraus_pick(const float2* ev, int S, const float* coef, int K, const float* x, int64_t x_stride,
                              int64_t B, int32_t* pick, float2* scale, float* p, cudaStream_t st);
cudaError_t launch_kraus_pick_bwd(const float2* gscale, const int32_t* pick, const float* p, int K,
                                  const float* coef, int S, int64_t B, float2* gev, cudaStream_t st);

}  // namespace tcg

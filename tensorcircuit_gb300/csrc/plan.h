// plan.h — host-side planner: gate list -> passes -> stages -> device program.
#pragma once
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <memory>

#include "../../include/tcgb300.h"
#include "engine.h"
#include "jit.h"

namespace tcg {

// One direction of a plan (forward, backward, or a Pauli-term measurement),
// flattened into the arrays the kernels read.
struct Program {
  int n = 0;
  int L = 0;                 // tile bits of every pass
  int R = 0;                 // register bits of the kernel it targets
  std::vector<DevPass> passes;
  std::vector<DevStage> stages;
  std::vector<DevOp> ops;
  std::vector<SlotOut> slot_out;
  std::vector<uint32_t> runs;
  std::vector<int64_t> entries;  // distinct accumulator outputs (sorted)
  std::vector<ZEnt> zents;       // OP_ZRUN entries
  int max_slots = 0;         // largest stage slot count
  int64_t nout = 0;          // per-circuit accumulator outputs (complex entries)
  int zrun_max = 32;         // longest run of Z-string rotations fused into one
                             // OP_ZRUN (1 = none; term runs always up to 32)

  // device copy, one per CUDA device, uploaded on first use
  struct DevCopy { void* base = nullptr; ProgramView view{}; };
  std::map<int, DevCopy> dev;
  std::mutex mu;

  // tensor-core passes (forward programs; tcpass.cu): source gates per pass,
  // the fused blocks of the passes that qualify; the error flag of their
  // bounded waits sits in the device copy (ProgramView::tc_err)
  std::vector<std::vector<int>> pass_gates;
  std::vector<TcPassDesc> tc_passes;
  std::vector<TcBlock> tc_blocks;
  std::vector<TcGate> tc_gates;
  std::vector<int> tc_of_pass;     // per pass: index into tc_passes, or -1
  std::vector<int> tc_prefer;      // per tensor pass: 1 if the cost model picks it
  int tc_slots = 0;                // fused matrices per circuit

  // specialised kernels per mode (jit.cpp), built on demand
  std::unique_ptr<JitKernels> jit[4];
  int calls[4] = {0, 0, 0, 0};
  std::mutex jit_mu;
};

struct PlanOpts {
  int tile_bits_fwd = 12;  // 2^(12-4) = 256 threads per CTA
  int tile_bits_bwd = 12;
  int max_stage_slots = 64;
  int zrun_max = 32;       // fusion width of commuting Z-string rotations
};

// A planned gate (global-bit form).
struct PGate {
  int kind;            // TCG_GATE_DENSE / TCG_GATE_DIAG / TCG_GATE_PAULI_ROT
  int k;
  int gbits[TCG_MAX_GATE_QUBITS];  // global index bits, first = sub-index MSB
  int64_t mat_off;
  int64_t grad_off;
  uint64_t xmask = 0, zmask = 0;   // PAULI_ROT: X/Y and Z/Y global masks
};

// Build a gate program for `gates` in execution order (`reverse` for the
// adjoint sweep: passes/stages are laid out in the order they execute).
int build_gate_program(int n, const std::vector<PGate>& gates, int L, int R,
                       bool reverse, int max_slots, Program* out);

// Build a measurement program for Pauli terms (global-bit masks).  Terms whose
// X/Y bits cannot fit the register layout are returned in `direct`.
int build_term_program(int n, const std::vector<tcg_pauli>& terms, int L, int R,
                       int max_slots, Program* out, std::vector<int>* direct);

// Fuse the dense gates of every forward pass that qualifies into blocks of at
// most kTcBlockBits tile bits (tensor-core passes, tcpass.cu).
void plan_tensor_passes(Program* P, const std::vector<PGate>& gates);

// Upload (once per device) and return the device view.
int program_device_view(Program* p, ProgramView* view);
void program_free(Program* p);

}  // namespace tcg

struct tcg_plan {
  int n = 0;
  int ngates = 0;
  int64_t grad_entries = 0;   // max grad_off + entries over gates
  bool has_grad = false;
  tcg::Program fwd;
  tcg::Program bwd;
};

struct tcg_mplan {
  int n = 0;
  int nterms = 0;
  std::vector<tcg_pauli> terms;
  tcg::Program prog;
  std::vector<int> direct;    // terms run by the plain kernel
  // device copies of terms[] and direct[] per device
  struct Dev { void* base = nullptr; tcg_pauli* terms = nullptr; int* direct = nullptr; int64_t* direct_entries = nullptr; };
  std::map<int, Dev> dev;
  std::mutex mu;
};

// engine.h — internal data structures shared by the host planner (plan.cpp)
// and the CUDA pass kernels (pass.cuh).  Not part of the C ABI.
//
// Execution model.  A circuit's gate list is cut into PASSES.  A pass holds a
// set of L "local" amplitude-index bits (the low LO bits always included, so
// every tile is a set of 2^(L-LO) contiguous runs of 2^LO amplitudes); one CTA
// owns one TILE = the 2^L amplitudes that differ only in the local bits, so a
// pass reads and writes the state exactly once.  Inside a pass the gates run
// in STAGES: a stage picks R of the L local bits as REGISTER bits, every thread
// holds the 2^R amplitudes of one register group, and the stage's gates run on
// those registers with no further memory traffic (dense gates on register
// bits, diagonal gates on any bits, Pauli terms whose X/Y bits are register
// bits).  Between two stages the tile goes through shared memory once to
// change which bits are register bits.
#pragma once
#include <cstdint>

namespace tcg {

constexpr int kLo = 5;            // low index bits always local (256 B runs)
constexpr int kMaxTileBits = 13;  // 2^13 amplitudes = 64 KiB per tile
constexpr int kMaxPassBits = 20;  // non-local bits of one circuit (n <= 33)
constexpr int kMinQubits = 6;     // smaller circuits are padded by the host
constexpr int kMaxQubits = 32;

// device op kinds
enum OpKind : int32_t {
  OP_DENSE1 = 0,   // 1-qubit dense on register position p0
  OP_DENSE2 = 1,   // 2-qubit dense on register positions (p0 = sub-index MSB, p1)
  OP_DIAG = 2,     // k-qubit diagonal on global bits gb[0..k-1] (gb[0] = MSB)
  OP_DENSEK = 3,   // k-qubit dense on tile bits tb[0..k-1], run on the smem tile
  OP_EXPECT = 4,   // Pauli term: acc += conj(psi[a]) s(a) psi[a ^ x]
  OP_PACC = 5,     // Pauli term: mu[a] += c s(a) psi[a ^ x]
  OP_PROT = 6,     // Pauli rotation cos(phi) I - i sin(phi) P (X/Y bits in
                   // registers: xreg; Z/Y global mask: zmask; nY)
  OP_ZRUN = 7      // run of k commuting Z-string rotations, entries
                   // zents[mat_off .. mat_off + k), applied as one phase
};

// One rotation of an OP_ZRUN run: exp(-i phi Z_S) with e^{i phi} at
// mats[mat_off]; zreg = register positions of the Z bits (the phase class),
// zmask = all Z bits (global).
struct ZEnt {
  uint32_t zmask;
  int32_t zreg;
  int32_t slot;      // gradient slot, -1 = none
  int32_t pad;
  int64_t mat_off;
  int64_t grad_off;
};

// One device op, 48 bytes.
struct DevOp {
  int32_t kind;
  int32_t k;
  int32_t p[6];        // register positions (DENSE1/2), tile bits (DENSEK),
                       // global bits (DIAG)
  int32_t xreg;        // EXPECT/PACC: register-position mask of the X/Y bits
  int32_t nY;          // EXPECT/PACC: number of Y factors (phase (-i)^nY)
  uint32_t zmask;      // EXPECT/PACC: global Z/Y mask
  int32_t slot;        // first accumulator slot in the stage (or -1)
  int64_t mat_off;     // per-circuit matrix offset (complex entries); term id
  int64_t grad_off;    // per-circuit gradient offset, -1 = none
};

struct DevStage {
  int32_t R;             // register bits (<= template R of the kernel)
  int32_t smem_stage;    // 1: ops run on the smem tile (OP_DENSEK only)
  int32_t lanes_low;     // 1: lane bits are tile bits 0..4 in order
  int32_t nthread_bits;  // L - R
  int32_t reg_tile[6];   // tile bit of register bit i
  int32_t thr_tile[16];  // tile bit of thread-id bit i
  int32_t op_begin, op_end;
  int32_t nslots;        // accumulator slots (complex) used by the stage
  int32_t slot_out_begin, slot_out_end; // entries of pass slot->output map
};

struct DevPass {
  int32_t L;                 // local bits
  int32_t nnonlocal;         // n - L
  int32_t lbits[kMaxTileBits];       // global bit of tile bit i
  int32_t nlbits[kMaxQubits];        // global bits that are not local
  int32_t stage_begin, stage_end;
  int32_t runs_off;          // offset of the 2^(L-LO) run table in the program
  int32_t pad;
};

// slot -> output mapping written at the end of each stage
struct SlotOut {
  int32_t slot;      // stage slot index
  int32_t pad;
  int64_t out_off;   // per-circuit output offset (complex entries)
};

// ---- tensor-core passes (tcpass.cu).  A forward pass whose gates all act on
// its 12 local bits can instead run as a short sequence of FUSED BLOCKS: each
// block is the product of consecutive gates of the pass on at most 6 tile
// bits, a 64 x 64 complex matrix applied to the tile as a complex GEMM on the
// tensor cores (64 block entries x 64 columns per tile).
constexpr int kTcTileBits = 12;   // tile bits of a tensor-core pass
constexpr int kTcBlockBits = 6;   // qubits of one fused block
constexpr int kTcMatBytes = 32768;  // one fused block: fp16 hi + lo planes, 16 KiB each

// A source gate of a fused block, in block-bit form.
struct TcGate {
  int32_t kind;      // TCG_GATE_DENSE / TCG_GATE_DIAG / TCG_GATE_PAULI_ROT
  int32_t k;
  int32_t pos[6];    // block bit of gate qubit i (gate qubit 0 = sub-index MSB)
  int32_t xmask;     // PAULI_ROT: block-bit mask of the X/Y factors
  int32_t zmask;     // PAULI_ROT: block-bit mask of the Z/Y factors
  int32_t nY;        // PAULI_ROT: number of Y factors
  int32_t pad;
  int64_t mat_off;   // per-circuit matrix offset (complex entries)
};

// Operand planes of a block in shared memory (bytes): re hi, re lo, im hi,
// im lo; the im planes sit 64 bytes further so that re and im rows of one
// store fall in different banks.  The fp32 copy of a tile before it goes
// back to HBM uses the same region: re at 0, im at kTcPlaneIm.
constexpr uint32_t kTcPlaneLo = 8192;
constexpr uint32_t kTcPlaneIm = 16448;
constexpr uint32_t kTcBRegion = 32832;

struct TcBlock {
  int32_t bbits[6];  // tile bit of block-index bit i
  int32_t cbits[6];  // tile bit of column-index bit i
  int32_t gate_begin, gate_end;  // source gates, in application order
  int32_t slot;      // fused-matrix slot (per circuit) of this block
  int32_t pairbit;   // column bit whose two values share one 32-bit word of
                     // the next block's planes (-1: 16-bit stores)
  // Where the epilogue writes output (block entry i, column n): byte offset
  // raddr[i] ^ caddr[n] in the next block's operand planes, or, after the
  // pass's last block, in the fp32 tile copy.  Both maps are linear over
  // GF(2) (a bit permutation, then the staging swizzle), hence the XOR.
  uint32_t raddr[64];
  uint32_t caddr[64];
};

struct TcPassDesc {
  int32_t pass;      // pass index in the program
  int32_t block_begin, block_end;
  int32_t ldpair;    // tile bit 0 is the first block's K bit 0: 32-bit stores
  uint32_t ldaddr[12];  // operand-plane byte offset of tile bit t, first block
};

// Whole device program of one plan direction, in one device allocation.
struct ProgramView {
  const DevPass* passes;
  const DevStage* stages;
  const DevOp* ops;
  const SlotOut* slot_out;
  const uint32_t* runs;   // run tables
  const int64_t* entries; // distinct accumulator outputs, for the final reduce
  int64_t nentries;
  const ZEnt* zents;      // entries of OP_ZRUN runs
  const TcPassDesc* tc_passes;  // tensor-core passes (forward programs)
  const TcBlock* tc_blocks;
  const TcGate* tc_gates;
  unsigned int* tc_err;         // sticky flag: a tensor-core pass's wait ran out
};

}  // namespace tcg

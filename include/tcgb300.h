/*
 * tcgb300.h — C ABI of the GB300 statevector engine for TensorCircuit's
 * parameterized-circuit path.
 *
 * The engine replaces the tensor-network contraction that TensorCircuit runs
 * for `Circuit.wavefunction()` / `expectation_ps()` / `sample()` and the
 * taped autodiff behind `backend.vvag`.  Every entry point is stream ordered,
 * takes plain device pointers owned by the caller (torch tensors on the Python
 * side), and returns an int status (TCG_OK == 0).  No entry point exits,
 * aborts or traps; device-side problems come back as a status.
 *
 * State layout (same as the reference): a circuit on n qubits is a complex64
 * vector of 2^n amplitudes, qubit 0 is the MOST significant bit of the
 * amplitude index (tensorcircuit/basecircuit.py:213-215 wires gate leg i to
 * the i-th front edge; tests/test_circuit.py:21-44 pins
 * `wavefunction()[2] == 8` for `unitary(0, 1, arange(16))`).  A batch of B
 * circuits with the same structure is B such vectors back to back.
 *
 * Gate matrices follow the reference's `reshapem` convention
 * (tensorcircuit/backends/abstract_backend.py:403-414): a k-qubit gate is a
 * 2^k x 2^k row-major matrix M[out, in], and the first listed qubit is the
 * most significant bit of the k-bit sub-index.
 */
#ifndef TCGB300_H
#define TCGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------
 * Mirrors the reference's error behaviour: duplicated qubits are an
 * AssertionError there (tensorcircuit/basecircuit.py:143), measuring two
 * operators on one index a ValueError (basecircuit.py:306-307), anything a
 * backend lacks a NotImplementedError (backends/abstract_backend.py:914-928).
 * The Python layer maps these codes back to those exception types. */
enum {
  TCG_OK = 0,
  TCG_ERR_INVALID_ARG = 1,   /* bad size, null pointer, qubit out of range */
  TCG_ERR_DUP_QUBIT = 2,     /* a gate lists the same qubit twice */
  TCG_ERR_UNSUPPORTED = 3,   /* valid request this engine does not implement */
  TCG_ERR_CUDA = 4,          /* a CUDA runtime call failed */
  TCG_ERR_SCRATCH = 5,       /* caller-provided scratch is too small */
  TCG_ERR_OOM = 6,           /* a host or device allocation failed */
  TCG_ERR_TOO_LARGE = 7,     /* request exceeds a fixed internal capacity (each
                                entry point that returns it states its limit) */
  TCG_ERR_TIMEOUT = 8        /* a bounded device-side wait ran out of time */
};

/* ---- gate program --------------------------------------------------------- */
enum {
  TCG_GATE_DENSE = 0,     /* 2^nq x 2^nq matrix, row-major M[out, in]        */
  TCG_GATE_DIAG = 1,      /* diagonal gate: 2^nq entries d[idx]                */
  TCG_GATE_PAULI_ROT = 2  /* cos(phi) I - i sin(phi) P for a Pauli string P  */
};

#define TCG_MAX_GATE_QUBITS 6

typedef struct tcg_gate {
  int32_t kind;                         /* TCG_GATE_*                        */
  int32_t nq;                           /* 1 .. TCG_MAX_GATE_QUBITS          */
  int32_t qubits[TCG_MAX_GATE_QUBITS];  /* qubit indices, first = sub-index MSB */
  int32_t pauli[TCG_MAX_GATE_QUBITS];   /* PAULI_ROT: 1=X 2=Y 3=Z per qubit  */
  int64_t mat_off;   /* complex64 offset of this gate's entries in the
                        per-circuit matrix buffer: 4^nq (dense), 2^nq
                        (diagonal), or 1 = cos(phi) + i sin(phi) (Pauli
                        rotation; rx(theta) is phi = theta/2, P = X)      */
  int64_t grad_off;  /* complex64 offset of this gate's cotangent in the
                        per-circuit gradient buffer, or -1 when no gradient
                        is wanted.  Dense/diagonal: one entry per matrix
                        entry (torch convention dL/dRe + i dL/dIm).  Pauli
                        rotation: one entry, (dL/dphi, 0).                */
} tcg_gate;

typedef struct tcg_plan tcg_plan; /* opaque, host side; owns a small device
                                     copy of its pass program               */

typedef struct tcg_plan_opts {
  int32_t tile_bits;     /* local index bits held by one CTA, 5..12 (larger values
                            are clamped to 12: 256 threads per CTA); 0 = 12 */
  int32_t max_stage_grad_entries; /* cap on cotangent entries per stage; 0 = default */
  int32_t zrun_max;      /* fusion width of commuting Z-string rotations: the
                            longest run applied as one phase op (1..32, 1 = each
                            rotation on its own); 0 = default (32)          */
} tcg_plan_opts;

typedef struct tcg_plan_stats {
  int32_t nqubits;
  int32_t ngates;
  int32_t npasses;       /* HBM passes over the state per forward sweep   */
  int32_t nstages;       /* register layouts summed over passes           */
  int32_t tile_bits;
  int64_t grad_entries;  /* complex64 cotangent entries per circuit       */
} tcg_plan_stats;

/* Replaces: the gate queue built by AbstractCircuit._meta_apply /
 * BaseCircuit.apply_general_gate (tensorcircuit/abstractcircuit.py:218-326,
 * tensorcircuit/basecircuit.py:120-245) plus the contraction path search of
 * cons._base (tensorcircuit/cons.py:523-631).  Plans the gate list into HBM
 * passes; the result is reusable for any batch and any matrix values. */
int tcg_plan_create(int32_t nqubits, const tcg_gate* gates, int32_t ngates,
                    const tcg_plan_opts* opts, tcg_plan** out);
int tcg_plan_destroy(tcg_plan* plan);
int tcg_plan_get_stats(const tcg_plan* plan, tcg_plan_stats* out);

/* Tensor-core passes (no reference counterpart; part of what replaces the
 * per-gate contraction of tensorcircuit/cons.py:605-623).  A forward pass
 * whose gates all act on its 12 local bits may run as fused blocks: each block
 * is the product of consecutive gates on at most 6 bits, applied to every
 * tile as a complex GEMM on the tensor cores (tcgen05, fp16 hi/lo operand
 * split, fp32 accumulation).  Which passes do so follows the environment
 * variable TCG_TC (0 none, 1 every pass that qualifies, unset the passes the
 * planner's cost model prefers).  A call with such passes takes its fused
 * matrices (32 KiB per block and circuit) from a stream-ordered allocation on
 * its own stream, from a library memory pool per device that keeps up to
 * 1 GiB between calls, and frees it in stream order when it returns (under
 * stream capture the allocation becomes the graph's own memory nodes).
 * tcg_plan_tensor_passes returns how many forward passes take that path. */
int tcg_plan_tensor_passes(const tcg_plan* plan);
/* Sets the policy TCG_TC selects (0, 1 or 2 = cost model) for later calls of
 * every plan; returns the previous one (another value only queries). */
int32_t tcg_set_tensor_policy(int32_t policy);
/* Synchronises the stream; TCG_ERR_TIMEOUT if a bounded device-side wait of
 * an earlier tensor-core pass ran out of time (its results are then invalid),
 * else TCG_OK.  Clears the flag. */
int tcg_plan_check(const tcg_plan* plan, void* stream);
/* Diagnostics (no reference counterpart): one tensor-core MMA probe,
 * d[128][n] = a[128][k] b[n][k]^T for fp16 row-major a, b (device memory,
 * k in {16, 32, 48, 64}, n a multiple of 32 up to 256), fp32 d, through the
 * same shared-memory operand layout, descriptors and tensor-memory readback
 * as the tensor-core passes.  *err (device) is set if its wait ran out. */
int tcg_debug_tc_mma(const void* a, const void* b, float* d, int32_t k, int32_t n, unsigned int* err,
                     void* stream);
/* Diagnostics: host pointers to the fused-block program of a plan's forward
 * sweep: arrays[0..3] = tensor-pass descriptors, blocks, source gates, the
 * cost model's per-pass preference (int32); counts and element sizes in bytes
 * likewise (all three arrays hold 4 elements). */
int tcg_debug_tc_program(const tcg_plan* plan, const void** arrays, int64_t* counts, int64_t* sizes);

/* Replaces: Circuit.wavefunction() (tensorcircuit/circuit.py:792-810), i.e.
 * the contractor loop of cons._base (tensorcircuit/cons.py:605-623).
 * psi [batch][2^n] holds the input states on entry and the output states on
 * return (in place).  mats holds batch rows of mat_stride complex64 entries. */
int tcg_forward(const tcg_plan* plan, void* psi, int64_t batch,
                const void* mats, int64_t mat_stride, void* stream);

/* tcg_forward with the input states read from elsewhere (no reference
 * counterpart: it saves the copy of the input into the output buffer).  The
 * first pass reads psi_in[b * in_stride ..] (in_stride 0: one state for every
 * circuit, e.g. |0...0>; psi_in == psi with in_stride 2^n is tcg_forward) and
 * every pass writes psi [batch][2^n]. */
int tcg_forward_from(const tcg_plan* plan, const void* psi_in, int64_t in_stride, void* psi,
                     int64_t batch, const void* mats, int64_t mat_stride, void* stream);

/* Replaces: the reverse-mode AD that backend.vvag runs through the taped
 * tensordots (tensorcircuit/backends/pytorch_backend.py:673-709).  Adjoint
 * sweep: on entry psi = output states, mu = cotangent of the output (torch
 * convention, dL/dRe + i dL/dIm); on return psi = input states, mu = the
 * cotangent of the input states and grads[b][grad_off + e] = the cotangent
 * of matrix entry e of each gate with grad_off >= 0.
 * scratch: tcg_backward_scratch_bytes(plan, batch) bytes of device memory. */
size_t tcg_backward_scratch_bytes(const tcg_plan* plan, int64_t batch);
int tcg_backward(const tcg_plan* plan, void* psi, void* mu, int64_t batch,
                 const void* mats, int64_t mat_stride, void* grads,
                 int64_t grad_stride, void* scratch, size_t scratch_bytes,
                 void* stream);
/* tcg_backward with the output states read from psi_out [batch][2^n]
 * (left unchanged) instead of psi: psi is written with the input states, so
 * the caller keeps its output states without copying them first. */
int tcg_backward_from(const tcg_plan* plan, const void* psi_out, void* psi, void* mu,
                      int64_t batch, const void* mats, int64_t mat_stride, void* grads,
                      int64_t grad_stride, void* scratch, size_t scratch_bytes,
                      void* stream);

/* ---- observables ---------------------------------------------------------- */

/* A Pauli string over qubits, as masks over AMPLITUDE-INDEX bits
 * (bit b <-> qubit n-1-b): xmask has X or Y positions, zmask Z or Y
 * positions.  (P psi)[a] = (-i)^{#Y} (-1)^{popcount(a & zmask)} psi[a ^ xmask].
 * The reference builds the same operator from its ps codes 1=X, 2=Y, 3=Z
 * (tensorcircuit/abstractcircuit.py:1208-1288, quantum.py:1025-1045). */
typedef struct tcg_pauli {
  uint64_t xmask;
  uint64_t zmask;
} tcg_pauli;

typedef struct tcg_mplan tcg_mplan; /* opaque measurement plan for a term list */

/* Plans a list of Pauli terms into read-only passes (terms whose X/Y
 * positions fit one tile are grouped; the rest get one plain pass each). */
int tcg_mplan_create(int32_t nqubits, const tcg_pauli* terms, int32_t nterms,
                     tcg_mplan** out);
int tcg_mplan_destroy(tcg_mplan* plan);
/* number of read passes over the state one expectation call makes */
int tcg_mplan_passes(const tcg_mplan* plan);

/* Replaces: AbstractCircuit.expectation_ps (tensorcircuit/abstractcircuit.py:
 * 1208-1288) -> Circuit.expectation (tensorcircuit/circuit.py:914-981), one
 * sandwich contraction per term there.  Here all terms of the plan are read
 * from the state in the plan's passes.
 * out[b][t] = <psi_b| P_t |psi_b> as complex128 (re, im interleaved).
 * scratch: tcg_expect_scratch_bytes(plan, batch) bytes. */
size_t tcg_expect_scratch_bytes(const tcg_mplan* plan, int64_t batch);
int tcg_expect_pauli(const tcg_mplan* plan, const void* psi, int64_t batch,
                     double* out, void* scratch, size_t scratch_bytes,
                     void* stream);

/* Allocation-free Pauli expectations.  No counterpart in the reference: it
 * exists for callers that cannot allocate device memory -- hosts whose device
 * memory lives in a pool this ABI cannot reach (a runtime that hands over
 * only pre-allocated buffers), and loops that cannot afford cudaMalloc's
 * implicit synchronisation.  Same result as
 * tcg_expect_pauli (out[b][t] = <psi_b|P_t|psi_b>, complex128) without a plan
 * and without any allocation: the partial sums go to a fixed 8 MiB device
 * array inside the library.  Limits: nterms <= 64, batch <= 65535 and
 * batch * nterms <= 6898; larger requests return TCG_ERR_TOO_LARGE.  The
 * first call on each device looks up the array's device address (make it
 * before any stream capture).  All calls share the array: calls that overlap
 * on the GPU (different streams, no ordering between them) race. */
int tcg_expect_pauli_noalloc(const void* psi, int32_t nqubits, int64_t batch,
                             const tcg_pauli* terms, int32_t nterms, double* out,
                             void* stream);

/* Cotangent seed for Pauli observables: mu[b] += sum_t coef[b][t] P_t psi[b]
 * (coef real fp32, coef_stride floats per circuit).  With coef = 2 Re(g_t)
 * this is the cotangent the reference's AD propagates into the state for
 * outputs <P_t> with incoming gradients g_t. */
int tcg_pauli_accumulate(const tcg_mplan* plan, const void* psi, void* mu,
                         int64_t batch, const float* coef, int64_t coef_stride,
                         void* stream);
/* flags: TCG_ACC_OVERWRITE = mu[b] = sum_t ... (mu's old contents are not
 * read, so it needs no zero fill first). */
#define TCG_ACC_OVERWRITE 1
int tcg_pauli_accumulate_ex(const tcg_mplan* plan, const void* psi, void* mu,
                            int64_t batch, const float* coef, int64_t coef_stride,
                            int32_t flags, void* stream);

/* ---- sampling --------------------------------------------------------------
 * Replaces: BaseCircuit.sample(allow_state=True, status=u)
 * (tensorcircuit/basecircuit.py:525-616) -> backend.probability_sample
 * (tensorcircuit/backends/abstract_backend.py:1124-1157): normalise |psi|^2,
 * cumulative sum, r = cdf[-1] * (1 - u), left searchsorted.
 * Declared CDF arithmetic (integer, so every parallel scan order gives the
 * same bits):  w(x) = floor(x^2 * 2^60) for an fp32 component x, computed
 * exactly from its bits (0 for zero/subnormal x);  q[a] = w(re) + w(im);
 * cdf = inclusive uint64 prefix sum of q;  target
 * t = (uint64) floor((1.0 - (double)u) * (double)cdf[last]) in double;
 * out = first index with cdf[index] >= t, clamped to 2^n - 1.
 * Preconditions: |re|, |im| < 2 and sum |psi|^2 < 16 (true for states).
 * psi [batch][2^n]; u [batch][u_stride] (u_stride 0 shares one draw vector);
 * out [batch][nshots].  scratch: tcg_sample_scratch_bytes(n, batch) bytes. */
size_t tcg_sample_scratch_bytes(int32_t nqubits, int64_t batch);
int tcg_sample(const void* psi, int32_t nqubits, int64_t batch, const float* u,
               int64_t u_stride, int64_t nshots, int64_t* out, void* scratch,
               size_t scratch_bytes, void* stream);

/* Replaces: the Monte-Carlo step of Circuit._general_kraus_2
 * (tensorcircuit/circuit.py:635-694): branch probabilities
 * p_i = sum_s Re(ev[b][s]) coef[i][s] (ev: complex64 [batch][nstrings] Pauli
 * expectations, coef: fp32 [nkraus][nstrings] expansion of K_i^dag K_i), the
 * pick of Circuit.unitary_kraus (tensorcircuit/circuit.py:541-556) from the
 * uniform x[b * x_stride] (x_stride 0 shares one draw), and the rescale
 * 1 / (sqrt(p_pick) + 1e-10) as complex64 (imaginary part 0).  p receives
 * the fp32 [batch][nkraus] probabilities. */
int tcg_kraus_pick(const void* ev, int32_t nstrings, const float* coef, int32_t nkraus,
                   const float* x, int64_t x_stride, int64_t batch, int32_t* pick,
                   void* scale, float* p, void* stream);
/* Backward of tcg_kraus_pick: gev[b][s] = (g_b (-1 / (sqrt(p_r) + 1e-10)^2)
 * / (2 sqrt(p_r)) coef[r][s], 0) for g_b = Re(gscale[b]), r = pick[b]. */
int tcg_kraus_pick_backward(const void* gscale, const int32_t* pick, const float* p,
                            int32_t nkraus, const float* coef, int32_t nstrings,
                            int64_t batch, void* gev, void* stream);

/* Replaces: BaseCircuit.probability (tensorcircuit/basecircuit.py:510-523):
 * p[a] = |psi[a]|^2 in fp32 (computed as re^2 + im^2). */
int tcg_probability(const void* psi, int64_t len, float* p, void* stream);

/* Inner products <a_b|b_b> for batch rows of len amplitudes, complex128 out. */
int tcg_inner(const void* a, const void* b, int64_t len, int64_t batch,
              double* out, void* scratch, size_t scratch_bytes, void* stream);
size_t tcg_inner_scratch_bytes(int64_t len, int64_t batch);

/* ---- misc ------------------------------------------------------------------ */
const char* tcg_status_string(int32_t status);
/* 2: tcg_gate gained `pauli` (Pauli-rotation gates); uneven batches added.
 * 3: tcg_plan_opts gained `zrun_max` (its size changed: callers built against
 *    an older header must rebuild); tcg_ubatch_create_ex added. */
int32_t tcg_abi_version(void);

/* ---- uneven batches --------------------------------------------------------
 * Many parameterized circuits of different qubit counts and depths, each with
 * its own energy <H_c> = offset_c + sum_t coef_c[t] <psi_c|P_t|psi_c>, value
 * and adjoint gradient of every circuit in ONE call: one persistent kernel
 * launch per sweep (forward, measure, Pauli accumulate, adjoint) covers all
 * circuits, so the call is a fixed sequence of eight kernels that a CUDA
 * graph can capture.  Replaces the reference's loop of per-circuit
 * `K.value_and_grad(f)` calls (tensorcircuit/backends/pytorch_backend.py:
 * 533-544 over circuits built with tensorcircuit/templates/blocks.py:84-110
 * and measured with tensorcircuit/templates/measurements.py:290-335), which
 * has no batched form for circuits whose sizes differ.
 *
 * Parameterized gates must be Pauli rotations (TCG_GATE_PAULI_ROT) whose
 * angle is phi = mat_scale[e] * params_c[mat_param[e]] for their matrix entry
 * e; every other entry is a constant.  Gradients are d<H_c>/d params_c. */
typedef struct tcg_ubatch tcg_ubatch;

typedef struct tcg_ubatch_circuit {
  int32_t nqubits;          /* >= tile_bits of the batch                    */
  int32_t ngates;
  const tcg_gate* gates;    /* mat_off / grad_off index the circuit's own
                               matrix buffer; grad_off >= 0 only on
                               parameterized Pauli rotations                */
  int64_t nmat;             /* complex entries of the circuit's matrices    */
  const float* mat_const;   /* host, 2*nmat floats: constant entries        */
  const int64_t* mat_param; /* host, nmat: parameter of a rotation entry,
                               -1 for a constant entry                      */
  const float* mat_scale;   /* host, nmat: phi = scale * theta              */
  int32_t nparams;
  int32_t nterms;
  const tcg_pauli* terms;   /* host, nterms                                  */
  const float* coef;        /* host, nterms                                  */
  double offset;
} tcg_ubatch_circuit;

/* tile_bits: local index bits per tile, 5 < tile_bits <= 12 and <= every
 * circuit's qubit count (the autotuner's knob).  Host arrays are copied. */
int tcg_ubatch_create(const tcg_ubatch_circuit* circuits, int32_t ncircuits, int32_t tile_bits,
                      tcg_ubatch** out);
/* The same with the planner's options: opts->tile_bits as above (required),
 * opts->zrun_max the Z-rotation fusion width (0 = default), and
 * opts->max_stage_grad_entries (0 = default).  The batch autotuner searches
 * tile width and fusion width through this entry point. */
int tcg_ubatch_create_ex(const tcg_ubatch_circuit* circuits, int32_t ncircuits, const tcg_plan_opts* opts,
                         tcg_ubatch** out);
int tcg_ubatch_destroy(tcg_ubatch* batch);

/* nparams_total = sum of nparams (the layout of params and grads: circuit 0's
 * parameters first); state_entries = sum of 2^n; scratch_bytes = device
 * scratch one call needs (states, cotangents, matrices, partial sums). */
int tcg_ubatch_info(const tcg_ubatch* batch, int64_t* nparams_total, int64_t* state_entries,
                    size_t* scratch_bytes);

/* Complex-entry offset of circuit c's state inside the scratch buffer (the
 * states sit at the start of scratch, back to back).  After a call with
 * grads == NULL it holds the circuit's final state; a call with gradients
 * uncomputes it back to |0...0> during the adjoint sweep. */
int64_t tcg_ubatch_state_offset(const tcg_ubatch* batch, int32_t c);

/* energies[c] (float32) for every circuit and, when grads is not NULL,
 * grads[nparams_total] (float32).  params: device float32 [nparams_total].
 * Reductions run in float64 in a fixed order (deterministic). */
int tcg_ubatch_value_and_grad(tcg_ubatch* batch, const float* params, float* energies, float* grads,
                              void* scratch, size_t scratch_bytes, void* stream);

/* Work of one call per sweep (index 0 forward, 1 adjoint, 2 measure,
 * 3 Pauli accumulate): tiles processed and algorithmic HBM bytes (16 per
 * amplitude for the forward sweep, 32 adjoint, 8 measure, 24 accumulate). */
int tcg_ubatch_stats(const tcg_ubatch* batch, int64_t* tiles, double* alg_bytes);

/* Synchronises the stream and reports TCG_ERR_TIMEOUT if a dependency wait
 * of an earlier call ran out of time (its results are then invalid), else
 * TCG_OK; clears the flag.  The flag lives in the scratch buffer: zero the
 * scratch once before its first use so that it starts clear. */
int tcg_ubatch_check(tcg_ubatch* batch, void* scratch, void* stream);

/* Limit of one device-side dependency wait of later calls (default 2 s);
 * a wait that runs out makes the launch skip every later wait and finish,
 * and tcg_ubatch_check report TCG_ERR_TIMEOUT. */
int tcg_ubatch_set_wait_limit(tcg_ubatch* batch, uint64_t wait_ns);
/* Diagnostics (no reference counterpart): overwrite the dependency count of
 * segment `seg` of sweep `sweep` (0 forward, 1 adjoint, 2 measure, 3 Pauli
 * accumulate) in the batch's device tables, so that tests can make a wait
 * run out (a count no sweep reaches) without faulting anything: the results
 * of the calls that follow are invalid. */
int tcg_debug_ubatch_set_need(tcg_ubatch* batch, int32_t sweep, int32_t seg, uint32_t need);

/* ---- learned warm start (no reference counterpart) ---------------------------
 * Kernels of the network that maps Hamiltonian couplings to circuit angles
 * (tensorcircuit_gb300/warmstart.py).  Row-major float32 weights w[out][in];
 * activations bfloat16 (x_bf16 / y_bf16 = 1) or float32; float32 accumulation.
 * act: 0 identity, 1 GELU (tanh form). */
int tcg_mlp_linear_forward(const void* x, int32_t x_bf16, const float* w, const float* bias,
                           int64_t batch, int32_t in, int32_t out, int32_t act, float* pre,
                           void* y, int32_t y_bf16, void* stream);
/* dz = dy * act'(pre); dw = dz^T x (overwritten); db = column sums of dz
 * (overwritten); dx = dz w when dx is not NULL.  Fixed-order reductions. */
int tcg_mlp_linear_backward(const float* dy, const float* pre, int32_t act, const void* x,
                            int32_t x_bf16, const float* w, int64_t batch, int32_t in, int32_t out,
                            float* dz, float* dw, float* db, float* dx, void* stream);
/* Angle regression loss mean(1 - cos(pred - target)) over n entries:
 * dpred = sin(pred - target) / n, partial[nblocks] = per-block loss sums. */
int tcg_periodic_loss(const float* pred, const float* target, int64_t n, float* dpred,
                      float* partial, int32_t nblocks, void* stream);
/* Adam (bias-corrected, step >= 1) on n float32 parameters in place. */
int tcg_adam_update(float* p, const float* g, float* m, float* v, int64_t n, float lr, float beta1,
                    float beta2, float eps, int32_t step, void* stream);

/* Diagnostics (no reference counterpart): host pointers to a plan's pass
 * program so tests can replay its index arithmetic on the CPU.  which = 0
 * forward, 1 adjoint, 2 the measurement program of an mplan (pass the
 * mplan as `plan`).  arrays[0..5] = passes, stages, ops, slot_out, runs,
 * Z-rotation run entries; counts[0..5] their lengths; sizes[0..5] the
 * element sizes in bytes (all three arrays hold 6 elements). */
int tcg_debug_program(const void* plan, int32_t which, const void** arrays,
                      int64_t* counts, int64_t* sizes);

/* Number of kernel launches this library has issued since it was loaded
 * (all entry points, all devices). */
int64_t tcg_launch_count(void);

/* Specialised kernels (no reference counterpart).  A plan direction whose
 * kernels have run twice is translated into straight-line CUDA for its exact
 * gate layout and compiled once with NVRTC for sm_103a (environment variable
 * TCG_JIT: 0 = never, 1 = from the first call, unset = after two calls;
 * cubins are cached under TCG_JIT_CACHE or ~/.cache/tcgb300).  This reports
 * state (0 not built, 1 built, -1 failed, in which case the generic kernels
 * keep running) and copies into `text` (cap bytes) the compile log
 * (what = 0, ptxas register report included) or the generated source
 * (what = 1).  which/mode as for tcg_debug_program; mode 0 forward,
 * 1 adjoint, 2 measure, 3 Pauli accumulate. */
int tcg_debug_jit(const void* plan, int32_t which, int32_t mode, int32_t* state,
                  char* text, int64_t cap, int32_t what);

#ifdef __cplusplus
}
#endif

#endif /* TCGB300_H */

/*
 * bfgpu.h — C ABI of the GB300 (sm_103a) statevector engine for Butterfly's
 * gate-application hot path.
 *
 * The reference (Butterfly, Mojo) has no FFI on this path; its seam is
 *   fn execute(mut state: QuantumState, circuit: QuantumCircuit,
 *              ctx: ExecContext = ExecContext()) raises
 * (butterfly/core/executors.mojo:723-730), dispatched through the
 * function-pointer registry ExecutorFn / ExecutorEntry
 * (butterfly/core/executors.mojo:611-712) on ctx.execution_strategy
 * (butterfly/utils/context.mojo:33-40).  The entry points below are what a
 * GPU ExecutorFn binds: the state moves to the device once, the circuit is
 * flattened into an array of bf_op records, and bf_execute replaces the
 * per-transformation dispatch of execute_with_handlers
 * (butterfly/core/executors.mojo:268-319).
 *
 * Conventions
 *  - Every function returns an int status: BF_OK (0) or a negative BF_E* code.
 *    The message of the last failure on the calling thread is returned by
 *    bf_last_error().  No C++ exception crosses this boundary.
 *  - Qubit q is bit q of the amplitude index (little-endian), exactly as in
 *    the reference (transformations_scalar.mojo:87, stride = 1 << target).
 *  - The caller owns host arrays; the library owns device memory.
 *  - Each state owns one CUDA stream. Work on one state is stream-ordered;
 *    different states may run concurrently.  bf_execute only enqueues unless
 *    opts->sync is non-zero; bf_state_download_soa / bf_state_sync block.
 *  - Sizes are in elements unless stated otherwise.
 */
#ifndef BFGPU_H
#define BFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BFGPU_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
  BF_OK = 0,
  BF_EINVAL = -1,        /* invalid argument / circuit fails validation   */
  BF_ENOMEM = -2,        /* device or pinned allocation failed            */
  BF_ECUDA = -3,         /* CUDA runtime error (message has the details)  */
  BF_EUNSUPPORTED = -4,  /* valid request the library does not handle   */
  BF_ETIMEDOUT = -5,     /* bounded wait expired (serving loop)           */
  BF_EBUSY = -6          /* admission refused: not enough free HBM/slots  */
};

/* ---- state element types ----------------------------------------------- */
enum {
  BF_C128 = 0,   /* complex128: interleaved (re, im) FP64 pairs, FP64 math  */
  BF_C64 = 1     /* complex64:  interleaved (re, im) FP32 pairs, FP32 math  */
};

/* ---- gate kinds: values mirror GateKind (butterfly/core/gates.mojo:63-92) */
enum {
  BF_GATE_H = 0,
  BF_GATE_P = 1,
  BF_GATE_X = 2,
  BF_GATE_Y = 3,
  BF_GATE_Z = 4,
  BF_GATE_RX = 5,
  BF_GATE_RY = 6,
  BF_GATE_RZ = 7,
  BF_GATE_CUSTOM = 8   /* explicit 2x2 matrix in bf_op.mat                 */
};

/* ---- op kinds: one per Transformation variant (circuit.mojo:230-239) ---- */
enum {
  BF_OP_GATE = 0,      /* GateTransformation: controls + target + gate       */
  BF_OP_SWAP = 1,      /* SwapTransformation(a=target, b=target2)            */
  BF_OP_QREV = 2,      /* QubitReversalTransformation(targets; none = all)   */
  BF_OP_UNITARY = 3,   /* UnitaryTransformation(u, target, m=target2)        */
  BF_OP_CUNITARY = 4,  /* ControlledUnitaryTransformation(u, control, target, m) */
  BF_OP_BITREV = 5,    /* classical bit_reverse_tr(targets; none = all)      */
  BF_OP_PERMUTE = 6,   /* classical permute_qubits_tr(order)                 */
  BF_OP_CSWAP = 7,     /* classical swap_tr(a, b) (apply_swap)               */
  BF_OP_MEASURE = 8,   /* MeasurementTransformation (apply_measure): qubits =
                          targets, data = per-target values as doubles (-1 free,
                          0, 1) or NULL (all free), arg = seed (< 0: clock)   */
  BF_OP_GROVER_DIFFUSER = 9,   /* classical apply_grover_diffuser(qubits; none = all):
                                  x <- 2 mean - x over each target block      */
  BF_OP_GROVER_INVERSION0 = 10, /* classical apply_grover_inversion_0(qubits; none =
                                  all): negate the all-zero target amplitude  */
  BF_OP_CLASSICAL_ORACLE = 11, /* classical_oracle (grover.mojo:64-66): negate the
                                  amplitudes at the basis indices data[0..nqubits)
                                  (integers held exactly as doubles)          */
  BF_OP_MODEXP = 12,           /* apply_modexp (algos/shor.mojo:56-96): data =
                                  {n_exp, n_value, a, N} (nqubits = 4); the state
                                  has n_exp + n_value qubits, x = the low n_exp
                                  bits, y = the rest; |x, y> -> |x, y a^x mod N>
                                  for y < N, unchanged for y >= N              */
  BF_OP_MODEXP_INV = 13        /* apply_modexp_inverse (algos/shor.mojo:99-140):
                                  the same with a^-x mod N                    */
};

/* bf_op.flags */
#define BF_OPF_FUSE_WITH_NEXT 1u  /* this gate and the next one form a
                                     FusedPairTransformation (circuit.mojo:70-88) */

/*
 * One transformation.  Layout is fixed (128 bytes, 8-byte aligned) so that a
 * Mojo / ctypes / cgo caller can build the array without this header.
 *   GATE:      gate, target, controls (bitmask; ncontrols = its popcount and
 *              mirrors ControlKind), arg (angle for P/RX/RY/RZ), mat (CUSTOM).
 *   SWAP/CSWAP: target = a, target2 = b.
 *   QREV/BITREV/PERMUTE: qubits[0..nqubits) (nqubits = 0 means "all" for
 *              QREV/BITREV).
 *   UNITARY:   target, target2 = m, data = 2^m x 2^m complex row-major as
 *              interleaved (re, im) doubles.
 *   CUNITARY:  as UNITARY plus controls = 1 << control, ncontrols = 1.
 */
typedef struct bf_op {
  int32_t kind;
  int32_t gate;
  int32_t target;
  int32_t target2;
  uint64_t controls;
  int32_t ncontrols;
  uint32_t flags;
  double arg;
  double mat[8];            /* re00 im00 re01 im01 re10 im10 re11 im11 */
  const double* data;
  const int32_t* qubits;
  int64_t nqubits;
} bf_op;

/* ---- execution strategies ------------------------------------------------
 * Values 0..7 are the reference's ExecutionStrategy (context.mojo:33-40) and
 * are accepted only to be rejected with BF_EUNSUPPORTED (they are CPU paths).
 * BF_STRATEGY_GPU runs one kernel per transformation (the per-gate path);
 * BF_STRATEGY_GPU_FUSED groups consecutive gates into shared-memory tile
 * passes (the fused-grid path).                                              */
enum {
  BF_STRATEGY_GPU = 8,
  BF_STRATEGY_GPU_FUSED = 9
};

/* specialised-kernel switches, mirroring ExecContext.simd_use_specialized_*
 * (context.mojo:79-85). */
#define BF_SPEC_H   1u
#define BF_SPEC_P   2u
#define BF_SPEC_CP  4u
#define BF_SPEC_X   8u
#define BF_SPEC_CX  16u
#define BF_SPEC_RY  32u
#define BF_SPEC_CRY 64u
#define BF_SPEC_ALL 127u

typedef struct bf_exec_opts {
  int32_t strategy;          /* BF_STRATEGY_GPU or BF_STRATEGY_GPU_FUSED       */
  int32_t validate;          /* mirrors ExecContext.validate_circuit (default 1) */
  uint32_t specialized;      /* BF_SPEC_* mask (default BF_SPEC_ALL)           */
  int32_t tile_qubits;       /* fusion width of a tile pass; 0 = autotuned     */
  int32_t sync;              /* non-zero: block until the work has finished    */
  int32_t renormalize;       /* 0 (default): a complex64 state ends with the
                                norm it had before the circuit (double-float
                                norms, FP64 factor); -1: never.  complex128
                                states are never rescaled.                    */
  int32_t tensor_blocks;     /* 1 (default): tile passes may group their gates
                                into 5-qubit blocks applied as tensor-core
                                GEMMs (states of >= 12 qubits; per pass, where
                                cheaper): 3xTF32 for complex64; for complex128
                                exact products of five or six base-256 digits in bf16
                                (circuits of norm-preserving ops only).
                                0: CUDA-core tile passes only               */
  int32_t plan_dtype;        /* bf_plan_stats only: plan as for a BF_C128
                                (default) or BF_C64 state                   */
} bf_exec_opts;

/* Fills *opts with the defaults above (strategy GPU_FUSED). */
int bf_exec_opts_init(bf_exec_opts* opts);

/* ---- library ------------------------------------------------------------- */
int bf_version(int32_t* abi_version);
/* Copies the last error message of the calling thread (NUL-terminated). */
int bf_last_error(char* buf, size_t len);

/* ---- state lifecycle (QuantumState, butterfly/core/state.mojo:19-98) ------ */
typedef struct bf_state bf_state;

/* Allocates 2^num_qubits amplitudes on the current device, set to |0...0>
 * like State(n) (state.mojo:26-33). */
int bf_state_create(int32_t num_qubits, int32_t dtype, bf_state** out);
int bf_state_destroy(bf_state* st);
int bf_state_info(const bf_state* st, int32_t* num_qubits, int32_t* dtype);
/* |idx> basis state. */
int bf_state_set_basis(bf_state* st, uint64_t idx);
/* Host SoA arrays re[2^n], im[2^n] (the reference's layout, state.mojo:20-21)
 * to and from the device's interleaved layout, pageable or page-locked host
 * memory alike.  Upload returns once re and im have been read (the caller
 * may reuse them at once; the conversion on the device is stream-ordered
 * before later work on the state).  Download blocks until re and im hold
 * the amplitudes.  Both move 4 Mi-amplitude chunks through two device
 * buffers so that one chunk's host copy overlaps the next chunk's
 * conversion.  Transfers of at least one chunk from or to pageable arrays
 * go through the state's pinned host buffers (128 MiB, allocated on first
 * use), filled or drained by a pool of library host threads while the DMA
 * engine moves the other chunk. */
int bf_state_upload_soa(bf_state* st, const double* re, const double* im);
int bf_state_download_soa(bf_state* st, double* re, double* im);
/* Copies amplitudes [offset, offset+count) to host SoA arrays (blocks). */
int bf_state_download_range(bf_state* st, uint64_t offset, uint64_t count,
                            double* re, double* im);
int bf_state_sync(bf_state* st);
/* The state's cudaStream_t, for callers that order their own work on it. */
int bf_state_stream(bf_state* st, void** stream);

/* ---- execution (execute, butterfly/core/executors.mojo:723-730) ---------- */
/* Plans are cached per state (the last four, keyed by the exact op list with
 * its data and the options that shape a plan). */
int bf_execute(bf_state* st, const bf_op* ops, int64_t nops,
               const bf_exec_opts* opts);

/* Number of kernel launches bf_execute issued on this state since creation
 * (or since the last reset), for launch accounting. */
int bf_state_launch_count(const bf_state* st, uint64_t* launches, int32_t reset);

/* Pass timing: while enabled, bf_execute brackets every pass with CUDA events
 * on the state's stream.  bf_state_pass_times waits for the stream and writes,
 * per pass class, the number of timed passes and their summed device time in
 * ms (arrays of BF_PASS_CLASSES), then clears the record.  The classes: */
enum {
  BF_PASS_GATE = 0,          /* per-gate kernels                          */
  BF_PASS_TILE = 1,          /* CUDA-core shared-memory tile passes        */
  BF_PASS_BLOCK_TF32 = 2,    /* complex64 3xTF32 tensor-core block passes  */
  BF_PASS_BLOCK_DIGITS = 3,  /* complex128 digit tensor-core block passes  */
  BF_PASS_OTHER = 4,         /* permutations, Grover, measurement, modexp  */
  BF_PASS_CLASSES = 5
};
int bf_state_pass_timing(bf_state* st, int32_t enable);
int bf_state_pass_times(bf_state* st, int64_t* counts, double* ms);
/* complex128 digit passes: how many 4096-amplitude tiles ran with five and
 * with six base-256 digits since the state was created (or since the last
 * reset).  A tile takes five digits (the same fixed-point values, its top
 * digit being zero) when its norm is below 2^-9 of the state's digit scale;
 * waits for the state's stream.  No counterpart in the reference. */
int bf_state_digit_tiles(bf_state* st, uint64_t* five, uint64_t* six, int32_t reset);

/* ---- reductions ---------------------------------------------------------- */
/* sum |amp|^2, accumulated in FP64 (state.mojo:482-501 accumulates in the
 * state's type). */
int bf_norm2(bf_state* st, double* out);

/* <a|b> = sum conj(a_i) b_i of two states with the same qubit count, either
 * dtype, accumulated in double-float and summed in FP64; waits for both
 * states' pending work.  No counterpart in the reference: the fidelity
 * |<a|b>|^2 of a complex64 result against a complex128 one. */
int bf_inner(bf_state* a, bf_state* b, double* re, double* im);

/* ---- measurement and readout (apply_measure, state.mojo:447-553) ---------- */
/* Outcome probabilities over `qubits`: values[k] = 0 or 1 restricts to
 * amplitudes whose qubit k reads that value, -1 leaves it free (values may be
 * NULL: all free).  out[o] for the 2^f outcomes of the f free qubits, bit j of
 * o = the j-th free qubit in list order; f <= 20.  Blocks. */
int bf_probabilities(bf_state* st, const int32_t* qubits, const int8_t* values,
                     int32_t nqubits, double* out);
/* apply_measure: draws an outcome of the free targets with the reference's
 * generator (seed mod 2^31-1, times 48271 mod 2^31-1, scaled by the total
 * probability; a negative seed draws from the clock), collapses the state
 * onto it and renormalises by 1/sqrt(p).  Returns the outcome (bit j = j-th
 * free target) and its probability p.  Errors as the reference:
 * "Measurement probability is zero".  Blocks. */
int bf_measure(bf_state* st, const int32_t* targets, const int8_t* values,
               int32_t ntargets, int64_t seed, uint64_t* outcome,
               double* probability);
/* The k (1..64) most probable basis states, by descending |amp|^2, ties by
 * ascending index.  Blocks. */
int bf_probs_topk(bf_state* st, int32_t k, uint64_t* indices, double* probs);

/* ---- batches of independent circuits -------------------------------------
 * No single counterpart in the reference (its benches run circuits one at a
 * time through execute).  Many small circuits (1..30 qubits each, gate
 * transformations only) run from |0...0> in ONE persistent cooperative
 * launch: each circuit is planned into tile passes (tile width
 * opts->tile_qubits, or with 0 a width per qubit count picked by timing the
 * candidates at creation, see bf_batch_tuning), every tile of every pass
 * is a task, tasks are taken from an atomic ticket in pass-major order and a
 * task waits (bounded) for its circuit's previous pass.  The run is captured
 * into a CUDA graph at creation and replayed by bf_batch_run.
 * ops[c] / nops[c]: circuit c; the arrays are read during the call only. */
typedef struct bf_batch bf_batch;
int bf_batch_create(int32_t ncircuits, const int32_t* num_qubits,
                    const bf_op* const* ops, const int64_t* nops,
                    int32_t dtype, const bf_exec_opts* opts, bf_batch** out);
/* Runs every circuit from |0...0> (replays the graph); sync != 0 blocks and
 * reports BF_ETIMEDOUT if a task's bounded wait expired. */
int bf_batch_run(bf_batch* b, int32_t sync);
int bf_batch_sync(bf_batch* b);
/* Amplitudes of circuit c as SoA doubles (2^n each); blocks. */
int bf_batch_download(bf_batch* b, int32_t circuit, double* re, double* im);
int bf_batch_stats(bf_batch* b, int64_t* tasks, int64_t* passes,
                   uint64_t* state_bytes, int32_t* graph_captured,
                   uint64_t* launches);
int bf_batch_stream(bf_batch* b, void** stream);
/* The autotuning record of a batch created with opts->tile_qubits == 0.
 * For every qubit count n above 8 in the batch, each candidate tile width
 * (8..min(n, 12)) was timed on a sample of the batch's n-qubit circuits at
 * creation (one run of the sample, ms), and the fastest was kept for those
 * circuits (chosen = 1).  Writes up to cap rows and the row count. */
int bf_batch_tuning(bf_batch* b, int32_t* qubits, int32_t* widths, double* ms,
                    int32_t* chosen, int32_t cap, int32_t* count);
int bf_batch_destroy(bf_batch* b);

/* ---- serving: continuous batching of requests ------------------------------
 * No counterpart in the reference.  A request is a circuit (bf_op records,
 * copied at submission) with a qubit count and a dtype; it runs from
 * |0...0> and returns its top-k outcomes.  `slots` worker threads, each with
 * its own stream and state, admit the oldest queued request whose
 * statevector footprint 2^n * (8 | 16) B fits in the HBM budget left by the
 * running ones; states are allocated and freed stream-ordered, and requests
 * in different slots overlap on the device.  Requests whose estimated cost
 * (2^n * ops) is large wait in their own queue, cheapest first, served by
 * `large_slots` slots at the lowest stream priority while no small request
 * waits; a slot that frees up takes the oldest small request first and runs
 * it at the highest stream priority. */
typedef struct bf_server bf_server;
typedef struct bf_server_opts {
  int32_t slots;              /* concurrent requests; 0 = 12, at most 64       */
  int32_t tile_qubits;        /* fusion width; 0 = default                     */
  int32_t topk;               /* outcomes returned per request, 1..16; 0 = 16 */
  int32_t large_slots;        /* slots that run large requests; 0: all but a
                                 third of the slots (at least 2)           */
  uint64_t hbm_budget_bytes;  /* statevector bytes admitted at once;
                                 0 = 80 % of the free HBM at creation         */
  uint64_t large_cost;        /* a request is large when 2^n * ops exceeds
                                 this; 0 = 2^28                               */
} bf_server_opts;
typedef struct bf_result {
  uint64_t id;
  int32_t status;             /* BF_OK or the request's error code             */
  int32_t num_qubits;
  int32_t dtype;
  int32_t slot;
  int32_t k;
  int32_t reserved;
  double t_submit, t_start, t_done;   /* seconds on a monotonic clock          */
  uint64_t top_index[16];
  double top_prob[16];
  char message[128];
} bf_result;
typedef struct bf_server_counters {
  uint64_t submitted, completed, failed, queued, running;
  uint64_t bytes_in_use, peak_bytes, budget_bytes;
} bf_server_counters;
int bf_server_create(const bf_server_opts* opts, bf_server** out);
/* Queues a request; BF_EBUSY if its state can never fit the budget. */
int bf_server_submit(bf_server* s, int32_t num_qubits, int32_t dtype,
                     const bf_op* ops, int64_t nops, uint64_t* request_id);
/* Moves up to `max` finished results to out (oldest first). */
int bf_server_poll(bf_server* s, bf_result* out, int32_t max, int32_t* count);
/* Waits (bounded) until nothing is queued or running: BF_ETIMEDOUT else. */
int bf_server_wait_idle(bf_server* s, int64_t timeout_ms);
int bf_server_stats(bf_server* s, bf_server_counters* out);
/* Finishes the running requests, drops the queued ones, frees everything. */
int bf_server_destroy(bf_server* s);

/* ---- sum |amp|^2 without allocating ---------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: code running while its stream is captured into a CUDA graph, a
 * plugin inside a host framework whose allocator owns all device memory, or a
 * real-time path that cannot take cudaMalloc's implicit synchronisation.
 * d_amps: num_amps interleaved amplitudes (dtype BF_C128 or BF_C64) in the
 * caller's device memory; d_out: one double in the caller's device memory,
 * written with sum |amp|^2 (double-float accumulation), stream-ordered on
 * `stream` (a cudaStream_t; NULL = the default stream).  Nothing is
 * allocated: the partial sums use a 512 KiB array built into the library
 * (held by every GPU that loads it), which limits num_amps to 2^31; larger
 * inputs are rejected with BF_EINVAL, and so are d_amps not aligned to its
 * amplitude size (16 B for BF_C128, 8 B for BF_C64) and d_out not aligned to
 * 8 B, before anything is launched.  The first call on a device resolves
 * that array's address; make it before capturing a stream.  The address is
 * kept for the life of the process: after cudaDeviceReset on a device, do
 * not call this again there.  All calls share the array, so calls that
 * overlap on the GPU race: serialise them.  The sum is accumulated in
 * double-float (FP32's exponent range): components below about 1.1e-19 in
 * magnitude add nothing, and one of 1.8e19 or more overflows. */
int bf_norm2_noalloc(const void* d_amps, uint64_t num_amps, int32_t dtype,
                     double* d_out, void* stream);

/* ---- circuit wire formats ------------------------------------------------
 * An op list owns its records and the data / qubit arrays they point to.
 * bf_qasm3_parse reads the QASM3 subset of parse_qasm3_string
 * (butterfly/utils/qasm3_import.mojo:52-123: a qubit declaration, h, x,
 * p(angle), cp(angle); angles as numbers, pi, -pi, k*pi, pi/k, k/pi) with the
 * same error messages.  bf_ops_serialize writes a self-contained binary form
 * of any op array (little-endian: "BFOP", version 1, num_qubits, op count,
 * then per op its 104 fixed bytes, nqubits, and its data and qubit arrays);
 * with buf NULL it only reports the size.  bf_ops_deserialize reads it back.
 * No counterpart in the reference for the binary form. */
typedef struct bf_oplist bf_oplist;
int bf_qasm3_parse(const char* text, bf_oplist** out);
int bf_ops_serialize(int32_t num_qubits, const bf_op* ops, int64_t nops,
                     void* buf, size_t cap, size_t* len);
int bf_ops_deserialize(const void* buf, size_t len, bf_oplist** out);
/* the list's ops (valid until bf_oplist_destroy) and its qubit count */
int bf_oplist_view(const bf_oplist* list, const bf_op** ops, int64_t* nops,
                   int32_t* num_qubits);
int bf_oplist_destroy(bf_oplist* list);
/* submits a serialized op list (see bf_server_submit) */
int bf_server_submit_serialized(bf_server* server, const void* buf, size_t len,
                                int32_t dtype, uint64_t* id);

/* ---- host-only entry points (no device needed) --------------------------- */
/* validate_circuit (butterfly/core/executors.mojo:129-185) for a state of
 * num_qubits qubits. */
int bf_validate(int32_t num_qubits, const bf_op* ops, int64_t nops);
/* Plans ops as bf_execute would and reports the launches it would issue and
 * the algorithmic bytes they move, in units of the state's size S.
 * tile_passes counts every tile pass; block_passes of them run on the
 * tensor cores (tensor_blocks set), with `blocks` 5-qubit blocks in all. */
int bf_plan_stats(int32_t num_qubits, const bf_op* ops, int64_t nops,
                  const bf_exec_opts* opts, int64_t* tile_passes,
                  int64_t* gate_kernels, int64_t* other_passes,
                  double* bytes_in_S, int64_t* block_passes,
                  int64_t* blocks);

#ifdef __cplusplus
}
#endif

#endif /* BFGPU_H */

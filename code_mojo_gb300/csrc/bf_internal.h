// bf_internal.h — shared declarations of the bfgpu engine (host + device).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bfgpu.h"

namespace bf {

// ---------------------------------------------------------------------------
// Errors: host code throws bf::Error; the C ABI converts it to a status code
// and a thread-local message.
struct Error {
  int code;
  std::string msg;
};
[[noreturn]] void fail(int code, const char* fmt, ...);
void check_cuda(cudaError_t e, const char* what);
#define BF_CUDA(call) ::bf::check_cuda((call), #call)

// ---------------------------------------------------------------------------
// Devices.  Kernel attributes (cudaFuncSetAttribute) belong to one device,
// and the entry points may be called from several threads at once, so each
// launcher configures its kernels once per device under a lock.
constexpr int kMaxDevices = 64;
class PerDeviceOnce {
 public:
  // Runs f() the first time it is called with the current device `dev`.
  template <class F>
  void run(int dev, F&& f) {
    if (dev < 0 || dev >= kMaxDevices) fail(BF_EUNSUPPORTED, "device ordinal %d out of range", dev);
    const uint64_t bit = 1ull << dev;
    if (done_.load(std::memory_order_acquire) & bit) return;
    std::lock_guard<std::mutex> lock(mu_);
    if (done_.load(std::memory_order_relaxed) & bit) return;
    f();
    done_.fetch_or(bit, std::memory_order_release);
  }

 private:
  std::atomic<uint64_t> done_{0};
  std::mutex mu_;
};

// Makes `dev` the calling thread's current device for the guard's lifetime
// and restores the caller's device afterwards.  Every entry point that takes
// a state, batch or server runs its work under one, so a handle created on
// one GPU keeps launching there whatever device the calling thread has set.
class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev_) != cudaSuccess) {
      cudaGetLastError();
      prev_ = -1;
    }
    if (dev >= 0 && prev_ != dev) {
      BF_CUDA(cudaSetDevice(dev));
      switched_ = true;
    }
  }
  ~DeviceGuard() {
    if (switched_ && prev_ >= 0) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

 private:
  int prev_ = -1;
  bool switched_ = false;
};
int current_device();

// ---------------------------------------------------------------------------
// Compute precision of a state.
//   F64 : complex128 storage, FP64 arithmetic (DFMA).
//   DF  : complex128 storage, double-float arithmetic (FP32 hi+lo pairs, the
//         error-free transformations of Dekker 1971 / Knuth TAOCP vol. 2) with
//         the FP64 <-> pair conversions done in integer arithmetic.
//   F32 : complex64 storage, FP32 arithmetic.
enum Prec { PREC_F64 = 0, PREC_DF = 1, PREC_F32 = 2 };

// ---------------------------------------------------------------------------
// A lowered single-target gate (after kind/arg -> matrix on the host).
enum GKind : int32_t {
  GK_DENSE = 0,  // full 2x2 complex matrix m
  GK_H = 1,      // Hadamard: (u+v)*s, (u-v)*s with s = 0.7071067811865476
  GK_SWAP = 2,   // X: exchange the pair
  GK_PHASE = 3,  // diag(1, e^{i theta}): m[6], m[7] = cos, sin (P, Z, CP, CZ, MCP)
  GK_DIAG = 4,   // diag(d0, d1): m[0..1] = d0, m[6..7] = d1 (RZ)
  GK_RY = 5,     // real rotation [[c,-s],[s,c]]: m[0] = c, m[4] = s
  GK_DENSE_R = 6, // full 2x2 matrix whose m00 is real (m[1] == 0), as in every U3
  GK_UNITARY = 7  // dense 2^um x 2^um matrix on qubits target .. target + um - 1
};

// Dense unitaries of up to this many qubits join fused runs (tile passes
// and tensor-core blocks, whose 5 qubits bound it); wider ones run as their
// own pass.
constexpr int kTileUnitaryMax = 5;

struct GateInstr {
  int32_t kind;     // GKind
  int32_t target;   // GK_UNITARY: the lowest of its qubits
  uint64_t cmask;   // control qubits (all must be 1)
  double m[8];      // re00 im00 re01 im01 re10 im10 re11 im11
  float mhl[16];    // the same eight values as (hi, lo) FP32 pairs
  int32_t um;       // GK_UNITARY: qubit count (2..kTileUnitaryMax); 0 otherwise
  int32_t uoff;     // GK_UNITARY: offset (in doubles) of its row-major
                    // interleaved matrix in the run's unitary pool
};

inline bool gk_is_diagonal(int k) { return k == GK_PHASE || k == GK_DIAG; }
// qubits a gate acts on non-diagonally, and all the qubits it touches
inline uint64_t gate_xmask(const GateInstr& g) {
  if (g.kind == GK_UNITARY) return ((1ull << g.um) - 1ull) << g.target;
  return gk_is_diagonal(g.kind) ? 0ull : 1ull << g.target;
}
inline uint64_t gate_amask(const GateInstr& g) {
  const uint64_t t = g.kind == GK_UNITARY ? ((1ull << g.um) - 1ull) << g.target : 1ull << g.target;
  return g.cmask | t;
}

// Per-gate algorithmic bytes of one pass (read + write of every amplitude the
// gate must touch), in units of the state's byte size S.
double gate_bytes_fraction(const GateInstr& g);

// ---------------------------------------------------------------------------
// Tile pass: one shared-memory resident block of 2^K amplitudes per CTA,
// indexed by the tile qubits q[0..K) (ascending, q[j] = j for j < low).
constexpr int kMaxTileQubits = 13;
constexpr int kTileLowQubits = 5;

struct TileOp {
  int32_t kind;       // GKind
  int32_t tloc;       // local bit of the target, or -1 (diagonal gate whose
                      // target lies outside the tile); GK_UNITARY: local bit
                      // of its lowest qubit (its qubits are consecutive
                      // tile qubits, so they sit at tloc .. tloc + um - 1)
  int32_t tglob;      // global target qubit
  uint32_t cmask_loc; // control bits inside the tile (local positions)
  uint64_t cmask_out; // control bits outside the tile (global positions)
  double m[8];
  float mhl[16];
  int32_t um;         // GK_UNITARY: qubit count; 0 otherwise
  int32_t uoff;       // GK_UNITARY: offset (in doubles) of its matrix in the
                      // program's unitary pool
};

struct TilePass {
  int32_t K;
  int32_t L;   // q[j] = j for j < L (the always-resident low qubits)
  int32_t q[kMaxTileQubits];
  std::vector<TileOp> ops;
};

// ---------------------------------------------------------------------------
// Tensor-core block passes (complex64): a 12-qubit tile whose gates are
// grouped into blocks of 5 tile qubits, each applied as one 32x32 complex
// matrix.  A block's matrix may depend on up to 3 qubits outside the tile
// (controls, or targets of diagonal gates); its 2^nout variants are stored
// consecutively, variant v for outside bits (bit k of v = qubit outpos[k]).
constexpr int kBlockTileQubits = 12;
constexpr uint32_t kBlockImageBytes = 32768;  // one matrix: TF32 hi and lo parts, swizzled
constexpr int kBlockThreads = 512;            // threads of the 3xTF32 block kernel
constexpr int kBlockThreadElems = 8;          // amplitudes each of its threads moves per block
constexpr int kDigitThreads = 1024;           // threads of the digit block kernel (4 amplitudes each)
constexpr int kBlockTableEntries = 4096;      // one destination table: threads x amplitudes
constexpr int kMaxPassBlocks = 32;

struct Blk5 {
  uint32_t tmask;     // the block's 5 local positions (bits of the 12-bit tile index)
  int32_t nout;
  int32_t outpos[3];
  uint32_t img;       // image index of variant 0
  uint32_t offs;      // index (units of kBlockTableEntries) of the
                      // shared-memory destinations of this block's results
  uint32_t load_offs; // first block of a pass: destinations of the loaded tile
};

// Two operand formats for the blocks:
//   BLOCK_TF32   complex64: FP32 operands split into TF32 hi and lo (3xTF32);
//                a matrix image is 32 KiB.
//   BLOCK_DIGITS complex128: values as 6 signed base-256 digits held exactly
//                in bf16 (x / scale = 2^-8 sum_i d_i 2^-8i); the digit
//                products accumulate exactly in FP32 per digit level; a
//                matrix image is 6 digit planes of 8 KiB.
enum BlockFormat { BLOCK_TF32 = 0, BLOCK_DIGITS = 1 };
constexpr int kDigits = 6;
constexpr uint32_t kDigitImageBytes = kDigits * 8192;

// Partitions the ops of a 12-qubit tile pass into blocks and appends their
// matrix images and destination tables (u16 per thread and element: the
// next block's operand offset in the format's units, or after the last
// block the tile element); false when an op cannot be placed (more than 5
// tile qubits or more than 3 outside qubits on its own), the pass needs more
// than min(kMaxPassBlocks, max_blocks) blocks (checked before any matrix is
// built), or (BLOCK_DIGITS) a block's matrix is not unitary to 1e-12.
// `umats` is the unitary pool that GK_UNITARY ops index (may be null when
// the pass has none).
bool plan_blocks(const TilePass& tp, std::vector<Blk5>& blocks, std::vector<unsigned char>& images,
                 std::vector<uint16_t>& offsets, BlockFormat format = BLOCK_TF32, int max_blocks = kMaxPassBlocks,
                 const double* umats = nullptr);
#ifdef __CUDACC__
#define BF_HOST_DEVICE __host__ __device__
#else
#define BF_HOST_DEVICE
#endif
// operand layout shared by the planner and the kernel: byte offset of
// complex element (row g, column j) in a K-major, 128-byte-swizzled operand
BF_HOST_DEVICE inline uint32_t block_operand_offset(uint32_t g, uint32_t j) {
  return ((j >> 4) << 14) + (g << 7) + ((((j & 15) >> 1) ^ (g & 7)) << 4) + ((j & 1) << 3);
}
// byte offset of complex element (row g, column j) in one bf16 digit plane:
// K-major rows of 64 bf16 (re, im interleaved), 16-byte chunks swizzled by
// the row's low three bits; 16 KiB per plane
BF_HOST_DEVICE inline uint32_t digit_operand_offset(uint32_t g, uint32_t j) {
  return (g << 7) + ((((j >> 2) ^ (g & 7))) << 4) + ((j & 3) << 2);
}
// The matrix image of a 32x32 complex matrix u (row-major, interleaved
// re/im): the real 64x64 operand R^T, split into TF32 hi and lo parts, in
// the swizzled K-major layout of the block kernel.
void block_image(const double* u, unsigned char* img);

// ---------------------------------------------------------------------------
struct PlanCache;  // a state's recent plans (api.cpp)

// The device state.
struct State {
  int32_t n = 0;
  int32_t dtype = BF_C128;
  int32_t prec = PREC_F64;
  uint64_t N = 0;
  void* amp = nullptr;        // interleaved complex, 16 B (C128) or 8 B (C64)
  void* scratch = nullptr;    // second state-sized buffer, lazily allocated
  cudaStream_t stream = nullptr;
  int device = 0;
  int num_sms = 0;
  uint64_t launches = 0;
  // program buffer for tile ops (device) and its pinned host staging
  TileOp* d_prog = nullptr;
  TileOp* h_prog = nullptr;
  size_t prog_cap = 0;
  cudaEvent_t prog_event = nullptr;
  bool prog_event_live = false;
  // staging for SoA <-> interleaved conversion: two chunk buffers, so that
  // the copy of one chunk (on copy_stream) overlaps the conversion kernel of
  // the other (on stream); the events order the two streams per buffer
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t stage_copied[2] = {nullptr, nullptr};  // copy into / out of buffer k done
  cudaEvent_t stage_done[2] = {nullptr, nullptr};    // conversion kernel on buffer k done
  cudaEvent_t stage_start = nullptr;                 // the state's earlier work
  // pinned host staging for large transfers from or to pageable host arrays
  // (two chunk buffers, re and im each): host threads copy between the
  // caller's arrays and these while the DMA engine moves the other buffer
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  // dense unitary matrix (device copy of the current op's matrix)
  double* d_umat = nullptr;
  // norms before / after a complex64 circuit and the rescale factor
  double* d_renorm = nullptr;
  size_t renorm_cap = 0;
  // reduction partials
  double* d_partial = nullptr;
  double* h_partial = nullptr;
  size_t partial_cap = 0;
  // error flag of kernels with bounded waits (device word, pinned copy)
  int* d_flag = nullptr;
  int* h_flag = nullptr;
  bool flag_used = false;
  // the state runs in a server slot that shares the GPU with other slots:
  // long persistent kernels (grid-wide Grover loops) are not used
  bool shared_gpu = false;
  // block descriptors and matrix images of tensor-core passes (device) and
  // their pinned staging; uploaded with the tile program
  unsigned char* d_aux = nullptr;
  unsigned char* h_aux = nullptr;
  size_t aux_cap = 0;
  // scale exponent of the complex128 digit passes (device int)
  int* d_scale = nullptr;
  // digit passes' tiles run with five and with six digits (device u64 x 2)
  unsigned long long* d_digit_tiles = nullptr;
  // recent plans and the one whose program is on the device
  PlanCache* plans = nullptr;
  uint64_t uploaded_plan = 0;
  // pass timing: event pairs around each pass while enabled (pool reused)
  bool pass_timing = false;
  std::vector<cudaEvent_t> pass_events;
  std::vector<int> pass_class;   // class of recorded pair k (events 2k, 2k+1)

  // pinned host buffers outgrown while copies from them may be in flight;
  // freed with the state (cudaFreeHost can synchronise the device)
  std::vector<void*> retired_host;

  size_t amp_bytes() const { return dtype == BF_C128 ? 16 : 8; }
  size_t bytes() const { return (size_t)N * amp_bytes(); }
};

// Work buffers of a state are (re)allocated stream-ordered on its own stream
// (cudaMallocAsync / cudaFreeAsync) so that growing one never waits for
// kernels of other states; pinned host buffers that are outgrown are retired
// until the state is released.
void* dev_alloc(State& st, size_t bytes);   // throws BF_ENOMEM
void dev_free(State& st, void* p);
void* host_alloc(size_t bytes);             // pinned; throws BF_ENOMEM
void host_retire(State& st, void* p);
void upload_program_reserve(State& st, size_t ops);
// The state's device error flag (allocated and zeroed on first use); kernels
// with bounded waits set it.  flag_readback queues its copy to the host after
// such kernels; sync_state synchronises the stream and throws BF_ETIMEDOUT
// (clearing the flag) when a wait had expired.
int* state_flag(State& st);
void flag_readback(State& st);
void sync_state(State& st);

// ---------------------------------------------------------------------------
// Kernel launchers (device code lives in the .cu files).
void launch_gate(State& s, const GateInstr& g);
// d_umats: the device copy of the program's unitary pool (null without GK_UNITARY ops)
void launch_tile_pass(State& s, const TileOp* d_ops, int nops, const TilePass& p, const double* d_umats = nullptr);
void launch_block_pass(State& st, const Blk5* d_blocks, int nblocks, const unsigned char* d_images,
                       const uint16_t* d_offsets, const TilePass& p);
// complex128 digit blocks (BLOCK_DIGITS); d_exp holds the scale exponent
// that launch_digit_scale computed from the state's norm
// in_fixed: the state holds the previous digit pass's output as int64 pairs
// (the integers V of the unit 2^-48 of the scale, not FP64 values);
// out_fixed: write them so for the next digit pass.  Between two digit
// passes of one circuit the state is in this form; any other reader needs
// FP64, so the pass before it writes FP64.
void launch_block_pass_digits(State& st, const Blk5* d_blocks, int nblocks, const unsigned char* d_images,
                              const uint16_t* d_offsets, const TilePass& p, const int* d_exp, bool in_fixed = false,
                              bool out_fixed = false);
void launch_digit_scale(State& st, int* d_exp);
// the device counters of five- and six-digit tiles (allocated and zeroed on first use)
unsigned long long* digit_tile_counters(State& st);
void launch_norm2_partials(State& st, unsigned blocks);  // into st.d_partial (ensure_partials first)
void launch_bitrev_full(State& s);
void launch_permute(State& s, const int32_t* src_bit_of_dst);  // dst bit j <- src bit perm[j]
void launch_swap_bits(State& s, int a, int b);
// |x, y> -> |x, y * base^x mod N> (y < N) over the whole state, x the low n_exp bits
void launch_modexp(State& s, int n_exp, uint64_t base, uint64_t modulus);
void launch_unitary(State& s, const double* h_u, int target, int m, int control);
void launch_set_basis(State& s, uint64_t idx);
void launch_interleave(State& s, const double* d_re, const double* d_im, uint64_t off, uint64_t cnt);
void launch_deinterleave(State& s, double* d_re, double* d_im, uint64_t off, uint64_t cnt);
double reduce_norm2(State& s);
// <a|b> = sum conj(a_i) b_i (states of equal size, either dtype); synchronises a
void inner_product(State& a, State& b, double* re, double* im);
// complex64: restore the norm measured by launch_norm_before (or 1), stream-ordered
void launch_norm_before(State& st);
void launch_renormalize(State& st, bool unit_before);
void ensure_partials(State& st, size_t blocks);  // 2*blocks doubles, device + pinned host
void marginal_probs(State& st, const int32_t* q, const int8_t* values, int32_t nq, std::vector<double>& out);
void measure(State& st, const int32_t* q, const int8_t* values, int32_t nq, int64_t seed, uint64_t* outcome,
             double* prob);
void probs_topk(State& st, int k, uint64_t* idx, double* probs);
void launch_grover_inversion0(State& st, const int32_t* q, int32_t nq);
void launch_grover_diffuser(State& st, const int32_t* q, int32_t nq);
void launch_classical_oracle(State& st, const double* idx, int64_t count);
// iters x (negate marked[0..nmarked), diffuser over every qubit) in one launch
void launch_grover_loop(State& st, const uint64_t* marked, int nmarked, int iters);
int grover_loop_max_marked();
// sum |amp|^2 of caller memory with the library's static scratch (noalloc.cu)
void norm2_noalloc(const void* d_amps, uint64_t num_amps, int32_t dtype, double* d_out, cudaStream_t stream);

int tile_max_qubits(const State& s);

// ---------------------------------------------------------------------------
// Host planner and lowering.
GateInstr lower_gate(const bf_op& o, uint32_t specialized);
void validate_ops(int n, const bf_op* ops, int64_t nops);
// Groups a run of gates into tile passes (tile width K); gates for which a
// per-gate kernel moves fewer bytes than a tile pass stay single.
struct PlanStep {
  bool is_tile;
  GateInstr gate;  // when !is_tile
  TilePass tile;   // when is_tile
};
// block_units > 0: tile passes may run as tensor-core blocks, one block
// costing that many dense gates of the CUDA-core tile kernel; a pass whose
// blocks would be cheaper gets its tile chosen for work per unit of
// block-pass time rather than work per pass, a pass costing pass_cost
// blocks besides its blocks.  keep_wide_unitaries: a pass that would hold
// only a dense unitary of 4 or 5 qubits stays a pass (the complex128 digit
// blocks run it faster than the double-float unitary kernel)
std::vector<PlanStep> plan_gates(int n, const std::vector<GateInstr>& gates, int K, bool allow_single = true,
                                 double block_units = 0, double pass_cost = 2.5, bool keep_wide_unitaries = false);

// bf_execute's body on a prepared state; stream, event and SM count of a
// state; releasing every buffer a state owns (api.cpp).
void execute_ops(State& st, const bf_op* ops, int64_t nops, bf_exec_opts o);
void init_state_runtime(State& st);
void release_state_members(State& st);

// Batches of independent circuits (batch.cu).
struct Batch;
Batch* batch_create(int ncirc, const int32_t* nq, const bf_op* const* ops, const int64_t* nops, int dtype,
                    const bf_exec_opts& o, int prec);
void batch_run(Batch& b, bool sync);
void batch_sync(Batch& b);
void batch_download(Batch& b, int c, double* re, double* im);
void batch_destroy(Batch* b);
void batch_stats(const Batch& b, int64_t* tasks, int64_t* passes, uint64_t* state_bytes, int32_t* graph,
                 uint64_t* launches);
void* batch_stream(const Batch& b);
int batch_device(const Batch& b);
void batch_tuning(const Batch& b, int32_t* qubits, int32_t* widths, double* ms, int32_t* chosen, int32_t cap,
                  int32_t* count);

// Wire formats (wire.cpp).
struct OpList;
size_t op_data_len(const bf_op& o);    // doubles behind op.data for its kind
size_t op_qubits_len(const bf_op& o);  // int32s behind op.qubits for its kind
OpList* qasm3_parse(const char* text);
std::vector<unsigned char> ops_serialize(int32_t n, const bf_op* ops, int64_t nops);
OpList* ops_deserialize(const void* blob, size_t len);
void oplist_view(const OpList& L, const bf_op** ops, int64_t* nops, int32_t* n);
void oplist_destroy(OpList* L);

// Serving loop (server.cpp).
struct Server;
Server* server_create(const bf_server_opts& opts);
uint64_t server_submit(Server& sv, int32_t n, int32_t dtype, const bf_op* ops, int64_t nops);
int server_poll(Server& sv, bf_result* out, int max);
bool server_wait_idle(Server& sv, int64_t timeout_ms);
void server_stats(Server& sv, bf_server_counters& s);
void server_destroy(Server* sv);
int server_device(const Server& sv);

}  // namespace bf

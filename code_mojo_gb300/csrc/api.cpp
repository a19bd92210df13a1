// api.cpp — the C ABI (include/bfgpu.h): state lifecycle, boundary copies,
// and bf_execute, the GPU counterpart of execute_with_handlers
// (butterfly/core/executors.mojo:268-319).
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include <unistd.h>

#include "bf_internal.h"

namespace bf {

static thread_local std::string g_last_error;

template <class F>
static int guarded(F&& f) {
  try {
    f();
    return BF_OK;
  } catch (const Error& e) {
    g_last_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return BF_ENOMEM;
  } catch (...) {
    g_last_error = "unexpected internal error";
    return BF_ECUDA;
  }
}

static int default_tile_qubits(const State& st) {
  // 2^11 amplitudes (32 KiB at complex128) per CTA: six resident CTAs per SM.
  (void)st;
  return 11;
}

static int env_int(const char* name, int dflt) {
  const char* v = std::getenv(name);
  return (v && *v) ? std::atoi(v) : dflt;
}

// ---- stream-ordered work buffers ------------------------------------------------
void* dev_alloc(State& st, size_t bytes) {
  void* p = nullptr;
  if (cudaMallocAsync(&p, std::max<size_t>(bytes, 256), st.stream) != cudaSuccess) {
    cudaGetLastError();
    fail(BF_ENOMEM, "cannot allocate %zu bytes of device work space", bytes);
  }
  return p;
}

void dev_free(State& st, void* p) {
  if (p) cudaFreeAsync(p, st.stream);
}

void* host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaHostAlloc(&p, std::max<size_t>(bytes, 64), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    fail(BF_ENOMEM, "cannot allocate %zu bytes of pinned host memory", bytes);
  }
  return p;
}

void host_retire(State& st, void* p) {
  if (p) st.retired_host.push_back(p);
}

unsigned long long* digit_tile_counters(State& st) {
  if (!st.d_digit_tiles) {
    st.d_digit_tiles = static_cast<unsigned long long*>(dev_alloc(st, 2 * sizeof(unsigned long long)));
    BF_CUDA(cudaMemsetAsync(st.d_digit_tiles, 0, 2 * sizeof(unsigned long long), st.stream));
  }
  return st.d_digit_tiles;
}

int* state_flag(State& st) {
  if (!st.d_flag) {
    st.d_flag = static_cast<int*>(dev_alloc(st, 16));
    st.h_flag = static_cast<int*>(host_alloc(16));
    *st.h_flag = 0;
    BF_CUDA(cudaMemsetAsync(st.d_flag, 0, 16, st.stream));
  }
  st.flag_used = true;
  return st.d_flag;
}

void flag_readback(State& st) {
  if (!st.flag_used) return;
  BF_CUDA(cudaMemcpyAsync(st.h_flag, st.d_flag, sizeof(int), cudaMemcpyDeviceToHost, st.stream));
  st.flag_used = false;
}

void sync_state(State& st) {
  BF_CUDA(cudaStreamSynchronize(st.stream));
  if (st.h_flag && *st.h_flag) {
    *st.h_flag = 0;
    BF_CUDA(cudaMemsetAsync(st.d_flag, 0, sizeof(int), st.stream));
    fail(BF_ETIMEDOUT, "a bounded wait on the device expired; the state's contents are undefined");
  }
}

// ---- program buffer for tile ops ---------------------------------------------
void upload_program_reserve(State& st, size_t ops) {
  if (ops <= st.prog_cap) return;
  size_t cap = std::max(ops, st.prog_cap * 2);
  // copies out of the old pinned buffer may still be in flight: retire it
  host_retire(st, st.h_prog);
  st.h_prog = nullptr;
  dev_free(st, st.d_prog);  // stream-ordered: kernels already queued keep their copy
  st.d_prog = nullptr;
  st.prog_cap = 0;
  st.d_prog = static_cast<TileOp*>(dev_alloc(st, cap * sizeof(TileOp)));
  st.h_prog = static_cast<TileOp*>(host_alloc(cap * sizeof(TileOp)));
  st.prog_cap = cap;
  st.prog_event_live = false;
}

// Everything a plan uploads: tile ops, and in the auxiliary buffer the
// tensor-core passes' block descriptors, (at a 256-byte boundary) their
// matrix images and destination tables, then (at a 16-byte boundary) the
// unitary pool that the tile ops of dense unitaries index.
struct Program {
  std::vector<TileOp> ops;
  std::vector<Blk5> blocks;
  std::vector<unsigned char> images;
  std::vector<uint16_t> offsets;
  std::vector<double> umats;
  size_t images_offset() const { return (blocks.size() * sizeof(Blk5) + 255) & ~(size_t)255; }
  size_t offsets_offset() const { return images_offset() + images.size(); }
  size_t umats_offset() const { return (offsets_offset() + offsets.size() * sizeof(uint16_t) + 15) & ~(size_t)15; }
  size_t aux_bytes() const {
    if (blocks.empty() && umats.empty()) return 0;
    return umats_offset() + umats.size() * sizeof(double);
  }
};

// id: the plan's cache id (0: not cached); a program already on the device
// for the same id is not uploaded again
static void upload_program(State& st, const Program& pg, uint64_t id) {
  const std::vector<TileOp>& prog = pg.ops;
  const size_t aux = pg.aux_bytes();
  if (prog.empty() && aux == 0) return;
  if (id != 0 && st.uploaded_plan == id) return;
  st.uploaded_plan = id;
  if (st.prog_event_live) BF_CUDA(cudaEventSynchronize(st.prog_event));
  if (!prog.empty()) {
    upload_program_reserve(st, prog.size());
    std::memcpy(st.h_prog, prog.data(), prog.size() * sizeof(TileOp));
    BF_CUDA(cudaMemcpyAsync(st.d_prog, st.h_prog, prog.size() * sizeof(TileOp), cudaMemcpyHostToDevice, st.stream));
  }
  if (aux) {
    if (aux > st.aux_cap) {
      size_t cap = std::max(aux, 2 * st.aux_cap);
      host_retire(st, st.h_aux);
      dev_free(st, st.d_aux);
      st.h_aux = nullptr;
      st.d_aux = nullptr;
      st.aux_cap = 0;
      st.d_aux = static_cast<unsigned char*>(dev_alloc(st, cap));
      st.h_aux = static_cast<unsigned char*>(host_alloc(cap));
      st.aux_cap = cap;
    }
    std::memcpy(st.h_aux, pg.blocks.data(), pg.blocks.size() * sizeof(Blk5));
    std::memcpy(st.h_aux + pg.images_offset(), pg.images.data(), pg.images.size());
    std::memcpy(st.h_aux + pg.offsets_offset(), pg.offsets.data(), pg.offsets.size() * sizeof(uint16_t));
    std::memcpy(st.h_aux + pg.umats_offset(), pg.umats.data(), pg.umats.size() * sizeof(double));
    BF_CUDA(cudaMemcpyAsync(st.d_aux, st.h_aux, aux, cudaMemcpyHostToDevice, st.stream));
  }
  BF_CUDA(cudaEventRecord(st.prog_event, st.stream));
  st.prog_event_live = true;
}

// ---- execution -------------------------------------------------------------
// A step is one launch (or a launch group) in op order.
struct Step {
  enum Kind {
    GATE, TILE, TBLOCK, BITREV, PERMUTE, SWAPBITS, UNITARY, MEASURE, DIFFUSER, INVERSION0, ORACLE, GROVER_LOOP,
    MODEXP
  } kind;
  GateInstr gate;
  TilePass tile;            // ops moved into the program; tile.ops emptied
  size_t prog_off = 0;
  int nprog = 0;
  std::vector<int32_t> src_of;
  int a = 0, b = 0;
  std::vector<double> u;
  int ut = 0, um = 0, uc = -1;
  std::vector<int32_t> mq;   // measured qubits
  std::vector<int8_t> mv;    // their values (-1 free)
  int64_t seed = -1;
  std::vector<uint64_t> marked;  // Grover loop: indices the oracle negates
  int reps = 0;                  // Grover loop: iterations
  size_t blk_off = 0;            // tensor-core pass: its blocks in the program
  int nblk = 0;
  uint64_t base = 0, modulus = 0;  // modexp: a (or a^-1 mod N) and N; a = n_exp
  bool digits = false;             // tensor-core pass in the complex128 digit form
  bool unitaries = false;          // tile pass: holds dense unitaries (GK_UNITARY ops)
};

// a^-1 mod N for gcd(a, N) = 1 (extended Euclid, as modinv in algos/shor.mojo:46-53)
static int64_t modinv(int64_t a, int64_t N) {
  int64_t r0 = N, r1 = a, t0 = 0, t1 = 1;
  while (r1 != 0) {
    int64_t q = r0 / r1, r = r0 - q * r1, t = t0 - q * t1;
    r0 = r1;
    r1 = r;
    t0 = t1;
    t1 = t;
  }
  return ((t0 % N) + N) % N;
}

// Grover loop detection: the number of consecutive (classical oracle with
// the same index list, diffuser over every qubit) pairs starting at ops[i],
// or 0 when the oracle's odd-multiplicity indices exceed the loop's limit.
static bool full_diffuser(int n, const bf_op& o) {
  if (o.kind != BF_OP_GROVER_DIFFUSER) return false;
  if (o.nqubits == 0) return true;
  if (o.nqubits != n || !o.qubits) return false;
  uint64_t seen = 0;
  for (int k = 0; k < n; ++k) {
    int q = o.qubits[k];
    if (q < 0 || q >= n || ((seen >> q) & 1)) return false;
    seen |= 1ull << q;
  }
  return true;
}

static int64_t grover_loop_reps(int n, const bf_op* ops, int64_t nops, int64_t i) {
  const bf_op& o = ops[i];
  if (o.nqubits < 0 || o.nqubits > grover_loop_max_marked() || (o.nqubits > 0 && !o.data)) return 0;
  int64_t reps = 0;
  for (int64_t j = i; j + 1 < nops; j += 2) {
    const bf_op& a = ops[j];
    if (a.kind != BF_OP_CLASSICAL_ORACLE || a.nqubits != o.nqubits || !full_diffuser(n, ops[j + 1])) break;
    if (o.nqubits > 0 && (!a.data || std::memcmp(a.data, o.data, (size_t)o.nqubits * sizeof(double)) != 0)) break;
    ++reps;
  }
  return reps;
}

static bool is_h(const bf_op& o) { return o.ncontrols == 0 && o.gate == BF_GATE_H; }
static bool is_p(const bf_op& o) { return o.ncontrols == 0 && o.gate == BF_GATE_P; }
static bool is_cp(const bf_op& o) { return o.ncontrols == 1 && o.gate == BF_GATE_P; }

// 4x4 composition of a FusedPairTransformation that matches none of the sparse
// kernels (transformations_fusion.mojo:277-310): m = M1 * M0 on (q_low, q_low+1).
static void fused_pair_matrix(const bf_op& t0, const bf_op& t1, int& q_low, std::vector<double>& out) {
  auto gm = [](const bf_op& o, double* m) {
    GateInstr g = lower_gate(o, 0);
    std::memcpy(m, g.m, 8 * sizeof(double));
  };
  auto ctz = [](uint64_t v) { return v ? __builtin_ctzll(v) : 0; };
  int c0 = t0.ncontrols == 1 ? ctz(t0.controls) : 0;
  int c1 = t1.ncontrols == 1 ? ctz(t1.controls) : 0;
  q_low = t0.target;
  if (t0.ncontrols == 1) q_low = std::min(q_low, c0);
  q_low = std::min(q_low, t1.target);
  if (t1.ncontrols == 1) q_low = std::min(q_low, c1);
  auto to4 = [&](const bf_op& o, int ctl, double* M) {  // 16 complex, row-major
    double g[8];
    gm(o, g);
    for (int i = 0; i < 32; ++i) M[i] = 0;
    auto G = [&](int r, int c, int part) { return g[2 * (2 * r + c) + part]; };
    if (o.ncontrols == 1) {
      for (int b0 = 0; b0 < 2; ++b0)
        for (int b1 = 0; b1 < 2; ++b1) {
          int in = b0 + 2 * b1;
          int cb = ctl == q_low ? b0 : b1;
          int tb = o.target == q_low ? b0 : b1;
          if (cb == 0) {
            M[2 * (in * 4 + in)] = 1;
          } else {
            for (int ot = 0; ot < 2; ++ot) {
              int ob0 = b0, ob1 = b1;
              if (o.target == q_low) ob0 = ot; else ob1 = ot;
              int oi = ob0 + 2 * ob1;
              M[2 * (oi * 4 + in)] = G(ot, tb, 0);
              M[2 * (oi * 4 + in) + 1] = G(ot, tb, 1);
            }
          }
        }
    } else if (o.target == q_low) {
      for (int b1 = 0; b1 < 2; ++b1)
        for (int r0 = 0; r0 < 2; ++r0)
          for (int c0_ = 0; c0_ < 2; ++c0_) {
            int idx = (r0 + 2 * b1) * 4 + c0_ + 2 * b1;
            M[2 * idx] = G(r0, c0_, 0);
            M[2 * idx + 1] = G(r0, c0_, 1);
          }
    } else {
      for (int b0 = 0; b0 < 2; ++b0)
        for (int r1 = 0; r1 < 2; ++r1)
          for (int c1_ = 0; c1_ < 2; ++c1_) {
            int idx = (b0 + 2 * r1) * 4 + b0 + 2 * c1_;
            M[2 * idx] = G(r1, c1_, 0);
            M[2 * idx + 1] = G(r1, c1_, 1);
          }
    }
  };
  double m0[32], m1[32];
  to4(t0, c0, m0);
  to4(t1, c1, m1);
  out.assign(32, 0.0);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double sr = 0, si = 0;
      for (int k = 0; k < 4; ++k) {
        double ar = m1[2 * (r * 4 + k)], ai = m1[2 * (r * 4 + k) + 1];
        double br = m0[2 * (k * 4 + c)], bi = m0[2 * (k * 4 + c) + 1];
        sr = sr + (ar * br - ai * bi);
        si = si + (ar * bi + ai * br);
      }
      out[2 * (r * 4 + c)] = sr;
      out[2 * (r * 4 + c) + 1] = si;
    }
}

// Grover loops run for states of up to kLoopAlwaysQubits qubits, and for
// larger ones only when grover_loop_large (a server slot keeps long searches
// as short per-op kernels so that other requests get SMs between them).
constexpr int kLoopAlwaysQubits = 22;

// Tensor cores or CUDA cores for one 12-qubit pass: the CUDA-core tile
// kernel's work in units of one dense gate over the tile, against the blocks
// the pass needs (one block costs about kBlockUnits dense gates: measured on
// the 30-qubit complex64 layered circuit, 2.6 ms per block against 0.81 ms
// per dense gate, beyond the 2.6 ms that moving the state costs either way).
constexpr double kBlockUnits = 3.3;

static double cuda_core_units(const TilePass& tp) {
  double u = 0;
  for (const TileOp& t : tp.ops) {
    if (t.tloc < 0) {
      u += 0.4;  // diagonal gate on an outside target: one multiply per amplitude
      continue;
    }
    switch (t.kind) {
      case GK_SWAP: u += 0.5; break;
      case GK_PHASE: u += 0.4; break;
      case GK_DIAG: u += 0.6; break;
      case GK_UNITARY: u += (double)(1 << (t.um - 1)); break;  // 2^m products per amplitude
      default: u += 1.0; break;
    }
  }
  return u;
}

// complex128 digit blocks against the double-float tile kernel: one block
// costs about this many double-float dense gates (on the 30-qubit layered
// circuit a digit pass costs about 8 ms plus 5.8 ms per block, a dense gate
// in a double-float tile pass about 2.4 ms).  Measured against 5.0: the
// 30-qubit circuit 1144 against 1152 ms, value encoding at 22, 24 and 25
// (fused pairs) qubits 1.95 / 5.25 / 10.8 against 2.47 / 7.00 / 13.6 ms.
constexpr double kDigitBlockUnits = 2.5;

// A block pass costs about this many blocks besides its blocks (loading,
// converting and storing the tile).
constexpr double kPassCostBlocks = 2.5;

// True when every op keeps the state's norm (unitary gates and unitaries to
// 1e-12, permutations and the classical Grover and modexp passes; not
// measurement): the digit form's scale, taken from the norm before the
// circuit, then holds for every pass.
static bool norm_preserving(const bf_op* ops, int64_t nops) {
  auto unitary = [](const double* m, int dim) {
    for (int r = 0; r < dim; ++r)
      for (int c = 0; c < dim; ++c) {
        double re = 0, im = 0;
        for (int k = 0; k < dim; ++k) {
          const double ar = m[2 * (k * dim + r)], ai = -m[2 * (k * dim + r) + 1];  // conj(m[k][r])
          const double br = m[2 * (k * dim + c)], bi = m[2 * (k * dim + c) + 1];
          re += ar * br - ai * bi;
          im += ar * bi + ai * br;
        }
        if (std::fabs(re - (r == c ? 1.0 : 0.0)) > 1e-12 || std::fabs(im) > 1e-12) return false;
      }
    return true;
  };
  for (int64_t i = 0; i < nops; ++i) {
    const bf_op& op = ops[i];
    if (op.kind == BF_OP_MEASURE) return false;
    if (op.kind == BF_OP_GATE) {
      GateInstr g = lower_gate(op, 0);
      if (!unitary(g.m, 2)) return false;
    } else if (op.kind == BF_OP_UNITARY || op.kind == BF_OP_CUNITARY) {
      if (op.target2 <= 0 || op.target2 > 6 || !op.data || !unitary(op.data, 1 << op.target2)) return false;
    }
  }
  return true;
}

// tensor: tile passes as tensor-core block passes (12-qubit tiles), in
// `format` (BLOCK_TF32 for complex64, BLOCK_DIGITS for complex128)
static void build_steps(int n, const bf_op* ops, int64_t nops, const bf_exec_opts& o, std::vector<Step>& steps,
                        Program& pg, bool grover_loop_large = true, bool tensor = false,
                        BlockFormat format = BLOCK_TF32) {
  std::vector<TileOp>& prog = pg.ops;
  const bool fused = o.strategy == BF_STRATEGY_GPU_FUSED;
  tensor = tensor && fused && n >= kBlockTileQubits;
  if (tensor && format == BLOCK_DIGITS) tensor = norm_preserving(ops, nops);
  const double block_units = format == BLOCK_DIGITS ? kDigitBlockUnits : kBlockUnits;
  // a pass's own cost in blocks (load, conversion, stores); BFGPU_PASS_COST
  // overrides it for planner experiments
  const char* pc = std::getenv("BFGPU_PASS_COST");
  const double pass_cost = (pc && *pc) ? std::atof(pc) : kPassCostBlocks;
  const int K = tensor ? kBlockTileQubits : (o.tile_qubits > 0 ? o.tile_qubits : 11);
  std::vector<GateInstr> run;
  auto flush = [&]() {
    if (run.empty()) return;
    for (auto& ps : plan_gates(n, run, K, true, tensor ? block_units : 0.0, pass_cost,
                               tensor && format == BLOCK_DIGITS)) {
      Step s;
      if (ps.is_tile && tensor && ps.tile.K == kBlockTileQubits && ps.tile.L == kTileLowQubits) {
        size_t b0 = pg.blocks.size(), i0 = pg.images.size(), o0 = pg.offsets.size();
        // the most blocks for which the block pass is still the cheaper form
        const double cu = cuda_core_units(ps.tile);
        int max_blocks = 0;
        while (max_blocks < kMaxPassBlocks && (double)(max_blocks + 1) * block_units < cu) ++max_blocks;
        if (max_blocks > 0 &&
            plan_blocks(ps.tile, pg.blocks, pg.images, pg.offsets, format, max_blocks, pg.umats.data()) &&
            (double)(pg.blocks.size() - b0) * block_units < cu) {
          s.kind = Step::TBLOCK;
          s.digits = format == BLOCK_DIGITS;
          s.tile = ps.tile;
          s.tile.ops.clear();
          s.blk_off = b0;
          s.nblk = (int)(pg.blocks.size() - b0);
          steps.push_back(std::move(s));
          continue;
        }
        pg.blocks.resize(b0);
        pg.images.resize(i0);
        pg.offsets.resize(o0);
      }
      if (ps.is_tile) {
        s.kind = Step::TILE;
        s.tile = ps.tile;
        s.prog_off = prog.size();
        s.nprog = (int)ps.tile.ops.size();
        for (const TileOp& t : ps.tile.ops) s.unitaries |= t.kind == GK_UNITARY;
        prog.insert(prog.end(), ps.tile.ops.begin(), ps.tile.ops.end());
        s.tile.ops.clear();
      } else if (ps.gate.kind == GK_UNITARY) {
        // a unitary the planner left on its own: its dense kernel
        const GateInstr& g = ps.gate;
        s.kind = Step::UNITARY;
        const double* u = pg.umats.data() + g.uoff;
        s.u.assign(u, u + 2 * ((size_t)1 << (2 * g.um)));
        s.ut = g.target;
        s.um = g.um;
        s.uc = g.cmask ? __builtin_ctzll(g.cmask) : -1;
      } else {
        s.kind = Step::GATE;
        s.gate = ps.gate;
      }
      steps.push_back(std::move(s));
    }
    run.clear();
  };
  auto emit_gate = [&](const GateInstr& g) {
    if (fused) {
      run.push_back(g);
    } else {
      Step s;
      s.kind = Step::GATE;
      s.gate = g;
      steps.push_back(std::move(s));
    }
  };
  auto emit_perm = [&](const std::vector<int32_t>& src_of) {
    flush();
    bool full = true;
    for (int p = 0; p < n; ++p) full &= (src_of[p] == n - 1 - p);
    Step s;
    s.kind = full ? Step::BITREV : Step::PERMUTE;
    s.src_of = src_of;
    steps.push_back(std::move(s));
  };
  // a fused run's tile keeps its low min(K - 1, 5) qubits (all of them when
  // it spans the state); an m-qubit unitary joins only when it fits beside them
  const int run_low = K >= n ? std::min(K, kTileLowQubits) : std::min(K - 1, kTileLowQubits);
  auto emit_unitary = [&](const double* data, int t, int m, int ctl) {
    if (m <= 0) return;
    if (fused && m >= 2 && m <= kTileUnitaryMax && (K >= n || K - run_low >= m)) {
      // a dense unitary of a fused run: applied inside the tile pass (or
      // multiplied into a tensor-core block) with the gates around it
      GateInstr g;
      std::memset(&g, 0, sizeof g);
      g.kind = GK_UNITARY;
      g.target = t;
      g.cmask = ctl >= 0 ? 1ull << ctl : 0ull;
      g.um = m;
      g.uoff = (int32_t)pg.umats.size();
      pg.umats.insert(pg.umats.end(), data, data + 2 * ((size_t)1 << (2 * m)));
      run.push_back(g);
      return;
    }
    if (m == 1) {  // a 2x2: the gate kernels (and tile passes) take it
      bf_op g;
      std::memset(&g, 0, sizeof g);
      g.kind = BF_OP_GATE;
      g.gate = BF_GATE_CUSTOM;
      g.target = t;
      if (ctl >= 0) {
        g.controls = 1ull << ctl;
        g.ncontrols = 1;
      }
      std::memcpy(g.mat, data, 8 * sizeof(double));
      emit_gate(lower_gate(g, o.specialized));
      return;
    }
    flush();
    Step s;
    s.kind = Step::UNITARY;
    s.u.assign(data, data + 2 * ((size_t)1 << (2 * m)));
    s.ut = t;
    s.um = m;
    s.uc = ctl;
    steps.push_back(std::move(s));
  };

  for (int64_t i = 0; i < nops; ++i) {
    const bf_op& op = ops[i];
    switch (op.kind) {
      case BF_OP_GATE: {
        if ((op.flags & BF_OPF_FUSE_WITH_NEXT) && i + 1 < nops) {
          // FusedPairTransformation (apply_fused_pair, transformations_fusion.mojo:221-310)
          const bf_op& t1 = ops[i + 1];
          bool special = (is_cp(op) && is_cp(t1) && op.controls == t1.controls && op.target != t1.target) ||
                         (is_h(op) && is_h(t1) && op.target != t1.target) ||
                         (is_p(op) && is_p(t1) && op.target != t1.target) ||
                         (is_h(op) && is_p(t1) && op.target != t1.target) ||
                         (is_p(op) && is_h(t1) && op.target != t1.target);
          if (fused) {
            // a fused pair is its two gates in order: both join the run that
            // the tile planner fuses, whatever the pair's kind (the
            // reference's 4x4 product for H+CP and the like is the same map)
            run.push_back(lower_gate(op, o.specialized));
            run.push_back(lower_gate(t1, o.specialized));
          } else if (special) {
            // one pass for both gates: a two-gate run through the tile planner
            std::vector<GateInstr> pair = {lower_gate(op, o.specialized), lower_gate(t1, o.specialized)};
            {
              std::vector<GateInstr> saved;
              saved.swap(run);
              run = pair;
              flush();
              run.swap(saved);
            }
          } else {
            int q_low = 0;
            std::vector<double> m;
            fused_pair_matrix(op, t1, q_low, m);
            if (q_low + 2 > n) fail(BF_EINVAL, "Target range out of bounds");
            emit_unitary(m.data(), q_low, 2, -1);
          }
          ++i;
        } else {
          emit_gate(lower_gate(op, o.specialized));
        }
        break;
      }
      case BF_OP_SWAP:   // apply_swap_with_cx (executors.mojo:231-241): three CX = one exchange
      case BF_OP_CSWAP:  // apply_swap (state.mojo:434-444)
        if (op.target != op.target2) {
          flush();
          Step s;
          s.kind = Step::SWAPBITS;
          s.a = op.target;
          s.b = op.target2;
          steps.push_back(std::move(s));
        }
        break;
      case BF_OP_QREV: {  // apply_qubit_reversal_with_cx (executors.mojo:244-265)
        std::vector<int> t;
        if (op.nqubits == 0) for (int q = 0; q < n; ++q) t.push_back(q);
        else t.assign(op.qubits, op.qubits + op.nqubits);
        std::sort(t.begin(), t.end());
        std::vector<int32_t> src_of(n);
        for (int p = 0; p < n; ++p) src_of[p] = p;
        for (size_t k = 0; k < t.size() / 2; ++k) std::swap(src_of[t[k]], src_of[t[t.size() - 1 - k]]);
        emit_perm(src_of);
        break;
      }
      case BF_OP_BITREV: {  // apply_bit_reverse (state.mojo:383-390)
        std::vector<int32_t> src_of(n);
        for (int p = 0; p < n; ++p) src_of[p] = p;
        if (op.nqubits == 0) {
          for (int p = 0; p < n; ++p) src_of[p] = n - 1 - p;
        } else if (op.nqubits > 1) {
          std::vector<int> t(op.qubits, op.qubits + op.nqubits);
          std::sort(t.begin(), t.end());
          int k = (int)t.size();
          for (int b = 0; b < k; ++b) src_of[t[b]] = t[k - 1 - b];
        }
        emit_perm(src_of);
        break;
      }
      case BF_OP_PERMUTE: {  // apply_permute_qubits (state.mojo:393-431)
        if (op.nqubits == 0) break;
        std::vector<int32_t> src_of(op.qubits, op.qubits + op.nqubits);
        emit_perm(src_of);
        break;
      }
      case BF_OP_MEASURE: {  // MeasurementTransformation -> apply_measure (state.mojo:447-553)
        flush();
        Step s;
        s.kind = Step::MEASURE;
        s.mq.assign(op.qubits, op.qubits + op.nqubits);
        for (int64_t k = 0; k < op.nqubits; ++k) s.mv.push_back(op.data ? (int8_t)op.data[k] : (int8_t)-1);
        s.seed = (int64_t)op.arg;
        steps.push_back(std::move(s));
        break;
      }
      case BF_OP_CLASSICAL_ORACLE: {  // classical_oracle (grover.mojo:64-66)
        flush();
        int64_t reps = grover_loop_reps(n, ops, nops, i);
        if (reps >= 2 && (grover_loop_large || n <= kLoopAlwaysQubits)) {
          // repeated (oracle, full diffuser) iterations: one cooperative loop
          std::vector<uint64_t> idx;
          for (int64_t k = 0; k < op.nqubits; ++k) idx.push_back((uint64_t)op.data[k]);
          std::sort(idx.begin(), idx.end());
          Step s;
          s.kind = Step::GROVER_LOOP;
          for (size_t k = 0; k < idx.size();) {  // an index listed twice is negated twice
            size_t e = k;
            while (e < idx.size() && idx[e] == idx[k]) ++e;
            if ((e - k) & 1) s.marked.push_back(idx[k]);
            k = e;
          }
          s.reps = (int)reps;
          steps.push_back(std::move(s));
          i += 2 * reps - 1;
          break;
        }
        Step s;
        s.kind = Step::ORACLE;
        s.u.assign(op.data, op.data + op.nqubits);
        steps.push_back(std::move(s));
        break;
      }
      case BF_OP_GROVER_DIFFUSER:     // apply_grover_diffuser (grover_classical.mojo:284-326)
      case BF_OP_GROVER_INVERSION0: {  // apply_grover_inversion_0 (grover_classical.mojo:262-281)
        flush();
        Step s;
        s.kind = op.kind == BF_OP_GROVER_DIFFUSER ? Step::DIFFUSER : Step::INVERSION0;
        s.mq.assign(op.qubits, op.qubits + op.nqubits);
        steps.push_back(std::move(s));
        break;
      }
      case BF_OP_MODEXP:
      case BF_OP_MODEXP_INV: {  // apply_modexp(_inverse) (algos/shor.mojo:56-140)
        flush();
        Step s;
        s.kind = Step::MODEXP;
        s.a = (int)op.data[0];
        const int64_t N = (int64_t)op.data[3];
        const int64_t a = (((int64_t)op.data[2] % N) + N) % N;
        s.modulus = (uint64_t)N;
        s.base = (uint64_t)(op.kind == BF_OP_MODEXP ? a : modinv(a, N));
        steps.push_back(std::move(s));
        break;
      }
      case BF_OP_UNITARY:
        emit_unitary(op.data, op.target, op.target2, -1);
        break;
      case BF_OP_CUNITARY:
        emit_unitary(op.data, op.target, op.target2, __builtin_ctzll(op.controls));
        break;
      default:
        fail(BF_EINVAL, "Unknown transformation type: %d", op.kind);
    }
  }
  flush();
}

static int pass_class_of(const Step& s) {
  switch (s.kind) {
    case Step::GATE: return BF_PASS_GATE;
    case Step::TILE: return BF_PASS_TILE;
    case Step::TBLOCK: return s.digits ? BF_PASS_BLOCK_DIGITS : BF_PASS_BLOCK_TF32;
    default: return BF_PASS_OTHER;
  }
}

// The next free event of the timing pool (created on first use).
static cudaEvent_t pass_event(State& st, size_t k) {
  while (st.pass_events.size() <= k) {
    cudaEvent_t e;
    BF_CUDA(cudaEventCreate(&e));
    st.pass_events.push_back(e);
  }
  return st.pass_events[k];
}

static void run_steps(State& st, const std::vector<Step>& steps, const Program& pg, uint64_t plan_id) {
  upload_program(st, pg, plan_id);
  bool scaled = false;
  auto digit_pass = [&](size_t i) { return i < steps.size() && steps[i].kind == Step::TBLOCK && steps[i].digits; };
  for (size_t si = 0; si < steps.size(); ++si) {
    const Step& s = steps[si];
    if (s.kind == Step::TBLOCK && s.digits && !scaled) {
      // the digit scale, from the norm before the first digit pass
      if (!st.d_scale) st.d_scale = static_cast<int*>(dev_alloc(st, 16));
      launch_digit_scale(st, st.d_scale);
      scaled = true;
    }
    const size_t ev = 2 * st.pass_class.size();
    if (st.pass_timing) BF_CUDA(cudaEventRecord(pass_event(st, ev), st.stream));
    switch (s.kind) {
      case Step::GATE: launch_gate(st, s.gate); break;
      case Step::TILE:
        launch_tile_pass(st, st.d_prog + s.prog_off, s.nprog, s.tile,
                         s.unitaries ? reinterpret_cast<const double*>(st.d_aux + pg.umats_offset()) : nullptr);
        break;
      case Step::TBLOCK:
        if (s.digits) {
          // consecutive digit passes hand the state over as its fixed-point
          // integers; the first reads FP64 and the last writes it
          launch_block_pass_digits(st, reinterpret_cast<const Blk5*>(st.d_aux) + s.blk_off, s.nblk,
                                   st.d_aux + pg.images_offset(),
                                   reinterpret_cast<const uint16_t*>(st.d_aux + pg.offsets_offset()), s.tile,
                                   st.d_scale, si > 0 && digit_pass(si - 1), digit_pass(si + 1));
        } else {
          launch_block_pass(st, reinterpret_cast<const Blk5*>(st.d_aux) + s.blk_off, s.nblk,
                            st.d_aux + pg.images_offset(),
                            reinterpret_cast<const uint16_t*>(st.d_aux + pg.offsets_offset()), s.tile);
        }
        break;
      case Step::BITREV: launch_bitrev_full(st); break;
      case Step::PERMUTE: launch_permute(st, s.src_of.data()); break;
      case Step::SWAPBITS: launch_swap_bits(st, s.a, s.b); break;
      case Step::UNITARY: launch_unitary(st, s.u.data(), s.ut, s.um, s.uc); break;
      case Step::MEASURE:
        measure(st, s.mq.data(), s.mv.data(), (int32_t)s.mq.size(), s.seed, nullptr, nullptr);
        break;
      case Step::DIFFUSER: launch_grover_diffuser(st, s.mq.data(), (int32_t)s.mq.size()); break;
      case Step::INVERSION0: launch_grover_inversion0(st, s.mq.data(), (int32_t)s.mq.size()); break;
      case Step::ORACLE: launch_classical_oracle(st, s.u.data(), (int64_t)s.u.size()); break;
      case Step::GROVER_LOOP: launch_grover_loop(st, s.marked.data(), (int)s.marked.size(), s.reps); break;
      case Step::MODEXP: launch_modexp(st, s.a, s.base, s.modulus); break;
    }
    if (st.pass_timing) {
      BF_CUDA(cudaEventRecord(pass_event(st, ev + 1), st.stream));
      st.pass_class.push_back(pass_class_of(s));
    }
  }
}

static void free_state(State* st);

// A state's last few plans, keyed by the exact op list (each op with its data
// and qubit lists) and the options that shape a plan: running a circuit again
// skips planning and, while its program is still on the device, the upload.
struct PlanCache {
  struct Entry {
    std::vector<unsigned char> key;
    std::vector<Step> steps;
    Program prog;
    uint64_t id = 0;
  };
  static constexpr size_t kEntries = 4;
  std::vector<Entry> entries;  // most recent first
  uint64_t next_id = 1;
};

static void plan_key(std::vector<unsigned char>& k, const State& st, const bf_op* ops, int64_t nops,
                     const bf_exec_opts& o, BlockFormat format) {
  auto put = [&](const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    k.insert(k.end(), c, c + n);
  };
  const int32_t head[8] = {st.n, st.dtype, (int32_t)format, st.shared_gpu ? 1 : 0, o.strategy, o.tile_qubits,
                           (int32_t)o.specialized, o.tensor_blocks};
  k.reserve(sizeof head + (size_t)nops * sizeof(bf_op));
  put(head, sizeof head);
  for (int64_t i = 0; i < nops; ++i) {
    bf_op c = ops[i];
    c.data = nullptr;
    c.qubits = nullptr;
    put(&c, sizeof c);
    if (ops[i].data) put(ops[i].data, op_data_len(ops[i]) * sizeof(double));
    if (ops[i].qubits) put(ops[i].qubits, op_qubits_len(ops[i]) * sizeof(int32_t));
  }
}

void execute_ops(State& st, const bf_op* ops, int64_t nops, bf_exec_opts o) {
  if (o.strategy >= 0 && o.strategy <= 7)
    fail(BF_EUNSUPPORTED, "Execution strategy %d is a CPU strategy; use BF_STRATEGY_GPU(_FUSED)", o.strategy);
  if (o.strategy != BF_STRATEGY_GPU && o.strategy != BF_STRATEGY_GPU_FUSED)
    fail(BF_EINVAL, "Unknown execution strategy: %d", o.strategy);
  if (o.tile_qubits < 0 || o.tile_qubits > kMaxTileQubits)
    fail(BF_EINVAL, "tile_qubits must be in [0, %d]", kMaxTileQubits);
  if (o.tile_qubits == 0) o.tile_qubits = env_int("BFGPU_TILE_QUBITS", default_tile_qubits(st));
  if (o.validate) validate_ops(st.n, ops, nops);
  if (const char* tb = std::getenv("BFGPU_TENSOR_BLOCKS")) o.tensor_blocks = std::atoi(tb);
  const BlockFormat format = st.dtype == BF_C128 ? BLOCK_DIGITS : BLOCK_TF32;
  std::vector<unsigned char> key;
  plan_key(key, st, ops, nops, o, format);
  if (!st.plans) st.plans = new PlanCache();
  auto& entries = st.plans->entries;
  size_t hit = entries.size();
  for (size_t e = 0; e < entries.size(); ++e)
    if (entries[e].key == key) {
      hit = e;
      break;
    }
  if (hit == entries.size()) {
    PlanCache::Entry ne;
    build_steps(st.n, ops, nops, o, ne.steps, ne.prog, !st.shared_gpu, o.tensor_blocks != 0, format);
    ne.key = std::move(key);
    ne.id = st.plans->next_id++;
    entries.insert(entries.begin(), std::move(ne));
    if (entries.size() > PlanCache::kEntries) entries.pop_back();
  } else if (hit != 0) {
    std::rotate(entries.begin(), entries.begin() + (std::ptrdiff_t)hit, entries.begin() + (std::ptrdiff_t)hit + 1);
  }
  const PlanCache::Entry& plan = entries.front();
  // FP32 matrices are unitary only to ~6e-8, and that error changes the norm
  // coherently at every gate; the complex64 form restores the input norm.
  // renormalize == 2 (internal): the input is known to have unit norm.
  bool renorm = st.dtype == BF_C64 && nops > 0 && o.renormalize >= 0;
  if (renorm && o.renormalize != 2) launch_norm_before(st);
  run_steps(st, plan.steps, plan.prog, plan.id);
  if (renorm) launch_renormalize(st, o.renormalize == 2);
  flag_readback(st);
}

void init_state_runtime(State& st) {
  BF_CUDA(cudaGetDevice(&st.device));
  BF_CUDA(cudaDeviceGetAttribute(&st.num_sms, cudaDevAttrMultiProcessorCount, st.device));
  BF_CUDA(cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking));
  BF_CUDA(cudaEventCreateWithFlags(&st.prog_event, cudaEventDisableTiming));
}

void release_state_members(State& st) {
  if (st.stream) {
    dev_free(st, st.d_prog);
    dev_free(st, st.d_partial);
    dev_free(st, st.d_renorm);
    dev_free(st, st.d_flag);
    dev_free(st, st.d_aux);
    dev_free(st, st.d_scale);
    dev_free(st, st.d_digit_tiles);
    cudaStreamSynchronize(st.stream);
  }
  delete st.plans;
  st.plans = nullptr;
  if (st.amp) cudaFree(st.amp);
  if (st.scratch) cudaFree(st.scratch);
  if (st.h_prog) cudaFreeHost(st.h_prog);
  if (st.d_stage) cudaFree(st.d_stage);
  if (st.h_stage) cudaFreeHost(st.h_stage);
  for (int k = 0; k < 2; ++k) {
    if (st.stage_copied[k]) cudaEventDestroy(st.stage_copied[k]);
    if (st.stage_done[k]) cudaEventDestroy(st.stage_done[k]);
  }
  if (st.stage_start) cudaEventDestroy(st.stage_start);
  if (st.copy_stream) cudaStreamDestroy(st.copy_stream);
  if (st.h_partial) cudaFreeHost(st.h_partial);
  if (st.h_flag) cudaFreeHost(st.h_flag);
  if (st.h_aux) cudaFreeHost(st.h_aux);
  for (cudaEvent_t e : st.pass_events) cudaEventDestroy(e);
  st.pass_events.clear();
  if (st.d_umat) cudaFree(st.d_umat);
  for (void* p : st.retired_host) cudaFreeHost(p);
  if (st.prog_event) cudaEventDestroy(st.prog_event);
  if (st.stream) cudaStreamDestroy(st.stream);
  st = State();
}

static void free_state(State* st) {
  if (!st) return;
  release_state_members(*st);
  delete st;
}

// Boundary copies move the host SoA arrays in chunks of kStageElems
// amplitudes through two device staging buffers (re and im of one chunk
// each): the copy of chunk k+1 on the copy stream runs while the conversion
// kernel of chunk k runs on the state's stream.
static constexpr uint64_t kStageElems = 1ull << 22;  // 4 Mi amplitudes (64 MiB of re + im) per chunk

static void ensure_stage(State& st) {
  const size_t want = (size_t)std::min<uint64_t>(st.N, kStageElems) * 2 * sizeof(double) * 2;
  if (!st.copy_stream) {
    BF_CUDA(cudaStreamCreateWithFlags(&st.copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      BF_CUDA(cudaEventCreateWithFlags(&st.stage_copied[k], cudaEventDisableTiming));
      BF_CUDA(cudaEventCreateWithFlags(&st.stage_done[k], cudaEventDisableTiming));
    }
    BF_CUDA(cudaEventCreateWithFlags(&st.stage_start, cudaEventDisableTiming));
  }
  if (st.stage_bytes >= want) return;
  BF_CUDA(cudaStreamSynchronize(st.stream));
  BF_CUDA(cudaStreamSynchronize(st.copy_stream));
  if (st.d_stage) cudaFree(st.d_stage);
  st.d_stage = nullptr;
  st.stage_bytes = 0;
  if (cudaMalloc(&st.d_stage, want) != cudaSuccess) {
    cudaGetLastError();
    fail(BF_ENOMEM, "cannot allocate %zu bytes of boundary staging", want);
  }
  st.stage_bytes = want;
}

// re and im halves of staging buffer k
static double* stage_re(State& st, int k) {
  const uint64_t chunk = std::min<uint64_t>(st.N, kStageElems);
  return static_cast<double*>(st.d_stage) + (size_t)k * 2 * chunk;
}
static double* stage_im(State& st, int k) { return stage_re(st, k) + std::min<uint64_t>(st.N, kStageElems); }

// ---- host threads for copies between pageable arrays and pinned staging ----
// A copy from pageable memory goes through the driver's own staging, one
// CPU thread at a time.  For large transfers the library instead copies
// each chunk between the caller's arrays and pinned buffers with a pool of
// host threads (the calling thread takes a share too) while the DMA engine
// moves the previous chunk.
class CopyPool {
 public:
  // created on first use and never destroyed: its idle workers end with the
  // process (a destructor would join them, and in a forked child, whose
  // workers do not exist, the join would fail)
  static CopyPool& get() {
    static CopyPool* pool = new CopyPool();
    return *pool;
  }
  // dst[0, bytes) = src[0, bytes), split over the workers and the caller.
  // One job at a time (callers on other threads wait their turn); in a
  // process forked after the pool started, whose workers do not exist, the
  // caller copies alone.
  void copy(void* dst, const void* src, size_t bytes) {
    if (getpid() != pid_) {
      std::memcpy(dst, src, bytes);
      return;
    }
    std::lock_guard<std::mutex> one_job(job_m_);
    const size_t parts = workers_.size() + 1;
    const size_t part = ((bytes / parts) + 255) & ~(size_t)255;
    {
      std::lock_guard<std::mutex> lk(m_);
      dst_ = static_cast<char*>(dst);
      src_ = static_cast<const char*>(src);
      bytes_ = bytes;
      part_ = part;
      pending_ = (int)workers_.size();
      ++gen_;
    }
    cv_.notify_all();
    run_part(workers_.size());  // the caller's share: the last part
    std::unique_lock<std::mutex> lk(m_);
    done_.wait(lk, [&] { return pending_ == 0; });
  }
 private:
  CopyPool() : pid_(getpid()) {
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned n = std::max(1u, std::min(16u, hw ? hw : 4u)) - 1;
    for (unsigned i = 0; i < n; ++i) {
      workers_.emplace_back([this, i] { loop(i); });
      workers_.back().detach();
    }
  }
  void run_part(size_t i) {
    const size_t lo = std::min(bytes_, i * part_), hi = std::min(bytes_, lo + part_);
    if (i == workers_.size()) {
      if (lo < bytes_) std::memcpy(dst_ + lo, src_ + lo, bytes_ - lo);
    } else if (hi > lo) {
      std::memcpy(dst_ + lo, src_ + lo, hi - lo);
    }
  }
  void loop(size_t i) {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
      }
      run_part(i);
      std::lock_guard<std::mutex> lk(m_);
      if (--pending_ == 0) done_.notify_one();
    }
  }
  const pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex job_m_;  // held by the caller for a whole job
  std::mutex m_;
  std::condition_variable cv_, done_;
  uint64_t gen_ = 0;
  int pending_ = 0;
  char* dst_ = nullptr;
  const char* src_ = nullptr;
  size_t bytes_ = 0, part_ = 0;
};

// Host arrays the DMA engine cannot read directly (ordinary pageable
// memory), for transfers of at least one whole chunk: these go through the
// pinned staging.
static bool use_host_staging(const State& st, uint64_t count, const void* re, const void* im) {
  if (count < kStageElems) return false;
  for (const void* p : {re, im}) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (at.type != cudaMemoryTypeUnregistered) return false;
  }
  (void)st;
  return true;
}

static void ensure_host_stage(State& st) {
  const size_t want = (size_t)kStageElems * 2 * sizeof(double) * 2;
  if (st.h_stage_bytes >= want) return;
  if (st.h_stage) cudaFreeHost(st.h_stage);
  st.h_stage = nullptr;
  st.h_stage_bytes = 0;
  st.h_stage = host_alloc(want);
  st.h_stage_bytes = want;
}
static double* hstage_re(State& st, int k) { return static_cast<double*>(st.h_stage) + (size_t)k * 2 * kStageElems; }
static double* hstage_im(State& st, int k) { return hstage_re(st, k) + kStageElems; }

// Host SoA -> device.  Returns once every byte of re and im has been copied
// out of host memory (the conversion kernels may still run, stream-ordered
// before any later work on the state), so the caller may reuse the arrays.
static void upload_soa(State& st, const double* re, const double* im) {
  ensure_stage(st);
  if (use_host_staging(st, st.N, re, im)) {
    // host threads fill pinned buffer k while the DMA of the other runs
    ensure_host_stage(st);
    CopyPool& pool = CopyPool::get();
    const uint64_t chunk = kStageElems;
    BF_CUDA(cudaEventRecord(st.stage_start, st.stream));
    BF_CUDA(cudaStreamWaitEvent(st.copy_stream, st.stage_start, 0));
    int k = 0;
    for (uint64_t off = 0; off < st.N; off += chunk, k ^= 1) {
      const uint64_t cnt = std::min(chunk, st.N - off);
      // pinned buffer k is free once the DMA of two chunks back is done
      if (off >= 2 * chunk) BF_CUDA(cudaEventSynchronize(st.stage_copied[k]));
      pool.copy(hstage_re(st, k), re + off, cnt * sizeof(double));
      pool.copy(hstage_im(st, k), im + off, cnt * sizeof(double));
      if (off >= 2 * chunk) BF_CUDA(cudaStreamWaitEvent(st.copy_stream, st.stage_done[k], 0));
      BF_CUDA(cudaMemcpyAsync(stage_re(st, k), hstage_re(st, k), cnt * sizeof(double), cudaMemcpyHostToDevice,
                              st.copy_stream));
      BF_CUDA(cudaMemcpyAsync(stage_im(st, k), hstage_im(st, k), cnt * sizeof(double), cudaMemcpyHostToDevice,
                              st.copy_stream));
      BF_CUDA(cudaEventRecord(st.stage_copied[k], st.copy_stream));
      BF_CUDA(cudaStreamWaitEvent(st.stream, st.stage_copied[k], 0));
      launch_interleave(st, stage_re(st, k), stage_im(st, k), off, cnt);
      BF_CUDA(cudaEventRecord(st.stage_done[k], st.stream));
    }
    BF_CUDA(cudaStreamSynchronize(st.copy_stream));
    return;
  }
  const uint64_t chunk = std::min<uint64_t>(st.N, kStageElems);
  // the staging buffers' earlier users are on the state's stream
  BF_CUDA(cudaEventRecord(st.stage_start, st.stream));
  BF_CUDA(cudaStreamWaitEvent(st.copy_stream, st.stage_start, 0));
  int k = 0;
  for (uint64_t off = 0; off < st.N; off += chunk, k ^= 1) {
    const uint64_t cnt = std::min(chunk, st.N - off);
    if (off >= 2 * chunk) BF_CUDA(cudaStreamWaitEvent(st.copy_stream, st.stage_done[k], 0));
    BF_CUDA(cudaMemcpyAsync(stage_re(st, k), re + off, cnt * sizeof(double), cudaMemcpyHostToDevice,
                            st.copy_stream));
    BF_CUDA(cudaMemcpyAsync(stage_im(st, k), im + off, cnt * sizeof(double), cudaMemcpyHostToDevice,
                            st.copy_stream));
    BF_CUDA(cudaEventRecord(st.stage_copied[k], st.copy_stream));
    BF_CUDA(cudaStreamWaitEvent(st.stream, st.stage_copied[k], 0));
    launch_interleave(st, stage_re(st, k), stage_im(st, k), off, cnt);
    BF_CUDA(cudaEventRecord(st.stage_done[k], st.stream));
  }
  BF_CUDA(cudaStreamSynchronize(st.copy_stream));
}

// Device amplitudes [offset, offset + count) -> host SoA; blocks until the
// host arrays hold them.  The conversion of chunk c+1 is queued before the
// copy of chunk c, because a copy into pageable host memory returns only
// once it has finished.
static void download_soa(State& st, uint64_t offset, uint64_t count, double* re, double* im) {
  if (count == 0) {
    sync_state(st);
    return;
  }
  ensure_stage(st);
  const uint64_t chunk = std::min<uint64_t>(st.N, kStageElems);
  const uint64_t nchunks = (count + chunk - 1) / chunk;
  BF_CUDA(cudaEventRecord(st.stage_start, st.copy_stream));
  BF_CUDA(cudaStreamWaitEvent(st.stream, st.stage_start, 0));
  if (use_host_staging(st, count, re, im)) {
    // the DMA of chunk c+1 into pinned buffer (c+1) & 1 runs while host
    // threads copy chunk c out of buffer c & 1
    ensure_host_stage(st);
    CopyPool& pool = CopyPool::get();
    auto convert_and_fetch = [&](uint64_t c) {
      const int k = (int)(c & 1);
      const uint64_t cnt = std::min(chunk, count - c * chunk);
      if (c >= 2) BF_CUDA(cudaStreamWaitEvent(st.stream, st.stage_copied[k], 0));
      launch_deinterleave(st, stage_re(st, k), stage_im(st, k), offset + c * chunk, cnt);
      BF_CUDA(cudaEventRecord(st.stage_done[k], st.stream));
      BF_CUDA(cudaStreamWaitEvent(st.copy_stream, st.stage_done[k], 0));
      BF_CUDA(cudaMemcpyAsync(hstage_re(st, k), stage_re(st, k), cnt * sizeof(double), cudaMemcpyDeviceToHost,
                              st.copy_stream));
      BF_CUDA(cudaMemcpyAsync(hstage_im(st, k), stage_im(st, k), cnt * sizeof(double), cudaMemcpyDeviceToHost,
                              st.copy_stream));
      BF_CUDA(cudaEventRecord(st.stage_copied[k], st.copy_stream));
    };
    convert_and_fetch(0);
    for (uint64_t c = 0; c < nchunks; ++c) {
      // pinned buffer (c+1) & 1 was emptied by the host copy of chunk c-1
      if (c + 1 < nchunks) convert_and_fetch(c + 1);
      const int k = (int)(c & 1);
      const uint64_t cnt = std::min(chunk, count - c * chunk);
      BF_CUDA(cudaEventSynchronize(st.stage_copied[k]));
      pool.copy(re + c * chunk, hstage_re(st, k), cnt * sizeof(double));
      pool.copy(im + c * chunk, hstage_im(st, k), cnt * sizeof(double));
    }
    sync_state(st);
    return;
  }
  auto convert = [&](uint64_t c) {
    const int k = (int)(c & 1);
    if (c >= 2) BF_CUDA(cudaStreamWaitEvent(st.stream, st.stage_copied[k], 0));
    launch_deinterleave(st, stage_re(st, k), stage_im(st, k), offset + c * chunk, std::min(chunk, count - c * chunk));
    BF_CUDA(cudaEventRecord(st.stage_done[k], st.stream));
  };
  convert(0);
  for (uint64_t c = 0; c < nchunks; ++c) {
    if (c + 1 < nchunks) convert(c + 1);
    const int k = (int)(c & 1);
    const uint64_t cnt = std::min(chunk, count - c * chunk);
    BF_CUDA(cudaStreamWaitEvent(st.copy_stream, st.stage_done[k], 0));
    BF_CUDA(cudaMemcpyAsync(re + c * chunk, stage_re(st, k), cnt * sizeof(double), cudaMemcpyDeviceToHost,
                            st.copy_stream));
    BF_CUDA(cudaMemcpyAsync(im + c * chunk, stage_im(st, k), cnt * sizeof(double), cudaMemcpyDeviceToHost,
                            st.copy_stream));
    BF_CUDA(cudaEventRecord(st.stage_copied[k], st.copy_stream));
  }
  BF_CUDA(cudaStreamSynchronize(st.copy_stream));
  sync_state(st);
}

}  // namespace bf

using namespace bf;

static inline State* S_(bf_state* h) { return reinterpret_cast<State*>(h); }
static inline const State* S_(const bf_state* h) { return reinterpret_cast<const State*>(h); }

extern "C" {

int bf_exec_opts_init(bf_exec_opts* o) {
  if (!o) return BF_EINVAL;
  std::memset(o, 0, sizeof *o);
  o->strategy = BF_STRATEGY_GPU_FUSED;
  o->validate = 1;
  o->specialized = BF_SPEC_ALL;
  o->tile_qubits = 0;
  o->sync = 0;
  o->tensor_blocks = 1;
  return BF_OK;
}

int bf_version(int32_t* v) {
  if (!v) return BF_EINVAL;
  *v = BFGPU_ABI_VERSION;
  return BF_OK;
}

int bf_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return BF_EINVAL;
  size_t k = std::min(len - 1, g_last_error.size());
  std::memcpy(buf, g_last_error.data(), k);
  buf[k] = 0;
  return BF_OK;
}

int bf_state_create(int32_t n, int32_t dtype, bf_state** out) {
  return guarded([&]() {
    if (!out) fail(BF_EINVAL, "out is null");
    *out = nullptr;
    if (n < 1 || n > 40) fail(BF_EINVAL, "num_qubits must be in [1, 40], got %d", n);
    if (dtype != BF_C128 && dtype != BF_C64) fail(BF_EINVAL, "unknown dtype %d", dtype);
    State* st = new State();
    try {
      st->n = n;
      st->dtype = dtype;
      st->N = 1ull << n;
      // complex128 computes in double-float unless BFGPU_C128_MATH=f64
      const char* math = std::getenv("BFGPU_C128_MATH");
      if (dtype == BF_C64) st->prec = PREC_F32;
      else st->prec = (math && std::strcmp(math, "f64") == 0) ? PREC_F64 : PREC_DF;
      init_state_runtime(*st);
      if (cudaMalloc(&st->amp, st->bytes()) != cudaSuccess) {
        cudaGetLastError();
        st->amp = nullptr;
        fail(BF_ENOMEM, "cannot allocate %zu bytes for a %d-qubit state", st->bytes(), n);
      }
      launch_set_basis(*st, 0);
    } catch (...) {
      free_state(st);
      throw;
    }
    *out = reinterpret_cast<bf_state*>(st);
  });
}

int bf_state_destroy(bf_state* hst) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st) return;
    DeviceGuard dg(st->device);
    free_state(st);
  });
}

int bf_state_info(const bf_state* hst, int32_t* n, int32_t* dtype) {
  const State* st = S_(hst);
  return guarded([&]() {
    if (!st) fail(BF_EINVAL, "state is null");
    if (n) *n = st->n;
    if (dtype) *dtype = st->dtype;
  });
}

int bf_state_set_basis(bf_state* hst, uint64_t idx) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st) fail(BF_EINVAL, "state is null");
    DeviceGuard dg(st->device);
    if (idx >= st->N) fail(BF_EINVAL, "basis index %llu out of range", (unsigned long long)idx);
    launch_set_basis(*st, idx);
  });
}

int bf_state_upload_soa(bf_state* hst, const double* re, const double* im) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || !re || !im) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(st->device);
    upload_soa(*st, re, im);
  });
}

int bf_state_download_range(bf_state* hst, uint64_t offset, uint64_t count, double* re, double* im) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || (count && (!re || !im))) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(st->device);
    if (offset > st->N || count > st->N - offset) fail(BF_EINVAL, "range out of bounds");
    download_soa(*st, offset, count, re, im);
  });
}

int bf_state_download_soa(bf_state* hst, double* re, double* im) {
  State* st = S_(hst);
  if (!st) {
    g_last_error = "state is null";
    return BF_EINVAL;
  }
  return bf_state_download_range(hst, 0, st->N, re, im);
}

int bf_state_sync(bf_state* hst) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st) fail(BF_EINVAL, "state is null");
    DeviceGuard dg(st->device);
    sync_state(*st);
  });
}

int bf_state_stream(bf_state* hst, void** stream) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || !stream) fail(BF_EINVAL, "null argument");
    *stream = (void*)st->stream;
  });
}

int bf_state_launch_count(const bf_state* hst, uint64_t* launches, int32_t reset) {
  const State* st = S_(hst);
  return guarded([&]() {
    if (!st || !launches) fail(BF_EINVAL, "null argument");
    *launches = st->launches;
    if (reset) const_cast<State*>(st)->launches = 0;
  });
}

int bf_state_pass_timing(bf_state* hst, int32_t enable) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st) fail(BF_EINVAL, "state is null");
    st->pass_timing = enable != 0;
  });
}

int bf_state_pass_times(bf_state* hst, int64_t* counts, double* ms) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || !counts || !ms) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(st->device);
    for (int c = 0; c < BF_PASS_CLASSES; ++c) {
      counts[c] = 0;
      ms[c] = 0;
    }
    BF_CUDA(cudaStreamSynchronize(st->stream));
    for (size_t k = 0; k < st->pass_class.size(); ++k) {
      float t = 0;
      BF_CUDA(cudaEventElapsedTime(&t, st->pass_events[2 * k], st->pass_events[2 * k + 1]));
      ++counts[st->pass_class[k]];
      ms[st->pass_class[k]] += t;
    }
    st->pass_class.clear();
  });
}

int bf_state_digit_tiles(bf_state* hst, uint64_t* five, uint64_t* six, int32_t reset) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || !five || !six) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(st->device);
    unsigned long long h[2] = {0, 0};
    if (st->d_digit_tiles) {
      BF_CUDA(cudaMemcpyAsync(h, st->d_digit_tiles, sizeof h, cudaMemcpyDeviceToHost, st->stream));
      if (reset) BF_CUDA(cudaMemsetAsync(st->d_digit_tiles, 0, sizeof h, st->stream));
      BF_CUDA(cudaStreamSynchronize(st->stream));
    }
    *five = h[0];
    *six = h[1];
  });
}

int bf_execute(bf_state* hst, const bf_op* ops, int64_t nops, const bf_exec_opts* opts) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st) fail(BF_EINVAL, "state is null");
    DeviceGuard dg(st->device);
    bf_exec_opts o;
    if (opts) o = *opts;
    else bf_exec_opts_init(&o);
    execute_ops(*st, ops, nops, o);
    if (o.sync) sync_state(*st);
  });
}

int bf_norm2(bf_state* hst, double* out) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || !out) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(st->device);
    *out = reduce_norm2(*st);
  });
}

int bf_inner(bf_state* ha, bf_state* hb, double* re, double* im) {
  State* a = S_(ha);
  State* b = S_(hb);
  return guarded([&]() {
    if (!a || !b || !re || !im) fail(BF_EINVAL, "null argument");
    if (a->device != b->device) fail(BF_EINVAL, "the two states live on different devices (%d, %d)", a->device, b->device);
    DeviceGuard dg(a->device);
    inner_product(*a, *b, re, im);
  });
}

int bf_probabilities(bf_state* hst, const int32_t* qubits, const int8_t* values, int32_t nq, double* out) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || !out) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(st->device);
    std::vector<double> p;
    marginal_probs(*st, qubits, values, nq, p);
    std::memcpy(out, p.data(), p.size() * sizeof(double));
  });
}

int bf_measure(bf_state* hst, const int32_t* targets, const int8_t* values, int32_t ntargets, int64_t seed,
               uint64_t* outcome, double* probability) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st) fail(BF_EINVAL, "state is null");
    DeviceGuard dg(st->device);
    measure(*st, targets, values, ntargets, seed, outcome, probability);
  });
}

int bf_probs_topk(bf_state* hst, int32_t k, uint64_t* indices, double* probs) {
  State* st = S_(hst);
  return guarded([&]() {
    if (!st || !indices || !probs) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(st->device);
    probs_topk(*st, k, indices, probs);
  });
}

// ---- batches -------------------------------------------------------------------
static inline Batch* B_(bf_batch* h) { return reinterpret_cast<Batch*>(h); }

int bf_batch_create(int32_t ncirc, const int32_t* num_qubits, const bf_op* const* ops, const int64_t* nops,
                    int32_t dtype, const bf_exec_opts* opts, bf_batch** out) {
  return guarded([&]() {
    if (!out) fail(BF_EINVAL, "out is null");
    *out = nullptr;
    if (dtype != BF_C128 && dtype != BF_C64) fail(BF_EINVAL, "unknown dtype %d", dtype);
    bf_exec_opts o;
    if (opts) o = *opts;
    else bf_exec_opts_init(&o);
    if (o.tile_qubits < 0 || o.tile_qubits > kMaxTileQubits)
      fail(BF_EINVAL, "tile_qubits must be in [0, %d]", kMaxTileQubits);
    const char* math = std::getenv("BFGPU_C128_MATH");
    int prec = dtype == BF_C64 ? PREC_F32 : ((math && std::strcmp(math, "f64") == 0) ? PREC_F64 : PREC_DF);
    *out = reinterpret_cast<bf_batch*>(batch_create(ncirc, num_qubits, ops, nops, dtype, o, prec));
  });
}

int bf_batch_run(bf_batch* h, int32_t sync) {
  return guarded([&]() {
    if (!h) fail(BF_EINVAL, "batch is null");
    DeviceGuard dg(batch_device(*B_(h)));
    batch_run(*B_(h), sync != 0);
  });
}

int bf_batch_sync(bf_batch* h) {
  return guarded([&]() {
    if (!h) fail(BF_EINVAL, "batch is null");
    DeviceGuard dg(batch_device(*B_(h)));
    batch_sync(*B_(h));
  });
}

int bf_batch_download(bf_batch* h, int32_t circuit, double* re, double* im) {
  return guarded([&]() {
    if (!h || !re || !im) fail(BF_EINVAL, "null argument");
    DeviceGuard dg(batch_device(*B_(h)));
    batch_download(*B_(h), circuit, re, im);
  });
}

int bf_batch_stats(bf_batch* h, int64_t* tasks, int64_t* passes, uint64_t* state_bytes, int32_t* graph,
                   uint64_t* launches) {
  return guarded([&]() {
    if (!h) fail(BF_EINVAL, "batch is null");
    batch_stats(*B_(h), tasks, passes, state_bytes, graph, launches);
  });
}

int bf_batch_tuning(bf_batch* h, int32_t* qubits, int32_t* widths, double* ms, int32_t* chosen, int32_t cap,
                    int32_t* count) {
  return guarded([&]() {
    if (!h || !count) fail(BF_EINVAL, "null argument");
    batch_tuning(*B_(h), qubits, widths, ms, chosen, cap, count);
  });
}

int bf_batch_stream(bf_batch* h, void** stream) {
  return guarded([&]() {
    if (!h || !stream) fail(BF_EINVAL, "null argument");
    *stream = batch_stream(*B_(h));
  });
}

int bf_batch_destroy(bf_batch* h) {
  return guarded([&]() {
    if (!h) return;
    DeviceGuard dg(batch_device(*B_(h)));
    batch_destroy(B_(h));
  });
}

int bf_norm2_noalloc(const void* d_amps, uint64_t num_amps, int32_t dtype, double* d_out, void* stream) {
  return guarded([&]() { norm2_noalloc(d_amps, num_amps, dtype, d_out, static_cast<cudaStream_t>(stream)); });
}

// ---- serving -----------------------------------------------------------------
static inline Server* V_(bf_server* h) { return reinterpret_cast<Server*>(h); }

int bf_server_create(const bf_server_opts* opts, bf_server** out) {
  return guarded([&]() {
    if (!out) fail(BF_EINVAL, "out is null");
    *out = nullptr;
    bf_server_opts o;
    std::memset(&o, 0, sizeof o);
    if (opts) o = *opts;
    if (o.tile_qubits < 0 || o.tile_qubits > kMaxTileQubits)
      fail(BF_EINVAL, "tile_qubits must be in [0, %d]", kMaxTileQubits);
    *out = reinterpret_cast<bf_server*>(server_create(o));
  });
}

int bf_server_submit(bf_server* h, int32_t n, int32_t dtype, const bf_op* ops, int64_t nops, uint64_t* id) {
  return guarded([&]() {
    if (!h) fail(BF_EINVAL, "server is null");
    uint64_t r = server_submit(*V_(h), n, dtype, ops, nops);
    if (id) *id = r;
  });
}

int bf_server_poll(bf_server* h, bf_result* out, int32_t max, int32_t* count) {
  return guarded([&]() {
    if (!h || (max > 0 && !out)) fail(BF_EINVAL, "null argument");
    int k = server_poll(*V_(h), out, max);
    if (count) *count = k;
  });
}

int bf_server_wait_idle(bf_server* h, int64_t timeout_ms) {
  return guarded([&]() {
    if (!h) fail(BF_EINVAL, "server is null");
    if (!server_wait_idle(*V_(h), timeout_ms)) fail(BF_ETIMEDOUT, "server still busy after %lld ms", (long long)timeout_ms);
  });
}

int bf_server_stats(bf_server* h, bf_server_counters* out) {
  return guarded([&]() {
    if (!h || !out) fail(BF_EINVAL, "null argument");
    server_stats(*V_(h), *out);
  });
}

int bf_server_destroy(bf_server* h) {
  return guarded([&]() {
    if (!h) return;
    DeviceGuard dg(server_device(*V_(h)));
    server_destroy(V_(h));
  });
}

// Host-only: validates and plans ops for a state of n qubits without a
// device, reporting how many tile passes, per-gate kernels and other passes
// bf_execute would launch and the algorithmic bytes they move (units of S).
int bf_plan_stats(int32_t n, const bf_op* ops, int64_t nops, const bf_exec_opts* opts, int64_t* tile_passes,
                  int64_t* gate_kernels, int64_t* other_passes, double* bytes_in_S, int64_t* block_passes,
                  int64_t* blocks) {
  return guarded([&]() {
    if (n < 1 || n > 40) fail(BF_EINVAL, "num_qubits must be in [1, 40], got %d", n);
    bf_exec_opts o;
    if (opts) o = *opts;
    else bf_exec_opts_init(&o);
    if (o.tile_qubits <= 0) o.tile_qubits = 11;
    if (o.validate) validate_ops(n, ops, nops);
    std::vector<Step> steps;
    Program prog;
    build_steps(n, ops, nops, o, steps, prog, true, o.tensor_blocks != 0,
                o.plan_dtype == BF_C64 ? BLOCK_TF32 : BLOCK_DIGITS);
    int64_t t = 0, g = 0, x = 0, bp = 0, nb = 0;
    double bytes = 0;
    for (auto& s : steps) {
      if (s.kind == Step::TBLOCK) {
        ++bp;
        nb += s.nblk;
      }
      if (s.kind == Step::TILE || s.kind == Step::TBLOCK) {
        ++t;
        bytes += 2.0;
      } else if (s.kind == Step::GATE) {
        ++g;
        bytes += gate_bytes_fraction(s.gate);
      } else if (s.kind == Step::GROVER_LOOP) {
        ++x;
        bytes += 2.0 * (s.reps + 1);
      } else {
        ++x;
        bytes += (s.kind == Step::SWAPBITS) ? 1.0
                 : (s.kind == Step::DIFFUSER ? 3.0 : (s.kind == Step::ORACLE ? 0.0 : 2.0));
      }
    }
    if (tile_passes) *tile_passes = t;
    if (gate_kernels) *gate_kernels = g;
    if (other_passes) *other_passes = x;
    if (bytes_in_S) *bytes_in_S = bytes;
    if (block_passes) *block_passes = bp;
    if (blocks) *blocks = nb;
  });
}

// ---- wire formats ---------------------------------------------------------------
static inline OpList* L_(bf_oplist* h) { return reinterpret_cast<OpList*>(h); }
static inline const OpList* LC_(const bf_oplist* h) { return reinterpret_cast<const OpList*>(h); }

int bf_qasm3_parse(const char* text, bf_oplist** out) {
  return guarded([&]() {
    if (!out) fail(BF_EINVAL, "out is null");
    *out = reinterpret_cast<bf_oplist*>(qasm3_parse(text));
  });
}

int bf_ops_serialize(int32_t n, const bf_op* ops, int64_t nops, void* buf, size_t cap, size_t* len) {
  return guarded([&]() {
    if (!len) fail(BF_EINVAL, "len is null");
    std::vector<unsigned char> blob = ops_serialize(n, ops, nops);
    *len = blob.size();
    if (!buf) return;
    if (cap < blob.size()) fail(BF_EINVAL, "buffer of %zu bytes is smaller than the %zu needed", cap, blob.size());
    std::memcpy(buf, blob.data(), blob.size());
  });
}

int bf_ops_deserialize(const void* buf, size_t len, bf_oplist** out) {
  return guarded([&]() {
    if (!out) fail(BF_EINVAL, "out is null");
    *out = reinterpret_cast<bf_oplist*>(ops_deserialize(buf, len));
  });
}

int bf_oplist_view(const bf_oplist* h, const bf_op** ops, int64_t* nops, int32_t* n) {
  return guarded([&]() {
    if (!h) fail(BF_EINVAL, "list is null");
    oplist_view(*LC_(h), ops, nops, n);
  });
}

int bf_oplist_destroy(bf_oplist* h) {
  return guarded([&]() { oplist_destroy(L_(h)); });
}

int bf_server_submit_serialized(bf_server* h, const void* buf, size_t len, int32_t dtype, uint64_t* id) {
  return guarded([&]() {
    if (!h || !id) fail(BF_EINVAL, "null argument");
    OpList* L = ops_deserialize(buf, len);
    const bf_op* ops = nullptr;
    int64_t nops = 0;
    int32_t n = 0;
    oplist_view(*L, &ops, &nops, &n);
    try {
      *id = server_submit(*V_(h), n, dtype, ops, nops);  // copies the ops
    } catch (...) {
      oplist_destroy(L);
      throw;
    }
    oplist_destroy(L);
  });
}

// Host-only validation (validate_circuit, executors.mojo:129-185).
int bf_validate(int32_t n, const bf_op* ops, int64_t nops) {
  return guarded([&]() { validate_ops(n, ops, nops); });
}

}  // extern "C"

// batch.cu — many independent circuits in one persistent launch.
//
// Every circuit of a batch is planned into tile passes (the same planner and
// tile body as a single state).  A task is one tile of one pass of one
// circuit; tasks are ordered pass-major, (pass index, circuit, tile), and the
// CTAs of one cooperative launch take them from an atomic ticket.  A task of
// pass p waits until its circuit has finished every tile of passes < p: the
// tasks it waits for hold smaller tickets, so they are already running on
// co-resident CTAs and the wait always ends.  The wait is bounded anyway
// (spin_limit polls); on expiry the CTA records an error flag, skips its
// task and the host reports BF_ETIMEDOUT.
//
// The states of all circuits live in one pooled buffer.  A run (|0...0> for
// every state, then all tasks) is captured once into a CUDA graph and
// replayed by bf_batch_run.
#include <algorithm>
#include <cstring>
#include <vector>

#include "tile_body.cuh"

namespace bf {

// Task kinds: a tile of a pass; for complex64, after a circuit's last pass,
// a contiguous chunk's sum |amp|^2 (added to the circuit's norm) and then
// the chunk's rescale to unit norm.
enum : uint32_t { TASK_TILE = 0, TASK_NORM = 1, TASK_SCALE = 2 };

struct BatchTask {
  uint32_t circuit;
  uint32_t pass;   // index into the pass table (its geometry gives the chunk size)
  uint32_t tile;
  uint32_t need;   // tasks of this circuit that must have finished
  uint32_t kind;
  uint32_t pad;
};

struct BatchPass {
  uint64_t offset;  // first amplitude of the circuit's state in the pool
  TileGeom geo;
  uint32_t op_begin;
  uint32_t nops;
};

struct BatchDesc {
  void* pool;
  double* norm;    // per circuit, complex64 renormalisation
  const BatchTask* tasks;
  const BatchPass* passes;
  const TileOp* ops;
  unsigned int* done;
  unsigned long long* ticket;
  int* error;
  unsigned long long ntasks;
  unsigned int spin_limit;
};

template <class P>
__global__ void __launch_bounds__(kTileThreads) k_batch(const BatchDesc d) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long t_sh;
  __shared__ int ok_sh;
  for (;;) {
    if (threadIdx.x == 0) t_sh = atomicAdd(d.ticket, 1ull);
    __syncthreads();
    const unsigned long long t = t_sh;
    __syncthreads();
    if (t >= d.ntasks) break;  // CTA-uniform
    const BatchTask task = d.tasks[t];
    if (threadIdx.x == 0) {
      int ok = 1;
      const volatile unsigned int* dn = d.done + task.circuit;
      unsigned int polls = 0;
      while (*dn < task.need) {
        if (++polls > d.spin_limit) {
          ok = 0;
          atomicExch(d.error, 1);
          break;
        }
        __nanosleep(128);
      }
      __threadfence();
      ok_sh = ok;
    }
    __syncthreads();
    if (ok_sh) {
      const BatchPass& bp = d.passes[task.pass];
      if (task.kind == TASK_TILE) {
        TileGeom geo = bp.geo;
        run_tile<P, true>(static_cast<typename P::Glob*>(d.pool) + bp.offset, d.ops + bp.op_begin, (int)bp.nops,
                          geo, task.tile, smem_raw);
      } else if constexpr (sizeof(typename P::Glob) == 8) {
        float2* base = reinterpret_cast<float2*>(d.pool) + bp.offset + ((uint64_t)task.tile << bp.geo.K);
        const int cnt = 1 << bp.geo.K;
        if (task.kind == TASK_NORM) {
          dfl acc{0.f, 0.f};
          for (int e = threadIdx.x; e < cnt; e += kTileThreads) {
            float2 v = __ldcg(base + e);
            acc = df_add(acc, df_dot2(dfl{v.x, 0.f}, dfl{v.x, 0.f}, dfl{v.y, 0.f}, dfl{v.y, 0.f}));
          }
          double* red = reinterpret_cast<double*>(smem_raw);
          red[threadIdx.x] = (double)acc.hi + (double)acc.lo;
          __syncthreads();
          for (int off = kTileThreads / 2; off > 0; off >>= 1) {
            if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
            __syncthreads();
          }
          if (threadIdx.x == 0) atomicAdd(d.norm + task.circuit, red[0]);
        } else {
          const double nrm = __ldcg(d.norm + task.circuit);
          const double f = nrm > 0 ? 1.0 / sqrt(nrm) : 1.0;
          const float hi = (float)f, lo = (float)(f - (double)hi);
          for (int e = threadIdx.x; e < cnt; e += kTileThreads) {
            float2 v = __ldcg(base + e);
            v.x = fmaf(v.x, hi, v.x * lo);
            v.y = fmaf(v.y, hi, v.y * lo);
            base[e] = v;
          }
        }
      }
    }
    __threadfence();  // every thread's stores are visible device-wide ...
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(d.done + task.circuit, 1u);  // ... before the task counts as done
  }
}

template <class T>
__global__ void k_batch_basis(T* pool, const uint64_t* offsets, int ncirc);
template <>
__global__ void k_batch_basis<double2>(double2* pool, const uint64_t* offsets, int ncirc) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncirc) pool[offsets[c]] = make_double2(1.0, 0.0);
}
template <>
__global__ void k_batch_basis<float2>(float2* pool, const uint64_t* offsets, int ncirc) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncirc) pool[offsets[c]] = make_float2(1.0f, 0.0f);
}

struct BatchTuneRow {
  int32_t qubits, width, circuits, chosen;
  double ms;  // one run of the sample batch
};

struct Batch {
  int device = 0, num_sms = 0;
  int dtype = BF_C64, prec = PREC_F32;
  int ncirc = 0;
  std::vector<int32_t> nq;
  std::vector<uint64_t> offsets;  // in amplitudes
  uint64_t pool_amps = 0;
  size_t smem = 0;
  void* pool = nullptr;
  BatchTask* d_tasks = nullptr;
  BatchPass* d_passes = nullptr;
  TileOp* d_ops = nullptr;
  uint64_t* d_offsets = nullptr;
  unsigned int* d_done = nullptr;
  double* d_norm = nullptr;
  unsigned long long* d_ticket = nullptr;
  int* d_error = nullptr;
  int* h_error = nullptr;
  uint64_t ntasks = 0, npasses = 0;
  unsigned grid = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  uint64_t launches = 0;
  // autotuning record: per qubit count, the candidate tile widths timed on a
  // sample of the batch's circuits of that size, and the width chosen
  std::vector<BatchTuneRow> tuning;
  size_t amp_bytes() const { return dtype == BF_C128 ? 16 : 8; }
};

template <class P>
static void enqueue_run(Batch& b) {
  BF_CUDA(cudaMemsetAsync(b.pool, 0, b.pool_amps * b.amp_bytes(), b.stream));
  k_batch_basis<typename P::Glob><<<(b.ncirc + 255) / 256, 256, 0, b.stream>>>(
      static_cast<typename P::Glob*>(b.pool), b.d_offsets, b.ncirc);
  BF_CUDA(cudaGetLastError());
  BF_CUDA(cudaMemsetAsync(b.d_done, 0, b.ncirc * sizeof(unsigned int), b.stream));
  BF_CUDA(cudaMemsetAsync(b.d_norm, 0, b.ncirc * sizeof(double), b.stream));
  BF_CUDA(cudaMemsetAsync(b.d_ticket, 0, sizeof(unsigned long long), b.stream));
  BF_CUDA(cudaMemsetAsync(b.d_error, 0, sizeof(int), b.stream));
  BatchDesc d;
  d.pool = b.pool;
  d.norm = b.d_norm;
  d.tasks = b.d_tasks;
  d.passes = b.d_passes;
  d.ops = b.d_ops;
  d.done = b.d_done;
  d.ticket = b.d_ticket;
  d.error = b.d_error;
  d.ntasks = b.ntasks;
  d.spin_limit = 1u << 24;  // x 128 ns sleeps: about 2 s before the error flag
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(b.grid);
  cfg.blockDim = dim3(kTileThreads);
  cfg.dynamicSmemBytes = b.smem;
  cfg.stream = b.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BF_CUDA(cudaLaunchKernelEx(&cfg, k_batch<P>, d));
  BF_CUDA(cudaMemcpyAsync(b.h_error, b.d_error, sizeof(int), cudaMemcpyDeviceToHost, b.stream));
}

static void enqueue(Batch& b) {
  switch (b.prec) {
    case PREC_F64: enqueue_run<PolF64>(b); break;
    case PREC_DF: enqueue_run<PolDF>(b); break;
    default: enqueue_run<PolF32>(b); break;
  }
}

// The kernel's shared-memory limit is set once per device to the largest a
// batch can ask for (a 13-qubit tile), so batches of different tile sizes,
// created on any thread, never lower it under one another.
template <class P>
static void size_grid(Batch& b) {
  static PerDeviceOnce configured;  // one per instantiation of P
  configured.run(b.device, [] {
    const size_t most = std::max<size_t>(tile_smem_bytes<P>(kMaxTileQubits, 0), kTileThreads * sizeof(double));
    BF_CUDA(cudaFuncSetAttribute(k_batch<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most));
  });
  int per_sm = 0;
  BF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<P>, kTileThreads, b.smem));
  if (per_sm < 1) fail(BF_EUNSUPPORTED, "batch kernel cannot be resident with %zu bytes of shared memory", b.smem);
  b.grid = (unsigned)(per_sm * b.num_sms);
}

static void free_batch(Batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->pool);
  cudaFree(b->d_tasks);
  cudaFree(b->d_passes);
  cudaFree(b->d_ops);
  cudaFree(b->d_offsets);
  cudaFree(b->d_done);
  cudaFree(b->d_norm);
  cudaFree(b->d_ticket);
  cudaFree(b->d_error);
  if (b->h_error) cudaFreeHost(b->h_error);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

template <class T>
static void dev_upload(T** dst, const std::vector<T>& v) {
  size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
  if (cudaMalloc(dst, bytes) != cudaSuccess) {
    cudaGetLastError();
    *dst = nullptr;
    fail(BF_ENOMEM, "cannot allocate %zu bytes of batch tables", bytes);
  }
  if (!v.empty()) BF_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

// Builds a batch whose circuits of n qubits use tiles of up to width_of_n[n]
// qubits; the kernel's shared memory is at least smem_floor (so that sample
// batches run at the occupancy of the widest candidate); `capture` records
// the run into a CUDA graph.
static Batch* build_batch(int ncirc, const int32_t* nq, const bf_op* const* ops, const int64_t* nops, int dtype,
                          const bf_exec_opts& o, int prec, const int* width_of_n, size_t smem_floor, bool capture) {
  if (ncirc < 1) fail(BF_EINVAL, "a batch needs at least one circuit");
  if (!nq || !ops || !nops) fail(BF_EINVAL, "null argument");
  Batch* b = new Batch();
  try {
    b->dtype = dtype;
    b->prec = prec;
    b->ncirc = ncirc;
    BF_CUDA(cudaGetDevice(&b->device));
    BF_CUDA(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device));
    std::vector<BatchPass> passes;
    std::vector<TileOp> prog;
    // per circuit: passes (each with its tile count)
    std::vector<std::vector<uint32_t>> circ_passes(ncirc);
    uint64_t off = 0;
    size_t smem = 0;
    for (int c = 0; c < ncirc; ++c) {
      int n = nq[c];
      if (n < 1 || n > 30) fail(BF_EINVAL, "circuit %d: num_qubits must be in [1, 30], got %d", c, n);
      validate_ops(n, ops[c], nops[c]);
      std::vector<GateInstr> gates;
      for (int64_t i = 0; i < nops[c]; ++i) {
        const bf_op& op = ops[c][i];
        if (op.kind != BF_OP_GATE || (op.flags & BF_OPF_FUSE_WITH_NEXT))
          fail(BF_EUNSUPPORTED, "circuit %d: batches take gate transformations only (op %lld)", c, (long long)i);
        gates.push_back(lower_gate(op, o.specialized));
      }
      b->nq.push_back(n);
      b->offsets.push_back(off);
      off += ((1ull << n) + 31) & ~31ull;  // 256-byte aligned starts
      int K = std::min(n, width_of_n[n]);
      for (auto& ps : plan_gates(n, gates, K, /*allow_single=*/false)) {
        BatchPass bp;
        std::memset(&bp, 0, sizeof bp);
        bp.offset = b->offsets.back();
        bp.geo.K = ps.tile.K;
        bp.geo.L = ps.tile.L;
        for (int j = 0; j < ps.tile.K; ++j) bp.geo.q[j] = ps.tile.q[j];
        bp.op_begin = (uint32_t)prog.size();
        bp.nops = (uint32_t)ps.tile.ops.size();
        prog.insert(prog.end(), ps.tile.ops.begin(), ps.tile.ops.end());
        circ_passes[c].push_back((uint32_t)passes.size());
        passes.push_back(bp);
        size_t sm = 0;
        switch (prec) {
          case PREC_F64: sm = tile_smem_bytes<PolF64>(bp.geo.K, bp.geo.L); break;
          case PREC_DF: sm = tile_smem_bytes<PolDF>(bp.geo.K, bp.geo.L); break;
          default: sm = tile_smem_bytes<PolF32>(bp.geo.K, bp.geo.L); break;
        }
        smem = std::max(smem, sm);
      }
    }
    b->pool_amps = off;
    b->smem = std::max<size_t>(std::max(smem, smem_floor), kTileThreads * sizeof(double));  // the norm stage reduces in it
    // tasks, pass-major
    std::vector<BatchTask> tasks;
    size_t max_p = 0;
    for (auto& cp : circ_passes) max_p = std::max(max_p, cp.size());
    // complex64: two more stages per circuit, norm then rescale
    const size_t extra = (dtype == BF_C64) ? 2 : 0;
    std::vector<uint32_t> done_before(ncirc, 0);
    for (size_t p = 0; p < max_p + extra; ++p)
      for (int c = 0; c < ncirc; ++c) {
        size_t np = circ_passes[c].size();
        if (np == 0 || p >= np + extra) continue;
        uint32_t kind = p < np ? TASK_TILE : (p == np ? TASK_NORM : TASK_SCALE);
        uint32_t pi = circ_passes[c][std::min(p, np - 1)];
        uint32_t tiles = (uint32_t)(1ull << (b->nq[c] - passes[pi].geo.K));
        for (uint32_t t = 0; t < tiles; ++t) tasks.push_back(BatchTask{(uint32_t)c, pi, t, done_before[c], kind, 0});
        done_before[c] += tiles;
      }
    b->ntasks = tasks.size();
    b->npasses = passes.size();
    size_t pool_bytes = b->pool_amps * b->amp_bytes();
    if (cudaMalloc(&b->pool, pool_bytes) != cudaSuccess) {
      cudaGetLastError();
      b->pool = nullptr;
      fail(BF_ENOMEM, "cannot allocate %zu bytes for the batch states", pool_bytes);
    }
    dev_upload(&b->d_tasks, tasks);
    dev_upload(&b->d_passes, passes);
    dev_upload(&b->d_ops, prog);
    dev_upload(&b->d_offsets, b->offsets);
    std::vector<unsigned int> zeros(ncirc, 0);
    dev_upload(&b->d_done, zeros);
    std::vector<double> dz(ncirc, 0.0);
    dev_upload(&b->d_norm, dz);
    std::vector<unsigned long long> z1(1, 0);
    dev_upload(&b->d_ticket, z1);
    std::vector<int> z2(1, 0);
    dev_upload(&b->d_error, z2);
    if (cudaHostAlloc(&b->h_error, sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      b->h_error = nullptr;
      fail(BF_ENOMEM, "cannot allocate the batch status word");
    }
    *b->h_error = 0;
    BF_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    switch (prec) {
      case PREC_F64: size_grid<PolF64>(*b); break;
      case PREC_DF: size_grid<PolDF>(*b); break;
      default: size_grid<PolF32>(*b); break;
    }
    // capture one run into a graph; if this stack cannot capture it, runs
    // are enqueued directly
    cudaGraph_t g = nullptr;
    if (capture && cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      bool ok = true;
      try {
        enqueue(*b);
      } catch (const Error&) {
        ok = false;
      }
      cudaError_t e = cudaStreamEndCapture(b->stream, &g);
      if (ok && e == cudaSuccess && g && cudaGraphInstantiate(&b->graph, g, 0) == cudaSuccess) {
        // captured
      } else {
        b->graph = nullptr;
      }
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
    }
  } catch (...) {
    free_batch(b);
    throw;
  }
  return b;
}

// Batch autotuning.  The candidates are tile widths 8..12 (at most n).  For
// each qubit count n of the batch, a sample of its circuits of that size
// (repeated when there are fewer, sized so that the sample fills the GPU as
// the whole batch does) runs once per candidate, every candidate at the shared memory of the widest one, and
// the width with the shortest run is kept.  This is the counterpart of the
// reference's tunable grid split (grid_col_bits, executors.mojo:213-228),
// chosen by measurement instead of a fixed rule.
constexpr int kTuneSample = 1024;
constexpr int kTuneMinWidth = 8, kTuneMaxWidth = 12;

template <class P>
static size_t tile_smem_of(int K) {
  return tile_smem_bytes<P>(K, std::min(K - 1, kTileLowQubits));
}

static double time_batch(Batch& b) {
  cudaEvent_t e0, e1;
  BF_CUDA(cudaEventCreate(&e0));
  BF_CUDA(cudaEventCreate(&e1));
  float best = 0.f;
  try {
    batch_run(b, true);  // warm-up
    for (int r = 0; r < 2; ++r) {
      BF_CUDA(cudaEventRecord(e0, b.stream));
      batch_run(b, false);
      BF_CUDA(cudaEventRecord(e1, b.stream));
      batch_sync(b);
      float ms = 0.f;
      BF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = r == 0 ? ms : std::min(best, ms);
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

static void tune_widths(int ncirc, const int32_t* nq, const bf_op* const* ops, const int64_t* nops, int dtype,
                        const bf_exec_opts& o, int prec, int* width_of_n, std::vector<BatchTuneRow>& rows) {
  size_t floor = 0;
  switch (prec) {
    case PREC_F64: floor = tile_smem_of<PolF64>(kTuneMaxWidth); break;
    case PREC_DF: floor = tile_smem_of<PolDF>(kTuneMaxWidth); break;
    default: floor = tile_smem_of<PolF32>(kTuneMaxWidth); break;
  }
  for (int n = 1; n <= 30; ++n) {
    std::vector<int> members;
    for (int c = 0; c < ncirc; ++c)
      if (nq[c] == n) members.push_back(c);
    if (members.empty() || n <= kTuneMinWidth) continue;
    // enough circuits that even the widest candidate's pass level holds
    // about 1024 tiles, 16 to kTuneSample of them: the batch being tuned
    // runs thousands of circuits at once, and a sample that leaves wide
    // tiles short of CTAs favours narrow ones (with 4096 tiles of the
    // narrowest width instead, the tuned 4096-circuit batch ran at 0.90 of
    // the fixed 12-qubit width)
    const int wmax = std::min(n, kTuneMaxWidth);
    const int sample = std::max(16, std::min(kTuneSample, 1024 >> std::min(n - wmax, 10)));
    std::vector<int32_t> snq;
    std::vector<const bf_op*> sops;
    std::vector<int64_t> snops;
    for (int k = 0; k < sample; ++k) {
      const int c = members[(size_t)k % members.size()];
      snq.push_back(n);
      sops.push_back(ops[c]);
      snops.push_back(nops[c]);
    }
    const size_t first = rows.size();
    for (int w = kTuneMinWidth; w <= std::min(n, kTuneMaxWidth); ++w) {
      int widths[31];
      for (int m = 0; m <= 30; ++m) widths[m] = w;
      Batch* t = build_batch(sample, snq.data(), sops.data(), snops.data(), dtype, o, prec, widths, floor, false);
      double ms = 0;
      try {
        ms = time_batch(*t);
      } catch (...) {
        free_batch(t);
        throw;
      }
      free_batch(t);
      rows.push_back(BatchTuneRow{n, w, sample, 0, ms});
    }
    // the widest width within 3% of the fastest: fewer passes, and the
    // sample's timing noise is about that size
    double best = rows[first].ms;
    for (size_t r = first; r < rows.size(); ++r) best = std::min(best, rows[r].ms);
    int best_w = width_of_n[n];
    for (size_t r = first; r < rows.size(); ++r)
      if (rows[r].ms <= 1.03 * best) best_w = rows[r].width;
    width_of_n[n] = best_w;
    for (size_t r = first; r < rows.size(); ++r) rows[r].chosen = rows[r].width == best_w ? 1 : 0;
  }
}

Batch* batch_create(int ncirc, const int32_t* nq, const bf_op* const* ops, const int64_t* nops, int dtype,
                    const bf_exec_opts& o, int prec) {
  if (ncirc < 1) fail(BF_EINVAL, "a batch needs at least one circuit");
  if (!nq || !ops || !nops) fail(BF_EINVAL, "null argument");
  // widths: the caller's, or 12 refined by measurement (o.tile_qubits == 0)
  int width_of_n[31];
  for (int m = 0; m <= 30; ++m) width_of_n[m] = o.tile_qubits > 0 ? o.tile_qubits : 12;
  std::vector<BatchTuneRow> rows;
  if (o.tile_qubits == 0) {
    for (int c = 0; c < ncirc; ++c) {
      if (nq[c] < 1 || nq[c] > 30) fail(BF_EINVAL, "circuit %d: num_qubits must be in [1, 30], got %d", c, nq[c]);
      validate_ops(nq[c], ops[c], nops[c]);
    }
    tune_widths(ncirc, nq, ops, nops, dtype, o, prec, width_of_n, rows);
  }
  Batch* b = build_batch(ncirc, nq, ops, nops, dtype, o, prec, width_of_n, 0, true);
  b->tuning = std::move(rows);
  return b;
}

void batch_tuning(const Batch& b, int32_t* qubits, int32_t* widths, double* ms, int32_t* chosen, int32_t cap,
                  int32_t* count) {
  const int32_t m = (int32_t)b.tuning.size();
  if (count) *count = m;
  for (int32_t r = 0; r < m && r < cap; ++r) {
    if (qubits) qubits[r] = b.tuning[r].qubits;
    if (widths) widths[r] = b.tuning[r].width;
    if (ms) ms[r] = b.tuning[r].ms;
    if (chosen) chosen[r] = b.tuning[r].chosen;
  }
}

void batch_run(Batch& b, bool sync) {
  if (b.graph) BF_CUDA(cudaGraphLaunch(b.graph, b.stream));
  else enqueue(b);
  b.launches += 2;  // basis kernel + persistent kernel
  if (sync) {
    BF_CUDA(cudaStreamSynchronize(b.stream));
    if (*b.h_error) fail(BF_ETIMEDOUT, "batch: a task waited past its bound for its circuit's previous pass");
  }
}

void batch_sync(Batch& b) {
  BF_CUDA(cudaStreamSynchronize(b.stream));
  if (*b.h_error) fail(BF_ETIMEDOUT, "batch: a task waited past its bound for its circuit's previous pass");
}

void batch_download(Batch& b, int c, double* re, double* im) {
  if (c < 0 || c >= b.ncirc) fail(BF_EINVAL, "circuit index %d out of range", c);
  batch_sync(b);
  uint64_t N = 1ull << b.nq[c];
  size_t eb = b.amp_bytes();
  std::vector<unsigned char> h(N * eb);
  BF_CUDA(cudaMemcpy(h.data(), static_cast<unsigned char*>(b.pool) + b.offsets[c] * eb, N * eb,
                     cudaMemcpyDeviceToHost));
  for (uint64_t i = 0; i < N; ++i) {
    if (eb == 16) {
      const double* p = reinterpret_cast<const double*>(h.data()) + 2 * i;
      re[i] = p[0];
      im[i] = p[1];
    } else {
      const float* p = reinterpret_cast<const float*>(h.data()) + 2 * i;
      re[i] = (double)p[0];
      im[i] = (double)p[1];
    }
  }
}

void batch_destroy(Batch* b) { free_batch(b); }

void batch_stats(const Batch& b, int64_t* tasks, int64_t* passes, uint64_t* state_bytes, int32_t* graph,
                 uint64_t* launches) {
  if (tasks) *tasks = (int64_t)b.ntasks;
  if (passes) *passes = (int64_t)b.npasses;
  if (state_bytes) *state_bytes = b.pool_amps * b.amp_bytes();
  if (graph) *graph = b.graph ? 1 : 0;
  if (launches) *launches = b.launches;
}

void* batch_stream(const Batch& b) { return (void*)b.stream; }

int batch_device(const Batch& b) { return b.device; }

}  // namespace bf

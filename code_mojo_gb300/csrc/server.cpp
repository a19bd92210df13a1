// server.cpp — a serving loop with continuous batching.
//
// Requests (a circuit as bf_op records, a qubit count, a dtype) are queued
// on submission with a copy of their ops.  `slots` worker threads, each
// owning one CUDA stream and one device state, take the oldest request
// whose statevector footprint 2^n * (8 | 16) B fits in the HBM budget that
// the running requests leave, allocate its state stream-ordered
// (cudaMallocAsync, so nothing synchronises the device), run the fused plan
// from |0...0>, read back its top-k outcomes and free the state.  Slots run
// concurrently on their own streams, so requests that arrive while others
// run are admitted as soon as a slot and the memory are free, and their
// kernels overlap on the device.  Each request records its submission,
// start and completion times.
//
// Scheduling: a request is large when 2^n * ops exceeds large_cost.  Small
// requests wait in a FIFO and every slot that frees up takes the oldest one
// before any large work; large ones wait in a queue ordered by that cost
// (cheapest first: under an offered load above capacity this completes the
// most requests, and the biggest ones wait) and run only on the large slots
// while no small request waits.  Each slot owns a stream of the highest and
// one of the lowest priority and runs small requests on the first, large
// ones on the second, so the block scheduler hands SMs that free up to the
// short requests first.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "bf_internal.h"

namespace bf {

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct ServedRequest {
  uint64_t id = 0;
  int32_t n = 0;
  int32_t dtype = BF_C64;
  std::vector<bf_op> ops;
  std::vector<std::vector<double>> data;     // owned copies of op.data
  std::vector<std::vector<int32_t>> qubits;  // owned copies of op.qubits
  double t_submit = 0;
  bool large = false;
  double cost = 0;  // 2^n * ops
  uint64_t bytes() const { return (1ull << n) * (dtype == BF_C128 ? 16 : 8); }
};

struct Server {
  bf_server_opts opts;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ServedRequest*> queue;         // small requests, oldest first
  std::vector<ServedRequest*> large_queue;  // large requests: a heap, cheapest on top
  std::vector<bf_result> done;
  uint64_t next_id = 1, bytes_in_use = 0, peak_bytes = 0, budget = 0;
  uint64_t submitted = 0, completed = 0, failed = 0, running = 0;
  bool stop = false;
  std::vector<std::thread> workers;
};

static ServedRequest* copy_request(int32_t n, int32_t dtype, const bf_op* ops, int64_t nops) {
  auto* r = new ServedRequest();
  r->n = n;
  r->dtype = dtype;
  r->ops.assign(ops, ops + nops);
  r->data.resize(nops);
  r->qubits.resize(nops);
  for (int64_t i = 0; i < nops; ++i) {
    bf_op& o = r->ops[i];
    const size_t nq = op_qubits_len(o);
    if (o.qubits && nq > 0) {
      r->qubits[i].assign(o.qubits, o.qubits + nq);
      o.qubits = r->qubits[i].data();
    }
    const size_t nd = op_data_len(o);
    if (o.data && nd > 0) {
      r->data[i].assign(o.data, o.data + nd);
      o.data = r->data[i].data();
    }
  }
  return r;
}

// heap order: the cheapest request (then the oldest) on top
static bool cheaper_last(const ServedRequest* a, const ServedRequest* b) {
  if (a->cost != b->cost) return a->cost > b->cost;
  return a->id > b->id;
}

static void serve_one(Server& sv, State& st, ServedRequest& r, bf_result& res) {
  st.n = r.n;
  st.N = 1ull << r.n;
  st.dtype = r.dtype;
  if (r.dtype == BF_C64) st.prec = PREC_F32;
  else {
    const char* math = std::getenv("BFGPU_C128_MATH");
    st.prec = (math && std::strcmp(math, "f64") == 0) ? PREC_F64 : PREC_DF;
  }
  void* amp = nullptr;
  cudaError_t e = cudaMallocAsync(&amp, st.bytes(), st.stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(BF_ENOMEM, "cannot allocate %zu bytes for request %llu", st.bytes(), (unsigned long long)r.id);
  }
  st.amp = amp;
  struct Free {
    State& st;
    ~Free() {
      if (st.amp) cudaFreeAsync(st.amp, st.stream);
      st.amp = nullptr;
    }
  } guard{st};
  launch_set_basis(st, 0);
  bf_exec_opts o;
  std::memset(&o, 0, sizeof o);
  o.strategy = BF_STRATEGY_GPU_FUSED;
  o.validate = 1;
  o.specialized = BF_SPEC_ALL;
  o.tile_qubits = sv.opts.tile_qubits;
  // no tensor-core passes: their persistent grids take every SM's shared
  // memory for the whole pass, which the other slots' kernels then wait for
  o.tensor_blocks = 0;
  o.renormalize = 2;  // starts from |0...0>: unit norm
  execute_ops(st, r.ops.data(), (int64_t)r.ops.size(), o);
  int k = std::min<int>(sv.opts.topk, (int)std::min<uint64_t>(16, st.N));
  res.k = k;
  probs_topk(st, k, res.top_index, res.top_prob);  // synchronises the slot's stream
}

static void worker_main(Server* sv, int slot) {
  cudaSetDevice(sv->device);
  State st;
  cudaStream_t s_hi = nullptr, s_lo = nullptr;
  bool ready = true;
  try {
    init_state_runtime(st);
    // the slot shares the GPU: no grid-wide persistent loops
    st.shared_gpu = true;
    // small requests on a stream of the highest priority, large ones on a
    // stream of the lowest
    int lo = 0, hi = 0;
    BF_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    BF_CUDA(cudaStreamDestroy(st.stream));
    st.stream = nullptr;
    BF_CUDA(cudaStreamCreateWithPriority(&s_hi, cudaStreamNonBlocking, hi));
    BF_CUDA(cudaStreamCreateWithPriority(&s_lo, cudaStreamNonBlocking, lo));
    st.stream = s_hi;
    // size the work buffers for the typical request up front
    upload_program_reserve(st, 16384);
    ensure_partials(st, 1 << 15);
    BF_CUDA(cudaStreamSynchronize(st.stream));
  } catch (const Error&) {
    ready = false;
  }
  for (;;) {
    ServedRequest* r = nullptr;
    const bool large_slot = slot < sv->opts.large_slots;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      auto fits_small = [&]() {
        return !sv->queue.empty() && sv->bytes_in_use + sv->queue.front()->bytes() <= sv->budget;
      };
      auto fits_large = [&]() {
        return !sv->large_queue.empty() && sv->bytes_in_use + sv->large_queue.front()->bytes() <= sv->budget;
      };
      sv->cv_work.wait_for(lk, std::chrono::milliseconds(5),
                           [&]() { return sv->stop || fits_small() || (large_slot && fits_large()); });
      if (sv->stop) break;
      if (fits_small()) {
        r = sv->queue.front();
        sv->queue.pop_front();
      } else if (large_slot && fits_large()) {
        std::pop_heap(sv->large_queue.begin(), sv->large_queue.end(), cheaper_last);
        r = sv->large_queue.back();
        sv->large_queue.pop_back();
      } else {
        continue;
      }
      sv->bytes_in_use += r->bytes();
      sv->peak_bytes = std::max(sv->peak_bytes, sv->bytes_in_use);
      sv->running++;
    }
    bf_result res;
    std::memset(&res, 0, sizeof res);
    res.id = r->id;
    res.num_qubits = r->n;
    res.dtype = r->dtype;
    res.slot = slot;
    res.t_submit = r->t_submit;
    res.t_start = now_s();
    try {
      if (!ready) fail(BF_ECUDA, "slot %d could not create its streams", slot);
      cudaStream_t want = r->large ? s_lo : s_hi;
      if (st.stream != want) {  // the other stream's work (an earlier request) is done first
        BF_CUDA(cudaStreamSynchronize(st.stream));
        st.stream = want;
      }
      serve_one(*sv, st, *r, res);
      res.status = BF_OK;
    } catch (const Error& e) {
      res.status = e.code;
      std::snprintf(res.message, sizeof res.message, "%s", e.msg.c_str());
    } catch (...) {
      res.status = BF_ECUDA;
      std::snprintf(res.message, sizeof res.message, "unexpected error");
    }
    res.t_done = now_s();
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->bytes_in_use -= r->bytes();
      sv->running--;
      if (res.status == BF_OK) sv->completed++;
      else sv->failed++;
      sv->done.push_back(res);
    }
    delete r;
    sv->cv_work.notify_all();
    sv->cv_done.notify_all();
  }
  st.amp = nullptr;
  // the state's members go with its current stream; the other one is idle
  cudaStream_t other = st.stream == s_hi ? s_lo : s_hi;
  if (other) {
    cudaStreamSynchronize(other);
    cudaStreamDestroy(other);
  }
  release_state_members(st);
}

Server* server_create(const bf_server_opts& opts) {
  auto* sv = new Server();
  sv->opts = opts;
  if (sv->opts.slots <= 0) sv->opts.slots = 12;
  if (sv->opts.slots > 64) fail(BF_EINVAL, "at most 64 slots");
  // a third of the slots (at least 2) serve small requests only
  if (sv->opts.large_slots <= 0) sv->opts.large_slots = std::max(1, sv->opts.slots - std::max(2, sv->opts.slots / 3));
  if (sv->opts.large_slots > sv->opts.slots) fail(BF_EINVAL, "large_slots exceeds slots");
  if (sv->opts.large_cost == 0) sv->opts.large_cost = 1ull << 28;
  if (sv->opts.topk <= 0) sv->opts.topk = 16;
  if (sv->opts.topk > 16) fail(BF_EINVAL, "topk must be in [1, 16]");
  BF_CUDA(cudaGetDevice(&sv->device));
  size_t free_b = 0, total_b = 0;
  BF_CUDA(cudaMemGetInfo(&free_b, &total_b));
  sv->budget = opts.hbm_budget_bytes ? opts.hbm_budget_bytes : (uint64_t)(0.8 * (double)free_b);
  // keep freed request memory in the stream-ordered pool for the next request
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, sv->device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  cudaGetLastError();
  for (int s = 0; s < sv->opts.slots; ++s) sv->workers.emplace_back(worker_main, sv, s);
  return sv;
}

uint64_t server_submit(Server& sv, int32_t n, int32_t dtype, const bf_op* ops, int64_t nops) {
  if (n < 1 || n > 34) fail(BF_EINVAL, "num_qubits must be in [1, 34], got %d", n);
  if (dtype != BF_C128 && dtype != BF_C64) fail(BF_EINVAL, "unknown dtype %d", dtype);
  if (nops < 0 || (nops > 0 && !ops)) fail(BF_EINVAL, "ops is null");
  validate_ops(n, ops, nops);
  ServedRequest* r = copy_request(n, dtype, ops, nops);
  if (r->bytes() > sv.budget) {
    delete r;
    fail(BF_EBUSY, "a %d-qubit state needs more than the server's HBM budget", n);
  }
  r->cost = (double)(1ull << n) * (double)std::max<int64_t>(1, nops);
  r->large = r->cost > (double)sv.opts.large_cost;
  uint64_t id;
  {
    std::lock_guard<std::mutex> lk(sv.mu);
    // a slot may take, run and free the request as soon as the lock is released
    id = r->id = sv.next_id++;
    r->t_submit = now_s();
    if (r->large) {
      sv.large_queue.push_back(r);
      std::push_heap(sv.large_queue.begin(), sv.large_queue.end(), cheaper_last);
    } else {
      sv.queue.push_back(r);
    }
    sv.submitted++;
  }
  sv.cv_work.notify_all();
  return id;
}

int server_poll(Server& sv, bf_result* out, int max) {
  std::lock_guard<std::mutex> lk(sv.mu);
  int k = (int)std::min<size_t>((size_t)std::max(0, max), sv.done.size());
  for (int i = 0; i < k; ++i) out[i] = sv.done[i];
  sv.done.erase(sv.done.begin(), sv.done.begin() + k);
  return k;
}

bool server_wait_idle(Server& sv, int64_t timeout_ms) {
  std::unique_lock<std::mutex> lk(sv.mu);
  return sv.cv_done.wait_for(lk, std::chrono::milliseconds(std::max<int64_t>(0, timeout_ms)),
                             [&]() { return sv.queue.empty() && sv.large_queue.empty() && sv.running == 0; });
}

void server_stats(Server& sv, bf_server_counters& s) {
  std::lock_guard<std::mutex> lk(sv.mu);
  s.submitted = sv.submitted;
  s.completed = sv.completed;
  s.failed = sv.failed;
  s.queued = sv.queue.size() + sv.large_queue.size();
  s.running = sv.running;
  s.bytes_in_use = sv.bytes_in_use;
  s.peak_bytes = sv.peak_bytes;
  s.budget_bytes = sv.budget;
}

void server_destroy(Server* sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto& t : sv->workers) t.join();
  for (auto* r : sv->queue) delete r;
  for (auto* r : sv->large_queue) delete r;
  delete sv;
}

int server_device(const Server& sv) { return sv.device; }

}  // namespace bf

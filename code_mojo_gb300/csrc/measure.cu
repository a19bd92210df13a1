// measure.cu — measurement and readout of a device state.
//
//  * bf_probabilities: outcome probabilities over a list of qubits (the
//    reduction of apply_measure, state.mojo:466-501), optionally restricted
//    to amplitudes whose other listed qubits have fixed values.
//  * bf_measure: apply_measure (state.mojo:447-553) — reduction, the
//    reference's seeded draw (seed mod 2^31-1, times 48271 mod 2^31-1,
//    scaled by the total), collapse onto the drawn outcome and
//    renormalisation by 1/sqrt(p).
//  * bf_probs_topk: the k most probable basis states.
// Reductions accumulate |amp|^2 in double-float per thread and finish in
// FP64 on the host.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

constexpr int kMeasThreads = 256;
constexpr int kMaxOutcomeBits = 20;

struct MargArgs {
  uint64_t fixed_mask;   // listed qubits with a fixed value
  uint64_t fixed_val;    // their required bits
  int32_t nfree;         // free (outcome) qubits
  int8_t free_pos[kMaxOutcomeBits];
  int32_t nins;          // all listed qubits, ascending (inserted as zeros)
  int8_t ins[64];
  uint64_t rest;         // amplitudes per outcome: N >> nins
  uint64_t chunk;        // amplitudes per CTA
  uint32_t chunks;       // CTAs per outcome
};

template <class T>
__device__ __forceinline__ dfl prob_df(T a);
template <>
__device__ __forceinline__ dfl prob_df<double2>(double2 a) {
  dfl r = df_from_double(a.x), i = df_from_double(a.y);
  return df_dot2(r, r, i, i);
}
template <>
__device__ __forceinline__ dfl prob_df<float2>(float2 a) {
  dfl r{a.x, 0.f}, i{a.y, 0.f};
  return df_dot2(r, r, i, i);
}

__device__ __forceinline__ dfl block_sum_df(dfl acc) {
  __shared__ dfl wsum[kMeasThreads / 32];
  for (int off = 16; off > 0; off >>= 1) {
    dfl o{__shfl_down_sync(0xffffffffu, acc.hi, off), __shfl_down_sync(0xffffffffu, acc.lo, off)};
    acc = df_add(acc, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  acc = dfl{0.f, 0.f};
  if (warp == 0) {
    acc = lane < kMeasThreads / 32 ? wsum[lane] : dfl{0.f, 0.f};
    for (int off = 16; off > 0; off >>= 1) {
      dfl o{__shfl_down_sync(0xffffffffu, acc.hi, off), __shfl_down_sync(0xffffffffu, acc.lo, off)};
      acc = df_add(acc, o);
    }
  }
  return acc;
}

// CTA (outcome o = blockIdx.y, chunk c = blockIdx.x) sums |amp|^2 over the
// amplitudes whose listed qubits read (fixed values, bits of o).
template <class T>
__global__ void __launch_bounds__(kMeasThreads) k_marginal(const T* __restrict__ s, const MargArgs a,
                                                           double* __restrict__ partial) {
  const uint64_t o = blockIdx.x / a.chunks;
  const uint64_t cidx = blockIdx.x % a.chunks;
  uint64_t sel = a.fixed_val;
  for (int k = 0; k < a.nfree; ++k)
    if ((o >> k) & 1) sel |= 1ull << a.free_pos[k];
  const uint64_t begin = cidx * a.chunk;
  const uint64_t end = min(begin + a.chunk, a.rest);
  dfl acc{0.f, 0.f};
  for (uint64_t r = begin + threadIdx.x; r < end; r += kMeasThreads) {
    uint64_t x = r;
    for (int i = 0; i < a.nins; ++i) x = insert_zero_bit(x, a.ins[i]);
    acc = df_add(acc, prob_df<T>(s[x | sel]));
  }
  acc = block_sum_df(acc);
  if (threadIdx.x == 0) {
    size_t slot = blockIdx.x;
    partial[2 * slot] = (double)acc.hi;
    partial[2 * slot + 1] = (double)acc.lo;
  }
}

// collapse: keep (and scale) the amplitudes whose listed qubits read `want`
template <class P>
__global__ void __launch_bounds__(256) k_collapse(typename P::Glob* __restrict__ s, uint64_t N, uint64_t mask,
                                                  uint64_t want, double inv) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  typename P::Coef g;
  // coefficient (inv, 0) in the policy's representation
  double m[8] = {inv, 0, 0, 0, 0, 0, 0, 0};
  float hl[16];
  hl[0] = __double2float_rn(inv);  // one FP64 op per thread: negligible
  hl[1] = (float)(inv - (double)hl[0]);
  for (int i = 2; i < 16; ++i) hl[i] = 0.f;
  g = P::coef(m, hl);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += step) {
    typename P::R x = P::from_glob(s[i]);
    if ((i & mask) == want) {
      P::cmul(x, g, 0);
    } else {
      x = P::zero();
    }
    s[i] = P::to_glob(x);
  }
}

static void check_qubits(const State& st, const int32_t* q, int32_t nq) {
  if (nq < 0 || (nq > 0 && !q)) fail(BF_EINVAL, "qubit list is null");
  uint64_t seen = 0;
  for (int i = 0; i < nq; ++i) {
    if (q[i] < 0 || q[i] >= st.n) fail(BF_EINVAL, "Target out of bounds: %d", q[i]);
    if ((seen >> q[i]) & 1) fail(BF_EINVAL, "Duplicate target: %d", q[i]);
    seen |= 1ull << q[i];
  }
}

// Outcome probabilities over the free qubits (values[k] < 0) of `q`; the
// others must read values[k].  out[o], bit k of o = k-th free qubit.
void marginal_probs(State& st, const int32_t* q, const int8_t* values, int32_t nq, std::vector<double>& out) {
  check_qubits(st, q, nq);
  MargArgs a;
  std::memset(&a, 0, sizeof a);
  std::vector<int> all(q, q + nq);
  std::sort(all.begin(), all.end());
  a.nins = nq;
  for (int i = 0; i < nq; ++i) a.ins[i] = (int8_t)all[i];
  for (int i = 0; i < nq; ++i) {
    int v = values ? values[i] : -1;
    if (v < 0) {
      if (a.nfree >= kMaxOutcomeBits) fail(BF_EUNSUPPORTED, "more than %d free measured qubits", kMaxOutcomeBits);
      a.free_pos[a.nfree++] = (int8_t)q[i];
    } else {
      a.fixed_mask |= 1ull << q[i];
      if (v) a.fixed_val |= 1ull << q[i];
    }
  }
  a.rest = st.N >> nq;
  const uint64_t outcomes = 1ull << a.nfree;
  // aim for ~4 CTAs per SM in total, at least 4096 amplitudes per CTA
  uint64_t want_ctas = std::max<uint64_t>(1, (uint64_t)st.num_sms * 4 / outcomes);
  a.chunk = std::max<uint64_t>(4096, (a.rest + want_ctas - 1) / want_ctas);
  a.chunks = (uint32_t)((a.rest + a.chunk - 1) / a.chunk);
  size_t slots = (size_t)outcomes * a.chunks;
  ensure_partials(st, slots);
  if (slots > 0x7fffffffull) fail(BF_EUNSUPPORTED, "too many outcome slots");
  dim3 grid((unsigned)slots);
  if (st.dtype == BF_C128)
    k_marginal<double2><<<grid, kMeasThreads, 0, st.stream>>>(static_cast<const double2*>(st.amp), a, st.d_partial);
  else
    k_marginal<float2><<<grid, kMeasThreads, 0, st.stream>>>(static_cast<const float2*>(st.amp), a, st.d_partial);
  BF_CUDA(cudaGetLastError());
  st.launches++;
  BF_CUDA(cudaMemcpyAsync(st.h_partial, st.d_partial, 2 * slots * sizeof(double), cudaMemcpyDeviceToHost,
                          st.stream));
  sync_state(st);
  out.assign(outcomes, 0.0);
  for (uint64_t o = 0; o < outcomes; ++o) {
    double hi = 0, lo = 0;
    for (uint32_t c = 0; c < a.chunks; ++c) {
      hi += st.h_partial[2 * (o * a.chunks + c)];
      lo += st.h_partial[2 * (o * a.chunks + c) + 1];
    }
    out[o] = hi + lo;
  }
}

void measure(State& st, const int32_t* q, const int8_t* values, int32_t nq, int64_t seed, uint64_t* outcome,
             double* prob) {
  if (nq == 0) {
    if (outcome) *outcome = 0;
    if (prob) *prob = 1.0;
    return;
  }
  std::vector<double> p;
  marginal_probs(st, q, values, nq, p);
  double total = 0;
  for (double v : p) total += v;
  if (!(total > 0)) fail(BF_EINVAL, "Measurement probability is zero");
  // the reference's draw (state.mojo:506-525); a negative seed is replaced
  // by a clock-derived one there as well
  if (seed < 0) seed = (int64_t)std::chrono::steady_clock::now().time_since_epoch().count() & 0x7fffffffffffll;
  int64_t rng = seed % 2147483647;
  rng = (rng * 48271) % 2147483647;
  double r = (double)rng / (double)2147483647 * total;
  uint64_t chosen = 0;
  double acc = 0;
  for (uint64_t i = 0; i < p.size(); ++i) {
    acc += p[i];
    if (r <= acc) {
      chosen = i;
      break;
    }
  }
  double cp = p[chosen];
  if (!(cp > 0)) fail(BF_EINVAL, "Measurement outcome probability is zero");
  double inv = 1.0 / std::sqrt(cp);
  uint64_t mask = 0, want = 0;
  int k = 0;
  for (int i = 0; i < nq; ++i) {
    mask |= 1ull << q[i];
    int v = values ? values[i] : -1;
    int bit = v >= 0 ? v : (int)((chosen >> k++) & 1);
    if (bit) want |= 1ull << q[i];
  }
  unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((st.N + 255) / 256, (uint64_t)st.num_sms * 16));
  switch (st.prec) {
    case PREC_F64:
      k_collapse<PolF64><<<blocks, 256, 0, st.stream>>>(static_cast<double2*>(st.amp), st.N, mask, want, inv);
      break;
    case PREC_DF:
      k_collapse<PolDF><<<blocks, 256, 0, st.stream>>>(static_cast<double2*>(st.amp), st.N, mask, want, inv);
      break;
    default:
      k_collapse<PolF32><<<blocks, 256, 0, st.stream>>>(static_cast<float2*>(st.amp), st.N, mask, want, inv);
      break;
  }
  BF_CUDA(cudaGetLastError());
  st.launches++;
  if (outcome) *outcome = chosen;
  if (prob) *prob = cp;
}

// ---- top-k ------------------------------------------------------------------
// Each CTA keeps the running top kTopK of its grid-stride share in shared
// memory: a chunk of 256 probabilities is added, and kTopK rounds of a
// block-wide argmax pick the new top kTopK from the 256 + kTopK candidates.
// Candidates are ordered by (probability desc, index asc).  The host merges
// the per-CTA lists.
constexpr int kTopK = 64;

struct Cand {
  float hi, lo;
  uint64_t idx;
};

__device__ __forceinline__ bool cand_better(const Cand& a, const Cand& b) {
  if (a.hi != b.hi) return a.hi > b.hi;
  if (a.lo != b.lo) return a.lo > b.lo;
  return a.idx < b.idx;
}

template <class T>
__global__ void __launch_bounds__(kMeasThreads) k_topk(const T* __restrict__ s, uint64_t N, int k,
                                                       Cand* __restrict__ out) {
  __shared__ Cand pool[kMeasThreads + kTopK];
  __shared__ Cand best[kTopK];
  __shared__ int pick;
  const int tid = threadIdx.x;
  if (tid < kTopK) best[tid] = Cand{-1.f, 0.f, ~0ull};
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * kMeasThreads;
  for (uint64_t base = (uint64_t)blockIdx.x * kMeasThreads; base < N; base += stride) {
    uint64_t i = base + tid;
    Cand c{-1.f, 0.f, ~0ull};
    if (i < N) {
      dfl p = prob_df<T>(s[i]);
      c = Cand{p.hi, p.lo, i};
    }
    // skip the selection when no new probability beats the current k-th
    if (!__syncthreads_or(cand_better(c, best[k - 1]) ? 1 : 0)) continue;
    pool[tid] = c;
    if (tid < k) pool[kMeasThreads + tid] = best[tid];
    else if (tid < kTopK) pool[kMeasThreads + tid] = Cand{-1.f, 0.f, ~0ull};
    __syncthreads();
    // k rounds of argmax over the kMeasThreads + kTopK pool
    for (int r = 0; r < k; ++r) {
      int bi = tid;
      Cand bc = pool[tid];
      if (tid < kTopK && cand_better(pool[kMeasThreads + tid], bc)) {
        bc = pool[kMeasThreads + tid];
        bi = kMeasThreads + tid;
      }
      for (int off = 16; off > 0; off >>= 1) {
        Cand oc;
        oc.hi = __shfl_down_sync(0xffffffffu, bc.hi, off);
        oc.lo = __shfl_down_sync(0xffffffffu, bc.lo, off);
        oc.idx = __shfl_down_sync(0xffffffffu, bc.idx, off);
        int ob = __shfl_down_sync(0xffffffffu, bi, off);
        if (cand_better(oc, bc)) {
          bc = oc;
          bi = ob;
        }
      }
      __shared__ Cand wc[kMeasThreads / 32];
      __shared__ int wi[kMeasThreads / 32];
      if ((tid & 31) == 0) {
        wc[tid >> 5] = bc;
        wi[tid >> 5] = bi;
      }
      __syncthreads();
      if (tid == 0) {
        Cand b = wc[0];
        int bb = wi[0];
        for (int w = 1; w < kMeasThreads / 32; ++w)
          if (cand_better(wc[w], b)) {
            b = wc[w];
            bb = wi[w];
          }
        best[r] = b;
        pick = bb;
      }
      __syncthreads();
      if (tid == 0) pool[pick] = Cand{-2.f, 0.f, ~0ull};
      __syncthreads();
    }
  }
  if (tid < k) out[(size_t)blockIdx.x * k + tid] = best[tid];
}

void probs_topk(State& st, int k, uint64_t* idx, double* probs) {
  if (k < 1 || k > kTopK) fail(BF_EINVAL, "k must be in [1, %d]", kTopK);
  if ((uint64_t)k > st.N) fail(BF_EINVAL, "k exceeds the number of amplitudes");
  unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((st.N + kMeasThreads - 1) / kMeasThreads,
                                                                        (uint64_t)st.num_sms * 2));
  size_t need = (size_t)blocks * k * sizeof(Cand);
  ensure_partials(st, (need + 2 * sizeof(double) - 1) / (2 * sizeof(double)));
  Cand* d = reinterpret_cast<Cand*>(st.d_partial);
  if (st.dtype == BF_C128)
    k_topk<double2><<<blocks, kMeasThreads, 0, st.stream>>>(static_cast<const double2*>(st.amp), st.N, k, d);
  else
    k_topk<float2><<<blocks, kMeasThreads, 0, st.stream>>>(static_cast<const float2*>(st.amp), st.N, k, d);
  BF_CUDA(cudaGetLastError());
  st.launches++;
  std::vector<Cand> h((size_t)blocks * k);
  BF_CUDA(cudaMemcpyAsync(h.data(), d, need, cudaMemcpyDeviceToHost, st.stream));
  sync_state(st);
  std::sort(h.begin(), h.end(), [](const Cand& a, const Cand& b) {
    double pa = (double)a.hi + (double)a.lo, pb = (double)b.hi + (double)b.lo;
    if (pa != pb) return pa > pb;
    return a.idx < b.idx;
  });
  for (int i = 0; i < k; ++i) {
    idx[i] = h[i].idx;
    probs[i] = (double)h[i].hi + (double)h[i].lo;
  }
}

}  // namespace bf

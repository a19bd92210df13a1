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
// Each warp keeps a sorted list of its best candidates in registers: list
// position j sits in lane j % 32, slot j / 32.  One ballot tests 32
// probabilities against the warp's k-th best; the few lanes that beat it are
// inserted one at a time with shuffles.  After the first few thousand
// amplitudes almost no chunk holds one, so the pass streams the state at the
// cost of the ballot.  An FP32 estimate of |amp|^2 from the leading bits of
// each component skips the exact double-float square for amplitudes that
// cannot reach the k-th best.  The CTA's warps merge their lists through
// shared memory, and a one-CTA kernel merges the CTAs' lists, so the host
// reads back the k winners only.  Candidates are ordered by (probability
// desc, index asc).
constexpr int kTopK = 64;
constexpr int kTopUnroll = 4;            // loads in flight per thread
constexpr int kTopMergeThreads = 1024;
// The estimate is at least (1 - 2^-18) of the exact |amp|^2 and the k-th
// best's hi part is within 2^-24 of its value, so an amplitude that beats
// the k-th best has an estimate above its hi part times 1 - 2^-16.
constexpr float kTopSlack = 1.0f - 1.0f / 65536.0f;

struct Cand {
  float hi, lo;
  uint64_t idx;
};

__device__ __forceinline__ Cand cand_none() { return Cand{-1.f, 0.f, ~0ull}; }

__device__ __forceinline__ bool cand_better(const Cand& a, const Cand& b) {
  if (a.hi != b.hi) return a.hi > b.hi;
  if (a.lo != b.lo) return a.lo > b.lo;
  return a.idx < b.idx;
}

__device__ __forceinline__ Cand shfl_cand(const Cand& c, int src) {
  return Cand{__shfl_sync(0xffffffffu, c.hi, src), __shfl_sync(0xffffffffu, c.lo, src),
              __shfl_sync(0xffffffffu, c.idx, src)};
}

__device__ __forceinline__ Cand shfl_up_cand(const Cand& c) {
  return Cand{__shfl_up_sync(0xffffffffu, c.hi, 1), __shfl_up_sync(0xffffffffu, c.lo, 1),
              __shfl_up_sync(0xffffffffu, c.idx, 1)};
}

// |x| truncated to the 21 leading significant bits of the FP64 (its high
// word), as FP32; 0 below the FP32 range, +inf above it (and for Inf/NaN) so
// that the exact path decides those.
__device__ __forceinline__ float lead_abs(double x) {
  const unsigned hw = (unsigned)((unsigned long long)__double_as_longlong(x) >> 32);
  const int ef = (int)((hw >> 20) & 0x7ffu) - 896;
  if (ef <= 0) return 0.f;
  if (ef >= 255) return __int_as_float(0x7f800000);
  return __int_as_float((ef << 23) | (int)((hw & 0xfffffu) << 3));
}

// An FP32 estimate of |a|^2 that is at least (1 - 2^-18) of the exact value
// (two 2^-20 truncations squared, two FP32 roundings).
template <class T>
__device__ __forceinline__ float prob_estimate(T a);
template <>
__device__ __forceinline__ float prob_estimate<double2>(double2 a) {
  const float r = lead_abs(a.x), i = lead_abs(a.y);
  return fmaf(r, r, __fmul_rn(i, i));
}
template <>
__device__ __forceinline__ float prob_estimate<float2>(float2 a) {
  return fmaf(a.x, a.x, __fmul_rn(a.y, a.y));
}

// A warp's k best candidates, sorted, KB slots per lane (KB = 1 for k <= 32,
// 2 for k <= 64).  Unused positions hold cand_none().
template <int KB>
struct WarpTop {
  Cand s[KB];

  __device__ __forceinline__ void init() {
#pragma unroll
    for (int b = 0; b < KB; ++b) s[b] = cand_none();
  }
  // position k - 1, in every lane
  __device__ __forceinline__ Cand kth(int k) const {
    if (KB == 2 && k > 32) return shfl_cand(s[KB - 1], k - 33);
    return shfl_cand(s[0], k - 1);
  }
  // insert the warp-uniform x at its rank; the last position falls off
  __device__ __forceinline__ void insert(const Cand& x, int lane) {
    int pos = __popc(__ballot_sync(0xffffffffu, cand_better(s[0], x)));
    if (KB == 2) pos += __popc(__ballot_sync(0xffffffffu, cand_better(s[KB - 1], x)));
    const Cand up0 = shfl_up_cand(s[0]);
    if (KB == 2) {
      Cand up1 = shfl_up_cand(s[KB - 1]);
      const Cand last0 = shfl_cand(s[0], 31);
      if (lane == 0) up1 = last0;
      const int j = lane + 32;
      s[KB - 1] = j < pos ? s[KB - 1] : (j == pos ? x : up1);
    }
    s[0] = lane < pos ? s[0] : (lane == pos ? x : up0);
  }
  // one candidate per lane (where `valid`); thr is the k-th best and follows
  // the insertions
  __device__ __forceinline__ void offer(const Cand& c, bool valid, Cand& thr, int k, int lane) {
    unsigned m = __ballot_sync(0xffffffffu, valid && cand_better(c, thr));
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      const Cand x = shfl_cand(c, src);
      if (cand_better(x, thr)) {
        insert(x, lane);
        thr = kth(k);
      }
    }
  }
  __device__ __forceinline__ void store(Cand* dst, int k, int lane) const {
#pragma unroll
    for (int b = 0; b < KB; ++b)
      if (lane + 32 * b < k) dst[lane + 32 * b] = s[b];
  }
};

// The CTA's WARPS lists -> warp 0's list (valid in warp 0 only).
template <int KB, int WARPS>
__device__ __forceinline__ void merge_warps(WarpTop<KB>& top, Cand& thr, Cand (*lists)[kTopK], int k) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  top.store(lists[warp], k, lane);
  __syncthreads();
  if (warp != 0) return;
  for (int w = 1; w < WARPS; ++w)
    for (int j0 = 0; j0 < k; j0 += 32) {
      const int j = j0 + lane;
      top.offer(j < k ? lists[w][j] : cand_none(), j < k, thr, k, lane);
    }
}

template <class T, int KB>
__global__ void __launch_bounds__(kMeasThreads) k_topk(const T* __restrict__ s, uint64_t N, int k,
                                                       Cand* __restrict__ out) {
  constexpr int kWarps = kMeasThreads / 32;
  __shared__ Cand lists[kWarps][kTopK];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpTop<KB> top;
  top.init();
  Cand thr = cand_none();
  const uint64_t chunk = 32ull * kTopUnroll;
  const uint64_t step = (uint64_t)gridDim.x * kWarps * chunk;
  for (uint64_t base = ((uint64_t)blockIdx.x * kWarps + warp) * chunk; base < N; base += step) {
    T v[kTopUnroll];
#pragma unroll
    for (int u = 0; u < kTopUnroll; ++u) {
      const uint64_t i = base + 32 * u + lane;
      v[u] = i < N ? s[i] : T{};
    }
#pragma unroll
    for (int u = 0; u < kTopUnroll; ++u) {
      const uint64_t i = base + 32 * u + lane;
      const bool valid = i < N && prob_estimate<T>(v[u]) >= thr.hi * kTopSlack;
      Cand c{0.f, 0.f, i};
      if (valid) {
        const dfl p = prob_df<T>(v[u]);
        c.hi = p.hi;
        c.lo = p.lo;
      }
      top.offer(c, valid, thr, k, lane);
    }
  }
  merge_warps<KB, kWarps>(top, thr, lists, k);
  if (warp == 0) top.store(out + (size_t)blockIdx.x * k, k, lane);
}

// m candidates (the CTAs' lists) -> the k best, sorted.
template <int KB>
__global__ void __launch_bounds__(kTopMergeThreads) k_topk_merge(const Cand* __restrict__ in, int m, int k,
                                                                 Cand* __restrict__ out) {
  constexpr int kWarps = kTopMergeThreads / 32;
  __shared__ Cand lists[kWarps][kTopK];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpTop<KB> top;
  top.init();
  Cand thr = cand_none();
  for (int j0 = warp * 32; j0 < m; j0 += kTopMergeThreads) {
    const int j = j0 + lane;
    top.offer(j < m ? in[j] : cand_none(), j < m, thr, k, lane);
  }
  merge_warps<KB, kWarps>(top, thr, lists, k);
  if (warp == 0) top.store(out, k, lane);
}

template <class T, int KB>
static void launch_topk(State& st, unsigned blocks, int k, Cand* part, Cand* fin) {
  k_topk<T, KB><<<blocks, kMeasThreads, 0, st.stream>>>(static_cast<const T*>(st.amp), st.N, k, part);
  BF_CUDA(cudaGetLastError());
  k_topk_merge<KB><<<1, kTopMergeThreads, 0, st.stream>>>(part, (int)blocks * k, k, fin);
  BF_CUDA(cudaGetLastError());
  st.launches += 2;
}

void probs_topk(State& st, int k, uint64_t* idx, double* probs) {
  if (k < 1 || k > kTopK) fail(BF_EINVAL, "k must be in [1, %d]", kTopK);
  if ((uint64_t)k > st.N) fail(BF_EINVAL, "k exceeds the number of amplitudes");
  static_assert(sizeof(Cand) == 2 * sizeof(double), "a candidate fills one partial-sum slot");
  const uint64_t per_cta = (uint64_t)kMeasThreads * kTopUnroll;
  const unsigned blocks = (unsigned)std::max<uint64_t>(
      1, std::min<uint64_t>((st.N + per_cta - 1) / per_cta, (uint64_t)st.num_sms * 4));
  ensure_partials(st, (size_t)blocks * k + k);
  Cand* part = reinterpret_cast<Cand*>(st.d_partial);
  Cand* fin = part + (size_t)blocks * k;
  const bool wide = k > 32;
  if (st.dtype == BF_C128) {
    if (wide) launch_topk<double2, 2>(st, blocks, k, part, fin);
    else launch_topk<double2, 1>(st, blocks, k, part, fin);
  } else {
    if (wide) launch_topk<float2, 2>(st, blocks, k, part, fin);
    else launch_topk<float2, 1>(st, blocks, k, part, fin);
  }
  Cand* h = reinterpret_cast<Cand*>(st.h_partial);
  BF_CUDA(cudaMemcpyAsync(h, fin, (size_t)k * sizeof(Cand), cudaMemcpyDeviceToHost, st.stream));
  sync_state(st);
  for (int i = 0; i < k; ++i) {
    idx[i] = h[i].idx;
    probs[i] = (double)h[i].hi + (double)h[i].lo;
  }
}

}  // namespace bf

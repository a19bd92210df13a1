// grover.cu — the Grover diffuser and inversion about |0> as classical
// passes (apply_grover_diffuser / apply_grover_inversion_0,
// butterfly/algos/grover_classical.mojo:262-326), replacing their gate
// decompositions (H^k X^k MCP(pi) X^k H^k) with one reduction and one update.
//
// For every assignment b of the qubits outside `targets` (a block of 2^k
// amplitudes over the targets):
//   inversion:  x[b, 0] <- -x[b, 0]
//   diffuser:   x[b, t] <- 2 * mean_b - x[b, t],  mean_b = sum_t x[b, t] / 2^k
// The reference writes the imaginary part as -2 * mean_im - x_im
// (grover_classical.mojo:318); this pass uses 2 * mean - x for both parts,
// the inversion about the mean for complex amplitudes.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

struct DiffArgs {
  int32_t low;               // 1: the targets are qubits 0..k-1 (index = b << k | t)
  int32_t k;                 // targets
  int8_t tpos[64];           // target positions, ascending
  int32_t nother;
  int8_t opos[64];           // other positions, ascending
  uint64_t blocks;           // 2^(n-k)
  uint64_t chunk;            // target-subspace amplitudes per CTA
  uint32_t chunks;           // CTAs per block
};

__device__ __forceinline__ uint64_t deposit_pos(uint64_t x, const int8_t* pos, int cnt) {
  uint64_t r = 0;
  for (int j = 0; j < cnt; ++j) r |= ((x >> j) & 1ull) << pos[j];
  return r;
}

__device__ __forceinline__ uint64_t diff_index(const DiffArgs& a, uint64_t b, uint64_t t) {
  if (a.low) return (b << a.k) | t;
  return deposit_pos(b, a.opos, a.nother) | deposit_pos(t, a.tpos, a.k);
}

// negate the amplitudes whose target bits are all zero (sign bits only: exact)
template <class T>
__global__ void __launch_bounds__(256) k_inversion0(T* __restrict__ s, uint64_t count, DiffArgs a) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < count; b += step) {
    uint64_t i = diff_index(a, b, 0);
    T v = s[i];
    v.x = -v.x;
    v.y = -v.y;
    s[i] = v;
  }
}

// CTA (block b, chunk c) sums its share of block b's amplitudes (double-float)
template <class T>
__device__ __forceinline__ void amp_df(T g, dfl& re, dfl& im);
template <>
__device__ __forceinline__ void amp_df<double2>(double2 g, dfl& re, dfl& im) {
  re = df_from_double(g.x);
  im = df_from_double(g.y);
}
template <>
__device__ __forceinline__ void amp_df<float2>(float2 g, dfl& re, dfl& im) {
  re = dfl{g.x, 0.f};
  im = dfl{g.y, 0.f};
}

template <class T>
__global__ void __launch_bounds__(256) k_diff_sum(const T* __restrict__ s, DiffArgs a, float4* __restrict__ partial) {
  const uint64_t b = blockIdx.x / a.chunks, c = blockIdx.x % a.chunks;
  const uint64_t sub = 1ull << a.k;
  const uint64_t begin = c * a.chunk, end = min(begin + a.chunk, sub);
  dfl sr{0.f, 0.f}, si{0.f, 0.f};
  for (uint64_t t = begin + threadIdx.x; t < end; t += blockDim.x) {
    dfl xr, xi;
    amp_df<T>(s[diff_index(a, b, t)], xr, xi);
    sr = df_add(sr, xr);
    si = df_add(si, xi);
  }
  __shared__ dfl wr[8], wi[8];
  for (int off = 16; off > 0; off >>= 1) {
    sr = df_add(sr, dfl{__shfl_down_sync(0xffffffffu, sr.hi, off), __shfl_down_sync(0xffffffffu, sr.lo, off)});
    si = df_add(si, dfl{__shfl_down_sync(0xffffffffu, si.hi, off), __shfl_down_sync(0xffffffffu, si.lo, off)});
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    wr[warp] = sr;
    wi[warp] = si;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    dfl r = wr[0], im = wi[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      r = df_add(r, wr[w]);
      im = df_add(im, wi[w]);
    }
    partial[blockIdx.x] = make_float4(r.hi, r.lo, im.hi, im.lo);
  }
}

// one CTA per block b: 2 * mean_b in double-float from its chunk partials
__global__ void __launch_bounds__(256) k_diff_mean(const float4* __restrict__ partial, DiffArgs a,
                                                   float4* __restrict__ mean2) {
  const uint64_t b = blockIdx.x;
  dfl r{0.f, 0.f}, im{0.f, 0.f};
  for (uint32_t c = threadIdx.x; c < a.chunks; c += blockDim.x) {
    float4 p = partial[b * a.chunks + c];
    r = df_add(r, dfl{p.x, p.y});
    im = df_add(im, dfl{p.z, p.w});
  }
  __shared__ dfl wr[8], wi[8];
  for (int off = 16; off > 0; off >>= 1) {
    r = df_add(r, dfl{__shfl_down_sync(0xffffffffu, r.hi, off), __shfl_down_sync(0xffffffffu, r.lo, off)});
    im = df_add(im, dfl{__shfl_down_sync(0xffffffffu, im.hi, off), __shfl_down_sync(0xffffffffu, im.lo, off)});
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    wr[warp] = r;
    wi[warp] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      wr[0] = df_add(wr[0], wr[w]);
      wi[0] = df_add(wi[0], wi[w]);
    }
    // scale by 2 / 2^k: a power of two, exact on both parts
    const float sc = ldexpf(1.0f, 1 - a.k);
    mean2[b] = make_float4(wr[0].hi * sc, wr[0].lo * sc, wi[0].hi * sc, wi[0].lo * sc);
  }
}

template <class P>
__global__ void __launch_bounds__(256) k_diff_update(typename P::Glob* __restrict__ s, DiffArgs a,
                                                     const float4* __restrict__ mean2) {
  const uint64_t sub = 1ull << a.k;
  const uint64_t total = a.blocks * sub;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < total; j += step) {
    const uint64_t b = j >> a.k, t = j & (sub - 1);
    const uint64_t i = diff_index(a, b, t);
    const float4 m = mean2[b];
    typename P::R x = P::from_glob(s[i]);
    if constexpr (std::is_same<P, PolDF>::value) {
      x.re = df_sub(dfl{m.x, m.y}, x.re);
      x.im = df_sub(dfl{m.z, m.w}, x.im);
    } else if constexpr (std::is_same<P, PolF32>::value) {
      x.re = (m.x + m.y) - x.re;
      x.im = (m.z + m.w) - x.im;
    } else {
      x.re = ((double)m.x + (double)m.y) - x.re;
      x.im = ((double)m.z + (double)m.w) - x.im;
    }
    s[i] = P::to_glob(x);
  }
}

// small target sets (k <= kSmallDiff): one thread per block, sum then update
constexpr int kSmallDiff = 8;

template <class P>
__global__ void __launch_bounds__(256) k_diff_small(typename P::Glob* __restrict__ s, DiffArgs a) {
  const uint64_t sub = 1ull << a.k;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < a.blocks; b += step) {
    const uint64_t base = deposit_pos(b, a.opos, a.nother);
    dfl sr{0.f, 0.f}, si{0.f, 0.f};
    for (uint64_t t = 0; t < sub; ++t) {
      dfl xr, xi;
      amp_df<typename P::Glob>(s[base | deposit_pos(t, a.tpos, a.k)], xr, xi);
      sr = df_add(sr, xr);
      si = df_add(si, xi);
    }
    const float sc = ldexpf(1.0f, 1 - a.k);
    const float4 m = make_float4(sr.hi * sc, sr.lo * sc, si.hi * sc, si.lo * sc);
    for (uint64_t t = 0; t < sub; ++t) {
      const uint64_t i = base | deposit_pos(t, a.tpos, a.k);
      typename P::R x = P::from_glob(s[i]);
      if constexpr (std::is_same<P, PolDF>::value) {
        x.re = df_sub(dfl{m.x, m.y}, x.re);
        x.im = df_sub(dfl{m.z, m.w}, x.im);
      } else if constexpr (std::is_same<P, PolF32>::value) {
        x.re = (m.x + m.y) - x.re;
        x.im = (m.z + m.w) - x.im;
      } else {
        x.re = ((double)m.x + (double)m.y) - x.re;
        x.im = ((double)m.z + (double)m.w) - x.im;
      }
      s[i] = P::to_glob(x);
    }
  }
}

static DiffArgs diff_args(const State& st, const int32_t* q, int32_t nq) {
  DiffArgs a;
  std::memset(&a, 0, sizeof a);
  uint64_t tm = 0;
  if (nq == 0) tm = (st.n >= 64) ? ~0ull : ((1ull << st.n) - 1);
  for (int i = 0; i < nq; ++i) {
    if (q[i] < 0 || q[i] >= st.n) fail(BF_EINVAL, "Target out of bounds: %d", q[i]);
    if ((tm >> q[i]) & 1) fail(BF_EINVAL, "Duplicate target: %d", q[i]);
    tm |= 1ull << q[i];
  }
  for (int b = 0; b < st.n; ++b) {
    if ((tm >> b) & 1) a.tpos[a.k++] = (int8_t)b;
    else a.opos[a.nother++] = (int8_t)b;
  }
  a.blocks = 1ull << a.nother;
  a.low = (a.k == 0) || (a.tpos[a.k - 1] == a.k - 1);  // ascending: targets are 0..k-1
  return a;
}

// classical_oracle (grover.mojo:64-66): negate listed amplitudes, eight per launch
struct OracleIdx {
  int32_t count;
  uint64_t idx[8];
};

template <class T>
__global__ void k_negate(T* s, OracleIdx a) {
  if ((int)threadIdx.x < a.count) {
    T v = s[a.idx[threadIdx.x]];
    v.x = -v.x;
    v.y = -v.y;
    s[a.idx[threadIdx.x]] = v;
  }
}

void launch_classical_oracle(State& st, const double* idx, int64_t count) {
  for (int64_t k = 0; k < count; k += 8) {
    OracleIdx a;
    a.count = (int32_t)std::min<int64_t>(8, count - k);
    for (int j = 0; j < a.count; ++j) a.idx[j] = (uint64_t)idx[k + j];
    // a repeated index is negated twice, as in the reference's loop
    bool dup = false;
    for (int i = 0; i < a.count; ++i)
      for (int j = i + 1; j < a.count; ++j) dup |= a.idx[i] == a.idx[j];
    if (dup) {
      for (int j = 0; j < a.count; ++j) {
        OracleIdx one;
        one.count = 1;
        one.idx[0] = a.idx[j];
        if (st.dtype == BF_C128) k_negate<double2><<<1, 32, 0, st.stream>>>(static_cast<double2*>(st.amp), one);
        else k_negate<float2><<<1, 32, 0, st.stream>>>(static_cast<float2*>(st.amp), one);
        st.launches++;
      }
    } else {
      if (st.dtype == BF_C128) k_negate<double2><<<1, 32, 0, st.stream>>>(static_cast<double2*>(st.amp), a);
      else k_negate<float2><<<1, 32, 0, st.stream>>>(static_cast<float2*>(st.amp), a);
      st.launches++;
    }
    BF_CUDA(cudaGetLastError());
  }
}

void launch_grover_inversion0(State& st, const int32_t* q, int32_t nq) {
  DiffArgs a = diff_args(st, q, nq);
  unsigned g = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((a.blocks + 255) / 256, (uint64_t)st.num_sms * 16));
  if (st.dtype == BF_C128) k_inversion0<double2><<<g, 256, 0, st.stream>>>(static_cast<double2*>(st.amp), a.blocks, a);
  else k_inversion0<float2><<<g, 256, 0, st.stream>>>(static_cast<float2*>(st.amp), a.blocks, a);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

template <class P>
static void diffuser_p(State& st, DiffArgs& a) {
  if (a.k <= kSmallDiff) {
    unsigned g = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((a.blocks + 255) / 256, (uint64_t)st.num_sms * 16));
    k_diff_small<P><<<g, 256, 0, st.stream>>>(static_cast<typename P::Glob*>(st.amp), a);
    BF_CUDA(cudaGetLastError());
    st.launches++;
    return;
  }
  const uint64_t sub = 1ull << a.k;
  // short CTAs (16 Ki amplitudes each) so that other streams' kernels get SMs
  // between them
  a.chunk = std::min<uint64_t>(sub, 1ull << 14);
  a.chunks = (uint32_t)((sub + a.chunk - 1) / a.chunk);
  uint64_t slots = a.blocks * a.chunks;
  if (slots > 0x7fffffffull) fail(BF_EUNSUPPORTED, "too many diffuser blocks");
  // partials (float4 per slot) then 2*mean (float4 per block), in the partials buffer
  size_t need = (size_t)(slots + a.blocks) * sizeof(float4);
  ensure_partials(st, (need + 2 * sizeof(double) - 1) / (2 * sizeof(double)));
  float4* partial = reinterpret_cast<float4*>(st.d_partial);
  float4* mean2 = partial + slots;
  auto* s = static_cast<typename P::Glob*>(st.amp);
  k_diff_sum<typename P::Glob><<<(unsigned)slots, 256, 0, st.stream>>>(s, a, partial);
  if (a.blocks > 0x7fffffffull) fail(BF_EUNSUPPORTED, "too many diffuser blocks");
  k_diff_mean<<<(unsigned)a.blocks, 256, 0, st.stream>>>(partial, a, mean2);
  // one element per thread: short CTAs
  unsigned g = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((st.N + 255) / 256, 0x7fffffffull));
  k_diff_update<P><<<g, 256, 0, st.stream>>>(s, a, mean2);
  BF_CUDA(cudaGetLastError());
  st.launches += 3;
}

void launch_grover_diffuser(State& st, const int32_t* q, int32_t nq) {
  DiffArgs a = diff_args(st, q, nq);
  switch (st.prec) {
    case PREC_F64: diffuser_p<PolF64>(st, a); break;
    case PREC_DF: diffuser_p<PolDF>(st, a); break;
    default: diffuser_p<PolF32>(st, a); break;
  }
}

// ---- Grover search loop ------------------------------------------------------
// `iters` repetitions of (classical oracle, diffuser over every qubit) -- the
// body of grover_search with the classical replacements (grover.mojo:64-94,
// grover_classical.mojo:284-326) -- in one cooperative launch.  Each CTA owns
// a fixed contiguous chunk of the state.  Pass p (0..iters) reads the chunk,
// applies the diffuser update of iteration p-1 (x <- 2*mean - x, the mean
// coming from the partial sums of pass p-1), then the oracle of iteration p
// (negate the marked amplitudes) and sums the result for the next mean; one
// grid barrier separates the passes.  Per iteration this is one read and one
// write of the state and no launch, against three launches and 1.5 passes for
// the per-op form.  The partial sums alternate between two buffers, so a CTA
// that runs ahead into pass p+1 never overwrites sums another CTA is still
// reading in pass p.
struct LoopArgs {
  uint64_t N;
  uint64_t chunk;         // amplitudes per CTA
  int32_t iters;
  int32_t nmarked;        // indices negated by the oracle (odd multiplicity)
  uint64_t marked[8];
  int32_t n;              // qubits: 2 * mean = sum * 2^(1-n)
  uint32_t spin_limit;    // polls of 64 ns before a barrier wait gives up
  float4* partial;        // 2 x gridDim.x
  unsigned int* bar;      // arrival counter, zero at launch
  int* flag;              // set to 1 when a barrier wait expires
};

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// all CTAs of the grid: returns false (CTA-uniform) when the wait expired
__device__ __forceinline__ bool loop_barrier(const LoopArgs& a, unsigned int target) {
  __shared__ int ok_sh;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(a.bar, 1u);
    unsigned int polls = 0;
    while (ld_acquire_u32(a.bar) < target) {
      if (++polls > a.spin_limit) {
        ok = 0;
        atomicExch(a.flag, 1);
        break;
      }
      __nanosleep(64);
    }
    ok_sh = ok;
  }
  __syncthreads();
  return ok_sh != 0;
}

__device__ __forceinline__ void block_sum2(dfl& r, dfl& im, dfl* wr, dfl* wi) {
  for (int off = 16; off > 0; off >>= 1) {
    r = df_add(r, dfl{__shfl_down_sync(0xffffffffu, r.hi, off), __shfl_down_sync(0xffffffffu, r.lo, off)});
    im = df_add(im, dfl{__shfl_down_sync(0xffffffffu, im.hi, off), __shfl_down_sync(0xffffffffu, im.lo, off)});
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    wr[warp] = r;
    wi[warp] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      wr[0] = df_add(wr[0], wr[w]);
      wi[0] = df_add(wi[0], wi[w]);
    }
    r = wr[0];
    im = wi[0];
  }
}

template <class P>
__device__ __forceinline__ void loop_update(typename P::R& x, const float4 m) {
  if constexpr (std::is_same<P, PolDF>::value) {
    x.re = df_sub(dfl{m.x, m.y}, x.re);
    x.im = df_sub(dfl{m.z, m.w}, x.im);
  } else if constexpr (std::is_same<P, PolF32>::value) {
    x.re = (m.x + m.y) - x.re;
    x.im = (m.z + m.w) - x.im;
  } else {
    x.re = ((double)m.x + (double)m.y) - x.re;
    x.im = ((double)m.z + (double)m.w) - x.im;
  }
}

template <class P>
__device__ __forceinline__ void loop_accumulate(const typename P::R& x, dfl& sr, dfl& si) {
  if constexpr (std::is_same<P, PolDF>::value) {
    sr = df_add(sr, x.re);
    si = df_add(si, x.im);
  } else if constexpr (std::is_same<P, PolF32>::value) {
    sr = df_add(sr, dfl{x.re, 0.f});
    si = df_add(si, dfl{x.im, 0.f});
  } else {
    sr = df_add(sr, df_from_double(x.re));
    si = df_add(si, df_from_double(x.im));
  }
}

template <class P>
__device__ __forceinline__ void loop_negate(typename P::R& x) {
  if constexpr (std::is_same<P, PolDF>::value) {
    x.re = df_neg(x.re);
    x.im = df_neg(x.im);
  } else {
    x.re = -x.re;
    x.im = -x.im;
  }
}

template <class P>
__global__ void __launch_bounds__(256) k_grover_loop(typename P::Glob* __restrict__ s, LoopArgs a) {
  __shared__ dfl wr[8], wi[8];
  __shared__ float4 m2_sh;
  const uint64_t begin = (uint64_t)blockIdx.x * a.chunk;
  const uint64_t end = min(begin + a.chunk, a.N);
  const unsigned int G = gridDim.x;
  const float sc = ldexpf(1.0f, 1 - a.n);
  for (int p = 0; p <= a.iters; ++p) {
    float4 m2 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p > 0) {
      const float4* part = a.partial + (size_t)((p - 1) & 1) * G;
      dfl r{0.f, 0.f}, im{0.f, 0.f};
      for (unsigned int c = threadIdx.x; c < G; c += blockDim.x) {
        float4 q = __ldcg(part + c);
        r = df_add(r, dfl{q.x, q.y});
        im = df_add(im, dfl{q.z, q.w});
      }
      block_sum2(r, im, wr, wi);
      if (threadIdx.x == 0) m2_sh = make_float4(r.hi * sc, r.lo * sc, im.hi * sc, im.lo * sc);
      __syncthreads();
      m2 = m2_sh;
    }
    const bool last = p == a.iters;
    dfl sr{0.f, 0.f}, si{0.f, 0.f};
    // eight loads in flight per thread before any use
    constexpr int kU = 8;
    for (uint64_t base = begin + threadIdx.x; base < end; base += kU * blockDim.x) {
      typename P::Glob v[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint64_t i = base + (uint64_t)u * blockDim.x;
        if (i < end) v[u] = s[i];
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint64_t i = base + (uint64_t)u * blockDim.x;
        if (i >= end) break;
        typename P::R x = P::from_glob(v[u]);
        if (p > 0) loop_update<P>(x, m2);
        if (!last) {
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (k < a.nmarked && i == a.marked[k]) loop_negate<P>(x);
          loop_accumulate<P>(x, sr, si);
        }
        s[i] = P::to_glob(x);
      }
    }
    if (last) break;
    __syncthreads();  // wr/wi reuse
    block_sum2(sr, si, wr, wi);
    if (threadIdx.x == 0) a.partial[(size_t)(p & 1) * G + blockIdx.x] = make_float4(sr.hi, sr.lo, si.hi, si.lo);
    if (G > 1) {
      if (!loop_barrier(a, (unsigned int)(p + 1) * G)) return;
    } else {
      __syncthreads();
    }
  }
}

// Cluster form, for states that fit in the shared memory of one thread-block
// cluster (up to 16 CTAs of 128 KiB): each CTA keeps its chunk in shared
// memory for all iterations, the partial sums travel through distributed
// shared memory and the hardware cluster barrier separates the passes -- no
// global traffic between the first load and the last store, and no waits of
// our own.
constexpr int kClusterThreads = 512;
constexpr uint32_t kClusterChunkBytes = 128 * 1024;

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::
          : "memory");
}

__device__ __forceinline__ float4 ld_cluster_f4(const float4* local, uint32_t rank) {
  uint32_t la = (uint32_t)__cvta_generic_to_shared(local), ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(rank));
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(ra)
               : "memory");
  return v;
}

template <class P>
__global__ void __launch_bounds__(kClusterThreads) k_grover_cluster(typename P::Glob* __restrict__ s, LoopArgs a,
                                                                      uint32_t csize) {
  using S = typename P::Smem;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S* amp = reinterpret_cast<S*>(smem_raw);
  __shared__ float4 part[2];  // this CTA's partial sums, by pass parity
  __shared__ dfl wr[kClusterThreads / 32], wi[kClusterThreads / 32];
  __shared__ float4 m2_sh;
  const uint32_t rank = cluster_rank();
  const int cnt = (int)a.chunk;
  const uint64_t begin = (uint64_t)rank * a.chunk;
  for (int e = threadIdx.x; e < cnt; e += kClusterThreads) amp[e] = P::to_smem(P::from_glob(s[begin + e]));
  __syncthreads();
  const float sc = ldexpf(1.0f, 1 - a.n);
  for (int p = 0; p <= a.iters; ++p) {
    float4 m2 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p > 0) {
      if (threadIdx.x < 32) {  // every CTA sums the cluster's partials in the same order
        dfl r{0.f, 0.f}, im{0.f, 0.f};
        if (threadIdx.x < csize) {
          const float4 q = ld_cluster_f4(&part[(p - 1) & 1], threadIdx.x);
          r = dfl{q.x, q.y};
          im = dfl{q.z, q.w};
        }
        for (int off = 16; off > 0; off >>= 1) {
          r = df_add(r, dfl{__shfl_down_sync(0xffffffffu, r.hi, off), __shfl_down_sync(0xffffffffu, r.lo, off)});
          im = df_add(im, dfl{__shfl_down_sync(0xffffffffu, im.hi, off), __shfl_down_sync(0xffffffffu, im.lo, off)});
        }
        if (threadIdx.x == 0) m2_sh = make_float4(r.hi * sc, r.lo * sc, im.hi * sc, im.lo * sc);
      }
      __syncthreads();
      m2 = m2_sh;
    }
    const bool last = p == a.iters;
    dfl sr{0.f, 0.f}, si{0.f, 0.f};
    for (int e = threadIdx.x; e < cnt; e += kClusterThreads) {
      typename P::R x = P::from_smem(amp[e]);
      if (p > 0) loop_update<P>(x, m2);
      if (!last) {
        const uint64_t i = begin + (uint64_t)e;
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (k < a.nmarked && i == a.marked[k]) loop_negate<P>(x);
        loop_accumulate<P>(x, sr, si);
      }
      amp[e] = P::to_smem(x);
    }
    if (last) break;
    block_sum2(sr, si, wr, wi);
    if (threadIdx.x == 0) part[p & 1] = make_float4(sr.hi, sr.lo, si.hi, si.lo);
    cluster_sync_all();
  }
  __syncthreads();
  for (int e = threadIdx.x; e < cnt; e += kClusterThreads) s[begin + e] = P::to_glob(P::from_smem(amp[e]));
  // the other CTAs may still be reading this CTA's partials
  cluster_sync_all();
}

// launches the cluster form when the state fits; false otherwise
template <class P>
static bool try_grover_cluster(State& st, LoopArgs& a) {
  const uint64_t cap = kClusterChunkBytes / sizeof(typename P::Smem);
  uint32_t C = 1;
  while ((uint64_t)C * cap < st.N) C <<= 1;
  if (C > 16) return false;
  a.chunk = st.N / C;
  const size_t smem = (size_t)a.chunk * sizeof(typename P::Smem);
  static PerDeviceOnce configured;  // one per instantiation of P
  configured.run(st.device, [] {
    BF_CUDA(cudaFuncSetAttribute(k_grover_cluster<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kClusterChunkBytes));
    BF_CUDA(cudaFuncSetAttribute(k_grover_cluster<P>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  });
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, k_grover_cluster<P>, &cfg) != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    return false;
  }
  BF_CUDA(cudaLaunchKernelEx(&cfg, k_grover_cluster<P>, static_cast<typename P::Glob*>(st.amp), a, C));
  st.launches++;
  return true;
}

int grover_loop_max_marked() { return 8; }

void launch_grover_loop(State& st, const uint64_t* marked, int nmarked, int iters) {
  if (iters <= 0) return;
  if (nmarked < 0 || nmarked > 8) fail(BF_EINVAL, "internal: %d oracle indices in a Grover loop", nmarked);
  LoopArgs a;
  std::memset(&a, 0, sizeof a);
  a.N = st.N;
  a.n = st.n;
  a.iters = iters;
  a.nmarked = nmarked;
  for (int k = 0; k < nmarked; ++k) a.marked[k] = marked[k];
  switch (st.prec) {
    case PREC_F64:
      if (try_grover_cluster<PolF64>(st, a)) return;
      break;
    case PREC_DF:
      if (try_grover_cluster<PolDF>(st, a)) return;
      break;
    default:
      if (try_grover_cluster<PolF32>(st, a)) return;
      break;
  }
  a.spin_limit = 1u << 25;  // x 64 ns sleeps: about 2 s
  // chunks of at least 4096 amplitudes
  int per_sm = 0;
  const void* fn = nullptr;
  switch (st.prec) {
    case PREC_F64: fn = (const void*)k_grover_loop<PolF64>; break;
    case PREC_DF: fn = (const void*)k_grover_loop<PolDF>; break;
    default: fn = (const void*)k_grover_loop<PolF32>; break;
  }
  BF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0));
  uint64_t resident = (uint64_t)std::max(1, per_sm) * (uint64_t)st.num_sms;
  // a server slot shares the GPU: its loop holds at most kSharedLoopCtas
  // SMs' worth of CTAs for the whole search, so the other slots keep the rest
  // (per-op kernels instead would issue four launches per iteration from
  // every slot at once)
  constexpr uint64_t kSharedLoopCtas = 16;
  const uint64_t cap = st.shared_gpu ? kSharedLoopCtas : (uint64_t)2 * st.num_sms;
  uint64_t G = std::max<uint64_t>(1, std::min<uint64_t>(std::min(cap, resident), st.N >> 12));
  a.chunk = (st.N + G - 1) / G;
  a.chunk = (a.chunk + 255) & ~255ull;
  G = (st.N + a.chunk - 1) / a.chunk;
  // partial sums (2 x G float4), the arrival counter after them
  size_t bytes = 2 * G * sizeof(float4) + 16;
  ensure_partials(st, (bytes + 2 * sizeof(double) - 1) / (2 * sizeof(double)));
  a.partial = reinterpret_cast<float4*>(st.d_partial);
  a.bar = reinterpret_cast<unsigned int*>(reinterpret_cast<char*>(st.d_partial) + 2 * G * sizeof(float4));
  a.flag = state_flag(st);
  BF_CUDA(cudaMemsetAsync(a.bar, 0, sizeof(unsigned int), st.stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)G);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  switch (st.prec) {
    case PREC_F64: BF_CUDA(cudaLaunchKernelEx(&cfg, k_grover_loop<PolF64>, static_cast<double2*>(st.amp), a)); break;
    case PREC_DF: BF_CUDA(cudaLaunchKernelEx(&cfg, k_grover_loop<PolDF>, static_cast<double2*>(st.amp), a)); break;
    default: BF_CUDA(cudaLaunchKernelEx(&cfg, k_grover_loop<PolF32>, static_cast<float2*>(st.amp), a)); break;
  }
  st.launches++;
}

}  // namespace bf

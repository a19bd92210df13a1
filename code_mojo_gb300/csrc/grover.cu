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

}  // namespace bf

// state_ops.cu — state initialisation, SoA <-> interleaved conversion at the
// boundary, the |amp|^2 reduction, and dense m-qubit unitaries.
#include <algorithm>
#include <vector>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

// ---- |idx> (State(n) is |0...0>, state.mojo:26-33) -------------------------
template <class T>
__global__ void k_set_one(T* s, uint64_t idx);
template <>
__global__ void k_set_one<double2>(double2* s, uint64_t idx) { s[idx] = make_double2(1.0, 0.0); }
template <>
__global__ void k_set_one<float2>(float2* s, uint64_t idx) { s[idx] = make_float2(1.0f, 0.0f); }

void launch_set_basis(State& st, uint64_t idx) {
  BF_CUDA(cudaMemsetAsync(st.amp, 0, st.bytes(), st.stream));
  if (st.dtype == BF_C128) k_set_one<double2><<<1, 1, 0, st.stream>>>(static_cast<double2*>(st.amp), idx);
  else k_set_one<float2><<<1, 1, 0, st.stream>>>(static_cast<float2*>(st.amp), idx);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

// ---- SoA (re[], im[], the reference's layout) <-> interleaved --------------
__global__ void __launch_bounds__(256) k_interleave_c128(double2* __restrict__ s, const double* __restrict__ re,
                                                         const double* __restrict__ im, uint64_t cnt) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += step)
    s[i] = make_double2(re[i], im[i]);
}
__global__ void __launch_bounds__(256) k_interleave_c64(float2* __restrict__ s, const double* __restrict__ re,
                                                        const double* __restrict__ im, uint64_t cnt) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += step)
    s[i] = make_float2((float)re[i], (float)im[i]);
}
__global__ void __launch_bounds__(256) k_deinterleave_c128(const double2* __restrict__ s, double* __restrict__ re,
                                                           double* __restrict__ im, uint64_t cnt) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += step) {
    double2 v = s[i];
    re[i] = v.x;
    im[i] = v.y;
  }
}
__global__ void __launch_bounds__(256) k_deinterleave_c64(const float2* __restrict__ s, double* __restrict__ re,
                                                          double* __restrict__ im, uint64_t cnt) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += step) {
    float2 v = s[i];
    re[i] = (double)v.x;
    im[i] = (double)v.y;
  }
}

static unsigned grid_for(const State& st, uint64_t cnt) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((cnt + 255) / 256, (uint64_t)st.num_sms * 16));
}

void launch_interleave(State& st, const double* d_re, const double* d_im, uint64_t off, uint64_t cnt) {
  if (st.dtype == BF_C128)
    k_interleave_c128<<<grid_for(st, cnt), 256, 0, st.stream>>>(static_cast<double2*>(st.amp) + off, d_re, d_im, cnt);
  else
    k_interleave_c64<<<grid_for(st, cnt), 256, 0, st.stream>>>(static_cast<float2*>(st.amp) + off, d_re, d_im, cnt);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_deinterleave(State& st, double* d_re, double* d_im, uint64_t off, uint64_t cnt) {
  if (st.dtype == BF_C128)
    k_deinterleave_c128<<<grid_for(st, cnt), 256, 0, st.stream>>>(static_cast<const double2*>(st.amp) + off, d_re,
                                                                   d_im, cnt);
  else
    k_deinterleave_c64<<<grid_for(st, cnt), 256, 0, st.stream>>>(static_cast<const float2*>(st.amp) + off, d_re,
                                                                  d_im, cnt);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

// ---- sum |amp|^2 --------------------------------------------------------
// Each thread accumulates in double-float (about 48 significant bits), the
// block combines its warps with shuffles, and the per-block partials are
// summed on the host in FP64.
__device__ __forceinline__ dfl df_shfl_add(dfl v, int off) {
  dfl o;
  o.hi = __shfl_down_sync(0xffffffffu, v.hi, off);
  o.lo = __shfl_down_sync(0xffffffffu, v.lo, off);
  return df_add(v, o);
}

template <class T>
__device__ __forceinline__ dfl amp_norm2_df(T a);
template <>
__device__ __forceinline__ dfl amp_norm2_df<double2>(double2 a) {
  dfl r = df_from_double(a.x), i = df_from_double(a.y);
  return df_dot2(r, r, i, i);
}
template <>
__device__ __forceinline__ dfl amp_norm2_df<float2>(float2 a) {
  dfl r{a.x, 0.f}, i{a.y, 0.f};
  return df_dot2(r, r, i, i);
}

template <class T>
__global__ void __launch_bounds__(256) k_norm2(const T* __restrict__ s, uint64_t N, double* __restrict__ partial) {
  __shared__ dfl wsum[8];
  dfl acc{0.f, 0.f};
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += step)
    acc = df_add(acc, amp_norm2_df<T>(s[i]));
  for (int off = 16; off > 0; off >>= 1) acc = df_shfl_add(acc, off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  if (warp == 0) {
    acc = lane < (int)(blockDim.x >> 5) ? wsum[lane] : dfl{0.f, 0.f};
    for (int off = 16; off > 0; off >>= 1) acc = df_shfl_add(acc, off);
    if (lane == 0) {
      partial[2 * blockIdx.x] = (double)acc.hi;
      partial[2 * blockIdx.x + 1] = (double)acc.lo;
    }
  }
}

void ensure_partials(State& st, size_t blocks) {
  if (st.partial_cap >= blocks) return;
  blocks = std::max(blocks, 2 * st.partial_cap);
  dev_free(st, st.d_partial);
  host_retire(st, st.h_partial);
  st.d_partial = nullptr;
  st.h_partial = nullptr;
  st.partial_cap = 0;
  st.d_partial = static_cast<double*>(dev_alloc(st, 2 * blocks * sizeof(double)));
  st.h_partial = static_cast<double*>(host_alloc(2 * blocks * sizeof(double)));
  st.partial_cap = blocks;
}

double reduce_norm2(State& st) {
  unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((st.N + 255) / 256, (uint64_t)st.num_sms * 8));
  ensure_partials(st, blocks);
  if (st.dtype == BF_C128)
    k_norm2<double2><<<blocks, 256, 0, st.stream>>>(static_cast<const double2*>(st.amp), st.N, st.d_partial);
  else
    k_norm2<float2><<<blocks, 256, 0, st.stream>>>(static_cast<const float2*>(st.amp), st.N, st.d_partial);
  BF_CUDA(cudaGetLastError());
  st.launches++;
  BF_CUDA(cudaMemcpyAsync(st.h_partial, st.d_partial, 2 * blocks * sizeof(double), cudaMemcpyDeviceToHost,
                          st.stream));
  sync_state(st);
  double hi = 0, lo = 0;
  for (unsigned b = 0; b < blocks; ++b) {
    hi += st.h_partial[2 * b];
    lo += st.h_partial[2 * b + 1];
  }
  return hi + lo;
}

// ---- <a|b> ------------------------------------------------------------------
// sum conj(a_i) b_i over two states of the same size and either dtype, in
// double-float per thread; partials (re.hi, re.lo, im.hi, im.lo) per block
// summed on the host in FP64.  Used for the fidelity of a complex64 result
// against a complex128 one.
template <class T>
__device__ __forceinline__ void amp_df2(T a, dfl& re, dfl& im);
template <>
__device__ __forceinline__ void amp_df2<double2>(double2 a, dfl& re, dfl& im) {
  re = df_from_double(a.x);
  im = df_from_double(a.y);
}
template <>
__device__ __forceinline__ void amp_df2<float2>(float2 a, dfl& re, dfl& im) {
  re = dfl{a.x, 0.f};
  im = dfl{a.y, 0.f};
}

template <class TA, class TB>
__global__ void __launch_bounds__(256) k_inner(const TA* __restrict__ a, const TB* __restrict__ b, uint64_t N,
                                               double* __restrict__ partial) {
  __shared__ dfl wr[8], wi[8];
  dfl sr{0.f, 0.f}, si{0.f, 0.f};
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += step) {
    dfl ar, ai, br, bi;
    amp_df2<TA>(a[i], ar, ai);
    amp_df2<TB>(b[i], br, bi);
    sr = df_add(sr, df_dot2(ar, br, ai, bi));           // re(conj(a) b) = ar br + ai bi
    si = df_add(si, df_dot2(ar, bi, df_neg(ai), br));   // im(conj(a) b) = ar bi - ai br
  }
  for (int off = 16; off > 0; off >>= 1) {
    sr = df_shfl_add(sr, off);
    si = df_shfl_add(si, off);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    wr[warp] = sr;
    wi[warp] = si;
  }
  __syncthreads();
  if (warp == 0) {
    sr = lane < (int)(blockDim.x >> 5) ? wr[lane] : dfl{0.f, 0.f};
    si = lane < (int)(blockDim.x >> 5) ? wi[lane] : dfl{0.f, 0.f};
    for (int off = 16; off > 0; off >>= 1) {
      sr = df_shfl_add(sr, off);
      si = df_shfl_add(si, off);
    }
    if (lane == 0) {
      partial[4 * blockIdx.x] = (double)sr.hi;
      partial[4 * blockIdx.x + 1] = (double)sr.lo;
      partial[4 * blockIdx.x + 2] = (double)si.hi;
      partial[4 * blockIdx.x + 3] = (double)si.lo;
    }
  }
}

void inner_product(State& a, State& b, double* re, double* im) {
  if (a.n != b.n) fail(BF_EINVAL, "inner product of states with %d and %d qubits", a.n, b.n);
  unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((a.N + 255) / 256, (uint64_t)a.num_sms * 8));
  ensure_partials(a, 2 * (size_t)blocks);
  // b's pending work must finish before a's stream reads it
  cudaEvent_t ev;
  BF_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  BF_CUDA(cudaEventRecord(ev, b.stream));
  BF_CUDA(cudaStreamWaitEvent(a.stream, ev, 0));
  BF_CUDA(cudaEventDestroy(ev));
  const bool a128 = a.dtype == BF_C128, b128 = b.dtype == BF_C128;
  if (a128 && b128)
    k_inner<double2, double2><<<blocks, 256, 0, a.stream>>>(static_cast<const double2*>(a.amp),
                                                            static_cast<const double2*>(b.amp), a.N, a.d_partial);
  else if (a128)
    k_inner<double2, float2><<<blocks, 256, 0, a.stream>>>(static_cast<const double2*>(a.amp),
                                                           static_cast<const float2*>(b.amp), a.N, a.d_partial);
  else if (b128)
    k_inner<float2, double2><<<blocks, 256, 0, a.stream>>>(static_cast<const float2*>(a.amp),
                                                           static_cast<const double2*>(b.amp), a.N, a.d_partial);
  else
    k_inner<float2, float2><<<blocks, 256, 0, a.stream>>>(static_cast<const float2*>(a.amp),
                                                          static_cast<const float2*>(b.amp), a.N, a.d_partial);
  BF_CUDA(cudaGetLastError());
  a.launches++;
  BF_CUDA(cudaMemcpyAsync(a.h_partial, a.d_partial, 4 * (size_t)blocks * sizeof(double), cudaMemcpyDeviceToHost,
                          a.stream));
  sync_state(a);
  double r = 0, i = 0;
  for (unsigned k = 0; k < blocks; ++k) {
    r += a.h_partial[4 * k] + a.h_partial[4 * k + 1];
    i += a.h_partial[4 * k + 2] + a.h_partial[4 * k + 3];
  }
  *re = r;
  *im = i;
}

// ---- renormalisation (complex64 states) -------------------------------------
// FP32 gate matrices are unitary only to ~6e-8 and that error changes the
// norm coherently at every gate, so the complex64 form restores the norm
// the state had before the circuit: sum |amp|^2 in double-float before and
// after (k_norm2 partials), one thread forms sqrt(before / after) in FP64 and
// stores it as an FP32 (hi, lo) pair, and every amplitude is multiplied by
// hi + lo (x*hi + x*lo with one FMA: unbiased).  All stream-ordered.
__device__ __forceinline__ double sum_partials(const double* __restrict__ partial, int blocks) {
  __shared__ double sh[256];
  double acc = 0;
  for (int b = threadIdx.x; b < blocks; b += blockDim.x) acc += partial[2 * b] + partial[2 * b + 1];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

// before == nullptr: the norm before the circuit is 1
__global__ void k_norm_factor(const double* __restrict__ before, const double* __restrict__ after, int blocks,
                              float* __restrict__ factor) {
  double b = before ? sum_partials(before, blocks) : 1.0;
  double a = sum_partials(after, blocks);
  if (threadIdx.x == 0) {
    double f = (a > 0 && b > 0) ? sqrt(b / a) : 1.0;
    float hi = (float)f;
    factor[0] = hi;
    factor[1] = (float)(f - (double)hi);
  }
}

__global__ void __launch_bounds__(256) k_scale_c64(float2* __restrict__ s, uint64_t N, const float* __restrict__ factor) {
  const float hi = factor[0], lo = factor[1];
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += step) {
    float2 v = s[i];
    v.x = fmaf(v.x, hi, v.x * lo);
    v.y = fmaf(v.y, hi, v.y * lo);
    s[i] = v;
  }
}

static unsigned renorm_blocks(const State& st) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((st.N + 255) / 256, (uint64_t)st.num_sms * 8));
}

// The state's own buffer (not the shared reduction partials, which the
// circuit's diffusers and measurements reuse in between):
// [before: 2*blocks][after: 2*blocks][factor]
static void ensure_renorm(State& st, unsigned blocks) {
  size_t need = 4 * (size_t)blocks + 2;
  if (st.renorm_cap >= need) return;
  dev_free(st, st.d_renorm);
  st.d_renorm = nullptr;
  st.renorm_cap = 0;
  st.d_renorm = static_cast<double*>(dev_alloc(st, need * sizeof(double)));
  st.renorm_cap = need;
}

// sum |amp|^2 partials (hi, lo per CTA) into st.d_partial, stream-ordered
void launch_norm2_partials(State& st, unsigned blocks) {
  if (st.dtype == BF_C128)
    k_norm2<double2><<<blocks, 256, 0, st.stream>>>(static_cast<const double2*>(st.amp), st.N, st.d_partial);
  else
    k_norm2<float2><<<blocks, 256, 0, st.stream>>>(static_cast<const float2*>(st.amp), st.N, st.d_partial);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_norm_before(State& st) {
  if (st.dtype != BF_C64) return;
  unsigned blocks = renorm_blocks(st);
  ensure_renorm(st, blocks);
  k_norm2<float2><<<blocks, 256, 0, st.stream>>>(static_cast<const float2*>(st.amp), st.N, st.d_renorm);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_renormalize(State& st, bool unit_before) {
  if (st.dtype != BF_C64) fail(BF_EUNSUPPORTED, "renormalisation is for complex64 states");
  unsigned blocks = renorm_blocks(st);
  ensure_renorm(st, blocks);
  double* before = st.d_renorm;
  double* after = st.d_renorm + 2 * blocks;
  float* factor = reinterpret_cast<float*>(st.d_renorm + 4 * blocks);
  k_norm2<float2><<<blocks, 256, 0, st.stream>>>(static_cast<const float2*>(st.amp), st.N, after);
  k_norm_factor<<<1, 256, 0, st.stream>>>(unit_before ? nullptr : before, after, (int)blocks, factor);
  k_scale_c64<<<grid_for(st, st.N), 256, 0, st.stream>>>(static_cast<float2*>(st.amp), st.N, factor);
  BF_CUDA(cudaGetLastError());
  st.launches += 3;
}

// ---- dense m-qubit unitary on contiguous qubits [t, t+m) ------------------
// apply_unitary / apply_controlled_unitary (transformations_unitary.mojo:
// 22-139): groups of 2^m amplitudes base + (k << t); out[row] =
// sum_col u[row*dim + col] * in[col].  For m >= 4 a CTA of 256 threads
// holds G = 256 / dim groups in shared memory and thread (g, row) forms one
// output; smaller unitaries run in registers (k_unitary_reg).
constexpr int kUniThreads = 256;
constexpr int kUniMaxM = 6;

struct UniArgs {
  uint64_t groups;    // number of groups to process
  int32_t t, m, dim, G;
  uint64_t cbit;      // control bit (0 = uncontrolled)
  int32_t nfix;
  int8_t fix[8];      // inserted-zero positions, ascending
};

template <class P>
__global__ void __launch_bounds__(kUniThreads) k_unitary(typename P::Glob* __restrict__ s,
                                                         const double* __restrict__ u, const UniArgs a) {
  using R = typename P::R;
  using Sm = typename P::Smem;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Sm* mat = reinterpret_cast<Sm*>(smem_raw);                       // dim*dim
  Sm* xin = mat + (size_t)a.dim * a.dim;                             // G*dim
  const int dim = a.dim, G = a.G, tid = threadIdx.x;
  for (int e = tid; e < dim * dim; e += kUniThreads) {
    typename P::Glob gv;
    if constexpr (sizeof(typename P::Glob) == 16) gv = make_double2(u[2 * e], u[2 * e + 1]);
    else gv = make_float2((float)u[2 * e], (float)u[2 * e + 1]);
    mat[e] = P::to_smem(P::from_glob(gv));
  }
  const bool t0 = (a.t == 0);
  for (uint64_t gbase = (uint64_t)blockIdx.x * G; gbase < a.groups; gbase += (uint64_t)gridDim.x * G) {
    __syncthreads();
    // load: consecutive threads walk the contiguous direction
    {
      int g = t0 ? tid / dim : tid % G;
      int c = t0 ? tid % dim : tid / G;
      uint64_t gi = gbase + g;
      if (gi < a.groups) {
        uint64_t x = gi;
        for (int i = 0; i < a.nfix; ++i) x = insert_zero_bit(x, a.fix[i]);
        x |= a.cbit;
        xin[g * dim + c] = P::to_smem(P::from_glob(s[x | ((uint64_t)c << a.t)]));
      }
    }
    __syncthreads();
    int g = tid / dim, row = tid % dim;
    uint64_t gi = gbase + g;
    R acc;
    if (gi < a.groups) {
      acc = P::zero();
      for (int c = 0; c < dim; ++c)
        acc = P::fma(P::from_smem(mat[row * dim + c]), P::from_smem(xin[g * dim + c]), acc);
    }
    __syncthreads();
    if (gi < a.groups) xin[g * dim + row] = P::to_smem(acc);
    __syncthreads();
    {
      int g2 = t0 ? tid / dim : tid % G;
      int c2 = t0 ? tid % dim : tid / G;
      uint64_t gj = gbase + g2;
      if (gj < a.groups) {
        uint64_t x = gj;
        for (int i = 0; i < a.nfix; ++i) x = insert_zero_bit(x, a.fix[i]);
        x |= a.cbit;
        s[x | ((uint64_t)c2 << a.t)] = P::to_glob(P::from_smem(xin[g2 * dim + c2]));
      }
    }
  }
}

// m <= 3: each thread holds whole groups of 2^m amplitudes in registers
// (all loads issued before the matrix-vector product), the matrix staged in
// shared memory; consecutive threads take consecutive groups, so for a
// target block above the low 5 qubits every load and store instruction of
// a warp is one contiguous run.
template <class P, int M>
__global__ void __launch_bounds__(kUniThreads) k_unitary_reg(typename P::Glob* __restrict__ s,
                                                             const double* __restrict__ u, const UniArgs a) {
  using R = typename P::R;
  using Sm = typename P::Smem;
  constexpr int D = 1 << M;
  __shared__ Sm mat[D * D];
  for (int e = threadIdx.x; e < D * D; e += kUniThreads) {
    typename P::Glob gv;
    if constexpr (sizeof(typename P::Glob) == 16) gv = make_double2(u[2 * e], u[2 * e + 1]);
    else gv = make_float2((float)u[2 * e], (float)u[2 * e + 1]);
    mat[e] = P::to_smem(P::from_glob(gv));
  }
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * kUniThreads;
  for (uint64_t gi = (uint64_t)blockIdx.x * kUniThreads + threadIdx.x; gi < a.groups; gi += stride) {
    uint64_t x = gi;
#pragma unroll
    for (int i = 0; i < M + 1; ++i)  // the targets and at most one control
      if (i < a.nfix) x = insert_zero_bit(x, a.fix[i]);
    x |= a.cbit;
    R v[D];
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = P::from_glob(s[x | ((uint64_t)c << a.t)]);
    // one output row at a time keeps the register count near the group's
#pragma unroll 1
    for (int r = 0; r < D; ++r) {
      R acc = P::zero();
#pragma unroll
      for (int c = 0; c < D; ++c) acc = P::fma(P::from_smem(mat[r * D + c]), v[c], acc);
      s[x | ((uint64_t)r << a.t)] = P::to_glob(acc);
    }
  }
}

template <class P>
static void launch_unitary_p(State& st, const double* h_u, int t, int m, int control) {
  int dim = 1 << m;
  UniArgs a;
  a.t = t;
  a.m = m;
  a.dim = dim;
  a.G = kUniThreads / dim;
  a.cbit = control >= 0 ? (1ull << control) : 0ull;
  std::vector<int> pos;
  for (int k = 0; k < m; ++k) pos.push_back(t + k);
  if (control >= 0) pos.push_back(control);
  std::sort(pos.begin(), pos.end());
  a.nfix = (int)pos.size();
  for (int i = 0; i < a.nfix; ++i) a.fix[i] = (int8_t)pos[i];
  a.groups = st.N >> a.nfix;
  if (a.groups == 0) return;
  size_t mbytes = (size_t)dim * dim * 2 * sizeof(double);
  if (!st.d_umat) {
    if (cudaMalloc(&st.d_umat, (size_t)64 * 64 * 2 * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      st.d_umat = nullptr;
      fail(BF_ENOMEM, "cannot allocate the unitary matrix buffer");
    }
  }
  double* d_u = st.d_umat;
  BF_CUDA(cudaMemcpyAsync(d_u, h_u, mbytes, cudaMemcpyHostToDevice, st.stream));
  if (m <= 3) {
    const uint64_t ctas = std::min<uint64_t>((a.groups + kUniThreads - 1) / kUniThreads, (uint64_t)st.num_sms * 8);
    typename P::Glob* amp = static_cast<typename P::Glob*>(st.amp);
    if (m == 1) k_unitary_reg<P, 1><<<(unsigned)ctas, kUniThreads, 0, st.stream>>>(amp, d_u, a);
    else if (m == 2) k_unitary_reg<P, 2><<<(unsigned)ctas, kUniThreads, 0, st.stream>>>(amp, d_u, a);
    else k_unitary_reg<P, 3><<<(unsigned)ctas, kUniThreads, 0, st.stream>>>(amp, d_u, a);
    BF_CUDA(cudaGetLastError());
    st.launches++;
    return;
  }
  size_t smem = ((size_t)dim * dim + kUniThreads) * sizeof(typename P::Smem);
  static PerDeviceOnce configured;  // one per instantiation of P
  configured.run(st.device, [] {
    BF_CUDA(cudaFuncSetAttribute(k_unitary<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(((size_t)64 * 64 + kUniThreads) * sizeof(typename P::Smem))));
  });
  uint64_t ctas = std::min<uint64_t>((a.groups + a.G - 1) / a.G, (uint64_t)st.num_sms * 8);
  k_unitary<P><<<(unsigned)ctas, kUniThreads, smem, st.stream>>>(static_cast<typename P::Glob*>(st.amp), d_u, a);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_unitary(State& st, const double* h_u, int t, int m, int control) {
  if (m < 1 || m > kUniMaxM) fail(BF_EUNSUPPORTED, "dense unitary on %d qubits (supported: 1..%d)", m, kUniMaxM);
  switch (st.prec) {
    case PREC_F64: launch_unitary_p<PolF64>(st, h_u, t, m, control); break;
    case PREC_DF: launch_unitary_p<PolDF>(st, h_u, t, m, control); break;
    default: launch_unitary_p<PolF32>(st, h_u, t, m, control); break;
  }
}

}  // namespace bf

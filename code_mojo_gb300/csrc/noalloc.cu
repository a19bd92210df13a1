// noalloc.cu — sum |amp|^2 for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: code running while a CUDA stream is
// being captured into a graph (allocation is illegal there), plugins that
// live inside a host framework whose allocator owns every device byte, and
// real-time paths where cudaMalloc's implicit device synchronisation is not
// acceptable.  bf_norm2_noalloc serves them: the caller passes the
// amplitudes and the output slot (both device pointers) and a stream, and
// the per-block partial sums live in a fixed array in this file,
// g_norm2_scratch, instead of memory allocated per call.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds its 512 KiB until the process exits.  It bounds the input at
// kNoAllocMaxAmps amplitudes (2^31).  All calls on a device share it and it
// keeps the last call's contents; a call writes every partial it later reads,
// so nothing needs clearing first.  Calls whose kernels overlap on the GPU
// (on different streams, or from different threads without ordering) race on
// the array and may return wrong sums: serialise them.
//
// Range: the sum is accumulated in double-float, whose exponent range is
// FP32's.  Components of magnitude below about 1.1e-19 add nothing (their
// squares flush to zero: at most 2^31 x 1.2e-38 in all), and a component of
// magnitude 1.8e19 or more overflows the sum.  Normalised states are far
// inside that range.
#include <mutex>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

constexpr int kNoAllocThreads = 256;
constexpr uint64_t kNoAllocAmpsPerBlock = 1ull << 16;        // 256 per thread
constexpr int kNoAllocMaxBlocks = 1 << 15;                   // partials held
constexpr uint64_t kNoAllocMaxAmps = kNoAllocAmpsPerBlock * kNoAllocMaxBlocks;  // 2^31

// (hi, lo) pair per block: 2^16 doubles = 512 KiB.
static __device__ __align__(256) double g_norm2_scratch[2 * kNoAllocMaxBlocks];

__device__ __forceinline__ dfl na_shfl_add(dfl v, int off) {
  dfl o;
  o.hi = __shfl_down_sync(0xffffffffu, v.hi, off);
  o.lo = __shfl_down_sync(0xffffffffu, v.lo, off);
  return df_add(v, o);
}

__device__ __forceinline__ dfl na_block_sum(dfl acc) {
  __shared__ dfl wsum[kNoAllocThreads / 32];
  for (int off = 16; off > 0; off >>= 1) acc = na_shfl_add(acc, off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wsum[warp] = acc;
  __syncthreads();
  acc = dfl{0.f, 0.f};
  if (warp == 0) {
    acc = lane < kNoAllocThreads / 32 ? wsum[lane] : dfl{0.f, 0.f};
    for (int off = 16; off > 0; off >>= 1) acc = na_shfl_add(acc, off);
  }
  return acc;  // valid in thread 0
}

// Block b reduces amplitudes [b * 2^16, (b+1) * 2^16) and stores its
// double-float partial in scratch[2b], scratch[2b+1].
template <class T>
__global__ void __launch_bounds__(kNoAllocThreads) k_norm2_chunks(const T* __restrict__ s, uint64_t n,
                                                                  double* __restrict__ scratch) {
  const uint64_t begin = (uint64_t)blockIdx.x * kNoAllocAmpsPerBlock;
  const uint64_t end = min(begin + kNoAllocAmpsPerBlock, n);
  dfl acc{0.f, 0.f};
  for (uint64_t i = begin + threadIdx.x; i < end; i += kNoAllocThreads) {
    T a = s[i];
    dfl re, im;
    if constexpr (sizeof(T) == 16) {
      re = df_from_double(((const double2&)a).x);
      im = df_from_double(((const double2&)a).y);
    } else {
      re = dfl{((const float2&)a).x, 0.f};
      im = dfl{((const float2&)a).y, 0.f};
    }
    acc = df_add(acc, df_dot2(re, re, im, im));
  }
  acc = na_block_sum(acc);
  if (threadIdx.x == 0) {
    scratch[2 * blockIdx.x] = (double)acc.hi;
    scratch[2 * blockIdx.x + 1] = (double)acc.lo;
  }
}

// One block sums the `blocks` partials and writes the FP64 result.
__global__ void __launch_bounds__(kNoAllocThreads) k_norm2_finish(const double* __restrict__ scratch, int blocks,
                                                                  double* __restrict__ out) {
  dfl acc{0.f, 0.f};
  for (int b = threadIdx.x; b < blocks; b += kNoAllocThreads) {
    acc = df_add(acc, df_from_double(scratch[2 * b]));
    acc = df_add(acc, df_from_double(scratch[2 * b + 1]));
  }
  acc = na_block_sum(acc);
  if (threadIdx.x == 0) *out = df_to_double(acc);
}

// Device address of g_norm2_scratch, resolved once per device with that
// device current.  The host-side name g_norm2_scratch is only a stand-in for
// the symbol and must never be passed to a kernel.  The table is never
// cleared: after cudaDeviceReset (or any teardown of the device's primary
// context) the cached address is stale, so a process that resets a device
// must not call bf_norm2_noalloc on it again.
static void* noalloc_scratch_for_current_device() {
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  int dev = 0;
  BF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) fail(BF_EUNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_norm2_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fail(BF_ECUDA, "cudaGetSymbolAddress(g_norm2_scratch) failed on device %d: %s", dev, cudaGetErrorString(e));
    }
    addr[dev] = p;
  }
  return addr[dev];
}

void norm2_noalloc(const void* d_amps, uint64_t num_amps, int32_t dtype, double* d_out, cudaStream_t stream) {
  if (!d_amps || !d_out) fail(BF_EINVAL, "bf_norm2_noalloc: null device pointer");
  if (dtype != BF_C128 && dtype != BF_C64) fail(BF_EINVAL, "bf_norm2_noalloc: unknown dtype %d", dtype);
  if (num_amps == 0) fail(BF_EINVAL, "bf_norm2_noalloc: no amplitudes");
  // The kernels read whole double2 (16 B) or float2 (8 B) amplitudes and
  // write one double; a misaligned pointer would fault on the device and
  // poison the caller's context, so it is refused here, before any launch.
  const uintptr_t amp_align = dtype == BF_C128 ? 16u : 8u;
  if (reinterpret_cast<uintptr_t>(d_amps) % amp_align != 0)
    fail(BF_EINVAL, "bf_norm2_noalloc: d_amps must be %u-byte aligned for this dtype", (unsigned)amp_align);
  if (reinterpret_cast<uintptr_t>(d_out) % 8u != 0) fail(BF_EINVAL, "bf_norm2_noalloc: d_out must be 8-byte aligned");
  if (num_amps > kNoAllocMaxAmps)
    fail(BF_EINVAL,
         "bf_norm2_noalloc: %llu amplitudes exceed the maximum of %llu (2^31) set by its static scratch; "
         "use bf_norm2 on a bf_state",
         (unsigned long long)num_amps, (unsigned long long)kNoAllocMaxAmps);
  double* scratch = static_cast<double*>(noalloc_scratch_for_current_device());
  const int blocks = (int)((num_amps + kNoAllocAmpsPerBlock - 1) / kNoAllocAmpsPerBlock);
  if (dtype == BF_C128)
    k_norm2_chunks<double2><<<blocks, kNoAllocThreads, 0, stream>>>(static_cast<const double2*>(d_amps), num_amps,
                                                                     scratch);
  else
    k_norm2_chunks<float2><<<blocks, kNoAllocThreads, 0, stream>>>(static_cast<const float2*>(d_amps), num_amps,
                                                                    scratch);
  BF_CUDA(cudaGetLastError());
  k_norm2_finish<<<1, kNoAllocThreads, 0, stream>>>(scratch, blocks, d_out);
  BF_CUDA(cudaGetLastError());
}

}  // namespace bf

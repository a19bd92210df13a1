// tblock.cu — complex64 tile passes whose gates are fused into 5-qubit
// blocks (32x32 complex unitaries) applied on the tensor cores.
//
// The reference fuses neighbouring gates into dense 2^m x 2^m unitaries and
// applies them by gather -> matrix-vector -> scatter
// (transformations_fusion.mojo:539-876, transformations_unitary.mojo:22-75).
// Here a CTA holds a 12-qubit tile (4096 amplitudes) and applies a sequence
// of 5-qubit blocks whose qubits are all tile qubits.  For one block the tile
// is a 128 x 32 complex matrix X (rows: the 7 other tile qubits; columns:
// the block's 5 qubits) and the block is X <- X U^T, i.e. as a real GEMM
//   D[128 x 64] = A[128 x 64] * R[64 x 64],   A = X with (re, im) interleaved,
// R[2l+c][2j+d] built from U[j][l].  It runs as tcgen05.mma kind::tf32
// (M=128, N=64, K=8 per instruction) with FP32 accumulation in tensor
// memory, in 3xTF32 form: A = Ab + As and R = Rb + Rs with Ab, Rb rounded
// to TF32 and As, Rs the remainders, D = As*Rb + Ab*Rs + Ab*Rb (the As*Rs
// term is below FP32 resolution).  Relative error per block is about 2^-21,
// against 2^-11 for plain TF32.
//
// Per tile: coalesced 16-byte loads -> split into the two A operands in
// shared memory (K-major, 128-byte swizzle) -> per block: one thread issues
// 24 MMAs and commits them to an mbarrier, the epilogue reads D from tensor
// memory (tcgen05.ld 32x32b), and writes it either as the next block's A
// operands (a bit permutation of the tile index) or, after the last block,
// straight to the state.  Where each
// thread's 8 results go is a per-block table computed by the planner (one
// 16-byte load per thread per block), which also orders each block's rows so
// that a warp's operand stores spread over the swizzled 16-byte chunks.  The block
// matrices (pre-split and pre-swizzled on the host, 32 KiB each) stream in
// with cp.async.bulk behind the MMAs of the previous block.  Gates with
// controls (or diagonal targets) outside the tile select one of up to 8
// precomputed variants of their block's matrix from the CTA's fixed
// outside bits.
//
// Every wait is bounded: on expiry the CTA sets the state's error flag,
// waits (bounded) for its own copy in flight, frees its tensor memory and
// returns.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

constexpr int kBlkThreads = kBlockThreads;
constexpr int kColGroups = kBlkThreads / 128;      // warps sharing one 32-lane group of D
constexpr int kColsPerWarp = 64 / kColGroups;      // FP32 columns of D per warp
constexpr int kCplxPerThread = kColsPerWarp / 2;   // complex results per thread per block
constexpr int kLoadIters = 4096 / (2 * kBlkThreads);  // 16-byte loads per thread per tile
constexpr uint32_t kAOpBytes = 128 * 64 * 4;  // 32 KiB: 128 rows x 64 FP32
constexpr uint32_t kSmemA0 = 0;               // Ab
constexpr uint32_t kSmemA1 = kAOpBytes;       // As
constexpr uint32_t kSmemB = 2 * kAOpBytes;    // Rb (2 x 8 KiB), Rs (2 x 8 KiB)
constexpr uint32_t kSmemHoff = kSmemB + kBlockImageBytes;
constexpr uint32_t kSmemBar = kSmemHoff + 128 * 8;
constexpr uint32_t kSmemBlk = kSmemBar + 32;   // the pass's block descriptors
constexpr uint32_t kSmemUsed = kSmemBlk + kMaxPassBlocks * sizeof(Blk5);
constexpr uint32_t kSmemAlloc = kSmemUsed + 1024;  // slack for 1024-byte alignment
constexpr uint32_t kTmemCols = 64;

struct BlkPassArgs {
  float2* s;
  const Blk5* blocks;
  const unsigned char* images;  // kBlockImageBytes per image, 16-byte aligned
  uint64_t ntiles;
  int32_t nblocks;
  int32_t q[kBlockTileQubits];  // tile qubits; q[j] = j for j < 5
  const uint16_t* offsets;      // destination tables (kBlkThreads x 8 per table)
  int* flag;
  uint32_t spin_limit;
};

// ---- PTX wrappers ------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for the phase with parity `parity`; false when it expired
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 64) __nanosleep(32);
  }
  return false;
}

// one 32 KiB block image: global -> shared, completing on `bar`
__device__ __forceinline__ void load_image(uint32_t dst, const void* src, uint32_t bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kBlockImageBytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(kBlockImageBytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor (tcgen05): K-major operand with the
// 128-byte swizzle; 8-row core-matrix groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 lanes x 16 consecutive FP32 columns: thread `lane` of the warp gets
// row (32 * (warp % 4) + lane), columns col..col+15
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- operand layout ----------------------------------------------------------
// TF32 rounding to nearest (ties away from zero) of an FP32 value: the tensor
// cores read the top 19 bits of each operand.
__device__ __forceinline__ float tf32_round(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// The low part is the exact remainder x - tf32(x); the tensor cores read its
// top 19 bits (|error| <= 2^-21 |x|, no bias: the remainder takes either sign).
__device__ __forceinline__ void put_split(unsigned char* sm, uint32_t off, float re, float im) {
  const float rb = tf32_round(re), ib = tf32_round(im);
  *reinterpret_cast<float2*>(sm + kSmemA0 + off) = make_float2(rb, ib);
  *reinterpret_cast<float2*>(sm + kSmemA1 + off) = make_float2(re - rb, im - ib);
}

// this thread's 8 destinations in a table: operand byte offset / 8, or after
// the last block the tile element
__device__ __forceinline__ uint4 my_dests(const uint16_t* offsets, uint32_t table) {
  return __ldg(reinterpret_cast<const uint4*>(offsets + (size_t)table * kBlockTableEntries + threadIdx.x * 8));
}

__device__ __forceinline__ uint32_t dest_at(const uint4& d, int e) {
  const uint32_t w = e < 2 ? d.x : (e < 4 ? d.y : (e < 6 ? d.z : d.w));
  return (e & 1) ? (w >> 16) : (w & 0xFFFFu);
}

__device__ __forceinline__ uint32_t variant_of(const Blk5& b, uint64_t obase) {
  uint32_t v = 0;
  for (int k = 0; k < b.nout; ++k) v |= (uint32_t)((obase >> b.outpos[k]) & 1ull) << k;
  return v;
}

__global__ void __launch_bounds__(kBlkThreads, 2) k_tblock(const BlkPassArgs a) {
  extern __shared__ unsigned char smem_raw[];
  // 1024-byte alignment for the swizzled operands
  unsigned char* sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* hoff = reinterpret_cast<uint64_t*>(sm + kSmemHoff);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kSmemBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kSmemBar + 16);
  int* ok_slot = reinterpret_cast<int*>(sm + kSmemBar + 20);
  Blk5* blk = reinterpret_cast<Blk5*>(sm + kSmemBlk);
  const uint32_t bar_b = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]);
  const int tid = threadIdx.x, warp = tid >> 5;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
    mbar_init(bar_b, 1);
    mbar_init(bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int h = tid; h < 128; h += kBlkThreads) {  // local bits 5..11 -> global offsets
    uint64_t off = 0;
    for (int j = 0; j < 7; ++j)
      if ((h >> j) & 1) off |= 1ull << a.q[5 + j];
    hoff[h] = off;
  }
  if (tid < a.nblocks * (int)(sizeof(Blk5) / 16))
    reinterpret_cast<uint4*>(blk)[tid] = __ldg(reinterpret_cast<const uint4*>(a.blocks) + tid);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // this warp's rows and columns of D
  const uint32_t colh = (uint32_t)(warp >> 2);  // columns kColsPerWarp*colh ..
  const uint32_t taddr = tmem + ((32u * (warp & 3)) << 16) + (uint32_t)kColsPerWarp * colh;
  static_assert(kColsPerWarp == 16, "the epilogue reads 16 columns per warp");

  // instruction descriptor: D FP32, A and B TF32, both K-major, N = 64, M = 128
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
  const uint32_t sA0 = smem_u32(sm + kSmemA0), sA1 = smem_u32(sm + kSmemA1), sB = smem_u32(sm + kSmemB);

  uint32_t ph_b = 0, ph_mma = 0;
  bool b_in_flight = false;     // thread 0: an image copy has not been waited for
  int mma_lost_phase = -1;      // thread 0: MMAs whose completion wait expired
  bool failed = false;

  auto tile_base = [&](uint64_t tile) {
    uint64_t ob = tile;
    for (int j = 0; j < kBlockTileQubits; ++j) ob = insert_zero_bit(ob, a.q[j]);
    return ob;
  };

  // tile bases step by masked addition (base(t + g) = ((base(t) | ~free) + base(g)) & free)
  uint64_t tpos = 0;
  for (int j = 0; j < kBlockTileQubits; ++j) tpos |= 1ull << a.q[j];
  const uint64_t free_pos = ((a.ntiles << kBlockTileQubits) - 1) & ~tpos;
  const uint64_t grid_base = tile_base(gridDim.x);
  auto step_base = [&](uint64_t b) { return ((b | ~free_pos) + grid_base) & free_pos; };
  uint64_t tile = blockIdx.x;
  uint64_t obase = tile_base(tile);
  if (tid == 0 && tile < a.ntiles) {
    const Blk5& b0 = blk[0];
    load_image(sB, a.images + (size_t)(b0.img + variant_of(b0, obase)) * kBlockImageBytes, bar_b);
    b_in_flight = true;
  }

  static_assert(kLoadIters * 2 == kBlockThreadElems, "one destination table entry per loaded amplitude");
  const uint4 load_dest = my_dests(a.offsets, blk[0].load_offs);
  for (; tile < a.ntiles && !failed; tile += gridDim.x, obase = step_base(obase)) {
    // load: 16 bytes at a time, split into the block-0 operands
    float4 v[kLoadIters];
#pragma unroll
    for (int it = 0; it < kLoadIters; ++it) {
      const uint32_t i0 = (uint32_t)(it * kBlkThreads + tid) * 2u;
      v[it] = __ldcs(reinterpret_cast<const float4*>(a.s + (obase | (i0 & 31u) | hoff[i0 >> 5])));
    }
#pragma unroll
    for (int it = 0; it < kLoadIters; ++it) {
      put_split(sm, dest_at(load_dest, 2 * it) << 3, v[it].x, v[it].y);
      put_split(sm, dest_at(load_dest, 2 * it + 1) << 3, v[it].z, v[it].w);
    }
    fence_proxy_async();
    __syncthreads();

    for (int bi = 0; bi < a.nblocks; ++bi) {
      const bool more = bi + 1 < a.nblocks;
      const uint4 dest = my_dests(a.offsets, blk[bi].offs);
      if (tid == 0) {
        int ok = mbar_wait(bar_b, ph_b, a.spin_limit) ? 1 : 0;
        if (ok) {
          b_in_flight = false;
          tc_fence_after();
          uint32_t acc = 0;
          // small products first: As*Rb, Ab*Rs, then Ab*Rb
#pragma unroll
          for (int pass = 0; pass < 3; ++pass) {
            const uint32_t abase = pass == 0 ? sA1 : sA0;
            const uint32_t bbase = pass == 1 ? sB + 16384u : sB;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
              const uint64_t ad = sdesc(abase + (uint32_t)(s >> 2) * 16384u + (uint32_t)(s & 3) * 32u);
              const uint64_t bd = sdesc(bbase + (uint32_t)(s >> 2) * 8192u + (uint32_t)(s & 3) * 32u);
              mma_tf32(tmem, ad, bd, idesc, acc);
              acc = 1;
            }
          }
          mma_commit(bar_mma);
          // the next image's address while the MMAs run
          const unsigned char* next_img = nullptr;
          if (more) {
            next_img = a.images + (size_t)(blk[bi + 1].img + variant_of(blk[bi + 1], obase)) * kBlockImageBytes;
          } else if (tile + gridDim.x < a.ntiles) {
            next_img = a.images + (size_t)(blk[0].img + variant_of(blk[0], step_base(obase))) * kBlockImageBytes;
          }
          ok = mbar_wait(bar_mma, ph_mma, a.spin_limit) ? 1 : 0;
          if (!ok) mma_lost_phase = (int)ph_mma;
          // the B buffer is free once the MMAs are done: fetch the next image
          if (ok && next_img) {
            load_image(sB, next_img, bar_b);
            b_in_flight = true;
          }
        }
        if (!ok) atomicExch(a.flag, 1);
        *ok_slot = ok;
      }
      ph_b ^= 1u;
      ph_mma ^= 1u;
      __syncthreads();
      if (!*ok_slot) {
        failed = true;
        break;
      }
      tc_fence_after();
      float d[kColsPerWarp];
      tmem_ld16(taddr, d);
      if (more) {
#pragma unroll
        for (int c = 0; c < kCplxPerThread; ++c) put_split(sm, dest_at(dest, c) << 3, d[2 * c], d[2 * c + 1]);
        fence_proxy_async();
      } else {
        // the results straight to the state (the table gives their tile
        // elements): the 30-qubit circuit took 397 ms this way, 402 ms with
        // the tile staged in shared memory for 16-byte stores
#pragma unroll
        for (int c = 0; c < kCplxPerThread; ++c) {
          const uint32_t ie = dest_at(dest, c);
          __stcs(a.s + (obase | (ie & 31u) | hoff[ie >> 5]), make_float2(d[2 * c], d[2 * c + 1]));
        }
      }
      tc_fence_before();
      __syncthreads();
    }
    if (failed) break;
  }

  // nothing of ours may be in flight when the tensor memory is freed
  if (tid == 0) {
    if (b_in_flight && !mbar_wait(bar_b, ph_b, a.spin_limit)) atomicExch(a.flag, 1);
    if (mma_lost_phase >= 0 && !mbar_wait(bar_mma, (uint32_t)mma_lost_phase, a.spin_limit)) atomicExch(a.flag, 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ---- complex128: digit blocks on the bf16 tensor cores -----------------------
// A complex128 value x becomes D signed base-256 digits, x / s = 2^-8 sum_i
// d_i 2^-8(i + 6 - D) (i < D) with d_i integers of at most 8 bits plus sign,
// each exact in bf16; the matrix likewise as six digits (r = 2^-8 sum_j e_j
// 2^-8j).  For every digit level s = i + j <= D the 4 MMAs of each kept pair
// (i, j) (kind::f16, bf16 inputs, K = 16) accumulate sum_K d_i e_j into one
// FP32 accumulator; every product and partial sum is an integer below 2^24,
// so the accumulation is exact whatever the order.  The epilogue turns the
// D + 1 level sums back into the next block's digits by carries between
// levels (FP32 on exact integers), or after the last block into the FP64
// result.
//
// The state is a fixed-point number: one scale s = 2^e (s >= 2 ||state||,
// from the norm before the first digit pass) and the unit 2^-48 s, so every
// amplitude of a unitary circuit is an integer V of that unit with |V| <
// 2^47 (six digits).  A block pass mixes amplitudes only within a tile, so
// a tile's norm is the same after every block; when it is below 2^-9 s,
// every value of the tile stays below 2^39 units through the pass and the
// top digit is zero: the tile runs in D = 5 digits (20 digit pairs instead
// of 26) with the same unit, so the five- and six-digit forms hold the same
// integers and give the same bits.  The norm test is an exact integer bound
// per warp (sq_bound_units), decided at the barrier that follows the
// conversion: a tile that fails it is converted again in six digits.  On
// the 30-qubit circuit a tile holds about 2^-9 of the norm, so nearly every
// tile runs five digits.  Dropping the levels s > D and rounding below the
// unit leave errors of about one unit per block.  A pass runs in this form
// only when all its blocks are unitary.
constexpr uint32_t kDgPlane = 16384;                       // 128 rows x 64 bf16
constexpr uint32_t kDgSmemB = kDigits * kDgPlane;          // 6 A planes (5 used by five-digit tiles), then B
constexpr uint32_t kDgSmemHoff = kDgSmemB + 2 * kDigitImageBytes;  // two image buffers
constexpr uint32_t kDgSmemBar = kDgSmemHoff + 128 * 8;  // 2 image barriers, 1 MMA barrier, tmem slot, tile counts
constexpr uint32_t kDgSmemBlk = kDgSmemBar + 128;       // the pass's block descriptors
static_assert(sizeof(Blk5) == 32 && kDgSmemBlk % 16 == 0, "block descriptors are copied as 16-byte words");
constexpr uint32_t kDgSmemUsed = kDgSmemBlk + kMaxPassBlocks * sizeof(Blk5);
constexpr uint32_t kDgSmemAlloc = kDgSmemUsed + 1024;
constexpr uint32_t kDgTmemCols = 512;                      // up to 7 levels x 64 columns
constexpr int kDgThreads = kDigitThreads;                  // 32 warps: 8 per 32-lane group of D
constexpr int kDgCols = 64 / (kDgThreads / 128);           // FP32 columns of a level per warp
constexpr int kDgCplx = kDgCols / 2;                       // complex results per thread per block
constexpr int kDgLoadIters = 4096 / (2 * kDgThreads);      // amplitude pairs per thread per tile
constexpr int kDgFewDigits = 5;                            // digits of a tile with a small norm
constexpr uint32_t kDgWarpBound = 1u << 27;                // a warp's norm bound below this: five digits
static_assert(kDgCols == 8 && kDgLoadIters * 2 == kBlockTableEntries / kDgThreads, "digit kernel thread layout");

// The MMA groups of one block: A plane i against B planes j0 .. j0+nj-1, in
// issue order; the first group to reach a level initialises it.  Six
// digits: the 26 pairs with i + j <= 6.  Five digits: the 20 pairs with
// i <= 4, j <= 5, i + j <= 5.
struct DgGroup {
  int i, j0, nj, init;
};
#define BF_DG_GROUPS6                                                                                 \
  {                                                                                                   \
    {0, 0, 4, 1}, {0, 4, 2, 1}, /* levels 0..5 first written */                                       \
        {1, 5, 1, 1},           /* level 6 first written */                                           \
        {1, 0, 4, 0}, {1, 4, 1, 0}, {2, 0, 4, 0}, {2, 4, 1, 0}, {3, 0, 4, 0}, {4, 0, 3, 0}, {5, 0, 2, 0} \
  }
#define BF_DG_GROUPS5                                                                                 \
  {                                                                                                   \
    {0, 0, 4, 1}, {0, 4, 2, 1}, /* levels 0..5 first written */                                       \
        {1, 0, 4, 0}, {1, 4, 1, 0}, {2, 0, 4, 0}, {3, 0, 3, 0}, {4, 0, 2, 0}                          \
  }

// 8 columns of the thread's TMEM lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])
               :
               : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// this thread's 4 destinations in a table
__device__ __forceinline__ uint2 my_dests4(const uint16_t* offsets, uint32_t table) {
  return __ldg(reinterpret_cast<const uint2*>(offsets + (size_t)table * kBlockTableEntries + threadIdx.x * 4));
}
__device__ __forceinline__ uint32_t dest_at4(const uint2& d, int e) {
  const uint32_t w = e < 2 ? d.x : d.y;
  return (e & 1) ? (w >> 16) : (w & 0xFFFFu);
}

struct DgPassArgs {
  double2* s;
  const Blk5* blocks;
  const unsigned char* images;  // kDigitImageBytes per image
  const uint16_t* offsets;
  uint64_t ntiles;
  int32_t nblocks;
  int32_t q[kBlockTileQubits];
  const int* scale_exp;         // device: the state's scale 2^e_g
  int* flag;
  uint32_t spin_limit;
  int32_t scale_shift;          // added to the state's scale exponent (0; a test moves it)
  int32_t five_digits;          // 1: tiles below the norm bound run five digits; 0: six always
  unsigned long long* digit_tiles;  // optional: [0] five-digit tiles, [1] six-digit tiles (counted per CTA)
  int32_t in_fixed;             // 1: the state holds the previous digit pass's integers V (int64 pairs)
  int32_t out_fixed;            // 1: write V itself for the next digit pass instead of FP64
};

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void load_image_bytes(uint32_t dst, const void* src, uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// rint(t / 256) for |t| < 2^30: t / 256 is exact, and the FMA rounds its sum
// with 1.5 * 2^23 once, to an integer
__device__ __forceinline__ float rint_div256(float t) {
  return __fsub_rn(__fmaf_rn(t, 0.00390625f, 12582912.0f), 12582912.0f);
}

// The carry step of two values at once in packed FP32 pairs (f32x2, one
// instruction for both lanes, each lane rounded exactly as its scalar
// form): t = d + c, q = rint(t / 256) as in rint_div256, d = t - 256 q,
// c = q.
__device__ __forceinline__ void carry_pair(float& d0, float& d1, float& c0, float& c1) {
  const unsigned long long inv256 = 0x3B8000003B800000ull;  // (2^-8, 2^-8)
  const unsigned long long magic = 0x4B4000004B400000ull;   // (1.5 * 2^23, 1.5 * 2^23)
  const unsigned long long m256 = 0xC3800000C3800000ull;    // (-256, -256)
  unsigned long long d, c, t, u, q;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(d0), "f"(d1));
  asm("mov.b64 %0, {%1, %2};" : "=l"(c) : "f"(c0), "f"(c1));
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(t) : "l"(d), "l"(c));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(u) : "l"(t), "l"(inv256), "l"(magic));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(q) : "l"(u), "l"(magic));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(q), "l"(m256), "l"(t));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d0), "=f"(d1) : "l"(d));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(c0), "=f"(c1) : "l"(q));
}

// two 8-column TMEM loads in flight, one wait; the wait names the registers
// so that no use of them is scheduled before it
__device__ __forceinline__ void tmem_ld8x2(uint32_t ta, uint32_t tb, float* va, float* vb) {
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(ta));
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                 "=r"(r[15])
               : "r"(tb));
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15])
               :
               : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    va[i] = __uint_as_float(r[i]);
    vb[i] = __uint_as_float(r[8 + i]);
  }
}
__device__ __forceinline__ int int_of_small(float x) {  // exact integer-valued |x| < 2^22
  return __float_as_int(__fadd_rn(x, 12582912.0f)) - 0x4B400000;
}
// two exact small-integer floats -> (bf16 lo | bf16 hi << 16)
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// byte j (0..3) of w minus 128, as an exact float: the byte goes into the
// low mantissa bits of 1.5 * 2^23
__device__ __forceinline__ float byte_digit(uint32_t w, int j) {
  return __int_as_float((int)__byte_perm(w, 0x4B400000u, 0x7640u + (uint32_t)j)) - 12583040.0f;
}

// V = round(x * 2^sh) to nearest, ties to even, |V| < 2^(8D - 1), as D
// balanced base-256 digits d (d[D-1] the lowest).  A value a digit pass wrote
// is an integer of the unit already and converts exactly; other values (the
// first digit pass of a circuit) round once, and ties round to even so that
// the rounding has no bias (away from zero would grow every tie's
// magnitude, and the norm with them).  With W = V + 128 (1 + 2^8 + ... +
// 2^(8(D-1))) every
// byte of W is its digit plus 128 (the added 128s absorb the borrows), and
// the top digit is W / 2^(8(D-1)) - 128.  False when |x * 2^sh| >= 2^(8D-1)
// (the scale does not cover x).
template <int D>
__device__ __forceinline__ bool digits_of(double x, int sh, float* d) {
  static_assert(D == 5 || D == 6, "five or six digits");
  const long long b = __double_as_longlong(x);
  const int ex = (int)((uint32_t)(b >> 52) & 0x7ffu);
  const int k = ex - 1075 + sh;  // |x| 2^sh = m 2^k
  long long V = 0;
  bool ok = true;
  if (ex != 0 && k > -64) {
    if (k > 8 * D - 54) {
      ok = false;
    } else {
      const long long m = (b & 0x000FFFFFFFFFFFFFll) | 0x0010000000000000ll;
      // add half - 1 plus the kept low bit: rounds up above one half, and at
      // exactly one half only when the kept part is odd
      V = (m + (1ll << (-k - 1)) - 1 + ((m >> (-k)) & 1)) >> (-k);
    }
  }
  if (b < 0) V = -V;
  const unsigned long long W = (unsigned long long)(V + (D == 6 ? 0x808080808080ll : 0x8080808080ll));
  const uint32_t wl = (uint32_t)W, wh = (uint32_t)(W >> 32);
  d[D - 1] = byte_digit(wl, 0);
  d[D - 2] = byte_digit(wl, 1);
  d[D - 3] = byte_digit(wl, 2);
  d[D - 4] = byte_digit(wl, 3);
  if (D == 6) {
    d[1] = byte_digit(wh, 0);
    d[0] = __int_as_float((int)(0x4B400000u | (wh >> 8))) - 12583040.0f;
  } else {
    d[0] = __int_as_float((int)(0x4B400000u | wh)) - 12583040.0f;
  }
  return ok;
}

// V * 2^e as a double, |V| < 2^53 (exact)
__device__ __forceinline__ double double_of(long long V, int e) {
  if (V == 0) return 0.0;
  const unsigned long long sgn = V < 0 ? 0x8000000000000000ull : 0ull;
  const unsigned long long a = (unsigned long long)(V < 0 ? -V : V);
  const int lz = __clzll(a);
  const unsigned long long mant = (a << (lz - 11)) & 0x000FFFFFFFFFFFFFull;
  const long long E = (long long)(63 - lz) + 1023 + e;
  if (E <= 0) return 0.0;
  return __longlong_as_double((long long)(sgn | ((unsigned long long)E << 52) | mant));
}

// An integer upper bound of x^2 in units of 2^(2e - 50) (s = 2^e the
// state's scale), clamped to kDgWarpBound: with ex the biased exponent of x
// and m8 its top 8 mantissa bits, |x| < (257 + m8) 2^(ex - 1031), so x^2 <
// (257 + m8)^2 2^k units with k = 2 (ex - e) - 2012, rounded up.  Zero gives
// 0, a subnormal 1.  A tile whose warps each sum below kDgWarpBound units
// has ||tile||^2 < 32 * 2^27 * 2^(2e - 50) = (2^-9 s)^2.  Integer sums are
// exact and independent of the reduction order.
__device__ __forceinline__ uint32_t sq_bound_units(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  if (b == 0) return 0;
  const int ex = (int)(b >> 52);
  if (ex == 0) return 1;
  const uint32_t u = 257u + (uint32_t)((b >> 44) & 255u);
  const uint32_t u2 = u * u;  // below 2^19
  const int k = 2 * (ex - e) - 2012;
  if (k >= 11) return kDgWarpBound;               // u2 >= 2^16: the term alone reaches the bound
  if (k >= 0) return min(u2 << k, kDgWarpBound);  // below 2^29 before the min
  if (k <= -19) return 1;
  return (u2 + (1u << -k) - 1) >> -k;
}

// digits_of for a value already held as its integer V of the unit (the
// output of the previous digit pass): the same digits, no rounding
template <int D>
__device__ __forceinline__ bool digits_of_fixed(long long V, float* d) {
  const bool ok = V < (1ll << (8 * D - 1)) && V > -(1ll << (8 * D - 1));
  const unsigned long long W = (unsigned long long)(V + (D == 6 ? 0x808080808080ll : 0x8080808080ll));
  const uint32_t wl = (uint32_t)W, wh = (uint32_t)(W >> 32);
  d[D - 1] = byte_digit(wl, 0);
  d[D - 2] = byte_digit(wl, 1);
  d[D - 3] = byte_digit(wl, 2);
  d[D - 4] = byte_digit(wl, 3);
  if (D == 6) {
    d[1] = byte_digit(wh, 0);
    d[0] = __int_as_float((int)(0x4B400000u | (wh >> 8))) - 12583040.0f;
  } else {
    d[0] = __int_as_float((int)(0x4B400000u | wh)) - 12583040.0f;
  }
  return ok;
}

// sq_bound_units of x = V 2^(e - 48) from V: the exponent difference ex - e
// is lead + 975 (lead = the position of V's leading one), so k = 2 lead - 62
// whatever the scale, and m8 is the 8 bits below the leading one
__device__ __forceinline__ uint32_t sq_bound_units_fixed(long long V) {
  if (V == 0) return 0;
  const unsigned long long a = (unsigned long long)(V < 0 ? -V : V);
  const int lead = 63 - __clzll(a);
  const uint32_t m8 = (uint32_t)((lead >= 8 ? a >> (lead - 8) : a << (8 - lead)) & 255u);
  const uint32_t u = 257u + m8;
  const uint32_t u2 = u * u;
  const int k = 2 * lead - 62;
  if (k >= 11) return kDgWarpBound;
  if (k >= 0) return min(u2 << k, kDgWarpBound);
  if (k <= -19) return 1;
  return (u2 + (1u << -k) - 1) >> -k;
}

template <int D>
__device__ __forceinline__ DgGroup dg_group(int gi) {
  if constexpr (D == 6) {
    constexpr DgGroup g[10] = BF_DG_GROUPS6;
    return g[gi];
  } else {
    constexpr DgGroup g[7] = BF_DG_GROUPS5;
    return g[gi];
  }
}
template <int D>
constexpr int kDgGroupCount = D == 6 ? 10 : 7;

// The CTA's pipeline state, carried from tile to tile.  Block k of the CTA
// (counting every tile's blocks) uses image buffer k & 1, whose barrier is
// then in its phase (k >> 1) & 1, and the MMA barrier in phase k & 1.
struct DgPipe {
  uint32_t kimg;       // blocks this CTA has run
  int b_in_flight;     // thread 0: image loads not yet waited for (by buffer bit)
  bool issued;         // thread 0: MMAs issued for the current block
  int mma_lost_phase;  // thread 0: MMA phase whose wait expired
  bool range_ok;
};

// What every tile of the launch shares.
struct DgFixed {
  unsigned char* sm;
  const Blk5* blk;
  const uint64_t* hoff;
  uint32_t sA, sB, tmem, tlane, bar_b, bar_mma, idesc_base;
  uint64_t free_pos, grid_base;  // next tile's base: ((base | ~free_pos) + grid_base) & free_pos
};

// the 4 MMAs (K = 16 each) of one group: A plane i against nj stacked B
// planes j0.. (N = 64 nj) into levels i + j0 .. i + j0 + nj - 1, consecutive
// 64-column ranges of tensor memory; an initialising group overwrites at
// K step 0, the others accumulate
__device__ __forceinline__ void dg_mma_group(const DgFixed& f, uint32_t sBk, const DgGroup gr) {
  const uint32_t idn = f.idesc_base | ((uint32_t)(8 * gr.nj) << 17);
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const uint64_t ad = sdesc(f.sA + (uint32_t)gr.i * kDgPlane + (uint32_t)ks * 32u);
    const uint64_t bd = sdesc(sBk + (uint32_t)gr.j0 * 8192u + (uint32_t)ks * 32u);
    mma_bf16(f.tmem + 64u * (uint32_t)(gr.i + gr.j0), ad, bd, idn, (gr.init && ks == 0) ? 0u : 1u);
  }
}

// Thread 0, before the first MMA of the CTA's block k: waits (bounded) for
// its image in buffer k & 1; false when the wait expired.
__device__ __forceinline__ bool dg_wait_image(const DgFixed& f, const DgPassArgs& a, DgPipe& p, uint32_t k) {
  const uint32_t kb = k & 1u;
  if (!mbar_wait(f.bar_b + 8u * kb, (k >> 1) & 1u, a.spin_limit)) return false;
  p.b_in_flight &= ~(1 << kb);
  tc_fence_after();
  return true;
}

// Thread 0, after the last MMA of the CTA's block k (block bi of the pass):
// commits them to the MMA barrier and loads the image of the block after it
// (the pass's next block, or the next tile's first) into the other buffer,
// whose last reader (block k - 1's MMAs) has completed.
__device__ __forceinline__ void dg_commit(const DgFixed& f, const DgPassArgs& a, DgPipe& p, uint32_t k, int bi,
                                          uint64_t obase, bool has_next) {
  mma_commit(f.bar_mma);
  p.issued = true;
  const Blk5* nb = nullptr;
  uint64_t nbase = obase;
  if (bi + 1 < a.nblocks) {
    nb = &f.blk[bi + 1];
  } else if (has_next) {
    nb = &f.blk[0];
    nbase = ((obase | ~f.free_pos) + f.grid_base) & f.free_pos;
  }
  if (nb) {
    const uint32_t kn = (k + 1) & 1u;
    load_image_bytes(f.sB + kn * kDigitImageBytes,
                     a.images + (size_t)(nb->img + variant_of(*nb, nbase)) * kDigitImageBytes, f.bar_b + 8u * kn,
                     kDigitImageBytes);
    p.b_in_flight |= 1 << kn;
  }
}

// The pass's blocks on one tile whose A planes hold its D digits, then its
// results (FP64 of unit 2^(e - 48), or the integers themselves for the next
// digit pass) back to the state.  False when a bounded wait expired (the
// CTA then stops).
template <int D>
__device__ __forceinline__ bool dg_tile(const DgPassArgs& a, const DgFixed& f, DgPipe& p, uint64_t obase,
                                        bool has_next, int e) {
  const int tid = threadIdx.x;
  unsigned char* sm = f.sm;
  // the tile's first block: every group, after the conversion's barrier
  bool issue_lost = false;  // thread 0: the image of the block to run never arrived
  if (tid == 0) {
    if (dg_wait_image(f, a, p, p.kimg)) {
      const uint32_t sBk = f.sB + (p.kimg & 1u) * kDigitImageBytes;
#pragma unroll
      for (int gi = 0; gi < kDgGroupCount<D>; ++gi) dg_mma_group(f, sBk, dg_group<D>(gi));
      dg_commit(f, a, p, p.kimg, 0, obase, has_next);
    } else {
      issue_lost = true;
    }
  }
  for (int bi = 0; bi < a.nblocks; ++bi) {
    const bool more = bi + 1 < a.nblocks;
    const uint32_t k = p.kimg;  // this block
    const uint32_t sBn = f.sB + ((k + 1) & 1u) * kDigitImageBytes;
    const uint2 dest = my_dests4(a.offsets, f.blk[bi].offs);
    bool lost = issue_lost;     // no MMAs were issued: the wait below expires too
    if (!mbar_wait(f.bar_mma, k & 1u, a.spin_limit)) lost = true;
    tc_fence_after();
    // Level s holds digit position s + 1 of the result.  From the lowest
    // level up: t = sum + carry, digit = t - 256 round(t / 256), carry the
    // rest; positions D and D + 1 only round; position 0 is the last carry.
    float carry[kDgCols];
#pragma unroll
    for (int c = 0; c < kDgCols; ++c) carry[c] = 0.f;
    auto carry_step = [&](float* d) {
#pragma unroll
      for (int c = 0; c < kDgCols; c += 2) carry_pair(d[c], d[c + 1], carry[c], carry[c + 1]);
    };
    if (more) {
      // positions 1 .. D-1 and 0 become the next block's A planes
      auto level = [&](const int s, float* d) {
        carry_step(d);
        if (s + 1 <= D - 1) {
#pragma unroll
          for (int c = 0; c < kDgCplx; ++c)
            *reinterpret_cast<uint32_t*>(sm + (uint32_t)(s + 1) * kDgPlane + (dest_at4(dest, c) << 2)) =
                pack_bf16(d[2 * c], d[2 * c + 1]);
        }
      };
#pragma unroll
      for (int s = D; s >= 1; s -= 2) {
        float d0[kDgCols], d1[kDgCols];
        tmem_ld8x2(f.tlane + 64u * (uint32_t)s, f.tlane + 64u * (uint32_t)(s - 1), d0, d1);
        level(s, d0);
        level(s - 1, d1);
      }
      if ((D + 1) & 1) {
        float d0[kDgCols];
        tmem_ld8(f.tlane, d0);
        level(0, d0);
      }
#pragma unroll
      for (int c = 0; c < kDgCplx; ++c)
        *reinterpret_cast<uint32_t*>(sm + (dest_at4(dest, c) << 2)) = pack_bf16(carry[2 * c], carry[2 * c + 1]);
      fence_proxy_async();
    } else {
      // after the last block the result is V = hi 2^24 + lo, the three
      // lowest positions in lo and the others in hi (32-bit each); each
      // thread stores its results straight to the state (the table gives
      // their tile elements), which measured faster than staging the tile
      // in shared memory for coalesced row stores (22.2 against 24.6 ms per
      // 30-qubit pass)
      int lo[kDgCols], hi[kDgCols];
#pragma unroll
      for (int c = 0; c < kDgCols; ++c) {
        lo[c] = 0;
        hi[c] = 0;
      }
      auto level = [&](const int s, float* d) {
        carry_step(d);
        const int pos = s + 1;
        if (pos <= D - 1) {
          if (pos >= D - 3) {
#pragma unroll
            for (int c = 0; c < kDgCols; ++c) lo[c] += int_of_small(d[c]) * (1 << (8 * (D - 1 - pos)));
          } else {
#pragma unroll
            for (int c = 0; c < kDgCols; ++c) hi[c] += int_of_small(d[c]) * (1 << (8 * (D - 4 - pos)));
          }
        }
      };
#pragma unroll
      for (int s = D; s >= 1; s -= 2) {
        float d0[kDgCols], d1[kDgCols];
        tmem_ld8x2(f.tlane + 64u * (uint32_t)s, f.tlane + 64u * (uint32_t)(s - 1), d0, d1);
        level(s, d0);
        level(s - 1, d1);
      }
      if ((D + 1) & 1) {
        float d0[kDgCols];
        tmem_ld8(f.tlane, d0);
        level(0, d0);
      }
#pragma unroll
      for (int c = 0; c < kDgCplx; ++c) {
        const long long vr = (long long)(hi[2 * c] + int_of_small(carry[2 * c]) * (1 << (8 * (D - 4)))) *
                                 16777216ll +
                             (long long)lo[2 * c];
        const long long vi = (long long)(hi[2 * c + 1] + int_of_small(carry[2 * c + 1]) * (1 << (8 * (D - 4)))) *
                                 16777216ll +
                             (long long)lo[2 * c + 1];
        const uint32_t ie = dest_at4(dest, c);  // the result's tile element
        __stcs(a.s + (obase | (ie & 31u) | f.hoff[ie >> 5]),
               a.out_fixed ? make_double2(__longlong_as_double(vr), __longlong_as_double(vi))
                           : make_double2(double_of(vr, e - 48), double_of(vi, e - 48)));
      }
    }
    if (tid == 0 && lost && p.issued) p.mma_lost_phase = (int)(k & 1u);
    ++p.kimg;
    tc_fence_before();
    if (__syncthreads_or(lost ? 1 : 0)) {
      if (tid == 0) atomicExch(a.flag, 1);
      return false;
    }
    // the next block's MMAs, once every thread has written its A planes
    issue_lost = false;
    if (more && tid == 0) {
      tc_fence_after();
      if (dg_wait_image(f, a, p, k + 1)) {
#pragma unroll
        for (int gi = 0; gi < kDgGroupCount<D>; ++gi) dg_mma_group(f, sBn, dg_group<D>(gi));
        dg_commit(f, a, p, k + 1, bi + 1, obase, has_next);
      } else {
        issue_lost = true;
      }
    }
  }
  return true;
}

__global__ void __launch_bounds__(kDgThreads, 1) k_tblock_dg(const DgPassArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* hoff = reinterpret_cast<uint64_t*>(sm + kDgSmemHoff);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kDgSmemBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kDgSmemBar + 72);
  Blk5* blk = reinterpret_cast<Blk5*>(sm + kDgSmemBlk);
  // bars[0], bars[1]: image buffers; bars[2]: the MMAs of a block
  const uint32_t bar_b = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[2]);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kDgTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
    mbar_init(bar_b, 1);
    mbar_init(bar_b + 8u, 1);
    mbar_init(bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int h = tid; h < 128; h += kDgThreads) {
    uint64_t off = 0;
    for (int j = 0; j < 7; ++j)
      if ((h >> j) & 1) off |= 1ull << a.q[5 + j];
    hoff[h] = off;
  }
  if (tid < a.nblocks * (int)(sizeof(Blk5) / 16))
    reinterpret_cast<uint4*>(blk)[tid] = __ldg(reinterpret_cast<const uint4*>(a.blocks) + tid);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t colh = (uint32_t)(warp >> 2);  // 8 column groups of 8
  DgFixed f;
  f.sm = sm;
  f.blk = blk;
  f.hoff = hoff;
  f.sA = smem_u32(sm);
  f.sB = smem_u32(sm + kDgSmemB);
  f.tmem = tmem;
  f.tlane = tmem + ((32u * (warp & 3)) << 16) + (uint32_t)kDgCols * colh;
  f.bar_b = bar_b;
  f.bar_mma = bar_mma;
  // kind::f16: D FP32, A and B BF16, both K-major, M = 128 (N set per MMA)
  f.idesc_base = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 4) << 24);
  const int e = *a.scale_exp + a.scale_shift;
  const int sh = 48 - e;  // x / 2^e * 2^48 = x * 2^sh: the value in units

  DgPipe p;
  p.kimg = 0;
  p.b_in_flight = 0;
  p.issued = false;
  p.mma_lost_phase = -1;
  p.range_ok = true;
  uint32_t* tiles_by_digits = reinterpret_cast<uint32_t*>(sm + kDgSmemBar + 80);  // five, six (thread 0)
  if (tid == 0) tiles_by_digits[0] = tiles_by_digits[1] = 0;

  auto tile_base = [&](uint64_t tile) {
    uint64_t ob = tile;
    for (int j = 0; j < kBlockTileQubits; ++j) ob = insert_zero_bit(ob, a.q[j]);
    return ob;
  };

  // Tile bases step by masked addition: with the tile positions filled with
  // ones, adding the base of gridDim.x carries across them, so base(t + g) =
  // ((base(t) | ~free) + base(g)) & free.
  uint64_t tpos = 0;
  for (int j = 0; j < kBlockTileQubits; ++j) tpos |= 1ull << a.q[j];
  const uint64_t free_pos = ((a.ntiles << kBlockTileQubits) - 1) & ~tpos;
  const uint64_t grid_base = tile_base(gridDim.x);
  auto step_base = [&](uint64_t b) { return ((b | ~free_pos) + grid_base) & free_pos; };
  f.free_pos = free_pos;
  f.grid_base = grid_base;
  uint64_t tile = blockIdx.x;
  uint64_t obase = tile_base(tile);
  if (tid == 0 && tile < a.ntiles) {
    const Blk5& b0 = blk[0];
    load_image_bytes(f.sB, a.images + (size_t)(b0.img + variant_of(b0, obase)) * kDigitImageBytes, bar_b,
                     kDigitImageBytes);
    p.b_in_flight |= 1;
  }
  const uint2 load_dest = my_dests4(a.offsets, blk[0].load_offs);

  bool failed = false;
  for (; tile < a.ntiles && !failed; tile += gridDim.x, obase = step_base(obase)) {
    const bool has_next = tile + gridDim.x < a.ntiles;
    // load: 4 amplitudes per thread, all loads issued first
    double2 v[2 * kDgLoadIters];
#pragma unroll
    for (int it = 0; it < kDgLoadIters; ++it) {
      const uint32_t i0 = (uint32_t)(it * kDgThreads + tid) * 2u;
      const double2* src = a.s + (obase | (i0 & 31u) | hoff[i0 >> 5]);
      v[2 * it] = __ldcs(src);
      v[2 * it + 1] = __ldcs(src + 1);
    }
    // the next tile's 128 rows of 32 amplitudes (512 contiguous bytes each:
    // the tile holds qubits 0..4) into L2 while this tile computes, one
    // 128-byte line per thread of the first 512 (per-thread prefetches
    // measured faster than one bulk prefetch per row: 24.6 against 25.5 ms
    // per 30-qubit pass)
    if (tid < 512 && has_next) {
      const double2* line = a.s + (step_base(obase) | ((uint32_t)(tid & 3) * 8u) | hoff[tid >> 2]);
      asm volatile("prefetch.global.L2 [%0];" ::"l"(line) : "memory");
    }
    // Five digits unless a value needs six or the tile's norm may reach
    // 2^-9 s: each warp sums its exact bound (a thread's own sum is clamped
    // just below the bound, and flagged when it reaches it, so that the warp
    // sum cannot overflow), and the barrier after the conversion ORs the
    // verdicts.
    bool six = false;
    uint32_t tb = 0;
#pragma unroll
    for (int el = 0; el < 2 * kDgLoadIters; ++el) {
      float dr[kDgFewDigits], di[kDgFewDigits];
      if (a.in_fixed) {
        const long long vr = __double_as_longlong(v[el].x), vi = __double_as_longlong(v[el].y);
        six |= !digits_of_fixed<kDgFewDigits>(vr, dr);
        six |= !digits_of_fixed<kDgFewDigits>(vi, di);
        tb += sq_bound_units_fixed(vr) + sq_bound_units_fixed(vi);
      } else {
        six |= !digits_of<kDgFewDigits>(v[el].x, sh, dr);
        six |= !digits_of<kDgFewDigits>(v[el].y, sh, di);
        tb += sq_bound_units(v[el].x, e) + sq_bound_units(v[el].y, e);
      }
      const uint32_t off = dest_at4(load_dest, el) << 2;
#pragma unroll
      for (int q = 0; q < kDgFewDigits; ++q)
        *reinterpret_cast<uint32_t*>(sm + (uint32_t)q * kDgPlane + off) = pack_bf16(dr[q], di[q]);
    }
    const bool big = tb >= kDgWarpBound;
    const uint32_t ws = __reduce_add_sync(0xffffffffu, big ? kDgWarpBound - 1 : tb);
    six |= big || ws >= kDgWarpBound || !a.five_digits;
    fence_proxy_async();
    bool ok;
    if (__syncthreads_or(six ? 1 : 0)) {
#pragma unroll
      for (int el = 0; el < 2 * kDgLoadIters; ++el) {
        float dr[kDigits], di[kDigits];
        if (a.in_fixed) {
          p.range_ok &= digits_of_fixed<kDigits>(__double_as_longlong(v[el].x), dr);
          p.range_ok &= digits_of_fixed<kDigits>(__double_as_longlong(v[el].y), di);
        } else {
          p.range_ok &= digits_of<kDigits>(v[el].x, sh, dr);
          p.range_ok &= digits_of<kDigits>(v[el].y, sh, di);
        }
        const uint32_t off = dest_at4(load_dest, el) << 2;
#pragma unroll
        for (int q = 0; q < kDigits; ++q)
          *reinterpret_cast<uint32_t*>(sm + (uint32_t)q * kDgPlane + off) = pack_bf16(dr[q], di[q]);
      }
      fence_proxy_async();
      __syncthreads();
      if (tid == 0) ++tiles_by_digits[1];
      ok = dg_tile<kDigits>(a, f, p, obase, has_next, e);
    } else {
      if (tid == 0) ++tiles_by_digits[0];
      ok = dg_tile<kDgFewDigits>(a, f, p, obase, has_next, e);
    }
    if (!ok) failed = true;
  }
  if (!p.range_ok) atomicExch(a.flag, 2);
  if (tid == 0 && a.digit_tiles) {
    atomicAdd(a.digit_tiles, (unsigned long long)tiles_by_digits[0]);
    atomicAdd(a.digit_tiles + 1, (unsigned long long)tiles_by_digits[1]);
  }

  if (tid == 0) {
    // a load in flight into buffer k completes the phase of the next block
    // that would have used it
    for (uint32_t k = 0; k < 2; ++k) {
      if (!(p.b_in_flight & (1 << k))) continue;
      const uint32_t next_use = (p.kimg & 1u) == k ? p.kimg : p.kimg + 1;
      if (!mbar_wait(bar_b + 8u * k, (next_use >> 1) & 1u, a.spin_limit)) atomicExch(a.flag, 1);
    }
    if (p.mma_lost_phase >= 0 && !mbar_wait(bar_mma, (uint32_t)p.mma_lost_phase, a.spin_limit))
      atomicExch(a.flag, 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kDgTmemCols) : "memory");
}

// scale exponent e (scale = 2^e >= 2 * norm) from norm-squared partials
__global__ void k_digit_scale(const double* __restrict__ partial, int blocks, int* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double hi = 0, lo = 0;
  for (int b = 0; b < blocks; ++b) {
    hi += partial[2 * b];
    lo += partial[2 * b + 1];
  }
  const double nrm = sqrt(hi + lo) * (1.0 + 1e-6);
  int e = 1;
  if (nrm > 0) {
    int k = 0;
    frexp(nrm, &k);  // nrm < 2^k
    e = k + 1;
  }
  *out = e;
}

void launch_digit_scale(State& st, int* d_exp) {
  const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((st.N + 255) / 256, (uint64_t)st.num_sms * 8));
  ensure_partials(st, blocks);
  launch_norm2_partials(st, blocks);
  k_digit_scale<<<1, 32, 0, st.stream>>>(st.d_partial, (int)blocks, d_exp);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_block_pass_digits(State& st, const Blk5* d_blocks, int nblocks, const unsigned char* d_images,
                              const uint16_t* d_offsets, const TilePass& p, const int* d_exp, bool in_fixed,
                              bool out_fixed) {
  if (st.dtype != BF_C128) fail(BF_EINVAL, "internal: digit blocks need a complex128 state");
  if (p.K != kBlockTileQubits || st.n < kBlockTileQubits) fail(BF_EINVAL, "internal: block pass needs a 12-qubit tile");
  if (nblocks < 1 || nblocks > kMaxPassBlocks) fail(BF_EINVAL, "internal: block pass of %d blocks", nblocks);
  if (((uintptr_t)d_blocks & 15u) != 0) fail(BF_EINVAL, "internal: block descriptors must be 16-byte aligned");
  if (((uintptr_t)d_images & 15u) != 0 || ((uintptr_t)d_offsets & 15u) != 0)
    fail(BF_EINVAL, "internal: block images and tables must be 16-byte aligned");
  DgPassArgs a;
  std::memset(&a, 0, sizeof a);
  for (int j = 0; j < kBlockTileQubits; ++j) {
    a.q[j] = p.q[j];
    if (j < 5 && p.q[j] != j) fail(BF_EINVAL, "internal: block tile must hold qubits 0..4");
  }
  a.s = static_cast<double2*>(st.amp);
  a.blocks = d_blocks;
  a.images = d_images;
  a.offsets = d_offsets;
  a.nblocks = nblocks;
  a.ntiles = st.N >> kBlockTileQubits;
  a.scale_exp = d_exp;
  a.flag = state_flag(st);
  a.spin_limit = 1u << 24;
  // A test may raise the scale by 2^shift (a coarser unit) so that the
  // tiles of a small state fall below 2^-9 of it and run five digits.
  const char* shift = std::getenv("BFGPU_DIGIT_SCALE_SHIFT");
  a.scale_shift = (shift && *shift) ? std::atoi(shift) : 0;
  // five-digit tiles hold the same integers as six-digit ones; a test may
  // turn them off to compare the two bit for bit
  const char* five = std::getenv("BFGPU_DIGIT_FIVE");
  a.five_digits = (five && *five == '0') ? 0 : 1;
  a.digit_tiles = digit_tile_counters(st);
  a.in_fixed = in_fixed ? 1 : 0;
  a.out_fixed = out_fixed ? 1 : 0;
  static PerDeviceOnce configured;
  configured.run(st.device, [] {
    BF_CUDA(cudaFuncSetAttribute(k_tblock_dg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDgSmemAlloc));
    BF_CUDA(cudaFuncSetAttribute(k_tblock_dg, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  });
  uint64_t grid = std::min<uint64_t>(a.ntiles, (uint64_t)st.num_sms);
  k_tblock_dg<<<(unsigned)grid, kDgThreads, kDgSmemAlloc, st.stream>>>(a);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_block_pass(State& st, const Blk5* d_blocks, int nblocks, const unsigned char* d_images,
                       const uint16_t* d_offsets, const TilePass& p) {
  if (st.dtype != BF_C64) fail(BF_EINVAL, "internal: tensor-core blocks need a complex64 state");
  if (p.K != kBlockTileQubits || st.n < kBlockTileQubits) fail(BF_EINVAL, "internal: block pass needs a 12-qubit tile");
  if (nblocks < 1 || nblocks > kMaxPassBlocks) fail(BF_EINVAL, "internal: block pass of %d blocks", nblocks);
  if (((uintptr_t)d_blocks & 15u) != 0) fail(BF_EINVAL, "internal: block descriptors must be 16-byte aligned");
  if (((uintptr_t)d_images & 15u) != 0) fail(BF_EINVAL, "internal: block images must be 16-byte aligned");
  BlkPassArgs a;
  std::memset(&a, 0, sizeof a);
  for (int j = 0; j < kBlockTileQubits; ++j) {
    a.q[j] = p.q[j];
    if (j < 5 && p.q[j] != j) fail(BF_EINVAL, "internal: block tile must hold qubits 0..4");
  }
  a.s = static_cast<float2*>(st.amp);
  a.blocks = d_blocks;
  a.images = d_images;
  a.offsets = d_offsets;
  if (((uintptr_t)d_offsets & 15u) != 0) fail(BF_EINVAL, "internal: block tables must be 16-byte aligned");
  a.nblocks = nblocks;
  a.ntiles = st.N >> kBlockTileQubits;
  a.flag = state_flag(st);
  a.spin_limit = 1u << 24;
  static PerDeviceOnce configured;
  configured.run(st.device, [] {
    BF_CUDA(cudaFuncSetAttribute(k_tblock, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemAlloc));
    // the whole L1/shared split as shared memory: two CTAs per SM
    BF_CUDA(cudaFuncSetAttribute(k_tblock, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  });
  // two CTAs per SM when the shared memory holds them (one CTA's MMAs then
  // overlap the other's loads and conversions); the occupancy calculator
  // can report one under the default carveout, so count from the SM's size
  int smem_sm = 0;
  BF_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, st.device));
  int per_sm = std::max(1, std::min(2, smem_sm / (int)(kSmemAlloc + 1024)));
  uint64_t grid = std::min<uint64_t>(a.ntiles, (uint64_t)per_sm * st.num_sms);
  k_tblock<<<(unsigned)grid, kBlkThreads, kSmemAlloc, st.stream>>>(a);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

}  // namespace bf

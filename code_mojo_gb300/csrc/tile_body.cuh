// tile_body.cuh — the shared-memory tile pass body, used by the single-state
// tile kernel (tile.cu) and the batched persistent kernel (batch.cu).
#pragma once

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

constexpr int kTileThreads = 256;

struct TileGeom {
  int32_t K;
  int32_t L;        // low qubits (q[j] = j for j < L)
  int32_t q[kMaxTileQubits];
};

// One tile: load the 2^K amplitudes of tile `tile` (the non-tile qubits set
// to the bits of `tile`), apply ops[0..nops) in shared memory, store.  Called
// by every thread of a CTA of kTileThreads threads; `smem_raw` holds
// tile_smem_bytes(K, L) bytes.
// kL2Loads: read the state with L2-only loads (__ldcg).  Needed when other
// CTAs of the same launch wrote these amplitudes earlier (L1 is not coherent
// across SMs); a separate launch per pass does not need it.
template <class P, bool kL2Loads = false>
__device__ __forceinline__ void run_tile(typename P::Glob* __restrict__ s, const TileOp* __restrict__ ops, int nops,
                                         const TileGeom& geo, uint64_t tile, unsigned char* smem_raw) {
  using R = typename P::R;
  using S = typename P::Smem;
  const int K = geo.K, L = geo.L;
  const int TS = 1 << K;
  S* amp = reinterpret_cast<S*>(smem_raw);
  uint64_t* hoff = reinterpret_cast<uint64_t*>(smem_raw + (size_t)TS * sizeof(S));
  const int tid = threadIdx.x;

  // global index of local element 0: `tile` with zero bits inserted at the
  // tile positions (ascending).
  uint64_t obase = tile;
  for (int j = 0; j < K; ++j) obase = insert_zero_bit(obase, geo.q[j]);

  const int H = K - L;
  for (int h = tid; h < (1 << H); h += kTileThreads) {
    uint64_t off = 0;
    for (int j = 0; j < H; ++j)
      if ((h >> j) & 1) off |= 1ull << geo.q[L + j];
    hoff[h] = off;
  }
  __syncthreads();

  const int lowmask = (1 << L) - 1;
  for (int e = tid; e < TS; e += kTileThreads) {
    uint64_t gi = obase | (uint64_t)(e & lowmask) | hoff[e >> L];
    amp[e] = P::to_smem(P::from_glob(kL2Loads ? __ldcg(s + gi) : s[gi]));
  }
  __syncthreads();

  for (int i = 0; i < nops; ++i) {
    const TileOp* op = ops + i;
    const uint64_t cmo = __ldg(&op->cmask_out);
    if ((obase & cmo) != cmo) continue;  // CTA-uniform
    const int kind = __ldg(&op->kind);
    const int tloc = __ldg(&op->tloc);
    const uint32_t cml = __ldg(&op->cmask_loc);
    const typename P::Coef g = P::coef(op->m, op->mhl);
    if (tloc >= 0) {
      const int tb = 1 << tloc;
      for (int p = tid; p < (TS >> 1); p += kTileThreads) {
        int i0 = (int)insert_zero_bit((uint64_t)p, tloc);
        if ((i0 & cml) != cml) continue;
        int i1 = i0 | tb;
        if (kind == GK_SWAP) {
          S t = amp[i0];
          amp[i0] = amp[i1];
          amp[i1] = t;
        } else if (kind == GK_PHASE) {
          R v = P::from_smem(amp[i1]);
          P::cmul(v, g, 6);
          amp[i1] = P::to_smem(v);
        } else {
          R u = P::from_smem(amp[i0]), v = P::from_smem(amp[i1]);
          apply_pair<P>(kind, u, v, g);
          amp[i0] = P::to_smem(u);
          amp[i1] = P::to_smem(v);
        }
      }
    } else {
      // diagonal gate, target outside the tile: one entry for the whole CTA
      const int tg = __ldg(&op->tglob);
      const int bit = (int)((obase >> tg) & 1);
      if (kind == GK_PHASE && bit == 0) continue;  // CTA-uniform
      const typename P::E c = bit ? g.v[6] : g.v[0], sn = bit ? g.v[7] : g.v[1];
      for (int e = tid; e < TS; e += kTileThreads) {
        if ((e & cml) != cml) continue;
        R x = P::from_smem(amp[e]);
        P::cmul_by(x, c, sn);
        amp[e] = P::to_smem(x);
      }
    }
    __syncthreads();
  }

  for (int e = tid; e < TS; e += kTileThreads) {
    uint64_t gi = obase | (uint64_t)(e & lowmask) | hoff[e >> L];
    s[gi] = P::to_glob(P::from_smem(amp[e]));
  }
}

template <class P>
inline size_t tile_smem_bytes(int K, int L) {
  return ((size_t)1 << K) * sizeof(typename P::Smem) + ((size_t)1 << (K - L)) * sizeof(uint64_t);
}

}  // namespace bf

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

// One in-tile gate over all its pairs: the gate kind and whether it has
// controls inside the tile are compile-time, so the pair loop carries no
// dispatch; indices are 32-bit (a tile has at most 2^13 amplitudes).
template <class P, int KIND, bool kCtl>
__device__ __forceinline__ void tile_pairs(typename P::Smem* amp, int TS, int tloc, uint32_t cml,
                                           const typename P::Coef& g) {
  using R = typename P::R;
  using S = typename P::Smem;
  const uint32_t low = (1u << tloc) - 1u, tb = 1u << tloc;
#pragma unroll 2
  for (int p = threadIdx.x; p < (TS >> 1); p += kTileThreads) {
    const uint32_t i0 = (((uint32_t)p & ~low) << 1) | ((uint32_t)p & low);
    if (kCtl && (i0 & cml) != cml) continue;
    const uint32_t i1 = i0 | tb;
    if (KIND == GK_SWAP) {
      S t = amp[i0];
      amp[i0] = amp[i1];
      amp[i1] = t;
    } else if (KIND == GK_PHASE) {
      R v = P::from_smem(amp[i1]);
      P::cmul(v, g, 6);
      amp[i1] = P::to_smem(v);
    } else {
      R u = P::from_smem(amp[i0]), v = P::from_smem(amp[i1]);
      apply_pair<P>(KIND, u, v, g);
      amp[i0] = P::to_smem(u);
      amp[i1] = P::to_smem(v);
    }
  }
}

template <class P, bool kCtl>
__device__ __forceinline__ void tile_gate(int kind, typename P::Smem* amp, int TS, int tloc, uint32_t cml,
                                          const typename P::Coef& g) {
  switch (kind) {
    case GK_DENSE: tile_pairs<P, GK_DENSE, kCtl>(amp, TS, tloc, cml, g); break;
    case GK_H: tile_pairs<P, GK_H, kCtl>(amp, TS, tloc, cml, g); break;
    case GK_SWAP: tile_pairs<P, GK_SWAP, kCtl>(amp, TS, tloc, cml, g); break;
    case GK_PHASE: tile_pairs<P, GK_PHASE, kCtl>(amp, TS, tloc, cml, g); break;
    case GK_DIAG: tile_pairs<P, GK_DIAG, kCtl>(amp, TS, tloc, cml, g); break;
    case GK_DENSE_R: tile_pairs<P, GK_DENSE_R, kCtl>(amp, TS, tloc, cml, g); break;
    default: tile_pairs<P, GK_RY, kCtl>(amp, TS, tloc, cml, g); break;
  }
}

// One in-tile dense unitary on the consecutive local bits tloc .. tloc+UM-1:
// each thread takes whole groups of 2^UM amplitudes (the other bits fixed),
// reads them, forms U x (rows of the row-major matrix `um` in shared memory)
// and writes it back in place.
template <class P, int UM, bool kCtl>
__device__ __forceinline__ void tile_unitary(typename P::Smem* amp, int TS, int tloc, uint32_t cml,
                                             const typename P::Smem* um) {
  using R = typename P::R;
  constexpr int D = 1 << UM;
  const uint32_t low = (1u << tloc) - 1u;
  for (int g = threadIdx.x; g < (TS >> UM); g += kTileThreads) {
    const uint32_t base = (((uint32_t)g & ~low) << UM) | ((uint32_t)g & low);
    if (kCtl && (base & cml) != cml) continue;
    R x[D];
#pragma unroll
    for (int c = 0; c < D; ++c) x[c] = P::from_smem(amp[base | ((uint32_t)c << tloc)]);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      R acc = P::zero();
#pragma unroll
      for (int c = 0; c < D; ++c) acc = P::fma(P::from_smem(um[r * D + c]), x[c], acc);
      amp[base | ((uint32_t)r << tloc)] = P::to_smem(acc);
    }
  }
}

// A wider in-tile unitary (UM = 4 or 5 qubits): a thread's outputs (rows of
// groups) are formed from the group's inputs in shared memory into
// registers, 2 per thread at a time over whole groups, then written after
// a barrier (the groups of one round are disjoint from the next round's).
// The staged matrix is transposed (`umt[c * D + r]`), so that the lanes of a
// warp, which take consecutive rows of a group, read consecutive entries.
// Every thread runs the same number of rounds (the barriers are uniform).
template <class P, int UM, bool kCtl>
__device__ __forceinline__ void tile_unitary_wide(typename P::Smem* amp, int TS, int tloc, uint32_t cml,
                                                  const typename P::Smem* umt) {
  using R = typename P::R;
  constexpr int D = 1 << UM;
  constexpr int kPer = 2;  // outputs per thread per round (more cost registers of every unitary pass)
  const uint32_t low = (1u << tloc) - 1u;
  for (int round = 0; round < TS; round += kPer * kTileThreads) {
    R out[kPer];
    uint32_t where[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int o = round + j * kTileThreads + (int)threadIdx.x;
      where[j] = 0xffffffffu;
      if (o >= TS) continue;
      const uint32_t g = (uint32_t)o >> UM, r = (uint32_t)o & (D - 1);
      const uint32_t base = ((g & ~low) << UM) | (g & low);
      if (kCtl && (base & cml) != cml) continue;
      R acc = P::zero();
#pragma unroll 1
      for (int c = 0; c < D; ++c)
        acc = P::fma(P::from_smem(umt[c * D + r]), P::from_smem(amp[base | ((uint32_t)c << tloc)]), acc);
      out[j] = acc;
      where[j] = base | (r << tloc);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kPer; ++j)
      if (where[j] != 0xffffffffu) amp[where[j]] = P::to_smem(out[j]);
  }
}

// bytes of shared memory before the staged unitary matrix (16-byte aligned)
template <class P>
__host__ __device__ inline size_t tile_umat_offset(int K, int L) {
  return ((((size_t)1 << K) * sizeof(typename P::Smem) + ((size_t)1 << (K - L)) * sizeof(uint64_t)) + 15) &
         ~(size_t)15;
}

// One tile: load the 2^K amplitudes of tile `tile` (the non-tile qubits set
// to the bits of `tile`), apply ops[0..nops) in shared memory, store.  Called
// by every thread of a CTA of kTileThreads threads; `smem_raw` holds
// tile_smem_bytes(K, L) bytes.
// kL2Loads: read the state with L2-only loads (__ldcg).  Needed when other
// CTAs of the same launch wrote these amplitudes earlier (L1 is not coherent
// across SMs); a separate launch per pass does not need it.
// kUnitaries: the ops may include GK_UNITARY (their register-heavy loop is
// compiled only into this form; passes without them keep the lean one);
// umats is then the unitary pool (row-major interleaved FP64), and
// `smem_raw` also holds the staged matrix (tile_smem_bytes(K, L, true)).
template <class P, bool kL2Loads = false, bool kUnitaries = false>
__device__ __forceinline__ void run_tile(typename P::Glob* __restrict__ s, const TileOp* __restrict__ ops, int nops,
                                         const TileGeom& geo, uint64_t tile, unsigned char* smem_raw,
                                         const double* __restrict__ umats = nullptr) {
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
    if (kUnitaries && kind == GK_UNITARY) {
      // stage the matrix, then every group of the tile
      const int um = __ldg(&op->um);
      const double* u = umats + __ldg(&op->uoff);
      S* mat = reinterpret_cast<S*>(smem_raw + tile_umat_offset<P>(K, L));
      const int dim = 1 << um;
      for (int e = tid; e < dim * dim; e += kTileThreads) {
        typename P::Glob gv;
        if constexpr (sizeof(typename P::Glob) == 16) gv = make_double2(__ldg(u + 2 * e), __ldg(u + 2 * e + 1));
        else gv = make_float2((float)__ldg(u + 2 * e), (float)__ldg(u + 2 * e + 1));
        // row-major for the narrow forms, transposed for the wide ones
        const int at = um <= 3 ? e : (e % dim) * dim + e / dim;
        mat[at] = P::to_smem(P::from_glob(gv));
      }
      __syncthreads();
      switch (um) {
        case 2:
          if (cml) tile_unitary<P, 2, true>(amp, TS, tloc, cml, mat);
          else tile_unitary<P, 2, false>(amp, TS, tloc, 0u, mat);
          break;
        case 3:
          if (cml) tile_unitary<P, 3, true>(amp, TS, tloc, cml, mat);
          else tile_unitary<P, 3, false>(amp, TS, tloc, 0u, mat);
          break;
        case 4:
          if (cml) tile_unitary_wide<P, 4, true>(amp, TS, tloc, cml, mat);
          else tile_unitary_wide<P, 4, false>(amp, TS, tloc, 0u, mat);
          break;
        default:
          if (cml) tile_unitary_wide<P, 5, true>(amp, TS, tloc, cml, mat);
          else tile_unitary_wide<P, 5, false>(amp, TS, tloc, 0u, mat);
          break;
      }
      __syncthreads();
      continue;
    }
    const typename P::Coef g = P::coef(op->m, op->mhl);
    if (tloc >= 0) {
      if (cml) tile_gate<P, true>(kind, amp, TS, tloc, cml, g);
      else tile_gate<P, false>(kind, amp, TS, tloc, 0u, g);
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

// shared memory of run_tile; with_unitary: room for a staged
// 2^kTileUnitaryMax-square matrix
template <class P>
inline size_t tile_smem_bytes(int K, int L, bool with_unitary = false) {
  if (with_unitary)
    return tile_umat_offset<P>(K, L) + ((size_t)1 << (2 * kTileUnitaryMax)) * sizeof(typename P::Smem);
  return ((size_t)1 << K) * sizeof(typename P::Smem) + ((size_t)1 << (K - L)) * sizeof(uint64_t);
}

}  // namespace bf

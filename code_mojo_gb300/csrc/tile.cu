// tile.cu — fused tile pass: each CTA loads the 2^K amplitudes that share
// one assignment of the non-tile qubits into shared memory, applies an
// ordered list of gates there, and writes them back: one HBM read + write
// for the whole group of gates.
//
// GPU form of the reference's fused-grid strategy (GRID_FUSED: row-local
// groups applied one row at a time, executors.mojo:1062-1093) and of its
// L2 column tiling (transformations_grid.mojo:21, 367-555): the "row" is the
// set of K tile qubits, which need not be contiguous.  The low
// kTileLowQubits qubits are always part of the tile so that every global
// access moves runs of 2^5 contiguous amplitudes (512 B at complex128).
//
// A gate fits a tile pass when its target is a tile qubit; its controls may
// be anywhere (a control outside the tile is constant over the CTA, so the
// CTA applies the gate or skips it).  A diagonal gate fits whatever its
// qubits: a target outside the tile only selects which diagonal entry the
// whole CTA multiplies by.
#include <algorithm>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

constexpr int kTileThreads = 256;

struct TileGeom {
  int32_t K;
  int32_t L;        // low qubits (q[j] = j for j < L)
  int32_t q[kMaxTileQubits];
};

template <class P>
__global__ void __launch_bounds__(kTileThreads) k_tile(typename P::Glob* __restrict__ s,
                                                       const TileOp* __restrict__ ops, int nops,
                                                       const TileGeom geo) {
  using R = typename P::R;
  using S = typename P::Smem;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = geo.K, L = geo.L;
  const int TS = 1 << K;
  S* amp = reinterpret_cast<S*>(smem_raw);
  uint64_t* hoff = reinterpret_cast<uint64_t*>(smem_raw + (size_t)TS * sizeof(S));
  const int tid = threadIdx.x;

  // global index of local element 0: blockIdx.x with zero bits inserted at
  // the tile positions (ascending).
  uint64_t obase = blockIdx.x;
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
    amp[e] = P::to_smem(P::from_glob(s[gi]));
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
static size_t tile_smem_bytes(int K, int L) {
  return ((size_t)1 << K) * sizeof(typename P::Smem) + ((size_t)1 << (K - L)) * sizeof(uint64_t);
}

template <class P>
static void launch_tile_p(State& st, const TileOp* d_ops, int nops, const TilePass& p) {
  TileGeom geo;
  geo.K = p.K;
  geo.L = p.L;
  if (geo.L < 0 || geo.L > std::min(p.K, kTileLowQubits)) fail(BF_EINVAL, "internal: bad tile low width %d", geo.L);
  for (int j = 0; j < p.K; ++j) geo.q[j] = p.q[j];
  for (int j = 0; j < geo.L; ++j)
    if (geo.q[j] != j) fail(BF_EINVAL, "internal: tile qubits must start with 0..%d", geo.L - 1);
  size_t smem = tile_smem_bytes<P>(p.K, geo.L);
  static int configured[3] = {0, 0, 0};
  int idx = st.prec;
  if (!configured[idx]) {
    BF_CUDA(cudaFuncSetAttribute(k_tile<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tile_smem_bytes<P>(kMaxTileQubits, 0)));
    configured[idx] = 1;
  }
  uint64_t blocks = st.N >> p.K;
  if (blocks > 0x7fffffffull) fail(BF_EUNSUPPORTED, "tile grid too large");
  k_tile<P><<<(unsigned)blocks, kTileThreads, smem, st.stream>>>(static_cast<typename P::Glob*>(st.amp), d_ops,
                                                                 nops, geo);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_tile_pass(State& st, const TileOp* d_ops, int nops, const TilePass& p) {
  switch (st.prec) {
    case PREC_F64: launch_tile_p<PolF64>(st, d_ops, nops, p); break;
    case PREC_DF: launch_tile_p<PolDF>(st, d_ops, nops, p); break;
    default: launch_tile_p<PolF32>(st, d_ops, nops, p); break;
  }
}

int tile_max_qubits(const State&) { return kMaxTileQubits; }

}  // namespace bf

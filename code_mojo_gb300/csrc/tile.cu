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

#include "tile_body.cuh"

namespace bf {

// kUnitaries: the pass holds dense unitaries (a separate form, so that
// passes without them keep the gate loop's small register count)
template <class P, bool kUnitaries>
__global__ void __launch_bounds__(kTileThreads) k_tile(typename P::Glob* __restrict__ s,
                                                       const TileOp* __restrict__ ops, int nops,
                                                       const TileGeom geo, const double* __restrict__ umats) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  run_tile<P, false, kUnitaries>(s, ops, nops, geo, blockIdx.x, smem_raw, umats);
}


template <class P>
static void launch_tile_p(State& st, const TileOp* d_ops, int nops, const TilePass& p, const double* d_umats) {
  TileGeom geo;
  geo.K = p.K;
  geo.L = p.L;
  if (geo.L < 0 || geo.L > std::min(p.K, kTileLowQubits)) fail(BF_EINVAL, "internal: bad tile low width %d", geo.L);
  for (int j = 0; j < p.K; ++j) geo.q[j] = p.q[j];
  for (int j = 0; j < geo.L; ++j)
    if (geo.q[j] != j) fail(BF_EINVAL, "internal: tile qubits must start with 0..%d", geo.L - 1);
  const bool uni = d_umats != nullptr;
  size_t smem = tile_smem_bytes<P>(p.K, geo.L, uni);
  static PerDeviceOnce configured;  // one per instantiation of P
  configured.run(st.device, [] {
    BF_CUDA(cudaFuncSetAttribute(k_tile<P, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tile_smem_bytes<P>(kMaxTileQubits, 0)));
    BF_CUDA(cudaFuncSetAttribute(k_tile<P, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tile_smem_bytes<P>(kMaxTileQubits, 0, true)));
  });
  uint64_t blocks = st.N >> p.K;
  if (blocks > 0x7fffffffull) fail(BF_EUNSUPPORTED, "tile grid too large");
  auto* amp = static_cast<typename P::Glob*>(st.amp);
  if (uni) k_tile<P, true><<<(unsigned)blocks, kTileThreads, smem, st.stream>>>(amp, d_ops, nops, geo, d_umats);
  else k_tile<P, false><<<(unsigned)blocks, kTileThreads, smem, st.stream>>>(amp, d_ops, nops, geo, nullptr);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_tile_pass(State& st, const TileOp* d_ops, int nops, const TilePass& p, const double* d_umats) {
  switch (st.prec) {
    case PREC_F64: launch_tile_p<PolF64>(st, d_ops, nops, p, d_umats); break;
    case PREC_DF: launch_tile_p<PolDF>(st, d_ops, nops, p, d_umats); break;
    default: launch_tile_p<PolF32>(st, d_ops, nops, p, d_umats); break;
  }
}

int tile_max_qubits(const State&) { return kMaxTileQubits; }

}  // namespace bf

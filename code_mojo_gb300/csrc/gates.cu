// gates.cu — per-gate kernels: one HBM pass per (possibly controlled)
// single-target gate.  GPU form of the reference's per-gate strategies
// (transformations_scalar.mojo:63-594, transformations_simd_parallel.mojo).
//
// Mapping: the pair bases of a gate are the indices whose fixed bits
// (controls and target) are set to (1.., 0); thread k builds its base by
// inserting zero bits at the fixed positions (ascending) into k and OR-ing the
// control mask, so only the controlled subspace is read and written: a CX
// moves S bytes, a CP S/2, exactly the algorithmic bytes of the gate.
#include <algorithm>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

struct GateArgs {
  uint64_t count;   // pair bases (or amplitudes, for GK_PHASE)
  uint64_t cmask;   // controls | (target bit for GK_PHASE)
  int32_t target;
  int32_t nfix;
  int8_t fix[64];   // fixed bit positions, ascending
  double m[8];
  float mhl[16];
};

// Each thread takes gate_unroll pair bases a grid-stride apart and issues
// all their loads before any arithmetic, so that enough bytes are in flight
// to keep HBM busy (a state far larger than L2 is read once: streaming loads
// and stores).  Measured at 30 qubits: the arithmetic kinds at complex128
// keep two (more registers cut occupancy), the data-movement kinds eight.
template <class P, int KIND>
__host__ __device__ constexpr int gate_unroll() {
  return (KIND == GK_SWAP || KIND == GK_PHASE) ? 8 : (sizeof(typename P::Glob) == 16 ? 2 : 4);
}

template <class P, int KIND>
__global__ void __launch_bounds__(256) k_gate(typename P::Glob* __restrict__ s, const GateArgs a) {
  using R = typename P::R;
  using G = typename P::Glob;
  constexpr int kGateUnroll = gate_unroll<P, KIND>();
  const typename P::Coef g = P::coef(a.m, a.mhl);
  const uint64_t tbit = 1ull << a.target;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k0 < a.count; k0 += kGateUnroll * step) {
    uint64_t x[kGateUnroll];
    G u[kGateUnroll], v[kGateUnroll];
#pragma unroll
    for (int j = 0; j < kGateUnroll; ++j) {
      const uint64_t k = k0 + (uint64_t)j * step;
      uint64_t xx = k;
      for (int i = 0; i < a.nfix; ++i) xx = insert_zero_bit(xx, a.fix[i]);
      x[j] = xx | a.cmask;
      if (k < a.count) {
        u[j] = __ldcs(s + x[j]);  // GK_PHASE: x already carries the target bit
        if (KIND != GK_PHASE) v[j] = __ldcs(s + (x[j] | tbit));
      }
    }
#pragma unroll
    for (int j = 0; j < kGateUnroll; ++j) {
      if (k0 + (uint64_t)j * step >= a.count) break;
      if (KIND == GK_PHASE) {
        R w = P::from_glob(u[j]);
        P::cmul(w, g, 6);
        __stcs(s + x[j], P::to_glob(w));
      } else if (KIND == GK_SWAP) {  // pure data movement, no conversion
        __stcs(s + x[j], v[j]);
        __stcs(s + (x[j] | tbit), u[j]);
      } else {
        R p = P::from_glob(u[j]), q = P::from_glob(v[j]);
        apply_pair<P>(KIND, p, q, g);
        __stcs(s + x[j], P::to_glob(p));
        __stcs(s + (x[j] | tbit), P::to_glob(q));
      }
    }
  }
}

template <class P>
static void launch_gate_p(State& st, const GateInstr& g) {
  GateArgs a;
  a.target = g.target;
  uint64_t fixed = g.cmask | (1ull << g.target);
  a.nfix = 0;
  for (int b = 0; b < 64; ++b)
    if ((fixed >> b) & 1) a.fix[a.nfix++] = (int8_t)b;
  a.count = st.N >> a.nfix;
  a.cmask = g.cmask | (g.kind == GK_PHASE ? (1ull << g.target) : 0ull);
  for (int i = 0; i < 8; ++i) a.m[i] = g.m[i];
  for (int i = 0; i < 16; ++i) a.mhl[i] = g.mhl[i];
  if (a.count == 0) return;
  uint64_t blocks = std::min<uint64_t>((a.count + 255) / 256, (uint64_t)st.num_sms * 16);
  auto* s = static_cast<typename P::Glob*>(st.amp);
  switch (g.kind) {
    case GK_DENSE: k_gate<P, GK_DENSE><<<(unsigned)blocks, 256, 0, st.stream>>>(s, a); break;
    case GK_H: k_gate<P, GK_H><<<(unsigned)blocks, 256, 0, st.stream>>>(s, a); break;
    case GK_SWAP: k_gate<P, GK_SWAP><<<(unsigned)blocks, 256, 0, st.stream>>>(s, a); break;
    case GK_PHASE: k_gate<P, GK_PHASE><<<(unsigned)blocks, 256, 0, st.stream>>>(s, a); break;
    case GK_DIAG: k_gate<P, GK_DIAG><<<(unsigned)blocks, 256, 0, st.stream>>>(s, a); break;
    case GK_RY: k_gate<P, GK_RY><<<(unsigned)blocks, 256, 0, st.stream>>>(s, a); break;
    case GK_DENSE_R: k_gate<P, GK_DENSE_R><<<(unsigned)blocks, 256, 0, st.stream>>>(s, a); break;
    default: fail(BF_EINVAL, "internal: unknown lowered gate kind %d", g.kind);
  }
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_gate(State& st, const GateInstr& g) {
  switch (st.prec) {
    case PREC_F64: launch_gate_p<PolF64>(st, g); break;
    case PREC_DF: launch_gate_p<PolDF>(st, g); break;
    default: launch_gate_p<PolF32>(st, g); break;
  }
}

// swap_bits_state (state.mojo:304-317) in one pass: exchange the amplitudes
// with (bit a, bit b) = (1, 0) and (0, 1).  Touches half the state.
template <class T>
__global__ void __launch_bounds__(256) k_swap_bits(T* __restrict__ s, uint64_t count, int lo, int hi,
                                                   uint64_t abit, uint64_t bbit) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += step) {
    uint64_t x = insert_zero_bit(insert_zero_bit(k, lo), hi);
    T u = s[x | abit], v = s[x | bbit];
    s[x | abit] = v;
    s[x | bbit] = u;
  }
}

void launch_swap_bits(State& st, int a, int b) {
  if (a == b) return;
  int lo = std::min(a, b), hi = std::max(a, b);
  uint64_t count = st.N >> 2;
  if (count == 0) return;
  uint64_t blocks = std::min<uint64_t>((count + 255) / 256, (uint64_t)st.num_sms * 16);
  if (st.dtype == BF_C128)
    k_swap_bits<double2><<<(unsigned)blocks, 256, 0, st.stream>>>(static_cast<double2*>(st.amp), count, lo, hi,
                                                                   1ull << a, 1ull << b);
  else
    k_swap_bits<float2><<<(unsigned)blocks, 256, 0, st.stream>>>(static_cast<float2*>(st.amp), count, lo, hi,
                                                                  1ull << a, 1ull << b);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

}  // namespace bf

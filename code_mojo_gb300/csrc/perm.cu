// perm.cu — qubit permutations as data movement (bit-exact by construction).
//
//  * Full bit reversal (bit_reverse_state, state.mojo:131-204) in place as a
//    tiled shared-memory transpose: with the index split as
//    [h: top 5 bits][m: middle n-10 bits][l: low 5 bits], rev(i) =
//    [rev l][rev m][rev h], so the 32x32 tile at middle value m exchanges
//    with the transposed, bit-reversed tile at rev(m).  One CTA owns the
//    pair (m, rev m); every global access is a 512 B run (complex128).
//  * Any other permutation of qubit positions (partial reversal,
//    permute_qubits, qubit reversal of a subset) out of place into the
//    scratch buffer, the two buffers then swapped: complex128 states from
//    10 qubits up as shared-memory tiles whose reads and writes both run
//    over the low 5 qubits (k_permute_tiles: 2S of DRAM traffic, 0.43 ms at
//    26 qubits), otherwise as a gather dst[j] = src[map(j)] with map(j)
//    assembled from a per-CTA table of 8-bit chunks (k_permute, whose
//    scattered 16-byte reads moved 3.9S and took 0.64 ms at 26 qubits,
//    complex128).
#include <algorithm>
#include <cstring>
#include <utility>

#include "amp_math.cuh"
#include "bf_internal.h"

namespace bf {

constexpr int kRevT = 5;             // tile edge bits
constexpr int kRevW = 1 << kRevT;    // 32
constexpr int kRevPitch = kRevW + 1; // padded row (bank spread for the transpose)

__device__ __forceinline__ uint32_t rev_bits_u32(uint32_t x, int nbits) {
  return nbits == 0 ? 0u : (__brev(x) >> (32 - nbits));
}

template <class T>
__global__ void __launch_bounds__(256) k_bitrev_tiles(T* __restrict__ s, int n) {
  __shared__ T ta[kRevW * kRevPitch];
  __shared__ T tb[kRevW * kRevPitch];
  const int M = n - 2 * kRevT;
  const uint32_t m = blockIdx.x;
  const uint32_t mr = rev_bits_u32(m, M);
  if (mr < m) return;  // the partner CTA owns this pair (CTA-uniform exit)
  const int hshift = n - kRevT;
  const bool self = (mr == m);
  for (int e = threadIdx.x; e < kRevW * kRevW; e += blockDim.x) {
    int h = e >> kRevT, l = e & (kRevW - 1);
    uint64_t ia = ((uint64_t)h << hshift) | ((uint64_t)m << kRevT) | (uint64_t)l;
    ta[h * kRevPitch + l] = s[ia];
    if (!self) {
      uint64_t ib = ((uint64_t)h << hshift) | ((uint64_t)mr << kRevT) | (uint64_t)l;
      tb[h * kRevPitch + l] = s[ib];
    }
  }
  __syncthreads();
  const T* src_for_a = self ? ta : tb;
  for (int e = threadIdx.x; e < kRevW * kRevW; e += blockDim.x) {
    int h = e >> kRevT, l = e & (kRevW - 1);
    int rl = (int)rev_bits_u32((uint32_t)l, kRevT), rh = (int)rev_bits_u32((uint32_t)h, kRevT);
    uint64_t ia = ((uint64_t)h << hshift) | ((uint64_t)m << kRevT) | (uint64_t)l;
    s[ia] = src_for_a[rl * kRevPitch + rh];
    if (!self) {
      uint64_t ib = ((uint64_t)h << hshift) | ((uint64_t)mr << kRevT) | (uint64_t)l;
      s[ib] = ta[rl * kRevPitch + rh];
    }
  }
}

struct PermArgs {
  int32_t n;
  int32_t src_of[64];  // destination bit p takes source bit src_of[p]
};

template <class T>
__global__ void __launch_bounds__(256) k_permute(const T* __restrict__ src, T* __restrict__ dst, uint64_t N,
                                                 const PermArgs a) {
  __shared__ uint64_t lut[5][256];
  const int nchunks = (a.n + 7) / 8;
  for (int e = threadIdx.x; e < nchunks * 256; e += blockDim.x) {
    int c = e >> 8, v = e & 255;
    uint64_t off = 0;
    for (int b = 0; b < 8; ++b) {
      int p = c * 8 + b;
      if (p < a.n && ((v >> b) & 1)) off |= 1ull << a.src_of[p];
    }
    lut[c][v] = off;
  }
  __syncthreads();
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += step) {
    uint64_t i = 0;
    for (int c = 0; c < nchunks; ++c) i |= lut[c][(j >> (8 * c)) & 255];
    dst[j] = src[i];
  }
}

// A permutation as tiles whose global reads and writes both run over the
// low 5 qubits: P is the set of destination positions below 5 or fed from a
// source position below 5 (at most 10), S the source positions feeding P.
// A CTA takes one assignment of the other destination bits and moves the
// 2^|P| amplitudes that vary in P: it reads them in source order (the low 5
// bits of the element number are source bits 0..4: 32-amplitude runs) into
// shared memory at their destination element, then writes them in
// destination order (the low 5 bits are destination bits 0..4).
struct PermTiles {
  int32_t np;             // |P|
  int32_t pdst[10];       // P, ascending (pdst[0..4] = 0..4)
  int32_t psrc[10];       // S, ascending (psrc[0..4] = 0..4)
  int32_t e_of_f[10];     // source-order bit k (position psrc[k]) = destination-order bit e_of_f[k]
  int32_t nq;             // the other destination positions, ascending, and their source positions
  int32_t qdst[40];
  int32_t qsrc[40];
};

template <class T>
__global__ void __launch_bounds__(256) k_permute_tiles(const T* __restrict__ src, T* __restrict__ dst,
                                                       const PermTiles t) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);
  // element-number halves (low 5 bits, the rest) -> destination element,
  // source offset of the high bits, destination offset of the high bits
  __shared__ uint32_t e_lo[32], e_hi[32];
  __shared__ uint64_t s_hi[32], d_hi[32];
  if (threadIdx.x < 32) {
    const uint32_t v = threadIdx.x;
    uint32_t el = 0, eh = 0;
    uint64_t sh = 0, dh = 0;
    for (int k = 0; k < 5; ++k)
      if ((v >> k) & 1) el |= 1u << t.e_of_f[k];
    for (int k = 0; k + 5 < t.np; ++k)
      if ((v >> k) & 1) {
        eh |= 1u << t.e_of_f[5 + k];
        sh |= 1ull << t.psrc[5 + k];
        dh |= 1ull << t.pdst[5 + k];
      }
    e_lo[v] = el;
    e_hi[v] = eh;
    s_hi[v] = sh;
    d_hi[v] = dh;
  }
  // this CTA's destination bits outside P, and the source bits they take
  uint64_t dbase = 0, sbase = 0;
  for (int k = 0; k < t.nq; ++k)
    if (((uint64_t)blockIdx.x >> k) & 1) {
      dbase |= 1ull << t.qdst[k];
      sbase |= 1ull << t.qsrc[k];
    }
  __syncthreads();
  const int count = 1 << t.np;
  for (int f = threadIdx.x; f < count; f += blockDim.x)
    tile[e_lo[f & 31] | e_hi[f >> 5]] = src[sbase | (uint64_t)(f & 31) | s_hi[f >> 5]];
  __syncthreads();
  for (int e = threadIdx.x; e < count; e += blockDim.x) dst[dbase | (uint64_t)(e & 31) | d_hi[e >> 5]] = tile[e];
}

void ensure_scratch(State& st) {
  if (st.scratch) return;
  cudaError_t e = cudaMalloc(&st.scratch, st.bytes());
  if (e != cudaSuccess) {
    cudaGetLastError();
    st.scratch = nullptr;
    fail(BF_ENOMEM, "cannot allocate %zu bytes of permutation scratch", st.bytes());
  }
}

void launch_bitrev_full(State& st) {
  if (st.n < 2 * kRevT) {
    int32_t src_of[64];
    for (int p = 0; p < st.n; ++p) src_of[p] = st.n - 1 - p;
    launch_permute(st, src_of);
    return;
  }
  unsigned blocks = 1u << (st.n - 2 * kRevT);
  if (st.dtype == BF_C128)
    k_bitrev_tiles<double2><<<blocks, 256, 0, st.stream>>>(static_cast<double2*>(st.amp), st.n);
  else
    k_bitrev_tiles<float2><<<blocks, 256, 0, st.stream>>>(static_cast<float2*>(st.amp), st.n);
  BF_CUDA(cudaGetLastError());
  st.launches++;
}

void launch_permute(State& st, const int32_t* src_of) {
  bool identity = true;
  for (int p = 0; p < st.n; ++p) identity &= (src_of[p] == p);
  if (identity) return;
  if (st.n > 40) fail(BF_EUNSUPPORTED, "permutation of more than 40 qubits");
  ensure_scratch(st);
  PermArgs a;
  a.n = st.n;
  for (int p = 0; p < 64; ++p) a.src_of[p] = p < st.n ? src_of[p] : 0;
  if (st.n >= 10 && st.dtype == BF_C128) {
    // the tiled form (global accesses in 32-amplitude runs); at complex64
    // the gather below measured faster (0.26 against 0.36 ms at 26 qubits:
    // its 8-byte reads waste less of a sector, the tiles' runs are half as
    // long)
    PermTiles t;
    std::memset(&t, 0, sizeof t);
    bool inP[64] = {false}, fromP[64] = {false};
    for (int p = 0; p < st.n; ++p)
      if (p < 5 || src_of[p] < 5) {
        inP[p] = true;
        fromP[src_of[p]] = true;
      }
    for (int p = 0; p < st.n; ++p) {
      if (inP[p]) t.pdst[t.np++] = p;
      else t.qdst[t.nq++] = p;
    }
    int ns = 0;
    for (int q = 0; q < st.n; ++q)
      if (fromP[q]) t.psrc[ns++] = q;
    for (int k = 0; k < t.np; ++k)  // source bit psrc[k] feeds destination position p = pdst[e]
      for (int e = 0; e < t.np; ++e)
        if (src_of[t.pdst[e]] == t.psrc[k]) t.e_of_f[k] = e;
    for (int k = 0; k < t.nq; ++k) t.qsrc[k] = src_of[t.qdst[k]];
    const size_t smem = ((size_t)1 << t.np) * (st.dtype == BF_C128 ? sizeof(double2) : sizeof(float2));
    const uint64_t tiles = st.N >> t.np;
    if (tiles > 0x7fffffffull) fail(BF_EUNSUPPORTED, "permutation grid too large");
    if (st.dtype == BF_C128)
      k_permute_tiles<double2><<<(unsigned)tiles, 256, smem, st.stream>>>(
          static_cast<const double2*>(st.amp), static_cast<double2*>(st.scratch), t);
    else
      k_permute_tiles<float2><<<(unsigned)tiles, 256, smem, st.stream>>>(
          static_cast<const float2*>(st.amp), static_cast<float2*>(st.scratch), t);
    BF_CUDA(cudaGetLastError());
    st.launches++;
    std::swap(st.amp, st.scratch);
    return;
  }
  uint64_t blocks = std::min<uint64_t>((st.N + 255) / 256, (uint64_t)st.num_sms * 16);
  if (st.dtype == BF_C128)
    k_permute<double2><<<(unsigned)blocks, 256, 0, st.stream>>>(static_cast<const double2*>(st.amp),
                                                                static_cast<double2*>(st.scratch), st.N, a);
  else
    k_permute<float2><<<(unsigned)blocks, 256, 0, st.stream>>>(static_cast<const float2*>(st.amp),
                                                               static_cast<float2*>(st.scratch), st.N, a);
  BF_CUDA(cudaGetLastError());
  st.launches++;
  std::swap(st.amp, st.scratch);
}

// ---- modular exponentiation (Shor's order finding) -----------------------------
// apply_modexp / apply_modexp_inverse (algos/shor.mojo:56-140) as one
// out-of-place gather: amplitude (x, y) moves to (x, y * base^x mod N) for
// y < N, where x is the low n_exp bits and y the rest; y >= N stays.  For
// gcd(base, N) = 1 this is a permutation.  base^x mod N comes from a table
// built on the device (x < 2^22) or from square-and-multiply per amplitude.
__device__ __forceinline__ uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t m) {
  return (uint64_t)(((unsigned __int128)a * b) % m);
}

__device__ __forceinline__ uint64_t powmod64(uint64_t base, uint64_t e, uint64_t m) {
  uint64_t r = 1 % m, b = base % m;
  while (e) {
    if (e & 1) r = mulmod64(r, b, m);
    b = mulmod64(b, b, m);
    e >>= 1;
  }
  return r;
}

__global__ void k_powtable(uint64_t* __restrict__ table, uint64_t count, uint64_t base, uint64_t m) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < count; x += step)
    table[x] = powmod64(base, x, m);
}

template <class T>
__global__ void __launch_bounds__(256) k_modexp(const T* __restrict__ in, T* __restrict__ out, uint64_t N,
                                                int n_exp, uint64_t base, uint64_t m,
                                                const uint64_t* __restrict__ table) {
  const uint64_t xmask = (1ull << n_exp) - 1;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N; idx += step) {
    const uint64_t x = idx & xmask, y = idx >> n_exp;
    uint64_t y_out = y;
    if (y < m) y_out = mulmod64(y, table ? __ldg(table + x) : powmod64(base, x, m), m);
    out[x | (y_out << n_exp)] = in[idx];
  }
}

// The same map as a gather over slabs, for a value register of at most
// 10 qubits and an invertible base: a CTA takes XW consecutive exponents x
// (XW amplitudes = 128 bytes of each row y) and every row, reads the slab
// into shared memory with 128-byte row reads, and writes each output row
// (x, y_out) from (x, y_out * base^-x mod N) with 128-byte row writes.  The
// scatter form above writes single amplitudes to scattered rows (partial
// DRAM sectors: 5 S of traffic for 2 S of algorithmic bytes at 26 qubits).
template <class T, int XW>
__global__ void __launch_bounds__(256) k_modexp_slab(const T* __restrict__ in, T* __restrict__ out, int n_exp,
                                                     uint32_t Y, uint32_t m, const uint64_t* __restrict__ inv_table) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* slab = reinterpret_cast<T*>(smem_raw);  // Y rows of XW amplitudes
  const uint64_t x0 = (uint64_t)blockIdx.x * XW;
  const uint32_t total = Y * XW;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    const uint32_t y = t / XW, xi = t % XW;
    slab[t] = in[(x0 + xi) | ((uint64_t)y << n_exp)];
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    const uint32_t y_out = t / XW, xi = t % XW;
    uint32_t y_in = y_out;
    if (y_out < m) y_in = (uint32_t)(((uint64_t)y_out * __ldg(inv_table + x0 + xi)) % m);
    out[(x0 + xi) | ((uint64_t)y_out << n_exp)] = slab[y_in * XW + xi];
  }
}

// a^-1 mod m (extended Euclid), or 0 when gcd(a, m) != 1
static uint64_t inverse_mod(uint64_t a, uint64_t m) {
  int64_t r0 = (int64_t)m, r1 = (int64_t)(a % m), t0 = 0, t1 = 1;
  while (r1 != 0) {
    const int64_t q = r0 / r1, r = r0 - q * r1, t = t0 - q * t1;
    r0 = r1;
    r1 = r;
    t0 = t1;
    t1 = t;
  }
  if (r0 != 1) return 0;
  return (uint64_t)((t0 % (int64_t)m + (int64_t)m) % (int64_t)m);
}

template <class T>
static bool launch_modexp_slab(State& st, int n_exp, uint64_t base, uint64_t modulus) {
  constexpr int XW = 128 / (int)sizeof(T);
  const int ny = st.n - n_exp;
  if (ny > 10 || n_exp < 7 || n_exp > 22 || modulus > (1ull << ny)) return false;
  const uint64_t inv = inverse_mod(base, modulus);
  if (inv == 0) return false;  // not a permutation: the scatter form keeps the reference's behaviour
  const uint64_t xcount = 1ull << n_exp;
  uint64_t* table = static_cast<uint64_t*>(dev_alloc(st, xcount * sizeof(uint64_t)));
  const unsigned tb = (unsigned)std::min<uint64_t>((xcount + 255) / 256, (uint64_t)st.num_sms * 16);
  k_powtable<<<tb, 256, 0, st.stream>>>(table, xcount, inv, modulus);
  BF_CUDA(cudaGetLastError());
  st.launches++;
  const uint32_t Y = 1u << ny;
  const size_t smem = (size_t)Y * XW * sizeof(T);
  static PerDeviceOnce configured;  // one per instantiation of T
  configured.run(st.device, [] {
    BF_CUDA(cudaFuncSetAttribute(k_modexp_slab<T, 128 / (int)sizeof(T)>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(1024 * 128)));
  });
  k_modexp_slab<T, XW><<<(unsigned)(xcount / XW), 256, smem, st.stream>>>(
      static_cast<const T*>(st.amp), static_cast<T*>(st.scratch), n_exp, Y, (uint32_t)modulus, table);
  BF_CUDA(cudaGetLastError());
  st.launches++;
  dev_free(st, table);  // stream-ordered: after the gather
  std::swap(st.amp, st.scratch);
  return true;
}

void launch_modexp(State& st, int n_exp, uint64_t base, uint64_t modulus) {
  if (n_exp <= 0 || n_exp >= st.n) fail(BF_EINVAL, "internal: modexp register of %d qubits", n_exp);
  if (modulus < 2) fail(BF_EINVAL, "internal: modexp modulus %llu", (unsigned long long)modulus);
  ensure_scratch(st);
  if (st.dtype == BF_C128 ? launch_modexp_slab<double2>(st, n_exp, base, modulus)
                          : launch_modexp_slab<float2>(st, n_exp, base, modulus))
    return;
  uint64_t* table = nullptr;
  const uint64_t xcount = 1ull << n_exp;
  if (n_exp <= 22) {
    table = static_cast<uint64_t*>(dev_alloc(st, xcount * sizeof(uint64_t)));
    unsigned tb = (unsigned)std::min<uint64_t>((xcount + 255) / 256, (uint64_t)st.num_sms * 16);
    k_powtable<<<tb, 256, 0, st.stream>>>(table, xcount, base, modulus);
    BF_CUDA(cudaGetLastError());
    st.launches++;
  }
  uint64_t blocks = std::min<uint64_t>((st.N + 255) / 256, (uint64_t)st.num_sms * 16);
  if (st.dtype == BF_C128)
    k_modexp<double2><<<(unsigned)blocks, 256, 0, st.stream>>>(static_cast<const double2*>(st.amp),
                                                               static_cast<double2*>(st.scratch), st.N, n_exp, base,
                                                               modulus, table);
  else
    k_modexp<float2><<<(unsigned)blocks, 256, 0, st.stream>>>(static_cast<const float2*>(st.amp),
                                                              static_cast<float2*>(st.scratch), st.N, n_exp, base,
                                                              modulus, table);
  BF_CUDA(cudaGetLastError());
  st.launches++;
  if (table) dev_free(st, table);  // stream-ordered: after the gather
  std::swap(st.amp, st.scratch);
}

}  // namespace bf

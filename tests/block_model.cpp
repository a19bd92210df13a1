// block_model.cpp — a host functional model of the tensor-core block passes,
// for the CPU tests (tests/test_block_model.py).
//
// It plans a circuit exactly as the engine does (the library's own
// lower_gate, plan_gates and plan_blocks), then executes every block pass the
// way the kernels move data: the load-phase destination table fills the
// operand slots, each block multiplies the operand rows by its matrix decoded
// from the matrix image (variant chosen by the tile's outside bits), the
// block's destination table scatters the results into the next block's
// operand slots or, after the last block, into the staging slots, and the
// staged tile is stored.  Arithmetic is complex FP64 on the decoded matrices,
// so the result checks the planner's grouping, orders, images and tables
// against the oracle without a GPU.  Passes that are not planned as blocks
// and single-gate steps are applied gate by gate.
//
// Mode digits-exact follows the complex128 digit kernel's arithmetic step
// by step instead: the state's scale from the norm before the first digit
// pass and its unit 2^-48 of it (BFGPU_DIGIT_SCALE_SHIFT raises the scale as
// it does for the kernel); per tile, the digit count (five when every warp's
// exact integer bound puts the tile's norm below 2^-9 of the scale and every
// value fits, six otherwise); each value rounded to that many balanced
// base-256 digits of the unit, exact
// integer level sums of the kept digit pairs (20 or 26), the carries with
// round-half-even, and the FP64 result after the last block, so that the
// model gives the bits the kernel gives.  It prints the passes by kind and
// the tiles run with five and with six digits.
//
//   block_model <digits|digits-exact|tf32> <ops file (binary op list)> <state in> <state out>
//
// The state files hold 2^n interleaved complex128 values.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <vector>

#include "../code_mojo_gb300/csrc/bf_internal.h"

using namespace bf;
using cd = std::complex<double>;

static uint64_t insert_zero(uint64_t x, int pos) {
  const uint64_t m = (1ull << pos) - 1;
  return ((x & ~m) << 1) | (x & m);
}

// one 2x2 gate (controls all 1) on the global state
static void apply_gate(std::vector<cd>& s, int n, int target, uint64_t cmask, const double* m) {
  const cd m00(m[0], m[1]), m01(m[2], m[3]), m10(m[4], m[5]), m11(m[6], m[7]);
  const uint64_t half = 1ull << (n - 1);
  for (uint64_t p = 0; p < half; ++p) {
    const uint64_t i0 = insert_zero(p, target), i1 = i0 | (1ull << target);
    if ((i0 & cmask) != cmask) continue;
    const cd a = s[i0], b = s[i1];
    s[i0] = m00 * a + m01 * b;
    s[i1] = m10 * a + m11 * b;
  }
}

// a dense 2^m x 2^m unitary (row-major, interleaved) on qubits t .. t+m-1
static void apply_unitary(std::vector<cd>& s, int n, int t, int m, uint64_t cmask, const double* u) {
  const int D = 1 << m;
  const uint64_t groups = 1ull << (n - m), low = (1ull << t) - 1;
  std::vector<cd> x((size_t)D);
  for (uint64_t g = 0; g < groups; ++g) {
    const uint64_t base = ((g & ~low) << m) | (g & low);
    if ((base & cmask) != cmask) continue;
    for (int c = 0; c < D; ++c) x[(size_t)c] = s[base | ((uint64_t)c << t)];
    for (int r = 0; r < D; ++r) {
      cd acc(0.0, 0.0);
      for (int c = 0; c < D; ++c) acc += cd(u[2 * (r * D + c)], u[2 * (r * D + c) + 1]) * x[(size_t)c];
      s[base | ((uint64_t)r << t)] = acc;
    }
  }
}

static std::vector<double> g_pool;  // the unitary pool of the circuit's dense unitaries

static void apply_tile_op(std::vector<cd>& s, int n, const TilePass& tp, const TileOp& t) {
  uint64_t cm = t.cmask_out;
  for (int j = 0; j < tp.K; ++j)
    if ((t.cmask_loc >> j) & 1u) cm |= 1ull << tp.q[j];
  if (t.kind == GK_UNITARY) {
    apply_unitary(s, n, tp.q[t.tloc], t.um, cm, g_pool.data() + t.uoff);
    return;
  }
  if (t.tloc >= 0) {
    apply_gate(s, n, tp.q[t.tloc], cm, t.m);
    return;
  }
  // diagonal gate whose target lies outside the tile
  const cd e0(t.m[0], t.m[1]), e1(t.m[6], t.m[7]);
  for (uint64_t i = 0; i < s.size(); ++i)
    if ((i & cm) == cm) s[i] *= ((i >> t.tglob) & 1) ? e1 : e0;
}

// the 32x32 matrix u[j][l] of one image
static void decode_image(const unsigned char* img, bool digits, cd* u) {
  for (int n = 0; n < 64; ++n)
    for (int k = 0; k < 64; k += 2) {  // c = 0: R^T[n][2l] = (Re u[j][l], Im u[j][l]) for d = 0, 1
      double v;
      if (digits) {
        const size_t off = (size_t)n * 128 + (size_t)((((2 * k) >> 4) ^ (n & 7)) << 4) + (size_t)((2 * k) & 15);
        long long V = 0;
        for (int p = 0; p < kDigits; ++p) {
          uint16_t h;
          std::memcpy(&h, img + (size_t)p * 8192 + off, 2);
          const uint32_t bits = (uint32_t)h << 16;
          float f;
          std::memcpy(&f, &bits, 4);
          V = V * 256 + (long long)f;
        }
        v = std::ldexp((double)V, -48);
      } else {
        const size_t off = (size_t)(k >> 5) * 8192 + (size_t)n * 128 + (size_t)((((k & 31) >> 2) ^ (n & 7)) << 4) +
                           (size_t)((k & 3) << 2);
        float big, small;
        std::memcpy(&big, img + off, 4);
        std::memcpy(&small, img + 16384 + off, 4);
        v = (double)big + (double)small;
      }
      const int j = n >> 1, l = k >> 1;
      if ((n & 1) == 0) u[j * 32 + l].real(v);
      else u[j * 32 + l].imag(v);
    }
}

// ---- the digit kernel's arithmetic ------------------------------------------

// round(x * 2^sh) (to nearest, ties to even, on the magnitude) as D balanced
// base-256 digits, d[D-1] the lowest
static void value_digits_of(double x, int sh, int D, int* d) {
  long long V = (long long)std::nearbyint(std::ldexp(std::fabs(x), sh));
  if (x < 0) V = -V;
  for (int j = D - 1; j >= 1; --j) {
    const long long t = ((V & 255) ^ 128) - 128;
    d[j] = (int)t;
    V = (V - t) >> 8;
  }
  d[0] = (int)V;
}

// the kernel's integer bound of x^2 in units of 2^(2e - 50), clamped to
// 2^27: (257 + the top 8 mantissa bits)^2 2^k, k = 2 (ex - e) - 2012,
// rounded up
static uint32_t sq_bound_units(double x, int e) {
  const uint32_t cap = 1u << 27;
  unsigned long long b;
  std::memcpy(&b, &x, 8);
  b &= 0x7FFFFFFFFFFFFFFFull;
  if (b == 0) return 0;
  const int ex = (int)(b >> 52);
  if (ex == 0) return 1;
  const uint32_t u = 257u + (uint32_t)((b >> 44) & 255u);
  const uint32_t u2 = u * u;
  const int k = 2 * (ex - e) - 2012;
  if (k >= 11) return cap;
  if (k >= 0) return std::min(u2 << k, cap);
  if (k <= -19) return 1;
  return (u2 + (1u << -k) - 1) >> -k;
}

// the kernel's digit count for a tile: five unless a value needs six digits
// (|x| 2^sh >= 2^39) or a warp's bound (its threads' sums, each clamped just
// below 2^27 and flagged when it reaches it) reaches 2^27
static int tile_digit_count(const std::vector<double>& vals_by_thread, int e, int sh) {
  const uint32_t cap = 1u << 27;
  bool six = false;
  const int T = kDigitThreads, per = (int)(vals_by_thread.size() / T);
  for (int w = 0; w < T / 32 && !six; ++w) {
    uint32_t ws = 0;
    for (int l = 0; l < 32; ++l) {
      uint32_t tb = 0;
      for (int k = 0; k < per; ++k) {
        const double x = vals_by_thread[(size_t)(w * 32 + l) * per + k];
        tb += sq_bound_units(x, e);
        if (std::ldexp(std::fabs(x), sh) >= 549755813888.0) six = true;  // 2^39
      }
      if (tb >= cap) six = true;
      ws += tb >= cap ? cap - 1 : tb;
    }
    if (ws >= cap) six = true;
  }
  return six ? 6 : 5;
}

// the six digits e_0..e_5 of every entry of an image's 64x64 real matrix, [n][k]
static void image_digits(const unsigned char* img, int (*b)[64][64]) {
  for (int n = 0; n < 64; ++n)
    for (int k = 0; k < 64; ++k) {
      const size_t off = (size_t)n * 128 + (size_t)((((2 * k) >> 4) ^ (n & 7)) << 4) + (size_t)((2 * k) & 15);
      for (int p = 0; p < kDigits; ++p) {
        uint16_t h;
        std::memcpy(&h, img + (size_t)p * 8192 + off, 2);
        const uint32_t bits = (uint32_t)h << 16;
        float f;
        std::memcpy(&f, &bits, 4);
        b[p][n][k] = (int)f;
      }
    }
}

static void run_digit_pass_exact(std::vector<cd>& s, int n, const TilePass& tp, const std::vector<Blk5>& blocks,
                                 const std::vector<unsigned char>& images, const std::vector<uint16_t>& offsets,
                                 int e_scale, bool five_digits, long long* tiles_by_digits) {
  const int T = kDigitThreads, E = kBlockTableEntries / T;
  std::vector<int> g_of(4096), j_of(4096);
  for (uint32_t g = 0; g < 128; ++g)
    for (uint32_t j = 0; j < 32; ++j) {
      const uint32_t slot = digit_operand_offset(g, j) >> 2;
      g_of[slot] = (int)g;
      j_of[slot] = (int)j;
    }
  uint64_t hoff[128];
  for (int h = 0; h < 128; ++h) {
    hoff[h] = 0;
    for (int j = 0; j < 7; ++j)
      if ((h >> j) & 1) hoff[h] |= 1ull << tp.q[5 + j];
  }
  struct Slot { int re[kDigits], im[kDigits]; };
  std::vector<Slot> opnd(4096), next(4096);
  std::vector<double> stage_re(4096), stage_im(4096);
  static int b[kDigits][64][64];
  std::vector<int> a((size_t)kDigits * 128 * 64);
  const uint64_t ntiles = 1ull << (n - kBlockTileQubits);
  for (uint64_t tile = 0; tile < ntiles; ++tile) {
    uint64_t obase = tile;
    for (int j = 0; j < kBlockTileQubits; ++j) obase = insert_zero(obase, tp.q[j]);
    auto gi = [&](uint32_t i) { return obase | (i & 31u) | hoff[i >> 5]; };
    const uint16_t* load = offsets.data() + (size_t)blocks[0].load_offs * kBlockTableEntries;
    // the values each thread loads, in its order: amplitudes i0, i0 + 1 of
    // i0 = (it * T + t) * 2, real then imaginary part
    const int sh = 48 - e_scale;
    std::vector<double> by_thread((size_t)T * E * 2);
    for (int t = 0; t < T; ++t)
      for (int e = 0; e < E; ++e) {
        const uint32_t i = (uint32_t)(((e >> 1) * T + t) * 2 + (e & 1));
        by_thread[((size_t)t * E + e) * 2] = s[gi(i)].real();
        by_thread[((size_t)t * E + e) * 2 + 1] = s[gi(i)].imag();
      }
    const int D = five_digits ? tile_digit_count(by_thread, e_scale, sh) : 6;
    ++tiles_by_digits[D == 5 ? 0 : 1];
    for (int t = 0; t < T; ++t)
      for (int e = 0; e < E; ++e) {
        const uint32_t i = (uint32_t)(((e >> 1) * T + t) * 2 + (e & 1));
        Slot& sl = opnd[load[t * E + e]];
        value_digits_of(s[gi(i)].real(), sh, D, sl.re);
        value_digits_of(s[gi(i)].imag(), sh, D, sl.im);
      }
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const Blk5& bk = blocks[bi];
      const bool last = bi + 1 == blocks.size();
      uint32_t v = 0;
      for (int k = 0; k < bk.nout; ++k) v |= (uint32_t)((obase >> bk.outpos[k]) & 1ull) << k;
      image_digits(images.data() + (size_t)(bk.img + v) * kDigitImageBytes, b);
      for (int slot = 0; slot < 4096; ++slot)
        for (int i = 0; i < D; ++i) {
          a[((size_t)i * 128 + g_of[slot]) * 64 + 2 * j_of[slot]] = opnd[slot].re[i];
          a[((size_t)i * 128 + g_of[slot]) * 64 + 2 * j_of[slot] + 1] = opnd[slot].im[i];
        }
      const uint16_t* dest = offsets.data() + (size_t)bk.offs * kBlockTableEntries;
      for (int t = 0; t < T; ++t)
        for (int e = 0; e < E; ++e) {
          const int w = t >> 5, lane = t & 31;
          const int g = 32 * (w & 3) + lane, jo = E * (w >> 2) + e;
          int dig[2][kDigits];
          long long V[2];
          for (int d = 0; d < 2; ++d) {
            const int nn = 2 * jo + d;
            // levels 0..D: the pairs i < D, j < 6 with i + j = level
            long long Lv[kDigits + 1];
            for (int lv = 0; lv <= D; ++lv) {
              Lv[lv] = 0;
              for (int i = 0; i <= lv && i < D; ++i) {
                const int j = lv - i;
                if (j >= kDigits) continue;
                const int* ar = &a[((size_t)i * 128 + g) * 64];
                for (int k = 0; k < 64; ++k) Lv[lv] += (long long)ar[k] * b[j][nn][k];
              }
            }
            // carries from the lowest level up, rounding half to even
            double carry = 0;
            for (int lv = D; lv >= 0; --lv) {
              const double t2 = (double)Lv[lv] + carry;
              const double q = std::nearbyint(t2 / 256.0);
              if (lv + 1 <= D - 1) dig[d][lv + 1] = (int)(t2 - 256.0 * q);
              carry = q;
            }
            dig[d][0] = (int)carry;
            V[d] = 0;
            for (int p2 = 0; p2 < D; ++p2) V[d] = V[d] * 256 + dig[d][p2];
          }
          const uint16_t to = dest[t * E + e];
          if (last) {
            stage_re[to] = std::ldexp((double)V[0], e_scale - 48);
            stage_im[to] = std::ldexp((double)V[1], e_scale - 48);
          } else {
            for (int p2 = 0; p2 < D; ++p2) {
              next[to].re[p2] = dig[0][p2];
              next[to].im[p2] = dig[1][p2];
            }
          }
        }
      if (!last) opnd.swap(next);
    }
    // the digit kernel's last table names each result's tile element
    for (uint32_t i = 0; i < 4096; ++i) s[gi(i)] = cd(stage_re[i], stage_im[i]);
  }
}

static void run_block_pass(std::vector<cd>& s, int n, const TilePass& tp, const std::vector<Blk5>& blocks,
                           const std::vector<unsigned char>& images, const std::vector<uint16_t>& offsets,
                           bool digits) {
  const int T = digits ? kDigitThreads : kBlockThreads, E = kBlockTableEntries / T;
  const uint32_t image_bytes = digits ? kDigitImageBytes : kBlockImageBytes;
  // operand slot <-> (row g, complex column j)
  std::vector<int> g_of(4096), j_of(4096);
  for (uint32_t g = 0; g < 128; ++g)
    for (uint32_t j = 0; j < 32; ++j) {
      const uint32_t slot = digits ? digit_operand_offset(g, j) >> 2 : block_operand_offset(g, j) >> 3;
      g_of[slot] = (int)g;
      j_of[slot] = (int)j;
    }
  uint64_t hoff[128];
  for (int h = 0; h < 128; ++h) {
    hoff[h] = 0;
    for (int j = 0; j < 7; ++j)
      if ((h >> j) & 1) hoff[h] |= 1ull << tp.q[5 + j];
  }
  const uint64_t ntiles = 1ull << (n - kBlockTileQubits);
  std::vector<cd> opnd(4096), next(4096), u(1024);
  for (uint64_t tile = 0; tile < ntiles; ++tile) {
    uint64_t obase = tile;
    for (int j = 0; j < kBlockTileQubits; ++j) obase = insert_zero(obase, tp.q[j]);
    auto gi = [&](uint32_t i) { return obase | (i & 31u) | hoff[i >> 5]; };
    const uint16_t* load = offsets.data() + (size_t)blocks[0].load_offs * kBlockTableEntries;
    for (int t = 0; t < T; ++t)
      for (int e = 0; e < E; ++e) {
        const uint32_t i = (uint32_t)(((e >> 1) * T + t) * 2 + (e & 1));
        opnd[load[t * E + e]] = s[gi(i)];
      }
    for (size_t b = 0; b < blocks.size(); ++b) {
      const Blk5& bk = blocks[b];
      uint32_t v = 0;
      for (int k = 0; k < bk.nout; ++k) v |= (uint32_t)((obase >> bk.outpos[k]) & 1ull) << k;
      decode_image(images.data() + (size_t)(bk.img + v) * image_bytes, digits, u.data());
      // rows of the operand: a[g][l]
      std::vector<cd> a(128 * 32), d(128 * 32);
      for (int slot = 0; slot < 4096; ++slot) a[g_of[slot] * 32 + j_of[slot]] = opnd[slot];
      for (int g = 0; g < 128; ++g)
        for (int j = 0; j < 32; ++j) {
          cd acc = 0;
          for (int l = 0; l < 32; ++l) acc += u[j * 32 + l] * a[g * 32 + l];
          d[g * 32 + j] = acc;
        }
      const uint16_t* dest = offsets.data() + (size_t)bk.offs * kBlockTableEntries;
      for (int t = 0; t < T; ++t)
        for (int e = 0; e < E; ++e) {
          const int w = t >> 5, lane = t & 31;
          const int g = 32 * (w & 3) + lane, j = E * (w >> 2) + e;
          next[dest[t * E + e]] = d[g * 32 + j];
        }
      opnd.swap(next);
    }
    // opnd now holds the results by tile element
    for (uint32_t i = 0; i < 4096; ++i) s[gi(i)] = opnd[i];
  }
}

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: block_model <digits|tf32> <ops> <state in> <state out>\n");
    return 2;
  }
  const bool exact = std::strcmp(argv[1], "digits-exact") == 0;
  const bool digits = exact || std::strcmp(argv[1], "digits") == 0;
  int e_scale = 0;  // the digit scale, from the norm before the first digit pass
  // the kernel's test overrides: the scale raised by 2^shift, five-digit
  // tiles turned off
  const char* shift_env = std::getenv("BFGPU_DIGIT_SCALE_SHIFT");
  const int scale_shift = (shift_env && *shift_env) ? std::atoi(shift_env) : 0;
  const char* five_env = std::getenv("BFGPU_DIGIT_FIVE");
  const bool five_digits = !(five_env && *five_env == '0');
  long long tiles_by_digits[2] = {0, 0};
  std::ifstream fo(argv[2], std::ios::binary);
  std::vector<char> blob((std::istreambuf_iterator<char>(fo)), {});
  bf_oplist* list = nullptr;
  if (bf_ops_deserialize(blob.data(), blob.size(), &list) != BF_OK) return 3;
  const bf_op* ops;
  int64_t nops;
  int32_t n;
  bf_oplist_view(list, &ops, &nops, &n);
  std::vector<cd> s((size_t)1 << n);
  std::ifstream fi(argv[3], std::ios::binary);
  fi.read(reinterpret_cast<char*>(s.data()), (std::streamsize)(s.size() * sizeof(cd)));
  std::vector<GateInstr> gates;
  for (int64_t i = 0; i < nops; ++i) {
    const bf_op& o = ops[i];
    if ((o.kind == BF_OP_UNITARY || o.kind == BF_OP_CUNITARY) && o.target2 >= 2 && o.target2 <= kTileUnitaryMax) {
      // a dense unitary of a fused run, as the engine plans it
      GateInstr g;
      std::memset(&g, 0, sizeof g);
      g.kind = GK_UNITARY;
      g.target = o.target;
      g.cmask = o.kind == BF_OP_CUNITARY ? o.controls : 0ull;
      g.um = o.target2;
      g.uoff = (int32_t)g_pool.size();
      g_pool.insert(g_pool.end(), o.data, o.data + 2 * ((size_t)1 << (2 * o.target2)));
      gates.push_back(g);
      continue;
    }
    if (o.kind != BF_OP_GATE) return 4;  // the model covers gates and small unitaries
    gates.push_back(lower_gate(o, BF_SPEC_ALL));
  }
  int block_passes = 0, tile_passes = 0, gate_steps = 0;
  for (const PlanStep& ps : plan_gates(n, gates, kBlockTileQubits, true, digits ? 5.0 : 3.3)) {
    if (!ps.is_tile) {
      if (ps.gate.kind == GK_UNITARY)
        apply_unitary(s, n, ps.gate.target, ps.gate.um, ps.gate.cmask, g_pool.data() + ps.gate.uoff);
      else
        apply_gate(s, n, ps.gate.target, ps.gate.cmask, ps.gate.m);
      ++gate_steps;
      continue;
    }
    std::vector<Blk5> blocks;
    std::vector<unsigned char> images;
    std::vector<uint16_t> offsets;
    if (ps.tile.K == kBlockTileQubits && ps.tile.L == kTileLowQubits &&
        plan_blocks(ps.tile, blocks, images, offsets, digits ? BLOCK_DIGITS : BLOCK_TF32, kMaxPassBlocks,
                    g_pool.data())) {
      if (exact) {
        if (e_scale == 0) {
          double nrm2 = 0;
          for (const cd& x : s) nrm2 += std::norm(x);
          int k = 0;
          std::frexp(std::sqrt(nrm2) * (1.0 + 1e-6), &k);
          e_scale = nrm2 > 0 ? k + 1 : 1;
        }
        run_digit_pass_exact(s, n, ps.tile, blocks, images, offsets, e_scale + scale_shift, five_digits,
                             tiles_by_digits);
      } else {
        run_block_pass(s, n, ps.tile, blocks, images, offsets, digits);
      }
      ++block_passes;
    } else {
      for (const TileOp& t : ps.tile.ops) apply_tile_op(s, n, ps.tile, t);
      ++tile_passes;
    }
  }
  std::ofstream fw(argv[4], std::ios::binary);
  fw.write(reinterpret_cast<const char*>(s.data()), (std::streamsize)(s.size() * sizeof(cd)));
  std::printf("%d %d %d %lld %lld\n", block_passes, tile_passes, gate_steps, tiles_by_digits[0], tiles_by_digits[1]);
  return 0;
}

// blocks.cpp — host side of the tensor-core block passes: groups the gates of
// a 12-qubit tile pass into 5-qubit blocks and builds each block's 32x32
// matrix, split and laid out for the kernel in tblock.cu.
//
// This is the GPU form of the reference's dense fusion
// (fuse_contiguous_target_pairs, transformations_fusion.mojo:539-876: runs
// of gates on neighbouring qubits multiplied into one 2^m x 2^m unitary on
// the host and applied by apply_unitary, transformations_unitary.mojo:22-75),
// widened to any 5 qubits of the tile and to gates that are not adjacent in
// the op list.
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "bf_internal.h"

namespace bf {

using cd = std::complex<double>;

static float tf32_round_host(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u = (u + 0x1000u) & 0xFFFFE000u;
  std::memcpy(&x, &u, 4);
  return x;
}

// byte offset of element (row n, column k) of a 64 x 64 FP32 K-major operand
// stored as two 128-byte-wide spans (k < 32, k >= 32) of 8 KiB, the 16-byte
// chunks of each 128-byte row swizzled by the row's low three bits
static size_t image_off(int n, int k) {
  return (size_t)(k >> 5) * 8192 + (size_t)n * 128 + (size_t)((((k & 31) >> 2) ^ (n & 7)) << 4) + (size_t)((k & 3) << 2);
}

// out_j = sum_l u[j][l] x_l on interleaved (re, im) vectors is the real
// product out = x R with R[2l+c][2j+d]:
//   R[2l][2j] = Re u[j][l]   R[2l+1][2j] = -Im u[j][l]
//   R[2l][2j+1] = Im u[j][l] R[2l+1][2j+1] = Re u[j][l]
// The kernel's B operand is R^T (rows n = output column, K-major).
void block_image(const double* u, unsigned char* img) {
  std::memset(img, 0, kBlockImageBytes);
  for (int n = 0; n < 64; ++n)
    for (int k = 0; k < 64; ++k) {
      const int j = n >> 1, d = n & 1, l = k >> 1, c = k & 1;
      const double re = u[2 * (j * 32 + l)], im = u[2 * (j * 32 + l) + 1];
      const double v = c == 0 ? (d == 0 ? re : im) : (d == 0 ? -im : re);
      const float big = tf32_round_host((float)v);
      const float small = tf32_round_host((float)(v - (double)big));
      std::memcpy(img + image_off(n, k), &big, 4);
      std::memcpy(img + 16384 + image_off(n, k), &small, 4);
    }
}

// Digits of a value v with |v| <= 1 as r = 2^-8 sum_j e_j 2^-8j: balanced
// base-256 digits e_1..e_5 in [-128, 127] and the leading e_0 in [-256, 256],
// from the nearest integer to v * 2^48.
static void value_digits(double v, int* e) {
  // v * 2^48 is exact and below 2^49 in magnitude, so adding one half is
  // exact too and truncation rounds halves away from zero (as llround)
  const double r = v * 281474976710656.0;
  const long long V = (long long)(r + (r >= 0 ? 0.5 : -0.5));
  // with W = V + 128 (1 + 2^8 + ... + 2^32) + 512 * 2^40 (nonnegative for
  // |V| <= 2^49), each of the five low bytes of W is its digit plus 128 (the
  // added 128s absorb the borrows) and the leading digit is W / 2^40 - 512
  const unsigned long long W = (unsigned long long)(V + 0x8080808080ll + (512ll << 40));
  for (int j = kDigits - 1; j >= 1; --j) e[j] = (int)((W >> (8 * (kDigits - 1 - j))) & 255u) - 128;
  e[0] = (int)(W >> 40) - 512;
}

static uint16_t bf16_of_int(int d) {  // exact for |d| <= 256
  float f = (float)d;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}

// The digit image of a 32x32 complex matrix: R^T as in block_image, each
// entry as 6 bf16 digit planes (plane j holds e_j), K-major with the
// 128-byte swizzle, 8 KiB per plane.
void block_image_digits(const double* u, unsigned char* img) {
  static const std::array<uint16_t, 513> bf16_of = [] {
    std::array<uint16_t, 513> t{};
    for (int d = -256; d <= 256; ++d) t[(size_t)(d + 256)] = bf16_of_int(d);
    return t;
  }();
  uint16_t* planes = reinterpret_cast<uint16_t*>(img);
  for (int n = 0; n < 64; ++n)
    for (int k = 0; k < 64; ++k) {
      const int j = n >> 1, d = n & 1, l = k >> 1, c = k & 1;
      const double re = u[2 * (j * 32 + l)], im = u[2 * (j * 32 + l) + 1];
      const double v = c == 0 ? (d == 0 ? re : im) : (d == 0 ? -im : re);
      int e[kDigits];
      value_digits(v, e);
      const size_t off = ((size_t)n * 128 + (size_t)((((2 * k) >> 4) ^ (n & 7)) << 4) + (size_t)((2 * k) & 15)) / 2;
      if (e[0] < -256 || e[0] > 256) fail(BF_EINVAL, "internal: block matrix entry %g outside the digit range", v);
      for (int p = 0; p < kDigits; ++p) planes[(size_t)p * 4096 + off] = bf16_of[(size_t)(e[p] + 256)];
    }
}

namespace {

struct BlockBuild {
  uint32_t qset = 0;   // local positions used by its ops
  uint64_t outs = 0;   // outside qubits its ops depend on
  std::vector<const TileOp*> ops;
};

uint32_t local_set(const TileOp& t) {
  if (t.kind == GK_UNITARY) return t.cmask_loc | (((1u << t.um) - 1u) << t.tloc);
  return t.cmask_loc | (t.tloc >= 0 ? (1u << t.tloc) : 0u);
}
uint64_t outside_set(const TileOp& t) { return t.cmask_out | (t.tloc < 0 ? (1ull << t.tglob) : 0ull); }

}  // namespace

namespace {

// Index maps of one block: the 5 block qubits T in column order J (column
// bit k = local position J[k]) and the row order R (row bit r = local
// position R[r]).
struct BlockMap {
  uint32_t T = 0;
  int J[5] = {0, 0, 0, 0, 0};
  int R[7] = {0, 0, 0, 0, 0, 0, 0};
  uint32_t dep_g(uint32_t g) const {
    uint32_t i = 0;
    for (int r = 0; r < 7; ++r) i |= ((g >> r) & 1u) << R[r];
    return i;
  }
  uint32_t dep_j(uint32_t j) const {
    uint32_t i = 0;
    for (int k = 0; k < 5; ++k) i |= ((j >> k) & 1u) << J[k];
    return i;
  }
  void ext(uint32_t i, uint32_t& g, uint32_t& j) const {
    g = 0;
    j = 0;
    for (int r = 0; r < 7; ++r) g |= ((i >> R[r]) & 1u) << r;
    for (int k = 0; k < 5; ++k) j |= ((i >> J[k]) & 1u) << k;
  }
};


// Block maps whose operand writes avoid shared-memory bank conflicts.  An
// epilogue (or the load phase) writes one word per lane; the lanes that share
// a store wavefront vary `nlanes` local positions P (the writer's row bits
// 0..nlanes-1; the load phase's positions 1..nlanes) and the word of element
// (row g, column j) lies in a bank whose index has bits j0..j(nlow-1) and
// j(nlow+m) ^ g(m) for m = 0..2 (the 128-byte swizzle XORs the row's low three
// bits onto the 16-byte chunk): 4-byte digit words, nlow = 2 and 32 lanes;
// 8-byte TF32 pairs, nlow = 1 and a half-warp of 16 lanes per wavefront.  The
// wavefront is conflict-free when the positions of P, seen from the next
// block, supply each of those bank bits once: nlow of them as its lowest
// column bits, the others as column bits nlow.. or row bits 0..2.  So each
// block takes nlow positions of the writer's P as its lowest column bits
// (padding its qubit set from P when it has fewer), the rest of P on the
// matching column or row bits, and puts the next block's new qubits among its
// own lane rows.
std::vector<BlockMap> conflict_free_maps(const std::vector<uint32_t>& qsets, int nlow, int nlanes) {
  std::vector<BlockMap> maps;
  uint32_t P = ((1u << nlanes) - 1u) << 1;  // load phase: lanes walk local positions 1..nlanes
  for (size_t b = 0; b < qsets.size(); ++b) {
    BlockMap m;
    uint32_t T = qsets[b];
    for (int pos = 0; pos < kBlockTileQubits && __builtin_popcount(T) < 5; ++pos)
      if (((P >> pos) & 1u) && !((T >> pos) & 1u) && __builtin_popcount(P & T) < nlow) T |= 1u << pos;
    for (int pos = 0; pos < kBlockTileQubits && __builtin_popcount(T) < 5; ++pos) T |= 1u << pos;
    m.T = T;
    int A[5], nA = 0, B[7], nB = 0;
    for (int pos = 0; pos < kBlockTileQubits; ++pos)
      if ((P >> pos) & 1u) {
        if ((T >> pos) & 1u) A[nA++] = pos;
        else B[nB++] = pos;
      }
    int J[5] = {-1, -1, -1, -1, -1}, R[7] = {-1, -1, -1, -1, -1, -1, -1};
    int ia = 0, ib = 0;
    for (int k = 0; k < nlow && ia < nA; ++k) J[k] = A[ia++];
    for (int m2 = 0; m2 < 3; ++m2) {  // bank bit nlow + m2: column bit nlow + m2 or row bit m2
      if (ia < nA) J[nlow + m2] = A[ia++];
      else if (ib < nB) R[m2] = B[ib++];
    }
    for (int r = 3; r < 7 && ib < nB; ++r) R[r] = B[ib++];
    uint32_t used = 0;
    for (int k = 0; k < 5; ++k)
      if (J[k] >= 0) used |= 1u << J[k];
    for (int k = 0, pos = 0; k < 5; ++k) {
      if (J[k] >= 0) continue;
      while (!((T >> pos) & 1u) || ((used >> pos) & 1u)) ++pos;
      J[k] = pos;
      used |= 1u << pos;
    }
    for (int r = 0; r < 7; ++r)
      if (R[r] >= 0) used |= 1u << R[r];
    // the next block's qubits that are not ours go to the free lane rows first
    const uint32_t next = b + 1 < qsets.size() ? qsets[b + 1] & ~T : 0u;
    for (int pass = 0; pass < 2; ++pass)
      for (int r = 0; r < 7; ++r) {
        if (R[r] >= 0 || (pass == 0 && r >= nlanes)) continue;
        for (int pos = 0; pos < kBlockTileQubits; ++pos) {
          if (((used | T) >> pos) & 1u) continue;
          if (pass == 0 && !((next >> pos) & 1u)) continue;
          R[r] = pos;
          used |= 1u << pos;
          break;
        }
      }
    std::memcpy(m.J, J, sizeof J);
    std::memcpy(m.R, R, sizeof R);
    maps.push_back(m);
    P = 0;
    for (int r = 0; r < nlanes; ++r) P |= 1u << R[r];
  }
  return maps;
}

}  // namespace

bool plan_blocks(const TilePass& tp, std::vector<Blk5>& blocks, std::vector<unsigned char>& images,
                 std::vector<uint16_t>& offsets, BlockFormat format, int max_blocks, const double* umats) {
  const uint32_t image_bytes = format == BLOCK_DIGITS ? kDigitImageBytes : kBlockImageBytes;
  // destination of complex element (g, j) of a block's operands, in the
  // units of the kernel's table (TF32: bytes / 8; digits: bytes / 4 in a plane)
  auto dest = [&](uint32_t g, uint32_t j) {
    return format == BLOCK_DIGITS ? (uint16_t)(digit_operand_offset(g, j) >> 2)
                                  : (uint16_t)(block_operand_offset(g, j) >> 3);
  };
  if (tp.K != kBlockTileQubits) return false;
  std::vector<BlockBuild> bl;
  // Each op goes into the earliest block at or after the last block that
  // shares a tile qubit with it (everything after that block acts on other
  // tile qubits, and gates on disjoint tile qubits commute for a fixed
  // assignment of the outside qubits), if the block stays within 5 tile
  // qubits and 3 outside qubits; otherwise into a new block at the end.
  for (const TileOp& t : tp.ops) {
    const uint32_t Q = local_set(t);
    const uint64_t O = outside_set(t);
    if (__builtin_popcount(Q) > 5 || __builtin_popcountll(O) > 3) return false;
    int last = -1;
    for (int b = 0; b < (int)bl.size(); ++b)
      if (bl[b].qset & Q) last = b;
    int place = -1;
    for (int b = std::max(last, 0); b < (int)bl.size(); ++b)
      if (__builtin_popcount(bl[b].qset | Q) <= 5 && __builtin_popcountll(bl[b].outs | O) <= 3) {
        place = b;
        break;
      }
    if (place < 0) {
      bl.emplace_back();
      place = (int)bl.size() - 1;
    }
    bl[place].qset |= Q;
    bl[place].outs |= O;
    bl[place].ops.push_back(&t);
  }

  // more blocks than the pass is worth: decided before any matrix is built
  if ((int)bl.size() > std::min(kMaxPassBlocks, max_blocks)) return false;
  std::vector<BlockMap> maps;
  const size_t first = blocks.size();
  {
    std::vector<uint32_t> qsets;
    for (auto& b : bl) qsets.push_back(b.qset);
    // digit words: 4 bytes, 32 lanes per wavefront; TF32 pairs: 8 bytes, 16
    maps = format == BLOCK_DIGITS ? conflict_free_maps(qsets, 2, 5) : conflict_free_maps(qsets, 1, 4);
  }
  for (size_t bi = 0; bi < bl.size(); ++bi) {
    const BlockBuild& b = bl[bi];
    const uint32_t T = maps[bi].T;
    int rank_of[kBlockTileQubits];
    for (int pos = 0; pos < kBlockTileQubits; ++pos) rank_of[pos] = -1;
    for (int k = 0; k < 5; ++k) rank_of[maps[bi].J[k]] = k;
    Blk5 d;
    std::memset(&d, 0, sizeof d);
    d.tmask = T;
    for (int q = 0; q < 64; ++q)
      if ((b.outs >> q) & 1ull) d.outpos[d.nout++] = q;
    d.img = (uint32_t)(images.size() / image_bytes);
    const int variants = 1 << d.nout;
    std::vector<cd> U(32 * 32);
    std::vector<double> flat(2 * 32 * 32);
    for (int v = 0; v < variants; ++v) {
      std::fill(U.begin(), U.end(), cd(0.0, 0.0));
      for (int i = 0; i < 32; ++i) U[i * 32 + i] = cd(1.0, 0.0);
      auto out_bit = [&](int q) {
        for (int k = 0; k < d.nout; ++k)
          if (d.outpos[k] == q) return (v >> k) & 1;
        return 0;
      };
      for (const TileOp* t : b.ops) {
        bool active = true;  // outside controls all set in this variant
        for (int q = 0; q < 64; ++q)
          if (((t->cmask_out >> q) & 1ull) && !out_bit(q)) active = false;
        if (!active) continue;
        uint32_t cb = 0;
        for (int pos = 0; pos < kBlockTileQubits; ++pos)
          if ((t->cmask_loc >> pos) & 1u) cb |= 1u << rank_of[pos];
        if (t->kind == GK_UNITARY) {
          // dense 2^um x 2^um on local bits tloc .. tloc+um-1 (unitary bit i
          // at block rank rank_of[tloc + i]): every column of U, every group
          // of rows that share the other bits and meet the controls
          if (!umats) return false;
          const int D = 1 << t->um;
          const double* um = umats + t->uoff;
          int rk[kTileUnitaryMax];
          uint32_t umask = 0;
          for (int i = 0; i < t->um; ++i) {
            rk[i] = rank_of[t->tloc + i];
            umask |= 1u << rk[i];
          }
          cd x[1 << kTileUnitaryMax];
          for (int r0 = 0; r0 < 32; ++r0) {
            if ((r0 & umask) || (r0 & cb) != cb) continue;
            auto row = [&](int a) {
              int r = r0;
              for (int i = 0; i < t->um; ++i)
                if ((a >> i) & 1) r |= 1 << rk[i];
              return r;
            };
            for (int c = 0; c < 32; ++c) {
              for (int a = 0; a < D; ++a) x[a] = U[row(a) * 32 + c];
              for (int a = 0; a < D; ++a) {
                cd acc(0.0, 0.0);
                for (int b = 0; b < D; ++b) acc += cd(um[2 * (a * D + b)], um[2 * (a * D + b) + 1]) * x[b];
                U[row(a) * 32 + c] = acc;
              }
            }
          }
          continue;
        }
        const double* m = t->m;
        if (t->tloc < 0) {  // diagonal gate on an outside target: one entry for the variant
          const cd e = out_bit(t->tglob) ? cd(m[6], m[7]) : cd(m[0], m[1]);
          for (int row = 0; row < 32; ++row)
            if ((row & cb) == cb)
              for (int c = 0; c < 32; ++c) U[row * 32 + c] *= e;
          continue;
        }
        const int tb = rank_of[t->tloc];
        const cd m00(m[0], m[1]), m01(m[2], m[3]), m10(m[4], m[5]), m11(m[6], m[7]);
        for (int r0 = 0; r0 < 32; ++r0) {
          if ((r0 >> tb) & 1) continue;
          if ((r0 & cb) != cb) continue;
          const int r1 = r0 | (1 << tb);
          for (int c = 0; c < 32; ++c) {
            const cd x0 = U[r0 * 32 + c], x1 = U[r1 * 32 + c];
            U[r0 * 32 + c] = m00 * x0 + m01 * x1;
            U[r1 * 32 + c] = m10 * x0 + m11 * x1;
          }
        }
      }
      for (int i = 0; i < 32 * 32; ++i) {
        flat[2 * i] = U[i].real();
        flat[2 * i + 1] = U[i].imag();
      }
      if (format == BLOCK_DIGITS) {
        // the digit form is exact only for entries of modulus <= 1: unitary
        // blocks (U^H U = I to 1e-12; columns as contiguous re / im vectors)
        double cre[32][32], cim[32][32];
        for (int k = 0; k < 32; ++k)
          for (int r = 0; r < 32; ++r) {
            cre[r][k] = U[k * 32 + r].real();
            cim[r][k] = U[k * 32 + r].imag();
          }
        double worst2 = 0;
        for (int r = 0; r < 32; ++r)
          for (int c = r; c < 32; ++c) {
            double ar = 0, ai = 0;
            for (int k = 0; k < 32; ++k) {
              ar += cre[r][k] * cre[c][k] + cim[r][k] * cim[c][k];
              ai += cre[r][k] * cim[c][k] - cim[r][k] * cre[c][k];
            }
            if (r == c) ar -= 1.0;
            worst2 = std::max(worst2, ar * ar + ai * ai);
          }
        if (worst2 > 1e-24) return false;
      }
      size_t at = images.size();
      images.resize(at + image_bytes);
      if (format == BLOCK_DIGITS) block_image_digits(flat.data(), images.data() + at);
      else block_image(flat.data(), images.data() + at);
    }
    blocks.push_back(d);
  }

  // destination tables: u16 per (thread, amplitude) of the format's kernel;
  // the index maps of every block as lookup tables (tile element -> row
  // and column, and back)
  struct MapLut {
    uint16_t g_of[4096], j_of[4096];
    uint16_t from_g[128], from_j[32];
  };
  std::vector<MapLut> lut(maps.size());
  for (size_t k = 0; k < maps.size(); ++k) {
    for (uint32_t i = 0; i < 4096; ++i) {
      uint32_t g, j;
      maps[k].ext(i, g, j);
      lut[k].g_of[i] = (uint16_t)g;
      lut[k].j_of[i] = (uint16_t)j;
    }
    for (uint32_t g = 0; g < 128; ++g) lut[k].from_g[g] = (uint16_t)maps[k].dep_g(g);
    for (uint32_t j = 0; j < 32; ++j) lut[k].from_j[j] = (uint16_t)maps[k].dep_j(j);
  }
  const int T = format == BLOCK_DIGITS ? kDigitThreads : kBlockThreads;
  const int E = kBlockTableEntries / T;
  const size_t table = (size_t)kBlockTableEntries;
  auto new_table = [&]() {
    size_t at = offsets.size();
    offsets.resize(at + table);
    return at;
  };
  {  // load phase: thread t, element e = 2 * it + h holds tile element (it * T + t) * 2 + h
    size_t at = new_table();
    blocks[first].load_offs = (uint32_t)(at / table);
    for (int t = 0; t < T; ++t)
      for (int e = 0; e < E; ++e) {
        const uint32_t i = (uint32_t)(((e >> 1) * T + t) * 2 + (e & 1));
        offsets[at + (size_t)t * E + e] = dest(lut[0].g_of[i], lut[0].j_of[i]);
      }
  }
  for (size_t k = 0; k < maps.size(); ++k) {
    // epilogue: thread t reads D row 32 (warp % 4) + lane, columns of
    // complex elements E (warp / 4) + e
    size_t at = new_table();
    blocks[first + k].offs = (uint32_t)(at / table);
    for (int t = 0; t < T; ++t)
      for (int e = 0; e < E; ++e) {
        const uint32_t w = (uint32_t)t >> 5, lane = (uint32_t)t & 31u;
        const uint32_t g = 32u * (w & 3u) + lane, j = (uint32_t)E * (w >> 2) + (uint32_t)e;
        const uint32_t i = (uint32_t)lut[k].from_g[g] | lut[k].from_j[j];
        uint16_t v;
        if (k + 1 < maps.size()) {
          v = dest(lut[k + 1].g_of[i], lut[k + 1].j_of[i]);
        } else {
          // after the last block: the tile element itself (both kernels
          // store their results straight to the state)
          v = (uint16_t)i;
        }
        offsets[at + (size_t)t * E + e] = v;
      }
  }
  return true;
}

}  // namespace bf

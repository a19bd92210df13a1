// planner.cpp — host-side lowering, validation and tile-pass planning.
// No device code: everything here runs (and is tested) without a GPU.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "bf_internal.h"

namespace bf {

void fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw Error{code, buf};
}

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(e == cudaErrorMemoryAllocation ? BF_ENOMEM : BF_ECUDA, "%s: %s", what, cudaGetErrorString(e));
  }
}

int current_device() {
  int dev = 0;
  BF_CUDA(cudaGetDevice(&dev));
  return dev;
}

// ---- validation: validate_circuit (executors.mojo:78-185) ----------------
static void check_qubit(int idx, int n, const char* label) {
  if (idx < 0 || idx >= n) fail(BF_EINVAL, "%s out of bounds: %d", label, idx);
}

void validate_ops(int n, const bf_op* ops, int64_t nops) {
  if (nops < 0) fail(BF_EINVAL, "negative op count");
  if (nops > 0 && ops == nullptr) fail(BF_EINVAL, "ops is null");
  for (int64_t i = 0; i < nops; ++i) {
    const bf_op& o = ops[i];
    switch (o.kind) {
      case BF_OP_GATE: {
        check_qubit(o.target, n, "Target");
        if (o.gate < 0 || o.gate > BF_GATE_CUSTOM) fail(BF_EINVAL, "Unknown gate kind: %d", o.gate);
        if (n < 64 && (o.controls >> n)) fail(BF_EINVAL, "Control out of bounds: %d", 63 - __builtin_clzll(o.controls));
        if (o.ncontrols < 0 || __builtin_popcountll(o.controls) != o.ncontrols)
          fail(BF_EINVAL, "Gate control kind mismatch: expected %d controls, mask holds %d", o.ncontrols,
               __builtin_popcountll(o.controls));
        if (o.flags & BF_OPF_FUSE_WITH_NEXT) {
          if (i + 1 >= nops || ops[i + 1].kind != BF_OP_GATE)
            fail(BF_EINVAL, "fused pair: the gate flagged FUSE_WITH_NEXT must be followed by a gate");
        }
        break;
      }
      case BF_OP_SWAP:
      case BF_OP_CSWAP:
        check_qubit(o.target, n, "Target");
        check_qubit(o.target2, n, "Target");
        break;
      case BF_OP_QREV:
      case BF_OP_BITREV:
      case BF_OP_PERMUTE:
      case BF_OP_GROVER_DIFFUSER:
      case BF_OP_GROVER_INVERSION0: {
        if (o.nqubits < 0 || (o.nqubits > 0 && o.qubits == nullptr)) fail(BF_EINVAL, "qubit list is null");
        for (int64_t k = 0; k < o.nqubits; ++k) check_qubit(o.qubits[k], n, "Target");
        if (o.kind == BF_OP_BITREV || o.kind == BF_OP_GROVER_DIFFUSER || o.kind == BF_OP_GROVER_INVERSION0) {
          uint64_t seen = 0;
          for (int64_t k = 0; k < o.nqubits; ++k) {
            if ((seen >> o.qubits[k]) & 1) fail(BF_EINVAL, "Duplicate target: %d", o.qubits[k]);
            seen |= 1ull << o.qubits[k];
          }
        }
        if (o.kind == BF_OP_PERMUTE && o.nqubits != 0) {
          if (o.nqubits != n) fail(BF_EINVAL, "Permutation size mismatch: %lld", (long long)o.nqubits);
          uint64_t seen = 0;
          for (int64_t k = 0; k < o.nqubits; ++k) {
            if ((seen >> o.qubits[k]) & 1) fail(BF_EINVAL, "Duplicate permutation value: %d", o.qubits[k]);
            seen |= 1ull << o.qubits[k];
          }
        }
        break;
      }
      case BF_OP_MODEXP:
      case BF_OP_MODEXP_INV: {  // apply_modexp(_inverse) checks (algos/shor.mojo:60-76, 103-119)
        const char* name = o.kind == BF_OP_MODEXP ? "MOD_EXP" : "MOD_EXP_INV";
        if (o.nqubits < 4 || !o.data) fail(BF_EINVAL, "%s expects 4 parameters: n_exp, n_value, a, N", name);
        for (int k = 0; k < 4; ++k)
          if (o.data[k] != std::floor(o.data[k]) || std::fabs(o.data[k]) > 9.0e15)
            fail(BF_EINVAL, "%s parameters must be integers", name);
        const int64_t ne = (int64_t)o.data[0], nv = (int64_t)o.data[1], a = (int64_t)o.data[2], N = (int64_t)o.data[3];
        if (ne <= 0 || nv <= 0) fail(BF_EINVAL, "%s expects positive register sizes", name);
        if (N <= 1) fail(BF_EINVAL, "%s expects modulus > 1", name);
        int64_t x = ((a % N) + N) % N, y = N;  // gcd(a, N)
        while (y != 0) {
          int64_t t = x % y;
          x = y;
          y = t;
        }
        if (x != 1) fail(BF_EINVAL, "%s expects a and modulus to be coprime", name);
        if (ne + nv != n) fail(BF_EINVAL, "State size mismatch for %s", name);
        break;
      }
      case BF_OP_CLASSICAL_ORACLE: {
        if (o.nqubits < 0 || (o.nqubits > 0 && o.data == nullptr)) fail(BF_EINVAL, "oracle index list is null");
        double N = std::ldexp(1.0, n);
        for (int64_t k = 0; k < o.nqubits; ++k) {
          double v = o.data[k];
          if (!(v >= 0 && v < N) || v != std::floor(v)) fail(BF_EINVAL, "Oracle index out of range: %.17g", v);
        }
        break;
      }
      case BF_OP_MEASURE: {
        if (o.nqubits < 0 || (o.nqubits > 0 && o.qubits == nullptr)) fail(BF_EINVAL, "qubit list is null");
        uint64_t seen = 0;
        for (int64_t k = 0; k < o.nqubits; ++k) {
          check_qubit(o.qubits[k], n, "Target");
          if ((seen >> o.qubits[k]) & 1) fail(BF_EINVAL, "Duplicate target: %d", o.qubits[k]);
          seen |= 1ull << o.qubits[k];
          if (o.data && !(o.data[k] == -1.0 || o.data[k] == 0.0 || o.data[k] == 1.0))
            fail(BF_EINVAL, "Measurement values must be -1 (free), 0 or 1");
        }
        break;
      }
      case BF_OP_UNITARY:
      case BF_OP_CUNITARY: {
        int m = o.target2;
        if (m > 0 && (o.target < 0 || o.target + m > n)) fail(BF_EINVAL, "Target range out of bounds");
        if (o.kind == BF_OP_CUNITARY) {
          if (o.ncontrols != 1 || __builtin_popcountll(o.controls) != 1)
            fail(BF_EINVAL, "Controlled unitary expects exactly one control");
          int c = __builtin_ctzll(o.controls);
          check_qubit(c, n, "Control");
          if (m > 0 && c >= o.target && c < o.target + m) fail(BF_EINVAL, "Control overlaps target range");
        }
        if (m > 0 && o.data == nullptr) fail(BF_EINVAL, "Unitary data is null");
        break;
      }
      default:
        fail(BF_EINVAL, "Unknown transformation type: %d", o.kind);
    }
  }
}

// ---- lowering: GateInfo kind/arg -> matrix (gates.mojo:5-61) ---------------
static void gate_matrix(int kind, double a, const double* mat, double* m) {
  const double s = std::sqrt(0.5);
  auto set = [&](double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7) {
    m[0] = a0; m[1] = a1; m[2] = a2; m[3] = a3; m[4] = a4; m[5] = a5; m[6] = a6; m[7] = a7;
  };
  switch (kind) {
    case BF_GATE_H: set(s, 0, s, 0, s, 0, -s, 0); break;
    case BF_GATE_P: set(1, 0, 0, 0, 0, 0, std::cos(a), std::sin(a)); break;
    case BF_GATE_X: set(0, 0, 1, 0, 1, 0, 0, 0); break;
    case BF_GATE_Y: set(0, 0, 0, -1, 0, 1, 0, 0); break;
    case BF_GATE_Z: set(1, 0, 0, 0, 0, 0, -1, 0); break;
    case BF_GATE_RX: set(std::cos(a / 2), 0, 0, -std::sin(a / 2), 0, -std::sin(a / 2), std::cos(a / 2), 0); break;
    case BF_GATE_RY: set(std::cos(a / 2), 0, -std::sin(a / 2), 0, std::sin(a / 2), 0, std::cos(a / 2), 0); break;
    case BF_GATE_RZ: set(std::cos(a / 2), -std::sin(a / 2), 0, 0, 0, 0, std::cos(a / 2), std::sin(a / 2)); break;
    default: std::memcpy(m, mat, 8 * sizeof(double)); break;
  }
}

static void split_pairs(GateInstr& g) {
  for (int i = 0; i < 8; ++i) {
    float hi = (float)g.m[i];
    g.mhl[2 * i] = hi;
    g.mhl[2 * i + 1] = (float)(g.m[i] - (double)hi);
  }
}

// Chooses the cheapest kernel form that computes the same matrix: the
// reference's specialised H/P/X/RY/CP/CX/CRY kernels (transformations_scalar.mojo
// :178-566) plus diagonal and permutation detection for any other kind.
GateInstr lower_gate(const bf_op& o, uint32_t spec) {
  GateInstr g;
  std::memset(&g, 0, sizeof g);
  g.target = o.target;
  g.cmask = o.controls;
  gate_matrix(o.gate, o.arg, o.mat, g.m);
  const double* m = g.m;
  const bool ctl0 = o.ncontrols == 0, ctl1 = o.ncontrols == 1;
  bool off_zero = m[2] == 0 && m[3] == 0 && m[4] == 0 && m[5] == 0;
  bool diag_zero = m[0] == 0 && m[1] == 0 && m[6] == 0 && m[7] == 0;
  if (o.gate == BF_GATE_H && ctl0 && (spec & BF_SPEC_H)) {
    g.kind = GK_H;
  } else if (diag_zero && m[2] == 1 && m[3] == 0 && m[4] == 1 && m[5] == 0) {
    g.kind = GK_SWAP;  // X, CX, CCX, MCX (and a CUSTOM X)
  } else if (off_zero && m[0] == 1 && m[1] == 0) {
    g.kind = GK_PHASE;  // P, Z, CP, CZ, MCP
  } else if (off_zero) {
    g.kind = GK_DIAG;  // RZ and other diagonals
  } else if ((o.gate == BF_GATE_RY && ((ctl0 && (spec & BF_SPEC_RY)) || (ctl1 && (spec & BF_SPEC_CRY)))) ||
             (m[1] == 0 && m[3] == 0 && m[5] == 0 && m[7] == 0 && m[0] == m[6] && m[2] == -m[4])) {
    g.kind = GK_RY;  // real rotation [[c, -s], [s, c]]
  } else {
    g.kind = m[1] == 0 ? GK_DENSE_R : GK_DENSE;  // U3: m00 = cos(theta/2) is real
  }
  split_pairs(g);
  return g;
}

double gate_bytes_fraction(const GateInstr& g) {
  int c = __builtin_popcountll(g.cmask);
  double f = (g.kind == GK_PHASE) ? 1.0 : 2.0;  // P touches half the amplitudes
  return f / std::ldexp(1.0, c);
}

// ---- tile-pass planning -----------------------------------------------------
// Greedy, order-respecting grouping.  Scanning the remaining gates in order,
// a gate joins the current pass if it commutes with every gate deferred so
// far and its target is (or can become) a tile qubit; otherwise it is
// deferred.  Two gates commute when, on every qubit they share, both act
// diagonally (controls always do; a diagonal gate does on its target).
static TileOp to_tile_op(const GateInstr& g, const int* loc_of) {
  TileOp t;
  std::memset(&t, 0, sizeof t);
  t.kind = g.kind;
  t.tglob = g.target;
  t.tloc = loc_of[g.target];
  t.um = g.um;
  t.uoff = g.uoff;
  for (int b = 0; b < 64; ++b) {
    if (!((g.cmask >> b) & 1)) continue;
    if (loc_of[b] >= 0) t.cmask_loc |= 1u << loc_of[b];
    else t.cmask_out |= 1ull << b;
  }
  std::memcpy(t.m, g.m, sizeof t.m);
  std::memcpy(t.mhl, g.mhl, sizeof t.mhl);
  return t;
}

// The work (per-gate bytes, in units of S) a tile pass over the qubit set
// inQ takes from the remaining gates: a gate joins when its non-diagonal
// target is in the set and it commutes with every gate deferred before it.
static double pass_work(const std::vector<const GateInstr*>& remaining, uint64_t inQ, uint64_t all) {
  uint64_t blockedX = 0, blockedAll = 0;
  double w = 0;
  for (const GateInstr* g : remaining) {
    const uint64_t Xg = gate_xmask(*g);
    const uint64_t Ag = gate_amask(*g);
    if (!(Xg & blockedAll) && !(Ag & blockedX) && !(Xg & ~inQ)) {
      w += gate_bytes_fraction(*g);
    } else {
      blockedX |= Xg;
      blockedAll |= Ag;
      if ((blockedX & all) == all) break;  // every later gate meets a deferred one
    }
  }
  return w;
}

// The tensor-core blocks a pass over inQ would need: its gates grouped into
// blocks of at most 5 tile qubits and 3 outside qubits, each gate into the
// earliest block at or after the last one that shares a tile qubit with it
// (the grouping of plan_blocks); large when a gate cannot be placed.
static int pass_blocks(const std::vector<const GateInstr*>& remaining, uint64_t inQ, uint64_t all) {
  uint64_t blockedX = 0, blockedAll = 0;
  uint64_t bq[64], bo[64];
  int nb = 0;
  for (const GateInstr* g : remaining) {
    const uint64_t Xg = gate_xmask(*g);
    const uint64_t Ag = gate_amask(*g);
    if ((Xg & blockedAll) || (Ag & blockedX) || (Xg & ~inQ)) {
      blockedX |= Xg;
      blockedAll |= Ag;
      if ((blockedX & all) == all) break;
      continue;
    }
    const uint64_t Q = Ag & inQ, O = Ag & ~inQ;
    if (__builtin_popcountll(Q) > 5 || __builtin_popcountll(O) > 3) return 1000;
    int last = -1;
    for (int b = 0; b < nb; ++b)
      if (bq[b] & Q) last = b;
    int place = -1;
    for (int b = std::max(last, 0); b < nb; ++b)
      if (__builtin_popcountll(bq[b] | Q) <= 5 && __builtin_popcountll(bo[b] | O) <= 3) {
        place = b;
        break;
      }
    if (place < 0) {
      if (nb == 64) return 1000;
      bq[nb] = 0;
      bo[nb] = 0;
      place = nb++;
    }
    bq[place] |= Q;
    bo[place] |= O;
  }
  return nb;
}

// The CUDA-core tile kernel's cost of the gates a pass over inQ takes, in
// dense-gate units (dense 1, exchange 0.5, phase 0.4, other diagonal 0.6, a
// diagonal gate on an outside target 0.4, an m-qubit unitary 2^(m-1): its
// 2^m complex products per amplitude against a dense gate's 2).
static double pass_core_units(const std::vector<const GateInstr*>& remaining, uint64_t inQ, uint64_t all) {
  uint64_t blockedX = 0, blockedAll = 0;
  double u = 0;
  for (const GateInstr* g : remaining) {
    const uint64_t tb = 1ull << g->target;
    const uint64_t Xg = gate_xmask(*g);
    const uint64_t Ag = gate_amask(*g);
    if ((Xg & blockedAll) || (Ag & blockedX) || (Xg & ~inQ)) {
      blockedX |= Xg;
      blockedAll |= Ag;
      if ((blockedX & all) == all) break;
      continue;
    }
    if (g->kind == GK_UNITARY) u += (double)(1 << (g->um - 1));
    else if (!(tb & inQ)) u += 0.4;
    else if (g->kind == GK_SWAP) u += 0.5;
    else if (g->kind == GK_PHASE) u += 0.4;
    else if (g->kind == GK_DIAG) u += 0.6;
    else u += 1.0;
  }
  return u;
}

std::vector<PlanStep> plan_gates(int n, const std::vector<GateInstr>& gates, int K, bool allow_single,
                                 double block_units, double pass_cost, bool keep_wide_unitaries) {
  std::vector<PlanStep> steps;
  if (gates.empty()) return steps;
  K = std::max(1, std::min(K, std::min(n, kMaxTileQubits)));
  // Low qubits always in the tile; when the tile is narrower than the state
  // at least one slot stays free, so every pass can take the next gate.
  const int L = (K >= n) ? std::min(K, kTileLowQubits) : std::min(K - 1, kTileLowQubits);
  const uint64_t low = (L >= 64) ? ~0ull : ((1ull << L) - 1);
  std::vector<const GateInstr*> remaining;
  for (auto& g : gates) remaining.push_back(&g);
  while (!remaining.empty()) {
    // the tile's qubits: first the targets in order of appearance among the
    // gates that could still join (first come), then single swaps of a chosen
    // qubit for another target while that improves the pass: more work, or
    // for passes that run as tensor-core blocks more work per unit of time
    // (a pass costs about as much as pass_cost blocks besides its blocks)
    uint64_t inQ = low;
    int nQ = L;
    // the qubits the remaining gates touch: once the deferred gates act
    // non-diagonally on all of them, no later gate can join a pass
    uint64_t all = 0;
    for (const GateInstr* g : remaining) all |= gate_amask(*g);
    {
      uint64_t blockedX = 0, blockedAll = 0;
      for (const GateInstr* g : remaining) {
        const uint64_t Xg = gate_xmask(*g);
        const uint64_t Ag = gate_amask(*g);
        bool fits = false;
        if (!(Xg & blockedAll) && !(Ag & blockedX)) {
          const int extra = __builtin_popcountll(Xg & ~inQ);
          if (extra == 0) {
            fits = true;
          } else if (nQ + extra <= K) {
            inQ |= Xg;
            nQ += extra;
            fits = true;
          }
        }
        if (!fits) {
          blockedX |= Xg;
          blockedAll |= Ag;
          if ((blockedX & all) == all) break;
        }
      }
    }
    if (nQ == K && K < n) {
      uint64_t targets = 0;
      for (const GateInstr* g : remaining) targets |= gate_xmask(*g);
      auto search = [&](uint64_t start, auto score) {
        uint64_t set = start;
        double best = score(set);
        for (int round = 0; round < 8; ++round) {
          uint64_t best_set = set;
          for (int a = 0; a < n; ++a) {
            if (!((set >> a) & 1) || ((low >> a) & 1)) continue;
            for (int b = 0; b < n; ++b) {
              if (((set >> b) & 1) || !((targets >> b) & 1)) continue;
              const uint64_t cand = (set & ~(1ull << a)) | (1ull << b);
              const double w = score(cand);
              if (w > best + 1e-9) {
                best = w;
                best_set = cand;
              }
            }
          }
          if (best_set == set) break;
          set = best_set;
        }
        return set;
      };
      auto work = [&](uint64_t set) { return pass_work(remaining, set, all); };
      const uint64_t start = inQ;
      bool chosen = false;
      const uint64_t by_work = search(start, work);
      if (block_units > 0) {
        // Passes that may run as tensor-core blocks: the tile that takes the
        // most work per unit of time as blocks (a pass costs about pass_cost
        // blocks besides its blocks), kept when its blocks beat the CUDA-core kernel
        // on the same gates and it does more work per unit of time than the
        // most-work tile does on the CUDA cores (same pass cost; a block
        // costs block_units dense gates).
        auto block_rate = [&](uint64_t c) { return work(c) / (pass_cost + pass_blocks(remaining, c, all)); };
        const uint64_t set = search(start, block_rate);
        const double core = pass_core_units(remaining, set, all);
        const double core_rate = work(by_work) / (pass_cost + pass_core_units(remaining, by_work, all) / block_units);
        if ((double)pass_blocks(remaining, set, all) * block_units < core && block_rate(set) >= core_rate) {
          inQ = set;
          chosen = true;
        }
      }
      if (!chosen) inQ = by_work;
    }
    std::vector<const GateInstr*> taken, deferred;
    {
      uint64_t blockedX = 0, blockedAll = 0;
      size_t i = 0;
      for (; i < remaining.size(); ++i) {
        const GateInstr* g = remaining[i];
        const uint64_t Xg = gate_xmask(*g);
        const uint64_t Ag = gate_amask(*g);
        if (!(Xg & blockedAll) && !(Ag & blockedX) && !(Xg & ~inQ)) {
          taken.push_back(g);
        } else {
          deferred.push_back(g);
          blockedX |= Xg;
          blockedAll |= Ag;
          if ((blockedX & all) == all) {
            ++i;
            break;
          }
        }
      }
      deferred.insert(deferred.end(), remaining.begin() + (std::ptrdiff_t)i, remaining.end());
    }
    if (taken.empty()) fail(BF_EINVAL, "internal: tile planner made no progress (K=%d, n=%d)", K, n);
    double single_bytes = 0;
    bool wide_unitary = false;
    for (const GateInstr* g : taken) {
      single_bytes += gate_bytes_fraction(*g);
      wide_unitary |= g->kind == GK_UNITARY && g->um >= 4;
    }
    // a tile pass moves 2S; the gates on their own move no more.  With
    // keep_wide_unitaries a unitary of 4 or 5 qubits stays a pass (one
    // tensor-core block): on its own, a double-float kernel does 2^m complex
    // products per amplitude (at 26 qubits a lone 5-qubit unitary took 8.2
    // ms that way and 1.9 ms as a digit pass; a 3-qubit one 1.8 ms either
    // way, so it keeps its kernel)
    if (allow_single && single_bytes <= 2.0 && !(wide_unitary && keep_wide_unitaries)) {
      for (const GateInstr* g : taken) {
        PlanStep st;
        st.is_tile = false;
        st.gate = *g;
        steps.push_back(st);
      }
    } else {
      // pad the tile with the lowest unused qubits up to K
      for (int q = 0; q < n && nQ < K; ++q)
        if (!((inQ >> q) & 1)) {
          inQ |= 1ull << q;
          nQ++;
        }
      PlanStep st;
      st.is_tile = true;
      st.tile.K = nQ;
      st.tile.L = L;
      int loc_of[64];
      for (int q = 0; q < 64; ++q) loc_of[q] = -1;
      int j = 0;
      for (int q = 0; q < n; ++q)
        if ((inQ >> q) & 1) {
          st.tile.q[j] = q;
          loc_of[q] = j;
          ++j;
        }
      for (const GateInstr* g : taken) st.tile.ops.push_back(to_tile_op(*g, loc_of));
      steps.push_back(std::move(st));
    }
    remaining.swap(deferred);
  }
  return steps;
}

}  // namespace bf

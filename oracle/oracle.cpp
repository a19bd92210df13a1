// oracle.cpp — CPU restatement of Butterfly's SCALAR strategy and a chunked
// multi-threaded port of its SIMD_PARALLEL strategy.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and
// bench.py's CPU legs as the checker / timed baseline, never by the engine.
// Built with -ffp-contract=off so that every expression rounds exactly as
// written, on x86-64 and on aarch64 alike.
//
// Each function names the reference code (paths inside learnqc/code_mojo)
// whose loop order and arithmetic it restates.

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

struct Cplx {
  double re, im;
};
typedef Cplx Gate2[2][2];

struct OrError {
  std::string msg;
  int code;
};

[[noreturn]] void fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw OrError{buf, code};
}

struct St {
  int n;
  size_t N;
  double* re;
  double* im;
};

struct Ctx {
  uint32_t spec;   // BF_SPEC_* (ExecContext.simd_use_specialized_*)
  int threads;     // worker threads of the parallel port
  int chunks;      // work items per gate (get_num_chunks)
  int strategy;
};

// ---- gates (butterfly/core/gates.mojo:5-61, cis utils/common.mojo:8-9) ----
Cplx cis(double t) { return Cplx{cos(t), sin(t)}; }

void gate_matrix(int kind, double a, const double* mat, Gate2 g) {
  const double s = sqrt(0.5);  // sq_half_re, types.mojo:23
  auto set = [&](Cplx a00, Cplx a01, Cplx a10, Cplx a11) {
    g[0][0] = a00; g[0][1] = a01; g[1][0] = a10; g[1][1] = a11;
  };
  switch (kind) {
    case BF_GATE_H: set({s, 0}, {s, 0}, {s, 0}, {-s, 0}); break;
    case BF_GATE_P: set({1, 0}, {0, 0}, {0, 0}, cis(a)); break;
    case BF_GATE_X: set({0, 0}, {1, 0}, {1, 0}, {0, 0}); break;
    case BF_GATE_Y: set({0, 0}, {0, -1}, {0, 1}, {0, 0}); break;
    case BF_GATE_Z: set({1, 0}, {0, 0}, {0, 0}, {-1, 0}); break;
    case BF_GATE_RX:
      set({cos(a / 2), 0}, {0, -sin(a / 2)}, {0, -sin(a / 2)}, {cos(a / 2), 0});
      break;
    case BF_GATE_RY:
      set({cos(a / 2), 0}, {-sin(a / 2), 0}, {sin(a / 2), 0}, {cos(a / 2), 0});
      break;
    case BF_GATE_RZ:
      set({cos(a / 2), -sin(a / 2)}, {0, 0}, {0, 0}, {cos(a / 2), sin(a / 2)});
      break;
    case BF_GATE_CUSTOM:
      set({mat[0], mat[1]}, {mat[2], mat[3]}, {mat[4], mat[5]}, {mat[6], mat[7]});
      break;
    default: fail(BF_EINVAL, "Unknown gate kind: %d", kind);
  }
}

// ---- parallel helper: the chunking of transformations_simd_parallel.mojo:
// min(chunks, blocks) workers, each owning contiguous blocks (:13-37). -------
template <class F>
void for_blocks(const Ctx& c, size_t total_blocks, F&& body) {
  if (total_blocks == 0) return;
  if (c.strategy != OR_SIMD_PARALLEL) {
    body(0, total_blocks);
    return;
  }
  size_t items = (size_t)std::max(1, c.chunks);
  size_t workers = std::min(items, total_blocks);
  size_t per = std::max<size_t>(1, total_blocks / items);
  if (workers <= 1) {
    body(0, total_blocks);
    return;
  }
  std::vector<std::thread> pool;
  size_t nthreads = std::min<size_t>(workers, (size_t)std::max(1, c.threads));
  // items are distributed round-robin over the threads (parallelize's pool)
  for (size_t t = 0; t < nthreads; ++t) {
    pool.emplace_back([&, t]() {
      for (size_t w = t; w < workers; w += nthreads) {
        size_t b0 = w * per;
        size_t b1 = (w == workers - 1) ? total_blocks : (w + 1) * per;
        body(b0, b1);
      }
    });
  }
  for (auto& th : pool) th.join();
}

// ---- process_pair_scalar (transformations_scalar.mojo:10-40) -------------
inline void process_pair(St& s, const Gate2 g, size_t k0, size_t k1) {
  double u_re = s.re[k0], u_im = s.im[k0], v_re = s.re[k1], v_im = s.im[k1];
  s.re[k0] = u_re * g[0][0].re - u_im * g[0][0].im + v_re * g[0][1].re - v_im * g[0][1].im;
  s.im[k0] = u_re * g[0][0].im + u_im * g[0][0].re + v_re * g[0][1].im + v_im * g[0][1].re;
  s.re[k1] = u_re * g[1][0].re - u_im * g[1][0].im + v_re * g[1][1].re - v_im * g[1][1].im;
  s.im[k1] = u_re * g[1][0].im + u_im * g[1][0].re + v_re * g[1][1].im + v_im * g[1][1].re;
}

// Pair enumeration.  SCALAR walks j in [0, N/2) with idx = 2j - r, r wrapping
// at stride (transformations_scalar.mojo:111-117); the parallel port walks
// contiguous 2*stride blocks (transformations_simd_parallel.mojo:341-357).
// Both visit every pair base (bit `target` clear) exactly once.
template <class F>
void for_pairs(St& s, const Ctx& c, int target, F&& f) {
  size_t stride = (size_t)1 << target;
  if (c.strategy == OR_SCALAR) {
    size_t r = 0;
    for (size_t j = 0; j < s.N / 2; ++j) {
      size_t idx = 2 * j - r;
      f(idx, idx + stride);
      r += 1;
      if (r == stride) r = 0;
    }
    return;
  }
  for_blocks(c, s.N / (2 * stride), [&](size_t b0, size_t b1) {
    for (size_t b = b0; b < b1; ++b) {
      size_t k = b * 2 * stride;
      for (size_t m = 0; m < stride; ++m) f(k + m, k + m + stride);
    }
  });
}

inline bool bit_set(size_t m, int k) { return (m >> k) & 1; }

// transform_h_scalar (:233-286)
void transform_h(St& s, const Ctx& c, int t) {
  const double sq_half = 0.7071067811865476;
  for_pairs(s, c, t, [&](size_t i, size_t j) {
    double u_re = s.re[i], u_im = s.im[i], v_re = s.re[j], v_im = s.im[j];
    s.re[i] = (u_re + v_re) * sq_half;
    s.im[i] = (u_im + v_im) * sq_half;
    s.re[j] = (u_re - v_re) * sq_half;
    s.im[j] = (u_im - v_im) * sq_half;
  });
}

// transform_p_scalar (:289-336)
void transform_p(St& s, const Ctx& c, int t, double theta) {
  double cs = cos(theta), sn = sin(theta);
  for_pairs(s, c, t, [&](size_t, size_t j) {
    double v_re = s.re[j], v_im = s.im[j];
    s.re[j] = v_re * cs - v_im * sn;
    s.im[j] = v_re * sn + v_im * cs;
  });
}

// transform_x_scalar (:178-230)
void transform_x(St& s, const Ctx& c, int t) {
  for_pairs(s, c, t, [&](size_t i, size_t j) {
    std::swap(s.re[i], s.re[j]);
    std::swap(s.im[i], s.im[j]);
  });
}

// transform_ry_scalar (:339-394)
void transform_ry(St& s, const Ctx& c, int t, double theta) {
  double cs = cos(theta / 2), sn = sin(theta / 2);
  for_pairs(s, c, t, [&](size_t i, size_t j) {
    double u_re = s.re[i], u_im = s.im[i], v_re = s.re[j], v_im = s.im[j];
    s.re[i] = u_re * cs - v_re * sn;
    s.im[i] = u_im * cs - v_im * sn;
    s.re[j] = u_re * sn + v_re * cs;
    s.im[j] = u_im * sn + v_im * cs;
  });
}

// transform_scalar (:63-117): specialised dispatch, else the generic pair.
void transform(St& s, const Ctx& c, int t, const Gate2 g, int kind, double arg) {
  if (kind == BF_GATE_H && (c.spec & BF_SPEC_H)) return transform_h(s, c, t);
  if (kind == BF_GATE_P && (c.spec & BF_SPEC_P)) return transform_p(s, c, t, arg);
  if (kind == BF_GATE_X && (c.spec & BF_SPEC_X)) return transform_x(s, c, t);
  if (kind == BF_GATE_RY && (c.spec & BF_SPEC_RY)) return transform_ry(s, c, t, arg);
  for_pairs(s, c, t, [&](size_t i, size_t j) { process_pair(s, g, i, j); });
}

// c_transform_scalar (:120-175) and its specialised CP/CX/CRY (:397-566)
void c_transform(St& s, const Ctx& c, int ctl, int t, const Gate2 g, int kind,
                 double arg) {
  if (kind == BF_GATE_P && (c.spec & BF_SPEC_CP)) {
    double cs = cos(arg), sn = sin(arg);
    for_pairs(s, c, t, [&](size_t i, size_t j) {
      if (!bit_set(i, ctl)) return;
      double v_re = s.re[j], v_im = s.im[j];
      s.re[j] = v_re * cs - v_im * sn;
      s.im[j] = v_re * sn + v_im * cs;
    });
    return;
  }
  if (kind == BF_GATE_X && (c.spec & BF_SPEC_CX)) {
    for_pairs(s, c, t, [&](size_t i, size_t j) {
      if (!bit_set(i, ctl)) return;
      std::swap(s.re[i], s.re[j]);
      std::swap(s.im[i], s.im[j]);
    });
    return;
  }
  if (kind == BF_GATE_RY && (c.spec & BF_SPEC_CRY)) {
    double cs = cos(arg / 2), sn = sin(arg / 2);
    for_pairs(s, c, t, [&](size_t i, size_t j) {
      if (!bit_set(i, ctl)) return;
      double u_re = s.re[i], u_im = s.im[i], v_re = s.re[j], v_im = s.im[j];
      s.re[i] = u_re * cs - v_re * sn;
      s.im[i] = u_im * cs - v_im * sn;
      s.re[j] = u_re * sn + v_re * cs;
      s.im[j] = u_im * sn + v_im * cs;
    });
    return;
  }
  for_pairs(s, c, t, [&](size_t i, size_t j) {
    if (bit_set(i, ctl)) process_pair(s, g, i, j);
  });
}

// mc_transform_scalar (:569-594): generic pair under a control mask.
void mc_transform(St& s, const Ctx& c, uint64_t mask, int t, const Gate2 g) {
  for_pairs(s, c, t, [&](size_t i, size_t j) {
    if ((i & mask) == mask) process_pair(s, g, i, j);
  });
}

// ---- dense m-qubit unitaries (transformations_unitary.mojo:22-139) --------
void apply_unitary(St& s, const double* u, int target, int m, int control) {
  if (m <= 0) return;
  size_t dim = (size_t)1 << m;
  size_t stride = (size_t)1 << target;
  size_t block = (size_t)1 << (target + m);
  std::vector<double> tr(dim), ti(dim), orr(dim), oi(dim);
  for (size_t high = 0; high < s.N; high += block) {
    for (size_t low = 0; low < stride; ++low) {
      size_t base = high + low;
      if (control >= 0 && (base & ((size_t)1 << control)) == 0) continue;
      for (size_t k = 0; k < dim; ++k) {
        size_t idx = base + (k << target);
        tr[k] = s.re[idx];
        ti[k] = s.im[idx];
      }
      for (size_t row = 0; row < dim; ++row) {
        double sr = 0, si = 0;
        for (size_t col = 0; col < dim; ++col) {
          double ur = u[2 * (row * dim + col)], ui = u[2 * (row * dim + col) + 1];
          sr += ur * tr[col] - ui * ti[col];
          si += ur * ti[col] + ui * tr[col];
        }
        orr[row] = sr;
        oi[row] = si;
      }
      for (size_t k = 0; k < dim; ++k) {
        size_t idx = base + (k << target);
        s.re[idx] = orr[k];
        s.im[idx] = oi[k];
      }
    }
  }
}

// ---- fused pair kernels (fused_kernels_sparse_global.mojo:8-250) ----------
inline size_t insert_zero_bit(size_t x, int pos) {  // utils/bit_utils.mojo:5-10
  size_t mask = ((size_t)1 << pos) - 1;
  return ((x & ~mask) << 1) | (x & mask);
}

void fused_hh(St& s, int t1, int t2) {
  int hi = std::max(t1, t2), lo = std::min(t1, t2);
  size_t sl = (size_t)1 << lo, sh = (size_t)1 << hi;
  const double scale = 0.5;
  for (size_t k = 0; k < (s.N >> 2); ++k) {
    size_t i0 = insert_zero_bit(insert_zero_bit(k, lo), hi);
    size_t i1 = i0 + sl, i2 = i0 + sh, i3 = i1 + sh;
    double r0 = s.re[i0], m0 = s.im[i0], r1 = s.re[i1], m1 = s.im[i1];
    double r2 = s.re[i2], m2 = s.im[i2], r3 = s.re[i3], m3 = s.im[i3];
    double s01r = r0 + r1, s01i = m0 + m1, d01r = r0 - r1, d01i = m0 - m1;
    double s23r = r2 + r3, s23i = m2 + m3, d23r = r2 - r3, d23i = m2 - m3;
    s.re[i0] = (s01r + s23r) * scale; s.im[i0] = (s01i + s23i) * scale;
    s.re[i1] = (d01r + d23r) * scale; s.im[i1] = (d01i + d23i) * scale;
    s.re[i2] = (s01r - s23r) * scale; s.im[i2] = (s01i - s23i) * scale;
    s.re[i3] = (d01r - d23r) * scale; s.im[i3] = (d01i - d23i) * scale;
  }
}

void fused_hp(St& s, int th, int tp, double theta) {
  size_t sh = (size_t)1 << th, sp = (size_t)1 << tp;
  int lo = std::min(th, tp), hi = std::max(th, tp);
  const double sq_half = 0.7071067811865476;
  double cs = cos(theta), sn = sin(theta);
  for (size_t k = 0; k < (s.N >> 2); ++k) {
    size_t i0 = insert_zero_bit(insert_zero_bit(k, lo), hi);
    size_t ih = i0 | sh, ip = i0 | sp, ihp = i0 | sh | sp;
    double r0 = s.re[i0], m0 = s.im[i0], rh = s.re[ih], mh = s.im[ih];
    double rp = s.re[ip], mp = s.im[ip], rhp = s.re[ihp], mhp = s.im[ihp];
    double n_r0 = (r0 + rh) * sq_half, n_i0 = (m0 + mh) * sq_half;
    double n_rh = (r0 - rh) * sq_half, n_ih = (m0 - mh) * sq_half;
    double n_rp = (rp + rhp) * sq_half, n_ip = (mp + mhp) * sq_half;
    double n_rhp = (rp - rhp) * sq_half, n_ihp = (mp - mhp) * sq_half;
    s.re[i0] = n_r0; s.im[i0] = n_i0;
    s.re[ih] = n_rh; s.im[ih] = n_ih;
    s.re[ip] = n_rp * cs - n_ip * sn; s.im[ip] = n_rp * sn + n_ip * cs;
    s.re[ihp] = n_rhp * cs - n_ihp * sn; s.im[ihp] = n_rhp * sn + n_ihp * cs;
  }
}

void fused_pp(St& s, int t1, int t2, double th1, double th2) {
  int hi = t1, lo = t2;
  if (t2 > t1) { hi = t2; lo = t1; std::swap(th1, th2); }
  size_t sl = (size_t)1 << lo, sh = (size_t)1 << hi;
  double c1 = cos(th1), s1 = sin(th1), c2 = cos(th2), s2 = sin(th2);
  double c12 = cos(th1 + th2), s12 = sin(th1 + th2);
  for (size_t k = 0; k < (s.N >> 2); ++k) {
    size_t i0 = insert_zero_bit(insert_zero_bit(k, lo), hi);
    size_t i1 = i0 | sl, i2 = i0 | sh, i3 = i1 | sh;
    double r1 = s.re[i1], m1 = s.im[i1];
    s.re[i1] = r1 * c2 - m1 * s2; s.im[i1] = r1 * s2 + m1 * c2;
    double r2 = s.re[i2], m2 = s.im[i2];
    s.re[i2] = r2 * c1 - m2 * s1; s.im[i2] = r2 * s1 + m2 * c1;
    double r3 = s.re[i3], m3 = s.im[i3];
    s.re[i3] = r3 * c12 - m3 * s12; s.im[i3] = r3 * s12 + m3 * c12;
  }
}

void fused_shared_c_pp(St& s, int ctl, int t1, int t2, double th1, double th2) {
  int b[3] = {ctl, t1, t2};
  std::sort(b, b + 3);
  size_t sc = (size_t)1 << ctl, s1 = (size_t)1 << t1, s2 = (size_t)1 << t2;
  double c1 = cos(th1), n1 = sin(th1), c2 = cos(th2), n2 = sin(th2);
  double c12 = cos(th1 + th2), n12 = sin(th1 + th2);
  for (size_t k = 0; k < (s.N >> 3); ++k) {
    size_t i0 = insert_zero_bit(insert_zero_bit(insert_zero_bit(k, b[0]), b[1]), b[2]);
    size_t cb = i0 | sc;
    size_t a = cb | s1;
    double r = s.re[a], m = s.im[a];
    s.re[a] = r * c1 - m * n1; s.im[a] = r * n1 + m * c1;
    a = cb | s2;
    r = s.re[a]; m = s.im[a];
    s.re[a] = r * c2 - m * n2; s.im[a] = r * n2 + m * c2;
    a = cb | s1 | s2;
    r = s.re[a]; m = s.im[a];
    s.re[a] = r * c12 - m * n12; s.im[a] = r * n12 + m * c12;
  }
}

// 4x4 helpers of transformations_fusion.mojo:51-103 (complex products as
// (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re)).
void gate_to_4x4(const Gate2 g, int q_low, int target, Cplx* m) {
  for (int i = 0; i < 16; ++i) m[i] = Cplx{0, 0};
  if (target == q_low) {
    for (int b1 = 0; b1 < 2; ++b1)
      for (int r0 = 0; r0 < 2; ++r0)
        for (int c0 = 0; c0 < 2; ++c0) m[(r0 + 2 * b1) * 4 + c0 + 2 * b1] = g[r0][c0];
  } else {
    for (int b0 = 0; b0 < 2; ++b0)
      for (int r1 = 0; r1 < 2; ++r1)
        for (int c1 = 0; c1 < 2; ++c1) m[(b0 + 2 * r1) * 4 + b0 + 2 * c1] = g[r1][c1];
  }
}

void cgate_to_4x4(const Gate2 g, int q_low, int control, int target, Cplx* m) {
  for (int i = 0; i < 16; ++i) m[i] = Cplx{0, 0};
  for (int b0 = 0; b0 < 2; ++b0)
    for (int b1 = 0; b1 < 2; ++b1) {
      int in = b0 + 2 * b1;
      int cb = control == q_low ? b0 : b1;
      int tb = target == q_low ? b0 : b1;
      if (cb == 0) {
        m[in * 4 + in] = Cplx{1, 0};
      } else {
        for (int ot = 0; ot < 2; ++ot) {
          int ob0 = b0, ob1 = b1;
          if (target == q_low) ob0 = ot; else ob1 = ot;
          m[(ob0 + 2 * ob1) * 4 + in] = g[ot][tb];
        }
      }
    }
}

void matmul4(const Cplx* a, const Cplx* b, Cplx* out) {
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      Cplx sum{0, 0};
      for (int k = 0; k < 4; ++k) {
        Cplx x = a[r * 4 + k], y = b[k * 4 + c];
        sum.re = sum.re + (x.re * y.re - x.im * y.im);
        sum.im = sum.im + (x.re * y.im + x.im * y.re);
      }
      out[r * 4 + c] = sum;
    }
}

bool is_h(const bf_op& o) { return o.ncontrols == 0 && o.gate == BF_GATE_H; }
bool is_p(const bf_op& o) { return o.ncontrols == 0 && o.gate == BF_GATE_P; }
bool is_cp(const bf_op& o) { return o.ncontrols == 1 && o.gate == BF_GATE_P; }
int lowest_bit(uint64_t m) { return m ? __builtin_ctzll(m) : 0; }

// apply_fused_pair (transformations_fusion.mojo:221-310)
void apply_fused_pair(St& s, const bf_op& t0, const bf_op& t1) {
  if (is_cp(t0) && is_cp(t1) && t0.controls == t1.controls) {
    int ctl = lowest_bit(t0.controls);
    if (t0.target > t1.target)
      fused_shared_c_pp(s, ctl, t0.target, t1.target, t0.arg, t1.arg);
    else
      fused_shared_c_pp(s, ctl, t1.target, t0.target, t1.arg, t0.arg);
    return;
  }
  if (is_h(t0) && is_h(t1)) return fused_hh(s, t0.target, t1.target);
  if (is_p(t0) && is_p(t1)) {
    if (t0.target > t1.target) fused_pp(s, t0.target, t1.target, t0.arg, t1.arg);
    else fused_pp(s, t1.target, t0.target, t1.arg, t0.arg);
    return;
  }
  if (is_h(t0) && is_p(t1)) return fused_hp(s, t0.target, t1.target, t1.arg);
  if (is_p(t0) && is_h(t1)) return fused_hp(s, t1.target, t0.target, t0.arg);
  int c0 = t0.ncontrols == 1 ? lowest_bit(t0.controls) : 0;
  int c1 = t1.ncontrols == 1 ? lowest_bit(t1.controls) : 0;
  int q_low = t0.target;
  if (t0.ncontrols == 1) q_low = std::min(q_low, c0);
  q_low = std::min(q_low, t1.target);
  if (t1.ncontrols == 1) q_low = std::min(q_low, c1);
  Gate2 g0, g1;
  gate_matrix(t0.gate, t0.arg, t0.mat, g0);
  gate_matrix(t1.gate, t1.arg, t1.mat, g1);
  Cplx m0[16], m1[16], m[16];
  if (t0.ncontrols == 1) cgate_to_4x4(g0, q_low, c0, t0.target, m0);
  else gate_to_4x4(g0, q_low, t0.target, m0);
  if (t1.ncontrols == 1) cgate_to_4x4(g1, q_low, c1, t1.target, m1);
  else gate_to_4x4(g1, q_low, t1.target, m1);
  matmul4(m1, m0, m);
  double u[32];
  for (int i = 0; i < 16; ++i) { u[2 * i] = m[i].re; u[2 * i + 1] = m[i].im; }
  apply_unitary(s, u, q_low, 2, -1);
}

// ---- permutations (state.mojo:131-445, utils/common.mojo:12-19) ---------
size_t rev_bits(size_t i, int n) {
  size_t r = 0;
  for (int b = 0; b < n; ++b) r |= ((i >> b) & 1) << (n - 1 - b);
  return r;
}

// bit_reverse_state (:131-204): out[i] = in[rev(i)] into fresh arrays.
void bit_reverse_full(St& s) {
  std::vector<double> nr(s.N), ni(s.N);
  for (size_t i = 0; i < s.N; ++i) {
    size_t r = rev_bits(i, s.n);
    nr[i] = s.re[r];
    ni[i] = s.im[r];
  }
  memcpy(s.re, nr.data(), s.N * sizeof(double));
  memcpy(s.im, ni.data(), s.N * sizeof(double));
}

// partial_bit_reverse_state (:252-301)
void bit_reverse_partial(St& s, std::vector<int> t) {
  int k = (int)t.size();
  if (k <= 1) return;
  std::sort(t.begin(), t.end());
  for (size_t il = 0; il < s.N; ++il) {
    size_t is = 0;
    for (int b = 0; b < k; ++b)
      if ((il >> t[b]) & 1) is |= (size_t)1 << b;
    size_t js = 0;
    for (int b = 0; b < k; ++b)
      if ((is >> b) & 1) js |= (size_t)1 << (k - 1 - b);
    if (is < js) {
      size_t jl = il;
      for (int b = 0; b < k; ++b) {
        if ((js >> b) & 1) jl |= (size_t)1 << t[b];
        else jl &= ~((size_t)1 << t[b]);
      }
      std::swap(s.re[il], s.re[jl]);
      std::swap(s.im[il], s.im[jl]);
    }
  }
}

// swap_bits_state (:304-317) with swap_bits_index (common.mojo:12-19)
void swap_bits(St& s, int a, int b) {
  if (a == b) return;
  for (size_t i = 0; i < s.N; ++i) {
    size_t x = ((i >> a) ^ (i >> b)) & 1;
    size_t j = i ^ ((x << a) | (x << b));
    if (j > i) {
      std::swap(s.re[i], s.re[j]);
      std::swap(s.im[i], s.im[j]);
    }
  }
}

// apply_permute_qubits (:393-431)
void permute_qubits(St& s, const int32_t* order, int64_t cnt) {
  if (cnt == 0) return;
  if (cnt != s.n) fail(BF_EINVAL, "Permutation size mismatch: %lld", (long long)cnt);
  std::vector<bool> seen(s.n, false);
  for (int i = 0; i < s.n; ++i) {
    int v = order[i];
    if (v < 0 || v >= s.n) fail(BF_EINVAL, "Invalid permutation value: %d", v);
    if (seen[v]) fail(BF_EINVAL, "Duplicate permutation value: %d", v);
    seen[v] = true;
  }
  std::vector<int> perm(s.n);
  for (int i = 0; i < s.n; ++i) perm[i] = i;
  for (int i = 0; i < s.n; ++i) {
    if (perm[i] == order[i]) continue;
    int j = i + 1;
    while (j < s.n && perm[j] != order[i]) ++j;
    if (j >= s.n) fail(BF_EINVAL, "Invalid permutation order");
    swap_bits(s, i, j);
    std::swap(perm[i], perm[j]);
  }
}

// ---- modular exponentiation (algos/shor.mojo:11-140) ------------------------
int64_t gcd64(int64_t a, int64_t b) {  // gcd (:11-18)
  int64_t x = a, y = b;
  while (y != 0) {
    int64_t t = x % y;
    x = y;
    y = t;
  }
  return x < 0 ? -x : x;
}

uint64_t mulmod_u64(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)(((unsigned __int128)a * b) % m); }

int64_t modexp64(int64_t base, int64_t e, int64_t m) {  // modexp (:21-32)
  if (m <= 1) return 0;
  uint64_t r = 1 % (uint64_t)m, b = (uint64_t)(((base % m) + m) % m);
  while (e > 0) {
    if (e & 1) r = mulmod_u64(r, b, (uint64_t)m);
    b = mulmod_u64(b, b, (uint64_t)m);
    e >>= 1;
  }
  return (int64_t)r;
}

int64_t modinv64(int64_t a, int64_t m) {  // modinv via egcd (:39-53)
  int64_t r0 = m, r1 = ((a % m) + m) % m, t0 = 0, t1 = 1;
  while (r1 != 0) {
    int64_t q = r0 / r1, r = r0 - q * r1, t = t0 - q * t1;
    r0 = r1;
    r1 = r;
    t0 = t1;
    t1 = t;
  }
  return r0 != 1 ? 0 : ((t0 % m) + m) % m;
}

// out[x | y_out << n_exp] = in[idx], y_out = y * a^x mod N (or a^-x) for y < N
void apply_modexp(St& s, int n_exp, int n_value, int64_t a, int64_t N, bool inverse) {
  std::vector<double> ore(s.N, 0.0), oim(s.N, 0.0);
  const size_t xm = ((size_t)1 << n_exp) - 1, ym = ((size_t)1 << n_value) - 1;
  for (size_t idx = 0; idx < s.N; ++idx) {
    size_t x = idx & xm, y = (idx >> n_exp) & ym, y_out = y;
    if ((int64_t)y < N) {
      int64_t ax = modexp64(a, (int64_t)x, N);
      if (inverse) ax = modinv64(ax, N);
      y_out = (size_t)mulmod_u64(y, (uint64_t)ax, (uint64_t)N);
    }
    size_t out = x | (y_out << n_exp);
    ore[out] = s.re[idx];
    oim[out] = s.im[idx];
  }
  std::memcpy(s.re, ore.data(), s.N * sizeof(double));
  std::memcpy(s.im, oim.data(), s.N * sizeof(double));
}

// ---- validation (executors.mojo:78-185) -----------------------------------
void check_qubit(int idx, int n, const char* label) {
  if (idx < 0 || idx >= n) fail(BF_EINVAL, "%s out of bounds: %d", label, idx);
}

void validate(const St& s, const bf_op* ops, int64_t nops) {
  int n = s.n;
  for (int64_t i = 0; i < nops; ++i) {
    const bf_op& o = ops[i];
    switch (o.kind) {
      case BF_OP_GATE: {
        check_qubit(o.target, n, "Target");
        if (o.ncontrols < 0 || __builtin_popcountll(o.controls) != o.ncontrols)
          fail(BF_EINVAL, "Gate control kind mismatch: %d controls in a mask of %d",
               o.ncontrols, __builtin_popcountll(o.controls));
        if (n < 64 && (o.controls >> n))
          fail(BF_EINVAL, "Control out of bounds: %d", 63 - __builtin_clzll(o.controls));
        if (o.gate < 0 || o.gate > BF_GATE_CUSTOM) fail(BF_EINVAL, "Unknown gate kind: %d", o.gate);
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
        for (int64_t k = 0; k < o.nqubits; ++k) check_qubit(o.qubits[k], n, "Target");
        break;
      case BF_OP_MEASURE:
      case BF_OP_GROVER_DIFFUSER:
      case BF_OP_GROVER_INVERSION0:
        for (int64_t k = 0; k < o.nqubits; ++k) check_qubit(o.qubits[k], n, "Target");
        break;
      case BF_OP_CLASSICAL_ORACLE:
        for (int64_t k = 0; k < o.nqubits; ++k)
          if (!(o.data[k] >= 0 && o.data[k] < (double)s.N) || o.data[k] != floor(o.data[k]))
            fail(BF_EINVAL, "Oracle index out of range: %.17g", o.data[k]);
        break;
      case BF_OP_MODEXP:
      case BF_OP_MODEXP_INV: {  // algos/shor.mojo:60-76
        const char* name = o.kind == BF_OP_MODEXP ? "MOD_EXP" : "MOD_EXP_INV";
        if (o.nqubits < 4 || !o.data) fail(BF_EINVAL, "%s expects 4 parameters: n_exp, n_value, a, N", name);
        int64_t ne = (int64_t)o.data[0], nv = (int64_t)o.data[1], a = (int64_t)o.data[2], N = (int64_t)o.data[3];
        if (ne <= 0 || nv <= 0) fail(BF_EINVAL, "%s expects positive register sizes", name);
        if (N <= 1) fail(BF_EINVAL, "%s expects modulus > 1", name);
        if (gcd64(a, N) != 1) fail(BF_EINVAL, "%s expects a and modulus to be coprime", name);
        if (ne + nv != n) fail(BF_EINVAL, "State size mismatch for %s", name);
        break;
      }
      case BF_OP_UNITARY:
      case BF_OP_CUNITARY: {
        int m = o.target2;
        if (m > 0 && (o.target < 0 || o.target + m > n)) fail(BF_EINVAL, "Target range out of bounds");
        if (o.kind == BF_OP_CUNITARY) {
          if (o.ncontrols != 1 || __builtin_popcountll(o.controls) != 1)
            fail(BF_EINVAL, "Controlled unitary expects exactly one control");
          int c = lowest_bit(o.controls);
          check_qubit(c, n, "Control");
          if (m > 0 && c >= o.target && c < o.target + m) fail(BF_EINVAL, "Control overlaps target range");
        }
        if (m > 0 && o.data == nullptr) fail(BF_EINVAL, "Unitary data is null");
        break;
      }
      default: fail(BF_EINVAL, "Unknown transformation type: %d", o.kind);
    }
  }
}

// ---- executor (execute_with_handlers, executors.mojo:268-319) -------------
void cx(St& s, const Ctx& c, int ctl, int t) {  // handle_cx_scalar (:368-372)
  Gate2 g;
  gate_matrix(BF_GATE_X, 0, nullptr, g);
  if (c.strategy == OR_SCALAR) c_transform(s, c, ctl, t, g, BF_GATE_X, 0);
  else mc_transform(s, c, (uint64_t)1 << ctl, t, g);  // handle_cx_simd_parallel
}

void gate_op(St& s, const Ctx& c, const bf_op& o) {
  Gate2 g;
  gate_matrix(o.gate, o.arg, o.mat, g);
  if (o.ncontrols == 0) {
    // handle_gate_scalar / handle_gate_simd_parallel share this dispatch for
    // the specialised kinds, then the generic pair kernel.
    transform(s, c, o.target, g, o.gate, o.arg);
  } else if (o.ncontrols == 1) {
    int ctl = lowest_bit(o.controls);
    if (c.strategy == OR_SCALAR) {
      c_transform(s, c, ctl, o.target, g, o.gate, o.arg);
    } else {
      bool spec = (o.gate == BF_GATE_P && (c.spec & BF_SPEC_CP)) ||
                  (o.gate == BF_GATE_X && (c.spec & BF_SPEC_CX)) ||
                  (o.gate == BF_GATE_RY && (c.spec & BF_SPEC_CRY));
      if (spec) c_transform(s, c, ctl, o.target, g, o.gate, o.arg);
      else mc_transform(s, c, o.controls, o.target, g);
    }
  } else {
    mc_transform(s, c, o.controls, o.target, g);
  }
}

void run(St& s, const Ctx& c, const bf_op* ops, int64_t nops, bool do_validate) {
  if (do_validate) validate(s, ops, nops);
  for (int64_t i = 0; i < nops; ++i) {
    const bf_op& o = ops[i];
    switch (o.kind) {
      case BF_OP_GATE:
        if ((o.flags & BF_OPF_FUSE_WITH_NEXT) && i + 1 < nops && ops[i + 1].kind == BF_OP_GATE) {
          apply_fused_pair(s, o, ops[i + 1]);
          ++i;
        } else {
          gate_op(s, c, o);
        }
        break;
      case BF_OP_SWAP:  // apply_swap_with_cx (:231-241)
        if (o.target != o.target2) {
          cx(s, c, o.target, o.target2);
          cx(s, c, o.target2, o.target);
          cx(s, c, o.target, o.target2);
        }
        break;
      case BF_OP_QREV: {  // apply_qubit_reversal_with_cx (:244-265)
        std::vector<int> t;
        if (o.nqubits == 0) for (int q = 0; q < s.n; ++q) t.push_back(q);
        else t.assign(o.qubits, o.qubits + o.nqubits);
        std::sort(t.begin(), t.end());
        size_t half = t.size() / 2;
        for (size_t k = 0; k < half; ++k) {
          int a = t[k], b = t[t.size() - 1 - k];
          if (a == b) continue;
          cx(s, c, a, b);
          cx(s, c, b, a);
          cx(s, c, a, b);
        }
        break;
      }
      case BF_OP_UNITARY:
        apply_unitary(s, o.data, o.target, o.target2, -1);
        break;
      case BF_OP_CUNITARY:
        apply_unitary(s, o.data, o.target, o.target2, lowest_bit(o.controls));
        break;
      case BF_OP_BITREV:  // apply_bit_reverse (:383-390)
        if (o.nqubits == 0) bit_reverse_full(s);
        else bit_reverse_partial(s, std::vector<int>(o.qubits, o.qubits + o.nqubits));
        break;
      case BF_OP_PERMUTE:
        permute_qubits(s, o.qubits, o.nqubits);
        break;
      case BF_OP_CSWAP:  // apply_swap (:434-444)
        swap_bits(s, o.target, o.target2);
        break;
      case BF_OP_GROVER_DIFFUSER:     // apply_grover_diffuser (grover_classical.mojo:284-326)
      case BF_OP_GROVER_INVERSION0: {  // apply_grover_inversion_0 (grover_classical.mojo:262-281)
        std::vector<bool> is_t(s.n, o.nqubits == 0);
        for (int64_t k = 0; k < o.nqubits; ++k) is_t[o.qubits[k]] = true;
        std::vector<int> tg, other;
        if (o.nqubits == 0) for (int q = 0; q < s.n; ++q) tg.push_back(q);
        else tg.assign(o.qubits, o.qubits + o.nqubits);
        for (int q = 0; q < s.n; ++q) if (!is_t[q]) other.push_back(q);
        size_t blocks = (size_t)1 << other.size(), bs = (size_t)1 << tg.size();
        for (size_t b = 0; b < blocks; ++b) {
          size_t base = 0;
          for (size_t i = 0; i < other.size(); ++i) if ((b >> i) & 1) base |= (size_t)1 << other[i];
          if (o.kind == BF_OP_GROVER_INVERSION0) {
            s.re[base] = -s.re[base];
            s.im[base] = -s.im[base];
            continue;
          }
          auto idx_of = [&](size_t tm) {
            size_t idx = base;
            for (size_t j = 0; j < tg.size(); ++j) if ((tm >> j) & 1) idx |= (size_t)1 << tg[j];
            return idx;
          };
          double sr = 0, si = 0;
          for (size_t tm = 0; tm < bs; ++tm) { size_t i = idx_of(tm); sr += s.re[i]; si += s.im[i]; }
          // 2 * mean for both parts (the reference negates the imaginary one,
          // grover_classical.mojo:318, which is not the inversion about the mean)
          double ar = 2.0 * (1.0 / (double)bs) * sr, ai = 2.0 * (1.0 / (double)bs) * si;
          for (size_t tm = 0; tm < bs; ++tm) {
            size_t i = idx_of(tm);
            s.re[i] = ar - s.re[i];
            s.im[i] = ai - s.im[i];
          }
        }
        break;
      }
      case BF_OP_MODEXP:       // apply_modexp (algos/shor.mojo:56-96)
      case BF_OP_MODEXP_INV:   // apply_modexp_inverse (algos/shor.mojo:99-140)
        apply_modexp(s, (int)o.data[0], (int)o.data[1], (int64_t)o.data[2], (int64_t)o.data[3],
                     o.kind == BF_OP_MODEXP_INV);
        break;
      case BF_OP_CLASSICAL_ORACLE:  // classical_oracle (grover.mojo:64-66)
        for (int64_t k = 0; k < o.nqubits; ++k) {
          size_t i = (size_t)o.data[k];
          s.re[i] = -s.re[i];
          s.im[i] = -s.im[i];
        }
        break;
      case BF_OP_MEASURE: {  // MeasurementTransformation -> apply_measure (:447-553)
        std::vector<int8_t> v;
        for (int64_t k = 0; k < o.nqubits; ++k) v.push_back(o.data ? (int8_t)o.data[k] : (int8_t)-1);
        char err[512];
        int rc = or_measure(s.n, s.re, s.im, o.qubits, v.data(), (int32_t)o.nqubits, (int64_t)o.arg, nullptr,
                            nullptr, err, sizeof err);
        if (rc != 0) fail(rc, "%s", err);
        break;
      }
      default:
        fail(BF_EINVAL, "Unknown transformation type: %d", o.kind);
    }
  }
}

void set_err(char* err, size_t len, const std::string& m) {
  if (err && len) {
    size_t k = std::min(len - 1, m.size());
    memcpy(err, m.data(), k);
    err[k] = 0;
  }
}

// ---- classical QFT (butterfly/algos/qft_classical.mojo) -------------------
void fft_in_place(std::vector<double>& re, std::vector<double>& im, bool inverse) {
  size_t n = re.size();
  if (n <= 1) return;
  int log_n = 0;
  while (((size_t)1 << log_n) < n) ++log_n;
  for (size_t i = 0; i < n; ++i) {  // _bit_reverse_in_place (:51-75)
    size_t j = rev_bits(i, log_n);
    if (i < j) { std::swap(re[i], re[j]); std::swap(im[i], im[j]); }
  }
  double sign = inverse ? -1.0 : 1.0;
  const double two_pi = 2.0 * M_PI;
  for (size_t step = 2; step <= n; step *= 2) {  // _fft_in_place (:78-119)
    size_t half = step / 2;
    double theta = sign * two_pi / (double)step;
    double wmr = cos(theta), wmi = sin(theta);
    for (size_t k = 0; k < n; k += step) {
      double wr = 1, wi = 0;
      for (size_t j = 0; j < half; ++j) {
        double tr = wr * re[k + j + half] - wi * im[k + j + half];
        double ti = wr * im[k + j + half] + wi * re[k + j + half];
        double ur = re[k + j], ui = im[k + j];
        re[k + j] = ur + tr; im[k + j] = ui + ti;
        re[k + j + half] = ur - tr; im[k + j + half] = ui - ti;
        double nwr = wr * wmr - wi * wmi;
        double nwi = wr * wmi + wi * wmr;
        wr = nwr; wi = nwi;
      }
    }
  }
}

// ---- fusion rewrites (transformations_fusion.mojo:24-908) ------------------
// A second restatement of the reference's fusion passes, over op records,
// so that the host mirror's rewrite (code_mojo_gb300/fusion.py) is checked
// against an independent one.  An item is a gate (one record), a fused pair
// (two records, the first flagged BF_OPF_FUSE_WITH_NEXT), a 1- or 2-qubit
// unitary, a controlled 1-qubit unitary, or any other record passed through.
enum ItemKind { IT_GATE, IT_PAIR, IT_UNITARY, IT_CUNITARY, IT_OTHER };
struct Item {
  ItemKind kind = IT_OTHER;
  bf_op op[2] = {};           // IT_GATE / IT_OTHER: op[0]; IT_PAIR: both
  std::vector<Cplx> u;        // IT_UNITARY (2x2 or 4x4) / IT_CUNITARY (2x2), row-major
  int target = 0, m = 0, control = -1;
};

// ControlKind of a gate record: 0 none, 1 one control, 2 several
int control_kind(const bf_op& o) { return o.ncontrols == 0 ? 0 : (o.ncontrols == 1 ? 1 : 2); }
int control_of(const bf_op& o) { return control_kind(o) == 1 ? lowest_bit(o.controls) : 0; }
bool is_special(const bf_op& o) { return is_h(o) || is_p(o) || is_cp(o); }

Item gate_item(const bf_op& o) {
  Item it;
  it.kind = IT_GATE;
  it.op[0] = o;
  return it;
}

// can_fuse_special_pair (:181-219)
bool can_fuse_special(const bf_op& t0, const bf_op& t1) {
  if (control_kind(t0) == 2 || control_kind(t1) == 2) return false;
  if (is_cp(t0) && is_cp(t1) && t0.controls == t1.controls && t0.target != t1.target) return true;
  int lo = t0.target, hi = t0.target;
  auto widen = [&](int q) { lo = std::min(lo, q); hi = std::max(hi, q); };
  if (control_kind(t0) == 1) widen(control_of(t0));
  if (control_kind(t1) == 1) widen(control_of(t1));
  widen(t1.target);
  if (hi - lo != 1) return false;
  return (is_h(t0) && is_h(t1)) || (is_p(t0) && is_p(t1)) || (is_h(t0) && is_cp(t1)) || (is_cp(t0) && is_h(t1));
}

// fuse_special_pair_gates (:312-333)
std::vector<Item> special_pairs(const std::vector<Item>& in) {
  std::vector<Item> out;
  for (size_t i = 0; i < in.size(); ++i) {
    if (i + 1 < in.size() && in[i].kind == IT_GATE && in[i + 1].kind == IT_GATE &&
        can_fuse_special(in[i].op[0], in[i + 1].op[0])) {
      Item it;
      it.kind = IT_PAIR;
      it.op[0] = in[i].op[0];
      it.op[1] = in[i + 1].op[0];
      it.op[0].flags |= BF_OPF_FUSE_WITH_NEXT;
      out.push_back(it);
      ++i;
      continue;
    }
    out.push_back(in[i]);
  }
  return out;
}

// 4x4 of a gate record on the pair (q_low, q_low + 1); try_pair_matrix
// (:129-161) for the specialised form
bool pair_4x4(const bf_op& g, int q_low, int q_high, bool special_only, Cplx* m) {
  if (special_only && !is_special(g)) return false;
  Gate2 gm;
  gate_matrix(g.gate, g.arg, g.mat, gm);
  if (control_kind(g) == 0) {
    if (g.target != q_low && g.target != q_high) return false;
    gate_to_4x4(gm, q_low, g.target, m);
    return true;
  }
  if (control_kind(g) != 1) return false;
  const int c = control_of(g);
  if (c == g.target || (c != q_low && c != q_high) || (g.target != q_low && g.target != q_high)) return false;
  cgate_to_4x4(gm, q_low, c, g.target, m);
  return true;
}

void bounds(const bf_op& g, int* lo, int* hi) {  // gate_bounds (:106-117)
  *lo = *hi = g.target;
  if (control_kind(g) == 1) {
    *lo = std::min(*lo, control_of(g));
    *hi = std::max(*hi, control_of(g));
  }
}

// fuse_contiguous_target_pairs (:539-687) and its specialised form (:689-876)
std::vector<Item> contiguous_pairs(const std::vector<Item>& in, bool special) {
  std::vector<Item> out;
  bool pending = false, paired = false;
  bf_op p{};
  Cplx acc[16];
  int lo = 0, hi = 0;
  auto flush = [&]() {
    if (paired) {
      Item it;
      it.kind = IT_UNITARY;
      it.u = std::vector<Cplx>(std::begin(acc), std::end(acc));
      it.target = lo;
      it.m = 2;
      out.push_back(it);
    } else if (pending) {
      out.push_back(gate_item(p));
    }
    pending = paired = false;
  };
  auto start = [&](const bf_op& g) {
    flush();
    p = g;
    pending = true;
  };
  for (const Item& it : in) {
    bool passes = it.kind != IT_GATE;
    if (!passes) {
      const bf_op& g = it.op[0];
      passes = special ? (control_kind(g) == 2 || !is_special(g)) : control_kind(g) != 0;
    }
    if (passes) {
      flush();
      out.push_back(it);
      continue;
    }
    const bf_op& g = it.op[0];
    if (!pending) {
      start(g);
      continue;
    }
    if (!paired) {
      const bool same = g.target == p.target &&
                        (!special || (control_kind(g) == control_kind(p) && control_of(g) == control_of(p)));
      if (!same) {
        int l0, h0, l1, h1;
        bounds(p, &l0, &h0);
        bounds(g, &l1, &h1);
        const int l = special ? std::min(l0, l1) : std::min(p.target, g.target);
        const int h = special ? std::max(h0, h1) : std::max(p.target, g.target);
        Cplx m0[16], m1[16];
        if (h - l == 1 && pair_4x4(p, l, h, special, m0) && pair_4x4(g, l, h, special, m1)) {
          matmul4(m1, m0, acc);
          lo = l;
          hi = h;
          paired = true;
          continue;
        }
      }
      start(g);
      continue;
    }
    Cplx m1[16], nxt[16];
    if (pair_4x4(g, lo, hi, special, m1)) {
      matmul4(m1, acc, nxt);
      std::copy(nxt, nxt + 16, acc);
      continue;
    }
    start(g);
  }
  flush();
  return out;
}

// fuse_same_target_gates (:427-537) with flush_active (:335-392)
std::vector<Item> same_target_runs(const std::vector<Item>& in) {
  std::vector<Item> out;
  bool active = false, phase = false;
  int count = 0;
  bf_op first{};
  Gate2 prod;
  double phase_sum = 0;
  auto flush = [&]() {
    if (!active) return;
    if (phase) {
      bf_op g = first;
      g.gate = BF_GATE_P;
      g.arg = phase_sum;
      out.push_back(gate_item(g));
    } else if (count == 1) {
      out.push_back(gate_item(first));
    } else {
      Item it;
      it.kind = control_kind(first) == 0 ? IT_UNITARY : IT_CUNITARY;
      it.u = {prod[0][0], prod[0][1], prod[1][0], prod[1][1]};
      it.target = first.target;
      it.m = 1;
      it.control = control_kind(first) == 0 ? -1 : control_of(first);
      out.push_back(it);
    }
    active = false;
  };
  for (const Item& it : in) {
    if (it.kind != IT_GATE || control_kind(it.op[0]) == 2) {
      flush();
      out.push_back(it);
      continue;
    }
    const bf_op& g = it.op[0];
    Gate2 gm;
    gate_matrix(g.gate, g.arg, g.mat, gm);
    if (active && g.target == first.target && control_kind(g) == control_kind(first) &&
        control_of(g) == control_of(first)) {
      Gate2 next;  // mul_gate(new, product) (:24-33)
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
          Cplx sum{0, 0};
          for (int k = 0; k < 2; ++k) {
            sum.re = sum.re + (gm[i][k].re * prod[k][j].re - gm[i][k].im * prod[k][j].im);
            sum.im = sum.im + (gm[i][k].re * prod[k][j].im + gm[i][k].im * prod[k][j].re);
          }
          next[i][j] = sum;
        }
      std::memcpy(prod, next, sizeof prod);
      ++count;
      if (phase && g.gate == BF_GATE_P) phase_sum += g.arg;
      else phase = false;
      continue;
    }
    flush();
    active = true;
    first = g;
    count = 1;
    std::memcpy(prod, gm, sizeof prod);
    phase = g.gate == BF_GATE_P;
    phase_sum = phase ? g.arg : 0.0;
  }
  flush();
  return out;
}

}  // namespace

extern "C" {

int or_execute(int32_t n, double* re, double* im, const bf_op* ops, int64_t nops,
               int32_t strategy, int32_t threads, int32_t chunks, uint32_t specialized,
               int32_t validate_flag, char* err, size_t errlen) {
  try {
    if (n < 0 || n > 40) fail(BF_EINVAL, "State size must be a power of two");
    if (strategy != OR_SCALAR && strategy != OR_SIMD_PARALLEL)
      fail(BF_EUNSUPPORTED, "Unknown execution strategy: %d", strategy);
    St s{n, (size_t)1 << n, re, im};
    Ctx c;
    c.spec = specialized;
    c.strategy = strategy;
    c.threads = threads > 0 ? threads : or_num_cores();
    c.chunks = chunks > 0 ? chunks : c.threads;
    run(s, c, ops, nops, validate_flag != 0);
    return BF_OK;
  } catch (const OrError& e) {
    set_err(err, errlen, e.msg);
    return e.code;
  }
}

// _apply_qft_like (qft_classical.mojo:122-210)
int or_qft_classical(int32_t n, double* re, double* im, const int32_t* targets,
                     int32_t ntargets, int32_t inverse, int32_t swap, char* err,
                     size_t errlen) {
  try {
    St s{n, (size_t)1 << n, re, im};
    std::vector<int> t;
    if (ntargets == 0) for (int q = 0; q < n; ++q) t.push_back(q);
    else {
      std::vector<bool> seen(n, false);
      for (int i = 0; i < ntargets; ++i) {
        int q = targets[i];
        if (q < 0 || q >= n) fail(BF_EINVAL, "Target out of bounds: %d", q);
        if (seen[q]) fail(BF_EINVAL, "Duplicate target: %d", q);
        seen[q] = true;
        t.push_back(q);
      }
    }
    if (t.empty()) return BF_OK;
    bool lsb_first = true;
    for (size_t i = 1; i < t.size(); ++i)
      if (t[i] <= t[i - 1]) { lsb_first = false; break; }
    bool pre = false, post = false;
    if (inverse) {
      if (lsb_first) post = !swap;
      else { pre = true; post = swap; }
    } else {
      if (lsb_first) pre = !swap;
      else { pre = swap; post = true; }
    }
    auto bitrev = [&]() {
      if ((int)t.size() == n) bit_reverse_full(s);
      else bit_reverse_partial(s, t);
    };
    if (pre) bitrev();
    std::vector<bool> is_t(n, false);
    for (int q : t) is_t[q] = true;
    std::vector<int> other;
    for (int q = 0; q < n; ++q) if (!is_t[q]) other.push_back(q);
    size_t nt = t.size(), bs = (size_t)1 << nt;
    double scale = 1.0 / sqrt((double)bs);
    std::vector<double> tr(bs), ti(bs);
    for (size_t blk = 0; blk < ((size_t)1 << other.size()); ++blk) {
      size_t base = 0;
      for (size_t i = 0; i < other.size(); ++i)
        if ((blk >> i) & 1) base |= (size_t)1 << other[i];
      auto idx_of = [&](size_t tm) {
        size_t idx = base;
        for (size_t j = 0; j < nt; ++j)
          if ((tm >> j) & 1) idx |= (size_t)1 << (lsb_first ? t[j] : t[nt - 1 - j]);
        return idx;
      };
      for (size_t tm = 0; tm < bs; ++tm) { size_t i = idx_of(tm); tr[tm] = re[i]; ti[tm] = im[i]; }
      fft_in_place(tr, ti, inverse != 0);
      for (size_t tm = 0; tm < bs; ++tm) { size_t i = idx_of(tm); re[i] = tr[tm] * scale; im[i] = ti[tm] * scale; }
    }
    if (post) bitrev();
    return BF_OK;
  } catch (const OrError& e) {
    set_err(err, errlen, e.msg);
    return e.code;
  }
}

// apply_measure (state.mojo:447-553), the sequential loops as written.
// values[k]: -1 free, 0/1 fixed.  Returns the chosen outcome and its
// probability; collapses (re, im) in place.
int or_measure(int32_t n, double* re, double* im, const int32_t* targets, const int8_t* values,
               int32_t nt, int64_t seed, uint64_t* outcome, double* prob, char* err, size_t errlen) {
  try {
    size_t N = (size_t)1 << n;
    for (int j = 0; j < nt; ++j)
      if (targets[j] < 0 || targets[j] >= n) fail(BF_EINVAL, "Target out of bounds: %d", targets[j]);
    std::vector<int> free_t, free_pos(nt);
    for (int j = 0; j < nt; ++j) {
      if (values && values[j] >= 0) free_pos[j] = -1;
      else { free_pos[j] = (int)free_t.size(); free_t.push_back(targets[j]); }
    }
    size_t oc = (size_t)1 << free_t.size();
    std::vector<double> op(oc, 0.0);
    double total = 0;
    for (size_t i = 0; i < N; ++i) {
      bool match = true;
      for (int j = 0; j < nt; ++j)
        if (values && values[j] >= 0 && (int)((i >> targets[j]) & 1) != values[j]) { match = false; break; }
      if (!match) continue;
      size_t o = 0;
      for (size_t k = 0; k < free_t.size(); ++k)
        if ((i >> free_t[k]) & 1) o |= (size_t)1 << k;
      double p = re[i] * re[i] + im[i] * im[i];
      op[o] = op[o] + p;
      total += p;
    }
    if (total <= 0) fail(BF_EINVAL, "Measurement probability is zero");
    int64_t rng = seed % 2147483647;
    rng = (rng * 48271) % 2147483647;
    double r = (double)rng / (double)2147483647 * total;
    size_t chosen = 0;
    double acc = 0;
    for (size_t i = 0; i < oc; ++i) {
      acc += op[i];
      if (r <= acc) { chosen = i; break; }
    }
    double cp = op[chosen];
    if (cp <= 0) fail(BF_EINVAL, "Measurement outcome probability is zero");
    double inv = 1.0 / sqrt(cp);
    for (size_t i = 0; i < N; ++i) {
      bool match = true;
      for (int j = 0; j < nt; ++j) {
        int bit = (int)((i >> targets[j]) & 1);
        int want = (values && values[j] >= 0) ? values[j] : (int)((chosen >> free_pos[j]) & 1);
        if (bit != want) { match = false; break; }
      }
      if (match) { re[i] = re[i] * inv; im[i] = im[i] * inv; }
      else { re[i] = 0.0; im[i] = 0.0; }
    }
    if (outcome) *outcome = chosen;
    if (prob) *prob = cp;
    return BF_OK;
  } catch (const OrError& e) {
    set_err(err, errlen, e.msg);
    return e.code;
  }
}

// The k most probable indices, by descending re^2 + im^2, ties by index.
void or_topk(int32_t n, const double* re, const double* im, int32_t k, uint64_t* idx, double* prob) {
  size_t N = (size_t)1 << n;
  std::vector<std::pair<double, uint64_t>> v(N);
  for (size_t i = 0; i < N; ++i) v[i] = {re[i] * re[i] + im[i] * im[i], i};
  std::partial_sort(v.begin(), v.begin() + k, v.end(), [](const auto& a, const auto& b) {
    if (a.first != b.first) return a.first > b.first;
    return a.second < b.second;
  });
  for (int i = 0; i < k; ++i) { idx[i] = v[i].second; prob[i] = v[i].first; }
}

void or_bit_reverse_indices(int32_t n, uint64_t* out_index) {
  size_t N = (size_t)1 << n;
  for (size_t i = 0; i < N; ++i) out_index[i] = rev_bits(i, n);
}

double or_norm2(int32_t n, const double* re, const double* im) {
  size_t N = (size_t)1 << n;
  double acc = 0;
  for (size_t i = 0; i < N; ++i) acc += re[i] * re[i] + im[i] * im[i];
  return acc;
}

int32_t or_num_cores(void) {
  unsigned c = std::thread::hardware_concurrency();
  return c ? (int32_t)c : 1;
}

// fuse_circuit / fuse_circuit_specialized_pairs (transformations_fusion.mojo:
// 879-908): contiguous pairs (or special pairs), then same-target runs
int or_fuse(int32_t mode, const bf_op* in, int64_t nin, bf_op* out, int64_t out_cap, double* mats,
            int64_t mats_cap, int64_t* nout, char* err, size_t errlen) {
  try {
    if (!nout || (nin > 0 && !in)) fail(BF_EINVAL, "null argument");
    std::vector<Item> items;
    for (int64_t i = 0; i < nin; ++i) {
      const bf_op& o = in[i];
      if (o.kind == BF_OP_GATE && (o.flags & BF_OPF_FUSE_WITH_NEXT) && i + 1 < nin) {
        Item it;  // an existing fused pair passes through
        it.kind = IT_PAIR;
        it.op[0] = o;
        it.op[1] = in[i + 1];
        items.push_back(it);
        ++i;
      } else if (o.kind == BF_OP_GATE) {
        items.push_back(gate_item(o));
      } else {
        Item it;
        it.kind = IT_OTHER;
        it.op[0] = o;
        items.push_back(it);
      }
    }
    items = same_target_runs(mode == 1 ? special_pairs(items) : contiguous_pairs(items, false));
    int64_t k = 0, d = 0;
    auto put = [&](const bf_op& o) {
      if (k < out_cap && out) out[k] = o;
      ++k;
    };
    for (const Item& it : items) {
      if (it.kind == IT_GATE || it.kind == IT_OTHER) {
        put(it.op[0]);
      } else if (it.kind == IT_PAIR) {
        put(it.op[0]);
        put(it.op[1]);
      } else {
        bf_op o;
        std::memset(&o, 0, sizeof o);
        o.kind = it.kind == IT_UNITARY ? BF_OP_UNITARY : BF_OP_CUNITARY;
        o.target = it.target;
        o.target2 = it.m;
        if (it.kind == IT_CUNITARY) {
          o.controls = 1ull << it.control;
          o.ncontrols = 1;
        }
        const int64_t need = 2 * (int64_t)it.u.size();
        if (mats && d + need <= mats_cap) {
          for (size_t e = 0; e < it.u.size(); ++e) {
            mats[d + 2 * (int64_t)e] = it.u[e].re;
            mats[d + 2 * (int64_t)e + 1] = it.u[e].im;
          }
          o.data = mats + d;
        }
        d += need;
        put(o);
      }
    }
    *nout = k;
    if (k > out_cap || (mats_cap < d)) fail(BF_EINVAL, "output too small: %lld ops, %lld doubles needed",
                                           (long long)k, (long long)d);
    return BF_OK;
  } catch (const OrError& e) {
    set_err(err, errlen, e.msg);
    return e.code;
  }
}

}  // extern "C"

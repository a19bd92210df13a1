// amp_math.cuh — per-precision amplitude arithmetic used by every kernel.
//
// Three policies share one interface so that each kernel is written once:
//   PolF64 : double2 in HBM, FP64 registers (DFMA).
//   PolDF  : double2 in HBM, double-float registers: each FP64 value is held
//            as an unevaluated sum hi + lo of two FP32 numbers (about 48
//            significant bits).  Products and sums use the error-free
//            transformations TwoSum (Knuth, TAOCP vol. 2, 4.2.2), Fast2Sum and
//            TwoProduct-by-FMA (Dekker 1971).  FP64 -> pair and pair -> FP64
//            conversions are done with integer bit arithmetic, so the slow
//            FP64 pipe of this part is never used on the hot path.
//   PolF32 : float2 in HBM, FP32 registers.
//
// Gate coefficients arrive in two forms prepared on the host: m[8] as FP64
// and mhl[16] as (hi, lo) FP32 pairs of the same eight values (hi = the
// FP64 value rounded to FP32, lo = the rounded remainder).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bf {

constexpr double kSqHalf = 0.7071067811865476;  // sq_half in transform_h_scalar
constexpr float kSqHalfHi = (float)kSqHalf;      // kSqHalf as an FP32 pair
constexpr float kSqHalfLo = (float)(kSqHalf - (double)kSqHalfHi);

// ---------------------------------------------------------------------------
// double-float primitives (all operations round-to-nearest FP32; no
// contraction is possible in the add/sub sequences; products use explicit
// fmaf so the compiler's contraction cannot change them).
struct dfl {
  float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dfl df_norm(float s, float e) {
  dfl r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}

// x + y with one TwoSum on the leading parts (absolute error ~2^-48 of the
// larger operand, which is the error measure amplitude parity uses).
__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
  float s, e;
  two_sum(x.hi, y.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
  return df_norm(s, e);
}

__device__ __forceinline__ dfl df_neg(dfl x) { return dfl{-x.hi, -x.lo}; }
__device__ __forceinline__ dfl df_sub(dfl x, dfl y) { return df_add(x, df_neg(y)); }

// x * c
__device__ __forceinline__ dfl df_mul(dfl x, dfl c) {
  float p = __fmul_rn(x.hi, c.hi);
  float e = fmaf(x.hi, c.hi, -p);
  e = fmaf(x.hi, c.lo, e);
  e = fmaf(x.lo, c.hi, e);
  return df_norm(p, e);
}

// a0*b0 + a1*b1 + a2*b2 + a3*b3: products by TwoProduct, leading parts summed
// by a TwoSum chain, all error terms added in FP32, one final renormalisation.
__device__ __forceinline__ dfl df_dot4(dfl a0, dfl b0, dfl a1, dfl b1, dfl a2,
                                        dfl b2, dfl a3, dfl b3) {
  float p0 = __fmul_rn(a0.hi, b0.hi), e0 = fmaf(a0.hi, b0.hi, -p0);
  float p1 = __fmul_rn(a1.hi, b1.hi), e1 = fmaf(a1.hi, b1.hi, -p1);
  float p2 = __fmul_rn(a2.hi, b2.hi), e2 = fmaf(a2.hi, b2.hi, -p2);
  float p3 = __fmul_rn(a3.hi, b3.hi), e3 = fmaf(a3.hi, b3.hi, -p3);
  e0 = fmaf(a0.hi, b0.lo, fmaf(a0.lo, b0.hi, e0));
  e1 = fmaf(a1.hi, b1.lo, fmaf(a1.lo, b1.hi, e1));
  e2 = fmaf(a2.hi, b2.lo, fmaf(a2.lo, b2.hi, e2));
  e3 = fmaf(a3.hi, b3.lo, fmaf(a3.lo, b3.hi, e3));
  float s, t1, t2, t3;
  two_sum(p0, p1, s, t1);
  two_sum(s, p2, s, t2);
  two_sum(s, p3, s, t3);
  float err = __fadd_rn(__fadd_rn(__fadd_rn(e0, e1), __fadd_rn(e2, e3)),
                        __fadd_rn(__fadd_rn(t1, t2), t3));
  return df_norm(s, err);
}

// a0*b0 + a1*b1 + a2*b2, as df_dot4
__device__ __forceinline__ dfl df_dot3(dfl a0, dfl b0, dfl a1, dfl b1, dfl a2, dfl b2) {
  float p0 = __fmul_rn(a0.hi, b0.hi), e0 = fmaf(a0.hi, b0.hi, -p0);
  float p1 = __fmul_rn(a1.hi, b1.hi), e1 = fmaf(a1.hi, b1.hi, -p1);
  float p2 = __fmul_rn(a2.hi, b2.hi), e2 = fmaf(a2.hi, b2.hi, -p2);
  e0 = fmaf(a0.hi, b0.lo, fmaf(a0.lo, b0.hi, e0));
  e1 = fmaf(a1.hi, b1.lo, fmaf(a1.lo, b1.hi, e1));
  e2 = fmaf(a2.hi, b2.lo, fmaf(a2.lo, b2.hi, e2));
  float s, t1, t2;
  two_sum(p0, p1, s, t1);
  two_sum(s, p2, s, t2);
  float err = __fadd_rn(__fadd_rn(e0, e1), __fadd_rn(e2, __fadd_rn(t1, t2)));
  return df_norm(s, err);
}

// a0*b0 + a1*b1
__device__ __forceinline__ dfl df_dot2(dfl a0, dfl b0, dfl a1, dfl b1) {
  float p0 = __fmul_rn(a0.hi, b0.hi), e0 = fmaf(a0.hi, b0.hi, -p0);
  float p1 = __fmul_rn(a1.hi, b1.hi), e1 = fmaf(a1.hi, b1.hi, -p1);
  e0 = fmaf(a0.hi, b0.lo, fmaf(a0.lo, b0.hi, e0));
  e1 = fmaf(a1.hi, b1.lo, fmaf(a1.lo, b1.hi, e1));
  float s, t;
  two_sum(p0, p1, s, t);
  return df_norm(s, __fadd_rn(__fadd_rn(e0, e1), t));
}

// FP64 bits -> (hi, lo).  hi keeps the leading 24 significant bits
// (truncated); lo is the remaining 29 bits rounded to the nearest 23
// (|x - hi - lo| <= 2^-47 |x|, unbiased, so errors do not drift over many
// passes).  |x| below 2^-126 is flushed to zero (absolute error < 1.2e-38);
// the lo part of |x| below 2^-80 is dropped (absolute error < 2^-103).
// Inf/NaN map to NaN so that they stay visible.
__device__ __forceinline__ dfl df_from_double(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  unsigned sign = hw & 0x80000000u;
  int e = (int)((hw >> 20) & 0x7ffu);
  int ef = e - 896;  // FP32 biased exponent of hi
  unsigned mant23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
  dfl r;
  if (ef <= 0) {
    r.hi = 0.f;
    r.lo = 0.f;
    return r;
  }
  if (e == 0x7ff || ef >= 255) {
    r.hi = __int_as_float(0x7fc00000);
    r.lo = 0.f;
    return r;
  }
  r.hi = __int_as_float((int)(sign | ((unsigned)ef << 23) | mant23));
  // rounded top 23 of the 29 remainder bits; a carry to 2^23 still decodes
  // correctly below (0x4B800000 - 2^23 = 2^23)
  unsigned r23 = ((lw & 0x1fffffffu) + 32u) >> 6;
  int es = e - 942;  // FP32 biased exponent of 2^(e - 1069)
  float lo = 0.f;
  if (es >= 1) {
    float rf = __fsub_rn(__int_as_float((int)(0x4B000000u | r23)), 8388608.0f);
    lo = __fmul_rn(rf, __int_as_float(es << 23));
  }
  r.lo = __int_as_float(__float_as_int(lo) ^ (int)sign);
  return r;
}

// (hi, lo) -> FP64, rounded to nearest (ties away from zero) in integer
// arithmetic: M = hi's 24-bit significand << 29 plus lo aligned to it.
__device__ __forceinline__ double df_to_double(dfl v) {
  unsigned hb = (unsigned)__float_as_int(v.hi), lb = (unsigned)__float_as_int(v.lo);
  int eh = (int)((hb >> 23) & 0xffu);
  if (eh == 0) return 0.0;  // hi is zero (or FP32-subnormal): value below 2^-126
  if (eh == 0xff) return __longlong_as_double(0x7ff8000000000000ll);
  // 2 guard bits below the FP64 significand: M has 55 bits at scale 2^-2
  long long M = (long long)((hb & 0x7fffffu) | 0x800000u) << 31;
  int el = (int)((lb >> 23) & 0xffu);
  if (el != 0) {
    long long ml = (long long)((lb & 0x7fffffu) | 0x800000u);
    int sh = eh - el;  // >= 0 for a normalised pair
    long long L;
    if (sh <= 31) L = ml << (31 - sh);
    else if (sh < 31 + 25) L = (ml + (1ll << (sh - 32))) >> (sh - 31);
    else L = 0;
    if ((hb ^ lb) & 0x80000000u) M -= L; else M += L;
  }
  int E = eh + 896;  // FP64 biased exponent for M in [2^54, 2^55)
  int drop = 2;
  if (M >= (1ll << 55)) {
    drop = 3;
    E += 1;
  } else if (M < (1ll << 54)) {
    drop = 1;
    E -= 1;
  }
  M = (M + (1ll << (drop - 1))) >> drop;
  if (M >= (1ll << 53)) {  // rounding carried into a new bit
    M >>= 1;
    E += 1;
  }
  unsigned long long bits = ((unsigned long long)(hb & 0x80000000u) << 32) |
                            ((unsigned long long)E << 52) |
                            ((unsigned long long)M & 0xfffffffffffffull);
  return __longlong_as_double((long long)bits);
}

// ---------------------------------------------------------------------------
// Policies.

struct PolF64 {
  using Glob = double2;
  using Smem = double2;
  using E = double;
  struct R {
    double re, im;
  };
  struct Coef {
    double v[8];
  };
  static constexpr int kStoreBytes = 16;

  __device__ static __forceinline__ R from_glob(Glob a) { return R{a.x, a.y}; }
  __device__ static __forceinline__ Glob to_glob(R r) { return make_double2(r.re, r.im); }
  __device__ static __forceinline__ R from_smem(Smem a) { return R{a.x, a.y}; }
  __device__ static __forceinline__ Smem to_smem(R r) { return make_double2(r.re, r.im); }
  __device__ static __forceinline__ Coef coef(const double* m, const float*) {
    Coef c;
#pragma unroll
    for (int i = 0; i < 8; ++i) c.v[i] = m[i];
    return c;
  }
  // the term order of process_pair_scalar (transformations_scalar.mojo:17-40)
  __device__ static __forceinline__ void dense(R& u, R& v, const Coef& g) {
    const double* m = g.v;
    R a = u, b = v;
    u.re = a.re * m[0] - a.im * m[1] + b.re * m[2] - b.im * m[3];
    u.im = a.re * m[1] + a.im * m[0] + b.re * m[3] + b.im * m[2];
    v.re = a.re * m[4] - a.im * m[5] + b.re * m[6] - b.im * m[7];
    v.im = a.re * m[5] + a.im * m[4] + b.re * m[7] + b.im * m[6];
  }
  __device__ static __forceinline__ void dense_r(R& u, R& v, const Coef& g) { dense(u, v, g); }
  __device__ static __forceinline__ void hadamard(R& u, R& v) {
    R a = u, b = v;
    u.re = (a.re + b.re) * kSqHalf;
    u.im = (a.im + b.im) * kSqHalf;
    v.re = (a.re - b.re) * kSqHalf;
    v.im = (a.im - b.im) * kSqHalf;
  }
  __device__ static __forceinline__ void ry(R& u, R& v, const Coef& g) {
    double c = g.v[0], s = g.v[4];
    R a = u, b = v;
    u.re = a.re * c - b.re * s;
    u.im = a.im * c - b.im * s;
    v.re = a.re * s + b.re * c;
    v.im = a.im * s + b.im * c;
  }
  __device__ static __forceinline__ R zero() { return R{0.0, 0.0}; }
  // acc + a * b, with apply_unitary's term order (transformations_unitary.mojo:67-68)
  __device__ static __forceinline__ R fma(R a, R b, R acc) {
    return R{acc.re + (a.re * b.re - a.im * b.im), acc.im + (a.re * b.im + a.im * b.re)};
  }
  // multiply by the complex coefficient (v[k], v[k+1])
  __device__ static __forceinline__ void cmul(R& x, const Coef& g, int k) { cmul_by(x, g.v[k], g.v[k + 1]); }
  __device__ static __forceinline__ void cmul_by(R& x, E c, E s) {
    R a = x;
    x.re = a.re * c - a.im * s;
    x.im = a.re * s + a.im * c;
  }
};

struct PolDF {
  using Glob = double2;
  using Smem = float4;  // (re.hi, re.lo, im.hi, im.lo)
  using E = dfl;
  struct R {
    dfl re, im;
  };
  struct Coef {
    dfl v[8];
  };
  static constexpr int kStoreBytes = 16;

  __device__ static __forceinline__ R from_glob(Glob a) {
    return R{df_from_double(a.x), df_from_double(a.y)};
  }
  __device__ static __forceinline__ Glob to_glob(R r) {
    return make_double2(df_to_double(r.re), df_to_double(r.im));
  }
  __device__ static __forceinline__ R from_smem(Smem a) {
    return R{dfl{a.x, a.y}, dfl{a.z, a.w}};
  }
  __device__ static __forceinline__ Smem to_smem(R r) {
    return make_float4(r.re.hi, r.re.lo, r.im.hi, r.im.lo);
  }
  __device__ static __forceinline__ Coef coef(const double*, const float* hl) {
    Coef c;
#pragma unroll
    for (int i = 0; i < 8; ++i) c.v[i] = dfl{hl[2 * i], hl[2 * i + 1]};
    return c;
  }
  __device__ static __forceinline__ void dense(R& u, R& v, const Coef& g) {
    const dfl* m = g.v;
    R a = u, b = v;
    u.re = df_dot4(a.re, m[0], df_neg(a.im), m[1], b.re, m[2], df_neg(b.im), m[3]);
    u.im = df_dot4(a.re, m[1], a.im, m[0], b.re, m[3], b.im, m[2]);
    v.re = df_dot4(a.re, m[4], df_neg(a.im), m[5], b.re, m[6], df_neg(b.im), m[7]);
    v.im = df_dot4(a.re, m[5], a.im, m[4], b.re, m[7], b.im, m[6]);
  }
  // m00 real (m[1] == 0): the a-terms of u need one product each
  __device__ static __forceinline__ void dense_r(R& u, R& v, const Coef& g) {
    const dfl* m = g.v;
    R a = u, b = v;
    u.re = df_dot3(a.re, m[0], b.re, m[2], df_neg(b.im), m[3]);
    u.im = df_dot3(a.im, m[0], b.re, m[3], b.im, m[2]);
    v.re = df_dot4(a.re, m[4], df_neg(a.im), m[5], b.re, m[6], df_neg(b.im), m[7]);
    v.im = df_dot4(a.re, m[5], a.im, m[4], b.re, m[7], b.im, m[6]);
  }
  __device__ static __forceinline__ void hadamard(R& u, R& v) {
    const dfl s = dfl{kSqHalfHi, kSqHalfLo};
    R a = u, b = v;
    u.re = df_mul(df_add(a.re, b.re), s);
    u.im = df_mul(df_add(a.im, b.im), s);
    v.re = df_mul(df_sub(a.re, b.re), s);
    v.im = df_mul(df_sub(a.im, b.im), s);
  }
  __device__ static __forceinline__ void ry(R& u, R& v, const Coef& g) {
    dfl c = g.v[0], s = g.v[4];
    R a = u, b = v;
    u.re = df_dot2(a.re, c, df_neg(b.re), s);
    u.im = df_dot2(a.im, c, df_neg(b.im), s);
    v.re = df_dot2(a.re, s, b.re, c);
    v.im = df_dot2(a.im, s, b.im, c);
  }
  __device__ static __forceinline__ R zero() { return R{dfl{0.f, 0.f}, dfl{0.f, 0.f}}; }
  __device__ static __forceinline__ R fma(R a, R b, R acc) {
    return R{df_add(acc.re, df_dot2(a.re, b.re, df_neg(a.im), b.im)),
             df_add(acc.im, df_dot2(a.re, b.im, a.im, b.re))};
  }
  __device__ static __forceinline__ void cmul(R& x, const Coef& g, int k) { cmul_by(x, g.v[k], g.v[k + 1]); }
  __device__ static __forceinline__ void cmul_by(R& x, E c, E s) {
    R a = x;
    x.re = df_dot2(a.re, c, df_neg(a.im), s);
    x.im = df_dot2(a.re, s, a.im, c);
  }
};

struct PolF32 {
  using Glob = float2;
  using Smem = float2;
  using E = float;
  struct R {
    float re, im;
  };
  struct Coef {
    float v[8];
  };
  static constexpr int kStoreBytes = 8;

  __device__ static __forceinline__ R from_glob(Glob a) { return R{a.x, a.y}; }
  __device__ static __forceinline__ Glob to_glob(R r) { return make_float2(r.re, r.im); }
  __device__ static __forceinline__ R from_smem(Smem a) { return R{a.x, a.y}; }
  __device__ static __forceinline__ Smem to_smem(R r) { return make_float2(r.re, r.im); }
  __device__ static __forceinline__ Coef coef(const double*, const float* hl) {
    Coef c;
#pragma unroll
    for (int i = 0; i < 8; ++i) c.v[i] = hl[2 * i];
    return c;
  }
  __device__ static __forceinline__ void dense(R& u, R& v, const Coef& g) {
    const float* m = g.v;
    R a = u, b = v;
    u.re = a.re * m[0] - a.im * m[1] + b.re * m[2] - b.im * m[3];
    u.im = a.re * m[1] + a.im * m[0] + b.re * m[3] + b.im * m[2];
    v.re = a.re * m[4] - a.im * m[5] + b.re * m[6] - b.im * m[7];
    v.im = a.re * m[5] + a.im * m[4] + b.re * m[7] + b.im * m[6];
  }
  // sqrt(0.5) rounded to FP32 is 1.7e-8 low: multiplying by it would shrink
  // the norm at every H.  x*hi + x*lo with one FMA keeps the product within
  // half an ulp of x*sqrt(0.5), so no bias builds up.
  __device__ static __forceinline__ float mul_sq_half(float x) { return fmaf(x, kSqHalfHi, x * kSqHalfLo); }
  __device__ static __forceinline__ void dense_r(R& u, R& v, const Coef& g) { dense(u, v, g); }
  __device__ static __forceinline__ void hadamard(R& u, R& v) {
    R a = u, b = v;
    u.re = mul_sq_half(a.re + b.re);
    u.im = mul_sq_half(a.im + b.im);
    v.re = mul_sq_half(a.re - b.re);
    v.im = mul_sq_half(a.im - b.im);
  }
  __device__ static __forceinline__ void ry(R& u, R& v, const Coef& g) {
    float c = g.v[0], s = g.v[4];
    R a = u, b = v;
    u.re = a.re * c - b.re * s;
    u.im = a.im * c - b.im * s;
    v.re = a.re * s + b.re * c;
    v.im = a.im * s + b.im * c;
  }
  __device__ static __forceinline__ R zero() { return R{0.f, 0.f}; }
  __device__ static __forceinline__ R fma(R a, R b, R acc) {
    return R{acc.re + (a.re * b.re - a.im * b.im), acc.im + (a.re * b.im + a.im * b.re)};
  }
  __device__ static __forceinline__ void cmul(R& x, const Coef& g, int k) { cmul_by(x, g.v[k], g.v[k + 1]); }
  __device__ static __forceinline__ void cmul_by(R& x, E c, E s) {
    R a = x;
    x.re = a.re * c - a.im * s;
    x.im = a.re * s + a.im * c;
  }
};

// Applies one lowered gate kind to the pair (u, v) = (bit 0, bit 1).
template <class P>
__device__ __forceinline__ void apply_pair(int kind, typename P::R& u,
                                           typename P::R& v,
                                           const typename P::Coef& g) {
  switch (kind) {
    case 0: P::dense(u, v, g); break;            // GK_DENSE
    case 1: P::hadamard(u, v); break;            // GK_H
    case 2: { typename P::R t = u; u = v; v = t; break; }  // GK_SWAP
    case 3: P::cmul(v, g, 6); break;             // GK_PHASE
    case 4: P::cmul(u, g, 0); P::cmul(v, g, 6); break;  // GK_DIAG
    case 6: P::dense_r(u, v, g); break;          // GK_DENSE_R
    default: P::ry(u, v, g); break;              // GK_RY
  }
}

__device__ __forceinline__ uint64_t insert_zero_bit(uint64_t x, int pos) {
  uint64_t mask = (1ull << pos) - 1;
  return ((x & ~mask) << 1) | (x & mask);
}

}  // namespace bf

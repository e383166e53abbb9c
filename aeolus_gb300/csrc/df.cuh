// Double-float ("df") arithmetic: a value is hi + lo with two f32 words
// (~48-bit significand), built from error-free transforms (Knuth two-sum,
// FMA two-product; Dekker 1971, Hida-Li-Bailey 2001).  Used by the split-
// precision row stage, where GB300's f32 pipe is ~64x its f64 pipe.
#pragma once

#include <cuda_runtime.h>

namespace aeolus {

struct df {
  float hi, lo;
};

struct cdf {  // complex df, 16 bytes (same footprint as double2)
  df re, im;
};

__device__ __forceinline__ df df_make(float h, float l) { return df{h, l}; }

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return df{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = a + b;
  return df{s, b - (s - a)};
}

// Accurate addition: error ~2^-48 relative to the result.
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}

// Faster addition (Dekker): error ~2^-48 relative to |a| + |b| rather than
// to the result -- the backward-stable bound an FFT butterfly needs.
__device__ __forceinline__ df df_add_fast(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}

// df + float: two-sum of the high words, the low word folded in once.
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// Multiplication by a power of two (exact).
__device__ __forceinline__ df df_scale2(df a, float p2) { return df{a.hi * p2, a.lo * p2}; }

// ---------------------------------------------------------------------
// Two double-floats side by side.  An f2 word holds two f32 lanes, and
// Blackwell's packed two-lane FP32 instructions (add/sub/mul/fma .f32x2)
// operate on both with one instruction, each lane rounded exactly as its
// scalar form: df2 arithmetic below is the df arithmetic above in the same
// order of operations, two values at a time, in half the instructions.
typedef unsigned long long f2;

__device__ __forceinline__ f2 f2_pack(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2 r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 f2_neg(f2 a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ f2 f2_splat(float a) { return f2_pack(a, a); }

struct df2 {
  f2 hi, lo;
};

__device__ __forceinline__ df2 df2_pack(df a, df b) { return df2{f2_pack(a.hi, b.hi), f2_pack(a.lo, b.lo)}; }
__device__ __forceinline__ void df2_unpack(df2 v, df& a, df& b) {
  f2_unpack(v.hi, a.hi, b.hi);
  f2_unpack(v.lo, a.lo, b.lo);
}
__device__ __forceinline__ df2 two_sum2(f2 a, f2 b) {
  const f2 s = f2_add(a, b);
  const f2 bb = f2_sub(s, a);
  return df2{s, f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb))};
}
__device__ __forceinline__ df2 fast_two_sum2(f2 a, f2 b) {
  const f2 s = f2_add(a, b);
  return df2{s, f2_sub(b, f2_sub(s, a))};
}
__device__ __forceinline__ df2 df2_add_fast(df2 a, df2 b) {
  df2 s = two_sum2(a.hi, b.hi);
  s.lo = f2_add(s.lo, f2_add(a.lo, b.lo));
  return fast_two_sum2(s.hi, s.lo);
}
__device__ __forceinline__ df2 df2_neg(df2 a) { return df2{f2_neg(a.hi), f2_neg(a.lo)}; }
// df_add of two pairs (the accurate addition, same operations lane by lane).
__device__ __forceinline__ df2 df2_add(df2 a, df2 b) {
  df2 s = two_sum2(a.hi, b.hi);
  const df2 t = two_sum2(a.lo, b.lo);
  s.lo = f2_add(s.lo, t.hi);
  s = fast_two_sum2(s.hi, s.lo);
  s.lo = f2_add(s.lo, t.lo);
  return fast_two_sum2(s.hi, s.lo);
}
__device__ __forceinline__ df2 df2_mul(df2 a, df2 b) {
  const f2 p = f2_mul(a.hi, b.hi);
  f2 e = f2_fma(a.hi, b.hi, f2_neg(p));
  e = f2_fma(a.hi, b.lo, e);
  e = f2_fma(a.lo, b.hi, e);
  return fast_two_sum2(p, e);
}
__device__ __forceinline__ df2 df2_scale2(df2 a, f2 p2) { return df2{f2_mul(a.hi, p2), f2_mul(a.lo, p2)}; }

__device__ __forceinline__ df2 df2_splat(df a) { return df2{f2_splat(a.hi), f2_splat(a.lo)}; }
__device__ __forceinline__ df2 df2_sub_fast(df2 a, df2 b) { return df2_add_fast(a, df2_neg(b)); }
// i a for a complex value in the lanes (re, im): (-im, re).
__device__ __forceinline__ f2 f2_times_i(f2 a) { return ((a >> 32) | (a << 32)) ^ 0x80000000ull; }
__device__ __forceinline__ df2 df2_times_i(df2 a) { return df2{f2_times_i(a.hi), f2_times_i(a.lo)}; }

// FP64 <-> double-float by integer operations on the bit patterns (no FP64
// instruction; GB300's FP64 pipe is ~1/64 of its f32 pipe).
// x as hi + lo: hi = x truncated to 24 significant bits, lo = the other 29
// bits rounded to a float, so |x - hi - lo| <= 2^-48 |x| and |lo| < ulp(hi).
// |x| below 2^-126 gives 0; |x| of 2^128 or more (and NaN) +-infinity.
__device__ __forceinline__ df df_of_f64(double x) {
  const unsigned l = static_cast<unsigned>(__double2loint(x)), h = static_cast<unsigned>(__double2hiint(x));
  const unsigned sg = h & 0x80000000u, ah = h & 0x7FFFFFFFu;
  const int ex = static_cast<int>(ah >> 20);  // biased exponent: 2^(ex - 1023) <= |x|
  if (ex < 897) return df{0.f, 0.f};
  if (ex > 1150) return df{__uint_as_float(sg | 0x7F800000u), 0.f};
  const float hi = __uint_as_float(sg | __funnelshift_l(l, ah - (896u << 20), 3));
  // (l mod 2^29) 2^(ex - 1075) = ((l mod 2^29) 2^-52) 2^(ex - 1023)
  const float r = __uint2float_rn(l & 0x1FFFFFFFu) * 2.220446049250313080847e-16f;
  const float lo = r * __uint_as_float(static_cast<unsigned>(ex - 896) << 23);
  return df{hi, sg ? -lo : lo};
}
// A complex FP64 value as a df2 with the lanes (re, im).
__device__ __forceinline__ df2 df2_of_f64x2(double2 v) { return df2_pack(df_of_f64(v.x), df_of_f64(v.y)); }
// A float as the FP64 of the same value (denormal floats as 0), by its bits.
__device__ __forceinline__ double f64_of_f32(float f) {
  const unsigned u = __float_as_uint(f), e = (u >> 23) & 0xFFu;
  if (e == 0) return 0.0;
  const unsigned hw = (u & 0x80000000u) | ((e == 255u ? 2047u : e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
  return __hiloint2double(static_cast<int>(hw), static_cast<int>(u << 29));
}
// hi + lo rounded to FP64: the two words converted exactly, one FP64 addition.
__device__ __forceinline__ double f64_of_df(df v) { return f64_of_f32(v.hi) + f64_of_f32(v.lo); }
__device__ __forceinline__ double2 f64x2_of_df2(df2 v) {
  df a, b;
  df2_unpack(v, a, b);
  return make_double2(f64_of_df(a), f64_of_df(b));
}

// From / to double (f64 conversions: used only at stage boundaries).
__device__ __forceinline__ df df_from_double(double x) {
  const float h = __double2float_rn(x);
  return df{h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return cdf{df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ cdf cdf_addf(cdf a, cdf b) { return cdf{df_add_fast(a.re, b.re), df_add_fast(a.im, b.im)}; }
__device__ __forceinline__ cdf cdf_subf(cdf a, cdf b) {
  return cdf{df_add_fast(a.re, df_neg(b.re)), df_add_fast(a.im, df_neg(b.im))};
}
// Complex product with the faster additions (twiddle rotations).
__device__ __forceinline__ cdf cdf_mulf(cdf a, cdf b) {
  return cdf{df_add_fast(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))),
             df_add_fast(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ cdf cdf_sub(cdf a, cdf b) { return cdf{df_sub(a.re, b.re), df_sub(a.im, b.im)}; }
__device__ __forceinline__ cdf cdf_mul(cdf a, cdf b) {
  return cdf{df_sub(df_mul(a.re, b.re), df_mul(a.im, b.im)), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ cdf cdf_conj(cdf a) { return cdf{a.re, df_neg(a.im)}; }
__device__ __forceinline__ cdf cdf_i(cdf a) { return cdf{df_neg(a.im), a.re}; }  // i * a
__device__ __forceinline__ cdf cdf_scale(df s, cdf a) { return cdf{df_mul(s, a.re), df_mul(s, a.im)}; }
__device__ __forceinline__ cdf cdf_scale2(float p2, cdf a) { return cdf{df_scale2(a.re, p2), df_scale2(a.im, p2)}; }
__device__ __forceinline__ cdf cdf_zero() { return cdf{df{0.f, 0.f}, df{0.f, 0.f}}; }

__device__ __forceinline__ cdf cdf_from_double2(double2 v) { return cdf{df_from_double(v.x), df_from_double(v.y)}; }
__device__ __forceinline__ double2 cdf_to_double2(cdf v) { return make_double2(df_to_double(v.re), df_to_double(v.im)); }

// Twiddles are stored as float4 (re.hi, re.lo, im.hi, im.lo).
__device__ __forceinline__ cdf cdf_from_f4(float4 v) { return cdf{df{v.x, v.y}, df{v.z, v.w}}; }

// Per-row constants handed to the pointwise functors' df_op.
struct RowDf {
  df invc;  // 1 / cos(latitude) (clamped)
  df fj;    // planetary vorticity at the row (2 Omega sin lat), 0 if unused
  float c;  // cos(latitude) (for guards)
};

}  // namespace aeolus

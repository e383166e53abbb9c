// 64-bit fixed-point arithmetic of the split-precision longitude stage.
//
// A row of one field is held as integers X_k with one block exponent S
// (value X_k 2^S).  FFT additions are then exact 64-bit integer additions
// (two instructions, against ~11 f32 operations for a double-float sum), and
// a twiddle product is a 64 x 62-bit product truncated to 64 bits, built
// from 32-bit wide multiply-adds on 31-bit limbs:
//
//   x = xh 2^30 + xl (xl in [0, 2^30)),  W = w 2^61 = wh 2^31 + wl (wl in [0, 2^31))
//   x w = xh wh + (xh wl + 2 xl wh) 2^-31 + xl wl 2^-61
//
// The last term (< 1) is dropped and the middle one floored: the product is
// within 3 units of x w.  Every operand of a product stays below 2^59 in
// magnitude (so xh fits 29 bits and the limb sums stay below 2^63); the row
// stage picks the block exponent of its inputs from the transform length
// so that no butterfly can overflow.
//
// Spectra between the tensor-core stages and the row stage travel as
// packed words: a signed mantissa M (|M| <= 2^52) in bits 63..10 and an
// exponent e in [-512, 511] in bits 9..0, value M 2^e -- a 64-bit
// floating-point format whose encode / decode are a few integer operations.
//
// Products use explicit mad.wide.s32 (one wide multiply-add each); no 64-bit
// integer <-> float conversion is used anywhere, as those run on the FP64
// pipe.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

namespace aeolus {

struct cfx {
  long long re, im;
};

// Q61 twiddle / constant as 31-bit limbs: w 2^61 = h 2^31 + l.
struct FxK {
  int h, l;
};
struct FxW {  // complex twiddle, 16 bytes
  int ch, cl, sh, sl;
};

// Constants of the radix-3/5/8 butterflies.
struct FxConst {
  FxK h3, c1, c2, s1, s2, r2;
};

// Q61 limbs of a constant |v| <= 1 v 2^61 = h 2^31 + l, l in [0, 2^31).
inline FxK fx_const(double v) {
  const long long W = std::llrint(std::ldexp(v, 61));
  return FxK{static_cast<int>(W >> 31), static_cast<int>(W & 0x7FFFFFFFLL)};
}

// Butterfly constants: sin(2pi/3), cos(2pi/5), cos(4pi/5), sin(2pi/5), sin(4pi/5), 1/sqrt(2).
inline FxConst fx_consts() {
  return FxConst{fx_const(0.86602540378443864676), fx_const(0.30901699437494742410),
                 fx_const(-0.80901699437494742410), fx_const(0.95105651629515357212),
                 fx_const(0.58778525229247312917), fx_const(0.70710678118654752440)};
}

// a b + c with a 32 x 32 -> 64-bit signed product (one wide multiply-add).
__device__ __forceinline__ long long fx_madw(int a, int b, long long c) {
  long long d;
  asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
  return d;
}

__device__ __forceinline__ void fx_split(long long x, int& h, int& l2) {
  h = static_cast<int>(x >> 30);
  l2 = static_cast<int>(static_cast<unsigned>(x) << 1) & 0x7FFFFFFE;  // 2 (x mod 2^30)
}

// x * k (k real, |k| <= 1).
__device__ __forceinline__ long long fx_mulk(long long x, FxK k) {
  int h, l2;
  fx_split(x, h, l2);
  const long long t = fx_madw(l2, k.h, fx_madw(h, k.l, 0LL));
  return fx_madw(h, k.h, t >> 31);
}

// x * w (CONJ: x * conj(w)), |w| = 1.
template <bool CONJ>
__device__ __forceinline__ cfx fx_cmul(cfx x, FxW w) {
  int ah, al, bh, bl;
  fx_split(x.re, ah, al);
  fx_split(x.im, bh, bl);
  // re = a c -+ b s
  const int bhs = CONJ ? bh : -bh, bls = CONJ ? bl : -bl;
  const long long tr = fx_madw(bls, w.sh, fx_madw(bhs, w.sl, fx_madw(al, w.ch, fx_madw(ah, w.cl, 0LL))));
  const long long re = fx_madw(ah, w.ch, fx_madw(bhs, w.sh, tr >> 31));
  // im = +-a s + b c
  const int ahs = CONJ ? -ah : ah, als = CONJ ? -al : al;
  const long long ti = fx_madw(bl, w.ch, fx_madw(bh, w.cl, fx_madw(als, w.sh, fx_madw(ahs, w.sl, 0LL))));
  const long long im = fx_madw(ahs, w.sh, fx_madw(bh, w.ch, ti >> 31));
  return cfx{re, im};
}

__device__ __forceinline__ FxW fx_ldw(const FxW* p) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p));
  return FxW{v.x, v.y, v.z, v.w};
}

__device__ __forceinline__ cfx fx_add(cfx a, cfx b) { return cfx{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cfx fx_sub(cfx a, cfx b) { return cfx{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cfx fx_conj(cfx a) { return cfx{a.re, -a.im}; }
// sg i a for sg = +1 (POS) or -1
template <bool POS>
__device__ __forceinline__ cfx fx_i(cfx a) {
  return POS ? cfx{-a.im, a.re} : cfx{a.im, -a.re};
}

// Bit length of |x| (0 for x = 0).
__device__ __forceinline__ int fx_bitlen(long long x) {
  const unsigned long long a = static_cast<unsigned long long>(x < 0 ? -x : x);
  return 64 - __clzll(static_cast<long long>(a));
}

// x 2^-s rounded to an integer (round half up) for s >= 1; s is clamped to
// [1, 63] (s >= 63 gives 0 for |x| < 2^62; zero words may ask for s < 1).
__device__ __forceinline__ long long fx_rshift(long long x, int s) {
  s = max(1, min(s, 63));
  return (x + (1LL << (s - 1))) >> s;
}

// ---------------------------------------------------------- packed words
// Words are normalised: a nonzero mantissa has 52 or 53 significant bits
// (|M| in [2^51, 2^52]) unless the exponent sits at its lower limit, so
// |value| < 2^(e + 53) for every word and aligning a word to any block
// exponent at least that large is a right shift.
constexpr int kPackMant = 52;  // |M| <= 2^52
constexpr int kPackEmin = -512, kPackEmax = 511;
constexpr int kPackNone = -100000;  // magnitude bound of a zero word

__device__ __forceinline__ long long pk_mant(long long w) { return w >> 10; }
__device__ __forceinline__ int pk_exp(long long w) {
  return static_cast<int>(static_cast<unsigned>(w) << 22) >> 22;
}
// g with |value| < 2^g (kPackNone for zero).
__device__ __forceinline__ int pk_mag(long long w) { return w == 0 ? kPackNone : pk_exp(w) + kPackMant + 1; }

// M 2^e (|M| < 2^63) as a normalised packed word, mantissa rounded to 52 bits.
__device__ __forceinline__ long long pk_pack(long long M, int e) {
  if (M == 0) return 0;
  const int sh = fx_bitlen(M) - kPackMant;  // > 0: round right, <= 0: exact left shift
  long long N = sh > 0 ? (M + (1LL << (sh - 1))) >> sh : M << (-sh);
  e += sh;
  if (e < kPackEmin) {  // below the exponent range: denormal mantissa
    N = fx_rshift(N, kPackEmin - e);
    e = kPackEmin;
  } else if (e > kPackEmax) {  // beyond any finite double-float: saturate
    N = N > 0 ? (1LL << kPackMant) : -(1LL << kPackMant);
    e = kPackEmax;
  }
  return static_cast<long long>(static_cast<unsigned long long>(N) << 10) | (e & 1023);
}

// Packed word aligned to block exponent S >= its magnitude bound - 52:
// rint(M 2^(e - S)).
__device__ __forceinline__ long long pk_align(long long w, int S) { return fx_rshift(pk_mant(w), S - pk_exp(w)); }

// 2^p as a float in two factors (p1 + p2 = p, each a normal float).
__device__ __forceinline__ float fx_pow2f(int p) { return __int_as_float((p + 127) << 23); }
__device__ __forceinline__ void fx_pow2_split(int p, float& a, float& b) {
  const int p1 = max(-126, min(127, p));
  const int p2 = max(-126, min(127, p - p1));
  a = fx_pow2f(p1);
  b = fx_pow2f(p2);
}

}  // namespace aeolus

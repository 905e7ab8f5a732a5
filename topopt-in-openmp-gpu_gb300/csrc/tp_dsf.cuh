// Double-single arithmetic shared by the level-0 operator and the coarse
// band Cholesky.
#pragma once
#include <cuda_runtime.h>

namespace tp {

// Double-single arithmetic: a value is the unevaluated sum h + l of two FP32
// numbers (Dekker, "A floating-point technique for extending the available
// precision", 1971; the sum's error term is Knuth's two-sum). The FP64 pipe of
// this part issues one warp instruction per ~67 cycles per SM sub-partition,
// the FP32 pipe one per cycle, so an FP64 operand in memory can be worked on
// as a pair of floats for a fraction of the FP64 time.
// The sum of element contributions needs each operation's error bounded
// relative to its operands, as an FP64 evaluation bounds it by 2^-53
// (|a| + |b|), not relative to its result. Here: a + b takes the exact
// two-sum of the high parts and adds the low parts and the two-sum's error
// in FP32; a * b takes the exact product of the high parts (an FMA gives its
// error) plus the cross terms. Both are left unnormalised (l is not folded
// back into h), which keeps the bounds at ~2^-45 (|a| + |b|) and ~2^-45 |a| |b|
// -- l only ever holds rounding-sized terms -- for 8 and 4 instructions
// instead of 11 and 7; the sum h + l is formed in FP64 once, on output.
// The _rn intrinsics keep the compiler from contracting the error terms.
// 8-byte aligned, so a pair moves to and from shared memory as one access.
struct __align__(8) Dsf {
  float h, l;
  Dsf() = default;
  __device__ __forceinline__ Dsf(float v) : h(v), l(0.f) {}
  __device__ __forceinline__ Dsf(float a, float b) : h(a), l(b) {}
};
__device__ __forceinline__ Dsf operator+(Dsf a, Dsf b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));  // a.h + b.h - s, exactly
  return Dsf(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ Dsf operator-(Dsf a) { return Dsf(-a.h, -a.l); }
__device__ __forceinline__ Dsf operator-(Dsf a, Dsf b) { return a + (-b); }
__device__ __forceinline__ Dsf operator*(Dsf a, Dsf b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);  // the rounding error of p, exactly
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return Dsf(p, e);
}
__device__ __forceinline__ Dsf& operator+=(Dsf& a, Dsf b) { return a = a + b; }
__device__ __forceinline__ Dsf& operator-=(Dsf& a, Dsf b) { return a = a - b; }

// double -> double-single with integer operations only (the FP64 pipe stays
// free): h keeps the sign, the exponent and the leading 23 stored mantissa
// bits (truncated), l the remaining 29 bits rounded to 24, scaled by
// 2^-52 * 2^(e-1023) (two normal factors; one factor 2^(e-1075) would
// underflow below |v| = 2^-74). Within 2^-47 |v| down to |v| ~ 2^-102,
// where l turns subnormal; magnitudes below FP32's normal range become 0,
// above it infinity, NaN stays NaN.
__device__ __forceinline__ Dsf ds_from(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const unsigned sg = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7ffu);  // biased by 1023
  if (e < 897) return Dsf(0.f);              // |v| < 2^-126
  if (e > 1150) {                            // |v| >= 2^128, inf, NaN
    const bool nan = e == 2047 && ((hw & 0xfffffu) | lw) != 0u;
    return Dsf(__uint_as_float(nan ? 0x7fc00000u : (sg | 0x7f800000u)));
  }
  const float h = __uint_as_float(sg | ((unsigned)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
  // the low 29 mantissa bits carry weight 2^(e - 1023 - 52)
  const float l = __fmul_rn(__fmul_rn(__int2float_rn((int)(lw & 0x1fffffffu)), 0x1p-52f),
                            __uint_as_float((unsigned)(e - 896) << 23));
  return Dsf(h, sg ? -l : l);
}
// float -> double bits with integer operations, exact as the conversion is:
// on this part a conversion to FP64 holds the FP64 pipe as long as an add
// does (~67 cycles per warp instruction), so ds_to would otherwise cost three
// FP64 instructions instead of one. Subnormal floats are normalised; NaN
// keeps its payload with the quiet bit set.
__host__ __device__ __forceinline__ unsigned long long f32_to_f64_bits(unsigned u) {
  const unsigned long long sg = (unsigned long long)(u >> 31) << 63;
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e == 0xffu) return sg | (0x7ffULL << 52) | ((unsigned long long)m << 29) | (m ? (1ULL << 51) : 0ULL);
  if (e != 0u) return sg | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
  if (m == 0u) return sg;
#ifdef __CUDA_ARCH__
  const int p = 31 - __clz((int)m);  // top bit of a subnormal's mantissa, 0..22: value 2^(p-149) * 1.f
#else
  const int p = 31 - __builtin_clz(m);
#endif
  return sg | ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xfffffffffffffULL);
}
__device__ __forceinline__ double ds_to(Dsf a) {
  return __longlong_as_double((long long)f32_to_f64_bits(__float_as_uint(a.h))) +
         __longlong_as_double((long long)f32_to_f64_bits(__float_as_uint(a.l)));
}

// 1/sqrt(d): the FP32 estimate h = rsqrtf(d) refined by one Newton step for
// the reciprocal square root, r = h + h (1 - d h^2) / 2, with 1 - d h^2
// formed from the exact square of h and d's two parts (1 - p is exact for
// p near 1). From rsqrtf's few-ulp estimate the step leaves under 2^-42
// relative error.
__device__ __forceinline__ Dsf ds_rsqrt(Dsf d) {
  const float x = __fadd_rn(d.h, d.l);
  const float h = rsqrtf(x);
  const float th = __fmul_rn(h, h);
  const float tl = __fmaf_rn(h, h, -th);  // h^2 = th + tl exactly
  const float p = __fmul_rn(d.h, th);
  float pe = __fmaf_rn(d.h, th, -p);
  pe = __fmaf_rn(d.h, tl, pe);
  pe = __fmaf_rn(d.l, th, pe);            // d h^2 = p + pe
  const float e = __fsub_rn(__fsub_rn(1.0f, p), pe);
  return Dsf(h, __fmul_rn(__fmul_rn(0.5f, h), e));
}
// 1/d: the FP32 reciprocal h refined by one Newton step, r = h + h (1 - d h)
__device__ __forceinline__ Dsf ds_rcp(Dsf d) {
  const float x = __fadd_rn(d.h, d.l);
  const float h = __frcp_rn(x);
  const float p = __fmul_rn(d.h, h);
  float pe = __fmaf_rn(d.h, h, -p);
  pe = __fmaf_rn(d.l, h, pe);  // d h = p + pe
  const float e = __fsub_rn(__fsub_rn(1.0f, p), pe);
  return Dsf(h, __fmul_rn(h, e));
}
__device__ __forceinline__ Dsf& operator*=(Dsf& a, Dsf b) { return a = a * b; }
__device__ __forceinline__ float ds_val(Dsf a) { return __fadd_rn(a.h, a.l); }
__device__ __forceinline__ Dsf ds_sel(bool c, Dsf a, Dsf b) { return Dsf(c ? a.h : b.h, c ? a.l : b.l); }
__device__ __forceinline__ Dsf ds_shfl(Dsf v, int src) {
  return Dsf(__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src));
}

// Two double-single values in the halves of float2 registers: each FP32 step
// of Dsf's + and * becomes one f32x2 instruction for both values. The halves
// round to nearest independently, so each is the scalar result bit for bit.
// The operand a is the same in both halves and comes with its negated parts,
// so that the product's error terms can be formed negated where the scalar
// form negates an operand: fma(-x, y, z) = -fma(x, y, -z) exactly (round to
// nearest is odd-symmetric), and the sum never waits on a negation.
struct Dsf2 {
  float2 h, l;
};
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// acc + (a * b), a = (ah, -nah, -nal): p = a.h b.h, ne = -(the product's error)
__device__ __forceinline__ void ds2_add_prod(Dsf2& acc, float2 ah, float2 nah, float2 nal, float2 bh, float2 bl) {
  const float2 p = __fmul2_rn(ah, bh);
  float2 ne = __ffma2_rn(nah, bh, p);
  ne = __ffma2_rn(nah, bl, ne);
  ne = __ffma2_rn(nal, bh, ne);
  const float2 s = __fadd2_rn(acc.h, p);
  const float2 bb = f2sub(s, acc.h);
  const float2 e = __fadd2_rn(f2sub(acc.h, f2sub(s, bb)), f2sub(p, bb));
  acc.l = __fadd2_rn(e, f2sub(acc.l, ne));
  acc.h = s;
}

// storage (double) <-> value type V of a kernel written for both
template <typename V>
__device__ __forceinline__ V ds_in(double v);
template <>
__device__ __forceinline__ double ds_in<double>(double v) { return v; }
template <>
__device__ __forceinline__ Dsf ds_in<Dsf>(double v) { return ds_from(v); }
__device__ __forceinline__ double ds_out(double v) { return v; }
__device__ __forceinline__ double ds_out(Dsf v) { return ds_to(v); }

}  // namespace tp

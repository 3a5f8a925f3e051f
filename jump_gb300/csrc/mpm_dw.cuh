// mpm_dw.cuh -- double-word FP32 arithmetic for the MPM_PREC_DW step.
//
// A double-word ("DW") value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi)/2: 48 significant bits, relative rounding unit u^2 with
// u = 2^-24 (FP64 has 2^-53).  On GB300 the FP32 pipe issues 64 times as many
// lane operations per clock as the FP64 pipe, so a DW operation of 6-16 FP32
// instructions is several times cheaper than one FP64 instruction.
//
// Building blocks (each written from the published algorithm):
//  * TwoSum (Knuth, TAOCP vol. 2): s + e == a + b exactly, 6 additions;
//  * Fast2Sum (Dekker 1971): the same when the exponent of a >= that of b, 3;
//  * TwoProd with an FMA: p + e == a b exactly, 2;
//  * the double-word sum, products and their error bounds of M. Joldes,
//    J.-M. Muller, V. Popescu, "Tight and rigorous error bounds for basic
//    building blocks of double-word arithmetic", ACM TOMS 44(2), 2017:
//    SloppyDWPlusDW (absolute error a small multiple of u^2 (|x| + |y|)),
//    DWTimesFP3 and DWTimesDW3 (relative error a small multiple of u^2);
//  * square root and reciprocal by one Newton step from the correctly
//    rounded FP32 result, the residual formed exactly with TwoProd / FMA
//    (A. Karp, P. Markstein, "High-precision division and square root",
//    ACM TOMS 23(4), 1997).
// Every operation is written with the _rn intrinsics, so the compiler neither
// contracts nor reassociates the error terms away.
//
// FP64 <-> DW conversions run on the integer pipe: the hardware conversions
// issue on the FP64 pipe, which is the resource this arithmetic saves.
#pragma once

#include "mpm_common.cuh"

namespace jmpm {

struct dw {
  float hi, lo;
};

__device__ __forceinline__ dw dw_make(float h, float l) {
  dw r;
  r.hi = h;
  r.lo = l;
  return r;
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// SloppyDWPlusDW
__device__ __forceinline__ dw operator+(dw x, dw y) {
  float sh, sl, zh, zl;
  two_sum(x.hi, y.hi, sh, sl);
  const float w = __fadd_rn(sl, __fadd_rn(x.lo, y.lo));
  fast_two_sum(sh, w, zh, zl);
  return dw_make(zh, zl);
}

__device__ __forceinline__ dw operator-(dw x) { return dw_make(-x.hi, -x.lo); }
__device__ __forceinline__ dw operator-(dw x, dw y) { return x + (-y); }

// DWTimesDW3
__device__ __forceinline__ dw operator*(dw x, dw y) {
  float ch, cl1, zh, zl;
  two_prod(x.hi, y.hi, ch, cl1);
  const float tl1 = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.lo));
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  fast_two_sum(ch, __fadd_rn(cl1, cl2), zh, zl);
  return dw_make(zh, zl);
}

// DWTimesFP3
__device__ __forceinline__ dw operator*(dw x, float y) {
  float ch, cl1, zh, zl;
  two_prod(x.hi, y, ch, cl1);
  fast_two_sum(ch, __fmaf_rn(x.lo, y, cl1), zh, zl);
  return dw_make(zh, zl);
}

// x times a power of two or a sign (+-1, 0): exact, barring underflow
__device__ __forceinline__ dw dw_scale(dw x, float s) { return dw_make(__fmul_rn(x.hi, s), __fmul_rn(x.lo, s)); }

// c + a b: the product's pieces (DWTimesDW3 before its renormalisation) added
// to c as in SloppyDWPlusDW, one renormalisation in all
__device__ __forceinline__ dw dw_fma(dw a, dw b, dw c) {
  float ph, pl, sh, sl, zh, zl;
  two_prod(a.hi, b.hi, ph, pl);
  pl = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.lo, pl)));
  two_sum(c.hi, ph, sh, sl);
  fast_two_sum(sh, __fadd_rn(sl, __fadd_rn(c.lo, pl)), zh, zl);
  return dw_make(zh, zl);
}

// A sum of DW products kept as its leading float sum s (each product's
// leading part added by TwoSum) and the float sum c of every error term, so a
// term costs TwoProd, two cross FMAs, TwoSum and two adds; one TwoSum turns
// (s, c) into a DW at the end (s may cancel below c, so not Fast2Sum).  The
// error stays a small multiple of u^2 times the sum of the terms' magnitudes.
struct dw_acc {
  float s, c;
};

__device__ __forceinline__ void acc_fma(dw_acc& acc, dw a, dw b) {
  float ph, pl, sh, sl;
  two_prod(a.hi, b.hi, ph, pl);
  pl = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, pl));
  two_sum(acc.s, ph, sh, sl);
  acc.s = sh;
  acc.c = __fadd_rn(acc.c, __fadd_rn(sl, pl));
}

__device__ __forceinline__ dw acc_value(dw_acc acc) {
  float zh, zl;
  two_sum(acc.s, acc.c, zh, zl);
  return dw_make(zh, zl);
}

__device__ __forceinline__ dw dw_sqr(dw x) {
  float ph, pl, zh, zl;
  two_prod(x.hi, x.hi, ph, pl);
  pl = __fmaf_rn(__fadd_rn(x.hi, x.hi), x.lo, __fmaf_rn(x.lo, x.lo, pl));
  fast_two_sum(ph, pl, zh, zl);
  return dw_make(zh, zl);
}

// sqrt(q) for q >= 0 (0 otherwise): y = RN(sqrt(q.hi)), then
// sqrt(q) = y + (q - y^2) / (2 y) to second order in the residual, which is
// formed exactly (q.hi - RN(y^2) is exact by Sterbenz's lemma)
__device__ __forceinline__ dw dw_sqrt(dw q) {
  if (!(q.hi > 0.f)) return dw_make(0.f, 0.f);
  const float y = __fsqrt_rn(q.hi);
  float p, e, zh, zl;
  two_prod(y, y, p, e);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(q.hi, p), e), q.lo);
  fast_two_sum(y, __fmul_rn(r, __fdividef(0.5f, y)), zh, zl);  // 2-ulp quotient: the term is ~u y
  return dw_make(zh, zl);
}

// 1 / x for x != 0: r = RN(1 / x.hi), then 1/x = r + r (1 - x r) to second
// order, the residual 1 - x r from FMAs
__device__ __forceinline__ dw dw_recip(dw x) {
  const float r = __frcp_rn(x.hi);
  const float e = __fmaf_rn(-x.lo, r, __fmaf_rn(-x.hi, r, 1.0f));
  float zh, zl;
  fast_two_sum(r, __fmul_rn(r, e), zh, zl);
  return dw_make(zh, zl);
}

// x > 0 (a renormalised DW has hi == 0 only when lo == 0)
__device__ __forceinline__ bool dw_pos(dw x) { return x.hi > 0.f; }

// 1 - x for 0 <= x <= 1 (the upper hat value from the lower one)
__device__ __forceinline__ dw dw_one_minus(dw x) {
  float s, e, zh, zl;
  two_sum(1.0f, -x.hi, s, e);
  fast_two_sum(s, __fsub_rn(e, x.lo), zh, zl);
  return dw_make(zh, zl);
}

// FP64 -> DW on the integer pipe: hi is the double rounded to 24 significant
// bits (ties to even), lo the remainder (at most 29 bits) rounded to 24 bits,
// so hi + lo equals x to a relative 2^-49, for magnitudes in [2^-126, 2^128).
// Smaller magnitudes flush to a signed zero, larger ones give +-Inf, NaN a
// NaN; no path issues an FP64 instruction.
__device__ __forceinline__ dw dw_from(double x) {
  const unsigned bh = unsigned(__double2hiint(x)), bl = unsigned(__double2loint(x));
  const unsigned ex = (bh >> 20) & 0x7ffu;
  const unsigned sign = bh & 0x80000000u;
  if (ex - 897u > 253u) {
    const bool nan = ex == 0x7ffu && ((bh & 0x000fffffu) | bl) != 0u;
    const unsigned h = ex < 897u ? sign : (sign | 0x7f800000u | (nan ? 0x00400000u : 0u));
    return dw_make(__uint_as_float(h), 0.f);
  }
  // round the 52 fraction bits to their top 23: add 2^28 - 1 + bit 29, clear bits 0..28
  const unsigned sl = bl + (0x0fffffffu + ((bl >> 29) & 1u));
  const unsigned rh = bh + (sl < bl ? 1u : 0u);
  const unsigned rl = sl & 0xe0000000u;
  // the rounded double as float bits: exponent - 896 and the 23 fraction bits
  // (a carry into the exponent past the float range gives Inf)
  const float hi = __uint_as_float((__funnelshift_l(rl, rh, 3) - (0x180u << 23)) | sign);
  // x - hi = sign * delta units of x's last place, 2^(ex - 1075) = 2^-52 * 2^(ex - 1023)
  const int delta = int(bl - rl);
  const float sc = __uint_as_float(((ex - 896u) << 23) | sign);
  const float lo = __fmul_rn(__fmul_rn(__int2float_rn(delta), 0x1p-52f), sc);
  return dw_make(hi, lo);
}

// float -> FP64 bits on the integer pipe: normal numbers exactly, subnormals
// flushed to a signed zero, Inf and NaN kept
__device__ __forceinline__ double f64_of(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = u & 0x7f800000u, s = u & 0x80000000u;
  unsigned hi = s | (((u & 0x7fffffffu) >> 3) + 0x38000000u);
  hi = e == 0x7f800000u ? (s | 0x7ff00000u | ((u >> 3) & 0x000fffffu)) : hi;
  hi = e == 0u ? s : hi;
  return __hiloint2double(int(hi), e == 0u ? 0 : int(u << 29));
}

// DW -> FP64: both parts exactly, added in one FP64 add
__device__ __forceinline__ double dw_to_f64(dw x) { return __dadd_rn(f64_of(x.hi), f64_of(x.lo)); }

// old + x for an FP64 value old and a DW increment x: the increment rounded to
// FP64 and added to old, so old keeps its 53 bits (two FP64 adds)
__device__ __forceinline__ double f64_plus_dw(double old, dw x) { return __dadd_rn(old, dw_to_f64(x)); }

// the grid update's DW record of node i (NodeP::dw4, 3D): vdt and dv, or
// zeros when vdt == dv == nullptr
__device__ __forceinline__ void put_node_dw(float4* r, int64_t i, const double* vdt, const double* dv) {
  if (!vdt) {
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    r[3 * i] = z;
    r[3 * i + 1] = z;
    r[3 * i + 2] = z;
    return;
  }
  const dw v0 = dw_from(vdt[0]), v1 = dw_from(vdt[1]), v2 = dw_from(vdt[2]);
  const dw d0 = dw_from(dv[0]), d1 = dw_from(dv[1]), d2 = dw_from(dv[2]);
  r[3 * i] = make_float4(v0.hi, v0.lo, v1.hi, v1.lo);
  r[3 * i + 1] = make_float4(v2.hi, v2.lo, d0.hi, d0.lo);
  r[3 * i + 2] = make_float4(d1.hi, d1.lo, d2.hi, d2.lo);
}

// a host-split FP64 constant (hi = float(d), lo = float(d - hi))
__device__ __forceinline__ dw dw_c(const float (&c)[2]) { return dw_make(c[0], c[1]); }

}  // namespace jmpm

// Double-float arithmetic for complex128 gates on GB300.
//
// GB300 issues FP64 at about 1/64 of its FP32 rate, so a complex128 gate
// that does its arithmetic in FP64 is bound by the FP64 pipe, not by HBM.
// The gate kernels instead carry each amplitude component as an unevaluated
// pair of floats (hi + lo) and each matrix entry as an exact triple
// (hi + mid + lo), and compute with FP32 / INT32 instructions only:
//
//   * df_split: a double -> pair by integer bit operations: hi is the double
//     rounded to 24 significant bits, lo the signed remainder rounded to
//     24 bits, so |x - hi - lo| <= 2^-48 |x|;
//   * df_entry: a double -> exact triple (24 + 24 + 5 bits), each part
//     rounded to nearest;
//   * products through fma (Dekker): m * a = p + e with p = RN(m.hi * a.hi),
//     its exact rounding error, and the cross terms m.hi * a.lo and
//     m.mid * a.hi accumulated into e.  The terms of order 2^-48 (m.mid *
//     a.lo, m.lo * a.hi) are left out, as are the roundings of e: every
//     leading word is rounded to nearest, so the low words carry either
//     sign and what is left out has no bias (a truncating split would
//     shrink every product by about 2^-48.6 and drift the norm);
//   * sums of products use Knuth's TwoSum on the leading parts and add the
//     error terms, then one fast renormalisation (Dekker's Fast2Sum);
//   * df_join: pair -> double by integer operations on the bit pattern of
//     hi, adding lo as a rounded integer number of double ulps of hi.
//
// The relative error of one gate is a few units of 2^-47, unbiased; the
// complex128 engine keeps native FP64 arithmetic as an option
// (gbsv_set_c128_arith).  The float range bounds the operands: a thread
// whose largest amplitude component lies outside [2^-40, 2^60] (and is not
// zero), or an operator whose largest entry does, runs native FP64.
// Inside that range, components below 2^-80 keep no low word and those
// below 2^-126 become zero (absolute errors below 2^-103 and 2^-126), and
// entries below 2^-74 become zero.
//
// All float additions and products go through the _rn intrinsics so the
// compiler cannot contract them into fma, which would break TwoSum.  The
// same code compiles for the host with -ffp-contract=off (the host test
// checks it against exact rational arithmetic).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define GBSV_HD __host__ __device__ __forceinline__
#else
#define GBSV_HD inline
#endif
#ifndef __CUDA_ARCH__
#include <math.h>
#include <string.h>
#endif

namespace gbsv {

struct DF {  // hi + lo
  float hi, lo;
};
struct DE {  // hi + mid + lo, exactly a double
  float hi, mid, lo;
};

GBSV_HD float df_add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
GBSV_HD float df_sub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
GBSV_HD float df_mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
GBSV_HD float df_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}
GBSV_HD uint32_t df_fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  memcpy(&b, &x, 4);
  return b;
#endif
}
GBSV_HD float df_float(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, 4);
  return x;
#endif
}
GBSV_HD uint32_t df_hiword(double x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2hiint(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return (uint32_t)(b >> 32);
#endif
}
GBSV_HD uint32_t df_loword(double x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2loint(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return (uint32_t)b;
#endif
}
GBSV_HD double df_make(uint32_t hw, uint32_t lw) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hw, (int)lw);
#else
  const uint64_t b = ((uint64_t)hw << 32) | lw;
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
// integer <-> float conversions, rounding to nearest (the XU pipe on the
// device, off the ALU pipe that carries the bit operations)
GBSV_HD float df_i2f(int32_t x) {
#ifdef __CUDA_ARCH__
  return __int2float_rn(x);
#else
  return (float)x;
#endif
}
GBSV_HD int32_t df_f2i(float x) {
#ifdef __CUDA_ARCH__
  return __float2int_rn(x);
#else
  return (int32_t)nearbyintf(x);
#endif
}
// bits [29, 61) of the 64-bit word hw:lw
GBSV_HD uint32_t df_shr29(uint32_t hw, uint32_t lw) {
#ifdef __CUDA_ARCH__
  return __funnelshift_r(lw, hw, 29);
#else
  return (lw >> 29) | (hw << 3);
#endif
}

// Exponent field (biased, 11 bits) of the double whose high word is hw.
GBSV_HD uint32_t df_expo(uint32_t hw) { return (hw >> 20) & 0x7ffu; }

// The range test: the largest exponent field among a thread's amplitude
// components (and, separately, among the operator's entries) lies in
// [DF_EMIN, DF_EMAX], or every component is zero.
constexpr uint32_t DF_EMIN = 1023 - 40, DF_EMAX = 1023 + 60;

GBSV_HD DF df_split(double x) {
  const uint32_t hw = df_hiword(x), lw = df_loword(x);
  const uint32_t sign = hw & 0x80000000u;
  const uint32_t eb = hw & 0x7ff00000u;  // exponent field, in place
  // hi: the double rounded to 24 significant bits (adding half of bit 29
  // to the bit pattern; a carry moves into the exponent), then the
  // exponent rebias 1023 -> 127 on the 9 low exponent bits (the result
  // lies in [1, 254] for e in [897, 1150], so it fits 8 bits)
  const uint64_t rb = (((uint64_t)hw << 32) | lw) + (1u << 28);
  const uint32_t hb =
      (df_shr29((uint32_t)(rb >> 32), (uint32_t)rb) + 0x40000000u) | sign;
  // lo = x - hi: the 29 bits below hi as a signed count (bit 28 set means
  // hi was rounded up), times 2^(e - 1075) with the original exponent e,
  // whose float exponent field e - 948 comes from the 9 low exponent bits
  // (mod 512) for e in [949, 1083]
  const int32_t rest = (int32_t)(lw << 3) >> 3;
  const uint32_t sb = (((hw << 3) - (436u << 23)) & 0x7f800000u) | sign;
  const float lo = df_mul_rn(df_i2f(rest), df_float(sb));
  DF d;
  d.hi = eb >= (897u << 20) ? df_float(hb) : 0.f;  // |x| >= 2^-126
  d.lo = eb >= (949u << 20) ? lo : 0.f;            // scale a normal float
  return d;
}

// Exact triple of a double with |x| in [2^-74, 2^127) (or zero; smaller
// values become zero): hi = x rounded to a float, mid = the remainder
// rounded, lo = what is left (at most 5 significant bits).  Each
// subtraction is exact, and both low words carry either sign.
GBSV_HD DE df_entry(double x) {
  DE d{0.f, 0.f, 0.f};
  if ((df_hiword(x) & 0x7ff00000u) < (949u << 20)) return d;
  d.hi = (float)x;
  const double r1 = x - (double)d.hi;
  d.mid = (float)r1;
  d.lo = (float)(r1 - (double)d.mid);
  return d;
}

// m * a = p + e to about 2^-48 relative, with the pair a and the triple m
struct DFP {
  float p, e;
};
GBSV_HD DFP df_prod(const DE& m, const DF& a) {
  DFP r;
  r.p = df_mul_rn(m.hi, a.hi);
  float e = df_fma(m.hi, a.hi, -r.p);
  e = df_fma(m.hi, a.lo, e);
  e = df_fma(m.mid, a.hi, e);
  r.e = e;
  return r;
}
GBSV_HD DFP df_neg(DFP x) {
  x.p = -x.p;
  x.e = -x.e;
  return x;
}
GBSV_HD DF df_neg(DF x) {
  x.hi = -x.hi;
  x.lo = -x.lo;
  return x;
}

// Fast2Sum: hi + lo == a + b when |a| >= |b| or a == 0
GBSV_HD DF df_fast2(float a, float b) {
  DF r;
  r.hi = df_add_rn(a, b);
  r.lo = df_sub_rn(b, df_sub_rn(r.hi, a));
  return r;
}
// TwoSum: s + err == a + b exactly
GBSV_HD float df_two_sum(float a, float b, float& err) {
  const float s = df_add_rn(a, b);
  const float bb = df_sub_rn(s, a);
  err = df_add_rn(df_sub_rn(a, df_sub_rn(s, bb)), df_sub_rn(b, bb));
  return s;
}

// Sums of products.  N = true renormalises the result (|lo| <= ulp(hi)/2,
// what df_join needs); N = false leaves lo at a few ulps of hi, which the
// products of the next gate take as they are (fused stages renormalise
// once, before the join).
template <bool N>
GBSV_HD DF df_fin(float s, float el) {
  if constexpr (N) return df_fast2(s, el);
  DF r;
  r.hi = s;
  r.lo = el;
  return r;
}
template <bool N = true>
GBSV_HD DF df_one(DFP x) { return df_fin<N>(x.p, x.e); }
template <bool N = true>
GBSV_HD DF df_sum2(DFP x, DFP y) {
  float es;
  const float s = df_two_sum(x.p, y.p, es);
  return df_fin<N>(s, df_add_rn(es, df_add_rn(x.e, y.e)));
}
template <bool N = true>
GBSV_HD DF df_sum4(DFP x, DFP y, DFP z, DFP w) {
  float e1, e2, e3;
  const float s1 = df_two_sum(x.p, y.p, e1);
  const float s2 = df_two_sum(z.p, w.p, e2);
  const float s = df_two_sum(s1, s2, e3);
  const float el = df_add_rn(df_add_rn(df_add_rn(x.e, y.e),
                                       df_add_rn(z.e, w.e)),
                             df_add_rn(df_add_rn(e1, e2), e3));
  return df_fin<N>(s, el);
}
template <bool N = true>
GBSV_HD DF df_sum8(const DFP* x) {
  float e[7];
  const float s0 = df_two_sum(x[0].p, x[1].p, e[0]);
  const float s1 = df_two_sum(x[2].p, x[3].p, e[1]);
  const float s2 = df_two_sum(x[4].p, x[5].p, e[2]);
  const float s3 = df_two_sum(x[6].p, x[7].p, e[3]);
  const float t0 = df_two_sum(s0, s1, e[4]);
  const float t1 = df_two_sum(s2, s3, e[5]);
  const float s = df_two_sum(t0, t1, e[6]);
  float el = df_add_rn(df_add_rn(x[0].e, x[1].e), df_add_rn(x[2].e, x[3].e));
  el = df_add_rn(el, df_add_rn(df_add_rn(x[4].e, x[5].e),
                               df_add_rn(x[6].e, x[7].e)));
  el = df_add_rn(el, df_add_rn(df_add_rn(e[0], e[1]), df_add_rn(e[2], e[3])));
  el = df_add_rn(el, df_add_rn(df_add_rn(e[4], e[5]), e[6]));
  return df_fin<N>(s, el);
}
// an unnormalised pair made exact and normalised (TwoSum)
GBSV_HD DF df_norm(DF x) {
  DF r;
  r.hi = df_two_sum(x.hi, x.lo, r.lo);
  return r;
}
// Exact sum of two pairs, renormalised
GBSV_HD DF df_add(DF x, DF y) {
  float es;
  const float s = df_two_sum(x.hi, y.hi, es);
  return df_fast2(s, df_add_rn(es, df_add_rn(x.lo, y.lo)));
}

// hi + lo rounded to a double, for a normalised pair (|lo| <= ulp(hi),
// any output of df_fast2, df_sum*, df_split).  lo is added to the bit
// pattern of hi as a count of double ulps of hi: lo * 2^(179 - e_hi),
// signed relative to hi's magnitude (2^(180 - e_hi) when lo lowers a
// power of two, whose lower neighbours are half an ulp apart), rounded to
// an integer by the conversion unit.  Below |hi| = 2^-75 lo is dropped
// (an absolute error below 2^-99).
GBSV_HD double df_join(DF x) {
  const uint32_t hb = df_fbits(x.hi);
  const uint32_t sign = hb & 0x80000000u;
  const uint32_t ehb = hb & 0x7f800000u;
  float v = df_mul_rn(x.lo, df_float((0x99000000u - ehb) ^ sign));
  if ((hb & 0x7fffffu) == 0 && v < 0.f) v = df_add_rn(v, v);
  const int32_t la = ehb >= (52u << 23) ? df_f2i(v) : 0;
  // hi as a double: exponent 127 -> 1023, 23 mantissa bits at the top
  const uint32_t dh = (((hb >> 3) & 0x0fffffffu) + (896u << 20)) | sign;
  const uint32_t dl = hb << 29;
  const uint64_t b =
      (((uint64_t)dh << 32) | dl) + (uint64_t)(int64_t)la;
  return ehb == 0 ? df_make(sign, 0u)
                  : df_make((uint32_t)(b >> 32), (uint32_t)b);
}

// ----------------------------------------------------- complex forms ----
// The gate kernels' arithmetic on one amplitude pair, shared with the host
// test.  Amplitudes are pairs per component, entries exact triples.
struct DC {
  DF re, im;
};
struct DEC {
  DE re, im;
};

GBSV_HD DC df_split2(double re, double im) {
  DC a;
  a.re = df_split(re);
  a.im = df_split(im);
  return a;
}
GBSV_HD DEC df_entry2(double re, double im) {
  DEC m;
  m.re = df_entry(re);
  m.im = df_entry(im);
  return m;
}

// m0 a0 + m1 a1, complex entries
template <bool N = true>
GBSV_HD DC df_row2(const DEC& m0, const DC& a0, const DEC& m1,
                   const DC& a1) {
  DC y;
  y.re = df_sum4<N>(df_prod(m0.re, a0.re), df_neg(df_prod(m0.im, a0.im)),
                 df_prod(m1.re, a1.re), df_neg(df_prod(m1.im, a1.im)));
  y.im = df_sum4<N>(df_prod(m0.re, a0.im), df_prod(m0.im, a0.re),
                 df_prod(m1.re, a1.im), df_prod(m1.im, a1.re));
  return y;
}
// m0 a0 + m1 a1, real entries
template <bool N = true>
GBSV_HD DC df_row2_real(const DE& m0, const DC& a0, const DE& m1,
                        const DC& a1) {
  DC y;
  y.re = df_sum2<N>(df_prod(m0, a0.re), df_prod(m1, a1.re));
  y.im = df_sum2<N>(df_prod(m0, a0.im), df_prod(m1, a1.im));
  return y;
}
// r a0 + (i s) a1, real r and s (the rows of RX-like matrices)
template <bool N = true>
GBSV_HD DC df_row2_rx(const DE& r, const DC& a0, const DE& s, const DC& a1) {
  DC y;
  y.re = df_sum2<N>(df_prod(r, a0.re), df_neg(df_prod(s, a1.im)));
  y.im = df_sum2<N>(df_prod(r, a0.im), df_prod(s, a1.re));
  return y;
}
// m a, complex m
template <bool N = true>
GBSV_HD DC df_cmul(const DEC& m, const DC& a) {
  DC y;
  y.re = df_sum2<N>(df_prod(m.re, a.re), df_neg(df_prod(m.im, a.im)));
  y.im = df_sum2<N>(df_prod(m.re, a.im), df_prod(m.im, a.re));
  return y;
}
// r a, real r
template <bool N = true>
GBSV_HD DC df_rmul(const DE& r, const DC& a) {
  DC y;
  y.re = df_one<N>(df_prod(r, a.re));
  y.im = df_one<N>(df_prod(r, a.im));
  return y;
}
// (i s) a, real s
template <bool N = true>
GBSV_HD DC df_imul(const DE& s, const DC& a) {
  DC y;
  y.re = df_neg(df_one<N>(df_prod(s, a.im)));
  y.im = df_one<N>(df_prod(s, a.re));
  return y;
}

// sum_j m_j a_j over four complex entries (one row of a 4x4)
template <bool N = true>
GBSV_HD DC df_row4(const DEC* m, const DC* a) {
  DFP pr[8], pi[8];
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int j = 0; j < 4; ++j) {
    pr[2 * j] = df_prod(m[j].re, a[j].re);
    pr[2 * j + 1] = df_neg(df_prod(m[j].im, a[j].im));
    pi[2 * j] = df_prod(m[j].re, a[j].im);
    pi[2 * j + 1] = df_prod(m[j].im, a[j].re);
  }
  DC y;
  y.re = df_sum8<N>(pr);
  y.im = df_sum8<N>(pi);
  return y;
}

// sum_b m_b x_b over D complex terms (one row of a D x D operator): a
// compensated dot product (the leading parts summed with TwoSum, their
// errors and the products' error words summed beside them, as in Ogita,
// Rump and Oishi's Dot2), renormalised once at the end.
template <int D>
GBSV_HD DC df_rowD(const DEC* m, const DC* x) {
  float sr = 0.f, er = 0.f, si = 0.f, ei = 0.f;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int b = 0; b < D; ++b) {
    const DFP rr = df_prod(m[b].re, x[b].re);
    const DFP ii = df_neg(df_prod(m[b].im, x[b].im));
    const DFP ri = df_prod(m[b].re, x[b].im);
    const DFP ir = df_prod(m[b].im, x[b].re);
    float t;
    sr = df_two_sum(sr, rr.p, t);
    er = df_add_rn(er, df_add_rn(t, rr.e));
    sr = df_two_sum(sr, ii.p, t);
    er = df_add_rn(er, df_add_rn(t, ii.e));
    si = df_two_sum(si, ri.p, t);
    ei = df_add_rn(ei, df_add_rn(t, ri.e));
    si = df_two_sum(si, ir.p, t);
    ei = df_add_rn(ei, df_add_rn(t, ir.e));
  }
  DC y;
  y.re = df_norm(DF{sr, er});
  y.im = df_norm(DF{si, ei});
  return y;
}

// ---- sine and cosine in pairs --------------------------------------------
// sin and cos of a double angle with |theta| <= 2^20, as pairs, written
// from the mathematics: Cody and Waite's reduction theta = k pi/2 + r with
// pi/2 held as three floats C1 + C2 + C3 (72 bits; each k Ci taken exactly
// by fma, theta.hi - k C1 exact by Sterbenz's lemma for k != 0, the other
// parts summed with TwoSum and their errors kept beside), then the Taylor
// series of sin and cos on |r| <= pi/4 (plus a rounding margin): the
// coefficients 1/n! whose terms exceed about 2^-25 of the result as pairs,
// the remaining tail in FP32.  The constants are the floats nearest to
// pi/2's parts, 2/pi and the pair splits of (-1)^j / n!, computed from
// exact rationals.
struct DSC {
  DF s, c;
};

GBSV_HD float df_rint(float x) {
#ifdef __CUDA_ARCH__
  return rintf(x);
#else
  return nearbyintf(x);
#endif
}

// a * b for two pairs: the leading product exactly, the cross terms into
// the error word
GBSV_HD DFP df_prod2(DF a, DF b) {
  DFP r;
  r.p = df_mul_rn(a.hi, b.hi);
  float e = df_fma(a.hi, b.hi, -r.p);
  e = df_fma(a.hi, b.lo, e);
  e = df_fma(a.lo, b.hi, e);
  r.e = e;
  return r;
}
// a * b + c, renormalised
GBSV_HD DF df_mad2(DF a, DF b, DF c) {
  const DFP p = df_prod2(a, b);
  float es;
  const float s = df_two_sum(p.p, c.hi, es);
  return df_fast2(s, df_add_rn(es, df_add_rn(p.e, c.lo)));
}

GBSV_HD DSC df_sincos(double theta) {
  constexpr float PIO2_1 = 0x1.921fb6p+0f, PIO2_2 = -0x1.777a5cp-25f,
                  PIO2_3 = -0x1.ee59dap-50f, TWO_OVER_PI = 0x1.45f306p-1f;
  // sin r = r + r z S(z), z = r^2: S0..S3 as pairs, S4..S7 in FP32
  const DF S0{-0x1.555556p-3f, 0x1.555556p-28f};
  const DF S1{0x1.111112p-7f, -0x1.dddddep-32f};
  const DF S2{-0x1.a01a02p-13f, 0x1.7f97fap-39f};
  const DF S3{0x1.71de3ap-19f, 0x1.55b1ccp-45f};
  constexpr float S4 = -0x1.ae6456p-26f, S5 = 0x1.612462p-33f,
                  S6 = -0x1.ae7f3ep-41f, S7 = 0x1.952c78p-49f;
  // cos r = 1 + z C(z): C0..C4 as pairs, C5..C8 in FP32
  const DF C0{-0.5f, 0.f};
  const DF C1{0x1.555556p-5f, -0x1.555556p-30f};
  const DF C2{-0x1.6c16c2p-10f, 0x1.27d27ep-35f};
  const DF C3{0x1.a01a02p-16f, -0x1.7f97fap-42f};
  const DF C4{-0x1.27e4fcp-22f, 0x1.10ec14p-47f};
  constexpr float C5 = 0x1.1eed8ep-29f, C6 = -0x1.93974ap-37f,
                  C7 = 0x1.ae7f3ep-45f, C8 = -0x1.682786p-53f;

  const DE t = df_entry(theta);
  const float kf = df_rint(df_mul_rn(t.hi, TWO_OVER_PI));
  const float p1 = df_mul_rn(kf, PIO2_1), e1 = df_fma(kf, PIO2_1, -p1);
  const float p2 = df_mul_rn(kf, PIO2_2), e2 = df_fma(kf, PIO2_2, -p2);
  const float p3 = df_mul_rn(kf, PIO2_3);
  float s = df_sub_rn(t.hi, p1);
  float q, err;
  s = df_two_sum(s, -e1, err);
  s = df_two_sum(s, t.mid, q);
  err = df_add_rn(err, q);
  s = df_two_sum(s, -p2, q);
  err = df_add_rn(err, q);
  err = df_add_rn(err, df_sub_rn(df_sub_rn(t.lo, e2), p3));
  const DF r = df_fast2(s, err);
  const DFP zp = df_prod2(r, r);
  const DF z = df_fast2(zp.p, zp.e);

  float ts = df_fma(z.hi, S7, S6);
  ts = df_fma(z.hi, ts, S5);
  ts = df_fma(z.hi, ts, S4);
  DF as = df_mad2(z, DF{ts, 0.f}, S3);
  as = df_mad2(z, as, S2);
  as = df_mad2(z, as, S1);
  as = df_mad2(z, as, S0);
  const DFP wp = df_prod2(z, as);
  const DF sr = df_mad2(r, df_fast2(wp.p, wp.e), r);

  float tc = df_fma(z.hi, C8, C7);
  tc = df_fma(z.hi, tc, C6);
  tc = df_fma(z.hi, tc, C5);
  DF ac = df_mad2(z, DF{tc, 0.f}, C4);
  ac = df_mad2(z, ac, C3);
  ac = df_mad2(z, ac, C2);
  ac = df_mad2(z, ac, C1);
  ac = df_mad2(z, ac, C0);
  const DF cr = df_mad2(z, ac, DF{1.f, 0.f});

  // quadrant k mod 4
  const int quad = ((int)kf) & 3;
  DSC o;
  o.s = (quad & 1) ? cr : sr;
  o.c = (quad & 1) ? sr : cr;
  if (quad == 2 || quad == 3) o.s = df_neg(o.s);
  if (quad == 1 || quad == 2) o.c = df_neg(o.c);
  return o;
}

}  // namespace gbsv

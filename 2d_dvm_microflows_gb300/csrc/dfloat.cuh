// dfloat.cuh -- FP64-accurate arithmetic on the FP32 pipe.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so the streaming kernels keep their values in
// FP64 memory but do their arithmetic on unevaluated sums of two floats (hi + lo), with the
// error-free transformations of Knuth (TwoSum), Dekker (Fast2Sum) and the FMA product
// error (TwoProd). A double enters by an integer split of its bit pattern (no FP64
// instruction) into hi = its leading 24 significant bits and lo = the next 24 bits, rounded
// (relative error at most 2^-47, about 7e-15); values below 2^-126 enter as zero (their
// absolute size, under 1.2e-38, is far below the FP64 rounding of any cell total). A result
// leaves as hi + lo converted bit-exactly to doubles and added with one FP64 add.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dvm {

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl dfl_make(float h, float l) {
  dfl r;
  r.hi = h;
  r.lo = l;
  return r;
}

// Split of a double into hi + lo by integer operations on its bits.
__device__ __forceinline__ dfl dfl_from_double(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const uint32_t bh = static_cast<uint32_t>(b >> 32), bl = static_cast<uint32_t>(b);
  const uint32_t sign = bh & 0x80000000u;
  const int e = static_cast<int>((bh >> 20) & 0x7ffu);  // biased FP64 exponent
  const int ef = e - 896;                                // biased FP32 exponent of hi
  // mantissa bits 51..29 -> hi, bits 28..5 -> lo (23 bits plus the rounding bit 5)
  const uint32_t mhi = ((bh & 0xfffffu) << 3) | (bl >> 29);
  const uint32_t mlo = ((bl >> 6) & 0x7fffffu) + ((bl >> 5) & 1u);
  dfl r;
  if (ef <= 0) {             // |x| < 2^-126 (zero, FP64 subnormals, tiny values)
    r.hi = 0.f;
    r.lo = 0.f;
    return r;
  }
  if (ef >= 255) {           // |x| >= 2^128 or inf / NaN: FP32 inf / NaN (bit operations
                             // only, so that no FP64 conversion is issued on the hot path)
    const bool nan = (e == 2047) && (((bh & 0xfffffu) | bl) != 0u);
    r.hi = __int_as_float(static_cast<int>(sign | 0x7f800000u | (nan ? 0x400000u : 0u)));
    r.lo = 0.f;
    return r;
  }
  r.hi = __int_as_float(static_cast<int>(sign | (static_cast<uint32_t>(ef) << 23) | mhi));
  const int el = ef - 23;    // exponent of the lo magic number
  if (el <= 0) {
    r.lo = 0.f;
  } else {
    // (1 + mlo 2^-23) 2^(E-23) - 2^(E-23) = mlo 2^(E-46), exact; a carry of the rounding
    // into the exponent field gives 2^(E-22) - 2^(E-23) = 2^23 2^(E-46), also exact
    const float magic = __int_as_float(static_cast<int>((static_cast<uint32_t>(el) << 23) + mlo));
    const float base = __int_as_float(static_cast<int>(static_cast<uint32_t>(el) << 23));
    const float l = __fsub_rn(magic, base);
    r.lo = sign ? -l : l;
  }
  return r;
}

// Exact float -> double by integer operations (no FP64 conversion is issued): normal
// floats by rebiasing the exponent, FP32 subnormals (the lo part of values below about
// 2^-102) by normalising their mantissa, and inf / NaN carried over.
__device__ __forceinline__ double dbl_from_float(float v) {
  const uint32_t u = static_cast<uint32_t>(__float_as_int(v));
  const uint32_t ex = (u >> 23) & 0xffu;
  const uint32_t m = u & 0x7fffffu;
  const uint32_t sign = u & 0x80000000u;
  uint32_t hi, lo;
  if (ex == 0u) {
    if (m == 0u) return __hiloint2double(static_cast<int>(sign), 0);
    const int p = 31 - __clz(static_cast<int>(m));            // top bit, 0..22
    const unsigned long long mm =
        (static_cast<unsigned long long>(m) << (52 - p)) & ((1ull << 52) - 1);
    hi = sign | (static_cast<uint32_t>(p + 874) << 20) | static_cast<uint32_t>(mm >> 32);
    lo = static_cast<uint32_t>(mm);
  } else {
    hi = sign | ((ex == 255u ? 2047u : ex + 896u) << 20) | (m >> 3) |
         ((ex == 255u && m != 0u) ? 0x80000u : 0u);  // NaN stays NaN
    lo = m << 29;
  }
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

__device__ __forceinline__ double dfl_to_double(dfl a) {
  return dbl_from_float(a.hi) + dbl_from_float(a.lo);
}

// Exact float -> double for a normal float or zero (no subnormal, inf or NaN handling):
// the short form for values known to lie well inside the float range.
__device__ __forceinline__ double dbl_from_normal_float(float v) {
  const uint32_t u = static_cast<uint32_t>(__float_as_int(v));
  const uint32_t hi = (u & 0x80000000u) | (((u >> 23) & 0xffu) + 896u) << 20 | ((u & 0x7fffffu) >> 3);
  const uint32_t lo = u << 29;
  return (u & 0x7fffffffu) ? __hiloint2double(static_cast<int>(hi), static_cast<int>(lo)) : 0.0;
}

// Pair -> double for pairs of normal floats (hi in the normal range, lo normal or zero).
__device__ __forceinline__ double dfl_to_double_normal(dfl a) {
  return dbl_from_normal_float(a.hi) + dbl_from_normal_float(a.lo);
}

// float -> double for any float: inf and NaN carry over exactly, a subnormal (below
// 1.2e-38) may come out off by up to its own size; the short form for values added into
// FP64 state, where that is far below the FP64 rounding of the state.
__device__ __forceinline__ double dbl_from_float_fast(float v) {
  const uint32_t u = static_cast<uint32_t>(__float_as_int(v));
  if ((u & 0x7f800000u) == 0x7f800000u) return dbl_from_float(v);
  return dbl_from_normal_float(v);
}

// Pair -> double for a hi of any finite, infinite or NaN value with a lo below it: inf and
// NaN carry over through hi, and an FP32-subnormal part (below 1.2e-38) may come out off
// by up to its own size, far below the FP64 rounding of any value the kernels keep.
__device__ __forceinline__ double dfl_to_double_fast(dfl a) {
  const uint32_t u = static_cast<uint32_t>(__float_as_int(a.hi));
  if ((u & 0x7f800000u) == 0x7f800000u) return dbl_from_float(a.hi);
  return dbl_from_normal_float(a.hi) + dbl_from_normal_float(a.lo);
}

// Knuth's TwoSum: s + e = a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Dekker's Fast2Sum (|a| >= |b| or a == 0): s + e = a + b exactly.
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dfl dfl_norm(float h, float l) {
  dfl r;
  fast_two_sum(h, l, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ dfl dfl_add(dfl a, dfl b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return dfl_norm(s, e);
}

__device__ __forceinline__ dfl dfl_neg(dfl a) { return dfl_make(-a.hi, -a.lo); }

__device__ __forceinline__ dfl dfl_sub(dfl a, dfl b) { return dfl_add(a, dfl_neg(b)); }

__device__ __forceinline__ dfl dfl_abs(dfl a) {
  return (a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f)) ? dfl_neg(a) : a;
}

// FP32 reciprocal and reciprocal square root estimates (MUFU, about 1 ulp); the callers
// correct them with an exactly formed remainder.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Product with the FMA error term (the lo*lo term, below 2^-48 relative, is dropped).
__device__ __forceinline__ dfl dfl_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dfl_norm(p, e);
}

// a * b as a double: the product's hi and its error term go to FP64 unnormalised, since the
// FP64 add rounds their exact sum, which renormalising (an error-free transformation) would
// not change. The hi goes through the hardware's float-to-double conversion (exact, on the
// FP64 pipe) and the error term through the integer one: the collide kernel, which alone
// uses this, balances its issue slots and its FP64 pipe best that way (measured against
// both conversions of either kind).
__device__ __forceinline__ double dfl_mul_to_double(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return static_cast<double>(p) + dbl_from_normal_float(e);
}

__device__ __forceinline__ dfl dfl_scale(dfl a, float s) {  // s a power of two
  return dfl_make(a.hi * s, a.lo * s);
}

// Division with one correction step (Karp-Markstein style): q1 = a/b in FP32, the
// remainder a - q1 b formed exactly by FMA, divided again (about 2^-45 relative).
__device__ __forceinline__ dfl dfl_div(dfl a, dfl b) {
  const float rb = rcp_approx(b.hi);
  const float q1 = __fmul_rn(a.hi, rb);
  const float p = __fmul_rn(q1, b.hi);
  const float e = __fmaf_rn(q1, b.hi, -p);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), __fmaf_rn(q1, b.lo, e)), a.lo);
  const float q2 = __fmul_rn(r, rb);
  return dfl_norm(q1, q2);
}

// Square root from the reciprocal square root estimate y: s = a y, then s + (a - s^2) y / 2.
__device__ __forceinline__ dfl dfl_sqrt(dfl a) {
  if (!(a.hi > 0.f)) return dfl_make(0.f, 0.f);
  const float y = rsqrt_approx(a.hi);
  const float s = __fmul_rn(a.hi, y);
  const float p = __fmul_rn(s, s);
  const float e = __fmaf_rn(s, s, -p);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), a.lo);
  return dfl_norm(s, __fmul_rn(r, 0.5f * y));
}

// ---- x^q for a positive pair: x^q = 2^(q log2 x) ------------------------------------------
// The relative speed's g^(2 - 2 omega) on grids without a speed table: an FP64 pow per
// sample costs the collide kernel as much as the rest of its work together, the FP64 pipe
// issuing at 1/64 of the FP32 rate. Methods (from the mathematics, not from any library):
//   log2 x = e + log2 m: x = 2^e m with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh s,
//     s = (m - 1)/(m + 1), |s| <= 0.1716, t = s^2 <= 0.0295, ln m = 2 s (1 + t/3 + t^2/5 +
//     ... + t^9/19); the terms from t^4 on (below 7e-8 of the sum) in FP32, the others in
//     pairs.
//   q log2 x = q e + q log2 m: q is held as three floats (all 53 bits of the double), so
//     q e is formed exactly by error-free products and only its fraction and q log2 m
//     (each below 1 in size) go through pair arithmetic.
//   2^y: y = n + j/32 + u with integer n, j in [-16, 16] and |u| <= 1/64; 2^y =
//     2^n 2^(j/32) e^v, v = u ln 2, |v| <= 0.0109, 2^(j/32) from a 33-entry pair table and
//     e^v by its Taylor series to v^6 (v^4 on in FP32) -- the table-driven reduction of
//     P. T. P. Tang, ACM Trans. Math. Softw. 15 (1989) 144-157.
// Each pair step rounds at about 2^-48 of a value below 1 in size: the result is within
// about 1e-14 relative whatever the size of q log2 x.
constexpr int kExp2TabN = 33;  // 2^(j/32), j = -16 .. 16

// Entry t of the table (2^((t - 16)/32) as a normalised pair) from the FP64 exp2.
__device__ __forceinline__ float2 exp2_table_entry(int t) {
  const dfl v = dfl_from_double(exp2(static_cast<double>(t - 16) * 0.03125));
  const dfl n = dfl_norm(v.hi, v.lo);
  return make_float2(n.hi, n.lo);
}

// A double as three floats whose sum is the double (exactly, for normal results).
struct flt3 {
  float hi, mid, lo;
};

__device__ __forceinline__ flt3 flt3_from_double(double q) {
  flt3 r;
  r.hi = __double2float_rn(q);
  const double r1 = q - static_cast<double>(r.hi);
  r.mid = __double2float_rn(r1);
  r.lo = __double2float_rn(r1 - static_cast<double>(r.mid));
  return r;
}

__device__ __forceinline__ float pow2f_exact(int a) {  // 2^a, -126 <= a <= 127
  return __int_as_float((a + 127) << 23);
}

// log2 m of a pair x with a positive normal hi, x = 2^e m, m in [sqrt(1/2), sqrt(2)).
__device__ __forceinline__ dfl dfl_log2_split(dfl x, int& e) {
  const int bits = __float_as_int(x.hi);
  e = ((bits >> 23) & 0xff) - 127;
  const float mh = __int_as_float((bits & 0x007fffff) | 0x3f800000);  // in [1, 2)
  if (mh > 1.41421354f) e += 1;                                       // m < sqrt(2)
  const float sc = pow2f_exact(-e);
  const dfl m = dfl_make(x.hi * sc, x.lo * sc);                       // exact
  const dfl one = dfl_make(1.f, 0.f);
  const dfl num = dfl_sub(m, one), den = dfl_add(m, one);
  dfl s = dfl_div(num, den);
  // one more correction of the quotient: s + (num - s den)/den (dfl_div alone holds about
  // 2^-45 of s, the leading term of ln m)
  s = dfl_add(s, dfl_make(__fmul_rn(dfl_sub(num, dfl_mul(s, den)).hi, rcp_approx(den.hi)), 0.f));
  const dfl t = dfl_mul(s, s);
  const float th = t.hi;
  // 1/9 + t/11 + ... + t^5/19 in FP32
  const float r4 = fmaf(th, fmaf(th, fmaf(th, fmaf(th, fmaf(th, 1.f / 19.f, 1.f / 17.f),
                                                   1.f / 15.f), 1.f / 13.f), 1.f / 11.f),
                        1.f / 9.f);
  const dfl c3 = dfl_make(0x1.555556p-2f, -0x1.555556p-27f);
  const dfl c5 = dfl_make(0x1.99999ap-3f, -0x1.99999ap-29f);
  const dfl c7 = dfl_make(0x1.24924ap-3f, -0x1.b6db6ep-28f);
  const dfl inv_ln2 = dfl_make(0x1.715476p+0f, 0x1.4ae0c0p-26f);
  const dfl A = dfl_add(c7, dfl_mul(t, dfl_make(r4, 0.f)));
  const dfl B = dfl_add(c5, dfl_mul(t, A));
  const dfl P = dfl_add(c3, dfl_mul(t, B));
  const dfl s2 = dfl_scale(s, 2.f);
  const dfl lnm = dfl_add(s2, dfl_mul(dfl_mul(s2, t), P));
  return dfl_mul(lnm, inv_ln2);
}

// 2^(n + y) for an integer n and a pair |y| below a few units, n + y within [-126, 127].
__device__ __forceinline__ dfl dfl_exp2_split(int n, dfl y, const float2* tab) {
  const float ny = rintf(y.hi);
  const dfl f = dfl_sub(y, dfl_make(ny, 0.f));
  const float j = rintf(f.hi * 32.f);
  const dfl u = dfl_sub(f, dfl_make(j * 0.03125f, 0.f));
  const dfl v = dfl_mul(u, dfl_make(0x1.62e430p-1f, -0x1.05c610p-29f));  // u ln 2
  const dfl v2 = dfl_mul(v, v);
  const float vh = v.hi;
  const float tail = v2.hi * v2.hi * fmaf(vh, fmaf(vh, 1.f / 720.f, 1.f / 120.f), 1.f / 24.f);
  const dfl v3s = dfl_mul(dfl_mul(v2, v), dfl_make(0x1.555556p-3f, -0x1.555556p-28f));  // v^3/6
  // e^v - 1, below 0.011 in size, so that 2^(j/32) e^v = T + T (e^v - 1) rounds only the
  // small correction and the final sum
  const dfl em1 = dfl_add(v, dfl_add(dfl_scale(v2, 0.5f), dfl_add(v3s, dfl_make(tail, 0.f))));
  const int ji = min(max(static_cast<int>(j) + 16, 0), kExp2TabN - 1);
  const dfl T = dfl_make(tab[ji].x, tab[ji].y);
  const dfl R = dfl_add(T, dfl_mul(T, em1));
  const float sc = pow2f_exact(n + static_cast<int>(ny));
  return dfl_make(R.hi * sc, R.lo * sc);
}

// x^q for a pair x with a positive normal hi and q given as three floats.
__device__ __forceinline__ dfl dfl_pow(dfl x, flt3 q, const float2* tab) {
  int e;
  const dfl lm = dfl_log2_split(x, e);
  // q e exactly: hi and mid products with their FMA error terms, lo e below 2^-70 of q e
  const float fe = static_cast<float>(e);
  const float p1 = q.hi * fe, e1 = fmaf(q.hi, fe, -p1);
  const float p2 = q.mid * fe, e2 = fmaf(q.mid, fe, -p2);
  const float n1 = rintf(p1);  // |p1| < 2^24: p1 - n1 is exact
  dfl y = dfl_make(p1 - n1, 0.f);
  y = dfl_add(y, dfl_make(p2, 0.f));
  y = dfl_add(y, dfl_make(e1, 0.f));
  y = dfl_add(y, dfl_make(e2 + q.lo * fe, 0.f));
  y = dfl_add(y, dfl_mul(lm, dfl_norm(q.hi, q.mid)));
  return dfl_exp2_split(static_cast<int>(n1), y, tab);
}

// A running sum, renormalised after every term so that lo stays within half an ulp of hi
// and each term adds at most about 2^-48 of the sum in rounding.
struct dacc {
  float hi, lo;
};

__device__ __forceinline__ void dacc_zero(dacc& s) {
  s.hi = 0.f;
  s.lo = 0.f;
}

__device__ __forceinline__ void dacc_add(dacc& s, dfl x) {
  float t, e;
  two_sum(s.hi, x.hi, t, e);
  fast_two_sum(t, __fadd_rn(e, __fadd_rn(s.lo, x.lo)), s.hi, s.lo);
}

// s += x * c (c a constant pair).
__device__ __forceinline__ void dacc_fma(dacc& s, dfl x, dfl c) {
  const float p = __fmul_rn(x.hi, c.hi);
  float e = __fmaf_rn(x.hi, c.hi, -p);
  e = __fmaf_rn(x.hi, c.lo, e);
  e = __fmaf_rn(x.lo, c.hi, e);
  float t, e2;
  two_sum(s.hi, p, t, e2);
  fast_two_sum(t, __fadd_rn(e2, __fadd_rn(s.lo, e)), s.hi, s.lo);
}

__device__ __forceinline__ double dacc_to_double(const dacc& s) {
  return dbl_from_float(s.hi) + dbl_from_float(s.lo);
}

// Block-wide sums of NV pairs without FP64 shuffles or adds: warp butterflies on the
// (hi, lo) floats with pair additions, then warp 0 over the warp totals. Thread 0 gets
// the totals as doubles in out; s_red must hold NV * 32 float2.
template <int NV>
__device__ __forceinline__ void block_sum_dfl(dacc (&v)[NV], float2* s_red, double (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  dfl x[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    x[q] = dfl_norm(v[q].hi, v[q].lo);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dfl y;
      y.hi = __shfl_xor_sync(0xffffffffu, x[q].hi, o);
      y.lo = __shfl_xor_sync(0xffffffffu, x[q].lo, o);
      x[q] = dfl_add(x[q], y);
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) s_red[q * 32 + warp] = make_float2(x[q].hi, x[q].lo);
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const float2 t = lane < nw ? s_red[q * 32 + lane] : make_float2(0.f, 0.f);
      dfl y = dfl_make(t.x, t.y);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dfl z;
        z.hi = __shfl_xor_sync(0xffffffffu, y.hi, o);
        z.lo = __shfl_xor_sync(0xffffffffu, y.lo, o);
        y = dfl_add(y, z);
      }
      out[q] = dfl_to_double(y);
    }
  }
}

// Block-wide sums of NV pairs through shared memory: every thread stores its NV pairs,
// then warp w sums quantities w, w + warps, ... (each lane a strided subset of the threads,
// then a butterfly), so a thread does the butterfly for NV / warps quantities instead of
// all NV. s_buf holds NV * blockDim.x float2, s_out NV float2; thread 0 gets the totals.
template <int NV>
__device__ __forceinline__ void block_sum_dfl_t(dacc (&v)[NV], float2* s_buf, float2* s_out,
                                                double (&out)[NV]) {
  const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, warp = t >> 5, nw = nt >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const dfl x = dfl_norm(v[q].hi, v[q].lo);
    s_buf[q * nt + t] = make_float2(x.hi, x.lo);
  }
  __syncthreads();
  for (int q = warp; q < NV; q += nw) {
    dacc acc;
    dacc_zero(acc);
    for (int i = lane; i < nt; i += 32) {
      const float2 y = s_buf[q * nt + i];
      dacc_add(acc, dfl_make(y.x, y.y));
    }
    dfl x = dfl_norm(acc.hi, acc.lo);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dfl y;
      y.hi = __shfl_xor_sync(0xffffffffu, x.hi, o);
      y.lo = __shfl_xor_sync(0xffffffffu, x.lo, o);
      x = dfl_add(x, y);
    }
    if (lane == 0) s_out[q] = make_float2(x.hi, x.lo);
  }
  __syncthreads();
  if (t == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) out[q] = dfl_to_double(dfl_make(s_out[q].x, s_out[q].y));
  }
}

}  // namespace dvm

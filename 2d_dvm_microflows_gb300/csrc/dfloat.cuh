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

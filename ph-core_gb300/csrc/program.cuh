// program.cuh -- the fixed-opcode accumulator machine evaluated per element.
//
// Values live in slots of type S: uint32_t when every type the program
// touches is 32-bit or narrower (Float32, Int32, Bool), uint64_t otherwise.
// Float32 and Int32 occupy the low 32 bits, Int64 and Float64 all 64, Bool is
// 0/1.  Every instruction is uniform across the grid, so each instruction is
// dispatched ONCE per thread (uniform branches) and then applied to the V
// elements the thread holds in registers; per element only the arithmetic
// itself runs.  Semantics follow Crystal 1.0 numbers (checked Int32/Int64
// + - *, floor division and modulo, Int / Int -> Float64, Float ** Int by
// binary exponentiation), matching the CPU oracle.  Translation units that
// include this file are compiled with -fmad=false: every Float32 operation
// rounds once, as on the host.
#pragma once

#include <cstring>
#include <type_traits>

#include "common.cuh"

namespace phcu {

// ----------------------------------------------------------- slot access
template <typename S>
__device__ __forceinline__ float sf32(S s) { return __uint_as_float((uint32_t)s); }
template <typename S>
__device__ __forceinline__ S pf32(float f) { return (S)__float_as_uint(f); }
template <typename S>
__device__ __forceinline__ int32_t si32(S s) { return (int32_t)(uint32_t)s; }
template <typename S>
__device__ __forceinline__ S pi32(int32_t v) { return (S)(uint32_t)v; }
__device__ __forceinline__ double sf64(uint64_t s) { return __longlong_as_double((long long)s); }
__device__ __forceinline__ uint64_t pf64(double f) { return (uint64_t)__double_as_longlong(f); }

// ----------------------------------------------------------------- loads
// One element of type dtype at p as a slot (the caller switches on dtype
// outside its element loops).
template <typename S, int ES>
__device__ __forceinline__ S ld_elem(const char* p) {
  if constexpr (ES == 4) return (S)__ldg((const uint32_t*)p);
  else if constexpr (ES == 8) return (S)__ldg((const unsigned long long*)p);
  else return (S)(*(const uint8_t*)p != 0);
}
template <typename S, int ES>
__device__ __forceinline__ void st_elem(char* p, S v) {
  if constexpr (ES == 4) *(uint32_t*)p = (uint32_t)v;
  else if constexpr (ES == 8) *(unsigned long long*)p = (unsigned long long)v;
  else *(uint8_t*)p = (uint8_t)(v & 1u);
}

// VEC consecutive elements starting at p (aligned to min(16, VEC*ES) bytes).
template <typename S, int ES, int VEC>
__device__ __forceinline__ void ld_vec(const char* p, S* v) {
  if constexpr (VEC == 8 && ES != 1) {  // two (ES=4) or four (ES=8) 16-byte accesses
    ld_vec<S, ES, 4>(p, v);
    ld_vec<S, ES, 4>(p + 4 * ES, v + 4);
  } else if constexpr (ES == 4) {
    if constexpr (VEC == 4) {
      uint4 x = __ldg((const uint4*)p);
      v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else if constexpr (VEC == 2) {
      uint2 x = __ldg((const uint2*)p);
      v[0] = x.x; v[1] = x.y;
    } else {
      v[0] = __ldg((const uint32_t*)p);
    }
  } else if constexpr (ES == 8) {
    if constexpr (VEC == 4) {
      ulonglong2 x = __ldg((const ulonglong2*)p);
      ulonglong2 y = __ldg((const ulonglong2*)(p + 16));
      v[0] = (S)x.x; v[1] = (S)x.y; v[2] = (S)y.x; v[3] = (S)y.y;
    } else if constexpr (VEC == 2) {
      ulonglong2 x = __ldg((const ulonglong2*)p);
      v[0] = (S)x.x; v[1] = (S)x.y;
    } else {
      v[0] = (S)__ldg((const unsigned long long*)p);
    }
  } else {
#pragma unroll
    for (int i = 0; i < VEC; i++) v[i] = (S)(p[i] != 0);
  }
}

template <typename S, int ES, int VEC>
__device__ __forceinline__ void st_vec(char* p, const S* v) {
  if constexpr (VEC == 8 && ES != 1) {
    st_vec<S, ES, 4>(p, v);
    st_vec<S, ES, 4>(p + 4 * ES, v + 4);
  } else if constexpr (ES == 4) {
    if constexpr (VEC == 4) *(uint4*)p = make_uint4((uint32_t)v[0], (uint32_t)v[1], (uint32_t)v[2], (uint32_t)v[3]);
    else if constexpr (VEC == 2) *(uint2*)p = make_uint2((uint32_t)v[0], (uint32_t)v[1]);
    else *(uint32_t*)p = (uint32_t)v[0];
  } else if constexpr (ES == 8) {
    if constexpr (VEC == 4) {
      *(ulonglong2*)p = make_ulonglong2(v[0], v[1]);
      *(ulonglong2*)(p + 16) = make_ulonglong2(v[2], v[3]);
    } else if constexpr (VEC == 2) {
      *(ulonglong2*)p = make_ulonglong2(v[0], v[1]);
    } else {
      *(unsigned long long*)p = v[0];
    }
  } else {
#pragma unroll
    for (int i = 0; i < VEC; i++) p[i] = (char)(v[i] & 1u);
  }
}

// VEC elements of one operand in a vector mode: VM_VEC (unit stride),
// VM_VEC_REV (stride -1, vector at the low end, reversed), VM_SCALAR.
template <typename S, int ES, int VEC>
__device__ __forceinline__ void ld_operand(const char* p, int64_t inner_stride, int vmode, S* v) {
  if (vmode == VM_VEC) {
    ld_vec<S, ES, VEC>(p, v);
  } else if (vmode == VM_VEC_REV) {
    S t[VEC];
    ld_vec<S, ES, VEC>(p - (VEC - 1) * ES, t);
#pragma unroll
    for (int i = 0; i < VEC; i++) v[i] = t[VEC - 1 - i];
  } else {
#pragma unroll
    for (int i = 0; i < VEC; i++) v[i] = ld_elem<S, ES>(p + i * inner_stride * ES);
  }
}

template <typename S, int ES, int VEC>
__device__ __forceinline__ void st_operand(char* p, int64_t inner_stride, int vmode, const S* v) {
  if (vmode == VM_VEC) {
    st_vec<S, ES, VEC>(p, v);
  } else {
#pragma unroll
    for (int i = 0; i < VEC; i++) st_elem<S, ES>(p + i * inner_stride * ES, v[i]);
  }
}

// ------------------------------------------------------- conversions
template <typename S>
__device__ __forceinline__ S convert_slot(S s, int from, int to) {
  if (from == to) return s;
  if constexpr (sizeof(S) == 4) {
    switch (from) {
      case PHCU_BOOL:
      case PHCU_I32: {
        int32_t x = (from == PHCU_BOOL) ? (int32_t)(s & 1u) : si32(s);
        if (to == PHCU_F32) return pf32<S>((float)x);
        if (to == PHCU_I32) return pi32<S>(x);
        return (S)(x != 0);
      }
      case PHCU_F32: {
        float x = sf32(s);
        if (to == PHCU_I32) return pi32<S>((int32_t)x);
        return (S)(x != 0.0f);
      }
    }
    return s;
  } else {
    switch (from) {
      case PHCU_BOOL:
      case PHCU_I32:
      case PHCU_I64: {
        int64_t x = (from == PHCU_BOOL) ? (int64_t)(s & 1u) : (from == PHCU_I32) ? (int64_t)si32(s) : (int64_t)s;
        switch (to) {
          case PHCU_I32: return (S)(uint32_t)(int32_t)x;
          case PHCU_I64: return (S)x;
          case PHCU_F32: return pf32<S>((float)x);
          case PHCU_F64: return pf64((double)x);
          case PHCU_BOOL: return x != 0;
        }
        break;
      }
      case PHCU_F32: {
        float x = sf32(s);
        switch (to) {
          case PHCU_F64: return pf64((double)x);
          case PHCU_I32: return (S)(uint32_t)(int32_t)x;
          case PHCU_I64: return (S)(int64_t)x;
          case PHCU_BOOL: return x != 0.0f;
        }
        break;
      }
      case PHCU_F64: {
        double x = sf64(s);
        switch (to) {
          case PHCU_F32: return pf32<S>((float)x);
          case PHCU_I32: return (S)(uint32_t)(int32_t)x;
          case PHCU_I64: return (S)(int64_t)x;
          case PHCU_BOOL: return x != 0.0;
        }
        break;
      }
    }
    return s;
  }
}

// ------------------------------------------------------ integer helpers
__device__ __forceinline__ int64_t floordiv_i64(int64_t a, int64_t b) {
  int64_t q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) q -= 1;
  return q;
}
__device__ __forceinline__ int64_t floormod_i64(int64_t a, int64_t b) {
  int64_t r = a % b;
  if (r != 0 && ((r < 0) != (b < 0))) r += b;
  return r;
}
__device__ __forceinline__ int32_t chk_add32(int32_t a, int32_t b, uint32_t& st) {
  int32_t r = (int32_t)((uint32_t)a + (uint32_t)b);
  if (((a ^ r) & (b ^ r)) < 0) st |= PHCU_ST_OVERFLOW;
  return r;
}
__device__ __forceinline__ int32_t chk_sub32(int32_t a, int32_t b, uint32_t& st) {
  int32_t r = (int32_t)((uint32_t)a - (uint32_t)b);
  if (((a ^ b) & (a ^ r)) < 0) st |= PHCU_ST_OVERFLOW;
  return r;
}
__device__ __forceinline__ int32_t chk_mul32(int32_t a, int32_t b, uint32_t& st) {
  int64_t r = (int64_t)a * b;
  if (r != (int32_t)r) st |= PHCU_ST_OVERFLOW;
  return (int32_t)(uint32_t)(uint64_t)r;
}
__device__ __forceinline__ int64_t chk_add64(int64_t a, int64_t b, uint32_t& st) {
  int64_t r = (int64_t)((uint64_t)a + (uint64_t)b);
  if (((a ^ r) & (b ^ r)) < 0) st |= PHCU_ST_OVERFLOW;
  return r;
}
__device__ __forceinline__ int64_t chk_sub64(int64_t a, int64_t b, uint32_t& st) {
  int64_t r = (int64_t)((uint64_t)a - (uint64_t)b);
  if (((a ^ b) & (a ^ r)) < 0) st |= PHCU_ST_OVERFLOW;
  return r;
}
__device__ __forceinline__ int64_t chk_mul64(int64_t a, int64_t b, uint32_t& st) {
  int64_t r = (int64_t)((uint64_t)a * (uint64_t)b);
  if (__mul64hi(a, b) != (r >> 63)) st |= PHCU_ST_OVERFLOW;
  return r;
}
template <typename I>
__device__ __forceinline__ I wrap_mul(I a, I b) {
  using U = typename std::conditional<sizeof(I) == 4, uint32_t, uint64_t>::type;
  return (I)((U)a * (U)b);
}

// Int#** (checked) and Int#&** (wrapping): binary exponentiation.
template <typename I>
__device__ __forceinline__ I int_pow(I base, int64_t e, bool wrapping, uint32_t& st) {
  if (e < 0) {
    st |= PHCU_ST_ARGUMENT;
    return 0;
  }
  I result = 1, k = base;
  while (e > 0) {
    if (e & 1) {
      if (wrapping) result = wrap_mul<I>(result, k);
      else if constexpr (sizeof(I) == 4) result = chk_mul32(result, k, st);
      else result = chk_mul64(result, k, st);
    }
    e >>= 1;
    if (e > 0) {
      if (wrapping) k = wrap_mul<I>(k, k);
      else if constexpr (sizeof(I) == 4) k = chk_mul32(k, k, st);
      else k = chk_mul64(k, k, st);
    }
  }
  return result;
}

// LLVM powi semantics: binary exponentiation, reciprocal for negative exponents
// (the method of compiler-rt's __powisf2/__powidf2).
template <typename F>
__device__ __forceinline__ F powi(F a, int32_t b) {
  const bool recip = b < 0;
  F r = (F)1;
  for (;;) {
    if (b & 1) r = r * a;
    b /= 2;
    if (b == 0) break;
    a = a * a;
  }
  return recip ? (F)1 / r : r;
}

// Crystal `Int32 / Int32` is `x.to_f64 / y.to_f64`: the IEEE double quotient,
// correctly rounded to nearest-even.  GB300's FP64 rate makes a double
// division cost about as much as reading the operands many times over, so the
// quotient is computed exactly with 32-bit integer long division instead
// (schoolbook division with estimated digits, Knuth TAOCP vol. 2, 4.3.1, in
// the redundant signed-digit form of SRT division): normalise |x| and |y| so
// both lie in [2^30, 2^31) (divisor b'), take the integer part of their
// quotient m in [1, 2) and then three 18-bit fraction digits.  Each digit is
// round(r * 2^18 / b') estimated from the top 22 bits of the signed remainder
// r and an FP32 reciprocal of b' (within 0.19 of the exact real quotient), and
// is never corrected: the new remainder r * 2^18 - q * b' lies in (-b', b'),
// fits an int32, and the next digit absorbs its sign.  The fraction
// F = d0 * 2^36 + d1 * 2^18 + d2 then satisfies m * 2^54 = 2^54 + F + r3 / b'.
// No quotient of two Int32 lies exactly halfway between two doubles (an odd
// number above 2^53 would have to divide |x| <= 2^31), so rounding to nearest is
// (F + 2) >> 2, or (F + 1) >> 2 when r3 < 0.  Every |quotient| of two non-zero
// Int32 lies in [2^-31, 2^31], so the result is always normal.
__device__ __forceinline__ uint64_t int32_div_f64_bits(int32_t x, int32_t y) {
  const uint32_t a = x < 0 ? 0u - (uint32_t)x : (uint32_t)x;
  const uint32_t b = y < 0 ? 0u - (uint32_t)y : (uint32_t)y;
  if (b == 0 || a == 0) {
    if (b != 0) return (uint64_t)((uint32_t)y >> 31) << 63;                    // +0.0 / y = +-0.0
    if (a == 0) return 0x7ff8000000000000ull;                                  // 0 / 0 = NaN
    return ((uint64_t)((uint32_t)x >> 31) << 63) | 0x7ff0000000000000ull;      // x / 0 = +-Inf (sign of x)
  }
  const int za = __clz(a), zb = __clz(b);
  // leading one at bit 30 (|Int32| <= 2^31 leaves bit 0 of a << za clear)
  const uint32_t an = (a << za) >> 1, bn = (b << zb) >> 1;
  const uint32_t c = an < bn;  // m = 2 an / bn, one binade lower
  int32_t r = (int32_t)((an << c) - bn);
  const int e = zb - za - (int)c;
  // bn * 2^-27 in [8, 16) as an FP32 built from the top 24 bits of bn
  // (truncated: within 1 ulp); rcp.approx adds at most 1 ulp, so rc is
  // 2^27 / bn within 2 ulp and moves an estimate below 2^18 by under 1/16
  float rc;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rc) : "f"(__uint_as_float(0x40800000u + (bn >> 7))));
  int32_t d[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    // r >> 9 in [-2^22, 2^22) converts exactly through the 1.5 * 2^23 offset;
    // the dropped bits move the estimate by under 2^9 * 2^18 / 2^30 = 1/8
    const float rh = __int_as_float(0x4b400000 + (r >> 9)) - 12582912.0f;
    // rounded to an integer by the same offset, read back from the bits
    const int32_t q = __float_as_int(__fmaf_rn(rh, rc, 12582912.0f)) - 0x4b400000;
    r = (int32_t)(((uint32_t)r << 18) - (uint32_t)q * bn);  // exact: the true value lies in (-bn, bn)
    d[k] = q;
  }
  const int64_t F = ((((int64_t)d[0] << 18) + d[1]) << 18) + d[2];
  const uint64_t mant = (uint64_t)(F + 2 - (r < 0)) >> 2;
  const uint64_t sign = (uint64_t)(((uint32_t)x ^ (uint32_t)y) & 0x80000000u) << 32;
  return sign + ((uint64_t)(e + 1023) << 52) + mant;
}

// ------------------------------------------------- vector op kernels
// Each applies one binary operator to V element pairs (dispatch done once).
#define PHCU_LOOP _Pragma("unroll") for (int v = 0; v < V; v++)

template <typename S, int V>
__device__ __forceinline__ void bin_f32(int op, int bt, S* a, const S* b, uint32_t& st) {
  if (op == PHCU_OP_POW && is_int_t(bt)) {
    PHCU_LOOP a[v] = pf32<S>(powi<float>(sf32(a[v]), bt == PHCU_I32 ? si32(b[v]) : (int32_t)(int64_t)b[v]));
    return;
  }
  switch (op) {
    case PHCU_OP_ADD: PHCU_LOOP a[v] = pf32<S>(sf32(a[v]) + sf32(b[v])); break;
    case PHCU_OP_SUB: PHCU_LOOP a[v] = pf32<S>(sf32(a[v]) - sf32(b[v])); break;
    case PHCU_OP_MUL: PHCU_LOOP a[v] = pf32<S>(sf32(a[v]) * sf32(b[v])); break;
    case PHCU_OP_DIV: PHCU_LOOP a[v] = pf32<S>(sf32(a[v]) / sf32(b[v])); break;
    case PHCU_OP_FLOORDIV: PHCU_LOOP a[v] = pf32<S>(floorf(sf32(a[v]) / sf32(b[v]))); break;
    case PHCU_OP_MOD:
      PHCU_LOOP {
        const float x = sf32(a[v]), y = sf32(b[v]);
        if (y == 0.0f) {
          st |= PHCU_ST_DIVZERO;
          a[v] = pf32<S>(0.0f);
        } else {
          const float q = floorf(x / y);
          const float m = y * q;
          a[v] = pf32<S>(x - m);
        }
      }
      break;
    case PHCU_OP_POW: PHCU_LOOP a[v] = pf32<S>(powf(sf32(a[v]), sf32(b[v]))); break;
    case PHCU_OP_GT: PHCU_LOOP a[v] = sf32(a[v]) > sf32(b[v]); break;
    case PHCU_OP_LT: PHCU_LOOP a[v] = sf32(a[v]) < sf32(b[v]); break;
    case PHCU_OP_GE: PHCU_LOOP a[v] = sf32(a[v]) >= sf32(b[v]); break;
    case PHCU_OP_LE: PHCU_LOOP a[v] = sf32(a[v]) <= sf32(b[v]); break;
    case PHCU_OP_EQ: PHCU_LOOP a[v] = sf32(a[v]) == sf32(b[v]); break;
    case PHCU_OP_CMP:
      PHCU_LOOP {
        const float x = sf32(a[v]), y = sf32(b[v]);
        a[v] = pi32<S>((x > y) - (x < y));
      }
      break;
  }
}

template <typename S, int V>
__device__ __forceinline__ void bin_i32(int op, S* a, const S* b, uint32_t& st) {
  switch (op) {
    case PHCU_OP_ADD: PHCU_LOOP a[v] = pi32<S>(chk_add32(si32(a[v]), si32(b[v]), st)); break;
    case PHCU_OP_SUB: PHCU_LOOP a[v] = pi32<S>(chk_sub32(si32(a[v]), si32(b[v]), st)); break;
    case PHCU_OP_MUL: PHCU_LOOP a[v] = pi32<S>(chk_mul32(si32(a[v]), si32(b[v]), st)); break;
    case PHCU_OP_DIV:
      if constexpr (sizeof(S) == 8) {
        PHCU_LOOP a[v] = int32_div_f64_bits(si32(a[v]), si32(b[v]));
      }
      break;
    case PHCU_OP_FLOORDIV:
      PHCU_LOOP {
        const int32_t x = si32(a[v]), y = si32(b[v]);
        if (y == 0) {
          st |= PHCU_ST_DIVZERO;
          a[v] = 0;
        } else if (x == INT32_MIN && y == -1) {
          st |= PHCU_ST_OVERFLOW;
        } else {
          a[v] = pi32<S>((int32_t)floordiv_i64(x, y));
        }
      }
      break;
    case PHCU_OP_MOD:
      PHCU_LOOP {
        const int32_t x = si32(a[v]), y = si32(b[v]);
        if (y == 0) {
          st |= PHCU_ST_DIVZERO;
          a[v] = 0;
        } else if (y == -1) {
          a[v] = 0;
        } else {
          a[v] = pi32<S>((int32_t)floormod_i64(x, y));
        }
      }
      break;
    case PHCU_OP_POW: PHCU_LOOP a[v] = pi32<S>(int_pow<int32_t>(si32(a[v]), si32(b[v]), false, st)); break;
    case PHCU_OP_WADD: PHCU_LOOP a[v] = pi32<S>((int32_t)((uint32_t)a[v] + (uint32_t)b[v])); break;
    case PHCU_OP_WSUB: PHCU_LOOP a[v] = pi32<S>((int32_t)((uint32_t)a[v] - (uint32_t)b[v])); break;
    case PHCU_OP_WMUL: PHCU_LOOP a[v] = pi32<S>((int32_t)((uint32_t)a[v] * (uint32_t)b[v])); break;
    case PHCU_OP_WPOW: PHCU_LOOP a[v] = pi32<S>(int_pow<int32_t>(si32(a[v]), si32(b[v]), true, st)); break;
    case PHCU_OP_AND: PHCU_LOOP a[v] = pi32<S>(si32(a[v]) & si32(b[v])); break;
    case PHCU_OP_OR: PHCU_LOOP a[v] = pi32<S>(si32(a[v]) | si32(b[v])); break;
    case PHCU_OP_XOR: PHCU_LOOP a[v] = pi32<S>(si32(a[v]) ^ si32(b[v])); break;
    case PHCU_OP_GT: PHCU_LOOP a[v] = si32(a[v]) > si32(b[v]); break;
    case PHCU_OP_LT: PHCU_LOOP a[v] = si32(a[v]) < si32(b[v]); break;
    case PHCU_OP_GE: PHCU_LOOP a[v] = si32(a[v]) >= si32(b[v]); break;
    case PHCU_OP_LE: PHCU_LOOP a[v] = si32(a[v]) <= si32(b[v]); break;
    case PHCU_OP_EQ: PHCU_LOOP a[v] = si32(a[v]) == si32(b[v]); break;
    case PHCU_OP_CMP:
      PHCU_LOOP {
        const int32_t x = si32(a[v]), y = si32(b[v]);
        a[v] = pi32<S>((x > y) - (x < y));
      }
      break;
  }
}

template <int V>
__device__ __forceinline__ void bin_f64(int op, int bt, uint64_t* a, const uint64_t* b, uint32_t& st) {
  if (op == PHCU_OP_POW && is_int_t(bt)) {
    PHCU_LOOP a[v] = pf64(powi<double>(sf64(a[v]), bt == PHCU_I32 ? si32(b[v]) : (int32_t)(int64_t)b[v]));
    return;
  }
  switch (op) {
    case PHCU_OP_ADD: PHCU_LOOP a[v] = pf64(sf64(a[v]) + sf64(b[v])); break;
    case PHCU_OP_SUB: PHCU_LOOP a[v] = pf64(sf64(a[v]) - sf64(b[v])); break;
    case PHCU_OP_MUL: PHCU_LOOP a[v] = pf64(sf64(a[v]) * sf64(b[v])); break;
    case PHCU_OP_DIV: PHCU_LOOP a[v] = pf64(sf64(a[v]) / sf64(b[v])); break;
    case PHCU_OP_FLOORDIV: PHCU_LOOP a[v] = pf64(floor(sf64(a[v]) / sf64(b[v]))); break;
    case PHCU_OP_MOD:
      PHCU_LOOP {
        const double x = sf64(a[v]), y = sf64(b[v]);
        if (y == 0.0) {
          st |= PHCU_ST_DIVZERO;
          a[v] = pf64(0.0);
        } else {
          const double q = floor(x / y);
          const double m = y * q;
          a[v] = pf64(x - m);
        }
      }
      break;
    case PHCU_OP_POW: PHCU_LOOP a[v] = pf64(pow(sf64(a[v]), sf64(b[v]))); break;
    case PHCU_OP_GT: PHCU_LOOP a[v] = sf64(a[v]) > sf64(b[v]); break;
    case PHCU_OP_LT: PHCU_LOOP a[v] = sf64(a[v]) < sf64(b[v]); break;
    case PHCU_OP_GE: PHCU_LOOP a[v] = sf64(a[v]) >= sf64(b[v]); break;
    case PHCU_OP_LE: PHCU_LOOP a[v] = sf64(a[v]) <= sf64(b[v]); break;
    case PHCU_OP_EQ: PHCU_LOOP a[v] = sf64(a[v]) == sf64(b[v]); break;
    case PHCU_OP_CMP:
      PHCU_LOOP {
        const double x = sf64(a[v]), y = sf64(b[v]);
        a[v] = (uint64_t)(uint32_t)((x > y) - (x < y));
      }
      break;
  }
}

template <int V>
__device__ __forceinline__ void bin_i64(int op, uint64_t* a, const uint64_t* b, uint32_t& st) {
  switch (op) {
    case PHCU_OP_ADD: PHCU_LOOP a[v] = (uint64_t)chk_add64((int64_t)a[v], (int64_t)b[v], st); break;
    case PHCU_OP_SUB: PHCU_LOOP a[v] = (uint64_t)chk_sub64((int64_t)a[v], (int64_t)b[v], st); break;
    case PHCU_OP_MUL: PHCU_LOOP a[v] = (uint64_t)chk_mul64((int64_t)a[v], (int64_t)b[v], st); break;
    case PHCU_OP_DIV: PHCU_LOOP a[v] = pf64((double)(int64_t)a[v] / (double)(int64_t)b[v]); break;
    case PHCU_OP_FLOORDIV:
      PHCU_LOOP {
        const int64_t x = (int64_t)a[v], y = (int64_t)b[v];
        if (y == 0) {
          st |= PHCU_ST_DIVZERO;
          a[v] = 0;
        } else if (x == INT64_MIN && y == -1) {
          st |= PHCU_ST_OVERFLOW;
        } else {
          a[v] = (uint64_t)floordiv_i64(x, y);
        }
      }
      break;
    case PHCU_OP_MOD:
      PHCU_LOOP {
        const int64_t x = (int64_t)a[v], y = (int64_t)b[v];
        if (y == 0) {
          st |= PHCU_ST_DIVZERO;
          a[v] = 0;
        } else if (y == -1) {
          a[v] = 0;
        } else {
          a[v] = (uint64_t)floormod_i64(x, y);
        }
      }
      break;
    case PHCU_OP_POW: PHCU_LOOP a[v] = (uint64_t)int_pow<int64_t>((int64_t)a[v], (int64_t)b[v], false, st); break;
    case PHCU_OP_WADD: PHCU_LOOP a[v] = a[v] + b[v]; break;
    case PHCU_OP_WSUB: PHCU_LOOP a[v] = a[v] - b[v]; break;
    case PHCU_OP_WMUL: PHCU_LOOP a[v] = a[v] * b[v]; break;
    case PHCU_OP_WPOW: PHCU_LOOP a[v] = (uint64_t)int_pow<int64_t>((int64_t)a[v], (int64_t)b[v], true, st); break;
    case PHCU_OP_AND: PHCU_LOOP a[v] = a[v] & b[v]; break;
    case PHCU_OP_OR: PHCU_LOOP a[v] = a[v] | b[v]; break;
    case PHCU_OP_XOR: PHCU_LOOP a[v] = a[v] ^ b[v]; break;
    case PHCU_OP_GT: PHCU_LOOP a[v] = (int64_t)a[v] > (int64_t)b[v]; break;
    case PHCU_OP_LT: PHCU_LOOP a[v] = (int64_t)a[v] < (int64_t)b[v]; break;
    case PHCU_OP_GE: PHCU_LOOP a[v] = (int64_t)a[v] >= (int64_t)b[v]; break;
    case PHCU_OP_LE: PHCU_LOOP a[v] = (int64_t)a[v] <= (int64_t)b[v]; break;
    case PHCU_OP_EQ: PHCU_LOOP a[v] = a[v] == b[v]; break;
    case PHCU_OP_CMP:
      PHCU_LOOP {
        const int64_t x = (int64_t)a[v], y = (int64_t)b[v];
        a[v] = (uint64_t)(uint32_t)((x > y) - (x < y));
      }
      break;
  }
}

template <typename S, int V>
__device__ __forceinline__ void bin_bool(int op, S* a, const S* b) {
  switch (op) {
    case PHCU_OP_AND: PHCU_LOOP a[v] = (a[v] & b[v]) & 1u; break;
    case PHCU_OP_OR: PHCU_LOOP a[v] = (a[v] | b[v]) & 1u; break;
    case PHCU_OP_XOR: PHCU_LOOP a[v] = (a[v] ^ b[v]) & 1u; break;
    case PHCU_OP_EQ: PHCU_LOOP a[v] = (a[v] & 1u) == (b[v] & 1u); break;
  }
}

template <typename S, int V>
__device__ __forceinline__ void un_vec(int op, int T, S* a, uint32_t& st) {
  if (op == PHCU_I_POS) return;
  if (op == PHCU_I_NEG) {
    switch (T) {
      case PHCU_F32: PHCU_LOOP a[v] = pf32<S>(-sf32(a[v])); break;
      case PHCU_I32:
        PHCU_LOOP {
          const int32_t x = si32(a[v]);
          if (x == INT32_MIN) st |= PHCU_ST_OVERFLOW;
          else a[v] = pi32<S>(-x);
        }
        break;
      case PHCU_F64:
        if constexpr (sizeof(S) == 8) { PHCU_LOOP a[v] = pf64(-sf64(a[v])); }
        break;
      case PHCU_I64:
        if constexpr (sizeof(S) == 8) {
          PHCU_LOOP {
            const int64_t x = (int64_t)a[v];
            if (x == INT64_MIN) st |= PHCU_ST_OVERFLOW;
            else a[v] = (uint64_t)(-x);
          }
        }
        break;
    }
    return;
  }
  // NOT
  if (T == PHCU_I32) {
    PHCU_LOOP a[v] = pi32<S>(~si32(a[v]));
  } else if (T == PHCU_I64) {
    PHCU_LOOP a[v] = ~a[v];
  }
}

template <typename S, int V>
__device__ __forceinline__ void cvt_vec(S* a, int from, int to) {
  if (from == to) return;
  // one dispatch on the (from, to) pair, then a straight loop of that conversion
#define PHCU_CVT(F, T_) \
  case (F) * 8 + (T_): PHCU_LOOP a[v] = convert_slot<S>(a[v], (F), (T_)); return;
  switch (from * 8 + to) {
    PHCU_CVT(PHCU_BOOL, PHCU_I32) PHCU_CVT(PHCU_BOOL, PHCU_F32) PHCU_CVT(PHCU_I32, PHCU_BOOL)
    PHCU_CVT(PHCU_I32, PHCU_F32) PHCU_CVT(PHCU_F32, PHCU_BOOL) PHCU_CVT(PHCU_F32, PHCU_I32)
    default: break;
  }
  if constexpr (sizeof(S) == 8) {
    switch (from * 8 + to) {
      PHCU_CVT(PHCU_BOOL, PHCU_I64) PHCU_CVT(PHCU_BOOL, PHCU_F64) PHCU_CVT(PHCU_I32, PHCU_I64)
      PHCU_CVT(PHCU_I32, PHCU_F64) PHCU_CVT(PHCU_I64, PHCU_BOOL) PHCU_CVT(PHCU_I64, PHCU_I32)
      PHCU_CVT(PHCU_I64, PHCU_F32) PHCU_CVT(PHCU_I64, PHCU_F64) PHCU_CVT(PHCU_F32, PHCU_I64)
      PHCU_CVT(PHCU_F32, PHCU_F64) PHCU_CVT(PHCU_F64, PHCU_BOOL) PHCU_CVT(PHCU_F64, PHCU_I32)
      PHCU_CVT(PHCU_F64, PHCU_I64) PHCU_CVT(PHCU_F64, PHCU_F32)
      default: break;
    }
  }
#undef PHCU_CVT
  PHCU_LOOP a[v] = convert_slot<S>(a[v], from, to);
}

// x ** e for an exponent shared by all V elements (an immediate): the same
// multiply sequence as powi(), with the loop control uniform across the warp.
template <typename S, int V>
__device__ __forceinline__ void powi_uniform(S* a, int T, int32_t e) {
  const bool recip = e < 0;
  if (T == PHCU_F32) {
    float x[V], r[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      x[v] = sf32(a[v]);
      r[v] = 1.0f;
    }
    for (int32_t b = e;;) {
      if (b & 1) {
#pragma unroll
        for (int v = 0; v < V; v++) r[v] = r[v] * x[v];
      }
      b /= 2;
      if (b == 0) break;
#pragma unroll
      for (int v = 0; v < V; v++) x[v] = x[v] * x[v];
    }
    if (recip) {
#pragma unroll
      for (int v = 0; v < V; v++) a[v] = pf32<S>(1.0f / r[v]);
    } else {
#pragma unroll
      for (int v = 0; v < V; v++) a[v] = pf32<S>(r[v]);
    }
  } else if constexpr (sizeof(S) == 8) {
    double x[V], r[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      x[v] = sf64(a[v]);
      r[v] = 1.0;
    }
    for (int32_t b = e;;) {
      if (b & 1) {
#pragma unroll
        for (int v = 0; v < V; v++) r[v] = r[v] * x[v];
      }
      b /= 2;
      if (b == 0) break;
#pragma unroll
      for (int v = 0; v < V; v++) x[v] = x[v] * x[v];
    }
    if (recip) {
#pragma unroll
      for (int v = 0; v < V; v++) a[v] = pf64(1.0 / r[v]);
    } else {
#pragma unroll
      for (int v = 0; v < V; v++) a[v] = pf64(r[v]);
    }
  }
}

// A plain binary program, [ACC = IN0; ACC = ACC op IN1; optional CVT], run in
// place on input 0's registers (no accumulator or operand copies).
template <typename S, int V>
__device__ __forceinline__ void run_binop(const phcu_program_t& P, S* a, const S* b, uint32_t& st) {
  const int op = P.code[1].op, T = P.code[1].type, bt = P.code[1].btype;
  switch (T) {
    case PHCU_F32: bin_f32<S, V>(op, bt, a, b, st); break;
    case PHCU_I32: bin_i32<S, V>(op, a, b, st); break;
    case PHCU_BOOL: bin_bool<S, V>(op, a, b); break;
    case PHCU_F64:
      if constexpr (sizeof(S) == 8) bin_f64<V>(op, bt, a, b, st);
      break;
    case PHCU_I64:
      if constexpr (sizeof(S) == 8) bin_i64<V>(op, a, b, st);
      break;
  }
  if (P.n_instr == 3) cvt_vec<S, V>(a, P.code[2].type, (int)P.code[2].imm.i);
}

// ------------------------------------------- pre-decoded arithmetic forms
// The library's private copy of a program carries, in pad[0] of each
// instruction, one of these ids when the instruction is a Float32 or Int32
// operator whose operand B is an input or an immediate of the compute type.
// The interpreter then runs it with one uniform branch on the operand source
// and no operand copy, conversion check or type dispatch.  FX_NONE (0) leaves
// the instruction to the general path.
enum : uint8_t {
  FX_NONE = 0,
  FX_F32_LD, FX_F32_ADD, FX_F32_SUB, FX_F32_MUL, FX_F32_DIV, FX_F32_RSUB, FX_F32_RDIV,
  FX_I32_LD, FX_I32_ADD, FX_I32_SUB, FX_I32_MUL, FX_I32_RSUB, FX_I32_WADD, FX_I32_WSUB, FX_I32_WMUL,
  FX_I32_RWSUB, FX_I32_AND, FX_I32_OR, FX_I32_XOR,
};

// Host: writes the pre-decoded ids into a program copy (pad[0] of every
// instruction; anything a caller left there is overwritten).  An Int32
// immediate of a Float32 instruction is converted here, round to nearest as
// the device conversion does, so the instruction qualifies.
inline void predecode_program(phcu_program_t* P) {
  for (int i = 0; i < P->n_instr && i < PHCU_MAX_INSTR; i++) {
    phcu_instr_t& I = P->code[i];
    I.pad[0] = FX_NONE;
    if (!(I.src < MAXIN || I.src == PHCU_SRC_IMM)) continue;
    if (I.src == PHCU_SRC_IMM && I.type == PHCU_F32 && I.btype == PHCU_I32 && I.op != PHCU_OP_POW) {
      const float f = (float)(int32_t)(uint32_t)(uint64_t)I.imm.i;
      uint32_t bits;
      memcpy(&bits, &f, 4);
      I.imm.i = (int64_t)bits;
      I.btype = PHCU_F32;
    }
    if (I.btype != I.type) continue;
    const bool swap = (I.flags & 1) != 0;
    if (I.type == PHCU_F32) {
      switch (I.op) {
        case PHCU_I_LD: I.pad[0] = FX_F32_LD; break;
        case PHCU_OP_ADD: I.pad[0] = FX_F32_ADD; break;
        case PHCU_OP_MUL: I.pad[0] = FX_F32_MUL; break;
        case PHCU_OP_SUB: I.pad[0] = swap ? FX_F32_RSUB : FX_F32_SUB; break;
        case PHCU_OP_DIV: I.pad[0] = swap ? FX_F32_RDIV : FX_F32_DIV; break;
      }
    } else if (I.type == PHCU_I32) {
      switch (I.op) {
        case PHCU_I_LD: I.pad[0] = FX_I32_LD; break;
        case PHCU_OP_ADD: I.pad[0] = FX_I32_ADD; break;
        case PHCU_OP_MUL: I.pad[0] = FX_I32_MUL; break;
        case PHCU_OP_SUB: I.pad[0] = swap ? FX_I32_RSUB : FX_I32_SUB; break;
        case PHCU_OP_WADD: I.pad[0] = FX_I32_WADD; break;
        case PHCU_OP_WMUL: I.pad[0] = FX_I32_WMUL; break;
        case PHCU_OP_WSUB: I.pad[0] = swap ? FX_I32_RWSUB : FX_I32_WSUB; break;
        case PHCU_OP_AND: I.pad[0] = FX_I32_AND; break;
        case PHCU_OP_OR: I.pad[0] = FX_I32_OR; break;
        case PHCU_OP_XOR: I.pad[0] = FX_I32_XOR; break;
      }
    }
  }
}

// ACC = f(ACC, B) with B = the immediate or input `src`, chosen by one
// uniform branch.
template <typename S, int NIN, int V, typename F>
__device__ __forceinline__ void fx_apply(int src, S imm, S* acc, const S (&in)[NIN > 0 ? NIN : 1][V], F f) {
  if (src == PHCU_SRC_IMM) {
    PHCU_LOOP acc[v] = f(acc[v], imm);
    return;
  }
  if constexpr (NIN > 3) {
    if (src == 3) {
      PHCU_LOOP acc[v] = f(acc[v], in[3][v]);
      return;
    }
  }
  if constexpr (NIN > 2) {
    if (src == 2) {
      PHCU_LOOP acc[v] = f(acc[v], in[2][v]);
      return;
    }
  }
  if constexpr (NIN > 1) {
    if (src == 1) {
      PHCU_LOOP acc[v] = f(acc[v], in[1][v]);
      return;
    }
  }
  PHCU_LOOP acc[v] = f(acc[v], in[0][v]);
}

// Runs one pre-decoded instruction (fx != FX_NONE).
template <typename S, int NIN, int V>
__device__ __forceinline__ void run_fx(int fx, int src, S imm, S* acc, const S (&in)[NIN > 0 ? NIN : 1][V],
                                       uint32_t& st) {
#define PHCU_FX(ID, EXPR) \
  case ID: fx_apply<S, NIN, V>(src, imm, acc, in, [&](S a, S b) -> S { return EXPR; }); break;
  switch (fx) {
    PHCU_FX(FX_F32_LD, b)
    PHCU_FX(FX_F32_ADD, pf32<S>(sf32(a) + sf32(b)))
    PHCU_FX(FX_F32_SUB, pf32<S>(sf32(a) - sf32(b)))
    PHCU_FX(FX_F32_MUL, pf32<S>(sf32(a) * sf32(b)))
    PHCU_FX(FX_F32_DIV, pf32<S>(sf32(a) / sf32(b)))
    PHCU_FX(FX_F32_RSUB, pf32<S>(sf32(b) - sf32(a)))
    PHCU_FX(FX_F32_RDIV, pf32<S>(sf32(b) / sf32(a)))
    PHCU_FX(FX_I32_LD, b)
    PHCU_FX(FX_I32_ADD, pi32<S>(chk_add32(si32(a), si32(b), st)))
    PHCU_FX(FX_I32_SUB, pi32<S>(chk_sub32(si32(a), si32(b), st)))
    PHCU_FX(FX_I32_MUL, pi32<S>(chk_mul32(si32(a), si32(b), st)))
    PHCU_FX(FX_I32_RSUB, pi32<S>(chk_sub32(si32(b), si32(a), st)))
    PHCU_FX(FX_I32_WADD, pi32<S>((int32_t)((uint32_t)a + (uint32_t)b)))
    PHCU_FX(FX_I32_WSUB, pi32<S>((int32_t)((uint32_t)a - (uint32_t)b)))
    PHCU_FX(FX_I32_WMUL, pi32<S>((int32_t)((uint32_t)a * (uint32_t)b)))
    PHCU_FX(FX_I32_RWSUB, pi32<S>((int32_t)((uint32_t)b - (uint32_t)a)))
    PHCU_FX(FX_I32_AND, pi32<S>((int32_t)((uint32_t)a & (uint32_t)b)))
    PHCU_FX(FX_I32_OR, pi32<S>((int32_t)((uint32_t)a | (uint32_t)b)))
    PHCU_FX(FX_I32_XOR, pi32<S>((int32_t)((uint32_t)a ^ (uint32_t)b)))
  }
#undef PHCU_FX
}

// A program every instruction of which has a pre-decoded form or is
// `Float ** Int` with an immediate exponent (host check: program_is_fx).
// Kernels built for such programs compile only these two paths: no operand
// copies, conversions or type dispatch, so they need fewer registers.
// A power by an immediate integer exponent (uniform across the grid): the
// reduced interpreter runs it as binary exponentiation of its own, for Float
// (LLVM powi) and for Int32 / Int64 (checked, or wrapping for &**).
inline bool fx_power(const phcu_instr_t& I) {
  if (I.src != PHCU_SRC_IMM || (I.flags & 1) || !is_int_t(I.btype)) return false;
  if (I.op == PHCU_OP_POW) return is_float_t(I.type) || is_int_t(I.type);
  return I.op == PHCU_OP_WPOW && is_int_t(I.type);
}

inline bool program_is_fx(const phcu_program_t& P) {
  if (P.n_instr < 1) return false;
  for (int i = 0; i < P.n_instr; i++) {
    const phcu_instr_t& I = P.code[i];
    if (I.pad[0] != FX_NONE) continue;
    if (fx_power(I)) continue;
    return false;
  }
  return true;
}

template <typename S, int V>
__device__ __forceinline__ void powi_uniform(S* a, int T, int32_t e);

template <typename S, int NIN, int V>
__device__ __forceinline__ void run_program_fx(const phcu_program_t& P, const S (&in)[NIN > 0 ? NIN : 1][V],
                                               S (&acc)[V], uint32_t& st) {
  const int ni = P.n_instr;
  for (int pc = 0; pc < ni; pc++) {
    const int fx = P.code[pc].pad[0];
    if (fx != FX_NONE) {
      run_fx<S, NIN, V>(fx, P.code[pc].src, (S)(uint64_t)P.code[pc].imm.i, acc, in, st);
    } else {
      // the exponent as the general interpreter reads the immediate slot
      const phcu_instr_t& I = P.code[pc];
      const bool wrap = I.op == PHCU_OP_WPOW;
      if (I.type == PHCU_I32) {
        const int64_t e = (int32_t)(uint32_t)I.imm.i;
#pragma unroll
        for (int v = 0; v < V; v++) acc[v] = pi32<S>(int_pow<int32_t>(si32(acc[v]), e, wrap, st));
      } else if (I.type == PHCU_I64) {
        if constexpr (sizeof(S) == 8) {
          const int64_t e = (int64_t)I.imm.i;
#pragma unroll
          for (int v = 0; v < V; v++) acc[v] = (S)int_pow<int64_t>((int64_t)acc[v], e, wrap, st);
        }
      } else {
        const int64_t e = I.imm.i;
        powi_uniform<S, V>(acc, I.type, I.btype == PHCU_I32 ? (int32_t)(uint32_t)e : (int32_t)e);
      }
    }
  }
}

// ------------------------------------------------------ the interpreter
// ACC = ACC op B on V elements in the compute type T (B already of type T, or
// an integer exponent of a float power).
template <typename S, int V>
__device__ __forceinline__ void bin_dispatch(int op, int T, int bt, S* acc, const S* b, uint32_t& st) {
  switch (T) {
    case PHCU_F32: bin_f32<S, V>(op, bt, acc, b, st); break;
    case PHCU_I32: bin_i32<S, V>(op, acc, b, st); break;
    case PHCU_BOOL: bin_bool<S, V>(op, acc, b); break;
    case PHCU_F64:
      if constexpr (sizeof(S) == 8) bin_f64<V>(op, bt, acc, b, st);
      break;
    case PHCU_I64:
      if constexpr (sizeof(S) == 8) bin_i64<V>(op, acc, b, st);
      break;
  }
}

// Runs the program on V elements: in[k][v] are the loaded inputs, acc[v]
// receives the result.  STASH=false instantiations require a program without
// ST0/ST1 and without stash operands (the host checks).
template <typename S, int NIN, int V, bool STASH>
__device__ __forceinline__ void run_program(const phcu_program_t& P, const S (&in)[NIN > 0 ? NIN : 1][V], S (&acc)[V],
                                            uint32_t& st) {
  S s0[STASH ? V : 1], s1[STASH ? V : 1];
  const int ni = P.n_instr;
  for (int pc = 0; pc < ni; pc++) {
    const int fx = P.code[pc].pad[0];
    if (fx != FX_NONE) {
      run_fx<S, NIN, V>(fx, P.code[pc].src, (S)(uint64_t)P.code[pc].imm.i, acc, in, st);
      continue;
    }
    const int op = P.code[pc].op;
    const int T = P.code[pc].type;
    if constexpr (STASH) {
      if (op == PHCU_I_ST0) {
        PHCU_LOOP s0[v] = acc[v];
        continue;
      }
      if (op == PHCU_I_ST1) {
        PHCU_LOOP s1[v] = acc[v];
        continue;
      }
    }
    if (op == PHCU_I_CVT) {
      cvt_vec<S, V>(acc, T, (int)P.code[pc].imm.i);
      continue;
    }
    if (op == PHCU_I_NEG || op == PHCU_I_NOT || op == PHCU_I_POS) {
      un_vec<S, V>(op, T, acc, st);
      continue;
    }
    const int src = P.code[pc].src;
    if (op == PHCU_OP_POW && src == PHCU_SRC_IMM && is_float_t(T) && is_int_t(P.code[pc].btype) &&
        !(P.code[pc].flags & 1)) {
      const int64_t e = P.code[pc].imm.i;
      powi_uniform<S, V>(acc, T, P.code[pc].btype == PHCU_I32 ? (int32_t)(uint32_t)e : (int32_t)e);
      continue;
    }
    int bt = P.code[pc].btype;
    const bool int_exp = (op == PHCU_OP_POW) && is_float_t(T) && is_int_t(bt);
    // operand B
    S b[V];
    if (src == PHCU_SRC_IMM) {  // an immediate is converted once, then broadcast
      S imm = (S)(uint64_t)P.code[pc].imm.i;
      if (!int_exp && bt != T) {
        imm = convert_slot<S>(imm, bt, T);
        bt = T;
      }
      PHCU_LOOP b[v] = imm;
    } else if (STASH && src == PHCU_SRC_S0) {
      PHCU_LOOP b[v] = s0[v];
    } else if (STASH && src == PHCU_SRC_S1) {
      PHCU_LOOP b[v] = s1[v];
    } else {
      PHCU_LOOP b[v] = in[0][v];
      if constexpr (NIN > 1) {
        if (src == 1) { PHCU_LOOP b[v] = in[1][v]; }
      }
      if constexpr (NIN > 2) {
        if (src == 2) { PHCU_LOOP b[v] = in[2][v]; }
      }
      if constexpr (NIN > 3) {
        if (src == 3) { PHCU_LOOP b[v] = in[3][v]; }
      }
    }
    if (!int_exp && bt != T) {
      cvt_vec<S, V>(b, bt, T);
      bt = T;
    }
    if (op == PHCU_I_LD) {
      PHCU_LOOP acc[v] = b[v];
      continue;
    }
    if constexpr (STASH) {
      if (op == PHCU_I_SEL) {
        PHCU_LOOP acc[v] = (s0[v] & 1u) ? b[v] : acc[v];
        continue;
      }
    }
    if (P.code[pc].flags & 1) {  // ACC = B op ACC
      PHCU_LOOP {
        const S t = acc[v];
        acc[v] = b[v];
        b[v] = t;
      }
    }
    bin_dispatch<S, V>(op, T, bt, acc, b, st);
  }
}

#undef PHCU_LOOP

}  // namespace phcu

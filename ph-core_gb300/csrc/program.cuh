// program.cuh -- the fixed-opcode accumulator machine evaluated per element.
//
// Values live in 64-bit slots: Float32 and Int32 in the low 32 bits, Int64 and
// Float64 in all 64, Bool as 0/1.  Every instruction is uniform across the
// grid, so the switches below are uniform branches; each thread applies an
// instruction to VEC elements held in registers.  Semantics follow Crystal 1.0
// numbers (checked Int32/Int64 + - *, floor division and modulo, Int / Int ->
// Float64, Float ** Int by binary exponentiation), matching the CPU oracle.
// This translation unit is compiled with -fmad=false: no FMA contraction, so
// every Float32 operation rounds once, as on the host.
#pragma once

#include "common.cuh"

namespace phcu {

__device__ __forceinline__ float sf32(uint64_t s) { return __uint_as_float((uint32_t)s); }
__device__ __forceinline__ uint64_t pf32(float f) { return (uint64_t)__float_as_uint(f); }
__device__ __forceinline__ double sf64(uint64_t s) { return __longlong_as_double((long long)s); }
__device__ __forceinline__ uint64_t pf64(double f) { return (uint64_t)__double_as_longlong(f); }
__device__ __forceinline__ int32_t si32(uint64_t s) { return (int32_t)(uint32_t)s; }
__device__ __forceinline__ uint64_t pi32(int32_t v) { return (uint64_t)(uint32_t)v; }
__device__ __forceinline__ int64_t si64(uint64_t s) { return (int64_t)s; }
__device__ __forceinline__ uint64_t pi64(int64_t v) { return (uint64_t)v; }

// ---------------------------------------------------------------- loads
template <int VEC>
__device__ __forceinline__ void load_scalar(const char* p, int64_t stride_bytes, int dtype,
                                            uint64_t (&v)[VEC]) {
#pragma unroll
  for (int i = 0; i < VEC; i++) {
    const char* q = p + i * stride_bytes;
    switch (dtype) {
      case PHCU_BOOL: v[i] = (*(const uint8_t*)q) ? 1u : 0u; break;
      case PHCU_I32:
      case PHCU_F32: v[i] = (uint64_t)__ldg((const uint32_t*)q); break;
      default: v[i] = (uint64_t)__ldg((const unsigned long long*)q); break;
    }
  }
}

// VEC consecutive elements starting at p (aligned to min(16, VEC*es) bytes).
template <int VEC>
__device__ __forceinline__ void load_vec(const char* p, int dtype, uint64_t (&v)[VEC]) {
  const int es = dtype_size(dtype);
  if (es == 4) {
    if constexpr (VEC == 4) {
      uint4 x = __ldg((const uint4*)p);
      v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else if constexpr (VEC == 2) {
      uint2 x = __ldg((const uint2*)p);
      v[0] = x.x; v[1] = x.y;
    } else {
      v[0] = __ldg((const uint32_t*)p);
    }
  } else if (es == 8) {
    if constexpr (VEC == 4) {
      ulonglong2 x = __ldg((const ulonglong2*)p);
      ulonglong2 y = __ldg((const ulonglong2*)(p + 16));
      v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
    } else if constexpr (VEC == 2) {
      ulonglong2 x = __ldg((const ulonglong2*)p);
      v[0] = x.x; v[1] = x.y;
    } else {
      v[0] = __ldg((const unsigned long long*)p);
    }
  } else {  // bool
#pragma unroll
    for (int i = 0; i < VEC; i++) v[i] = p[i] ? 1u : 0u;
  }
}

template <int VEC>
__device__ __forceinline__ void store_scalar(char* p, int64_t stride_bytes, int dtype,
                                             const uint64_t (&v)[VEC]) {
#pragma unroll
  for (int i = 0; i < VEC; i++) {
    char* q = p + i * stride_bytes;
    switch (dtype) {
      case PHCU_BOOL: *(uint8_t*)q = (uint8_t)(v[i] & 1u); break;
      case PHCU_I32:
      case PHCU_F32: *(uint32_t*)q = (uint32_t)v[i]; break;
      default: *(unsigned long long*)q = (unsigned long long)v[i]; break;
    }
  }
}

template <int VEC>
__device__ __forceinline__ void store_vec(char* p, int dtype, const uint64_t (&v)[VEC]) {
  const int es = dtype_size(dtype);
  if (es == 4) {
    if constexpr (VEC == 4) {
      *(uint4*)p = make_uint4((uint32_t)v[0], (uint32_t)v[1], (uint32_t)v[2], (uint32_t)v[3]);
    } else if constexpr (VEC == 2) {
      *(uint2*)p = make_uint2((uint32_t)v[0], (uint32_t)v[1]);
    } else {
      *(uint32_t*)p = (uint32_t)v[0];
    }
  } else if (es == 8) {
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

// Loads VEC elements of one operand in the given vector mode.
template <int VEC>
__device__ __forceinline__ void load_operand(const char* p, int64_t inner_stride, int dtype, int vmode,
                                             uint64_t (&v)[VEC]) {
  const int es = dtype_size(dtype);
  if (vmode == VM_VEC) {
    load_vec<VEC>(p, dtype, v);
  } else if (vmode == VM_VEC_REV) {
    uint64_t t[VEC];
    load_vec<VEC>(p - (VEC - 1) * es, dtype, t);
#pragma unroll
    for (int i = 0; i < VEC; i++) v[i] = t[VEC - 1 - i];
  } else {
    load_scalar<VEC>(p, inner_stride * es, dtype, v);
  }
}

// -------------------------------------------------------- conversions
__device__ __forceinline__ uint64_t convert_slot(uint64_t s, int from, int to) {
  if (from == to) return s;
  switch (from) {
    case PHCU_BOOL:
    case PHCU_I32: {
      int64_t x = (from == PHCU_BOOL) ? (int64_t)(s & 1u) : (int64_t)si32(s);
      switch (to) {
        case PHCU_I32: return pi32((int32_t)x);
        case PHCU_I64: return pi64(x);
        case PHCU_F32: return pf32((float)x);
        case PHCU_F64: return pf64((double)x);
        case PHCU_BOOL: return x != 0;
      }
      break;
    }
    case PHCU_I64: {
      int64_t x = si64(s);
      switch (to) {
        case PHCU_I32: return pi32((int32_t)x);
        case PHCU_F32: return pf32((float)x);
        case PHCU_F64: return pf64((double)x);
        case PHCU_BOOL: return x != 0;
      }
      break;
    }
    case PHCU_F32: {
      float x = sf32(s);
      switch (to) {
        case PHCU_F64: return pf64((double)x);
        case PHCU_I32: return pi32((int32_t)x);
        case PHCU_I64: return pi64((int64_t)x);
        case PHCU_BOOL: return x != 0.0f;
      }
      break;
    }
    case PHCU_F64: {
      double x = sf64(s);
      switch (to) {
        case PHCU_F32: return pf32((float)x);
        case PHCU_I32: return pi32((int32_t)x);
        case PHCU_I64: return pi64((int64_t)x);
        case PHCU_BOOL: return x != 0.0;
      }
      break;
    }
  }
  return s;
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

template <typename I>
__device__ __forceinline__ I wrap_mul(I a, I b) {
  using U = typename std::conditional<sizeof(I) == 4, uint32_t, uint64_t>::type;
  return (I)((U)a * (U)b);
}

__device__ __forceinline__ int32_t chk_add32(int32_t a, int32_t b, uint32_t& st) {
  int64_t r = (int64_t)a + b;
  if (r != (int32_t)r) st |= PHCU_ST_OVERFLOW;
  return (int32_t)(uint32_t)(uint64_t)r;
}
__device__ __forceinline__ int32_t chk_sub32(int32_t a, int32_t b, uint32_t& st) {
  int64_t r = (int64_t)a - b;
  if (r != (int32_t)r) st |= PHCU_ST_OVERFLOW;
  return (int32_t)(uint32_t)(uint64_t)r;
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
  int64_t hi = __mul64hi(a, b);
  if (hi != (r >> 63)) st |= PHCU_ST_OVERFLOW;
  return r;
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
      else if (sizeof(I) == 4) result = (I)chk_mul32((int32_t)result, (int32_t)k, st);
      else result = (I)chk_mul64((int64_t)result, (int64_t)k, st);
    }
    e >>= 1;
    if (e > 0) {
      if (wrapping) k = wrap_mul<I>(k, k);
      else if (sizeof(I) == 4) k = (I)chk_mul32((int32_t)k, (int32_t)k, st);
      else k = (I)chk_mul64((int64_t)k, (int64_t)k, st);
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

// ------------------------------------------------ one binary operation
// a OP b in compute type T; b already converted to T unless op is POW with
// an integer exponent (bt = the exponent's type).
__device__ __forceinline__ uint64_t bin_op(int op, int T, int bt, uint64_t a, uint64_t b, uint32_t& st) {
  switch (T) {
    case PHCU_F32: {
      float x = sf32(a);
      if (op == PHCU_OP_POW && is_int_t(bt)) {
        int32_t e = (bt == PHCU_I32) ? si32(b) : (int32_t)si64(b);
        return pf32(powi<float>(x, e));
      }
      float y = sf32(b);
      switch (op) {
        case PHCU_OP_ADD: return pf32(x + y);
        case PHCU_OP_SUB: return pf32(x - y);
        case PHCU_OP_MUL: return pf32(x * y);
        case PHCU_OP_DIV: return pf32(x / y);
        case PHCU_OP_FLOORDIV: return pf32(floorf(x / y));
        case PHCU_OP_MOD: {
          if (y == 0.0f) { st |= PHCU_ST_DIVZERO; return pf32(0.0f); }
          float q = floorf(x / y);
          float mm = y * q;
          return pf32(x - mm);
        }
        case PHCU_OP_POW: return pf32(powf(x, y));
        case PHCU_OP_GT: return x > y;
        case PHCU_OP_LT: return x < y;
        case PHCU_OP_GE: return x >= y;
        case PHCU_OP_LE: return x <= y;
        case PHCU_OP_EQ: return x == y;
        case PHCU_OP_CMP: return pi32((x > y) - (x < y));
      }
      return 0;
    }
    case PHCU_F64: {
      double x = sf64(a);
      if (op == PHCU_OP_POW && is_int_t(bt)) {
        int32_t e = (bt == PHCU_I32) ? si32(b) : (int32_t)si64(b);
        return pf64(powi<double>(x, e));
      }
      double y = sf64(b);
      switch (op) {
        case PHCU_OP_ADD: return pf64(x + y);
        case PHCU_OP_SUB: return pf64(x - y);
        case PHCU_OP_MUL: return pf64(x * y);
        case PHCU_OP_DIV: return pf64(x / y);
        case PHCU_OP_FLOORDIV: return pf64(floor(x / y));
        case PHCU_OP_MOD: {
          if (y == 0.0) { st |= PHCU_ST_DIVZERO; return pf64(0.0); }
          double q = floor(x / y);
          double mm = y * q;
          return pf64(x - mm);
        }
        case PHCU_OP_POW: return pf64(pow(x, y));
        case PHCU_OP_GT: return x > y;
        case PHCU_OP_LT: return x < y;
        case PHCU_OP_GE: return x >= y;
        case PHCU_OP_LE: return x <= y;
        case PHCU_OP_EQ: return x == y;
        case PHCU_OP_CMP: return pi32((x > y) - (x < y));
      }
      return 0;
    }
    case PHCU_I32: {
      int32_t x = si32(a), y = si32(b);
      switch (op) {
        case PHCU_OP_ADD: return pi32(chk_add32(x, y, st));
        case PHCU_OP_SUB: return pi32(chk_sub32(x, y, st));
        case PHCU_OP_MUL: return pi32(chk_mul32(x, y, st));
        case PHCU_OP_DIV: return pf64((double)x / (double)y);
        case PHCU_OP_FLOORDIV:
          if (y == 0) { st |= PHCU_ST_DIVZERO; return 0; }
          if (x == INT32_MIN && y == -1) { st |= PHCU_ST_OVERFLOW; return pi32(x); }
          return pi32((int32_t)floordiv_i64(x, y));
        case PHCU_OP_MOD:
          if (y == 0) { st |= PHCU_ST_DIVZERO; return 0; }
          if (y == -1) return 0;
          return pi32((int32_t)floormod_i64(x, y));
        case PHCU_OP_POW: return pi32(int_pow<int32_t>(x, y, false, st));
        case PHCU_OP_WADD: return pi32((int32_t)((uint32_t)x + (uint32_t)y));
        case PHCU_OP_WSUB: return pi32((int32_t)((uint32_t)x - (uint32_t)y));
        case PHCU_OP_WMUL: return pi32(wrap_mul<int32_t>(x, y));
        case PHCU_OP_WPOW: return pi32(int_pow<int32_t>(x, y, true, st));
        case PHCU_OP_AND: return pi32(x & y);
        case PHCU_OP_OR: return pi32(x | y);
        case PHCU_OP_XOR: return pi32(x ^ y);
        case PHCU_OP_GT: return x > y;
        case PHCU_OP_LT: return x < y;
        case PHCU_OP_GE: return x >= y;
        case PHCU_OP_LE: return x <= y;
        case PHCU_OP_EQ: return x == y;
        case PHCU_OP_CMP: return pi32((x > y) - (x < y));
      }
      return 0;
    }
    case PHCU_I64: {
      int64_t x = si64(a), y = si64(b);
      switch (op) {
        case PHCU_OP_ADD: return pi64(chk_add64(x, y, st));
        case PHCU_OP_SUB: return pi64(chk_sub64(x, y, st));
        case PHCU_OP_MUL: return pi64(chk_mul64(x, y, st));
        case PHCU_OP_DIV: return pf64((double)x / (double)y);
        case PHCU_OP_FLOORDIV:
          if (y == 0) { st |= PHCU_ST_DIVZERO; return 0; }
          if (x == INT64_MIN && y == -1) { st |= PHCU_ST_OVERFLOW; return pi64(x); }
          return pi64(floordiv_i64(x, y));
        case PHCU_OP_MOD:
          if (y == 0) { st |= PHCU_ST_DIVZERO; return 0; }
          if (y == -1) return 0;
          return pi64(floormod_i64(x, y));
        case PHCU_OP_POW: return pi64(int_pow<int64_t>(x, y, false, st));
        case PHCU_OP_WADD: return pi64((int64_t)((uint64_t)x + (uint64_t)y));
        case PHCU_OP_WSUB: return pi64((int64_t)((uint64_t)x - (uint64_t)y));
        case PHCU_OP_WMUL: return pi64(wrap_mul<int64_t>(x, y));
        case PHCU_OP_WPOW: return pi64(int_pow<int64_t>(x, y, true, st));
        case PHCU_OP_AND: return pi64(x & y);
        case PHCU_OP_OR: return pi64(x | y);
        case PHCU_OP_XOR: return pi64(x ^ y);
        case PHCU_OP_GT: return x > y;
        case PHCU_OP_LT: return x < y;
        case PHCU_OP_GE: return x >= y;
        case PHCU_OP_LE: return x <= y;
        case PHCU_OP_EQ: return x == y;
        case PHCU_OP_CMP: return pi32((x > y) - (x < y));
      }
      return 0;
    }
    case PHCU_BOOL: {
      uint64_t x = a & 1u, y = b & 1u;
      switch (op) {
        case PHCU_OP_AND: return x & y;
        case PHCU_OP_OR: return x | y;
        case PHCU_OP_XOR: return x ^ y;
        case PHCU_OP_EQ: return x == y;
      }
      return 0;
    }
  }
  return 0;
}

__device__ __forceinline__ uint64_t un_op(int op, int T, uint64_t a, uint32_t& st) {
  switch (op) {
    case PHCU_I_POS: return a;
    case PHCU_I_NEG:
      switch (T) {
        case PHCU_F32: return pf32(-sf32(a));
        case PHCU_F64: return pf64(-sf64(a));
        case PHCU_I32: {
          int32_t x = si32(a);
          if (x == INT32_MIN) { st |= PHCU_ST_OVERFLOW; return a; }
          return pi32(-x);
        }
        case PHCU_I64: {
          int64_t x = si64(a);
          if (x == INT64_MIN) { st |= PHCU_ST_OVERFLOW; return a; }
          return pi64(-x);
        }
      }
      return a;
    case PHCU_I_NOT:
      if (T == PHCU_I32) return pi32(~si32(a));
      if (T == PHCU_I64) return pi64(~si64(a));
      return a;
  }
  return a;
}

// ------------------------------------------------------ the interpreter
template <int NIN, int VEC>
__device__ __forceinline__ void run_program(const phcu_program_t& P, const uint64_t (&in)[NIN > 0 ? NIN : 1][VEC],
                                            uint64_t (&acc)[VEC], uint32_t& st) {
  uint64_t s0[VEC], s1[VEC];
#pragma unroll
  for (int v = 0; v < VEC; v++) { acc[v] = 0; s0[v] = 0; s1[v] = 0; }
  const int ni = P.n_instr;
  for (int pc = 0; pc < ni; pc++) {
    const phcu_instr_t& I = P.code[pc];
    const int op = I.op;
    if (op == PHCU_I_ST0) {
#pragma unroll
      for (int v = 0; v < VEC; v++) s0[v] = acc[v];
      continue;
    }
    if (op == PHCU_I_ST1) {
#pragma unroll
      for (int v = 0; v < VEC; v++) s1[v] = acc[v];
      continue;
    }
    if (op == PHCU_I_CVT) {
      const int to = (int)I.imm.i;
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] = convert_slot(acc[v], I.type, to);
      continue;
    }
    if (op == PHCU_I_NEG || op == PHCU_I_NOT || op == PHCU_I_POS) {
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] = un_op(op, I.type, acc[v], st);
      continue;
    }
    // operand B
    uint64_t b[VEC];
    switch (I.src) {
      case PHCU_SRC_IMM: {
        const uint64_t imm = (uint64_t)I.imm.i;
#pragma unroll
        for (int v = 0; v < VEC; v++) b[v] = imm;
        break;
      }
      case PHCU_SRC_S0:
#pragma unroll
        for (int v = 0; v < VEC; v++) b[v] = s0[v];
        break;
      case PHCU_SRC_S1:
#pragma unroll
        for (int v = 0; v < VEC; v++) b[v] = s1[v];
        break;
      default: {
        const int k = I.src;
#pragma unroll
        for (int v = 0; v < VEC; v++) b[v] = in[0][v];
        if constexpr (NIN > 1) {
          if (k == 1) {
#pragma unroll
            for (int v = 0; v < VEC; v++) b[v] = in[1][v];
          }
        }
        if constexpr (NIN > 2) {
          if (k == 2) {
#pragma unroll
            for (int v = 0; v < VEC; v++) b[v] = in[2][v];
          }
        }
        if constexpr (NIN > 3) {
          if (k == 3) {
#pragma unroll
            for (int v = 0; v < VEC; v++) b[v] = in[3][v];
          }
        }
        break;
      }
    }
    if (op == PHCU_I_LD) {
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] = convert_slot(b[v], I.btype, I.type);
      continue;
    }
    const int T = I.type;
    int bt = I.btype;
    const bool int_exp = (op == PHCU_OP_POW) && is_float_t(T) && is_int_t(bt);
    if (!int_exp && bt != T) {
#pragma unroll
      for (int v = 0; v < VEC; v++) b[v] = convert_slot(b[v], bt, T);
      bt = T;
    }
    if (I.flags & 1) {
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] = bin_op(op, T, bt, b[v], acc[v], st);
    } else {
#pragma unroll
      for (int v = 0; v < VEC; v++) acc[v] = bin_op(op, T, bt, acc[v], b[v], st);
    }
  }
}

}  // namespace phcu

// eval.cu -- strided gather/scatter and fused elementwise entry points.
//
// One kernel family serves copies (the empty program), fills (no inputs),
// single infix operators and whole fused chains.  Two launch shapes:
//
//  ROW  -- the output and every input share the innermost canonical axis.
//          Each thread handles several chunks of VEC consecutive elements;
//          operands with unit (or reversed unit) inner stride use 128-bit
//          accesses.
//  TILE -- the output is contiguous along axis W while (some) inputs are
//          contiguous along another axis R (permuted views).  A 64x64 tile of
//          each such input is read coalesced along R into shared memory, then
//          read back transposed so the output is written coalesced along W.
// Kernels are instantiated in eval_inst_*.cu; this file plans and dispatches.
#include "eval_kernels.cuh"

#include <cudaTypedefs.h>

#include <cstdlib>

namespace phcu {

int32_t launch_eval_u32_lo(const EvalArgs& A);
int32_t launch_eval_u32_hi(const EvalArgs& A);
int32_t launch_eval_u64_lo(const EvalArgs& A);
int32_t launch_eval_u64_hi(const EvalArgs& A);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda); null when unavailable or when PHCU_TILE_TMA=0 selects the
// register/cp.async staged tile path.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    const char* env = std::getenv("PHCU_TILE_TMA");
    if (env && std::atoi(env) == 0) return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }
    return (PFN_cuTensorMapEncodeTiled_v12000)f;
  }();
  return fn;
}

// Describes every staged input of a TILE plan as a tensor map over the plan's
// axes [R, W, batch axes in order].  A batch axis the input walks backwards
// is described forwards from its last element, with its coordinate mirrored
// in the kernel.  False (the staged tile path is used) unless each staged
// input has 4-byte elements, unit stride along R, a positive stride along W,
// strides that are multiples of 16 bytes, a 16-byte aligned first address,
// and the plan has at most 5 axes.
static bool encode_tile_maps(const EvalPlan& p, TmaMaps* m) {
  if (p.mode != MODE_TILE || p.sp.rank < 2 || p.sp.rank > 5 || p.staged == 0) return false;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const int W = p.sp.rank - 1, R = p.raxis;
  int s = 0;
  for (int k = 0; k < p.nin; k++) {
    if (!(p.staged & (1u << k))) continue;
    const Operand& o = p.in[k];
    if (dtype_size(o.dtype) != 4 || o.stride[R] != 1 || o.stride[W] <= 0) return false;
    const char* first = o.base;
    uint32_t flip = 0;
    cuuint64_t dims[5], strides[4];
    cuuint32_t box[5], estr[5] = {1, 1, 1, 1, 1};
    dims[0] = (cuuint64_t)p.sp.shape[R];
    box[0] = TMA_BOX_R;
    m->ext[0] = (int32_t)p.sp.shape[R];
    int d = 1;
    auto add_axis = [&](int a, cuuint32_t b) {
      int64_t sb = o.stride[a] * 4;
      if (sb < 0) {  // walk it forwards from its last element
        first += (p.sp.shape[a] - 1) * sb;
        sb = -sb;
        flip |= 1u << d;
      }
      if (sb == 0 || (sb & 15) != 0 || sb >= ((int64_t)1 << 40)) return false;
      dims[d] = (cuuint64_t)p.sp.shape[a];
      strides[d - 1] = (cuuint64_t)sb;
      box[d] = b;
      m->ext[d] = (int32_t)p.sp.shape[a];
      d++;
      return true;
    };
    if (!add_axis(W, TILE)) return false;
    for (int a = 0; a < W; a++)
      if (a != R && !add_axis(a, 1)) return false;
    if (((uintptr_t)first & 15u) != 0) return false;
    const CUresult r = enc(&m->map[s], CU_TENSOR_MAP_DATA_TYPE_UINT32, (cuuint32_t)d, (void*)first, dims, strides,
                           box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    m->ndim = d;
    m->flip[s] = flip;
    s++;
  }
  return s > 0;
}

int32_t launch_eval(const EvalArgs& A0) {
  if (A0.plan.nin < 0 || A0.plan.nin > MAXIN) return fail(PHCU_ERR_INVALID, "too many inputs (%d)", A0.plan.nin);
  EvalArgs A = A0;
  predecode_program(&A.prog);
  TmaMaps maps;
  A.tma = encode_tile_maps(A.plan, &maps) ? &maps : nullptr;
  const bool narrow = program_is_32bit(A.prog, A.plan);
  if (narrow) return A.plan.nin <= 2 ? launch_eval_u32_lo(A) : launch_eval_u32_hi(A);
  return A.plan.nin <= 2 ? launch_eval_u64_lo(A) : launch_eval_u64_hi(A);
}
// Launches an already planned operation (used by the batched executor's per-op replay).
int32_t launch_eval_plan(const EvalPlan& plan, const phcu_program_t& prog) {
  EvalArgs A;
  A.plan = plan;
  A.prog = prog;
  A.status = ctx().status;
  return launch_eval(A);
}

// ------------------------------------------------------- program checks
int32_t check_program(const phcu_program_t* prog, int nin) {
  if (!prog) return fail(PHCU_ERR_INVALID, "null program");
  if (prog->n_instr < 0 || prog->n_instr > PHCU_MAX_INSTR)
    return fail(PHCU_ERR_INVALID, "program length %d outside 0..%d", prog->n_instr, PHCU_MAX_INSTR);
  for (int i = 0; i < prog->n_instr; i++) {
    const phcu_instr_t& I = prog->code[i];
    if (!dtype_valid(I.type)) return fail(PHCU_ERR_INVALID, "instruction %d: bad type %d", i, I.type);
    bool needs_b = !(I.op == PHCU_I_ST0 || I.op == PHCU_I_ST1 || I.op == PHCU_I_CVT || I.op == PHCU_I_NEG ||
                     I.op == PHCU_I_NOT || I.op == PHCU_I_POS);
    if (needs_b) {
      if (!(I.src < nin || I.src == PHCU_SRC_IMM || I.src == PHCU_SRC_S0 || I.src == PHCU_SRC_S1))
        return fail(PHCU_ERR_INVALID, "instruction %d: operand source %d not available", i, I.src);
      if (!dtype_valid(I.btype)) return fail(PHCU_ERR_INVALID, "instruction %d: bad operand type", i);
    }
    if (!(I.op < PHCU_OP_NBINARY || (I.op >= PHCU_I_LD && I.op <= PHCU_I_SEL)))
      return fail(PHCU_ERR_INVALID, "instruction %d: unknown opcode %d", i, I.op);
    if (I.op == PHCU_I_CVT && !dtype_valid((int)I.imm.i))
      return fail(PHCU_ERR_INVALID, "instruction %d: bad conversion target", i);
  }
  return PHCU_OK;
}

// Evaluates with inputs that may overlap the output: an input that overlaps
// the output with a different mapping is first copied to a temporary.  Every
// argument is checked before the context is asked for, so argument errors
// come back the same with or without a device.
int32_t eval_views(const phcu_program_t* prog, const phcu_view_t* inputs, int nin, const phcu_view_t* out,
                   int force_mode = -1) {
  PHCU_TRY(check_view(out, "output"));
  if (nin < 0 || nin > MAXIN) return fail(PHCU_ERR_INVALID, "n_inputs %d outside 0..%d", nin, MAXIN);
  if (nin > 0 && !inputs) return fail(PHCU_ERR_INVALID, "null input array");
  for (int k = 0; k < nin; k++) PHCU_TRY(check_input_view(&inputs[k], "input"));
  PHCU_TRY(check_program(prog, nin));
  if (prog->out_type != out->dtype)
    return fail(PHCU_ERR_INVALID, "program result type %d differs from output dtype %d", prog->out_type, out->dtype);
  PHCU_TRY(require_ctx());

  phcu_view_t staged[MAXIN];
  void* temps[MAXIN] = {nullptr};
  const phcu_view_t* ins[MAXIN];
  int32_t rc = PHCU_OK;
  for (int k = 0; k < nin; k++) ins[k] = &inputs[k];
  for (int k = 0; k < nin && rc == PHCU_OK; k++) {
    if (views_overlap(&inputs[k], out) && !views_identical(&inputs[k], out)) {
      // materialise this input first (lexicographic, contiguous)
      const phcu_view_t& v = inputs[k];
      int64_t n = view_size(&v);
      rc = scratch_alloc((size_t)n * dtype_size(v.dtype), &temps[k]);
      if (rc != PHCU_OK) break;
      phcu_view_t t;
      memset(&t, 0, sizeof(t));
      t.base = temps[k];
      t.dtype = v.dtype;
      t.rank = v.rank;
      int64_t s = 1;
      for (int i = v.rank - 1; i >= 0; i--) {
        t.shape[i] = v.shape[i];
        t.stride[i] = s;
        s *= v.shape[i];
      }
      EvalArgs C;
      phcu_program_t cp;
      memset(&cp, 0, sizeof(cp));
      cp.n_instr = 1;
      cp.out_type = v.dtype;
      cp.code[0].op = PHCU_I_LD;
      cp.code[0].src = 0;
      cp.code[0].type = (uint8_t)v.dtype;
      cp.code[0].btype = (uint8_t)v.dtype;
      const phcu_view_t* one[1] = {&v};
      rc = make_plan(&t, one, 1, &C.plan);
      C.prog = cp;
      C.status = ctx().status;
      if (rc == PHCU_OK && C.plan.mode != MODE_EMPTY) rc = launch_eval(C);
      staged[k] = t;
      ins[k] = &staged[k];
    }
  }
  if (rc == PHCU_OK) {
    EvalArgs A;
    rc = make_plan(out, ins, nin, &A.plan, force_mode);
    if (rc == PHCU_OK && A.plan.mode != MODE_EMPTY) {
      A.prog = *prog;
      A.status = ctx().status;
      rc = launch_eval(A);
    }
  }
  for (int k = 0; k < nin; k++) scratch_free(temps[k]);  // stream-ordered after the launches
  return rc;
}

// ------------------------------------------------ Crystal result types
int32_t result_dtype(int op, int ta, int tb, int* tout) {
  if (ta == PHCU_BOOL || tb == PHCU_BOOL) {
    if (op == PHCU_OP_EQ) { *tout = PHCU_BOOL; return PHCU_OK; }
    if (ta == PHCU_BOOL && tb == PHCU_BOOL && (op == PHCU_OP_AND || op == PHCU_OP_OR || op == PHCU_OP_XOR)) {
      *tout = PHCU_BOOL;
      return PHCU_OK;
    }
    return fail(PHCU_ERR_UNSUPPORTED, "operator %d is not defined for Bool operands", op);
  }
  if (op == PHCU_OP_GT || op == PHCU_OP_LT || op == PHCU_OP_GE || op == PHCU_OP_LE || op == PHCU_OP_EQ) {
    *tout = PHCU_BOOL;
    return PHCU_OK;
  }
  if (op == PHCU_OP_CMP) { *tout = PHCU_I32; return PHCU_OK; }
  if (op == PHCU_OP_AND || op == PHCU_OP_OR || op == PHCU_OP_XOR) {
    if (!is_int_t(ta) || !is_int_t(tb)) return fail(PHCU_ERR_UNSUPPORTED, "bitwise operator on a float operand");
    *tout = ta;
    return PHCU_OK;
  }
  if (is_int_t(ta) && is_int_t(tb)) {
    *tout = (op == PHCU_OP_DIV) ? PHCU_F64 : ta;
    return PHCU_OK;
  }
  if (op == PHCU_OP_WADD || op == PHCU_OP_WSUB || op == PHCU_OP_WMUL || op == PHCU_OP_WPOW)
    return fail(PHCU_ERR_UNSUPPORTED, "wrapping operator on a float operand");
  if (is_int_t(ta) && is_float_t(tb) && op == PHCU_OP_POW) { *tout = PHCU_F64; return PHCU_OK; }
  *tout = (ta == PHCU_F64 || tb == PHCU_F64) ? PHCU_F64 : PHCU_F32;
  return PHCU_OK;
}

// compute type of `a op b` before the result conversion
static int compute_type(int op, int ta, int tb) {
  if (ta == PHCU_BOOL && tb == PHCU_BOOL) return PHCU_BOOL;
  if (is_int_t(ta) && is_int_t(tb)) return ta;
  if (is_int_t(ta) && is_float_t(tb) && op == PHCU_OP_POW) return PHCU_F64;
  return (ta == PHCU_F64 || tb == PHCU_F64) ? PHCU_F64 : PHCU_F32;
}

// Builds the one-operator program ACC = IN0 op B.
static int32_t binary_program(int op, int ta, int tb, int src_b, const phcu_scalar_t* imm, int scalar_left,
                              phcu_program_t* P) {
  int tout;
  PHCU_TRY(result_dtype(op, ta, tb, &tout));
  memset(P, 0, sizeof(*P));
  if (ta == PHCU_BOOL || tb == PHCU_BOOL) {
    if (!(ta == PHCU_BOOL && tb == PHCU_BOOL)) {
      // Bool == number is always false (different types)
      P->n_instr = 1;
      P->code[0].op = PHCU_I_LD;
      P->code[0].src = PHCU_SRC_IMM;
      P->code[0].type = PHCU_BOOL;
      P->code[0].btype = PHCU_BOOL;
      P->code[0].imm.i = 0;
      P->out_type = PHCU_BOOL;
      return PHCU_OK;
    }
  }
  int T = compute_type(op, ta, tb);
  if (op == PHCU_OP_POW && is_float_t(ta) && is_int_t(tb)) T = ta;  // powi keeps the base type
  int n = 0;
  // ACC = IN0 (converted to T unless it is an integer exponent of a float base)
  auto slot_of = [](const phcu_scalar_t* s) -> int64_t {
    switch (s->dtype) {
      case PHCU_F32: { float f = (float)s->v.f; uint32_t u; memcpy(&u, &f, 4); return (int64_t)u; }
      case PHCU_F64: { int64_t u; memcpy(&u, &s->v.f, 8); return u; }
      case PHCU_I32: return (int64_t)(uint32_t)(int32_t)s->v.i;
      case PHCU_BOOL: return s->v.i ? 1 : 0;
      default: return s->v.i;
    }
  };
  if (scalar_left) {
    // scalar op IN0: ACC = scalar, B = IN0
    if (op == PHCU_OP_POW && is_float_t(ta) && is_int_t(tb)) {
      // float scalar ** int array: powi(scalar, x)
      phcu_instr_t& a = P->code[n++];
      a.op = PHCU_I_LD; a.src = 0; a.type = (uint8_t)tb; a.btype = (uint8_t)tb;
      phcu_instr_t& s0 = P->code[n++];
      s0.op = PHCU_I_ST0; s0.type = (uint8_t)tb;
      phcu_instr_t& l = P->code[n++];
      l.op = PHCU_I_LD; l.src = PHCU_SRC_IMM; l.type = (uint8_t)T; l.btype = (uint8_t)ta; l.imm.i = slot_of(imm);
      phcu_instr_t& pw = P->code[n++];
      pw.op = PHCU_OP_POW; pw.src = PHCU_SRC_S0; pw.type = (uint8_t)T; pw.btype = (uint8_t)tb;
    } else {
      phcu_instr_t& l = P->code[n++];
      l.op = PHCU_I_LD; l.src = PHCU_SRC_IMM; l.type = (uint8_t)T; l.btype = (uint8_t)ta; l.imm.i = slot_of(imm);
      phcu_instr_t& o = P->code[n++];
      o.op = (uint8_t)op; o.src = 0; o.type = (uint8_t)T; o.btype = (uint8_t)tb;
    }
  } else {
    phcu_instr_t& l = P->code[n++];
    l.op = PHCU_I_LD; l.src = 0; l.type = (uint8_t)T; l.btype = (uint8_t)ta;
    phcu_instr_t& o = P->code[n++];
    o.op = (uint8_t)op;
    o.src = (uint8_t)src_b;
    o.type = (uint8_t)T;
    o.btype = (uint8_t)tb;
    if (src_b == PHCU_SRC_IMM) o.imm.i = slot_of(imm);
  }
  // result type of the operator in T
  int rt = T;
  if (op == PHCU_OP_GT || op == PHCU_OP_LT || op == PHCU_OP_GE || op == PHCU_OP_LE || op == PHCU_OP_EQ) rt = PHCU_BOOL;
  else if (op == PHCU_OP_CMP) rt = PHCU_I32;
  else if (op == PHCU_OP_DIV && is_int_t(T)) rt = PHCU_F64;
  if (rt != tout) {
    phcu_instr_t& c = P->code[n++];
    c.op = PHCU_I_CVT; c.type = (uint8_t)rt; c.imm.i = tout;
  }
  P->n_instr = n;
  P->out_type = tout;
  return PHCU_OK;
}

}  // namespace phcu

using namespace phcu;

extern "C" {

int32_t phcu_result_dtype(int32_t op, int32_t ta, int32_t tb, int32_t* tout) {
  int t;
  PHCU_TRY(result_dtype(op, ta, tb, &t));
  *tout = t;
  return PHCU_OK;
}

int32_t phcu_copy(const phcu_view_t* dst, const phcu_view_t* src) {
  PHCU_TRY(check_view(dst, "dst"));
  PHCU_TRY(check_view(src, "src"));
  if (dst->dtype != src->dtype)
    return fail(PHCU_ERR_INVALID, "phcu_copy: dtype %d -> %d (copies do not convert)", src->dtype, dst->dtype);
  if (view_size(dst) != view_size(src))
    return fail(PHCU_ERR_SHAPE, "phcu_copy: source has %lld elements, destination %lld", (long long)view_size(src),
                (long long)view_size(dst));
  phcu_program_t P;
  memset(&P, 0, sizeof(P));
  P.n_instr = 1;
  P.out_type = dst->dtype;
  P.code[0].op = PHCU_I_LD;
  P.code[0].src = 0;
  P.code[0].type = (uint8_t)dst->dtype;
  P.code[0].btype = (uint8_t)dst->dtype;
  return eval_views(&P, src, 1, dst);
}

int32_t phcu_fill(const phcu_view_t* dst, const phcu_scalar_t* value) {
  PHCU_TRY(check_view(dst, "dst"));
  if (!value) return fail(PHCU_ERR_INVALID, "phcu_fill: null value");
  phcu_program_t P;
  memset(&P, 0, sizeof(P));
  P.n_instr = 1;
  P.out_type = dst->dtype;
  phcu_instr_t& I = P.code[0];
  I.op = PHCU_I_LD;
  I.src = PHCU_SRC_IMM;
  I.type = (uint8_t)dst->dtype;
  I.btype = (uint8_t)value->dtype;
  switch (value->dtype) {
    case PHCU_F32: { float f = (float)value->v.f; uint32_t u; memcpy(&u, &f, 4); I.imm.i = u; break; }
    case PHCU_F64: memcpy(&I.imm.i, &value->v.f, 8); break;
    case PHCU_I32: I.imm.i = (int64_t)(uint32_t)(int32_t)value->v.i; break;
    case PHCU_BOOL: I.imm.i = value->v.i ? 1 : 0; break;
    default: I.imm.i = value->v.i;
  }
  return eval_views(&P, nullptr, 0, dst);
}

int32_t phcu_eval(const phcu_program_t* prog, const phcu_view_t* inputs, int32_t n_inputs, const phcu_view_t* out) {
  return eval_views(prog, inputs, n_inputs, out);
}

int32_t phcu_binary(int32_t op, const phcu_view_t* a, const phcu_view_t* b, const phcu_view_t* out) {
  PHCU_TRY(require_ctx());
  PHCU_TRY(check_view(a, "a"));
  PHCU_TRY(check_view(b, "b"));
  if (op < 0 || op >= PHCU_OP_NBINARY) return fail(PHCU_ERR_INVALID, "unknown operator %d", op);
  phcu_program_t P;
  PHCU_TRY(binary_program(op, a->dtype, b->dtype, 1, nullptr, 0, &P));
  phcu_view_t ins[2] = {*a, *b};
  return eval_views(&P, ins, 2, out);
}

int32_t phcu_binary_scalar(int32_t op, const phcu_view_t* a, const phcu_scalar_t* s, int32_t scalar_left,
                           const phcu_view_t* out) {
  PHCU_TRY(require_ctx());
  PHCU_TRY(check_view(a, "a"));
  if (!s || !dtype_valid(s->dtype)) return fail(PHCU_ERR_INVALID, "bad scalar");
  if (op < 0 || op >= PHCU_OP_NBINARY) return fail(PHCU_ERR_INVALID, "unknown operator %d", op);
  phcu_program_t P;
  if (scalar_left) PHCU_TRY(binary_program(op, s->dtype, a->dtype, PHCU_SRC_IMM, s, 1, &P));
  else PHCU_TRY(binary_program(op, a->dtype, s->dtype, PHCU_SRC_IMM, s, 0, &P));
  return eval_views(&P, a, 1, out);
}

int32_t phcu_unary(int32_t uop, const phcu_view_t* a, const phcu_view_t* out) {
  PHCU_TRY(require_ctx());
  PHCU_TRY(check_view(a, "a"));
  int t = a->dtype;
  if (t == PHCU_BOOL) return fail(PHCU_ERR_UNSUPPORTED, "unary operator on Bool");
  if (uop == PHCU_UOP_NOT && !is_int_t(t)) return fail(PHCU_ERR_UNSUPPORTED, "~ on a float operand");
  phcu_program_t P;
  memset(&P, 0, sizeof(P));
  P.n_instr = 2;
  P.out_type = t;
  P.code[0].op = PHCU_I_LD;
  P.code[0].src = 0;
  P.code[0].type = (uint8_t)t;
  P.code[0].btype = (uint8_t)t;
  P.code[1].op = uop == PHCU_UOP_NEG ? PHCU_I_NEG : uop == PHCU_UOP_NOT ? PHCU_I_NOT : PHCU_I_POS;
  P.code[1].type = (uint8_t)t;
  return eval_views(&P, a, 1, out);
}

}  // extern "C"

// Host-only check of the library's program pre-decoding (program.cuh):
// builds programs, runs predecode_program / program_is_fx and prints one JSON
// line per case.  Compiled and run by tests/test_predecode.py (no GPU).
#include <cstdio>

#include "program.cuh"

using namespace phcu;

static phcu_instr_t ins(int op, int src, int type, int btype, int flags, int64_t imm) {
  phcu_instr_t I;
  memset(&I, 0, sizeof(I));
  I.op = (uint8_t)op;
  I.src = (uint8_t)src;
  I.type = (uint8_t)type;
  I.btype = (uint8_t)btype;
  I.flags = (uint8_t)flags;
  I.imm.i = imm;
  return I;
}

static void run(const char* name, std::initializer_list<phcu_instr_t> code, int garbage = 0) {
  phcu_program_t P;
  memset(&P, 0, sizeof(P));
  P.n_instr = (int32_t)code.size();
  int k = 0;
  for (const phcu_instr_t& I : code) {
    P.code[k] = I;
    P.code[k].pad[0] = (uint8_t)garbage;
    k++;
  }
  predecode_program(&P);
  printf("{\"case\": \"%s\", \"is_fx\": %d, \"fx\": [", name, program_is_fx(P) ? 1 : 0);
  for (int i = 0; i < P.n_instr; i++) printf("%s%d", i ? ", " : "", P.code[i].pad[0]);
  printf("], \"btype\": [");
  for (int i = 0; i < P.n_instr; i++) printf("%s%d", i ? ", " : "", P.code[i].btype);
  printf("], \"imm\": [");
  for (int i = 0; i < P.n_instr; i++) printf("%s%lld", i ? ", " : "", (long long)P.code[i].imm.i);
  printf("]}\n");
}

int main() {
  printf("{\"names\": {\"FX_NONE\": %d, \"FX_F32_LD\": %d, \"FX_F32_ADD\": %d, \"FX_F32_SUB\": %d, \"FX_F32_MUL\": %d, "
         "\"FX_F32_DIV\": %d, \"FX_F32_RSUB\": %d, \"FX_F32_RDIV\": %d, \"FX_I32_LD\": %d, \"FX_I32_ADD\": %d, "
         "\"FX_I32_SUB\": %d, \"FX_I32_MUL\": %d, \"FX_I32_RSUB\": %d, \"FX_I32_WADD\": %d, \"FX_I32_WSUB\": %d, "
         "\"FX_I32_WMUL\": %d, \"FX_I32_RWSUB\": %d, \"FX_I32_AND\": %d, \"FX_I32_OR\": %d, \"FX_I32_XOR\": %d}}\n",
         FX_NONE, FX_F32_LD, FX_F32_ADD, FX_F32_SUB, FX_F32_MUL, FX_F32_DIV, FX_F32_RSUB, FX_F32_RDIV, FX_I32_LD,
         FX_I32_ADD, FX_I32_SUB, FX_I32_MUL, FX_I32_RSUB, FX_I32_WADD, FX_I32_WSUB, FX_I32_WMUL, FX_I32_RWSUB,
         FX_I32_AND, FX_I32_OR, FX_I32_XOR);
  const int F = PHCU_F32, I32 = PHCU_I32, F64 = PHCU_F64, IMM = PHCU_SRC_IMM;
  // ((x + 4) ** 2) * y - z
  run("chain", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_ADD, IMM, F, I32, 0, 4), ins(PHCU_OP_POW, IMM, F, I32, 0, 2),
                ins(PHCU_OP_MUL, 1, F, F, 0, 0), ins(PHCU_OP_SUB, 2, F, F, 0, 0)});
  run("swapped_f32", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_SUB, 1, F, F, 1, 0), ins(PHCU_OP_DIV, 1, F, F, 1, 0),
                      ins(PHCU_OP_ADD, 1, F, F, 1, 0), ins(PHCU_OP_MUL, 1, F, F, 1, 0)});
  run("int32_forms", {ins(PHCU_I_LD, 0, I32, I32, 0, 0), ins(PHCU_OP_SUB, 1, I32, I32, 1, 0),
                      ins(PHCU_OP_WSUB, 1, I32, I32, 1, 0), ins(PHCU_OP_WSUB, 1, I32, I32, 0, 0),
                      ins(PHCU_OP_WADD, 1, I32, I32, 0, 0), ins(PHCU_OP_WMUL, 1, I32, I32, 0, 0),
                      ins(PHCU_OP_AND, 1, I32, I32, 0, 0), ins(PHCU_OP_OR, 1, I32, I32, 0, 0),
                      ins(PHCU_OP_XOR, 1, I32, I32, 0, 0), ins(PHCU_OP_MUL, 1, I32, I32, 0, 0),
                      ins(PHCU_OP_ADD, 1, I32, I32, 0, 0)});
  // a comparison, a Float64 operator, a stash operand and a Float64 immediate stay general
  run("general", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_GT, 1, F, F, 0, 0)});
  run("float64", {ins(PHCU_I_LD, 0, F64, F64, 0, 0), ins(PHCU_OP_ADD, 1, F64, F64, 0, 0)});
  run("stash", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_ADD, PHCU_SRC_S0, F, F, 0, 0)});
  run("f64_immediate", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_ADD, IMM, F, F64, 0, 0x4004000000000000ll)});
  // a swapped power and a conversion keep the program out of the reduced interpreter
  run("swapped_pow", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_POW, IMM, F, I32, 1, 2)});
  run("conversion", {ins(PHCU_I_LD, 0, I32, I32, 0, 0), ins(PHCU_I_CVT, 0, I32, 0, 0, PHCU_F32)}, 99);
  // Int32 immediates of Float32 operators, rounded to nearest even
  run("immediates", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_ADD, IMM, F, I32, 0, -3),
                     ins(PHCU_OP_MUL, IMM, F, I32, 0, 16777217), ins(PHCU_OP_SUB, IMM, F, I32, 0, 16777219)});
  // whatever a caller left in pad[0] is overwritten
  run("garbage", {ins(PHCU_I_LD, 0, F, F, 0, 0), ins(PHCU_OP_FLOORDIV, 1, F, F, 0, 0)}, 7);
  return 0;
}

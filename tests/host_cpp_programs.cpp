// Prints the device programs that the C++ host mirror's fused expressions
// (ph-core_gb300/host/phase.hpp: Sym, CuProcView, the program compiler)
// compile to; tests/test_host_cpp_programs.py compares them with the Python
// mirror's compile_program.  Host logic only: nothing here calls the library.
//
//   host_cpp_programs expr   one expression per stdin line:
//                            <out type> <prefix expression>, with
//                            i <slot> <type> | c <type> <value> |
//                            b <op> <lhs> <rhs> | u <op> <operand>
//   host_cpp_programs sym    the fixed expressions built with Sym operators
//   host_cpp_programs proc   CuProcView chains over placeholder operands
//
// Output per program: "P <raises> <n> <out type> | <op src type btype flags
// imm>;..." or "ERR <exception>"; proc mode adds "L <offset> <shape> : <stride>"
// per operand view.
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>

#include "phase.hpp"

using namespace phase;
using detail::ExprP;

static void print_program(const phcu_program_t& p, bool raises) {
  std::cout << "P " << (raises ? 1 : 0) << " " << p.n_instr << " " << p.out_type << " |";
  for (int i = 0; i < p.n_instr; i++) {
    const phcu_instr_t& c = p.code[i];
    std::cout << " " << (int)c.op << " " << (int)c.src << " " << (int)c.type << " " << (int)c.btype << " "
              << (int)c.flags << " " << c.imm.i << ";";
  }
  std::cout << "\n";
}

static void compile_and_print(const ExprP& e, int32_t out_type) {
  try {
    bool raises = false;
    const phcu_program_t p = detail::compile_program(e, out_type, &raises);
    print_program(p, raises);
  } catch (const NotImplementedError&) {
    std::cout << "ERR NotImplementedError\n";
  }
}

static ExprP parse(std::istream& in) {
  std::string k;
  in >> k;
  if (k == "i") {
    int32_t slot, t;
    in >> slot >> t;
    return detail::input(slot, t);
  }
  if (k == "c") {
    int32_t t;
    std::string v;
    in >> t >> v;
    if (t == PHCU_F32) return detail::constant((float)std::strtod(v.c_str(), nullptr));
    if (t == PHCU_F64) return detail::constant(std::strtod(v.c_str(), nullptr));
    if (t == PHCU_I32) return detail::constant((int32_t)std::stoll(v));
    return detail::constant((int64_t)std::stoll(v));
  }
  int32_t op;
  in >> op;
  if (k == "u") return detail::unary_expr(op, parse(in));
  ExprP l = parse(in);
  ExprP r = parse(in);
  return detail::binary_expr(op, l, r);
}

static void expr_mode() {
  std::string line;
  while (std::getline(std::cin, line)) {
    if (line.empty()) continue;
    std::istringstream in(line);
    int32_t out_type;
    in >> out_type;
    try {
      compile_and_print(parse(in), out_type);
    } catch (const NotImplementedError&) {
      std::cout << "ERR NotImplementedError\n";
    }
  }
}

template <typename R>
static void show(const Sym<R>& s) {
  compile_and_print(s.e, DType<R>::id);
}

static void sym_mode() {
  const auto x = Sym<float>::input(0), y = Sym<float>::input(1), z = Sym<float>::input(2), w = Sym<float>::input(3);
  const auto a = Sym<int32_t>::input(0), b = Sym<int32_t>::input(1);
  const auto d = Sym<double>::input(2);
  const auto l = Sym<int64_t>::input(3);
  show(pow(x + 4, 2) * y - z);                         // the fused chain ((x + 4) ** 2) * y - z
  show((x + y + z - w * 4) * 0.2f);                    // a four-point update
  show(a / b);                                         // Int32 / Int32 -> Float64
  show(a * 0.5f + x);                                  // Int32 * Float32 -> Float32
  show(x * y - z * w);                                 // both operands compound: one stash
  show((x * y - z * w) * ((x + y) - (z + w)));         // two stashes
  show(7 - x * 3);                                     // constant on the left: swapped operands
  show(-a + b);                                        // checked Int32 negation
  show(pow(x, 3));                                     // Float32 ** Int32
  show(pow(a, x));                                     // Int32 ** Float32 -> Float64
  show(pow(a, b));                                     // checked Int32 power
  show(wpow(a, 3));                                    // wrapping Int32 power
  show(wadd(a, b) - wmul(a, 5));                       // wrapping arithmetic
  show(floordiv(a, 3) % 7);                            // floored division and modulo
  show((a & b) ^ (a | 12));                            // bitwise
  show(d * x + 1.5);                                   // Float64 with Float32
  show(l + a);                                         // Int64 + Int32 -> Int64
  show(a + l);                                         // Int32 + Int64 -> Int32
  show(x / 0.0f);                                      // IEEE division
  show(x % 2.5f);                                      // Float32 modulo
  show(pow(x * y, z - w));                             // Float32 ** Float32 with a stash
  show(2 - (x - (y - (z - w))));                       // right-leaning chain
  try {
    show(((x * y - z * w) * (x - y * z)) - ((x + y) * (z - w * x)));  // needs a third stash
  } catch (const NotImplementedError&) {
    std::cout << "ERR NotImplementedError\n";
  }
}

static detail::Leaf leaf(int64_t offset, const std::vector<int64_t>& shape, int32_t dtype) {
  return detail::Leaf{nullptr, Affine{offset, shape, row_major(shape)}, dtype};
}

template <typename T>
static void show(const CuProcView<T>& p) {
  bool raises = false;
  const phcu_program_t prog = p.program(&raises);
  print_program(prog, raises);
  for (const auto& lf : p.leaves()) {
    std::cout << "L " << lf.aff.offset;
    for (int64_t s : lf.aff.shape) std::cout << " " << s;
    std::cout << " :";
    for (int64_t s : lf.aff.stride) std::cout << " " << s;
    std::cout << "\n";
  }
}

static void proc_mode() {
  // Placeholder operand views: no buffers; distinct offsets keep them apart.
  const std::vector<int64_t> sh = {4, 3, 2};
  const CuProcView<float> x({leaf(0, sh, PHCU_F32)}, detail::input(0, PHCU_F32), sh);
  const CuProcView<float> y({leaf(1000, sh, PHCU_F32)}, detail::input(0, PHCU_F32), sh);
  const CuProcView<float> z({leaf(2000, sh, PHCU_F32)}, detail::input(0, PHCU_F32), sh);
  const CuProcView<int32_t> a({leaf(3000, sh, PHCU_I32)}, detail::input(0, PHCU_I32), sh);
  const auto chain = x.process([](auto e) { return pow(e + 4, 2); }) * y - z;
  show(chain);
  show(chain.permute({2, 0, 1}).view({all(), rng(std::nullopt, std::nullopt, -1)}));
  show(x * x + x);                                  // one operand view, one slot
  show((x - y) * (y - x));                          // shared operands across both sides
  show(a.process([](auto e) { return e * 2; }) / a + x);
  show(x.process([](auto) { return 1.5f; }));       // a constant block
  show(-(a * 3));
  show(x.view({idx(1)}) + y.view({idx(2)}));        // dropped axis: distinct views
  show(x.reverse() * 2.0);
  try {
    show(x + y.view({rng(0, 2)}));
  } catch (const ShapeError& e) {
    std::cout << "ERR ShapeError " << e.what() << "\n";
  }
  // Five distinct operand views: to_cu() refuses these (more than
  // PHCU_MAX_INPUTS) before any device call.
  const CuProcView<float> w({leaf(4000, sh, PHCU_F32)}, detail::input(0, PHCU_F32), sh);
  std::cout << "N " << ((x + y) * (z - a) + w).leaves().size() << "\n";
}

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "expr";
  if (mode == "expr") expr_mode();
  else if (mode == "sym") sym_mode();
  else if (mode == "proc") proc_mode();
  else return 2;
  return 0;
}

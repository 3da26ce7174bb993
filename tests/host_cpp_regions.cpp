// Reads region cases from stdin and prints what the C++ host mirror
// (ph-core_gb300/host/phase.hpp) makes of them; driven by
// tests/test_host_cpp.py.  One case per line:
//   N <rank> <bound...> <nlits> <lit>... <op>      IndexRegion::make (bounded)
//   A <nlits> <lit>... <op>                        IndexRegion::absolute
// with <lit> = I <index> | R <first|n> <last|n> <step|n> <exclusive 0/1> and
// <op> = none | rev | fits|trim|trans|incl|l2a <n> <values...>.
// Output: "OK <n> <reduced shape...> | <first step last size>..." for a
// region, "BOOL 0|1", "COORD <values...>" or "ERR <exception>".  Host logic
// only: nothing here calls the library.
#include <iostream>
#include <sstream>
#include <string>

#include "phase.hpp"

static std::optional<int64_t> opt(const std::string& t) {
  if (t == "n") return std::nullopt;
  return std::stoll(t);
}

static std::vector<int64_t> ints(std::istream& in) {
  size_t n = 0;
  in >> n;
  std::vector<int64_t> v(n);
  for (auto& x : v) in >> x;
  return v;
}

static void print(const phase::IndexRegion& r) {
  const std::vector<int64_t> sh = r.shape();
  std::cout << "OK " << sh.size();
  for (int64_t v : sh) std::cout << " " << v;
  std::cout << " |";
  for (const auto& a : r.axes) std::cout << " " << a.first << " " << a.step << " " << a.last << " " << a.size;
  std::cout << "\n";
}

int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    if (line.empty()) continue;
    std::istringstream in(line);
    std::string mode;
    in >> mode;
    std::vector<int64_t> bound;
    if (mode == "N") {
      size_t rank = 0;
      in >> rank;
      bound.resize(rank);
      for (auto& b : bound) in >> b;
    }
    size_t nlits = 0;
    in >> nlits;
    std::vector<phase::Lit> lits;
    for (size_t i = 0; i < nlits; i++) {
      std::string kind;
      in >> kind;
      if (kind == "I") {
        int64_t v;
        in >> v;
        lits.push_back(phase::idx(v));
      } else {
        std::string f, l, s;
        int x;
        in >> f >> l >> s >> x;
        lits.push_back(phase::rng(opt(f), opt(l), opt(s), x != 0));
      }
    }
    std::string op;
    in >> op;
    try {
      phase::IndexRegion r = mode == "N" ? phase::IndexRegion::make(lits, bound) : phase::IndexRegion::absolute(lits);
      // Every result is computed before anything is printed, so a raise
      // leaves no half-written line.
      if (op == "fits" || op == "incl") {
        const bool b = op == "fits" ? r.fits_in(ints(in)) : r.includes(ints(in));
        std::cout << "BOOL " << (b ? 1 : 0) << "\n";
      } else if (op == "l2a") {
        const std::vector<int64_t> c = r.local_to_absolute(ints(in));
        std::cout << "COORD";
        for (int64_t v : c) std::cout << " " << v;
        std::cout << "\n";
      } else {
        if (op == "trim") r.trim(ints(in));
        if (op == "rev") r.reverse();
        if (op == "trans") r.translate(ints(in));
        print(r);
      }
    } catch (const phase::DimensionError&) {
      std::cout << "ERR DimensionError\n";
    } catch (const phase::IndexError&) {
      std::cout << "ERR IndexError\n";
    } catch (const phase::ArgumentError&) {
      std::cout << "ERR ArgumentError\n";
    }
  }
  return 0;
}

// Reads region literals from stdin and prints the C++ host mirror's
// canonical IndexRegion (ph-core_gb300/host/phase.hpp) or the exception it
// raises; driven by tests/test_host_cpp.py.  One case per line:
//   <rank> <bound...> <nlits> { I <index> | R <first|n> <last|n> <step|n> <exclusive 0/1> }...
// Output per case: "OK <n> <reduced shape...> | <first step last size>..." or
// "ERR <exception>".  Host logic only: nothing here calls the library.
#include <iostream>
#include <sstream>
#include <string>

#include "phase.hpp"

static std::optional<int64_t> opt(const std::string& t) {
  if (t == "n") return std::nullopt;
  return std::stoll(t);
}

int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    if (line.empty()) continue;
    std::istringstream in(line);
    size_t rank = 0, nlits = 0;
    in >> rank;
    std::vector<int64_t> bound(rank);
    for (auto& b : bound) in >> b;
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
    try {
      const phase::IndexRegion r = phase::IndexRegion::make(lits, bound);
      const std::vector<int64_t> sh = r.shape();
      std::cout << "OK " << sh.size();
      for (int64_t v : sh) std::cout << " " << v;
      std::cout << " |";
      for (const auto& a : r.axes) std::cout << " " << a.first << " " << a.step << " " << a.last << " " << a.size;
      std::cout << "\n";
    } catch (const phase::DimensionError&) {
      std::cout << "ERR DimensionError\n";
    } catch (const phase::IndexError&) {
      std::cout << "ERR IndexError\n";
    }
  }
  return 0;
}

// Reads one affine layout and a new shape per line,
//   <offset> <rank> <shape...> <stride...> <new rank> <new shape...>
// and prints what the C++ host mirror's affine_reshape makes of it:
//   OK <offset> <stride...>   or   NONE   (strides cannot express it).
// tests/test_host_cpp.py compares the answers with the Python mirror's.
#include <iostream>
#include <sstream>
#include <string>

#include "phase.hpp"

using namespace phase;

int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream in(line);
    Affine a;
    size_t rank = 0, nrank = 0;
    in >> a.offset >> rank;
    a.shape.resize(rank);
    a.stride.resize(rank);
    for (auto& v : a.shape) in >> v;
    for (auto& v : a.stride) in >> v;
    in >> nrank;
    std::vector<int64_t> ns(nrank);
    for (auto& v : ns) in >> v;
    const std::optional<Affine> r = affine_reshape(a, ns);
    if (!r) {
      std::cout << "NONE\n";
      continue;
    }
    std::cout << "OK " << r->offset;
    for (int64_t s : r->stride) std::cout << " " << s;
    std::cout << "\n";
  }
  return 0;
}

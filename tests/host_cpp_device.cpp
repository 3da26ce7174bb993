// Runs the C++ host mirror (ph-core_gb300/host/phase.hpp) on the device:
// reads a.f32/b.f32/a.i32/b.i32 (16x12x10, row-major) from the directory
// given as argv[1], writes each result as <name>.bin there and prints one line
// per result or raised exception; tests/test_gpu_host_cpp.py compares them
// with the oracle.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>

#include "phase.hpp"

using namespace phase;

static std::string dir;

template <typename T>
static std::vector<T> load(const std::string& name, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(dir + "/" + name, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
  if (!f) throw std::runtime_error("cannot read " + name);
  return v;
}

template <typename T>
static void save(const std::string& name, const std::vector<T>& v) {
  std::ofstream f(dir + "/" + name + ".bin", std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
  std::cout << "ok " << name << " " << v.size() << "\n";
}

template <typename F>
static void expect_raise(const std::string& name, F f) {
  try {
    f();
    std::cout << "noraise " << name << "\n";
  } catch (const DimensionError&) {
    std::cout << "raised " << name << " DimensionError\n";
  } catch (const ShapeError&) {
    std::cout << "raised " << name << " ShapeError\n";
  } catch (const IndexError&) {
    std::cout << "raised " << name << " IndexError\n";
  } catch (const OverflowError&) {
    std::cout << "raised " << name << " OverflowError\n";
  }
}

template <typename T>
static void run(const std::string& tag) {
  const std::vector<int64_t> shape = {16, 12, 10};
  const size_t n = 16 * 12 * 10;
  const CuNArray<T> A = CuNArray<T>::of_buffer(shape, load<T>("a." + tag, n));
  const CuNArray<T> B = CuNArray<T>::of_buffer(shape, load<T>("b." + tag, n));
  const CuView<T> ap = A.permute({2, 0, 1}), bp = B.permute({2, 0, 1});
  const std::vector<Lit> rev = {all(), rng(std::nullopt, std::nullopt, -1), all()};
  const CuView<T> ar = A.view(rev), br = B.view(rev);
  save(tag + "_perm", ap.to_vector());
  save(tag + "_rev", ar.to_vector());
  save(tag + "_add_perm", (ap + bp).to_vector());
  save(tag + "_sub_rev", (ar - br).to_vector());
  save(tag + "_div_perm", (ap / bp).to_vector());
  if (std::is_floating_point<T>::value) save(tag + "_mul_rev", (ar * br).to_vector());
  else save(tag + "_mul_rev", wmul(ar, br).to_vector());
  save(tag + "_scal", (T(7) - (ap * T(3))).to_vector());
  for (int k = 0; k < 3; k++) {
    save(tag + "_sum" + std::to_string(k), sum(ap, k).to_vector());
    save(tag + "_max" + std::to_string(k), max(ar, k).to_vector());
    save(tag + "_argmax" + std::to_string(k), argmax(ap, k).to_vector());
  }
  save(tag + "_sumall", std::vector<T>{sum(A)});
  save(tag + "_argmaxall", argmax(ar));
  save(tag + "_chunk", A.get_chunk({idx(1), rng(0, 10, 3, true), rng(-1, 2)}).to_vector());
  CuNArray<T> C = CuNArray<T>::fill({10, 16, 12}, T(5));
  C.set_chunk(rev, ap);
  C.set_chunk({idx(2), rng(0, 3)}, T(-1));
  save(tag + "_scatter", C.to_vector());
  expect_raise(tag + "_shape", [&] { return ap + ar; });
  expect_raise(tag + "_index", [&] { return A.view({rng(0, 16)}); });
  expect_raise(tag + "_dim", [&] { return A.view({all(), all(), all(), all()}); });
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  dir = argv[1];
  try {
    init(0);
    run<float>("f32");
    run<int32_t>("i32");
    const CuNArray<int32_t> big = CuNArray<int32_t>::fill({64}, 1 << 30);
    expect_raise("overflow", [&] { return big + big; });
    save("wrapped", wadd(big, big).to_vector());
  } catch (const std::exception& e) {
    std::cout << "error " << e.what() << "\n";
    return 1;
  }
  return 0;
}

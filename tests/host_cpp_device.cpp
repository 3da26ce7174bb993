// Runs the C++ host mirror (ph-core_gb300/host/phase.hpp) on the device:
// reads a.f32/b.f32/a.i32/b.i32 (16x12x10, row-major) from the directory
// given as argv[1], writes each result as <name>.bin there and prints one line
// per result or raised exception; tests/test_gpu_host_cpp.py compares them
// with the oracle.  With argv[2] = "proc" it runs the fused expressions
// (CuProcView) instead of the eager operators; with "more" element access,
// slices, comparisons, masked writes, equality, in-place maps, reshape, tile,
// concatenate and push.
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
  } catch (const NotImplementedError&) {
    std::cout << "raised " << name << " NotImplementedError\n";
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

// Fused chains: one phcu_eval per materialisation.
template <typename T>
static void run_proc(const std::string& tag) {
  const std::vector<int64_t> shape = {16, 12, 10};
  const size_t n = 16 * 12 * 10;
  const CuNArray<T> A = CuNArray<T>::of_buffer(shape, load<T>("a." + tag, n));
  const CuNArray<T> B = CuNArray<T>::of_buffer(shape, load<T>("b." + tag, n));
  const std::vector<Lit> rev = {all(), rng(std::nullopt, std::nullopt, -1), all()};
  // ((x + 4) ** 2) * y - z over an array and two reversed views
  const auto chain = A.process([](auto e) { return pow(e + 4, 2); }) * B.view(rev) - A.view(rev);
  save(tag + "_proc_chain", chain.to_vector());
  save(tag + "_proc_chain_perm", chain.permute({2, 0, 1}).reverse().to_vector());
  save(tag + "_proc_chain_max1", max(chain, 1).to_vector());
  save(tag + "_proc_chain_argmax0", argmax(chain, 0).to_vector());
  save(tag + "_proc_sum1", sum(A.process() * 3 - B.view(rev), 1).to_vector());  // within Int32
  save(tag + "_proc_chain_chunk", chain.get_chunk({idx(3), rng(0, 10, 3, true)}).to_vector());
  CuNArray<T> C = CuNArray<T>::fill(shape, T(0));
  C.set_chunk(rev, A.process() + B);
  save(tag + "_proc_set", C.to_vector());
  CuNArray<T> D = A.clone();
  // a source one row ahead of the rows it writes: element by element, every
  // read comes before the write that reaches it, so the result is the reference's
  D.set_chunk({rng(0, -2)}, D.view({rng(1, -1)}).process() * 2);
  save(tag + "_proc_overlap", D.to_vector());
  // one row behind: the reference would read rows it has already written
  expect_raise(tag + "_proc_overlap_behind", [&] {
    CuNArray<T> E = A.clone();
    E.set_chunk({rng(1, -1)}, E.view({rng(0, -2)}).process() * 2);
    return E;
  });
  save(tag + "_proc_const", A.process([](auto) { return 2.5f; }).to_vector());
  // five distinct operand views (A, B, A and B reversed on axis 1, A reversed
  // on every axis; CuView - CuView alone would be eager): more than one device
  // program reads, so the expression runs as two programs
  save(tag + "_proc_five", ((A.process() + B) * (A.view(rev).process() - B.view(rev)) + A.reverse()).to_vector());
}

// Element access, slices, comparisons, masked writes, equality and in-place maps.
template <typename T>
static void run_more(const std::string& tag) {
  const std::vector<int64_t> shape = {16, 12, 10};
  const size_t n = 16 * 12 * 10;
  const CuNArray<T> A = CuNArray<T>::of_buffer(shape, load<T>("a." + tag, n));
  const CuNArray<T> B = CuNArray<T>::of_buffer(shape, load<T>("b." + tag, n));
  const std::vector<Lit> rev = {all(), rng(std::nullopt, std::nullopt, -1), all()};
  CuNArray<T> D = A.clone();
  D.map_inplace([](auto e) { return e * 3 + 1; });
  save(tag + "_map_inplace", D.to_vector());
  CuNArray<T> E = A.clone();
  E.map_with_inplace(B.view(rev), [](auto x, auto y) { return x - y * 2; });
  save(tag + "_map_with_inplace", E.to_vector());
  save(tag + "_get", std::vector<T>{A.get({3, -1, 2}), A.get({-16, 0, -1})});
  CuNArray<T> F = A.clone();
  F.set_element({0, 0, 0}, T(42));
  F.set_element({-1, -1, -1}, T(-7));
  save(tag + "_set_element", F.to_vector());
  expect_raise(tag + "_get_index", [&] { return A.get({16, 0, 0}); });
  expect_raise(tag + "_get_dim", [&] { return A.get({1, 2}); });
  const std::vector<CuNArray<T>> sl = A.slices(1);
  std::cout << "nslices " << tag << " " << sl.size() << "\n";
  save(tag + "_slice5", sl[5].to_vector());
  const CuNArray<Bool> m = gt(A, B);
  save(tag + "_gt", m.to_vector());
  CuNArray<T> G = A.clone();
  G.set_mask(m, T(0));
  save(tag + "_mask_value", G.to_vector());
  CuNArray<T> H = A.clone();
  H.set_mask(m, B.view(rev));
  save(tag + "_mask_src", H.to_vector());
  expect_raise(tag + "_mask_shape", [&] {
    CuNArray<T> X = A.clone();
    X.set_mask(gt(A.permute({2, 0, 1}), B.permute({2, 0, 1})), T(1));
    return X;
  });
  std::cout << "equals " << tag << " same " << equals(A, A.clone()) << "\n";
  std::cout << "equals " << tag << " other " << equals(A, B) << "\n";
  std::cout << "equals " << tag << " reversed " << equals(A.view(rev), A.view(rev).to_cu()) << "\n";
  std::cout << "equals " << tag << " shape " << equals(A.view({}), A.permute({2, 0, 1})) << "\n";
  // reshape: a permuted view (copied first), an affine one, the array itself
  save(tag + "_reshape_perm", A.permute({2, 0, 1}).reshape({10, 192}).to_vector());
  save(tag + "_reshape_rows", A.view({rng(2, 9)}).reshape({8, 120}).to_vector());
  save(tag + "_reshape_rev", A.view(rev).reshape({16, 120}).to_vector());
  save(tag + "_reshape_array", A.reshape({120, 16}).to_vector());
  expect_raise(tag + "_reshape_size", [&] { return A.view({}).reshape({7, 7}); });
  // tile, concatenate, push
  const CuNArray<T> S = A.get_chunk({rng(0, 3), rng(0, 4), rng(0, 5)});
  save(tag + "_tile", CuNArray<T>::tile(S.view(rev), {2, 3, 1}).to_vector());
  save(tag + "_concat", CuNArray<T>::concatenate({A.view(rev), B.view({})}, 1).to_vector());
  expect_raise(tag + "_concat_dim", [&] { return CuNArray<T>::concatenate({A.view({}), A.permute({2, 0, 1})}, 0); });
  CuNArray<T> P = A.clone();
  P.push(B.view({}));
  save(tag + "_push", P.to_vector());
  // in-place maps with the element's index and coordinates
  CuNArray<T> I = A.clone();
  I.map_with_index_inplace([](auto e, auto i) { return e + i; });
  save(tag + "_map_with_index", I.to_vector());
  CuNArray<T> K = A.clone();
  K.map_with_coord_inplace([](auto e, const auto& c) { return e * c[0] - c[2]; });
  save(tag + "_map_with_coord", K.to_vector());
}

static void run_proc_mixed() {
  const std::vector<int64_t> shape = {16, 12, 10};
  const size_t n = 16 * 12 * 10;
  const CuNArray<float> A = CuNArray<float>::of_buffer(shape, load<float>("a.f32", n));
  const CuNArray<int32_t> Ai = CuNArray<int32_t>::of_buffer(shape, load<int32_t>("a.i32", n));
  const CuNArray<int32_t> Bi = CuNArray<int32_t>::of_buffer(shape, load<int32_t>("b.i32", n));
  save("proc_mixed", ((Ai.process() * 0.5f + A) / 3.0).to_vector());      // Int32 * Float32, then Float64
  save("proc_div", (Ai.permute({2, 0, 1}).process() / Bi.permute({2, 0, 1})).to_vector());  // Float64
  const CuNArray<int32_t> big = CuNArray<int32_t>::fill({64}, 1 << 30);
  expect_raise("proc_overflow", [&] { return (big.process() * 4 + big).to_cu(); });
  save("proc_wrapped", wadd(wmul(big.process(), 4), big).to_vector());
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  dir = argv[1];
  if (argc > 2 && std::string(argv[2]) == "more") {
    try {
      init(0);
      run_more<float>("f32");
      run_more<int32_t>("i32");
    } catch (const std::exception& e) {
      std::cout << "error " << e.what() << "\n";
      return 1;
    }
    return 0;
  }
  if (argc > 2 && std::string(argv[2]) == "proc") {
    try {
      init(0);
      run_proc<float>("f32");
      run_proc<int32_t>("i32");
      run_proc_mixed();
    } catch (const std::exception& e) {
      std::cout << "error " << e.what() << "\n";
      return 1;
    }
    return 0;
  }
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

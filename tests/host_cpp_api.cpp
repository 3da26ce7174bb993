// Compile-only check of the C++ host mirror's public surface
// (ph-core_gb300/host/phase.hpp) as a caller uses it: views,
// eager operators with Crystal's result types, fused CuProcView chains,
// reductions, chunk reads and writes, element access, slices, comparisons,
// masked writes, equality, in-place maps, reshape, tile, concatenate, push,
// region operations.  The static
// assertions pin the result types; tests/test_host_cpp_programs.py compiles
// this file with warnings as errors.  Nothing here runs.
#include <type_traits>

#include "phase.hpp"

using namespace phase;

template <typename A, typename B>
constexpr bool same = std::is_same<A, B>::value;

void api(const std::vector<float>& host_f, const std::vector<int32_t>& host_i) {
  init(0);
  auto a = CuNArray<float>::of_buffer({512, 512, 256}, host_f);
  auto b = CuNArray<float>::of_buffer({512, 512, 256}, host_f);
  auto ai = CuNArray<int32_t>::of_buffer({512, 512, 256}, host_i);
  auto bi = CuNArray<int32_t>::of_buffer({512, 512, 256}, host_i);
  auto c = CuNArray<float>::fill({256, 512, 512}, 0.0f);
  auto p = a.permute({2, 0, 1});
  auto r = a.view({all(), rng(std::nullopt, std::nullopt, -1), all()});
  CuNArray<float> s = p + b.permute({2, 0, 1});
  CuNArray<int32_t> i = argmax(s, 2);
  CuNArray<double> q = ai.permute({2, 0, 1}) / bi.permute({2, 0, 1});
  c.set_chunk({all(), rng(std::nullopt, std::nullopt, -1), all()}, p);
  c.set_chunk({idx(0)}, 1.5f);
  CuNArray<int32_t> w = wmul(ai, bi);

  // fused chains
  auto x = CuNArray<float>::of_buffer({64, 128, 128, 64}, host_f);
  auto y = x.clone();
  auto z = x.clone();
  auto chain = x.process([](auto e) { return pow(e + 4, 2); }) * y - z;
  static_assert(same<decltype(chain), CuProcView<float>>, "Float32 chain");
  CuNArray<float> out = chain.to_cu();
  CuNArray<float> s1 = sum(chain, 1);
  CuNArray<int32_t> am = argmax(chain, 3);
  CuNArray<float> corner = chain.get_chunk({idx(0), rng(0, 3)});
  auto mixed = ai.permute({2, 0, 1}).process() * 0.5f + a.permute({2, 0, 1});
  static_assert(same<decltype(mixed), CuProcView<float>>, "Int32 * Float32 is Float32");
  auto quot = ai.process() / bi;
  static_assert(same<decltype(quot), CuProcView<double>>, "Int32 / Int32 is Float64");
  auto ipow = pow(ai.process(), 1.5f);
  static_assert(same<decltype(ipow), CuProcView<double>>, "Int32 ** Float32 is Float64");
  auto fpow = pow(a.process(), 3);
  static_assert(same<decltype(fpow), CuProcView<float>>, "Float32 ** Int32 stays Float32");
  auto wrap = wadd(wmul(ai.process(), 4), bi);
  static_assert(same<decltype(wrap), CuProcView<int32_t>>, "wrapping Int32");
  auto wide = ai.process() + int64_t(1);
  static_assert(same<decltype(wide), CuProcView<int32_t>>, "Int32 + Int64 is Int32 (the receiver's type)");
  auto bits = (ai.process() & bi) ^ 7;
  static_assert(same<decltype(bits), CuProcView<int32_t>>, "bitwise");
  auto neg = -(a.process() * 2.0);
  static_assert(same<decltype(neg), CuProcView<double>>, "Float32 * Float64 is Float64");
  auto cst = a.process([](auto) { return 2.5f; });
  static_assert(same<decltype(cst), CuProcView<float>>, "a constant block");
  c.set_chunk({all(), all(), all()}, p.process() * 2);
  float total = sum(chain);
  std::vector<int64_t> where = argmax(chain.permute().reverse());

  // element access, slices, comparisons, masks, equality, in-place maps
  float e0 = a.get({0, -1, 3});
  a.set_element({1, 2, 3}, 4.0f);
  std::vector<CuNArray<float>> sl = a.slices(2);
  CuNArray<Bool> m = gt(a, b);
  static_assert(same<decltype(lt(ai, bi)), CuNArray<Bool>>, "comparisons give Bool arrays");
  std::vector<Bool> mh = m.to_vector();
  a.set_mask(m, 0.0f);
  a.set_mask(m, b.view({}));
  bool eqs = equals(a, b) || equals<int32_t>(ai, bi);
  CuNArray<float>& self = a.map_inplace([](auto e) { return e * 3 + 1; });
  ai.map_with_inplace(bi.view({}), [](auto u, auto v) { return u - v * 2; });
  a.map_with_inplace(ai.view({}), [](auto u, auto v) { return u * v; });  // Float32 * Int32 stays Float32
  a.map_with_index_inplace([](auto e, auto k) { return e + k; });
  ai.map_with_coord_inplace([](auto e, const auto& cd) { return e * cd[0] - cd[2]; });

  // reshape, tile, concatenate, push
  CuView<float> rv = p.reshape({256, 512 * 512});
  CuNArray<float> ra = a.reshape({512 * 512, 256});
  CuNArray<float> tl = CuNArray<float>::tile(a.get_chunk({rng(0, 1)}), {2, 1, 3});
  CuNArray<float> cc = CuNArray<float>::concatenate({a.view({}), b.view({})}, 2);
  ai.push(bi.view({}));

  // region operations
  IndexRegion reg = IndexRegion::absolute({rng(3, 20, 4), rng(7, std::nullopt, -2)});
  bool fits = reg.fits_in({21, 8});
  bool has = reg.includes({7, 5});
  reg.translate({-3, 0});
  reg.reverse();
  std::vector<int64_t> abs = reg.local_to_absolute({1, 2});
  reg.trim({10, 4});
  (void)i, (void)q, (void)w, (void)out, (void)s1, (void)am, (void)corner, (void)total, (void)where;
  (void)fits, (void)has, (void)abs, (void)r, (void)e0, (void)sl, (void)mh, (void)eqs, (void)self, (void)rv, (void)ra, (void)tl, (void)cc;
}

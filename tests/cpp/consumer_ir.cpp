// Consumer-side check of the C++ front end without a device: builds the
// expressions of the reference configurations as typed expressions through
// include/aether and prints the aether-ir/1 text each serialises to, one per
// line, for the Python test to compare with the Python front end's text.
#include <aether/aether.h>

#include <cstdio>

using namespace aether;

template <class T, std::size_t... Es>
auto fake(std::uintptr_t addr, std::size_t n) {
    return aether::detail::plane_view<T, Es...>(reinterpret_cast<T*>(addr), quantized_capacity(n), n);
}

template <class V, class E>
void emit(const char* name, const V&, const E& typed, const char* op = "set") {
    const Expr e(typed);
    ir::Context ctx;
    const std::string text = plan_text(aether::detail::dtype_name<typename V::value_type>(),
                                       dst_shape(ir::shape_of(typename V::element_extents{}), e), op, e, ctx);
    std::printf("%s\t%s\t%zu\t%zu\t%zu\n", name, text.c_str(), ctx.operands.size(), ctx.scalars.size(), ctx.keys.size());
}

int main() {
    const std::size_t n = 1000;
    auto a = fake<double, 3>(0x10000, n), b = fake<double, 3>(0x20000, n), c = fake<double, 3>(0x30000, n);
    auto d0 = fake<double, 3>(0x40000, n), d = fake<double, 3>(0x50000, n);
    emit("cfg1", d, a + b * c + cwiseSin(a) * cwiseExp((c * c) * -1.0));
    emit("cfg2a", d, cwiseSqrt(a * a + b * b) * cwiseLog1p(cwiseAbs(c)) + cwiseRsqrt(constant<extents<3>>(1.0) + d0 * d0));
    random::Generator g(42);
    emit("uniform", a, g.substream(0).uniform<double, 3>(-1.0, 1.0));
    auto z = fake<double>(0x60000, n);
    emit("normal", z, random::Generator(7).substream(4).normal<double, 1>(0.0, 1.0));
    Item<double, 3> m3, s3, l3;
    m3(0) = -1.0; m3(1) = 0.0; m3(2) = 2.5;
    s3(0) = 0.5; s3(1) = 1.0; s3(2) = 3.0;
    l3(0) = 0.5; l3(1) = 2.0; l3(2) = 8.0;
    emit("normal_item", a, random::Generator(21).substream(0).normal<double, 3>(m3, s3));
    emit("exponential_item", a, random::Generator(21).substream(2).exponential<double, 3>(l3));
    auto q = fake<double, 4>(0x70000, n);
    auto m = fake<double, 3, 3>(0x80000, n), mi = fake<double, 3, 3>(0x90000, n);
    emit("cross", d, a.cross(b));
    emit("qrot", d, q.quatRotate(b));
    emit("inv", mi, select(cwiseAbs(per_sample::det(m)) > 1e-300, m.inverse(), constant<extents<3, 3>>(0.0)));
    auto x = fake<float, 8>(0xA0000, n), y = fake<float, 8>(0xB0000, n);
    auto s = fake<float>(0xC0000, n);
    emit("dot8", s, per_sample::dot(x, y));
    emit("axpy_add", d, a * 2.5 + b / 4.0, "add");
    emit("minmax", d, cwiseMax(cwiseMin(a, b), -0.5) - clamp(c, -0.25, 0.25));
    emit("structural", d, m.row<1>() + m.col<2>() + m.transpose() * a);
    emit("literal", d, a * literal(0.1) + literal(-3.0));
    return 0;
}

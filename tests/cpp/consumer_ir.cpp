// Consumer-side check of the C++ front end without a device: builds the
// expressions of the reference configurations through include/aether and
// prints the aether-ir/1 text of each assignment, one per line, for the
// Python test to compare with the Python front end's text.
#include <aether/aether.h>

#include <cstdio>

using namespace aether;

template <class T, std::size_t... Es>
View<T, Es...> fake(std::uintptr_t addr, std::size_t n) {
    return View<T, Es...>(reinterpret_cast<T*>(addr), quantized_capacity(n), n);
}

template <class T, std::size_t... Es>
void emit(const char* name, const View<T, Es...>&, const Expr& e, const char* op = "set") {
    ir::Context ctx;
    const std::string text = plan_text(aether::detail::dtype_name<T>(), dst_shape(View<T, Es...>::shape(), e), op, e, ctx);
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
    auto q = fake<double, 4>(0x70000, n);
    auto m = fake<double, 3, 3>(0x80000, n), mi = fake<double, 3, 3>(0x90000, n);
    emit("cross", d, a.cross(b));
    emit("qrot", d, q.quatRotate(b));
    emit("inv", mi, select(cwiseAbs(m.det()) > 1e-300, m.inverse(), constant<extents<3, 3>>(0.0)));
    auto x = fake<float, 8>(0xA0000, n), y = fake<float, 8>(0xB0000, n);
    auto s = fake<float>(0xC0000, n);
    emit("dot8", s, x.dot(y));
    emit("axpy_add", d, a * 2.5 + b / 4.0, "add");
    emit("minmax", d, cwiseMax(cwiseMin(a, b), -0.5) - clamp(c, -0.25, 0.25));
    emit("structural", d, m.expr().row(1) + m.expr().col(2) + m.expr().transpose().matvec(a));
    emit("literal", d, a * literal(0.1) + literal(-3.0));
    return 0;
}

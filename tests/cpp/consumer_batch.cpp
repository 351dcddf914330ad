// Batches and serving through the C++ headers: uneven arrays of the cross
// product and the guarded 3x3 inverse in one launch and in a graph replay,
// compared with one plain assignment per array; then a server answering the
// same cross products from host bytes, compared with the plain results.
#include <aether/aether.h>

#include <cstdio>
#include <cstring>
#include <vector>

using namespace aether;

int main() {
    const std::size_t sizes[] = {37, 1000, 4097, 12345, 64, 777};
    random::Generator g(11);
    std::vector<std::unique_ptr<Array<double, 3>>> as, bs, outs, refs;
    std::vector<std::unique_ptr<Array<double, 3, 3>>> ms, minv, mref;
    gb300::Batch batch;
    for (std::size_t k = 0; k < 6; ++k) {
        const std::size_t n = sizes[k];
        as.emplace_back(new Array<double, 3>(n));
        bs.emplace_back(new Array<double, 3>(n));
        outs.emplace_back(new Array<double, 3>(n));
        refs.emplace_back(new Array<double, 3>(n));
        as.back()->deviceView() = g.substream(2 * k).uniform<double, 3>(-1.0, 1.0);
        bs.back()->deviceView() = g.substream(2 * k + 1).uniform<double, 3>(-1.0, 1.0);
        refs.back()->deviceView() = as.back()->deviceView().cross(bs.back()->deviceView());
        batch.add(outs.back()->deviceView(), as.back()->deviceView().cross(bs.back()->deviceView()));
        ms.emplace_back(new Array<double, 3, 3>(n));
        minv.emplace_back(new Array<double, 3, 3>(n));
        mref.emplace_back(new Array<double, 3, 3>(n));
        ms.back()->deviceView() = Expr(g.substream(100 + k).uniform<double, 9>(-1.0, 1.0)).reshape({3, 3});
        auto M = ms.back()->deviceView();
        const Expr inv = select(cwiseAbs(per_sample::det(M)) > 1e-300, M.inverse(), constant<extents<3, 3>>(0.0));
        mref.back()->deviceView() = inv;
        batch.add(minv.back()->deviceView(), inv);
    }
    auto same = [](auto& x, auto& y) {
        x.download();
        y.download();
        return std::memcmp(x.hostView().data(), y.hostView().data(), x.bytes()) == 0;
    };
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 0) {
            batch.launch();
        } else {
            void* s = nullptr;
            if (aether_stream_create(0, &s) != AETHER_OK) return 1;
            for (auto& o : outs) o->deviceView() = o->deviceView() * 0.0;
            aether_stream_sync(0, nullptr);
            batch.capture(s);
            batch.replay(s);
            aether_stream_sync(0, s);
            aether_stream_destroy(s);
        }
        for (std::size_t k = 0; k < 6; ++k)
            if (!same(*outs[k], *refs[k]) || !same(*minv[k], *mref[k])) {
                std::printf("batch pass %d item %zu differs\n", pass, k);
                return 1;
            }
    }
    if (batch.info().n_plans != 2) return 1;

    // serving: the cross products again, operands from the arrays' host copies
    auto pa = aether::detail::plane_view<double, 3>(reinterpret_cast<double*>(16), 0, 0);
    auto pb = aether::detail::plane_view<double, 3>(reinterpret_cast<double*>(32), 0, 0);
    gb300::Server srv(64ull << 20);
    const int cross = srv.add_shape({pa, pb}, pa.cross(pb), "f64", {3});
    srv.open();
    std::vector<uint64_t> tickets;
    std::vector<std::vector<double>> got(6);
    for (std::size_t k = 0; k < 6; ++k) {
        as[k]->download();   // the server reads the operands' host copies
        bs[k]->download();
        got[k].assign(3 * quantized_capacity(sizes[k]), 0.0);
        tickets.push_back(srv.submit(cross, sizes[k], {1000 + 2 * k, 1001 + 2 * k},
                                     {as[k]->hostView().data(), bs[k]->hostView().data()}, got[k].data()));
    }
    for (std::size_t k = 0; k < 6; ++k) {
        srv.wait(tickets[k]);
        auto r = refs[k]->hostView();
        for (int c = 0; c < 3; ++c)
            if (std::memcmp(&got[k][c * quantized_capacity(sizes[k])], r.data() + c * refs[k]->capacity(),
                            sizes[k] * sizeof(double)) != 0) {
                std::printf("served item %zu differs\n", k);
                return 1;
            }
    }
    std::printf("batch and serve ok\n");
    return 0;
}

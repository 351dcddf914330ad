// aether/array.h -- SoA arrays and their views.
//
// Array<T, Es...> (array/Array.h:82-364): n samples of a T-valued tensor of
// static component extents Es..., stored plane by plane: component c of
// sample i at c * capacity() + i, capacity() = n rounded up to 32 samples
// (array/Array.h:288-304). An Array owns a pinned host copy and a device copy
// (chunk/Chunk.h:111-260), both allocated through the C-ABI; upload() and
// download() move the whole capacity (array/Array.h:250-268).
//
// hostView() reads and writes the host copy with v(c..., i) (view/View.h:
// 234-246); deviceView() is an expression leaf over the device copy and the
// destination of an assignment: `d.deviceView() = a.deviceView() + ...;`
// evaluates the tree for every sample in one kernel (aether/eval.h).
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>

#include "aether/expr.h"
#include "aether_gb300.h"

namespace aether {

/** A raw cudaStream_t; nullptr is the legacy default stream. */
using Stream = void*;

namespace detail {

template <class T>
constexpr const char* dtype_name() {
    static_assert(std::is_same<T, double>::value || std::is_same<T, float>::value,
                  "aether arrays hold double or float");
    return std::is_same<T, double>::value ? "f64" : "f32";
}

inline std::string last_error() {
    const char* m = aether_last_error();
    return m ? m : "unknown error";
}

/** One chunk allocated through the C-ABI (chunk/Chunk.h:111-260). */
class Chunk {
public:
    Chunk() = default;
    Chunk(int kind, std::size_t bytes, const char* where) : kind_(kind), bytes_(bytes) {
        void* h = nullptr;
        void* p = nullptr;
        if (aether_chunk_alloc(kind, 0, bytes, nullptr, &h, &p) != AETHER_OK)
            throw Error::memory("Chunk::allocate", where, bytes, last_error());
        handle_.reset(h);
        ptr_ = p;
    }
    void* get() const { return ptr_; }
    std::size_t bytes() const { return bytes_; }
    int kind() const { return kind_; }

private:
    struct Release {
        void operator()(void* h) const {
            if (h) aether_chunk_release(h);
        }
    };
    std::unique_ptr<void, Release> handle_;
    void* ptr_ = nullptr;
    int kind_ = AETHER_MEM_CPU;
    std::size_t bytes_ = 0;
};

inline void copy(void* dst, int dst_kind, const void* src, int src_kind, std::size_t bytes, Stream s, const char* op) {
    if (aether_copy(dst_kind, 0, dst, src_kind, 0, src, bytes, s) != AETHER_OK)
        throw Error::memory(op, dst_kind == AETHER_MEM_DEVICE ? "device 0" : "host", bytes, last_error());
}

inline void sync(Stream s) {
    if (aether_stream_sync(0, s) != AETHER_OK) throw Error("stream_sync failed (" + last_error() + ")");
}

}  // namespace detail

/** A host view: element access v(c0, ..., i) over the pinned host copy. */
template <class T, std::size_t... Es>
class HostView {
public:
    HostView(T* data, std::size_t pitch, std::size_t n) : data_(data), pitch_(pitch), n_(n) {}
    template <class... I>
    T& operator()(I... idx) const {
        static_assert(sizeof...(I) == sizeof...(Es) + 1 || (sizeof...(Es) == 0 && sizeof...(I) == 1),
                      "one index per component extent, then the sample");
        const std::size_t ix[] = {std::size_t(idx)...};
        constexpr std::size_t ext[] = {Es..., 1};
        std::size_t c = 0;
        for (std::size_t k = 0; k + 1 < sizeof...(I); ++k) c = c * ext[k] + ix[k];
        return data_[c * pitch_ + ix[sizeof...(I) - 1]];
    }
    std::size_t samples() const { return n_; }
    std::size_t pitch() const { return pitch_; }
    T* data() const { return data_; }

private:
    T* data_;
    std::size_t pitch_, n_;
};

template <class T, std::size_t... Es>
class View;

/** A device view: an expression leaf and an assignment destination. */
template <class T, std::size_t... Es>
class View {
public:
    using element_type = T;
    static constexpr int comps = int((std::size_t(1) * ... * Es));

    View(T* data, std::size_t pitch, std::size_t n) : data_(data), pitch_(pitch), n_(n) {}

    static ir::Shape shape() { return ir::shape_of(extents<Es...>{}); }
    T* data() const { return data_; }
    std::size_t pitch() const { return pitch_; }
    std::size_t samples() const { return n_; }

    /** The view as an expression leaf (view/View.h:369-377). */
    Expr expr() const {
        auto n = std::make_shared<ir::Leaf>();
        n->ptr = data_;
        n->pitch = pitch_;
        n->dtype = detail::dtype_name<T>();
        n->shape = shape();
        return Expr(n);
    }
    operator Expr() const { return expr(); }

    /** Static component I of a vector view as a rank-0 view (View::component<I>,
     *  view/View.h:315-332). */
    template <std::size_t I>
    View<T> component() const {
        static_assert(sizeof...(Es) == 1, "component<I> of a vector view");
        return View<T>(data_ + I * pitch_, pitch_, n_);
    }

    // Assignment launches one kernel (expr/Assign.h:251-346); defined in aether/eval.h.
    View& operator=(const Expr& e);
    View& operator+=(const Expr& e);
    View& operator-=(const Expr& e);
    View& operator=(const View& o) { return *this = o.expr(); }

    // member surface forwarded to the expression
    Expr dot(const Expr& o) const { return expr().dot(o); }
    Expr squaredNorm() const { return expr().squaredNorm(); }
    Expr norm() const { return expr().norm(); }
    Expr cross(const Expr& o) const { return expr().cross(o); }
    Expr quatRotate(const Expr& v) const { return expr().quatRotate(v); }
    Expr quatMul(const Expr& o) const { return expr().quatMul(o); }
    Expr inverse() const { return expr().inverse(); }
    Expr det() const { return expr().det(); }
    Expr transpose() const { return expr().transpose(); }
    Expr unitVector() const { return expr().unitVector(); }

private:
    T* data_;
    std::size_t pitch_, n_;
};

// Arithmetic on views goes through their expressions.
#define AETHER_GB300_VIEW_OP(OPER)                                                                     \
    template <class T, std::size_t... Es>                                                              \
    Expr operator OPER(const View<T, Es...>& a, const Expr& b) { return a.expr() OPER b; }           \
    template <class T, std::size_t... Es>                                                              \
    Expr operator OPER(const Expr& a, const View<T, Es...>& b) { return a OPER b.expr(); }           \
    template <class T, std::size_t... Es, class U, std::size_t... Fs>                                  \
    Expr operator OPER(const View<T, Es...>& a, const View<U, Fs...>& b) { return a.expr() OPER b.expr(); } \
    template <class T, std::size_t... Es>                                                              \
    Expr operator OPER(const View<T, Es...>& a, double s) { return a.expr() OPER s; }                 \
    template <class T, std::size_t... Es>                                                              \
    Expr operator OPER(double s, const View<T, Es...>& a) { return s OPER a.expr(); }
AETHER_GB300_VIEW_OP(+)
AETHER_GB300_VIEW_OP(-)
AETHER_GB300_VIEW_OP(*)
#undef AETHER_GB300_VIEW_OP
template <class T, std::size_t... Es>
Expr operator/(const View<T, Es...>& a, double s) { return a.expr() / s; }
template <class T, std::size_t... Es>
Expr operator-(const View<T, Es...>& a) { return -a.expr(); }

/** Samples rounded up to the 32-sample capacity quantum. */
inline std::size_t quantized_capacity(std::size_t n) { return (n + 31) / 32 * 32; }

template <class T, std::size_t... Es>
class Array {
public:
    using element_type = T;
    using ViewT = View<T, Es...>;
    using HostViewT = HostView<T, Es...>;
    static constexpr std::size_t components = (std::size_t(1) * ... * Es);

    explicit Array(std::size_t n_samples)
        : n_(n_samples), cap_(quantized_capacity(n_samples)),
          host_(AETHER_MEM_PINNED, bytes_(), "host (pinned)"),
          dev_(AETHER_MEM_DEVICE, bytes_(), "device 0") {}

    std::size_t samples() const { return n_; }
    std::size_t capacity() const { return cap_; }
    std::size_t bytes() const { return bytes_(); }

    HostViewT hostView() { return HostViewT(static_cast<T*>(host_.get()), cap_, n_); }
    ViewT deviceView() { return ViewT(static_cast<T*>(dev_.get()), cap_, n_); }
    ViewT view() { return deviceView(); }

    /** Blocking host -> device copy of the whole capacity. */
    void upload() {
        upload(nullptr);
        detail::sync(nullptr);
    }
    void download() {
        download(nullptr);
        detail::sync(nullptr);
    }
    /** Stream-ordered copies (array/Array.h:266-268). */
    void upload(Stream s) { detail::copy(dev_.get(), AETHER_MEM_DEVICE, host_.get(), AETHER_MEM_PINNED, bytes_(), s, "upload"); }
    void download(Stream s) { detail::copy(host_.get(), AETHER_MEM_PINNED, dev_.get(), AETHER_MEM_DEVICE, bytes_(), s, "download"); }

private:
    std::size_t bytes_() const { return components * cap_ * sizeof(T); }
    std::size_t n_, cap_;
    detail::Chunk host_, dev_;
};

/** Batched views by shape (aether.h:234-260). */
template <class T>
using ScalarView = View<T>;
template <class T, std::size_t N>
using VecView = View<T, N>;
template <class T, std::size_t R, std::size_t C>
using MatView = View<T, R, C>;
using Vec3dView = VecView<double, 3>;
using Mat33dView = MatView<double, 3, 3>;

}  // namespace aether

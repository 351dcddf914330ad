// aether/reshape.h -- reshaping a view's sample mode (view/Reshape.h,
// view/MakeReshape.h).
//
// aether::reshaped<Ms...>(view) takes a layout_right view whose modes are
// static except the trailing sample mode and replaces that mode by the modes
// Ms..., exactly one of which is `dyn`: the product of the static Ms must
// divide view.samples() (an aether::Error otherwise), and the dynamic one
// takes the quotient. The result is a layout_right view over the same data
// (no copy), so element (c..., m...) is the flat element the row-major
// folding of the sample index names.
#pragma once

#include <cstddef>
#include <string>
#include <utility>

#include "aether/array.h"

namespace aether {

namespace detail {

template <class Prefix, std::size_t... Ms>
struct reshape_extents;
template <std::size_t... P, std::size_t... Ms>
struct reshape_extents<std::index_sequence<P...>, Ms...> {
    using type = extents<P..., Ms...>;
};

// The static modes before the sample mode of extents<Es...>.
template <std::size_t... Es, std::size_t... K>
constexpr auto leading_modes(std::index_sequence<K...>) {
    return std::index_sequence<pick<Es...>(K)...>{};
}
template <std::size_t... Es>
using leading_modes_t = decltype(leading_modes<Es...>(std::make_index_sequence<sizeof...(Es) - 1>{}));

}  // namespace detail

/** The trailing sample mode of `view` reshaped into Ms... (one of them dyn). */
template <std::size_t... Ms, class T, std::size_t... Es, bool Vo, bool RO>
View<T, typename detail::reshape_extents<detail::leading_modes_t<Es...>, Ms...>::type, layout_right, Vo, RO> reshaped(
    const View<T, extents<Es...>, layout_right, Vo, RO>& view) {
    static_assert(sizeof...(Es) >= 1, "reshaped: a view of rank >= 1");
    static_assert(detail::pick<Es...>(sizeof...(Es) - 1) == dyn, "reshaped: the trailing mode must be the sample mode");
    static_assert(detail::count_dyn<Es...>::value == 1, "reshaped: every mode before the sample mode must be static");
    static_assert(detail::count_dyn<Ms...>::value == 1, "reshaped<Ms...>: exactly one of Ms... must be dyn");
    using X = typename detail::reshape_extents<detail::leading_modes_t<Es...>, Ms...>::type;
    constexpr std::size_t fixed = ((Ms == dyn ? std::size_t(1) : Ms) * ... * std::size_t(1));
    const std::size_t samples = view.samples();
    if (samples % fixed != 0)
        throw Error::memory("reshaped", "view", samples * sizeof(T),
                            "static mode product " + std::to_string(fixed) + " does not divide samples()=" +
                                std::to_string(samples));
    return View<T, X, layout_right, Vo, RO>(view.data(), typename layout_right::template mapping<X>(X(samples / fixed)),
                                            view.device());
}

}  // namespace aether

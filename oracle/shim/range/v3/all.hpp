// Test infrastructure (oracle only): a minimal stand-in for the parts of
// range-v3 0.12 that the reference's join path names (views::enumerate,
// views::transform, views::join, ranges::to), mapped onto C++23 <ranges>.
// It lets the unmodified reference sources compile for the oracle build;
// nothing in the shipped library includes it.
#pragma once
#include <iterator>
#include <ranges>
#include <utility>

namespace ranges {
namespace views {
inline constexpr auto enumerate = std::views::enumerate;
inline constexpr auto transform = std::views::transform;
inline constexpr auto join      = std::views::join_with;
}  // namespace views

template <class C>
struct to_container_tag {};

// ranges::to<C>() — collects a range into container C.
template <class C>
constexpr to_container_tag<C> to() {
    return {};
}

template <std::ranges::input_range R, class C>
C operator|(R&& r, to_container_tag<C>) {
    C out;
    for (auto&& x : r) out.push_back(static_cast<typename C::value_type>(x));
    return out;
}
}  // namespace ranges

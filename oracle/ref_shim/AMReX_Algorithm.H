#pragma once
#include <algorithm>
namespace amrex {
template <class T> constexpr T const& max(T const& a, T const& b) { return std::max(a, b); }
template <class T> constexpr T const& min(T const& a, T const& b) { return std::min(a, b); }
}

#pragma once
#include "AMReX_REAL.H"
#include <stdexcept>
#include <string>
namespace amrex {
[[noreturn]] inline void Abort(std::string const& msg) { throw std::runtime_error(msg); }
[[noreturn]] inline void Abort(char const* msg) { throw std::runtime_error(msg); }
inline void Warning(std::string const&) {}
template <typename... T> inline void ignore_unused(T const&...) {}
}

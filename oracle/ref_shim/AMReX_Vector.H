#pragma once
#include <vector>
namespace amrex { template <class T> using Vector = std::vector<T>; }

#pragma once
#include <stdexcept>
#define AMREX_ALWAYS_ASSERT(x) do { if (!(x)) throw std::runtime_error("assert: " #x); } while (0)
#define AMREX_ASSERT(x) AMREX_ALWAYS_ASSERT(x)

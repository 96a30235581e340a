#pragma once
#include <string>
namespace amrex {
struct ParmParse {
    explicit ParmParse(std::string const& = std::string()) {}
    template <class T> bool query(char const*, T&) const { return false; }
};
}

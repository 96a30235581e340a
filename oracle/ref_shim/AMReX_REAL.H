// Minimal stand-in for the AMReX headers the reference's table, path, RNG and
// kinematics sources include.  Only used to compile those reference sources
// into the checker under oracle/_ref; never part of the shipped library.
#pragma once
namespace amrex {
using Real = double;
using ParticleReal = double;
using Long = long long;
}

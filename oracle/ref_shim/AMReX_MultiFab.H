#pragma once
#include "amrex_single_box.hpp"

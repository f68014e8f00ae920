// Definitions of the opaque handle types of the C ABI (include/sysu_cfd.h).
#pragma once

#include "solver.hpp"

struct sysu_case {
    sysu::Case cs;
};

struct sysu_solver {
    sysu::SimpleSolver *impl;
};

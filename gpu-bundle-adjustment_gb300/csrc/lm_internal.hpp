#pragma once
// Internal entry of the LM loop, shared by gba::solve_bal_gpu and the C ABI.

#include <chrono>

#include "gba/lm.hpp"

namespace gba {

class Solver;

// Runs the LM iterations on an already-built solver; t0 is the solve start
// used for the trajectory timestamps.
LMResult run_lm(Solver& s, const LMOptions& opts, std::chrono::steady_clock::time_point t0);

}  // namespace gba

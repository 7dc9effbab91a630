#pragma once
// Learned block-Jacobi correction: a per-camera MLP (BF16 weights, FP32
// accumulation) whose output corrects the Cholesky factor of each damped
// diagonal block S_cc used by the mixed-form PCG.

#include <string>

namespace gba {

class Solver;

class LearnedPreconditioner {
public:
    explicit LearnedPreconditioner(const std::string& path);
    ~LearnedPreconditioner();
    // Replaces the block-Jacobi factors in s.Pfac_ by the corrected factors.
    void correct_factors(Solver& s, double lambda);

    struct Impl;
    Impl* impl = nullptr;
};

}  // namespace gba

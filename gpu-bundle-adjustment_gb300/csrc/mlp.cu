// Learned block-Jacobi correction (per-camera MLP).

#include "common.cuh"
#include "mlp.hpp"
#include "solver.hpp"

namespace gba {

struct LearnedPreconditioner::Impl {};

LearnedPreconditioner::LearnedPreconditioner(const std::string&) {
    throw std::invalid_argument("learned preconditioner not available in this build");
}
LearnedPreconditioner::~LearnedPreconditioner() { delete impl; }
void LearnedPreconditioner::correct_factors(Solver&, double) {}

Solver::~Solver() { delete model_; }

void Solver::load_model(const std::string& path) {
    delete model_;
    model_ = nullptr;
    model_ = new LearnedPreconditioner(path);
}

}  // namespace gba

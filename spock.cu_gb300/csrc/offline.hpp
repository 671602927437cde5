// Offline cache of the dynamics projection and the AVaR nullspace projectors, computed on the
// GPU in FP64 (offline.cu).
#pragma once

#include <vector>

#include "problem.hpp"

namespace spock {

// Column-major per node, the layouts of dynamics_{P,K,lowCholesky,ABKTr,APB}.bt.
struct OfflineCache {
    std::vector<double> P, K, lowChol, ABKTr, APB;
};

// From the problem's [A B] per node and its tree; throws std::invalid_argument when a factor
// I + sum B'PB is not positive definite, std::runtime_error on a CUDA failure.
OfflineCache offlineDynamicsGpu(const HostProblem &p, int device);

// risk_NNtr: the projector I - S'(SS')^-1 S onto the kernel of each nonleaf node's padded AVaR
// matrix, (4E+1) x (4E+1) per nonleaf node, column-major.
std::vector<double> offlineNullspaceGpu(const HostProblem &p, int device);

}  // namespace spock

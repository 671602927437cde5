// Drives the C++ interface (include/spock_gb300.hpp) the way the reference's example programs
// drive theirs (examples/random/main.cu:41-70): tree -> problem -> builder -> cache -> solve.
//   wrapper_main load  <folder>                 sizes of the tree (host only)
//   wrapper_main bad   <folder>                 expects std::invalid_argument
//   wrapper_main solve <folder> <tol> <x0...>   FP64 runSpock, prints status, iterations, u_0
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "spock_gb300.hpp"

using namespace spock_gb300;

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    const char *mode = argv[1];
    if (!std::strcmp(mode, "bad")) {
        try {
            ScenarioTree<double> tree(argv[2]);
        } catch (const std::invalid_argument &e) {
            std::printf("invalid_argument %s\n", e.what());
            return 0;
        }
        return 1;
    }
    ScenarioTree<double> tree(argv[2]);
    ProblemData<double> data(tree);
    if (!std::strcmp(mode, "load")) {
        std::printf("%zu %zu %zu %zu %zu %zu %.17g\n", tree.numEvents(), tree.numNodes(), tree.numNonleafNodes(),
                    tree.numStages(), tree.numStates(), tree.numInputs(), data.stepSize());
        return 0;
    }
    if (!std::strcmp(mode, "solve") && argc >= 4) {
        const double tol = std::atof(argv[3]);
        std::vector<double> x0;
        for (int k = 4; k < argc; k++) x0.push_back(std::atof(argv[k]));
        CacheBuilder<double> builder(tree, data);
        Cache<double> cache = builder.tol(tol).maxIters(5000).enableDebug(false).build();
        const int status = cache.runSpock(x0);
        std::vector<double> u = cache.inputs();
        std::printf("%d %zu %s\n", status, cache.solveIter(), toString(status));
        for (size_t k = 0; k < tree.numInputs(); k++) std::printf("%.17g\n", u[k]);
        // Cache::getDual at the solution: the dual of T(z*) for z*'s own primal, which at a
        // converged point is within the tolerance of z*'s dual
        std::vector<double> z = cache.solution(), zp(z.begin(), z.begin() + (long)cache.sizePrimal());
        std::vector<double> dual = cache.getDual(zp);
        double gap = 0;
        for (size_t k = 0; k < dual.size(); k++) {
            const double e = std::fabs(dual[k] - z[cache.sizePrimal() + k]);
            gap = e > gap ? e : gap;
        }
        std::printf("getDual %.3g\n", gap);
        CacheBuilder<double> debugBuilder(tree, data);
        debugBuilder.enableDebug();  // the reference's default argument (cache.cuh:1204)
        return 0;
    }
    return 2;
}

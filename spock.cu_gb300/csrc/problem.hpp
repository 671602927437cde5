// Host-side problem data: everything a SPOCK solve reads, loaded from a data folder.
//
// The folder format is the one the reference's offline factory writes and its C++ loaders
// read (src/tree.cuh:102-179, src/problem.cuh:126-153, src/dynamics.cuh:40-72,
// src/costs.cuh:85-113/228-250/329-366, src/constraints.cuh:129-150/216-243/316-360,
// src/risks.cuh:26-33/81-97): `data.json` plus one `.bt` tensor per array.  Tensors are read
// as `_d` (FP64) when present and otherwise `_f` (FP32); index arrays are `_u` (uint64).
#pragma once

#include <string>
#include <vector>

namespace spock {

enum CostKind { kCostQuadratic = 0, kCostLinear = 1, kCostQuadraticPlusLinear = 2 };
// kConRectangleInputBall (nonleaf only, no reference counterpart): box bounds on x and the ball
// ||u||_2 <= nlRadius on the inputs; its dual block is [x; u] as for a rectangle.
enum ConstraintKind {
    kConNone = 0,
    kConRectangle = 1,
    kConPolyhedron = 2,
    kConPolyhedronWithIdentity = 3,
    kConRectangleInputBall = 4
};

struct HostProblem {
    std::string path;
    char dtype = 'd';  // suffix of the folder's floating-point tensors: 'd' (FP64) or 'f' (FP32)
    // tree (tree.cuh:48-76)
    long numEvents = 0, numNodes = 0, numNonleaf = 0, numLeaf = 0, numStages = 0;
    long nx = 0, nu = 0;
    std::vector<long> stages, ancestors, childFrom, numChildren, stageFrom, stageTo;
    std::vector<double> probabilities, condProbabilities;
    // problem (problem.cuh:383-398)
    bool affine = false, preconditioned = false;
    int costNonleaf = kCostQuadratic, costLeaf = kCostQuadratic;
    int conNonleaf = kConNone, conLeaf = kConNone;
    double alpha = 1., stepSize = 0.;
    long nullDim = 0, yDim = 0;
    std::vector<double> scaling;  // nx + nu, ones when not preconditioned
    // dynamics cache, column-major per node
    std::vector<double> BTr, AB, K, ABKTr, P, APB, lowChol, e, Pe;
    // costs
    std::vector<double> sqrtQ, sqrtR, q, r, translation, gradient;  // nonleaf, per node
    std::vector<double> leafSqrtQ, leafQ, leafTranslation, leafGradient;  // one set for all leaves
    // constraints: bounds laid out exactly like the dual block they bound
    std::vector<double> nlLower, nlUpper, lLower, lUpper, nlGamma, lGamma;
    long nlGammaRows = 0, lGammaRows = 0;
    double nlRadius = 0.;  // kConRectangleInputBall
    // risk
    std::vector<double> NNtr, b;
    // iterate layout (cache.cuh:481-497, 529-581)
    long sizeU = 0, sizeX = 0, sizeY = 0, sizeT = 0, sizeS = 0, sizePrim = 0;
    long sizeI = 0, sizeII = 0, sizeIII = 0, sizeIV = 0, sizeV = 0, sizeVI = 0, sizeDual = 0;
    long dimIV = 0, dimVI = 0, dimIII = 0, dimV = 0;  // per-node block sizes

    // Throws std::invalid_argument.  With withoutCache the offline cache (dynamics_P, _K,
    // _lowCholesky, _ABKTr, _APB, risk_NNtr) may be absent and is then zero, and stepSize may be
    // zero: the state of a folder whose problem data is written and whose cache is not yet.
    static HostProblem load(const std::string &folder, bool withoutCache = false);
    long sizeIterate() const { return sizePrim + sizeDual; }
    double minScaling() const;
};

// Write the offline cache of `p` (dynamics_P, _K, _lowCholesky, _ABKTr, _APB, risk_NNtr) into
// its folder with the folder's own suffix, and set the stepSize of its data.json to p.stepSize
// (the other keys are kept as they are).
void writeOfflineCache(const HostProblem &p);

}  // namespace spock

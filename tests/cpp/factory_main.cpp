// Test driver of the C++ problem generator (include/spock_gb300_factory.hpp).
//
//   factory_main data <spec_dir> <out_dir>   write the problem data only (host code)
//   factory_main full <spec_dir> <out_dir>   ... and the offline cache on GPU 0; prints the step
//   factory_main bad  <case>                 one invalid input; prints the exception's kind
//
// <spec_dir> holds spec.txt (one "key value" per line: tree markov|iid, horizon, stopping,
// nx, nu, events, dynamics linear|affine, cost, leaf, nlcon, lcon, alpha, precondition,
// scale, dtype, radius) and the input matrices as `_d.bt` tensors, one matrix per event:
// tree_P, tree_v / tree_d, dyn_A, dyn_B, dyn_c, cost_Q, cost_R, cost_q, cost_r, leaf_Q, leaf_q
// and the constraint bounds nl_* / l_* (lb, ub, G, glb, gub).
#include <spock_gb300_factory.hpp>

#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>

using namespace spock::factory;

namespace {

std::string dirOf(std::string d) { return d.back() == '/' ? d : d + "/"; }

std::vector<double> vec(const std::string &dir, const std::string &name) {
    uint64_t dims[3];
    return readTensor(dir + name + "_d.bt", dims);
}

// Matrix k of a (rows, cols, mats) tensor.
Matrix mat(const std::string &dir, const std::string &name, long k = 0) {
    uint64_t dims[3];
    const auto v = readTensor(dir + name + "_d.bt", dims);
    Matrix m((long)dims[0], (long)dims[1]);
    const size_t per = (size_t)(dims[0] * dims[1]);
    std::copy(v.begin() + (long)(per * (size_t)k), v.begin() + (long)(per * (size_t)(k + 1)), m.a.begin());
    return m;
}

std::vector<double> column(const std::string &dir, const std::string &name, long k) { return mat(dir, name, k).a; }

Constraint constraint(const std::string &dir, const std::string &kind, const std::string &p, long nu, double radius) {
    if (kind == "no") return Constraint::none();
    if (kind == "rectangle") return Constraint::rectangle(vec(dir, p + "lb"), vec(dir, p + "ub"));
    if (kind == "polyhedron") return Constraint::polyhedron(mat(dir, p + "G"), vec(dir, p + "glb"), vec(dir, p + "gub"));
    if (kind == "polyhedronWithIdentity")
        return Constraint::polyhedronWithIdentity(Constraint::rectangle(vec(dir, p + "lb"), vec(dir, p + "ub")),
                                                  Constraint::polyhedron(mat(dir, p + "G"), vec(dir, p + "glb"), vec(dir, p + "gub")));
    if (kind == "rectangleInputBall") return Constraint::rectangleInputBall(vec(dir, p + "lb"), vec(dir, p + "ub"), nu, radius);
    throw std::invalid_argument("unknown constraint kind " + kind);
}

ProblemFactory fromSpec(const std::string &dir, char &dtype) {
    std::map<std::string, std::string> s;
    std::ifstream f(dir + "spec.txt");
    std::string k, v;
    while (f >> k >> v) s[k] = v;
    const long N = std::stol(s.at("horizon")), tau = std::stol(s.at("stopping")), nx = std::stol(s.at("nx")),
               nu = std::stol(s.at("nu")), K = std::stol(s.at("events"));
    ScenarioTree tree = s.at("tree") == "markov" ? MarkovChain(mat(dir, "tree_P"), vec(dir, "tree_v"), N, tau).build()
                                                 : IidProcess(vec(dir, "tree_d"), N, tau).build();
    ProblemFactory fac(tree, nx, nu);
    std::vector<Dynamics> dyn;
    std::vector<Cost> cost;
    const std::string ck = s.at("cost"), lk = s.at("leaf");
    for (long e = 0; e < K; e++) {
        dyn.push_back(s.at("dynamics") == "affine" ? Dynamics::affine(mat(dir, "dyn_A", e), mat(dir, "dyn_B", e), column(dir, "dyn_c", e))
                                                   : Dynamics::linear(mat(dir, "dyn_A", e), mat(dir, "dyn_B", e)));
        if (ck == "quadratic") cost.push_back(Cost::quadratic(mat(dir, "cost_Q", e), mat(dir, "cost_R", e)));
        else if (ck == "quadraticPlusLinear")
            cost.push_back(Cost::quadraticPlusLinear(mat(dir, "cost_Q", e), column(dir, "cost_q", e), mat(dir, "cost_R", e),
                                                     column(dir, "cost_r", e)));
        else cost.push_back(Cost::linear(column(dir, "cost_q", e), column(dir, "cost_r", e)));
    }
    fac.withDynamicsEvents(dyn).withCostNonleafEvents(cost);
    if (lk == "quadratic") fac.withCostLeaf(Cost::quadraticLeaf(mat(dir, "leaf_Q")));
    else if (lk == "quadraticPlusLinear") fac.withCostLeaf(Cost::quadraticPlusLinearLeaf(mat(dir, "leaf_Q"), vec(dir, "leaf_q")));
    else fac.withCostLeaf(Cost::linearLeaf(vec(dir, "leaf_q")));
    const double radius = s.count("radius") ? std::stod(s.at("radius")) : 0.;
    fac.withConstraintNonleaf(constraint(dir, s.at("nlcon"), "nl_", nu, radius));
    fac.withConstraintLeaf(constraint(dir, s.at("lcon"), "l_", nu, radius));
    fac.withRisk(AVaR(std::stod(s.at("alpha"))));
    fac.withPreconditioning(s.at("precondition") == "1");
    if (s.count("scale")) fac.withCostScaling(std::stod(s.at("scale")));
    dtype = s.count("dtype") ? s.at("dtype")[0] : 'd';
    return fac;
}

int bad(const std::string &which) {
    try {
        Matrix P(2, 2);
        P(0, 0) = .5;
        P(0, 1) = .6;  // row sums to 1.1
        P(1, 1) = 1.;
        if (which == "markov") MarkovChain(P, {.5, .5}, 3).build();
        if (which == "iid") IidProcess({.5, .4}, 3).build();
        if (which == "stopping") IidProcess({.5, .5}, 3, 4).build();
        if (which == "horizon") MarkovChain(Matrix::identity(2), {.5, .5}, 0).build();
        if (which == "alpha") AVaR(1.5);
        if (which == "rectangle") Constraint::rectangle({1., 0.}, {0., 1.});
        if (which == "leafcost") {
            ScenarioTree t = IidProcess({.5, .5}, 2).build();
            ProblemFactory(t, 1, 1).withCostLeaf(Cost::quadratic(Matrix::identity(1), Matrix::identity(1)));
        }
        std::cout << "no exception\n";
    } catch (const std::invalid_argument &e) {
        std::cout << "invalid_argument " << e.what() << "\n";
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 3) {
        std::cerr << "usage: factory_main data|full <spec_dir> <out_dir> | bad <case>\n";
        return 2;
    }
    const std::string mode = argv[1];
    if (mode == "bad") return bad(argv[2]);
    if (argc < 4) return 2;
    try {
        char dtype = 'd';
        ProblemFactory fac = fromSpec(dirOf(argv[2]), dtype);
        if (mode == "data") {
            fac.writeProblemData(argv[3], dtype);
            std::cout << "ok\n";
        } else {
            std::printf("%.17g\n", fac.generateProblem(argv[3], dtype, 0));
        }
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    return 0;
}

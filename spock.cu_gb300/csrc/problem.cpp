// Data-folder loader for HostProblem (see problem.hpp for the format references).
#include "problem.hpp"

#include <cctype>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <sstream>
#include <stdexcept>

namespace spock {
namespace {

[[noreturn]] void fail(const std::string &msg) { throw std::invalid_argument(msg); }

// ---- minimal JSON: the data.json written by the factory is a flat object whose values are
// numbers, booleans, strings or one level of nested objects of strings/numbers.
struct Json {
    std::map<std::string, std::string> kv;  // "a" -> raw value, "a.b" -> raw nested value

    static Json parse(const std::string &text) {
        Json j;
        size_t i = 0;
        auto ws = [&]() { while (i < text.size() && std::isspace((unsigned char)text[i])) i++; };
        auto str = [&]() {
            if (text[i] != '"') fail("[data.json] expected string");
            size_t s = ++i;
            while (i < text.size() && text[i] != '"') i++;
            return text.substr(s, i++ - s);
        };
        auto scalar = [&]() {
            ws();
            if (text[i] == '"') return str();
            size_t s = i;
            while (i < text.size() && text[i] != ',' && text[i] != '}' && !std::isspace((unsigned char)text[i])) i++;
            return text.substr(s, i - s);
        };
        std::string prefix;
        ws();
        if (i >= text.size() || text[i] != '{') fail("[data.json] not an object");
        i++;
        int depth = 1;
        while (depth > 0) {
            ws();
            if (i >= text.size()) fail("[data.json] unexpected end of file");
            if (text[i] == ',') { i++; continue; }
            if (text[i] == '}') { depth--; i++; prefix.clear(); continue; }
            std::string key = str();
            ws();
            if (text[i] != ':') fail("[data.json] expected ':' after " + key);
            i++;
            ws();
            if (text[i] == '{') {
                if (depth > 1) fail("[data.json] nesting too deep");
                prefix = key + ".";
                depth++;
                i++;
                continue;
            }
            j.kv[prefix + key] = scalar();
        }
        return j;
    }
    const std::string &get(const std::string &k) const {
        auto it = kv.find(k);
        if (it == kv.end()) fail("[data.json] missing key '" + k + "'");
        return it->second;
    }
    long integer(const std::string &k) const { return std::stol(get(k)); }
    double number(const std::string &k) const { return std::stod(get(k)); }
    bool boolean(const std::string &k) const {
        const auto &v = get(k);
        if (v == "true") return true;
        if (v == "false") return false;
        fail("[data.json] key '" + k + "' is not a boolean");
    }
};

struct Tensor {
    uint64_t rows = 0, cols = 0, mats = 0;
    std::vector<double> data;
    size_t numel() const { return (size_t)(rows * cols * mats); }
};

bool exists(const std::string &fn) { return std::ifstream(fn).good(); }

std::vector<char> slurp(const std::string &fn) {
    std::ifstream f(fn, std::ios::binary);
    if (!f) fail("cannot open " + fn);
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

// `.bt`: uint64 rows, cols, mats, then rows*cols*mats values, column-major per matrix.
Tensor readTensor(const std::string &dir, const std::string &name) {
    std::string fn = dir + name + "_d.bt";
    int bytes = 8;
    if (!exists(fn)) {
        fn = dir + name + "_f.bt";
        bytes = 4;
    }
    auto buf = slurp(fn);
    Tensor t;
    if (buf.size() < 24) fail("[" + fn + "] truncated header");
    std::memcpy(&t.rows, buf.data(), 8);
    std::memcpy(&t.cols, buf.data() + 8, 8);
    std::memcpy(&t.mats, buf.data() + 16, 8);
    const size_t n = t.numel();
    if (buf.size() != 24 + n * (size_t)bytes)
        fail("[" + fn + "] size " + std::to_string(buf.size()) + " does not match dims");
    t.data.resize(n);
    for (size_t k = 0; k < n; k++) {
        if (bytes == 8) std::memcpy(&t.data[k], buf.data() + 24 + 8 * k, 8);
        else {
            float v;
            std::memcpy(&v, buf.data() + 24 + 4 * k, 4);
            t.data[k] = v;
        }
    }
    return t;
}

std::vector<long> readIndex(const std::string &dir, const std::string &name) {
    const std::string fn = dir + name + "_u.bt";
    auto buf = slurp(fn);
    if (buf.size() < 24) fail("[" + fn + "] truncated header");
    uint64_t h[3];
    std::memcpy(h, buf.data(), 24);
    const size_t n = (size_t)(h[0] * h[1] * h[2]);
    if (buf.size() != 24 + 8 * n) fail("[" + fn + "] size does not match dims");
    std::vector<long> out(n);
    for (size_t k = 0; k < n; k++) {
        uint64_t v;
        std::memcpy(&v, buf.data() + 24 + 8 * k, 8);
        out[k] = (v == std::numeric_limits<uint64_t>::max()) ? -1 : (long)v;
    }
    return out;
}

std::vector<double> expect(const Tensor &t, size_t n, const std::string &what) {
    if (t.numel() != n)
        fail("[" + what + "] has " + std::to_string(t.numel()) + " entries, expected " + std::to_string(n));
    return t.data;
}

int costKind(const std::string &s) {
    if (s == "quadratic") return kCostQuadratic;
    if (s == "linear") return kCostLinear;
    if (s == "quadraticPlusLinear") return kCostQuadraticPlusLinear;
    fail("[parseCost] Cost type " + s + " is not supported. Supported types include: quadratic, linear, quadraticPlusLinear");
}

int conKind(const std::string &s) {
    if (s == "no") return kConNone;
    if (s == "rectangle") return kConRectangle;
    if (s == "polyhedron") return kConPolyhedron;
    if (s == "polyhedronWithIdentity") return kConPolyhedronWithIdentity;
    if (s == "rectangleInputBall") return kConRectangleInputBall;
    fail("[parseConstraint] Constraint type " + s + " is not supported. Supported types include: none, rectangle, polyhedron, polyhedronWithIdentity, rectangleInputBall");
}

// Bounds for one constraint part laid out like its dual block (constraints.cuh:32-37, 129-150,
// 216-243, 316-360); the root's state bounds of a nonleaf rectangle are +-inf (constraints.cuh:142-148).
// Rectangle bounds laid out like the dual block; the root's states are free (constraints.cuh:142-148).
void loadConstraintRect(HostProblem &p, const std::string &dir, const std::string &part, long dpn, long nodes,
                        std::vector<double> &lo, std::vector<double> &hi, long &per) {
    const std::vector<double> ilb = expect(readTensor(dir, part + "ILB"), dpn, part + "ILB");
    const std::vector<double> iub = expect(readTensor(dir, part + "IUB"), dpn, part + "IUB");
    const double inf = std::numeric_limits<double>::infinity();
    per = dpn;
    lo.assign(per * nodes, 0.);
    hi.assign(per * nodes, 0.);
    for (long i = 0; i < nodes; i++)
        for (long k = 0; k < dpn; k++) {
            const bool freeRoot = i == 0 && k < p.nx;
            lo[i * dpn + k] = freeRoot ? -inf : ilb[k];
            hi[i * dpn + k] = freeRoot ? inf : iub[k];
        }
}

void loadConstraint(HostProblem &p, const std::string &dir, bool leaf) {
    const std::string part = leaf ? "leafConstraint" : "nonleafConstraint";
    const int kind = leaf ? p.conLeaf : p.conNonleaf;
    const long dpn = leaf ? p.nx : p.nx + p.nu;
    const long nodes = leaf ? p.numLeaf : p.numNonleaf;
    auto &lo = leaf ? p.lLower : p.nlLower;
    auto &hi = leaf ? p.lUpper : p.nlUpper;
    auto &G = leaf ? p.lGamma : p.nlGamma;
    long &gRows = leaf ? p.lGammaRows : p.nlGammaRows;
    long &per = leaf ? p.dimV : p.dimIII;
    std::vector<double> ilb, iub, glb, gub;
    gRows = 0;
    if (kind == kConNone) { per = 0; return; }
    if (kind == kConRectangleInputBall) {
        if (leaf) fail("[" + part + "] an input ball constrains nonleaf nodes only");
        p.nlRadius = expect(readTensor(dir, part + "Radius"), 1, part + "Radius")[0];
        if (!(p.nlRadius > 0)) fail("[" + part + "Radius] must be positive");
        loadConstraintRect(p, dir, part, dpn, nodes, lo, hi, per);
        return;
    }
    if (kind == kConRectangle || kind == kConPolyhedronWithIdentity) {
        ilb = expect(readTensor(dir, part + "ILB"), dpn, part + "ILB");
        iub = expect(readTensor(dir, part + "IUB"), dpn, part + "IUB");
    }
    if (kind == kConPolyhedron || kind == kConPolyhedronWithIdentity) {
        Tensor g = readTensor(dir, part + "Gamma");
        if ((long)g.cols != dpn) fail("[" + part + "Gamma] wrong number of columns");
        gRows = (long)g.rows;
        G = g.data;
        glb = expect(readTensor(dir, part + "GLB"), gRows, part + "GLB");
        gub = expect(readTensor(dir, part + "GUB"), gRows, part + "GUB");
    }
    per = (kind == kConRectangle ? dpn : 0) + (kind == kConPolyhedron ? gRows : 0) +
          (kind == kConPolyhedronWithIdentity ? dpn + gRows : 0);
    lo.assign(per * nodes, 0.);
    hi.assign(per * nodes, 0.);
    const double inf = std::numeric_limits<double>::infinity();
    if (kind == kConRectangle) {
        for (long i = 0; i < nodes; i++)
            for (long k = 0; k < dpn; k++) {
                const bool freeRoot = !leaf && i == 0 && k < p.nx;
                lo[i * dpn + k] = freeRoot ? -inf : ilb[k];
                hi[i * dpn + k] = freeRoot ? inf : iub[k];
            }
    } else if (kind == kConPolyhedron) {
        for (long i = 0; i < nodes; i++)
            for (long k = 0; k < gRows; k++) { lo[i * gRows + k] = glb[k]; hi[i * gRows + k] = gub[k]; }
    } else {
        for (long i = 0; i < nodes; i++) {
            for (long k = 0; k < dpn; k++) { lo[i * dpn + k] = ilb[k]; hi[i * dpn + k] = iub[k]; }
            for (long k = 0; k < gRows; k++) {
                lo[nodes * dpn + i * gRows + k] = glb[k];
                hi[nodes * dpn + i * gRows + k] = gub[k];
            }
        }
    }
}

}  // namespace

double HostProblem::minScaling() const { return *std::min_element(scaling.begin(), scaling.end()); }

HostProblem HostProblem::load(const std::string &folder, bool withoutCache) {
    HostProblem p;
    std::string dir = folder;
    if (!dir.empty() && dir.back() != '/') dir += '/';
    p.path = dir;
    const std::string jsonFile = dir + "data.json";
    if (!exists(jsonFile)) fail("[Tree] cannot open " + jsonFile);
    auto raw = slurp(jsonFile);
    const Json js = Json::parse(std::string(raw.begin(), raw.end()));
    p.numEvents = js.integer("numEvents");
    p.numNonleaf = js.integer("numNonleafNodes");
    p.numNodes = js.integer("numNodes");
    p.numStages = js.integer("numStages");
    p.nx = js.integer("numStates");
    p.nu = js.integer("numInputs");
    p.numLeaf = p.numNodes - p.numNonleaf;
    p.nullDim = js.integer("rowsNNtr");
    p.yDim = p.nullDim - 2 * p.numEvents;
    p.stepSize = js.number("stepSize");
    p.preconditioned = js.boolean("preconditioned");
    const std::string dyn = js.get("dynamics.type");
    if (dyn == "linear") p.affine = false;
    else if (dyn == "affine") p.affine = true;
    else fail("[parseDynamics] Dynamics type " + dyn + " is not supported. Supported types include: linear, affine");
    p.costNonleaf = costKind(js.get("cost.nonleaf"));
    p.costLeaf = costKind(js.get("cost.leaf"));
    p.conNonleaf = conKind(js.get("constraint.nonleaf"));
    p.conLeaf = conKind(js.get("constraint.leaf"));
    const std::string risk = js.get("risk.type");
    if (risk != "avar") fail("[parseRisk] Risk type " + risk + " is not supported. Supported types include: avar");
    p.alpha = js.kv.count("risk.alpha") ? js.number("risk.alpha") : 1.;
    if (p.numNodes < 2 || p.numNonleaf < 1 || p.numStages < 2 || p.nx < 1 || p.nu < 1 || p.numEvents < 1)
        fail("[Tree] invalid sizes in data.json");
    if (!(p.stepSize > 0) && !(withoutCache && p.stepSize == 0)) fail("[Problem] stepSize must be positive");
    p.dtype = exists(dir + "dynamics_AB_d.bt") ? 'd' : 'f';

    const long n = p.numNodes, nnl = p.numNonleaf, nx = p.nx, nu = p.nu;
    p.stages = readIndex(dir, "stages");
    p.ancestors = readIndex(dir, "ancestors");
    p.childFrom = readIndex(dir, "childrenFrom");
    p.numChildren = readIndex(dir, "numChildren");
    p.stageFrom = readIndex(dir, "stageFrom");
    p.stageTo = readIndex(dir, "stageTo");
    if ((long)p.ancestors.size() != n || (long)p.childFrom.size() != nnl || (long)p.numChildren.size() != nnl ||
        (long)p.stageFrom.size() != p.numStages || (long)p.stageTo.size() != p.numStages)
        fail("[Tree] index tensors do not match data.json sizes");
    for (long i = 0; i < nnl; i++) {
        const long c0 = p.childFrom[i], nc = p.numChildren[i];
        if (nc < 1 || nc > p.numEvents || c0 < 1 || c0 + nc > n) fail("[Tree] invalid children of node " + std::to_string(i));
        for (long j = c0; j < c0 + nc; j++)
            if (p.ancestors[j] != i) fail("[Tree] children/ancestors mismatch at node " + std::to_string(j));
    }
    for (long j = 1; j < n; j++)
        if (p.ancestors[j] < 0 || p.ancestors[j] >= j) fail("[Tree] invalid ancestor of node " + std::to_string(j));
    p.probabilities = expect(readTensor(dir, "probabilities"), n, "probabilities");
    p.condProbabilities = expect(readTensor(dir, "conditionalProbabilities"), n, "conditionalProbabilities");

    p.BTr = expect(readTensor(dir, "dynamics_BTr"), nu * nx * n, "dynamics_BTr");
    p.AB = expect(readTensor(dir, "dynamics_AB"), nx * (nx + nu) * n, "dynamics_AB");
    // the offline cache: zeros in place of files not yet written when withoutCache is set
    auto cache = [&](const std::string &name, long count) {
        if (withoutCache && !exists(dir + name + "_d.bt") && !exists(dir + name + "_f.bt"))
            return std::vector<double>((size_t)count, 0.);
        return expect(readTensor(dir, name), count, name);
    };
    p.K = cache("dynamics_K", nu * nx * nnl);
    p.ABKTr = cache("dynamics_ABKTr", nx * nx * n);
    p.P = cache("dynamics_P", nx * nx * n);
    p.APB = cache("dynamics_APB", nx * nu * n);
    p.lowChol = cache("dynamics_lowCholesky", nu * nu * nnl);
    if (p.affine) {
        p.e = expect(readTensor(dir, "dynamics_c"), nx * n, "dynamics_c");
        p.Pe.assign(nx * n, 0.);  // Pe = P e per node (dynamics.cuh:236)
        for (long j = 0; j < n; j++)
            for (long c = 0; c < nx; c++)
                for (long r = 0; r < nx; r++) p.Pe[j * nx + r] += p.P[j * nx * nx + c * nx + r] * p.e[j * nx + c];
    }
    if (p.costNonleaf == kCostLinear) {
        p.gradient = expect(readTensor(dir, "nonleafCost_gradient"), (nx + nu) * n, "nonleafCost_gradient");
    } else {
        p.sqrtQ = expect(readTensor(dir, "nonleafCost_sqrtQ"), nx * nx * n, "nonleafCost_sqrtQ");
        p.sqrtR = expect(readTensor(dir, "nonleafCost_sqrtR"), nu * nu * n, "nonleafCost_sqrtR");
        p.translation = expect(readTensor(dir, "nonleafCost_translation"), (nx + nu + 2) * n, "nonleafCost_translation");
        if (p.costNonleaf == kCostQuadraticPlusLinear) {
            p.q = expect(readTensor(dir, "nonleafCost_q"), nx * n, "nonleafCost_q");
            p.r = expect(readTensor(dir, "nonleafCost_r"), nu * n, "nonleafCost_r");
        }
    }
    if (p.costLeaf == kCostLinear) {
        p.leafGradient = expect(readTensor(dir, "leafCost_gradient"), nx, "leafCost_gradient");
    } else {
        p.leafSqrtQ = expect(readTensor(dir, "leafCost_sqrtQ"), nx * nx, "leafCost_sqrtQ");
        p.leafTranslation = expect(readTensor(dir, "leafCost_translation"), nx + 2, "leafCost_translation");
        if (p.costLeaf == kCostQuadraticPlusLinear) p.leafQ = expect(readTensor(dir, "leafCost_q"), nx, "leafCost_q");
    }
    loadConstraint(p, dir, false);
    loadConstraint(p, dir, true);
    p.NNtr = cache("risk_NNtr", p.nullDim * p.nullDim * nnl);
    p.b = expect(readTensor(dir, "risk_b"), p.yDim * nnl, "risk_b");
    if (p.preconditioned) p.scaling = expect(readTensor(dir, "scaling"), nx + nu, "scaling");
    else p.scaling.assign(nx + nu, 1.);
    for (double s : p.scaling)
        if (!(s > 0)) fail("[Problem] preconditioning scaling must be positive");

    p.sizeU = nu * nnl;
    p.sizeX = nx * n;
    p.sizeY = p.yDim * nnl;
    p.sizeT = n;
    p.sizeS = n;
    p.sizePrim = p.sizeU + p.sizeX + p.sizeY + p.sizeT + p.sizeS;
    p.dimIV = p.costNonleaf == kCostLinear ? 2 : nx + nu + 2;
    p.dimVI = p.costLeaf == kCostLinear ? 2 : nx + 2;
    p.sizeI = p.yDim * nnl;
    p.sizeII = nnl;
    p.sizeIII = p.dimIII * nnl;
    p.sizeIV = p.dimIV * n;
    p.sizeV = p.dimV * p.numLeaf;
    p.sizeVI = p.dimVI * p.numLeaf;
    p.sizeDual = p.sizeI + p.sizeII + p.sizeIII + p.sizeIV + p.sizeV + p.sizeVI;
    return p;
}

namespace {

void writeTensor(const std::string &dir, const std::string &name, char dt, const std::vector<double> &v,
                 uint64_t rows, uint64_t cols, uint64_t mats) {
    if ((size_t)(rows * cols * mats) != v.size()) fail("[" + name + "] size does not match its dims");
    const std::string fn = dir + name + "_" + dt + ".bt";
    std::ofstream f(fn, std::ios::binary | std::ios::trunc);
    if (!f) fail("cannot write " + fn);
    const uint64_t h[3] = {rows, cols, mats};
    f.write(reinterpret_cast<const char *>(h), sizeof h);
    if (dt == 'd') {
        f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(double)));
    } else {
        std::vector<float> w(v.begin(), v.end());
        f.write(reinterpret_cast<const char *>(w.data()), (std::streamsize)(w.size() * sizeof(float)));
    }
    if (!f) fail("cannot write " + fn);
}

}  // namespace

void writeOfflineCache(const HostProblem &p) {
    const std::string &dir = p.path;
    const uint64_t n = p.numNodes, nnl = p.numNonleaf, nx = p.nx, nu = p.nu, nd = p.nullDim;
    writeTensor(dir, "dynamics_P", p.dtype, p.P, nx, nx, n);
    writeTensor(dir, "dynamics_K", p.dtype, p.K, nu, nx, nnl);
    writeTensor(dir, "dynamics_lowCholesky", p.dtype, p.lowChol, nu, nu, nnl);
    writeTensor(dir, "dynamics_ABKTr", p.dtype, p.ABKTr, nx, nx, n);
    writeTensor(dir, "dynamics_APB", p.dtype, p.APB, nx, nu, n);
    writeTensor(dir, "risk_NNtr", p.dtype, p.NNtr, nd, nd, nnl);
    // data.json: replace the value of "stepSize" in place
    const std::string fn = dir + "data.json";
    auto raw = slurp(fn);
    std::string text(raw.begin(), raw.end());
    size_t k = text.find("\"stepSize\"");
    if (k == std::string::npos) fail("[data.json] missing key 'stepSize'");
    k = text.find(':', k);
    if (k == std::string::npos) fail("[data.json] malformed stepSize");
    size_t a = k + 1;
    while (a < text.size() && std::isspace((unsigned char)text[a])) a++;
    size_t b = a;
    while (b < text.size() && text[b] != ',' && text[b] != '}' && !std::isspace((unsigned char)text[b])) b++;
    char num[64];
    std::snprintf(num, sizeof num, "%.17g", p.stepSize);
    text.replace(a, b - a, num);
    std::ofstream f(fn, std::ios::binary | std::ios::trunc);
    if (!f) fail("cannot write " + fn);
    f << text;
    if (!f) fail("cannot write " + fn);
}

}  // namespace spock

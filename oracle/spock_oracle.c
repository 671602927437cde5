/*
 * FP64 CPU oracle for the SPOCK solve -- TEST INFRASTRUCTURE ONLY (see spock_oracle.h).
 *
 * Restates, in plain C and double precision, the algorithm of ruairimoran/spock.cu:
 *   - file formats: data.json keys (api/python/spock/jinja2.py:1-33), `.bt` tensors
 *     (3 x uint64 dims + column-major payload, tests/julia/modelFactory/src/modelFactory.jl:26-60);
 *   - L and L* (src/operator.cuh:40-82, src/costs.cuh:126-195, 261-292, 379-458,
 *     src/constraints.cuh:96-108, 158-190, 251-285, 386-425), written with the semantics of the
 *     reference's Python operators (api/python/spock/problem.py:273-365, build.py:257-292,
 *     411-441, 592-634, 890-1014) that its operator fixtures were generated from;
 *   - the dynamics projection (src/dynamics.cuh:74-174), the AVaR kernel projection
 *     (src/cache.cuh:650-676), the dual projections (src/cache.cuh:678-698,
 *     src/definitions.cu:38-52, 301-443, src/risks.cuh:81-106);
 *   - the CP step (src/cache.cuh:748-801), M inner product (cache.cuh:721-742), error check
 *     (cache.cuh:909-961), Anderson direction (cache.cuh:860-904) and the SuperMann / CP loops
 *     (cache.cuh:966-1132);
 *   - the offline cache (problem.py:192-231) and step size (problem.py:402-417).
 * On request it also emulates single precision (or_set_emulation, spock_oracle.h), to explain
 * the iteration counts of the FP32 GPU path; mode 0, the default, is the plain FP64 restatement.
 */
#include "spock_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

enum { COST_QUAD = 0, COST_LIN = 1, COST_QPL = 2 };
/* CON_RECTBALL (nonleaf only, no counterpart in the reference): a box on [x; u] with infinite
 * input bounds, plus ||u||_2 <= radius at every nonleaf node. */
enum { CON_NO = 0, CON_RECT = 1, CON_POLY = 2, CON_POLYID = 3, CON_RECTBALL = 4 };

struct OrProblem {
    long ne, n, nnl, nl, ns, nx, nu, nxu;
    long *stages, *anc, *chFrom, *numCh, *stageFrom, *stageTo;
    double *prob, *cprob;
    int affine, costNl, costL, conNl, conL, precond;
    double alpha, step;
    double nlRadius; /* CON_RECTBALL */
    double *scaling;
    long nullDim, yDim;
    /* dynamics (per node) */
    double *BTr, *AB, *K, *ABKTr, *P, *APB, *chol, *e, *Pe;
    /* nonleaf cost (per node, incl. root) */
    double *nlSqrtQ, *nlSqrtR, *nlq, *nlr, *nlTrans, *nlGrad;
    /* leaf cost (one set, shared by all leaves) */
    double *lSqrtQ, *lq, *lTrans, *lGrad;
    /* constraints: bounds laid out exactly like the dual block */
    double *nlLb, *nlUb, *lLb, *lUb, *nlGamma, *lGamma;
    long nlGRows, lGRows;
    /* risk */
    double *NNtr, *b;
    /* sizes and offsets */
    long sU, sX, sY, sT, sS, sPrim, sI, sII, sIII, sIV, sV, sVI, sDual, sZ;
    long oX, oY, oT, oS, oII, oIII, oIV, oV, oVI;
    long dIV, dVI;
};

static char g_err[2048];

/* FP32 emulation mode (spock_oracle.h, OR_EMU_*); 0 keeps every operation in double. */
static int g_emu = 0;
void or_set_emulation(int mode) { g_emu = mode; }
/* Nonzero while a region whose products OR_EMU_ACCX_* exempts from OR_EMU_ACC runs (per thread:
 * the batch solves run one instance per thread). */
static __thread int g_exact = 0;
static void r32(double *v, long n) {
    for (long i = 0; i < n; i++) v[i] = (double)(float)v[i];
}
#define EMU_VEC(v, n) do { if (g_emu & OR_EMU_VEC) r32((v), (n)); } while (0)

const char *or_last_error(void) { return g_err; }

#define FAIL(...) do { snprintf(g_err, sizeof g_err, __VA_ARGS__); goto fail; } while (0)

/* ------------------------------------------------------------------ file I/O */

static char *slurp(const char *fn, long *len) {
    FILE *f = fopen(fn, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *buf = (char *)malloc((size_t)n + 1);
    if (buf && fread(buf, 1, (size_t)n, f) != (size_t)n) { free(buf); buf = NULL; }
    fclose(f);
    if (buf) buf[n] = 0;
    if (len) *len = n;
    return buf;
}

/* Read a .bt tensor; kind 'd' (double) or 'u' (uint64 -> long). Returns element count or -1. */
static long read_bt(const char *dir, const char *name, char kind, void **out, long dims[3]) {
    char fn[1024];
    snprintf(fn, sizeof fn, "%s%s_%c.bt", dir, name, kind);
    long len = 0;
    char *buf = slurp(fn, &len);
    if (!buf) return -1;
    if (len < 24) { free(buf); return -1; }
    uint64_t h[3];
    memcpy(h, buf, 24);
    long n = (long)(h[0] * h[1] * h[2]);
    if (len != 24 + n * 8) { free(buf); return -1; }
    if (dims) { dims[0] = (long)h[0]; dims[1] = (long)h[1]; dims[2] = (long)h[2]; }
    if (kind == 'd') {
        double *a = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        memcpy(a, buf + 24, (size_t)n * 8);
        if (g_emu & OR_EMU_DATA) r32(a, n);
        *out = a;
    } else {
        long *a = (long *)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
        for (long i = 0; i < n; i++) {
            uint64_t v;
            memcpy(&v, buf + 24 + 8 * i, 8);
            a[i] = (v == UINT64_MAX) ? -1 : (long)v;
        }
        *out = a;
    }
    free(buf);
    return n;
}

static const char *json_find(const char *js, const char *key) {
    char pat[128];
    snprintf(pat, sizeof pat, "\"%s\"", key);
    const char *p = strstr(js, pat);
    if (!p) return NULL;
    p += strlen(pat);
    while (*p && *p != ':') p++;
    return *p ? p + 1 : NULL;
}

static int json_num(const char *js, const char *key, double *v) {
    const char *p = json_find(js, key);
    if (!p) return 0;
    *v = strtod(p, NULL);
    return 1;
}

static int json_str(const char *js, const char *key, char *out, size_t cap) {
    const char *p = json_find(js, key);
    if (!p) return 0;
    while (*p && *p != '"') p++;
    if (!*p) return 0;
    p++;
    size_t i = 0;
    while (*p && *p != '"' && i + 1 < cap) out[i++] = *p++;
    out[i] = 0;
    return 1;
}

/* value of `sub` inside the object that follows `obj` */
static int json_sub_str(const char *js, const char *obj, const char *sub, char *out, size_t cap) {
    const char *p = json_find(js, obj);
    if (!p) return 0;
    const char *end = strchr(p, '}');
    if (!end) return 0;
    size_t n = (size_t)(end - p);
    char *tmp = (char *)malloc(n + 1);
    memcpy(tmp, p, n);
    tmp[n] = 0;
    int ok = json_str(tmp, sub, out, cap);
    free(tmp);
    return ok;
}

static int parse_cost(const char *s) {
    if (!strcmp(s, "quadratic")) return COST_QUAD;
    if (!strcmp(s, "linear")) return COST_LIN;
    if (!strcmp(s, "quadraticPlusLinear")) return COST_QPL;
    return -1;
}

static int parse_con(const char *s) {
    if (!strcmp(s, "no")) return CON_NO;
    if (!strcmp(s, "rectangle")) return CON_RECT;
    if (!strcmp(s, "polyhedron")) return CON_POLY;
    if (!strcmp(s, "polyhedronWithIdentity")) return CON_POLYID;
    if (!strcmp(s, "rectangleInputBall")) return CON_RECTBALL;
    return -1;
}

void or_free(OrProblem *p) {
    if (!p) return;
    void *ptrs[] = {p->stages, p->anc, p->chFrom, p->numCh, p->stageFrom, p->stageTo, p->prob, p->cprob,
                    p->scaling, p->BTr, p->AB, p->K, p->ABKTr, p->P, p->APB, p->chol, p->e, p->Pe,
                    p->nlSqrtQ, p->nlSqrtR, p->nlq, p->nlr, p->nlTrans, p->nlGrad, p->lSqrtQ, p->lq,
                    p->lTrans, p->lGrad, p->nlLb, p->nlUb, p->lLb, p->lUb, p->nlGamma, p->lGamma,
                    p->NNtr, p->b};
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) free(ptrs[i]);
    free(p);
}

#define NEED(expr, what) do { if ((expr) < 0) FAIL("cannot read %s", what); } while (0)

/* Build bounds for a constraint block (constraints.cuh:129-150, 216-243, 316-360). */
static int load_constraint(OrProblem *p, const char *dir, int leaf, int type, long nodes,
                           double **lbOut, double **ubOut, double **gOut, long *gRows, long *size) {
    const char *part = leaf ? "leafConstraint" : "nonleafConstraint";
    char nm[128];
    long dpn = leaf ? p->nx : p->nxu;
    double *ilb = NULL, *iub = NULL, *g = NULL, *glb = NULL, *gub = NULL;
    long dims[3];
    *gRows = 0;
    *size = 0;
    *lbOut = *ubOut = *gOut = NULL;
    if (type == CON_NO) return 0;
    if (type == CON_RECTBALL) {
        double *rad = NULL;
        if (leaf) return -1;
        snprintf(nm, sizeof nm, "%sRadius", part);
        if (read_bt(dir, nm, 'd', (void **)&rad, dims) != 1) return -1;
        p->nlRadius = rad[0];
        free(rad);
        type = CON_RECT; /* bounds exactly as a rectangle */
    }
    if (type == CON_RECT || type == CON_POLYID) {
        snprintf(nm, sizeof nm, "%sILB", part);
        if (read_bt(dir, nm, 'd', (void **)&ilb, dims) != dpn) return -1;
        snprintf(nm, sizeof nm, "%sIUB", part);
        if (read_bt(dir, nm, 'd', (void **)&iub, dims) != dpn) return -1;
    }
    if (type == CON_POLY || type == CON_POLYID) {
        snprintf(nm, sizeof nm, "%sGamma", part);
        if (read_bt(dir, nm, 'd', (void **)&g, dims) < 0) return -1;
        if (dims[1] != dpn) return -1;
        *gRows = dims[0];
        snprintf(nm, sizeof nm, "%sGLB", part);
        if (read_bt(dir, nm, 'd', (void **)&glb, dims) != *gRows) return -1;
        snprintf(nm, sizeof nm, "%sGUB", part);
        if (read_bt(dir, nm, 'd', (void **)&gub, dims) != *gRows) return -1;
    }
    long per = (type == CON_RECT ? dpn : 0) + (type == CON_POLY ? *gRows : 0) +
               (type == CON_POLYID ? dpn + *gRows : 0);
    *size = per * nodes;
    double *lb = (double *)malloc(sizeof(double) * (size_t)(*size));
    double *ub = (double *)malloc(sizeof(double) * (size_t)(*size));
    if (type == CON_RECT) {
        for (long i = 0; i < nodes; i++)
            for (long k = 0; k < dpn; k++) {
                lb[i * dpn + k] = ilb[k];
                ub[i * dpn + k] = iub[k];
                if (!leaf && i == 0 && k < p->nx) { lb[k] = -INFINITY; ub[k] = INFINITY; }
            }
    } else if (type == CON_POLY) {
        for (long i = 0; i < nodes; i++)
            for (long k = 0; k < *gRows; k++) { lb[i * *gRows + k] = glb[k]; ub[i * *gRows + k] = gub[k]; }
    } else {
        long off = dpn * nodes;
        for (long i = 0; i < nodes; i++) {
            for (long k = 0; k < dpn; k++) { lb[i * dpn + k] = ilb[k]; ub[i * dpn + k] = iub[k]; }
            for (long k = 0; k < *gRows; k++) {
                lb[off + i * *gRows + k] = glb[k];
                ub[off + i * *gRows + k] = gub[k];
            }
        }
    }
    free(ilb); free(iub); free(glb); free(gub);
    *lbOut = lb;
    *ubOut = ub;
    *gOut = g;
    return 0;
}

OrProblem *or_load(const char *dir) {
    OrProblem *p = (OrProblem *)calloc(1, sizeof(OrProblem));
    char fn[1024], s1[64];
    snprintf(fn, sizeof fn, "%sdata.json", dir);
    char *js = slurp(fn, NULL);
    double v;
    long dims[3];
    if (!js) FAIL("cannot open %s", fn);
#define JN(key, dst) do { if (!json_num(js, key, &v)) FAIL("missing key %s", key); dst = v; } while (0)
    JN("numEvents", p->ne);
    JN("numNonleafNodes", p->nnl);
    JN("numNodes", p->n);
    JN("numStages", p->ns);
    JN("numStates", p->nx);
    JN("numInputs", p->nu);
    JN("rowsNNtr", p->nullDim);
    JN("stepSize", p->step);
    p->nl = p->n - p->nnl;
    p->nxu = p->nx + p->nu;
    p->yDim = p->nullDim - 2 * p->ne;
    {
        const char *pc = json_find(js, "preconditioned");
        if (!pc) FAIL("missing key preconditioned");
        while (*pc == ' ') pc++;
        p->precond = (strncmp(pc, "true", 4) == 0);
    }
    if (!json_sub_str(js, "dynamics", "type", s1, sizeof s1)) FAIL("missing dynamics.type");
    if (!strcmp(s1, "linear")) p->affine = 0;
    else if (!strcmp(s1, "affine")) p->affine = 1;
    else FAIL("dynamics type %s not supported", s1);
    if (!json_sub_str(js, "cost", "nonleaf", s1, sizeof s1) || (p->costNl = parse_cost(s1)) < 0) FAIL("cost.nonleaf");
    if (!json_sub_str(js, "cost", "leaf", s1, sizeof s1) || (p->costL = parse_cost(s1)) < 0) FAIL("cost.leaf");
    if (!json_sub_str(js, "constraint", "nonleaf", s1, sizeof s1) || (p->conNl = parse_con(s1)) < 0)
        FAIL("constraint.nonleaf");
    if (!json_sub_str(js, "constraint", "leaf", s1, sizeof s1) || (p->conL = parse_con(s1)) < 0)
        FAIL("constraint.leaf");
    if (!json_sub_str(js, "risk", "type", s1, sizeof s1) || strcmp(s1, "avar")) FAIL("risk type");
    {
        const char *pr = json_find(js, "risk");
        const char *pa = pr ? strstr(pr, "\"alpha\"") : NULL;
        p->alpha = pa ? strtod(strchr(pa, ':') + 1, NULL) : 1.0;
    }
    free(js);
    js = NULL;

    long n = p->n, nnl = p->nnl, nx = p->nx, nu = p->nu;
    NEED(read_bt(dir, "stages", 'u', (void **)&p->stages, NULL), "stages");
    NEED(read_bt(dir, "ancestors", 'u', (void **)&p->anc, NULL), "ancestors");
    NEED(read_bt(dir, "childrenFrom", 'u', (void **)&p->chFrom, NULL), "childrenFrom");
    NEED(read_bt(dir, "numChildren", 'u', (void **)&p->numCh, NULL), "numChildren");
    NEED(read_bt(dir, "stageFrom", 'u', (void **)&p->stageFrom, NULL), "stageFrom");
    NEED(read_bt(dir, "stageTo", 'u', (void **)&p->stageTo, NULL), "stageTo");
    NEED(read_bt(dir, "probabilities", 'd', (void **)&p->prob, NULL), "probabilities");
    NEED(read_bt(dir, "conditionalProbabilities", 'd', (void **)&p->cprob, NULL), "conditionalProbabilities");
    if (read_bt(dir, "dynamics_BTr", 'd', (void **)&p->BTr, dims) != nu * nx * n) FAIL("dynamics_BTr");
    if (read_bt(dir, "dynamics_AB", 'd', (void **)&p->AB, dims) != nx * (nx + nu) * n) FAIL("dynamics_AB");
    if (read_bt(dir, "dynamics_K", 'd', (void **)&p->K, dims) != nu * nx * nnl) FAIL("dynamics_K");
    if (read_bt(dir, "dynamics_ABKTr", 'd', (void **)&p->ABKTr, dims) != nx * nx * n) FAIL("dynamics_ABKTr");
    if (read_bt(dir, "dynamics_P", 'd', (void **)&p->P, dims) != nx * nx * n) FAIL("dynamics_P");
    if (read_bt(dir, "dynamics_APB", 'd', (void **)&p->APB, dims) != nx * nu * n) FAIL("dynamics_APB");
    if (read_bt(dir, "dynamics_lowCholesky", 'd', (void **)&p->chol, dims) != nu * nu * nnl)
        FAIL("dynamics_lowCholesky");
    if (p->affine) {
        if (read_bt(dir, "dynamics_c", 'd', (void **)&p->e, dims) != nx * n) FAIL("dynamics_c");
        p->Pe = (double *)calloc((size_t)(nx * n), sizeof(double)); /* Pe = P e (dynamics.cuh:236) */
        for (long j = 0; j < n; j++)
            for (long r = 0; r < nx; r++) {
                double acc = 0;
                for (long c = 0; c < nx; c++) acc += p->P[j * nx * nx + c * nx + r] * p->e[j * nx + c];
                p->Pe[j * nx + r] = acc;
            }
    }
    /* nonleaf cost */
    if (p->costNl == COST_LIN) {
        if (read_bt(dir, "nonleafCost_gradient", 'd', (void **)&p->nlGrad, dims) != p->nxu * n)
            FAIL("nonleafCost_gradient");
    } else {
        if (read_bt(dir, "nonleafCost_sqrtQ", 'd', (void **)&p->nlSqrtQ, dims) != nx * nx * n) FAIL("nonleafCost_sqrtQ");
        if (read_bt(dir, "nonleafCost_sqrtR", 'd', (void **)&p->nlSqrtR, dims) != nu * nu * n) FAIL("nonleafCost_sqrtR");
        if (read_bt(dir, "nonleafCost_translation", 'd', (void **)&p->nlTrans, dims) != (p->nxu + 2) * n)
            FAIL("nonleafCost_translation");
        if (p->costNl == COST_QPL) {
            if (read_bt(dir, "nonleafCost_q", 'd', (void **)&p->nlq, dims) != nx * n) FAIL("nonleafCost_q");
            if (read_bt(dir, "nonleafCost_r", 'd', (void **)&p->nlr, dims) != nu * n) FAIL("nonleafCost_r");
        }
    }
    if (p->costL == COST_LIN) {
        if (read_bt(dir, "leafCost_gradient", 'd', (void **)&p->lGrad, dims) != nx) FAIL("leafCost_gradient");
    } else {
        if (read_bt(dir, "leafCost_sqrtQ", 'd', (void **)&p->lSqrtQ, dims) != nx * nx) FAIL("leafCost_sqrtQ");
        if (read_bt(dir, "leafCost_translation", 'd', (void **)&p->lTrans, dims) != nx + 2)
            FAIL("leafCost_translation");
        if (p->costL == COST_QPL && read_bt(dir, "leafCost_q", 'd', (void **)&p->lq, dims) != nx)
            FAIL("leafCost_q");
    }
    if (load_constraint(p, dir, 0, p->conNl, nnl, &p->nlLb, &p->nlUb, &p->nlGamma, &p->nlGRows, &p->sIII))
        FAIL("nonleaf constraint files");
    if (load_constraint(p, dir, 1, p->conL, p->nl, &p->lLb, &p->lUb, &p->lGamma, &p->lGRows, &p->sV))
        FAIL("leaf constraint files");
    if (read_bt(dir, "risk_NNtr", 'd', (void **)&p->NNtr, dims) != p->nullDim * p->nullDim * nnl) FAIL("risk_NNtr");
    if (read_bt(dir, "risk_b", 'd', (void **)&p->b, dims) != p->yDim * nnl) FAIL("risk_b");
    if (p->precond) {
        if (read_bt(dir, "scaling", 'd', (void **)&p->scaling, dims) != p->nxu) FAIL("scaling");
    } else {
        p->scaling = (double *)malloc(sizeof(double) * (size_t)p->nxu);
        for (long i = 0; i < p->nxu; i++) p->scaling[i] = 1.0;
    }
    /* sizes (cache.cuh:481-497) */
    p->sU = nu * nnl;
    p->sX = nx * n;
    p->sY = p->yDim * nnl;
    p->sT = n;
    p->sS = n;
    p->sPrim = p->sU + p->sX + p->sY + p->sT + p->sS;
    p->oX = p->sU;
    p->oY = p->oX + p->sX;
    p->oT = p->oY + p->sY;
    p->oS = p->oT + p->sT;
    p->sI = p->yDim * nnl;
    p->sII = nnl;
    p->dIV = (p->costNl == COST_LIN) ? 2 : p->nxu + 2;
    p->dVI = (p->costL == COST_LIN) ? 2 : nx + 2;
    p->sIV = p->dIV * n;
    p->sVI = p->dVI * p->nl;
    p->oII = p->sI;
    p->oIII = p->oII + p->sII;
    p->oIV = p->oIII + p->sIII;
    p->oV = p->oIV + p->sIV;
    p->oVI = p->oV + p->sV;
    p->sDual = p->oVI + p->sVI;
    p->sZ = p->sPrim + p->sDual;
    return p;
fail:
    free(js);
    or_free(p);
    return NULL;
}

void or_sizes(const OrProblem *p, long *o) {
    o[0] = p->n; o[1] = p->nnl; o[2] = p->ns; o[3] = p->nx; o[4] = p->nu; o[5] = p->ne;
    o[6] = p->yDim; o[7] = p->nullDim; o[8] = p->sPrim; o[9] = p->sDual; o[10] = p->precond;
}

double or_step_size(const OrProblem *p) { return p->step; }

void or_scaling(const OrProblem *p, double *out) { memcpy(out, p->scaling, sizeof(double) * (size_t)p->nxu); }

/* ------------------------------------------------------------------ small dense helpers */

/* y (+)= M x, M column-major r x c */
static inline void matvec(const double *M, long r, long c, const double *x, double *y, int add) {
    if ((g_emu & OR_EMU_ACC) && !g_exact) {
        for (long i = 0; i < r; i++) {
            float acc = add ? (float)y[i] : 0.f;
            for (long k = 0; k < c; k++) acc = fmaf((float)M[k * r + i], (float)x[k], acc);
            y[i] = acc;
        }
        return;
    }
    if (!add) for (long i = 0; i < r; i++) y[i] = 0;
    for (long k = 0; k < c; k++) {
        const double xk = x[k];
        const double *col = M + k * r;
        for (long i = 0; i < r; i++) y[i] += col[i] * xk;
    }
}

/* y (+)= M' x, M column-major r x c, x length r, y length c */
static inline void matTvec(const double *M, long r, long c, const double *x, double *y, int add) {
    if ((g_emu & OR_EMU_ACC) && !g_exact) {
        for (long k = 0; k < c; k++) {
            float acc = 0.f;
            for (long i = 0; i < r; i++) acc = fmaf((float)M[k * r + i], (float)x[i], acc);
            y[k] = add ? (double)(float)(y[k] + acc) : acc;
        }
        return;
    }
    for (long k = 0; k < c; k++) {
        const double *col = M + k * r;
        double acc = 0;
        for (long i = 0; i < r; i++) acc += col[i] * x[i];
        y[k] = add ? y[k] + acc : acc;
    }
}

/* y = M x for the forward rollout (`states` = 1 for [A B][x; u], 0 for K x): as matvec, or
 * (OR_EMU_FWD64) accumulated in double, or (OR_EMU_FWDC, OR_EMU_FWDCX) float with compensation -- Ogita, Rump & Oishi, "Accurate sum and dot
 * product", SIAM J. Sci. Comput. 26 (2005), algorithm Dot2: each product split into its
 * rounded value and exact error by an FMA, each sum by Knuth's TwoSum. */
static void matvec_fwd(const double *M, long r, long c, const double *x, double *y, int states) {
    const int comp = (g_emu & OR_EMU_FWDC) || ((g_emu & OR_EMU_FWDCX) && states);
    const int kahan = (g_emu & OR_EMU_FWDK) != 0;
    if (!(g_emu & OR_EMU_ACC) || !((g_emu & OR_EMU_FWD64) || comp || kahan)) { matvec(M, r, c, x, y, 0); return; }
    if (g_emu & OR_EMU_FWD64) {
        for (long i = 0; i < r; i++) {
            double acc = 0;
            for (long k = 0; k < c; k++) acc += M[k * r + i] * x[k];
            y[i] = acc;
        }
        return;
    }
    if (kahan && !comp) { /* Kahan: s += a*b (rounded) with a running correction */
        for (long i = 0; i < r; i++) {
            float s = 0.f, cr = 0.f;
            for (long k = 0; k < c; k++) {
                const float yv = (float)M[k * r + i] * (float)x[k] - cr;
                const float t = s + yv;
                cr = (t - s) - yv;
                s = t;
            }
            y[i] = s;
        }
        return;
    }
    for (long i = 0; i < r; i++) {
        float s = 0.f, comp = 0.f;
        for (long k = 0; k < c; k++) {
            const float a = (float)M[k * r + i], b = (float)x[k];
            const float pr = a * b, e = fmaf(a, b, -pr);
            const float t = s + pr, bv = t - s;
            comp += ((s - (t - bv)) + (pr - bv)) + e;
            s = t;
        }
        y[i] = s + comp;
    }
}

static inline double dotv(const double *a, const double *b, long n) {
    double s = 0;
    for (long i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* ------------------------------------------------------------------ L and L* */

static void op_impl(const OrProblem *p, const double *prim, double *dual);
static void adj_impl(const OrProblem *p, const double *dual, double *prim);

void or_op(const OrProblem *p, const double *prim, double *dual) {
    const int saved = g_exact;
    if (g_emu & OR_EMU_ACCX_OPS) g_exact = 1;
    op_impl(p, prim, dual);
    g_exact = saved;
}

void or_adj(const OrProblem *p, const double *dual, double *prim) {
    const int saved = g_exact;
    if (g_emu & OR_EMU_ACCX_OPS) g_exact = 1;
    adj_impl(p, dual, prim);
    g_exact = saved;
}

static void op_impl(const OrProblem *p, const double *prim, double *dual) {
    const long nx = p->nx, nu = p->nu, nxu = p->nxu, yD = p->yDim, n = p->n, nnl = p->nnl;
    const double *u = prim, *x = prim + p->oX, *y = prim + p->oY, *t = prim + p->oT, *s = prim + p->oS;
    double *I = dual, *II = dual + p->oII, *III = dual + p->oIII, *IV = dual + p->oIV, *V = dual + p->oV,
           *VI = dual + p->oVI;
    double xu[1024];
    memset(dual, 0, sizeof(double) * (size_t)p->sDual);
    /* I, II (operator.cuh:44-49) */
    for (long i = 0; i < nnl; i++) {
        memcpy(I + i * yD, y + i * yD, sizeof(double) * (size_t)yD);
        II[i] = s[i] - dotv(p->b + i * yD, y + i * yD, yD);
    }
    /* III: nonleaf constraint */
    for (long i = 0; i < nnl && p->conNl != CON_NO; i++) {
        memcpy(xu, x + i * nx, sizeof(double) * (size_t)nx);
        memcpy(xu + nx, u + i * nu, sizeof(double) * (size_t)nu);
        if (p->conNl == CON_RECT || p->conNl == CON_RECTBALL) memcpy(III + i * nxu, xu, sizeof(double) * (size_t)nxu);
        else if (p->conNl == CON_POLY) matvec(p->nlGamma, p->nlGRows, nxu, xu, III + i * p->nlGRows, 0);
        else {
            memcpy(III + i * nxu, xu, sizeof(double) * (size_t)nxu);
            matvec(p->nlGamma, p->nlGRows, nxu, xu, III + nnl * nxu + i * p->nlGRows, 0);
        }
    }
    /* IV: nonleaf cost on every non-root node, reading the ancestor's (x, u) */
    for (long j = 1; j < n; j++) {
        const long a = p->anc[j];
        const double *xa = x + a * nx, *ua = u + a * nu;
        if (p->costNl == COST_LIN) {
            const double *g = p->nlGrad + j * nxu;
            IV[j] = dotv(g, xa, nx) + dotv(g + nx, ua, nu);
        } else {
            double *o = IV + j * (nxu + 2);
            matvec(p->nlSqrtQ + j * nx * nx, nx, nx, xa, o, 0);
            matvec(p->nlSqrtR + j * nu * nu, nu, nu, ua, o + nx, 0);
            double h = 0.5 * t[j];
            if (p->costNl == COST_QPL) h -= 0.5 * (dotv(p->nlq + j * nx, xa, nx) + dotv(p->nlr + j * nu, ua, nu));
            o[nxu] = h;
            o[nxu + 1] = h;
        }
    }
    if (p->costNl == COST_LIN) memcpy(IV + n, t, sizeof(double) * (size_t)n);
    /* V, VI: leaf constraint and leaf cost */
    for (long jj = 0; jj < p->nl; jj++) {
        const double *xj = x + (nnl + jj) * nx;
        if (p->conL == CON_RECT) memcpy(V + jj * nx, xj, sizeof(double) * (size_t)nx);
        else if (p->conL == CON_POLY) matvec(p->lGamma, p->lGRows, nx, xj, V + jj * p->lGRows, 0);
        else if (p->conL == CON_POLYID) {
            memcpy(V + jj * nx, xj, sizeof(double) * (size_t)nx);
            matvec(p->lGamma, p->lGRows, nx, xj, V + p->nl * nx + jj * p->lGRows, 0);
        }
        const double sj = s[nnl + jj];
        if (p->costL == COST_LIN) {
            VI[jj] = dotv(p->lGrad, xj, nx);
            VI[p->nl + jj] = sj;
        } else {
            double *o = VI + jj * (nx + 2);
            matvec(p->lSqrtQ, nx, nx, xj, o, 0);
            double h = 0.5 * sj;
            if (p->costL == COST_QPL) h -= 0.5 * dotv(p->lq, xj, nx);
            o[nx] = h;
            o[nx + 1] = h;
        }
    }
    EMU_VEC(dual, p->sDual);
}

static void adj_impl(const OrProblem *p, const double *dual, double *prim) {
    const long nx = p->nx, nu = p->nu, nxu = p->nxu, yD = p->yDim, n = p->n, nnl = p->nnl;
    double *u = prim, *x = prim + p->oX, *y = prim + p->oY, *t = prim + p->oT, *s = prim + p->oS;
    const double *I = dual, *II = dual + p->oII, *III = dual + p->oIII, *IV = dual + p->oIV, *V = dual + p->oV,
                 *VI = dual + p->oVI;
    double xu[1024];
    memset(prim, 0, sizeof(double) * (size_t)p->sPrim);
    for (long i = 0; i < nnl; i++) {
        s[i] = II[i];
        for (long k = 0; k < yD; k++) y[i * yD + k] = I[i * yD + k] - p->b[i * yD + k] * II[i];
    }
    for (long i = 0; i < nnl && p->conNl != CON_NO; i++) {
        if (p->conNl == CON_RECT || p->conNl == CON_RECTBALL) memcpy(xu, III + i * nxu, sizeof(double) * (size_t)nxu);
        else if (p->conNl == CON_POLY) matTvec(p->nlGamma, p->nlGRows, nxu, III + i * p->nlGRows, xu, 0);
        else {
            memcpy(xu, III + i * nxu, sizeof(double) * (size_t)nxu);
            matTvec(p->nlGamma, p->nlGRows, nxu, III + nnl * nxu + i * p->nlGRows, xu, 1);
        }
        memcpy(x + i * nx, xu, sizeof(double) * (size_t)nx);
        memcpy(u + i * nu, xu + nx, sizeof(double) * (size_t)nu);
    }
    for (long j = 1; j < n; j++) {
        const long a = p->anc[j];
        double *xa = x + a * nx, *ua = u + a * nu;
        if (p->costNl == COST_LIN) {
            const double g = IV[j];
            const double *gr = p->nlGrad + j * nxu;
            for (long k = 0; k < nx; k++) xa[k] += gr[k] * g;
            for (long k = 0; k < nu; k++) ua[k] += gr[nx + k] * g;
        } else {
            const double *d = IV + j * (nxu + 2);
            matvec(p->nlSqrtQ + j * nx * nx, nx, nx, d, xa, 1);
            matvec(p->nlSqrtR + j * nu * nu, nu, nu, d + nx, ua, 1);
            const double d23 = d[nxu] + d[nxu + 1];
            if (p->costNl == COST_QPL) {
                for (long k = 0; k < nx; k++) xa[k] -= 0.5 * p->nlq[j * nx + k] * d23;
                for (long k = 0; k < nu; k++) ua[k] -= 0.5 * p->nlr[j * nu + k] * d23;
            }
            t[j] = 0.5 * d23;
        }
    }
    if (p->costNl == COST_LIN) memcpy(t, IV + n, sizeof(double) * (size_t)n);
    for (long jj = 0; jj < p->nl; jj++) {
        double *xj = x + (nnl + jj) * nx;
        if (p->conL == CON_RECT) memcpy(xj, V + jj * nx, sizeof(double) * (size_t)nx);
        else if (p->conL == CON_POLY) matTvec(p->lGamma, p->lGRows, nx, V + jj * p->lGRows, xj, 0);
        else if (p->conL == CON_POLYID) {
            memcpy(xj, V + jj * nx, sizeof(double) * (size_t)nx);
            matTvec(p->lGamma, p->lGRows, nx, V + p->nl * nx + jj * p->lGRows, xj, 1);
        }
        if (p->costL == COST_LIN) {
            for (long k = 0; k < nx; k++) xj[k] += p->lGrad[k] * VI[jj];
            s[nnl + jj] = VI[p->nl + jj];
        } else {
            const double *d = VI + jj * (nx + 2);
            matvec(p->lSqrtQ, nx, nx, d, xj, 1);
            const double d23 = d[nx] + d[nx + 1];
            if (p->costL == COST_QPL)
                for (long k = 0; k < nx; k++) xj[k] -= 0.5 * p->lq[k] * d23;
            s[nnl + jj] = 0.5 * d23;
        }
    }
    EMU_VEC(prim, p->sPrim);
}

/* ------------------------------------------------------------------ proximal pieces */

static void chol_solve(const double *L, long m, double *b) {
    for (long i = 0; i < m; i++) { /* L y = b */
        double acc = b[i];
        for (long k = 0; k < i; k++) acc -= L[k * m + i] * b[k];
        b[i] = acc / L[i * m + i];
    }
    for (long i = m - 1; i >= 0; i--) { /* L' d = y */
        double acc = b[i];
        for (long k = i + 1; k < m; k++) acc -= L[i * m + k] * b[k];
        b[i] = acc / L[i * m + i];
    }
}

/* Dynamics projection (dynamics.cuh:74-174). q, d: node workspaces. */
void or_project_dynamics(const OrProblem *p, const double *x0, double *x, double *u) {
    const long nx = p->nx, nu = p->nu, n = p->n, nnl = p->nnl;
    double *q = (double *)malloc(sizeof(double) * (size_t)(nx * n));
    double *d = (double *)malloc(sizeof(double) * (size_t)(nu * nnl));
    double tmp[1024];
    for (long j = nnl; j < n; j++)
        for (long k = 0; k < nx; k++) q[j * nx + k] = -x[j * nx + k];
    const int saved = g_exact;
    if (g_emu & OR_EMU_ACCX_BACK) g_exact = 1;
    for (long stage = p->ns - 2; stage >= 0; stage--) {
        for (long i = p->stageFrom[stage]; i <= p->stageTo[stage]; i++) {
            const long c0 = p->chFrom[i], nc = p->numCh[i];
            double *di = d + i * nu;
            if (p->affine)
                for (long j = c0; j < c0 + nc; j++)
                    for (long k = 0; k < nx; k++) q[j * nx + k] += p->Pe[j * nx + k];
            for (long k = 0; k < nu; k++) di[k] = u[i * nu + k];
            for (long j = c0; j < c0 + nc; j++) { /* d -= B' q over children */
                matvec(p->BTr + j * nu * nx, nu, nx, q + j * nx, tmp, 0);
                for (long k = 0; k < nu; k++) di[k] -= tmp[k];
            }
            chol_solve(p->chol + i * nu * nu, nu, di);
            EMU_VEC(di, nu);
            if (stage > 0) {
                double *qi = q + i * nx;
                for (long k = 0; k < nx; k++) qi[k] = 0;
                for (long j = c0; j < c0 + nc; j++) {
                    matvec(p->APB + j * nx * nu, nx, nu, di, qi, 1);
                    matvec(p->ABKTr + j * nx * nx, nx, nx, q + j * nx, qi, 1);
                }
                for (long k = 0; k < nu; k++) tmp[k] = di[k] - u[i * nu + k];
                matTvec(p->K + i * nu * nx, nu, nx, tmp, qi, 1); /* K' (d - u) */
                for (long k = 0; k < nx; k++) qi[k] -= x[i * nx + k];
                EMU_VEC(qi, nx);
            }
        }
    }
    g_exact = saved;
    for (long k = 0; k < nx; k++) x[k] = x0[k];
    EMU_VEC(x, nx);
    for (long stage = 0; stage < p->ns - 1; stage++) {
        for (long i = p->stageFrom[stage]; i <= p->stageTo[stage]; i++) {
            double *ui = u + i * nu;
            matvec_fwd(p->K + i * nu * nx, nu, nx, x + i * nx, ui, 0);
            for (long k = 0; k < nu; k++) ui[k] += d[i * nu + k];
            EMU_VEC(ui, nu);
            memcpy(tmp, x + i * nx, sizeof(double) * (size_t)nx);
            memcpy(tmp + nx, ui, sizeof(double) * (size_t)nu);
            for (long j = p->chFrom[i]; j < p->chFrom[i] + p->numCh[i]; j++) {
                matvec_fwd(p->AB + j * nx * p->nxu, nx, p->nxu, tmp, x + j * nx, 1);
                if (p->affine)
                    for (long k = 0; k < nx; k++) x[j * nx + k] += p->e[j * nx + k];
                EMU_VEC(x + j * nx, nx);
            }
        }
    }
    free(q);
    free(d);
}

/* AVaR epigraph: project (y_i, t[ch(i)], s[ch(i)]) on ker[E' -I -I] (cache.cuh:650-676). */
void or_project_kernel(const OrProblem *p, double *y, double *t, double *s) {
    const long yD = p->yDim, nd = p->nullDim, E = p->ne;
    double v[512], w[512];
    for (long i = 0; i < p->nnl; i++) {
        const long c0 = p->chFrom[i], nc = p->numCh[i];
        memset(v, 0, sizeof(double) * (size_t)nd);
        memcpy(v, y + i * yD, sizeof(double) * (size_t)yD);
        for (long k = 0; k < nc; k++) { v[yD + k] = t[c0 + k]; v[yD + E + k] = s[c0 + k]; }
        matvec(p->NNtr + i * nd * nd, nd, nd, v, w, 0);
        EMU_VEC(w, nd);
        memcpy(y + i * yD, w, sizeof(double) * (size_t)yD);
        for (long k = 0; k < nc; k++) { t[c0 + k] = w[yD + k]; s[c0 + k] = w[yD + E + k]; }
    }
}

/* k_projectRectangle (definitions.cu:38-48), elementwise. */
void or_project_box(double *v, const double *lb, const double *ub, long n) {
    for (long i = 0; i < n; i++) {
        const int lower = v[i] <= lb[i], upper = v[i] >= ub[i];
        const double lbi = isinf(lb[i]) ? 0 : lower * lb[i];
        const double ubi = isinf(ub[i]) ? 0 : upper * ub[i];
        v[i] = v[i] * (1 - lower) * (1 - upper) + lbi + ubi;
    }
}

/* SOC projection of each column (Parikh & Boyd section 6.3.2; definitions.cu:301-428). */
void or_project_soc_columns(double *data, long dim, long ncones) {
    for (long c = 0; c < ncones; c++) {
        double *v = data + c * dim;
        double ss = 0;
        for (long k = 0; k < dim - 1; k++) ss += v[k] * v[k];
        const double nrm = sqrt(ss), tt = v[dim - 1];
        const int i1 = nrm <= tt;
        const int i2 = (nrm <= -tt) && !i1;
        const int i3 = !i1 && !i2;
        const double sc = (nrm + tt) / (2. * nrm + (1 - i3));
        if (i2) { for (long k = 0; k < dim; k++) v[k] = 0; }
        else if (i3) {
            for (long k = 0; k < dim - 1; k++) v[k] *= sc;
            v[dim - 1] = sc * nrm;
        }
    }
}

/* Linear-cost epigraph set: clamp `sum` from above by `set` (costs.cuh:296-301). */
static void project_linear_epi(double *blk, long nodes) {
    for (long i = 0; i < nodes; i++) {
        double lb = -INFINITY, ub = blk[nodes + i];
        or_project_box(blk + i, &lb, &ub, 1);
    }
}

/* Projection of the dual workspace on the constraint set C (cache.cuh:684-698). */
void or_project_dual(const OrProblem *p, double *dual) {
    const long yD = p->yDim;
    double *I = dual, *II = dual + p->oII;
    for (long i = 0; i < p->nnl; i++) { /* AVaR dual cone: first 2*numCh entries >= 0 */
        const long m = 2 * p->numCh[i];
        for (long k = 0; k < m; k++) {
            double *a = I + i * yD + k;
            if (*a < 0.) *a = (1 - 1) * *a;
        }
    }
    for (long i = 0; i < p->nnl; i++) II[i] = fmax(0., II[i]);
    if (p->sIII) or_project_box(dual + p->oIII, p->nlLb, p->nlUb, p->sIII);
    if (p->conNl == CON_RECTBALL) /* ||u|| <= radius: u * min(1, radius / ||u||) */
        for (long i = 0; i < p->nnl; i++) {
            double *u = dual + p->oIII + i * p->nxu + p->nx;
            const double nrm = sqrt(dotv(u, u, p->nu));
            if (nrm > p->nlRadius)
                for (long k = 0; k < p->nu; k++) u[k] *= p->nlRadius / nrm;
        }
    if (p->costNl == COST_LIN) project_linear_epi(dual + p->oIV, p->n);
    else or_project_soc_columns(dual + p->oIV, p->nxu + 2, p->n);
    if (p->sV) or_project_box(dual + p->oV, p->lLb, p->lUb, p->sV);
    if (p->costL == COST_LIN) project_linear_epi(dual + p->oVI, p->nl);
    else or_project_soc_columns(dual + p->oVI, p->nx + 2, p->nl);
    EMU_VEC(dual, p->sDual);
}

/* One Chambolle-Pock step: cand = T(z) (cache.cuh:748-801). x0s is the scaled initial state. */
typedef struct {
    double *pw, *pd, *dw, *dc;
} Work;

static void work_alloc(const OrProblem *p, Work *w) {
    w->pw = (double *)malloc(sizeof(double) * (size_t)p->sPrim);
    w->pd = (double *)malloc(sizeof(double) * (size_t)p->sPrim);
    w->dw = (double *)malloc(sizeof(double) * (size_t)p->sDual);
    w->dc = (double *)malloc(sizeof(double) * (size_t)p->sDual);
}

static void work_free(Work *w) { free(w->pw); free(w->pd); free(w->dw); free(w->dc); }

static void cp_step(const OrProblem *p, Work *w, const double *x0s, const double *z, double *cand) {
    const long sp = p->sPrim, sd = p->sDual;
    const double g = p->step, gi = 1. / p->step;
    const double *zp = z, *zd = z + sp;
    double *cp = cand, *cd = cand + sp;
    /* modifyPrimal: p - gamma L* d */
    or_adj(p, zd, w->pw);
    for (long i = 0; i < sp; i++) w->pw[i] = w->pw[i] * -g + zp[i];
    EMU_VEC(w->pw, sp);
    /* proximalPrimal: s_root -= gamma; dynamics; kernels */
    w->pw[p->oS] -= g;
    EMU_VEC(w->pw + p->oS, 1);
    or_project_dynamics(p, x0s, w->pw + p->oX, w->pw);
    or_project_kernel(p, w->pw + p->oY, w->pw + p->oT, w->pw + p->oS);
    memcpy(cp, w->pw, sizeof(double) * (size_t)sp);
    /* modifyDual: d + gamma L(2 pbar - p) */
    for (long i = 0; i < sp; i++) w->pd[i] = 2. * cp[i] - zp[i];
    EMU_VEC(w->pd, sp);
    or_op(p, w->pd, w->dw);
    for (long i = 0; i < sd; i++) w->dw[i] = w->dw[i] * g + zd[i];
    EMU_VEC(w->dw, sd);
    /* proximalDual (Moreau): cand = gamma (v - proj_C(v)), v = dbar/gamma + translation */
    for (long i = 0; i < sd; i++) w->dw[i] *= gi;
    if (p->costNl != COST_LIN)
        for (long i = 0; i < p->sIV; i++) w->dw[p->oIV + i] += p->nlTrans[i];
    if (p->costL != COST_LIN)
        for (long jj = 0; jj < p->nl; jj++)
            for (long k = 0; k < p->nx + 2; k++) w->dw[p->oVI + jj * (p->nx + 2) + k] += p->lTrans[k];
    EMU_VEC(w->dw, sd);
    memcpy(cd, w->dw, sizeof(double) * (size_t)sd);
    or_project_dual(p, w->dw);
    for (long i = 0; i < sd; i++) cd[i] = (cd[i] - w->dw[i]) * g;
    EMU_VEC(cd, sd);
}

void or_cp_step(const OrProblem *p, const double *x0s, const double *z, double *cand) {
    Work w;
    work_alloc(p, &w);
    cp_step(p, &w, x0s, z, cand);
    work_free(&w);
}

/* M y = y - gamma [L* y_d; L y_p]   (cache.cuh:721-734) */
static void apply_m(const OrProblem *p, const double *yv, double *my) {
    const long sp = p->sPrim;
    or_adj(p, yv + sp, my);
    or_op(p, yv, my + sp);
    for (long i = 0; i < p->sZ; i++) my[i] = yv[i] - p->step * my[i];
    EMU_VEC(my, p->sZ);
}

double or_dot_m(const OrProblem *p, const double *x, const double *y) {
    double *my = (double *)malloc(sizeof(double) * (size_t)p->sZ);
    apply_m(p, y, my);
    double r = dotv(x, my, p->sZ);
    free(my);
    return r;
}

/* Least squares min ||A g - b|| by Householder QR (what QRFactoriser::leastSquares computes
 * with cuSOLVER geqrf/ormqr/trsm at cache.cuh:879-888).  A is n x m column-major (copied). */
static void lstsq_qr(const double *A0, long n, long m, const double *b0, double *g) {
    double *A = (double *)malloc(sizeof(double) * (size_t)(n * m));
    double *b = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(A, A0, sizeof(double) * (size_t)(n * m));
    memcpy(b, b0, sizeof(double) * (size_t)n);
    for (long k = 0; k < m; k++) {
        double *a = A + k * n;
        double nrm = 0;
        for (long i = k; i < n; i++) nrm += a[i] * a[i];
        nrm = sqrt(nrm);
        if (nrm == 0) continue;
        const double alpha = a[k] > 0 ? -nrm : nrm;
        const double v0 = a[k] - alpha;
        /* v = [v0, a[k+1:]]; H = I - 2 v v'/(v'v) */
        double vv = v0 * v0;
        for (long i = k + 1; i < n; i++) vv += a[i] * a[i];
        a[k] = v0;
        for (long j = k + 1; j < m; j++) {
            double *c = A + j * n;
            double dp = 0;
            for (long i = k; i < n; i++) dp += a[i] * c[i];
            const double f = 2. * dp / vv;
            for (long i = k; i < n; i++) c[i] -= f * a[i];
        }
        double dp = 0;
        for (long i = k; i < n; i++) dp += a[i] * b[i];
        const double f = 2. * dp / vv;
        for (long i = k; i < n; i++) b[i] -= f * a[i];
        a[k] = alpha; /* R(k,k) */
    }
    for (long k = m - 1; k >= 0; k--) {
        double acc = b[k];
        for (long j = k + 1; j < m; j++) acc -= A[j * n + k] * g[j];
        g[k] = acc / A[k * n + k];
    }
    free(A);
    free(b);
}

/* OR_EMU_GRAM: min ||A g - b|| by the normal equations, as a GPU controller with float data
 * solves it -- Gram matrix and right-hand side accumulated with float FMAs over blocks of 256
 * rows and summed in double, a ridge of 1e-7 x the largest diagonal entry, FP64 Cholesky.
 * Returns 0 on breakdown (the caller then takes the plain residual direction). */
static int gram_solve(const double *A, long n, long m, const double *b, double *g) {
    double G[64], h[64], L[64], y[8];
    if (m > 8) return 0;
    for (long i = 0; i < m; i++)
        for (long j = 0; j <= m; j++) {
            if (j < m && j > i) continue;
            const double *v = j < m ? A + j * n : b;
            double s = 0;
            for (long c = 0; c < n; c += 256) {
                float acc = 0.f;
                for (long k = c; k < c + 256 && k < n; k++) acc = fmaf((float)A[i * n + k], (float)v[k], acc);
                s += acc;
            }
            if (j < m) G[i * m + j] = G[j * m + i] = s;
            else h[i] = s;
        }
    double dmax = 0;
    for (long i = 0; i < m; i++) dmax = fmax(dmax, G[i * m + i]);
    if (!(dmax > 0)) return 0;
    for (long j = 0; j < m; j++) {
        double s = G[j * m + j] + 1e-7 * dmax;
        for (long k = 0; k < j; k++) s -= L[j * m + k] * L[j * m + k];
        if (!(s > 0)) return 0;
        const double d = sqrt(s);
        L[j * m + j] = d;
        for (long i = j + 1; i < m; i++) {
            double a = G[i * m + j];
            for (long k = 0; k < j; k++) a -= L[i * m + k] * L[j * m + k];
            L[i * m + j] = a / d;
        }
    }
    for (long i = 0; i < m; i++) {
        double a = h[i];
        for (long k = 0; k < i; k++) a -= L[i * m + k] * y[k];
        y[i] = a / L[i * m + i];
    }
    for (long i = m - 1; i >= 0; i--) {
        double a = y[i];
        for (long k = i + 1; k < m; k++) a -= L[k * m + i] * g[k];
        g[i] = a / L[i * m + i];
    }
    for (long i = 0; i < m; i++)
        if (!isfinite(g[i])) return 0;
    return 1;
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static double max_abs(const double *v, long n) {
    double m = 0;
    for (long i = 0; i < n; i++) {
        const double a = fabs(v[i]);
        if (a > m || isnan(a)) m = a;
    }
    return m;
}

typedef struct {
    const OrProblem *p;
    const OrOptions *o;
    double tolAbs, tolRel, tol;
    int errInit;
    int status;
    long iters;
    double err;
    double t0;
} Ctl;

static void ctl_init(Ctl *c, const OrProblem *p, const OrOptions *o) {
    c->p = p;
    c->o = o;
    c->tolAbs = o->tol_abs;
    c->tolRel = o->tol_rel;
    if (p->precond) { /* cache.cuh:302-306 */
        double mn = p->scaling[0];
        for (long i = 1; i < p->nxu; i++) mn = fmin(mn, p->scaling[i]);
        c->tolAbs *= mn;
        c->tolRel *= mn;
    }
    c->tol = 0;
    c->errInit = 1;
    c->status = -1;
    c->iters = 0;
    c->err = INFINITY;
    c->t0 = now_s();
}

/* computeError (cache.cuh:909-961), given r = z - T(z) and m = M r (so r/gamma - [L* r_d; L r_p]
 * equals m / gamma). */
static void ctl_check(Ctl *c, long idx, const double *mr, long nz) {
    if (idx % 25 != 0) return;
    const double e = max_abs(mr, nz) / c->p->step;
    if (c->errInit) {
        c->tol = fmax(c->tolAbs, c->tolRel * e);
        c->status = -1;
        c->errInit = 0;
    } else {
        c->err = e;
        if (e <= c->tol) c->status = 0;
        if (c->o->max_outer && idx >= c->o->max_outer) c->status = 1;
        if (c->o->max_time_secs > 0 && idx % 1000 == 0 && now_s() - c->t0 >= c->o->max_time_secs) c->status = 2;
        if (c->status != -1) c->iters = idx;
    }
}

static void scale_x0(const OrProblem *p, const double *x0, double *x0s) {
    for (long i = 0; i < p->nx; i++) x0s[i] = x0[i] * p->scaling[i];
}

int or_run_cp(const OrProblem *p, const OrOptions *o, const double *x0, double *z, int warm, OrStats *st) {
    const long nz = p->sZ;
    double x0s[1024];
    scale_x0(p, x0, x0s);
    double *cand = (double *)malloc(sizeof(double) * (size_t)nz);
    double *r = (double *)malloc(sizeof(double) * (size_t)nz);
    double *mr = (double *)malloc(sizeof(double) * (size_t)nz);
    Work w;
    work_alloc(p, &w);
    if (!warm) memset(z, 0, sizeof(double) * (size_t)nz);
    Ctl c;
    ctl_init(&c, p, o);
    long calls = 0;
    for (long i = 0;; i++) {
        cp_step(p, &w, x0s, z, cand);
        calls++;
        if (i % 25 == 0) {
            for (long k = 0; k < nz; k++) r[k] = z[k] - cand[k];
            apply_m(p, r, mr);
            ctl_check(&c, i, mr, nz);
        }
        memcpy(z, cand, sizeof(double) * (size_t)nz);
        if (c.status != -1) break;
    }
    if (st) {
        memset(st, 0, sizeof *st);
        st->status = c.status; st->iters = c.iters; st->calls_T = calls; st->tol = c.tol; st->err = c.err;
        st->seconds = now_s() - c.t0;
    }
    work_free(&w);
    free(cand); free(r); free(mr);
    return c.status;
}

int or_run_spock(const OrProblem *p, const OrOptions *o, const double *x0, double *z, int warm, OrStats *st) {
    const long nz = p->sZ, m = o->anderson;
    const double c0 = .99, c1 = .99, c2 = .99, beta = .5, sigma = .1, lambda = 1.;
    double x0s[1024];
    scale_x0(p, x0, x0s);
    const size_t B = sizeof(double) * (size_t)nz;
    double *cand = (double *)malloc(B), *prev = (double *)malloc(B), *rprev = (double *)malloc(B);
    double *backup = (double *)malloc(B), *r = (double *)malloc(B), *mr = (double *)malloc(B);
    double *dz = (double *)malloc(B), *dr = (double *)malloc(B), *dir = (double *)malloc(B);
    double *dsc = (double *)malloc(B);
    double *andZ = (double *)calloc((size_t)(nz * m), sizeof(double));
    double *andR = (double *)calloc((size_t)(nz * m), sizeof(double));
    double gam[64];
    Work w;
    work_alloc(p, &w);
    if (!warm) {
        memset(z, 0, B);
        for (long i = 0; i < nz; i++) { prev[i] = 1.; rprev[i] = 1.; } /* cache.cuh:624-632 */
    } else {
        EMU_VEC(z, nz);
        memcpy(prev, z, B);
        memset(rprev, 0, B);
    }
    Ctl c;
    ctl_init(&c, p, o);
    long calls = 0, k0 = 0, k1 = 0, k2 = 0, k2bt = 0, k3 = 0;
    double zeta = INFINITY, wv = INFINITY, wSafe = INFINITY, wTilde = INFINITY, rho = 0, tau = 0;
    for (long iOut = 0;; iOut++) {
        if (iOut != 0) memcpy(z, cand, B);
        cp_step(p, &w, x0s, z, cand);
        calls++;
        for (long k = 0; k < nz; k++) r[k] = z[k] - cand[k];
        EMU_VEC(r, nz);
        apply_m(p, r, mr);
        ctl_check(&c, iOut, mr, nz);
        if (c.status != -1) { memcpy(z, cand, B); break; }
        memcpy(backup, cand, B);
        wv = sqrt(dotv(r, mr, nz));
        for (long k = 0; k < nz; k++) { dz[k] = z[k] - prev[k]; dr[k] = r[k] - rprev[k]; }
        memcpy(prev, z, B);
        memcpy(rprev, r, B);
        /* updateDirection (cache.cuh:860-904); the column shift has memmove semantics */
        if (m > 1) {
            memmove(andZ + nz, andZ, B * (size_t)(m - 1));
            memmove(andR + nz, andR, B * (size_t)(m - 1));
        }
        EMU_VEC(dz, nz);
        EMU_VEC(dr, nz);
        for (long k = 0; k < nz; k++) { andR[k] = dr[k]; andZ[k] = dz[k] - dr[k]; }
        EMU_VEC(andZ, nz);
        int useAnd = iOut >= m;
        if (useAnd && (g_emu & OR_EMU_GRAM)) useAnd = gram_solve(andR, nz, m, r, gam);
        else if (useAnd) lstsq_qr(andR, nz, m, r, gam);
        if (useAnd) {
            for (long k = 0; k < nz; k++) {
                double acc = 0;
                for (long j = 0; j < m; j++) acc += andZ[j * nz + k] * gam[j];
                dir[k] = -acc - r[k];
            }
        } else {
            for (long k = 0; k < nz; k++) dir[k] = -r[k];
        }
        EMU_VEC(dir, nz);
        if (wv <= c0 * zeta) { /* K0: blind update */
            for (long k = 0; k < nz; k++) cand[k] = prev[k] + dir[k];
            EMU_VEC(cand, nz);
            zeta = wv;
            k0++;
            continue;
        }
        tau = 1.;
        for (long iIn = 0; iIn < o->max_inner; iIn++) {
            for (long k = 0; k < nz; k++) { dsc[k] = dir[k] * tau; z[k] = prev[k] + dsc[k]; }
            EMU_VEC(dsc, nz);
            EMU_VEC(z, nz);
            cp_step(p, &w, x0s, z, cand);
            calls++;
            for (long k = 0; k < nz; k++) r[k] = z[k] - cand[k];
            EMU_VEC(r, nz);
            apply_m(p, r, mr);
            wTilde = sqrt(dotv(r, mr, nz));
            if (wv <= wSafe && wTilde <= c1 * wv) { /* K1: educated update */
                memcpy(cand, z, B);
                wSafe = wTilde + pow(c2, (double)iOut);
                k1++;
                break;
            }
            rho = wTilde * wTilde - dotv(mr, dsc, nz); /* r'M(tau d) = (M r)'(tau d) */
            if (rho >= sigma * wTilde * wv) { /* K2: safeguard */
                const double f = lambda * rho / (wTilde * wTilde);
                for (long k = 0; k < nz; k++) cand[k] = prev[k] - r[k] * f;
                EMU_VEC(cand, nz);
                k2++;
                break;
            } else {
                tau *= beta;
                k2bt++;
            }
            if (iIn >= o->max_inner - 1) { /* K3: restore */
                memcpy(cand, backup, B);
                k3++;
            }
        }
    }
    if (st) {
        st->status = c.status; st->iters = c.iters; st->calls_T = calls; st->tol = c.tol; st->err = c.err;
        st->k0 = k0; st->k1 = k1; st->k2 = k2; st->k2bt = k2bt; st->k3 = k3;
        st->seconds = now_s() - c.t0;
    }
    work_free(&w);
    free(cand); free(prev); free(rprev); free(backup); free(r); free(mr); free(dz); free(dr);
    free(dir); free(dsc); free(andZ); free(andR);
    return c.status;
}

void or_states_inputs(const OrProblem *p, const double *z, double *states, double *inputs) {
    for (long j = 0; j < p->n; j++)
        for (long k = 0; k < p->nx; k++) states[j * p->nx + k] = z[p->oX + j * p->nx + k] / p->scaling[k];
    for (long i = 0; i < p->nnl; i++)
        for (long k = 0; k < p->nu; k++) inputs[i * p->nu + k] = z[i * p->nu + k] / p->scaling[p->nx + k];
}

/* ------------------------------------------------------------------ many instances on threads */

typedef struct {
    const OrProblem *p;
    const OrOptions *o;
    long begin, end;
    const double *x0s;
    int *status;
    long *iters;
    double *u0;
    double *zs;
    int warm;
    long *calls;
} Job;

static void *job_run(void *arg) {
    Job *j = (Job *)arg;
    const OrProblem *p = j->p;
    double *z = (double *)malloc(sizeof(double) * (size_t)p->sZ);
    for (long k = j->begin; k < j->end; k++) {
        OrStats st;
        if (j->warm) memcpy(z, j->zs + k * p->sZ, sizeof(double) * (size_t)p->sZ);
        or_run_spock(p, j->o, j->x0s + k * p->nx, z, j->warm, &st);
        j->status[k] = st.status;
        j->iters[k] = st.iters;
        if (j->calls) j->calls[k] = st.calls_T;
        for (long q = 0; q < p->nu; q++) j->u0[k * p->nu + q] = z[q] / p->scaling[p->nx + q];
        if (j->zs) memcpy(j->zs + k * p->sZ, z, sizeof(double) * (size_t)p->sZ);
    }
    free(z);
    return NULL;
}

double or_solve_many(const OrProblem *p, const OrOptions *o, long count, const double *x0s, int threads,
                     int *status, long *iters, double *u0, double *zs) {
    return or_solve_many_warm(p, o, count, x0s, threads, status, iters, u0, zs, 0, NULL);
}

double or_solve_many_warm(const OrProblem *p, const OrOptions *o, long count, const double *x0s, int threads,
                          int *status, long *iters, double *u0, double *zs, int warm, long *calls) {
    if (warm && !zs) return -1.;
    if (threads < 1) threads = 1;
    if (threads > count) threads = (int)count;
    pthread_t th[256];
    Job jobs[256];
    if (threads > 256) threads = 256;
    const double t0 = now_s();
    for (int t = 0; t < threads; t++) {
        jobs[t].p = p; jobs[t].o = o; jobs[t].x0s = x0s; jobs[t].status = status; jobs[t].iters = iters;
        jobs[t].u0 = u0; jobs[t].zs = zs; jobs[t].warm = warm; jobs[t].calls = calls;
        jobs[t].begin = count * t / threads;
        jobs[t].end = count * (t + 1) / threads;
        pthread_create(&th[t], NULL, job_run, &jobs[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    return now_s() - t0;
}

/* ------------------------------------------------------------------ offline cache */

static void chol_lower(const double *A, long m, double *L) {
    memset(L, 0, sizeof(double) * (size_t)(m * m));
    for (long j = 0; j < m; j++) {
        double s = A[j * m + j];
        for (long k = 0; k < j; k++) s -= L[k * m + j] * L[k * m + j];
        L[j * m + j] = sqrt(s);
        for (long i = j + 1; i < m; i++) {
            double a = A[j * m + i];
            for (long k = 0; k < j; k++) a -= L[k * m + i] * L[k * m + j];
            L[j * m + i] = a / L[j * m + j];
        }
    }
}

void or_offline_dynamics(const OrProblem *p, const double *AB, double *P, double *K, double *lowChol,
                         double *ABKTr, double *APB) {
    const long nx = p->nx, nu = p->nu, nxu = p->nxu, n = p->n, nnl = p->nnl;
    double *sumR = (double *)malloc(sizeof(double) * (size_t)(nu * nu));
    double *sumK = (double *)malloc(sizeof(double) * (size_t)(nu * nx));
    double *PB = (double *)malloc(sizeof(double) * (size_t)(nx * nu));
    double *PA = (double *)malloc(sizeof(double) * (size_t)(nx * nx));
    double *Abk = (double *)malloc(sizeof(double) * (size_t)(nx * nx));
    double *PAbk = (double *)malloc(sizeof(double) * (size_t)(nx * nx));
    double *col = (double *)malloc(sizeof(double) * (size_t)(nx > nu ? nx : nu));
    memset(P, 0, sizeof(double) * (size_t)(nx * nx * n));
    memset(ABKTr, 0, sizeof(double) * (size_t)(nx * nx * n));
    memset(APB, 0, sizeof(double) * (size_t)(nx * nu * n));
    for (long j = nnl; j < n; j++)
        for (long k = 0; k < nx; k++) P[j * nx * nx + k * nx + k] = 1.;
#define AJ(j, r, c) AB[(j) * nx * nxu + (c) * nx + (r)]
#define BJ(j, r, c) AB[(j) * nx * nxu + (nx + (c)) * nx + (r)]
    for (long i = nnl - 1; i >= 0; i--) {
        memset(sumR, 0, sizeof(double) * (size_t)(nu * nu));
        memset(sumK, 0, sizeof(double) * (size_t)(nu * nx));
        const long c0 = p->chFrom[i], nc = p->numCh[i];
        for (long j = c0; j < c0 + nc; j++) {
            const double *Pj = P + j * nx * nx;
            for (long c = 0; c < nu; c++) /* PB = P_j B_j */
                for (long r = 0; r < nx; r++) {
                    double a = 0;
                    for (long k = 0; k < nx; k++) a += Pj[k * nx + r] * BJ(j, k, c);
                    PB[c * nx + r] = a;
                }
            for (long c = 0; c < nx; c++)
                for (long r = 0; r < nx; r++) {
                    double a = 0;
                    for (long k = 0; k < nx; k++) a += Pj[k * nx + r] * AJ(j, k, c);
                    PA[c * nx + r] = a;
                }
            for (long c = 0; c < nu; c++)
                for (long r = 0; r < nu; r++) {
                    double a = 0;
                    for (long k = 0; k < nx; k++) a += BJ(j, k, r) * PB[c * nx + k];
                    sumR[c * nu + r] += a;
                }
            for (long c = 0; c < nx; c++)
                for (long r = 0; r < nu; r++) {
                    double a = 0;
                    for (long k = 0; k < nx; k++) a += BJ(j, k, r) * PA[c * nx + k];
                    sumK[c * nu + r] += a;
                }
        }
        for (long k = 0; k < nu; k++) sumR[k * nu + k] += 1.;
        double *L = lowChol + i * nu * nu;
        chol_lower(sumR, nu, L);
        double *Ki = K + i * nu * nx;
        for (long c = 0; c < nx; c++) {
            for (long r = 0; r < nu; r++) col[r] = -sumK[c * nu + r];
            chol_solve(L, nu, col);
            for (long r = 0; r < nu; r++) Ki[c * nu + r] = col[r];
        }
        double *Pi = P + i * nx * nx;
        for (long c = 0; c < nx; c++)
            for (long r = 0; r < nx; r++) {
                double a = (r == c) ? 1. : 0.;
                for (long k = 0; k < nu; k++) a += Ki[r * nu + k] * Ki[c * nu + k];
                Pi[c * nx + r] = a;
            }
        for (long j = c0; j < c0 + nc; j++) {
            const double *Pj = P + j * nx * nx;
            for (long c = 0; c < nx; c++) /* Abk = A_j + B_j K_i */
                for (long r = 0; r < nx; r++) {
                    double a = AJ(j, r, c);
                    for (long k = 0; k < nu; k++) a += BJ(j, r, k) * Ki[c * nu + k];
                    Abk[c * nx + r] = a;
                }
            for (long c = 0; c < nx; c++)
                for (long r = 0; r < nx; r++) ABKTr[j * nx * nx + c * nx + r] = Abk[r * nx + c];
            for (long c = 0; c < nx; c++)
                for (long r = 0; r < nx; r++) {
                    double a = 0;
                    for (long k = 0; k < nx; k++) a += Pj[k * nx + r] * Abk[c * nx + k];
                    PAbk[c * nx + r] = a;
                }
            for (long c = 0; c < nx; c++)
                for (long r = 0; r < nx; r++) {
                    double a = 0;
                    for (long k = 0; k < nx; k++) a += Abk[r * nx + k] * PAbk[c * nx + k];
                    Pi[c * nx + r] += a;
                }
            for (long c = 0; c < nu; c++)
                for (long r = 0; r < nx; r++) {
                    double a = 0;
                    for (long k = 0; k < nx; k++) {
                        double pb = 0;
                        for (long q = 0; q < nx; q++) pb += Pj[q * nx + k] * BJ(j, q, c);
                        a += Abk[r * nx + k] * pb;
                    }
                    APB[j * nx * nu + c * nx + r] = a;
                }
        }
    }
#undef AJ
#undef BJ
    free(sumR); free(sumK); free(PB); free(PA); free(Abk); free(PAbk); free(col);
}

/* Projector onto null([E' -I -I]) for node i, padded to 4E+1 (problem.py:215-231):
 * P = I - S'(SS')^{-1}S with S the numCh nonzero rows. */
void or_offline_kernel(const OrProblem *p, double alpha, long node, double *nntr) {
    const long nd = p->nullDim, E = p->ne, yD = p->yDim, nc = p->numCh[node];
    double *S = (double *)calloc((size_t)(nc * nd), sizeof(double)); /* row-major nc x nd */
    for (long k = 0; k < nc; k++) {
        S[k * nd + k] = alpha;
        S[k * nd + nc + k] = -1.;
        S[k * nd + 2 * nc] = 1.;
        S[k * nd + yD + k] = -1.;
        S[k * nd + yD + E + k] = -1.;
    }
    double *G = (double *)calloc((size_t)(nc * nc), sizeof(double)), *L = (double *)calloc((size_t)(nc * nc), sizeof(double));
    for (long a = 0; a < nc; a++)
        for (long b = 0; b < nc; b++) G[b * nc + a] = dotv(S + a * nd, S + b * nd, nd);
    chol_lower(G, nc, L);
    double *col = (double *)malloc(sizeof(double) * (size_t)nc);
    for (long c = 0; c < nd; c++) {
        for (long a = 0; a < nc; a++) col[a] = S[a * nd + c];
        chol_solve(L, nc, col); /* (SS')^{-1} S e_c */
        for (long r = 0; r < nd; r++) {
            double a = 0;
            for (long k = 0; k < nc; k++) a += S[k * nd + r] * col[k];
            nntr[c * nd + r] = (r == c ? 1. : 0.) - a;
        }
    }
    free(S); free(G); free(L); free(col);
}

double or_norm_L_sq(const OrProblem *p, long iters) {
    double *v = (double *)malloc(sizeof(double) * (size_t)p->sPrim);
    double *d = (double *)malloc(sizeof(double) * (size_t)p->sDual);
    double *w = (double *)malloc(sizeof(double) * (size_t)p->sPrim);
    for (long i = 0; i < p->sPrim; i++) v[i] = 1. + 0.001 * (double)(i % 17);
    double lam = 0;
    for (long it = 0; it < iters; it++) {
        const double nv = sqrt(dotv(v, v, p->sPrim));
        for (long i = 0; i < p->sPrim; i++) v[i] /= nv;
        or_op(p, v, d);
        or_adj(p, d, w);
        const double l = dotv(v, w, p->sPrim);
        memcpy(v, w, sizeof(double) * (size_t)p->sPrim);
        if (it > 10 && fabs(l - lam) <= 1e-15 * fabs(l)) { lam = l; break; }
        lam = l;
    }
    free(v); free(d); free(w);
    return lam;
}

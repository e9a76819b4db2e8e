/*
 * CPU oracle for the darcy MG-PCG solve path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference algorithm (darcy-cpp v1.0.0). Every
 * function names the reference lines it follows; loop order, operation order
 * and OpenMP structure (static schedules, the 4096-cell serial guard, the
 * simd reductions) are kept so that, built with the same flags, a one-thread
 * run reproduces the reference bit for bit and a many-thread run has the same
 * cost profile. Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it; the GPU library neither links nor calls it.
 */
#include "darcy_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(__GNUC__)
#define RESTRICT __restrict__
#else
#define RESTRICT
#endif

#define DO_PRAGMA(x) _Pragma(#x)
#ifdef _OPENMP
#define OMP(x) DO_PRAGMA(omp x)
#else
#define OMP(x)
#endif

/* level.hpp:74 and blas.hpp:24: below this size a loop runs serially. */
#define MIN_PARALLEL 4096
/* multigrid.hpp:148 */
#define COARSEST_SWEEPS 8
/* multigrid.hpp:46 */
#define MAX_LEVELS 32

static void set_err(char* err, int err_len, const char* msg) {
    if (err && err_len > 0) {
        strncpy(err, msg, (size_t)err_len - 1);
        err[err_len - 1] = '\0';
    }
}

/* ------------------------------------------------------------------ blas */

/* blas.hpp:27-35 */
static double b_dot(const double* RESTRICT x, const double* RESTRICT y, int64_t n) {
    double s = 0.0;
    OMP(parallel for simd reduction(+ : s) schedule(static) if (n >= MIN_PARALLEL))
    for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

/* blas.hpp:50-56: y = x + beta * y */
static void b_xpby(const double* RESTRICT x, double beta, double* RESTRICT y, int64_t n) {
    OMP(parallel for simd schedule(static) if (n >= MIN_PARALLEL))
    for (int64_t i = 0; i < n; ++i) y[i] = x[i] + beta * y[i];
}

/* blas.hpp:62-77: u += alpha p; r -= alpha ap; return ||r||^2 */
static double b_cg_update(double alpha, const double* RESTRICT p, const double* RESTRICT ap,
                          double* RESTRICT u, double* RESTRICT r, int64_t n) {
    double rr = 0.0;
    OMP(parallel for simd reduction(+ : rr) schedule(static) if (n >= MIN_PARALLEL))
    for (int64_t i = 0; i < n; ++i) {
        u[i] += alpha * p[i];
        const double ri = r[i] - alpha * ap[i];
        r[i] = ri;
        rr += ri * ri;
    }
    return rr;
}

/* blas.hpp:79-84 */
static void b_fill(double* RESTRICT x, double v, int64_t n) {
    OMP(parallel for simd schedule(static) if (n >= MIN_PARALLEL))
    for (int64_t i = 0; i < n; ++i) x[i] = v;
}

/* ----------------------------------------------------------------- level */

typedef struct {
    int64_t n, size;
    int parallel;
    double *e, *w, *nn, *s, *diag, *inv_diag; /* level.hpp:253 */
} level_t;

static int level_alloc(level_t* L, int64_t n) {
    L->n = n;
    L->size = n * n;
    L->parallel = L->size >= MIN_PARALLEL;
    double* block = (double*)malloc(sizeof(double) * 6 * (size_t)L->size);
    if (!block) return -1;
    L->e = block;
    L->w = block + L->size;
    L->nn = block + 2 * L->size;
    L->s = block + 3 * L->size;
    L->diag = block + 4 * L->size;
    L->inv_diag = block + 5 * L->size;
    return 0;
}

static void level_free(level_t* L) {
    free(L->e);
    L->e = NULL;
}

/* level.hpp:57 */
static inline double harmonic_mean(double x, double y) { return 2.0 * x * y / (x + y); }

/* level.hpp:79-97: harmonic faces, boundary face = own permeability. */
static void level_build(level_t* L, const double* RESTRICT a) {
    const int64_t n = L->n;
    OMP(parallel for schedule(static) if (L->parallel))
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = 0; j < n; ++j) {
            const int64_t k = i * n + j;
            const double c = a[k];
            L->e[k] = (j + 1 < n) ? harmonic_mean(c, a[k + 1]) : c;
            L->w[k] = (j > 0) ? harmonic_mean(c, a[k - 1]) : c;
            L->nn[k] = (i + 1 < n) ? harmonic_mean(c, a[k + n]) : c;
            L->s[k] = (i > 0) ? harmonic_mean(c, a[k - n]) : c;
            const double d = L->e[k] + L->w[k] + L->nn[k] + L->s[k];
            L->diag[k] = d;
            L->inv_diag[k] = 1.0 / d;
        }
    }
}

/* level.hpp:105-119: y = A x */
static void level_apply(const level_t* L, const double* RESTRICT x, double* RESTRICT y) {
    const int64_t n = L->n;
    OMP(parallel for schedule(static) if (L->parallel))
    for (int64_t i = 0; i < n; ++i) {
        const int64_t row = i * n;
        for (int64_t j = 0; j < n; ++j) {
            const int64_t k = row + j;
            double v = L->diag[k] * x[k];
            if (j + 1 < n) v -= L->e[k] * x[k + 1];
            if (j > 0) v -= L->w[k] * x[k - 1];
            if (i + 1 < n) v -= L->nn[k] * x[k + n];
            if (i > 0) v -= L->s[k] * x[k - n];
            y[k] = v;
        }
    }
}

/* level.hpp:122-137: r = b - A x */
static void level_residual(const level_t* L, const double* RESTRICT x, const double* RESTRICT b,
                           double* RESTRICT r) {
    const int64_t n = L->n;
    OMP(parallel for schedule(static) if (L->parallel))
    for (int64_t i = 0; i < n; ++i) {
        const int64_t row = i * n;
        for (int64_t j = 0; j < n; ++j) {
            const int64_t k = row + j;
            double v = L->diag[k] * x[k];
            if (j + 1 < n) v -= L->e[k] * x[k + 1];
            if (j > 0) v -= L->w[k] * x[k - 1];
            if (i + 1 < n) v -= L->nn[k] * x[k + n];
            if (i > 0) v -= L->s[k] * x[k - n];
            r[k] = b[k] - v;
        }
    }
}

/* level.hpp:145-161: one colour of red-black Gauss-Seidel, in place. */
static void level_gs(const level_t* L, double* RESTRICT x, const double* RESTRICT b, int colour) {
    const int64_t n = L->n;
    OMP(parallel for schedule(static) if (L->parallel))
    for (int64_t i = 0; i < n; ++i) {
        const int64_t row = i * n;
        for (int64_t j = (i + colour) & 1; j < n; j += 2) {
            const int64_t k = row + j;
            double v = b[k];
            if (j + 1 < n) v += L->e[k] * x[k + 1];
            if (j > 0) v += L->w[k] * x[k - 1];
            if (i + 1 < n) v += L->nn[k] * x[k + n];
            if (i > 0) v += L->s[k] * x[k - n];
            x[k] = v * L->inv_diag[k];
        }
    }
}

/* level.hpp:164 */
static int64_t coarse_side(int64_t n) { return (n + 1) / 2; }

/* level.hpp:171-211: Galerkin coarse operator by face summation. */
static int level_coarsen(const level_t* F, level_t* C) {
    if (level_alloc(C, coarse_side(F->n)) != 0) return -1;
    const int64_t n = F->n, nc = C->n;
    OMP(parallel for schedule(static) if (F->parallel))
    for (int64_t I = 0; I < nc; ++I) {
        const int64_t i0 = 2 * I;
        const int64_t i1 = (2 * I + 1 < n) ? 2 * I + 1 : 2 * I;
        for (int64_t J = 0; J < nc; ++J) {
            const int64_t j0 = 2 * J;
            const int64_t j1 = (2 * J + 1 < n) ? 2 * J + 1 : 2 * J;
            double ce = 0.0, cw = 0.0, cn = 0.0, cs = 0.0;
            for (int64_t i = i0; i <= i1; ++i) {
                ce += F->e[i * n + j1];
                cw += F->w[i * n + j0];
            }
            for (int64_t j = j0; j <= j1; ++j) {
                cn += F->nn[i1 * n + j];
                cs += F->s[i0 * n + j];
            }
            const int64_t k = I * nc + J;
            C->e[k] = ce;
            C->w[k] = cw;
            C->nn[k] = cn;
            C->s[k] = cs;
            const double d = ce + cw + cn + cs;
            C->diag[k] = d;
            C->inv_diag[k] = 1.0 / d;
        }
    }
    return 0;
}

/* level.hpp:214-227: r_c = P^T r (sum over each 2x2 aggregate). */
static void level_restrict(int64_t n, int parallel, const double* RESTRICT fine, double* RESTRICT coarse) {
    const int64_t nc = coarse_side(n);
    OMP(parallel for schedule(static) if (parallel))
    for (int64_t I = 0; I < nc; ++I) {
        const int64_t i1 = (2 * I + 1 < n) ? 2 * I + 1 : 2 * I;
        for (int64_t J = 0; J < nc; ++J) {
            const int64_t j1 = (2 * J + 1 < n) ? 2 * J + 1 : 2 * J;
            double s = 0.0;
            for (int64_t i = 2 * I; i <= i1; ++i)
                for (int64_t j = 2 * J; j <= j1; ++j) s += fine[i * n + j];
            coarse[I * nc + J] = s;
        }
    }
}

/* level.hpp:230-237: x += P x_c (injection into the 2x2 children). */
static void level_prolong_add(int64_t n, int parallel, const double* RESTRICT coarse, double* RESTRICT fine) {
    const int64_t nc = coarse_side(n);
    OMP(parallel for schedule(static) if (parallel))
    for (int64_t i = 0; i < n; ++i) {
        const int64_t I = i / 2;
        for (int64_t j = 0; j < n; ++j) fine[i * n + j] += coarse[I * nc + j / 2];
    }
}

/* ------------------------------------------------------------- multigrid */

typedef struct {
    int pre, post, cycle;
    int num_levels;
    level_t lv[MAX_LEVELS];
    double *x[MAX_LEVELS], *b[MAX_LEVELS], *r[MAX_LEVELS];
} mg_t;

static void mg_free(mg_t* M) {
    for (int l = 0; l < M->num_levels; ++l) {
        level_free(&M->lv[l]);
        free(M->x[l]);
    }
    M->num_levels = 0;
}

/* multigrid.hpp:55-71: coarsen until a level is 1 x 1 (min_coarse_n = 1),
 * capped at max_levels = 32. Takes ownership of `fine`. */
static int mg_build(mg_t* M, level_t fine, int pre, int post, int cycle) {
    memset(M, 0, sizeof(*M));
    M->pre = pre;
    M->post = post;
    M->cycle = cycle;
    M->lv[0] = fine;
    M->num_levels = 1;
    while (M->num_levels < MAX_LEVELS) {
        const level_t* top = &M->lv[M->num_levels - 1];
        if (top->n <= 1) break;
        if (level_coarsen(top, &M->lv[M->num_levels]) != 0) {
            mg_free(M);
            return -1;
        }
        M->num_levels++;
    }
    for (int l = 0; l < M->num_levels; ++l) {
        const size_t m = (size_t)M->lv[l].size;
        double* block = (double*)calloc(3 * m, sizeof(double));
        if (!block) {
            mg_free(M);
            return -1;
        }
        M->x[l] = block;
        M->b[l] = block + m;
        M->r[l] = block + 2 * m;
    }
    return 0;
}

/* multigrid.hpp:129-146 */
static void mg_coarsest(const level_t* A, double* x, const double* b) {
    if (A->size == 1) {
        x[0] = b[0] * A->inv_diag[0];
        return;
    }
    for (int s = 0; s < COARSEST_SWEEPS; ++s) {
        level_gs(A, x, b, 0);
        level_gs(A, x, b, 1);
    }
    for (int s = 0; s < COARSEST_SWEEPS; ++s) {
        level_gs(A, x, b, 1);
        level_gs(A, x, b, 0);
    }
}

/* multigrid.hpp:97-127: recursive V (cycle 1) / W (cycle 2) cycle. */
static void mg_run_cycle(const mg_t* M, int l) {
    const level_t* A = &M->lv[l];
    double* x = M->x[l];
    const double* b = M->b[l];
    if (l + 1 == M->num_levels) {
        mg_coarsest(A, x, b);
        return;
    }
    for (int s = 0; s < M->pre; ++s) {
        level_gs(A, x, b, 0);
        level_gs(A, x, b, 1);
    }
    level_residual(A, x, b, M->r[l]);
    level_restrict(A->n, A->parallel, M->r[l], M->b[l + 1]);
    b_fill(M->x[l + 1], 0.0, M->lv[l + 1].size);
    for (int g = 0; g < M->cycle; ++g) mg_run_cycle(M, l + 1);
    level_prolong_add(A->n, A->parallel, M->x[l + 1], x);
    for (int s = 0; s < M->post; ++s) {
        level_gs(A, x, b, 1);
        level_gs(A, x, b, 0);
    }
}

/* multigrid.hpp:88-93: z = M^{-1} r from a zero initial guess. */
static void mg_apply(const mg_t* M, const double* r, double* z) {
    const int64_t m = M->lv[0].size;
    memcpy(M->b[0], r, sizeof(double) * (size_t)m);
    b_fill(M->x[0], 0.0, m);
    mg_run_cycle(M, 0);
    memcpy(z, M->x[0], sizeof(double) * (size_t)m);
}

/* ---------------------------------------------------------------- solver */

/* solver.hpp:68-77 */
static int validate_permeability(const double* a, int64_t size, char* err, int err_len) {
    for (int64_t i = 0; i < size; ++i) {
        if (!(a[i] > 0.0) || !isfinite(a[i])) {
            char msg[200];
            snprintf(msg, sizeof msg,
                     "permeability must be finite and strictly positive everywhere; "
                     "offending value at flat index %lld",
                     (long long)i);
            set_err(err, err_len, msg);
            return ORACLE_INVALID;
        }
    }
    return ORACLE_OK;
}

static int validate_options(int64_t n, const oracle_options* o, char* err, int err_len) {
    /* solver.hpp:85-87 */
    if (n < 1) {
        set_err(err, err_len, "grid size must be at least 1");
        return ORACLE_INVALID;
    }
    if (o->tol <= 0.0) {
        set_err(err, err_len, "tol must be positive");
        return ORACLE_INVALID;
    }
    if (o->max_iter < 1) {
        set_err(err, err_len, "max_iter must be at least 1");
        return ORACLE_INVALID;
    }
    if (o->preconditioner < 0 || o->preconditioner > 2) {
        set_err(err, err_len, "unknown preconditioner");
        return ORACLE_INVALID;
    }
    /* bindings.cpp:43-46 */
    if (o->pre_sweeps < 1 || o->post_sweeps < 1) {
        set_err(err, err_len, "pre_sweeps and post_sweeps must be at least 1");
        return ORACLE_INVALID;
    }
    if (o->cycle_index < 1 || o->cycle_index > 2) {
        set_err(err, err_len, "cycle_index must be 1 (V-cycle) or 2 (W-cycle)");
        return ORACLE_INVALID;
    }
    return ORACLE_OK;
}

/* solver.hpp:83-174 (u0 == NULL), plus a warm start from u0 when given. */
static int pcg(const double* a, const double* rhs, const double* u0, int64_t n, const oracle_options* o,
               double* u, double* history, oracle_result* res, char* err, int err_len) {
    int rc = validate_options(n, o, err, err_len);
    if (rc) return rc;
    const int64_t size = n * n;
    rc = validate_permeability(a, size, err, err_len);
    if (rc) return rc;

    const double h = 1.0 / (double)(n + 1);
    const double h2 = h * h;

    level_t fine;
    if (level_alloc(&fine, n) != 0) return ORACLE_NOMEM;
    level_build(&fine, a);

    memset(res, 0, sizeof(*res));
    res->levels = 1;
    res->residual = 0.0;
    for (int64_t i = 0; i < size; ++i) u[i] = 0.0;

    double* work = (double*)malloc(sizeof(double) * 5 * (size_t)size);
    if (!work) {
        level_free(&fine);
        return ORACLE_NOMEM;
    }
    double *b = work, *r = work + size, *z = work + 2 * size, *p = work + 3 * size, *ap = work + 4 * size;
    for (int64_t i = 0; i < size; ++i) b[i] = rhs[i] * h2;

    const double b_norm = sqrt(b_dot(b, b, size));
    if (b_norm == 0.0) { /* solver.hpp:104-108 */
        res->converged = 1;
        free(work);
        level_free(&fine);
        return ORACLE_OK;
    }

    mg_t mg;
    int have_mg = 0;
    if (o->preconditioner == ORACLE_PC_MULTIGRID) {
        if (mg_build(&mg, fine, o->pre_sweeps, o->post_sweeps, o->cycle_index) != 0) {
            free(work);
            return ORACLE_NOMEM;
        }
        have_mg = 1;
        res->levels = mg.num_levels;
    }
    const level_t* A = have_mg ? &mg.lv[0] : &fine;

    /* r = b, or r = b - A u0 for a warm start. */
    if (u0) {
        for (int64_t i = 0; i < size; ++i) u[i] = u0[i];
        level_residual(A, u, b, r);
    } else {
        memcpy(r, b, sizeof(double) * (size_t)size);
    }

#define PRECONDITION(in, to)                                                           \
    do {                                                                               \
        if (o->preconditioner == ORACLE_PC_NONE) {                                     \
            memcpy((to), (in), sizeof(double) * (size_t)size);                         \
        } else if (o->preconditioner == ORACLE_PC_JACOBI) {                            \
            for (int64_t q = 0; q < size; ++q) (to)[q] = (in)[q] * A->inv_diag[q];     \
        } else {                                                                       \
            mg_apply(&mg, (in), (to));                                                 \
        }                                                                              \
    } while (0)

    int hlen = 0;
    if (u0) {
        /* Warm start: the first residual is measured, not assumed to be 1. */
        res->residual = sqrt(b_dot(r, r, size)) / b_norm;
        if (o->record_history && history) history[hlen++] = res->residual;
        if (res->residual < o->tol) {
            res->converged = 1;
            goto done;
        }
    } else {
        res->residual = 1.0;
        if (o->record_history && history) history[hlen++] = 1.0;
    }

    PRECONDITION(r, z);
    memcpy(p, z, sizeof(double) * (size_t)size);
    double rz = b_dot(r, z, size);

    for (int it = 0; it < o->max_iter; ++it) {
        level_apply(A, p, ap);
        const double p_ap = b_dot(p, ap, size);
        if (!(fabs(p_ap) > 0.0) || !isfinite(p_ap)) { /* solver.hpp:149-155 */
            res->iterations = it;
            res->converged = 0;
            goto done;
        }
        const double alpha = rz / p_ap;
        const double rr = b_cg_update(alpha, p, ap, u, r, size);
        res->residual = sqrt(rr) / b_norm;
        res->iterations = it + 1;
        if (o->record_history && history) history[hlen++] = res->residual;
        if (res->residual < o->tol) {
            res->converged = 1;
            break;
        }
        PRECONDITION(r, z);
        const double rz_new = b_dot(r, z, size);
        const double beta = rz_new / rz;
        rz = rz_new;
        b_xpby(z, beta, p, size);
    }
#undef PRECONDITION
done:
    res->history_len = hlen;
    free(work);
    if (have_mg)
        mg_free(&mg);
    else
        level_free(&fine);
    return ORACLE_OK;
}

int oracle_solve(const double* a, const double* f, int64_t n, const oracle_options* opt, double* u,
                 double* history, oracle_result* res, char* err, int err_len) {
    return pcg(a, f, NULL, n, opt, u, history, res, err, err_len);
}

int oracle_solve_x0(const double* a, const double* f, const double* u0, int64_t n,
                    const oracle_options* opt, double* u, oracle_result* res, char* err, int err_len) {
    return pcg(a, f, u0, n, opt, u, NULL, res, err, err_len);
}

/* bindings.cpp:140-197: samples in parallel, kernels inside each solve serial
 * (nested regions are inactive); the first failure is reported after the join. */
int oracle_solve_batch(const double* a, const double* f, int64_t batch, int64_t n,
                       const oracle_options* opt, int threads, double* u, int* iterations,
                       double* residuals, int* converged, char* err, int err_len) {
    const int64_t stride = n * n;
    int failed = 0;
    int fail_rc = ORACLE_OK;
    oracle_options o = *opt;
    o.record_history = 0;
#ifdef _OPENMP
    const int nthreads = threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
#endif
    OMP(parallel for schedule(dynamic) num_threads(nthreads))
    for (int64_t s = 0; s < batch; ++s) {
        oracle_result r;
        char local_err[256] = {0};
        const int rc = pcg(a + s * stride, f, NULL, n, &o, u + s * stride, NULL, &r, local_err,
                           (int)sizeof local_err);
        if (rc == ORACLE_OK) {
            iterations[s] = r.iterations;
            residuals[s] = r.residual;
            converged[s] = r.converged;
        } else {
            OMP(critical)
            {
                if (!failed) {
                    failed = 1;
                    fail_rc = rc;
                    set_err(err, err_len, local_err);
                }
            }
        }
    }
    return fail_rc;
}

/* bindings.cpp:199-216 */
int oracle_apply_operator(const double* a, const double* x, int64_t n, double* y, char* err, int err_len) {
    if (n < 1) {
        set_err(err, err_len, "a must be a square 2-D array with at least one cell");
        return ORACLE_INVALID;
    }
    int rc = validate_permeability(a, n * n, err, err_len);
    if (rc) return rc;
    level_t L;
    if (level_alloc(&L, n) != 0) return ORACLE_NOMEM;
    level_build(&L, a);
    level_apply(&L, x, y);
    level_free(&L);
    return ORACLE_OK;
}

/* bindings.cpp:218-245 */
int oracle_apply_preconditioner(const double* a, const double* r, int64_t n, int pre_sweeps,
                                int post_sweeps, int cycle_index, double* z, char* err, int err_len) {
    if (n < 1) {
        set_err(err, err_len, "a must be a square 2-D array with at least one cell");
        return ORACLE_INVALID;
    }
    int rc = validate_permeability(a, n * n, err, err_len);
    if (rc) return rc;
    if (pre_sweeps < 1 || post_sweeps < 1) {
        set_err(err, err_len, "sweeps must be at least 1");
        return ORACLE_INVALID;
    }
    if (cycle_index < 1 || cycle_index > 2) {
        set_err(err, err_len, "cycle_index must be 1 or 2");
        return ORACLE_INVALID;
    }
    level_t L;
    if (level_alloc(&L, n) != 0) return ORACLE_NOMEM;
    level_build(&L, a);
    mg_t mg;
    if (mg_build(&mg, L, pre_sweeps, post_sweeps, cycle_index) != 0) return ORACLE_NOMEM;
    mg_apply(&mg, r, z);
    mg_free(&mg);
    return ORACLE_OK;
}

int oracle_num_levels(int64_t n) {
    int levels = 1;
    while (n > 1 && levels < MAX_LEVELS) {
        n = coarse_side(n);
        ++levels;
    }
    return levels;
}

int64_t oracle_hierarchy(const double* a, int64_t n, double* out, int64_t capacity) {
    level_t L;
    if (n < 1 || level_alloc(&L, n) != 0) return -1;
    level_build(&L, a);
    mg_t mg;
    if (mg_build(&mg, L, 1, 1, 2) != 0) return -1;
    int64_t off = 0;
    for (int l = 0; l < mg.num_levels; ++l) {
        const level_t* V = &mg.lv[l];
        if (off + 6 * V->size > capacity) {
            mg_free(&mg);
            return -1;
        }
        memcpy(out + off, V->e, sizeof(double) * 6 * (size_t)V->size);
        off += 6 * V->size;
    }
    mg_free(&mg);
    return off;
}

static int level_from_a(level_t* L, const double* a, int64_t n) {
    if (n < 1 || level_alloc(L, n) != 0) return -1;
    level_build(L, a);
    return 0;
}

int oracle_level_gs(const double* a, int64_t n, double* x, const double* b, int colour) {
    level_t L;
    if (level_from_a(&L, a, n)) return -1;
    level_gs(&L, x, b, colour);
    level_free(&L);
    return 0;
}

int oracle_level_residual(const double* a, int64_t n, const double* x, const double* b, double* r) {
    level_t L;
    if (level_from_a(&L, a, n)) return -1;
    level_residual(&L, x, b, r);
    level_free(&L);
    return 0;
}

int oracle_level_restrict(int64_t n, const double* fine, double* coarse) {
    level_restrict(n, n * n >= MIN_PARALLEL, fine, coarse);
    return 0;
}

int oracle_level_prolong_add(int64_t n, const double* coarse, double* fine) {
    level_prolong_add(n, n * n >= MIN_PARALLEL, coarse, fine);
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

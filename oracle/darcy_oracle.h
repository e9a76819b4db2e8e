/*
 * CPU oracle for the darcy MG-PCG solve path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (darcy-cpp v1.0.0,
 * include/darcy/{level,multigrid,solver,blas}.hpp and src/bindings.cpp), used by
 * the tests as the parity reference and by bench.py as the timed CPU baseline.
 * The GPU library never links, loads or calls this code.
 *
 * Parity pin: tests/test_oracle.py checks this restatement against golden
 * vectors produced by the reference itself (its own headers compiled by
 * oracle/build_ref.sh), see tests/golden/make_golden.py.
 */
#ifndef DARCY_ORACLE_H
#define DARCY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Preconditioner codes, reference include/darcy/solver.hpp:31-35. */
enum { ORACLE_PC_NONE = 0, ORACLE_PC_JACOBI = 1, ORACLE_PC_MULTIGRID = 2 };

/* Return codes. */
enum { ORACLE_OK = 0, ORACLE_INVALID = 1, ORACLE_NOMEM = 2 };

typedef struct {
    double tol;          /* solver.hpp:41 */
    int max_iter;        /* solver.hpp:42 */
    int preconditioner;  /* solver.hpp:43 */
    int pre_sweeps;      /* multigrid.hpp:31 */
    int post_sweeps;     /* multigrid.hpp:33 */
    int cycle_index;     /* multigrid.hpp:42 */
    int record_history;  /* solver.hpp:45 */
} oracle_options;

typedef struct {
    int iterations;
    double residual;
    int converged;
    int levels;
    int history_len; /* entries written to the caller's history buffer */
} oracle_result;

/* darcy::solve (solver.hpp:83-174). `u` (n*n) is written; `history` may be
 * NULL or hold max_iter + 1 doubles. `threads` > 0 sets the OpenMP team size
 * for this call, 0 keeps the current setting. */
int oracle_solve(const double* a, const double* f, int64_t n, const oracle_options* opt, double* u,
                 double* history, oracle_result* res, char* err, int err_len);

/* Warm-started variant: PCG from u0 instead of 0 (same stopping test,
 * ||r|| / ||b|| < tol with r = b - A u0). Not in the reference; used to assess
 * the learned warm start. */
int oracle_solve_x0(const double* a, const double* f, const double* u0, int64_t n,
                    const oracle_options* opt, double* u, oracle_result* res, char* err, int err_len);

/* _core.solve_batch (bindings.cpp:140-197): OpenMP schedule(dynamic) over
 * samples with `threads` threads (0 = omp_get_max_threads()). */
int oracle_solve_batch(const double* a, const double* f, int64_t batch, int64_t n,
                       const oracle_options* opt, int threads, double* u, int* iterations,
                       double* residuals, int* converged, char* err, int err_len);

/* _core.apply_operator (bindings.cpp:199-216). */
int oracle_apply_operator(const double* a, const double* x, int64_t n, double* y, char* err, int err_len);

/* _core.apply_preconditioner (bindings.cpp:218-245). */
int oracle_apply_preconditioner(const double* a, const double* r, int64_t n, int pre_sweeps,
                                int post_sweeps, int cycle_index, double* z, char* err, int err_len);

/* Number of levels the hierarchy has for an n x n grid (multigrid.hpp:55-64). */
int oracle_num_levels(int64_t n);

/* Dump the whole hierarchy: for level l with side n_l and m_l = n_l^2 cells,
 * writes e, w, n, s, diag, inv_diag (6 * m_l doubles, in that order) into
 * `out` at the running offset. Returns the number of doubles written, or -1. */
int64_t oracle_hierarchy(const double* a, int64_t n, double* out, int64_t capacity);

/* Single-level kernels for unit tests of the GPU kernels. */
int oracle_level_gs(const double* a, int64_t n, double* x, const double* b, int colour);
int oracle_level_residual(const double* a, int64_t n, const double* x, const double* b, double* r);
int oracle_level_restrict(int64_t n, const double* fine, double* coarse);
int oracle_level_prolong_add(int64_t n, const double* coarse, double* fine);

int oracle_max_threads(void);
void oracle_set_threads(int t);

#ifdef __cplusplus
}
#endif
#endif

// C-ABI shim over the REFERENCE's own headers (darcy-cpp v1.0.0,
// include/darcy/*.hpp), compiled by oracle/build_ref.py from the checkout (or
// from the unmodified copies it stages in baseline/_ref/_src for a machine
// without one) into oracle/_ref/ (never committed). Test infrastructure only: it lets the
// golden-vector script and the oracle tests run the reference itself, so the
// C restatement in darcy_oracle.c is pinned against the real thing.
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "darcy/solver.hpp"

namespace {
void put(char* err, int len, const char* msg) {
    if (err && len > 0) {
        std::strncpy(err, msg, static_cast<std::size_t>(len) - 1);
        err[len - 1] = '\0';
    }
}
darcy::SolveOptions make(double tol, int max_iter, int pc, int pre, int post, int cycle, int hist) {
    darcy::SolveOptions o;
    o.tol = tol;
    o.max_iter = max_iter;
    o.preconditioner = pc == 0 ? darcy::Preconditioner::None
                       : pc == 1 ? darcy::Preconditioner::Jacobi
                                 : darcy::Preconditioner::Multigrid;
    o.multigrid.pre_sweeps = pre;
    o.multigrid.post_sweeps = post;
    o.multigrid.cycle_index = cycle;
    o.record_history = hist != 0;
    return o;
}
}  // namespace

extern "C" {

// darcy::solve (solver.hpp:83). Returns 0, or 1 with `err` filled.
int ref_solve(const double* a, const double* f, int64_t n, double tol, int max_iter, int pc, int pre,
              int post, int cycle, int hist, double* u, double* history, int* iterations,
              double* residual, int* converged, int* levels, int* history_len, char* err, int err_len) {
    try {
        const darcy::SolveResult r = darcy::solve(a, f, n, make(tol, max_iter, pc, pre, post, cycle, hist));
        std::memcpy(u, r.u.data(), sizeof(double) * r.u.size());
        *iterations = r.iterations;
        *residual = r.residual;
        *converged = r.converged ? 1 : 0;
        *levels = r.levels;
        *history_len = static_cast<int>(r.history.size());
        if (history)
            std::memcpy(history, r.history.data(), sizeof(double) * r.history.size());
        return 0;
    } catch (const std::exception& e) {
        put(err, err_len, e.what());
        return 1;
    }
}

int ref_apply_operator(const double* a, const double* x, int64_t n, double* y) {
    darcy::Level level(a, n);
    level.apply(x, y);
    return 0;
}

int ref_apply_preconditioner(const double* a, const double* r, int64_t n, int pre, int post, int cycle,
                             double* z) {
    darcy::MultigridOptions o;
    o.pre_sweeps = pre;
    o.post_sweeps = post;
    o.cycle_index = cycle;
    darcy::Multigrid mg(darcy::Level(a, n), o);
    mg.apply(r, z);
    return 0;
}

// Hierarchy dump in the same layout as oracle_hierarchy: per level e, w, n, s,
// diag, inv_diag. Faces are recovered through apply() on unit vectors since the
// Level class keeps them private: the column of A for cell k holds -face
// values at the neighbours and diag at k.
int64_t ref_hierarchy(const double* a, int64_t n, double* out, int64_t capacity) {
    darcy::Multigrid mg(darcy::Level(a, n), darcy::MultigridOptions{});
    int64_t off = 0;
    for (int l = 0; l < mg.num_levels(); ++l) {
        const darcy::Level& L = mg.level(l);
        const int64_t m = L.size(), nl = L.n();
        if (off + 6 * m > capacity) return -1;
        std::vector<double> unit(static_cast<std::size_t>(m), 0.0), col(static_cast<std::size_t>(m));
        double* e = out + off;
        double* w = e + m;
        double* nn = w + m;
        double* s = nn + m;
        double* d = s + m;
        double* inv = d + m;
        for (int64_t k = 0; k < m; ++k) {
            e[k] = w[k] = nn[k] = s[k] = 0.0;
        }
        for (int64_t k = 0; k < m; ++k) {
            unit[static_cast<std::size_t>(k)] = 1.0;
            L.apply(unit.data(), col.data());
            unit[static_cast<std::size_t>(k)] = 0.0;
            const int64_t i = k / nl, j = k % nl;
            // A[k-1][k] = -e[k-1] (east face of the west neighbour), etc.
            if (j > 0) e[k - 1] = -col[static_cast<std::size_t>(k - 1)];
            if (j + 1 < nl) w[k + 1] = -col[static_cast<std::size_t>(k + 1)];
            if (i > 0) nn[k - nl] = -col[static_cast<std::size_t>(k - nl)];
            if (i + 1 < nl) s[k + nl] = -col[static_cast<std::size_t>(k + nl)];
            d[k] = L.diag()[static_cast<std::size_t>(k)];
            inv[k] = L.inv_diag()[static_cast<std::size_t>(k)];
        }
        off += 6 * m;
    }
    return off;
}

int ref_num_levels(const double* a, int64_t n) {
    darcy::Multigrid mg(darcy::Level(a, n), darcy::MultigridOptions{});
    return mg.num_levels();
}

// _core.solve_batch's sample loop (bindings.cpp:166-188), restated.
int ref_solve_batch(const double* a, const double* f, int64_t batch, int64_t n, double tol, int max_iter,
                    int pc, int pre, int post, int cycle, int threads, double* u, int* iterations,
                    double* residuals, int* converged) {
    const darcy::SolveOptions o = make(tol, max_iter, pc, pre, post, cycle, 0);
    const int64_t stride = n * n;
    int failed = 0;
#ifdef _OPENMP
    const int nthreads = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
#endif
    for (int64_t s = 0; s < batch; ++s) {
        try {
            const darcy::SolveResult r = darcy::solve(a + s * stride, f, n, o);
            std::memcpy(u + s * stride, r.u.data(), sizeof(double) * static_cast<std::size_t>(stride));
            iterations[s] = r.iterations;
            residuals[s] = r.residual;
            converged[s] = r.converged ? 1 : 0;
        } catch (...) {
#pragma omp atomic write
            failed = 1;
        }
    }
    return failed;
}

void ref_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#endif
}
}

// Host-side view of the device engine: the structs shared between the kernel
// translation unit and the orchestration code, and the launch wrappers.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

#include "../../include/darcy_gpu.h"

#include "common.cuh"
#include "setup.cuh"

namespace dgpu {

// Device-resident state of one PCG solve (grid engine). Every loop kernel
// reads `done` on entry and returns if it is set; the last block of the
// reducing kernels updates the scalars (solver.hpp:146-172 restated).
struct CgState {
    double rz;        // r . z of the current direction
    double rzo;       // r_new . z_old (flexible beta of the mixed form)
    double beta;      // p = z + beta p
    double alpha;     // rz / (p . Ap)
    double bnorm;     // ||b||
    double residual;  // ||r|| / ||b|| (recursive residual, as the reference reports)
    double true_residual;  // ||b - A u|| / ||b|| recomputed after the loop
    double tol;
    double fscalar;   // constant forcing when no f array is given
    int it;
    int max_iter;
    int done;
    int converged;
    int record_history;
    int use_cond;                 // a graph conditional handle is live
    cudaGraphConditionalHandle cond;
    double* history;              // max_iter + 1 entries, or null
    unsigned long long bad;       // first invalid permeability index, or ~0
    unsigned ticket[4];           // reduction tickets
};

// One problem of a batched (block-engine) solve.
struct BatchArgs {
    int count;
    const int* order;           // processing order, largest first
    const int* side;            // n per problem
    const int64_t* off;         // first cell of each problem in the packed arrays
    const double* a;            // packed permeability
    const double* f;            // packed forcing, or null for the scalar
    double fscalar;
    int f_shared;               // f is one n*n array shared by every problem
    const double* u0;           // packed warm start, or null
    int u0_fallback;            // a warm start no better than zero in estimated energy norm is replaced by zero
    double* u;                  // packed solution (device)
    int* iterations;
    double* residual;
    int* converged;
    int* levels;
    double* true_residual;
    unsigned long long* bad;    // per problem, ~0 if valid
    double* history;            // count == 1 only: max_iter + 1 entries
    unsigned* work;             // dynamic work counter (zeroed before launch)
    char* scratch;              // per-CTA arena
    size_t scratch_stride;
    size_t smem_budget;         // dynamic shared memory per CTA for the coarse levels
    double tol;
    int max_iter;
    int pc;                     // 0 none, 1 jacobi, 2 multigrid
    int pre, post, gamma;
    int record_history;
};

}  // namespace dgpu

#include "fused.cuh"  // needs CgState

namespace dgpu {

constexpr int kPcNone = 0, kPcJacobi = 1, kPcMultigrid = 2;
constexpr int kThreads = 256;     // grid-engine block size
constexpr int kMaxBlocks = 152 * 8;

inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of per-CTA scratch the batched engine needs for a side-n problem.
size_t block_arena_bytes(int n, bool mixed, size_t smem_budget);
int num_levels_for(int n);

// Message returned by dgpu_last_error() on this thread (solver.cu).
void set_last_error(const char* msg);

// Learned warm start (learn.cu), for the batched solve.
int net_predict_on_stream(dgpu_net* net, const double* d_a, double fscalar, int64_t count, double* d_u0,
                          cudaStream_t stream, std::string* msg);
int net_side(const dgpu_net* net);
int64_t net_launches(const dgpu_net* net);

// Programmatic dependent launch for the grid engine's kernels (on by
// default; DARCY_GPU_PDL=0 turns it off).
void set_programmatic_launch(bool on);
bool programmatic_launch();

// ---- launch wrappers (kernels.cu) ----
void launch_build_fine(const double* a, const Lvl64& L, unsigned long long* bad, cudaStream_t s);
void launch_coarsen(const Lvl64& F, const Lvl64& C, cudaStream_t s);
void launch_to_fp32(const Lvl64& L, float* e, float* nf, float* d, float* id, float* elo, float* nlo, float* dlo,
                    cudaStream_t s);

void launch_cg_init(const double* f, double h2, int64_t m, double* b, double* r, double* u, double* p,
                    float* b0f, float* b0lo, const double* u0, const Lvl64& L0, CgState* st, double* partials,
                    cudaStream_t s);
template <class T>
void launch_gs(const Lvl<T>& L, int colour, bool zero, CgState* st, cudaStream_t s);
template <class T>
void launch_residual_restrict(const Lvl<T>& L, T* bc, CgState* st, cudaStream_t s);
void launch_residual_restrict_df(const Lvl<float>& L, const float* elo, const float* nlo, const float* dlo,
                                 const float* blo, float* bc, CgState* st, cudaStream_t s);
template <class T>
void launch_prolong_gs1(const Lvl<T>& L, const T* xc, CgState* st, cudaStream_t s);
template <class T>
void launch_gs0_dot(const Lvl<T>& L, const double* r, CgState* st, double* partials, cudaStream_t s);
template <class T>
void launch_tail(const Lvl<T>* lv_dev, int l0, int nlev, int pre, int post, int gamma, int top_calls,
                 const double* id64, CgState* st, int threads, cudaStream_t s);
// Dense coarse-tail operator: columns (setup) and application (per visit).
void launch_tail_columns(const Lvl64* h_dev, const Lvl64* h_host, int l0, int nlev, int pre, int post, int gamma,
                         int top_calls, int N, double* Td, float* Tf, cudaStream_t s);
template <class T>
void launch_tail_matvec(const T* M, int N, const T* b, T* x, CgState* st, cudaStream_t s);
// Fused level visits (pre_sweeps = post_sweeps = 1): tile-staged red+black
// sweeps + residual + restriction, and prolongation + black+red sweeps
// (+ r . z on level 0). xin == null: iterate known to be zero.
template <class T>
void launch_visit_pre(const VisitLevel<T>& V, const T* xin, T* xout, T* bc, cudaStream_t s);
template <class T>
void launch_visit_mid(const VisitLevel<T>& V, const T* xin, const T* xc, T* xout, T* bc, cudaStream_t s);
template <class T>
void launch_visit_post(const VisitLevel<T>& V, const T* xin, const T* xc, T* xout, const double* r, CgState* st,
                       double* partials, cudaStream_t s);
template <class T>
void launch_dot_rz(const T* z, const double* r, int64_t m, CgState* st, double* partials, cudaStream_t s);
void launch_precond_diag(const double* r, const double* id, double* z, int64_t m, CgState* st,
                         double* partials, cudaStream_t s);
template <class Z>
void launch_xpby(const Z* z, double* p, int64_t m, CgState* st, cudaStream_t s);
void launch_apply_dot(const Lvl64& L, const double* p, double* ap, CgState* st, double* partials,
                      cudaStream_t s);
void launch_cg_update(const double* p, const double* ap, double* u, double* r, float* b0f, float* b0lo,
                      const float* zold, int64_t m, CgState* st, double* partials, cudaStream_t s);
void launch_true_residual(const Lvl64& L, const double* u, const double* b, double* scratch, CgState* st,
                          double* partials, cudaStream_t s);
void launch_apply(const Lvl64& L, const double* x, double* y, cudaStream_t s);
void launch_check_conversions(const double* x, int64_t m, float* hi, float* lo, float* rounded, double* widened,
                              unsigned long long* mismatches, cudaStream_t s);
template <class T>
void launch_copy_cast(const double* src, T* dst, int64_t m, cudaStream_t s);
template <class T>
void launch_copy_back(const T* src, double* dst, int64_t m, cudaStream_t s);

template <class T>
void launch_block_solve(const BatchArgs& args, int ctas, int threads, cudaStream_t s);
template <class T>
int block_solve_occupancy(int threads, size_t smem);


}  // namespace dgpu

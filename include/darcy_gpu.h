/*
 * darcy_gpu.h -- C ABI of the GB300 engine for the darcy MG-PCG solve path.
 *
 * libdarcy_gpu.so exports exactly the functions below: plain C types, host
 * pointers (or, for the *_device variants, device pointers), no C++ or torch
 * types. It is the layer that sits under the Python extension `_core`
 * (darcy_cpp_gb300/csrc/bindings.cpp), which keeps the reference's Python
 * signatures, messages and result types.
 *
 * Semantics follow the reference (darcy-cpp v1.0.0):
 *   - inputs are borrowed and never modified, outputs are written in full;
 *   - invalid shapes/values/parameters return DGPU_INVALID_INPUT with the
 *     reference's message text in dgpu_last_error();
 *   - non-convergence and CG breakdown are NOT errors: stats.converged = 0.
 *
 * All entry points are serialised per context (one internal mutex); a context
 * owns its CUDA stream, device buffers and captured graphs.
 */
#ifndef DARCY_GPU_H
#define DARCY_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define DGPU_OK 0
#define DGPU_INVALID_INPUT 1 /* reference: darcy::InvalidInput -> ValueError   */
#define DGPU_CUDA_ERROR 2    /* a CUDA call failed; message in dgpu_last_error */
#define DGPU_NO_MEMORY 3     /* device allocation failed                       */
#define DGPU_TIMEOUT 4       /* a bounded device-side wait gave up             */

/* Preconditioners, reference include/darcy/solver.hpp:31-35. */
#define DGPU_PC_NONE 0
#define DGPU_PC_JACOBI 1
#define DGPU_PC_MULTIGRID 2

/* Arithmetic forms. FP64: every step in double, the drop-in for darcy::solve.
 * MIXED: the multigrid cycle (smoothing, residual, transfers) in FP32 inside
 * the FP64 CG recurrence; Galerkin assembly, the coarsest solve, dots and the
 * true residual stay in FP64. */
#define DGPU_FORM_FP64 0
#define DGPU_FORM_MIXED 1

typedef struct dgpu_context dgpu_context;

/* reference SolveOptions (solver.hpp:40-46) + MultigridOptions
 * (multigrid.hpp:29-47) + the arithmetic form. */
typedef struct {
    double tol;         /* relative residual ||b - Au|| / ||b||, > 0        */
    int max_iter;       /* >= 1                                              */
    int preconditioner; /* DGPU_PC_*                                         */
    int pre_sweeps;     /* >= 1                                              */
    int post_sweeps;    /* >= 1                                              */
    int cycle_index;    /* 1 = V-cycle, 2 = W-cycle                          */
    int record_history; /* keep the per-iteration relative residual         */
    int form;           /* DGPU_FORM_*                                       */
} dgpu_options;

/* reference SolveResult (solver.hpp:48-56) without the arrays. */
typedef struct {
    int iterations;
    double residual;      /* recursive relative residual, as the reference reports */
    int converged;
    int levels;           /* multigrid levels (1 without multigrid, or f == 0) */
    int history_len;      /* entries written to history_out                    */
    double true_residual; /* ||b - A u|| / ||b|| recomputed on the device     */
    double device_ms;     /* CUDA-event time of the device work of this call   */
    int64_t kernel_launches; /* kernels this call launched on the device      */
} dgpu_stats;

/* One row of dgpu_profile_kernels. */
typedef struct {
    char name[48];
    double avg_ms;           /* mean device time of one launch (CUDA events)   */
    double bytes;            /* algorithmic bytes one launch moves             */
    double launches_per_iteration;
} dgpu_kernel_time;

/* Context lifetime. device < 0 selects the current device. */
int dgpu_create(int device, dgpu_context** out);
void dgpu_destroy(dgpu_context* ctx);

/* Message of the last failed call on this thread ("" if none). */
const char* dgpu_last_error(void);

/* Fill `out` (capacity bytes) with "name | SMs | compute capability | ...". */
int dgpu_device_info(dgpu_context* ctx, char* out, int capacity);

/* darcy::solve, reference solver.hpp:83-174 behind _core.solve
 * (src/bindings.cpp:117-138). a: n*n permeability; f: n*n forcing or NULL to
 * use f_scalar everywhere (bindings.cpp:51-63); u0: n*n warm start or NULL
 * (additive extension); u_out: n*n; history_out: NULL or max_iter + 1.
 * Host u_out buffers are written while the GPU computes (one element per
 * page, so that the copy out finds its pages mapped): they must not alias an
 * input. The same holds for every host-array entry point below. */
int dgpu_solve(dgpu_context* ctx, const double* a, const double* f, double f_scalar, int64_t n,
               const dgpu_options* opt, const double* u0, double* u_out, double* history_out,
               dgpu_stats* stats);

/* Same, on device-resident buffers (no host copies; `stream` may be NULL for
 * the context's stream, else a cudaStream_t the work is ordered after). */
int dgpu_solve_device(dgpu_context* ctx, const double* d_a, const double* d_f, double f_scalar, int64_t n,
                      const dgpu_options* opt, const double* d_u0, double* d_u, dgpu_stats* stats,
                      void* stream);

/* _core.solve_batch, reference src/bindings.cpp:140-197: `batch` problems of
 * one side n, packed (batch, n, n). f: NULL (f_scalar), one n*n array shared
 * by every sample (f_per_sample = 0, the reference's behaviour) or a packed
 * (batch, n, n) array (f_per_sample = 1). Outputs per sample. levels may be NULL.
 * Problems of side >= 384 run as up to four concurrent single solves (one
 * plan and stream each), smaller ones as one launch with one problem per CTA. */
int dgpu_solve_batch(dgpu_context* ctx, const double* a, const double* f, double f_scalar, int f_per_sample,
                     int64_t batch, int64_t n, const dgpu_options* opt, const double* u0, double* u_out,
                     int* iterations, double* residuals, int* converged, int* levels);

/* Same, on device-resident arrays (d_a, d_f, d_u0, d_u: device pointers,
 * packed as above); per-sample results in host arrays; device_ms (may be
 * NULL) receives the device time of the solve. Routed as dgpu_solve_batch.
 * Ordered after `stream` (may be NULL); returns when the results are written.
 * No reference counterpart. */
int dgpu_solve_batch_device(dgpu_context* ctx, const double* d_a, const double* d_f, double f_scalar,
                            int f_per_sample, int64_t batch, int64_t n, const dgpu_options* opt, const double* d_u0,
                            double* d_u, int* iterations, double* residuals, int* converged, int* levels,
                            double* device_ms, void* stream);

/* Kernels the context's last solve call launched on the device (a single
 * solve, a batch of any engine, or a learned batch). No reference counterpart. */
int64_t dgpu_last_launches(const dgpu_context* ctx);

/* Uneven-size batch (additive extension of solve_batch): problem p has side
 * sides[p] and occupies cells [off_p, off_p + sides[p]^2) of the packed
 * arrays, off_p being the running sum. f/u0 follow the same packing or NULL.
 * Each problem is routed as in dgpu_solve_batch: the small ones share one
 * launch, those of side >= 384 follow as concurrent single solves. */
int dgpu_solve_uneven(dgpu_context* ctx, int64_t count, const int64_t* sides, const double* a,
                      const double* f, double f_scalar, const dgpu_options* opt, const double* u0,
                      double* u_out, int* iterations, double* residuals, int* converged, int* levels);

/* _core.apply_operator, reference src/bindings.cpp:199-216: y = A x. */
int dgpu_apply_operator(dgpu_context* ctx, const double* a, const double* x, int64_t n, double* y);

/* _core.apply_preconditioner, reference src/bindings.cpp:218-245: one cycle
 * from a zero initial guess, z = M r. */
int dgpu_apply_preconditioner(dgpu_context* ctx, const double* a, const double* r, int64_t n, int pre_sweeps,
                              int post_sweeps, int cycle_index, int form, double* z);

/* Hierarchy dump for parity tests (reference level.hpp:79-97, :171-211): per
 * level l, e, w, n, s, diag, inv_diag (6 * n_l^2 doubles) at the running
 * offset. Returns the number of doubles written, or -1. */
int64_t dgpu_hierarchy(dgpu_context* ctx, const double* a, int64_t n, double* out, int64_t capacity);

/* Number of multigrid levels for an n x n grid (multigrid.hpp:55-64). */
int dgpu_num_levels(int64_t n);

/* Time the kernels of one CG iteration of the grid engine in isolation on
 * the field `a` (after one full solve): each of the finest-level kernels and
 * the dense coarse-tail product is launched `reps` times back to back inside a
 * CUDA graph between CUDA events on the context stream. Writes up to `cap`
 * rows and their count. Measurement hook; no counterpart in the reference. */
int dgpu_profile_kernels(dgpu_context* ctx, const double* a, int64_t n, const dgpu_options* opt, int reps,
                         dgpu_kernel_time* out, int cap, int* count);

/* Allocation-free z = M r (one multigrid cycle from a zero guess) for callers
 * that cannot allocate device memory while they run -- code inside a host
 * that owns all device memory itself (a serving pool, a framework allocator)
 * or a loop that must not enter cudaMalloc/cudaFree, which can synchronise
 * the device. No counterpart in the reference. The caller passes device
 * buffers a, r, z (n*n doubles each) and an optional cudaStream_t; the
 * scratch is a fixed 2 MiB array inside the library, present on every device
 * that loads it until the process exits, so n is limited to 1..128 (larger n
 * returns DGPU_INVALID_INPUT). No context is needed and nothing is allocated;
 * each call looks up the array's device address on the current device (the
 * first call on a device loads the library's device code there). All calls
 * share the one array, so calls that overlap on the GPU race; serialise them.
 * The call is synchronous: it waits for the stream and reads back a status
 * word (to report invalid permeability) before it returns, so it must never
 * be made on a stream that is being captured. */
int dgpu_apply_preconditioner_noalloc(const double* d_a, const double* d_r, int64_t n, int pre_sweeps,
                                      int post_sweeps, int cycle_index, double* d_z, void* stream);

/* Write `bytes` of device memory on the context stream (evicts L2 between
 * timed runs). */
int dgpu_flush_l2(dgpu_context* ctx, int64_t bytes);

/* Self-check of the engine's FP64<->FP32 conversions done on the integer and
 * FP32 pipes (the mixed form's CG kernels use them in place of the conversion
 * instructions): for each x[k] (host array), hi = (float)x, lo = (float)(x -
 * hi), rounded = (float)x by the rounding-only helper, widened = (double)hi.
 * Returns how many elements differ in any bit from the instruction forms, or
 * -1 on error. Test hook; no counterpart in the reference. */
int64_t dgpu_check_conversions(dgpu_context* ctx, const double* x, int64_t count, float* hi, float* lo,
                               float* rounded, double* widened);

/* Random two-phase fields on the GPU for training sets: the reference
 * generator's construction (python/darcy/fields.py:31-83: spectral amplitudes
 * tau^(alpha-1) (pi^2 |k|^2 + tau^2)^(-alpha/2), orthonormal inverse DCT,
 * threshold at zero -> hi / lo) with counter-based noise (Philox-4x32-10,
 * Box-Muller), so the fields match the host generator in distribution, not
 * bit for bit. out: count x n x n doubles (n <= 128), on the device when
 * out_on_device, else host memory; raw != 0 writes the unthresholded field. */
int dgpu_random_fields(int64_t n, int64_t count, unsigned long long seed, double alpha, double tau, double hi,
                       double lo, int raw, double* out, int out_on_device, void* stream);

/* ------------------------------------------------------------------------
 * Learned warm start. No counterpart in the reference (which always starts
 * PCG from u0 = 0, solver.hpp:96-102): a 6-layer 3x3 convolutional network
 * (2 -> 32 x 5 -> 1 channels, GELU, BF16 weights and activations, FP32
 * accumulation) maps (log a, f) on a side x side grid to a guess of u, which
 * the solve then refines to the same tolerance. Training data are (a, u)
 * pairs the solver produced (for example dgpu_solve_batch at tol 1e-10).
 * One network per grid side (even, 8..512).
 * Parameters are one FP32 vector: per layer l, w_l[cout][tap * cin + ci]
 * (tap = 3 * (dy + 1) + (dx + 1)), then b_l[cout]. Training minimises the
 * prediction's error in the energy norm of each sample's own operator (the
 * norm CG minimises), relative to the solution's, unless set otherwise. */
typedef struct dgpu_net dgpu_net;

#define DGPU_NET_TENSOR 0 /* 32 -> 32 convolutions on the tensor cores (default) */
#define DGPU_NET_SIMT 1   /* same arithmetic on the CUDA cores (cross-check)      */

/* New network on the current device, He-uniform weights from `seed`. */
int dgpu_net_create(int side, unsigned long long seed, dgpu_net** out);
void dgpu_net_destroy(dgpu_net* net);
int64_t dgpu_net_num_params(const dgpu_net* net);
int dgpu_net_side(const dgpu_net* net);
int dgpu_net_get_params(dgpu_net* net, float* out);
/* Replaces the parameters and resets the Adam moments. */
int dgpu_net_set_params(dgpu_net* net, const float* in);
/* Input/output scaling {mean of log a, std of log a, RMS of u at f = fref,
 * fref}; set by the first dgpu_net_load_pairs unless set here first. */
int dgpu_net_get_scaling(dgpu_net* net, double* out4);
int dgpu_net_set_scaling(dgpu_net* net, const double* in4);
int dgpu_net_set_engine(dgpu_net* net, int engine);
/* Test hook (no counterpart in the reference): how many times each
 * tensor-core convolution CTA polls its first MMA-completion mbarrier before
 * declaring the wait lost (default and maximum 2^24). 0 makes that wait run
 * out at once, so the timeout path can be exercised without a fault: the
 * kernel records the error, drains the MMA in flight with the full budget,
 * frees its tensor memory and returns, and the call reports DGPU_TIMEOUT.
 * Pass 1 << 24 to restore the default. */
int dgpu_net_set_first_wait(dgpu_net* net, long long polls);

#define DGPU_NET_LOSS_ENERGY 0 /* e^T A e / u^T A u per sample, batch mean (default) */
#define DGPU_NET_LOSS_MSE 1    /* mean of (u0 - u)^2 over all cells, u scaled to unit RMS */
int dgpu_net_set_loss(dgpu_net* net, int kind);
/* Host arrays: a and u packed (count, side, side); f NULL (f = 1) or one
 * scalar forcing per sample. Replaces the resident training set. */
int dgpu_net_load_pairs(dgpu_net* net, const double* a, const double* u, const double* f, int64_t count);
/* `steps` Adam steps (betas 0.9 / 0.999, eps 1e-8) on mini-batches drawn
 * without replacement from the resident set (a new permutation per epoch,
 * fixed by `seed`); the loss of each step goes to losses[steps] (may be NULL). */
int dgpu_net_train(dgpu_net* net, int64_t steps, int batch, float lr, unsigned long long seed, float* losses);
/* The loss and its gradient with respect to every parameter for one batch
 * of host samples (no update). */
int dgpu_net_gradients(dgpu_net* net, const double* a, const double* u, const double* f, int64_t count,
                       float* grad, float* loss);
/* The network's input for `count` samples, as it enters the first layer
 * (after BF16 rounding): out[count][side][side][2] = ((log a - mean) / std,
 * (f / fref) U1) where U1 is the grid's a = 1, f = 1 solution at unit RMS. */
int dgpu_net_features(dgpu_net* net, const double* a, const double* f, int64_t count, float* out);
/* u0 for `count` samples (host arrays). */
int dgpu_net_predict(dgpu_net* net, const double* a, const double* f, int64_t count, double* u0);
/* Same on device arrays, ordered after / before `stream` (may be NULL). */
int dgpu_net_predict_device(dgpu_net* net, const double* d_a, const double* d_f, int64_t count, double* d_u0,
                            void* stream);
/* Kernels launched by the network's last call. */
int64_t dgpu_net_last_launches(const dgpu_net* net);
/* Text description of the network and its launch shapes. */
int dgpu_net_info(dgpu_net* net, char* out, int capacity);

/* dgpu_solve_batch with the warm start predicted on the device by `net`
 * (whose side must equal n): the prediction never leaves the GPU. f is the
 * scalar f_scalar for every sample. */
int dgpu_solve_batch_learned(dgpu_context* ctx, dgpu_net* net, const double* a, double f_scalar, int64_t batch,
                             int64_t n, const dgpu_options* opt, double* u_out, int* iterations, double* residuals,
                             int* converged, int* levels);

#ifdef __cplusplus
}
#endif
#endif

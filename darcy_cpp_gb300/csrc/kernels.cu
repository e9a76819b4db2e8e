// sm_103a kernels of the darcy GB300 engine.
//
// Two engines share the level operations of common.cuh:
//   * the grid engine (one solve spread over the whole GPU): one kernel per
//     phase on the large levels, the coarse tail handed to one CTA, the PCG
//     scalars kept on the device so that no iteration waits for the host;
//   * the block engine (batched solves): one CTA runs a whole PCG solve of one
//     problem, pulling problems from a work counter, largest first.
#include <math.h>

#include <cstdlib>
#include <type_traits>
#include <algorithm>
#include <mutex>
#include <map>

#include "block.cuh"
#include "cycle.cuh"
#include "engine.h"
#include "fused.cuh"

namespace dgpu {

// ------------------------------------------------------------ small helpers

// Grid of the streaming (grid-stride) kernels: one wave of resident CTAs --
// SMs x the CTAs per SM this kernel's registers allow -- or fewer when the
// work is smaller, and never more than kMaxBlocks (the reduction partials).
// A fixed 1216 (8 per SM) ran 1.33 waves for the 40-register kernels (6 CTAs
// per SM): the last third of a wave took as long as a whole one.
template <typename... KArgs>
static int grid_fill(void (*kern)(KArgs...), int64_t work, int threads = kThreads) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> cap;
    int dev = 0;
    cudaGetDevice(&dev);
    int c;
    {
        std::lock_guard<std::mutex> lock(mu);
        const auto key = std::make_pair((const void*)kern, dev);
        auto it = cap.find(key);
        if (it == cap.end()) {
            int sms = 0, per = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, 0);
            it = cap.emplace(key, std::max(1, std::min(kMaxBlocks, std::max(sms, 1) * std::max(per, 1)))).first;
        }
        c = it->second;
    }
    int64_t g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > c) g = c;
    return (int)g;
}

// Launches of the grid engine go through launch_k: with programmatic
// serialization on (set_programmatic_launch), graph edges between them become
// programmatic so each kernel's launch overlaps its predecessor's tail.
static bool g_pdl = false;
void set_programmatic_launch(bool on) { g_pdl = on; }
bool programmatic_launch() { return g_pdl; }

template <typename... KArgs, typename... Args>
static void launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    if (!g_pdl) {
        kern<<<grid, block, smem, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

__device__ __forceinline__ void stop_loop(CgState* st) {
    if (st->use_cond) cudaGraphSetConditional(st->cond, 0u);
}

// Two-value variant of grid_sum_last.
__device__ __forceinline__ bool grid_sum2_last(double v1, double v2, double* partials, unsigned* ticket,
                                               double* scratch, double& t1, double& t2) {
    __shared__ bool s_last;
    const double b1 = block_sum_wide(v1, scratch);
    const double b2 = block_sum_wide(v2, scratch);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = b1;
        partials[2 * blockIdx.x + 1] = b2;
        __threadfence();
        s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double a1 = 0.0, a2 = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
        a1 += ((volatile double*)partials)[2 * q];
        a2 += ((volatile double*)partials)[2 * q + 1];
    }
    t1 = block_sum_wide(a1, scratch);
    t2 = block_sum_wide(a2, scratch);
    if (threadIdx.x == 0) *ticket = 0;
    return true;
}


// ------------------------------------------------------------- setup kernels

__global__ void k_build_fine(const double* __restrict__ a, Lvl64 L, unsigned long long* bad) {
    pdl_enter();
    build_fine<GridScope>(a, L, bad);
}
__global__ void k_coarsen(Lvl64 F, Lvl64 C) {
    pdl_enter(); coarsen<GridScope>(F, C); }
__global__ void k_to_fp32(Lvl64 L, float* e, float* nf, float* d, float* id, float* elo, float* nlo, float* dlo) {
    pdl_enter();
    to_fp32<GridScope>(L, e, nf, d, id, elo, nlo, dlo);
}

void launch_build_fine(const double* a, const Lvl64& L, unsigned long long* bad, cudaStream_t s) {
    launch_k(k_build_fine, grid_fill(k_build_fine, (int64_t)L.n * L.n), kThreads, 0, s, a, L, bad);
}
void launch_coarsen(const Lvl64& F, const Lvl64& C, cudaStream_t s) {
    launch_k(k_coarsen, grid_fill(k_coarsen, (int64_t)C.n * C.n), kThreads, 0, s, F, C);
}
void launch_to_fp32(const Lvl64& L, float* e, float* nf, float* d, float* id, float* elo, float* nlo, float* dlo,
                    cudaStream_t s) {
    launch_k(k_to_fp32, grid_fill(k_to_fp32, (int64_t)L.n * L.n), kThreads, 0, s, L, e, nf, d, id, elo, nlo, dlo);
}

// ---------------------------------------------------------------- PCG kernels

// b = f h^2 (solver.hpp:98-102), r = b (or b - A u0 for a warm start), u = 0
// (or u0), p = 0, ||b|| and the initial residual (solver.hpp:104-108, :143-144).
__global__ void k_cg_init(const double* __restrict__ f, double h2, int64_t m,
                          double* __restrict__ b, double* __restrict__ r, double* __restrict__ u,
                          double* __restrict__ p, float* __restrict__ b0f, float* __restrict__ b0lo,
                          const double* __restrict__ u0, Lvl64 L0, CgState* st, double* partials) {
    pdl_enter();
    __shared__ double red[kThreads];
    double sb = 0.0, sr = 0.0;
    const int n = L0.n;
    const double fscalar = st->fscalar;
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) {
        const double bk = (f ? f[k] : fscalar) * h2;
        double rk = bk;
        if (u0) {
            const int i = (int)k / n, j = (int)k - i * n;  // n^2 < 2^31
            rk = bk - apply_cell(L0, u0, i, j);
            u[k] = u0[k];
        } else {
            u[k] = 0.0;
        }
        b[k] = bk;
        r[k] = rk;
        p[k] = 0.0;
        if (b0f) {
            float hi, lo;
            split_f64(rk, hi, lo);
            b0f[k] = hi;
            b0lo[k] = lo;
        }
        sb += bk * bk;
        sr += rk * rk;
    }
    double tb, tr;
    if (!grid_sum2_last(sb, sr, partials, &st->ticket[0], red, tb, tr)) return;
    if (threadIdx.x == 0) {
        st->bnorm = sqrt(tb);
        st->it = 0;
        st->beta = 0.0;
        st->converged = 0;
        st->done = 0;
        if (st->bad != ~0ull) {  // invalid permeability: reported by the host, no iteration
            st->residual = 0.0;
            st->done = 1;
        } else if (st->bnorm == 0.0) {  // f == 0: u == 0 exactly, no iteration
            st->residual = 0.0;
            st->converged = 1;
            st->done = 1;
        } else {
            st->residual = u0 ? sqrt(tr) / st->bnorm : 1.0;
            if (u0 && st->residual < st->tol) {
                st->converged = 1;
                st->done = 1;
            }
        }
        if (st->record_history && st->history) st->history[0] = st->residual;
    }
}

// Level kernels: each returns at once when the solve has finished, so a
// converged iteration's remaining graph nodes cost only their launch.
template <class T>
__global__ void k_gs(Lvl<T> L, int c, bool zero, const CgState* st) {
    pdl_enter();
    if (st && st->done) return;
    gs_colour<GridScope>(L, c, zero);
}
template <class T>
__global__ void k_residual_restrict(Lvl<T> L, T* bc, const CgState* st) {
    pdl_enter();
    if (st && st->done) return;
    residual_restrict<GridScope>(L, bc);
}
// The FP32 cycle's residual + restriction in double-float arithmetic on FP32
// pipes: coefficients as hi + lo pairs, b with its lo part on level 0 (blo,
// else null), error-free products and compensated sums, summed per 2 x 2
// aggregate. Same operation order as the fused pre-visit (k_visit_pre), so
// both give the same bits.
__global__ void k_residual_restrict_df(Lvl<float> L, const float* __restrict__ elo, const float* __restrict__ nlo,
                                       const float* __restrict__ dlo, const float* __restrict__ blo,
                                       float* __restrict__ bc, const CgState* st) {
    pdl_enter();
    if (st && st->done) return;
    const int n = L.n, nc = (n + 1) / 2;
    const int64_t mc = (int64_t)nc * nc;
    for (int64_t K = GridScope::start(); K < mc; K += GridScope::stride()) {
        const int I = (int)(K / nc), J = (int)(K - (int64_t)I * nc);
        DF acc{0.f, 0.f};
        for (int di = 0; di < 2; ++di) {
            const int i = 2 * I + di;
            if (i >= n) break;
            for (int dj = 0; dj < 2; ++dj) {
                const int j = 2 * J + dj;
                if (j >= n) break;
                const int64_t k = (int64_t)i * n + j;
                const float xe = j + 1 < n ? L.x[k + 1] : 0.f, ee = j + 1 < n ? L.e[k] : 0.f,
                            el = j + 1 < n ? elo[k] : 0.f;
                const float xw = j > 0 ? L.x[k - 1] : 0.f, ew = j > 0 ? L.e[k - 1] : 0.f,
                            wl = j > 0 ? elo[k - 1] : 0.f;
                const float xn = i + 1 < n ? L.x[k + n] : 0.f, en = i + 1 < n ? L.nf[k] : 0.f,
                            nl = i + 1 < n ? nlo[k] : 0.f;
                const float xs = i > 0 ? L.x[k - n] : 0.f, es = i > 0 ? L.nf[k - n] : 0.f,
                            sl = i > 0 ? nlo[k - n] : 0.f;
                df_add(acc, L.b[k], blo ? blo[k] : 0.f);
                df_axpy(acc, L.d[k], dlo[k], L.x[k], -1.f);
                df_axpy(acc, ee, el, xe, 1.f);
                df_axpy(acc, ew, wl, xw, 1.f);
                df_axpy(acc, en, nl, xn, 1.f);
                df_axpy(acc, es, sl, xs, 1.f);
            }
        }
        bc[K] = acc.hi + acc.lo;
    }
}
template <class T>
__global__ void k_prolong_gs1(Lvl<T> L, const T* xc, const CgState* st) {
    pdl_enter();
    if (st && st->done) return;
    prolong_gs1<GridScope>(L, xc);
}

// Last post-smoothing pass on level 0 (colour 0) fused with rz = r . z and
// beta = rz_new / rz (solver.hpp:167-171). z is the level-0 iterate; in the
// mixed form it is the FP32 iterate widened to FP64 on the fly.
//
// kPairs (even n): one thread per pair of horizontally adjacent cells, one of
// each colour: the colour-0 one is updated (the same arithmetic as
// gs_colour), both enter r . z, and r is read once as 16-byte pairs instead
// of once per colour loop.
template <class T, bool kPairs>
__global__ void k_gs0_dot(Lvl<T> L, const double* __restrict__ r, CgState* st, double* partials) {
    pdl_enter();
    __shared__ double red[kThreads];
    if (st->done) return;
    const int n = L.n;
    double acc = 0.0;
    if constexpr (kPairs) {
        const int64_t m2 = (int64_t)n * n / 2;
        for (int64_t q = GridScope::start(); q < m2; q += GridScope::stride()) {
            const int k0 = (int)(2 * q);  // n^2 < 2^31
            const int i = k0 / n, j0 = k0 - i * n;
            const int jc = j0 + (i & 1);  // the colour-0 cell of the pair
            const int kc = i * n + jc, ko = (i & 1) ? k0 : k0 + 1;
            T v = L.b[kc];
            if (jc + 1 < n) v += L.e[kc] * L.x[kc + 1];
            if (jc > 0) v += L.e[kc - 1] * L.x[kc - 1];
            if (i + 1 < n) v += L.nf[kc] * L.x[kc + n];
            if (i > 0) v += L.nf[kc - n] * L.x[kc - n];
            const T xn = v * L.id[kc];
            const T xo = L.x[ko];
            L.x[kc] = xn;
            const double2 rv = reinterpret_cast<const double2*>(r)[q];
            acc += rv.x * widen_f32((i & 1) ? xo : xn);
            acc += rv.y * widen_f32((i & 1) ? xn : xo);
        }
        double tot;
        if (!grid_sum_last(acc, partials, &st->ticket[1], red, tot)) return;
        if (threadIdx.x == 0) {
            st->beta = st->it == 0 ? 0.0 : (tot - st->rzo) / st->rz;
            st->rz = tot;
        }
        return;
    }
    const int64_t cnt0 = colour_count(n, 0);
    for (int64_t t = GridScope::start(); t < cnt0; t += GridScope::stride()) {
        int i, j;
        colour_cell(n, 0, t, i, j);
        const int64_t k = (int64_t)i * n + j;
        T v = L.b[k];
        if (j + 1 < n) v += L.e[k] * L.x[k + 1];
        if (j > 0) v += L.e[k - 1] * L.x[k - 1];
        if (i + 1 < n) v += L.nf[k] * L.x[k + n];
        if (i > 0) v += L.nf[k - n] * L.x[k - n];
        const T xn = v * L.id[k];
        L.x[k] = xn;
        acc += r[k] * widen_f32(xn);
    }
    const int64_t cnt1 = colour_count(n, 1);
    for (int64_t t = GridScope::start(); t < cnt1; t += GridScope::stride()) {
        int i, j;
        colour_cell(n, 1, t, i, j);
        const int64_t k = (int64_t)i * n + j;
        acc += r[k] * widen_f32(L.x[k]);
    }
    double tot;
    if (!grid_sum_last(acc, partials, &st->ticket[1], red, tot)) return;
    if (threadIdx.x == 0) {
        st->beta = st->it == 0 ? 0.0 : (tot - st->rzo) / st->rz;
        st->rz = tot;
    }
}

// rz = r . z after a preconditioner that ended elsewhere (coarse-tail-only
// hierarchies).
template <class T>
__global__ void k_dot_rz(const T* __restrict__ z, const double* __restrict__ r, int64_t m, CgState* st,
                         double* partials) {
    pdl_enter();
    __shared__ double red[kThreads];
    if (st->done) return;
    double acc = 0.0;
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) acc += r[k] * widen_f32(z[k]);
    double tot;
    if (!grid_sum_last(acc, partials, &st->ticket[1], red, tot)) return;
    if (threadIdx.x == 0) {
        st->beta = st->it == 0 ? 0.0 : (tot - st->rzo) / st->rz;
        st->rz = tot;
    }
}

// Jacobi (z = r / d) or no preconditioner (z = r), with rz and beta
// (solver.hpp:122-137, :167-171). id == null selects "none".
__global__ void k_precond_diag(const double* __restrict__ r, const double* __restrict__ id,
                               double* __restrict__ z, int64_t m, CgState* st, double* partials) {
    pdl_enter();
    __shared__ double red[kThreads];
    if (st->done) return;
    double acc = 0.0;
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) {
        const double zk = id ? r[k] * id[k] : r[k];
        z[k] = zk;
        acc += r[k] * zk;
    }
    double tot;
    if (!grid_sum_last(acc, partials, &st->ticket[1], red, tot)) return;
    if (threadIdx.x == 0) {
        st->beta = st->it == 0 ? 0.0 : (tot - st->rzo) / st->rz;
        st->rz = tot;
    }
}

// p = z + beta p (blas.hpp:50-56). First node of every loop iteration: it is
// also where a finished solve stops the device-side while loop.
template <class Z>
__global__ void k_xpby(const Z* __restrict__ z, double* __restrict__ p, int64_t m, CgState* st) {
    pdl_enter();
    if (st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) stop_loop(st);
        return;
    }
    const double beta = st->beta;
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) p[k] = widen_f32(z[k]) + beta * p[k];
}

// ap = A p and p . Ap, then alpha or a breakdown (solver.hpp:147-156).
//
// kPairs: two consecutive cells per thread (two independent FP64 chains, one
// 16-byte store of Ap); needs 16-byte aligned p and ap.
template <bool kPairs>
__global__ void k_apply_dot(Lvl64 L, const double* __restrict__ p, double* __restrict__ ap, CgState* st,
                            double* partials) {
    pdl_enter();
    __shared__ double red[kThreads];
    if (st->done) return;
    const int n = L.n;
    const int64_t m = (int64_t)n * n;
    double acc = 0.0;
    if constexpr (kPairs) {
        const int64_t m2 = m >> 1;
        for (int64_t q = GridScope::start(); q < m2; q += GridScope::stride()) {
            const int k0 = (int)(2 * q);  // n^2 < 2^31
            const int i0 = k0 / n, j0 = k0 - i0 * n;
            const int i1 = j0 + 1 < n ? i0 : i0 + 1, j1 = j0 + 1 < n ? j0 + 1 : 0;
            const double y0 = apply_cell(L, p, i0, j0);
            const double y1 = apply_cell(L, p, i1, j1);
            reinterpret_cast<double2*>(ap)[q] = make_double2(y0, y1);
            const double2 pv = reinterpret_cast<const double2*>(p)[q];
            acc += pv.x * y0;
            acc += pv.y * y1;
        }
        if ((m & 1) && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) {  // odd m: the last cell
            const double y = apply_cell(L, p, n - 1, n - 1);
            ap[m - 1] = y;
            acc += p[m - 1] * y;
        }
    } else {
        for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) {
            const int i = (int)k / n, j = (int)k - i * n;  // n^2 < 2^31
            const double y = apply_cell(L, p, i, j);
            ap[k] = y;
            acc += p[k] * y;
        }
    }
    double pap;
    if (!grid_sum_last(acc, partials, &st->ticket[2], red, pap)) return;
    if (threadIdx.x == 0) {
        if (!(fabs(pap) > 0.0) || !isfinite(pap)) {
            st->converged = 0;
            st->done = 1;
            stop_loop(st);
        } else {
            st->alpha = st->rz / pap;
        }
    }
}

// u += alpha p, r -= alpha Ap, ||r||^2 (blas.hpp:62-77), then the stopping
// test (solver.hpp:159-165). The mixed form also emits r in FP32 as the
// level-0 right-hand side of the cycle, and r_new . z_old for the flexible
// (Polak-Ribiere) beta: its FP32 cycle is a slightly inexact preconditioner,
// and beta = r_new.(z_new - z_old) / r_old.z_old keeps CG's convergence rate
// with it. For an exact preconditioner r_new . z_old = 0 and the two betas agree.
//
// kPairs: two adjacent cells per thread through 16-byte loads and stores, the
// two pairs of a thread's two grid strides loaded before any arithmetic, so
// more loads are in flight (a 1024^2 level gives a thread only ~3 cells).
// Needs 16-byte aligned p, ap, u, r, 8-byte aligned b0f, b0lo, and no zold;
// used for the FP64 form.
__device__ __forceinline__ void cg_cell(double alpha, double pk, double apk, double& uk, double& rk, float* hi,
                                        float* lo, double& acc) {
    uk += alpha * pk;
    rk = rk - alpha * apk;
    if (hi) split_f64(rk, *hi, *lo);
    acc += rk * rk;
}

template <bool kPairs>
__global__ void k_cg_update(const double* __restrict__ p, const double* __restrict__ ap, double* __restrict__ u,
                            double* __restrict__ r, float* __restrict__ b0f, float* __restrict__ b0lo,
                            const float* __restrict__ zold, int64_t m, CgState* st, double* partials) {
    pdl_enter();
    __shared__ double red[kThreads];
    if (st->done) return;
    const double alpha = st->alpha;
    double acc = 0.0, acc2 = 0.0;
    if constexpr (kPairs) {
        const int64_t m2 = m >> 1, gs = GridScope::stride();
        const double2* p2 = reinterpret_cast<const double2*>(p);
        const double2* a2 = reinterpret_cast<const double2*>(ap);
        double2* u2 = reinterpret_cast<double2*>(u);
        double2* r2 = reinterpret_cast<double2*>(r);
        const bool mixed = b0f != nullptr;
        float2 hi, lo;
        for (int64_t q0 = GridScope::start(); q0 < m2; q0 += 2 * gs) {
            const int64_t q1 = q0 + gs;
            const bool two = q1 < m2;
            const double2 pa = p2[q0], aa = a2[q0];
            double2 ua = u2[q0], ra = r2[q0];
            double2 pb{0.0, 0.0}, ab{0.0, 0.0}, ub{0.0, 0.0}, rb{0.0, 0.0};
            if (two) {
                pb = p2[q1];
                ab = a2[q1];
                ub = u2[q1];
                rb = r2[q1];
            }
            cg_cell(alpha, pa.x, aa.x, ua.x, ra.x, mixed ? &hi.x : nullptr, &lo.x, acc);
            cg_cell(alpha, pa.y, aa.y, ua.y, ra.y, mixed ? &hi.y : nullptr, &lo.y, acc);
            u2[q0] = ua;
            r2[q0] = ra;
            if (mixed) {
                reinterpret_cast<float2*>(b0f)[q0] = hi;
                reinterpret_cast<float2*>(b0lo)[q0] = lo;
            }
            if (two) {
                cg_cell(alpha, pb.x, ab.x, ub.x, rb.x, mixed ? &hi.x : nullptr, &lo.x, acc);
                cg_cell(alpha, pb.y, ab.y, ub.y, rb.y, mixed ? &hi.y : nullptr, &lo.y, acc);
                u2[q1] = ub;
                r2[q1] = rb;
                if (mixed) {
                    reinterpret_cast<float2*>(b0f)[q1] = hi;
                    reinterpret_cast<float2*>(b0lo)[q1] = lo;
                }
            }
        }
        if ((m & 1) && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) {  // odd m: the last cell
            const int64_t k = m - 1;
            double uk = u[k], rk = r[k];
            float h, l;
            cg_cell(alpha, p[k], ap[k], uk, rk, mixed ? &h : nullptr, &l, acc);
            u[k] = uk;
            r[k] = rk;
            if (mixed) {
                b0f[k] = h;
                b0lo[k] = l;
            }
        }
    } else
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) {
        u[k] += alpha * p[k];
        const double rk = r[k] - alpha * ap[k];
        r[k] = rk;
        if (b0f) {  // r as FP32 hi + lo for the FP32 cycle
            float hi, lo;
            split_f64(rk, hi, lo);
            b0f[k] = hi;
            b0lo[k] = lo;
        }
        if (zold) acc2 += rk * widen_f32(zold[k]);
        acc += rk * rk;
    }
    double rr, rzo = 0.0;
    if (zold) {
        if (!grid_sum2_last(acc, acc2, partials, &st->ticket[3], red, rr, rzo)) return;
    } else if (!grid_sum_last(acc, partials, &st->ticket[3], red, rr)) {  // r.r alone: half the reduction
        return;
    }
    if (threadIdx.x == 0) {
        st->rzo = zold ? rzo : 0.0;
        const double res = sqrt(rr) / st->bnorm;
        const int it = st->it + 1;
        st->residual = res;
        st->it = it;
        if (st->record_history && st->history) st->history[it] = res;
        if (res < st->tol) {
            st->converged = 1;
            st->done = 1;
        } else if (it >= st->max_iter) {
            st->done = 1;
        }
        if (st->done) stop_loop(st);
    }
}

// ||b - A u|| / ||b|| from scratch: the honest residual check. Also zeroes u
// when ||b|| == 0 (f == 0 returns u == 0 whatever the warm start).
__global__ void k_true_residual(Lvl64 L, double* __restrict__ u, const double* __restrict__ b, CgState* st,
                                double* partials) {
    pdl_enter();
    __shared__ double red[kThreads];
    const int n = L.n;
    const int64_t m = (int64_t)n * n;
    const bool zero_u = st->bnorm == 0.0;
    double acc = 0.0;
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) {
        if (zero_u) {
            u[k] = 0.0;
            continue;
        }
        const int i = (int)k / n, j = (int)k - i * n;  // n^2 < 2^31
        const double rk = b[k] - apply_cell(L, u, i, j);
        acc += rk * rk;
    }
    double tot;
    if (!grid_sum_last(acc, partials, &st->ticket[0], red, tot)) return;
    if (threadIdx.x == 0) st->true_residual = st->bnorm > 0.0 ? sqrt(tot) / st->bnorm : 0.0;
}

__global__ void k_apply(Lvl64 L, const double* __restrict__ x, double* __restrict__ y) {
    pdl_enter();
    const int n = L.n;
    const int64_t m = (int64_t)n * n;
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) {
        const int i = (int)k / n, j = (int)k - i * n;  // n^2 < 2^31
        y[k] = apply_cell(L, x, i, j);
    }
}

// The integer-pipe conversions of common.cuh against the conversion
// instructions, element by element: hi/lo from split_f64, (float)x from
// round_f64, (double)hi from widen_f32, and a count of elements where any of
// them differs in its bits from the instruction form.
__global__ void k_check_conversions(const double* __restrict__ x, int64_t m, float* __restrict__ hi,
                                    float* __restrict__ lo, float* __restrict__ rounded,
                                    double* __restrict__ widened, unsigned long long* mismatches) {
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) {
        const double v = x[k];
        float h, l;
        split_f64(v, h, l);
        const float rd = round_f64(v);
        const double w = widen_f32(h);
        const float hi_ref = (float)v;
        const float lo_ref = (float)(v - (double)hi_ref);
        const double w_ref = (double)h;
        const bool same = __float_as_uint(h) == __float_as_uint(hi_ref) && __float_as_uint(l) == __float_as_uint(lo_ref) &&
                          __float_as_uint(rd) == __float_as_uint(hi_ref) &&
                          __double_as_longlong(w) == __double_as_longlong(w_ref);
        hi[k] = h;
        lo[k] = l;
        rounded[k] = rd;
        widened[k] = w;
        if (!same) atomicAdd(mismatches, 1ull);
    }
}
void launch_check_conversions(const double* x, int64_t m, float* hi, float* lo, float* rounded, double* widened,
                              unsigned long long* mismatches, cudaStream_t s) {
    k_check_conversions<<<grid_fill(k_check_conversions, m), kThreads, 0, s>>>(x, m, hi, lo, rounded, widened,
                                                                             mismatches);
}

template <class T>
__global__ void k_copy_cast(const double* __restrict__ src, T* __restrict__ dst, int64_t m) {
    pdl_enter();
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) dst[k] = (T)src[k];
}
template <class T>
__global__ void k_copy_back(const T* __restrict__ src, double* __restrict__ dst, int64_t m) {
    pdl_enter();
    for (int64_t k = GridScope::start(); k < m; k += GridScope::stride()) dst[k] = (double)src[k];
}

// Coarse tail: one CTA runs `top_calls` cycles on levels l0 .. nlev-1.
template <class T>
__global__ void k_tail(const Lvl<T>* __restrict__ lv, int l0, int nlev, int pre, int post, int gamma,
                       int top_calls, const double* id64, const CgState* st) {
    pdl_enter();
    if (st && st->done) return;
    block_cycle<T>(lv, l0, nlev, pre, post, gamma, top_calls, id64);
}

// Dense coarse tail. The levels from l0 down form a fixed linear map
// b_{l0} -> x_{l0} ("x = 0, then top_calls cycles": multigrid.hpp:116-118 for
// l0 > 0, multigrid.hpp:88-93 for l0 = 0). Column j is that map applied to the
// unit vector e_j, computed by one CTA per column with the level vectors in
// shared memory and the coefficients read from the (FP64) hierarchy. Stored
// row-major, FP64 and optionally rounded to FP32 for the mixed form.
// k_tail_matvec reads T before its programmatic-launch wait, so this kernel
// waits for its predecessor but does not release its dependents early: the
// next kernel starts only once T is complete. (Under programmatic launch a
// kernel's pre-wait code overlaps only its immediate predecessor, which
// itself started after the kernel before it had completed; data written two
// or more kernels earlier is safe to read before the wait.)
__global__ void k_tail_columns(const Lvl64* __restrict__ h, int l0, int nlev, int pre, int post, int gamma,
                               int top_calls, int N, double* __restrict__ Td, float* __restrict__ Tf) {
    pdl_wait();
    extern __shared__ double sm_vec[];
    __shared__ Lvl<double> lv[kMaxLevels];
    if (threadIdx.x == 0) {
        double* ptr = sm_vec;
        for (int l = l0; l < nlev; ++l) {
            const Lvl64 H = h[l];
            const int m = H.n * H.n;
            lv[l] = Lvl<double>{H.n, H.e, H.nf, H.d, H.id, ptr, ptr + m};
            ptr += 2 * m;
        }
    }
    __syncthreads();
    const int j = blockIdx.x;
    double* b = lv[l0].b;
    for (int k = threadIdx.x; k < N; k += blockDim.x) b[k] = (k == j) ? 1.0 : 0.0;
    __syncthreads();
    block_cycle<double>(lv, l0, nlev, pre, post, gamma, top_calls, nullptr);
    const double* x = lv[l0].x;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        Td[(size_t)i * N + j] = x[i];
        if (Tf) Tf[(size_t)i * N + j] = (float)x[i];
    }
}

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// x_{l0} = T b_{l0}: one warp per row, b staged in shared memory, the row
// streamed with 16-byte loads (N is a square of a side <= 32; rows of
// N % 4 == 0 are read as 16-byte vectors, others scalar).
template <class T>
__device__ __forceinline__ T dot_row(const T* __restrict__ Mr, const T* __restrict__ b, int N, int lane) {
    T acc = T(0);
    if ((N & 3) == 0 && sizeof(T) == 4) {
        const float4* M4 = reinterpret_cast<const float4*>(Mr);
        const float4* b4 = reinterpret_cast<const float4*>(b);
#pragma unroll 8
        for (int c = lane; c < (N >> 2); c += 32) {
            const float4 m = __ldg(M4 + c), v = __ldg(b4 + c);
            acc += (T)m.x * (T)v.x + (T)m.y * (T)v.y + (T)m.z * (T)v.z + (T)m.w * (T)v.w;
        }
    } else if ((N & 1) == 0 && sizeof(T) == 8) {
        const double2* M2 = reinterpret_cast<const double2*>(Mr);
        const double2* b2 = reinterpret_cast<const double2*>(b);
#pragma unroll 8
        for (int c = lane; c < (N >> 1); c += 32) {
            const double2 m = __ldg(M2 + c), v = __ldg(b2 + c);
            acc += (T)m.x * (T)v.x;
            acc += (T)m.y * (T)v.y;
        }
    } else {
        for (int c = lane; c < N; c += 32) acc += Mr[c] * b[c];
    }
    return warp_sum_t(acc);
}

// x_{l0} = T b_{l0}: one warp per row. T is constant during a solve, so when
// a whole row fits in the warp's registers (N <= kTailRegCells, N a multiple
// of the vector width) each warp loads its row before waiting for the kernel
// that produces b: under programmatic launch that load overlaps the previous
// kernel, and only the read of b is left between the two. Accumulation order
// is dot_row's. Otherwise the row is prefetched to L2 and streamed.
constexpr int kTailRegCells = 1024;  // the largest tail: a 32 x 32 level
template <class T>
__device__ __forceinline__ void tail_acc(T& acc, const float4& m, const float4& v) {
    acc += (T)m.x * (T)v.x + (T)m.y * (T)v.y + (T)m.z * (T)v.z + (T)m.w * (T)v.w;
}
template <class T>
__device__ __forceinline__ void tail_acc(T& acc, const double2& m, const double2& v) {
    acc += (T)m.x * (T)v.x;
    acc += (T)m.y * (T)v.y;
}
template <class T>
__global__ void __launch_bounds__(128) k_tail_matvec(const T* __restrict__ M, int N, const T* __restrict__ b,
                                                     T* __restrict__ x, const CgState* st) {
    (void)st;  // scratch-only output: runs to completion even after convergence
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int kW = (int)(sizeof(V) / sizeof(T));
    constexpr int kPer = kTailRegCells / (32 * kW);  // vectors per lane for a whole row
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    if (N % kW == 0 && N <= kTailRegCells && nwarps >= N) {
        const int nv = N / kW;
        V mr[kPer];
        if (warp < N) {
            const V* Mr = reinterpret_cast<const V*>(M + (size_t)warp * N);
#pragma unroll
            for (int k = 0; k < kPer; ++k)
                if (lane + 32 * k < nv) mr[k] = __ldg(Mr + lane + 32 * k);
        }
        pdl_enter();
        if (warp < N) {
            const V* bv = reinterpret_cast<const V*>(b);
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < kPer; ++k)
                if (lane + 32 * k < nv) tail_acc<T>(acc, mr[k], __ldg(bv + lane + 32 * k));
            acc = warp_sum_t(acc);
            if (lane == 0) x[warp] = acc;
        }
        return;
    }
    if (warp < N) {
        const char* row = reinterpret_cast<const char*>(M + (size_t)warp * N);
        for (int off = lane * 128; off < N * (int)sizeof(T); off += 32 * 128)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(row + off));
    }
    pdl_enter();
    for (int row = warp; row < N; row += nwarps) {
        const T acc = dot_row<T>(M + (size_t)row * N, b, N, lane);
        if (lane == 0) x[row] = acc;
    }
}

// Fused visit kernels (fused.cuh): 16 x 32 tiles with 256 threads on large
// levels; 8 x 16 tiles with 128 threads where a level has few cells, so that
// small levels spread over more SMs and each thread stages less.
constexpr int kMaxTileGrid = kMaxBlocks;

template <int TH, int TW>
static inline int tiles_grid(int n) {
    const int64_t t = (int64_t)((n + TH - 1) / TH) * ((n + TW - 1) / TW);
    return (int)(t < kMaxTileGrid ? t : kMaxTileGrid);
}

// Threads of a visit CTA. 256 for both tile shapes: measured at 1024^2
// (mixed / FP64) 35.0 / 42.7 ms with 128 threads on the 8 x 16 tiles, 32.8 /
// 39.5 ms with 256 (more loads in flight while the halo is staged), 33.1 /
// 40.9 ms with 512; 512 on the 16 x 32 tiles measured slower as well.
constexpr int kVisitThreads = 256;
template <class T>
void launch_visit_pre(const VisitLevel<T>& V, const T* xin, T* xout, T* bc, cudaStream_t s) {
    if (V.n <= 256)
        launch_k(k_visit_pre<T, 8, 16>, tiles_grid<8, 16>(V.n), kVisitThreads, VisitSmem<T, 8, 16>::bytes, s, V, xin, xout, bc);
    else
        launch_k(k_visit_pre<T, 16, 32>, tiles_grid<16, 32>(V.n), kVisitThreads, VisitSmem<T, 16, 32>::bytes, s, V, xin, xout,
                 bc);
}
template <class T>
void launch_visit_mid(const VisitLevel<T>& V, const T* xin, const T* xc, T* xout, T* bc, cudaStream_t s) {
    if (V.n <= 256)
        launch_k(k_visit_mid<T, 8, 16>, tiles_grid<8, 16>(V.n), kVisitThreads, MidSmem<T, 8, 16>::bytes, s, V, xin, xc, xout,
                 bc);
    else
        launch_k(k_visit_mid<T, 16, 32>, tiles_grid<16, 32>(V.n), kVisitThreads, MidSmem<T, 16, 32>::bytes, s, V, xin, xc,
                 xout, bc);
}
template <class T>
void launch_visit_post(const VisitLevel<T>& V, const T* xin, const T* xc, T* xout, const double* r, CgState* st,
                       double* partials, cudaStream_t s) {
    if (V.n <= 256)
        launch_k(k_visit_post<T, 8, 16>, tiles_grid<8, 16>(V.n), kVisitThreads, PostSmem<T, 8, 16>::bytes, s, V, xin, xc, xout,
                 r, st, partials);
    else
        launch_k(k_visit_post<T, 16, 32>, tiles_grid<16, 32>(V.n), kVisitThreads, PostSmem<T, 16, 32>::bytes, s, V, xin, xc,
                 xout, r, st, partials);
}

// ------------------------------------------------------------ launch wrappers

void launch_cg_init(const double* f, double h2, int64_t m, double* b, double* r, double* u, double* p,
                    float* b0f, float* b0lo, const double* u0, const Lvl64& L0, CgState* st, double* partials,
                    cudaStream_t s) {
    launch_k(k_cg_init, grid_fill(k_cg_init, m), kThreads, 0, s, f, h2, m, b, r, u, p, b0f, b0lo, u0, L0, st, partials);
}
template <class T>
void launch_gs(const Lvl<T>& L, int colour, bool zero, CgState* st, cudaStream_t s) {
    launch_k(k_gs<T>, grid_fill(k_gs<T>, colour_count(L.n, colour)), kThreads, 0, s, L, colour, zero, st);
}
template <class T>
void launch_residual_restrict(const Lvl<T>& L, T* bc, CgState* st, cudaStream_t s) {
    const int64_t nc = (L.n + 1) / 2;
    launch_k(k_residual_restrict<T>, grid_fill(k_residual_restrict<T>, nc * nc), kThreads, 0, s, L, bc, st);
}
void launch_residual_restrict_df(const Lvl<float>& L, const float* elo, const float* nlo, const float* dlo,
                                 const float* blo, float* bc, CgState* st, cudaStream_t s) {
    const int64_t nc = (L.n + 1) / 2;
    launch_k(k_residual_restrict_df, grid_fill(k_residual_restrict_df, nc * nc), kThreads, 0, s, L, elo, nlo, dlo, blo, bc, st);
}
template <class T>
void launch_prolong_gs1(const Lvl<T>& L, const T* xc, CgState* st, cudaStream_t s) {
    launch_k(k_prolong_gs1<T>, grid_fill(k_prolong_gs1<T>, colour_count(L.n, 1)), kThreads, 0, s, L, xc, st);
}
template <class T>
void launch_gs0_dot(const Lvl<T>& L, const double* r, CgState* st, double* partials, cudaStream_t s) {
    if ((L.n & 1) == 0 && ((uintptr_t)r & 15) == 0)
        launch_k(k_gs0_dot<T, true>, grid_fill(k_gs0_dot<T, true>, colour_count(L.n, 0)), kThreads, 0, s, L, r, st,
                 partials);
    else
        launch_k(k_gs0_dot<T, false>, grid_fill(k_gs0_dot<T, false>, colour_count(L.n, 0)), kThreads, 0, s, L, r, st,
                 partials);
}
template <class T>
void launch_tail(const Lvl<T>* lv_dev, int l0, int nlev, int pre, int post, int gamma, int top_calls,
                 const double* id64, CgState* st, int threads, cudaStream_t s) {
    launch_k(k_tail<T>, 1, threads, 0, s, lv_dev, l0, nlev, pre, post, gamma, top_calls, id64, st);
}
void launch_tail_columns(const Lvl64* h_dev, const Lvl64* h_host, int l0, int nlev, int pre, int post, int gamma,
                         int top_calls, int N, double* Td, float* Tf, cudaStream_t s) {
    size_t smem = 0;
    for (int l = l0; l < nlev; ++l) smem += 2 * sizeof(double) * (size_t)h_host[l].n * h_host[l].n;
    cudaFuncSetAttribute(k_tail_columns, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    launch_k(k_tail_columns, N, 256, smem, s, h_dev, l0, nlev, pre, post, gamma, top_calls, N, Td, Tf);
}
template <class T>
void launch_tail_matvec(const T* M, int N, const T* b, T* x, CgState* st, cudaStream_t s) {
    // One row per warp. FP32: 128 threads (64 and 256 measured the same).
    // FP64: one warp per CTA, so the 1024 rows spread over 152 SMs as 6-7 per
    // SM instead of 4 or 8 (the FP64 FMAs decide the time): 4.08 -> 3.86 us.
    const int threads = sizeof(T) == 8 ? 32 : 128;
    int blocks = (N + threads / 32 - 1) / (threads / 32);
    if (blocks > kMaxBlocks) blocks = kMaxBlocks;
    launch_k(k_tail_matvec<T>, blocks, threads, 0, s, M, N, b, x, st);
}
template <class T>
void launch_dot_rz(const T* z, const double* r, int64_t m, CgState* st, double* partials, cudaStream_t s) {
    launch_k(k_dot_rz<T>, grid_fill(k_dot_rz<T>, m), kThreads, 0, s, z, r, m, st, partials);
}
void launch_precond_diag(const double* r, const double* id, double* z, int64_t m, CgState* st,
                         double* partials, cudaStream_t s) {
    launch_k(k_precond_diag, grid_fill(k_precond_diag, m), kThreads, 0, s, r, id, z, m, st, partials);
}
template <class Z>
void launch_xpby(const Z* z, double* p, int64_t m, CgState* st, cudaStream_t s) {
    launch_k(k_xpby<Z>, grid_fill(k_xpby<Z>, m), kThreads, 0, s, z, p, m, st);
}
void launch_apply_dot(const Lvl64& L, const double* p, double* ap, CgState* st, double* partials,
                      cudaStream_t s) {
    const int64_t m = (int64_t)L.n * L.n;
    if ((((uintptr_t)p | (uintptr_t)ap) & 15) == 0)
        launch_k(k_apply_dot<true>, grid_fill(k_apply_dot<true>, (m + 1) / 2), kThreads, 0, s, L, p, ap, st, partials);
    else
        launch_k(k_apply_dot<false>, grid_fill(k_apply_dot<false>, m), kThreads, 0, s, L, p, ap, st, partials);
}
void launch_cg_update(const double* p, const double* ap, double* u, double* r, float* b0f, float* b0lo,
                      const float* zold, int64_t m, CgState* st, double* partials, cudaStream_t s) {
    auto al = [](const void* q, uintptr_t a) { return ((uintptr_t)q & (a - 1)) == 0; };
    // Pairs for the FP64 form (1024^2: 14.9 -> 12.8 us); the mixed form's
    // pair kernel needs 72 registers and ran slower (18.8 -> 22.2 us).
    const bool pairs = !zold && al(p, 16) && al(ap, 16) && al(u, 16) && al(r, 16) && al(b0f, 8) && al(b0lo, 8);
    if (pairs)
        launch_k(k_cg_update<true>, grid_fill(k_cg_update<true>, (m + 1) / 2), kThreads, 0, s, p, ap, u, r, b0f, b0lo,
                 zold, m, st, partials);
    else
        launch_k(k_cg_update<false>, grid_fill(k_cg_update<false>, m), kThreads, 0, s, p, ap, u, r, b0f, b0lo, zold,
                 m, st, partials);
}
void launch_true_residual(const Lvl64& L, const double* u, const double* b, double*, CgState* st,
                          double* partials, cudaStream_t s) {
    launch_k(k_true_residual, grid_fill(k_true_residual, (int64_t)L.n * L.n), kThreads, 0, s, L, const_cast<double*>(u), b, st, partials);
}
void launch_apply(const Lvl64& L, const double* x, double* y, cudaStream_t s) {
    launch_k(k_apply, grid_fill(k_apply, (int64_t)L.n * L.n), kThreads, 0, s, L, x, y);
}
template <class T>
void launch_copy_cast(const double* src, T* dst, int64_t m, cudaStream_t s) {
    launch_k(k_copy_cast<T>, grid_fill(k_copy_cast<T>, m), kThreads, 0, s, src, dst, m);
}
template <class T>
void launch_copy_back(const T* src, double* dst, int64_t m, cudaStream_t s) {
    launch_k(k_copy_back<T>, grid_fill(k_copy_back<T>, m), kThreads, 0, s, src, dst, m);
}

// ================================================================ block engine

int num_levels_for(int n) { return carve<double>(n, nullptr, nullptr, 0, nullptr).nlev; }

size_t block_arena_bytes(int n, bool mixed, size_t sbudget) {
    return mixed ? carve<float>(n, nullptr, nullptr, sbudget, nullptr).global_bytes
                 : carve<double>(n, nullptr, nullptr, sbudget, nullptr).global_bytes;
}

// One whole PCG solve (solver.hpp:83-174) by one CTA.
template <class T>
__device__ void block_solve_one(const BatchArgs& A, int pid, const BlockViews<T>& V, double* red,
                                unsigned long long* s_bad) {
    const int n = A.side[pid];
    const int64_t m = (int64_t)n * n;
    const int64_t off = A.off[pid];
    double* u = A.u + off;
    double *b = V.cg[0], *r = V.cg[1], *p = V.cg[2], *ap = V.cg[3], *z = V.cg[4];
    const Lvl64* h = V.h;
    const int nlev = V.nlev;

    const unsigned long long bad = block_setup<T>(A, A.a + off, V, s_bad);
    if (bad != ~0ull) {
        if (threadIdx.x == 0) {
            A.bad[pid] = bad;
            A.iterations[pid] = 0;
            A.converged[pid] = 0;
            A.residual[pid] = 0.0;
            A.levels[pid] = 1;
            if (A.true_residual) A.true_residual[pid] = 0.0;
        }
        return;
    }

    const double hh = 1.0 / (double)(n + 1);
    const double h2 = hh * hh;
    const double* f = A.f ? (A.f_shared ? A.f : A.f + off) : nullptr;
    const double* u0 = A.u0 ? A.u0 + off : nullptr;
    const bool record = A.record_history && A.history && A.count == 1;
    // Standard beta, as in the grid engine (the flexible variant measured
    // worse for the FP32 cycle).
    constexpr bool flexible = false;

    double sb = 0.0;
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
        const double bk = (f ? f[k] : A.fscalar) * h2;
        b[k] = bk;
        u[k] = u0 ? u0[k] : 0.0;
        sb += bk * bk;
    }
    const double bnorm = sqrt(block_sum_wide(sb, red));
    int iterations = 0, converged = 0;
    double residual = 0.0;
    if (bnorm == 0.0) {
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
            u[k] = 0.0;
        }
        if (threadIdx.x == 0) {
            A.bad[pid] = ~0ull;
            A.iterations[pid] = 0;
            A.converged[pid] = 1;
            A.residual[pid] = 0.0;
            A.levels[pid] = 1;
            if (A.true_residual) A.true_residual[pid] = 0.0;
        }
        return;
    }

    double bu0 = 0.0;  // b . u0: estimates the solution's energy ||u||_A^2 = b . u for a close u0
    if (u0) {
        double sr = 0.0, sbu = 0.0;
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
            const int i = (int)k / n, j = (int)k - i * n;  // n^2 < 2^31
            const double rk = b[k] - apply_cell(h[0], u, i, j);
            r[k] = rk;
            sr += rk * rk;
            sbu += b[k] * u[k];
        }
        residual = sqrt(block_sum_wide(sr, red)) / bnorm;
        if (A.u0_fallback) bu0 = block_sum_wide(sbu, red);
    } else {
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) r[k] = b[k];
        residual = 1.0;
        __syncthreads();
    }
    if (record && threadIdx.x == 0) A.history[0] = residual;

    if (residual < A.tol) {
        converged = 1;
    } else {
        // (Leaving z in the FP32 iterate and widening it where p reads it, with
        // no FP64 z array, measured 2% slower: 4096 x 64^2 mixed 23.1 against
        // 22.7 ms.)
        double rz = block_precondition<T>(A, V, r, z, red);
        // A predicted start no better than zero is dropped for the zero start,
        // the fallback it is judged against. CG minimises the error's energy
        // norm; r0 . M r0 (the first preconditioned residual, computed here
        // anyway) estimates the start's ||u - u0||_A^2 and b . u0 the
        // solution's ||u||_A^2, so a start is kept while the first is below
        // the second. A rejected start costs one more cycle (z = M b).
        if (u0 && A.u0_fallback && !(rz < bu0)) {
            for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
                u[k] = 0.0;
                r[k] = b[k];
            }
            residual = 1.0;
            __syncthreads();
            rz = block_precondition<T>(A, V, r, z, red);
        }
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) p[k] = z[k];
        __syncthreads();
        // Even sides take the paired loops: two cells per thread, 16-byte
        // FP64 accesses (arena vectors are 256-byte aligned; u also needs an
        // even offset in the packed output).
        const bool pairs = (n & 1) == 0;
        const bool pairs_u = pairs && (((uintptr_t)u) & 15) == 0;
        for (int it = 0; it < A.max_iter; ++it) {
            const double pap = pairs ? block_apply_dot2(h[0], p, ap, red) : block_apply_dot(h[0], p, ap, red);
            if (!(fabs(pap) > 0.0) || !isfinite(pap)) {
                iterations = it;
                converged = 0;
                break;
            }
            const double alpha = rz / pap;
            double rr = 0.0, rzo = 0.0;
            // the FP32 cycle's input (r rounded) is written here, in the same pass
            const bool round_b = sizeof(T) == 4 && A.pc == kPcMultigrid;
            T* b32 = V.lv[0].b;
            if (pairs_u && !flexible) {
                double2* u2 = reinterpret_cast<double2*>(u);
                double2* r2 = reinterpret_cast<double2*>(r);
                const double2* p2 = reinterpret_cast<const double2*>(p);
                const double2* a2 = reinterpret_cast<const double2*>(ap);
                for (int64_t q = threadIdx.x; q < (m >> 1); q += blockDim.x) {
                    double2 uu = u2[q], rv = r2[q];
                    const double2 pp = p2[q], av = a2[q];
                    uu.x += alpha * pp.x;
                    uu.y += alpha * pp.y;
                    rv.x = rv.x - alpha * av.x;
                    rv.y = rv.y - alpha * av.y;
                    u2[q] = uu;
                    r2[q] = rv;
                    rr += rv.x * rv.x;
                    rr += rv.y * rv.y;
                    if (round_b) {
                        b32[2 * q] = narrow_to<T>(rv.x);
                        b32[2 * q + 1] = narrow_to<T>(rv.y);
                    }
                }
            } else {
                for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
                    u[k] += alpha * p[k];
                    const double rk = r[k] - alpha * ap[k];
                    r[k] = rk;
                    rr += rk * rk;
                    if (round_b) b32[k] = narrow_to<T>(rk);
                    if (flexible) rzo += rk * z[k];  // z still holds the previous direction's z
                }
            }
            residual = sqrt(block_sum_wide(rr, red)) / bnorm;
            if (flexible) rzo = block_sum_wide(rzo, red);
            iterations = it + 1;
            if (record && threadIdx.x == 0) A.history[it + 1] = residual;
            if (residual < A.tol) {
                converged = 1;
                break;
            }
            const double rz_new = block_precondition<T>(A, V, r, z, red, round_b);
            const double beta = (rz_new - rzo) / rz;
            rz = rz_new;
            if (pairs) {
                double2* p2 = reinterpret_cast<double2*>(p);
                const double2* z2 = reinterpret_cast<const double2*>(z);
                for (int64_t q = threadIdx.x; q < (m >> 1); q += blockDim.x) {
                    const double2 zz = z2[q];
                    double2 pp = p2[q];
                    pp.x = zz.x + beta * pp.x;
                    pp.y = zz.y + beta * pp.y;
                    p2[q] = pp;
                }
            } else {
                for (int64_t k = threadIdx.x; k < m; k += blockDim.x) p[k] = z[k] + beta * p[k];
            }
            __syncthreads();
        }
    }

    // Honest residual ||b - A u|| / ||b|| from scratch, when the caller asked
    // for it (one more FP64 operator pass per problem).
    double true_res = residual;
    __syncthreads();
    if (A.true_residual) {
        double tr = 0.0;
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
            const int i = (int)k / n, j = (int)k - i * n;  // n^2 < 2^31
            const double rk = b[k] - apply_cell(h[0], u, i, j);
            tr += rk * rk;
        }
        true_res = sqrt(block_sum_wide(tr, red)) / bnorm;
    }
    if (threadIdx.x == 0) {
        A.bad[pid] = ~0ull;
        A.iterations[pid] = iterations;
        A.converged[pid] = converged;
        A.residual[pid] = residual;
        A.levels[pid] = A.pc == kPcMultigrid ? nlev : 1;
        if (A.true_residual) A.true_residual[pid] = true_res;
    }
}

// Dynamic shared memory of a block-engine CTA: the coarse-level budget, then
// block_sum_wide's scratch, one double per thread.
__host__ __device__ inline size_t block_red_offset(size_t budget) { return (budget + 15) & ~(size_t)15; }
inline size_t block_smem_bytes(size_t budget, int threads) {
    return block_red_offset(budget) + sizeof(double) * (size_t)threads;
}

template <class T>
__global__ void __launch_bounds__(1024) k_block_solve(BatchArgs A) {
    __shared__ BlockViews<T> V;
    __shared__ int s_pid;
    __shared__ unsigned long long s_bad;
    extern __shared__ __align__(16) unsigned char block_smem[];
    double* red = reinterpret_cast<double*>(block_smem + block_red_offset(A.smem_budget));
    char* arena = A.scratch + (size_t)blockIdx.x * A.scratch_stride;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned w = atomicAdd(A.work, 1u);
            s_pid = w < (unsigned)A.count ? A.order[w] : -1;
            if (s_pid >= 0) carve<T>(A.side[s_pid], arena, (char*)block_smem, A.smem_budget, &V);
        }
        __syncthreads();
        const int pid = s_pid;
        if (pid < 0) return;
        block_solve_one<T>(A, pid, V, red, &s_bad);
        __syncthreads();
    }
}

template <class T>
int block_solve_occupancy(int threads, size_t smem) {
    // static + dynamic shared memory above 48 KiB needs the opt-in, so set it always
    const size_t bytes = block_smem_bytes(smem, threads);
    cudaFuncSetAttribute(k_block_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_block_solve<T>, threads, bytes) != cudaSuccess) n = 1;
    return n;
}
template <class T>
void launch_block_solve(const BatchArgs& args, int ctas, int threads, cudaStream_t s) {
    const size_t bytes = block_smem_bytes(args.smem_budget, threads);
    cudaFuncSetAttribute(k_block_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    k_block_solve<T><<<ctas, threads, bytes, s>>>(args);
}

// ------------------------------------------------------ explicit instantiation

#define DGPU_INSTANTIATE(T)                                                                                \
    template void launch_gs<T>(const Lvl<T>&, int, bool, CgState*, cudaStream_t);                          \
    template void launch_residual_restrict<T>(const Lvl<T>&, T*, CgState*, cudaStream_t);                  \
    template void launch_prolong_gs1<T>(const Lvl<T>&, const T*, CgState*, cudaStream_t);                  \
    template void launch_gs0_dot<T>(const Lvl<T>&, const double*, CgState*, double*, cudaStream_t);        \
    template void launch_tail<T>(const Lvl<T>*, int, int, int, int, int, int, const double*, CgState*, int, \
                                 cudaStream_t);                                                            \
    template void launch_dot_rz<T>(const T*, const double*, int64_t, CgState*, double*, cudaStream_t);     \
    template void launch_tail_matvec<T>(const T*, int, const T*, T*, CgState*, cudaStream_t);              \
    template void launch_visit_pre<T>(const VisitLevel<T>&, const T*, T*, T*, cudaStream_t);                 \
    template void launch_visit_mid<T>(const VisitLevel<T>&, const T*, const T*, T*, T*, cudaStream_t);        \
    template void launch_visit_post<T>(const VisitLevel<T>&, const T*, const T*, T*, const double*,          \
                                       CgState*, double*, cudaStream_t);                                   \
    template void launch_xpby<T>(const T*, double*, int64_t, CgState*, cudaStream_t);                      \
    template void launch_copy_cast<T>(const double*, T*, int64_t, cudaStream_t);                           \
    template void launch_copy_back<T>(const T*, double*, int64_t, cudaStream_t);                           \
    template void launch_block_solve<T>(const BatchArgs&, int, int, cudaStream_t);                          \
    template int block_solve_occupancy<T>(int, size_t);                                                    \


DGPU_INSTANTIATE(double)
DGPU_INSTANTIATE(float)

}  // namespace dgpu

// The coarse levels of the grid engine's W-cycle in one thread-block cluster.
//
// Below ~128 x 128 cells a level visit has too little work to fill the GPU
// and costs what its launch and its dependency on the previous kernel cost;
// the W-cycle visits level l 2^l times, so at 1024^2 the levels of side 128,
// 64 and 32 and their coarse tail account for ~70% of every iteration. Here
// one launch runs all `top_calls` cycles of the top coarse level (the
// parent's whole coarse-grid correction, multigrid.hpp:116-118) on a cluster
// of up to 8 CTAs (one per 16 rows of the top level, 1024 threads each):
//
//   * every level's rows are split the same way (CTA r owns rows
//     [r R_l, (r + 1) R_l), R_l = 16 >> (l - top)), so a 2 x 2 aggregate and
//     its coarse cell always live in the same CTA and restriction and
//     prolongation are local;
//   * each CTA keeps its rows of every level -- coefficients (with the FP32
//     lo parts of the mixed form), iterate and right-hand side -- in shared
//     memory for the whole launch, and reads the one row above / below that a
//     5-point update needs from its neighbour's shared memory (distributed
//     shared memory);
//   * phases (colour sweeps, residual + restriction, the dense tail product)
//     are separated by hardware cluster barriers;
//   * the levels of side <= 16 are the dense tail operator, each CTA holding
//     the rows of it that produce its own cells.
//
// The arithmetic is the fused visit kernels' (fused.cuh): the same update
// formula and order, the same double-float residual in the FP32 form.
#pragma once

#include <cooperative_groups.h>

#include "fused.cuh"

namespace dgpu {

constexpr int kClusterMaxLevels = 3;  // explicit levels: sides in (16, 128]
constexpr int kClusterTopRows = 16;   // rows of the top level per CTA
constexpr int kClusterMaxCtas = 8;
constexpr int kClusterThreads = 1024;

template <class T>
struct ClusterArgs {
    int nl;                                  // explicit levels (1..3), top first
    VisitLevel<T> lv[kClusterMaxLevels];     // their coefficients (global)
    int n_tail;                              // side of the tail level (<= 16)
    const T* tail;                           // N x N tail operator, N = n_tail^2, row-major
    const T* b_top;                          // right-hand side of the top level
    T* x_top;                                // its result
    int gamma;                               // cycle index
    int top_calls;                           // cycles run at the top level from x = 0
};

// Shared-memory layout, identical in every CTA of the cluster (element
// offsets in units of T).
struct ClusterLayout {
    int rows[kClusterMaxLevels + 1];         // rows per CTA, level i (index nl: the tail)
    int64_t e[kClusterMaxLevels], nf[kClusterMaxLevels], d[kClusterMaxLevels], id[kClusterMaxLevels];
    int64_t elo[kClusterMaxLevels], nlo[kClusterMaxLevels], dlo[kClusterMaxLevels];
    int64_t x[kClusterMaxLevels + 1], b[kClusterMaxLevels + 1];
    int64_t tslice, bfull;
    int64_t total;
};

template <class T>
__host__ __device__ inline ClusterLayout cluster_layout(const ClusterArgs<T>& A) {
    ClusterLayout L{};
    int64_t o = 0;
    const bool lo = sizeof(T) == 4;
    for (int i = 0; i <= A.nl; ++i) L.rows[i] = kClusterTopRows >> i;
    auto take = [&](int64_t count) {
        const int64_t at = o;
        o += (count + 1) & ~(int64_t)1;  // keep 16-byte alignment for doubles
        return at;
    };
    for (int i = 0; i < A.nl; ++i) {
        const int64_t c = (int64_t)L.rows[i] * A.lv[i].n;
        L.e[i] = take(c);
        L.nf[i] = take(c);
        L.d[i] = take(c);
        L.id[i] = take(c);
        if (lo) {
            L.elo[i] = take(c);
            L.nlo[i] = take(c);
            L.dlo[i] = take(c);
        }
        L.x[i] = take(c);
        L.b[i] = take(c);
    }
    const int64_t ct = (int64_t)L.rows[A.nl] * A.n_tail, N = (int64_t)A.n_tail * A.n_tail;
    L.x[A.nl] = take(ct);
    L.b[A.nl] = take(ct);
    L.bfull = take(N);
    L.tslice = take(ct * N);
    L.total = o;
    return L;
}

namespace clusterdetail {
namespace cgx = cooperative_groups;

// Value of array `off` (a per-level array of the layout) at cell (gi, gj) of
// a level with side n and R rows per CTA: local or in the owner's shared memory.
template <class T>
__device__ __forceinline__ T at(cgx::cluster_group& cl, T* base, int64_t off, int rank, int R, int n, int gi,
                                int gj) {
    const int owner = gi / R;
    const int64_t li = (int64_t)(gi - owner * R) * n + gj;
    if (owner == rank) return base[off + li];
    const T* rem = cl.map_shared_rank(base + off, owner);
    return rem[li];
}

}  // namespace clusterdetail

template <class T>
__global__ void __launch_bounds__(kClusterThreads) k_cluster_cycle(ClusterArgs<T> A) {
    namespace cgx = cooperative_groups;
    using clusterdetail::at;
    cgx::cluster_group cl = cgx::this_cluster();
    const int rank = (int)cl.block_rank();
    extern __shared__ __align__(16) unsigned char cluster_smem[];
    T* S = reinterpret_cast<T*>(cluster_smem);
    // layout and level table in shared memory (indexed by level at run time)
    __shared__ ClusterLayout L;
    __shared__ int lvn[kClusterMaxLevels];
    if (threadIdx.x == 0) {
        L = cluster_layout<T>(A);
        for (int i = 0; i < kClusterMaxLevels; ++i) lvn[i] = i < A.nl ? A.lv[i].n : 0;
    }
    __syncthreads();
    constexpr bool LO = sizeof(T) == 4;
    const int nl = A.nl, nt = A.n_tail, N = nt * nt;

    // ---- static data: coefficients of the own rows, the own rows of the tail operator
    for (int i = 0; i < nl; ++i) {
        const VisitLevel<T>& V = A.lv[i];
        const int n = V.n, R = L.rows[i];
        const int r0 = min(rank * R, n), r1 = min(r0 + R, n);
        const int cnt = (r1 - r0) * n;
        const int64_t g0 = (int64_t)r0 * n;
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            S[L.e[i] + q] = V.e[g0 + q];
            S[L.nf[i] + q] = V.nf[g0 + q];
            S[L.d[i] + q] = V.d[g0 + q];
            S[L.id[i] + q] = V.id[g0 + q];
            if (LO) {
                S[L.elo[i] + q] = V.elo[g0 + q];
                S[L.nlo[i] + q] = V.nlo[g0 + q];
                S[L.dlo[i] + q] = V.dlo[g0 + q];
            }
        }
    }
    {
        const int R = L.rows[nl];
        const int r0 = min(rank * R, nt), r1 = min(r0 + R, nt);
        const int64_t cells = (int64_t)(r1 - r0) * nt, k0 = (int64_t)r0 * nt;
        for (int64_t q = threadIdx.x; q < cells * N; q += blockDim.x) S[L.tslice + q] = A.tail[k0 * N + q];
    }
    pdl_enter();  // the previous kernel wrote b_top
    {
        const int n = lvn[0], R = L.rows[0];
        const int r0 = min(rank * R, n), r1 = min(r0 + R, n);
        for (int q = threadIdx.x; q < (r1 - r0) * n; q += blockDim.x) S[L.b[0] + q] = A.b_top[(int64_t)r0 * n + q];
    }
    cl.sync();

    // One colour pass on level i over the own cells of colour c; zero: the
    // iterate is known to be zero (first sweep of a call from the parent).
    auto sweep = [&](int i, int c, bool zero) {
        const int n = lvn[i], R = L.rows[i];
        const int r0 = min(rank * R, n), r1 = min(r0 + R, n);
        const int half = n >> 1, odd = n & 1;
        const int per_row = half + odd;  // upper bound of one colour's cells in a row
        for (int q = threadIdx.x; q < (r1 - r0) * per_row; q += blockDim.x) {
            const int lr = q / per_row, k = q - lr * per_row;
            const int gi = r0 + lr;
            const int gj = ((c - gi) & 1) + 2 * k;
            if (gj >= n) continue;
            const int64_t s = (int64_t)lr * n + gj;
            T v = S[L.b[i] + s];
            if (!zero) {
                if (gj + 1 < n) v += S[L.e[i] + s] * S[L.x[i] + s + 1];
                if (gj > 0) v += S[L.e[i] + s - 1] * S[L.x[i] + s - 1];
                if (gi + 1 < n) v += S[L.nf[i] + s] * at<T>(cl, S, L.x[i], rank, R, n, gi + 1, gj);
                if (gi > 0)
                    v += at<T>(cl, S, L.nf[i], rank, R, n, gi - 1, gj) * at<T>(cl, S, L.x[i], rank, R, n, gi - 1, gj);
            }
            S[L.x[i] + s] = v * S[L.id[i] + s];
        }
    };
    // Post-smoothing black pass with the prolongation folded in: neighbours
    // are read as x + x_coarse(aggregate), as the fused post-visit stages them.
    auto sweep_prolong = [&](int i) {
        const int n = lvn[i], R = L.rows[i];
        const int nc = (i + 1 < nl) ? lvn[i + 1] : nt, Rc = L.rows[i + 1];
        const int r0 = min(rank * R, n), r1 = min(r0 + R, n);
        const int per_row = (n >> 1) + (n & 1);
        auto xp = [&](int gi, int gj) {
            return at<T>(cl, S, L.x[i], rank, R, n, gi, gj) + at<T>(cl, S, L.x[i + 1], rank, Rc, nc, gi >> 1, gj >> 1);
        };
        for (int q = threadIdx.x; q < (r1 - r0) * per_row; q += blockDim.x) {
            const int lr = q / per_row, k = q - lr * per_row;
            const int gi = r0 + lr;
            const int gj = ((1 - gi) & 1) + 2 * k;
            if (gj >= n) continue;
            const int64_t s = (int64_t)lr * n + gj;
            T v = S[L.b[i] + s];
            if (gj + 1 < n) v += S[L.e[i] + s] * xp(gi, gj + 1);
            if (gj > 0) v += S[L.e[i] + s - 1] * xp(gi, gj - 1);
            if (gi + 1 < n) v += S[L.nf[i] + s] * xp(gi + 1, gj);
            if (gi > 0) v += at<T>(cl, S, L.nf[i], rank, R, n, gi - 1, gj) * xp(gi - 1, gj);
            S[L.x[i] + s] = v * S[L.id[i] + s];
        }
    };
    // Residual of level i summed over each own coarse cell's aggregate, into
    // the right-hand side of level i + 1 (index nl: the tail level).
    auto restrict_residual = [&](int i) {
        const int n = lvn[i], R = L.rows[i];
        const int nc = (i + 1 < nl) ? lvn[i + 1] : nt, Rc = L.rows[i + 1];
        const int c0 = min(rank * Rc, nc), c1 = min(c0 + Rc, nc);
        for (int q = threadIdx.x; q < (c1 - c0) * nc; q += blockDim.x) {
            const int I = c0 + q / nc, J = q - (q / nc) * nc;
            if constexpr (sizeof(T) == 8) {
                T acc = T(0);
                for (int di = 0; di < 2; ++di) {
                    const int gi = 2 * I + di;
                    if (gi >= n) break;
                    for (int dj = 0; dj < 2; ++dj) {
                        const int gj = 2 * J + dj;
                        if (gj >= n) break;
                        const int64_t s = (int64_t)(gi - rank * R) * n + gj;
                        const T xs = S[L.x[i] + s];
                        T v = S[L.d[i] + s] * xs;
                        if (gj + 1 < n) v -= S[L.e[i] + s] * S[L.x[i] + s + 1];
                        if (gj > 0) v -= S[L.e[i] + s - 1] * S[L.x[i] + s - 1];
                        if (gi + 1 < n) v -= S[L.nf[i] + s] * at<T>(cl, S, L.x[i], rank, R, n, gi + 1, gj);
                        if (gi > 0)
                            v -= at<T>(cl, S, L.nf[i], rank, R, n, gi - 1, gj) *
                                 at<T>(cl, S, L.x[i], rank, R, n, gi - 1, gj);
                        acc += S[L.b[i] + s] - v;
                    }
                }
                S[L.b[i + 1] + (int64_t)(I - c0) * nc + J] = acc;
            } else {
                DF acc{0.f, 0.f};
                for (int di = 0; di < 2; ++di) {
                    const int gi = 2 * I + di;
                    if (gi >= n) break;
                    for (int dj = 0; dj < 2; ++dj) {
                        const int gj = 2 * J + dj;
                        if (gj >= n) break;
                        const int64_t s = (int64_t)(gi - rank * R) * n + gj;
                        df_add(acc, S[L.b[i] + s], 0.f);
                        df_axpy(acc, S[L.d[i] + s], S[L.dlo[i] + s], S[L.x[i] + s], -1.f);
                        if (gj + 1 < n) df_axpy(acc, S[L.e[i] + s], S[L.elo[i] + s], S[L.x[i] + s + 1], 1.f);
                        if (gj > 0) df_axpy(acc, S[L.e[i] + s - 1], S[L.elo[i] + s - 1], S[L.x[i] + s - 1], 1.f);
                        if (gi + 1 < n)
                            df_axpy(acc, S[L.nf[i] + s], S[L.nlo[i] + s], at<T>(cl, S, L.x[i], rank, R, n, gi + 1, gj),
                                    1.f);
                        if (gi > 0)
                            df_axpy(acc, at<T>(cl, S, L.nf[i], rank, R, n, gi - 1, gj),
                                    at<T>(cl, S, L.nlo[i], rank, R, n, gi - 1, gj),
                                    at<T>(cl, S, L.x[i], rank, R, n, gi - 1, gj), 1.f);
                    }
                }
                S[L.b[i + 1] + (int64_t)(I - c0) * nc + J] = acc.hi + acc.lo;
            }
        }
    };
    // x_tail (own cells) = T b_tail, b_tail gathered from every CTA.
    auto tail_apply = [&]() {
        const int R = L.rows[nl];
        for (int k = threadIdx.x; k < N; k += blockDim.x) {
            const int gi = k / nt, gj = k - (k / nt) * nt;
            S[L.bfull + k] = at<T>(cl, S, L.b[nl], rank, R, nt, gi, gj);
        }
        __syncthreads();
        const int r0 = min(rank * R, nt), r1 = min(r0 + R, nt);
        const int cells = (r1 - r0) * nt;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int row = warp; row < cells; row += nw) {
            const T* Tr = S + L.tslice + (int64_t)row * N;
            T acc = T(0);
            for (int c = lane; c < N; c += 32) acc += Tr[c] * S[L.bfull + c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) S[L.x[nl] + row] = acc;
        }
    };

    // ---- the cycle: levels 0 .. nl-1 explicit, the tail below the last
    int calls[kClusterMaxLevels];
    unsigned zero_mask = 1u;
    int l = 0;
    calls[0] = A.top_calls;
    for (;;) {
        for (;;) {
            sweep(l, 0, (zero_mask >> l) & 1u);  // red
            cl.sync();
            sweep(l, 1, false);  // black
            cl.sync();
            zero_mask &= ~(1u << l);
            restrict_residual(l);
            cl.sync();
            if (l + 1 < nl) {
                ++l;
                calls[l] = A.gamma;
                zero_mask |= 1u << l;
                continue;
            }
            tail_apply();
            cl.sync();
            break;
        }
        // post-smoothing up the levels whose cycles are complete
        for (;;) {
            sweep_prolong(l);  // black, with the coarse correction
            cl.sync();
            sweep(l, 0, false);  // red
            cl.sync();
            if (--calls[l] > 0) break;  // this level's next cycle
            if (l == 0) break;
            --l;
        }
        if (l == 0 && calls[0] == 0) break;
    }

    {
        const int n = lvn[0], R = L.rows[0];
        const int r0 = min(rank * R, n), r1 = min(r0 + R, n);
        for (int q = threadIdx.x; q < (r1 - r0) * n; q += blockDim.x) A.x_top[(int64_t)r0 * n + q] = S[L.x[0] + q];
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

}  // namespace dgpu

// The multigrid cycle run by one CTA over a range of levels (block scope).
//
// Used two ways: as the whole preconditioner of a small problem (one CTA per
// problem in the batched engine), and as the coarse tail of a large solve,
// where the grid-wide kernels hand the levels at and below a cut-off side to
// one CTA per visit. The recursion of include/darcy/multigrid.hpp:97-127 is
// unrolled into an explicit per-level call counter so that every thread runs
// the same control flow and phases are separated by __syncthreads().
#pragma once

#include "common.cuh"

namespace dgpu {

// multigrid.hpp:129-146: a 1x1 level is solved exactly; a larger coarsest
// level (only reachable through the 32-level cap) gets 8 + 8 symmetric sweeps.
// The mixed form passes the FP64 reciprocal diagonal of the coarsest level so
// that its exact solve stays in FP64.
template <class T>
__device__ __forceinline__ void block_coarsest(const Lvl<T>& L, bool zero, const double* id64) {
    if (L.n == 1) {
        if (threadIdx.x == 0) {
            if (id64)
                L.x[0] = (T)((double)L.b[0] * id64[0]);
            else
                L.x[0] = L.b[0] * L.id[0];
        }
        __syncthreads();
        return;
    }
    for (int s = 0; s < 8; ++s) {
        gs_colour<BlockScope>(L, 0, zero && s == 0);
        __syncthreads();
        gs_colour<BlockScope>(L, 1, false);
        __syncthreads();
    }
    for (int s = 0; s < 8; ++s) {
        gs_colour<BlockScope>(L, 1, false);
        __syncthreads();
        gs_colour<BlockScope>(L, 0, false);
        __syncthreads();
    }
}

// x = Tt b for a dense N x N operator held by the block (shared or global
// memory): one warp per row, lanes across the row.
template <class T>
__device__ __forceinline__ void block_matvec(const T* __restrict__ Tt, int N, const T* b, T* x) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int row = warp; row < N; row += nw) {
        const T* Tr = Tt + row * N;
        T acc = T(0);
        for (int c = lane; c < N; c += 32) acc += Tr[c] * b[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) x[row] = acc;
    }
}

// Runs `top_calls` cycles at level l0 starting from x_{l0} = 0, on levels
// l0 .. nlev-1 of `lv` (nlev is the full hierarchy depth). With top_calls = 1
// and l0 = 0 this is Multigrid::apply (multigrid.hpp:88-93); with
// top_calls = cycle_index it is the body of the parent's recursion
// (multigrid.hpp:117-118) for the tail of a large solve.
//
// With Tt != null the levels from tl (> l0) down are not visited: the map
// they implement ("x_tl = 0, then gamma cycles") is the dense Tt, applied as
// one product per visit of level tl - 1.
template <class T>
__device__ void block_cycle(const Lvl<T>* lv, int l0, int nlev, int pre, int post, int gamma, int top_calls,
                            const double* id64_coarsest, const T* Tt = nullptr, int tl = 0) {
    int calls[kMaxLevels];
    unsigned zero_mask = 1u << l0;  // levels whose iterate is known to be zero
    int l = l0;
    calls[l0] = top_calls;
    const int last = Tt ? tl - 1 : nlev - 1;  // deepest level visited explicitly
    auto presmooth_restrict = [&](int lvl) {
        const Lvl<T>& A = lv[lvl];
        for (int s = 0; s < pre; ++s) {
            gs_colour<BlockScope>(A, 0, s == 0 && ((zero_mask >> lvl) & 1u));
            __syncthreads();
            gs_colour<BlockScope>(A, 1, false);
            __syncthreads();
        }
        zero_mask &= ~(1u << lvl);
        residual_restrict<BlockScope>(A, lv[lvl + 1].b);
        __syncthreads();
    };
    auto prolong_postsmooth = [&](int lvl) {
        const Lvl<T>& A = lv[lvl];
        prolong_gs1<BlockScope>(A, lv[lvl + 1].x);
        __syncthreads();
        gs_colour<BlockScope>(A, 0, false);
        __syncthreads();
        for (int s = 1; s < post; ++s) {
            gs_colour<BlockScope>(A, 1, false);
            __syncthreads();
            gs_colour<BlockScope>(A, 0, false);
            __syncthreads();
        }
    };
    for (;;) {
        while (l < last) {
            presmooth_restrict(l);
            ++l;
            calls[l] = gamma;
            zero_mask |= 1u << l;
        }
        if (Tt) {  // l == tl - 1: visit it, with the dense tail as its coarse correction
            presmooth_restrict(l);
            const int nt = lv[tl].n;
            block_matvec<T>(Tt, nt * nt, lv[tl].b, lv[tl].x);
            __syncthreads();
            prolong_postsmooth(l);
        } else {
            block_coarsest(lv[l], (zero_mask >> l) & 1u, id64_coarsest);
            zero_mask &= ~(1u << l);
        }
        for (;;) {
            if (--calls[l] > 0) break;  // run this level's cycle again
            if (l == l0) return;
            --l;
            prolong_postsmooth(l);
        }
    }
}

// ---------------------------------------------- many right-hand sides
//
// The same cycle applied to `nrhs` right-hand sides at once (right-hand side
// r of level l at x + r * n_l^2, b + r * n_l^2); used to build the dense tail
// operator of a block-engine problem, one column per right-hand side.

template <class T>
__device__ __forceinline__ void gs_colour_m(const Lvl<T> L, int c, bool zero, int nrhs) {
    const int n = L.n, m = n * n;
    const int cnt = (int)colour_count(n, c);
    for (int t = threadIdx.x; t < cnt * nrhs; t += blockDim.x) {
        const int rr = t / cnt, q = t - rr * cnt;
        int i, j;
        colour_cell(n, c, q, i, j);
        const int k = i * n + j;
        T* x = L.x + rr * m;
        T v = L.b[rr * m + k];
        if (!zero) {
            if (j + 1 < n) v += L.e[k] * x[k + 1];
            if (j > 0) v += L.e[k - 1] * x[k - 1];
            if (i + 1 < n) v += L.nf[k] * x[k + n];
            if (i > 0) v += L.nf[k - n] * x[k - n];
        }
        x[k] = v * L.id[k];
    }
}

template <class T>
__device__ __forceinline__ void residual_restrict_m(const Lvl<T> L, T* bc, int nrhs) {
    const int n = L.n, m = n * n, nc = (n + 1) / 2, mc = nc * nc;
    for (int t = threadIdx.x; t < mc * nrhs; t += blockDim.x) {
        const int rr = t / mc, K = t - rr * mc;
        const int I = K / nc, J = K - I * nc;
        const int i1 = (2 * I + 1 < n) ? 2 * I + 1 : 2 * I;
        const int j1 = (2 * J + 1 < n) ? 2 * J + 1 : 2 * J;
        Lvl<T> V = L;
        V.x = L.x + rr * m;
        V.b = L.b + rr * m;
        T s = T(0);
        for (int i = 2 * I; i <= i1; ++i)
            for (int j = 2 * J; j <= j1; ++j) s += cell_residual(V, i, j);
        bc[rr * mc + K] = s;
    }
}

template <class T>
__device__ __forceinline__ void prolong_gs1_m(const Lvl<T> L, const T* xc, int nrhs) {
    const int n = L.n, m = n * n, nc = (n + 1) / 2, mc = nc * nc;
    const int cnt = (int)colour_count(n, 1);
    for (int t = threadIdx.x; t < cnt * nrhs; t += blockDim.x) {
        const int rr = t / cnt, q = t - rr * cnt;
        int i, j;
        colour_cell(n, 1, q, i, j);
        const int k = i * n + j;
        const T* x = L.x + rr * m;
        const T* c = xc + rr * mc;
        T v = L.b[rr * m + k];
        if (j + 1 < n) v += L.e[k] * (x[k + 1] + c[(i >> 1) * nc + ((j + 1) >> 1)]);
        if (j > 0) v += L.e[k - 1] * (x[k - 1] + c[(i >> 1) * nc + ((j - 1) >> 1)]);
        if (i + 1 < n) v += L.nf[k] * (x[k + n] + c[((i + 1) >> 1) * nc + (j >> 1)]);
        if (i > 0) v += L.nf[k - n] * (x[k - n] + c[((i - 1) >> 1) * nc + (j >> 1)]);
        L.x[rr * m + k] = v * L.id[k];
    }
}

// id64: the FP64 reciprocal diagonal of the coarsest level (its 1 x 1 solve
// stays FP64 when the cycle is FP32), or null.
template <class T>
__device__ void block_cycle_m(const Lvl<T>* lv, int l0, int nlev, int pre, int post, int gamma, int top_calls,
                              int nrhs, const double* id64 = nullptr) {
    int calls[kMaxLevels];
    unsigned zero_mask = 1u << l0;
    int l = l0;
    calls[l0] = top_calls;
    for (;;) {
        while (l + 1 < nlev) {
            const Lvl<T>& A = lv[l];
            for (int s = 0; s < pre; ++s) {
                gs_colour_m<T>(A, 0, s == 0 && ((zero_mask >> l) & 1u), nrhs);
                __syncthreads();
                gs_colour_m<T>(A, 1, false, nrhs);
                __syncthreads();
            }
            zero_mask &= ~(1u << l);
            residual_restrict_m<T>(A, lv[l + 1].b, nrhs);
            __syncthreads();
            ++l;
            calls[l] = gamma;
            zero_mask |= 1u << l;
        }
        {  // coarsest level (multigrid.hpp:129-146)
            const Lvl<T>& A = lv[l];
            const bool zero = (zero_mask >> l) & 1u;
            if (A.n == 1) {
                for (int rr = threadIdx.x; rr < nrhs; rr += blockDim.x)
                    A.x[rr] = id64 ? (T)((double)A.b[rr] * id64[0]) : A.b[rr] * A.id[0];
                __syncthreads();
            } else {
                for (int s = 0; s < 8; ++s) {
                    gs_colour_m<T>(A, 0, zero && s == 0, nrhs);
                    __syncthreads();
                    gs_colour_m<T>(A, 1, false, nrhs);
                    __syncthreads();
                }
                for (int s = 0; s < 8; ++s) {
                    gs_colour_m<T>(A, 1, false, nrhs);
                    __syncthreads();
                    gs_colour_m<T>(A, 0, false, nrhs);
                    __syncthreads();
                }
            }
            zero_mask &= ~(1u << l);
        }
        for (;;) {
            if (--calls[l] > 0) break;
            if (l == l0) return;
            --l;
            const Lvl<T>& A = lv[l];
            prolong_gs1_m<T>(A, lv[l + 1].x, nrhs);
            __syncthreads();
            gs_colour_m<T>(A, 0, false, nrhs);
            __syncthreads();
            for (int s = 1; s < post; ++s) {
                gs_colour_m<T>(A, 1, false, nrhs);
                __syncthreads();
                gs_colour_m<T>(A, 0, false, nrhs);
                __syncthreads();
            }
        }
    }
}

}  // namespace dgpu

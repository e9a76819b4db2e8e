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

// Runs `top_calls` cycles at level l0 starting from x_{l0} = 0, on levels
// l0 .. nlev-1 of `lv` (nlev is the full hierarchy depth). With top_calls = 1
// and l0 = 0 this is Multigrid::apply (multigrid.hpp:88-93); with
// top_calls = cycle_index it is the body of the parent's recursion
// (multigrid.hpp:117-118) for the tail of a large solve.
template <class T>
__device__ void block_cycle(const Lvl<T>* lv, int l0, int nlev, int pre, int post, int gamma, int top_calls,
                            const double* id64_coarsest) {
    int calls[kMaxLevels];
    unsigned zero_mask = 1u << l0;  // levels whose iterate is known to be zero
    int l = l0;
    calls[l0] = top_calls;
    for (;;) {
        while (l + 1 < nlev) {
            const Lvl<T>& A = lv[l];
            for (int s = 0; s < pre; ++s) {
                gs_colour<BlockScope>(A, 0, s == 0 && ((zero_mask >> l) & 1u));
                __syncthreads();
                gs_colour<BlockScope>(A, 1, false);
                __syncthreads();
            }
            zero_mask &= ~(1u << l);
            residual_restrict<BlockScope>(A, lv[l + 1].b);
            __syncthreads();
            ++l;
            calls[l] = gamma;
            zero_mask |= 1u << l;
        }
        block_coarsest(lv[l], (zero_mask >> l) & 1u, id64_coarsest);
        zero_mask &= ~(1u << l);
        for (;;) {
            if (--calls[l] > 0) break;  // run this level's cycle again
            if (l == l0) return;
            --l;
            const Lvl<T>& A = lv[l];
            prolong_gs1<BlockScope>(A, lv[l + 1].x);
            __syncthreads();
            gs_colour<BlockScope>(A, 0, false);
            __syncthreads();
            for (int s = 1; s < post; ++s) {
                gs_colour<BlockScope>(A, 1, false);
                __syncthreads();
                gs_colour<BlockScope>(A, 0, false);
                __syncthreads();
            }
        }
    }
}

}  // namespace dgpu

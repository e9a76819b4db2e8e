// Block-engine building blocks: one CTA owns one problem (layout of its
// scratch, hierarchy setup, operator application, one preconditioner cycle).
// Shared by the batched engine (kernels.cu) and the allocation-free
// preconditioner entry point (noalloc.cu).
#pragma once

#include <math.h>

#include "cycle.cuh"
#include "engine.h"

namespace dgpu {

// y = A x at one cell, FP64 (level.hpp:105-119).
__device__ __forceinline__ double apply_cell(const Lvl64& L, const double* __restrict__ x, int i, int j) {
    const int n = L.n;
    const int64_t k = (int64_t)i * n + j;
    double v = L.d[k] * x[k];
    if (j + 1 < n) v -= L.e[k] * x[k + 1];
    if (j > 0) v -= L.e[k - 1] * x[k - 1];
    if (i + 1 < n) v -= L.nf[k] * x[k + n];
    if (i > 0) v -= L.nf[k - n] * x[k - n];
    return v;
}

// Per-CTA layout for one side-n problem. Global arena (L2-resident while the
// CTA works on the problem): the FP64 hierarchy (e, nf, d, id per level,
// wb/sb boundary vectors), the five FP64 CG vectors b, r, p, Ap, z, the
// cycle's own coefficient copies and iterate/right-hand side for the large
// levels, and the scratch used once per problem to build the dense tail.
// Shared memory: level 0's cycle data when all of it fits in `sbudget` bytes,
// then the dense tail operator, then the cycle's data for as many coarse
// levels as fit. Level 0 of an FP64 cycle works directly on r (right-hand
// side) and z (iterate).
//
// Dense tail: the levels from tl (the first level of side <= kBlockTailSide,
// when that is not level 0) down implement the fixed map "x = 0, then gamma
// cycles"; it is built once per problem as an N x N matrix (N = side_tl^2,
// one column per unit right-hand side, all columns at once) and the cycle
// applies it with one product per visit of level tl - 1 instead of visiting
// 2^k levels below. Same operator as the recursion, to rounding.
// Shared by host sizing and device carving (gbase/sbase == null: size only).
constexpr int kBlockTailSide = 8;

struct BlockLayout {
    size_t global_bytes, smem_bytes;
    int nlev, ls;
};

template <class T>
struct BlockViews {
    Lvl64 h[kMaxLevels];        // FP64 hierarchy
    Lvl<T> lv[kMaxLevels];      // the cycle's levels
    Lvl<T> lm[kMaxLevels];      // tail construction: the tail levels with N right-hand sides, in the
                                // cycle's precision (FP32 copies of the coefficients for the mixed form)
    double* cg[5];              // b, r, p, Ap, z
    T* tail;                    // dense tail operator (ntail x ntail), or null
    int nlev, tl, ntail;
};

template <class T>
__host__ __device__ BlockLayout carve(int n, char* gbase, char* sbase, size_t sbudget, BlockViews<T>* v) {
    size_t goff = 0, soff = 0;
    auto gtake = [&](size_t bytes) -> char* {
        char* ptr = gbase ? gbase + goff : nullptr;
        goff += (bytes + 255) & ~(size_t)255;
        return ptr;
    };
    auto stake = [&](size_t bytes) -> char* {
        char* ptr = sbase ? sbase + soff : nullptr;
        soff += (bytes + 15) & ~(size_t)15;
        return ptr;
    };
    int sides[kMaxLevels];
    int nlev = 0;
    for (int s = n; nlev < kMaxLevels;) {
        sides[nlev++] = s;
        if (s <= 1) break;
        s = (s + 1) / 2;
    }
    int tl = 0;
    for (int l = 1; l < nlev; ++l)
        if (sides[l] <= kBlockTailSide) {
            tl = l;
            break;
        }
    const int ntail = tl ? sides[tl] * sides[tl] : 0;
    const int cyc_levels = tl ? tl : nlev;  // levels the cycle itself visits
    const bool fp32 = sizeof(T) == 4;
    // Shared memory, in order of the traffic it saves: level 0's cycle data
    // when the whole of it fits (a visit of level l moves ~4^-l of level 0's
    // bytes and happens 2^l times per W-cycle, so level 0 carries about half
    // of a cycle's traffic: the coefficient copies, and for an FP32 cycle its
    // iterate and right-hand side too); then the tail operator (with level
    // tl's x and b, which it reads and writes); then the coarsest cycle levels
    // that still fit.
    auto arr = [](size_t cells) { return ((cells * sizeof(T) + 15) & ~(size_t)15); };
    const size_t l0_bytes = (fp32 ? 6 : 4) * arr((size_t)n * n);
    const bool l0_shared = nlev > 1 && cyc_levels >= 1 && l0_bytes <= sbudget;
    size_t need = l0_shared ? l0_bytes : 0;
    const size_t tail_bytes = tl ? arr((size_t)ntail * ntail) + 2 * arr((size_t)ntail) : 0;
    const bool tail_shared = tl && need + tail_bytes <= sbudget;
    if (tail_shared) need += tail_bytes;
    int ls = cyc_levels;
    for (int l = cyc_levels - 1; l >= 1; --l) {
        const size_t lvl = 6 * (((size_t)sides[l] * sides[l] * sizeof(T) + 15) & ~(size_t)15);
        if (need + lvl > sbudget) break;
        need += lvl;
        ls = l;
    }
    if (v) {
        v->nlev = nlev;
        v->tl = tl;
        v->ntail = ntail;
        v->tail = nullptr;
    }
    if (tl) {
        T* tp = (T*)(tail_shared ? stake(sizeof(T) * (size_t)ntail * ntail)
                                 : gtake(sizeof(T) * (size_t)ntail * ntail));
        if (v) v->tail = tp;
    }
    const size_t m0 = (size_t)n * n;
    for (int l = 0; l < nlev; ++l) {
        const size_t m = (size_t)sides[l] * sides[l];
        Lvl64 H;
        H.n = sides[l];
        H.e = (double*)gtake(8 * m);
        H.nf = (double*)gtake(8 * m);
        H.d = (double*)gtake(8 * m);
        H.id = (double*)gtake(8 * m);
        H.wb = (double*)gtake(8 * (size_t)sides[l]);
        H.sb = (double*)gtake(8 * (size_t)sides[l]);
        if (v) v->h[l] = H;
    }
    double* cgv[5];
    for (int q = 0; q < 5; ++q) cgv[q] = (double*)gtake(8 * m0);
    if (v)
        for (int q = 0; q < 5; ++q) v->cg[q] = cgv[q];
    for (int l = 0; l < nlev; ++l) {
        const size_t m = (size_t)sides[l] * sides[l];
        Lvl<T> V{};
        V.n = sides[l];
        if (tl && l > tl) {  // inside the tail: never visited by the cycle
            if (v) v->lv[l] = V;
            continue;
        }
        const bool shared = (l == 0 && l0_shared) || (l >= ls && l < cyc_levels) || (tail_shared && l == tl);
        auto take = [&](size_t bytes) { return shared ? stake(bytes) : gtake(bytes); };
        if (l < cyc_levels) {
            if (fp32 || shared) {
                V.e = (const T*)take(sizeof(T) * m);
                V.nf = (const T*)take(sizeof(T) * m);
                V.d = (const T*)take(sizeof(T) * m);
                V.id = (const T*)take(sizeof(T) * m);
            } else if (v) {
                V.e = (const T*)v->h[l].e;
                V.nf = (const T*)v->h[l].nf;
                V.d = (const T*)v->h[l].d;
                V.id = (const T*)v->h[l].id;
            }
        }
        if (l == 0 && !fp32) {
            V.x = (T*)cgv[4];  // z
            V.b = (T*)cgv[1];  // r
        } else {
            // level tl (the tail's input/output) only needs x and b
            V.x = (T*)take(sizeof(T) * m);
            V.b = (T*)take(sizeof(T) * m);
        }
        if (v) v->lv[l] = V;
    }
    if (tl) {  // tail construction scratch: every tail level with ntail right-hand sides
        for (int l = tl; l < nlev; ++l) {
            const size_t m = (size_t)sides[l] * sides[l];
            Lvl<T> M{};
            M.n = sides[l];
            M.x = (T*)gtake(sizeof(T) * m * ntail);
            M.b = (T*)gtake(sizeof(T) * m * ntail);
            if (fp32) {
                M.e = (const T*)gtake(sizeof(T) * m);
                M.nf = (const T*)gtake(sizeof(T) * m);
                M.d = (const T*)gtake(sizeof(T) * m);
                M.id = (const T*)gtake(sizeof(T) * m);
            } else if (v) {
                M.e = (const T*)v->h[l].e;
                M.nf = (const T*)v->h[l].nf;
                M.d = (const T*)v->h[l].d;
                M.id = (const T*)v->h[l].id;
            }
            if (v) v->lm[l] = M;
        }
    }
    return BlockLayout{goff, soff, nlev, ls};
}

// Cycle coefficients of level l in the cycle's precision (FP32 copies for the
// mixed form, shared-memory copies for the levels held on chip). The FP32
// reciprocal diagonal is the correctly rounded reciprocal of the FP32 d (the
// FP64 id, one FP64 division per cell, is built for FP32 cycles on the
// coarsest level only); FP64 copies take id as built.
template <class T>
__device__ __forceinline__ void block_copy_coeffs(const Lvl64& H, const Lvl<T>& V) {
    if (!V.e || (const void*)V.e == (const void*)H.e) return;  // not visited / FP64 used in place
    const int64_t m = (int64_t)H.n * H.n;
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
        ((T*)V.e)[k] = narrow_to<T>(H.e[k]);
        ((T*)V.nf)[k] = narrow_to<T>(H.nf[k]);
        const T dk = narrow_to<T>(H.d[k]);
        ((T*)V.d)[k] = dk;
        if constexpr (sizeof(T) == 4)
            ((T*)V.id)[k] = __frcp_rn(dk);
        else
            ((T*)V.id)[k] = H.id[k];
    }
}

// y = A x over a block, FP64, returning sum x . y.
__device__ __forceinline__ double block_apply_dot(const Lvl64& L, const double* x, double* y, double* red) {
    const int n = L.n;
    const int64_t m = (int64_t)n * n;
    double acc = 0.0;
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
        const int i = (int)k / n, j = (int)k - i * n;  // n^2 < 2^31
        const double v = apply_cell(L, x, i, j);
        y[k] = v;
        acc += x[k] * v;
    }
    return block_sum_wide(acc, red);
}

// The same for an even side, two horizontally adjacent cells per thread with
// 16-byte loads and stores (twice the bytes in flight per load instruction for
// this latency-bound loop); each cell's terms in apply_cell's order. All
// arrays 16-byte aligned (the arena's).
__device__ __forceinline__ double block_apply_dot2(const Lvl64& L, const double* x, double* y, double* red) {
    const int n = L.n, n2 = n >> 1;
    const int64_t m2 = (int64_t)n * n2;
    const double2* x2 = reinterpret_cast<const double2*>(x);
    const double2* d2 = reinterpret_cast<const double2*>(L.d);
    const double2* e2 = reinterpret_cast<const double2*>(L.e);
    const double2* nf2 = reinterpret_cast<const double2*>(L.nf);
    double acc = 0.0;
    for (int64_t q = threadIdx.x; q < m2; q += blockDim.x) {
        const int i = (int)q / n2, jp = (int)q - i * n2, j = 2 * jp;  // n^2 < 2^31
        const int64_t k = (int64_t)i * n + j;
        const double2 xc = x2[q], dd = d2[q], ee = e2[q];
        double v0 = dd.x * xc.x, v1 = dd.y * xc.y;
        v0 -= ee.x * xc.y;                            // east of j (j + 1 < n: j even, n even)
        if (j > 0) v0 -= L.e[k - 1] * x[k - 1];       // west of j
        if (j + 2 < n) v1 -= ee.y * x[k + 2];         // east of j + 1
        v1 -= ee.x * xc.x;                            // west of j + 1
        if (i + 1 < n) {
            const double2 nn = nf2[q], xn = x2[q + n2];
            v0 -= nn.x * xn.x;
            v1 -= nn.y * xn.y;
        }
        if (i > 0) {
            const double2 ns = nf2[q - n2], xs = x2[q - n2];
            v0 -= ns.x * xs.x;
            v1 -= ns.y * xs.y;
        }
        reinterpret_cast<double2*>(y)[q] = make_double2(v0, v1);
        acc += xc.x * v0;
        acc += xc.y * v1;
    }
    return block_sum_wide(acc, red);
}

// z = M r for one problem; returns r . z. For the FP32 cycle, r is rounded
// into the level-0 right-hand side and the FP32 iterate widened into z.
template <class T>
__device__ double block_precondition(const BatchArgs& A, const BlockViews<T>& V, const double* r, double* z,
                                     double* red, bool b_ready = false) {
    const int n = V.h[0].n;
    const int64_t m = (int64_t)n * n;
    double acc = 0.0;
    if (A.pc == kPcMultigrid) {
        const double* id64 = V.h[V.nlev - 1].id;  // FP64 exact coarsest solve (no-tail hierarchies)
        if (sizeof(T) == 4) {
            if (!b_ready) {  // (the CG update usually wrote the rounded r already)
                for (int64_t k = threadIdx.x; k < m; k += blockDim.x) V.lv[0].b[k] = narrow_to<T>(r[k]);
                __syncthreads();
            }
            block_cycle<T>(V.lv, 0, V.nlev, A.pre, A.post, A.gamma, 1, id64, V.tail, V.tl);
            if ((m & 1) == 0) {  // pairs: 8-byte FP32 and 16-byte FP64 accesses (arena-aligned)
                const float2* x2 = reinterpret_cast<const float2*>(V.lv[0].x);
                const double2* r2 = reinterpret_cast<const double2*>(r);
                for (int64_t q = threadIdx.x; q < (m >> 1); q += blockDim.x) {
                    const float2 xx = x2[q];
                    const double2 rr = r2[q];
                    const double z0 = widen_f32(xx.x), z1 = widen_f32(xx.y);
                    reinterpret_cast<double2*>(z)[q] = make_double2(z0, z1);
                    acc += rr.x * z0;
                    acc += rr.y * z1;
                }
            } else {
                for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
                    const double zk = widen_f32(V.lv[0].x[k]);
                    z[k] = zk;
                    acc += r[k] * zk;
                }
            }
        } else {
            block_cycle<T>(V.lv, 0, V.nlev, A.pre, A.post, A.gamma, 1, nullptr, V.tail, V.tl);
            if ((m & 1) == 0) {
                const double2* r2 = reinterpret_cast<const double2*>(r);
                const double2* z2 = reinterpret_cast<const double2*>(z);
                for (int64_t q = threadIdx.x; q < (m >> 1); q += blockDim.x) {
                    const double2 rr = r2[q], zz = z2[q];
                    acc += rr.x * zz.x;
                    acc += rr.y * zz.y;
                }
            } else {
                for (int64_t k = threadIdx.x; k < m; k += blockDim.x) acc += r[k] * z[k];
            }
        }
    } else {
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
            const double zk = A.pc == kPcJacobi ? r[k] * V.h[0].id[k] : r[k];
            z[k] = zk;
            acc += r[k] * zk;
        }
    }
    return block_sum_wide(acc, red);
}

// The dense tail of one problem: column j = the tail map applied to e_j, all
// columns at once, in the cycle's precision (the FP32 smoothing of the mixed
// form, with the exact 1 x 1 coarsest solve in FP64), stored row-major.
// Building it in FP64 cost the mixed form about a third of its FP64 work.
template <class T>
__device__ void block_build_tail(const BatchArgs& A, const BlockViews<T>& V) {
    const int tl = V.tl, N = V.ntail;
    const Lvl<T>& L = V.lm[tl];
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
        const int j = t / N, k = t - j * N;  // right-hand side j, cell k
        L.b[t] = (k == j) ? T(1) : T(0);
    }
    __syncthreads();
    block_cycle_m<T>(V.lm, tl, V.nlev, A.pre, A.post, A.gamma, A.gamma, N, V.h[V.nlev - 1].id);
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
        const int j = t / N, k = t - j * N;
        V.tail[k * N + j] = L.x[t];
    }
    __syncthreads();
}

// Build the hierarchy of one problem into the CTA's arena (and its dense
// tail). Returns the first invalid permeability index (~0 if valid).
template <class T>
__device__ unsigned long long block_setup(const BatchArgs& A, const double* a, const BlockViews<T>& V,
                                          unsigned long long* s_bad) {
    if (threadIdx.x == 0) *s_bad = ~0ull;
    __syncthreads();
    // FP64 reciprocal diagonals: every level for an FP64 cycle; level 0 for
    // the Jacobi preconditioner; otherwise the coarsest level's exact solve only.
    const bool fp64_id = sizeof(T) == 8 || A.pc != kPcMultigrid;
    build_fine_block(a, V.h[0], s_bad, fp64_id || V.nlev == 1);
    for (int l = 1; l < V.nlev; ++l) {
        coarsen<BlockScope>(V.h[l - 1], V.h[l], fp64_id || l == V.nlev - 1);
        __syncthreads();
    }
    if (A.pc == kPcMultigrid) {
        for (int l = 0; l < V.nlev; ++l) block_copy_coeffs<T>(V.h[l], V.lv[l]);
        for (int l = V.tl ? V.tl : V.nlev; l < V.nlev; ++l) block_copy_coeffs<T>(V.h[l], V.lm[l]);
        __syncthreads();
        if (V.tl && *s_bad == ~0ull) block_build_tail<T>(A, V);
    }
    __syncthreads();
    return *s_bad;
}

}  // namespace dgpu

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
// wb/sb boundary vectors), the five FP64 CG vectors b, r, p, Ap, z, and the
// cycle's own coefficient copies and iterate/right-hand side for the large
// levels. Shared memory: the same for every level from `ls` down, as many
// coarse levels as fit in `sbudget` bytes -- the W-cycle visits level l 2^l
// times, so the coarse levels are the ones whose latency matters. Level 0 of
// an FP64 cycle works directly on r (right-hand side) and z (iterate).
// Shared by host sizing and device carving (gbase/sbase == null: size only).
struct BlockLayout {
    size_t global_bytes, smem_bytes;
    int nlev, ls;
};

template <class T>
__host__ __device__ BlockLayout carve(int n, char* gbase, char* sbase, size_t sbudget, Lvl64* h, Lvl<T>* lv,
                                      double** cg) {
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
    int ls = nlev;
    size_t need = 0;
    for (int l = nlev - 1; l >= 1; --l) {
        const size_t lvl = 6 * (((size_t)sides[l] * sides[l] * sizeof(T) + 15) & ~(size_t)15);
        if (need + lvl > sbudget) break;
        need += lvl;
        ls = l;
    }
    const bool fp32 = sizeof(T) == 4;
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
        if (h) h[l] = H;
    }
    double* v[5];
    for (int q = 0; q < 5; ++q) v[q] = (double*)gtake(8 * m0);
    if (cg)
        for (int q = 0; q < 5; ++q) cg[q] = v[q];
    for (int l = 0; l < nlev; ++l) {
        const size_t m = (size_t)sides[l] * sides[l];
        const bool shared = l >= ls;
        auto take = [&](size_t bytes) { return shared ? stake(bytes) : gtake(bytes); };
        Lvl<T> V;
        V.n = sides[l];
        if (fp32 || shared) {
            V.e = (const T*)take(sizeof(T) * m);
            V.nf = (const T*)take(sizeof(T) * m);
            V.d = (const T*)take(sizeof(T) * m);
            V.id = (const T*)take(sizeof(T) * m);
        } else {
            V.e = h ? (const T*)h[l].e : nullptr;
            V.nf = h ? (const T*)h[l].nf : nullptr;
            V.d = h ? (const T*)h[l].d : nullptr;
            V.id = h ? (const T*)h[l].id : nullptr;
        }
        if (l == 0 && !fp32) {
            V.x = (T*)v[4];  // z
            V.b = (T*)v[1];  // r
        } else {
            V.x = (T*)take(sizeof(T) * m);
            V.b = (T*)take(sizeof(T) * m);
        }
        if (lv) lv[l] = V;
    }
    return BlockLayout{goff, soff, nlev, ls};
}

// Cycle coefficients of level l in the cycle's precision (FP32 copies for the
// mixed form, shared-memory copies for the levels held on chip).
template <class T>
__device__ __forceinline__ void block_copy_coeffs(const Lvl64& H, const Lvl<T>& V) {
    if ((const void*)V.e == (const void*)H.e) return;  // FP64 level used in place
    const int64_t m = (int64_t)H.n * H.n;
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
        ((T*)V.e)[k] = (T)H.e[k];
        ((T*)V.nf)[k] = (T)H.nf[k];
        ((T*)V.d)[k] = (T)H.d[k];
        ((T*)V.id)[k] = (T)H.id[k];
    }
}

// y = A x over a block, FP64, returning sum x . y (or x . x when want_xx).
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
    return block_sum(acc, red);
}

// z = M r for one problem; returns r . z. For the FP32 cycle, r is rounded
// into the level-0 right-hand side and the FP32 iterate widened into z.
template <class T>
__device__ double block_precondition(const BatchArgs& A, const Lvl64* h, const Lvl<T>* lv, int nlev,
                                     const double* r, double* z, double* red) {
    const int n = h[0].n;
    const int64_t m = (int64_t)n * n;
    double acc = 0.0;
    if (A.pc == kPcMultigrid) {
        if (sizeof(T) == 4) {
            for (int64_t k = threadIdx.x; k < m; k += blockDim.x) lv[0].b[k] = (T)r[k];
            __syncthreads();
            block_cycle<T>(lv, 0, nlev, A.pre, A.post, A.gamma, 1, h[nlev - 1].id);
            for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
                const double zk = (double)lv[0].x[k];
                z[k] = zk;
                acc += r[k] * zk;
            }
        } else {
            block_cycle<T>(lv, 0, nlev, A.pre, A.post, A.gamma, 1, nullptr);
            for (int64_t k = threadIdx.x; k < m; k += blockDim.x) acc += r[k] * z[k];
        }
    } else {
        for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
            const double zk = A.pc == kPcJacobi ? r[k] * h[0].id[k] : r[k];
            z[k] = zk;
            acc += r[k] * zk;
        }
    }
    return block_sum(acc, red);
}

// Build the hierarchy of one problem into the CTA's arena. Returns the first
// invalid permeability index (~0 if the field is valid).
template <class T>
__device__ unsigned long long block_setup(const BatchArgs& A, const double* a, const Lvl64* h, const Lvl<T>* lv,
                                          int nlev, unsigned long long* s_bad) {
    if (threadIdx.x == 0) *s_bad = ~0ull;
    __syncthreads();
    build_fine<BlockScope>(a, h[0], s_bad);
    __syncthreads();
    for (int l = 1; l < nlev; ++l) {
        coarsen<BlockScope>(h[l - 1], h[l]);
        __syncthreads();
    }
    if (A.pc == kPcMultigrid)
        for (int l = 0; l < nlev; ++l) block_copy_coeffs<T>(h[l], lv[l]);
    __syncthreads();
    return *s_bad;
}

}  // namespace dgpu

// Fused level visits for the grid engine: one kernel for everything before
// the coarse-grid correction, one for everything after it.
//
//   k_visit_pre : red sweep, black sweep, residual and 2x2 restriction
//                 (multigrid.hpp:108-115 with pre_sweeps = 1)
//   k_visit_post: prolongation, black sweep, red sweep, and on level 0 the
//                 r . z reduction (multigrid.hpp:119-126, solver.hpp:167-171)
//
// Each CTA owns a TH x TW tile (even origin, so it holds whole aggregates)
// and stages a halo in shared memory: red-black updates only look one cell
// away, so a tile can finish k dependent colour passes on its own if it
// recomputes k rings of halo. Cells outside the domain are staged as zero
// (x = 0 and face = 0), which reproduces the reference's skipped boundary
// terms exactly: adding e * 0 leaves the running sum bit-identical.
//
// Coefficients are the FP64 hierarchy in both forms. They do not change
// during a solve, so they are staged before the programmatic-launch wait and
// their load overlaps the previous kernel. The FP32 form converts them on the
// fly for its smoothing and keeps the residual it restricts in FP64: at high
// permeability contrast b - A x cancels to far below the size of its terms,
// and an FP32 residual there weakens the cycle enough to cost CG iterations.
//
// Both kernels read x from one buffer and write another (the halo of a
// neighbouring tile must see the values from before this pass), so the host
// alternates two iterate buffers per level. They do not look at the solve's
// `done` flag: after convergence the rest of that loop iteration only
// rewrites cycle scratch, which nothing reads.
#pragma once

#include "common.cuh"
#include "setup.cuh"

namespace dgpu {

template <int TH, int TW, int R>
struct Tile {
    static constexpr int SH = TH + 2 * R, SW = TW + 2 * R, S = SH * SW;
};

// Stage e, nf, id (and d when ds != null) of the tile + halo.
template <int TH, int TW, int R>
__device__ __forceinline__ void stage_coeffs(const Lvl64& H, int ti0, int tj0, double* es, double* ns, double* ds,
                                             double* is) {
    using G = Tile<TH, TW, R>;
    const int n = H.n;
    for (int q = threadIdx.x; q < G::S; q += blockDim.x) {
        const int li = q / G::SW, lj = q - li * G::SW;
        const int gi = ti0 - R + li, gj = tj0 - R + lj;
        double ev = 0.0, nv = 0.0, dv = 0.0, iv = 0.0;
        if (gi >= 0 && gi < n && gj >= 0 && gj < n) {
            const int k = gi * n + gj;
            ev = __ldg(H.e + k);
            nv = __ldg(H.nf + k);
            if (ds) dv = __ldg(H.d + k);
            iv = __ldg(H.id + k);
        }
        es[q] = ev;
        ns[q] = nv;
        if (ds) ds[q] = dv;
        is[q] = iv;
    }
}

// Stage x (+ the prolongation xc[aggregate] when xc != null) and b.
template <class T, int TH, int TW, int R>
__device__ __forceinline__ void stage_vectors(int n, const T* __restrict__ xin, const T* __restrict__ xc,
                                              const T* __restrict__ b, int ti0, int tj0, T* xs, T* bs) {
    using G = Tile<TH, TW, R>;
    const int nc = (n + 1) >> 1;
    for (int q = threadIdx.x; q < G::S; q += blockDim.x) {
        const int li = q / G::SW, lj = q - li * G::SW;
        const int gi = ti0 - R + li, gj = tj0 - R + lj;
        T xv = T(0), bv = T(0);
        if (gi >= 0 && gi < n && gj >= 0 && gj < n) {
            const int k = gi * n + gj;
            if (xin) xv = xin[k];
            if (xc) xv += xc[(gi >> 1) * nc + (gj >> 1)];
            bv = b[k];
        }
        xs[q] = xv;
        bs[q] = bv;
    }
}

// One colour pass on the staged tile over local rows/cols [lo, SH-lo) x
// [lo, SW-lo), in-domain cells of colour c only (level.hpp:145-161), in the
// cycle's precision T.
template <class T, int TH, int TW, int R>
__device__ __forceinline__ void stage_gs(int n, int ti0, int tj0, int lo, int c, T* xs, const double* es,
                                         const double* ns, const double* is, const T* bs) {
    using G = Tile<TH, TW, R>;
    const int h = G::SH - 2 * lo, w = G::SW - 2 * lo;
    for (int q = threadIdx.x; q < h * w; q += blockDim.x) {
        const int li = lo + q / w, lj = lo + (q - (q / w) * w);
        const int gi = ti0 - R + li, gj = tj0 - R + lj;
        if (((gi + gj) & 1) != c || gi < 0 || gi >= n || gj < 0 || gj >= n) continue;
        const int s = li * G::SW + lj;
        T v = bs[s];
        v += (T)es[s] * xs[s + 1];
        v += (T)es[s - 1] * xs[s - 1];
        v += (T)ns[s] * xs[s + G::SW];
        v += (T)ns[s - G::SW] * xs[s - G::SW];
        xs[s] = v * (T)is[s];
    }
}

template <class T, int TH, int TW>
struct VisitSmem {
    static constexpr int R = 3;
    static constexpr size_t bytes = (sizeof(double) * 4 + sizeof(T) * 2) * Tile<TH, TW, R>::S;
};
template <class T, int TH, int TW>
struct PostSmem {
    static constexpr size_t bytes = (sizeof(double) * 3 + sizeof(T) * 2) * Tile<TH, TW, 2>::S;
};

// Pre-smoothing (1 sweep: red then black), residual, restriction. xin == null
// means the iterate is known to be zero (first call from the parent). b64,
// when given, is the level's right-hand side in FP64 (level 0: the CG
// residual) for the residual; otherwise the staged b is used.
template <class T, int TH, int TW>
__global__ void __launch_bounds__(256) k_visit_pre(Lvl64 H, const T* __restrict__ b, const double* __restrict__ b64,
                                                   const T* __restrict__ xin, T* __restrict__ xout,
                                                   T* __restrict__ bc) {
    constexpr int R = 3;
    using G = Tile<TH, TW, R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* es = reinterpret_cast<double*>(smem_raw);
    double* ns = es + G::S;
    double* ds = ns + G::S;
    double* is = ds + G::S;
    T* xs = reinterpret_cast<T*>(is + G::S);
    T* bs = xs + G::S;
    const int n = H.n, nc = (n + 1) >> 1;
    const int tiles_x = (n + TW - 1) / TW, tiles = tiles_x * ((n + TH - 1) / TH);
    bool waited = false;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int ti0 = (tile / tiles_x) * TH, tj0 = (tile % tiles_x) * TW;
        stage_coeffs<TH, TW, R>(H, ti0, tj0, es, ns, ds, is);
        if (!waited) {  // coefficients are constant: fetched while the predecessor finishes
            pdl_enter();
            waited = true;
        }
        stage_vectors<T, TH, TW, R>(n, xin, nullptr, b, ti0, tj0, xs, bs);
        __syncthreads();
        stage_gs<T, TH, TW, R>(n, ti0, tj0, 1, 0, xs, es, ns, is, bs);  // red, rings <= 2
        __syncthreads();
        stage_gs<T, TH, TW, R>(n, ti0, tj0, 2, 1, xs, es, ns, is, bs);  // black, rings <= 1
        __syncthreads();
        // residual of each tile cell in FP64, summed per aggregate
        // (level.hpp:122-137, :214-227)
        for (int q = threadIdx.x; q < (TH / 2) * (TW / 2); q += blockDim.x) {
            const int ai = q / (TW / 2), aj = q - ai * (TW / 2);
            const int I = (ti0 >> 1) + ai, J = (tj0 >> 1) + aj;
            if (I >= nc || J >= nc) continue;
            double acc = 0.0;
            for (int di = 0; di < 2; ++di) {
                const int gi = 2 * I + di;
                if (gi >= n) break;
                for (int dj = 0; dj < 2; ++dj) {
                    const int gj = 2 * J + dj;
                    if (gj >= n) break;
                    const int s = (R + 2 * ai + di) * G::SW + (R + 2 * aj + dj);
                    double v = ds[s] * (double)xs[s];
                    v -= es[s] * (double)xs[s + 1];
                    v -= es[s - 1] * (double)xs[s - 1];
                    v -= ns[s] * (double)xs[s + G::SW];
                    v -= ns[s - G::SW] * (double)xs[s - G::SW];
                    const double bv = b64 ? b64[gi * n + gj] : (double)bs[s];
                    acc += bv - v;
                }
            }
            bc[I * nc + J] = (T)acc;
        }
        // the smoothed iterate of the tile
        for (int q = threadIdx.x; q < TH * TW; q += blockDim.x) {
            const int li = q / TW, lj = q - li * TW;
            const int gi = ti0 + li, gj = tj0 + lj;
            if (gi < n && gj < n) xout[gi * n + gj] = xs[(R + li) * G::SW + (R + lj)];
        }
        __syncthreads();
    }
    if (!waited) pdl_enter();
}

// Prolongation + post-smoothing (1 sweep: black then red). On level 0 (r
// given) also r . z and beta, like k_gs0_dot.
template <class T, int TH, int TW>
__global__ void __launch_bounds__(256) k_visit_post(Lvl64 H, const T* __restrict__ b, const T* __restrict__ xin,
                                                    const T* __restrict__ xc, T* __restrict__ xout,
                                                    const double* __restrict__ r, CgState* st, double* partials) {
    constexpr int R = 2;
    using G = Tile<TH, TW, R>;
    __shared__ double red[32];
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* es = reinterpret_cast<double*>(smem_raw);
    double* ns = es + G::S;
    double* is = ns + G::S;
    T* xs = reinterpret_cast<T*>(is + G::S);
    T* bs = xs + G::S;
    const int n = H.n;
    const int tiles_x = (n + TW - 1) / TW, tiles = tiles_x * ((n + TH - 1) / TH);
    double acc = 0.0;
    bool waited = false;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int ti0 = (tile / tiles_x) * TH, tj0 = (tile % tiles_x) * TW;
        stage_coeffs<TH, TW, R>(H, ti0, tj0, es, ns, nullptr, is);
        if (!waited) {
            pdl_enter();
            waited = true;
        }
        stage_vectors<T, TH, TW, R>(n, xin, xc, b, ti0, tj0, xs, bs);
        __syncthreads();
        stage_gs<T, TH, TW, R>(n, ti0, tj0, 1, 1, xs, es, ns, is, bs);  // black, rings <= 1
        __syncthreads();
        stage_gs<T, TH, TW, R>(n, ti0, tj0, 2, 0, xs, es, ns, is, bs);  // red, ring 0
        __syncthreads();
        for (int q = threadIdx.x; q < TH * TW; q += blockDim.x) {
            const int li = q / TW, lj = q - li * TW;
            const int gi = ti0 + li, gj = tj0 + lj;
            if (gi < n && gj < n) {
                const int k = gi * n + gj;
                const T v = xs[(R + li) * G::SW + (R + lj)];
                xout[k] = v;
                if (r) acc += r[k] * (double)v;
            }
        }
        __syncthreads();
    }
    if (!waited) pdl_enter();
    if (!r) return;
    double tot;
    if (!grid_sum_last(acc, partials, &st->ticket[1], red, tot)) return;
    if (threadIdx.x == 0) {
        st->beta = st->it == 0 ? 0.0 : (tot - st->rzo) / st->rz;
        st->rz = tot;
    }
}

}  // namespace dgpu

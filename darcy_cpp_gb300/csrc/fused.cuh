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
// Coefficients do not change during a solve (they are written by the setup
// kernels, which complete before the solve's loop starts), so they are
// staged before the programmatic-launch wait and their load overlaps the
// previous kernel; everything the previous kernel produces is read after it.
//
// FP32 cycle (mixed form). Smoothing and transfers run in FP32. The residual
// that is restricted is formed in double-float arithmetic -- FP32 hi/lo
// coefficient pairs, error-free products (FMA) and compensated sums -- which
// is accurate to ~2^-48 of its largest term while using only the FP32 pipes:
// at high permeability contrast b - A x cancels far below the size of its
// terms, where a plain FP32 residual weakens the cycle and costs CG
// iterations, and GB300's FP64 (and FP64<->FP32 conversion) rate is ~1/60 of
// its FP32 rate.
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

// Level data a fused visit reads. For T = double: the FP64 hierarchy, lo
// pointers null. For T = float: FP32 hi parts and the lo parts of e, nf, d
// (c = hi + lo to ~2^-48); blo is the lo part of b where it exists (level 0).
template <class T>
struct VisitLevel {
    int n;
    const T* e;
    const T* nf;
    const T* d;
    const T* id;
    const T* elo;
    const T* nlo;
    const T* dlo;
    const T* b;
    const T* blo;
};

// ---------------------------------------------------------- double-float
struct DF {
    float hi, lo;
};
// s + v, v = (vh, vl) with |vl| << |vh|: TwoSum on the hi parts.
__device__ __forceinline__ void df_add(DF& s, float vh, float vl) {
    const float t = s.hi + vh;
    const float bb = t - s.hi;
    const float err = (s.hi - (t - bb)) + (vh - bb);
    s.hi = t;
    s.lo += err + vl;
}
// s += sign * (ch + cl) * x, x exact in FP32: error-free hi product.
__device__ __forceinline__ void df_axpy(DF& s, float ch, float cl, float x, float sign) {
    const float p = ch * x;
    const float pe = fmaf(ch, x, -p);
    df_add(s, sign * p, sign * (pe + cl * x));
}

// -------------------------------------------------------------- staging

template <class T, int TH, int TW, int R, bool WITH_D, bool WITH_LO>
__device__ __forceinline__ void stage_coeffs(const VisitLevel<T>& V, int ti0, int tj0, T* es, T* ns, T* ds, T* is,
                                             T* elo, T* nlo, T* dlo) {
    using G = Tile<TH, TW, R>;
    const int n = V.n;
    for (int q = threadIdx.x; q < G::S; q += blockDim.x) {
        const int li = q / G::SW, lj = q - li * G::SW;
        const int gi = ti0 - R + li, gj = tj0 - R + lj;
        T ev = T(0), nv = T(0), dv = T(0), iv = T(0), el = T(0), nl = T(0), dl = T(0);
        if (gi >= 0 && gi < n && gj >= 0 && gj < n) {
            const int k = gi * n + gj;
            ev = __ldg(V.e + k);
            nv = __ldg(V.nf + k);
            if (WITH_D) dv = __ldg(V.d + k);
            iv = __ldg(V.id + k);
            if (WITH_LO) {
                el = __ldg(V.elo + k);
                nl = __ldg(V.nlo + k);
                if (WITH_D) dl = __ldg(V.dlo + k);
            }
        }
        es[q] = ev;
        ns[q] = nv;
        if (WITH_D) ds[q] = dv;
        is[q] = iv;
        if (WITH_LO) {
            elo[q] = el;
            nlo[q] = nl;
            if (WITH_D) dlo[q] = dl;
        }
    }
}

// x (+ the prolongation xc[aggregate] when xc != null), b and b's lo part.
template <class T, int TH, int TW, int R>
__device__ __forceinline__ void stage_vectors(const VisitLevel<T>& V, const T* __restrict__ xin,
                                              const T* __restrict__ xc, int ti0, int tj0, T* xs, T* bs, T* bls) {
    using G = Tile<TH, TW, R>;
    const int n = V.n, nc = (n + 1) >> 1;
    for (int q = threadIdx.x; q < G::S; q += blockDim.x) {
        const int li = q / G::SW, lj = q - li * G::SW;
        const int gi = ti0 - R + li, gj = tj0 - R + lj;
        T xv = T(0), bv = T(0), bl = T(0);
        if (gi >= 0 && gi < n && gj >= 0 && gj < n) {
            const int k = gi * n + gj;
            if (xin) xv = xin[k];
            if (xc) xv += xc[(gi >> 1) * nc + (gj >> 1)];
            bv = V.b[k];
            if (bls && V.blo) bl = V.blo[k];
        }
        xs[q] = xv;
        bs[q] = bv;
        if (bls) bls[q] = bl;
    }
}

// One colour pass over the in-domain cells of colour c inside local rows /
// cols [LO, S-LO): every row of the region holds exactly half its cells of
// each colour (the staged width is even), so cells are enumerated directly.
template <class T, int TH, int TW, int R, int LO>
__device__ __forceinline__ void stage_gs(int n, int ti0, int tj0, int c, T* xs, const T* es, const T* ns,
                                         const T* is, const T* bs) {
    using G = Tile<TH, TW, R>;
    constexpr int h = G::SH - 2 * LO, hw = (G::SW - 2 * LO) / 2;
    static_assert((G::SW - 2 * LO) % 2 == 0, "even staged width");
    for (int q = threadIdx.x; q < h * hw; q += blockDim.x) {
        const int r = q / hw, k = q - r * hw;
        const int li = LO + r;
        const int gi = ti0 - R + li;
        // first local column of colour c in this row
        const int par = (c - gi - (tj0 - R) - LO) & 1;
        const int lj = LO + par + 2 * k;
        const int gj = tj0 - R + lj;
        if (gi < 0 || gi >= n || gj < 0 || gj >= n) continue;
        const int s = li * G::SW + lj;
        T v = bs[s];
        v += es[s] * xs[s + 1];
        v += es[s - 1] * xs[s - 1];
        v += ns[s] * xs[s + G::SW];
        v += ns[s - G::SW] * xs[s - G::SW];
        xs[s] = v * is[s];
    }
}

template <class T, int TH, int TW>
struct VisitSmem {
    // FP64: e, nf, d, id, x, b. FP32: + e_lo, nf_lo, d_lo, b_lo.
    static constexpr int arrays = sizeof(T) == 8 ? 6 : 10;
    static constexpr size_t bytes = sizeof(T) * arrays * Tile<TH, TW, 3>::S;
};
template <class T, int TH, int TW>
struct PostSmem {
    static constexpr size_t bytes = sizeof(T) * 5 * Tile<TH, TW, 2>::S;
};

// Pre-smoothing (1 sweep: red then black), residual, restriction. xin == null
// means the iterate is known to be zero (first call from the parent).
template <class T, int TH, int TW>
__global__ void __launch_bounds__(256) k_visit_pre(VisitLevel<T> V, const T* __restrict__ xin, T* __restrict__ xout,
                                                   T* __restrict__ bc) {
    constexpr int R = 3;
    constexpr bool LO = sizeof(T) == 4;
    using G = Tile<TH, TW, R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* es = reinterpret_cast<T*>(smem_raw);
    T* ns = es + G::S;
    T* ds = ns + G::S;
    T* is = ds + G::S;
    T* xs = is + G::S;
    T* bs = xs + G::S;
    T* elo = LO ? bs + G::S : nullptr;
    T* nlo = LO ? elo + G::S : nullptr;
    T* dlo = LO ? nlo + G::S : nullptr;
    T* bls = LO ? dlo + G::S : nullptr;
    const int n = V.n, nc = (n + 1) >> 1;
    const int tiles_x = (n + TW - 1) / TW, tiles = tiles_x * ((n + TH - 1) / TH);
    bool waited = false;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int ti0 = (tile / tiles_x) * TH, tj0 = (tile % tiles_x) * TW;
        stage_coeffs<T, TH, TW, R, true, LO>(V, ti0, tj0, es, ns, ds, is, elo, nlo, dlo);
        if (!waited) {
            pdl_enter();
            waited = true;
        }
        stage_vectors<T, TH, TW, R>(V, xin, nullptr, ti0, tj0, xs, bs, bls);
        __syncthreads();
        stage_gs<T, TH, TW, R, 1>(n, ti0, tj0, 0, xs, es, ns, is, bs);  // red, rings <= 2
        __syncthreads();
        stage_gs<T, TH, TW, R, 2>(n, ti0, tj0, 1, xs, es, ns, is, bs);  // black, rings <= 1
        __syncthreads();
        // residual of each tile cell, summed per aggregate (level.hpp:122-137, :214-227)
        for (int q = threadIdx.x; q < (TH / 2) * (TW / 2); q += blockDim.x) {
            const int ai = q / (TW / 2), aj = q - ai * (TW / 2);
            const int I = (ti0 >> 1) + ai, J = (tj0 >> 1) + aj;
            if (I >= nc || J >= nc) continue;
            if constexpr (sizeof(T) == 8) {
                T acc = T(0);
                for (int di = 0; di < 2; ++di) {
                    if (2 * I + di >= n) break;
                    for (int dj = 0; dj < 2; ++dj) {
                        if (2 * J + dj >= n) break;
                        const int s = (R + 2 * ai + di) * G::SW + (R + 2 * aj + dj);
                        T v = ds[s] * xs[s];
                        v -= es[s] * xs[s + 1];
                        v -= es[s - 1] * xs[s - 1];
                        v -= ns[s] * xs[s + G::SW];
                        v -= ns[s - G::SW] * xs[s - G::SW];
                        acc += bs[s] - v;
                    }
                }
                bc[I * nc + J] = acc;
            } else {
                DF acc{0.f, 0.f};
                for (int di = 0; di < 2; ++di) {
                    if (2 * I + di >= n) break;
                    for (int dj = 0; dj < 2; ++dj) {
                        if (2 * J + dj >= n) break;
                        const int s = (R + 2 * ai + di) * G::SW + (R + 2 * aj + dj);
                        // r = b - d x + e xE + w xW + n xN + s xS
                        df_add(acc, bs[s], bls[s]);
                        df_axpy(acc, ds[s], dlo[s], xs[s], -1.f);
                        df_axpy(acc, es[s], elo[s], xs[s + 1], 1.f);
                        df_axpy(acc, es[s - 1], elo[s - 1], xs[s - 1], 1.f);
                        df_axpy(acc, ns[s], nlo[s], xs[s + G::SW], 1.f);
                        df_axpy(acc, ns[s - G::SW], nlo[s - G::SW], xs[s - G::SW], 1.f);
                    }
                }
                bc[I * nc + J] = acc.hi + acc.lo;
            }
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

// The W-cycle's second call of a level follows the first call's
// post-smoothing directly: post (prolongation, black, red) then pre (red,
// black, residual, restriction). The two red passes in the middle read the
// same black values and produce the same result, so one is kept: prolongation
// + black + red + black + residual/restriction in one kernel, halo 4.
template <class T, int TH, int TW>
struct MidSmem {
    static constexpr int arrays = sizeof(T) == 8 ? 6 : 10;
    static constexpr size_t bytes = sizeof(T) * arrays * Tile<TH, TW, 4>::S;
};

template <class T, int TH, int TW>
__global__ void __launch_bounds__(256) k_visit_mid(VisitLevel<T> V, const T* __restrict__ xin,
                                                   const T* __restrict__ xc, T* __restrict__ xout,
                                                   T* __restrict__ bc) {
    constexpr int R = 4;
    constexpr bool LO = sizeof(T) == 4;
    using G = Tile<TH, TW, R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* es = reinterpret_cast<T*>(smem_raw);
    T* ns = es + G::S;
    T* ds = ns + G::S;
    T* is = ds + G::S;
    T* xs = is + G::S;
    T* bs = xs + G::S;
    T* elo = LO ? bs + G::S : nullptr;
    T* nlo = LO ? elo + G::S : nullptr;
    T* dlo = LO ? nlo + G::S : nullptr;
    T* bls = LO ? dlo + G::S : nullptr;
    const int n = V.n, nc = (n + 1) >> 1;
    const int tiles_x = (n + TW - 1) / TW, tiles = tiles_x * ((n + TH - 1) / TH);
    bool waited = false;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int ti0 = (tile / tiles_x) * TH, tj0 = (tile % tiles_x) * TW;
        stage_coeffs<T, TH, TW, R, true, LO>(V, ti0, tj0, es, ns, ds, is, elo, nlo, dlo);
        if (!waited) {
            pdl_enter();
            waited = true;
        }
        stage_vectors<T, TH, TW, R>(V, xin, xc, ti0, tj0, xs, bs, bls);  // x + prolongation
        __syncthreads();
        stage_gs<T, TH, TW, R, 1>(n, ti0, tj0, 1, xs, es, ns, is, bs);  // post black, rings <= 3
        __syncthreads();
        stage_gs<T, TH, TW, R, 2>(n, ti0, tj0, 0, xs, es, ns, is, bs);  // red (post and pre), rings <= 2
        __syncthreads();
        stage_gs<T, TH, TW, R, 3>(n, ti0, tj0, 1, xs, es, ns, is, bs);  // pre black, rings <= 1
        __syncthreads();
        for (int q = threadIdx.x; q < (TH / 2) * (TW / 2); q += blockDim.x) {
            const int ai = q / (TW / 2), aj = q - ai * (TW / 2);
            const int I = (ti0 >> 1) + ai, J = (tj0 >> 1) + aj;
            if (I >= nc || J >= nc) continue;
            if constexpr (sizeof(T) == 8) {
                T acc = T(0);
                for (int di = 0; di < 2; ++di) {
                    if (2 * I + di >= n) break;
                    for (int dj = 0; dj < 2; ++dj) {
                        if (2 * J + dj >= n) break;
                        const int s = (R + 2 * ai + di) * G::SW + (R + 2 * aj + dj);
                        T v = ds[s] * xs[s];
                        v -= es[s] * xs[s + 1];
                        v -= es[s - 1] * xs[s - 1];
                        v -= ns[s] * xs[s + G::SW];
                        v -= ns[s - G::SW] * xs[s - G::SW];
                        acc += bs[s] - v;
                    }
                }
                bc[I * nc + J] = acc;
            } else {
                DF acc{0.f, 0.f};
                for (int di = 0; di < 2; ++di) {
                    if (2 * I + di >= n) break;
                    for (int dj = 0; dj < 2; ++dj) {
                        if (2 * J + dj >= n) break;
                        const int s = (R + 2 * ai + di) * G::SW + (R + 2 * aj + dj);
                        df_add(acc, bs[s], bls[s]);
                        df_axpy(acc, ds[s], dlo[s], xs[s], -1.f);
                        df_axpy(acc, es[s], elo[s], xs[s + 1], 1.f);
                        df_axpy(acc, es[s - 1], elo[s - 1], xs[s - 1], 1.f);
                        df_axpy(acc, ns[s], nlo[s], xs[s + G::SW], 1.f);
                        df_axpy(acc, ns[s - G::SW], nlo[s - G::SW], xs[s - G::SW], 1.f);
                    }
                }
                bc[I * nc + J] = acc.hi + acc.lo;
            }
        }
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
__global__ void __launch_bounds__(256) k_visit_post(VisitLevel<T> V, const T* __restrict__ xin,
                                                    const T* __restrict__ xc, T* __restrict__ xout,
                                                    const double* __restrict__ r, CgState* st, double* partials) {
    constexpr int R = 2;
    using G = Tile<TH, TW, R>;
    __shared__ double red[256];  // block_sum_wide: one double per thread
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* es = reinterpret_cast<T*>(smem_raw);
    T* ns = es + G::S;
    T* is = ns + G::S;
    T* xs = is + G::S;
    T* bs = xs + G::S;
    const int n = V.n;
    const int tiles_x = (n + TW - 1) / TW, tiles = tiles_x * ((n + TH - 1) / TH);
    double acc = 0.0;
    bool waited = false;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int ti0 = (tile / tiles_x) * TH, tj0 = (tile % tiles_x) * TW;
        stage_coeffs<T, TH, TW, R, false, false>(V, ti0, tj0, es, ns, nullptr, is, nullptr, nullptr, nullptr);
        if (!waited) {
            pdl_enter();
            waited = true;
        }
        stage_vectors<T, TH, TW, R>(V, xin, xc, ti0, tj0, xs, bs, nullptr);
        __syncthreads();
        stage_gs<T, TH, TW, R, 1>(n, ti0, tj0, 1, xs, es, ns, is, bs);  // black, rings <= 1
        __syncthreads();
        stage_gs<T, TH, TW, R, 2>(n, ti0, tj0, 0, xs, es, ns, is, bs);  // red, ring 0
        __syncthreads();
        for (int q = threadIdx.x; q < TH * TW; q += blockDim.x) {
            const int li = q / TW, lj = q - li * TW;
            const int gi = ti0 + li, gj = tj0 + lj;
            if (gi < n && gj < n) {
                const int k = gi * n + gj;
                const T v = xs[(R + li) * G::SW + (R + lj)];
                xout[k] = v;
                if (r) acc += r[k] * widen_f32(v);
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

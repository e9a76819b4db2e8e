// Hierarchy construction on the device, in FP64 (the Galerkin sums and the
// reciprocal diagonal are the steps whose accuracy the cycle rests on; an FP32
// cycle takes its reciprocal diagonal from the FP32 copy of d instead).
#pragma once

#include <math.h>

#include "common.cuh"

namespace dgpu {

// FP64 level storage, plus the boundary west/south faces used only here.
struct Lvl64 {
    int n;
    double* e;
    double* nf;
    double* d;
    double* id;
    double* wb;  // west boundary face of row i (cell (i, 0))
    double* sb;  // south boundary face of column j (cell (0, j))
};

// include/darcy/level.hpp:57. 2*x*y is (2x)*y: exact scaling then one rounded
// product, so harmonic(x, y) == harmonic(y, x) bit for bit.
__device__ __forceinline__ double harmonic(double x, double y) { return 2.0 * x * y / (x + y); }

// level.hpp:79-97 plus validate_permeability (solver.hpp:68-77): the first
// offending flat index is folded into *bad with atomicMin.
template <class S>
__device__ __forceinline__ void build_fine(const double* __restrict__ a, const Lvl64& L,
                                           unsigned long long* bad) {
    const int n = L.n;
    const int64_t m = (int64_t)n * n;
    for (int64_t k = S::start(); k < m; k += S::stride()) {
        const int i = (int)(k / n), j = (int)(k - (int64_t)i * n);
        const double c = a[k];
        if (!(c > 0.0) || !isfinite(c)) atomicMin(bad, (unsigned long long)k);
        const double e = (j + 1 < n) ? harmonic(c, a[k + 1]) : c;
        const double w = (j > 0) ? harmonic(c, a[k - 1]) : c;
        const double nn = (i + 1 < n) ? harmonic(c, a[k + n]) : c;
        const double s = (i > 0) ? harmonic(c, a[k - n]) : c;
        const double dd = e + w + nn + s;
        L.e[k] = e;
        L.nf[k] = nn;
        L.d[k] = dd;
        L.id[k] = 1.0 / dd;
        if (j == 0) L.wb[i] = w;
        if (i == 0) L.sb[j] = s;
    }
}

// build_fine for one CTA with every face computed once (one division per
// face instead of two; FP64 division is tens of instructions on the narrow
// FP64 pipe): the east/north faces and the boundary faces first, then the
// diagonal from the stored faces in build_fine's summation order. A cell's
// west/south face is its neighbour's east/north face, the same bits since
// harmonic() is symmetric, so the level equals build_fine's bit for bit.
// with_id false leaves id unwritten (the FP32 cycle computes its own
// reciprocal from the FP32 diagonal). Returns with the CTA synchronised.
__device__ __forceinline__ void build_fine_block(const double* __restrict__ a, const Lvl64& L,
                                                 unsigned long long* bad, bool with_id) {
    const int n = L.n;
    const int64_t m = (int64_t)n * n;
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
        const int i = (int)(k / n), j = (int)(k - (int64_t)i * n);
        const double c = a[k];
        if (!(c > 0.0) || !isfinite(c)) atomicMin(bad, (unsigned long long)k);
        L.e[k] = (j + 1 < n) ? harmonic(c, a[k + 1]) : c;
        L.nf[k] = (i + 1 < n) ? harmonic(c, a[k + n]) : c;
        if (j == 0) L.wb[i] = c;
        if (i == 0) L.sb[j] = c;
    }
    __syncthreads();
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
        const int i = (int)(k / n), j = (int)(k - (int64_t)i * n);
        const double w = (j > 0) ? L.e[k - 1] : L.wb[i];
        const double s = (i > 0) ? L.nf[k - n] : L.sb[j];
        const double dd = L.e[k] + w + L.nf[k] + s;
        L.d[k] = dd;
        if (with_id) L.id[k] = 1.0 / dd;
    }
    __syncthreads();
}

// Galerkin coarse operator P^T A P by face summation (level.hpp:171-211),
// including the width-one trailing aggregate of an odd grid. West/south fine
// faces come from the neighbour's east/north face (same bits) or, on the
// domain boundary, from wb/sb; summation order is the reference's. with_id
// false leaves id unwritten, as in build_fine_block.
template <class S>
__device__ __forceinline__ void coarsen(const Lvl64& F, const Lvl64& C, bool with_id = true) {
    const int n = F.n, nc = C.n;
    const int64_t mc = (int64_t)nc * nc;
    for (int64_t K = S::start(); K < mc; K += S::stride()) {
        const int I = (int)(K / nc), J = (int)(K - (int64_t)I * nc);
        const int i0 = 2 * I, i1 = (2 * I + 1 < n) ? 2 * I + 1 : 2 * I;
        const int j0 = 2 * J, j1 = (2 * J + 1 < n) ? 2 * J + 1 : 2 * J;
        double ce = 0.0, cw = 0.0, cn = 0.0, cs = 0.0;
        for (int i = i0; i <= i1; ++i) {
            ce += F.e[(int64_t)i * n + j1];
            cw += (j0 > 0) ? F.e[(int64_t)i * n + j0 - 1] : F.wb[i];
        }
        for (int j = j0; j <= j1; ++j) {
            cn += F.nf[(int64_t)i1 * n + j];
            cs += (i0 > 0) ? F.nf[(int64_t)(i0 - 1) * n + j] : F.sb[j];
        }
        const double dd = ce + cw + cn + cs;
        C.e[K] = ce;
        C.nf[K] = cn;
        C.d[K] = dd;
        if (with_id) C.id[K] = 1.0 / dd;
        if (J == 0) C.wb[I] = cw;
        if (I == 0) C.sb[J] = cs;
    }
}

// FP32 copy of a level's coefficients for the mixed-precision cycle. When
// the lo pointers are given, also the rounding remainders of e, nf, d
// (c - (double)(float)c, rounded to FP32): hi + lo carries ~48 bits.
template <class S>
__device__ __forceinline__ void to_fp32(const Lvl64& L, float* e, float* nf, float* d, float* id, float* elo,
                                        float* nlo, float* dlo) {
    const int64_t m = (int64_t)L.n * L.n;
    for (int64_t k = S::start(); k < m; k += S::stride()) {
        float eh, el, nh, nl, dh, dl;  // split_f64: the conversions' bits without the FP64 pipe
        split_f64(L.e[k], eh, el);
        split_f64(L.nf[k], nh, nl);
        split_f64(L.d[k], dh, dl);
        e[k] = eh;
        nf[k] = nh;
        d[k] = dh;
        id[k] = round_f64(L.id[k]);
        if (elo) {
            elo[k] = el;
            nlo[k] = nl;
            dlo[k] = dl;
        }
    }
}

}  // namespace dgpu

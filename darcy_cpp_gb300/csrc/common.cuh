// Shared device-side building blocks of the darcy GB300 engine.
//
// Data layout (one problem, one level of side n, m = n*n cells, row-major):
//   e[m]    east-face transmissibility of cell k (boundary face at j = n-1)
//   nf[m]   north-face transmissibility (boundary face at i = n-1)
//   d[m]    diagonal = e + w + n + s (boundary faces included)
//   id[m]   1 / d
// The west face of cell k is e[k-1] and the south face nf[k-n] for interior
// cells: the harmonic mean (and every Galerkin face sum) is symmetric in its
// two cells, bit for bit, so the reference's separate w/s arrays
// (include/darcy/level.hpp:253) carry no extra information except on the
// boundary, where they only enter d. Boundary west/south faces are kept in two
// n-vectors (wb, sb) for the coarsening step only.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace dgpu {

constexpr int kMaxLevels = 32;  // include/darcy/multigrid.hpp:46

template <class T>
struct Lvl {
    int n;              // side
    const T* e;         // east faces
    const T* nf;        // north faces
    const T* d;         // diagonal
    const T* id;        // 1 / diagonal
    T* x;               // iterate
    T* b;               // right-hand side
};

// Execution scopes: a phase is written once and run either by a whole grid
// (one kernel per phase) or by one CTA (phases separated by __syncthreads).
struct GridScope {
    __device__ static int64_t start() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ static int64_t stride() { return (int64_t)gridDim.x * blockDim.x; }
    __device__ static void sync() {}
};
struct BlockScope {
    __device__ static int64_t start() { return threadIdx.x; }
    __device__ static int64_t stride() { return blockDim.x; }
    __device__ static void sync() { __syncthreads(); }
};

// Number of cells of colour c ((i + j) % 2 == c) on an n x n grid.
__host__ __device__ inline int64_t colour_count(int n, int c) {
    return ((int64_t)n * n + 1 - c) / 2;
}

// t-th cell of colour c, in row-major order. Rows pair up: rows 2p and 2p+1
// together hold exactly n cells of each colour.
__device__ __forceinline__ void colour_cell(int n, int c, int64_t t, int& i, int& j) {
    const int p = (int)t / n;  // cells < 2^31: grids are capped at n = 46340
    const int r = (int)t - p * n;
    const int o0 = c & 1;
    const int cnt0 = (n - o0 + 1) >> 1;
    if (r < cnt0) {
        i = (int)(2 * p);
        j = o0 + 2 * r;
    } else {
        i = (int)(2 * p + 1);
        j = (o0 ^ 1) + 2 * (r - cnt0);
    }
}

// ---------------------------------------------------------------- level ops
//
// Operation order follows the reference loops (level.hpp:105-161): the
// diagonal term first, then east, west, north, south. The GPU contracts each
// multiply-add into an FMA, so results agree with the reference to rounding,
// not bit for bit.

// Red-black Gauss-Seidel, one colour, in place (level.hpp:145-161).
// `zero` means x is known to be 0: the update collapses to x = b / d.
template <class S, class T>
__device__ __forceinline__ void gs_colour(const Lvl<T> L, int c, bool zero) {
    const int n = L.n;
    const int64_t cnt = colour_count(n, c);
    for (int64_t t = S::start(); t < cnt; t += S::stride()) {
        int i, j;
        colour_cell(n, c, t, i, j);
        const int64_t k = (int64_t)i * n + j;
        T v = L.b[k];
        if (!zero) {
            if (j + 1 < n) v += L.e[k] * L.x[k + 1];
            if (j > 0) v += L.e[k - 1] * L.x[k - 1];
            if (i + 1 < n) v += L.nf[k] * L.x[k + n];
            if (i > 0) v += L.nf[k - n] * L.x[k - n];
        }
        L.x[k] = v * L.id[k];
    }
}

// Residual of one cell, r = b - A x (level.hpp:122-137).
template <class T>
__device__ __forceinline__ T cell_residual(const Lvl<T>& L, int i, int j) {
    const int n = L.n;
    const int64_t k = (int64_t)i * n + j;
    T v = L.d[k] * L.x[k];
    if (j + 1 < n) v -= L.e[k] * L.x[k + 1];
    if (j > 0) v -= L.e[k - 1] * L.x[k - 1];
    if (i + 1 < n) v -= L.nf[k] * L.x[k + n];
    if (i > 0) v -= L.nf[k - n] * L.x[k - n];
    return L.b[k] - v;
}

// Fused residual + restriction: b_c = P^T (b - A x), summed over each 2x2
// aggregate in the reference order (level.hpp:214-227). The coarse iterate is
// not zero-filled here: the first coarse smoothing pass runs in `zero` mode.
template <class S, class T>
__device__ __forceinline__ void residual_restrict(const Lvl<T> L, T* bc) {
    const int n = L.n, nc = (n + 1) / 2;
    const int64_t mc = (int64_t)nc * nc;
    for (int64_t K = S::start(); K < mc; K += S::stride()) {
        const int I = (int)(K / nc), J = (int)(K - (int64_t)I * nc);
        const int i0 = 2 * I, i1 = (2 * I + 1 < n) ? 2 * I + 1 : 2 * I;
        const int j0 = 2 * J, j1 = (2 * J + 1 < n) ? 2 * J + 1 : 2 * J;
        T s = T(0);
        for (int i = i0; i <= i1; ++i)
            for (int j = j0; j <= j1; ++j) s += cell_residual(L, i, j);
        bc[K] = s;
    }
}

// Prolongation x += P x_c fused into the first post-smoothing colour (1).
// A colour-1 update reads only colour-0 neighbours and never its own value,
// and the colour-0 pass that follows overwrites every colour-0 cell, so the
// injected correction only has to be seen through the neighbours here:
// exactly the values level.hpp:230-237 followed by :145-161 would use.
template <class S, class T>
__device__ __forceinline__ void prolong_gs1(const Lvl<T> L, const T* xc) {
    const int n = L.n, nc = (n + 1) / 2;
    const int64_t cnt = colour_count(n, 1);
    for (int64_t t = S::start(); t < cnt; t += S::stride()) {
        int i, j;
        colour_cell(n, 1, t, i, j);
        const int64_t k = (int64_t)i * n + j;
        const T* xr = xc + (int64_t)(i >> 1) * nc;
        T v = L.b[k];
        if (j + 1 < n) v += L.e[k] * (L.x[k + 1] + xr[(j + 1) >> 1]);
        if (j > 0) v += L.e[k - 1] * (L.x[k - 1] + xr[(j - 1) >> 1]);
        if (i + 1 < n) v += L.nf[k] * (L.x[k + n] + xc[(int64_t)((i + 1) >> 1) * nc + (j >> 1)]);
        if (i > 0) v += L.nf[k - n] * (L.x[k - n] + xc[(int64_t)((i - 1) >> 1) * nc + (j >> 1)]);
        L.x[k] = v * L.id[k];
    }
}

// ------------------------------------------------- programmatic launches
//
// Kernels of a solve graph are launched with programmatic stream
// serialization: a kernel may be scheduled while its predecessor is still
// running, waits in pdl_wait() for the predecessor's completion and memory
// flush, and immediately lets its own successor be scheduled (pdl_trigger).
// Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
    pdl_wait();
    pdl_trigger();
}

// ------------------------------------------------------------ reductions

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum: every thread gets the total. `scratch` holds at
// least blockDim.x / 32 doubles. Fixed order, so repeated runs agree bit for bit.
__device__ __forceinline__ double block_sum(double v, double* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (warp == 0) {
        t = lane < nw ? scratch[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) scratch[0] = t;
    }
    __syncthreads();
    t = scratch[0];
    __syncthreads();
    return t;
}

// Grid-wide deterministic sum: each block stores its partial, the last block
// to finish (ticket counter) adds the partials in block order. Returns true in
// every thread of the last block, with the total in `total`.
__device__ __forceinline__ bool grid_sum_last(double v, double* partials, unsigned* ticket, double* scratch,
                                              double& total) {
    __shared__ bool s_last;
    const double bs = block_sum(v, scratch);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        __threadfence();
        const unsigned got = atomicAdd(ticket, 1u);
        s_last = (got == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double acc = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) acc += ((volatile double*)partials)[q];
    total = block_sum(acc, scratch);
    if (threadIdx.x == 0) *ticket = 0;  // ready for the next launch
    return true;
}

}  // namespace dgpu

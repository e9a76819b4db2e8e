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

// ------------------------------------------- FP64 <-> FP32 off the FP64 pipe
//
// GB300 issues FP64 arithmetic and FP64<->FP32 conversions at ~2 per SM per
// clock (measured: 529 G FP64 FMA/s against 38.8 T FP32 FMA/s), so the mixed
// form's conversions are done on the integer and FP32 pipes where the value is
// in range, bit-identical to the conversion instructions (round to nearest,
// ties to even); other values take the instructions.

// The instruction forms for values outside the integer paths' range, kept out
// of line: inlined, the compiler may evaluate them for every value and select,
// which puts the FP64-pipe conversions back on the hot path.
static __device__ __noinline__ float2 split_f64_slow(double x) {
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}
static __device__ __noinline__ float round_f64_slow(double x) { return (float)x; }
static __device__ __noinline__ double widen_f32_slow(float v) { return (double)v; }

// (float)i, rounded to nearest even, for |i| <= 2^28 without a conversion
// instruction (GB300 issues int->float conversions on its narrow FP64 pipe):
// i = h * 2^12 + l with l in [0, 4096) and |h| <= 2^16, each made exact from
// its bits (2^23 + v has v as its low significand bits), then one FMA rounds
// h * 4096 + l once.
__device__ __forceinline__ float int29_to_float(int i) {
    const int h = i >> 12;  // floor(i / 4096)
    const unsigned l = (unsigned)i & 0xFFFu;
    const float hf = __uint_as_float(0x4B000000u | (unsigned)(h + (1 << 20))) - 9437184.0f;  // 2^23 + 2^20
    const float lf = __uint_as_float(0x4B000000u | l) - 8388608.0f;                         // 2^23
    return __fmaf_rn(hf, 4096.0f, lf);
}

// hi = (float)x, lo = (float)(x - (double)hi): x as FP32 hi + lo. The 53-bit
// significand is rounded to 24 bits on integers; the remainder x - hi is an
// integer of at most 29 bits times 2^(e-52), rounded to FP32 by
// int29_to_float and scaled by an exact power of two.
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7FFu) - 1023;
    if (e < -74 || e > 126) {
        if ((bits << 1) == 0ull) {  // +-0: hi keeps the sign, x - hi is +0
            hi = __uint_as_float((unsigned)(bits >> 32));
            lo = 0.f;
        } else {  // tiny, huge, inf, nan
            const float2 t = split_f64_slow(x);
            hi = t.x;
            lo = t.y;
        }
        return;
    }
    const unsigned long long sig = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    unsigned q = (unsigned)(sig >> 29);                 // leading 24 bits
    const unsigned rem = (unsigned)sig & 0x1FFFFFFFu;   // trailing 29 bits
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (q & 1u));
    const int diff = (int)rem - (up ? 0x20000000 : 0);  // |x| - |hi| in units of 2^(e-52)
    q += up ? 1u : 0u;
    int eh = e;
    if (q == (1u << 24)) {
        q >>= 1;
        ++eh;
    }
    const unsigned sgn = (unsigned)(bits >> 63) << 31;
    hi = __uint_as_float(sgn | ((unsigned)(eh + 127) << 23) | (q & 0x7FFFFFu));
    const float l = int29_to_float(diff) * __uint_as_float((unsigned)(e - 52 + 127) << 23);
    lo = diff == 0 ? 0.f : (sgn ? -l : l);  // x - hi == +0 when exact
}

// (float)x, the hi part of split_f64.
__device__ __forceinline__ float round_f64(double x) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7FFu) - 1023;
    if (e < -126 || e > 126) return (bits << 1) == 0ull ? __uint_as_float((unsigned)(bits >> 32)) : round_f64_slow(x);
    const unsigned long long sig = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    unsigned q = (unsigned)(sig >> 29);
    const unsigned rem = (unsigned)sig & 0x1FFFFFFFu;
    q += (rem > 0x10000000u || (rem == 0x10000000u && (q & 1u))) ? 1u : 0u;
    int eh = e;
    if (q == (1u << 24)) {
        q >>= 1;
        ++eh;
    }
    return __uint_as_float(((unsigned)(bits >> 63) << 31) | ((unsigned)(eh + 127) << 23) | (q & 0x7FFFFFu));
}

// (double)v, exact: the exponent rebiased and the significand shifted.
__device__ __forceinline__ double widen_f32(float v) {
    const unsigned b = __float_as_uint(v);
    const unsigned ex = b & 0x7F800000u;
    if (ex == 0u || ex == 0x7F800000u)  // zero, subnormal, inf, nan
        return (b << 1) == 0u ? __hiloint2double((int)b, 0) : widen_f32_slow(v);
    return __hiloint2double((int)((b & 0x80000000u) | (((b >> 3) & 0x0FFFFFFFu) + 0x38000000u)), (int)(b << 29));
}
__device__ __forceinline__ double widen_f32(double v) { return v; }

// x in the cycle's precision T: round_f64 for FP32, x itself for FP64.
template <class T>
__device__ __forceinline__ T narrow_to(double x) {
    if constexpr (sizeof(T) == 4)
        return round_f64(x);
    else
        return x;
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

// Deterministic block sum with few FP64 instructions. GB300 issues FP64 adds
// at ~1/64 of the FP32 rate, and a shuffle tree in every warp (five full-warp
// adds per warp and value) cost as much FP64 issue as a streaming kernel's own
// arithmetic at a few cells per thread (ncu: cg_update's FP64 pipe 71% busy
// with 3 FMAs per cell). Here every thread stores its value, lane i of warp 0
// adds values i, i + 32, ... (two interleaved chains, all lanes busy), then one
// shuffle tree: blockDim/32 + 4 full-warp adds per block instead of
// 5 blockDim/32 + 5. `scratch` holds blockDim.x doubles; blockDim.x is a
// multiple of 32. Fixed order; every thread gets the total.
__device__ __forceinline__ double block_sum_wide(double v, double* scratch) {
    const int t = threadIdx.x, nw = (int)(blockDim.x >> 5);
    __syncthreads();  // the previous call's readers are done with scratch
    scratch[t] = v;
    __syncthreads();
    if (t < 32) {
        double s0 = scratch[t], s1 = nw > 1 ? scratch[t + 32] : 0.0;
        for (int w = 2; w < nw; w += 2) {
            s0 += scratch[t + 32 * w];
            if (w + 1 < nw) s1 += scratch[t + 32 * (w + 1)];
        }
        const double s = warp_sum(s0 + s1);
        if (t == 0) scratch[0] = s;
    }
    __syncthreads();
    return scratch[0];
}

// Grid-wide deterministic sum: each block stores its partial, the last block
// to finish (ticket counter) adds the partials in block order. Returns true in
// every thread of the last block, with the total in `total`. `scratch` holds
// blockDim.x doubles (block_sum_wide).
__device__ __forceinline__ bool grid_sum_last(double v, double* partials, unsigned* ticket, double* scratch,
                                              double& total) {
    __shared__ bool s_last;
    const double bs = block_sum_wide(v, scratch);
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
    total = block_sum_wide(acc, scratch);
    if (threadIdx.x == 0) *ticket = 0;  // ready for the next launch
    return true;
}

}  // namespace dgpu

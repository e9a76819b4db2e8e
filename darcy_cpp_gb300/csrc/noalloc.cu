// Allocation-free preconditioner entry point.
//
// Some callers of this library cannot allocate device memory while they run:
// code inside a host that owns every device allocation itself (an inference
// server's memory pool, a framework allocator, a real-time loop that must not
// enter cudaMalloc/cudaFree because those may synchronise the device or take
// a driver lock), or code running where a fresh allocation would break a
// budget fixed up front. dgpu_apply_preconditioner_noalloc serves them: it
// computes z = M r (one multigrid cycle from a zero guess, the reference's
// Multigrid::apply, include/darcy/multigrid.hpp:88-93) for one problem of
// side n <= kNoAllocMaxSide, on device buffers the caller owns, and keeps its
// scratch -- the whole FP64 hierarchy, the cycle's vectors and a status word
// -- in the file-scope array below instead of allocating it.
//
// That array is sized for the largest accepted grid and lives on every device
// that loads the library until the process exits. All calls share it and it
// keeps the last call's contents, so calls that overlap on the GPU (different
// streams, or different host threads on one device) race on it; each call
// resets the status word it reads back and rebuilds everything else it uses.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/darcy_gpu.h"
#include "block.cuh"

namespace dgpu {

namespace {

constexpr int kNoAllocMaxSide = 128;
constexpr size_t kNoAllocBytes = size_t(2) << 20;  // 2 MiB per device
constexpr size_t kStatusOffset = kNoAllocBytes - 256;  // last 256 bytes: status word

// Scratch of the allocation-free entry point (see the file comment). In host
// code this name is only a stand-in for the device symbol: its device address
// comes from cudaGetSymbolAddress on the current device, on every call.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// One cycle z = M r for a side-n problem, one CTA, all scratch in `scratch`.
__global__ void __launch_bounds__(256) k_precondition_noalloc(unsigned char* scratch, int n, int pre, int post,
                                                               int gamma, const double* __restrict__ a,
                                                               const double* __restrict__ r, double* __restrict__ z) {
    __shared__ BlockViews<double> V;
    __shared__ double red[256];  // block_sum_wide: one double per thread
    __shared__ unsigned long long s_bad;
    if (threadIdx.x == 0) carve<double>(n, (char*)scratch, nullptr, 0, &V);
    __syncthreads();
    BatchArgs A{};
    A.pc = kPcMultigrid;
    A.pre = pre;
    A.post = post;
    A.gamma = gamma;
    const unsigned long long bad = block_setup<double>(A, a, V, &s_bad);
    unsigned long long* status = reinterpret_cast<unsigned long long*>(scratch + kStatusOffset);
    if (threadIdx.x == 0) *status = bad;
    if (bad != ~0ull) return;
    const int64_t m = (int64_t)n * n;
    double* rr = V.cg[1];
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) rr[k] = r[k];
    __syncthreads();
    block_precondition<double>(A, V, rr, V.cg[4], red);
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) z[k] = V.cg[4][k];
}

// Device address of the scratch array in the current device's context. It is
// looked up on every call (a table lookup once the module is loaded; the first
// call on a device loads it): a cached address would go stale when the
// context is reset (cudaDeviceReset reloads the module, and the array can
// move).
int scratch_address(void** out) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return (int)e;
    *out = ptr;
    return 0;
}

}  // namespace

}  // namespace dgpu

using namespace dgpu;

extern "C" int dgpu_apply_preconditioner_noalloc(const double* d_a, const double* d_r, int64_t n, int pre_sweeps,
                                                 int post_sweeps, int cycle_index, double* d_z, void* stream) {
    char msg[256];
    if (n < 1 || n > kNoAllocMaxSide) {
        std::snprintf(msg, sizeof msg,
                      "grid side %lld outside the allocation-free range 1..%d (its scratch is a fixed %zu-byte array)",
                      (long long)n, kNoAllocMaxSide, kNoAllocBytes);
        set_last_error(msg);
        return DGPU_INVALID_INPUT;
    }
    if (!d_a || !d_r || !d_z) {
        set_last_error("buffers must not be NULL");
        return DGPU_INVALID_INPUT;
    }
    // The reference's sweep and cycle checks (src/bindings.cpp:231-232). The
    // reference validates the permeability first (src/bindings.cpp:225); here
    // that check runs in the kernel, after these, so an input invalid both
    // ways reports the sweep/cycle error.
    if (pre_sweeps < 1 || post_sweeps < 1) {
        set_last_error("sweeps must be at least 1");
        return DGPU_INVALID_INPUT;
    }
    if (cycle_index < 1 || cycle_index > 2) {
        set_last_error("cycle_index must be 1 or 2");
        return DGPU_INVALID_INPUT;
    }
    const size_t need = carve<double>((int)n, nullptr, nullptr, 0, nullptr).global_bytes;
    if (need > kStatusOffset) {  // cannot happen for n <= kNoAllocMaxSide; kept as the invariant
        set_last_error("allocation-free scratch too small for this grid");
        return DGPU_INVALID_INPUT;
    }
    void* scratch = nullptr;
    const int se = scratch_address(&scratch);
    if (se != 0) {
        std::snprintf(msg, sizeof msg, "cudaGetSymbolAddress failed: %s", cudaGetErrorString((cudaError_t)se));
        set_last_error(msg);
        return DGPU_CUDA_ERROR;
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* base = (unsigned char*)scratch;
    k_precondition_noalloc<<<1, 256, 0, s>>>(base, (int)n, pre_sweeps, post_sweeps, cycle_index, d_a, d_r, d_z);
    unsigned long long bad = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, base + kStatusOffset, sizeof bad, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        std::snprintf(msg, sizeof msg, "CUDA error %s (%s) in dgpu_apply_preconditioner_noalloc", cudaGetErrorName(e),
                      cudaGetErrorString(e));
        set_last_error(msg);
        return DGPU_CUDA_ERROR;
    }
    if (bad != ~0ull) {
        std::snprintf(msg, sizeof msg,
                      "permeability must be finite and strictly positive everywhere; offending value at flat index %llu",
                      bad);
        set_last_error(msg);
        return DGPU_INVALID_INPUT;
    }
    set_last_error("");
    return DGPU_OK;
}

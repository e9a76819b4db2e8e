// Random two-phase permeability fields generated on the GPU.
//
// The construction is the reference generator's (python/darcy/fields.py:31-83,
// after Li et al., "Fourier Neural Operator for Parametric PDEs"): spectral
// amplitudes tau^(alpha-1) (pi^2 |k|^2 + tau^2)^(-alpha/2) with the k = 0 mode
// dropped, times standard normal noise, an orthonormal inverse 2-D DCT, then a
// threshold at zero (>= 0 -> hi, else lo). Here the noise comes from a
// counter-based generator (Philox-4x32-10, Salmon et al., SC 2011) through the
// Box-Muller transform, and the inverse DCT is two dense n x n products in
// shared memory (x = C^T X C, C the orthonormal DCT-II matrix), in FP32: the
// fields follow the host generator's distribution, not its bits (numpy's
// stream is not reproduced). Used to make training sets at sizes where the
// host generator dominates; one CTA per field, sides up to 128.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/darcy_gpu.h"
#include "engine.h"

namespace dgpu {
namespace {

constexpr int kMaxFieldSide = 128;
constexpr int kFieldThreads = 256;

struct U4 {
    uint32_t x, y, z, w;
};

// Philox-4x32 with 10 rounds: multipliers 0xD2511F53 / 0xCD9E8D57, key
// increments 0x9E3779B9 / 0xBB67AE85 (the published constants).
__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    }
    return c;
}

__device__ __forceinline__ float unit_open(uint32_t v) { return ((float)v + 0.5f) * 2.3283064365386963e-10f; }

__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
    const float r = sqrtf(-2.0f * logf(unit_open(a)));
    float s, c;
    sincospif(2.0f * unit_open(b), &s, &c);
    z0 = r * c;
    z1 = r * s;
}

__global__ void __launch_bounds__(kFieldThreads) k_random_fields(int n, int64_t count, int64_t f0, uint32_t k0,
                                                                 uint32_t k1,
                                                                 const float* __restrict__ amp,
                                                                 const float* __restrict__ C, double hi, double lo,
                                                                 int raw, double* __restrict__ out) {
    extern __shared__ float fsm[];
    float* sC = fsm;
    float* sX = fsm + n * n;
    float* sT = sX + n * n;
    const int m = n * n;
    for (int q = threadIdx.x; q < m; q += blockDim.x) sC[q] = C[q];
    for (int64_t f = blockIdx.x; f < count; f += gridDim.x) {
        // noise: four normals per Philox call, counter (group, field low, field
        // high, 0) with the field's index in the whole call (f0 + f)
        const uint64_t fid = (uint64_t)(f0 + f);
        for (int g = threadIdx.x; g < (m + 3) / 4; g += blockDim.x) {
            const U4 r = philox4x32_10(U4{(uint32_t)g, (uint32_t)fid, (uint32_t)(fid >> 32), 0u}, k0, k1);
            float z[4];
            box_muller(r.x, r.y, z[0], z[1]);
            box_muller(r.z, r.w, z[2], z[3]);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int q = 4 * g + e;
                if (q < m) sX[q] = amp[q] * z[e];
            }
        }
        __syncthreads();
        // T = C^T X
        for (int o = threadIdx.x; o < m; o += blockDim.x) {
            const int i = o / n, l = o - (o / n) * n;
            float acc = 0.f;
            for (int k = 0; k < n; ++k) acc += sC[k * n + i] * sX[k * n + l];
            sT[o] = acc;
        }
        __syncthreads();
        // x = T C, thresholded
        double* dst = out + f * (int64_t)m;
        for (int o = threadIdx.x; o < m; o += blockDim.x) {
            const int i = o / n, j = o - (o / n) * n;
            float acc = 0.f;
            for (int l = 0; l < n; ++l) acc += sT[i * n + l] * sC[l * n + j];
            dst[o] = raw ? (double)acc : (acc >= 0.f ? hi : lo);
        }
        __syncthreads();
    }
}

}  // namespace
}  // namespace dgpu

using namespace dgpu;

extern "C" int dgpu_random_fields(int64_t n, int64_t count, unsigned long long seed, double alpha, double tau,
                                  double hi, double lo, int raw, double* out, int out_on_device, void* stream) {
    char msg[256];
    if (n < 1 || n > kMaxFieldSide) {
        std::snprintf(msg, sizeof msg, "field side %lld outside 1..%d", (long long)n, kMaxFieldSide);
        set_last_error(msg);
        return DGPU_INVALID_INPUT;
    }
    if (count < 1 || !out) {
        set_last_error(count < 1 ? "need at least one field" : "buffers must not be NULL");
        return DGPU_INVALID_INPUT;
    }
    if (!raw && (!(hi > 0) || !(lo > 0))) {  // fields.py:72-83
        set_last_error("permeability phases must be strictly positive");
        return DGPU_INVALID_INPUT;
    }
    if (!std::isfinite(alpha) || !(tau > 0)) {
        set_last_error("alpha must be finite and tau positive");
        return DGPU_INVALID_INPUT;
    }
    const int N = (int)n, m = N * N;
    // amplitudes and the orthonormal DCT-II matrix, in FP64 on the host
    std::vector<float> amp(m), C(m);
    const double pi = 3.14159265358979323846;
    for (int kx = 0; kx < N; ++kx)
        for (int ky = 0; ky < N; ++ky) {
            const double spec = pi * pi * (double)(kx * kx + ky * ky) + tau * tau;
            amp[kx * N + ky] = (kx == 0 && ky == 0) ? 0.f : (float)(std::pow(tau, alpha - 1.0) * std::pow(spec, -alpha / 2.0));
        }
    for (int k = 0; k < N; ++k)
        for (int i = 0; i < N; ++i)
            C[k * N + i] = (float)(std::sqrt((k == 0 ? 1.0 : 2.0) / N) * std::cos(pi * k * (2 * i + 1) / (2.0 * N)));
    cudaStream_t s = (cudaStream_t)stream;
    float *d_amp = nullptr, *d_C = nullptr;
    double* d_out = nullptr;
    const int64_t chunk = out_on_device ? count : std::min<int64_t>(count, (int64_t)(256 << 20) / (8 * m));
    cudaError_t e = cudaMalloc(&d_amp, sizeof(float) * m);
    if (e == cudaSuccess) e = cudaMalloc(&d_C, sizeof(float) * m);
    if (e == cudaSuccess && !out_on_device) e = cudaMalloc(&d_out, sizeof(double) * m * chunk);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_amp, amp.data(), sizeof(float) * m, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_C, C.data(), sizeof(float) * m, cudaMemcpyHostToDevice, s);
    const size_t smem = sizeof(float) * 3 * (size_t)m;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_random_fields, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int sms = 0, dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int64_t at = 0; e == cudaSuccess && at < count; at += chunk) {
        const int64_t c = std::min(chunk, count - at);
        double* dst = out_on_device ? out + at * m : d_out;
        // counters carry the field's index in the whole call, so chunking does not change the fields
        k_random_fields<<<(unsigned)std::min<int64_t>(c, (int64_t)sms * 8), kFieldThreads, smem, s>>>(
            N, c, at, k0, k1, d_amp, d_C, hi, lo, raw, dst);
        e = cudaGetLastError();
        if (e == cudaSuccess && !out_on_device)
            e = cudaMemcpyAsync(out + at * m, d_out, sizeof(double) * m * c, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && !out_on_device) e = cudaStreamSynchronize(s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_amp);
    cudaFree(d_C);
    if (d_out) cudaFree(d_out);
    if (e != cudaSuccess) {
        std::snprintf(msg, sizeof msg, "CUDA error %s (%s) in dgpu_random_fields", cudaGetErrorName(e),
                      cudaGetErrorString(e));
        set_last_error(msg);
        return DGPU_CUDA_ERROR;
    }
    set_last_error("");
    return DGPU_OK;
}

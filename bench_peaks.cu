// bench_peaks.cu — device throughput probes used by bench.py as roofline
// denominators that no driver-side measurement provides: the FP32 FFMA rate
// (the bound of the kriging solve, which runs on the CUDA cores), the FP64
// DFMA rate (the bound of the plain FP64 path's solve), the FP32 rate of the
// solve's Gauss-Jordan update pattern at the solve's occupancy, and the rate
// at which kernels write page-locked host memory (the bound of the FP64
// output that sgs_plan_simulate writes straight into the caller's buffer).
// Measurement infrastructure beside the benchmark, built by bench.py as its
// own library (_build/libgeosgs_peaks.so); not part of the product or its
// C ABI.
#include <cuda_runtime.h>
#include <cstdint>

namespace {

// NR independent FFMA chains per thread; the result is stored so that the
// chains are not removed
template <int NR>
__global__ void ffma_chains_kernel(float* out, int iters, float a) {
    float r[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) r[j] = threadIdx.x * 1e-3f + j;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < NR; ++j) r[j] = __fmaf_rn(r[j], a, 0.5f);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < NR; ++j) s += r[j];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// NR independent DFMA chains per thread
template <int NR>
__global__ void dfma_chains_kernel(double* out, int iters, double a) {
    double r[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) r[j] = threadIdx.x * 1e-3 + j;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < NR; ++j) r[j] = __fma_rn(r[j], a, 0.5);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < NR; ++j) s += r[j];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// streaming 16-byte writes of n2 double2 values
__global__ void write_stream_kernel(double2* out, int64_t n2, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_double2(v, v + 1.0);
}

// The kriging solve's Gauss-Jordan update: per step every lane updates its
// two rows of 48 registers, each from the next register and a pivot-row
// coefficient read from shared memory (R[j] = R[j+1] - a * c[j]); the next
// step's factor depends on the update.  Two warps per block, as the solve.
constexpr int GJ_N = 48;
__global__ void gj_pattern_kernel(float* out, int steps) {
    __shared__ __align__(16) float cb[2 * 64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float* my = cb + w * 64;
    for (int i = lane; i < 64; i += 32) my[i] = 1e-3f * (i + 1);
    __syncwarp();
    float R0[GJ_N], R1[GJ_N];
#pragma unroll
    for (int j = 0; j < GJ_N; ++j) {
        R0[j] = lane * 1e-3f + j;
        R1[j] = lane * 2e-3f - j;
    }
    float a0 = 0.999f + lane * 1e-6f, a1 = 0.998f;
#pragma unroll 1
    for (int s = 0; s < steps; ++s) {
        const float4* c4 = reinterpret_cast<const float4*>(my);
#pragma unroll
        for (int j4 = 0; j4 < GJ_N / 4; ++j4) {
            const float4 v = c4[j4];
            const float c[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int j = 4 * j4 + t;
                if (j < GJ_N - 1) {
                    R0[j] = __fmaf_rn(-a0, c[t], R0[j + 1]);
                    R1[j] = __fmaf_rn(-a1, c[t], R1[j + 1]);
                }
            }
        }
        R0[GJ_N - 1] = a0;
        R1[GJ_N - 1] = a1;
        a0 = R0[0] * 1e-3f + 0.999f;
        a1 = R1[0] * 1e-3f + 0.998f;
    }
    float sum = 0.f;
#pragma unroll
    for (int j = 0; j < GJ_N; ++j) sum += R0[j] + R1[j];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

int sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

}  // namespace

// Best of three timed launches of 32 FFMA chains per thread, 8 blocks of 256
// threads per SM; *tflops = 2 x FFMA lanes per second / 1e12.  0 on success.
extern "C" int geosgs_peak_fp32(double* tflops) {
    const int nsm = sms();
    if (!tflops || nsm <= 0) return 1;
    const int blocks = nsm * 8, threads = 256, iters = 20000;
    float* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) return 2;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        ffma_chains_kernel<32><<<blocks, threads>>>(out, iters, 0.999f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || best <= 0.f) return 3;
    *tflops = 2.0 * (double)blocks * threads * iters * 32 / (best * 1e-3) / 1e12;
    return 0;
}

// Best of three timed launches of 16 DFMA chains per thread, 8 blocks of 256
// threads per SM; *tflops = 2 x DFMA lanes per second / 1e12.  0 on success.
extern "C" int geosgs_peak_fp64(double* tflops) {
    const int nsm = sms();
    if (!tflops || nsm <= 0) return 1;
    const int blocks = nsm * 8, threads = 256, iters = 1000;
    double* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return 2;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        dfma_chains_kernel<16><<<blocks, threads>>>(out, iters, 0.999);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || best <= 0.f) return 3;
    *tflops = 2.0 * (double)blocks * threads * iters * 16 / (best * 1e-3) / 1e12;
    return 0;
}

// Best of three timed kernels writing `bytes` (rounded down to 16) into
// page-locked host memory through its device address; *gbs = bytes / s / 1e9.
extern "C" int geosgs_peak_host_write(int64_t bytes, double* gbs) {
    const int nsm = sms();
    if (!gbs || nsm <= 0 || bytes < 16) return 1;
    const int64_t n2 = bytes / 16;
    void* h = nullptr;
    if (cudaHostAlloc(&h, (size_t)n2 * 16, cudaHostAllocMapped) != cudaSuccess) return 2;
    void* hd = nullptr;
    if (cudaHostGetDevicePointer(&hd, h, 0) != cudaSuccess) {
        cudaFreeHost(h);
        return 2;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        write_stream_kernel<<<nsm * 8, 256>>>(static_cast<double2*>(hd), n2, 1.0);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeHost(h);
    if (err != cudaSuccess || best <= 0.f) return 3;
    *gbs = (double)n2 * 16 / (best * 1e-3) / 1e9;
    return 0;
}

// Best of three device-to-page-locked-host copies (cudaMemcpyAsync, the
// copy engines) of `bytes`; *gbs = bytes / s / 1e9.  0 on success.
extern "C" int geosgs_peak_d2h_copy(int64_t bytes, double* gbs) {
    if (!gbs || bytes < 16) return 1;
    void* h = nullptr;
    void* d = nullptr;
    if (cudaHostAlloc(&h, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) return 2;
    if (cudaMalloc(&d, (size_t)bytes) != cudaSuccess) {
        cudaFreeHost(h);
        return 2;
    }
    cudaMemset(d, 1, (size_t)bytes);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        cudaMemcpyAsync(h, d, (size_t)bytes, cudaMemcpyDeviceToHost, 0);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    cudaFreeHost(h);
    if (err != cudaSuccess || best <= 0.f) return 3;
    *gbs = (double)bytes / (best * 1e-3) / 1e9;
    return 0;
}

// FP32 rate of the Gauss-Jordan update pattern with 10 resident warps per SM
// (the solve's occupancy): *tflops = 2 x FFMA lanes per second / 1e12.
extern "C" int geosgs_peak_gj_pattern(double* tflops) {
    const int nsm = sms();
    if (!tflops || nsm <= 0) return 1;
    const int blocks = nsm * 5, threads = 64, steps = 4000;
    float* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) return 2;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        gj_pattern_kernel<<<blocks, threads>>>(out, steps);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || best <= 0.f) return 3;
    *tflops = 2.0 * (double)blocks * threads * steps * (GJ_N - 1) * 2 / (best * 1e-3) / 1e12;
    return 0;
}

// sweep.cu — kernel (c): the level-scheduled value sweep over all
// realizations, and the layout conversions around it.
//
// Replaces the draw of randsingle's loop, v = mu_hat + sigma_hat * z
// (src/simulation/field/seqsim.jl:132,335-340, prior :109-111), for every
// realization at once.  Values are centred (v - mu) and node-major,
// V[node][Rp] with realizations contiguous, so one node's update reads each
// grid neighbour's row of realizations with coalesced vector loads:
//   V[g][r] = b0 + sum_j w_j V[nb_j][r] + sigma * z[g][r]
// All nodes of one dependency level are independent; levels run in order.
// The data's fixed values enter through b0 (computed by the solve).
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace sgs {

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
    __device__ static float4 load(const float* p) { return *reinterpret_cast<const float4*>(p); }
    __device__ static void store(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
};

struct D4 {
    double x, y, z, w;
};
__device__ __forceinline__ D4 load_d4(const double* p) {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    return {a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void store_d4(double* p, D4 v) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v.x, v.y);
    reinterpret_cast<double2*>(p)[1] = make_double2(v.z, v.w);
}

// Compensated dot product in FP32 (Dot2: Ogita, Rump & Oishi 2005, "Accurate
// sum and dot product"): the product w*x is split exactly into p + pe with an
// FMA, p is added to the running sum s with TwoSum (Knuth), and every
// rounding error, plus the low part of the weight, goes into the correction
// c.  s + c carries the dot product to about twice FP32 precision; only the
// final rounding to the stored FP32 value remains.
struct Dot2 {
    float s, c;
    __device__ __forceinline__ void init(float hi, float lo) {
        s = hi;
        c = lo;
    }
    __device__ __forceinline__ void add(float wh, float wl, float x) {
        const float p = __fmul_rn(wh, x);
        const float pe = __fmaf_rn(wh, x, -p);
        const float t = __fadd_rn(s, p);
        const float bp = __fsub_rn(t, s);
        const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
        s = t;
        c = __fadd_rn(c, __fadd_rn(e, __fmaf_rn(wl, x, pe)));
    }
    __device__ __forceinline__ float value() const { return __fadd_rn(s, c); }
};

// Update one node's chunk of 4 realizations (FP32 values, compensated sum).
__device__ __forceinline__ void sweep_item_fp32(const SweepTables<float>& t, int k, int64_t pos, int ch, int Rp,
                                                const float* __restrict__ z, uint64_t seed, float* __restrict__ V) {
    const int g = t.node[pos];
    const int m = t.m[pos];
    const float2 b0 = reinterpret_cast<const float2*>(t.b0)[pos];
    Dot2 a0, a1, a2, a3;
    a0.init(b0.x, b0.y);
    a1.init(b0.x, b0.y);
    a2.init(b0.x, b0.y);
    a3.init(b0.x, b0.y);
    const int32_t* idx = t.idx + pos * k;
    const float2* w = reinterpret_cast<const float2*>(t.w) + pos * k;
#pragma unroll 4
    for (int j = 0; j < m; ++j) {
        const float4 v = Vec4<float>::load(V + (int64_t)idx[j] * Rp + 4 * ch);
        const float2 wj = w[j];
        a0.add(wj.x, wj.y, v.x);
        a1.add(wj.x, wj.y, v.y);
        a2.add(wj.x, wj.y, v.z);
        a3.add(wj.x, wj.y, v.w);
    }
    const float4 zz = z ? Vec4<float>::load(z + (int64_t)g * Rp + 4 * ch) : normals4(seed, g, ch);
    const float2 sg = reinterpret_cast<const float2*>(t.sigma)[pos];
    a0.add(sg.x, sg.y, zz.x);
    a1.add(sg.x, sg.y, zz.y);
    a2.add(sg.x, sg.y, zz.z);
    a3.add(sg.x, sg.y, zz.w);
    Vec4<float>::store(V + (int64_t)g * Rp + 4 * ch, make_float4(a0.value(), a1.value(), a2.value(), a3.value()));
}

// Update one node's chunk of 4 realizations (FP64 values).
__device__ __forceinline__ void sweep_item_fp64(const SweepTables<double>& t, int k, int64_t pos, int ch, int Rp,
                                                const double* __restrict__ z, uint64_t seed, double* __restrict__ V) {
    const int g = t.node[pos];
    const int m = t.m[pos];
    const double b0 = t.b0[pos];
    D4 acc = {b0, b0, b0, b0};
    const int32_t* idx = t.idx + pos * k;
    const double* w = t.w + pos * k;
#pragma unroll 4
    for (int j = 0; j < m; ++j) {
        const D4 v = load_d4(V + (int64_t)idx[j] * Rp + 4 * ch);
        const double wj = w[j];
        acc.x = fma(wj, v.x, acc.x);
        acc.y = fma(wj, v.y, acc.y);
        acc.z = fma(wj, v.z, acc.z);
        acc.w = fma(wj, v.w, acc.w);
    }
    D4 zz;
    if (z) {
        zz = load_d4(z + (int64_t)g * Rp + 4 * ch);
    } else {
        const float4 f = normals4(seed, g, ch);
        zz = {(double)f.x, (double)f.y, (double)f.z, (double)f.w};
    }
    const double s = t.sigma[pos];
    acc.x = fma(s, zz.x, acc.x);
    acc.y = fma(s, zz.y, acc.y);
    acc.z = fma(s, zz.z, acc.z);
    acc.w = fma(s, zz.w, acc.w);
    store_d4(V + (int64_t)g * Rp + 4 * ch, acc);
}

// One level per launch: one thread per (node, chunk of 4 realizations).
template <typename T>
__global__ void __launch_bounds__(256) sweep_level_kernel(const SweepTables<T> t, int k, int64_t p0, int64_t p1, int Rp,
                                                          const T* __restrict__ z, uint64_t seed, T* __restrict__ V) {
    const int cpn = Rp >> 2;
    const int64_t total = (p1 - p0) * cpn;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        if constexpr (sizeof(T) == 4) sweep_item_fp32(t, k, p0 + i / cpn, (int)(i % cpn), Rp, z, seed, V);
        else sweep_item_fp64(t, k, p0 + i / cpn, (int)(i % cpn), Rp, z, seed, V);
    }
}

// All levels in one cooperative launch: the grid walks level after level and
// synchronizes between them (cooperative_groups grid barrier; every block of
// a cooperative launch is resident, so the barrier always completes).  This
// removes the per-level launch gaps that dominate sweeps with many small
// levels.
template <typename T>
__global__ void __launch_bounds__(256) sweep_all_kernel(const SweepTables<T> t, int k, const int32_t* __restrict__ loff,
                                                        int nlevels, int Rp, const T* __restrict__ z, uint64_t seed,
                                                        T* __restrict__ V) {
    cg::grid_group grid = cg::this_grid();
    const int cpn = Rp >> 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int l = 0; l < nlevels; ++l) {
        const int64_t p0 = loff[l], p1 = loff[l + 1];
        const int64_t total = (p1 - p0) * cpn;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
            if constexpr (sizeof(T) == 4) sweep_item_fp32(t, k, p0 + i / cpn, (int)(i % cpn), Rp, z, seed, V);
            else sweep_item_fp64(t, k, p0 + i / cpn, (int)(i % cpn), Rp, z, seed, V);
        }
        grid.sync();
    }
}

// One warp per node for rows of at most 32 chunks (R <= 128): lane = s * cpn +
// ch, where ch is the realization chunk and s one of S = 32 / cpn slices of
// the neighbour list.  Each lane accumulates every S-th neighbour, so the
// chain of dependent loads per lane is S times shorter than one thread per
// chunk walking all neighbours (the small levels are latency-bound); the S
// partial sums are then combined across lanes (error-free for the
// compensated FP32 sums).
__device__ __forceinline__ void dot2_merge(Dot2& a, float s2, float c2) {
    const DF t = df_two_sum(a.s, s2);
    a.s = t.hi;
    a.c = __fadd_rn(a.c, __fadd_rn(c2, t.lo));
}

template <typename T>
__global__ void __launch_bounds__(256) sweep_warp_kernel(const SweepTables<T> t, int k, int64_t p0, int64_t p1, int Rp,
                                                         int cpn, const T* __restrict__ z, uint64_t seed,
                                                         T* __restrict__ V) {
    const int lane = threadIdx.x & 31;
    const int ch = lane % cpn, s = lane / cpn, S = 32 / cpn;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t pos = p0 + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); pos < p1; pos += nw) {
        const int g = t.node[pos];
        const int m = t.m[pos];
        const int32_t* idx = t.idx + pos * k;
        if constexpr (sizeof(T) == 4) {
            Dot2 a0, a1, a2, a3;
            a0.init(0.f, 0.f);
            a1.init(0.f, 0.f);
            a2.init(0.f, 0.f);
            a3.init(0.f, 0.f);
            const float2* w = reinterpret_cast<const float2*>(t.w) + pos * k;
            for (int j = s; j < m; j += S) {
                const float4 v = Vec4<float>::load(V + (int64_t)idx[j] * Rp + 4 * ch);
                const float2 wj = w[j];
                a0.add(wj.x, wj.y, v.x);
                a1.add(wj.x, wj.y, v.y);
                a2.add(wj.x, wj.y, v.z);
                a3.add(wj.x, wj.y, v.w);
            }
            for (int o = cpn; o < 32; o <<= 1) {
                dot2_merge(a0, __shfl_xor_sync(FULL_MASK, a0.s, o), __shfl_xor_sync(FULL_MASK, a0.c, o));
                dot2_merge(a1, __shfl_xor_sync(FULL_MASK, a1.s, o), __shfl_xor_sync(FULL_MASK, a1.c, o));
                dot2_merge(a2, __shfl_xor_sync(FULL_MASK, a2.s, o), __shfl_xor_sync(FULL_MASK, a2.c, o));
                dot2_merge(a3, __shfl_xor_sync(FULL_MASK, a3.s, o), __shfl_xor_sync(FULL_MASK, a3.c, o));
            }
            if (s == 0) {
                const float2 b0 = reinterpret_cast<const float2*>(t.b0)[pos];
                dot2_merge(a0, b0.x, b0.y);
                dot2_merge(a1, b0.x, b0.y);
                dot2_merge(a2, b0.x, b0.y);
                dot2_merge(a3, b0.x, b0.y);
                const float4 zz = z ? Vec4<float>::load(z + (int64_t)g * Rp + 4 * ch) : normals4(seed, g, ch);
                const float2 sg = reinterpret_cast<const float2*>(t.sigma)[pos];
                a0.add(sg.x, sg.y, zz.x);
                a1.add(sg.x, sg.y, zz.y);
                a2.add(sg.x, sg.y, zz.z);
                a3.add(sg.x, sg.y, zz.w);
                Vec4<float>::store(V + (int64_t)g * Rp + 4 * ch,
                                   make_float4(a0.value(), a1.value(), a2.value(), a3.value()));
            }
        } else {
            D4 acc = {0.0, 0.0, 0.0, 0.0};
            const double* w = t.w + pos * k;
            for (int j = s; j < m; j += S) {
                const D4 v = load_d4(V + (int64_t)idx[j] * Rp + 4 * ch);
                const double wj = w[j];
                acc.x = fma(wj, v.x, acc.x);
                acc.y = fma(wj, v.y, acc.y);
                acc.z = fma(wj, v.z, acc.z);
                acc.w = fma(wj, v.w, acc.w);
            }
            for (int o = cpn; o < 32; o <<= 1) {
                acc.x += __shfl_xor_sync(FULL_MASK, acc.x, o);
                acc.y += __shfl_xor_sync(FULL_MASK, acc.y, o);
                acc.z += __shfl_xor_sync(FULL_MASK, acc.z, o);
                acc.w += __shfl_xor_sync(FULL_MASK, acc.w, o);
            }
            if (s == 0) {
                const double b0 = t.b0[pos];
                D4 zz;
                if (z) {
                    zz = load_d4(z + (int64_t)g * Rp + 4 * ch);
                } else {
                    const float4 f = normals4(seed, g, ch);
                    zz = {(double)f.x, (double)f.y, (double)f.z, (double)f.w};
                }
                const double sg = t.sigma[pos];
                acc.x = fma(sg, zz.x, acc.x + b0);
                acc.y = fma(sg, zz.y, acc.y + b0);
                acc.z = fma(sg, zz.z, acc.z + b0);
                acc.w = fma(sg, zz.w, acc.w + b0);
                store_d4(V + (int64_t)g * Rp + 4 * ch, acc);
            }
        }
    }
}

static int sweep_blocks(int64_t total) {
    int64_t b = (total + 255) / 256;
    if (b > (1 << 20)) b = 1 << 20;
    return (int)(b < 1 ? 1 : b);
}

// warp-per-node variant when a row has a power-of-two number of chunks <= 16
static bool use_warp_sweep(int Rp) {
    const int cpn = Rp / 4;
    return cpn <= 16 && (cpn & (cpn - 1)) == 0;
}

template <typename T>
static cudaError_t sweep_level(const SweepTables<T>& t, int k, int64_t p0, int64_t p1, int Rp, const T* z,
                               uint64_t seed, T* V, cudaStream_t s) {
    if (p1 <= p0) return cudaSuccess;
    if (use_warp_sweep(Rp)) {
        const int64_t nodes = p1 - p0;
        int64_t blocks = (nodes + 7) / 8;
        if (blocks > (1 << 20)) blocks = 1 << 20;
        sweep_warp_kernel<T><<<(int)blocks, 256, 0, s>>>(t, k, p0, p1, Rp, Rp / 4, z, seed, V);
    } else {
        sweep_level_kernel<T><<<sweep_blocks((p1 - p0) * (Rp / 4)), 256, 0, s>>>(t, k, p0, p1, Rp, z, seed, V);
    }
    return cudaGetLastError();
}

cudaError_t launch_sweep_fp32(const SweepTables<float>& t, int k, int64_t p0, int64_t p1, int Rp, const float* z,
                              uint64_t seed, float* V, cudaStream_t s) {
    return sweep_level<float>(t, k, p0, p1, Rp, z, seed, V, s);
}

cudaError_t launch_sweep_fp64(const SweepTables<double>& t, int k, int64_t p0, int64_t p1, int Rp, const double* z,
                              uint64_t seed, double* V, cudaStream_t s) {
    return sweep_level<double>(t, k, p0, p1, Rp, z, seed, V, s);
}

template <typename T>
static cudaError_t sweep_all(const SweepTables<T>& t, int k, const int32_t* loff, int nlevels, int Rp, const T* z,
                             uint64_t seed, T* V, cudaStream_t s) {
    int dev = 0, nsm = 0, coop = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return cudaErrorNotSupported;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_all_kernel<T>, 256, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorNotSupported;
    dim3 grid(nsm * per_sm), block(256);
    void* args[] = {(void*)&t, (void*)&k, (void*)&loff, (void*)&nlevels, (void*)&Rp, (void*)&z, (void*)&seed, (void*)&V};
    return cudaLaunchCooperativeKernel((const void*)sweep_all_kernel<T>, grid, block, args, 0, s);
}

cudaError_t launch_sweep_all_fp32(const SweepTables<float>& t, int k, const int32_t* loff, int nlevels, int Rp,
                                  const float* z, uint64_t seed, float* V, cudaStream_t s) {
    return sweep_all<float>(t, k, loff, nlevels, Rp, z, seed, V, s);
}

cudaError_t launch_sweep_all_fp64(const SweepTables<double>& t, int k, const int32_t* loff, int nlevels, int Rp,
                                  const double* z, uint64_t seed, double* V, cudaStream_t s) {
    return sweep_all<double>(t, k, loff, nlevels, Rp, z, seed, V, s);
}

// ---------------------------------------------------------------------------
// Tiled transposes between the caller's realization-major [R][N] double
// arrays and the node-major [N][Rp] rows (32x32 tiles through shared memory).
template <typename T>
__global__ void z_to_rows_kernel(const double* __restrict__ zin, int64_t N, int R, int Rp, T* __restrict__ z) {
    __shared__ double tile[32][33];
    const int64_t g0 = (int64_t)blockIdx.x * 32;
    const int r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int r = r0 + j;
        const int64_t g = g0 + threadIdx.x;
        tile[j][threadIdx.x] = (r < R && g < N) ? zin[(int64_t)r * N + g] : 0.0;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int64_t g = g0 + j;
        const int r = r0 + threadIdx.x;
        if (g < N && r < Rp) z[g * Rp + r] = (T)tile[threadIdx.x][j];
    }
}

template <typename T>
__global__ void rows_to_out_kernel(const T* __restrict__ V, int64_t N, int R, int Rp, double mu,
                                   double* __restrict__ out) {
    __shared__ double tile[32][33];
    const int64_t g0 = (int64_t)blockIdx.x * 32;
    const int r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int64_t g = g0 + j;
        const int r = r0 + threadIdx.x;
        tile[j][threadIdx.x] = (g < N && r < R) ? (double)V[g * Rp + r] : 0.0;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int r = r0 + j;
        const int64_t g = g0 + threadIdx.x;
        if (r < R && g < N) out[(int64_t)r * N + g] = tile[threadIdx.x][j] + mu;
    }
}

template <typename T>
static cudaError_t z_rows(const double* zin, int64_t N, int R, int Rp, T* z, cudaStream_t s) {
    dim3 grid((unsigned)((N + 31) / 32), (unsigned)((Rp + 31) / 32));
    z_to_rows_kernel<T><<<grid, dim3(32, 8), 0, s>>>(zin, N, R, Rp, z);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t rows_out(const T* V, int64_t N, int R, int Rp, double mu, double* out, cudaStream_t s) {
    dim3 grid((unsigned)((N + 31) / 32), (unsigned)((R + 31) / 32));
    rows_to_out_kernel<T><<<grid, dim3(32, 8), 0, s>>>(V, N, R, Rp, mu, out);
    return cudaGetLastError();
}

cudaError_t launch_z_to_rows_fp32(const double* zin, int64_t N, int R, int Rp, float* z, cudaStream_t s) {
    return z_rows<float>(zin, N, R, Rp, z, s);
}
cudaError_t launch_z_to_rows_fp64(const double* zin, int64_t N, int R, int Rp, double* z, cudaStream_t s) {
    return z_rows<double>(zin, N, R, Rp, z, s);
}
cudaError_t launch_rows_to_out_fp32(const float* V, int64_t N, int R, int Rp, double mu, double* out, cudaStream_t s) {
    return rows_out<float>(V, N, R, Rp, mu, out, s);
}
cudaError_t launch_rows_to_out_fp64(const double* V, int64_t N, int R, int Rp, double mu, double* out, cudaStream_t s) {
    return rows_out<double>(V, N, R, Rp, mu, out, s);
}

}  // namespace sgs

// sweep.cu — kernel (c): the level-scheduled value sweep over all
// realizations, and the layout conversions around it.
//
// Replaces the draw of randsingle's loop, v = mu_hat + sigma_hat * z
// (src/simulation/field/seqsim.jl:132,335-340, prior :109-111), for every
// realization at once.  Values are centred (v - mu) and node-major,
// V[node][Rp] with realizations contiguous, so one node's update reads each
// grid neighbour's row of realizations with coalesced vector loads:
//   V[g][r] = b0 + sum_j w_j V[nb_j][r] + sigma * z[g][r]
// All nodes of one dependency level are independent.  The default sweep is
// one persistent dataflow launch (sweep_flow_kernel) in which each node waits
// only for its own neighbours; per-level launches and a cooperative launch
// with grid barriers between levels are the alternatives.  The data's fixed
// values enter through b0 (computed by the solve).
#include <algorithm>

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

// Adds another compensated sum (s2, c2) to a (TwoSum of the leading parts).
__device__ __forceinline__ void dot2_merge(Dot2& a, float s2, float c2) {
    const DF t = df_two_sum(a.s, s2);
    a.s = t.hi;
    a.c = __fadd_rn(a.c, __fadd_rn(c2, t.lo));
}

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

// CH consecutive chunks of 4 realizations (ch .. ch + CH - 1 < cpn) of one
// node, FP32: CH independent row loads per neighbour in flight per thread.
template <int CH>
__device__ __forceinline__ void sweep_itemN_fp32(const SweepTables<float>& t, int k, int64_t pos, int ch, int Rp,
                                                 const float* __restrict__ z, uint64_t seed, float* __restrict__ V) {
    const int g = t.node[pos];
    const int m = t.m[pos];
    const float2 b0 = reinterpret_cast<const float2*>(t.b0)[pos];
    Dot2 a[4 * CH];
#pragma unroll
    for (int q = 0; q < 4 * CH; ++q) a[q].init(b0.x, b0.y);
    const int32_t* idx = t.idx + pos * k;
    const float2* w = reinterpret_cast<const float2*>(t.w) + pos * k;
#pragma unroll 4
    for (int j = 0; j < m; ++j) {
        const float* row = V + (int64_t)idx[j] * Rp + 4 * ch;
        float4 v[CH];
#pragma unroll
        for (int h = 0; h < CH; ++h) v[h] = Vec4<float>::load(row + 4 * h);
        const float2 wj = w[j];
#pragma unroll
        for (int h = 0; h < CH; ++h) {
            a[4 * h + 0].add(wj.x, wj.y, v[h].x);
            a[4 * h + 1].add(wj.x, wj.y, v[h].y);
            a[4 * h + 2].add(wj.x, wj.y, v[h].z);
            a[4 * h + 3].add(wj.x, wj.y, v[h].w);
        }
    }
    const float2 sg = reinterpret_cast<const float2*>(t.sigma)[pos];
#pragma unroll
    for (int h = 0; h < CH; ++h) {
        const float4 zz = z ? Vec4<float>::load(z + (int64_t)g * Rp + 4 * (ch + h)) : normals4(seed, g, ch + h);
        a[4 * h + 0].add(sg.x, sg.y, zz.x);
        a[4 * h + 1].add(sg.x, sg.y, zz.y);
        a[4 * h + 2].add(sg.x, sg.y, zz.z);
        a[4 * h + 3].add(sg.x, sg.y, zz.w);
        Vec4<float>::store(V + (int64_t)g * Rp + 4 * (ch + h),
                           make_float4(a[4 * h].value(), a[4 * h + 1].value(), a[4 * h + 2].value(), a[4 * h + 3].value()));
    }
}

// One level per launch, FP32, rows of a multiple of CH chunks: one thread
// per (node, CH consecutive chunks).
template <int CH>
__global__ void __launch_bounds__(256) sweep_levelN_kernel(const SweepTables<float> t, int k, int64_t p0, int64_t p1,
                                                           int Rp, const float* __restrict__ z, uint64_t seed,
                                                           float* __restrict__ V) {
    const int cpg = Rp / (4 * CH);  // chunk groups per node
    const int64_t total = (p1 - p0) * cpg;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x)
        sweep_itemN_fp32<CH>(t, k, p0 + i / cpg, CH * (int)(i % cpg), Rp, z, seed, V);
}

// One level per launch for levels of few nodes (FP32, rows of a multiple of
// 8 realizations): one block per node, its SPLIT_WARPS warps splitting the
// node's neighbour list (warp s takes every SPLIT_WARPS-th neighbour from
// s), each lane 2 chunks of 4 realizations (64 chunks per pass over the
// row), so each thread's chain of dependent row loads is SPLIT_WARPS times
// shorter; warp 0 merges the warps' compensated partial sums (error-free
// TwoSum merges) from shared memory, adds b0 and sigma z and stores.
constexpr int SPLIT_WARPS = 8;

__global__ void __launch_bounds__(SPLIT_WARPS * 32) sweep_split_kernel(const SweepTables<float> t, int k, int64_t p0,
                                                                       int64_t p1, int Rp, const float* __restrict__ z,
                                                                       uint64_t seed, float* __restrict__ V) {
    __shared__ float2 part[SPLIT_WARPS - 1][8][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int cpn = Rp >> 2;
    for (int64_t pos = p0 + blockIdx.x; pos < p1; pos += gridDim.x) {
        const int g = t.node[pos];
        const int m = t.m[pos];
        const int32_t* idx = t.idx + pos * k;
        const float2* w = reinterpret_cast<const float2*>(t.w) + pos * k;
        for (int c0 = 0; c0 < cpn; c0 += 64) {
            const int ch = c0 + 2 * lane;  // chunks ch and ch + 1 (cpn is even)
            const bool act = ch < cpn;
            Dot2 a[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) a[q].init(0.f, 0.f);
            if (act) {
#pragma unroll 2
                for (int j = wid; j < m; j += SPLIT_WARPS) {
                    const float* row = V + (int64_t)idx[j] * Rp + 4 * ch;
                    const float4 v0 = Vec4<float>::load(row);
                    const float4 v1 = Vec4<float>::load(row + 4);
                    const float2 wj = w[j];
                    a[0].add(wj.x, wj.y, v0.x);
                    a[1].add(wj.x, wj.y, v0.y);
                    a[2].add(wj.x, wj.y, v0.z);
                    a[3].add(wj.x, wj.y, v0.w);
                    a[4].add(wj.x, wj.y, v1.x);
                    a[5].add(wj.x, wj.y, v1.y);
                    a[6].add(wj.x, wj.y, v1.z);
                    a[7].add(wj.x, wj.y, v1.w);
                }
            }
            if (wid > 0)
#pragma unroll
                for (int q = 0; q < 8; ++q) part[wid - 1][q][lane] = make_float2(a[q].s, a[q].c);
            __syncthreads();
            if (wid == 0 && act) {
#pragma unroll 1
                for (int s = 0; s < SPLIT_WARPS - 1; ++s)
#pragma unroll
                    for (int q = 0; q < 8; ++q) dot2_merge(a[q], part[s][q][lane].x, part[s][q][lane].y);
                const float2 b0 = reinterpret_cast<const float2*>(t.b0)[pos];
                const float2 sg = reinterpret_cast<const float2*>(t.sigma)[pos];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float4 zz =
                        z ? Vec4<float>::load(z + (int64_t)g * Rp + 4 * (ch + h)) : normals4(seed, g, ch + h);
#pragma unroll
                    for (int q = 0; q < 4; ++q) dot2_merge(a[4 * h + q], b0.x, b0.y);
                    a[4 * h + 0].add(sg.x, sg.y, zz.x);
                    a[4 * h + 1].add(sg.x, sg.y, zz.y);
                    a[4 * h + 2].add(sg.x, sg.y, zz.z);
                    a[4 * h + 3].add(sg.x, sg.y, zz.w);
                    Vec4<float>::store(V + (int64_t)g * Rp + 4 * (ch + h),
                                       make_float4(a[4 * h].value(), a[4 * h + 1].value(), a[4 * h + 2].value(),
                                                   a[4 * h + 3].value()));
                }
            }
            __syncthreads();
        }
    }
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
                              uint64_t seed, float* V, cudaStream_t s, int pairs, int split) {
    // pairs: chunks of 4 realizations per thread (1, 2 or 4); split: one
    // block per node with the neighbour list split over its warps
    if (split && Rp % 8 == 0) {
        if (p1 <= p0) return cudaSuccess;
        const int64_t nodes = p1 - p0;
        sweep_split_kernel<<<(unsigned)std::min<int64_t>(nodes, 1 << 20), SPLIT_WARPS * 32, 0, s>>>(t, k, p0, p1, Rp,
                                                                                                   z, seed, V);
        return cudaGetLastError();
    }
    if ((pairs == 2 || pairs == 4) && Rp % (4 * pairs) == 0 && !use_warp_sweep(Rp)) {
        if (p1 <= p0) return cudaSuccess;
        if (pairs == 2)
            sweep_levelN_kernel<2><<<sweep_blocks((p1 - p0) * (Rp / 8)), 256, 0, s>>>(t, k, p0, p1, Rp, z, seed, V);
        else
            sweep_levelN_kernel<4><<<sweep_blocks((p1 - p0) * (Rp / 16)), 256, 0, s>>>(t, k, p0, p1, Rp, z, seed, V);
        return cudaGetLastError();
    }
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
// Dataflow sweep: the dependency levels in one persistent launch, with no
// barrier between levels.  Realizations are independent, so a node's row is
// cut into H pieces of P4 chunks of 4 realizations, and every (node, piece)
// is a work item with its own flag: piece q of a node waits only for piece q
// of its grid neighbours.  Items are numbered position-major (item = pos * H
// + q, positions in level order) and warps take `chunk` consecutive items per
// ticket.  A dependency always has a smaller item number (strictly lower
// level, same piece), and item numbers are taken in increasing order by
// warps that are running, so every wait ends: the smallest unfinished item
// can always proceed.  Waits are bounded anyway (wait_ns of wall-clock time);
// a warp that gives up sets err, skips the update but still raises its flag,
// and no warp takes new tickets once err is set.
//
// Memory ordering: the item's lanes store the piece, each fences (gpu
// scope), the warp synchronizes, lane 0 stores the flag; a reader's lanes
// load flags with acquire semantics, synchronize, then read rows with L2-only
// loads (ld.global.cg), so no stale L1 line of a row written by another SM is
// used.
//
// Lane layout inside a warp: W lanes per slice of the neighbour list (a
// power of two), S = 32 / W slices, each lane G chunks of the piece
// (P4 = W * G); the S partial sums are combined across lanes at the end.
__device__ __forceinline__ int ld_flag_acquire(const int32_t* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_flag(int32_t* p, int v) {
    asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait until piece q of every grid neighbour is stored in this sweep (flags
// of piece q: done_q); false when a wait gave up.  A legitimate wait can last
// as long as the longest dependency chain, so the bound is wall-clock time.
// The flag that ends a wait is read with acquire semantics, and the warp
// barrier orders it before every lane's reads of the neighbours' rows.
__device__ __forceinline__ bool flow_wait(const int32_t* __restrict__ idx, int m, const int32_t* done_q,
                                          const FlowArgs& f, int lane) {
    bool ok = true;
    // bounded by elapsed time and, should the timer stall, by a count of
    // polls (each takes at least the 64 ns back-off, so the count bound is
    // reached no earlier than the time bound)
    const uint64_t max_polls = f.wait_ns / 32 + 1024;
    for (int j = lane; j < m; j += 32) {
        const int32_t* flag = done_q + idx[j];
        uint64_t t0 = 0, polls = 0;
        while (ld_flag_acquire(flag) != f.epoch) {
            const uint64_t now = global_ns();
            if (t0 == 0) t0 = now;
            if (now - t0 > f.wait_ns || ++polls > max_polls) {
                ok = false;
                break;
            }
            __nanosleep(64);
        }
    }
    ok = __all_sync(FULL_MASK, ok);
    __syncwarp();
    return ok;
}

// One piece (chunks [c0, c0 + W*G) of the row, clipped to the row) of one
// node, FP32 values with compensated sums.
template <int G, bool CSR>
__device__ __forceinline__ void flow_piece_fp32(const SweepTables<float>& t, int k, int64_t pos, int g, int m, int Rp,
                                                int64_t Rs, int c0, int W, int lane, const float* __restrict__ z,
                                                uint64_t seed, float* __restrict__ V) {
    const int cpn = Rp >> 2;
    const int S = 32 / W, s = lane / W, cl = lane % W;
    const int64_t row = CSR ? t.off[pos] : pos * (int64_t)k;
    const int32_t* idx = t.idx + row;
    const float2* w = reinterpret_cast<const float2*>(t.w) + row;
    Dot2 a[G][4];
#pragma unroll
    for (int gi = 0; gi < G; ++gi)
#pragma unroll
        for (int q = 0; q < 4; ++q) a[gi][q].init(0.f, 0.f);
#pragma unroll 4
    for (int j = s; j < m; j += S) {
        const float4* row = reinterpret_cast<const float4*>(V + (int64_t)idx[j] * Rs);
        const float2 wj = w[j];
#pragma unroll
        for (int gi = 0; gi < G; ++gi) {
            const int ch = c0 + cl + gi * W;
            if (ch < cpn) {
                const float4 v = __ldcg(row + ch);
                a[gi][0].add(wj.x, wj.y, v.x);
                a[gi][1].add(wj.x, wj.y, v.y);
                a[gi][2].add(wj.x, wj.y, v.z);
                a[gi][3].add(wj.x, wj.y, v.w);
            }
        }
    }
    for (int o = W; o < 32; o <<= 1)
#pragma unroll
        for (int gi = 0; gi < G; ++gi)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                dot2_merge(a[gi][q], __shfl_xor_sync(FULL_MASK, a[gi][q].s, o),
                           __shfl_xor_sync(FULL_MASK, a[gi][q].c, o));
    if (s == 0) {
        const float2 b0 = reinterpret_cast<const float2*>(t.b0)[pos];
        const float2 sg = reinterpret_cast<const float2*>(t.sigma)[pos];
#pragma unroll
        for (int gi = 0; gi < G; ++gi) {
            const int ch = c0 + cl + gi * W;
            if (ch < cpn) {
                const float4 zz =
                    z ? *reinterpret_cast<const float4*>(z + (int64_t)g * Rs + 4 * ch) : normals4(seed, g, ch);
#pragma unroll
                for (int q = 0; q < 4; ++q) dot2_merge(a[gi][q], b0.x, b0.y);
                a[gi][0].add(sg.x, sg.y, zz.x);
                a[gi][1].add(sg.x, sg.y, zz.y);
                a[gi][2].add(sg.x, sg.y, zz.z);
                a[gi][3].add(sg.x, sg.y, zz.w);
                Vec4<float>::store(V + (int64_t)g * Rs + 4 * ch, make_float4(a[gi][0].value(), a[gi][1].value(),
                                                                             a[gi][2].value(), a[gi][3].value()));
            }
        }
    }
}

// The same for FP64 values (plain FMA sums).
template <int G, bool CSR>
__device__ __forceinline__ void flow_piece_fp64(const SweepTables<double>& t, int k, int64_t pos, int g, int m, int Rp,
                                                int64_t Rs, int c0, int W, int lane, const double* __restrict__ z,
                                                uint64_t seed, double* __restrict__ V, int pairs) {
    const int cpn = Rp >> 2;
    const int S = 32 / W, s = lane / W, cl = lane % W;
    const int64_t row = CSR ? t.off[pos] : pos * (int64_t)k;
    const int32_t* idx = t.idx + row;
    const double* w = t.w + row;
    // pairs: each 8-byte table entry holds an FP32 (hi, lo) pair
    auto entry = [pairs](const double* p, int64_t i) {
        if (pairs) {
            const float2 v = reinterpret_cast<const float2*>(p)[i];
            return (double)v.x + (double)v.y;
        }
        return p[i];
    };
    D4 a[G];
#pragma unroll
    for (int gi = 0; gi < G; ++gi) a[gi] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 4
    for (int j = s; j < m; j += S) {
        const double2* row = reinterpret_cast<const double2*>(V + (int64_t)idx[j] * Rs);
        const double wj = entry(w, j);
#pragma unroll
        for (int gi = 0; gi < G; ++gi) {
            const int ch = c0 + cl + gi * W;
            if (ch < cpn) {
                const double2 v0 = __ldcg(row + 2 * ch);
                const double2 v1 = __ldcg(row + 2 * ch + 1);
                a[gi].x = fma(wj, v0.x, a[gi].x);
                a[gi].y = fma(wj, v0.y, a[gi].y);
                a[gi].z = fma(wj, v1.x, a[gi].z);
                a[gi].w = fma(wj, v1.y, a[gi].w);
            }
        }
    }
    for (int o = W; o < 32; o <<= 1)
#pragma unroll
        for (int gi = 0; gi < G; ++gi) {
            a[gi].x += __shfl_xor_sync(FULL_MASK, a[gi].x, o);
            a[gi].y += __shfl_xor_sync(FULL_MASK, a[gi].y, o);
            a[gi].z += __shfl_xor_sync(FULL_MASK, a[gi].z, o);
            a[gi].w += __shfl_xor_sync(FULL_MASK, a[gi].w, o);
        }
    if (s == 0) {
        const double b0 = entry(t.b0, pos), sg = entry(t.sigma, pos);
#pragma unroll
        for (int gi = 0; gi < G; ++gi) {
            const int ch = c0 + cl + gi * W;
            if (ch < cpn) {
                D4 zz;
                if (z) {
                    zz = load_d4(z + (int64_t)g * Rs + 4 * ch);
                } else {
                    const float4 f = normals4(seed, g, ch);
                    zz = {(double)f.x, (double)f.y, (double)f.z, (double)f.w};
                }
                D4 r;
                r.x = fma(sg, zz.x, a[gi].x + b0);
                r.y = fma(sg, zz.y, a[gi].y + b0);
                r.z = fma(sg, zz.z, a[gi].z + b0);
                r.w = fma(sg, zz.w, a[gi].w + b0);
                store_d4(V + (int64_t)g * Rs + 4 * ch, r);
            }
        }
    }
}

// CSR: packed tables (t.off rows) and the seed read from f.seed_dev, the form
// used by batches of domains.
template <typename T, int G, int MINB, bool CSR>
__global__ void __launch_bounds__(256, MINB) sweep_flow_kernel(const SweepTables<T> t, int k, int Rp, int W,
                                                               const T* __restrict__ z, uint64_t seed,
                                                               T* __restrict__ V, const FlowArgs f) {
    const int lane = threadIdx.x & 31;
    const int64_t items = f.item1;
    const int P4 = W * G;
    const int64_t Rs = f.row_stride ? f.row_stride : Rp;
    if (CSR && f.seed_dev) seed = *f.seed_dev;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0)
            base = (*(volatile int32_t*)f.err) ? (unsigned long long)items
                                                 : f.item0 + atomicAdd(f.ticket, (unsigned long long)f.chunk);
        base = __shfl_sync(FULL_MASK, base, 0);
        if ((int64_t)base >= items) break;
        const int64_t end = min((int64_t)base + f.chunk, items);
        for (int64_t it = (int64_t)base; it < end; ++it) {
            const int64_t pos = it / f.H;
            const int q = (int)(it - pos * f.H);
            const int g = t.node[pos];
            if (f.node_class && f.node_class[g] != f.cls) continue;  // the other launch's node
            const int m = t.m[pos];
            int32_t* done_q = f.done + (int64_t)q * f.N;
            const bool ok = flow_wait(t.idx + (CSR ? t.off[pos] : pos * (int64_t)k), m, done_q, f, lane);
            if (ok) {
                if constexpr (sizeof(T) == 4)
                    flow_piece_fp32<G, CSR>(t, k, pos, g, m, Rp, Rs, q * P4, W, lane, z, seed, V);
                else
                    flow_piece_fp64<G, CSR>(t, k, pos, g, m, Rp, Rs, q * P4, W, lane, z, seed, V, CSR ? f.pairs : 0);
            } else if (lane == 0) {
                atomicExch(f.err, 1);
            }
            __threadfence();
            __syncwarp();
            if (lane == 0) st_flag(done_q + g, f.epoch);
        }
    }
}

// Self-test of the dataflow wait: one warp waits, with the sweep's own
// flow_wait, on a flag that nothing sets; the wait must give up after
// f.wait_ns and report it in *f.err, leaving the context usable.
__global__ void flow_wait_selftest_kernel(const int32_t* __restrict__ idx, const FlowArgs f) {
    const int lane = threadIdx.x & 31;
    const bool ok = flow_wait(idx, 1, f.done, f, lane);
    if (!ok && lane == 0) atomicExch(f.err, 1);
}

cudaError_t launch_flow_wait_selftest(const int32_t* idx, const FlowArgs& f, cudaStream_t s) {
    flow_wait_selftest_kernel<<<1, 32, 0, s>>>(idx, f);
    return cudaGetLastError();
}

// Flags of the positions [p0, p1) swept by per-level launches before a
// dataflow launch takes over (every piece).
__global__ void flow_mark_kernel(const int32_t* __restrict__ node, int64_t p0, int64_t p1, int H, int64_t N,
                                 int32_t* __restrict__ done, int32_t epoch) {
    const int64_t n = (p1 - p0) * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = p0 + i / H;
        const int q = (int)(i % H);
        done[(int64_t)q * N + node[pos]] = epoch;
    }
}

// Lane layout for a row of cpn chunks: W lanes per slice (0 = automatic),
// G chunks per lane; returns the pieces per row.
int flow_layout(int Rp, int& W, int& G) {
    const int cpn = Rp / 4;
    int p2 = 1;
    while (p2 < cpn && p2 < 32) p2 <<= 1;
    if (W <= 0 || W > p2) W = p2;
    if (G != 2) G = 1;
    if (W * G > cpn && G == 2) G = 1;
    return (cpn + W * G - 1) / (W * G);
}

template <typename T, int G, int MINB, bool CSR>
static cudaError_t flow_launch(const SweepTables<T>& t, int k, int Rp, int W, const T* z, uint64_t seed, T* V,
                               const FlowArgs& f, int nsm, cudaStream_t s) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_flow_kernel<T, G, MINB, CSR>, 256, 0);
    if (e != cudaSuccess) return e;
    if (f.blocks_per_sm > 0 && f.blocks_per_sm < per_sm) per_sm = f.blocks_per_sm;
    if (per_sm < 1) per_sm = 1;
    const int64_t items = (f.item1 - f.item0 + f.chunk - 1) / f.chunk;
    int64_t blocks = std::min<int64_t>((int64_t)nsm * per_sm, (items + 7) / 8);
    if (blocks < 1) blocks = 1;
    sweep_flow_kernel<T, G, MINB, CSR><<<(int)blocks, 256, 0, s>>>(t, k, Rp, W, z, seed, V, f);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t sweep_flow(const SweepTables<T>& t, int k, int Rp, int W, int G, const T* z, uint64_t seed, T* V,
                              const FlowArgs& f, int nsm, cudaStream_t s) {
    if (f.item1 <= f.item0) return cudaSuccess;
    if (t.off) {
        if (G == 2) return f.tight ? flow_launch<T, 2, 4, true>(t, k, Rp, W, z, seed, V, f, nsm, s)
                                   : flow_launch<T, 2, 1, true>(t, k, Rp, W, z, seed, V, f, nsm, s);
        return f.tight ? flow_launch<T, 1, 6, true>(t, k, Rp, W, z, seed, V, f, nsm, s)
                       : flow_launch<T, 1, 1, true>(t, k, Rp, W, z, seed, V, f, nsm, s);
    }
    if (G == 2) return f.tight ? flow_launch<T, 2, 4, false>(t, k, Rp, W, z, seed, V, f, nsm, s)
                               : flow_launch<T, 2, 1, false>(t, k, Rp, W, z, seed, V, f, nsm, s);
    return f.tight ? flow_launch<T, 1, 6, false>(t, k, Rp, W, z, seed, V, f, nsm, s)
                   : flow_launch<T, 1, 1, false>(t, k, Rp, W, z, seed, V, f, nsm, s);
}

cudaError_t launch_sweep_flow_fp32(const SweepTables<float>& t, int k, int Rp, int W, int G, const float* z,
                                   uint64_t seed, float* V, const FlowArgs& f, int nsm, cudaStream_t s) {
    return sweep_flow<float>(t, k, Rp, W, G, z, seed, V, f, nsm, s);
}

cudaError_t launch_sweep_flow_fp64(const SweepTables<double>& t, int k, int Rp, int W, int G, const double* z,
                                   uint64_t seed, double* V, const FlowArgs& f, int nsm, cudaStream_t s) {
    return sweep_flow<double>(t, k, Rp, W, G, z, seed, V, f, nsm, s);
}

cudaError_t launch_flow_mark(const int32_t* node, int64_t p0, int64_t p1, int H, int64_t N, int32_t* done,
                             int32_t epoch, cudaStream_t s) {
    if (p1 <= p0) return cudaSuccess;
    const int64_t n = (p1 - p0) * H;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 1 << 16);
    flow_mark_kernel<<<blocks, 256, 0, s>>>(node, p0, p1, H, N, done, epoch);
    return cudaGetLastError();
}

int sweep_flow_max_blocks_per_sm(bool fp64, int G, bool tight) {
    int per_sm = 0;
    if (fp64) {
        if (G == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, tight ? sweep_flow_kernel<double, 2, 4, false> : sweep_flow_kernel<double, 2, 1, false>, 256, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, tight ? sweep_flow_kernel<double, 1, 6, false> : sweep_flow_kernel<double, 1, 1, false>, 256, 0);
    } else {
        if (G == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, tight ? sweep_flow_kernel<float, 2, 4, false> : sweep_flow_kernel<float, 2, 1, false>, 256, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, tight ? sweep_flow_kernel<float, 1, 6, false> : sweep_flow_kernel<float, 1, 1, false>, 256, 0);
    }
    return per_sm;
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

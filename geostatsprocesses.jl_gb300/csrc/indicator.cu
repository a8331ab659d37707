// indicator.cu — sequential indicator simulation (SIS): the categorical
// counterpart of the sweep for an IndicatorProcess simulated with SEQSIM
// (src/simulation/field/seqsim.jl:247-261 one-hot transform, :292-310
// Kriging(func, prob) with a Categorical prior and conditional, :342-347
// categorical draw).
//
// For a separable (intrinsic) indicator covariance C_ab(h) = A_ab rho(h) —
// which includes the proportional transiogram t_ab(h) = p_b + (delta_ab -
// p_b) rho(h), where A = diag(p) - p p' — simple cokriging of isotopic
// indicators gives every category the same weights: those of simple kriging
// with rho (the weights of the plan's solve), so
//   p_l = prob_l + sum_i w_i (I_l(x_i) - prob_l)
//       = prob_l (1 - W) + sum_{grid nbrs of category l} w_j + D_l
// with W the sum of all weights and D_l the weights of data of category l
// (both written by the solve).  The conditional is Categorical(normalize(
// clamp(p, 0, 1), 1)); a node without a kriging system (fewer than
// minneighbors neighbours, or singular) has W = D = 0, i.e. the prior.
// The draw is the inverse cdf at a uniform u: the first category whose
// cumulative probability exceeds u.
//
// Categories are bytes, node-major [N][Rp] (4 realizations per 32-bit
// word); levels run in order, one thread per (node, 4 realizations).
// Per-category sums are compensated FP32 sums of (hi, lo) weights (about
// 1e-12), so the category decision equals an FP64 evaluation except at
// exact ties.
#include "common.cuh"

namespace sgs {

// four uniforms in (0, 1) of node g, realizations 4q..4q+3: (2m+1)/2^24 on
// the top 23 bits m of the Philox4x32-10 output words (counter: node,
// realization / 4, 0x5349), exact in FP32 and FP64
__device__ __forceinline__ float4 uniforms4(uint64_t seed, int64_t g, int q) {
    uint4 c = philox10(make_uint4((uint32_t)g, (uint32_t)((uint64_t)g >> 32), (uint32_t)q, 0x5349u),
                       (uint32_t)seed, (uint32_t)(seed >> 32));
    const float sc = 1.0f / 16777216.0f;
    return make_float4((float)((c.x >> 9) * 2u + 1u) * sc, (float)((c.y >> 9) * 2u + 1u) * sc,
                       (float)((c.z >> 9) * 2u + 1u) * sc, (float)((c.w >> 9) * 2u + 1u) * sc);
}

__device__ __forceinline__ int draw_category(const IndArgs& ia, const double* p, double u) {
    double q[IND_MAX_CAT];
    double s = 0.0;
#pragma unroll
    for (int l = 0; l < IND_MAX_CAT; ++l) {
        q[l] = l < ia.ncat ? fmin(fmax(p[l], 0.0), 1.0) : 0.0;
        s += q[l];
    }
    if (!(s > 0.0)) {  // every kriged probability clamped to 0: the prior
#pragma unroll
        for (int l = 0; l < IND_MAX_CAT; ++l) q[l] = l < ia.ncat ? ia.prob[l] : 0.0;
        s = 1.0;
    }
    double cum = 0.0;
#pragma unroll
    for (int l = 0; l < IND_MAX_CAT - 1; ++l) {
        if (l < ia.ncat - 1) {
            cum += q[l] / s;
            if (u < cum) return l;
        }
    }
    return ia.ncat - 1;
}

template <typename T>
__global__ void __launch_bounds__(256) sis_level_kernel(const SweepTables<T> t, int k, int64_t p0, int64_t p1, int Rp,
                                                        const IndArgs ia, const double* __restrict__ u, uint64_t seed,
                                                        uint8_t* __restrict__ C) {
    const int cpn = Rp >> 2;
    const int64_t total = (p1 - p0) * cpn;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = p0 + i / cpn;
        const int ch = (int)(i % cpn);
        const int g = t.node[pos];
        const int m = t.m[pos];
        const int32_t* idx = t.idx + pos * k;
        // per realization and category: the weights of grid neighbours of
        // that category (compensated FP32 sums, or FP64 for FP64 tables)
        float s[4][IND_MAX_CAT], c[4][IND_MAX_CAT];
        double d[4][IND_MAX_CAT];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int l = 0; l < IND_MAX_CAT; ++l) {
                s[r][l] = 0.f;
                c[r][l] = 0.f;
                d[r][l] = 0.0;
            }
        for (int j = 0; j < m; ++j) {
            const uint32_t cats = *reinterpret_cast<const uint32_t*>(C + (int64_t)idx[j] * Rp + 4 * ch);
            if constexpr (sizeof(T) == 4) {
                const float2 wj = reinterpret_cast<const float2*>(t.w)[pos * k + j];
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const int cr = (int)((cats >> (8 * r)) & 0xffu);
#pragma unroll
                    for (int l = 0; l < IND_MAX_CAT; ++l)
                        if (l == cr) {
                            const DF ts = df_two_sum(s[r][l], wj.x);
                            s[r][l] = ts.hi;
                            c[r][l] = __fadd_rn(c[r][l], __fadd_rn(ts.lo, wj.y));
                        }
                }
            } else {
                const double wj = t.w[pos * k + j];
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const int cr = (int)((cats >> (8 * r)) & 0xffu);
#pragma unroll
                    for (int l = 0; l < IND_MAX_CAT; ++l)
                        if (l == cr) d[r][l] += wj;
                }
            }
        }
        const double W = ia.wsum[pos];
        const double* D = ia.dsum + pos * ia.ncat;
        const float4 uf = u ? make_float4(0.f, 0.f, 0.f, 0.f) : uniforms4(seed, g, ch);
        const float ufa[4] = {uf.x, uf.y, uf.z, uf.w};
        uint32_t out = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            double p[IND_MAX_CAT];
#pragma unroll
            for (int l = 0; l < IND_MAX_CAT; ++l) {
                const double gsum = sizeof(T) == 4 ? (double)s[r][l] + (double)c[r][l] : d[r][l];
                p[l] = l < ia.ncat ? ia.prob[l] * (1.0 - W) + gsum + D[l] : 0.0;
            }
            const double ur = u ? u[(int64_t)g * Rp + 4 * ch + r] : (double)ufa[r];
            out |= (uint32_t)draw_category(ia, p, ur) << (8 * r);
        }
        *reinterpret_cast<uint32_t*>(C + (int64_t)g * Rp + 4 * ch) = out;
    }
}

template <typename T>
static cudaError_t sis_level(const SweepTables<T>& t, int k, int64_t p0, int64_t p1, int Rp, const IndArgs& ia,
                             const double* u, uint64_t seed, uint8_t* C, cudaStream_t s) {
    if (p1 <= p0) return cudaSuccess;
    int64_t blocks = ((p1 - p0) * (Rp / 4) + 255) / 256;
    if (blocks > (1 << 20)) blocks = 1 << 20;
    sis_level_kernel<T><<<(int)blocks, 256, 0, s>>>(t, k, p0, p1, Rp, ia, u, seed, C);
    return cudaGetLastError();
}

cudaError_t launch_sis_level_fp32(const SweepTables<float>& t, int k, int64_t p0, int64_t p1, int Rp,
                                  const IndArgs& ia, const double* u, uint64_t seed, uint8_t* C, cudaStream_t s) {
    return sis_level<float>(t, k, p0, p1, Rp, ia, u, seed, C, s);
}

cudaError_t launch_sis_level_fp64(const SweepTables<double>& t, int k, int64_t p0, int64_t p1, int Rp,
                                  const IndArgs& ia, const double* u, uint64_t seed, uint8_t* C, cudaStream_t s) {
    return sis_level<double>(t, k, p0, p1, Rp, ia, u, seed, C, s);
}

// node-major category bytes [N][Rp] -> realization-major int32 [R][N]
__global__ void cats_to_out_kernel(const uint8_t* __restrict__ C, int64_t N, int R, int Rp, int32_t* __restrict__ out) {
    const int64_t total = N * R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / N);
        const int64_t g = i - (int64_t)r * N;
        out[i] = C[g * Rp + r];
    }
}

cudaError_t launch_cats_to_out(const uint8_t* C, int64_t N, int R, int Rp, int32_t* out, cudaStream_t s) {
    const int64_t total = N * R;
    int64_t blocks = (total + 255) / 256;
    if (blocks > (1 << 20)) blocks = 1 << 20;
    if (blocks < 1) blocks = 1;
    cats_to_out_kernel<<<(int)blocks, 256, 0, s>>>(C, N, R, Rp, out);
    return cudaGetLastError();
}

}  // namespace sgs

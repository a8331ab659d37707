// ensemble.cu — per-node statistics of an ensemble of realizations, on the
// device: mean, variance, empirical cdf / ccdf at thresholds and quantiles.
//
// Replaces the reference's Ensemble statistics (src/ensembles.jl:42-52,
// reduced per node by ereduce, :76-85): mean, var (Statistics.var, corrected:
// divides by R - 1), cdf(e, x) = count(<= x) / R, ccdf(e, x) = count(> x) / R,
// quantile(e, p) = Statistics.quantile of the node's R values (the default
// definition: linear interpolation between order statistics, h = (R - 1) p,
// x[floor h] + (h - floor h) (x[floor h + 1] - x[floor h]) on the sorted
// values).  The realizations stay in HBM: the values are the node-major rows
// sgs_plan_simulate_device / sgs_batch_simulate_device write (row of R
// values, row stride >= R, float or double, centred), and `offset` (the
// process mean) is added to every value.
//
// One warp per node; sums in FP64; the quantile kernel sorts each row in
// shared memory (bitonic, R <= 1024).  Nothing is allocated: the threshold
// and probability lists (at most 32 per launch) travel in the kernel
// parameters, and the host wrapper launches once per 32 of them.
#include <algorithm>
#include <climits>
#include <cmath>

#include "common.cuh"

namespace sgs {

constexpr int ENS_WARPS = 8;
constexpr int ENS_LIST = 32;
constexpr int ENS_RMAX = 1024;

struct EnsArgs {
    const void* vals;
    int fp64;          // 1: double values, 0: float
    int64_t N;
    int R;
    int stride;        // row stride (elements)
    double offset;
    int nlist;         // entries of `list` used
    int list_stride;   // output row length (all entries of the full list)
    int list0;         // first output column of this launch
    double list[ENS_LIST];
};

__device__ __forceinline__ double ens_val(const EnsArgs& a, int64_t g, int r) {
    const int64_t i = g * a.stride + r;
    return (a.fp64 ? reinterpret_cast<const double*>(a.vals)[i] : (double)reinterpret_cast<const float*>(a.vals)[i]) +
           a.offset;
}

__device__ __forceinline__ double ens_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

__global__ void __launch_bounds__(ENS_WARPS * 32) ens_stats_kernel(const EnsArgs a, double* mean, double* var) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * ENS_WARPS;
    for (int64_t g = (int64_t)blockIdx.x * ENS_WARPS + (threadIdx.x >> 5); g < a.N; g += nw) {
        double s = 0.0;
        for (int r = lane; r < a.R; r += 32) s += ens_val(a, g, r);
        const double m = ens_warp_sum(s) / a.R;
        double q = 0.0;
        for (int r = lane; r < a.R; r += 32) {
            const double d = ens_val(a, g, r) - m;
            q += d * d;
        }
        q = ens_warp_sum(q);
        if (lane == 0) {
            if (mean) mean[g] = m;
            if (var) var[g] = a.R > 1 ? q / (a.R - 1) : nan("");
        }
    }
}

// cdf (complement = 0: count(v <= x) / R) or ccdf (1: count(v > x) / R)
__global__ void __launch_bounds__(ENS_WARPS * 32) ens_cdf_kernel(const EnsArgs a, int complement, double* out) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * ENS_WARPS;
    for (int64_t g = (int64_t)blockIdx.x * ENS_WARPS + (threadIdx.x >> 5); g < a.N; g += nw) {
        int cnt[ENS_LIST];
#pragma unroll
        for (int i = 0; i < ENS_LIST; ++i) cnt[i] = 0;
        for (int r0 = 0; r0 < a.R; r0 += 32) {
            const int r = r0 + lane;
            const bool in = r < a.R;
            const double v = in ? ens_val(a, g, r) : 0.0;
#pragma unroll
            for (int i = 0; i < ENS_LIST; ++i)
                if (i < a.nlist) {
                    const bool c = in && (complement ? v > a.list[i] : v <= a.list[i]);
                    cnt[i] += __popc(__ballot_sync(FULL_MASK, c));
                }
        }
        for (int i = lane; i < a.nlist; i += 32) {
            int c = 0;
#pragma unroll
            for (int j = 0; j < ENS_LIST; ++j)
                if (j == i) c = cnt[j];
            out[g * a.list_stride + a.list0 + i] = (double)c / a.R;
        }
    }
}

// quantiles: the row sorted in shared memory, then linear interpolation
__global__ void __launch_bounds__(ENS_WARPS * 32) ens_quantile_kernel(const EnsArgs a, double* out) {
    extern __shared__ double s_rows[];
    const int lane = threadIdx.x & 31;
    int P = 1;
    while (P < a.R) P <<= 1;
    double* x = s_rows + (size_t)(threadIdx.x >> 5) * P;
    const int64_t nw = (int64_t)gridDim.x * ENS_WARPS;
    for (int64_t g = (int64_t)blockIdx.x * ENS_WARPS + (threadIdx.x >> 5); g < a.N; g += nw) {
        for (int r = lane; r < P; r += 32) x[r] = r < a.R ? ens_val(a, g, r) : INFINITY;
        __syncwarp();
        for (int size = 2; size <= P; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int t = lane; t < (P >> 1); t += 32) {
                    const int i = (t / stride) * stride * 2 + (t % stride);
                    const int j = i + stride;
                    const bool asc = (i & size) == 0;
                    const double xi = x[i], xj = x[j];
                    if ((xi > xj) == asc) {
                        x[i] = xj;
                        x[j] = xi;
                    }
                }
                __syncwarp();
            }
        for (int i = lane; i < a.nlist; i += 32) {
            const double h = (a.R - 1) * a.list[i];
            const double fl = floor(h);
            const int lo = min(max((int)fl, 0), a.R - 1);
            const int hi = min(lo + 1, a.R - 1);
            out[g * a.list_stride + a.list0 + i] = x[lo] + (h - fl) * (x[hi] - x[lo]);
        }
        __syncwarp();
    }
}

}  // namespace sgs

using namespace sgs;

namespace {

int ens_fail(int code, const char* msg) {
    sgs::set_thread_error(msg);
    return code;
}

int ens_args(EnsArgs& a, const void* vals, int32_t precision, int64_t N, int32_t R, int32_t stride, double offset) {
    if (!vals || N < 0 || R < 1 || stride < R) return ens_fail(SGS_ERR_ARG, "invalid ensemble array");
    if (precision != SGS_PREC_FP64 && precision != SGS_PREC_FP32_REFINE) return ens_fail(SGS_ERR_ARG, "unknown precision");
    a = EnsArgs{};
    a.vals = vals;
    a.fp64 = precision == SGS_PREC_FP64;
    a.N = N;
    a.R = R;
    a.stride = stride;
    a.offset = offset;
    return SGS_OK;
}

int ens_grid(int64_t N) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (N + ENS_WARPS - 1) / ENS_WARPS;
    const int64_t cap = (int64_t)(nsm > 0 ? nsm : 1) * 16;
    return (int)std::max<int64_t>(1, std::min(want, cap));
}

int ens_done(cudaError_t e, const char* where) {
    if (e != cudaSuccess) {
        sgs::set_thread_error(std::string(where) + ": " + cudaGetErrorString(e));
        return SGS_ERR_CUDA;
    }
    return SGS_OK;
}

}  // namespace

extern "C" int sgs_ensemble_stats(const void* vals, int32_t precision, int64_t nnodes, int32_t nreals,
                                  int32_t row_stride, double offset, double* mean, double* var, void* stream) {
    EnsArgs a;
    int rc = ens_args(a, vals, precision, nnodes, nreals, row_stride, offset);
    if (rc) return rc;
    if (!mean && !var) return ens_fail(SGS_ERR_ARG, "no output");
    if (nnodes == 0) return SGS_OK;
    ens_stats_kernel<<<ens_grid(nnodes), ENS_WARPS * 32, 0, (cudaStream_t)stream>>>(a, mean, var);
    return ens_done(cudaGetLastError(), "sgs_ensemble_stats");
}

extern "C" int sgs_ensemble_cdf(const void* vals, int32_t precision, int64_t nnodes, int32_t nreals,
                                int32_t row_stride, double offset, const double* x, int32_t nx, int32_t complement,
                                double* out, void* stream) {
    EnsArgs a;
    int rc = ens_args(a, vals, precision, nnodes, nreals, row_stride, offset);
    if (rc) return rc;
    if (!x || nx < 1 || !out) return ens_fail(SGS_ERR_ARG, "invalid thresholds or output");
    if (nnodes == 0) return SGS_OK;
    a.list_stride = nx;
    for (int i0 = 0; i0 < nx; i0 += ENS_LIST) {
        a.list0 = i0;
        a.nlist = std::min(ENS_LIST, nx - i0);
        for (int i = 0; i < a.nlist; ++i) a.list[i] = x[i0 + i];
        ens_cdf_kernel<<<ens_grid(nnodes), ENS_WARPS * 32, 0, (cudaStream_t)stream>>>(a, complement ? 1 : 0, out);
        if ((rc = ens_done(cudaGetLastError(), "sgs_ensemble_cdf"))) return rc;
    }
    return SGS_OK;
}

extern "C" int sgs_ensemble_quantile(const void* vals, int32_t precision, int64_t nnodes, int32_t nreals,
                                     int32_t row_stride, double offset, const double* p, int32_t np, double* out,
                                     void* stream) {
    EnsArgs a;
    int rc = ens_args(a, vals, precision, nnodes, nreals, row_stride, offset);
    if (rc) return rc;
    if (!p || np < 1 || !out) return ens_fail(SGS_ERR_ARG, "invalid probabilities or output");
    if (nreals > ENS_RMAX) return ens_fail(SGS_ERR_ARG, "quantiles take at most 1024 realizations");
    for (int i = 0; i < np; ++i)
        if (!(p[i] >= 0.0 && p[i] <= 1.0)) return ens_fail(SGS_ERR_ARG, "probabilities must be in [0, 1]");
    if (nnodes == 0) return SGS_OK;
    int P = 1;
    while (P < nreals) P <<= 1;
    const size_t smem = (size_t)ENS_WARPS * P * sizeof(double);
    if ((rc = ens_done(cudaFuncSetAttribute(ens_quantile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem), "sgs_ensemble_quantile")))
        return rc;
    a.list_stride = np;
    for (int i0 = 0; i0 < np; i0 += ENS_LIST) {
        a.list0 = i0;
        a.nlist = std::min(ENS_LIST, np - i0);
        for (int i = 0; i < a.nlist; ++i) a.list[i] = p[i0 + i];
        ens_quantile_kernel<<<ens_grid(nnodes), ENS_WARPS * 32, smem, (cudaStream_t)stream>>>(a, out);
        if ((rc = ens_done(cudaGetLastError(), "sgs_ensemble_quantile"))) return rc;
    }
    return SGS_OK;
}

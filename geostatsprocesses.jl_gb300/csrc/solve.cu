// solve.cu — kernel (b): batched simple-kriging build + solve for every node.
//
// Replaces GeoStatsModels.fit(Kriging(f, mu), neighbourhood) + status +
// predictprob (src/simulation/field/seqsim.jl:124-131,302-304): the LHS
// C_ab = sill - gamma(x_a, x_b) (src/utils.jl:50-62), its Cholesky factor,
// the weights w = C^-1 c, the conditional variance sigma^2 = C(0) - w'c, and
// the prior fallback when the factorization fails or the node has fewer
// than minneighbors neighbours (seqsim.jl:109-111,127-131).
//
// One warp per system, LHS in shared memory.  Grid-grid covariances come
// from an FP64 table over integer lags (every neighbour of a node is a cell
// offset inside the search template, so pairwise lags are bounded); lags
// involving data points are evaluated directly in FP64.
//
// Precision modes:
//   FP64          FP64 LHS, Cholesky, weights (the plain path)
//   FP32+refine   FP32 LHS + Cholesky; iterative refinement with the FP64
//                 residual r = c - C w; FP64 variance.  A system whose FP32
//                 pivot falls below 1e-3*sill or whose refinement does not
//                 contract is queued and re-solved in FP64.
// Results are written in level order (the sweep's layout): the grid
// neighbours with their weights, and the data neighbours folded into the
// constant b0 = sum_data w_i (d_i - mu).
#include <cmath>

#include "common.cuh"

namespace sgs {

constexpr int SOLVE_WARPS = 4;

struct NbInfo {
    int c0, c1, c2;  // cell (grid neighbour or query)
    int did;         // data id, -1 for a grid node
};

__device__ __forceinline__ double lut_or_cov(const SolveArgs& a, int L0, int L1, int L2) {
    const CovLut& t = a.lut;
    if (t.c64 != nullptr && L0 >= -t.e[0] && L0 <= t.e[0] && L1 >= -t.e[1] && L1 <= t.e[1] &&
        L2 >= -t.e[2] && L2 <= t.e[2]) {
        return t.c64[(L0 + t.e[0]) + t.w[0] * ((L1 + t.e[1]) + t.w[1] * (L2 + t.e[2]))];
    }
    const GridDev& G = a.grid;
    return cov_fp64(a.vario, G.dim, dmul((double)L0, G.spacing[0]), dmul((double)L1, G.spacing[1]),
                    G.dim == 3 ? dmul((double)L2, G.spacing[2]) : 0.0);
}

__device__ __forceinline__ void point_of(const SolveArgs& a, const NbInfo& p, double* x) {
    const GridDev& G = a.grid;
    if (p.did < 0) {
        x[0] = centroid(G, 0, p.c0);
        x[1] = centroid(G, 1, p.c1);
        x[2] = G.dim == 3 ? centroid(G, 2, p.c2) : 0.0;
    } else {
        x[0] = a.data_xyz[3 * (int64_t)p.did + 0];
        x[1] = a.data_xyz[3 * (int64_t)p.did + 1];
        x[2] = a.data_xyz[3 * (int64_t)p.did + 2];
    }
}

// FP64 covariance between two points of the augmented set
__device__ __forceinline__ double kcov(const SolveArgs& a, const NbInfo& p, const NbInfo& q) {
    if (p.did < 0 && q.did < 0) return lut_or_cov(a, q.c0 - p.c0, q.c1 - p.c1, q.c2 - p.c2);
    double xp[3], xq[3];
    point_of(a, p, xp);
    point_of(a, q, xq);
    return cov_fp64(a.vario, a.grid.dim, dsub(xq[0], xp[0]), dsub(xq[1], xp[1]), dsub(xq[2], xp[2]));
}

// Right-looking Cholesky of the lower triangle of A (leading dimension ld)
// by one warp.  Fails (returns false) when a pivot is not > tau.
template <typename T>
__device__ bool warp_cholesky(T* A, int ld, int n, T tau, int lane) {
    for (int j = 0; j < n; ++j) {
        const T d = A[j * ld + j];
        if (!(d > tau)) return false;
        const T ljj = sqrt(d);
        const T inv = T(1) / ljj;
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) A[i * ld + j] *= inv;
        if (lane == 0) A[j * ld + j] = ljj;
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) {
            const T lij = A[i * ld + j];
            for (int l = j + 1; l <= i; ++l) A[i * ld + l] -= lij * A[l * ld + j];
        }
        __syncwarp();
    }
    return true;
}

// Solve L L^T x = b in place (x overwrites b), L from warp_cholesky.
template <typename T>
__device__ void warp_chol_solve(const T* A, int ld, int n, T* b, int lane) {
    for (int j = 0; j < n; ++j) {
        const T yj = b[j] / A[j * ld + j];
        __syncwarp();
        if (lane == 0) b[j] = yj;
        for (int i = j + 1 + lane; i < n; i += 32) b[i] -= A[i * ld + j] * yj;
        __syncwarp();
    }
    for (int j = n - 1; j >= 0; --j) {
        const T wj = b[j] / A[j * ld + j];
        __syncwarp();
        if (lane == 0) b[j] = wj;
        for (int i = lane; i < j; i += 32) b[i] -= A[j * ld + i] * wj;
        __syncwarp();
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL_MASK, v, o));
    return v;
}

template <typename T>
__host__ __device__ constexpr size_t warp_smem_bytes(int k) {
    // A (k x (k+1) of T), c and w (FP64), rhs (T), neighbour info
    return ((size_t)k * (k + 1) * sizeof(T) + 15) / 16 * 16 + 2 * (size_t)k * sizeof(double) +
           ((size_t)k * sizeof(T) + 15) / 16 * 16 + (size_t)k * sizeof(NbInfo);
}

// Write one position's sweep-table row (and the optional node-indexed export).
template <typename O>
__device__ void write_row(const SolveArgs& a, const SweepTables<O>& tab, int64_t pos, int g, int n,
                          const NbInfo* info, const double* w, double sigma, int status, int lane) {
    const int k = a.k;
    int m = 0;
    double b0 = 0.0;
    if (status == SGS_NODE_KRIGED_) {
        for (int base = 0; base < n; base += 32) {
            const int q = base + lane;
            const bool isgrid = q < n && info[q].did < 0;
            const unsigned b = __ballot_sync(FULL_MASK, isgrid);
            if (isgrid) {
                const int j = m + __popc(b & lanemask_lt());
                tab.idx[pos * k + j] = a.nbr[(int64_t)g * k + q];
                tab.w[pos * k + j] = (O)w[q];
            } else if (q < n) {
                b0 += w[q] * (a.data_val[info[q].did] - a.mu);
            }
            m += __popc(b);
        }
        b0 = warp_sum(b0);
    }
    if (lane == 0) {
        if (a.sum_m) atomicAdd(a.sum_m, (unsigned long long)m);
        tab.node[pos] = g;
        tab.m[pos] = m;
        tab.b0[pos] = (O)b0;
        tab.sigma[pos] = (O)sigma;
        a.status[g] = (int8_t)status;
    }
    if (a.w_full) {
        for (int q = lane; q < k; q += 32)
            a.w_full[(int64_t)g * k + q] = (status == SGS_NODE_KRIGED_ && q < n) ? w[q] : 0.0;
        if (lane == 0) a.sigma_full[g] = sigma;
    }
}

// T: factorization type; O: table type; REFINE: FP32 + FP64 refinement with
// fallback queue.  With a.list set, solves only the queued positions.
template <typename T, typename O, bool REFINE>
__global__ void __launch_bounds__(SOLVE_WARPS * 32) solve_kernel(const SolveArgs a, const SweepTables<O> tab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int k = a.k;
    const int ld = k + 1;
    unsigned char* base = smem + (size_t)wib * warp_smem_bytes<T>(k);
    T* A = reinterpret_cast<T*>(base);
    double* c = reinterpret_cast<double*>(base + ((size_t)k * ld * sizeof(T) + 15) / 16 * 16);
    double* w = c + k;
    T* rhs = reinterpret_cast<T*>(w + k);
    NbInfo* info = reinterpret_cast<NbInfo*>(reinterpret_cast<unsigned char*>(rhs) + ((size_t)k * sizeof(T) + 15) / 16 * 16);
    const GridDev& G = a.grid;
    const double sill = a.vario.sill;
    const double prior_sd = sqrt(sill);

    const int64_t count = a.list ? (int64_t)*a.nfallback : a.P;
    const int64_t nwarps = (int64_t)gridDim.x * SOLVE_WARPS;
    for (int64_t it = (int64_t)blockIdx.x * SOLVE_WARPS + wib; it < count; it += nwarps) {
        const int64_t pos = a.list ? (int64_t)a.list[it] : it;
        const int g = a.order[pos];
        const int n = a.cnt[g];
        if (n < a.nmin) {
            write_row<O>(a, tab, pos, g, n, info, w, prior_sd, SGS_NODE_PRIOR_NMIN_, lane);
            continue;
        }
        NbInfo self;
        cell_of(G, g, self.c0, self.c1, self.c2);
        self.did = -1;
        for (int q = lane; q < n; q += 32) {
            const int id = a.nbr[(int64_t)g * k + q];
            NbInfo in;
            if (id < G.N) {
                cell_of(G, id, in.c0, in.c1, in.c2);
                in.did = -1;
            } else {
                in.c0 = in.c1 = in.c2 = 0;
                in.did = id - (int)G.N;
            }
            info[q] = in;
        }
        __syncwarp();
        for (int q = lane; q < n; q += 32) c[q] = kcov(a, info[q], self);
        for (int r = 0; r < n; ++r)
            for (int q = lane; q <= r; q += 32) A[r * ld + q] = (T)kcov(a, info[q], info[r]);
        __syncwarp();

        bool ok;
        if (!REFINE) {
            ok = warp_cholesky<T>(A, ld, n, (T)a.tau, lane);
            if (ok) {
                for (int q = lane; q < n; q += 32) rhs[q] = (T)c[q];
                __syncwarp();
                warp_chol_solve<T>(A, ld, n, rhs, lane);
                for (int q = lane; q < n; q += 32) w[q] = (double)rhs[q];
                __syncwarp();
            }
        } else {
            const T guard = (T)(1e-3 * sill);
            ok = warp_cholesky<T>(A, ld, n, guard, lane);
            bool accept = ok;
            if (ok) {
                for (int q = lane; q < n; q += 32) rhs[q] = (T)c[q];
                __syncwarp();
                warp_chol_solve<T>(A, ld, n, rhs, lane);
                for (int q = lane; q < n; q += 32) w[q] = (double)rhs[q];
                __syncwarp();
                double prev = 0.0, last = 0.0;
                for (int s = 0; s < a.refine_steps; ++s) {
                    // FP64 residual r = c - C w, one row per lane
                    for (int i = lane; i < n; i += 32) {
                        double r = c[i];
                        for (int j = 0; j < n; ++j) r -= kcov(a, info[j], info[i]) * w[j];
                        rhs[i] = (T)r;
                    }
                    __syncwarp();
                    warp_chol_solve<T>(A, ld, n, rhs, lane);
                    double dmax = 0.0;
                    for (int q = lane; q < n; q += 32) {
                        const double dq = (double)rhs[q];
                        w[q] += dq;
                        dmax = fmax(dmax, fabs(dq));
                    }
                    __syncwarp();
                    prev = last;
                    last = warp_max(dmax);
                }
                // remaining error ~ contraction * last correction
                if (a.refine_steps >= 2) {
                    const double rho = prev > 0.0 ? last / prev : 0.0;
                    accept = rho < 0.5 && rho * last <= 1e-9 && isfinite(last);
                } else {
                    accept = isfinite(last);
                }
            }
            if (!accept) {
                if (lane == 0) a.fallback[atomicAdd(a.nfallback, 1)] = (int32_t)pos;
                continue;
            }
        }
        if (!ok) {
            write_row<O>(a, tab, pos, g, n, info, w, prior_sd, SGS_NODE_PRIOR_SINGULAR_, lane);
            continue;
        }
        double wc = 0.0;
        for (int q = lane; q < n; q += 32) wc += w[q] * c[q];
        wc = warp_sum(wc);
        const double var = sill - wc;
        write_row<O>(a, tab, pos, g, n, info, w, sqrt(var > 0.0 ? var : 0.0), SGS_NODE_KRIGED_, lane);
        __syncwarp();
    }
}

template <typename T, typename O, bool REFINE>
static cudaError_t launch_solve(const SolveArgs& a, const SweepTables<O>& t, cudaStream_t s) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = warp_smem_bytes<T>(a.k) * SOLVE_WARPS;
    cudaError_t e = cudaFuncSetAttribute(solve_kernel<T, O, REFINE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, solve_kernel<T, O, REFINE>, SOLVE_WARPS * 32, smem);
    if (per_sm < 1) per_sm = 1;
    int64_t want = a.list ? (int64_t)nsm * per_sm : (a.P + SOLVE_WARPS - 1) / SOLVE_WARPS;
    int blocks = (int)(want < (int64_t)nsm * per_sm ? want : (int64_t)nsm * per_sm);
    if (blocks < 1) blocks = 1;
    solve_kernel<T, O, REFINE><<<blocks, SOLVE_WARPS * 32, smem, s>>>(a, t);
    return cudaGetLastError();
}

cudaError_t launch_solve_fp64(const SolveArgs& a, const SweepTables<double>& t, cudaStream_t s) {
    return launch_solve<double, double, false>(a, t, s);
}

cudaError_t launch_solve_fp32(const SolveArgs& a, const SweepTables<float>& t, cudaStream_t s) {
    return launch_solve<float, float, true>(a, t, s);
}

cudaError_t launch_solve_fp64_into_fp32(const SolveArgs& a, const SweepTables<float>& t, cudaStream_t s) {
    return launch_solve<double, float, false>(a, t, s);
}

// ---------------------------------------------------------------------------
__global__ void fill_lut_kernel(const GridDev G, const VarioDev v, const CovLut t, double* c64, float* c32,
                                int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int L0 = (int)(i % t.w[0]) - t.e[0];
        const int64_t r = i / t.w[0];
        const int L1 = (int)(r % t.w[1]) - t.e[1];
        const int L2 = (int)(r / t.w[1]) - t.e[2];
        const double c = cov_fp64(v, G.dim, dmul((double)L0, G.spacing[0]), dmul((double)L1, G.spacing[1]),
                                  G.dim == 3 ? dmul((double)L2, G.spacing[2]) : 0.0);
        c64[i] = c;
        if (c32) c32[i] = (float)c;
    }
}

cudaError_t launch_fill_cov_lut(const GridDev& g, const VarioDev& v, CovLut lut, double* c64, float* c32,
                                cudaStream_t s) {
    const int64_t total = (int64_t)lut.w[0] * lut.w[1] * lut.w[2];
    int blocks = (int)((total + 255) / 256);
    if (blocks > 65535) blocks = 65535;
    fill_lut_kernel<<<blocks, 256, 0, s>>>(g, v, lut, c64, c32, total);
    return cudaGetLastError();
}

}  // namespace sgs

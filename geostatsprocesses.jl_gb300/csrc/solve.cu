// solve.cu — kernel (b): batched simple-kriging build + solve for every node.
//
// Replaces GeoStatsModels.fit(Kriging(f, mu), neighbourhood) + status +
// predictprob (src/simulation/field/seqsim.jl:124-131,302-304): the LHS
// C_ab = sill - gamma(x_a, x_b) (src/utils.jl:50-62), its Cholesky factor,
// the weights w = C^-1 c, the conditional variance sigma^2 = C(0) - w'c, and
// the prior fallback when the factorization fails or the node has fewer
// than minneighbors neighbours (seqsim.jl:109-111,127-131).
//
// One warp per system.  Grid-grid covariances come from a table over integer
// lags (every neighbour of a node is a cell offset inside the search
// template, so pairwise lags are bounded); lags involving data points are
// evaluated directly in FP64, 32 per warp pass.
//
// Precision modes:
//   FP64          FP64 LHS, right-looking Cholesky in shared memory, FP64
//                 weights (the plain path; also re-solves queued systems)
//   FP32+refine   register-resident Gauss-Jordan inverse of the FP32 LHS,
//                 refinement against a double-FP32 LHS with a compensated
//                 residual, double-FP32 variance (solve_fp32_kernel below)
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

// Indices of the neighbours that are data points, in order, into dl; returns
// their number (warp-uniform).
__device__ __forceinline__ int collect_data(const NbInfo* info, int n, int* dl, int lane) {
    int nd = 0;
    for (int b = 0; b < n; b += 32) {
        const int q = b + lane;
        const bool isdata = q < n && info[q].did >= 0;
        const unsigned bal = __ballot_sync(FULL_MASK, isdata);
        if (isdata) dl[nd + __popc(bal & lanemask_lt())] = q;
        nd += __popc(bal);
    }
    __syncwarp();
    return nd;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

template <typename T>
__host__ __device__ constexpr size_t warp_smem_bytes(int k) {
    // A (k x (k+1) of T), c and w (FP64), rhs (T), neighbour info
    return ((size_t)k * (k + 1) * sizeof(T) + 15) / 16 * 16 + 2 * (size_t)k * sizeof(double) +
           ((size_t)k * sizeof(T) + 15) / 16 * 16 + (size_t)k * sizeof(NbInfo);
}

// Indicator sums of one system (SolveArgs::ind_*): w holds the weights of the
// system's n neighbours (FP64 values `wq(q)`), kriged = false for a prior
// node (all sums zero).
template <typename WF>
__device__ __forceinline__ void write_indicator_sums(const SolveArgs& a, int64_t pos, int n, const NbInfo* info,
                                                     bool kriged, WF wq, int lane) {
    double ws = 0.0;
    double ds[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) ds[l] = 0.0;
    if (kriged)
        for (int q = lane; q < n; q += 32) {
            const double v = wq(q);
            ws += v;
            if (info[q].did >= 0) {
                const int c = a.ind_cat[info[q].did];
#pragma unroll
                for (int l = 0; l < 8; ++l)
                    if (l == c) ds[l] += v;
            }
        }
    ws = warp_sum(ws);
    if (lane == 0) a.ind_wsum[pos] = ws;
#pragma unroll
    for (int l = 0; l < 8; ++l)
        if (l < a.ncat) {
            const double v = warp_sum(ds[l]);
            if (lane == 0) a.ind_dsum[pos * a.ncat + l] = v;
        }
}

// Store an FP64 value into a table entry: as is, or as an FP32 (hi, lo) pair.
__device__ __forceinline__ void put(double* t, int64_t i, double v) { t[i] = v; }
__device__ __forceinline__ void put(float* t, int64_t i, double v) {
    const float hi = (float)v;
    t[2 * i] = hi;
    t[2 * i + 1] = (float)(v - (double)hi);
}

// Write one position's sweep-table row (and the optional node-indexed export).
template <typename O>
__device__ void write_row(const SolveArgs& a, const SweepTables<O>& tab, int64_t pos, int g, int n,
                          const NbInfo* info, const double* w, double sigma, int status, int lane) {
    const int k = a.k;
    const int64_t row = table_row(tab, pos, k);
    int m = 0;
    double b0 = 0.0, l1 = 0.0;
    if (status == SGS_NODE_KRIGED_) {
        for (int base = 0; base < n; base += 32) {
            const int q = base + lane;
            const bool isgrid = q < n && info[q].did < 0;
            const unsigned b = __ballot_sync(FULL_MASK, isgrid);
            if (isgrid) {
                const int j = m + __popc(b & lanemask_lt());
                tab.idx[row + j] = a.nbr[(int64_t)g * k + q] + (int32_t)a.node0;
                put(tab.w, row + j, w[q]);
                l1 += fabs(w[q]);
            } else if (q < n) {
                b0 += w[q] * (a.data_val[info[q].did] - a.mu);
            }
            m += __popc(b);
        }
        b0 = warp_sum(b0);
        if (a.wl1_max) {
            l1 = warp_sum(l1);
            if (lane == 0) atomicMax(a.wl1_max, __float_as_uint((float)l1));
        }
    }
    if (a.ind_wsum)
        write_indicator_sums(a, pos, n, info, status == SGS_NODE_KRIGED_, [&](int q) { return w[q]; }, lane);
    if (lane == 0) {
        if (a.sum_m) atomicAdd(a.sum_m, (unsigned long long)m);
        tab.node[pos] = g + (int32_t)a.node0;
        tab.m[pos] = m;
        put(tab.b0, pos, b0);
        put(tab.sigma, pos, sigma);
        a.status[g] = (int8_t)status;
    }
    if (a.w_full) {
        for (int q = lane; q < k; q += 32)
            a.w_full[(int64_t)g * k + q] = (status == SGS_NODE_KRIGED_ && q < n) ? w[q] : 0.0;
        if (lane == 0) a.sigma_full[g] = sigma;
    }
}

// One system (node g, sweep-table row pos) of the problem `a`, in this warp's
// shared-memory slot `base` laid out for up to kl neighbours (kl >= a.k, or
// >= the node's neighbour count).
template <typename T, typename O>
__device__ __forceinline__ void solve_system(const SolveArgs& a, const SweepTables<O>& tab, int64_t pos, int g,
                                             unsigned char* base, int kl, int lane) {
    const int k = a.k;
    const int ld = kl + 1;
    T* A = reinterpret_cast<T*>(base);
    double* c = reinterpret_cast<double*>(base + ((size_t)kl * ld * sizeof(T) + 15) / 16 * 16);
    double* w = c + kl;
    T* rhs = reinterpret_cast<T*>(w + kl);
    NbInfo* info = reinterpret_cast<NbInfo*>(reinterpret_cast<unsigned char*>(rhs) + ((size_t)kl * sizeof(T) + 15) / 16 * 16);
    const GridDev& G = a.grid;
    const double sill = a.vario.sill;
    const double prior_sd = sqrt(sill);
    {
        const int n = a.cnt[g];
        if (n < a.nmin) {
            write_row<O>(a, tab, pos, g, n, info, w, prior_sd, SGS_NODE_PRIOR_NMIN_, lane);
            return;
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
        for (int r = 0; r < n; ++r) {
            const NbInfo ir = info[r];
            if (ir.did >= 0) continue;
            for (int q = lane; q <= r; q += 32) {
                const NbInfo iq = info[q];
                if (iq.did < 0) A[r * ld + q] = (T)kcov(a, iq, ir);
            }
        }
        {
            int* dl = reinterpret_cast<int*>(rhs);
            const int nd = collect_data(info, n, dl, lane);
            for (int item = lane; item < nd * n; item += 32) {
                const int da = dl[item / n], q = item % n;
                const NbInfo iq = info[q];
                if (iq.did >= 0 && q > da) continue;
                A[(da >= q ? da : q) * ld + (da >= q ? q : da)] = (T)kcov(a, iq, info[da]);
            }
        }
        __syncwarp();

        const bool ok = warp_cholesky<T>(A, ld, n, (T)a.tau, lane);
        if (ok) {
            for (int q = lane; q < n; q += 32) rhs[q] = (T)c[q];
            __syncwarp();
            warp_chol_solve<T>(A, ld, n, rhs, lane);
            for (int q = lane; q < n; q += 32) w[q] = (double)rhs[q];
            __syncwarp();
        }
        if (!ok) {
            write_row<O>(a, tab, pos, g, n, info, w, prior_sd, SGS_NODE_PRIOR_SINGULAR_, lane);
            return;
        }
        double wc = 0.0;
        for (int q = lane; q < n; q += 32) wc += w[q] * c[q];
        wc = warp_sum(wc);
        const double var = sill - wc;
        write_row<O>(a, tab, pos, g, n, info, w, sqrt(var > 0.0 ? var : 0.0), SGS_NODE_KRIGED_, lane);
        __syncwarp();
    }
}

// The plain FP64 path (T = double): FP64 LHS, Cholesky and weights.  O is the
// table type: double for the FP64 path, float (hi, lo pairs) when it re-solves
// the systems the FP32 path queued.  With a.list set, solves only the queued
// positions.
template <typename T, typename O>
__global__ void __launch_bounds__(SOLVE_WARPS * 32) solve_kernel(const SolveArgs a, const SweepTables<O> tab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char* base = smem + (size_t)wib * warp_smem_bytes<T>(a.k);
    const int64_t count = a.list ? (int64_t)*a.nfallback : a.P;
    const int64_t nwarps = (int64_t)gridDim.x * SOLVE_WARPS;
    for (int64_t it = (int64_t)blockIdx.x * SOLVE_WARPS + wib; it < count; it += nwarps) {
        const int64_t pos = a.list ? (int64_t)a.list[it] : it;
        solve_system<T, O>(a, tab, pos, a.order[pos], base, a.k, lane);
    }
}

// Batch form: desc[0] positions list[desc[1] ...] of the level-ordered
// global node list `order`, each solved with its domain's descriptor (domain
// d owns global node ids [noff[d], noff[d+1])); shared memory laid out for kl
// neighbours.
template <typename T, typename O>
__global__ void __launch_bounds__(SOLVE_WARPS * 32)
solve_batch_kernel(const SolveArgs* __restrict__ doms, const int64_t* __restrict__ noff, int ndom,
                   const int32_t* __restrict__ order, const int32_t* __restrict__ list,
                   const int32_t* __restrict__ desc, int kl, const SweepTables<O> tab) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ SolveArgs s_dom[SOLVE_WARPS];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char* base = smem + (size_t)wib * warp_smem_bytes<T>(kl);
    const int64_t n = desc[0];
    const int32_t* lst = list + desc[1];
    const int64_t nwarps = (int64_t)gridDim.x * SOLVE_WARPS;
    int64_t lo = 0, hi = 0;
    for (int64_t it = (int64_t)blockIdx.x * SOLVE_WARPS + wib; it < n; it += nwarps) {
        const int64_t pos = lst[it];
        const int64_t gg = order[pos];
        if (gg < lo || gg >= hi) {
            const int d = find_domain(noff, ndom, gg);
            lo = noff[d];
            hi = noff[d + 1];
            __syncwarp();
            warp_copy_struct(&s_dom[wib], &doms[d], lane);
            __syncwarp();
        }
        solve_system<T, O>(s_dom[wib], tab, pos, (int)(gg - lo), base, kl, lane);
    }
}

template <typename T, typename O>
static cudaError_t launch_solve(const SolveArgs& a, const SweepTables<O>& t, cudaStream_t s) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = warp_smem_bytes<T>(a.k) * SOLVE_WARPS;
    cudaError_t e = cudaFuncSetAttribute(solve_kernel<T, O>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, solve_kernel<T, O>, SOLVE_WARPS * 32, smem);
    if (per_sm < 1) per_sm = 1;
    int64_t want = a.list ? (int64_t)nsm * per_sm : (a.P + SOLVE_WARPS - 1) / SOLVE_WARPS;
    int blocks = (int)(want < (int64_t)nsm * per_sm ? want : (int64_t)nsm * per_sm);
    if (blocks < 1) blocks = 1;
    solve_kernel<T, O><<<blocks, SOLVE_WARPS * 32, smem, s>>>(a, t);
    return cudaGetLastError();
}

cudaError_t launch_solve_fp64(const SolveArgs& a, const SweepTables<double>& t, cudaStream_t s) {
    return launch_solve<double, double>(a, t, s);
}

// ---------------------------------------------------------------------------
// FP32 path.  One warp per system, lane l owning rows l and l + 32 of the
// system in registers.  The LHS is normalized by the sill (a correlation
// matrix: pivots in (0, 1], weights unchanged) and kept in shared memory as
// double-FP32 pairs (hi + lo, about 48 bits); grid-grid entries come from the
// (hi, lo) lag table, entries involving a datum from one FP64 evaluation each,
// packed 32 per pass.  Its FP32 copy is inverted in registers by the
// Gauss-Jordan sweep operator (Goodnight 1979; no pivoting, which is stable
// for symmetric positive definite matrices, and whose k-th pivot is the same
// Schur complement a Cholesky factorization would test).  Every solve is then
// a lane-parallel matrix-vector product instead of a sequential triangular
// solve.  The weights are refined against the double-FP32 LHS: the residual
// r = c - K w is accumulated with compensated (Dot2) FP32 arithmetic, which
// carries the accuracy of an FP64 residual without GB300's narrow FP64 pipe.
// Weights, sigma^2 = sill (1 - w'c) and b0 stay double-FP32 and are written as
// (hi, lo) pairs for the compensated sweep.  A system with a pivot below
// 1e-3 (near-singular: the canonical 1e-10 decision needs FP64) or whose
// refinement does not contract is queued for the FP64 kernel.
constexpr int SOLVE32_WARPS = 2;
// resident blocks per SM the FP32 solve is compiled for.  Systems of up to 48
// neighbours: 7 x 2 warps at 128 registers a thread (a few spilled values,
// measured 7 % faster than 6 blocks at 168 registers without spills, and
// ahead of 8 blocks); up to 32 neighbours: 8 blocks at under 100 registers;
// up to 64 neighbours hold two rows of 64 registers and get 4 blocks
constexpr int solve32_min_blocks(int nmax) { return nmax > 48 ? 4 : (nmax > 32 ? 7 : 8); }

template <int NMAX>
struct Smem32 {
    // the double-FP32 LHS as its packed lower triangle (row r at r(r+1)/2):
    // half the shared memory of the square, so that the register file, not
    // shared memory, bounds the resident warps
    static constexpr size_t K = (size_t)NMAX * (NMAX + 1) / 2 * sizeof(DF);
    static constexpr size_t C = (size_t)NMAX * sizeof(DF);
    static constexpr size_t W = (size_t)NMAX * sizeof(DF);
    static constexpr int CB = NMAX > 32 ? 64 : 32;  // one entry per owned row
    static constexpr size_t V = (size_t)CB * sizeof(float);
    static constexpr size_t COL = 2 * (size_t)CB * sizeof(float);
    static constexpr size_t INFO = (size_t)NMAX * sizeof(NbInfo);
    static constexpr size_t LIN = (size_t)NMAX * sizeof(int);
    static constexpr size_t bytes = K + C + W + V + COL + INFO + LIN;
    static_assert(K % 16 == 0 && bytes % 16 == 0, "16-byte aligned per-warp layout");
};

// packed lower-triangle index of entry (i, j) of a symmetric matrix
__device__ __forceinline__ int tri(int i, int j) { return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// normalized double-FP32 covariance between two points of the augmented set
__device__ __forceinline__ DF kcov2n(const SolveArgs& a, const NbInfo& p, const NbInfo& q) {
    if (p.did < 0 && q.did < 0) {
        const CovLut& t = a.lut;
        const int L0 = q.c0 - p.c0, L1 = q.c1 - p.c1, L2 = q.c2 - p.c2;
        if (t.c2 != nullptr && L0 >= -t.e[0] && L0 <= t.e[0] && L1 >= -t.e[1] && L1 <= t.e[1] && L2 >= -t.e[2] &&
            L2 <= t.e[2]) {
            const float2 v = t.c2[(L0 + t.e[0]) + t.w[0] * ((L1 + t.e[1]) + t.w[1] * (L2 + t.e[2]))];
            return {v.x, v.y};
        }
    }
    return df_from_double(kcov(a, p, q) * a.inv_sill);
}

__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);
    return df_fast_two_sum(p, __fadd_rn(e, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi))));
}

// One system (node g, sweep-table row pos) of the problem `a` with at most
// NMAX neighbours, in this warp's shared-memory slot `base`.
template <int NMAX>
__device__ __forceinline__ void solve32_system(const SolveArgs& a, const SweepTables<float>& tab, int64_t pos, int g,
                                               unsigned char* base, int lane) {
    using S = Smem32<NMAX>;
    constexpr bool TWO = NMAX > 32;  // lanes own a second row
    DF* K = reinterpret_cast<DF*>(base);
    DF* c = reinterpret_cast<DF*>(base + S::K);
    DF* w = reinterpret_cast<DF*>(base + S::K + S::C);
    float* vec = reinterpret_cast<float*>(base + S::K + S::C + S::W);
    float* colb = reinterpret_cast<float*>(base + S::K + S::C + S::W + S::V);
    NbInfo* info = reinterpret_cast<NbInfo*>(base + S::K + S::C + S::W + S::V + S::COL);
    int* lin = reinterpret_cast<int*>(base + S::K + S::C + S::W + S::V + S::COL + S::INFO);
    const GridDev& G = a.grid;
    const int k = a.k;
    const DF sd_sill = df_sqrt(df_from_double(a.vario.sill));
    const float2* lut2 = a.lut.c2;
    const int lw0 = a.lut.w[0], lw1 = a.lut.w[1];
    const int lcentre = a.lut.e[0] + lw0 * (a.lut.e[1] + lw1 * a.lut.e[2]);
    const int ltotal = lw0 * lw1 * a.lut.w[2];
    const int i0 = lane, i1 = lane + 32;
    {
        const int n = a.cnt[g];
        int status = SGS_NODE_KRIGED_;
        DF sigma = sd_sill;
        if (n < a.nmin) {
            status = SGS_NODE_PRIOR_NMIN_;
        } else {
            NbInfo self;
            cell_of(G, g, self.c0, self.c1, self.c2);
            self.did = -1;
            bool fits = true;  // every grid neighbour within half the table's extents
            for (int q = lane; q < n; q += 32) {
                const int id = a.nbr[(int64_t)g * k + q];
                NbInfo in;
                if (id < G.N) {
                    cell_of(G, id, in.c0, in.c1, in.c2);
                    in.did = -1;
                    fits = fits && 2 * abs(in.c0 - self.c0) <= a.lut.e[0] && 2 * abs(in.c1 - self.c1) <= a.lut.e[1] &&
                           2 * abs(in.c2 - self.c2) <= a.lut.e[2];
                } else {
                    in.c0 = in.c1 = in.c2 = 0;
                    in.did = id - (int)G.N;
                }
                info[q] = in;
                // linear lag-table offset of the cell relative to the query: the
                // table index of a grid pair (q, r) is centre + lin[r] - lin[q]
                lin[q] = in.did < 0 ? (in.c0 - self.c0) + lw0 * ((in.c1 - self.c1) + lw1 * (in.c2 - self.c2)) : 0;
            }
            fits = __all_sync(FULL_MASK, fits);
            __syncwarp();
            if (lut2 && fits) {
                // every pairwise lag of grid neighbours is inside the table (a
                // plan's table spans twice the search template, so this always
                // holds there); the clamp only keeps reads in bounds.  Lane l
                // fills columns l and l + 32 of every row; it keeps their
                // offsets in registers, and row r's offset and kind come by
                // shuffle and ballot mask instead of shared-memory loads.
                const bool gA = lane < n && info[lane].did < 0;
                const bool gB = lane + 32 < n && info[lane + 32].did < 0;
                const int linA = gA ? lin[lane] : 0, linB = gB ? lin[lane + 32] : 0;
                const unsigned mA = __ballot_sync(FULL_MASK, gA), mB = __ballot_sync(FULL_MASK, gB);
                if (gA) {
                    const float2 v = lut2[min(max(lcentre - linA, 0), ltotal - 1)];
                    c[lane] = {v.x, v.y};
                } else if (lane < n) {
                    c[lane] = kcov2n(a, info[lane], self);
                }
                if (gB) {
                    const float2 v = lut2[min(max(lcentre - linB, 0), ltotal - 1)];
                    c[lane + 32] = {v.x, v.y};
                } else if (lane + 32 < n) {
                    c[lane + 32] = kcov2n(a, info[lane + 32], self);
                }
                for (int r = 0; r < n; ++r) {
                    const int linr = __shfl_sync(FULL_MASK, r < 32 ? linA : linB, r & 31);
                    if (!(((r < 32 ? mA : mB) >> (r & 31)) & 1u)) continue;  // warp-uniform: row r is a datum
                    const int base = lcentre + linr;
                    DF* Kr = K + r * (r + 1) / 2;
                    if (gA && lane <= r) {
                        const float2 v = lut2[min(max(base - linA, 0), ltotal - 1)];
                        Kr[lane] = {v.x, v.y};
                    }
                    if (gB && lane + 32 <= r) {
                        const float2 v = lut2[min(max(base - linB, 0), ltotal - 1)];
                        Kr[lane + 32] = {v.x, v.y};
                    }
                }
            } else {
                for (int q = lane; q < n; q += 32) c[q] = kcov2n(a, info[q], self);
                for (int r = 0; r < n; ++r) {
                    const NbInfo ir = info[r];
                    if (ir.did >= 0) continue;
                    for (int q = lane; q <= r; q += 32) {
                        const NbInfo iq = info[q];
                        if (iq.did < 0) K[r * (r + 1) / 2 + q] = kcov2n(a, iq, ir);
                    }
                }
            }
            {
                int* dl = reinterpret_cast<int*>(vec);
                const int nd = collect_data(info, n, dl, lane);
                for (int item = lane; item < nd * n; item += 32) {
                    const int da = dl[item / n], q = item % n;
                    const NbInfo iq = info[q];
                    if (iq.did >= 0 && q > da) continue;  // data-data pair once
                    K[tri(da, q)] = df_from_double(kcov(a, iq, info[da]) * a.inv_sill);
                }
            }
            __syncwarp();
            // ---- rows of the FP32 LHS into registers (identity padding) ----
            float R0[NMAX], R1[TWO ? NMAX : 1];
            const int t0 = i0 * (i0 + 1) / 2, t1 = i1 * (i1 + 1) / 2;  // own rows' starts
#pragma unroll
            for (int j = 0; j < NMAX; ++j) {
                R0[j] = (i0 < n && j < n) ? K[j <= i0 ? t0 + j : j * (j + 1) / 2 + i0].hi : (i0 == j ? 1.0f : 0.0f);
                if (TWO)
                    R1[j] = (i1 < n && j < n) ? K[j <= i1 ? t1 + j : j * (j + 1) / 2 + i1].hi : (i1 == j ? 1.0f : 0.0f);
            }
            // ---- Gauss-Jordan sweep with column rotation: R -> -K^-1 ----
            // At step kk register j holds column (kk + j) mod NMAX, so the pivot
            // column is always register 0 and every register index is static
            // in a rolled loop (a fully unrolled sweep overflows the
            // instruction cache).  The pivot column is broadcast through shared
            // memory already rotated (slot j <- row (kk + j + 1) mod NMAX, which
            // by symmetry is row kk's entry for register j + 1).  NMAX steps
            // bring the columns back in place; padding pivots are exactly 1.
            bool ok = true;
            const bool own0 = i0 < NMAX, own1 = TWO && i1 < NMAX;
#pragma unroll 1
            for (int kk = 0; kk < NMAX; ++kk) {
                const float d = __shfl_sync(FULL_MASK, kk < 32 ? R0[0] : R1[0], kk & 31);
                if (!(d > 1e-3f)) {  // warp-uniform
                    ok = false;
                    break;
                }
                // the inverse is a preconditioner only: the approximate
                // reciprocal (pivots lie in (1e-3, 1], no denormals) is enough
                float inv;
                asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(d));
                float* cb = colb + (kk & 1) * S::CB;
                if (own0) {
                    int p = i0 - kk - 1;
                    cb[p < 0 ? p + NMAX : p] = R0[0];
                }
                if (own1) {
                    int p = i1 - kk - 1;
                    cb[p < 0 ? p + NMAX : p] = R1[0];
                }
                __syncwarp();
                // owner row: A[k][j] / d == A[k][j] - (1 - 1/d) A[k][j]
                const float a0 = i0 == kk ? __fsub_rn(1.0f, inv) : __fmul_rn(R0[0], inv);
                const float a1 = TWO ? (i1 == kk ? __fsub_rn(1.0f, inv) : __fmul_rn(R1[0], inv)) : 0.0f;
                const float4* cb4 = reinterpret_cast<const float4*>(cb);  // 16-byte aligned
#pragma unroll
                for (int j4 = 0; j4 < NMAX / 4; ++j4) {
                    const float4 v = cb4[j4];
                    const float akv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int j = 4 * j4 + t;
                        if (j < NMAX - 1) {
                            R0[j] = __fmaf_rn(-a0, akv[t], R0[j + 1]);
                            if (TWO) R1[TWO ? j : 0] = __fmaf_rn(-a1, akv[t], R1[TWO ? j + 1 : 0]);
                        }
                    }
                }
                R0[NMAX - 1] = i0 == kk ? -inv : a0;
                if (TWO) R1[TWO ? NMAX - 1 : 0] = i1 == kk ? -inv : a1;
            }
            bool accept = ok;
            if (accept) {
                float s0 = 0.0f, s1 = 0.0f;
                if (a.w_init) {
                    // learned warm start: the refinement below starts from the
                    // network's prediction and must meet the same tolerance
                    if (i0 < n) s0 = a.w_init[(int64_t)g * k + i0];
                    if (TWO && i1 < n) s1 = a.w_init[(int64_t)g * k + i1];
                } else {
                    // w = K^-1 c = -R c
                    for (int q = lane; q < S::CB; q += 32) vec[q] = q < n ? c[q].hi : 0.0f;
                    __syncwarp();
#pragma unroll
                    for (int j = 0; j < NMAX; ++j) {
                        const float v = vec[j];
                        s0 = __fmaf_rn(-R0[j], v, s0);
                        if (TWO) s1 = __fmaf_rn(-R1[j], v, s1);
                    }
                }
                DF w0 = {s0, 0.0f}, w1 = {s1, 0.0f};
                if (i0 < n) w[i0] = w0;
                if (TWO && i1 < n) w[i1] = w1;
                __syncwarp();
                float prev = 0.0f, last = 0.0f;
                const int steps = a.refine_steps;
                // weights and residual the variance is evaluated with: the last
                // residual computed (it also drives the last correction)
                DF sw0 = w0, sw1 = w1;
                float sr0 = 0.0f, sr1 = 0.0f;
                // the correction computed from that residual (0 when none was)
                float sd0 = 0.0f, sd1 = 0.0f;
                // largest starting weight, for the one-correction estimate below
                float wmax = fmaxf(i0 < n ? fabsf(w0.hi) : 0.0f, TWO && i1 < n ? fabsf(w1.hi) : 0.0f);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) wmax = fmaxf(wmax, __shfl_xor_sync(FULL_MASK, wmax, o));
                bool early = false;
                for (int s = 0;; ++s) {
                    // residual r = c - K w in double-FP32, own rows
                    float r0 = 0.0f, r1 = 0.0f;
                    // row i of the packed triangle: entries t_i + j for j <= i,
                    // then down column i (j (j + 1) / 2 + i) for j > i
                    if (i0 < n) {
                        DFAcc acc;
                        acc.init(c[i0]);
                        int jt = 0;  // j (j + 1) / 2
                        for (int j = 0; j < n; ++j) {
                            acc.add_prod(df_neg(K[j <= i0 ? t0 + j : jt + i0]), w[j]);
                            jt += j + 1;
                        }
                        r0 = acc.value().hi;
                    }
                    if (TWO && i1 < n) {
                        DFAcc acc;
                        acc.init(c[i1]);
                        int jt = 0;
                        for (int j = 0; j < n; ++j) {
                            acc.add_prod(df_neg(K[j <= i1 ? t1 + j : jt + i1]), w[j]);
                            jt += j + 1;
                        }
                        r1 = acc.value().hi;
                    }
                    sw0 = w0;
                    sw1 = w1;
                    sr0 = r0;
                    sr1 = r1;
                    sd0 = sd1 = 0.0f;
                    if (s == steps) break;  // steps == 0: no correction
                    __syncwarp();
                    vec[i0] = r0;
                    if (TWO) vec[i1] = r1;
                    __syncwarp();
                    float d0 = 0.0f, d1 = 0.0f;
#pragma unroll
                    for (int j = 0; j < NMAX; ++j) {
                        const float v = vec[j];
                        d0 = __fmaf_rn(-R0[j], v, d0);
                        if (TWO) d1 = __fmaf_rn(-R1[j], v, d1);
                    }
                    float dmax = 0.0f;
                    sd0 = i0 < n ? d0 : 0.0f;
                    sd1 = TWO && i1 < n ? d1 : 0.0f;
                    if (i0 < n) {
                        const DF t = df_two_sum(w0.hi, d0);
                        w0 = df_fast_two_sum(t.hi, __fadd_rn(t.lo, w0.lo));
                        w[i0] = w0;
                        dmax = fabsf(d0);
                    }
                    if (TWO && i1 < n) {
                        const DF t = df_two_sum(w1.hi, d1);
                        w1 = df_fast_two_sum(t.hi, __fadd_rn(t.lo, w1.lo));
                        w[i1] = w1;
                        dmax = fmaxf(dmax, fabsf(d1));
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(FULL_MASK, dmax, o));
                    prev = last;
                    last = dmax;
                    __syncwarp();
                    if (s + 1 == steps) break;  // the final weights need no residual
                    // One correction is enough when the start was already good:
                    // the start's error is about |d| and the contraction factor
                    // of the FP32 inverse about |d| / |w|, so the corrected
                    // weights are off by about |d|^2 / |w| (measured on the
                    // 200x200x100 anisotropic systems: within a factor 4 of the
                    // true error, which is ~1e-12 there).
                    if (s == 0 && !a.w_init && last * last <= 1e-10f * wmax && isfinite(last)) {
                        early = true;
                        break;
                    }
                    // Later corrections: stop as soon as the contraction test
                    // below passes (a warm start from a prediction needs two).
                    if (s >= 1 && prev > 0.0f && last < 0.5f * prev && (last / prev) * last <= 1e-9f &&
                        isfinite(last)) {
                        early = true;
                        break;
                    }
                }
                // the remaining error is about the contraction factor times the
                // last correction
                if (early) {
                    accept = true;
                } else if (a.refine_steps >= 2) {
                    const float rho = prev > 0.0f ? last / prev : 0.0f;
                    accept = rho < 0.5f && rho * last <= 1e-9f && isfinite(last);
                } else {
                    accept = isfinite(last);
                }
                if (accept) {
                    // sigma^2 = sill S(w), S(w) = 1 - w'c - w'r with r = c - K w:
                    // equal to 1 - w'c at the exact weights, but stationary
                    // there (its error is (w - w*)' K (w - w*)), so it stays
                    // accurate where the variance cancels to ~0 (a node on a
                    // datum), where sqrt would magnify any error.  It is taken
                    // at the final weights w + d: S(w + d) = S(w) - 2 d'r +
                    // d' K d, and K d = r up to the inverse's error, so
                    // S(w + d) = S(w) - d'r with an error of order
                    // |d| |r| x that error.
                    DFAcc acc;
                    acc.init({0.0f, 0.0f});
                    if (i0 < n) {
                        acc.add_prod(sw0, df_add(c[i0], {sr0, 0.0f}));
                        acc.add_prod({sd0, 0.0f}, {sr0, 0.0f});
                    }
                    if (TWO && i1 < n) {
                        acc.add_prod(sw1, df_add(c[i1], {sr1, 0.0f}));
                        acc.add_prod({sd1, 0.0f}, {sr1, 0.0f});
                    }
                    const DF wc = warp_sum_df(acc.value());
                    sigma = df_mul(sd_sill, df_sqrt(df_add({1.0f, 0.0f}, df_neg(wc))));
                }
            }
            if (!accept) {
                if (lane == 0) a.fallback[atomicAdd(a.nfallback, 1)] = (int32_t)pos;
                __syncwarp();
                return;
            }
            if (a.w_init && a.n_warm && lane == 0) atomicAdd(a.n_warm, 1ull);
        }
        // ---- table row: grid neighbours with (hi, lo) weights, data folded into b0
        int m = 0;
        const int64_t row = table_row(tab, pos, k);
        DFAcc b0acc;
        b0acc.init({0.0f, 0.0f});
        float l1 = 0.0f;
        if (status == SGS_NODE_KRIGED_) {
            for (int b = 0; b < n; b += 32) {
                const int q = b + lane;
                const bool isgrid = q < n && info[q].did < 0;
                const unsigned bal = __ballot_sync(FULL_MASK, isgrid);
                if (isgrid) {
                    const int j = m + __popc(bal & lanemask_lt());
                    tab.idx[row + j] = a.nbr[(int64_t)g * k + q] + (int32_t)a.node0;
                    reinterpret_cast<float2*>(tab.w)[row + j] = make_float2(w[q].hi, w[q].lo);
                    l1 += fabsf(w[q].hi);
                } else if (q < n) {
                    b0acc.add_prod(w[q], df_from_double(a.data_val[info[q].did] - a.mu));
                }
                m += __popc(bal);
            }
            if (a.wl1_max) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) l1 += __shfl_xor_sync(FULL_MASK, l1, o);
                if (lane == 0) atomicMax(a.wl1_max, __float_as_uint(l1));
            }
        }
        const DF b0 = warp_sum_df(b0acc.value());
        if (a.ind_wsum)
            write_indicator_sums(a, pos, n, info, status == SGS_NODE_KRIGED_,
                                 [&](int q) { return (double)w[q].hi + (double)w[q].lo; }, lane);
        if (lane == 0) {
            if (a.sum_m) atomicAdd(a.sum_m, (unsigned long long)m);
            tab.node[pos] = g + (int32_t)a.node0;
            tab.m[pos] = m;
            reinterpret_cast<float2*>(tab.b0)[pos] = make_float2(b0.hi, b0.lo);
            reinterpret_cast<float2*>(tab.sigma)[pos] = make_float2(sigma.hi, sigma.lo);
            a.status[g] = (int8_t)status;
        }
        if (a.w_full) {
            for (int q = lane; q < k; q += 32)
                a.w_full[(int64_t)g * k + q] =
                    (status == SGS_NODE_KRIGED_ && q < n) ? (double)w[q].hi + (double)w[q].lo : 0.0;
            if (lane == 0) a.sigma_full[g] = (double)sigma.hi + (double)sigma.lo;
        }
        __syncwarp();
    }
}

template <int NMAX>
__global__ void __launch_bounds__(SOLVE32_WARPS * 32, solve32_min_blocks(NMAX)) solve_fp32_kernel(const SolveArgs a, const SweepTables<float> tab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char* base = smem + (size_t)wib * Smem32<NMAX>::bytes;
    const int64_t nwarps = (int64_t)gridDim.x * SOLVE32_WARPS;
    for (int64_t pos = (int64_t)blockIdx.x * SOLVE32_WARPS + wib; pos < a.P; pos += nwarps)
        solve32_system<NMAX>(a, tab, pos, a.order[pos], base, lane);
}

// Batch form of solve_fp32_kernel: desc[0] positions list[desc[1] ...]
// (systems with at most NMAX neighbours, from any domain), each solved with
// its domain's descriptor.
template <int NMAX>
__global__ void __launch_bounds__(SOLVE32_WARPS * 32, solve32_min_blocks(NMAX))
solve_fp32_batch_kernel(const SolveArgs* __restrict__ doms, const int64_t* __restrict__ noff, int ndom,
                        const int32_t* __restrict__ order, const int32_t* __restrict__ list,
                        const int32_t* __restrict__ desc, const SweepTables<float> tab) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ SolveArgs s_dom[SOLVE32_WARPS];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char* base = smem + (size_t)wib * Smem32<NMAX>::bytes;
    const int64_t n = desc[0];
    const int32_t* lst = list + desc[1];
    const int64_t nwarps = (int64_t)gridDim.x * SOLVE32_WARPS;
    int64_t lo = 0, hi = 0;
    for (int64_t it = (int64_t)blockIdx.x * SOLVE32_WARPS + wib; it < n; it += nwarps) {
        const int64_t pos = lst[it];
        const int64_t gg = order[pos];
        if (gg < lo || gg >= hi) {
            const int d = find_domain(noff, ndom, gg);
            lo = noff[d];
            hi = noff[d + 1];
            __syncwarp();
            warp_copy_struct(&s_dom[wib], &doms[d], lane);
            __syncwarp();
        }
        solve32_system<NMAX>(s_dom[wib], tab, pos, (int)(gg - lo), base, lane);
    }
}

template <int NMAX>
static cudaError_t launch_solve32(const SolveArgs& a, const SweepTables<float>& t, cudaStream_t s) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = Smem32<NMAX>::bytes * SOLVE32_WARPS;
    cudaError_t e = cudaFuncSetAttribute(solve_fp32_kernel<NMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, solve_fp32_kernel<NMAX>, SOLVE32_WARPS * 32, smem);
    if (per_sm < 1) per_sm = 1;
    int64_t want = (a.P + SOLVE32_WARPS - 1) / SOLVE32_WARPS;
    int blocks = (int)(want < (int64_t)nsm * per_sm ? want : (int64_t)nsm * per_sm);
    if (blocks < 1) blocks = 1;
    solve_fp32_kernel<NMAX><<<blocks, SOLVE32_WARPS * 32, smem, s>>>(a, t);
    return cudaGetLastError();
}

cudaError_t launch_solve_fp32(const SolveArgs& a, const SweepTables<float>& t, cudaStream_t s) {
    if (a.k <= 16) return launch_solve32<16>(a, t, s);
    if (a.k <= 32) return launch_solve32<32>(a, t, s);
    if (a.k <= 48) return launch_solve32<48>(a, t, s);
    return launch_solve32<64>(a, t, s);
}

cudaError_t launch_solve_fp64_into_fp32(const SolveArgs& a, const SweepTables<float>& t, cudaStream_t s) {
    return launch_solve<double, float>(a, t, s);
}

// ---------------------------------------------------------------------------
// Batches of domains.  Persistent grids (as many blocks as fit on the SMs)
// walk a device-resident list whose length is read on the device, so the
// launches need nothing from the host and can be captured in a graph.
template <int NMAX>
static cudaError_t launch_solve32_batch(const SolveArgs* doms, const int64_t* noff, int ndom, const int32_t* order,
                                        const int32_t* list, const int32_t* desc, const SweepTables<float>& t,
                                        int nsm, cudaStream_t s) {
    const size_t smem = Smem32<NMAX>::bytes * SOLVE32_WARPS;
    cudaError_t e = cudaFuncSetAttribute(solve_fp32_batch_kernel<NMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, solve_fp32_batch_kernel<NMAX>, SOLVE32_WARPS * 32, smem);
    if (per_sm < 1) per_sm = 1;
    solve_fp32_batch_kernel<NMAX><<<nsm * per_sm, SOLVE32_WARPS * 32, smem, s>>>(doms, noff, ndom, order, list, desc, t);
    return cudaGetLastError();
}

cudaError_t launch_solve_fp32_batch(int nmax, const SolveArgs* doms, const int64_t* noff, int ndom,
                                    const int32_t* order, const int32_t* list, const int32_t* desc,
                                    const SweepTables<float>& t, int nsm, cudaStream_t s) {
    switch (nmax) {
        case 8: return launch_solve32_batch<8>(doms, noff, ndom, order, list, desc, t, nsm, s);
        case 16: return launch_solve32_batch<16>(doms, noff, ndom, order, list, desc, t, nsm, s);
        case 32: return launch_solve32_batch<32>(doms, noff, ndom, order, list, desc, t, nsm, s);
        case 48: return launch_solve32_batch<48>(doms, noff, ndom, order, list, desc, t, nsm, s);
        case 64: return launch_solve32_batch<64>(doms, noff, ndom, order, list, desc, t, nsm, s);
        default: return cudaErrorInvalidValue;
    }
}

template <typename O>
static cudaError_t launch_solve64_batch(int kl, const SolveArgs* doms, const int64_t* noff, int ndom,
                                        const int32_t* order, const int32_t* list, const int32_t* desc,
                                        const SweepTables<O>& t, int nsm, cudaStream_t s) {
    if (kl < 1 || kl > KMAX) return cudaErrorInvalidValue;
    const size_t smem = warp_smem_bytes<double>(kl) * SOLVE_WARPS;
    cudaError_t e = cudaFuncSetAttribute(solve_batch_kernel<double, O>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, solve_batch_kernel<double, O>, SOLVE_WARPS * 32, smem);
    if (per_sm < 1) per_sm = 1;
    solve_batch_kernel<double, O><<<nsm * per_sm, SOLVE_WARPS * 32, smem, s>>>(doms, noff, ndom, order, list, desc, kl, t);
    return cudaGetLastError();
}

cudaError_t launch_solve_fp64_batch(int kl, const SolveArgs* doms, const int64_t* noff, int ndom,
                                    const int32_t* order, const int32_t* list, const int32_t* desc,
                                    const SweepTables<double>& t, int nsm, cudaStream_t s) {
    return launch_solve64_batch<double>(kl, doms, noff, ndom, order, list, desc, t, nsm, s);
}

cudaError_t launch_solve_fp64_into_fp32_batch(int kl, const SolveArgs* doms, const int64_t* noff, int ndom,
                                              const int32_t* order, const int32_t* list, const int32_t* desc,
                                              const SweepTables<float>& t, int nsm, cudaStream_t s) {
    return launch_solve64_batch<float>(kl, doms, noff, ndom, order, list, desc, t, nsm, s);
}

// ---------------------------------------------------------------------------
__global__ void tables_to_fp64_kernel(const SweepTables<float> src, SweepTables<double> dst, int64_t P,
                                      int64_t entries) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < entries; i += stride)
        dst.w[i] = (double)src.w[2 * i] + (double)src.w[2 * i + 1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P; i += stride) {
        dst.b0[i] = (double)src.b0[2 * i] + (double)src.b0[2 * i + 1];
        dst.sigma[i] = (double)src.sigma[2 * i] + (double)src.sigma[2 * i + 1];
    }
}

cudaError_t launch_tables_to_fp64(const SweepTables<float>& src, SweepTables<double>& dst, int64_t P, int64_t entries,
                                  cudaStream_t s) {
    dst.node = src.node;
    dst.m = src.m;
    dst.idx = src.idx;
    dst.off = src.off;
    const int64_t n = entries > P ? entries : P;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 65535) blocks = 65535;
    if (blocks < 1) blocks = 1;
    tables_to_fp64_kernel<<<blocks, 256, 0, s>>>(src, dst, P, entries);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
__global__ void fill_lut_kernel(const GridDev G, const VarioDev v, const CovLut t, double* c64, float2* c2,
                                int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int L0 = (int)(i % t.w[0]) - t.e[0];
        const int64_t r = i / t.w[0];
        const int L1 = (int)(r % t.w[1]) - t.e[1];
        const int L2 = (int)(r / t.w[1]) - t.e[2];
        const double c = cov_fp64(v, G.dim, dmul((double)L0, G.spacing[0]), dmul((double)L1, G.spacing[1]),
                                  G.dim == 3 ? dmul((double)L2, G.spacing[2]) : 0.0);
        if (c64) c64[i] = c;
        if (c2) {  // normalized by the sill, as (hi, lo) for the FP32 path
            const double cn = c / v.sill;
            const float hi = (float)cn;
            c2[i] = make_float2(hi, (float)(cn - (double)hi));
        }
    }
}

cudaError_t launch_fill_cov_lut(const GridDev& g, const VarioDev& v, CovLut lut, double* c64, float2* c2,
                                cudaStream_t s) {
    const int64_t total = (int64_t)lut.w[0] * lut.w[1] * lut.w[2];
    int blocks = (int)((total + 255) / 256);
    if (blocks > 65535) blocks = 65535;
    fill_lut_kernel<<<blocks, 256, 0, s>>>(g, v, lut, c64, c2, total);
    return cudaGetLastError();
}

}  // namespace sgs

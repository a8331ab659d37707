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
#include <algorithm>

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

// ---------------------------------------------------------------------------
// Full simple cokriging (SIS with a non-separable indicator covariance, e.g.
// structures of different ranges with their own coregionalization matrices):
// the reference's Kriging(f, prob) with a multivariate f solves, per node,
// one system over the n neighbours' L indicators (seqsim.jl:292-310).  LHS
// (nL x nL) blocks C(x_i - x_j), right-hand sides (nL x L) blocks
// C(x_i - x_0), C_ab(h) = sum_s coef[s][a][b] (sill_s - gamma_s(h)); FP64
// Cholesky by one warp with the canonical singular rule; then
//   p_t = prob_t + sum_i sum_a Lambda[(i, a), t] (I_a(x_i) - prob_a)
//       = cst_t + sum_{grid nbrs j} w[j][cat_j][t],
// the data's terms and every prob term folded into cst.
//
// Multivariate Gaussian simulation (GAUSS: a GaussianProcess whose function
// is such a model, seqsim.jl:277-290 Kriging(f, mu) with an MvNormal prior,
// predictprob's MvNormal conditional) solves the same systems with the L
// variables' values in place of indicators:
//   mu^_t = mu_t + sum_i sum_a Lambda[(i, a), t] (v_a(x_i) - mu_a)
//   S^    = C(0) - c' Lambda          (c: the right-hand sides, nL x L)
// and stores the lower Cholesky factor F of S^ (of C(0) for a node drawn from
// the prior): v = mu^ + F z.  F's rule: a pivot not above tau contributes
// nothing (its column of F is zero), so a conditional covariance that is zero
// up to rounding (a node on a datum) draws no noise.
constexpr int COK_WARPS = 2;

__host__ __device__ constexpr size_t cok_smem_per_warp(bool gauss) {
    return (size_t)COK_MAX * (COK_MAX + 1) * sizeof(double)                // LHS
           + (size_t)COK_MAX * IND_MAX_CAT * sizeof(double)                // right-hand sides -> weights
           + (size_t)COK_MAX * sizeof(double)                              // one column being solved
           + (gauss ? (size_t)COK_MAX * IND_MAX_CAT * sizeof(double) : 0)  // right-hand sides kept
           + (size_t)KMAX * 4 * sizeof(int);                               // neighbour cells / data ids
}

// lower Cholesky factor of the L x L symmetric matrix S (lower triangle,
// row-major) into F (full L x L, zero above the diagonal); pivots not above
// tau give zero columns
__device__ __forceinline__ void mv_factor(const double* S, int L, double tau, double* F) {
    for (int i = 0; i < L * L; ++i) F[i] = 0.0;
    for (int j = 0; j < L; ++j) {
        double d = S[j * L + j];
        for (int l = 0; l < j; ++l) d -= F[j * L + l] * F[j * L + l];
        if (!(d > tau)) continue;
        const double fjj = sqrt(d);
        F[j * L + j] = fjj;
        for (int i = j + 1; i < L; ++i) {
            double t = S[i * L + j];
            for (int l = 0; l < j; ++l) t -= F[i * L + l] * F[j * L + l];
            F[i * L + j] = t / fjj;
        }
    }
}

__device__ __forceinline__ double structure_cov(const VarioStructDev& v, int dim, double h0, double h1, double h2) {
    if (h0 == 0.0 && h1 == 0.0 && (dim == 2 || h2 == 0.0)) return v.sill;
    return v.sill - structure_gamma(v, dim, h0, h1, h2);
}

// lag between two points of the augmented set (grid cells or data), as the
// plain solve evaluates it
__device__ __forceinline__ void cok_lag(const SolveArgs& a, const int* ca, const int* cb, double* h) {
    const GridDev& G = a.grid;
    if (ca[3] < 0 && cb[3] < 0) {
        for (int j = 0; j < 3; ++j) h[j] = j < G.dim ? dmul((double)(cb[j] - ca[j]), G.spacing[j]) : 0.0;
        return;
    }
    double xa[3], xb[3];
    for (int j = 0; j < 3; ++j) {
        xa[j] = ca[3] < 0 ? (j < G.dim ? centroid(G, j, ca[j]) : 0.0) : a.data_xyz[3 * (int64_t)ca[3] + j];
        xb[j] = cb[3] < 0 ? (j < G.dim ? centroid(G, j, cb[j]) : 0.0) : a.data_xyz[3 * (int64_t)cb[3] + j];
        h[j] = dsub(xb[j], xa[j]);
    }
}

template <bool GAUSS>
__global__ void __launch_bounds__(COK_WARPS * 32) cok_solve_kernel(const SolveArgs a, const CokArgs c) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    unsigned char* base = smem + (size_t)wib * cok_smem_per_warp(GAUSS);
    double* A = reinterpret_cast<double*>(base);
    double* rhs = A + COK_MAX * (COK_MAX + 1);
    double* col = rhs + COK_MAX * IND_MAX_CAT;
    double* rhs0 = col + COK_MAX;  // GAUSS: the right-hand sides, kept
    int* cell = reinterpret_cast<int*>(GAUSS ? rhs0 + COK_MAX * IND_MAX_CAT : rhs0);  // [n][4]: c0, c1, c2,
                                                                                       // data id (-1: grid)
    const GridDev& G = a.grid;
    const int L = c.ncat, k = a.k, S = a.vario.ns;
    const int nwarps = gridDim.x * COK_WARPS;
    for (int64_t pos = (int64_t)blockIdx.x * COK_WARPS + wib; pos < a.P; pos += nwarps) {
        const int g = a.order[pos];
        const int n = a.cnt[g];
        const int m = n * L, ld = m + 1;
        int self[4];
        cell_of(G, g, self[0], self[1], self[2]);
        self[3] = -1;
        bool kriged = n >= a.nmin;
        if (kriged) {
            for (int q = lane; q < n; q += 32) {
                const int id = a.nbr[(int64_t)g * k + q];
                int* cq = cell + 4 * q;
                if (id < G.N) {
                    cell_of(G, id, cq[0], cq[1], cq[2]);
                    cq[3] = -1;
                } else {
                    cq[0] = cq[1] = cq[2] = 0;
                    cq[3] = id - (int)G.N;
                }
            }
            __syncwarp();
            // lower triangle of the LHS, one neighbour pair (i >= j) per lane
            for (int item = lane; item < n * (n + 1) / 2; item += 32) {
                int i = (int)((sqrt(8.0 * item + 1.0) - 1.0) * 0.5);
                while (i * (i + 1) / 2 > item) --i;
                while ((i + 1) * (i + 2) / 2 <= item) ++i;
                const int j = item - i * (i + 1) / 2;
                double h[3], cs[SGS_MAX_STRUCTURES];
                cok_lag(a, cell + 4 * j, cell + 4 * i, h);
                for (int s = 0; s < S; ++s) cs[s] = structure_cov(a.vario.st[s], G.dim, h[0], h[1], h[2]);
                for (int ai = 0; ai < L; ++ai)
                    for (int b = 0; b < L; ++b) {
                        const int r = i * L + ai, q = j * L + b;
                        if (q > r) continue;
                        double v = 0.0;
                        for (int s = 0; s < S; ++s) v += c.coef[(s * L + ai) * L + b] * cs[s];
                        A[r * ld + q] = v;
                    }
            }
            for (int i = lane; i < n; i += 32) {
                double h[3], cs[SGS_MAX_STRUCTURES];
                cok_lag(a, self, cell + 4 * i, h);
                for (int s = 0; s < S; ++s) cs[s] = structure_cov(a.vario.st[s], G.dim, h[0], h[1], h[2]);
                for (int ai = 0; ai < L; ++ai)
                    for (int t = 0; t < L; ++t) {
                        double v = 0.0;
                        for (int s = 0; s < S; ++s) v += c.coef[(s * L + ai) * L + t] * cs[s];
                        rhs[(i * L + ai) * IND_MAX_CAT + t] = v;
                        if constexpr (GAUSS) rhs0[(i * L + ai) * IND_MAX_CAT + t] = v;
                    }
            }
            __syncwarp();
            kriged = warp_cholesky<double>(A, ld, m, c.tau, lane);
        }
        if (kriged) {
            for (int t = 0; t < L; ++t) {
                for (int r = lane; r < m; r += 32) col[r] = rhs[r * IND_MAX_CAT + t];
                __syncwarp();
                warp_chol_solve<double>(A, ld, m, col, lane);
                for (int r = lane; r < m; r += 32) rhs[r * IND_MAX_CAT + t] = col[r];  // Lambda[(i, a), t]
                __syncwarp();
            }
        }
        if constexpr (GAUSS) {
            // conditional covariance C(0) - c' Lambda (the prior's C(0) for a
            // node without a system), lower triangle into col, then its factor
            for (int e = lane; e < L * L; e += 32) {
                const int t = e / L, u = e - t * L;
                if (u > t) continue;
                double v = 0.0;
                for (int s = 0; s < S; ++s) v += c.coef[(s * L + t) * L + u] * a.vario.st[s].sill;
                if (kriged)
                    for (int r = 0; r < m; ++r) v -= rhs0[r * IND_MAX_CAT + t] * rhs[r * IND_MAX_CAT + u];
                col[t * L + u] = v;
            }
            __syncwarp();
            if (lane == 0) {
                double F[IND_MAX_CAT * IND_MAX_CAT];
                mv_factor(col, L, c.tau, F);
                for (int i = 0; i < L * L; ++i) c.fac[pos * L * L + i] = F[i];
            }
            __syncwarp();
        }
        // outputs: grid neighbours compacted in neighbour order, prob and
        // data terms folded into cst
        int mg = 0;
        double cst[IND_MAX_CAT];
        for (int t = 0; t < IND_MAX_CAT; ++t) cst[t] = 0.0;
        if (kriged) {
            for (int b0 = 0; b0 < n; b0 += 32) {
                const int i = b0 + lane;
                const bool isgrid = i < n && cell[4 * i + 3] < 0;
                const unsigned bal = __ballot_sync(FULL_MASK, isgrid);
                if (i < n) {
                    if constexpr (GAUSS) {
                        const int d = isgrid ? -1 : cell[4 * i + 3];
                        for (int t = 0; t < L; ++t) {
                            double v = 0.0;
                            for (int ai = 0; ai < L; ++ai) {
                                const double lam = rhs[(i * L + ai) * IND_MAX_CAT + t];
                                v -= lam * c.prob[ai];
                                if (d >= 0) v += lam * c.data_val[(int64_t)d * L + ai];
                            }
                            cst[t] += v;
                        }
                    } else {
                        const int dcat = isgrid ? -1 : c.data_cat[cell[4 * i + 3]];
                        for (int t = 0; t < L; ++t) {
                            double v = 0.0;
                            for (int ai = 0; ai < L; ++ai) {
                                const double lam = rhs[(i * L + ai) * IND_MAX_CAT + t];
                                v -= lam * c.prob[ai];
                                if (ai == dcat) v += lam;
                            }
                            cst[t] += v;
                        }
                    }
                    if (isgrid) {
                        const int jj = mg + __popc(bal & lanemask_lt());
                        const int64_t e = pos * k + jj;
                        c.idx[e] = a.nbr[(int64_t)g * k + i];
                        for (int b = 0; b < L; ++b)
                            for (int t = 0; t < L; ++t)
                                c.w[(e * L + b) * L + t] = rhs[(i * L + b) * IND_MAX_CAT + t];
                    }
                }
                mg += __popc(bal);
            }
        }
        for (int t = 0; t < L; ++t) {
            double v = cst[t];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
            if (lane == 0) c.cst[pos * L + t] = c.prob[t] + v;
        }
        if (lane == 0) {
            c.m[pos] = mg;
            a.status[g] = (int8_t)(n < a.nmin ? SGS_NODE_PRIOR_NMIN_ : (kriged ? SGS_NODE_KRIGED_ : SGS_NODE_PRIOR_SINGULAR_));
        }
        __syncwarp();
    }
}

template <bool GAUSS>
static cudaError_t cok_solve(const SolveArgs& a, const CokArgs& c, cudaStream_t s) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = cok_smem_per_warp(GAUSS) * COK_WARPS;
    cudaError_t e =
        cudaFuncSetAttribute(cok_solve_kernel<GAUSS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cok_solve_kernel<GAUSS>, COK_WARPS * 32, smem);
    if (per_sm < 1) per_sm = 1;
    const int64_t want = (a.P + COK_WARPS - 1) / COK_WARPS;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)nsm * per_sm));
    cok_solve_kernel<GAUSS><<<blocks, COK_WARPS * 32, smem, s>>>(a, c);
    return cudaGetLastError();
}

cudaError_t launch_cok_solve(const SolveArgs& a, const CokArgs& c, bool gaussian, cudaStream_t s) {
    return gaussian ? cok_solve<true>(a, c, s) : cok_solve<false>(a, c, s);
}

// One level: one thread per (position, 4 realizations).
__global__ void __launch_bounds__(256) cok_level_kernel(const CokArgs c, const int32_t* __restrict__ node, int k,
                                                        int64_t p0, int64_t p1, int Rp, const double* __restrict__ u,
                                                        uint64_t seed, uint8_t* __restrict__ C) {
    const int cpn = Rp >> 2, L = c.ncat;
    IndArgs ia{};
    ia.ncat = L;
    for (int l = 0; l < IND_MAX_CAT; ++l) ia.prob[l] = c.prob[l];
    const int64_t total = (p1 - p0) * cpn;
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < total;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = p0 + it / cpn;
        const int ch = (int)(it % cpn);
        const int g = node[pos];
        const int m = c.m[pos];
        double p[4][IND_MAX_CAT];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int t = 0; t < IND_MAX_CAT; ++t) p[r][t] = t < L ? c.cst[pos * L + t] : 0.0;
        for (int j = 0; j < m; ++j) {
            const int64_t e = pos * k + j;
            const uint32_t cats = *reinterpret_cast<const uint32_t*>(C + (int64_t)c.idx[e] * Rp + 4 * ch);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int b = (int)((cats >> (8 * r)) & 0xffu);
                const double* wr = c.w + (e * L + b) * L;
#pragma unroll
                for (int t = 0; t < IND_MAX_CAT; ++t)
                    if (t < L) p[r][t] += wr[t];
            }
        }
        const float4 uf = u ? make_float4(0.f, 0.f, 0.f, 0.f) : uniforms4(seed, g, ch);
        const float ufa[4] = {uf.x, uf.y, uf.z, uf.w};
        uint32_t out = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const double ur = u ? u[(int64_t)g * Rp + 4 * ch + r] : (double)ufa[r];
            out |= (uint32_t)draw_category(ia, p[r], ur) << (8 * r);
        }
        *reinterpret_cast<uint32_t*>(C + (int64_t)g * Rp + 4 * ch) = out;
    }
}

cudaError_t launch_cok_level(const CokArgs& c, const int32_t* node, int k, int64_t p0, int64_t p1, int Rp,
                             const double* u, uint64_t seed, uint8_t* C, cudaStream_t s) {
    if (p1 <= p0) return cudaSuccess;
    int64_t blocks = ((p1 - p0) * (Rp / 4) + 255) / 256;
    if (blocks > (1 << 20)) blocks = 1 << 20;
    cok_level_kernel<<<(int)blocks, 256, 0, s>>>(c, node, k, p0, p1, Rp, u, seed, C);
    return cudaGetLastError();
}

// One level of the multivariate Gaussian sweep: one thread per (position,
// 4 realizations).  mu^_t = cst_t + sum_j sum_b w[j][b][t] v_b(x_j) over the
// system's grid neighbours, then v = mu^ + F z with z the given normals or
// the seeded ones of pseudo-node a*N + g (variable a of node g).
__global__ void __launch_bounds__(256) mv_level_kernel(const CokArgs c, const int32_t* __restrict__ node, int k,
                                                       int64_t N, int64_t p0, int64_t p1, int Rp,
                                                       const double* __restrict__ z, uint64_t seed,
                                                       double* __restrict__ V) {
    const int cpn = Rp >> 2, L = c.ncat;
    const int64_t total = (p1 - p0) * cpn;
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < total;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = p0 + it / cpn;
        const int ch = (int)(it % cpn);
        const int64_t g = node[pos];
        const int m = c.m[pos];
        double mu[4][IND_MAX_CAT];
#pragma unroll
        for (int t = 0; t < IND_MAX_CAT; ++t) {
            const double v = t < L ? c.cst[pos * L + t] : 0.0;
#pragma unroll
            for (int r = 0; r < 4; ++r) mu[r][t] = v;
        }
        for (int j = 0; j < m; ++j) {
            const int64_t e = pos * k + j;
            const int64_t nb = c.idx[e];
            for (int b = 0; b < L; ++b) {
                const double* vb = V + ((int64_t)b * N + nb) * Rp + 4 * ch;
                const double v0 = vb[0], v1 = vb[1], v2 = vb[2], v3 = vb[3];
                const double* wr = c.w + (e * L + b) * L;
#pragma unroll
                for (int t = 0; t < IND_MAX_CAT; ++t)
                    if (t < L) {
                        const double wt = wr[t];
                        mu[0][t] += wt * v0;
                        mu[1][t] += wt * v1;
                        mu[2][t] += wt * v2;
                        mu[3][t] += wt * v3;
                    }
            }
        }
        double zz[4][IND_MAX_CAT];
#pragma unroll
        for (int a = 0; a < IND_MAX_CAT; ++a) {
            if (a < L) {
                if (z) {
                    const double* za = z + ((int64_t)a * N + g) * Rp + 4 * ch;
                    zz[0][a] = za[0];
                    zz[1][a] = za[1];
                    zz[2][a] = za[2];
                    zz[3][a] = za[3];
                } else {
                    const float4 f = normals4(seed, (int64_t)a * N + g, ch);
                    zz[0][a] = f.x;
                    zz[1][a] = f.y;
                    zz[2][a] = f.z;
                    zz[3][a] = f.w;
                }
            } else {
                zz[0][a] = zz[1][a] = zz[2][a] = zz[3][a] = 0.0;
            }
        }
        const double* F = c.fac + pos * L * L;
#pragma unroll
        for (int t = 0; t < IND_MAX_CAT; ++t) {
            if (t < L) {
#pragma unroll
                for (int u = 0; u < IND_MAX_CAT; ++u)
                    if (u <= t) {
                        const double f = F[t * L + u];
#pragma unroll
                        for (int r = 0; r < 4; ++r) mu[r][t] += f * zz[r][u];
                    }
                double* vt = V + ((int64_t)t * N + g) * Rp + 4 * ch;
#pragma unroll
                for (int r = 0; r < 4; ++r) vt[r] = mu[r][t];
            }
        }
    }
}

cudaError_t launch_mv_level(const CokArgs& c, const int32_t* node, int k, int64_t N, int64_t p0, int64_t p1, int Rp,
                            const double* z, uint64_t seed, double* V, cudaStream_t s) {
    if (p1 <= p0) return cudaSuccess;
    int64_t blocks = ((p1 - p0) * (Rp / 4) + 255) / 256;
    if (blocks > (1 << 20)) blocks = 1 << 20;
    mv_level_kernel<<<(int)blocks, 256, 0, s>>>(c, node, k, N, p0, p1, Rp, z, seed, V);
    return cudaGetLastError();
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

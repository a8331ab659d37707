// search.cu — kernel (a): k-nearest neighbours among the data and the
// earlier-visited grid nodes inside the search neighbourhood, plus the
// dependency levels of the path's DAG and the level-ordered node list.
//
// Replaces search!(neighbors, center, searcher, mask=simulated)
// (src/simulation/field/seqsim.jl:107) for every node of the path at once:
// with the path fixed, node p's candidates are the data (always simulated,
// seqsim.jl:267-271) and the grid nodes of smaller path rank.
//
// One warp per node.  Grid candidates come from a template of cell offsets
// pre-sorted by (canonical FP64 d2, linear offset); scanning it 32 entries at
// a time and keeping offsets whose node is in the grid and has a smaller rank
// yields them in (d2, node id) order, so the first k kept are the k nearest.
// Data candidates come from a bucket grid, are tested with the same FP64
// metric and sorted in shared memory.  Both sorted lists merge into the
// node's neighbour row (ties: grid nodes first, their ids are smaller).
#include <climits>
#include <cmath>

#include "common.cuh"

namespace sgs {

constexpr int SEARCH_WARPS = 8;
constexpr int SCAN_STEPS = 4;  // template steps of 32 entries loaded per pass
constexpr int DCAP = 256;  // data candidate buffer per warp
// Early path ranks: a node of rank t has exactly t simulated grid nodes, the
// first t of the path.  While t is small against the template (T > 8 t, up
// to 2048), testing those t nodes costs less than scanning the template far
// enough to find k of them (the scan reads about k N / t entries).
constexpr int BRUTE_MAX = 2048;
constexpr int BRUTE_RATIO = 8;

// Squared distances are non-negative doubles, whose IEEE bit patterns order
// exactly like the values when read as int64, so the kernel compares and
// sorts them as integers (the integer ALU instead of GB300's narrow FP64 pipe).
__device__ __forceinline__ long long key_of(double d2) { return __double_as_longlong(d2); }

// Bitonic sort of n (<= DCAP) (key, idx) pairs in shared memory by one warp.
__device__ void warp_sort_pairs(long long* key, int32_t* idx, int n, int lane) {
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = n + lane; i < P; i += 32) {
        key[i] = LLONG_MAX;
        idx[i] = INT_MAX;
    }
    __syncwarp();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < (P >> 1); t += 32) {
                int i = (t / stride) * stride * 2 + (t % stride);
                int j = i + stride;
                bool asc = (i & size) == 0;
                long long ki = key[i], kj = key[j];
                int32_t ii = idx[i], ij = idx[j];
                bool gt = ki > kj || (ki == kj && ii > ij);
                if (gt == asc) {
                    key[i] = kj; key[j] = ki;
                    idx[i] = ij; idx[j] = ii;
                }
            }
            __syncwarp();
        }
    }
}

// Per-warp shared-memory buffers of the search.
struct SearchSmem {
    long long* gd2;   // [KMAX] grid candidates' d2 keys
    int32_t* gidx;    // [KMAX] their node ids
    long long* dd2;   // [DCAP] data candidates' d2 keys
    int32_t* didx;    // [DCAP] their augmented ids
    int32_t* squ;     // [64] screened data candidates
    int32_t* rstart;  // [32] first bucket-ordered datum of each of 32 bucket rows
    int32_t* roff;    // [32] their offsets in the concatenated candidate list
};

// The neighbour row of node g of the problem described by `a`; with COUNT,
// adds the candidates it examined to ex_grid / ex_data (warp-uniform).
template <bool COUNT>
__device__ __forceinline__ void search_node(const SearchArgs& a, int g, int lane, const SearchSmem& sm,
                                            unsigned long long& ex_grid, unsigned long long& ex_data) {
    long long* gd2 = sm.gd2;
    int32_t* gidx = sm.gidx;
    long long* dd2 = sm.dd2;
    const long long* tkey = reinterpret_cast<const long long*>(a.tmpl_d2);
    int32_t* didx = sm.didx;
    int32_t* squ = sm.squ;
    const GridDev& G = a.grid;
    const int k = a.k;
    const unsigned lt = lanemask_lt();
    {
        const int64_t t = a.rank[g];
        int i0, i1, i2;
        cell_of(G, g, i0, i1, i2);

        // ---- grid candidates from the sorted template ----
        // SCAN_STEPS steps of 32 entries per pass: the template entries and
        // rank gathers of all are issued before the first is used, and each
        // later step is taken only if the earlier ones left the row short
        // (the entries are processed in the same order as one step at a time)
        int ng = 0;
        const int T = a.data_only ? 0 : a.T;
        if (!a.data_only && t <= BRUTE_MAX && (int64_t)BRUTE_RATIO * t < T) {
            // the t earlier path nodes, with the template's canonical FP64 d2
            // (h_j = offset_j x spacing_j), inside the same neighbourhood,
            // kept by (d2, node id): the order of the template (d2, linear
            // offset), since for a fixed node the linear offset orders ids
            int nbuf = 0;
            if (COUNT) ex_grid += (unsigned long long)t;
            for (int base = 0; base < t; base += 32) {
                const int j = base + lane;
                int c = 0, c0 = 0, c1 = 0, c2 = 0;
                bool maybe = false;
                if (j < t) {
                    c = a.path[j];
                    cell_of(G, c, c0, c1, c2);
                    maybe = a.metric.kind == METRIC_NEAREST ||
                            metric_maybe_within(a.metric, G.dim, (float)(c0 - i0) * a.spacing_f[0],
                                                (float)(c1 - i1) * a.spacing_f[1],
                                                (float)(c2 - i2) * a.spacing_f[2], a.metric.bound_f);
                }
                bool ok = false;
                double d2 = 0.0;
                if (__any_sync(FULL_MASK, maybe) && maybe) {
                    d2 = metric_d2(a.metric, G.dim, dmul((double)(c0 - i0), G.spacing[0]),
                                   dmul((double)(c1 - i1), G.spacing[1]),
                                   G.dim == 3 ? dmul((double)(c2 - i2), G.spacing[2]) : 0.0);
                    ok = metric_inside(a.metric, d2);
                }
                const unsigned b = __ballot_sync(FULL_MASK, ok);
                if (ok) {
                    const int p = nbuf + __popc(b & lt);
                    dd2[p] = key_of(d2);
                    didx[p] = c;
                }
                nbuf += __popc(b);
                __syncwarp();
                if (nbuf > DCAP - 32) {
                    warp_sort_pairs(dd2, didx, nbuf, lane);
                    nbuf = min(nbuf, k);
                }
            }
            if (nbuf > 0) warp_sort_pairs(dd2, didx, nbuf, lane);
            ng = min(nbuf, k);
            for (int q = lane; q < ng; q += 32) {
                gd2[q] = dd2[q];
                gidx[q] = didx[q];
            }
            __syncwarp();
        }
        for (int base = 0; base < T && ng < k && !(t <= BRUTE_MAX && (int64_t)BRUTE_RATIO * t < T);
             base += 32 * SCAN_STEPS) {
            int c[SCAN_STEPS];
            bool in[SCAN_STEPS];
#pragma unroll
            for (int h = 0; h < SCAN_STEPS; ++h) {
                c[h] = 0;
                in[h] = false;
                const int j = base + 32 * h + lane;
                if (j < T) {
                    const TmplEntry e = a.tmpl[j];
                    const int c0 = i0 + e.dx, c1 = i1 + e.dy, c2 = i2 + e.dz;
                    if (c0 >= 0 && c0 < G.n[0] && c1 >= 0 && c1 < G.n[1] && c2 >= 0 && c2 < G.n[2]) {
                        c[h] = g + e.dlin;
                        in[h] = true;
                    }
                }
            }
            int rk[SCAN_STEPS];
#pragma unroll
            for (int h = 0; h < SCAN_STEPS; ++h) {
                rk[h] = in[h] ? a.rank[c[h]] : 0;
                if (COUNT) ex_grid += __popc(__ballot_sync(FULL_MASK, in[h]));
            }
#pragma unroll
            for (int h = 0; h < SCAN_STEPS; ++h) {
                if (ng >= k) break;  // warp-uniform
                const bool ok = in[h] && rk[h] < t;
                const unsigned b = __ballot_sync(FULL_MASK, ok);
                if (ok) {
                    const int p = ng + __popc(b & lt);
                    if (p < k) {
                        gidx[p] = c[h];
                        gd2[p] = tkey[base + 32 * h + lane];
                    }
                }
                ng += __popc(b);
            }
        }
        ng = min(ng, k);
        __syncwarp();

        // ---- data candidates, sorted ----
        // With k grid neighbours found, only data strictly nearer than the
        // k-th can enter the row (at equal distance grid nodes come first),
        // so that distance bounds the bucket box, the FP32 screen and the
        // exact test; otherwise every datum inside the neighbourhood counts.
        int nd = 0;
        if (a.D > 0) {
            const bool bounded = ng == k;
            const double tmax = bounded ? __longlong_as_double(gd2[k - 1]) : 0.0;
            const float tf = (float)tmax * 1.001f;
            const float rho = sqrtf(tf) + a.metric.dh_f;  // the bound's radius, metric units
            const float dimf = (float)G.dim;
            float bnd = a.metric.bound_f;
            if (bounded) {
                if (a.metric.kind == METRIC_NEAREST)
                    bnd = tf + 2.0f * sqrtf(dimf * tf) * a.metric.dh_f + dimf * a.metric.dh_f * a.metric.dh_f;
                else
                    bnd = fminf(bnd, tf + a.metric.slack_f);
            }
            double x[3];
            x[0] = centroid(G, 0, i0);
            x[1] = centroid(G, 1, i1);
            x[2] = G.dim == 3 ? centroid(G, 2, i2) : 0.0;
            int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
            for (int j = 0; j < G.dim; ++j) {
                if (a.metric.kind == METRIC_NEAREST && !bounded) {
                    lo[j] = 0;
                    hi[j] = a.nb[j] - 1;
                } else {
                    // bucket range of the bounding box (of the neighbourhood,
                    // or of its part within the bound), in FP32 with a margin
                    // of 1e-3 buckets on each side: far above the few FP32
                    // roundings here (~1e-5 buckets) and the FP32 rounding of
                    // the half extent, so the range is a superset
                    float ext = a.ext_f[j];
                    if (bounded) {
                        if (a.metric.kind == METRIC_ELLIPSOID) ext *= fminf(1.0f, rho);
                        else if (a.metric.kind == METRIC_ISO) ext = fminf(ext, rho);
                        else ext = rho;
                    }
                    const int ij = j == 0 ? i0 : (j == 1 ? i1 : i2);
                    const float xr = ((float)ij + 0.5f) * a.spacing_f[j];
                    const float l = floorf((xr - ext) * a.inv_bw_f[j] - 1e-3f);
                    const float h = floorf((xr + ext) * a.inv_bw_f[j] + 1e-3f);
                    lo[j] = (int)fmaxf(0.0f, fminf(l, (float)(a.nb[j] - 1)));
                    hi[j] = (int)fmaxf(0.0f, fminf(h, (float)(a.nb[j] - 1)));
                }
            }
            float xr[3];
            xr[0] = ((float)i0 + 0.5f) * a.spacing_f[0];
            xr[1] = ((float)i1 + 0.5f) * a.spacing_f[1];
            xr[2] = ((float)i2 + 0.5f) * a.spacing_f[2];
            int nbuf = 0, nq = 0;
            // exact FP64 test of queued candidates, one per lane (full warps,
            // so the FP64 path is not issued for a lone surviving lane)
            auto exact = [&](int cnt) {
                bool ok = false;
                double d2 = 0.0;
                int i = 0;
                if (lane < cnt) {
                    i = squ[lane];
                    const double h0 = dsub(a.dxyz[3 * (int64_t)i + 0], x[0]);
                    const double h1 = dsub(a.dxyz[3 * (int64_t)i + 1], x[1]);
                    const double h2 = G.dim == 3 ? dsub(a.dxyz[3 * (int64_t)i + 2], x[2]) : 0.0;
                    d2 = metric_d2(a.metric, G.dim, h0, h1, h2);
                    ok = metric_inside(a.metric, d2) && (!bounded || d2 < tmax);
                }
                const unsigned b = __ballot_sync(FULL_MASK, ok);
                if (ok) {
                    const int p = nbuf + __popc(b & lt);
                    dd2[p] = key_of(d2);
                    didx[p] = (int32_t)(G.N + a.did[i]);
                }
                nbuf += __popc(b);
                __syncwarp();
                if (nbuf > DCAP - 32) {
                    warp_sort_pairs(dd2, didx, nbuf, lane);
                    nbuf = min(nbuf, k);
                }
            };
            // Candidates: the bucket rows (by, bz) of the bounding box, 32 rows
            // at a time.  Lane r loads row r's range of bucket-ordered data,
            // a warp scan gives the rows' offsets in one concatenated list,
            // and the warp screens that list 32 candidates at a time (each
            // lane finds its candidate's row by binary search), so the
            // rows' loads overlap and lanes stay busy across short rows.
            const int n1 = hi[1] - lo[1] + 1;
            const int nrows = n1 * (hi[2] - lo[2] + 1);
            for (int r0 = 0; r0 < nrows; r0 += 32) {
                const int r = r0 + lane;
                int rs = 0, len = 0;
                if (r < nrows) {
                    const int row = a.nb[0] * ((lo[1] + r % n1) + a.nb[1] * (lo[2] + r / n1));
                    rs = a.bstart[row + lo[0]];
                    len = a.bstart[row + hi[0] + 1] - rs;
                }
                int incl = len;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL_MASK, incl, o);
                    if (lane >= o) incl += y;
                }
                const int total = __shfl_sync(FULL_MASK, incl, 31);
                if (COUNT) ex_data += (unsigned long long)total;
                sm.rstart[lane] = rs;
                sm.roff[lane] = incl - len;
                __syncwarp();
                for (int base = 0; base < total; base += 32) {
                    const int v = base + lane;
                    bool maybe = false;
                    int i = 0;
                    if (v < total) {
                        // last row whose offset is <= v holds candidate v
                        int rr = 0;
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1)
                            if (sm.roff[rr + step] <= v) rr += step;
                        i = sm.rstart[rr] + (v - sm.roff[rr]);
                        // FP32 screen on origin-relative FP32 coordinates;
                        // bound_f includes a slack above their rounding
                        const float4 p = a.dxyz_f[i];
                        maybe = metric_maybe_within(a.metric, G.dim, p.x - xr[0], p.y - xr[1], p.z - xr[2], bnd);
                    }
                    const unsigned b = __ballot_sync(FULL_MASK, maybe);
                    if (maybe) squ[nq + __popc(b & lt)] = i;
                    nq += __popc(b);
                    __syncwarp();
                    if (nq >= 32) {
                        exact(32);
                        const int rest = nq - 32;
                        const int vq = lane < rest ? squ[32 + lane] : 0;
                        __syncwarp();
                        if (lane < rest) squ[lane] = vq;
                        __syncwarp();
                        nq = rest;
                    }
                }
                __syncwarp();  // the row table is rewritten by the next 32 rows
            }
            if (nq > 0) exact(nq);
            if (nbuf > 0) warp_sort_pairs(dd2, didx, nbuf, lane);
            nd = min(nbuf, k);
        }

        // ---- merge (d2, id): grid entries precede data entries at equal d2 ----
        int32_t* out = a.nbr + (int64_t)g * k;
        int ngrid = 0;
        for (int q = lane; q < ng; q += 32) {
            const long long d = gd2[q];
            int lo = 0, hi = nd;  // data strictly nearer
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (dd2[mid] < d) lo = mid + 1; else hi = mid;
            }
            const int p = q + lo;
            if (p < k) {
                out[p] = gidx[q];
                ++ngrid;
            }
        }
        for (int q = lane; q < nd; q += 32) {
            const long long d = dd2[q];
            int lo = 0, hi = ng;  // grid at distance <= d
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (gd2[mid] <= d) lo = mid + 1; else hi = mid;
            }
            const int p = q + lo;
            if (p < k) out[p] = didx[q];
        }
        const int total = min(ng + nd, k);
        for (int p = total + lane; p < k; p += 32) out[p] = -1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ngrid += __shfl_xor_sync(FULL_MASK, ngrid, o);
        if (lane == 0) {
            a.cnt[g] = total;
            a.ngrid[g] = ngrid;
        }
        __syncwarp();
    }
}

#define SEARCH_SMEM_DECL                                                  \
    __shared__ long long s_gd2[SEARCH_WARPS][KMAX];                       \
    __shared__ int32_t s_gidx[SEARCH_WARPS][KMAX];                        \
    __shared__ long long s_dd2[SEARCH_WARPS][DCAP];                       \
    __shared__ int32_t s_didx[SEARCH_WARPS][DCAP];                        \
    __shared__ int32_t s_squ[SEARCH_WARPS][64];                           \
    __shared__ int32_t s_rows[SEARCH_WARPS][64];                          \
    const int lane = threadIdx.x & 31;                                    \
    const int wib = threadIdx.x >> 5;                                     \
    const SearchSmem sm{s_gd2[wib], s_gidx[wib], s_dd2[wib], s_didx[wib], s_squ[wib], s_rows[wib], s_rows[wib] + 32}

__global__ void __launch_bounds__(SEARCH_WARPS * 32) search_kernel(const SearchArgs a) {
    SEARCH_SMEM_DECL;
    const int64_t nwarps = (int64_t)gridDim.x * SEARCH_WARPS;
    // Nodes go in id order, so the warps of a block take neighbouring cells
    // and share the rank and data cache lines they scan; the result of a
    // node depends only on its path rank, not on when it is processed.
    unsigned long long ex_grid = 0, ex_data = 0;
    for (int64_t gg = (int64_t)blockIdx.x * SEARCH_WARPS + wib; gg < a.grid.N; gg += nwarps)
        search_node<true>(a, (int)gg, lane, sm, ex_grid, ex_data);
    if (a.scanned && lane == 0) {
        atomicAdd(&a.scanned[0], ex_grid);
        atomicAdd(&a.scanned[1], ex_data);
    }
}

// Every node of a batch of domains: global node ids [noff[d], noff[d+1])
// belong to domain d, described by doms[d] (its own grid, metric, template,
// data, path ranks and neighbour rows).  A warp copies its current domain's
// descriptor to shared memory when it moves into another domain.
__global__ void __launch_bounds__(SEARCH_WARPS * 32)
search_batch_kernel(const SearchArgs* __restrict__ doms, const int64_t* __restrict__ noff, int ndom) {
    SEARCH_SMEM_DECL;
    __shared__ SearchArgs s_dom[SEARCH_WARPS];
    const int64_t total = noff[ndom];
    const int64_t nwarps = (int64_t)gridDim.x * SEARCH_WARPS;
    int64_t lo = 0, hi = 0;
    unsigned long long ex_grid = 0, ex_data = 0;  // not counted for batches
    for (int64_t gg = (int64_t)blockIdx.x * SEARCH_WARPS + wib; gg < total; gg += nwarps) {
        if (gg < lo || gg >= hi) {
            const int d = find_domain(noff, ndom, gg);
            lo = noff[d];
            hi = noff[d + 1];
            __syncwarp();
            warp_copy_struct(&s_dom[wib], &doms[d], lane);
            __syncwarp();
        }
        search_node<false>(s_dom[wib], (int)(gg - lo), lane, sm, ex_grid, ex_data);
    }
}

cudaError_t launch_search_batch(const SearchArgs* doms, const int64_t* noff, int ndom, int64_t total, int nsm,
                                cudaStream_t s) {
    int64_t want = (total + SEARCH_WARPS - 1) / SEARCH_WARPS;
    int blocks = (int)(want < (int64_t)nsm * 8 ? want : (int64_t)nsm * 8);
    if (blocks < 1) blocks = 1;
    search_batch_kernel<<<blocks, SEARCH_WARPS * 32, 0, s>>>(doms, noff, ndom);
    return cudaGetLastError();
}

cudaError_t launch_search(const SearchArgs& a, cudaStream_t s) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int64_t want = (a.grid.N + SEARCH_WARPS - 1) / SEARCH_WARPS;
    int blocks = (int)(want < (int64_t)nsm * 8 ? want : (int64_t)nsm * 8);
    if (blocks < 1) blocks = 1;
    search_kernel<<<blocks, SEARCH_WARPS * 32, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Dependency levels: level(p) = 1 + max level of p's grid neighbours (0 when
// it has none).  Warps take LEVEL_CHUNK consecutive path ranks per ticket and
// process them in rank order; a node's neighbours all have smaller ranks,
// taken earlier by this warp or by warps that are resident and running, so
// every wait ends.  The kernel is bound by the latency of dependency chains:
// a warp that holds several ranks delays every chain through its later ones
// (16 ranks per ticket measured 7x slower than one), so LEVEL_CHUNK is 1.
// Each wait is still bounded (wait_level: a.wait_ns of wall-clock time, and
// no longer once another warp gave up); the kernel then raises the error
// flag, no warp takes a new ticket, and the host reports SGS_ERR_TIMEOUT.
// The deepest level is kept per warp and published once.
constexpr int LEVEL_CHUNK = 1;

__global__ void __launch_bounds__(256) levels_kernel(const LevelArgs a) {
    const int lane = threadIdx.x & 31;
    volatile int32_t* vlevel = a.level;
    const volatile int32_t* verr = a.err;
    int wmax = 0;
    for (int taken = 0;; ++taken) {
        int64_t t0 = 0;
        // after an error no new tickets (the flag is read every 16th ticket)
        if (lane == 0) t0 = ((taken & 15) == 15 && *verr) ? a.N : atomicAdd(a.ticket, LEVEL_CHUNK);
        t0 = __shfl_sync(FULL_MASK, t0, 0);
        if (t0 >= a.N) break;
        const int64_t t1 = min(t0 + (int64_t)LEVEL_CHUNK, a.N);
        for (int64_t t = t0; t < t1; ++t) {
            const int g = a.path[t];
            const int n = a.cnt[g];
            int lv = 0;
            for (int q = lane; q < n; q += 32) {
                const int c = a.nbr[(int64_t)g * a.k + q];
                if (c < a.N) lv = max(lv, wait_level(vlevel, c, a.err, a.wait_ns) + 1);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) lv = max(lv, __shfl_xor_sync(FULL_MASK, lv, o));
            if (lane == 0) atomicExch(&a.level[g], lv);
            wmax = max(wmax, lv);
        }
    }
    if (lane == 0) atomicMax(a.maxlevel, wmax);
}

// rank[path[t]] = t (rank preset to -1; a NULL path is the linear one and is
// written out), then a second pass: every entry in range, and every rank
// pointing back to its t — a repeated node leaves one of its ranks pointing
// elsewhere, and a node never visited is then impossible (N entries).
__global__ void path_rank_scatter_kernel(const int32_t* __restrict__ path, int64_t N, int32_t* __restrict__ path_out,
                                         int32_t* __restrict__ rank, int32_t* err) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = path ? (int64_t)path[t] : t;
        if (!path) path_out[t] = (int32_t)t;
        if (g < 0 || g >= N) {
            atomicOr(err, 1);
            continue;
        }
        rank[g] = (int32_t)t;
    }
}

__global__ void path_rank_check_kernel(const int32_t* __restrict__ path, int64_t N, const int32_t* __restrict__ rank,
                                       int32_t* err) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = path[t];
        if (g >= 0 && g < N && rank[g] != (int32_t)t) atomicOr(err, 2);
    }
}

cudaError_t launch_path_ranks(const int32_t* path, int64_t N, int32_t* path_out, int32_t* rank, int32_t* err, int nsm,
                              cudaStream_t s) {
    if (N <= 0) return cudaSuccess;
    path_rank_scatter_kernel<<<nsm * 8, 256, 0, s>>>(path, N, path_out, rank, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    path_rank_check_kernel<<<nsm * 8, 256, 0, s>>>(path_out, N, rank, err);
    return cudaGetLastError();
}

// The same for the path arena of a batch of domains: entry i of domain d
// (global ids [off[d], off[d+1])) holds a local node id; rank entries are
// local too.  *bad_domain (preset to nd by the caller) takes the smallest
// domain whose path is not a permutation of its nodes.
__global__ void batch_rank_scatter_kernel(const int32_t* __restrict__ path, const int64_t* __restrict__ off, int nd,
                                          int32_t* __restrict__ rank, int32_t* bad_domain) {
    const int64_t total = off[nd];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int d = find_domain(off, nd, i);
        const int64_t o = off[d], n = off[d + 1] - o, g = path[i];
        if (g < 0 || g >= n) {
            atomicMin(bad_domain, d);
            continue;
        }
        rank[o + g] = (int32_t)(i - o);
    }
}

__global__ void batch_rank_check_kernel(const int32_t* __restrict__ path, const int64_t* __restrict__ off, int nd,
                                        const int32_t* __restrict__ rank, int32_t* bad_domain) {
    const int64_t total = off[nd];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int d = find_domain(off, nd, i);
        const int64_t o = off[d], n = off[d + 1] - o, g = path[i];
        if (g >= 0 && g < n && rank[o + g] != (int32_t)(i - o)) atomicMin(bad_domain, d);
    }
}

cudaError_t launch_batch_path_ranks(const int32_t* path, const int64_t* off, int nd, int64_t total, int32_t* rank,
                                    int32_t* bad_domain, int nsm, cudaStream_t s) {
    if (total <= 0) return cudaSuccess;
    batch_rank_scatter_kernel<<<nsm * 8, 256, 0, s>>>(path, off, nd, rank, bad_domain);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    batch_rank_check_kernel<<<nsm * 8, 256, 0, s>>>(path, off, nd, rank, bad_domain);
    return cudaGetLastError();
}

cudaError_t launch_levels(const LevelArgs& a, int nsm, cudaStream_t s) {
    levels_kernel<<<nsm * 8, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// Counting sort of the nodes by level.  Each block takes a contiguous range
// of node ids and counts its levels in a shared-memory histogram, so global
// atomics are one per (block, level) instead of one per node; the fill pass
// reserves each level's slots for the block with one atomic per (block,
// level) and places its nodes from the shared bases.  Within a level, nodes
// come out grouped by block (ascending node-id ranges).  Level counts above
// LEVEL_HIST_MAX fall back to one global atomic per node.
constexpr int LEVEL_HIST_MAX = 12288;  // 48 KB of shared memory
constexpr int LEVEL_BLOCK_NODES = 8192;

__global__ void level_count_kernel(int64_t N, const int32_t* __restrict__ level, int nlevels,
                                   int32_t* __restrict__ lcount) {
    extern __shared__ int32_t h[];
    const int64_t g0 = (int64_t)blockIdx.x * LEVEL_BLOCK_NODES;
    const int64_t g1 = min(g0 + LEVEL_BLOCK_NODES, N);
    if (nlevels > LEVEL_HIST_MAX) {
        for (int64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) atomicAdd(&lcount[level[g]], 1);
        return;
    }
    for (int i = threadIdx.x; i < nlevels; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) atomicAdd(&h[level[g]], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < nlevels; i += blockDim.x)
        if (h[i]) atomicAdd(&lcount[i], h[i]);
}

__global__ void level_fill_kernel(int64_t N, const int32_t* __restrict__ level, int nlevels,
                                  const int32_t* __restrict__ loff, int32_t* __restrict__ lfill,
                                  int32_t* __restrict__ order) {
    extern __shared__ int32_t h[];
    const int64_t g0 = (int64_t)blockIdx.x * LEVEL_BLOCK_NODES;
    const int64_t g1 = min(g0 + LEVEL_BLOCK_NODES, N);
    if (nlevels > LEVEL_HIST_MAX) {
        for (int64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
            const int l = level[g];
            order[loff[l] + atomicAdd(&lfill[l], 1)] = (int32_t)g;
        }
        return;
    }
    for (int i = threadIdx.x; i < nlevels; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) atomicAdd(&h[level[g]], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < nlevels; i += blockDim.x)
        if (h[i]) h[i] = loff[i] + atomicAdd(&lfill[i], h[i]);
    __syncthreads();
    for (int64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) order[atomicAdd(&h[level[g]], 1)] = (int32_t)g;
}

cudaError_t launch_level_order(int64_t N, const int32_t* level, int nlevels, int32_t* lcount, int32_t* loff,
                               int32_t* lfill, int32_t* order, cudaStream_t s) {
    // lcount is counted here; the caller scans it into loff on the host
    // between the two phases, so this runs in two calls: order == nullptr ->
    // count, otherwise fill.
    const int64_t blocks = (N + LEVEL_BLOCK_NODES - 1) / LEVEL_BLOCK_NODES;
    if (blocks <= 0) return cudaSuccess;
    const size_t smem = nlevels <= LEVEL_HIST_MAX ? (size_t)nlevels * sizeof(int32_t) : 0;
    if (order == nullptr) {
        level_count_kernel<<<(unsigned)blocks, 256, smem, s>>>(N, level, nlevels, lcount);
    } else {
        level_fill_kernel<<<(unsigned)blocks, 256, smem, s>>>(N, level, nlevels, loff, lfill, order);
    }
    return cudaGetLastError();
}

}  // namespace sgs

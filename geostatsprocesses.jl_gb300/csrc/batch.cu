// batch.cu — batches of independent SGS problems ("domains"): one launch per
// phase over all domains' nodes, kriging systems solved in size classes,
// one persistent dataflow sweep, and CUDA graphs for the prepare sequence
// and the seeded sweep.
//
// The reference simulates one domain per rand call (src/simulation/field.jl:
// 73-124 -> preprocess / randsingle, src/simulation/field/seqsim.jl:50-156);
// a batch is the loop over such calls.  Domains are concatenated:
//   grid nodes   domain d owns global ids [noff[d], noff[d+1]); the path and
//                rank arenas use the same offsets (path entries and ranks
//                stay local to the domain)
//   neighbours   rows of k_d entries from nbr0[d] (local augmented ids, as a
//                plan's table), counts and grid counts by global id
//   levels       by global id; the level order lists global ids, so all
//                domains' level-0 nodes come first, then level 1, ...
//   sweep tables packed rows (CSR offsets by position in level order) of
//                global grid-neighbour ids and (hi, lo) or FP64 weights
//   values       node-major rows by global id
// Each kernel finds a work item's domain by binary search over noff and
// reads that domain's descriptor (SearchArgs / SolveArgs / LevelDom).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <string>
#include <memory>
#include <thread>
#include <vector>

#include "common.cuh"

using namespace sgs;

namespace sgs {

constexpr int NBIN = 5;
__host__ __device__ constexpr int bin_nmax(int b) { return b == 0 ? 8 : b == 1 ? 16 : b == 2 ? 32 : b == 3 ? 48 : 64; }
__device__ __forceinline__ int bin_of(int n) { return n <= 8 ? 0 : n <= 16 ? 1 : n <= 32 ? 2 : n <= 48 ? 3 : 4; }

struct LevelDom {
    int64_t node0;  // first global node id
    int64_t nbr0;   // first entry of the domain's neighbour rows
    int32_t N;      // grid nodes
    int32_t k;      // row length
};

// ---------------------------------------------------------------------------
// Dependency levels of all domains.  Tickets run over the concatenated path
// arena (domain after domain, path rank order inside a domain); a node's
// neighbours are earlier nodes of its own domain, so they hold smaller
// tickets, taken by running warps, and every wait ends.  Each wait is
// bounded anyway (wait_level: wait_ns of wall-clock time, then the error
// flag, after which no warp takes a new ticket).
__global__ void __launch_bounds__(256)
levels_batch_kernel(const LevelDom* __restrict__ doms, const int64_t* __restrict__ noff, int ndom,
                    const int32_t* __restrict__ path, const int32_t* __restrict__ nbr,
                    const int32_t* __restrict__ cnt, int32_t* level, unsigned long long* ticket, int32_t* maxlevel,
                    int32_t* err, uint64_t wait_ns) {
    const int lane = threadIdx.x & 31;
    const int64_t total = noff[ndom];
    volatile int32_t* vlevel = level;
    const volatile int32_t* verr = err;
    int wmax = 0;
    for (int taken = 0;; ++taken) {
        unsigned long long t = 0;
        // after an error no new tickets (the flag is read every 16th ticket)
        if (lane == 0) t = ((taken & 15) == 15 && *verr) ? (unsigned long long)total : atomicAdd(ticket, 1ull);
        t = __shfl_sync(FULL_MASK, t, 0);
        if ((int64_t)t >= total) break;
        const int d = find_domain(noff, ndom, (int64_t)t);
        const LevelDom D = doms[d];
        const int g = path[t];
        const int n = cnt[D.node0 + g];
        const int32_t* row = nbr + D.nbr0 + (int64_t)g * D.k;
        int lv = 0;
        for (int q = lane; q < n; q += 32) {
            const int c = row[q];
            if (c < D.N) lv = max(lv, wait_level(vlevel, D.node0 + c, err, wait_ns) + 1);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lv = max(lv, __shfl_xor_sync(FULL_MASK, lv, o));
        if (lane == 0) atomicExch(&level[D.node0 + g], lv);
        wmax = max(wmax, lv);
    }
    if (lane == 0) atomicMax(maxlevel, wmax);
}

// Counting sort by level with the level count read on the device (so the
// sequence needs no host round trip and can be captured): block histograms
// in shared memory up to BL_HIST levels, global atomics beyond.
constexpr int BL_HIST = 12288;
constexpr int BL_NODES = 8192;

__global__ void __launch_bounds__(256)
level_count_batch_kernel(int64_t N, const int32_t* __restrict__ level, const int32_t* __restrict__ maxlevel,
                         int32_t* __restrict__ lcount) {
    __shared__ int32_t h[BL_HIST];
    const int nlevels = *maxlevel + 1;
    const int64_t g0 = (int64_t)blockIdx.x * BL_NODES;
    const int64_t g1 = min(g0 + BL_NODES, N);
    if (nlevels > BL_HIST) {
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

__global__ void __launch_bounds__(256)
level_fill_batch_kernel(int64_t N, const int32_t* __restrict__ level, const int32_t* __restrict__ maxlevel,
                        const int32_t* __restrict__ loff, int32_t* __restrict__ lfill, int32_t* __restrict__ order) {
    __shared__ int32_t h[BL_HIST];
    const int nlevels = *maxlevel + 1;
    const int64_t g0 = (int64_t)blockIdx.x * BL_NODES;
    const int64_t g1 = min(g0 + BL_NODES, N);
    if (nlevels > BL_HIST) {
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

// Block-wide exclusive scan of one int64 per thread (blockDim.x a multiple
// of 32, at most 1024); returns the thread's prefix, *total the block sum.
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* s_warp, int64_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int64_t w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(FULL_MASK, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) s_warp[lane] = w;  // inclusive warp prefixes
    }
    __syncthreads();
    const int64_t before = wid > 0 ? s_warp[wid - 1] : 0;
    *total = s_warp[nw - 1];
    __syncthreads();
    return before + x - v;
}

// Level offsets loff[0..nlevels] from the counts (one block).
__global__ void __launch_bounds__(1024)
level_scan_kernel(const int32_t* __restrict__ maxlevel, const int32_t* __restrict__ lcount, int32_t* __restrict__ loff) {
    __shared__ int64_t s_warp[32];
    const int nlevels = *maxlevel + 1;
    int64_t carry = 0;
    for (int base = 0; base < nlevels; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int64_t v = i < nlevels ? lcount[i] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_scan(v, s_warp, &tot);
        if (i < nlevels) loff[i] = (int32_t)(carry + ex);
        carry += tot;
    }
    if (threadIdx.x == 0) loff[nlevels] = (int32_t)carry;
}

// CSR row starts of the sweep tables: off[p] = sum over positions q < p of
// the grid-neighbour count of node order[q]; off[n] = the total.  Three
// passes: tile sums, a one-block scan of the tile sums, tile rescans.
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_PER = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER;

__global__ void __launch_bounds__(SCAN_THREADS)
tile_sum_kernel(int64_t n, const int32_t* __restrict__ order, const int32_t* __restrict__ val, int64_t* __restrict__ tsum) {
    __shared__ int64_t s_warp[32];
    const int64_t p0 = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t s = 0;
    for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
        const int64_t p = p0 + i;
        if (p < n) s += val[order[p]];
    }
    int64_t tot;
    block_exclusive_scan(s, s_warp, &tot);
    if (threadIdx.x == 0) tsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) tile_scan_kernel(int64_t ntiles, int64_t* __restrict__ tsum) {
    __shared__ int64_t s_warp[32];
    int64_t carry = 0;
    for (int64_t base = 0; base < ntiles; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const int64_t v = i < ntiles ? tsum[i] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_scan(v, s_warp, &tot);
        if (i < ntiles) tsum[i] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS)
tile_apply_kernel(int64_t n, const int32_t* __restrict__ order, const int32_t* __restrict__ val,
                  const int64_t* __restrict__ tpre, int64_t* __restrict__ off) {
    __shared__ int64_t s_warp[32];
    const int64_t p0 = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER;
    int32_t v[SCAN_PER];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_PER; ++i) {
        const int64_t p = p0 + i;
        v[i] = p < n ? val[order[p]] : 0;
        s += v[i];
    }
    int64_t tot;
    int64_t run = tpre[blockIdx.x] + block_exclusive_scan(s, s_warp, &tot);
#pragma unroll
    for (int i = 0; i < SCAN_PER; ++i) {
        const int64_t p = p0 + i;
        if (p < n) off[p] = run;
        run += v[i];
        if (p == n - 1) off[n] = run;
    }
}

// Size classes of the systems: positions grouped by neighbour count into
// NBIN lists (one array, bin b at [start_b, start_b + count_b)).  desc gets
// {count_b, start_b} per bin for the solve launches.
constexpr int BIN_NODES = 8192;

__global__ void __launch_bounds__(256)
bin_count_kernel(int64_t n, const int32_t* __restrict__ order, const int32_t* __restrict__ cnt,
                 int32_t* __restrict__ bcount) {
    __shared__ int32_t h[NBIN];
    if (threadIdx.x < NBIN) h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t p0 = (int64_t)blockIdx.x * BIN_NODES;
    const int64_t p1 = min(p0 + BIN_NODES, n);
    for (int64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) atomicAdd(&h[bin_of(cnt[order[p]])], 1);
    __syncthreads();
    if (threadIdx.x < NBIN && h[threadIdx.x]) atomicAdd(&bcount[threadIdx.x], h[threadIdx.x]);
}

__global__ void __launch_bounds__(256)
bin_fill_kernel(int64_t n, const int32_t* __restrict__ order, const int32_t* __restrict__ cnt,
                const int32_t* __restrict__ bcount, int32_t* __restrict__ bfill, int32_t* __restrict__ list,
                int32_t* __restrict__ desc) {
    __shared__ int32_t h[NBIN], base[NBIN];
    if (threadIdx.x < NBIN) h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t p0 = (int64_t)blockIdx.x * BIN_NODES;
    const int64_t p1 = min(p0 + BIN_NODES, n);
    for (int64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) atomicAdd(&h[bin_of(cnt[order[p]])], 1);
    __syncthreads();
    if (threadIdx.x < NBIN) {
        int32_t start = 0;
        for (int b = 0; b < (int)threadIdx.x; ++b) start += bcount[b];
        base[threadIdx.x] = start + (h[threadIdx.x] ? atomicAdd(&bfill[threadIdx.x], h[threadIdx.x]) : 0);
        h[threadIdx.x] = 0;
        if (blockIdx.x == 0) {
            desc[2 * threadIdx.x] = bcount[threadIdx.x];
            desc[2 * threadIdx.x + 1] = start;
        }
    }
    __syncthreads();
    for (int64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const int b = bin_of(cnt[order[p]]);
        list[base[b] + atomicAdd(&h[b], 1)] = (int32_t)p;
    }
}

__global__ void sum_kernel(int64_t n, const int32_t* __restrict__ v, unsigned long long* __restrict__ out) {
    unsigned long long s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (unsigned long long)v[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

// *out += sum of m[p] over the table positions whose node has class 1 (its
// domain keeps FP64 values)
__global__ void sum_class_kernel(int64_t n, const int32_t* __restrict__ m, const int32_t* __restrict__ node,
                                 const uint8_t* __restrict__ cls, unsigned long long* __restrict__ out) {
    unsigned long long s = 0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        if (cls[node[p]]) s += (unsigned long long)m[p];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

__global__ void count_nonzero_kernel(int64_t n, const int8_t* __restrict__ v, unsigned long long* __restrict__ out) {
    unsigned long long s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += v[i] != 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

cudaError_t launch_count_nonzero(int64_t n, const int8_t* v, unsigned long long* out, int nsm, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    count_nonzero_kernel<<<nsm * 4, 256, 0, s>>>(n, v, out);
    return cudaGetLastError();
}

}  // namespace sgs

// ---------------------------------------------------------------------------
namespace {

const double kSingularTau = 1e-10;            // as for plans: pivot <= tau*sill -> prior
const int64_t kLutCap = (int64_t)1 << 19;     // lag-table entries per domain (4 MB of (hi, lo))

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct sgs_batch {
    std::string err;
    int device = 0, nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    int ndom = 0;
    int precision = SGS_PREC_FP32_REFINE;
    int kmax = 1;                  // largest maxneighbors of the batch
    int64_t Ntot = 0, Dtot = 0;
    int64_t lcap = 1;              // level-count capacity (largest domain + 1)
    std::vector<int64_t> noff;     // ndom + 1 global node offsets
    std::vector<int64_t> nbr0;     // neighbour-row arena offsets
    std::vector<int32_t> kd;       // maxneighbors per domain (after clamping)
    std::vector<double> mean;
    std::vector<SearchArgs> search;   // device pointers filled in
    std::vector<SolveArgs> solve;
    std::vector<Buf> bufs;
    // device
    int64_t* d_noff = nullptr;
    SearchArgs* d_search = nullptr;
    SolveArgs* d_solve = nullptr;
    LevelDom* d_ldom = nullptr;
    int32_t *d_path = nullptr, *d_nbr = nullptr, *d_cnt = nullptr, *d_ngrid = nullptr;
    int32_t *d_level = nullptr, *d_order = nullptr, *d_lcount = nullptr, *d_lfill = nullptr, *d_loff = nullptr;
    int8_t* d_status = nullptr;
    int64_t *d_toff = nullptr, *d_tsum = nullptr;
    int32_t *d_blist = nullptr, *d_bcount = nullptr, *d_bfill = nullptr, *d_bdesc = nullptr;
    int32_t *d_fallback = nullptr, *d_fbdesc = nullptr;
    int32_t* d_scratch = nullptr;  // [0] maxlevel [1] level-wait error
    unsigned long long* d_ticket = nullptr;  // levels ticket
    unsigned long long* d_sums = nullptr;    // [0] sum of grid neighbours (tables) [1] sum_m [2] priors
    unsigned long long* d_flow = nullptr;    // sweep ticket, error flag, second launch's ticket
    uint64_t* d_seed = nullptr;
    uint64_t* h_seed = nullptr;    // pinned
    int32_t* d_done = nullptr;
    int64_t done_cap = 0;
    int64_t table_entries = 0;
    SweepTables<float> t32{};
    SweepTables<double> t64{};
    bool allocated = false, prepared = false;
    // graphs
    // prepare graphs: [1] the whole sequence, [0] everything after the
    // search (the first prepare, whose table-sizing search already ran)
    cudaGraphExec_t prep_exec[2] = {nullptr, nullptr};
    int64_t prep_nodes[2] = {0, 0};
    cudaGraphExec_t sweep_exec = nullptr;
    int64_t sweep_nodes = 0;
    int sweep_Rp = 0;
    void* sweep_V = nullptr;
    cudaStream_t sweep_stream = nullptr;
    sgs_sweep_config sweep{SGS_SWEEP_FLOW, 1, 0, 1, 0, 0, 0, 0, 0, 0.f};
    bool sweep_graph_valid = false;
    bool sweep_pending = false;    // a device-resident sweep not yet checked
    unsigned int* d_wl1 = nullptr; // per domain: largest sum of |grid weights| (FP32 bits)
    // FP32 refinement with FP64 values for the domains whose weights amplify
    // the rounding of stored values (dom_fp64[d]); the value array then has
    // FP64 rows (Rp doubles per node), and the other domains keep FP32 values
    // in the first half of their rows, swept by a second launch (mixed)
    bool promote = false;          // some domain keeps FP64 values
    bool mixed = false;            // ... and some domain FP32 values
    std::vector<uint8_t> dom_fp64;
    uint8_t* d_cls = nullptr;      // per node: 1 = its domain keeps FP64 values
    bool sweep_promote = false;    // value layout the captured sweep graph was built for
    bool sweep_mixed = false;
    sgs_batch_info info{};
};

// the sweep's value type; promoted batches read the packed (hi, lo) FP32
// tables through an FP64-typed view (FlowArgs::pairs)
static bool values_fp64(const sgs_batch* B) { return B->precision == SGS_PREC_FP64 || B->promote; }
// domain d's values: FP64 rows, or FP32 rows (in the first half of each FP64
// row when the batch is mixed)
static bool domain_fp64(const sgs_batch* B, int d) {
    return B->precision == SGS_PREC_FP64 || (B->promote && (!B->mixed || B->dom_fp64[d]));
}
static SweepTables<double> sweep64(const sgs_batch* B) {
    if (!B->promote) return B->t64;
    SweepTables<double> v{};
    v.node = B->t32.node;
    v.m = B->t32.m;
    v.idx = B->t32.idx;
    v.w = reinterpret_cast<double*>(B->t32.w);
    v.b0 = reinterpret_cast<double*>(B->t32.b0);
    v.sigma = reinterpret_cast<double*>(B->t32.sigma);
    v.off = B->t32.off;
    return v;
}

namespace {

int berr(sgs_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    else sgs::set_thread_error(msg);
    return code;
}

int bcuda(sgs_batch* b, cudaError_t e, const char* where) {
    const int code = (e == cudaErrorMemoryAllocation) ? SGS_ERR_OOM : SGS_ERR_CUDA;
    return berr(b, code, std::string(where) + ": " + cudaGetErrorString(e));
}

#define BCK(b, call)                                        \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return bcuda(b, e_, #call);  \
    } while (0)

#define BLAUNCH(b, call)                                    \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return bcuda(b, e_, #call);  \
        ++launched;                                         \
    } while (0)

template <typename T>
int balloc(sgs_batch* b, T** out, size_t count) {
    *out = nullptr;
    if (count == 0) count = 1;
    void* p = nullptr;
    cudaError_t e = pool_alloc(&p, count * sizeof(T), b->device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        return berr(b, SGS_ERR_OOM, "allocation of " + std::to_string(count * sizeof(T)) + " bytes failed (" +
                                        std::to_string(fr) + " bytes free): split the batch");
    }
    b->bufs.push_back({p, count * sizeof(T)});
    b->info.device_bytes += (int64_t)(count * sizeof(T));
    *out = static_cast<T*>(p);
    return SGS_OK;
}

void bfree(sgs_batch* b, void* p) {
    if (!p) return;
    for (size_t i = 0; i < b->bufs.size(); ++i)
        if (b->bufs[i].p == p) {
            pool_free(p, b->stream);
            b->info.device_bytes -= (int64_t)b->bufs[i].bytes;
            b->bufs.erase(b->bufs.begin() + i);
            return;
        }
}

template <typename T>
int bupload_raw(sgs_batch* b, T** d, const T* h, size_t count) {
    int rc = balloc(b, d, count);
    if (rc) return rc;
    if (count) BCK(b, cudaMemcpyAsync(*d, h, count * sizeof(T), cudaMemcpyHostToDevice, b->stream));
    b->info.h2d_bytes += (int64_t)(count * sizeof(T));
    return SGS_OK;
}

template <typename T>
int bupload(sgs_batch* b, T** d, const std::vector<T>& h) {
    return bupload_raw(b, d, h.data(), h.size());
}

// A host arena that is not zero-filled on construction: the threads that
// fill it touch its pages first.
template <typename T>
struct HostArena {
    std::unique_ptr<T[]> p;
    size_t n = 0;
    explicit HostArena(size_t count) : p(new T[count ? count : 1]), n(count) {}
    T* data() { return p.get(); }
    const T* data() const { return p.get(); }
    size_t size() const { return n; }
};

template <typename T>
int bupload(sgs_batch* b, T** d, const HostArena<T>& h) {
    return bupload_raw(b, d, h.data(), h.size());
}

// 0 when the pair cannot be timed (the error is cleared, not left pending)
float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.f;
    }
    return ms;
}

// Lag-table half extents: twice the search template's (every pairwise lag
// of template offsets), shrunk until the table has at most kLutCap entries.
// Systems whose neighbours do not fit evaluate covariances directly.
void lut_extents(const HostDomain& H, int e[3]) {
    for (int j = 0; j < 3; ++j) e[j] = 2 * H.tmpl_ext[j];
    for (;;) {
        int64_t tot = 1;
        for (int j = 0; j < 3; ++j) tot *= 2 * (int64_t)e[j] + 1;
        if (tot <= kLutCap) return;
        int jm = 0;
        for (int j = 1; j < 3; ++j)
            if (e[j] > e[jm]) jm = j;
        e[jm] = std::max(0, e[jm] - std::max(1, e[jm] / 8));
    }
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" const char* sgs_batch_last_error(const sgs_batch* b) {
    return b ? b->err.c_str() : sgs_last_error(nullptr);
}

extern "C" void sgs_batch_destroy(sgs_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    // buffers may still be read by work queued on the caller's streams (the
    // device-pointer entry points): wait for the device, as a synchronous
    // free would
    cudaDeviceSynchronize();
    for (auto& e : b->prep_exec)
        if (e) cudaGraphExecDestroy(e);
    if (b->sweep_exec) cudaGraphExecDestroy(b->sweep_exec);
    for (auto& x : b->bufs) pool_free(x.p, b->stream);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->h_seed) cudaFreeHost(b->h_seed);
    for (auto& e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

static int batch_init(sgs_batch* B, const sgs_problem* pr, int nd) {
    if (nd < 1) return berr(B, SGS_ERR_ARG, "ndomains must be >= 1");
    B->ndom = nd;
    B->precision = pr[0].precision;
    B->device = pr[0].device;
    for (int d = 0; d < nd; ++d) {
        const std::string where = "domain " + std::to_string(d) + ": ";
        if (pr[d].precision != B->precision) return berr(B, SGS_ERR_ARG, where + "all domains need the same precision");
        if (pr[d].device != B->device) return berr(B, SGS_ERR_ARG, where + "all domains need the same device");
        if (pr[d].warm_start) return berr(B, SGS_ERR_ARG, where + "the learned warm start is not available in batches");
        if (pr[d].flags) return berr(B, SGS_ERR_ARG, where + "flags must be 0 in batches (the sweep is the dataflow form)");
    }
    // host set-up of every domain, in parallel (templates dominate)
    std::vector<HostDomain> H(nd);
    std::vector<std::string> errs(nd);
    std::vector<int> rcs(nd, SGS_OK);
    {
        const int nt = std::max(1, std::min<int>(nd, (int)std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back([&, t]() {
                for (int d = t; d < nd; d += nt) rcs[d] = host_domain(&pr[d], H[d], errs[d]);
            });
        for (auto& x : th) x.join();
    }
    for (int d = 0; d < nd; ++d)
        if (rcs[d] != SGS_OK) return berr(B, rcs[d], "domain " + std::to_string(d) + ": " + errs[d]);

    // global numbering
    B->noff.assign(nd + 1, 0);
    B->nbr0.assign(nd + 1, 0);
    std::vector<int64_t> doff(nd + 1, 0), toff(nd + 1, 0), boff(nd + 1, 0), loff(nd + 1, 0);
    std::vector<std::array<int, 3>> lute(nd);
    B->kd.resize(nd);
    B->mean.resize(nd);
    for (int d = 0; d < nd; ++d) {
        B->noff[d + 1] = B->noff[d] + H[d].N;
        B->nbr0[d + 1] = B->nbr0[d] + H[d].N * H[d].k;
        doff[d + 1] = doff[d] + H[d].D;
        toff[d + 1] = toff[d] + (int64_t)H[d].tmpl.size();
        boff[d + 1] = boff[d] + (int64_t)H[d].bstart.size();
        int e[3];
        lut_extents(H[d], e);
        lute[d] = {e[0], e[1], e[2]};
        loff[d + 1] = loff[d] + (2 * (int64_t)e[0] + 1) * (2 * (int64_t)e[1] + 1) * (2 * (int64_t)e[2] + 1);
        B->kd[d] = H[d].k;
        B->mean[d] = H[d].mean;
        B->kmax = std::max(B->kmax, H[d].k);
        B->lcap = std::max<int64_t>(B->lcap, H[d].N + 1);
    }
    B->Ntot = B->noff[nd];
    B->Dtot = doff[nd];
    if (B->Ntot >= (int64_t)INT32_MAX) return berr(B, SGS_ERR_ARG, "a batch holds fewer than 2^31 grid nodes");

    // device
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return berr(B, SGS_ERR_NODEVICE, "no CUDA device");
    }
    if (B->device < 0 || B->device >= ndev) return berr(B, SGS_ERR_ARG, "invalid device ordinal");
    BCK(B, cudaSetDevice(B->device));
    BCK(B, cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, B->device));
    BCK(B, cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
    for (auto& e : B->ev) BCK(B, cudaEventCreate(&e));
    BCK(B, cudaMallocHost(&B->h_seed, sizeof(uint64_t)));

    // arenas
    // path arena: local node ids per domain, as given (or the linear path);
    // the ranks are built and checked on the device
    HostArena<int32_t> path(B->Ntot), did(B->Dtot), bstart(boff[nd]);
    HostArena<TmplEntry> tmpl(toff[nd]);
    HostArena<double> td2(toff[nd]), xyz(3 * B->Dtot), val(B->Dtot), xyzb(3 * B->Dtot);
    HostArena<float4> xf(B->Dtot);
    {
        // the arenas (GBs of paths, ranks and templates) are filled by all
        // host threads, each domain's slices by one thread
        const int nt = std::max(1, std::min<int>(nd, (int)std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back([&, t]() {
                for (int d = t; d < nd; d += nt) {
                    const HostDomain& h = H[d];
                    int32_t* pd = path.data() + B->noff[d];
                    if (pr[d].path) std::copy(pr[d].path, pr[d].path + h.N, pd);
                    else for (int64_t t = 0; t < h.N; ++t) pd[t] = (int32_t)t;
                    std::copy(h.tmpl.begin(), h.tmpl.end(), tmpl.data() + toff[d]);
                    std::copy(h.tmpl_d2.begin(), h.tmpl_d2.end(), td2.data() + toff[d]);
                    std::copy(h.xyz.begin(), h.xyz.end(), xyz.data() + 3 * doff[d]);
                    std::copy(h.val.begin(), h.val.end(), val.data() + doff[d]);
                    std::copy(h.xyz_b.begin(), h.xyz_b.end(), xyzb.data() + 3 * doff[d]);
                    std::copy(h.did.begin(), h.did.end(), did.data() + doff[d]);
                    std::copy(h.xf.begin(), h.xf.end(), xf.data() + doff[d]);
                    std::copy(h.bstart.begin(), h.bstart.end(), bstart.data() + boff[d]);
                }
            });
        for (auto& x : th) x.join();
    }
    int rc;
    int32_t *d_rank, *d_did, *d_bstart;
    TmplEntry* d_tmpl;
    double *d_td2, *d_xyz, *d_val, *d_xyzb;
    float4* d_xf;
    float2* d_lut;
    if ((rc = bupload(B, &B->d_path, path))) return rc;
    if ((rc = bupload(B, &B->d_noff, B->noff))) return rc;
    {
        int32_t* d_bad = nullptr;
        if ((rc = balloc(B, &d_rank, B->Ntot)) || (rc = balloc(B, &d_bad, 1))) return rc;
        const int32_t nd32 = nd;
        BCK(B, cudaMemsetAsync(d_rank, 0xff, (size_t)B->Ntot * sizeof(int32_t), B->stream));
        BCK(B, cudaMemcpyAsync(d_bad, &nd32, sizeof(int32_t), cudaMemcpyHostToDevice, B->stream));
        BCK(B, launch_batch_path_ranks(B->d_path, B->d_noff, nd, B->Ntot, d_rank, d_bad, B->nsm, B->stream));
        B->info.launches += 2;
        int32_t bad = nd;
        BCK(B, cudaMemcpyAsync(&bad, d_bad, sizeof(int32_t), cudaMemcpyDeviceToHost, B->stream));
        BCK(B, cudaStreamSynchronize(B->stream));
        bfree(B, d_bad);
        if (bad < nd)
            return berr(B, SGS_ERR_ARG, "domain " + std::to_string(bad) + ": path is not a permutation of the grid nodes");
    }
    if ((rc = bupload(B, &d_tmpl, tmpl))) return rc;
    if ((rc = bupload(B, &d_td2, td2))) return rc;
    if ((rc = bupload(B, &d_xyz, xyz))) return rc;
    if ((rc = bupload(B, &d_val, val))) return rc;
    if ((rc = bupload(B, &d_xyzb, xyzb))) return rc;
    if ((rc = bupload(B, &d_did, did))) return rc;
    if ((rc = bupload(B, &d_bstart, bstart))) return rc;
    if ((rc = bupload(B, &d_xf, xf))) return rc;
    if ((rc = balloc(B, &d_lut, loff[nd]))) return rc;
    // results
    if ((rc = balloc(B, &B->d_nbr, B->nbr0[nd]))) return rc;
    if ((rc = balloc(B, &B->d_cnt, B->Ntot))) return rc;
    if ((rc = balloc(B, &B->d_ngrid, B->Ntot))) return rc;
    if ((rc = balloc(B, &B->d_level, B->Ntot))) return rc;
    if ((rc = balloc(B, &B->d_order, B->Ntot))) return rc;
    if ((rc = balloc(B, &B->d_status, B->Ntot))) return rc;
    if ((rc = balloc(B, &B->d_lcount, B->lcap))) return rc;
    if ((rc = balloc(B, &B->d_lfill, B->lcap))) return rc;
    if ((rc = balloc(B, &B->d_loff, B->lcap + 1))) return rc;
    if ((rc = balloc(B, &B->d_toff, B->Ntot + 1))) return rc;
    if ((rc = balloc(B, &B->d_tsum, (B->Ntot + SCAN_TILE - 1) / SCAN_TILE + 1))) return rc;
    if ((rc = balloc(B, &B->d_blist, B->Ntot))) return rc;
    if ((rc = balloc(B, &B->d_bcount, 2 * NBIN))) return rc;  // counts, fill cursors
    B->d_bfill = B->d_bcount + NBIN;
    if ((rc = balloc(B, &B->d_bdesc, 2 * NBIN))) return rc;
    if ((rc = balloc(B, &B->d_fallback, B->Ntot))) return rc;
    if ((rc = balloc(B, &B->d_fbdesc, 2))) return rc;
    if ((rc = balloc(B, &B->d_scratch, 4))) return rc;
    if ((rc = balloc(B, &B->d_ticket, 1))) return rc;
    if ((rc = balloc(B, &B->d_sums, 4))) return rc;
    if ((rc = balloc(B, &B->d_flow, 3))) return rc;
    if ((rc = balloc(B, &B->d_seed, 1))) return rc;
    if ((rc = balloc(B, &B->d_wl1, nd))) return rc;

    // descriptors
    B->search.resize(nd);
    B->solve.resize(nd);
    std::vector<LevelDom> ld(nd);
    for (int d = 0; d < nd; ++d) {
        const HostDomain& h = H[d];
        SearchArgs& sa = B->search[d];
        sa = SearchArgs{};
        search_args_of(h, sa);
        sa.tmpl = d_tmpl + toff[d];
        sa.tmpl_d2 = d_td2 + toff[d];
        sa.path = B->d_path + B->noff[d];
        sa.rank = d_rank + B->noff[d];
        sa.dxyz = d_xyzb + 3 * doff[d];
        sa.dxyz_f = d_xf + doff[d];
        sa.did = d_did + doff[d];
        sa.bstart = d_bstart + boff[d];
        sa.nbr = B->d_nbr + B->nbr0[d];
        sa.cnt = B->d_cnt + B->noff[d];
        sa.ngrid = B->d_ngrid + B->noff[d];

        SolveArgs& s = B->solve[d];
        s = SolveArgs{};
        s.grid = h.grid;
        s.vario = h.vario;
        s.lut.c64 = nullptr;
        s.lut.c2 = d_lut + loff[d];
        for (int j = 0; j < 3; ++j) {
            s.lut.e[j] = lute[d][j];
            s.lut.w[j] = 2 * lute[d][j] + 1;
        }
        s.k = h.k;
        s.nmin = h.nmin;
        s.mu = h.mean;
        s.tau = kSingularTau * h.vario.sill;
        s.inv_sill = 1.0 / h.vario.sill;
        s.refine_steps = pr[d].refine_steps;
        s.P = h.N;
        s.nbr = sa.nbr;
        s.cnt = sa.cnt;
        s.N = h.N;
        s.data_xyz = d_xyz + 3 * doff[d];
        s.data_val = d_val + doff[d];
        s.status = B->d_status + B->noff[d];
        s.fallback = B->d_fallback;
        s.nfallback = B->d_fbdesc;
        s.sum_m = B->d_sums + 1;
        s.wl1_max = B->d_wl1 + d;
        s.node0 = B->noff[d];

        ld[d] = LevelDom{B->noff[d], B->nbr0[d], (int32_t)h.N, h.k};
    }
    if ((rc = bupload(B, &B->d_search, B->search))) return rc;
    if ((rc = bupload(B, &B->d_solve, B->solve))) return rc;
    if ((rc = bupload(B, &B->d_ldom, ld))) return rc;
    // lag tables, one launch per domain (geometry and variogram only)
    for (int d = 0; d < nd; ++d) {
        cudaError_t e = launch_fill_cov_lut(H[d].grid, H[d].vario, B->solve[d].lut, nullptr, d_lut + loff[d], B->stream);
        if (e != cudaSuccess) return bcuda(B, e, "lag table");
        B->info.launches++;
    }
    BCK(B, cudaStreamSynchronize(B->stream));
    B->info.ndomains = nd;
    B->info.nnodes = B->Ntot;
    B->info.ndata = B->Dtot;
    return SGS_OK;
}

extern "C" int sgs_batch_create(const sgs_problem* problems, int32_t ndomains, sgs_batch** batch) {
    if (!problems || !batch) return berr(nullptr, SGS_ERR_ARG, "null argument");
    *batch = nullptr;
    sgs_batch* B = new sgs_batch();
    const int rc = batch_init(B, problems, ndomains);
    if (rc != SGS_OK) {
        sgs::set_thread_error(B->err);
        sgs_batch_destroy(B);
        return rc;
    }
    *batch = B;
    return SGS_OK;
}

// The prepare sequence: every launch is stream-ordered and reads its sizes
// on the device, so it is captured once and replayed.  The phase events are
// recorded as external event nodes (a plain record inside a capture only
// marks a dependency), so they time the replayed graph.
// with_search false: the sequence after the neighbour search (its results
// already in place)
static int enqueue_prepare(sgs_batch* B, int64_t& launched, bool with_search) {
    cudaStream_t st = B->stream;
    const int64_t N = B->Ntot;
    const int nd = B->ndom;
    if (with_search) {
        BCK(B, cudaEventRecordWithFlags(B->ev[0], st, cudaEventRecordExternal));
        BLAUNCH(B, launch_search_batch(B->d_search, B->d_noff, nd, N, B->nsm, st));
        BCK(B, cudaEventRecordWithFlags(B->ev[1], st, cudaEventRecordExternal));
    }
    // levels and level order
    BCK(B, cudaMemsetAsync(B->d_level, 0xff, N * sizeof(int32_t), st));
    BCK(B, cudaMemsetAsync(B->d_scratch, 0, 4 * sizeof(int32_t), st));
    BCK(B, cudaMemsetAsync(B->d_ticket, 0, sizeof(unsigned long long), st));
    BCK(B, cudaMemsetAsync(B->d_lcount, 0, B->lcap * sizeof(int32_t), st));
    BCK(B, cudaMemsetAsync(B->d_lfill, 0, B->lcap * sizeof(int32_t), st));
    levels_batch_kernel<<<B->nsm * 8, 256, 0, st>>>(B->d_ldom, B->d_noff, nd, B->d_path, B->d_nbr, B->d_cnt,
                                                     B->d_level, B->d_ticket, B->d_scratch, B->d_scratch + 1,
                                                     LEVEL_WAIT_NS);
    BLAUNCH(B, cudaGetLastError());
    const unsigned lb = (unsigned)((N + BL_NODES - 1) / BL_NODES);
    level_count_batch_kernel<<<lb, 256, 0, st>>>(N, B->d_level, B->d_scratch, B->d_lcount);
    BLAUNCH(B, cudaGetLastError());
    level_scan_kernel<<<1, 1024, 0, st>>>(B->d_scratch, B->d_lcount, B->d_loff);
    BLAUNCH(B, cudaGetLastError());
    level_fill_batch_kernel<<<lb, 256, 0, st>>>(N, B->d_level, B->d_scratch, B->d_loff, B->d_lfill, B->d_order);
    BLAUNCH(B, cudaGetLastError());
    // packed table rows and size classes
    const int64_t ntiles = (N + SCAN_TILE - 1) / SCAN_TILE;
    tile_sum_kernel<<<(unsigned)ntiles, SCAN_THREADS, 0, st>>>(N, B->d_order, B->d_ngrid, B->d_tsum);
    BLAUNCH(B, cudaGetLastError());
    tile_scan_kernel<<<1, 1024, 0, st>>>(ntiles, B->d_tsum);
    BLAUNCH(B, cudaGetLastError());
    tile_apply_kernel<<<(unsigned)ntiles, SCAN_THREADS, 0, st>>>(N, B->d_order, B->d_ngrid, B->d_tsum, B->d_toff);
    BLAUNCH(B, cudaGetLastError());
    BCK(B, cudaMemsetAsync(B->d_bcount, 0, 2 * NBIN * sizeof(int32_t), st));
    const unsigned bb = (unsigned)((N + BIN_NODES - 1) / BIN_NODES);
    bin_count_kernel<<<bb, 256, 0, st>>>(N, B->d_order, B->d_cnt, B->d_bcount);
    BLAUNCH(B, cudaGetLastError());
    bin_fill_kernel<<<bb, 256, 0, st>>>(N, B->d_order, B->d_cnt, B->d_bcount, B->d_bfill, B->d_blist, B->d_bdesc);
    BLAUNCH(B, cudaGetLastError());
    BCK(B, cudaEventRecordWithFlags(B->ev[2], st, cudaEventRecordExternal));
    // kriging systems by size class
    BCK(B, cudaMemsetAsync(B->d_fbdesc, 0, 2 * sizeof(int32_t), st));
    BCK(B, cudaMemsetAsync(B->d_sums + 1, 0, sizeof(unsigned long long), st));
    BCK(B, cudaMemsetAsync(B->d_wl1, 0, (size_t)B->ndom * sizeof(unsigned int), st));
    for (int b = 0; b < NBIN; ++b) {
        if (B->precision == SGS_PREC_FP64)
            BLAUNCH(B, launch_solve_fp64_batch(bin_nmax(b), B->d_solve, B->d_noff, nd, B->d_order, B->d_blist,
                                               B->d_bdesc + 2 * b, B->t64, B->nsm, st));
        else
            BLAUNCH(B, launch_solve_fp32_batch(bin_nmax(b), B->d_solve, B->d_noff, nd, B->d_order, B->d_blist,
                                               B->d_bdesc + 2 * b, B->t32, B->nsm, st));
    }
    if (B->precision != SGS_PREC_FP64)  // queued systems: FP64 re-solve (canonical decision)
        BLAUNCH(B, launch_solve_fp64_into_fp32_batch(B->kmax, B->d_solve, B->d_noff, nd, B->d_order, B->d_fallback,
                                                     B->d_fbdesc, B->t32, B->nsm, st));
    BCK(B, cudaEventRecordWithFlags(B->ev[3], st, cudaEventRecordExternal));
    return SGS_OK;
}

extern "C" int sgs_batch_prepare(sgs_batch* B) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    BCK(B, cudaSetDevice(B->device));
    cudaStream_t st = B->stream;
    int rc;
    int64_t launched = 0;
    bool searched = false;
    if (!B->allocated) {
        // size the packed sweep tables: one search, then the grid-neighbour
        // sum; this prepare then runs the rest of the sequence only
        BCK(B, cudaEventRecord(B->ev[0], st));
        BLAUNCH(B, launch_search_batch(B->d_search, B->d_noff, B->ndom, B->Ntot, B->nsm, st));
        BCK(B, cudaEventRecord(B->ev[1], st));
        searched = true;
        BCK(B, cudaMemsetAsync(B->d_sums, 0, sizeof(unsigned long long), st));
        sum_kernel<<<B->nsm * 4, 256, 0, st>>>(B->Ntot, B->d_ngrid, B->d_sums);
        BLAUNCH(B, cudaGetLastError());
        unsigned long long tot = 0;
        BCK(B, cudaMemcpyAsync(&tot, B->d_sums, sizeof(tot), cudaMemcpyDeviceToHost, st));
        BCK(B, cudaStreamSynchronize(st));
        B->info.d2h_bytes += sizeof(tot);
        B->table_entries = (int64_t)tot;
        const int64_t N = B->Ntot, E = std::max<int64_t>(1, B->table_entries);
        if (B->precision == SGS_PREC_FP64) {
            if ((rc = balloc(B, &B->t64.node, N))) return rc;
            if ((rc = balloc(B, &B->t64.m, N))) return rc;
            if ((rc = balloc(B, &B->t64.idx, E))) return rc;
            if ((rc = balloc(B, &B->t64.w, E))) return rc;
            if ((rc = balloc(B, &B->t64.b0, N))) return rc;
            if ((rc = balloc(B, &B->t64.sigma, N))) return rc;
            B->t64.off = B->d_toff;
        } else {
            if ((rc = balloc(B, &B->t32.node, N))) return rc;
            if ((rc = balloc(B, &B->t32.m, N))) return rc;
            if ((rc = balloc(B, &B->t32.idx, E))) return rc;
            if ((rc = balloc(B, &B->t32.w, 2 * E))) return rc;
            if ((rc = balloc(B, &B->t32.b0, 2 * N))) return rc;
            if ((rc = balloc(B, &B->t32.sigma, 2 * N))) return rc;
            B->t32.off = B->d_toff;
        }
        B->allocated = true;
        B->info.launches += launched;
        launched = 0;
    }
    const int gi = searched ? 0 : 1;
    if (!B->prep_exec[gi]) {
        cudaGraph_t g = nullptr;
        BCK(B, cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
        rc = enqueue_prepare(B, launched, !searched);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return bcuda(B, ce, "cudaStreamEndCapture (prepare)");
        ce = cudaGraphInstantiate(&B->prep_exec[gi], g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            B->prep_exec[gi] = nullptr;
            return bcuda(B, ce, "cudaGraphInstantiate (prepare)");
        }
        B->prep_nodes[gi] = launched;
    }
    BCK(B, cudaGraphLaunch(B->prep_exec[gi], st));
    B->info.graph_launches++;
    B->info.launches += B->prep_nodes[gi];
    // statistics (after the graph)
    BCK(B, cudaMemsetAsync(B->d_sums + 2, 0, sizeof(unsigned long long), st));
    count_nonzero_kernel<<<B->nsm * 4, 256, 0, st>>>(B->Ntot, B->d_status, B->d_sums + 2);
    BCK(B, cudaGetLastError());
    B->info.launches++;
    int32_t hs[4] = {0, 0, 0, 0};
    unsigned long long su[4] = {0, 0, 0, 0};
    int32_t hb[2 * NBIN], hf[2];
    std::vector<unsigned int> wl1(B->ndom);
    BCK(B, cudaMemcpyAsync(wl1.data(), B->d_wl1, wl1.size() * sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    BCK(B, cudaMemcpyAsync(hs, B->d_scratch, sizeof(hs), cudaMemcpyDeviceToHost, st));
    BCK(B, cudaMemcpyAsync(su, B->d_sums, sizeof(su), cudaMemcpyDeviceToHost, st));
    BCK(B, cudaMemcpyAsync(hb, B->d_bdesc, sizeof(hb), cudaMemcpyDeviceToHost, st));
    BCK(B, cudaMemcpyAsync(hf, B->d_fbdesc, sizeof(hf), cudaMemcpyDeviceToHost, st));
    BCK(B, cudaStreamSynchronize(st));
    B->info.d2h_bytes += sizeof(hs) + sizeof(su) + sizeof(hb) + sizeof(hf) + wl1.size() * sizeof(unsigned int);
    if (hs[1]) return berr(B, SGS_ERR_TIMEOUT, "dependency-level wait exceeded its bound");
    {
        // value precision per domain: FP64 values only where the domain's
        // weights amplify the rounding of stored FP32 values
        float fmax = 0.0f;
        int nfp64 = 0;
        B->dom_fp64.assign(B->ndom, 0);
        for (int d = 0; d < B->ndom; ++d) {
            float f;
            std::memcpy(&f, &wl1[d], sizeof(f));
            fmax = std::max(fmax, f);
            if (B->precision == SGS_PREC_FP32_REFINE && f > SGS_FP32_VALUE_L1_LIMIT) {
                B->dom_fp64[d] = 1;
                ++nfp64;
            }
        }
        B->info.weight_l1_max = fmax;
        B->promote = nfp64 > 0;
        B->mixed = nfp64 > 0 && nfp64 < B->ndom;
        if (B->mixed) {
            if (!B->d_cls) {
                int rc = balloc(B, &B->d_cls, B->Ntot);
                if (rc) return rc;
            }
            BCK(B, cudaMemsetAsync(B->d_cls, 0, (size_t)B->Ntot, st));
            for (int d = 0; d < B->ndom; ++d)
                if (B->dom_fp64[d])
                    BCK(B, cudaMemsetAsync(B->d_cls + B->noff[d], 1, (size_t)(B->noff[d + 1] - B->noff[d]), st));
        }
        B->info.values_fp64 = values_fp64(B) ? 1 : 0;
        B->info.domains_fp64 = B->precision == SGS_PREC_FP64 ? B->ndom : nfp64;
        // grid neighbours of the FP64-value domains' nodes (value traffic of
        // the sweep per precision class)
        if (B->mixed) {
            BCK(B, cudaMemsetAsync(B->d_sums + 3, 0, sizeof(unsigned long long), st));
            sum_class_kernel<<<B->nsm * 4, 256, 0, st>>>(B->Ntot, B->t32.m, B->t32.node, B->d_cls, B->d_sums + 3);
            BCK(B, cudaGetLastError());
            B->info.launches++;
            unsigned long long s64 = 0;
            BCK(B, cudaMemcpyAsync(&s64, B->d_sums + 3, sizeof(s64), cudaMemcpyDeviceToHost, st));
            BCK(B, cudaStreamSynchronize(st));
            B->info.d2h_bytes += sizeof(s64);
            B->info.sum_grid_neighbors_fp64 = (int64_t)s64;
        } else {
            B->info.sum_grid_neighbors_fp64 = values_fp64(B) ? (int64_t)su[1] : 0;
        }
    }
    B->info.nlevels = hs[0] + 1;
    B->info.sum_grid_neighbors = (int64_t)su[1];
    B->info.n_prior = (int64_t)su[2];
    B->info.n_fp64_fallback = B->precision == SGS_PREC_FP64 ? 0 : hf[0];
    for (int b = 0; b < NBIN; ++b) B->info.bin_systems[b] = hb[2 * b];
    B->info.ms_search = elapsed_ms(B->ev[0], B->ev[1]);
    B->info.ms_levels = elapsed_ms(B->ev[1], B->ev[2]);
    B->info.ms_solve = elapsed_ms(B->ev[2], B->ev[3]);
    B->info.ms_prepare = elapsed_ms(B->ev[0], B->ev[3]);
    B->prepared = true;
    return SGS_OK;
}

// The sweep: flags cleared, then one persistent dataflow launch over every
// position of the batch's level order.
static int enqueue_sweep(sgs_batch* B, int Rp, const void* z, void* V, cudaStream_t st, int64_t& launched) {
    const sgs_sweep_config& c = B->sweep;
    int W = c.lanes_w, G = c.lanes_g;
    const int H = flow_layout(Rp, W, G);
    const int64_t nflags = B->Ntot * H;
    if (nflags > B->done_cap) return berr(B, SGS_ERR_STATE, "sweep flags not allocated");
    BCK(B, cudaMemsetAsync(B->d_done, 0, nflags * sizeof(int32_t), st));
    BCK(B, cudaMemsetAsync(B->d_flow, 0, 3 * sizeof(unsigned long long), st));
    FlowArgs f{};
    f.item0 = 0;
    f.item1 = B->Ntot * H;
    f.N = B->Ntot;
    f.H = H;
    f.done = B->d_done;
    f.epoch = 1;
    f.ticket = B->d_flow;
    f.err = reinterpret_cast<int32_t*>(B->d_flow + 1);
    f.chunk = std::max(1, c.chunk);
    f.blocks_per_sm = c.blocks_per_sm;
    f.tight = c.tight;
    f.wait_ns = 10000000000ull;  // 10 s: far beyond any dependency chain
    f.seed_dev = B->d_seed;
    f.pairs = B->promote ? 1 : 0;
    if (B->mixed) {
        // two launches over disjoint domains: FP32 values in the first half
        // of each FP64 row, then the FP64 domains with their own ticket
        FlowArgs f32 = f;
        f32.pairs = 0;
        f32.row_stride = 2 * (int64_t)Rp;
        f32.node_class = B->d_cls;
        f32.cls = 0;
        BLAUNCH(B, launch_sweep_flow_fp32(B->t32, B->kmax, Rp, W, G, (const float*)z, 0, (float*)V, f32, B->nsm, st));
        FlowArgs f64 = f;
        f64.ticket = B->d_flow + 2;
        f64.node_class = B->d_cls;
        f64.cls = 1;
        BLAUNCH(B, launch_sweep_flow_fp64(sweep64(B), B->kmax, Rp, W, G, (const double*)z, 0, (double*)V, f64, B->nsm,
                                          st));
    } else if (values_fp64(B)) {
        BLAUNCH(B, launch_sweep_flow_fp64(sweep64(B), B->kmax, Rp, W, G, (const double*)z, 0, (double*)V, f, B->nsm, st));
    } else {
        BLAUNCH(B, launch_sweep_flow_fp32(B->t32, B->kmax, Rp, W, G, (const float*)z, 0, (float*)V, f, B->nsm, st));
    }
    return SGS_OK;
}

static int ensure_flags(sgs_batch* B, int Rp) {
    int W = B->sweep.lanes_w, G = B->sweep.lanes_g;
    const int64_t need = B->Ntot * flow_layout(Rp, W, G);
    if (need <= B->done_cap) return SGS_OK;
    BCK(B, cudaStreamSynchronize(B->stream));
    if (B->sweep_exec) {
        cudaGraphExecDestroy(B->sweep_exec);
        B->sweep_exec = nullptr;
    }
    bfree(B, B->d_done);
    B->d_done = nullptr;
    B->done_cap = 0;
    int rc;
    if ((rc = balloc(B, &B->d_done, need))) return rc;
    B->done_cap = need;
    return SGS_OK;
}

static int check_sweep_error(sgs_batch* B) {
    int32_t e = 0;
    BCK(B, cudaMemcpy(&e, B->d_flow + 1, sizeof(e), cudaMemcpyDeviceToHost));
    if (e) return berr(B, SGS_ERR_TIMEOUT, "dataflow sweep: a dependency wait exceeded its bound");
    return SGS_OK;
}

// Seeded sweep into V ([Ntot][Rp]) through the cached graph.
static int run_sweep_graph(sgs_batch* B, int Rp, uint64_t seed, void* V, cudaStream_t st) {
    int rc;
    if ((rc = ensure_flags(B, Rp))) return rc;
    if (!B->sweep_exec || B->sweep_Rp != Rp || B->sweep_V != V || B->sweep_stream != st || !B->sweep_graph_valid ||
        B->sweep_promote != B->promote || B->sweep_mixed != B->mixed) {
        if (B->sweep_exec) {
            BCK(B, cudaStreamSynchronize(B->sweep_stream ? B->sweep_stream : B->stream));
            cudaGraphExecDestroy(B->sweep_exec);
            B->sweep_exec = nullptr;
        }
        int64_t launched = 0;
        cudaGraph_t g = nullptr;
        BCK(B, cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
        rc = enqueue_sweep(B, Rp, nullptr, V, st, launched);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return bcuda(B, ce, "cudaStreamEndCapture (sweep)");
        ce = cudaGraphInstantiate(&B->sweep_exec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            B->sweep_exec = nullptr;
            return bcuda(B, ce, "cudaGraphInstantiate (sweep)");
        }
        B->sweep_nodes = launched;
        B->sweep_Rp = Rp;
        B->sweep_V = V;
        B->sweep_stream = st;
        B->sweep_promote = B->promote;
        B->sweep_mixed = B->mixed;
        B->sweep_graph_valid = true;
    }
    *B->h_seed = seed;
    BCK(B, cudaMemcpyAsync(B->d_seed, B->h_seed, sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    B->info.h2d_bytes += sizeof(uint64_t);
    BCK(B, cudaEventRecord(B->ev[4], st));
    BCK(B, cudaGraphLaunch(B->sweep_exec, st));
    BCK(B, cudaEventRecord(B->ev[5], st));
    B->info.graph_launches++;
    B->info.launches += B->sweep_nodes;
    return SGS_OK;
}

extern "C" int sgs_batch_simulate_device(sgs_batch* B, int32_t R, uint64_t seed, void* vals_dev, void* stream) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (!B->prepared) return berr(B, SGS_ERR_STATE, "simulate before prepare");
    if (R < 1 || !vals_dev) return berr(B, SGS_ERR_ARG, "invalid nreals or output");
    BCK(B, cudaSetDevice(B->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : B->stream;
    const int rc = run_sweep_graph(B, (R + 3) / 4 * 4, seed, vals_dev, st);
    if (rc == SGS_OK) B->sweep_pending = true;
    return rc;
}

extern "C" int sgs_batch_simulate(sgs_batch* B, int32_t R, const double* z, uint64_t seed, double* out) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (!B->prepared) return berr(B, SGS_ERR_STATE, "simulate before prepare");
    if (R < 1 || !out) return berr(B, SGS_ERR_ARG, "invalid nreals or output");
    BCK(B, cudaSetDevice(B->device));
    cudaStream_t st = B->stream;
    const int Rp = (R + 3) / 4 * 4;
    const bool f64 = values_fp64(B);
    const size_t es = f64 ? sizeof(double) : sizeof(float);
    int rc;
    unsigned char* V = nullptr;
    unsigned char* zr = nullptr;
    double* zin = nullptr;
    int64_t maxn = 0;
    for (int d = 0; d < B->ndom; ++d) maxn = std::max(maxn, B->noff[d + 1] - B->noff[d]);
    if ((rc = balloc(B, &V, (size_t)B->Ntot * Rp * es))) return rc;
    auto cleanup = [&]() {
        bfree(B, V);
        bfree(B, zr);
        bfree(B, zin);
    };
    int64_t launched = 0;
    if (z) {
        if ((rc = balloc(B, &zr, (size_t)B->Ntot * Rp * es)) ||
            (rc = balloc(B, &zin, (size_t)std::max<int64_t>(1, maxn) * R))) {
            cleanup();
            return rc;
        }
        BCK(B, cudaMemsetAsync(zr, 0, (size_t)B->Ntot * Rp * es, st));
        for (int d = 0; d < B->ndom; ++d) {
            const int64_t n0 = B->noff[d], n = B->noff[d + 1] - n0;
            BCK(B, cudaMemcpyAsync(zin, z + R * n0, (size_t)n * R * sizeof(double), cudaMemcpyHostToDevice, st));
            B->info.h2d_bytes += (int64_t)n * R * sizeof(double);
            if (domain_fp64(B, d)) BLAUNCH(B, launch_z_to_rows_fp64(zin, n, R, Rp, (double*)zr + n0 * Rp, st));
            else if (f64) BLAUNCH(B, launch_z_to_rows_fp32(zin, n, R, 2 * Rp, (float*)((double*)zr + n0 * Rp), st));
            else BLAUNCH(B, launch_z_to_rows_fp32(zin, n, R, Rp, (float*)zr + n0 * Rp, st));
        }
        if ((rc = ensure_flags(B, Rp))) {
            cleanup();
            return rc;
        }
        BCK(B, cudaEventRecord(B->ev[4], st));
        if ((rc = enqueue_sweep(B, Rp, zr, V, st, launched))) {
            cleanup();
            return rc;
        }
        BCK(B, cudaEventRecord(B->ev[5], st));
    } else if ((rc = run_sweep_graph(B, Rp, seed, V, st))) {
        cleanup();
        return rc;
    }
    // realization-major FP64 output by domain, the domain's mean added:
    // written by the transposing kernels straight into `out` when it is
    // page-locked host memory, else through a device buffer
    double* dout = pinned_device_view(out);
    for (int d = 0; dout && d < B->ndom; ++d) {
        const int64_t n0 = B->noff[d], n = B->noff[d + 1] - n0;
        if (domain_fp64(B, d))
            BLAUNCH(B, launch_rows_to_out_fp64((const double*)V + n0 * Rp, n, R, Rp, B->mean[d], dout + R * n0, st));
        else if (f64)
            BLAUNCH(B, launch_rows_to_out_fp32((const float*)((const double*)V + n0 * Rp), n, R, 2 * Rp, B->mean[d],
                                               dout + R * n0, st));
        else
            BLAUNCH(B, launch_rows_to_out_fp32((const float*)V + n0 * Rp, n, R, Rp, B->mean[d], dout + R * n0, st));
        B->info.d2h_bytes += (int64_t)n * R * sizeof(double);
    }
    double* ob = nullptr;
    const int64_t chunk_bytes = (int64_t)1 << 28;
    const int64_t ob_elems = std::max<int64_t>(1, std::min<int64_t>((int64_t)R * maxn, chunk_bytes / 8 + maxn));
    if (!dout && (rc = balloc(B, &ob, (size_t)ob_elems))) {
        cleanup();
        return rc;
    }
    for (int d = 0; !dout && d < B->ndom; ++d) {
        const int64_t n0 = B->noff[d], n = B->noff[d + 1] - n0;
        const int64_t rchunk = std::max<int64_t>(1, std::min<int64_t>(R, ob_elems / std::max<int64_t>(1, n)));
        for (int64_t r0 = 0; r0 < R; r0 += rchunk) {
            const int rn = (int)std::min<int64_t>(rchunk, R - r0);
            if (domain_fp64(B, d))
                BLAUNCH(B, launch_rows_to_out_fp64((const double*)V + n0 * Rp + r0, n, rn, Rp, B->mean[d], ob, st));
            else if (f64)
                BLAUNCH(B, launch_rows_to_out_fp32((const float*)((const double*)V + n0 * Rp) + r0, n, rn, 2 * Rp,
                                                   B->mean[d], ob, st));
            else
                BLAUNCH(B, launch_rows_to_out_fp32((const float*)V + n0 * Rp + r0, n, rn, Rp, B->mean[d], ob, st));
            BCK(B, cudaMemcpyAsync(out + R * n0 + r0 * n, ob, (size_t)n * rn * sizeof(double), cudaMemcpyDeviceToHost, st));
            B->info.d2h_bytes += (int64_t)n * rn * sizeof(double);
        }
    }
    BCK(B, cudaStreamSynchronize(st));
    B->info.launches += launched;
    rc = check_sweep_error(B);
    B->info.ms_sweep = elapsed_ms(B->ev[4], B->ev[5]);
    bfree(B, ob);
    cleanup();
    return rc;
}

extern "C" int sgs_batch_domain(const sgs_batch* B, int32_t d, int64_t* first, int64_t* nnodes) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (d < 0 || d >= B->ndom) return berr(const_cast<sgs_batch*>(B), SGS_ERR_ARG, "domain out of range");
    if (first) *first = B->noff[d];
    if (nnodes) *nnodes = B->noff[d + 1] - B->noff[d];
    return SGS_OK;
}

extern "C" int sgs_batch_domain_values_fp64(const sgs_batch* B, int32_t d, int32_t* fp64) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (!B->prepared) return berr(const_cast<sgs_batch*>(B), SGS_ERR_STATE, "values_fp64 before prepare");
    if (d < 0 || d >= B->ndom || !fp64) return berr(const_cast<sgs_batch*>(B), SGS_ERR_ARG, "domain out of range");
    *fp64 = domain_fp64(B, d) ? 1 : 0;
    return SGS_OK;
}

extern "C" int sgs_batch_neighbors(sgs_batch* B, int32_t d, int32_t* idx, int32_t* count) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (!B->prepared) return berr(B, SGS_ERR_STATE, "neighbors before prepare");
    if (d < 0 || d >= B->ndom) return berr(B, SGS_ERR_ARG, "domain out of range");
    BCK(B, cudaSetDevice(B->device));
    const int64_t n = B->noff[d + 1] - B->noff[d];
    if (idx) BCK(B, cudaMemcpy(idx, B->d_nbr + B->nbr0[d], (size_t)n * B->kd[d] * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (count) BCK(B, cudaMemcpy(count, B->d_cnt + B->noff[d], (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    B->info.d2h_bytes += (idx ? n * B->kd[d] * 4 : 0) + (count ? n * 4 : 0);
    return SGS_OK;
}

extern "C" int sgs_batch_weights(sgs_batch* B, int32_t d, double* weights, double* sigma, int32_t* status) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (!B->prepared) return berr(B, SGS_ERR_STATE, "weights before prepare");
    if (d < 0 || d >= B->ndom) return berr(B, SGS_ERR_ARG, "domain out of range");
    BCK(B, cudaSetDevice(B->device));
    cudaStream_t st = B->stream;
    const int64_t n = B->noff[d + 1] - B->noff[d];
    int rc;
    if (weights || sigma) {
        // re-run the solves with domain d's export pointers set
        double *wf = nullptr, *sf = nullptr;
        if ((rc = balloc(B, &wf, (size_t)n * B->kd[d]))) return rc;
        if ((rc = balloc(B, &sf, (size_t)n))) {
            bfree(B, wf);
            return rc;
        }
        SolveArgs s = B->solve[d];
        s.w_full = wf;
        s.sigma_full = sf;
        BCK(B, cudaMemcpyAsync(B->d_solve + d, &s, sizeof(s), cudaMemcpyHostToDevice, st));
        int64_t launched = 0;
        BCK(B, cudaMemsetAsync(B->d_fbdesc, 0, 2 * sizeof(int32_t), st));
        for (int b = 0; b < NBIN; ++b) {
            if (B->precision == SGS_PREC_FP64)
                BLAUNCH(B, launch_solve_fp64_batch(bin_nmax(b), B->d_solve, B->d_noff, B->ndom, B->d_order, B->d_blist,
                                                   B->d_bdesc + 2 * b, B->t64, B->nsm, st));
            else
                BLAUNCH(B, launch_solve_fp32_batch(bin_nmax(b), B->d_solve, B->d_noff, B->ndom, B->d_order, B->d_blist,
                                                   B->d_bdesc + 2 * b, B->t32, B->nsm, st));
        }
        if (B->precision != SGS_PREC_FP64)
            BLAUNCH(B, launch_solve_fp64_into_fp32_batch(B->kmax, B->d_solve, B->d_noff, B->ndom, B->d_order,
                                                         B->d_fallback, B->d_fbdesc, B->t32, B->nsm, st));
        BCK(B, cudaMemcpyAsync(B->d_solve + d, &B->solve[d], sizeof(s), cudaMemcpyHostToDevice, st));
        if (weights) BCK(B, cudaMemcpyAsync(weights, wf, (size_t)n * B->kd[d] * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (sigma) BCK(B, cudaMemcpyAsync(sigma, sf, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
        BCK(B, cudaStreamSynchronize(st));
        B->info.launches += launched;
        bfree(B, wf);
        bfree(B, sf);
    }
    if (status) {
        std::vector<int8_t> s8(n);
        BCK(B, cudaMemcpy(s8.data(), B->d_status + B->noff[d], n, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; ++i) status[i] = s8[i];
    }
    return SGS_OK;
}

extern "C" int sgs_batch_set_sweep(sgs_batch* B, const sgs_sweep_config* c) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (!c) return berr(B, SGS_ERR_ARG, "null sweep configuration");
    if (c->mode != SGS_SWEEP_FLOW) return berr(B, SGS_ERR_ARG, "batches sweep in the dataflow form only");
    if (c->chunk < 0 || c->chunk > 64 || c->blocks_per_sm < 0 || c->blocks_per_sm > 32 || c->lanes_g < 0 ||
        c->lanes_g > 2 || c->lanes_w < 0 || c->lanes_w > 32 || (c->lanes_w & (c->lanes_w - 1)) || c->tight < 0 ||
        c->tight > 1)
        return berr(B, SGS_ERR_ARG, "invalid dataflow sweep parameters");
    B->sweep = *c;
    B->sweep.level_lo = B->sweep.level_hi = B->sweep.split_nodes = 0;
    if (B->sweep.chunk < 1) B->sweep.chunk = 1;
    B->sweep_graph_valid = false;
    return SGS_OK;
}

extern "C" int sgs_batch_tune_sweep(sgs_batch* B, int32_t R, sgs_sweep_config* chosen, sgs_sweep_config* tried,
                                    int32_t max_tried, int32_t* ntried) {
    if (!B) return berr(nullptr, SGS_ERR_ARG, "null batch");
    if (!B->prepared) return berr(B, SGS_ERR_STATE, "tune before prepare");
    if (R < 1) return berr(B, SGS_ERR_ARG, "invalid nreals");
    BCK(B, cudaSetDevice(B->device));
    const int Rp = (R + 3) / 4 * 4, cpn = Rp / 4;
    const size_t es = values_fp64(B) ? sizeof(double) : sizeof(float);
    int rc;
    unsigned char* V = nullptr;
    if ((rc = balloc(B, &V, (size_t)B->Ntot * Rp * es))) return rc;
    const sgs_sweep_config saved = B->sweep;
    std::vector<sgs_sweep_config> done;
    int best = -1;
    cudaStream_t st = B->stream;
    auto time_one = [&](sgs_sweep_config c) -> int {
        B->sweep = c;
        int r;
        if ((r = ensure_flags(B, Rp))) return r;
        int64_t launched = 0;
        *B->h_seed = 7;
        BCK(B, cudaMemcpyAsync(B->d_seed, B->h_seed, sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        if ((r = enqueue_sweep(B, Rp, nullptr, V, st, launched))) return r;  // warm-up
        BCK(B, cudaEventRecord(B->ev[6], st));
        if ((r = enqueue_sweep(B, Rp, nullptr, V, st, launched))) return r;
        BCK(B, cudaEventRecord(B->ev[7], st));
        BCK(B, cudaStreamSynchronize(st));
        B->info.launches += launched;
        if ((r = check_sweep_error(B))) return r;
        c.ms = elapsed_ms(B->ev[6], B->ev[7]);
        done.push_back(c);
        if (best < 0 || c.ms < done[best].ms) best = (int)done.size() - 1;
        return SGS_OK;
    };
    int p2 = 1;
    while (p2 < cpn && p2 < 32) p2 <<= 1;
    rc = SGS_OK;
    for (int W = p2; !rc && W >= std::max(1, p2 / 4); W >>= 1)
        for (int G = 1; !rc && G <= (cpn >= 2 * W ? 2 : 1); ++G)
            for (int tight = 0; !rc && tight <= 1; ++tight)
                for (int chunk : {1, 2}) {
                    if (rc) break;
                    rc = time_one({SGS_SWEEP_FLOW, chunk, 0, G, W, 0, 0, tight, 0, 0.f});
                }
    bfree(B, V);
    if (rc || best < 0) {
        B->sweep = saved;
        B->sweep_graph_valid = false;
        return rc ? rc : berr(B, SGS_ERR_CUDA, "no sweep configuration could be timed");
    }
    B->sweep = done[best];
    B->sweep_graph_valid = false;
    if (chosen) *chosen = done[best];
    const int n = (int)done.size();
    if (tried)
        for (int i = 0; i < std::min(n, (int)max_tried); ++i) tried[i] = done[i];
    if (ntried) *ntried = n;
    return SGS_OK;
}

// Statistics; after a device-resident sweep this waits for it, times it and
// reports a failed dependency wait (SGS_ERR_TIMEOUT).
extern "C" int sgs_batch_info_get(const sgs_batch* B, sgs_batch_info* info) {
    if (!B || !info) return berr(nullptr, SGS_ERR_ARG, "null argument");
    sgs_batch* M = const_cast<sgs_batch*>(B);
    if (M->sweep_pending) {
        BCK(M, cudaSetDevice(M->device));
        BCK(M, cudaEventSynchronize(M->ev[5]));
        float ms = 0.f;
        BCK(M, cudaEventElapsedTime(&ms, M->ev[4], M->ev[5]));
        M->info.ms_sweep = ms;
        M->sweep_pending = false;
        const int rc = check_sweep_error(M);
        *info = M->info;
        return rc;
    }
    *info = M->info;
    return SGS_OK;
}

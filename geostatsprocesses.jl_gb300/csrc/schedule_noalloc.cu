// schedule_noalloc.cu — sgs_schedule_noalloc: the dependency-level schedule
// of a neighbour table (levels, level-ordered node list, level offsets)
// computed without allocating any memory.
//
// Who needs this: a caller that owns all device memory itself and must not
// have a library allocate behind its back — for example a host application
// whose memory pool has already reserved the device, so a cudaMalloc inside
// the library would fail or fragment it, or a time-critical loop where an
// allocation (which can synchronize the device) is not acceptable.  Such a
// caller passes every input and output buffer; the only working memory is
// the file-scope device array below, which exists once per device that loads
// the library and lives until the process exits.
//
// Limits and rules (also stated in include/geosgs.h):
//  * the inputs are checked on the device before they are used: path must
//    be a permutation of 0..N-1, every count in [0, maxneighbors], and every
//    grid neighbour (id < N) of a node must come earlier in the path than the
//    node; anything else is rejected with SGS_ERR_ARG and nothing is read or
//    written out of bounds;
//  * at most SGS_NOALLOC_MAX_LEVELS dependency levels; a larger schedule is
//    rejected with SGS_ERR_ARG before any per-level counter is touched;
//  * the array's device address is looked up (cudaGetSymbolAddress) on every
//    call, with the caller's device and context current, so a device reset or
//    another context never leaves a stale address behind;
//  * all calls on a device share the array, and each call clears what must
//    start at zero; calls that overlap on the GPU (other streams, other host
//    threads) race on it and must be serialized by the caller.
#include <algorithm>
#include <cstdio>
#include <string>

#include "../../include/geosgs.h"
#include "common.cuh"

namespace {

constexpr int kHeader = 64;  // ticket, max level, wait error, input error, padding
constexpr int kMaxLevels = SGS_NOALLOC_MAX_LEVELS;

// [0] ticket, [1] max level, [2] wait error flag, [3] input error code; then
// per-level counts and fill cursors, kMaxLevels each
static __device__ __align__(256) int32_t g_schedule_scratch[kHeader + 2 * kMaxLevels];

// input error codes (scratch[3], zero on entry); the first code raised is
// kept
enum : int32_t {
    kInOk = 0,
    kInPathRange = 1,      // a path entry outside [0, N)
    kInPathRepeat = 2,     // a node twice in the path
    kInCount = 3,          // a count outside [0, maxneighbors]
    kInNegNeighbour = 4,   // a negative id among a node's first count entries
    kInLaterNeighbour = 5  // a grid neighbour that does not come earlier in the path
};

__device__ __forceinline__ void raise_code(int32_t* code, int32_t c) { atomicCAS(code, kInOk, c); }

// Path ranks into rank[] (the caller's `order` buffer, all -1 on entry): a
// path entry out of range or repeated raises its code.  With no code raised,
// the N entries are N distinct ids in [0, N): a permutation.
__global__ void check_path_kernel(const int32_t* __restrict__ path, int64_t N, int32_t* rank, int32_t* code) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
        const int32_t g = path[t];
        if (g < 0 || g >= N) {
            raise_code(code, kInPathRange);
            continue;
        }
        if (atomicCAS(&rank[g], -1, (int32_t)t) != -1) raise_code(code, kInPathRepeat);
    }
}

// Every node's count and first count neighbour ids, against the ranks (run
// only when the path is a permutation, so every rank is set).
__global__ void check_table_kernel(const int32_t* __restrict__ nbr, const int32_t* __restrict__ count, int64_t N,
                                   int k, const int32_t* __restrict__ rank, int32_t* code) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
        const int32_t n = count[g];
        if (n < 0 || n > k) {
            raise_code(code, kInCount);
            continue;
        }
        const int32_t rg = rank[g];
        for (int q = 0; q < n; ++q) {
            const int32_t c = nbr[g * (int64_t)k + q];
            if (c < 0) {
                raise_code(code, kInNegNeighbour);
                break;
            }
            if (c < N && rank[c] >= rg) {
                raise_code(code, kInLaterNeighbour);
                break;
            }
        }
    }
}

const char* input_error_text(int32_t code) {
    switch (code) {
        case kInPathRange: return "path holds an entry outside [0, nnodes)";
        case kInPathRepeat: return "path holds a node twice (it must be a permutation of 0..nnodes-1)";
        case kInCount: return "a count is outside [0, maxneighbors]";
        case kInNegNeighbour: return "a negative neighbour id among a node's first count entries";
        case kInLaterNeighbour: return "a grid neighbour does not come earlier in the path than its node";
        default: return "invalid input";
    }
}

// the message is read back with sgs_last_error(NULL)
int fail(int code, const std::string& msg) {
    sgs::set_thread_error(msg);
    return code;
}

// exclusive scan of count[0..n) into off[0..n] by one block
__global__ void __launch_bounds__(1024) scan_offsets_kernel(const int32_t* count, int32_t n, int32_t* off) {
    __shared__ int32_t s[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int32_t base = 0; base < n; base += 1024) {
        const int32_t i = base + threadIdx.x;
        const int32_t v = i < n ? count[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
            const int32_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) off[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += s[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) off[n] = carry;
}

#define CKN(call)                                                                             \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(SGS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" int sgs_schedule_noalloc(const int32_t* path, const int32_t* nbr, const int32_t* count, int64_t nnodes,
                                    int32_t maxneighbors, int32_t* level, int32_t* order, int32_t* offsets,
                                    int32_t offsets_capacity, int32_t* nlevels, void* stream) {
    if (!path || !nbr || !count || !level || !order || !offsets || !nlevels)
        return fail(SGS_ERR_ARG, "null argument");
    if (nnodes < 1 || nnodes > (int64_t)INT32_MAX / 2) return fail(SGS_ERR_ARG, "nnodes must be in [1, 2^30)");
    if (maxneighbors < 1 || maxneighbors > sgs::KMAX) return fail(SGS_ERR_ARG, "maxneighbors must be in [1, 64]");
    if (offsets_capacity < 2) return fail(SGS_ERR_ARG, "offsets_capacity must be at least 2");
    int dev = 0, nsm = 0;
    CKN(cudaGetDevice(&dev));
    // the array's address in the current context, looked up on every call
    int32_t* scratch = nullptr;
    {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_schedule_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SGS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        }
        scratch = static_cast<int32_t*>(p);
    }
    CKN(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = (cudaStream_t)stream;
    const int check_blocks = (int)std::min<int64_t>((nnodes + 255) / 256, (int64_t)nsm * 16);

    // inputs: path ranks into the caller's order buffer, then the table
    CKN(cudaMemsetAsync(scratch, 0, kHeader * sizeof(int32_t), st));
    CKN(cudaMemsetAsync(order, 0xff, (size_t)nnodes * sizeof(int32_t), st));
    int32_t* code = scratch + 3;
    check_path_kernel<<<check_blocks, 256, 0, st>>>(path, nnodes, order, code);
    CKN(cudaGetLastError());
    int32_t hcode = 0;
    CKN(cudaMemcpyAsync(&hcode, code, sizeof(hcode), cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    if (hcode == kInOk) {
        check_table_kernel<<<check_blocks, 256, 0, st>>>(nbr, count, nnodes, maxneighbors, order, code);
        CKN(cudaGetLastError());
        CKN(cudaMemcpyAsync(&hcode, code, sizeof(hcode), cudaMemcpyDeviceToHost, st));
        CKN(cudaStreamSynchronize(st));
    }
    if (hcode != kInOk) return fail(SGS_ERR_ARG, input_error_text(hcode));

    // levels: the ticket kernel of the plan path, its counters in the scratch
    CKN(cudaMemsetAsync(level, 0xff, (size_t)nnodes * sizeof(int32_t), st));
    sgs::LevelArgs la{};
    la.N = nnodes;
    la.k = maxneighbors;
    la.path = path;
    la.nbr = nbr;
    la.cnt = count;
    la.level = level;
    la.ticket = scratch + 0;
    la.maxlevel = scratch + 1;
    la.err = scratch + 2;
    la.wait_ns = sgs::LEVEL_WAIT_NS;
    CKN(sgs::launch_levels(la, nsm, st));
    int32_t hdr[3] = {0, 0, 0};
    CKN(cudaMemcpyAsync(hdr, scratch, sizeof(hdr), cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    if (hdr[2]) return fail(SGS_ERR_TIMEOUT, "dependency-level wait exceeded its bound");
    const int32_t nl = hdr[1] + 1;
    if (nl > kMaxLevels)
        return fail(SGS_ERR_ARG, "the schedule has " + std::to_string(nl) + " levels; sgs_schedule_noalloc supports at most " +
                                     std::to_string(kMaxLevels));
    if (nl + 1 > offsets_capacity)
        return fail(SGS_ERR_ARG, "offsets needs " + std::to_string(nl + 1) + " entries, capacity is " +
                                     std::to_string(offsets_capacity));

    // level-ordered node list: count per level, scan into offsets, fill
    int32_t* lcount = scratch + kHeader;
    int32_t* lfill = scratch + kHeader + kMaxLevels;
    CKN(cudaMemsetAsync(lcount, 0, (size_t)nl * sizeof(int32_t), st));
    CKN(cudaMemsetAsync(lfill, 0, (size_t)nl * sizeof(int32_t), st));
    CKN(sgs::launch_level_order(nnodes, level, nl, lcount, nullptr, nullptr, nullptr, st));
    scan_offsets_kernel<<<1, 1024, 0, st>>>(lcount, nl, offsets);
    CKN(cudaGetLastError());
    CKN(sgs::launch_level_order(nnodes, level, nl, lcount, offsets, lfill, order, st));
    CKN(cudaStreamSynchronize(st));
    *nlevels = nl;
    return SGS_OK;
}

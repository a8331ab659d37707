// api.cu — the C ABI of libgeosgs.so (include/geosgs.h): plan creation,
// preparation (search, levels, solve), simulation (sweep) and the parity
// read-backs.  Host-side set-up that has to agree bit for bit with the
// oracle (the search template's distances) is compiled without FMA
// contraction (-ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/geosgs.h"
#include "internal.h"

using namespace sgs;

namespace {

thread_local std::string g_create_err;
const double kSingularTau = 1e-10;  // pivot <= tau*sill -> prior (SGS_NODE_PRIOR_SINGULAR)

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct sgs_plan {
    std::string err;
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    // learned warm start: the prediction runs on a second stream, started
    // right after the search, concurrently with the dependency levels
    cudaStream_t pred_stream = nullptr;
    cudaEvent_t pred_done = nullptr;
    bool pred_pending = false;
    // problem
    GridDev grid{};
    MetricDev metric{};
    VarioDev vario{};
    double mean = 0.0;
    int k = 0, nmin = 1;
    int precision = SGS_PREC_FP32_REFINE;
    int refine_steps = 2;
    int warm_start = 0;
    int flags = 0;
    int32_t* d_loff = nullptr;    // device level offsets (nlevels + 1)
    int64_t N = 0, D = 0;
    std::vector<TmplEntry> h_tmpl;
    std::vector<double> h_tmpl_d2;
    int tmpl_ext[3] = {0, 0, 0};
    // device: geometry and inputs
    std::vector<DevBuf> bufs;
    int32_t *d_path = nullptr, *d_rank = nullptr;
    TmplEntry* d_tmpl = nullptr;
    double* d_tmpl_d2 = nullptr;
    double *d_dxyz_b = nullptr, *d_dxyz = nullptr, *d_dval = nullptr;
    float4* d_dxyz_f = nullptr;
    int32_t *d_did = nullptr, *d_bstart = nullptr;
    int nb[3] = {1, 1, 1};
    double bw[3] = {1, 1, 1};
    // device: results
    int32_t *d_nbr = nullptr, *d_cnt = nullptr, *d_ngrid = nullptr;
    int32_t *d_level = nullptr, *d_order = nullptr, *d_scratch = nullptr;
    int8_t* d_status = nullptr;
    CovLut lut{};
    double* d_lut64 = nullptr;
    float2* d_lut2 = nullptr;
    SweepTables<float> t32{};
    SweepTables<double> t64{};
    int32_t *d_fallback = nullptr;
    std::vector<int32_t> h_loff;  // level offsets (nlevels+1)
    int nlevels = 0;
    bool prepared = false;
    bool sweep_timed = false;     // ev[5]/ev[6] bracket the last sweep
    unsigned long long* d_sum_m = nullptr;
    unsigned long long* d_stats = nullptr;  // [3] search candidates (grid, data), prior nodes
    float* d_nn = nullptr;        // warm-start network parameters
    float* d_winit = nullptr;     // warm-start predictions [N][k]
    int32_t* d_done = nullptr;    // dataflow sweep: per-node epoch flags
    unsigned long long* d_flow = nullptr;  // dataflow sweep: ticket, error flag
    int32_t flow_epoch = 0;
    sgs_sweep_config sweep{SGS_SWEEP_FLOW, 1, 0, 1, 0, 0, 0, 0, 0, 0.f};
    int64_t done_cap = 0;         // flags allocated in d_done (pieces x N)
    int last_sweep_mode = SGS_SWEEP_FLOW;  // mode of the last sweep launched
    int data_only = 0;            // neighbours from the data alone (sgs_krige)
    // indicator simulation (sgs_plan_set_indicator)
    int ind_ncat = 0;
    double ind_prob[IND_MAX_CAT] = {};
    int32_t* d_ind_cat = nullptr;
    double *d_ind_wsum = nullptr, *d_ind_dsum = nullptr;
    // full simple cokriging of the indicators (sgs_plan_set_indicator_cokriging):
    // coregionalization matrices per structure, per-position systems' outputs
    bool cok = false;
    double* d_cok_coef = nullptr;
    double cok_tau = 0.0;
    int32_t *d_cok_m = nullptr, *d_cok_idx = nullptr;
    double *d_cok_w = nullptr, *d_cok_cst = nullptr;
    int cok_L = 0;                // L the cokriging tables were allocated for
    // multivariate Gaussian simulation (sgs_plan_set_multivariate): the same
    // systems with the variables' means and the data's values, plus each
    // position's factor of its conditional covariance
    bool mv = false;
    int mv_nvars = 0;
    double mv_mean[IND_MAX_CAT] = {};
    double* d_mv_dval = nullptr;  // [D][L]
    double* d_mv_fac = nullptr;   // [N][L][L]
    // FP32 refinement whose weights amplify the rounding of FP32 values: the
    // sweep keeps FP64 values, from FP64 copies of the (hi, lo) tables
    unsigned int* d_wl1 = nullptr;
    bool promote = false;
    SweepTables<double> t64p{};
    sgs_info info{};
};

// the sweep's value type and the tables it reads
static bool values_fp64(const sgs_plan* P) { return P->precision == SGS_PREC_FP64 || P->promote; }
static const SweepTables<double>& sweep64(const sgs_plan* P) { return P->promote ? P->t64p : P->t64; }

// ---------------------------------------------------------------------------
namespace {

int set_err(sgs_plan* p, int code, const std::string& msg) {
    if (p) p->err = msg;
    else g_create_err = msg;
    return code;
}

int cuda_err(sgs_plan* p, cudaError_t e, const char* where) {
    const int code = (e == cudaErrorMemoryAllocation) ? SGS_ERR_OOM : SGS_ERR_CUDA;
    return set_err(p, code, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(plan, call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_err(plan, e_, #call); \
    } while (0)

// check a kernel launch wrapper's status and count the launch
#define LAUNCH(plan, n, call)                                \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_err(plan, e_, #call); \
        (plan)->info.launches += (n);                        \
    } while (0)

// plan scratch words: [0, 16) level-phase counters, flags and solve counters
// (cleared together before the level kernels), kPredErr the prediction's
// error flag
constexpr int kPredErr = 16;
constexpr int kScratchWords = 20;

template <typename T>
int dalloc(sgs_plan* p, T** out, size_t count) {
    *out = nullptr;
    if (count == 0) count = 1;
    void* ptr = nullptr;
    cudaError_t e = pool_alloc(&ptr, count * sizeof(T), p->device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(p, SGS_ERR_OOM, std::string("allocation of ") + std::to_string(count * sizeof(T)) + " bytes failed");
    }
    p->bufs.push_back({ptr, count * sizeof(T)});
    *out = static_cast<T*>(ptr);
    return SGS_OK;
}

void dfree(sgs_plan* p, void* ptr) {
    if (!ptr) return;
    for (size_t i = 0; i < p->bufs.size(); ++i)
        if (p->bufs[i].p == ptr) {
            pool_free(ptr, p->stream);
            p->bufs.erase(p->bufs.begin() + i);
            return;
        }
}

bool is_identity(const double* R, int dim) {
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
            if (R[i + 3 * j] != (i == j ? 1.0 : 0.0)) return false;
    return true;
}

void set_metric(MetricDev& m, int dim, int kind, const double* radii, const double* rot) {
    m.kind = kind;
    for (int j = 0; j < 3; ++j) {
        m.radii[j] = radii[j];
        m.inv[j] = 1.0 / radii[j];
    }
    for (int j = 0; j < 9; ++j) {
        m.R[j] = rot[j];
        m.Rf[j] = (float)rot[j];
    }
    for (int j = 0; j < 3; ++j) m.invf[j] = (float)m.inv[j];
    m.rr = radii[0] * radii[0];
    m.bound_f = (float)((kind == METRIC_ISO ? m.rr : 1.0) * (1.0 + 1e-3));
    for (int j = 0; j < 3; ++j) m.ext[j] = 0.0;
    if (kind == METRIC_ISO) {
        for (int j = 0; j < dim; ++j) m.ext[j] = radii[0];
    } else if (kind == METRIC_ELLIPSOID) {
        for (int i = 0; i < dim; ++i) {
            double s = 0.0;
            for (int j = 0; j < dim; ++j) {
                double t = rot[i + 3 * j] * radii[j];
                s += t * t;
            }
            m.ext[i] = std::sqrt(s);
        }
    }
}

// canonical squared distance (host): same operation order as the device's
// metric_d2 and the oracle; this file is compiled with -ffp-contract=off
double host_d2(const MetricDev& m, int dim, const double* h) {
    if (m.kind != METRIC_ELLIPSOID) {
        double s = h[0] * h[0];
        s = s + h[1] * h[1];
        if (dim == 3) s = s + h[2] * h[2];
        return s;
    }
    double s = 0.0;
    for (int j = 0; j < dim; ++j) {
        double u = m.R[0 + 3 * j] * h[0];
        u = u + m.R[1 + 3 * j] * h[1];
        if (dim == 3) u = u + m.R[2 + 3 * j] * h[2];
        double q = u * m.inv[j];
        s = (j == 0) ? q * q : s + q * q;
    }
    return s;
}

bool host_inside(const MetricDev& m, double d2) {
    if (m.kind == METRIC_ISO) return d2 <= m.rr;
    if (m.kind == METRIC_ELLIPSOID) return d2 <= 1.0;
    return true;
}

template <typename T>
int upload(sgs_plan* p, T** d, const T* h, size_t count) {
    int rc = dalloc(p, d, count);
    if (rc) return rc;
    if (count) CK(p, cudaMemcpyAsync(*d, h, count * sizeof(T), cudaMemcpyHostToDevice, p->stream));
    p->info.h2d_bytes += (int64_t)(count * sizeof(T));
    return SGS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// device memory pool (one per device, created on first use)
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};
cudaStream_t g_alloc_stream[kMaxDevices] = {};

cudaError_t device_pool(int device, cudaMemPool_t* pool, cudaStream_t* as) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pool[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t mp = nullptr;
        cudaError_t e = cudaMemPoolCreate(&mp, &props);
        if (e != cudaSuccess) return e;
        // keep freed memory for the next plan (a plan's buffers are GBs, and
        // mapping them anew each time costs milliseconds)
        uint64_t keep = UINT64_MAX;
        e = cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
        // the allocation stream belongs to the pool's device
        int cur = 0;
        cudaStream_t st = nullptr;
        if (e == cudaSuccess) e = cudaGetDevice(&cur);
        if (e == cudaSuccess && cur != device) e = cudaSetDevice(device);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (cur != device) cudaSetDevice(cur);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(mp);
            return e;
        }
        g_pool[device] = mp;
        g_alloc_stream[device] = st;
    }
    *pool = g_pool[device];
    *as = g_alloc_stream[device];
    return cudaSuccess;
}
}  // namespace

// Allocations run on a stream of their own that never carries kernels, and
// are waited for, so the memory is usable on any stream on return.  One
// retry after returning the pool's idle memory to the device.
cudaError_t sgs::pool_alloc(void** ptr, size_t bytes, int device) {
    *ptr = nullptr;
    cudaMemPool_t mp;
    cudaStream_t as;
    cudaError_t e = device_pool(device, &mp, &as);
    if (e != cudaSuccess) return e;
    e = cudaMallocFromPoolAsync(ptr, bytes, mp, as);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        cudaStreamSynchronize(as);
        cudaMemPoolTrimTo(mp, 0);
        e = cudaMallocFromPoolAsync(ptr, bytes, mp, as);
    }
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return e;
    }
    e = cudaStreamSynchronize(as);
    if (e != cudaSuccess) *ptr = nullptr;
    return e;
}

cudaError_t sgs::pool_free(void* ptr, cudaStream_t stream) {
    return ptr ? cudaFreeAsync(ptr, stream) : cudaSuccess;
}

extern "C" int sgs_trim_memory(int32_t device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return SGS_ERR_CUDA;
    }
    if (device >= n || device >= kMaxDevices) return SGS_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    for (int d = device < 0 ? 0 : device; d < (device < 0 ? std::min(n, kMaxDevices) : device + 1); ++d) {
        if (!g_pool[d]) continue;
        if (cudaSetDevice(d) != cudaSuccess || cudaStreamSynchronize(g_alloc_stream[d]) != cudaSuccess ||
            cudaMemPoolTrimTo(g_pool[d], 0) != cudaSuccess) {
            cudaGetLastError();
            return SGS_ERR_CUDA;
        }
    }
    return SGS_OK;
}

void sgs::set_thread_error(const char* msg) { g_create_err = msg; }

extern "C" const char* sgs_version(void) { return "geosgs 0.1.0 (sm_103a)"; }

// Diagnostic (exported, not part of the C ABI in include/geosgs.h): runs the
// dataflow sweep's bounded wait on a flag that nothing sets, with a limit of
// wait_ns.  *timed_out = 1 when the wait gave up and said so; *elapsed_ns =
// the launch's duration.  Returns 0, or a negative SGS_ERR_* code when the
// launch itself failed.
extern "C" int sgs_selftest_bounded_wait(int64_t wait_ns, int32_t* timed_out, int64_t* elapsed_ns) {
    if (!timed_out || !elapsed_ns || wait_ns <= 0) return SGS_ERR_ARG;
    *timed_out = 0;
    *elapsed_ns = 0;
    int32_t* d = nullptr;  // [0] the flag, [1] the error word, [2] the neighbour index (0)
    if (cudaMalloc(&d, 3 * sizeof(int32_t)) != cudaSuccess) {
        cudaGetLastError();
        return SGS_ERR_CUDA;
    }
    int rc = SGS_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    FlowArgs f{};
    f.done = d;
    f.err = d + 1;
    f.epoch = 1;
    f.wait_ns = (uint64_t)wait_ns;
    int32_t herr = 0;
    float ms = 0.f;
    if (cudaMemset(d, 0, 3 * sizeof(int32_t)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess || cudaEventRecord(e0) != cudaSuccess ||
        launch_flow_wait_selftest(d + 2, f, 0) != cudaSuccess || cudaEventRecord(e1) != cudaSuccess ||
        cudaEventSynchronize(e1) != cudaSuccess ||
        cudaMemcpy(&herr, d + 1, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        cudaGetLastError();
        rc = SGS_ERR_CUDA;
    }
    *timed_out = herr;
    *elapsed_ns = (int64_t)(ms * 1e6);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    return rc;
}

// Diagnostic (exported, not part of the C ABI in include/geosgs.h): runs the
// dependency-level kernel on a two-node table in which each node is the
// other's neighbour, so neither level can ever be known, with a wait limit
// of wait_ns.  *timed_out = 1 when the kernel gave up and said so;
// *elapsed_ns = the launch's duration.  Returns 0, or a negative SGS_ERR_*
// code when the launch itself failed.
extern "C" int sgs_selftest_levels_wait(int64_t wait_ns, int32_t* timed_out, int64_t* elapsed_ns) {
    if (!timed_out || !elapsed_ns || wait_ns <= 0) return SGS_ERR_ARG;
    *timed_out = 0;
    *elapsed_ns = 0;
    // [0,2) path, [2,4) neighbours, [4,6) counts, [6,8) levels, [8,12) ticket,
    // max level, error flag, spare
    const int32_t init[12] = {0, 1, 1, 0, 1, 1, -1, -1, 0, 0, 0, 0};
    int32_t* d = nullptr;
    if (cudaMalloc(&d, sizeof(init)) != cudaSuccess) {
        cudaGetLastError();
        return SGS_ERR_CUDA;
    }
    LevelArgs la{};
    la.N = 2;
    la.k = 1;
    la.path = d;
    la.nbr = d + 2;
    la.cnt = d + 4;
    la.level = d + 6;
    la.ticket = d + 8;
    la.maxlevel = d + 9;
    la.err = d + 10;
    la.wait_ns = (uint64_t)wait_ns;
    int rc = SGS_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int32_t herr = 0;
    float ms = 0.f;
    if (cudaMemcpy(d, init, sizeof(init), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
        cudaEventRecord(e0) != cudaSuccess || launch_levels(la, 1, 0) != cudaSuccess ||
        cudaEventRecord(e1) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaMemcpy(&herr, d + 10, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        cudaGetLastError();
        rc = SGS_ERR_CUDA;
    }
    *timed_out = herr;
    *elapsed_ns = (int64_t)(ms * 1e6);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    return rc;
}

extern "C" const char* sgs_last_error(const sgs_plan* plan) {
    return plan ? plan->err.c_str() : g_create_err.c_str();
}

extern "C" void sgs_plan_destroy(sgs_plan* p) {
    if (!p) return;
    cudaSetDevice(p->device);
    // the plan's buffers may still be read by work the caller queued on its
    // own streams (the device-pointer entry points): wait for the device, as
    // a synchronous free would
    cudaDeviceSynchronize();
    for (auto& b : p->bufs) pool_free(b.p, p->stream);
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (auto& e : p->ev)
        if (e) cudaEventDestroy(e);
    if (p->pred_done) cudaEventDestroy(p->pred_done);
    if (p->pred_stream) cudaStreamDestroy(p->pred_stream);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

// Host-side set-up of one problem: validation (argument errors as the
// reference's ArgumentError / @assert), the neighbourhood metric, the path
// and its ranks, the sorted offset template and the data buckets.  Shared by
// plans and batches of domains.
int sgs::host_domain(const sgs_problem* pr, HostDomain& H, std::string& err) {
#define HERR(msg)              \
    do {                       \
        err = (msg);           \
        return SGS_ERR_ARG;    \
    } while (0)
    const int dim = pr->dim;
    if (dim != 2 && dim != 3) HERR("dim must be 2 or 3");
    GridDev& G = H.grid;
    G.dim = dim;
    G.N = 1;
    for (int j = 0; j < 3; ++j) {
        G.n[j] = j < dim ? pr->dims[j] : 1;
        G.origin[j] = j < dim ? pr->origin[j] : 0.0;
        G.spacing[j] = j < dim ? pr->spacing[j] : 1.0;
        if (G.n[j] < 1) HERR("grid dims must be >= 1");
        if (!(G.spacing[j] > 0.0) || !std::isfinite(G.spacing[j]) || !std::isfinite(G.origin[j]))
            HERR("spacing must be finite and > 0");
        G.N *= G.n[j];
    }
    if (G.N > (int64_t)INT32_MAX / 2) HERR("grid too large (N must be < 2^30)");
    H.N = G.N;
    H.D = pr->ndata;
    if (H.D < 0 || (H.D > 0 && (!pr->data_coords || !pr->data_values))) HERR("invalid data arrays");
    if (H.N + H.D > (int64_t)INT32_MAX) HERR("too many points");
    for (int64_t i = 0; i < H.D * dim; ++i)
        if (!std::isfinite(pr->data_coords[i])) HERR("data coordinates must be finite");
    for (int64_t i = 0; i < H.D; ++i)
        if (!std::isfinite(pr->data_values[i])) HERR("data values must be finite");
    const sgs_variogram& v = pr->variogram;
    if (pr->nstructures < 0 || pr->nstructures >= SGS_MAX_STRUCTURES || (pr->nstructures > 0 && !pr->structures))
        HERR("nstructures must be in [0, SGS_MAX_STRUCTURES) with a structures array");
    // the model: `variogram` plus the nested structures, summed
    H.vario.ns = 1 + pr->nstructures;
    H.vario.sill = 0.0;
    H.vario.nugget = 0.0;
    double rmax = 0.0;  // range(f): the largest range of any structure
    for (int i = 0; i < H.vario.ns; ++i) {
        const sgs_variogram& u = i == 0 ? v : pr->structures[i - 1];
        if (u.type < SGS_SPHERICAL || u.type > SGS_GAUSSIAN) HERR("unknown variogram type");
        if (!(u.sill > 0.0) || !(u.nugget >= 0.0) || u.nugget > u.sill || !std::isfinite(u.sill))
            HERR("invalid sill/nugget");
        for (int j = 0; j < dim; ++j) {
            if (!(u.ranges[j] > 0.0) || !std::isfinite(u.ranges[j])) HERR("ranges must be finite and > 0");
            rmax = std::max(rmax, u.ranges[j]);
        }
        VarioStructDev& d = H.vario.st[i];
        d.type = u.type;
        d.sill = u.sill;
        d.nugget = u.nugget;
        for (int j = 0; j < 3; ++j) d.inv_range[j] = j < dim ? 1.0 / u.ranges[j] : 1.0;
        for (int j = 0; j < 9; ++j) d.R[j] = u.rotation[j];
        H.vario.sill += u.sill;
        H.vario.nugget += u.nugget;
    }
    H.vario.type = H.vario.st[0].type;
    for (int j = 0; j < 3; ++j) H.vario.inv_range[j] = H.vario.st[0].inv_range[j];
    for (int j = 0; j < 9; ++j) H.vario.R[j] = H.vario.st[0].R[j];
    if (!std::isfinite(pr->mean)) HERR("mean must be finite");
    H.mean = pr->mean;

    // seqsim.jl:202-208
    int64_t nmax = pr->maxneighbors, nmin = pr->minneighbors;
    if (nmax > H.N || nmax < 1) nmax = H.N;
    if (nmin > nmax || nmin < 1) nmin = 1;
    if (nmax > KMAX) HERR("maxneighbors above 64 is not supported on the GPU");
    H.k = (int)nmax;
    H.nmin = (int)nmin;
    if (pr->precision != SGS_PREC_FP64 && pr->precision != SGS_PREC_FP32_REFINE) HERR("unknown precision");
    if (pr->refine_steps < 0 || pr->refine_steps > 4) HERR("refine_steps must be in 0..4");

    // neighbourhood: seqsim.jl:171-177,221-227
    static const double I9[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (pr->search == SGS_SEARCH_RANGE) {
        double r[3] = {rmax, rmax, rmax};
        set_metric(H.metric, dim, METRIC_ISO, r, I9);
    } else if (pr->search == SGS_SEARCH_BALL) {
        for (int j = 0; j < dim; ++j)
            if (!(pr->ball.radii[j] > 0.0) || !std::isfinite(pr->ball.radii[j]))
                HERR("ball radii must be finite and > 0");
        bool iso = is_identity(pr->ball.rotation, dim);
        for (int j = 1; j < dim; ++j) iso = iso && pr->ball.radii[j] == pr->ball.radii[0];
        set_metric(H.metric, dim, iso ? METRIC_ISO : METRIC_ELLIPSOID, pr->ball.radii, pr->ball.rotation);
    } else if (pr->search == SGS_SEARCH_NEAREST) {
        double r[3] = {1, 1, 1};
        set_metric(H.metric, dim, METRIC_NEAREST, r, I9);
    } else {
        HERR("unknown search kind");
    }

    // the path is checked on the device, where its ranks are built
    // (launch_path_ranks, launch_batch_path_ranks)

    // template: cell offsets inside the neighbourhood in canonical order
    int64_t e[3] = {0, 0, 0};
    int64_t cells = 1;
    for (int j = 0; j < dim; ++j) {
        if (H.metric.kind == METRIC_NEAREST) e[j] = G.n[j] - 1;
        else e[j] = std::min<int64_t>(G.n[j] - 1, (int64_t)std::floor(H.metric.ext[j] / G.spacing[j]) + 1);
        cells *= 2 * e[j] + 1;
    }
    if (cells > (int64_t)1 << 28) HERR("search neighbourhood spans too many cells");
    struct Ent { double d2; int64_t lin; TmplEntry e; };
    std::vector<Ent> ents;
    for (int64_t c = -e[2]; c <= e[2]; ++c)
        for (int64_t b = -e[1]; b <= e[1]; ++b)
            for (int64_t a = -e[0]; a <= e[0]; ++a) {
                if (a == 0 && b == 0 && c == 0) continue;
                double h[3] = {(double)a * G.spacing[0], (double)b * G.spacing[1], dim == 3 ? (double)c * G.spacing[2] : 0.0};
                double d = host_d2(H.metric, dim, h);
                if (!host_inside(H.metric, d)) continue;
                int64_t lin = a + (int64_t)G.n[0] * (b + (int64_t)G.n[1] * c);
                ents.push_back({d, lin, TmplEntry{(int)a, (int)b, (int)c, (int)lin}});
            }
    std::sort(ents.begin(), ents.end(), [](const Ent& x, const Ent& y) {
        return x.d2 < y.d2 || (x.d2 == y.d2 && x.lin < y.lin);
    });
    H.tmpl.resize(ents.size());
    H.tmpl_d2.resize(ents.size());
    for (size_t i = 0; i < ents.size(); ++i) {
        H.tmpl[i] = ents[i].e;
        H.tmpl_d2[i] = ents[i].d2;
        H.tmpl_ext[0] = std::max(H.tmpl_ext[0], std::abs(ents[i].e.dx));
        H.tmpl_ext[1] = std::max(H.tmpl_ext[1], std::abs(ents[i].e.dy));
        H.tmpl_ext[2] = std::max(H.tmpl_ext[2], std::abs(ents[i].e.dz));
    }

    // data: id order (solve) and bucket order (search)
    H.xyz.assign((size_t)H.D * 3, 0.0);
    H.val.resize(H.D);
    for (int64_t i = 0; i < H.D; ++i) {
        for (int j = 0; j < dim; ++j) H.xyz[i * 3 + j] = pr->data_coords[i * dim + j];
        H.val[i] = pr->data_values[i];
    }
    const int B = 8;
    int64_t nbk = 1;
    for (int j = 0; j < 3; ++j) {
        H.nb[j] = (G.n[j] + B - 1) / B;
        H.bw[j] = G.spacing[j] * (double)B;
        nbk *= H.nb[j];
    }
    std::vector<int64_t> bid(H.D);
    H.bstart.assign(nbk + 1, 0);
    for (int64_t i = 0; i < H.D; ++i) {
        int64_t bc[3] = {0, 0, 0};
        for (int j = 0; j < dim; ++j) {
            double f = std::floor((H.xyz[i * 3 + j] - G.origin[j]) / H.bw[j]);
            f = std::max(0.0, std::min(f, (double)(H.nb[j] - 1)));
            bc[j] = (int64_t)f;
        }
        bid[i] = bc[0] + H.nb[0] * (bc[1] + H.nb[1] * bc[2]);
        H.bstart[bid[i] + 1]++;
    }
    for (int64_t b = 0; b < nbk; ++b) H.bstart[b + 1] += H.bstart[b];
    H.xyz_b.resize((size_t)H.D * 3);
    H.did.resize(H.D);
    {
        std::vector<int32_t> cur(H.bstart.begin(), H.bstart.end() - 1);
        for (int64_t i = 0; i < H.D; ++i) {
            const int32_t q = cur[bid[i]]++;
            H.did[q] = (int32_t)i;
            for (int j = 0; j < 3; ++j) H.xyz_b[(size_t)q * 3 + j] = H.xyz[i * 3 + j];
        }
    }
    // FP32 copies relative to the grid origin for the search's screen, and a
    // bound that covers their rounding: lags are off by at most dh per axis
    {
        H.xf.resize(H.D);
        double amax = 0.0;
        for (int j = 0; j < dim; ++j) amax = std::max(amax, (double)G.n[j] * G.spacing[j]);
        for (int64_t i = 0; i < H.D; ++i) {
            double r[3] = {0, 0, 0};
            for (int j = 0; j < dim; ++j) {
                r[j] = H.xyz_b[(size_t)i * 3 + j] - G.origin[j];
                amax = std::max(amax, std::fabs(r[j]));
            }
            H.xf[i] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.0f);
        }
        const double dh = 4.0 * amax * std::ldexp(1.0, -24) + 1e-30;
        MetricDev& m = H.metric;
        double slack = 0.0;
        if (m.kind == METRIC_ISO) {
            const double r = std::sqrt(m.rr);
            slack = 2.0 * r * dh * std::sqrt((double)dim) + dim * dh * dh;
        } else if (m.kind == METRIC_ELLIPSOID) {
            for (int j = 0; j < dim; ++j) {
                double dq = 0.0;
                for (int i = 0; i < dim; ++i) dq += std::fabs(m.R[i + 3 * j]);
                dq *= dh * m.inv[j];
                slack += 2.02 * dq + dq * dq;
            }
        }
        m.bound_f = (float)((m.kind == METRIC_ISO ? m.rr : 1.0) * (1.0 + 1e-3) + slack);
        if (m.kind == METRIC_NEAREST) m.bound_f = INFINITY;
        m.slack_f = (float)slack;
        m.dh_f = (float)(dh * (1.0 + 1e-3));
    }
    return SGS_OK;
#undef HERR
}

// Search arguments of a domain whose device arrays are set by the caller.
void sgs::search_args_of(const HostDomain& H, SearchArgs& sa) {
    sa.grid = H.grid;
    sa.metric = H.metric;
    sa.k = H.k;
    sa.T = (int)H.tmpl.size();
    sa.D = H.D;
    for (int j = 0; j < 3; ++j) {
        sa.nb[j] = H.nb[j];
        sa.bw[j] = H.bw[j];
        sa.inv_bw_f[j] = (float)(1.0 / H.bw[j]);
        sa.ext_f[j] = (float)H.metric.ext[j];
        sa.spacing_f[j] = (float)H.grid.spacing[j];
    }
}

static int plan_init(sgs_plan* P, const sgs_problem* pr) {
    HostDomain H;
    {
        std::string err;
        const int rc = host_domain(pr, H, err);  // path ranks on the device, below
        if (rc != SGS_OK) return set_err(P, rc, err);
    }
    P->grid = H.grid;
    P->metric = H.metric;
    P->vario = H.vario;
    P->mean = H.mean;
    P->N = H.N;
    P->D = H.D;
    P->k = H.k;
    P->nmin = H.nmin;
    P->precision = pr->precision;
    P->refine_steps = pr->refine_steps;
    P->warm_start = pr->warm_start;
    if (pr->flags & ~(SGS_FLAG_ONE_LAUNCH_SWEEP | SGS_FLAG_LEVEL_SWEEP | SGS_FLAG_NN_FP32 | SGS_FLAG_OUTPUT_STAGED))
        return set_err(P, SGS_ERR_ARG, "unknown flags");
    if ((pr->flags & SGS_FLAG_ONE_LAUNCH_SWEEP) && (pr->flags & SGS_FLAG_LEVEL_SWEEP))
        return set_err(P, SGS_ERR_ARG, "SGS_FLAG_ONE_LAUNCH_SWEEP and SGS_FLAG_LEVEL_SWEEP exclude each other");
    P->flags = pr->flags;
    P->sweep.mode = (pr->flags & SGS_FLAG_ONE_LAUNCH_SWEEP) ? SGS_SWEEP_COOPERATIVE
                    : (pr->flags & SGS_FLAG_LEVEL_SWEEP)   ? SGS_SWEEP_LEVELS
                                                           : SGS_SWEEP_FLOW;
    P->h_tmpl = std::move(H.tmpl);
    P->h_tmpl_d2 = std::move(H.tmpl_d2);
    for (int j = 0; j < 3; ++j) {
        P->tmpl_ext[j] = H.tmpl_ext[j];
        P->nb[j] = H.nb[j];
        P->bw[j] = H.bw[j];
    }

    // device
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(P, SGS_ERR_NODEVICE, "no CUDA device");
    }
    if (pr->device < 0 || pr->device >= ndev) return set_err(P, SGS_ERR_ARG, "invalid device ordinal");
    P->device = pr->device;
    CK(P, cudaSetDevice(P->device));
    CK(P, cudaDeviceGetAttribute(&P->nsm, cudaDevAttrMultiProcessorCount, P->device));
    CK(P, cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    for (auto& ev : P->ev) CK(P, cudaEventCreate(&ev));

    int rc;
    // the path as given (or the linear one), its ranks built and checked on
    // the device: rank[path[t]] = t, and the path a permutation of the nodes
    int32_t* d_perr = nullptr;
    if ((rc = dalloc(P, &P->d_rank, P->N)) || (rc = dalloc(P, &d_perr, 1))) return rc;
    if (pr->path) {
        if ((rc = upload(P, &P->d_path, pr->path, P->N))) return rc;
    } else if ((rc = dalloc(P, &P->d_path, P->N))) {
        return rc;
    }
    CK(P, cudaMemsetAsync(P->d_rank, 0xff, (size_t)P->N * sizeof(int32_t), P->stream));
    CK(P, cudaMemsetAsync(d_perr, 0, sizeof(int32_t), P->stream));
    LAUNCH(P, 2, launch_path_ranks(pr->path ? P->d_path : nullptr, P->N, P->d_path, P->d_rank, d_perr, P->nsm,
                                   P->stream));
    if ((rc = upload(P, &P->d_tmpl, P->h_tmpl.data(), P->h_tmpl.size()))) return rc;
    if ((rc = upload(P, &P->d_tmpl_d2, P->h_tmpl_d2.data(), P->h_tmpl_d2.size()))) return rc;
    if ((rc = upload(P, &P->d_dxyz, H.xyz.data(), H.xyz.size()))) return rc;
    if ((rc = upload(P, &P->d_dval, H.val.data(), H.val.size()))) return rc;
    if ((rc = upload(P, &P->d_dxyz_b, H.xyz_b.data(), H.xyz_b.size()))) return rc;
    if ((rc = upload(P, &P->d_did, H.did.data(), H.did.size()))) return rc;
    if ((rc = upload(P, &P->d_bstart, H.bstart.data(), H.bstart.size()))) return rc;
    if ((rc = upload(P, &P->d_dxyz_f, H.xf.data(), H.xf.size()))) return rc;
    int32_t perr = 0;
    CK(P, cudaMemcpyAsync(&perr, d_perr, sizeof(int32_t), cudaMemcpyDeviceToHost, P->stream));
    CK(P, cudaStreamSynchronize(P->stream));
    dfree(P, d_perr);
    if (perr) return set_err(P, SGS_ERR_ARG, "path is not a permutation of the grid nodes");

    P->info.nnodes = P->N;
    P->info.ndata = P->D;
    P->info.maxneighbors = P->k;
    P->info.minneighbors = P->nmin;
    P->info.template_size = (int32_t)P->h_tmpl.size();
    return SGS_OK;
}

extern "C" int sgs_plan_create(const sgs_problem* problem, sgs_plan** plan) {
    if (!problem || !plan) return set_err(nullptr, SGS_ERR_ARG, "null argument");
    *plan = nullptr;
    sgs_plan* P = new sgs_plan();
    const int rc = plan_init(P, problem);
    if (rc != SGS_OK) {
        g_create_err = P->err.empty() ? g_create_err : P->err;
        sgs_plan_destroy(P);
        return rc;
    }
    *plan = P;
    return SGS_OK;
}

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// Warm-start predictions [N][k] of the plan's network for every system: BF16
// on the tensor cores (tcgen05) or FP32 on the CUDA cores.  The tensor-core
// kernel's error flag is scratch[kPredErr] (read by the caller after a sync),
// outside the words the level phase clears, since the prediction can run
// beside it.
static int run_predict(sgs_plan* P, float* out, bool tensor_cores, cudaStream_t st) {
    if (tensor_cores) {
        CK(P, cudaMemsetAsync(P->d_scratch + kPredErr, 0, sizeof(int32_t), st));
        LAUNCH(P, 1, launch_nn_predict_tc(P->grid, P->vario, P->d_nbr, P->d_cnt, P->k, P->d_dxyz, P->d_nn, out,
                                          P->d_scratch + kPredErr, P->nsm, st));
    } else {
        LAUNCH(P, 1, launch_nn_predict_plan(P->grid, P->vario, P->d_nbr, P->d_cnt, P->k, P->d_dxyz, P->d_nn, out,
                                            st));
    }
    return SGS_OK;
}

static int run_solve(sgs_plan* P, double* w_full, double* sigma_full) {
    SolveArgs s{};
    s.grid = P->grid;
    s.vario = P->vario;
    s.lut = P->lut;
    s.k = P->k;
    s.nmin = P->nmin;
    s.mu = P->mean;
    s.tau = kSingularTau * P->vario.sill;
    s.inv_sill = 1.0 / P->vario.sill;
    s.refine_steps = P->refine_steps;
    s.P = P->N;
    s.order = P->d_order;
    s.nbr = P->d_nbr;
    s.cnt = P->d_cnt;
    s.N = P->N;
    s.data_xyz = P->d_dxyz;
    s.data_val = P->d_dval;
    s.status = P->d_status;
    s.w_full = w_full;
    s.sigma_full = sigma_full;
    s.sum_m = P->d_sum_m;
    s.wl1_max = P->d_wl1;
    CK(P, cudaMemsetAsync(P->d_wl1, 0, sizeof(unsigned int), P->stream));
    if (P->ind_ncat) {
        s.ind_cat = P->d_ind_cat;
        s.ncat = P->ind_ncat;
        s.ind_wsum = P->d_ind_wsum;
        s.ind_dsum = P->d_ind_dsum;
    }
    CK(P, cudaMemsetAsync(P->d_sum_m, 0, sizeof(unsigned long long), P->stream));
    if (P->precision == SGS_PREC_FP64) {
        LAUNCH(P, 1, launch_solve_fp64(s, P->t64, P->stream));
        P->info.n_fp64_fallback = 0;
        return SGS_OK;
    }
    int32_t* nfb = P->d_scratch;  // scratch[0]
    CK(P, cudaMemsetAsync(nfb, 0, sizeof(int32_t), P->stream));
    s.fallback = P->d_fallback;
    s.nfallback = nfb;
    unsigned long long* nwarm = reinterpret_cast<unsigned long long*>(P->d_scratch + 8);  // scratch[8..9]
    if (P->warm_start && P->d_nn) {
        // learned warm start: predictions for every node (launched after the
        // search by sgs_plan_prepare, or here), then the solve refines from them
        int rc;
        if (P->pred_pending) {
            CK(P, cudaStreamWaitEvent(P->stream, P->pred_done, 0));
            P->pred_pending = false;
        } else {
            if (!P->d_winit && (rc = dalloc(P, &P->d_winit, (size_t)P->N * P->k))) return rc;
            if ((rc = run_predict(P, P->d_winit, !(P->flags & SGS_FLAG_NN_FP32), P->stream))) return rc;
        }
        CK(P, cudaMemsetAsync(nwarm, 0, sizeof(unsigned long long), P->stream));
        s.w_init = P->d_winit;
        s.n_warm = nwarm;
        // a prediction is far less accurate than the FP32 inverse's own
        // solution, so warm-started systems take one more refinement step
        s.refine_steps = std::min(P->refine_steps + 1, 4);
    }
    LAUNCH(P, 1, launch_solve_fp32(s, P->t32, P->stream));
    // queued systems: re-solve in FP64 (the canonical decision and accuracy)
    s.list = P->d_fallback;
    s.w_init = nullptr;
    LAUNCH(P, 1, launch_solve_fp64_into_fp32(s, P->t32, P->stream));
    int32_t h = 0;
    unsigned long long hw = 0;
    CK(P, cudaMemcpyAsync(&h, nfb, sizeof(int32_t), cudaMemcpyDeviceToHost, P->stream));
    if (s.n_warm) CK(P, cudaMemcpyAsync(&hw, nwarm, sizeof(hw), cudaMemcpyDeviceToHost, P->stream));
    int32_t htc = 0;
    if (s.n_warm) CK(P, cudaMemcpyAsync(&htc, P->d_scratch + kPredErr, sizeof(int32_t), cudaMemcpyDeviceToHost, P->stream));
    CK(P, cudaStreamSynchronize(P->stream));
    P->info.d2h_bytes += sizeof(int32_t) + (s.n_warm ? sizeof(hw) + sizeof(htc) : 0);
    if (htc) return set_err(P, SGS_ERR_TIMEOUT, "tensor-core inference: an MMA completion wait exceeded its bound");
    P->info.n_fp64_fallback = h;
    P->info.n_warm_accepted = (int64_t)hw;
    return SGS_OK;
}

static CokArgs cok_args(const sgs_plan* P) {
    CokArgs c{};
    c.ncat = P->mv ? P->mv_nvars : P->ind_ncat;
    for (int l = 0; l < IND_MAX_CAT; ++l) c.prob[l] = P->mv ? P->mv_mean[l] : P->ind_prob[l];
    c.coef = P->d_cok_coef;
    c.data_cat = P->d_ind_cat;
    c.data_val = P->d_mv_dval;
    c.tau = P->cok_tau;
    c.m = P->d_cok_m;
    c.idx = P->d_cok_idx;
    c.w = P->d_cok_w;
    c.cst = P->d_cok_cst;
    c.fac = P->d_mv_fac;
    return c;
}

static void free_cok_tables(sgs_plan* P) {
    dfree(P, P->d_cok_m);
    dfree(P, P->d_cok_idx);
    dfree(P, P->d_cok_w);
    dfree(P, P->d_cok_cst);
    dfree(P, P->d_mv_fac);
    P->d_cok_m = P->d_cok_idx = nullptr;
    P->d_cok_w = P->d_cok_cst = P->d_mv_fac = nullptr;
    P->cok_L = 0;
}

extern "C" int sgs_plan_prepare(sgs_plan* P) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    CK(P, cudaSetDevice(P->device));
    const int64_t N = P->N;
    const int k = P->k;
    int rc;
    if (!P->d_nbr) {
        if ((rc = dalloc(P, &P->d_nbr, (size_t)N * k))) return rc;
        if ((rc = dalloc(P, &P->d_cnt, N))) return rc;
        if ((rc = dalloc(P, &P->d_ngrid, N))) return rc;
        if ((rc = dalloc(P, &P->d_level, N))) return rc;
        if ((rc = dalloc(P, &P->d_order, N))) return rc;
        if ((rc = dalloc(P, &P->d_status, N))) return rc;
        if ((rc = dalloc(P, &P->d_scratch, kScratchWords))) return rc;
        if ((rc = dalloc(P, &P->d_sum_m, 1))) return rc;
        if ((rc = dalloc(P, &P->d_stats, 3))) return rc;
        if ((rc = dalloc(P, &P->d_wl1, 1))) return rc;
    }
    cudaStream_t st = P->stream;

    // ---- (a) neighbour search ----
    SearchArgs sa{};
    sa.grid = P->grid;
    sa.metric = P->metric;
    sa.k = k;
    sa.T = (int)P->h_tmpl.size();
    sa.tmpl = P->d_tmpl;
    sa.tmpl_d2 = P->d_tmpl_d2;
    sa.path = P->d_path;
    sa.rank = P->d_rank;
    sa.D = P->D;
    sa.dxyz = P->d_dxyz_b;
    sa.dxyz_f = P->d_dxyz_f;
    sa.did = P->d_did;
    sa.bstart = P->d_bstart;
    for (int j = 0; j < 3; ++j) {
        sa.nb[j] = P->nb[j];
        sa.bw[j] = P->bw[j];
        sa.inv_bw_f[j] = (float)(1.0 / P->bw[j]);
        sa.ext_f[j] = (float)P->metric.ext[j];
        sa.spacing_f[j] = (float)P->grid.spacing[j];
    }
    sa.nbr = P->d_nbr;
    sa.cnt = P->d_cnt;
    sa.ngrid = P->d_ngrid;
    sa.data_only = P->data_only;
    sa.scanned = P->d_stats;
    CK(P, cudaMemsetAsync(P->d_stats, 0, 3 * sizeof(unsigned long long), st));
    CK(P, cudaEventRecord(P->ev[0], st));
    LAUNCH(P, 1, launch_search(sa, st));
    CK(P, cudaEventRecord(P->ev[1], st));

    // ---- learned warm start: predictions need only the neighbour rows, so
    // they run beside the dependency levels on a second stream ----
    if (P->warm_start && P->d_nn && P->precision != SGS_PREC_FP64) {
        if (!P->pred_stream) CK(P, cudaStreamCreateWithFlags(&P->pred_stream, cudaStreamNonBlocking));
        if (!P->pred_done) CK(P, cudaEventCreateWithFlags(&P->pred_done, cudaEventDisableTiming));
        if (!P->d_winit && (rc = dalloc(P, &P->d_winit, (size_t)N * k))) return rc;
        CK(P, cudaStreamWaitEvent(P->pred_stream, P->ev[1], 0));
        if ((rc = run_predict(P, P->d_winit, !(P->flags & SGS_FLAG_NN_FP32), P->pred_stream))) return rc;
        CK(P, cudaEventRecord(P->pred_done, P->pred_stream));
        P->pred_pending = true;
    }

    // ---- dependency levels and level order ----
    CK(P, cudaMemsetAsync(P->d_level, 0xff, N * sizeof(int32_t), st));
    CK(P, cudaMemsetAsync(P->d_scratch, 0, 16 * sizeof(int32_t), st));
    LevelArgs la{};
    la.N = N;
    la.k = k;
    la.path = P->d_path;
    la.nbr = P->d_nbr;
    la.cnt = P->d_cnt;
    la.level = P->d_level;
    la.ticket = P->d_scratch + 1;
    la.maxlevel = P->d_scratch + 2;
    la.err = P->d_scratch + 3;
    la.wait_ns = LEVEL_WAIT_NS;
    LAUNCH(P, 1, launch_levels(la, P->nsm, st));
    int32_t hs[4] = {0, 0, 0, 0};
    CK(P, cudaMemcpyAsync(hs, P->d_scratch, sizeof(hs), cudaMemcpyDeviceToHost, st));
    CK(P, cudaStreamSynchronize(st));
    P->info.d2h_bytes += sizeof(hs);
    if (hs[3]) return set_err(P, SGS_ERR_TIMEOUT, "dependency-level wait exceeded its bound");
    P->nlevels = hs[2] + 1;
    int32_t *d_lcount = nullptr, *d_lfill = nullptr;
    if ((rc = dalloc(P, &d_lcount, P->nlevels))) return rc;
    if ((rc = dalloc(P, &d_lfill, P->nlevels))) return rc;
    dfree(P, P->d_loff);  // level offsets stay for the one-launch sweep
    if ((rc = dalloc(P, &P->d_loff, P->nlevels + 1))) return rc;
    int32_t* d_loff = P->d_loff;
    CK(P, cudaMemsetAsync(d_lcount, 0, P->nlevels * sizeof(int32_t), st));
    CK(P, cudaMemsetAsync(d_lfill, 0, P->nlevels * sizeof(int32_t), st));
    LAUNCH(P, 1, launch_level_order(N, P->d_level, P->nlevels, d_lcount, nullptr, nullptr, nullptr, st));
    std::vector<int32_t> hc(P->nlevels);
    CK(P, cudaMemcpyAsync(hc.data(), d_lcount, P->nlevels * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK(P, cudaStreamSynchronize(st));
    P->info.d2h_bytes += P->nlevels * sizeof(int32_t);
    P->h_loff.assign(P->nlevels + 1, 0);
    for (int l = 0; l < P->nlevels; ++l) P->h_loff[l + 1] = P->h_loff[l] + hc[l];
    CK(P, cudaMemcpyAsync(d_loff, P->h_loff.data(), (P->nlevels + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    P->info.h2d_bytes += (P->nlevels + 1) * sizeof(int32_t);
    LAUNCH(P, 1, launch_level_order(N, P->d_level, P->nlevels, d_lcount, d_loff, d_lfill, P->d_order, st));
    CK(P, cudaEventRecord(P->ev[2], st));

    // ---- covariance table over the pairwise lags of template offsets ----
    if (!P->d_lut64) {
        int64_t total = 1;
        for (int j = 0; j < 3; ++j) {
            P->lut.e[j] = 2 * P->tmpl_ext[j];
            P->lut.w[j] = 2 * P->lut.e[j] + 1;
            total *= P->lut.w[j];
        }
        if (total <= ((int64_t)1 << 26)) {
            if ((rc = dalloc(P, &P->d_lut64, total))) return rc;
            if ((rc = dalloc(P, &P->d_lut2, total))) return rc;
            P->lut.c64 = P->d_lut64;
            P->lut.c2 = P->d_lut2;
            LAUNCH(P, 1, launch_fill_cov_lut(P->grid, P->vario, P->lut, P->d_lut64, P->d_lut2, st));
        } else {
            P->lut.c64 = nullptr;
            P->lut.c2 = nullptr;
        }
    }

    // ---- (b) kriging systems ----
    if (P->precision == SGS_PREC_FP64) {
        if (!P->t64.node) {
            if ((rc = dalloc(P, &P->t64.node, N))) return rc;
            if ((rc = dalloc(P, &P->t64.m, N))) return rc;
            if ((rc = dalloc(P, &P->t64.idx, (size_t)N * k))) return rc;
            if ((rc = dalloc(P, &P->t64.w, (size_t)N * k))) return rc;
            if ((rc = dalloc(P, &P->t64.b0, N))) return rc;
            if ((rc = dalloc(P, &P->t64.sigma, N))) return rc;
        }
    } else {
        if (!P->t32.node) {
            if ((rc = dalloc(P, &P->t32.node, N))) return rc;
            if ((rc = dalloc(P, &P->t32.m, N))) return rc;
            if ((rc = dalloc(P, &P->t32.idx, (size_t)N * k))) return rc;
            if ((rc = dalloc(P, &P->t32.w, (size_t)N * k * 2))) return rc;
            if ((rc = dalloc(P, &P->t32.b0, 2 * N))) return rc;
            if ((rc = dalloc(P, &P->t32.sigma, 2 * N))) return rc;
            if ((rc = dalloc(P, &P->d_fallback, N))) return rc;
        }
    }
    if (!P->d_flow && (rc = dalloc(P, &P->d_flow, 2))) return rc;
    if (P->ind_ncat && !P->d_ind_wsum) {
        if ((rc = dalloc(P, &P->d_ind_wsum, N))) return rc;
        if ((rc = dalloc(P, &P->d_ind_dsum, (size_t)N * P->ind_ncat))) return rc;
    }
    CK(P, cudaEventRecord(P->ev[3], st));
    if ((rc = run_solve(P, nullptr, nullptr))) return rc;
    {
        unsigned int wl1 = 0;
        CK(P, cudaMemcpyAsync(&wl1, P->d_wl1, sizeof(wl1), cudaMemcpyDeviceToHost, st));
        CK(P, cudaStreamSynchronize(st));
        P->info.d2h_bytes += sizeof(wl1);
        float f;
        std::memcpy(&f, &wl1, sizeof(f));
        P->info.weight_l1_max = f;
        P->promote = P->precision == SGS_PREC_FP32_REFINE && f > SGS_FP32_VALUE_L1_LIMIT && !P->data_only;
        P->info.values_fp64 = values_fp64(P) ? 1 : 0;
        if (P->promote) {
            if (!P->t64p.w) {
                if ((rc = dalloc(P, &P->t64p.w, (size_t)N * k))) return rc;
                if ((rc = dalloc(P, &P->t64p.b0, N))) return rc;
                if ((rc = dalloc(P, &P->t64p.sigma, N))) return rc;
            }
            LAUNCH(P, 1, launch_tables_to_fp64(P->t32, P->t64p, N, N * (int64_t)k, st));
        }
    }
    if (P->cok || P->mv) {
        // cokriging systems of every position (they replace the nodes' status)
        const int L = P->mv ? P->mv_nvars : P->ind_ncat;
        if (P->d_cok_m && P->cok_L != L) free_cok_tables(P);
        if (!P->d_cok_m) {
            if ((rc = dalloc(P, &P->d_cok_m, N))) return rc;
            if ((rc = dalloc(P, &P->d_cok_idx, (size_t)N * k))) return rc;
            if ((rc = dalloc(P, &P->d_cok_w, (size_t)N * k * L * L))) return rc;
            if ((rc = dalloc(P, &P->d_cok_cst, (size_t)N * L))) return rc;
            P->cok_L = L;
        }
        if (P->mv && !P->d_mv_fac)
            if ((rc = dalloc(P, &P->d_mv_fac, (size_t)N * L * L))) return rc;
        SolveArgs s{};
        s.grid = P->grid;
        s.vario = P->vario;
        s.k = P->k;
        s.nmin = P->nmin;
        s.P = P->N;
        s.order = P->d_order;
        s.nbr = P->d_nbr;
        s.cnt = P->d_cnt;
        s.N = P->N;
        s.data_xyz = P->d_dxyz;
        s.status = P->d_status;
        LAUNCH(P, 1, launch_cok_solve(s, cok_args(P), P->mv, st));
    }
    CK(P, cudaEventRecord(P->ev[4], st));
    LAUNCH(P, 1, launch_count_nonzero(N, P->d_status, P->d_stats + 2, P->nsm, st));
    CK(P, cudaStreamSynchronize(st));
    dfree(P, d_lcount);
    dfree(P, d_lfill);
    P->info.ms_search = elapsed(P->ev[0], P->ev[1]);
    P->info.ms_levels = elapsed(P->ev[1], P->ev[2]);
    P->info.ms_solve = elapsed(P->ev[3], P->ev[4]);
    P->info.nlevels = P->nlevels;
    {
        unsigned long long sm = 0, stats[3] = {0, 0, 0};
        CK(P, cudaMemcpy(&sm, P->d_sum_m, sizeof(sm), cudaMemcpyDeviceToHost));
        CK(P, cudaMemcpy(stats, P->d_stats, sizeof(stats), cudaMemcpyDeviceToHost));
        P->info.d2h_bytes += sizeof(sm) + sizeof(stats);
        P->info.search_grid_candidates = (int64_t)stats[0];
        P->info.search_data_candidates = (int64_t)stats[1];
        P->info.n_prior = (int64_t)stats[2];
        P->info.sum_grid_neighbors = (int64_t)sm;
    }
    P->prepared = true;
    return SGS_OK;
}

// error flag of the last dataflow sweep (the caller has synchronized)
static int check_flow_error(sgs_plan* P) {
    if (!P->d_flow || P->last_sweep_mode != SGS_SWEEP_FLOW) return SGS_OK;
    int32_t err = 0;
    CK(P, cudaMemcpy(&err, P->d_flow + 1, sizeof(err), cudaMemcpyDeviceToHost));
    if (err) return set_err(P, SGS_ERR_TIMEOUT, "dataflow sweep: a dependency wait exceeded its bound");
    return SGS_OK;
}

static int run_sweep(sgs_plan* P, int R, int Rp, const void* z, uint64_t seed, void* V, cudaStream_t st) {
    (void)R;
    const sgs_sweep_config& c = P->sweep;
    P->last_sweep_mode = c.mode;
    if (c.mode == SGS_SWEEP_COOPERATIVE) {
        // all levels in one cooperative launch (per-level launches if the
        // device or the launch configuration does not allow it)
        cudaError_t e;
        if (values_fp64(P))
            e = launch_sweep_all_fp64(sweep64(P), P->k, P->d_loff, P->nlevels, Rp, (const double*)z, seed, (double*)V, st);
        else
            e = launch_sweep_all_fp32(P->t32, P->k, P->d_loff, P->nlevels, Rp, (const float*)z, seed, (float*)V, st);
        if (e == cudaSuccess) {
            P->info.launches++;
            return SGS_OK;
        }
        cudaGetLastError();
        P->last_sweep_mode = SGS_SWEEP_LEVELS;
    } else if (c.mode == SGS_SWEEP_FLOW) {
        // leading levels by per-level launches, the rest in one dataflow launch
        int W = c.lanes_w, G = c.lanes_g;
        const int H = flow_layout(Rp, W, G);
        const int64_t nflags = P->N * H;
        if (nflags > P->done_cap) {
            CK(P, cudaStreamSynchronize(st));
            dfree(P, P->d_done);
            P->d_done = nullptr;
            P->done_cap = 0;
            int rc;
            if ((rc = dalloc(P, &P->d_done, nflags))) return rc;
            P->done_cap = nflags;
            CK(P, cudaMemsetAsync(P->d_done, 0, nflags * sizeof(int32_t), st));
            P->flow_epoch = 0;
        }
        if (P->flow_epoch >= 0x7ffffff0) {
            CK(P, cudaMemsetAsync(P->d_done, 0, P->done_cap * sizeof(int32_t), st));
            P->flow_epoch = 0;
        }
        // levels [lo, hi) by per-level launches, the rest by dataflow launches
        const int lo = std::max(0, std::min(c.level_lo, P->nlevels));
        const int hi = std::max(lo, std::min(c.level_hi, P->nlevels));
        const int64_t plo = P->h_loff[lo], phi = P->h_loff[hi];
        const int32_t epoch = ++P->flow_epoch;
        CK(P, cudaMemsetAsync(P->d_flow, 0, 2 * sizeof(unsigned long long), st));
        auto flow = [&](int64_t p0, int64_t p1) -> int {
            FlowArgs f{};
            f.item0 = p0 * H;
            f.item1 = p1 * H;
            f.N = P->N;
            f.H = H;
            f.done = P->d_done;
            f.epoch = epoch;
            f.ticket = P->d_flow;
            f.err = reinterpret_cast<int32_t*>(P->d_flow + 1);
            f.chunk = std::max(1, c.chunk);
            f.blocks_per_sm = c.blocks_per_sm;
            f.tight = c.tight;
            f.wait_ns = 10000000000ull;  // 10 s: far beyond any dependency chain
            cudaError_t e;
            if (values_fp64(P))
                e = launch_sweep_flow_fp64(sweep64(P), P->k, Rp, W, G, (const double*)z, seed, (double*)V, f, P->nsm, st);
            else
                e = launch_sweep_flow_fp32(P->t32, P->k, Rp, W, G, (const float*)z, seed, (float*)V, f, P->nsm, st);
            if (e != cudaSuccess) return cuda_err(P, e, "sweep launch");
            P->info.launches++;
            return SGS_OK;
        };
        int rc;
        if (plo > 0 && (rc = flow(0, plo))) return rc;
        for (int l = lo; l < hi; ++l) {
            const int64_t p0 = P->h_loff[l], p1 = P->h_loff[l + 1];
            cudaError_t e;
            if (values_fp64(P))
                e = launch_sweep_fp64(sweep64(P), P->k, p0, p1, Rp, (const double*)z, seed, (double*)V, st);
            else
                e = launch_sweep_fp32(P->t32, P->k, p0, p1, Rp, (const float*)z, seed, (float*)V, st, c.lanes_g,
                                      (p1 - p0) < (int64_t)c.split_nodes);
            if (e != cudaSuccess) return cuda_err(P, e, "sweep launch");
            if (p1 > p0) P->info.launches++;
        }
        if (phi < P->N) {
            const int32_t* node = values_fp64(P) ? sweep64(P).node : P->t32.node;
            if (phi > plo) LAUNCH(P, 1, launch_flow_mark(node, plo, phi, H, P->N, P->d_done, epoch, st));
            if (plo > 0) CK(P, cudaMemsetAsync(P->d_flow, 0, sizeof(unsigned long long), st));  // ticket only
            if ((rc = flow(phi, P->N))) return rc;
        }
        return SGS_OK;
    }
    for (int l = 0; l < P->nlevels; ++l) {
        const int64_t p0 = P->h_loff[l], p1 = P->h_loff[l + 1];
        cudaError_t e;
        if (values_fp64(P))
            e = launch_sweep_fp64(sweep64(P), P->k, p0, p1, Rp, (const double*)z, seed, (double*)V, st);
        else
            e = launch_sweep_fp32(P->t32, P->k, p0, p1, Rp, (const float*)z, seed, (float*)V, st, c.lanes_g,
                                  (p1 - p0) < (int64_t)c.split_nodes);
        if (e != cudaSuccess) return cuda_err(P, e, "sweep launch");
        if (p1 > p0) P->info.launches++;
    }
    return SGS_OK;
}

extern "C" int sgs_plan_simulate_device(sgs_plan* P, int32_t R, const void* z_dev, uint64_t seed, void* vals_dev,
                                        void* stream) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "simulate before prepare");
    if (R < 1 || !vals_dev) return set_err(P, SGS_ERR_ARG, "invalid nreals or output");
    CK(P, cudaSetDevice(P->device));
    const int Rp = (R + 3) / 4 * 4;
    cudaStream_t st = stream ? (cudaStream_t)stream : P->stream;
    CK(P, cudaEventRecord(P->ev[5], st));
    int rc = run_sweep(P, R, Rp, z_dev, seed, vals_dev, st);
    if (rc) return rc;
    CK(P, cudaEventRecord(P->ev[6], st));
    P->sweep_timed = true;
    return SGS_OK;
}

extern "C" int sgs_plan_simulate(sgs_plan* P, int32_t R, const double* z, uint64_t seed, double* out) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "simulate before prepare");
    if (R < 1 || !out) return set_err(P, SGS_ERR_ARG, "invalid nreals or output");
    CK(P, cudaSetDevice(P->device));
    const int64_t N = P->N;
    const int Rp = (R + 3) / 4 * 4;
    const size_t es = values_fp64(P) ? sizeof(double) : sizeof(float);
    cudaStream_t st = P->stream;
    int rc;
    void* V = nullptr;
    void* zr = nullptr;
    double* zin = nullptr;
    if ((rc = dalloc(P, (unsigned char**)&V, (size_t)N * Rp * es))) return rc;
    if (z) {
        if ((rc = dalloc(P, &zin, (size_t)N * R))) { dfree(P, V); return rc; }
        if ((rc = dalloc(P, (unsigned char**)&zr, (size_t)N * Rp * es))) { dfree(P, V); dfree(P, zin); return rc; }
        CK(P, cudaMemcpyAsync(zin, z, (size_t)N * R * sizeof(double), cudaMemcpyHostToDevice, st));
        P->info.h2d_bytes += (int64_t)N * R * sizeof(double);
        if (values_fp64(P)) LAUNCH(P, 1, launch_z_to_rows_fp64(zin, N, R, Rp, (double*)zr, st));
        else LAUNCH(P, 1, launch_z_to_rows_fp32(zin, N, R, Rp, (float*)zr, st));
    }
    CK(P, cudaEventRecord(P->ev[5], st));
    rc = run_sweep(P, R, Rp, zr, seed, V, st);
    if (rc) return rc;
    CK(P, cudaEventRecord(P->ev[6], st));
    // realization-major FP64 output: written by the transposing kernel
    // straight into `out` when it is page-locked host memory the device can
    // address, else in chunks of realizations through a device buffer
    double* dout = pinned_device_view(out);
    if (dout && (P->flags & SGS_FLAG_OUTPUT_STAGED)) {
        // chunks of realizations transposed on the plan's stream into two
        // device buffers in turn, each copied out by the copy engines on a
        // second stream while the next chunk is transposed
        const int64_t stage_bytes = (int64_t)1 << 28;
        const int64_t rc_n = std::max<int64_t>(1, std::min<int64_t>(R, stage_bytes / (N * (int64_t)sizeof(double))));
        double* sb[2] = {nullptr, nullptr};
        if ((rc = dalloc(P, &sb[0], (size_t)N * rc_n)) || (rc = dalloc(P, &sb[1], (size_t)N * rc_n))) {
            dfree(P, sb[0]);
            return rc;
        }
        cudaStream_t cs = nullptr;
        cudaEvent_t made[2] = {nullptr, nullptr}, moved[2] = {nullptr, nullptr};
        bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
        for (int b = 0; ok && b < 2; ++b)
            ok = cudaEventCreateWithFlags(&made[b], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&moved[b], cudaEventDisableTiming) == cudaSuccess;
        int64_t i = 0;
        for (int64_t r0 = 0; ok && r0 < R; r0 += rc_n, ++i) {
            const int rn = (int)std::min<int64_t>(rc_n, R - r0);
            const int b = (int)(i & 1);
            if (i >= 2) ok = ok && cudaStreamWaitEvent(st, moved[b], 0) == cudaSuccess;  // buffer free again
            const cudaError_t e = values_fp64(P)
                ? launch_rows_to_out_fp64((const double*)V + r0, N, rn, Rp, P->mean, sb[b], st)
                : launch_rows_to_out_fp32((const float*)V + r0, N, rn, Rp, P->mean, sb[b], st);
            ok = ok && e == cudaSuccess && cudaEventRecord(made[b], st) == cudaSuccess &&
                 cudaStreamWaitEvent(cs, made[b], 0) == cudaSuccess &&
                 cudaMemcpyAsync(out + r0 * N, sb[b], (size_t)N * rn * sizeof(double), cudaMemcpyDeviceToHost, cs) ==
                     cudaSuccess &&
                 cudaEventRecord(moved[b], cs) == cudaSuccess;
            P->info.launches++;
            P->info.d2h_bytes += (int64_t)N * rn * sizeof(double);
        }
        ok = ok && cudaStreamSynchronize(cs) == cudaSuccess;
        const cudaError_t err = cudaGetLastError();
        for (int b = 0; b < 2; ++b) {
            if (made[b]) cudaEventDestroy(made[b]);
            if (moved[b]) cudaEventDestroy(moved[b]);
        }
        if (cs) cudaStreamDestroy(cs);
        dfree(P, sb[0]);
        dfree(P, sb[1]);
        if (!ok) return cuda_err(P, err != cudaSuccess ? err : cudaErrorUnknown, "staged output");
    } else if (dout) {
        if (values_fp64(P))
            LAUNCH(P, 1, launch_rows_to_out_fp64((const double*)V, N, R, Rp, P->mean, dout, st));
        else
            LAUNCH(P, 1, launch_rows_to_out_fp32((const float*)V, N, R, Rp, P->mean, dout, st));
        P->info.d2h_bytes += (int64_t)N * R * sizeof(double);
    }
    const int64_t chunk_bytes = (int64_t)1 << 29;
    int64_t rchunk = std::max<int64_t>(1, std::min<int64_t>(R, chunk_bytes / (N * (int64_t)sizeof(double))));
    double* ob = nullptr;
    if (!dout && (rc = dalloc(P, &ob, (size_t)N * rchunk))) return rc;
    for (int64_t r0 = 0; !dout && r0 < R; r0 += rchunk) {
        const int rn = (int)std::min<int64_t>(rchunk, R - r0);
        // rows_to_out reads realizations [r0, r0+rn) of each row
        if (values_fp64(P))
            LAUNCH(P, 1, launch_rows_to_out_fp64((const double*)V + r0, N, rn, Rp, P->mean, ob, st));
        else
            LAUNCH(P, 1, launch_rows_to_out_fp32((const float*)V + r0, N, rn, Rp, P->mean, ob, st));
        CK(P, cudaMemcpyAsync(out + r0 * N, ob, (size_t)N * rn * sizeof(double), cudaMemcpyDeviceToHost, st));
        P->info.d2h_bytes += (int64_t)N * rn * sizeof(double);
    }
    CK(P, cudaStreamSynchronize(st));
    if ((rc = check_flow_error(P))) return rc;
    P->info.ms_sweep = elapsed(P->ev[5], P->ev[6]);
    P->sweep_timed = false;
    dfree(P, ob);
    dfree(P, V);
    if (zin) dfree(P, zin);
    if (zr) dfree(P, zr);
    return SGS_OK;
}

extern "C" int sgs_plan_neighbors(sgs_plan* P, int32_t* idx, int32_t* count) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "neighbors before prepare");
    CK(P, cudaSetDevice(P->device));
    if (idx) CK(P, cudaMemcpy(idx, P->d_nbr, (size_t)P->N * P->k * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (count) CK(P, cudaMemcpy(count, P->d_cnt, (size_t)P->N * sizeof(int32_t), cudaMemcpyDeviceToHost));
    P->info.d2h_bytes += (idx ? (int64_t)P->N * P->k * 4 : 0) + (count ? P->N * 4 : 0);
    return SGS_OK;
}

extern "C" int sgs_plan_weights(sgs_plan* P, double* weights, double* sigma, int32_t* status) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "weights before prepare");
    CK(P, cudaSetDevice(P->device));
    const int64_t N = P->N;
    int rc;
    if (weights || sigma) {
        double *wf = nullptr, *sf = nullptr;
        if ((rc = dalloc(P, &wf, (size_t)N * P->k))) return rc;
        if ((rc = dalloc(P, &sf, N))) { dfree(P, wf); return rc; }
        if ((rc = run_solve(P, wf, sf))) return rc;
        if (weights) CK(P, cudaMemcpyAsync(weights, wf, (size_t)N * P->k * sizeof(double), cudaMemcpyDeviceToHost, P->stream));
        if (sigma) CK(P, cudaMemcpyAsync(sigma, sf, (size_t)N * sizeof(double), cudaMemcpyDeviceToHost, P->stream));
        CK(P, cudaStreamSynchronize(P->stream));
        dfree(P, wf);
        dfree(P, sf);
    }
    if (status) {
        std::vector<int8_t> st8(N);
        CK(P, cudaMemcpy(st8.data(), P->d_status, N, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < N; ++i) status[i] = st8[i];
    }
    return SGS_OK;
}

extern "C" int sgs_plan_levels(sgs_plan* P, int32_t* level, int32_t* nlevels) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "levels before prepare");
    CK(P, cudaSetDevice(P->device));
    if (level) CK(P, cudaMemcpy(level, P->d_level, (size_t)P->N * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (nlevels) *nlevels = P->nlevels;
    return SGS_OK;
}

extern "C" int sgs_plan_info(const sgs_plan* P, sgs_info* info) {
    if (!P || !info) return set_err(nullptr, SGS_ERR_ARG, "null argument");
    *info = P->info;
    if (P->sweep_timed) {  // a device-resident sweep: time it once it has finished
        cudaSetDevice(P->device);
        if (cudaEventSynchronize(P->ev[6]) == cudaSuccess) info->ms_sweep = elapsed(P->ev[5], P->ev[6]);
        // a device-resident dataflow sweep reports a failed wait here
        return check_flow_error(const_cast<sgs_plan*>(P));
    }
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// learned warm start
extern "C" int sgs_plan_features_device(sgs_plan* P, float* feat_dev, void* stream) {
    if (!P || !feat_dev) return set_err(P, SGS_ERR_ARG, "null argument");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "features before prepare");
    CK(P, cudaSetDevice(P->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->stream;
    LAUNCH(P, 1, launch_nn_features(P->grid, P->vario, P->d_nbr, P->d_cnt, P->k, P->d_dxyz, feat_dev, st));
    CK(P, cudaStreamSynchronize(st));
    return SGS_OK;
}

extern "C" int sgs_plan_set_network(sgs_plan* P, const float* params) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    CK(P, cudaSetDevice(P->device));
    if (!params) {
        dfree(P, P->d_nn);
        P->d_nn = nullptr;
        return SGS_OK;
    }
    int rc;
    if (!P->d_nn && (rc = dalloc(P, &P->d_nn, SGS_NN_PARAMS))) return rc;
    CK(P, cudaMemcpy(P->d_nn, params, SGS_NN_PARAMS * sizeof(float), cudaMemcpyHostToDevice));
    P->info.h2d_bytes += SGS_NN_PARAMS * sizeof(float);
    return SGS_OK;
}

extern "C" int sgs_nn_forward(const float* params, const float* feat, const int32_t* count, int64_t nsys, int32_t k,
                              float* pred, void* stream) {
    if (!params || !feat || !count || !pred || nsys < 0 || k < 1 || k > KMAX)
        return set_err(nullptr, SGS_ERR_ARG, "invalid argument");
    if (nsys == 0) return SGS_OK;
    cudaError_t e = launch_nn_forward(params, feat, count, nsys, k, pred, (cudaStream_t)stream);
    return e == cudaSuccess ? SGS_OK : cuda_err(nullptr, e, "sgs_nn_forward");
}

extern "C" int sgs_nn_backward(const float* params, const float* feat, const int32_t* count, const float* target,
                               int64_t nsys, int32_t k, float* grad, float* loss, void* stream) {
    if (!params || !feat || !count || !target || !grad || !loss || nsys < 0 || k < 1 || k > KMAX)
        return set_err(nullptr, SGS_ERR_ARG, "invalid argument");
    if (nsys == 0) return SGS_OK;
    cudaError_t e = launch_nn_backward(params, feat, count, target, nsys, k, grad, loss, (cudaStream_t)stream);
    return e == cudaSuccess ? SGS_OK : cuda_err(nullptr, e, "sgs_nn_backward");
}

extern "C" int sgs_nn_adam(float* params, const float* grad, float* m, float* v, int32_t step, float lr, float scale,
                           void* stream) {
    if (!params || !grad || !m || !v || step < 1) return set_err(nullptr, SGS_ERR_ARG, "invalid argument");
    cudaError_t e = launch_nn_adam(params, grad, m, v, step, lr, scale, (cudaStream_t)stream);
    return e == cudaSuccess ? SGS_OK : cuda_err(nullptr, e, "sgs_nn_adam");
}

// ---------------------------------------------------------------------------
// Sweep configuration and its autotuner.
extern "C" int sgs_plan_set_sweep(sgs_plan* P, const sgs_sweep_config* c) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!c) return set_err(P, SGS_ERR_ARG, "null sweep configuration");
    if (c->mode < SGS_SWEEP_FLOW || c->mode > SGS_SWEEP_LEVELS) return set_err(P, SGS_ERR_ARG, "unknown sweep mode");
    if (c->mode == SGS_SWEEP_FLOW &&
        (c->chunk < 0 || c->chunk > 64 || c->blocks_per_sm < 0 || c->blocks_per_sm > 32 || c->lanes_g < 0 ||
         c->lanes_g > 2 || c->lanes_w < 0 || c->lanes_w > 32 || (c->lanes_w & (c->lanes_w - 1)) ||
         c->level_lo < 0 || c->level_hi < 0 || c->tight < 0 || c->tight > 1 || c->split_nodes < 0))
        return set_err(P, SGS_ERR_ARG, "invalid dataflow sweep parameters");
    if (c->mode == SGS_SWEEP_LEVELS && (c->lanes_g < 0 || c->lanes_g > 4 || c->lanes_g == 3 || c->split_nodes < 0))
        return set_err(P, SGS_ERR_ARG, "invalid per-level sweep parameters (lanes_g 0, 1, 2 or 4, split_nodes >= 0)");
    P->sweep = *c;
    if (P->sweep.chunk < 1) P->sweep.chunk = 1;
    return SGS_OK;
}

// time one sweep configuration (after a warm-up run); < 0 on failure
static int time_sweep(sgs_plan* P, const sgs_sweep_config& c, int R, int Rp, void* V, float* ms) {
    P->sweep = c;
    cudaStream_t st = P->stream;
    int rc;
    if ((rc = run_sweep(P, R, Rp, nullptr, 7, V, st))) return rc;
    CK(P, cudaEventRecord(P->ev[5], st));
    if ((rc = run_sweep(P, R, Rp, nullptr, 7, V, st))) return rc;
    CK(P, cudaEventRecord(P->ev[6], st));
    CK(P, cudaStreamSynchronize(st));
    if ((rc = check_flow_error(P))) return rc;
    *ms = elapsed(P->ev[5], P->ev[6]);
    return SGS_OK;
}

extern "C" int sgs_plan_tune_sweep(sgs_plan* P, int32_t R, sgs_sweep_config* chosen, sgs_sweep_config* tried,
                                   int32_t max_tried, int32_t* ntried) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "tune before prepare");
    if (R < 1) return set_err(P, SGS_ERR_ARG, "invalid nreals");
    CK(P, cudaSetDevice(P->device));
    const int Rp = (R + 3) / 4 * 4;
    const int cpn = Rp / 4;
    const bool fp64 = values_fp64(P);
    const size_t es = fp64 ? sizeof(double) : sizeof(float);
    void* V = nullptr;
    int rc;
    if ((rc = dalloc(P, (unsigned char**)&V, (size_t)P->N * Rp * es))) return rc;
    const sgs_sweep_config saved = P->sweep;
    std::vector<sgs_sweep_config> done;
    int best = -1;
    auto run = [&](sgs_sweep_config c) -> int {
        float ms = 0.f;
        int r = time_sweep(P, c, R, Rp, V, &ms);
        if (r) return r;
        c.ms = ms;
        done.push_back(c);
        if (best < 0 || ms < done[best].ms) best = (int)done.size() - 1;
        return SGS_OK;
    };
    // stage 1: per-level launches and whole-sweep dataflow mappings
    int p2 = 1;
    while (p2 < cpn && p2 < 32) p2 <<= 1;
    rc = run({SGS_SWEEP_LEVELS, 1, 0, 1, 0, 0, 0, 0, 0, 0.f});
    // per-level launches with 2 or 4 chunks of 4 realizations per thread
    for (int G = 2; !rc && !fp64 && G <= 4 && cpn > 16 && Rp % (4 * G) == 0; G *= 2)
        rc = run({SGS_SWEEP_LEVELS, 1, 0, G, 0, 0, 0, 0, 0, 0.f});
    // the best per-level form with small levels split over a block's warps
    if (!rc && !fp64 && Rp % 8 == 0) {
        int bl = -1;
        for (int i = 0; i < (int)done.size(); ++i)
            if (done[i].mode == SGS_SWEEP_LEVELS && (bl < 0 || done[i].ms < done[bl].ms)) bl = i;
        for (int thr : {256, 1024, 4096, 16384}) {
            if (rc || bl < 0) break;
            sgs_sweep_config c = done[bl];
            c.split_nodes = thr;
            rc = run(c);
        }
    }
    for (int W = p2; !rc && W >= std::max(1, p2 / 4); W >>= 1)
        for (int G = 1; !rc && G <= (cpn >= 2 * W ? 2 : 1); ++G)
            for (int tight = 0; !rc && tight <= 1; ++tight)
                for (int chunk : {1, 2}) {
                    if (rc) break;
                    rc = run({SGS_SWEEP_FLOW, chunk, 0, G, W, 0, 0, tight, 0, 0.f});
                }
    // stage 2: the best dataflow mapping, with the span of large levels
    // (from the first to the last level holding at least `thr` nodes) swept
    // by per-level launches instead
    if (!rc) {
        int bf = -1;
        for (int i = 0; i < (int)done.size(); ++i)
            if (done[i].mode == SGS_SWEEP_FLOW && (bf < 0 || done[i].ms < done[bf].ms)) bf = i;
        int last_lo = -1, last_hi = -1;
        for (int64_t thr : {(int64_t)P->nsm * 64, (int64_t)P->nsm * 16, (int64_t)P->nsm * 4}) {
            int lo = -1, hi = -1;
            for (int l = 0; l < P->nlevels; ++l)
                if (P->h_loff[l + 1] - P->h_loff[l] >= thr) {
                    if (lo < 0) lo = l;
                    hi = l + 1;
                }
            if (bf < 0 || lo < 0 || (lo == last_lo && hi == last_hi)) continue;
            last_lo = lo;
            last_hi = hi;
            sgs_sweep_config c = done[bf];
            c.level_lo = lo;
            c.level_hi = hi;
            if ((rc = run(c))) break;
        }
    }
    // stage 3: the small leading levels (a long chain of levels holding few
    // nodes) by one dataflow launch whose lanes split each neighbour list
    // (W lanes per slice, 32 / W slices), every level from the first one
    // holding at least `thr` nodes by the best per-level form
    if (!rc && !fp64) {
        int bl = -1;
        for (int i = 0; i < (int)done.size(); ++i)
            if (done[i].mode == SGS_SWEEP_LEVELS && (bl < 0 || done[i].ms < done[bl].ms)) bl = i;
        int last_lo = -1;
        for (int64_t thr : {(int64_t)P->nsm * 2, (int64_t)P->nsm * 8, (int64_t)P->nsm * 32}) {
            int lo = -1;
            for (int l = 0; l < P->nlevels && lo < 0; ++l)
                if (P->h_loff[l + 1] - P->h_loff[l] >= thr) lo = l;
            if (bl < 0 || lo <= 0 || lo == last_lo) continue;
            last_lo = lo;
            for (int W : {2, 4, 8}) {
                if (rc || W > p2) break;
                sgs_sweep_config c = done[bl];
                c.mode = SGS_SWEEP_FLOW;
                c.chunk = 1;
                c.lanes_w = W;
                c.level_lo = lo;
                c.level_hi = P->nlevels;
                // the per-level part keeps the best per-level form; the
                // dataflow part takes 2 chunks per lane only when they fit
                if (c.lanes_g > 2 || cpn < 2 * W) c.lanes_g = 1;
                rc = run(c);
            }
        }
    }
    dfree(P, V);
    if (rc || best < 0) {
        P->sweep = saved;
        return rc ? rc : set_err(P, SGS_ERR_CUDA, "no sweep configuration could be timed");
    }
    P->sweep = done[best];
    P->sweep_timed = false;
    if (chosen) *chosen = done[best];
    const int n = (int)done.size();
    if (tried)
        for (int i = 0; i < std::min(n, (int)max_tried); ++i) tried[i] = done[i];
    if (ntried) *ntried = n;
    return SGS_OK;
}

extern "C" int sgs_plan_predict_device(sgs_plan* P, float* out, int32_t tensor_cores, void* stream) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "predict before prepare");
    if (!P->d_nn) return set_err(P, SGS_ERR_STATE, "no network set (sgs_plan_set_network)");
    if (!out) return set_err(P, SGS_ERR_ARG, "null output");
    CK(P, cudaSetDevice(P->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->stream;
    int rc;
    if ((rc = run_predict(P, out, tensor_cores != 0, st))) return rc;
    int32_t htc = 0;
    if (tensor_cores) CK(P, cudaMemcpyAsync(&htc, P->d_scratch + kPredErr, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK(P, cudaStreamSynchronize(st));
    if (htc) return set_err(P, SGS_ERR_TIMEOUT, "tensor-core inference: an MMA completion wait exceeded its bound");
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Posterior mean by simple kriging from the data alone: a plan whose search
// keeps data candidates only, prepared as usual (every node then sits on
// dependency level 0), and each node's data term b0 = sum_i w_i (d_i - mu)
// and conditional deviation read back from the sweep tables.
extern "C" int sgs_krige(const sgs_problem* problem, double* mean, double* var) {
    if (!problem || !mean) return set_err(nullptr, SGS_ERR_ARG, "null argument");
    sgs_plan* P = new sgs_plan();
    auto fail = [&](int code) {
        g_create_err = P->err.empty() ? g_create_err : P->err;
        sgs_plan_destroy(P);
        return code;
    };
    int rc = plan_init(P, problem);
    if (rc != SGS_OK) return fail(rc);
    const int64_t N = P->N;
    if (P->D == 0) {  // no data: the prior (priormean, src/expectation/field/gaussian.jl:5-19)
        for (int64_t g = 0; g < N; ++g) {
            mean[g] = P->mean;
            if (var) var[g] = P->vario.sill;
        }
        sgs_plan_destroy(P);
        return SGS_OK;
    }
    P->warm_start = 0;
    P->data_only = 1;
    if ((rc = sgs_plan_prepare(P)) != SGS_OK) return fail(rc);
    std::vector<int32_t> node(N);
    std::vector<int8_t> st(N);
    std::vector<double> b0(N), sd(N);
    if (cudaMemcpy(st.data(), P->d_status, N, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(cuda_err(P, cudaGetLastError(), "status read-back"));
    if (P->precision == SGS_PREC_FP64) {
        if (cudaMemcpy(node.data(), P->t64.node, N * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(b0.data(), P->t64.b0, N * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(sd.data(), P->t64.sigma, N * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(cuda_err(P, cudaGetLastError(), "table read-back"));
    } else {
        std::vector<float> b2(2 * N), s2(2 * N);
        if (cudaMemcpy(node.data(), P->t32.node, N * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(b2.data(), P->t32.b0, N * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(s2.data(), P->t32.sigma, N * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(cuda_err(P, cudaGetLastError(), "table read-back"));
        for (int64_t p = 0; p < N; ++p) {
            b0[p] = (double)b2[2 * p] + (double)b2[2 * p + 1];
            sd[p] = (double)s2[2 * p] + (double)s2[2 * p + 1];
        }
    }
    const double nan = std::nan("");
    for (int64_t p = 0; p < N; ++p) {
        const int32_t g = node[p];
        const bool ok = st[g] == SGS_NODE_KRIGED;
        mean[g] = ok ? P->mean + b0[p] : nan;
        if (var) var[g] = ok ? sd[p] * sd[p] : nan;
    }
    sgs_plan_destroy(P);
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Sequential indicator simulation (indicator.cu): the plan's variogram is the
// categories' common correlogram, data_values are ignored in favour of the
// data categories.
extern "C" int sgs_plan_set_indicator(sgs_plan* P, int32_t ncat, const double* prob, const int32_t* data_cat) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (ncat < 2 || ncat > IND_MAX_CAT) return set_err(P, SGS_ERR_ARG, "ncat must be in 2..8");
    if (!prob) return set_err(P, SGS_ERR_ARG, "null probabilities");
    double s = 0.0;
    for (int l = 0; l < ncat; ++l) {
        if (!(prob[l] >= 0.0) || !std::isfinite(prob[l])) return set_err(P, SGS_ERR_ARG, "probabilities must be >= 0");
        s += prob[l];
    }
    if (!(s > 0.0)) return set_err(P, SGS_ERR_ARG, "probabilities must not all be 0");
    if (P->D > 0 && !data_cat) return set_err(P, SGS_ERR_ARG, "null data categories");
    std::vector<int32_t> cat(std::max<int64_t>(P->D, 1), 0);
    for (int64_t i = 0; i < P->D; ++i) {
        if (data_cat[i] < 0 || data_cat[i] >= ncat) return set_err(P, SGS_ERR_ARG, "data category out of range");
        cat[i] = data_cat[i];
    }
    CK(P, cudaSetDevice(P->device));
    if (P->ind_ncat != ncat) {  // table sizes change: reallocate at the next prepare
        dfree(P, P->d_ind_wsum);
        dfree(P, P->d_ind_dsum);
        P->d_ind_wsum = P->d_ind_dsum = nullptr;
    }
    dfree(P, P->d_ind_cat);
    P->d_ind_cat = nullptr;
    int rc;
    if ((rc = upload(P, &P->d_ind_cat, cat.data(), cat.size()))) return rc;
    CK(P, cudaStreamSynchronize(P->stream));
    P->ind_ncat = ncat;
    for (int l = 0; l < IND_MAX_CAT; ++l) P->ind_prob[l] = l < ncat ? prob[l] / s : 0.0;
    P->cok = false;
    P->mv = false;
    P->prepared = false;
    return SGS_OK;
}

extern "C" int sgs_plan_set_indicator_cokriging(sgs_plan* P, int32_t ncat, const double* prob, const int32_t* data_cat,
                                                const double* coef) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!coef) return set_err(P, SGS_ERR_ARG, "null coregionalization matrices");
    if (ncat >= 2 && (int64_t)ncat * P->k > COK_MAX)
        return set_err(P, SGS_ERR_ARG, "maxneighbors x categories must be at most 64 for cokriging");
    const int S = P->vario.ns;
    for (int i = 0; i < S * ncat * ncat && ncat >= 2 && ncat <= IND_MAX_CAT; ++i)
        if (!std::isfinite(coef[i])) return set_err(P, SGS_ERR_ARG, "coregionalization matrices must be finite");
    const int old_ncat = P->ind_ncat;
    int rc = sgs_plan_set_indicator(P, ncat, prob, data_cat);
    if (rc) return rc;
    if (old_ncat != ncat) free_cok_tables(P);  // table sizes change: reallocate at the next prepare
    // the singular rule's scale: the largest indicator variance
    double vmax = 0.0;
    for (int a = 0; a < ncat; ++a) {
        double v = 0.0;
        for (int s = 0; s < S; ++s) v += coef[((size_t)s * ncat + a) * ncat + a] * P->vario.st[s].sill;
        vmax = std::max(vmax, v);
    }
    if (!(vmax > 0.0)) return set_err(P, SGS_ERR_ARG, "the model's indicator variances must be positive");
    dfree(P, P->d_cok_coef);
    P->d_cok_coef = nullptr;
    std::vector<double> cf(coef, coef + (size_t)S * ncat * ncat);
    if ((rc = upload(P, &P->d_cok_coef, cf.data(), cf.size()))) return rc;
    CK(P, cudaStreamSynchronize(P->stream));
    P->cok_tau = kSingularTau * vmax;
    P->cok = true;
    return SGS_OK;
}

extern "C" int sgs_plan_simulate_indicator(sgs_plan* P, int32_t R, const double* u, uint64_t seed, int32_t* out) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->ind_ncat) return set_err(P, SGS_ERR_STATE, "no indicator set (sgs_plan_set_indicator)");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "simulate before prepare");
    if (R < 1 || !out) return set_err(P, SGS_ERR_ARG, "invalid nreals or output");
    CK(P, cudaSetDevice(P->device));
    const int64_t N = P->N;
    const int Rp = (R + 3) / 4 * 4;
    cudaStream_t st = P->stream;
    int rc;
    uint8_t* C = nullptr;
    double *uin = nullptr, *ur = nullptr;
    int32_t* od = nullptr;
    auto cleanup = [&]() {
        dfree(P, C);
        dfree(P, uin);
        dfree(P, ur);
        dfree(P, od);
    };
    if ((rc = dalloc(P, &C, (size_t)N * Rp))) return rc;
    if (u) {
        if ((rc = dalloc(P, &uin, (size_t)N * R)) || (rc = dalloc(P, &ur, (size_t)N * Rp))) {
            cleanup();
            return rc;
        }
        CK(P, cudaMemcpyAsync(uin, u, (size_t)N * R * sizeof(double), cudaMemcpyHostToDevice, st));
        P->info.h2d_bytes += (int64_t)N * R * sizeof(double);
        LAUNCH(P, 1, launch_z_to_rows_fp64(uin, N, R, Rp, ur, st));
    }
    IndArgs ia{};
    ia.ncat = P->ind_ncat;
    for (int l = 0; l < IND_MAX_CAT; ++l) ia.prob[l] = P->ind_prob[l];
    ia.wsum = P->d_ind_wsum;
    ia.dsum = P->d_ind_dsum;
    CK(P, cudaEventRecord(P->ev[5], st));
    for (int l = 0; l < P->nlevels; ++l) {
        const int64_t p0 = P->h_loff[l], p1 = P->h_loff[l + 1];
        cudaError_t e = P->cok ? launch_cok_level(cok_args(P), P->d_order, P->k, p0, p1, Rp, ur, seed, C, st)
                        : P->precision == SGS_PREC_FP64
                            ? launch_sis_level_fp64(P->t64, P->k, p0, p1, Rp, ia, ur, seed, C, st)
                            : launch_sis_level_fp32(P->t32, P->k, p0, p1, Rp, ia, ur, seed, C, st);
        if (e != cudaSuccess) {
            cleanup();
            return cuda_err(P, e, "indicator sweep launch");
        }
        if (p1 > p0) P->info.launches++;
    }
    CK(P, cudaEventRecord(P->ev[6], st));
    if ((rc = dalloc(P, &od, (size_t)N * R))) {
        cleanup();
        return rc;
    }
    LAUNCH(P, 1, launch_cats_to_out(C, N, R, Rp, od, st));
    CK(P, cudaMemcpyAsync(out, od, (size_t)N * R * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    P->info.d2h_bytes += (int64_t)N * R * sizeof(int32_t);
    CK(P, cudaStreamSynchronize(st));
    P->info.ms_sweep = elapsed(P->ev[5], P->ev[6]);
    cleanup();
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Multivariate Gaussian simulation (indicator.cu, the GAUSS form of the
// cokriging systems): a GaussianProcess whose function is a linear model of
// coregionalization over the plan's structures.
extern "C" int sgs_plan_set_multivariate(sgs_plan* P, int32_t nvars, const double* mean, const double* coef,
                                         const double* data_values) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (nvars < 1 || nvars > IND_MAX_CAT) return set_err(P, SGS_ERR_ARG, "nvars must be in 1..8");
    if ((int64_t)nvars * P->k > COK_MAX)
        return set_err(P, SGS_ERR_ARG, "maxneighbors x variables must be at most 64 for cokriging");
    if (!mean || !coef) return set_err(P, SGS_ERR_ARG, "null means or coregionalization matrices");
    if (P->D > 0 && !data_values) return set_err(P, SGS_ERR_ARG, "null data values");
    const int S = P->vario.ns, L = nvars;
    for (int a = 0; a < L; ++a)
        if (!std::isfinite(mean[a])) return set_err(P, SGS_ERR_ARG, "means must be finite");
    for (int s = 0; s < S; ++s)
        for (int a = 0; a < L; ++a)
            for (int b = 0; b < L; ++b) {
                const double v = coef[((size_t)s * L + a) * L + b];
                if (!std::isfinite(v)) return set_err(P, SGS_ERR_ARG, "coregionalization matrices must be finite");
                if (v != coef[((size_t)s * L + b) * L + a])
                    return set_err(P, SGS_ERR_ARG, "coregionalization matrices must be symmetric");
            }
    for (int64_t i = 0; i < P->D * L; ++i)
        if (!std::isfinite(data_values[i])) return set_err(P, SGS_ERR_ARG, "data values must be finite");
    // the singular rule's scale: the largest variance of a variable
    double vmax = 0.0;
    for (int a = 0; a < L; ++a) {
        double v = 0.0;
        for (int s = 0; s < S; ++s) v += coef[((size_t)s * L + a) * L + a] * P->vario.st[s].sill;
        vmax = std::max(vmax, v);
    }
    if (!(vmax > 0.0)) return set_err(P, SGS_ERR_ARG, "the model's variances must be positive");
    CK(P, cudaSetDevice(P->device));
    int rc;
    dfree(P, P->d_cok_coef);
    P->d_cok_coef = nullptr;
    std::vector<double> cf(coef, coef + (size_t)S * L * L);
    if ((rc = upload(P, &P->d_cok_coef, cf.data(), cf.size()))) return rc;
    dfree(P, P->d_mv_dval);
    P->d_mv_dval = nullptr;
    if (P->D > 0) {
        std::vector<double> dv(data_values, data_values + (size_t)P->D * L);
        if ((rc = upload(P, &P->d_mv_dval, dv.data(), dv.size()))) return rc;
    }
    CK(P, cudaStreamSynchronize(P->stream));
    // leave indicator mode: its per-position sums are not computed any more
    dfree(P, P->d_ind_wsum);
    dfree(P, P->d_ind_dsum);
    P->d_ind_wsum = P->d_ind_dsum = nullptr;
    P->ind_ncat = 0;
    P->cok = false;
    for (int a = 0; a < IND_MAX_CAT; ++a) P->mv_mean[a] = a < L ? mean[a] : 0.0;
    P->mv_nvars = L;
    P->cok_tau = kSingularTau * vmax;
    P->mv = true;
    P->prepared = false;
    return SGS_OK;
}

extern "C" int sgs_plan_simulate_multivariate(sgs_plan* P, int32_t R, const double* z, uint64_t seed, double* out) {
    if (!P) return set_err(nullptr, SGS_ERR_ARG, "null plan");
    if (!P->mv) return set_err(P, SGS_ERR_STATE, "no multivariate model set (sgs_plan_set_multivariate)");
    if (!P->prepared) return set_err(P, SGS_ERR_STATE, "simulate before prepare");
    if (R < 1 || !out) return set_err(P, SGS_ERR_ARG, "invalid nreals or output");
    CK(P, cudaSetDevice(P->device));
    const int L = P->mv_nvars;
    const int64_t N = P->N, NL = N * L;
    const int Rp = (R + 3) / 4 * 4;
    cudaStream_t st = P->stream;
    int rc;
    double *V = nullptr, *zin = nullptr, *zr = nullptr, *od = nullptr;
    auto cleanup = [&]() {
        dfree(P, V);
        dfree(P, zin);
        dfree(P, zr);
        dfree(P, od);
    };
    if ((rc = dalloc(P, &V, (size_t)NL * Rp))) return rc;
    if (z) {
        if ((rc = dalloc(P, &zin, (size_t)NL * R)) || (rc = dalloc(P, &zr, (size_t)NL * Rp))) {
            cleanup();
            return rc;
        }
        CK(P, cudaMemcpyAsync(zin, z, (size_t)NL * R * sizeof(double), cudaMemcpyHostToDevice, st));
        P->info.h2d_bytes += NL * R * (int64_t)sizeof(double);
        // nreals x (L N) -> rows [L N][Rp]: row a*N + g holds variable a of node g
        LAUNCH(P, 1, launch_z_to_rows_fp64(zin, NL, R, Rp, zr, st));
    }
    const CokArgs c = cok_args(P);
    CK(P, cudaEventRecord(P->ev[5], st));
    for (int l = 0; l < P->nlevels; ++l) {
        const int64_t p0 = P->h_loff[l], p1 = P->h_loff[l + 1];
        cudaError_t e = launch_mv_level(c, P->d_order, P->k, N, p0, p1, Rp, zr, seed, V, st);
        if (e != cudaSuccess) {
            cleanup();
            return cuda_err(P, e, "multivariate sweep launch");
        }
        if (p1 > p0) P->info.launches++;
    }
    CK(P, cudaEventRecord(P->ev[6], st));
    if ((rc = dalloc(P, &od, (size_t)NL * R))) {
        cleanup();
        return rc;
    }
    LAUNCH(P, 1, launch_rows_to_out_fp64(V, NL, R, Rp, 0.0, od, st));
    CK(P, cudaMemcpyAsync(out, od, (size_t)NL * R * sizeof(double), cudaMemcpyDeviceToHost, st));
    P->info.d2h_bytes += NL * R * (int64_t)sizeof(double);
    CK(P, cudaStreamSynchronize(st));
    P->info.ms_sweep = elapsed(P->ev[5], P->ev[6]);
    cleanup();
    return SGS_OK;
}

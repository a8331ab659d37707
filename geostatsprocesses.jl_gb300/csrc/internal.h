// internal.h — structures and launch wrappers shared by the host side of
// libgeosgs (api.cu) and the kernel files (search.cu, solve.cu, sweep.cu).
// Not part of the public ABI (include/geosgs.h is).
#pragma once

#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/geosgs.h"

namespace sgs {

constexpr int KMAX = 64;           // largest maxneighbors on the GPU
constexpr int METRIC_ISO = 0;
constexpr int METRIC_ELLIPSOID = 1;
constexpr int METRIC_NEAREST = 2;
constexpr int SGS_NODE_KRIGED_ = 0;          // mirrors SGS_NODE_* of geosgs.h
constexpr int SGS_NODE_PRIOR_NMIN_ = 1;
constexpr int SGS_NODE_PRIOR_SINGULAR_ = 2;

struct GridDev {
    int dim;
    int n[3];
    double origin[3];
    double spacing[3];
    int64_t N;
};

struct MetricDev {
    int kind;
    double rr;          // r*r (iso)
    double radii[3];
    double inv[3];      // 1 / radii, rounded once
    double R[9];        // column-major, leading dimension 3
    double ext[3];      // bounding-box half extents (physical units)
    float Rf[9];        // FP32 copies for the conservative prefilter
    float invf[3];
    float bound_f;      // FP32 prefilter bound: (1 + 1e-3) * (r*r or 1) + slack_f
                        // (+infinity for the unbounded nearest-neighbour metric)
    float slack_f;      // FP32 rounding allowance of the screen near the boundary
    float dh_f;         // bound on the FP32 rounding of an origin-relative coordinate
};

// One structure of a (nested) variogram model.
struct VarioStructDev {
    int type;
    double sill, nugget;
    double inv_range[3];
    double R[9];
};

// The process's variogram: ns structures summed (GeoStatsFunctions'
// NestedVariogram; ns = 1 for a single variogram).  type, inv_range and R
// repeat the first structure (the learned warm start's frame); sill and
// nugget are the model's, the structures' summed.
struct VarioDev {
    int type;
    double sill, nugget;
    double inv_range[3];
    double R[9];
    int ns;
    VarioStructDev st[SGS_MAX_STRUCTURES];
};

// Covariance lookup table over integer grid lags L in [-e, e] per axis:
// entry (L0+e0) + w0*((L1+e1) + w1*(L2+e2)), w = 2e+1.
struct CovLut {
    const double* c64;  // nullptr when absent
    const float2* c2;   // the covariances / sill as FP32 (hi, lo) pairs
    int e[3];
    int w[3];
};

// Offset template entry: cell offset and linear offset of a grid candidate.
struct TmplEntry {
    int dx, dy, dz, dlin;
};

struct SearchArgs {
    GridDev grid;
    MetricDev metric;
    int k;
    int T;                       // template entries
    const TmplEntry* tmpl;
    const double* tmpl_d2;
    const int32_t* path;
    const int32_t* rank;
    int64_t D;
    const double* dxyz;          // data coords, bucket order, D x 3
    const float4* dxyz_f;        // the same relative to the grid origin, FP32 (screen)
    const int32_t* did;          // data id of each bucket-ordered entry
    const int32_t* bstart;       // bucket start offsets (nb+1)
    int nb[3];
    double bw[3];                // bucket widths (physical)
    float inv_bw_f[3];           // FP32 1 / bucket width, for the bucket range
    float ext_f[3];              // FP32 bounding-box half extents
    float spacing_f[3];
    int32_t* nbr;                // N x k, node-indexed
    int32_t* cnt;                // N
    int32_t* ngrid;              // N: grid neighbours among them
    int data_only;               // 1: data candidates only (kriging from the data)
    // optional [2] (single-problem search only): candidates examined (grid:
    // earlier path nodes tested by the early ranks and template entries
    // inside the grid, each one path rank read; data: bucket entries
    // screened), summed once per warp
    unsigned long long* scanned;
};

// Longest wait of the dependency-level kernels for one neighbour's level.
// Their waits end by construction (a neighbour's path rank is smaller, and
// ranks are taken in increasing order by running warps), and the longest
// level computation measured (354 M nodes in one batch) takes 0.6 s in total,
// so a wait of 2 s only happens on a table that breaks the path order.
constexpr uint64_t LEVEL_WAIT_NS = 2000000000ull;

struct LevelArgs {
    int64_t N;
    int k;
    const int32_t* path;
    const int32_t* nbr;
    const int32_t* cnt;
    int32_t* level;              // N, -1 = not yet known
    int32_t* ticket;             // 1 counter
    int32_t* maxlevel;           // 1 counter
    int32_t* err;                // 1 flag
    uint64_t wait_ns;            // longest wait for one neighbour's level
};

// Sweep tables, indexed by position in level order.  For T = double one
// value per entry; for T = float every weight, b0 and sigma is stored as an
// unevaluated FP32 pair (hi, lo) with hi + lo equal to the FP64 value to
// about 2^-48 relative, consumed by the compensated (Dot2) FP32 sweep.
template <typename T>
struct SweepTables {
    static constexpr int S = sizeof(T) == 4 ? 2 : 1;  // entries per value
    int32_t* node;               // P -> node id
    int32_t* m;                  // grid neighbours used
    int32_t* idx;                // P x k grid neighbour node ids
    T* w;                        // P x k x S weights of those
    T* b0;                       // P x S: data term sum_i w_i (d_i - mu)
    T* sigma;                    // P x S: conditional std (sqrt(sill) for the prior)
    const int64_t* off;          // nullptr: row p starts at p * k; else CSR row starts
                                 // (P + 1), used by batches of domains
};

// Dataflow sweep state: warps take items (position in level order x piece of
// the row) from `ticket` and wait, per neighbour, until the neighbour's flag
// of the same piece equals epoch (set once that piece of this sweep is
// stored).
struct FlowArgs {
    int64_t item0;               // first item of this launch (earlier ones are done)
    int64_t item1;               // one past the last item of this launch
    int64_t N;                   // nodes (flag stride between pieces)
    int H;                       // pieces per row
    int32_t* done;               // H x N flags, piece-major
    int32_t epoch;               // > 0, new for every sweep over the same flags
    unsigned long long* ticket;  // 1 counter, zero at launch
    int32_t* err;                // 1 flag, zero at launch
    int chunk;                   // consecutive items taken per ticket
    int blocks_per_sm;           // resident blocks per SM to launch (<= occupancy)
    int tight;                   // 1: kernel compiled for higher residency (register cap)
    uint64_t wait_ns;            // longest wait for one flag before giving up
    const uint64_t* seed_dev;    // nullptr, or the draw seed in device memory (read at
                                 // launch; lets a captured graph take a new seed)
    int pairs;                   // FP64 values, packed tables: every 8-byte weight, b0
                                 // and sigma entry is an FP32 (hi, lo) pair
    int64_t row_stride;          // values between consecutive nodes' rows (0: Rp)
    const uint8_t* node_class;   // nullptr, or a class (0/1) per node: this launch
    int cls;                     // sweeps only the nodes of class cls, and another
                                 // launch the rest (their dependencies never cross)
};

struct SolveArgs {
    GridDev grid;
    VarioDev vario;
    CovLut lut;
    int k;
    int nmin;
    double mu;
    double tau;                  // singular pivot threshold (absolute)
    double inv_sill;             // 1 / sill (the FP32 path works on the correlation matrix)
    int refine_steps;
    int64_t P;                   // positions to solve
    const int32_t* order;        // P -> node
    const int32_t* nbr;
    const int32_t* cnt;
    int64_t N;
    const double* data_xyz;      // D x 3, data id order
    const double* data_val;
    int8_t* status;              // node-indexed
    double* w_full;              // optional N x k export of all weights (node-indexed)
    double* sigma_full;          // optional N
    int32_t* fallback;           // FP32 path: list of positions that need FP64
    int32_t* nfallback;
    const int32_t* list;         // FP64 re-solve: positions to solve (nullptr = all)
    unsigned long long* sum_m;   // accumulates the grid neighbours written to the tables
    const float* w_init;         // optional node-indexed [N][k] warm-start weights (FP32 path)
    unsigned long long* n_warm;  // counts systems accepted from the warm start
    int64_t node0;               // added to node ids written to the sweep tables (the
                                 // domain's first global id in a batch; 0 for a plan)
    // indicator simulation (nullptr otherwise): per position, the sum of all
    // weights and, per category, the sum of the weights of data of that
    // category (zero for prior nodes)
    const int32_t* ind_cat;      // D data categories, 0 .. ncat-1
    int ncat;
    double* ind_wsum;            // [P]
    double* ind_dsum;            // [P][ncat]
    unsigned int* wl1_max;       // optional: FP32 bit pattern of the largest sum of
                                 // |weights| of grid neighbours over the systems
};

// Sequential indicator simulation (indicator.cu).
constexpr int IND_MAX_CAT = 8;
struct IndArgs {
    int ncat;
    double prob[IND_MAX_CAT];    // prior probabilities (normalized)
    const double* wsum;          // [P] sum of a system's weights (0 for the prior)
    const double* dsum;          // [P][ncat] weights of data of each category
};
cudaError_t launch_sis_level_fp32(const SweepTables<float>& t, int k, int64_t p0, int64_t p1, int Rp,
                                  const IndArgs& ia, const double* u, uint64_t seed, uint8_t* C, cudaStream_t s);
cudaError_t launch_sis_level_fp64(const SweepTables<double>& t, int k, int64_t p0, int64_t p1, int Rp,
                                  const IndArgs& ia, const double* u, uint64_t seed, uint8_t* C, cudaStream_t s);
cudaError_t launch_cats_to_out(const uint8_t* C, int64_t N, int R, int Rp, int32_t* out, cudaStream_t s);

// Full simple cokriging of the indicators (indicator.cu) for a linear model
// of coregionalization C_ab(h) = sum_s coef[s][a][b] C_s(h) over the
// structures of the plan's variogram.  Unknowns per system: n x L <= COK_MAX.
// The same systems serve multivariate Gaussian simulation (a GaussianProcess
// whose function is such a model): there L is the number of variables,
// `prob` holds their means, the data's L values replace their categories and
// the solve also factors each node's conditional covariance.
constexpr int COK_MAX = 64;
struct CokArgs {
    int ncat;                    // L
    double prob[IND_MAX_CAT];    // prior probabilities (normalized); Gaussian: the means
    const double* coef;          // [S][L][L]
    const int32_t* data_cat;     // [D] data categories (indicator)
    const double* data_val;      // [D][L] data values (Gaussian)
    double tau;                  // singular pivot threshold (absolute)
    int32_t* m;                  // [P] grid neighbours of the position's system
    int32_t* idx;                // [P][k] their node ids
    double* w;                   // [P][k][L][L] weight of (grid neighbour j, its category b) for category t
    double* cst;                 // [P][L] prior term and the data's contribution
    double* fac;                 // [P][L][L] Gaussian: lower Cholesky factor of the conditional
                                 // covariance (of the prior's for prior nodes), row-major
};
// systems of every position (a: geometry, neighbours, order, status; the
// status of each node is overwritten with its cokriging status)
cudaError_t launch_cok_solve(const SolveArgs& a, const CokArgs& c, bool gaussian, cudaStream_t s);
cudaError_t launch_cok_level(const CokArgs& c, const int32_t* node, int k, int64_t p0, int64_t p1, int Rp,
                             const double* u, uint64_t seed, uint8_t* C, cudaStream_t s);
// One level of the multivariate Gaussian sweep.  V: values [L][N][Rp]
// (variable-major rows of Rp realizations); z: the normals in the same
// layout, or null for the seeded normals of pseudo-node a*N + g.
cudaError_t launch_mv_level(const CokArgs& c, const int32_t* node, int k, int64_t N, int64_t p0, int64_t p1, int Rp,
                            const double* z, uint64_t seed, double* V, cudaStream_t s);

// Host-side description of one problem (api.cu: host_domain): everything
// sgs_plan_create derives on the host before uploading.
struct HostDomain {
    GridDev grid{};
    MetricDev metric{};
    VarioDev vario{};
    double mean = 0.0;
    int k = 0, nmin = 1;
    int64_t N = 0, D = 0;
    std::vector<TmplEntry> tmpl;          // offsets sorted by (d2, linear offset)
    std::vector<double> tmpl_d2;
    int tmpl_ext[3] = {0, 0, 0};          // largest |offset| per axis
    std::vector<double> xyz, val;         // data, id order (xyz: D x 3)
    std::vector<double> xyz_b;            // data, bucket order
    std::vector<int32_t> did, bstart;     // data id per bucket entry; bucket starts
    std::vector<float4> xf;               // FP32 origin-relative coordinates, bucket order
    int nb[3] = {1, 1, 1};
    double bw[3] = {1, 1, 1};
};
// Validates *pr and fills H; SGS_OK or SGS_ERR_ARG with err set.  The path
// is left to the caller: plans and batches build and check its ranks on the
// device (launch_path_ranks, launch_batch_path_ranks).
int host_domain(const sgs_problem* pr, HostDomain& H, std::string& err);
// rank[path[t]] = t for a path of N nodes on the device (path NULL: the
// linear path, written into path_out), checking that the path is a
// permutation of [0, N): *err (zeroed by the caller) is set otherwise.
// path_out may equal path.
cudaError_t launch_path_ranks(const int32_t* path, int64_t N, int32_t* path_out, int32_t* rank, int32_t* err,
                              int nsm, cudaStream_t s);
// The same over a batch's path arena (local ids per domain, domains by the
// offsets off[0..nd]); *bad_domain (preset to nd) takes the smallest domain
// whose path is not a permutation.
cudaError_t launch_batch_path_ranks(const int32_t* path, const int64_t* off, int nd, int64_t total, int32_t* rank,
                                    int32_t* bad_domain, int nsm, cudaStream_t s);
// The geometry fields of a domain's SearchArgs (device pointers left as they are).
void search_args_of(const HostDomain& H, SearchArgs& sa);

// Device address of a page-locked host buffer (cudaHostAlloc'd or
// registered), or nullptr for any other pointer (pageable memory is never
// handed to a kernel).
inline double* pinned_device_view(double* host) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
    return static_cast<double*>(a.devicePointer);
}

// Message returned by sgs_last_error(NULL) on this host thread.
// Device memory of plans and batches comes from one stream-ordered pool per
// device that keeps freed memory for the next plan instead of returning it
// (sgs_trim_memory returns it).  pool_alloc: usable on every stream when it
// returns; pool_free: ordered after the work already queued on `stream`.
cudaError_t pool_alloc(void** ptr, size_t bytes, int device);
cudaError_t pool_free(void* ptr, cudaStream_t stream);

void set_thread_error(const char* msg);
inline void set_thread_error(const std::string& msg) { set_thread_error(msg.c_str()); }

// ---- launch wrappers (return cudaError_t of the launch) ----
cudaError_t launch_search(const SearchArgs& a, cudaStream_t s);
cudaError_t launch_levels(const LevelArgs& a, int nsm, cudaStream_t s);
cudaError_t launch_level_order(int64_t N, const int32_t* level, int nlevels, int32_t* lcount,
                               int32_t* loff, int32_t* lfill, int32_t* order, cudaStream_t s);
cudaError_t launch_solve_fp64(const SolveArgs& a, const SweepTables<double>& t, cudaStream_t s);
cudaError_t launch_solve_fp32(const SolveArgs& a, const SweepTables<float>& t, cudaStream_t s);
cudaError_t launch_solve_fp64_into_fp32(const SolveArgs& a, const SweepTables<float>& t, cudaStream_t s);
// batches of domains (doms: device descriptors, noff: ndom + 1 global node
// offsets, order: level-ordered global node ids; the positions to solve are
// list[desc[1] .. desc[1] + desc[0]), desc on the device)
// *out += the number of nonzero entries of v[0, n) (device counter)
cudaError_t launch_count_nonzero(int64_t n, const int8_t* v, unsigned long long* out, int nsm, cudaStream_t s);
cudaError_t launch_search_batch(const SearchArgs* doms, const int64_t* noff, int ndom, int64_t total, int nsm,
                                cudaStream_t s);
cudaError_t launch_solve_fp32_batch(int nmax, const SolveArgs* doms, const int64_t* noff, int ndom,
                                    const int32_t* order, const int32_t* list, const int32_t* desc,
                                    const SweepTables<float>& t, int nsm, cudaStream_t s);
cudaError_t launch_solve_fp64_batch(int kl, const SolveArgs* doms, const int64_t* noff, int ndom,
                                    const int32_t* order, const int32_t* list, const int32_t* desc,
                                    const SweepTables<double>& t, int nsm, cudaStream_t s);
cudaError_t launch_solve_fp64_into_fp32_batch(int kl, const SolveArgs* doms, const int64_t* noff, int ndom,
                                              const int32_t* order, const int32_t* list, const int32_t* desc,
                                              const SweepTables<float>& t, int nsm, cudaStream_t s);
// pairs = 2 or 4: one thread per 2 or 4 chunks of 4 realizations (rows of a
// multiple of 8 or 16 realizations, more than 64 of them); otherwise one
// thread per chunk.  split = 1 (rows of a multiple of 8 realizations): one
// block per node, the neighbour list split over its warps (small levels).
cudaError_t launch_sweep_fp32(const SweepTables<float>& t, int k, int64_t p0, int64_t p1, int Rp,
                              const float* z, uint64_t seed, float* V, cudaStream_t s, int pairs = 1,
                              int split = 0);
cudaError_t launch_sweep_fp64(const SweepTables<double>& t, int k, int64_t p0, int64_t p1, int Rp,
                              const double* z, uint64_t seed, double* V, cudaStream_t s);
// all levels in one cooperative launch (loff: device level offsets, nlevels + 1)
cudaError_t launch_sweep_all_fp32(const SweepTables<float>& t, int k, const int32_t* loff, int nlevels, int Rp,
                                  const float* z, uint64_t seed, float* V, cudaStream_t s);
cudaError_t launch_sweep_all_fp64(const SweepTables<double>& t, int k, const int32_t* loff, int nlevels, int Rp,
                                  const double* z, uint64_t seed, double* V, cudaStream_t s);
// all levels in one persistent dataflow launch (no level barriers); W lanes
// per slice of the neighbour list and G chunks of 4 realizations per lane,
// as returned by flow_layout, which also gives the pieces per row
int flow_layout(int Rp, int& W, int& G);
cudaError_t launch_flow_wait_selftest(const int32_t* idx, const FlowArgs& f, cudaStream_t s);
cudaError_t launch_sweep_flow_fp32(const SweepTables<float>& t, int k, int Rp, int W, int G, const float* z,
                                   uint64_t seed, float* V, const FlowArgs& f, int nsm, cudaStream_t s);
cudaError_t launch_sweep_flow_fp64(const SweepTables<double>& t, int k, int Rp, int W, int G, const double* z,
                                   uint64_t seed, double* V, const FlowArgs& f, int nsm, cudaStream_t s);
cudaError_t launch_flow_mark(const int32_t* node, int64_t p0, int64_t p1, int H, int64_t N, int32_t* done,
                             int32_t epoch, cudaStream_t s);
int sweep_flow_max_blocks_per_sm(bool fp64, int G, bool tight);
// host z (R x N, realization-major double) on device -> node-major [N][Rp] of T
cudaError_t launch_z_to_rows_fp32(const double* zin, int64_t N, int R, int Rp, float* z, cudaStream_t s);
cudaError_t launch_z_to_rows_fp64(const double* zin, int64_t N, int R, int Rp, double* z, cudaStream_t s);
// node-major centred values -> realization-major double with the mean added
cudaError_t launch_rows_to_out_fp32(const float* V, int64_t N, int R, int Rp, double mu, double* out, cudaStream_t s);
cudaError_t launch_rows_to_out_fp64(const double* V, int64_t N, int R, int Rp, double mu, double* out, cudaStream_t s);
// FP64 copies of packed (hi, lo) sweep tables: w of `entries` weights, b0 and
// sigma of P positions (node, m, idx and off are shared with the source)
cudaError_t launch_tables_to_fp64(const SweepTables<float>& src, SweepTables<double>& dst, int64_t P,
                                  int64_t entries, cudaStream_t s);
cudaError_t launch_fill_cov_lut(const GridDev& g, const VarioDev& v, CovLut lut, double* c64, float2* c2, cudaStream_t s);
// learned warm start (learned.cu)
cudaError_t launch_nn_features(const GridDev& G, const VarioDev& v, const int32_t* nbr, const int32_t* cnt, int k,
                               const double* data_xyz, float* feat, cudaStream_t s);
cudaError_t launch_nn_predict_plan(const GridDev& G, const VarioDev& v, const int32_t* nbr, const int32_t* cnt, int k,
                                   const double* data_xyz, const float* params, float* out, cudaStream_t s);
// BF16 tensor-core inference (learned_tc.cu); err: device flag set when an
// MMA completion wait gave up
cudaError_t launch_nn_predict_tc(const GridDev& G, const VarioDev& v, const int32_t* nbr, const int32_t* cnt, int k,
                                 const double* data_xyz, const float* params, float* out, int32_t* err, int nsm,
                                 cudaStream_t s);
cudaError_t launch_nn_forward(const float* params, const float* feat, const int32_t* count, int64_t nsys, int k,
                              float* pred, cudaStream_t s);
cudaError_t launch_nn_backward(const float* params, const float* feat, const int32_t* count, const float* target,
                               int64_t nsys, int k, float* grad, float* loss, cudaStream_t s);
cudaError_t launch_nn_adam(float* p, const float* g, float* m, float* v, int step, float lr, float scale,
                           cudaStream_t s);

}  // namespace sgs

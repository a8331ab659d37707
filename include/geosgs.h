/*
 * geosgs.h — C ABI of libgeosgs.so: sequential Gaussian simulation (SGS) of a
 * GaussianProcess on a Cartesian grid, on one GB300 GPU.
 *
 * This is the drop-in boundary for the SEQSIM method of GeoStatsProcesses.jl
 * (src/simulation/field/seqsim.jl).  The reference splits a simulation into
 *   preprocess(rng, process, method, init, domain, data)   seqsim.jl:50-70
 *   randsingle(rng, process, method, domain, data, preproc) seqsim.jl:72-156
 * called from rand(rng, process, domain, nreals; data, method)
 * (src/simulation/field.jl:73-124).  With one simulation path shared by all
 * realizations, everything randsingle computes per node except the draw
 * (neighbour search seqsim.jl:107, kriging fit seqsim.jl:124, conditional
 * seqsim.jl:127-131) depends only on geometry and path rank, so it moves into
 * a plan that is prepared once; the per-realization work becomes one batched,
 * level-scheduled sweep over all realizations.
 *
 * Conventions
 *  - All host buffers are owned by the caller; the library copies in and out
 *    and keeps no host pointer after a call returns.  A plan owns all device
 *    memory and one CUDA stream.  One host thread uses a plan at a time.
 *  - Every entry point returns 0 (SGS_OK) or a negative SGS_ERR_* code and
 *    never aborts; sgs_last_error() gives the message of the last failure.
 *  - Indices are 0-based.  Grid node id g = i0 + n0*(i1 + n1*i2) (first axis
 *    fastest, like Julia's LinearIndices).  The "augmented" point set of the
 *    reference (seqsim.jl:211-218) is grid nodes 0..N-1 followed by data
 *    points N..N+D-1 (seqsim.jl:267-271, ExplicitInit).
 *  - Host matrices of realizations are realization-major: element (r, g) at
 *    [r*N + g], i.e. an N x R column-major Julia matrix.
 */
#ifndef GEOSGS_H
#define GEOSGS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SGS_OK            0
#define SGS_ERR_ARG      -1  /* invalid argument (reference: ArgumentError / @assert) */
#define SGS_ERR_CUDA     -2  /* CUDA runtime error */
#define SGS_ERR_OOM      -3  /* device allocation failed */
#define SGS_ERR_TIMEOUT  -4  /* a bounded device wait ran out */
#define SGS_ERR_NUMERIC  -5  /* non-finite result */
#define SGS_ERR_STATE    -6  /* call out of order (e.g. simulate before prepare) */
#define SGS_ERR_NODEVICE -7  /* no CUDA device / library built without one */

/* ---- variogram families (GeoStatsFunctions, practical-range convention) - */
#define SGS_SPHERICAL    1
#define SGS_EXPONENTIAL  2
#define SGS_GAUSSIAN     3

/* ---- neighbourhood kinds (SEQSIM `neighborhood` option, seqsim.jl:171-177,221-227) */
#define SGS_SEARCH_RANGE   0  /* :range  -> isotropic ball of radius max(variogram ranges) */
#define SGS_SEARCH_BALL    1  /* MetricBall(radii, rotation)                               */
#define SGS_SEARCH_NEAREST 2  /* nothing -> k nearest with the Euclidean distance          */

/* ---- solve precision ---------------------------------------------------- */
#define SGS_PREC_FP64        0  /* FP64 LHS, Cholesky, weights and sweep          */
#define SGS_PREC_FP32_REFINE 1  /* FP32 LHS + Cholesky, FP64 refinement residual and
                                   variance, FP32 weights and sweep                 */

/* ---- sgs_problem.flags --------------------------------------------------- */
/* The default sweep is one persistent dataflow launch: warps take nodes in
   level order and wait (bounded) on per-node flags of their neighbours, with
   no barrier between levels.  These flags select the alternatives: */
#define SGS_FLAG_ONE_LAUNCH_SWEEP 1  /* one cooperative launch with a grid barrier
                                        between dependency levels */
#define SGS_FLAG_LEVEL_SWEEP      2  /* one launch per dependency level */
#define SGS_FLAG_NN_FP32          4  /* warm-start inference in FP32 on the CUDA cores
                                        instead of BF16 on the tensor cores */
#define SGS_FLAG_OUTPUT_STAGED    8  /* sgs_plan_simulate into page-locked memory:
                                        transpose chunks into device buffers and
                                        move them with the copy engines (overlapped),
                                        instead of kernels writing host memory */

/* ---- per-node solve status (sgs_plan_weights) --------------------------- */
#define SGS_NODE_KRIGED       0  /* conditional draw from simple kriging          */
#define SGS_NODE_PRIOR_NMIN   1  /* fewer than minneighbors neighbours: prior     */
#define SGS_NODE_PRIOR_SINGULAR 2/* Cholesky pivot <= 1e-10*sill: prior          */

/* Variogram gamma(h) = nugget*(h>0) + (sill-nugget)*f(h) with the
 * normalized anisotropic lag h = |diag(1/ranges) * R^T * lag|;
 * covariance C = sill - gamma (src/utils.jl:50-62). */
/* Nested models (GeoStatsFunctions' NestedVariogram, gamma = gamma_1 + ... +
 * gamma_m) are `variogram` plus sgs_problem.structures: every structure has its
 * own type, sill, nugget, ranges and rotation, and the model's sill, nugget
 * and range are the sums and the largest range (seqsim.jl:52 takes any
 * GeoStatsFunctions function as the process's func). */
#define SGS_MAX_STRUCTURES 4

typedef struct sgs_variogram {
    int32_t type;          /* SGS_SPHERICAL / SGS_EXPONENTIAL / SGS_GAUSSIAN */
    int32_t reserved;
    double  sill;
    double  nugget;
    double  ranges[3];     /* principal ranges (unused trailing entries ignored in 2D) */
    double  rotation[9];   /* column-major dim x dim (stride 3); column j = principal axis j */
} sgs_variogram;

/* Search neighbourhood for SGS_SEARCH_BALL: the ellipsoid
 * |diag(1/radii) * R^T * lag| <= 1.  Radii all equal with R = I is the
 * isotropic ball |lag| <= radius. */
typedef struct sgs_ball {
    double radii[3];
    double rotation[9];    /* same layout as sgs_variogram.rotation */
} sgs_ball;

/* Problem description: GaussianProcess(variogram, mean) on a CartesianGrid,
 * conditioned on point data, simulated with SEQSIM options. */
typedef struct sgs_problem {
    int32_t dim;              /* 2 or 3 */
    int32_t dims[3];          /* cells per axis */
    double  origin[3];        /* grid minimum corner */
    double  spacing[3];       /* cell sizes */
    int64_t ndata;            /* D >= 0 conditioning points */
    const double* data_coords;/* D x dim, row-major (point-major) */
    const double* data_values;/* D */
    sgs_variogram variogram;
    double  mean;             /* process mean mu (GaussianProcess.mean) */
    int32_t minneighbors;     /* SEQSIM.minneighbors (clamped as seqsim.jl:202-208) */
    int32_t maxneighbors;     /* SEQSIM.maxneighbors (<= 64 on the GPU) */
    int32_t search;           /* SGS_SEARCH_* */
    int32_t precision;        /* SGS_PREC_* */
    sgs_ball ball;            /* used when search == SGS_SEARCH_BALL */
    const int32_t* path;      /* N grid node ids, a permutation; NULL = LinearPath */
    int32_t refine_steps;     /* refinement steps for SGS_PREC_FP32_REFINE (0..4, default 2) */
    int32_t warm_start;       /* 1 = learned warm start of the kriging weights */
    int32_t device;           /* CUDA device ordinal */
    int32_t flags;            /* 0 or SGS_FLAG_* */
    int32_t nstructures;      /* further nested structures (0 .. SGS_MAX_STRUCTURES-1) */
    int32_t reserved2;
    const sgs_variogram* structures; /* nstructures structures added to `variogram` */
} sgs_problem;

typedef struct sgs_plan sgs_plan;

typedef struct sgs_info {
    int64_t nnodes;           /* N */
    int64_t ndata;            /* D */
    int32_t maxneighbors;     /* after clamping */
    int32_t minneighbors;
    int32_t nlevels;          /* depth of the path's dependency DAG */
    int32_t template_size;    /* grid offsets inside the search neighbourhood */
    int64_t n_prior;          /* nodes drawn from the prior */
    int64_t n_fp64_fallback;  /* FP32 systems re-solved in FP64 */
    int64_t n_warm_accepted;  /* systems whose learned warm start was accepted */
    double  ms_search, ms_levels, ms_solve, ms_sweep;  /* last device timings (CUDA events) */
    int64_t launches;         /* kernels launched by this plan so far */
    int64_t h2d_bytes;        /* bytes copied host -> device by this plan so far */
    int64_t d2h_bytes;        /* bytes copied device -> host by this plan so far */
    int64_t sum_grid_neighbors; /* sum over nodes of grid neighbours used by the sweep */
    double  weight_l1_max;    /* largest sum of |weights| of a node's grid neighbours:
                                 how much the sweep amplifies the rounding of stored
                                 values (nugget-free Gaussian models reach ~100) */
    int32_t values_fp64;      /* 1: the sweep keeps FP64 values (SGS_PREC_FP64, or
                                 SGS_PREC_FP32_REFINE with weight_l1_max above
                                 SGS_FP32_VALUE_L1_LIMIT); sgs_plan_simulate_device
                                 then takes double arrays                          */
    int32_t reserved;
    int64_t search_grid_candidates; /* candidates the last search examined, each one
                                       path-rank read: earlier path nodes tested by
                                       the first ranks, template offsets inside the grid */
    int64_t search_data_candidates; /* data bucket entries it screened */
} sgs_info;

/* SGS_PREC_FP32_REFINE stores values in FP32 while weight_l1_max stays below
 * this; above it the rounding of FP32 values, amplified by the weights, could
 * exceed 1e-6 relative, so the sweep keeps FP64 values (same weights). */
#define SGS_FP32_VALUE_L1_LIMIT 4.0

/* Validate the problem, copy geometry, data and path to the device.
 * Replaces preprocess(rng, process, ::SEQSIM, init, domain, data),
 * src/simulation/field/seqsim.jl:50-70 (_scale :162-189, _search :195-230,
 * _probmodel :277-290, _initialization :267-271). */
int sgs_plan_create(const sgs_problem* problem, sgs_plan** plan);

/* Run the realization-independent work on the device: neighbour search
 * (kernel a), dependency levels, simple-kriging build + solve (kernel b).
 * Replaces the per-node search!/fit/status/predictprob calls of the
 * randsingle loop, seqsim.jl:98-131, hoisted out of the realization loop. */
int sgs_plan_prepare(sgs_plan* plan);

/* Simulate nreals realizations (kernel c) and copy them to out (nreals x N,
 * realization-major, double).  z: standard-normal draws, nreals x N
 * realization-major (z[r*N+g] is the draw of node g in realization r), or
 * NULL to draw them on the device from `seed` (Philox4x32-10 + Box-Muller).
 * Replaces randsingle, seqsim.jl:72-156 (_draw! :335-340, prior :109-111,
 * output assembly :141-155), for a block of realizations. */
int sgs_plan_simulate(sgs_plan* plan, int32_t nreals, const double* z,
                      uint64_t seed, double* out);

/* Device-resident variant of sgs_plan_simulate: z_dev (node-major
 * [N][nreals rounded up to a multiple of 4], float when sgs_info.values_fp64
 * is 0 — SGS_PREC_FP32_REFINE with moderate weights — and double when it is
 * 1, or NULL for seeded draws) and vals_dev (node-major, same shape and type,
 * centred values v - mean) are device pointers; stream is a cudaStream_t
 * (NULL = the plan's stream).  Same reference counterpart as
 * sgs_plan_simulate. */
int sgs_plan_simulate_device(sgs_plan* plan, int32_t nreals, const void* z_dev,
                             uint64_t seed, void* vals_dev, void* stream);

/* Neighbour table: idx (N x maxneighbors, node-major, -1 padded) holds, for
 * each grid node, its neighbours in nearest-first order, and count (N) their
 * number.  Replaces search!(neighbors, center, searcher, mask=simulated),
 * seqsim.jl:107.  Either pointer may be NULL. */
int sgs_plan_neighbors(sgs_plan* plan, int32_t* idx, int32_t* count);

/* Kriging results per node: weights (N x maxneighbors, aligned with the
 * neighbour table, 0 padded), sigma (N, conditional standard deviation),
 * status (N, SGS_NODE_*).  Replaces GeoStatsModels.fit + status +
 * predictprob, seqsim.jl:124-131,302-304.  Any pointer may be NULL. */
int sgs_plan_weights(sgs_plan* plan, double* weights, double* sigma, int32_t* status);

/* Dependency level of every node (N) in the path's DAG; nlevels may be NULL.
 * Replaces the sequential visiting order of `for ind in traverse(domain,
 * path)`, seqsim.jl:98. */
int sgs_plan_levels(sgs_plan* plan, int32_t* level, int32_t* nlevels);

/* Plan statistics and last device timings. */
int sgs_plan_info(const sgs_plan* plan, sgs_info* info);

/* Release all device memory of the plan (waits for the device first, as a
 * synchronous free does).  NULL is ignored.  The memory returns to the
 * library's pool for the device, where the next plan or batch reuses it;
 * sgs_trim_memory hands it back to the device. */
void sgs_plan_destroy(sgs_plan* plan);

/* Return the device memory the library keeps for reuse (freed by destroyed
 * plans and batches, or between simulate calls) to `device`, or to every
 * device when device < 0.  Memory of live plans is not touched. */
int sgs_trim_memory(int32_t device);

/* Message of the last failure on this plan, or of the last failed
 * sgs_plan_create on this thread when plan is NULL. */
const char* sgs_last_error(const sgs_plan* plan);

/* Library version string. */
const char* sgs_version(void);

/* ---- learned warm start -------------------------------------------------
 * A small permutation-invariant network predicts each system's kriging
 * weights from per-neighbour features (normalized anisotropic lag to the
 * node, its norm, covariance / sill, nugget / sill, variogram family).  With
 * problem.warm_start = 1 and a network set on the plan, the FP32 solve starts
 * its refinement from the prediction instead of the FP32 solution and
 * accepts it only when the refined residual meets the usual tolerance; other
 * systems take the FP64 path.  No counterpart in the reference (it is part
 * of this method's GPU design); the training kernels run on device buffers
 * owned by the caller. */
#define SGS_NN_FEATURES 8
#define SGS_NN_PARAMS   2401

/* Features of every system (device out: N x maxneighbors x SGS_NN_FEATURES
 * floats, node-indexed, zero for missing neighbours). */
int sgs_plan_features_device(sgs_plan* plan, float* feat_dev, void* stream);
/* Set (or clear with NULL) the network used by the warm start: host array of
 * SGS_NN_PARAMS floats.  Takes effect at the next sgs_plan_prepare. */
int sgs_plan_set_network(sgs_plan* plan, const float* params);
/* Network forward pass: feat (nsys x k x F), count (nsys) -> pred (nsys x k). */
int sgs_nn_forward(const float* params, const float* feat, const int32_t* count, int64_t nsys, int32_t k,
                   float* pred, void* stream);
/* Adds the batch's mean-squared-error loss to *loss and its gradient to grad
 * (SGS_NN_PARAMS floats, zeroed by the caller), all device pointers. */
int sgs_nn_backward(const float* params, const float* feat, const int32_t* count, const float* target,
                    int64_t nsys, int32_t k, float* grad, float* loss, void* stream);
/* One Adam step (beta 0.9 / 0.999) on device arrays of SGS_NN_PARAMS floats,
 * with gradient scale `scale` (e.g. 1 / batch systems); step counts from 1. */
int sgs_nn_adam(float* params, const float* grad, float* m, float* v, int32_t step, float lr, float scale,
                void* stream);

/* Writes the warm-start network's predicted weights of every system of a
 * prepared plan (device array of nnodes x maxneighbors floats, zero past each
 * node's neighbour count): BF16 inference with FP32 accumulation on the
 * tensor cores (tensor_cores = 1) or FP32 on the CUDA cores (0).  No
 * counterpart in the reference.  Returns when the predictions are complete. */
int sgs_plan_predict_device(sgs_plan* plan, float* out_dev, int32_t tensor_cores, void* stream);

/* ---- sweep configuration and autotuning --------------------------------- */
#define SGS_SWEEP_FLOW        0  /* one persistent dataflow launch (default)      */
#define SGS_SWEEP_COOPERATIVE 1  /* one cooperative launch, grid barrier per level */
#define SGS_SWEEP_LEVELS      2  /* one launch per dependency level                */

typedef struct sgs_sweep_config {
    int32_t mode;             /* SGS_SWEEP_*                                         */
    int32_t chunk;            /* flow: work items a warp takes per ticket            */
    int32_t blocks_per_sm;    /* flow: resident 256-thread blocks per SM (0 = max)   */
    int32_t lanes_g;          /* flow: chunks of 4 realizations per lane, 1 or 2;
                                 levels (FP32, more than 64 realizations, a
                                 multiple of 4 * lanes_g): 2 or 4 chunks per
                                 thread                                        */
    int32_t lanes_w;          /* flow: lanes per slice of the neighbour list, a power
                                 of two <= 32 (0 = the row's chunks, at most 32);
                                 32 / lanes_w slices split the neighbour list and a
                                 row is cut into pieces of lanes_w * lanes_g chunks,
                                 each a separate work item                          */
    int32_t level_lo;         /* flow: dependency levels [level_lo, level_hi) are   */
    int32_t level_hi;         /* swept by per-level launches, the levels before and
                                 after them by one dataflow launch each             */
    int32_t tight;            /* flow: 1 = the kernel variant compiled for higher
                                 residency (register cap)                           */
    int32_t split_nodes;      /* levels (FP32, rows of a multiple of 8 realizations):
                                 levels of fewer nodes than this take one block per
                                 node, its 8 warps splitting the neighbour list
                                 (0 = never)                                       */
    float   ms;               /* sgs_plan_tune_sweep: measured time of this config   */
} sgs_sweep_config;

/* Sets how sgs_plan_simulate* run the sweep.  No counterpart in the reference
 * (its draw loop is serial, seqsim.jl:98-138); results are the same for every
 * configuration up to the order of FP32 roundings. */
int sgs_plan_set_sweep(sgs_plan* plan, const sgs_sweep_config* config);
/* Times the candidate sweep configurations for `nreals` realizations on the
 * prepared plan (each on a scratch value array, after one warm-up run), keeps
 * the fastest for later sgs_plan_simulate* calls and returns it in *chosen
 * (may be NULL).  tried (may be NULL) receives up to max_tried of the
 * configurations timed, and *ntried (may be NULL) their count. */
int sgs_plan_tune_sweep(sgs_plan* plan, int32_t nreals, sgs_sweep_config* chosen, sgs_sweep_config* tried,
                        int32_t max_tried, int32_t* ntried);

/* ---- batches of independent domains -------------------------------------
 * Many independent problems (each its own grid, data, variogram, mean,
 * neighbourhood, maxneighbors and path; one sgs_problem per domain) prepared
 * and simulated together: every phase is one launch over all domains' nodes
 * (search, dependency levels, level order, size bins), the kriging systems
 * are solved in size classes (at most 8, 16, 32, 48, 64 neighbours: one
 * launch each), and the sweep is one persistent dataflow launch.  The
 * prepare sequence and the seeded sweep are captured in CUDA graphs and
 * replayed by later calls.  Replaces a loop of rand(rng, process_d, domain_d,
 * nreals; data = data_d, method = SEQSIM(...)) calls over the domains
 * (src/simulation/field.jl:73-124), each of which runs preprocess /
 * randsingle (seqsim.jl:50-156) on its own.
 *
 * All domains use the same device and precision; warm_start and flags must
 * be 0.  Global node ids number the domains' grid nodes one after another:
 * domain d owns ids [first_d, first_d + N_d) (sgs_batch_domain).  Host
 * arrays of realizations are concatenated by domain: domain d's block is
 * nreals x N_d realization-major and starts at element nreals * first_d. */
typedef struct sgs_batch sgs_batch;

typedef struct sgs_batch_info {
    int32_t ndomains;
    int32_t nlevels;            /* deepest dependency level + 1 over all domains  */
    int64_t nnodes;             /* grid nodes of all domains                       */
    int64_t ndata;              /* conditioning points of all domains              */
    int64_t n_prior;            /* nodes drawn from the prior                      */
    int64_t n_fp64_fallback;    /* FP32 systems re-solved in FP64                  */
    int64_t sum_grid_neighbors; /* grid neighbours used by the sweep, all nodes    */
    int64_t bin_systems[5];     /* systems per size class (<= 8/16/32/48/64 nbrs)  */
    double  ms_search, ms_levels, ms_solve; /* phases of the last prepare          */
    double  ms_prepare;         /* the last prepare as a whole                     */
    double  ms_sweep;           /* the last sweep                                  */
    int64_t launches;           /* kernels launched, graph nodes included          */
    int64_t graph_launches;     /* CUDA graph launches                             */
    int64_t h2d_bytes, d2h_bytes;
    int64_t device_bytes;       /* device memory held by the batch                 */
    double  weight_l1_max;      /* as sgs_info: largest sum of |grid weights|       */
    int32_t values_fp64;        /* 1: the value array has FP64 rows (Rp doubles per
                                   node; sgs_batch_simulate_device takes double
                                   arrays); the rows of domains that keep FP32
                                   values then hold Rp floats in their first half
                                   (sgs_batch_domain_values_fp64)                  */
    int32_t domains_fp64;       /* domains whose values are FP64: with
                                   SGS_PREC_FP32_REFINE, only those whose weights
                                   exceed SGS_FP32_VALUE_L1_LIMIT                   */
    int64_t sum_grid_neighbors_fp64; /* the part of sum_grid_neighbors that belongs
                                   to the nodes of FP64-value domains              */
} sgs_batch_info;

/* Validate every problem (the first invalid one is named in the error) and
 * upload geometry, data, paths and search templates. */
int sgs_batch_create(const sgs_problem* problems, int32_t ndomains, sgs_batch** batch);
/* Neighbour search, levels, level order, size bins and kriging solves for
 * all domains.  The first call sizes the tables, then captures the sequence
 * in a CUDA graph; every call launches that graph. */
int sgs_batch_prepare(sgs_batch* batch);
/* Simulate nreals realizations of every domain into out (host, concatenated
 * by domain as above).  z: standard normals in the same layout, or NULL for
 * draws from `seed` (Philox4x32-10 keyed by seed, counter = global node id
 * and realization / 4). */
int sgs_batch_simulate(sgs_batch* batch, int32_t nreals, const double* z, uint64_t seed, double* out);
/* Seeded sweep into vals_dev: device array [nnodes][nreals rounded up to a
 * multiple of 4] of centred values (v - mean of the node's domain), float when
 * sgs_batch_info.values_fp64 is 0, double when it is 1, rows by global id.
 * Captured in a CUDA graph per (nreals, vals_dev, sweep configuration) and
 * replayed; stream is a cudaStream_t (NULL = the batch's stream). */
int sgs_batch_simulate_device(sgs_batch* batch, int32_t nreals, uint64_t seed, void* vals_dev, void* stream);
/* First global node id and node count of domain d. */
int sgs_batch_domain(const sgs_batch* batch, int32_t domain, int64_t* first, int64_t* nnodes);
/* Value precision of domain d after prepare: *fp64 = 1 when its values are
 * FP64 (SGS_PREC_FP64, or weights above SGS_FP32_VALUE_L1_LIMIT), 0 when they
 * are FP32.  The precision is decided per domain, so one domain whose
 * weights amplify rounding does not double the value traffic of the others.
 * No counterpart in the reference (its values are always FP64). */
int sgs_batch_domain_values_fp64(const sgs_batch* batch, int32_t d, int32_t* fp64);
/* Neighbour rows of domain d, as sgs_plan_neighbors (N_d x maxneighbors_d,
 * local augmented ids: grid nodes 0..N_d-1, data N_d..). */
int sgs_batch_neighbors(sgs_batch* batch, int32_t domain, int32_t* idx, int32_t* count);
/* Kriging weights, sigma and status of domain d, as sgs_plan_weights (the
 * weights are recomputed for the whole batch with an export). */
int sgs_batch_weights(sgs_batch* batch, int32_t domain, double* weights, double* sigma, int32_t* status);
/* Sweep configuration (mode must be SGS_SWEEP_FLOW; level_lo/level_hi are
 * ignored) and its autotuner over the dataflow mappings, as for plans. */
int sgs_batch_set_sweep(sgs_batch* batch, const sgs_sweep_config* config);
int sgs_batch_tune_sweep(sgs_batch* batch, int32_t nreals, sgs_sweep_config* chosen, sgs_sweep_config* tried,
                         int32_t max_tried, int32_t* ntried);
int sgs_batch_info_get(const sgs_batch* batch, sgs_batch_info* info);
/* Release all device memory and graphs.  NULL is ignored. */
void sgs_batch_destroy(sgs_batch* batch);
/* Message of the last failure on this batch, or of the last failed
 * sgs_batch_create on this thread when batch is NULL. */
const char* sgs_batch_last_error(const sgs_batch* batch);

/* Indicator simulation with full simple cokriging, for an indicator
 * covariance given as a linear model of coregionalization:
 * C_ab(h) = sum_s coef[s][a][b] C_s(h), C_s = sill_s - gamma_s over the
 * S = 1 + nstructures structures of the plan's variogram (coef: S x ncat x
 * ncat, row-major, symmetric).  Replaces Kriging(func, prob) with a
 * multivariate func in the indicator branches of SEQSIM
 * (src/simulation/field/seqsim.jl:292-310; IndicatorProcess(func, prob),
 * src/processes/field/indicator.jl:30-47), where the structures' ranges
 * differ and every category's weights are not those of one correlogram.
 * Each node solves one (n ncat x n ncat) system in FP64: maxneighbors x
 * ncat must be at most 64.  prob, data_cat and the draws as
 * sgs_plan_set_indicator / sgs_plan_simulate_indicator; prepare again after
 * setting it. */
int sgs_plan_set_indicator_cokriging(sgs_plan* plan, int32_t ncat, const double* prob, const int32_t* data_cat,
                                     const double* coef);
/* ---- sequential indicator simulation ------------------------------------
 * An IndicatorProcess(func, prob) simulated with SEQSIM
 * (src/processes/field/indicator.jl, src/simulation/field/seqsim.jl:247-261
 * one-hot data, :292-310 Kriging(func, prob) with a Categorical prior and
 * conditional, :342-347 categorical draw) for a separable indicator
 * covariance C_ab(h) = A_ab rho(h) — including the proportional transiogram
 * t_ab(h) = p_b + (delta_ab - p_b) rho(h) — where rho is the plan's
 * variogram model taken as the categories' common correlogram: every
 * category's simple cokriging weights are then rho's simple kriging weights,
 * and p_l = prob_l + sum_i w_i (I_l(x_i) - prob_l) is clamped to [0, 1],
 * normalized, and drawn from by the inverse cdf at a uniform.
 * sgs_plan_set_indicator (before sgs_plan_prepare): ncat categories (2..8),
 * prior probabilities prob (normalized here), data categories data_cat
 * (problem->ndata values in 0..ncat-1; the problem's data_values are not
 * used).  sgs_plan_simulate_indicator: out = nreals x N categories
 * (realization-major, int32); u = nreals x N uniforms in (0, 1) or NULL for
 * Philox4x32-10 uniforms from `seed`. */
#define SGS_IND_MAX_CATEGORIES 8
int sgs_plan_set_indicator(sgs_plan* plan, int32_t ncat, const double* prob, const int32_t* data_cat);
int sgs_plan_simulate_indicator(sgs_plan* plan, int32_t nreals, const double* u, uint64_t seed, int32_t* out);

/* ---- multivariate Gaussian simulation ------------------------------------
 * A GaussianProcess(func, mean) whose func has nvars > 1 variables, simulated
 * with SEQSIM (src/processes/field/gaussian.jl:22-35; seqsim.jl:277-290
 * Kriging(func, mean) with the prior MvNormal(mean, sill(func)), :302-304
 * predictprob's MvNormal conditional, :335-340 the draw of all variables of a
 * node at once).  func is a linear model of coregionalization over the
 * S = 1 + nstructures structures of the plan's variogram:
 * C_ab(h) = sum_s coef[s][a][b] C_s(h), C_s = sill_s - gamma_s (coef:
 * S x nvars x nvars, row-major, exactly symmetric).  Each node solves the
 * simple cokriging system of its n neighbours' nvars values (maxneighbors x
 * nvars at most 64) in FP64 with Cholesky (a pivot not above 1e-10 x the
 * largest variance: the node draws from the prior), and draws
 *   v = mu^ + F z,  mu^_t = mean_t + sum_i sum_a Lambda[(i, a), t] (v_a(x_i) - mean_a),
 * F the lower Cholesky factor of the conditional covariance C(0) - c' Lambda
 * (of C(0) for a prior node; a pivot not above the same threshold gives a zero
 * column, so a node on a datum draws no noise).
 * sgs_plan_set_multivariate (before sgs_plan_prepare): nvars in 1..8 (1 gives
 * simple kriging with the one structure set as univariate SEQSIM), the means,
 * coef, and data_values = problem->ndata x nvars values (the problem's own
 * data_values are not used).  sgs_plan_simulate_multivariate: out = nreals x
 * nvars x N values (realization-major, then variable, then node); z in the
 * same layout, or NULL for Philox4x32-10 normals from `seed` (those of
 * variable a of node g are the single-variable normals of node a*N + g). */
#define SGS_MV_MAX_VARIABLES 8
int sgs_plan_set_multivariate(sgs_plan* plan, int32_t nvars, const double* mean, const double* coef,
                              const double* data_values);
int sgs_plan_simulate_multivariate(sgs_plan* plan, int32_t nreals, const double* z, uint64_t seed, double* out);

/* ---- posterior mean (simple kriging from the data) ---------------------
 * Mean and variance of the process at every grid node conditioned on the
 * data alone: the reference's mean(process, domain; data) for a
 * GaussianProcess, which is simple kriging (posteriormean,
 * src/expectation/field/gaussian.jl:21-25, GeoStatsModels.fitpredict with
 * Kriging(func, mean)).  Each node takes its problem->maxneighbors nearest
 * data inside problem->search's neighbourhood (SGS_SEARCH_NEAREST: no
 * radius; the path is not used), mean = mu + w'(d - mu), var = C(0) - w'c.
 * Nodes with fewer than minneighbors data, or whose system is singular
 * (pivot <= 1e-10 sill), get NaN (the reference's `missing`); with no data
 * at all every node gets the prior: mu and the sill.  mean and var are host
 * arrays of N (var may be NULL).  Errors: sgs_last_error(NULL). */
int sgs_krige(const sgs_problem* problem, double* mean, double* var);

/* ---- ensemble statistics on the device ----------------------------------
 * Per-node statistics over nreals realizations held on the device in the
 * node-major layout of sgs_plan_simulate_device / sgs_batch_simulate_device
 * (rows of nreals values, row_stride elements apart; float when precision is
 * SGS_PREC_FP32_REFINE, double for SGS_PREC_FP64); `offset` is added to every
 * value (the process mean, as those values are centred).  Replaces the
 * Ensemble statistics of src/ensembles.jl:42-52 (mean, var with the n - 1
 * divisor, cdf, ccdf, quantile with linear interpolation between order
 * statistics).  Outputs are device arrays: mean / var (N; either may be
 * NULL), cdf (N x nx: fraction of values <= x[i], or > x[i] with complement
 * = 1), quantile (N x np, p[i] in [0, 1], nreals <= 1024).  x and p are
 * host arrays.  Nothing is allocated; stream is a cudaStream_t (NULL = the
 * default stream) and the calls return after launching.  Errors:
 * sgs_last_error(NULL). */
int sgs_ensemble_stats(const void* vals, int32_t precision, int64_t nnodes, int32_t nreals, int32_t row_stride,
                       double offset, double* mean, double* var, void* stream);
int sgs_ensemble_cdf(const void* vals, int32_t precision, int64_t nnodes, int32_t nreals, int32_t row_stride,
                     double offset, const double* x, int32_t nx, int32_t complement, double* out, void* stream);
int sgs_ensemble_quantile(const void* vals, int32_t precision, int64_t nnodes, int32_t nreals, int32_t row_stride,
                          double offset, const double* p, int32_t np, double* out, void* stream);

/* ---- allocation-free schedule ------------------------------------------ */
#define SGS_NOALLOC_MAX_LEVELS 262144

/* Dependency levels and the level-ordered node list of a neighbour table,
 * without allocating memory.  No counterpart in the reference: it is the
 * scheduling step of sgs_plan_prepare, offered on its own for callers that
 * cannot let a library allocate device memory (an application whose memory
 * pool already holds the device, or a loop where an allocation's implicit
 * device synchronization is not acceptable).  All pointers except nlevels
 * are device pointers owned by the caller: path (N), nbr (N x maxneighbors,
 * node-major, -1 padded, ids >= N are data), count (N); outputs level (N),
 * order (N, nodes grouped by level), offsets (nlevels + 1 entries, at most
 * offsets_capacity), and *nlevels on the host.  The inputs are checked on
 * the device first: path must be a permutation of 0..N-1, every count in
 * [0, maxneighbors], the first count ids of a row non-negative, and every
 * grid neighbour (id < N) of a node must come earlier in the path than the
 * node; otherwise SGS_ERR_ARG, with nothing read or written out of bounds.
 * stream is a cudaStream_t (NULL = default stream); the call synchronizes
 * it and returns when the results are complete.  Working memory is one
 * file-scope device array per device (about 2 MB) that stays until the
 * process exits: schedules with more than SGS_NOALLOC_MAX_LEVELS levels are
 * rejected with SGS_ERR_ARG.  Its device address is looked up on every call,
 * in the current context.  Calls on one device share the array: calls that
 * overlap on the GPU race and must be serialized by the caller.  Errors are
 * reported by sgs_last_error(NULL). */
int sgs_schedule_noalloc(const int32_t* path, const int32_t* nbr, const int32_t* count, int64_t nnodes,
                         int32_t maxneighbors, int32_t* level, int32_t* order, int32_t* offsets,
                         int32_t offsets_capacity, int32_t* nlevels, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GEOSGS_H */

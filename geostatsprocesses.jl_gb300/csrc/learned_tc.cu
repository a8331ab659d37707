// learned_tc.cu — inference of the warm-start network (learned.cu) on the
// 5th-generation tensor cores: BF16 operands in shared memory, FP32
// accumulators in tensor memory (TMEM), tcgen05.mma issued by one thread.
//
// A tile is 128 neighbour rows (one TMEM lane each): 4 systems of 32 rows
// when maxneighbors <= 32, 2 systems of 64 rows (padded) up to 64.  Per tile
//   layer 1   D1[128 x 32] = F[128 x 16] . W1^T[16 x 32]   (8 features, K
//             padded to 16 with zeros), then h = relu(D1 + b1) on the CUDA
//             cores (rows past a system's neighbour count are zeroed)
//   pooling   g_s = mean of h over system s's rows (warp reduce-scatter of
//             the column sums); u_s = W2b g_s + b2
//   layer 2   D2[128 x 32] = H[128 x 32] . W2a^T[32 x 32]   (two K = 16 steps,
//             into the TMEM columns D1 held: 32 columns per CTA)
//   output    y = w3 . relu(D2 + u_s) + b3 per row
// The 128 threads of the CTA own one row each: thread r computes row r's
// features, and warp w reads TMEM lanes [32w, 32w + 32) with tcgen05.ld.
//
// Operand layout in shared memory: K-major, no swizzle, in 8-row x 16-byte
// core matrices (element (r, k) at (r/8)*SBO + (k/8)*128 + (r%8)*16 +
// (k%8)*2 bytes): LBO = 128 bytes between core matrices along K, SBO between
// 8-row groups along M (A) or N (B).
//
// Every wait on the MMA completion barrier is bounded (2 s of wall-clock
// time): on expiry the kernel records an error, waits once more (bounded)
// for its MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>

#include "common.cuh"

namespace sgs {

namespace {

constexpr int TF = 8, TH = 32;  // features, hidden width (learned.cu)
constexpr int P_W1 = 0, P_B1 = TH * TF, P_W2A = P_B1 + TH, P_W2B = P_W2A + TH * TH, P_B2 = P_W2B + TH * TH,
              P_W3 = P_B2 + TH, P_B3 = P_W3 + TH;
constexpr int ROWS = 128;
constexpr int THREADS = 128;
constexpr uint32_t TMEM_COLS = 32;  // D1, then D2 in the same columns

// shared memory layout (bytes)
constexpr int SBO_A1 = 256, SBO_A2 = 512, SBO_B1 = 256, SBO_B2 = 512;
constexpr int OFF_A1 = 0;                        // 128 x 16 bf16: 4096
constexpr int OFF_A2 = OFF_A1 + 4096;            // 128 x 32 bf16: 8192
constexpr int OFF_B1 = OFF_A2 + 8192;            // 32 x 16 bf16: 1024
constexpr int OFF_B2 = OFF_B1 + 1024;            // 32 x 32 bf16: 2048
// FP32 parameters used on the CUDA cores: b1, W2b, b2, w3, b3
constexpr int Q_B1 = 0, Q_W2B = Q_B1 + TH, Q_B2 = Q_W2B + TH * TH, Q_W3 = Q_B2 + TH, Q_B3 = Q_W3 + TH,
              Q_N = Q_B3 + 1;
constexpr int OFF_P = OFF_B2 + 2048;
constexpr int OFF_GX = OFF_P + ((Q_N * 4 + 127) / 128) * 128;  // [4 warps][32] partial column sums
constexpr int OFF_U = OFF_GX + 4 * TH * 4;             // [4][32] W2b g + b2
constexpr int OFF_N = OFF_U + 4 * TH * 4;              // [4] neighbour counts
constexpr int OFF_BAR = OFF_N + 16;                    // mbarrier (8 bytes)
constexpr int OFF_TMEM = OFF_BAR + 8;                  // TMEM base address
constexpr int SMEM_BYTES = OFF_TMEM + 8;

// Sum of v[0..31] over the 32 lanes of the warp, reduce-scattered: lane l
// returns the sum of element l (31 shuffles instead of a shared-memory
// transpose).
__device__ __forceinline__ float warp_colsum(float* v, int lane) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const float keep = up ? v[i + o] : v[i];
            const float send = up ? v[i] : v[i + o];
            v[i] = keep + __shfl_xor_sync(FULL_MASK, send, o);
        }
    }
    return v[0];
}

__device__ __forceinline__ uint32_t cm_off(int r, int k, int sbo) {
    return (uint32_t)((r >> 3) * sbo + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// tcgen05 shared-memory matrix descriptor: start, LBO, SBO (>> 4), version 1
// (bits 46-47), no swizzle (bits 61-63 = 0), base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// bounded wait for the barrier phase with the given parity
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    uint64_t t0 = 0;
    // bounded by 2 s of elapsed time and by a count of polls
    for (uint32_t polls = 0; polls < (1u << 26); ++polls) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        const uint64_t t = now_ns();
        if (t0 == 0) t0 = t;
        if (t - t0 > 2000000000ull) return false;
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// 8 BF16 values (one 16-byte core-matrix row segment)
__device__ __forceinline__ void st_row8(unsigned char* base, uint32_t off, const float* v) {
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(base + off) = q;
}

// Features of one neighbour in FP32 (the FP64 definitions of learned.cu,
// evaluated in single precision: the result is rounded to BF16 anyway).
__device__ __forceinline__ void features_f32(const GridDev& G, const VarioDev& v, const float* Rf, const float* ir,
                                             int id, const int* cp, const double* data_xyz, float* f) {
    float h[3] = {0.f, 0.f, 0.f};
    if (id >= G.N) {
        const double* x = data_xyz + 3 * (int64_t)(id - G.N);
        for (int j = 0; j < G.dim; ++j) h[j] = (float)(centroid(G, j, cp[j]) - x[j]);
    } else {
        int cq[3];
        cell_of(G, id, cq[0], cq[1], cq[2]);
        for (int j = 0; j < G.dim; ++j) h[j] = (float)(cp[j] - cq[j]) * (float)G.spacing[j];
    }
    float s = 0.f;
    for (int j = 0; j < 3; ++j) {
        float t = 0.f;
        if (j < G.dim) {
            t = Rf[0 + 3 * j] * h[0] + Rf[1 + 3 * j] * h[1] + (G.dim == 3 ? Rf[2 + 3 * j] * h[2] : 0.f);
            t *= ir[j];
        }
        f[j] = t;
        s += t * t;
    }
    const float hn = sqrtf(s);
    f[3] = hn;
    const float sill = (float)v.sill, nug = (float)v.nugget;
    float c = 1.0f;
    if (v.ns > 1) {  // a nested model: its covariance summed over the structures
        c = (float)(cov_fp64(v, G.dim, (double)h[0], (double)h[1], (double)h[2]) / v.sill);
    } else if (hn > 0.f) {
        float fr;
        if (v.type == 1) fr = hn < 1.f ? 1.5f * hn - 0.5f * hn * hn * hn : 1.f;
        else if (v.type == 2) fr = 1.f - __expf(-3.f * hn);
        else fr = 1.f - __expf(-3.f * s);
        c = (sill - (nug + (sill - nug) * fr)) / sill;
    }
    f[4] = c;
    f[5] = nug / sill;
    f[6] = v.type == 2 ? 1.f : 0.f;
    f[7] = v.type == 3 ? 1.f : 0.f;
}

}  // namespace

__global__ void __launch_bounds__(THREADS) nn_predict_tc_kernel(const GridDev G, const VarioDev v,
                                                               const int32_t* __restrict__ nbr,
                                                               const int32_t* __restrict__ cnt, int k,
                                                               const double* __restrict__ data_xyz,
                                                               const float* __restrict__ params,
                                                               float* __restrict__ out, int32_t* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float* P = reinterpret_cast<float*>(sm + OFF_P);
    float* Gx = reinterpret_cast<float*>(sm + OFF_GX);
    float* Us = reinterpret_cast<float*>(sm + OFF_U);
    int* Ns = reinterpret_cast<int*>(sm + OFF_N);
    const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t bar = s_base + OFF_BAR;

    // ---- set-up: parameters, B operands, barrier, TMEM ----
    for (int i = tid; i < Q_N; i += THREADS) {
        float x;
        if (i < Q_W2B) x = params[P_B1 + i];
        else if (i < Q_B2) x = params[P_W2B + (i - Q_W2B)];
        else if (i < Q_W3) x = params[P_B2 + (i - Q_B2)];
        else if (i < Q_B3) x = params[P_W3 + (i - Q_W3)];
        else x = params[P_B3];
        P[i] = x;
    }
    for (int i = tid; i < 512 + 1024; i += THREADS) {
        // B1: W1 [32 n][16 k] (k >= 8 zero); B2: W2a [32 n][32 k]
        if (i < 512) {
            const int n = i >> 4, kk = i & 15;
            const float w = kk < TF ? params[P_W1 + n * TF + kk] : 0.f;
            *reinterpret_cast<__nv_bfloat16*>(sm + OFF_B1 + cm_off(n, kk, SBO_B1)) = __float2bfloat16_rn(w);
        } else {
            const int j = i - 512, n = j >> 5, kk = j & 31;
            *reinterpret_cast<__nv_bfloat16*>(sm + OFF_B2 + cm_off(n, kk, SBO_B2)) =
                __float2bfloat16_rn(params[P_W2A + n * TH + kk]);
        }
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_base + OFF_TMEM),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + OFF_TMEM);
    const uint32_t t_lane = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's TMEM lanes

    // variogram frame in FP32
    float Rf[9], ir[3];
    for (int j = 0; j < 9; ++j) Rf[j] = (float)v.R[j];
    for (int j = 0; j < 3; ++j) ir[j] = (float)v.inv_range[j];

    const int kp = k <= 32 ? 32 : 64;       // rows per system
    const int T = ROWS / kp;                // systems per tile
    const int64_t ntiles = (G.N + T - 1) / T;
    const uint32_t id1 = idesc_bf16(128, 32);
    const uint64_t a1 = smem_desc(s_base + OFF_A1, 128, SBO_A1), b1 = smem_desc(s_base + OFF_B1, 128, SBO_B1);
    const uint64_t a2 = smem_desc(s_base + OFF_A2, 128, SBO_A2), b2 = smem_desc(s_base + OFF_B2, 128, SBO_B2);
    uint32_t phase = 0;
    bool failed = false;

    for (int64_t tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int s = tid / kp, i = tid % kp;
        const int64_t g = tile * T + s;
        int n = 0;
        if (g < G.N) n = min(cnt[g], k);
        if (i == 0 && s < T) Ns[s] = n;
        const bool valid = g < G.N && i < n;
        // ---- features -> A1 (row tid) ----
        {
            float f[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) f[j] = 0.f;
            if (valid) {
                int cp[3];
                cell_of(G, (int)g, cp[0], cp[1], cp[2]);
                features_f32(G, v, Rf, ir, nbr[g * k + i], cp, data_xyz, f);
            }
            st_row8(sm + OFF_A1, cm_off(tid, 0, SBO_A1), f);
            st_row8(sm + OFF_A1, cm_off(tid, 8, SBO_A1), f + 8);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            mma_bf16(tmem, a1, b1, id1, 0u);
            mma_commit(bar);
        }
        bool ok = bar_wait(bar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();
        // ---- h = relu(D1 + b1) -> A2 (BF16); column sums of the warp's rows ----
        {
            float h[32];
            tmem_ld32(t_lane, h);
#pragma unroll
            for (int a = 0; a < 32; ++a) h[a] = valid ? fmaxf(h[a] + P[Q_B1 + a], 0.f) : 0.f;
#pragma unroll
            for (int c = 0; c < 4; ++c) st_row8(sm + OFF_A2, cm_off(tid, 8 * c, SBO_A2), h + 8 * c);
            Gx[warp * TH + lane] = warp_colsum(h, lane);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        // ---- pooled mean of system s = warp (kp = 32: warp s; kp = 64:
        // warps 2s, 2s + 1), then u = W2b g + b2 ----
        if (warp < T) {
            const int ss = warp, a = lane;
            const float sum = kp == 32 ? Gx[ss * TH + a] : Gx[2 * ss * TH + a] + Gx[(2 * ss + 1) * TH + a];
            const int ns = Ns[ss];
            const float gv = ns > 0 ? sum / (float)ns : 0.f;
            float z = P[Q_B2 + a];
#pragma unroll 8
            for (int b = 0; b < TH; ++b) z = fmaf(P[Q_W2B + a * TH + b], __shfl_sync(FULL_MASK, gv, b), z);
            Us[ss * TH + a] = z;
        }
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            mma_bf16(tmem, a2, b2, id1, 0u);
            mma_bf16(tmem, a2 + (256 >> 4), b2 + (256 >> 4), id1, 1u);  // K columns 16..31
            mma_commit(bar);
        }
        ok = bar_wait(bar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();
        // ---- y = w3 . relu(D2 + u) + b3 ----
        {
            float q[32];
            tmem_ld32(t_lane, q);
            float y = P[Q_B3];
#pragma unroll
            for (int a = 0; a < 32; ++a) y = fmaf(P[Q_W3 + a], fmaxf(q[a] + Us[s * TH + a], 0.f), y);
            if (g < G.N && i < k) out[g * k + i] = valid ? y : 0.f;
        }
        tc_fence_before();
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) atomicExch(err, 1);
        // an MMA may still be in flight: give it one more bounded wait
        bar_wait(bar, phase ^ 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

cudaError_t launch_nn_predict_tc(const GridDev& G, const VarioDev& v, const int32_t* nbr, const int32_t* cnt, int k,
                                 const double* data_xyz, const float* params, float* out, int32_t* err, int nsm,
                                 cudaStream_t s) {
    if (k < 1 || k > 64) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(nn_predict_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES);
    if (e != cudaSuccess) return e;
    // Resident CTAs per SM from the kernel's registers and shared memory and
    // the TMEM budget (512 columns per SM).  The occupancy query reported a
    // single CTA for this kernel, which left 7/8 of every SM idle; CTAs past
    // the true residency only queue (a CTA's TMEM allocation waits until a
    // resident CTA frees its columns, and resident CTAs never wait on others).
    cudaFuncAttributes fa{};
    e = cudaFuncGetAttributes(&fa, nn_predict_tc_kernel);
    if (e != cudaSuccess) return e;
    int dev = 0, smem_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const int by_regs = 65536 / std::max(1, fa.numRegs * THREADS);
    const int by_smem = smem_sm / (SMEM_BYTES + 1024);
    int per_sm = std::min(std::min(by_regs, by_smem), std::min(2048 / THREADS, (int)(512 / TMEM_COLS)));
    per_sm = std::max(1, per_sm);
    const int T = ROWS / (k <= 32 ? 32 : 64);
    const int64_t ntiles = (G.N + T - 1) / T;
    const int blocks = (int)std::min<int64_t>((int64_t)nsm * per_sm, ntiles);
    if (blocks < 1) return cudaSuccess;
    nn_predict_tc_kernel<<<blocks, THREADS, SMEM_BYTES, s>>>(G, v, nbr, cnt, k, data_xyz, params, out, err);
    return cudaGetLastError();
}

}  // namespace sgs

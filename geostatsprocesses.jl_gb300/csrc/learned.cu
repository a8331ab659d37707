// learned.cu — the kriging-weight network used as a learned warm start:
// features, forward (inference), backward (gradients) and Adam kernels.
//
// The network is permutation invariant over a system's neighbours (a
// DeepSets form): for neighbour i with features f_i
//     h_i = relu(W1 f_i + b1)                    (H = 32)
//     g   = mean_i h_i
//     q_i = relu(W2a h_i + W2b g + b2)
//     y_i = w3 . q_i + b3                        (predicted weight of i)
// Features (F = 8): the lag from the neighbour to the node in the
// variogram's normalized frame u = diag(1/ranges) R^T (x0 - x_i) (3), |u|,
// the covariance C(x_i, x0) / sill, nugget / sill, and the variogram family
// (exponential, gaussian flags; spherical is neither).  Training minimizes
// the mean squared error of y against the weights the method's own solver
// produced.  One warp per system throughout; parameters live in shared
// memory.
#include "common.cuh"

namespace sgs {

constexpr int NNF = 8;
constexpr int NNH = 32;
constexpr int NN_W1 = 0;                       // [H][F]
constexpr int NN_B1 = NN_W1 + NNH * NNF;       // [H]
constexpr int NN_W2A = NN_B1 + NNH;            // [H][H]
constexpr int NN_W2B = NN_W2A + NNH * NNH;     // [H][H]
constexpr int NN_B2 = NN_W2B + NNH * NNH;      // [H]
constexpr int NN_W3 = NN_B2 + NNH;             // [H]
constexpr int NN_B3 = NN_W3 + NNH;             // scalar
constexpr int NN_PARAMS = NN_B3 + 1;           // 2401
constexpr int NN_WARPS = 4;
constexpr int NN_LD = NNH + 1;                 // padded row of per-neighbour vectors

// Features of neighbour q of a system (see the file comment).
__device__ void nn_features(const GridDev& G, const VarioDev& v, const int* cq, const double* xq, bool qdata,
                            const int* cp, float* f) {
    double h[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < G.dim; ++j) {
        if (qdata) h[j] = centroid(G, j, cp[j]) - xq[j];
        else h[j] = (double)(cp[j] - cq[j]) * G.spacing[j];
    }
    float u[3] = {0.f, 0.f, 0.f};
    double s = 0.0;
    for (int j = 0; j < G.dim; ++j) {
        double t = v.R[0 + 3 * j] * h[0] + v.R[1 + 3 * j] * h[1];
        if (G.dim == 3) t += v.R[2 + 3 * j] * h[2];
        t *= v.inv_range[j];
        u[j] = (float)t;
        s += t * t;
    }
    f[0] = u[0];
    f[1] = u[1];
    f[2] = u[2];
    f[3] = (float)sqrt(s);
    f[4] = (float)(cov_fp64(v, G.dim, h[0], h[1], h[2]) / v.sill);
    f[5] = (float)(v.nugget / v.sill);
    f[6] = v.type == 2 ? 1.0f : 0.0f;
    f[7] = v.type == 3 ? 1.0f : 0.0f;
}

__global__ void nn_features_kernel(const GridDev G, const VarioDev v, const int32_t* nbr, const int32_t* cnt, int k,
                                   const double* data_xyz, float* feat) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t g = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); g < G.N; g += nw) {
        int cp[3];
        cell_of(G, (int)g, cp[0], cp[1], cp[2]);
        const int n = cnt[g];
        for (int q = lane; q < k; q += 32) {
            float f[NNF] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (q < n) {
                const int id = nbr[g * k + q];
                int cq[3] = {0, 0, 0};
                double xq[3] = {0, 0, 0};
                const bool isdata = id >= G.N;
                if (isdata) {
                    for (int j = 0; j < 3; ++j) xq[j] = data_xyz[3 * (int64_t)(id - G.N) + j];
                } else {
                    cell_of(G, id, cq[0], cq[1], cq[2]);
                }
                nn_features(G, v, cq, xq, isdata, cp, f);
            }
            float* o = feat + (g * k + q) * NNF;
#pragma unroll
            for (int j = 0; j < NNF; ++j) o[j] = f[j];
        }
    }
}

cudaError_t launch_nn_features(const GridDev& G, const VarioDev& v, const int32_t* nbr, const int32_t* cnt, int k,
                               const double* data_xyz, float* feat, cudaStream_t s) {
    int64_t blocks = (G.N + 7) / 8;
    if (blocks > 65535 * 8) blocks = 65535 * 8;
    nn_features_kernel<<<(int)blocks, 256, 0, s>>>(G, v, nbr, cnt, k, data_xyz, feat);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Forward pass of one system by one warp.  P: parameters (shared memory),
// f: features [n][F] (global), Hs/Qs: per-warp [64][NN_LD] scratch, gs/us:
// [H].  Leaves h_i in Hs, q_i in Qs (both post-activation), g in gs and
// W2b g + b2 in us; returns y for the lane's neighbours (i = lane, lane + 32).
__device__ void nn_forward_warp(const float* P, const float* f, int n, float* Hs, float* Qs, float* gs, float* us,
                                int lane, float y[2]) {
    for (int t = 0; t < 2; ++t) {
        const int i = lane + 32 * t;
        if (i < n) {
            float fi[NNF];
#pragma unroll
            for (int j = 0; j < NNF; ++j) fi[j] = f[i * NNF + j];
#pragma unroll 8
            for (int a = 0; a < NNH; ++a) {
                float z = P[NN_B1 + a];
#pragma unroll
                for (int j = 0; j < NNF; ++j) z = fmaf(P[NN_W1 + a * NNF + j], fi[j], z);
                Hs[i * NN_LD + a] = fmaxf(z, 0.0f);
            }
        }
    }
    __syncwarp();
    {
        float s = 0.0f;
        for (int i = 0; i < n; ++i) s += Hs[i * NN_LD + lane];
        gs[lane] = n > 0 ? s / (float)n : 0.0f;
    }
    __syncwarp();
    {
        float z = P[NN_B2 + lane];
        for (int b = 0; b < NNH; ++b) z = fmaf(P[NN_W2B + lane * NNH + b], gs[b], z);
        us[lane] = z;
    }
    __syncwarp();
    for (int t = 0; t < 2; ++t) {
        const int i = lane + 32 * t;
        y[t] = 0.0f;
        if (i < n) {
            float out = P[NN_B3];
#pragma unroll 4
            for (int a = 0; a < NNH; ++a) {
                float z = us[a];
                for (int b = 0; b < NNH; ++b) z = fmaf(P[NN_W2A + a * NNH + b], Hs[i * NN_LD + b], z);
                z = fmaxf(z, 0.0f);
                Qs[i * NN_LD + a] = z;
                out = fmaf(P[NN_W3 + a], z, out);
            }
            y[t] = out;
        }
    }
    __syncwarp();
}

struct NNSmem {
    float P[NN_PARAMS];
    float Hs[NN_WARPS][64 * NN_LD];
    float Qs[NN_WARPS][64 * NN_LD];
    float gs[NN_WARPS][NNH];
    float us[NN_WARPS][NNH];
};

__global__ void __launch_bounds__(NN_WARPS * 32) nn_forward_kernel(const float* __restrict__ params,
                                                                   const float* __restrict__ feat,
                                                                   const int32_t* __restrict__ count, int64_t nsys,
                                                                   int k, float* __restrict__ pred) {
    extern __shared__ __align__(16) unsigned char raw[];
    NNSmem& S = *reinterpret_cast<NNSmem*>(raw);
    for (int i = threadIdx.x; i < NN_PARAMS; i += blockDim.x) S.P[i] = params[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * NN_WARPS;
    for (int64_t s = (int64_t)blockIdx.x * NN_WARPS + wib; s < nsys; s += nw) {
        const int n = min(count[s], k);
        float y[2];
        nn_forward_warp(S.P, feat + s * k * NNF, n, S.Hs[wib], S.Qs[wib], S.gs[wib], S.us[wib], lane, y);
        for (int t = 0; t < 2; ++t) {
            const int i = lane + 32 * t;
            if (i < k) pred[s * k + i] = i < n ? y[t] : 0.0f;
        }
    }
}

// Loss and gradients of a batch: every system adds its mean squared error
// to *loss and its gradient to grad (accumulated per block in shared memory,
// then once per block into global memory).
__global__ void __launch_bounds__(NN_WARPS * 32) nn_backward_kernel(const float* __restrict__ params,
                                                                    const float* __restrict__ feat,
                                                                    const int32_t* __restrict__ count,
                                                                    const float* __restrict__ target, int64_t nsys,
                                                                    int k, float* grad, float* loss) {
    extern __shared__ __align__(16) unsigned char raw[];
    NNSmem& S = *reinterpret_cast<NNSmem*>(raw);
    float* G = reinterpret_cast<float*>(raw + sizeof(NNSmem));  // block gradient [NN_PARAMS]
    for (int i = threadIdx.x; i < NN_PARAMS; i += blockDim.x) {
        S.P[i] = params[i];
        G[i] = 0.0f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float* Hs = S.Hs[wib];
    float* Qs = S.Qs[wib];
    float* gs = S.gs[wib];
    float* us = S.us[wib];
    const int64_t nw = (int64_t)gridDim.x * NN_WARPS;
    float block_loss = 0.0f;
    for (int64_t s = (int64_t)blockIdx.x * NN_WARPS + wib; s < nsys; s += nw) {
        const int n = min(count[s], k);
        if (n <= 0) continue;
        const float* f = feat + s * k * NNF;
        float y[2];
        nn_forward_warp(S.P, f, n, Hs, Qs, gs, us, lane, y);
        // dL/dy_i = 2 (y_i - t_i) / n, kept per lane; squared error to the loss
        float dy[2] = {0.f, 0.f}, l2 = 0.0f;
        for (int t = 0; t < 2; ++t) {
            const int i = lane + 32 * t;
            if (i < n) {
                const float e = y[t] - target[s * k + i];
                dy[t] = 2.0f * e / (float)n;
                l2 += e * e;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) l2 += __shfl_xor_sync(FULL_MASK, l2, o);
        block_loss += l2 / (float)n;
        // output layer: dw3, db3; dz2_i = dy_i w3 (q_i > 0), stored over Qs
        // after its use (each lane owns its rows)
        float dyw[2] = {dy[0], dy[1]};
        __shared__ float dys[NN_WARPS][64];
        for (int t = 0; t < 2; ++t) {
            const int i = lane + 32 * t;
            if (i < 64) dys[wib][i] = i < n ? dyw[t] : 0.0f;
        }
        __syncwarp();
        {
            // lane a: dw3[a] = sum_i dy_i q_ia
            float acc = 0.0f;
            for (int i = 0; i < n; ++i) acc = fmaf(dys[wib][i], Qs[i * NN_LD + lane], acc);
            atomicAdd(&G[NN_W3 + lane], acc);
            if (lane == 0) {
                float sdy = 0.0f;
                for (int i = 0; i < n; ++i) sdy += dys[wib][i];
                atomicAdd(&G[NN_B3], sdy);
            }
        }
        __syncwarp();
        for (int t = 0; t < 2; ++t) {
            const int i = lane + 32 * t;
            if (i < n) {
                for (int a = 0; a < NNH; ++a) {
                    const float q = Qs[i * NN_LD + a];
                    Qs[i * NN_LD + a] = q > 0.0f ? dyw[t] * S.P[NN_W3 + a] : 0.0f;  // dz2
                }
            }
        }
        __syncwarp();
        // lane a owns row a of W2a / W2b: dW2a[a][b] = sum_i dz2_ia h_ib
        float sz = 0.0f;
        for (int i = 0; i < n; ++i) sz += Qs[i * NN_LD + lane];
        for (int b = 0; b < NNH; ++b) {
            float acc = 0.0f;
            for (int i = 0; i < n; ++i) acc = fmaf(Qs[i * NN_LD + lane], Hs[i * NN_LD + b], acc);
            atomicAdd(&G[NN_W2A + lane * NNH + b], acc);
            atomicAdd(&G[NN_W2B + lane * NNH + b], sz * gs[b]);
        }
        atomicAdd(&G[NN_B2 + lane], sz);
        // dg[b] = sum_a W2b[a][b] sz_a  (lane b); reuse us for dg / n
        us[lane] = sz;
        __syncwarp();
        float dg = 0.0f;
        for (int a = 0; a < NNH; ++a) dg = fmaf(S.P[NN_W2B + a * NNH + lane], us[a], dg);
        __syncwarp();
        gs[lane] = dg / (float)n;
        __syncwarp();
        // dh_i[b] = sum_a W2a[a][b] dz2_ia + dg_b / n; dz1 = dh (h > 0), over Hs
        for (int t = 0; t < 2; ++t) {
            const int i = lane + 32 * t;
            if (i < n) {
                float dh[NNH];
#pragma unroll
                for (int b = 0; b < NNH; ++b) dh[b] = gs[b];
                for (int a = 0; a < NNH; ++a) {
                    const float z = Qs[i * NN_LD + a];
#pragma unroll
                    for (int b = 0; b < NNH; ++b) dh[b] = fmaf(S.P[NN_W2A + a * NNH + b], z, dh[b]);
                }
#pragma unroll
                for (int b = 0; b < NNH; ++b) Hs[i * NN_LD + b] = Hs[i * NN_LD + b] > 0.0f ? dh[b] : 0.0f;
            }
        }
        __syncwarp();
        // lane a owns row a of W1: dW1[a][j] = sum_i dz1_ia f_ij
        {
            float acc[NNF] = {0, 0, 0, 0, 0, 0, 0, 0};
            float sb = 0.0f;
            for (int i = 0; i < n; ++i) {
                const float d = Hs[i * NN_LD + lane];
                sb += d;
#pragma unroll
                for (int j = 0; j < NNF; ++j) acc[j] = fmaf(d, f[i * NNF + j], acc[j]);
            }
#pragma unroll
            for (int j = 0; j < NNF; ++j) atomicAdd(&G[NN_W1 + lane * NNF + j], acc[j]);
            atomicAdd(&G[NN_B1 + lane], sb);
        }
        __syncwarp();
    }
    if (lane == 0) atomicAdd(loss, block_loss);
    __syncthreads();
    for (int i = threadIdx.x; i < NN_PARAMS; i += blockDim.x) atomicAdd(&grad[i], G[i]);
}

// Warm-start predictions for every node of a plan: features computed in
// shared memory, then the forward pass; out is node-indexed [N][k].
__global__ void __launch_bounds__(NN_WARPS * 32) nn_predict_plan_kernel(const GridDev G, const VarioDev v,
                                                                        const int32_t* __restrict__ nbr,
                                                                        const int32_t* __restrict__ cnt, int k,
                                                                        const double* __restrict__ data_xyz,
                                                                        const float* __restrict__ params,
                                                                        float* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char raw[];
    NNSmem& S = *reinterpret_cast<NNSmem*>(raw);
    float* F = reinterpret_cast<float*>(raw + sizeof(NNSmem));  // [NN_WARPS][64][NNF]
    for (int i = threadIdx.x; i < NN_PARAMS; i += blockDim.x) S.P[i] = params[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float* f = F + wib * 64 * NNF;
    const int64_t nw = (int64_t)gridDim.x * NN_WARPS;
    for (int64_t g = (int64_t)blockIdx.x * NN_WARPS + wib; g < G.N; g += nw) {
        int cp[3];
        cell_of(G, (int)g, cp[0], cp[1], cp[2]);
        const int n = min(cnt[g], k);
        for (int q = lane; q < n; q += 32) {
            const int id = nbr[g * k + q];
            int cq[3] = {0, 0, 0};
            double xq[3] = {0, 0, 0};
            const bool isdata = id >= G.N;
            if (isdata) {
                for (int j = 0; j < 3; ++j) xq[j] = data_xyz[3 * (int64_t)(id - G.N) + j];
            } else {
                cell_of(G, id, cq[0], cq[1], cq[2]);
            }
            nn_features(G, v, cq, xq, isdata, cp, f + q * NNF);
        }
        __syncwarp();
        float y[2];
        nn_forward_warp(S.P, f, n, S.Hs[wib], S.Qs[wib], S.gs[wib], S.us[wib], lane, y);
        for (int t = 0; t < 2; ++t) {
            const int i = lane + 32 * t;
            if (i < k) out[g * k + i] = i < n ? y[t] : 0.0f;
        }
    }
}

static int nn_blocks(int64_t nsys);

cudaError_t launch_nn_predict_plan(const GridDev& G, const VarioDev& v, const int32_t* nbr, const int32_t* cnt, int k,
                                   const double* data_xyz, const float* params, float* out, cudaStream_t s) {
    const size_t smem = sizeof(NNSmem) + (size_t)NN_WARPS * 64 * NNF * sizeof(float);
    cudaError_t e =
        cudaFuncSetAttribute(nn_predict_plan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    nn_predict_plan_kernel<<<nn_blocks(G.N), NN_WARPS * 32, smem, s>>>(G, v, nbr, cnt, k, data_xyz, params, out);
    return cudaGetLastError();
}

__global__ void nn_adam_kernel(float* p, const float* g, float* m, float* v, int step, float lr, float scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NN_PARAMS) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = g[i] * scale;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(b1, (float)step));
    const float vh = vi / (1.0f - powf(b2, (float)step));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

static int nn_blocks(int64_t nsys) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int64_t b = (nsys + NN_WARPS - 1) / NN_WARPS;
    const int64_t cap = (int64_t)nsm * 4;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

cudaError_t launch_nn_forward(const float* params, const float* feat, const int32_t* count, int64_t nsys, int k,
                              float* pred, cudaStream_t s) {
    const size_t smem = sizeof(NNSmem);
    cudaError_t e = cudaFuncSetAttribute(nn_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    nn_forward_kernel<<<nn_blocks(nsys), NN_WARPS * 32, smem, s>>>(params, feat, count, nsys, k, pred);
    return cudaGetLastError();
}

cudaError_t launch_nn_backward(const float* params, const float* feat, const int32_t* count, const float* target,
                               int64_t nsys, int k, float* grad, float* loss, cudaStream_t s) {
    const size_t smem = sizeof(NNSmem) + NN_PARAMS * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(nn_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    nn_backward_kernel<<<nn_blocks(nsys), NN_WARPS * 32, smem, s>>>(params, feat, count, target, nsys, k, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_nn_adam(float* p, const float* g, float* m, float* v, int step, float lr, float scale,
                           cudaStream_t s) {
    nn_adam_kernel<<<(NN_PARAMS + 255) / 256, 256, 0, s>>>(p, g, m, v, step, lr, scale);
    return cudaGetLastError();
}

}  // namespace sgs

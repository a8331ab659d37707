// common.cuh — device helpers shared by the SGS kernels: the canonical FP64
// lag metric, the variogram covariance, Philox draws and warp utilities.
//
// Canonical formulas (identical operation order on host and device; the
// device uses the _rn intrinsics so nothing is contracted into an FMA):
//   grid lag      h_j = (double)(i_c - i_p) * spacing_j
//   data lag      h_j = X_j - (origin_j + ((double)i_j + 0.5) * spacing_j)
//   isotropic     d2 = h0*h0 + h1*h1 (+ h2*h2), inside iff d2 <= r*r
//   ellipsoid     u_j = R(0,j)h0 + R(1,j)h1 (+ R(2,j)h2), q_j = u_j * inv_j
//                 with inv_j = 1 / radius_j rounded once, d2 = sum_j q_j^2,
//                 inside iff d2 <= 1
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "internal.h"

#define FULL_MASK 0xffffffffu

namespace sgs {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// canonical squared distance of a lag under a search metric
__device__ __forceinline__ double metric_d2(const MetricDev& m, int dim, double h0, double h1, double h2) {
    if (m.kind != METRIC_ELLIPSOID) {
        double s = dmul(h0, h0);
        s = dadd(s, dmul(h1, h1));
        if (dim == 3) s = dadd(s, dmul(h2, h2));
        return s;
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (j < dim) {
            double u = dmul(m.R[0 + 3 * j], h0);
            u = dadd(u, dmul(m.R[1 + 3 * j], h1));
            if (dim == 3) u = dadd(u, dmul(m.R[2 + 3 * j], h2));
            double q = dmul(u, m.inv[j]);
            s = (j == 0) ? dmul(q, q) : dadd(s, dmul(q, q));
        }
    }
    return s;
}

// FP32 evaluation of the same metric, used only to discard candidates that
// are clearly outside `bound` (bound_f, or a tighter bound for a smaller
// distance; each carries a 1e-3 relative margin and a slack above the FP32
// rounding of these few operations), so the FP64 decision is unchanged.
__device__ __forceinline__ bool metric_maybe_within(const MetricDev& m, int dim, float h0, float h1, float h2,
                                                    float bound) {
    float s;
    if (m.kind != METRIC_ELLIPSOID) {
        s = h0 * h0 + h1 * h1 + (dim == 3 ? h2 * h2 : 0.0f);
    } else {
        s = 0.0f;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            if (j < dim) {
                float u = m.Rf[0 + 3 * j] * h0 + m.Rf[1 + 3 * j] * h1 + (dim == 3 ? m.Rf[2 + 3 * j] * h2 : 0.0f);
                float q = u * m.invf[j];
                s += q * q;
            }
        }
    }
    return s <= bound;
}

__device__ __forceinline__ bool metric_inside(const MetricDev& m, double d2) {
    if (m.kind == METRIC_ISO) return d2 <= m.rr;
    if (m.kind == METRIC_ELLIPSOID) return d2 <= 1.0;
    return true;
}

// grid centroid coordinate along axis j
__device__ __forceinline__ double centroid(const GridDev& g, int j, int i) {
    double t = dadd((double)i, 0.5);
    t = dmul(t, g.spacing[j]);
    return dadd(g.origin[j], t);
}

__device__ __forceinline__ void cell_of(const GridDev& g, int node, int& i0, int& i1, int& i2) {
    i0 = node % g.n[0];
    int r = node / g.n[0];
    i1 = r % g.n[1];
    i2 = r / g.n[1];
}

// gamma(h) of one structure at a nonzero lag (GeoStatsFunctions conventions:
// practical ranges, nugget for nonzero lags only)
__device__ __forceinline__ double structure_gamma(const VarioStructDev& v, int dim, double h0, double h1, double h2) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (j < dim) {
            double u = v.R[0 + 3 * j] * h0 + v.R[1 + 3 * j] * h1;
            if (dim == 3) u += v.R[2 + 3 * j] * h2;
            double q = u * v.inv_range[j];
            s += q * q;
        }
    }
    double hn = sqrt(s);
    double f;
    if (v.type == 1) f = hn < 1.0 ? 1.5 * hn - 0.5 * hn * hn * hn : 1.0;
    else if (v.type == 2) f = 1.0 - exp(-3.0 * hn);
    else f = 1.0 - exp(-3.0 * s);
    return v.nugget + (v.sill - v.nugget) * f;
}

// covariance C(h) = sill - gamma(h) in FP64, gamma summed over the model's
// structures
__device__ __forceinline__ double cov_fp64(const VarioDev& v, int dim, double h0, double h1, double h2) {
    if (h0 == 0.0 && h1 == 0.0 && (dim == 2 || h2 == 0.0)) return v.sill;
    double g = structure_gamma(v.st[0], dim, h0, h1, h2);
    for (int i = 1; i < v.ns; ++i) g += structure_gamma(v.st[i], dim, h0, h1, h2);
    return v.sill - g;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw 2011) on counter (c0..c3), key (k0,k1)
__device__ __forceinline__ uint4 philox10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        uint4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// four standard normals of node g, realizations 4q..4q+3 (Box-Muller on
// 24-bit uniforms (2m+1)/2^24, exactly representable in float)
__device__ __forceinline__ float4 normals4(uint64_t seed, int64_t g, int q) {
    uint4 c = philox10(make_uint4((uint32_t)g, (uint32_t)((uint64_t)g >> 32), (uint32_t)q, 0u),
                       (uint32_t)seed, (uint32_t)(seed >> 32));
    const float sc = 1.0f / 16777216.0f;
    float u0 = (float)((c.x >> 9) * 2u + 1u) * sc;
    float u1 = (float)((c.y >> 9) * 2u + 1u) * sc;
    float u2 = (float)((c.z >> 9) * 2u + 1u) * sc;
    float u3 = (float)((c.w >> 9) * 2u + 1u) * sc;
    float r0 = sqrtf(-2.0f * logf(u0)), r1 = sqrtf(-2.0f * logf(u2));
    float s0, c0, s1, c1;
    sincospif(2.0f * u1, &s0, &c0);
    sincospif(2.0f * u3, &s1, &c1);
    return make_float4(r0 * c0, r0 * s0, r1 * c1, r1 * s1);
}

// ---- double-FP32 ("float-float") arithmetic: a value is an unevaluated sum
// hi + lo of two floats, |lo| <= ulp(hi)/2, about 48 significant bits.  Error-
// free transformations after Knuth (TwoSum), Dekker (Fast2Sum) and the FMA
// form of TwoProduct; every operation is an explicit _rn intrinsic so the
// compiler cannot contract or reorder them.
struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return {s, e};
}

__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DF df_from_double(double v) {
    const float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}

__device__ __forceinline__ DF df_add(DF a, DF b) {
    const DF s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ DF df_neg(DF a) { return {-a.hi, -a.lo}; }

// Compensated dot-product accumulator (Dot2, Ogita-Rump-Oishi 2005) with
// double-FP32 operands: adds (xh + xl) * (yh + yl) dropping only xl*yl.
struct DFAcc {
    float s, c;
    __device__ __forceinline__ void init(DF v) {
        s = v.hi;
        c = v.lo;
    }
    __device__ __forceinline__ void add_prod(DF x, DF y) {
        const float p = __fmul_rn(x.hi, y.hi);
        const float pe = __fmaf_rn(x.hi, y.hi, -p);
        const DF t = df_two_sum(s, p);
        s = t.hi;
        const float cross = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.hi));
        c = __fadd_rn(c, __fadd_rn(t.lo, __fadd_rn(pe, cross)));
    }
    __device__ __forceinline__ DF value() const { return df_two_sum(s, c); }
};

// square root of a non-negative double-FP32 value: FP32 root plus one
// Newton correction evaluated with an exact square (TwoProduct)
__device__ __forceinline__ DF df_sqrt(DF v) {
    if (!(v.hi > 0.0f)) return {0.0f, 0.0f};
    const float r = sqrtf(v.hi);
    const float p = __fmul_rn(r, r);
    const float pe = __fmaf_rn(r, r, -p);
    const float d = __fadd_rn(__fsub_rn(__fsub_rn(v.hi, p), pe), v.lo);
    return df_fast_two_sum(r, __fdiv_rn(d, __fmul_rn(2.0f, r)));
}

__device__ __forceinline__ DF shfl_xor_df(DF v, int o) {
    return {__shfl_xor_sync(FULL_MASK, v.hi, o), __shfl_xor_sync(FULL_MASK, v.lo, o)};
}

__device__ __forceinline__ DF warp_sum_df(DF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = df_add(v, shfl_xor_df(v, o));
    return v;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Level of node c once it is known (>= 0).  Bounded: the wait gives up after
// wait_ns of wall-clock time (or, should the timer stall, after a count of
// polls, each at least the 64 ns back-off, reached no earlier), and soon after
// another warp has raised *err.  The flag and the timer are read every 32nd
// poll only: the flag shares its cache line with the kernel's ticket counter,
// which every warp updates.  A warp that gives up raises *err; the returned
// level is then 0 and the caller's result is void.
__device__ __forceinline__ int wait_level(const volatile int32_t* vlevel, int64_t c, int32_t* err,
                                          uint64_t wait_ns) {
    int l = vlevel[c];
    if (l >= 0) return l;
    const volatile int32_t* verr = err;
    const uint64_t max_polls = wait_ns / 32 + 1024;
    uint64_t t0 = 0;
    for (uint64_t polls = 1;; ++polls) {
        __nanosleep(64);
        l = vlevel[c];
        if (l >= 0) return l;
        if ((polls & 31) == 0) {
            if (*verr) return 0;
            const uint64_t now = global_ns();
            if (t0 == 0) t0 = now;
            if (now - t0 > wait_ns || polls > max_polls) {
                atomicExch(err, 1);
                return 0;
            }
        }
    }
}

// Right-looking Cholesky of the lower triangle of A (leading dimension ld)
// by one warp.  Fails (returns false) when a pivot is not > tau.
template <typename T>
__device__ bool warp_cholesky(T* A, int ld, int n, T tau, int lane) {
    for (int j = 0; j < n; ++j) {
        const T d = A[j * ld + j];
        if (!(d > tau)) return false;
        const T ljj = sqrt(d);
        const T inv = T(1) / ljj;
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) A[i * ld + j] *= inv;
        if (lane == 0) A[j * ld + j] = ljj;
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) {
            const T lij = A[i * ld + j];
            for (int l = j + 1; l <= i; ++l) A[i * ld + l] -= lij * A[l * ld + j];
        }
        __syncwarp();
    }
    return true;
}

// Solve L L^T x = b in place (x overwrites b), L from warp_cholesky.
template <typename T>
__device__ void warp_chol_solve(const T* A, int ld, int n, T* b, int lane) {
    for (int j = 0; j < n; ++j) {
        const T yj = b[j] / A[j * ld + j];
        __syncwarp();
        if (lane == 0) b[j] = yj;
        for (int i = j + 1 + lane; i < n; i += 32) b[i] -= A[i * ld + j] * yj;
        __syncwarp();
    }
    for (int j = n - 1; j >= 0; --j) {
        const T wj = b[j] / A[j * ld + j];
        __syncwarp();
        if (lane == 0) b[j] = wj;
        for (int i = lane; i < j; i += 32) b[i] -= A[j * ld + i] * wj;
        __syncwarp();
    }
}

// ---- batches of domains: global numbering and per-domain descriptors ----
// Domain d owns the global ids [off[d], off[d+1]); returns d for id x
// (0 <= x < off[nd]) by binary search over the nd + 1 offsets.
__device__ __forceinline__ int find_domain(const int64_t* __restrict__ off, int nd, int64_t x) {
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Copy a descriptor (a plain struct, 4-byte multiple) from global into this
// warp's shared-memory slot, all lanes cooperating; the caller __syncwarp()s.
template <typename T>
__device__ __forceinline__ void warp_copy_struct(T* dst, const T* src, int lane) {
    static_assert(sizeof(T) % 4 == 0, "descriptor size");
    int* d = reinterpret_cast<int*>(dst);
    const int* s = reinterpret_cast<const int*>(src);
    for (int i = lane; i < (int)(sizeof(T) / 4); i += 32) d[i] = __ldg(s + i);
}

// First table entry of sweep-table row `pos`: rows of k entries, or CSR
// offsets when the tables are packed (batches of domains with different k).
template <typename T>
__device__ __forceinline__ int64_t table_row(const SweepTables<T>& t, int64_t pos, int k) {
    return t.off ? t.off[pos] : pos * (int64_t)k;
}

}  // namespace sgs

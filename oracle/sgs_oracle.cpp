// sgs_oracle.cpp — FP64 CPU oracle for sequential Gaussian simulation.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA library (see
// sgs_oracle.h).  Parity status: partially pinned (reference known-answer
// tests + closed forms + an independent numpy restatement; no reference
// outputs, since Julia is not available).
//
// Restated from GeoStatsProcesses.jl v0.13.0 (paths relative to the project):
//   control flow, prior branch, status fallback    src/simulation/field/seqsim.jl:72-156
//   nmin / nmax clamps                              src/simulation/field/seqsim.jl:202-208
//   augmented point set: grid, then data            src/simulation/field/seqsim.jl:211-218,267-271
//   :range neighbourhood = ball of radius range(f)  src/simulation/field/seqsim.jl:171-177
//   covariance = sill - variogram                   src/utils.jl:50-62
//   prior Normal(mu, sqrt(sill))                    src/simulation/field/seqsim.jl:277-290
//   draw mu_hat + sigma_hat * z                     src/simulation/field/seqsim.jl:335-340
// and from the published behaviour of the un-vendored dependencies
// (Meshes 0.57 KBallSearch/KNearestSearch: neighbours inside the ball that
// pass the mask, nearest first, at most k; GeoStatsFunctions 0.15
// spherical/exponential/gaussian variograms with the practical-range factor 3
// and the nugget applied for h > 0 only; GeoStatsModels 0.13 simple kriging:
// Cholesky of the covariance LHS, mean mu + w'(v - mu), variance
// C(0) - w'c, failure of the factorization -> prior).
//
// Canonical definitions this project fixes where the reference's result
// depends on tree traversal order or rounding:
//  * lag from a query grid node p to a candidate: (i_c - i_p) * spacing per
//    axis for grid candidates, X_c - centroid(p) for data candidates, where
//    centroid_j = origin_j + (i_j + 0.5) * spacing_j.  The reference's
//    similarity scaling (seqsim.jl:162-189) multiplies coordinates, ranges and
//    the ball by one factor and changes no distance order or covariance in
//    exact arithmetic, so everything is evaluated in unscaled units.
//  * isotropic ball: d2 = sum_j h_j^2, inside iff d2 <= r*r.  Ellipsoid:
//    u_j = sum_i R(i,j) h_i, q_j = u_j * (1 / radius_j) with the reciprocal
//    rounded once, d2 = sum_j q_j^2, inside iff d2 <= 1.  All sums in axis order, every operation rounded (built with
//    -ffp-contract=off; the GPU uses the _rn intrinsics).
//  * neighbour order: ascending (d2, augmented index).
//  * singular rule: the factorization fails when a pivot (before the square
//    root) is not > 1e-10 * sill; the node then takes the prior.
//  * variance: sigma^2 = max(sill - w'c, 0).
#include "sgs_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

const double kSingularTau = 1e-10;

struct Metric {
    int dim = 2;
    int kind = 0;        // 0 iso, 1 ellipsoid, 2 unbounded (nearest)
    double rr = 0.0;     // r*r for iso
    double radii[3] = {1, 1, 1};
    double inv[3] = {1, 1, 1};  // 1 / radii, rounded once
    double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    double ext[3] = {0, 0, 0};  // half extents of the bounding box (physical units)

    double d2(const double* h) const {
        if (kind != 1) {
            double s = h[0] * h[0];
            s = s + h[1] * h[1];
            if (dim == 3) s = s + h[2] * h[2];
            return s;
        }
        double s = 0.0;
        for (int j = 0; j < dim; ++j) {
            double u = R[0 + 3 * j] * h[0];
            u = u + R[1 + 3 * j] * h[1];
            if (dim == 3) u = u + R[2 + 3 * j] * h[2];
            double q = u * inv[j];
            s = (j == 0) ? q * q : s + q * q;
        }
        return s;
    }
    bool inside(double d) const {
        if (kind == 0) return d <= rr;
        if (kind == 1) return d <= 1.0;
        return true;
    }
};

struct Cand {
    double d2;
    int64_t idx;
    bool operator<(const Cand& o) const { return d2 < o.d2 || (d2 == o.d2 && idx < o.idx); }
};

struct Offset {
    int32_t o[3];
    int64_t lin;
    double d2;
};

}  // namespace

struct oracle_plan {
    int dim;
    int64_t n[3];
    double origin[3], spacing[3];
    int64_t N, D;
    std::vector<double> dx;   // D x 3 (padded)
    std::vector<double> dval; // D
    sgs_variogram vario;      // first structure
    std::vector<sgs_variogram> vs;  // every structure of the (nested) model
    std::vector<Metric> vms;        // their normalized lag metrics
    double sill = 1.0;        // the model's sill: the structures' sills summed
    // covariances of grid lags L (|L_j| <= lut_e[j]) computed once: entry
    // (L0 + e0) + w0 ((L1 + e1) + w1 (L2 + e2)) holds cov(L * spacing), the
    // value cov() gives for every grid pair with that lag
    std::vector<double> lut;
    int64_t lut_e[3] = {-1, -1, -1}, lut_w[3] = {0, 0, 0};
    double mean;
    int nmin, nmax;
    Metric search;
    Metric vmetric;           // variogram's normalized lag metric
    int64_t tmpl_ext[3] = {0, 0, 0};  // the offset template's extent per axis (cells)
    std::vector<int32_t> path, rank;
    std::vector<Offset> tmpl;
    // data buckets
    int64_t B = 8;
    int64_t nb[3];
    std::vector<int64_t> bstart;
    std::vector<int32_t> bdata;
    // results, node-indexed
    std::vector<int32_t> nbr, cnt;
    std::vector<uint8_t> searched, solved;
    std::vector<double> w, sigma;
    std::vector<int32_t> status;

    void cell(int64_t g, int64_t* i) const {
        i[0] = g % n[0];
        int64_t r = g / n[0];
        i[1] = r % n[1];
        i[2] = r / n[1];
    }
    double centroid(int64_t i, int j) const {
        double t = (double)i + 0.5;
        t = t * spacing[j];
        return origin[j] + t;
    }
    // lag from augmented point a to augmented point b
    void lag(int64_t a, int64_t b, double* h) const {
        h[0] = h[1] = h[2] = 0.0;
        if (a < N && b < N) {
            int64_t ia[3], ib[3];
            cell(a, ia);
            cell(b, ib);
            for (int j = 0; j < dim; ++j) h[j] = (double)(ib[j] - ia[j]) * spacing[j];
        } else {
            double pa[3], pb[3];
            point(a, pa);
            point(b, pb);
            for (int j = 0; j < dim; ++j) h[j] = pb[j] - pa[j];
        }
    }
    void point(int64_t a, double* x) const {
        if (a < N) {
            int64_t i[3];
            cell(a, i);
            for (int j = 0; j < dim; ++j) x[j] = centroid(i[j], j);
        } else {
            for (int j = 0; j < dim; ++j) x[j] = dx[(a - N) * 3 + j];
        }
    }
    // covariance of two points by their ids, given their cells (ca, cb;
    // unused for data): grid pairs through the lag table when it covers
    // their lag
    double cov_pair(int64_t a, int64_t b, const int64_t* ca, const int64_t* cb) const {
        double h[3];
        if (a < N && b < N && !lut.empty()) {
            int64_t off = 0, mult = 1;
            bool inside = true;
            for (int j = 0; j < dim; ++j) {
                const int64_t L = cb[j] - ca[j];
                inside = inside && L >= -lut_e[j] && L <= lut_e[j];
                off += (L + lut_e[j]) * mult;
                mult *= lut_w[j];
            }
            if (inside) return lut[(size_t)off];
        }
        lag(a, b, h);
        return cov(h);
    }
    // C(h) = sill - gamma(h), gamma = sum over the structures of
    // nugget_s + (sill_s - nugget_s) f_s(|h|_s) for h != 0 (utils.jl:50-62)
    double cov(const double* h) const {
        bool zero = true;
        for (int j = 0; j < dim; ++j) zero = zero && (h[j] == 0.0);
        if (zero) return sill;
        double gamma = 0.0;
        for (size_t i = 0; i < vs.size(); ++i) {
            const double s = vs[i].sill, ng = vs[i].nugget;
            const double hn = std::sqrt(vms[i].d2(h));
            double f;
            switch (vs[i].type) {
                case SGS_SPHERICAL: f = hn < 1.0 ? 1.5 * hn - 0.5 * hn * hn * hn : 1.0; break;
                case SGS_EXPONENTIAL: f = 1.0 - std::exp(-3.0 * hn); break;
                default: f = 1.0 - std::exp(-3.0 * hn * hn); break;
            }
            gamma = i == 0 ? ng + (s - ng) * f : gamma + (ng + (s - ng) * f);
        }
        return sill - gamma;
    }
};

static void set_metric(Metric& m, int dim, int kind, const double* radii, const double* rot) {
    m.dim = dim;
    m.kind = kind;
    for (int j = 0; j < 3; ++j) {
        m.radii[j] = radii[j];
        m.inv[j] = 1.0 / radii[j];
    }
    for (int j = 0; j < 9; ++j) m.R[j] = rot[j];
    if (kind == 0) {
        m.rr = radii[0] * radii[0];
        for (int j = 0; j < dim; ++j) m.ext[j] = radii[0];
    } else if (kind == 1) {
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

static bool is_identity(const double* R, int dim) {
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
            if (R[i + 3 * j] != (i == j ? 1.0 : 0.0)) return false;
    return true;
}

extern "C" const char* oracle_last_error(void) { return g_err.c_str(); }

extern "C" int oracle_create(const sgs_problem* p, oracle_plan** out) {
    if (!p || !out) return fail(SGS_ERR_ARG, "null argument");
    *out = nullptr;
    if (p->dim != 2 && p->dim != 3) return fail(SGS_ERR_ARG, "dim must be 2 or 3");
    auto* P = new oracle_plan();
    P->dim = p->dim;
    P->N = 1;
    for (int j = 0; j < 3; ++j) {
        P->n[j] = j < p->dim ? p->dims[j] : 1;
        P->origin[j] = j < p->dim ? p->origin[j] : 0.0;
        P->spacing[j] = j < p->dim ? p->spacing[j] : 1.0;
        if (P->n[j] < 1) { delete P; return fail(SGS_ERR_ARG, "grid dims must be >= 1"); }
        if (!(P->spacing[j] > 0.0)) { delete P; return fail(SGS_ERR_ARG, "spacing must be > 0"); }
        P->N *= P->n[j];
    }
    if (P->N > INT32_MAX / 2) { delete P; return fail(SGS_ERR_ARG, "grid too large"); }
    P->D = p->ndata;
    if (P->D < 0 || (P->D > 0 && (!p->data_coords || !p->data_values))) {
        delete P;
        return fail(SGS_ERR_ARG, "invalid data arrays");
    }
    P->dx.assign((size_t)P->D * 3, 0.0);
    P->dval.assign((size_t)P->D, 0.0);
    for (int64_t i = 0; i < P->D; ++i) {
        for (int j = 0; j < P->dim; ++j) P->dx[i * 3 + j] = p->data_coords[i * P->dim + j];
        P->dval[i] = p->data_values[i];
    }
    P->vario = p->variogram;
    const sgs_variogram& v = P->vario;
    if (p->nstructures < 0 || p->nstructures >= SGS_MAX_STRUCTURES || (p->nstructures > 0 && !p->structures)) {
        delete P;
        return fail(SGS_ERR_ARG, "invalid nested structures");
    }
    P->vs.assign(1, v);
    for (int i = 0; i < p->nstructures; ++i) P->vs.push_back(p->structures[i]);
    P->sill = 0.0;
    double rmax = 0.0;  // range(f): the largest range of any structure
    for (const sgs_variogram& u : P->vs) {
        if (u.type < SGS_SPHERICAL || u.type > SGS_GAUSSIAN) { delete P; return fail(SGS_ERR_ARG, "unknown variogram type"); }
        if (!(u.sill > 0.0) || u.nugget < 0.0 || u.nugget > u.sill) { delete P; return fail(SGS_ERR_ARG, "invalid sill/nugget"); }
        for (int j = 0; j < P->dim; ++j) {
            if (!(u.ranges[j] > 0.0)) { delete P; return fail(SGS_ERR_ARG, "ranges must be > 0"); }
            rmax = std::max(rmax, u.ranges[j]);
        }
        P->sill += u.sill;
        P->vms.emplace_back();
        set_metric(P->vms.back(), P->dim, 1, u.ranges, u.rotation);
    }
    P->mean = p->mean;
    set_metric(P->vmetric, P->dim, 1, v.ranges, v.rotation);

    // nmin / nmax clamps: seqsim.jl:202-208 (nelm = grid nodes)
    int64_t nmax = p->maxneighbors, nmin = p->minneighbors;
    if (nmax > P->N || nmax < 1) nmax = P->N;
    if (nmin > nmax || nmin < 1) nmin = 1;
    if (nmax > 4096) { delete P; return fail(SGS_ERR_ARG, "maxneighbors too large for the oracle"); }
    P->nmax = (int)nmax;
    P->nmin = (int)nmin;

    // search neighbourhood: seqsim.jl:171-177, 221-227
    if (p->search == SGS_SEARCH_RANGE) {
        double r[3] = {rmax, rmax, rmax};
        double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        set_metric(P->search, P->dim, 0, r, I);
    } else if (p->search == SGS_SEARCH_BALL) {
        const sgs_ball& b = p->ball;
        for (int j = 0; j < P->dim; ++j)
            if (!(b.radii[j] > 0.0)) { delete P; return fail(SGS_ERR_ARG, "ball radii must be > 0"); }
        bool iso = is_identity(b.rotation, P->dim);
        for (int j = 1; j < P->dim; ++j) iso = iso && b.radii[j] == b.radii[0];
        set_metric(P->search, P->dim, iso ? 0 : 1, b.radii, b.rotation);
    } else if (p->search == SGS_SEARCH_NEAREST) {
        double r[3] = {1, 1, 1};
        double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        set_metric(P->search, P->dim, 2, r, I);
    } else {
        delete P;
        return fail(SGS_ERR_ARG, "unknown search kind");
    }

    // path (LinearPath when NULL) and its ranks
    P->path.resize(P->N);
    P->rank.assign(P->N, -1);
    for (int64_t t = 0; t < P->N; ++t) {
        int64_t g = p->path ? p->path[t] : t;
        if (g < 0 || g >= P->N || P->rank[g] != -1) { delete P; return fail(SGS_ERR_ARG, "path is not a permutation of the grid nodes"); }
        P->path[t] = (int32_t)g;
        P->rank[g] = (int32_t)t;
    }

    // offset template in canonical order
    int64_t e[3] = {0, 0, 0};
    for (int j = 0; j < P->dim; ++j) {
        if (P->search.kind == 2) e[j] = P->n[j] - 1;
        else e[j] = std::min<int64_t>(P->n[j] - 1, (int64_t)std::floor(P->search.ext[j] / P->spacing[j]) + 1);
        P->tmpl_ext[j] = e[j];
    }
    for (int64_t c = -e[2]; c <= e[2]; ++c)
        for (int64_t b = -e[1]; b <= e[1]; ++b)
            for (int64_t a = -e[0]; a <= e[0]; ++a) {
                if (a == 0 && b == 0 && c == 0) continue;
                double h[3] = {(double)a * P->spacing[0], (double)b * P->spacing[1],
                               P->dim == 3 ? (double)c * P->spacing[2] : 0.0};
                double d = P->search.d2(h);
                if (!P->search.inside(d)) continue;
                Offset o;
                o.o[0] = (int32_t)a; o.o[1] = (int32_t)b; o.o[2] = (int32_t)c;
                o.lin = a + P->n[0] * (b + P->n[1] * c);
                o.d2 = d;
                P->tmpl.push_back(o);
            }
    std::sort(P->tmpl.begin(), P->tmpl.end(), [](const Offset& x, const Offset& y) {
        return x.d2 < y.d2 || (x.d2 == y.d2 && x.lin < y.lin);
    });

    // data buckets
    int64_t nbk = 1;
    for (int j = 0; j < 3; ++j) {
        P->nb[j] = (P->n[j] + P->B - 1) / P->B;
        nbk *= P->nb[j];
    }
    std::vector<int64_t> bid(P->D);
    P->bstart.assign(nbk + 1, 0);
    for (int64_t i = 0; i < P->D; ++i) {
        int64_t bc[3] = {0, 0, 0};
        for (int j = 0; j < P->dim; ++j) {
            double f = std::floor((P->dx[i * 3 + j] - P->origin[j]) / (P->spacing[j] * (double)P->B));
            bc[j] = std::min<int64_t>(P->nb[j] - 1, std::max<int64_t>(0, (int64_t)std::max(-1.0, std::min(f, 1e15))));
        }
        bid[i] = bc[0] + P->nb[0] * (bc[1] + P->nb[1] * bc[2]);
        P->bstart[bid[i] + 1]++;
    }
    for (int64_t b = 0; b < nbk; ++b) P->bstart[b + 1] += P->bstart[b];
    P->bdata.assign(P->D, 0);
    {
        std::vector<int64_t> cur(P->bstart.begin(), P->bstart.end() - 1);
        for (int64_t i = 0; i < P->D; ++i) P->bdata[cur[bid[i]]++] = (int32_t)i;
    }

    P->nbr.assign((size_t)P->N * P->nmax, -1);
    P->cnt.assign(P->N, 0);
    P->searched.assign(P->N, 0);
    P->solved.assign(P->N, 0);
    P->w.assign((size_t)P->N * P->nmax, 0.0);
    P->sigma.assign(P->N, 0.0);
    P->status.assign(P->N, SGS_NODE_PRIOR_NMIN);
    *out = P;
    return SGS_OK;
}

extern "C" void oracle_destroy(oracle_plan* p) { delete p; }

extern "C" int oracle_template_size(const oracle_plan* p) { return p ? (int)p->tmpl.size() : 0; }

// data candidates of query node g inside the neighbourhood, sorted canonically
static void data_candidates(const oracle_plan* P, int64_t g, bool brute, std::vector<Cand>& out) {
    out.clear();
    if (P->D == 0) return;
    int64_t ic[3];
    P->cell(g, ic);
    double x[3] = {0, 0, 0};
    for (int j = 0; j < P->dim; ++j) x[j] = P->centroid(ic[j], j);
    auto test = [&](int64_t i) {
        double h[3] = {0, 0, 0};
        for (int j = 0; j < P->dim; ++j) h[j] = P->dx[i * 3 + j] - x[j];
        double d = P->search.d2(h);
        if (P->search.inside(d)) out.push_back({d, P->N + i});
    };
    if (brute || P->search.kind == 2) {
        for (int64_t i = 0; i < P->D; ++i) test(i);
    } else {
        int64_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        for (int j = 0; j < P->dim; ++j) {
            double w = P->spacing[j] * (double)P->B;
            double a = std::floor((x[j] - P->search.ext[j] - P->origin[j]) / w) - 1;
            double b = std::floor((x[j] + P->search.ext[j] - P->origin[j]) / w) + 1;
            lo[j] = (int64_t)std::max(0.0, std::min(a, (double)(P->nb[j] - 1)));
            hi[j] = (int64_t)std::max(0.0, std::min(b, (double)(P->nb[j] - 1)));
        }
        for (int64_t c = lo[2]; c <= hi[2]; ++c)
            for (int64_t b = lo[1]; b <= hi[1]; ++b)
                for (int64_t a = lo[0]; a <= hi[0]; ++a) {
                    int64_t id = a + P->nb[0] * (b + P->nb[1] * c);
                    for (int64_t q = P->bstart[id]; q < P->bstart[id + 1]; ++q) test(P->bdata[q]);
                }
    }
    std::sort(out.begin(), out.end());
}

static void search_node(oracle_plan* P, int64_t t, int method, std::vector<Cand>& grid,
                        std::vector<Cand>& data) {
    const int64_t g = P->path[t];
    int64_t ic[3];
    P->cell(g, ic);
    const int k = P->nmax;
    grid.clear();
    if (method == ORACLE_SEARCH_BRUTE) {
        int64_t e[3] = {0, 0, 0};
        for (int j = 0; j < P->dim; ++j) {
            if (P->search.kind == 2) e[j] = P->n[j];
            else e[j] = (int64_t)std::floor(P->search.ext[j] / P->spacing[j]) + 2;
        }
        int64_t lo[3], hi[3];
        for (int j = 0; j < 3; ++j) {
            lo[j] = std::max<int64_t>(0, ic[j] - e[j]);
            hi[j] = std::min<int64_t>(P->n[j] - 1, ic[j] + e[j]);
        }
        for (int64_t c = lo[2]; c <= hi[2]; ++c)
            for (int64_t b = lo[1]; b <= hi[1]; ++b)
                for (int64_t a = lo[0]; a <= hi[0]; ++a) {
                    int64_t cg = a + P->n[0] * (b + P->n[1] * c);
                    if (cg == g || P->rank[cg] >= t) continue;
                    double h[3] = {(double)(a - ic[0]) * P->spacing[0], (double)(b - ic[1]) * P->spacing[1],
                                   P->dim == 3 ? (double)(c - ic[2]) * P->spacing[2] : 0.0};
                    double d = P->search.d2(h);
                    if (P->search.inside(d)) grid.push_back({d, cg});
                }
        std::sort(grid.begin(), grid.end());
    } else {
        for (const Offset& o : P->tmpl) {
            if ((int)grid.size() >= k) break;
            int64_t a = ic[0] + o.o[0], b = ic[1] + o.o[1], c = ic[2] + o.o[2];
            if (a < 0 || a >= P->n[0] || b < 0 || b >= P->n[1] || c < 0 || c >= P->n[2]) continue;
            int64_t cg = g + o.lin;
            if (P->rank[cg] < t) grid.push_back({o.d2, cg});
        }
    }
    data_candidates(P, g, method == ORACLE_SEARCH_BRUTE, data);
    // merge, keep the k best
    int32_t* nb = &P->nbr[(size_t)g * k];
    size_t i = 0, j = 0;
    int m = 0;
    while (m < k && (i < grid.size() || j < data.size())) {
        bool take_grid = j >= data.size() || (i < grid.size() && grid[i] < data[j]);
        nb[m++] = (int32_t)(take_grid ? grid[i++].idx : data[j++].idx);
    }
    for (int q = m; q < k; ++q) nb[q] = -1;
    P->cnt[g] = m;
    P->searched[g] = 1;
}

static int nthreads_or_all(int n) {
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

extern "C" int oracle_search(oracle_plan* P, int method, int64_t t0, int64_t t1, int64_t stride,
                             int nthreads) {
    if (!P) return fail(SGS_ERR_ARG, "null plan");
    if (stride < 1) stride = 1;
    t0 = std::max<int64_t>(0, t0);
    t1 = std::min<int64_t>(P->N, t1);
    const int nt = nthreads_or_all(nthreads);
#pragma omp parallel num_threads(nt)
    {
        std::vector<Cand> grid, data;
        grid.reserve(4096);
#pragma omp for schedule(dynamic, 256)
        for (int64_t t = t0; t < t1; t += stride) search_node(P, t, method, grid, data);
    }
    return SGS_OK;
}

static void solve_node(oracle_plan* P, int64_t g, std::vector<double>& K, std::vector<double>& c) {
    const int k = P->nmax;
    const int n = P->cnt[g];
    const int32_t* nb = &P->nbr[(size_t)g * k];
    double* w = &P->w[(size_t)g * k];
    for (int a = 0; a < k; ++a) w[a] = 0.0;
    P->solved[g] = 1;
    if (n < P->nmin) {  // seqsim.jl:109-111
        P->status[g] = SGS_NODE_PRIOR_NMIN;
        P->sigma[g] = std::sqrt(P->sill);
        return;
    }
    K.assign((size_t)n * n, 0.0);
    c.assign(n, 0.0);
    int64_t cells[3 * 64 + 3];  // grid cells of the neighbours (maxneighbors <= 64 on the GPU path)
    std::vector<int64_t> cells_big;
    int64_t* cl = cells;
    if (n > 64) {
        cells_big.resize(3 * (size_t)n);
        cl = cells_big.data();
    }
    for (int a = 0; a < n; ++a)
        if (nb[a] < P->N) P->cell(nb[a], cl + 3 * a);
    double h[3];
    for (int a = 0; a < n; ++a) {
        P->lag(g, nb[a], h);
        c[a] = P->cov(h);
        for (int b = 0; b <= a; ++b) K[(size_t)a * n + b] = P->cov_pair(nb[b], nb[a], cl + 3 * b, cl + 3 * a);
    }
    // Cholesky (lower, row a: L[a][b] for b <= a), pivot rule
    const double tau = kSingularTau * P->sill;
    for (int j = 0; j < n; ++j) {
        double s = K[(size_t)j * n + j];
        for (int l = 0; l < j; ++l) s -= K[(size_t)j * n + l] * K[(size_t)j * n + l];
        if (!(s > tau)) {  // seqsim.jl:127-131: status false -> prior
            P->status[g] = SGS_NODE_PRIOR_SINGULAR;
            P->sigma[g] = std::sqrt(P->sill);
            return;
        }
        double ljj = std::sqrt(s);
        K[(size_t)j * n + j] = ljj;
        for (int i = j + 1; i < n; ++i) {
            double t = K[(size_t)i * n + j];
            for (int l = 0; l < j; ++l) t -= K[(size_t)i * n + l] * K[(size_t)j * n + l];
            K[(size_t)i * n + j] = t / ljj;
        }
    }
    // forward and back substitution
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i) {
        double t = c[i];
        for (int l = 0; l < i; ++l) t -= K[(size_t)i * n + l] * y[l];
        y[i] = t / K[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double t = y[i];
        for (int l = i + 1; l < n; ++l) t -= K[(size_t)l * n + i] * w[l];
        w[i] = t / K[(size_t)i * n + i];
    }
    double wc = 0.0;
    for (int a = 0; a < n; ++a) wc += w[a] * c[a];
    double var = P->sill - wc;
    P->sigma[g] = std::sqrt(var > 0.0 ? var : 0.0);
    P->status[g] = SGS_NODE_KRIGED;
}

// Grid-lag covariance table, built once per plan before the first solve: lags
// up to twice the template's extent per axis (every pair of a node's grid
// neighbours), capped so the table stays below 2^22 entries.
static void build_lut(oracle_plan* P) {
    if (P->lut_e[0] >= 0) return;
    int64_t e[3] = {0, 0, 0}, total = 1;
    for (int j = 0; j < P->dim; ++j) e[j] = std::min<int64_t>(2 * P->tmpl_ext[j], P->n[j] - 1);
    for (;;) {
        total = 1;
        for (int j = 0; j < P->dim; ++j) total *= 2 * e[j] + 1;
        if (total <= ((int64_t)1 << 22)) break;
        for (int j = 0; j < P->dim; ++j) e[j] = e[j] * 3 / 4;
    }
    for (int j = 0; j < 3; ++j) {
        P->lut_e[j] = j < P->dim ? e[j] : 0;
        P->lut_w[j] = 2 * P->lut_e[j] + 1;
    }
    P->lut.assign((size_t)total, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < total; ++i) {
        int64_t r = i;
        double h[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < P->dim; ++j) {
            const int64_t L = r % P->lut_w[j] - P->lut_e[j];
            r /= P->lut_w[j];
            h[j] = (double)L * P->spacing[j];  // the lag() of a grid pair
        }
        P->lut[(size_t)i] = P->cov(h);
    }
}

extern "C" int oracle_solve(oracle_plan* P, int64_t t0, int64_t t1, int64_t stride, int nthreads) {
    if (!P) return fail(SGS_ERR_ARG, "null plan");
    build_lut(P);
    if (stride < 1) stride = 1;
    t0 = std::max<int64_t>(0, t0);
    t1 = std::min<int64_t>(P->N, t1);
    const int nt = nthreads_or_all(nthreads);
    int bad = 0;
#pragma omp parallel num_threads(nt)
    {
        std::vector<double> K, c;
#pragma omp for schedule(dynamic, 64) reduction(+ : bad)
        for (int64_t t = t0; t < t1; t += stride) {
            int64_t g = P->path[t];
            if (!P->searched[g]) { ++bad; continue; }
            solve_node(P, g, K, c);
        }
    }
    if (bad) return fail(SGS_ERR_STATE, "solve before search");
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Posterior mean of the process by simple kriging from the data alone
// (src/expectation/field/gaussian.jl:21-25: GeoStatsModels.fitpredict with
// Kriging(func, mean), restated): per node the k nearest data inside the
// neighbourhood in canonical order, the same FP64 SK system and Cholesky as
// solve_node, mean = mu + w'(d - mu), var = sill - w'c; NaN for fewer than
// nmin data or a singular system; the prior (mu, sill) when there is no data.
extern "C" int oracle_krige(oracle_plan* P, double* mean, double* var, int nthreads) {
    if (!P || !mean) return fail(SGS_ERR_ARG, "null argument");
    const double nan = std::nan("");
    if (P->D == 0) {
        for (int64_t g = 0; g < P->N; ++g) {
            mean[g] = P->mean;
            if (var) var[g] = P->sill;
        }
        return SGS_OK;
    }
    const int k = P->nmax;
    const int nt = nthreads_or_all(nthreads);
#pragma omp parallel num_threads(nt)
    {
        std::vector<Cand> data;
        std::vector<double> K, c;
#pragma omp for schedule(dynamic, 256)
        for (int64_t g = 0; g < P->N; ++g) {
            data_candidates(P, g, false, data);
            int32_t* nb = &P->nbr[(size_t)g * k];
            int m = 0;
            for (; m < k && m < (int)data.size(); ++m) nb[m] = (int32_t)data[m].idx;
            for (int q = m; q < k; ++q) nb[q] = -1;
            P->cnt[g] = m;
            P->searched[g] = 1;
            solve_node(P, g, K, c);
            if (P->status[g] != SGS_NODE_KRIGED) {
                mean[g] = nan;
                if (var) var[g] = nan;
                continue;
            }
            const double* w = &P->w[(size_t)g * k];
            double s = 0.0;
            for (int a = 0; a < m; ++a) s += w[a] * (P->dval[nb[a] - P->N] - P->mean);
            mean[g] = P->mean + s;
            if (var) var[g] = P->sigma[g] * P->sigma[g];
        }
    }
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw 2011, "Parallel random numbers:
// as easy as 1, 2, 3") and the Box-Muller transform; the seeded draws of the
// library follow the same definition.
static inline void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// uniform in (0,1) with 24 significant bits (exact in float and double)
static inline double u24(uint32_t x) { return (double)((x >> 9) * 2u + 1u) * (1.0 / 16777216.0); }

static inline double normal_of(uint64_t seed, int64_t g, int32_t r) {
    uint32_t c[4] = {(uint32_t)g, (uint32_t)((uint64_t)g >> 32), (uint32_t)(r >> 2), 0u};
    philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    int q = r & 3;
    double u0 = u24(c[q & 2]), u1 = u24(c[(q & 2) + 1]);
    double rad = std::sqrt(-2.0 * std::log(u0));
    const double two_pi = 6.283185307179586476925286766559;
    return (q & 1) ? rad * std::sin(two_pi * u1) : rad * std::cos(two_pi * u1);
}

extern "C" void oracle_normals(uint64_t seed, int64_t N, int32_t R, double* z) {
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < N; ++g)
        for (int32_t r = 0; r < R; ++r) z[(size_t)r * N + g] = normal_of(seed, g, r);
}

extern "C" int oracle_simulate(oracle_plan* P, int32_t R, const double* z, uint64_t seed,
                               double* out, int64_t t_end, int nthreads) {
    if (!P || !out || R < 0) return fail(SGS_ERR_ARG, "invalid argument");
    t_end = std::min<int64_t>(P->N, std::max<int64_t>(0, t_end));
    for (int64_t t = 0; t < t_end; ++t)
        if (!P->solved[P->path[t]]) return fail(SGS_ERR_STATE, "simulate before solve");
    const int nt = nthreads_or_all(nthreads);
    const int k = P->nmax;
    const double mu = P->mean, ssd = std::sqrt(P->sill);
#pragma omp parallel num_threads(nt)
    {
        std::vector<double> vals(P->N + P->D);
#pragma omp for schedule(dynamic, 1)
        for (int32_t r = 0; r < R; ++r) {
            std::fill(vals.begin(), vals.end(), std::nan(""));
            for (int64_t i = 0; i < P->D; ++i) vals[P->N + i] = P->dval[i];  // ExplicitInit
            for (int64_t t = 0; t < t_end; ++t) {
                const int64_t g = P->path[t];
                const double zz = z ? z[(size_t)r * P->N + g] : normal_of(seed, g, r);
                double v;
                if (P->status[g] != SGS_NODE_KRIGED) {
                    v = mu + ssd * zz;  // prior draw
                } else {
                    const int32_t* nb = &P->nbr[(size_t)g * k];
                    const double* w = &P->w[(size_t)g * k];
                    double m = mu;
                    for (int a = 0; a < P->cnt[g]; ++a) m += w[a] * (vals[nb[a]] - mu);
                    v = m + P->sigma[g] * zz;
                }
                vals[g] = v;
            }
            double* o = out + (size_t)r * P->N;
            for (int64_t g = 0; g < P->N; ++g) o[g] = vals[g];
        }
    }
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Sequential indicator simulation (IndicatorProcess + SEQSIM, seqsim.jl:
// 247-261 one-hot data, :292-310 Kriging(func, prob) with Categorical prior
// and conditional, :342-347 categorical draw), restated for a separable
// indicator covariance A_ab rho(h): every category's simple cokriging weights
// are rho's simple kriging weights w (this plan's solve), so
//   p_l = prob_l + sum_a w_a (I_l(x_a) - prob_l),
// clamped to [0, 1], normalized, and drawn from by the inverse cdf at u.
static inline double uniform_of(uint64_t seed, int64_t g, int32_t r) {
    uint32_t c[4] = {(uint32_t)g, (uint32_t)((uint64_t)g >> 32), (uint32_t)(r >> 2), 0x5349u};
    philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return u24(c[r & 3]);
}

extern "C" void oracle_uniforms(uint64_t seed, int64_t N, int32_t R, double* u) {
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < N; ++g)
        for (int32_t r = 0; r < R; ++r) u[(size_t)r * N + g] = uniform_of(seed, g, r);
}

extern "C" int oracle_simulate_indicator(oracle_plan* P, int32_t ncat, const double* prob, const int32_t* data_cat,
                                         int32_t R, const double* u, uint64_t seed, int32_t* out, int nthreads) {
    if (!P || !out || R < 0 || ncat < 2 || !prob) return fail(SGS_ERR_ARG, "invalid argument");
    double ps = 0.0;
    for (int l = 0; l < ncat; ++l) ps += prob[l];
    std::vector<double> pr(ncat);
    for (int l = 0; l < ncat; ++l) pr[l] = prob[l] / ps;
    const int k = P->nmax;
    const int nt = nthreads_or_all(nthreads);
#pragma omp parallel num_threads(nt)
    {
        std::vector<int32_t> cat(P->N + P->D);
        std::vector<double> p(ncat);
#pragma omp for schedule(dynamic, 1)
        for (int32_t r = 0; r < R; ++r) {
            std::fill(cat.begin(), cat.end(), -1);
            for (int64_t i = 0; i < P->D; ++i) cat[P->N + i] = data_cat[i];  // ExplicitInit
            for (int64_t t = 0; t < P->N; ++t) {
                const int64_t g = P->path[t];
                if (P->status[g] != SGS_NODE_KRIGED) {
                    for (int l = 0; l < ncat; ++l) p[l] = pr[l];
                } else {
                    const int32_t* nb = &P->nbr[(size_t)g * k];
                    const double* w = &P->w[(size_t)g * k];
                    for (int l = 0; l < ncat; ++l) {
                        double s = pr[l];
                        for (int a = 0; a < P->cnt[g]; ++a) s += w[a] * ((cat[nb[a]] == l ? 1.0 : 0.0) - pr[l]);
                        p[l] = s;
                    }
                }
                double tot = 0.0;
                for (int l = 0; l < ncat; ++l) {
                    p[l] = std::min(std::max(p[l], 0.0), 1.0);
                    tot += p[l];
                }
                if (!(tot > 0.0)) {
                    for (int l = 0; l < ncat; ++l) p[l] = pr[l];
                    tot = 1.0;
                }
                const double uu = u ? u[(size_t)r * P->N + g] : uniform_of(seed, g, r);
                int c = ncat - 1;
                double cum = 0.0;
                for (int l = 0; l < ncat - 1; ++l) {
                    cum += p[l] / tot;
                    if (uu < cum) {
                        c = l;
                        break;
                    }
                }
                cat[g] = c;
            }
            for (int64_t g = 0; g < P->N; ++g) out[(size_t)r * P->N + g] = cat[g];
        }
    }
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Sequential indicator simulation with full simple cokriging, for an
// indicator covariance given as a linear model of coregionalization
//   C_ab(h) = sum_s A_s[a][b] C_s(h),   C_s = sill_s - gamma_s (structure s)
// with the structures of the plan's (nested) variogram and symmetric L x L
// coefficient matrices A_s (coef: S x L x L, row-major).  With structures of
// different ranges the model is not separable, and every node solves the
// simple cokriging system of its n neighbours' L indicators (seqsim.jl:292-310,
// Kriging(f, prob) with a multivariate f): the (nL x nL) LHS has the blocks
// C(x_i - x_j), the L right-hand sides the blocks C(x_i - x_0); Cholesky with
// the canonical singular rule (a pivot not > 1e-10 x the largest variance
// sum_s A_s[a][a] sill_s); weights Lambda[(i, a), t] give
//   p_t = prob_t + sum_i sum_a Lambda[(i, a), t] (I_a(x_i) - prob_a),
// clamped to [0, 1], normalized and drawn from by the inverse cdf at u.
static double structure_cov(const oracle_plan* P, size_t s, const double* h) {
    bool zero = true;
    for (int j = 0; j < P->dim; ++j) zero = zero && (h[j] == 0.0);
    const sgs_variogram& v = P->vs[s];
    if (zero) return v.sill;
    const double hn = std::sqrt(P->vms[s].d2(h));
    double f;
    switch (v.type) {
        case SGS_SPHERICAL: f = hn < 1.0 ? 1.5 * hn - 0.5 * hn * hn * hn : 1.0; break;
        case SGS_EXPONENTIAL: f = 1.0 - std::exp(-3.0 * hn); break;
        default: f = 1.0 - std::exp(-3.0 * hn * hn); break;
    }
    return v.sill - (v.nugget + (v.sill - v.nugget) * f);
}

// Lower Cholesky factor F (L x L, zero above the diagonal) of the symmetric
// matrix S (lower triangle read); a pivot not above tau gives a zero column.
static void mv_factor(const double* S, int L, double tau, double* F) {
    for (int i = 0; i < L * L; ++i) F[i] = 0.0;
    for (int j = 0; j < L; ++j) {
        double d = S[j * L + j];
        for (int l = 0; l < j; ++l) d -= F[j * L + l] * F[j * L + l];
        if (!(d > tau)) continue;
        const double fjj = std::sqrt(d);
        F[j * L + j] = fjj;
        for (int i = j + 1; i < L; ++i) {
            double t = S[i * L + j];
            for (int l = 0; l < j; ++l) t -= F[i * L + l] * F[j * L + l];
            F[i * L + j] = t / fjj;
        }
    }
}

// The simple cokriging system of every node: status and Lambda (k*L x L);
// with `fac`, also the factor of the node's conditional covariance
// C(0) - c' Lambda (of C(0) for a node drawn from the prior).
static void cok_systems(oracle_plan* P, int L, const double* coef, double tau, std::vector<int8_t>& st,
                        std::vector<double>& lam, std::vector<double>* fac, int nt) {
    const int k = P->nmax, S = (int)P->vs.size();
    st.assign(P->N, (int8_t)SGS_NODE_PRIOR_NMIN);
    lam.assign((size_t)P->N * k * L * L, 0.0);
    std::vector<double> c0((size_t)L * L, 0.0);
    for (int a = 0; a < L; ++a)
        for (int b = 0; b < L; ++b)
            for (int s = 0; s < S; ++s) c0[(size_t)a * L + b] += coef[((size_t)s * L + a) * L + b] * P->vs[s].sill;
    if (fac) {
        fac->assign((size_t)P->N * L * L, 0.0);
        std::vector<double> f0((size_t)L * L);
        mv_factor(c0.data(), L, tau, f0.data());
        for (int64_t g = 0; g < P->N; ++g) std::copy(f0.begin(), f0.end(), fac->begin() + (size_t)g * L * L);
    }
#pragma omp parallel num_threads(nt)
    {
        std::vector<double> K, c, cs(S);
        double h[3];
#pragma omp for schedule(dynamic, 64)
        for (int64_t g = 0; g < P->N; ++g) {
            const int n = P->cnt[g];
            if (n < P->nmin) continue;
            const int m = n * L;
            const int32_t* nb = &P->nbr[(size_t)g * k];
            K.assign((size_t)m * m, 0.0);
            c.assign((size_t)m * L, 0.0);
            for (int i = 0; i < n; ++i) {
                P->lag(g, nb[i], h);
                for (int s = 0; s < S; ++s) cs[s] = structure_cov(P, s, h);
                for (int a = 0; a < L; ++a)
                    for (int t = 0; t < L; ++t) {
                        double v = 0.0;
                        for (int s = 0; s < S; ++s) v += coef[((size_t)s * L + a) * L + t] * cs[s];
                        c[(size_t)(i * L + a) * L + t] = v;
                    }
                for (int j = 0; j <= i; ++j) {
                    P->lag(nb[j], nb[i], h);
                    for (int s = 0; s < S; ++s) cs[s] = structure_cov(P, s, h);
                    for (int a = 0; a < L; ++a)
                        for (int b = 0; b < L; ++b) {
                            const int r = i * L + a, q = j * L + b;
                            if (q > r) continue;
                            double v = 0.0;
                            for (int s = 0; s < S; ++s) v += coef[((size_t)s * L + a) * L + b] * cs[s];
                            K[(size_t)r * m + q] = v;
                        }
                }
            }
            bool ok = true;
            for (int j = 0; j < m && ok; ++j) {
                double sj = K[(size_t)j * m + j];
                for (int l = 0; l < j; ++l) sj -= K[(size_t)j * m + l] * K[(size_t)j * m + l];
                if (!(sj > tau)) {
                    ok = false;
                    break;
                }
                const double ljj = std::sqrt(sj);
                K[(size_t)j * m + j] = ljj;
                for (int i = j + 1; i < m; ++i) {
                    double t = K[(size_t)i * m + j];
                    for (int l = 0; l < j; ++l) t -= K[(size_t)i * m + l] * K[(size_t)j * m + l];
                    K[(size_t)i * m + j] = t / ljj;
                }
            }
            if (!ok) {
                st[g] = (int8_t)SGS_NODE_PRIOR_SINGULAR;
                continue;
            }
            double* lg = &lam[(size_t)g * k * L * L];
            std::vector<double> y(m);
            for (int t = 0; t < L; ++t) {
                for (int i = 0; i < m; ++i) {
                    double v = c[(size_t)i * L + t];
                    for (int l = 0; l < i; ++l) v -= K[(size_t)i * m + l] * y[l];
                    y[i] = v / K[(size_t)i * m + i];
                }
                for (int i = m - 1; i >= 0; --i) {
                    double v = y[i];
                    for (int l = i + 1; l < m; ++l) v -= K[(size_t)l * m + i] * lg[(size_t)l * L + t];
                    lg[(size_t)i * L + t] = v / K[(size_t)i * m + i];
                }
            }
            st[g] = (int8_t)SGS_NODE_KRIGED;
            if (fac) {
                std::vector<double> sg((size_t)L * L);
                for (int t = 0; t < L; ++t)
                    for (int u = 0; u <= t; ++u) {
                        double v = c0[(size_t)t * L + u];
                        for (int r = 0; r < m; ++r) v -= c[(size_t)r * L + t] * lg[(size_t)r * L + u];
                        sg[(size_t)t * L + u] = v;
                    }
                mv_factor(sg.data(), L, tau, fac->data() + (size_t)g * L * L);
            }
        }
    }
}

extern "C" int oracle_simulate_cokriging(oracle_plan* P, int32_t ncat, const double* prob, const int32_t* data_cat,
                                         const double* coef, int32_t R, const double* u, uint64_t seed, int32_t* out,
                                         int nthreads) {
    if (!P || !out || R < 0 || ncat < 2 || ncat > 8 || !prob || !coef) return fail(SGS_ERR_ARG, "invalid argument");
    const int L = ncat, k = P->nmax, S = (int)P->vs.size();
    if (k * L > 64) return fail(SGS_ERR_ARG, "maxneighbors x categories above 64");
    double ps = 0.0;
    for (int l = 0; l < L; ++l) ps += prob[l];
    std::vector<double> pr(L);
    for (int l = 0; l < L; ++l) pr[l] = prob[l] / ps;
    double vmax = 0.0;  // largest variance of an indicator
    for (int a = 0; a < L; ++a) {
        double v = 0.0;
        for (int s = 0; s < S; ++s) v += coef[((size_t)s * L + a) * L + a] * P->vs[s].sill;
        vmax = std::max(vmax, v);
    }
    const double tau = kSingularTau * vmax;
    const int nt = nthreads_or_all(nthreads);
    std::vector<int8_t> st;
    std::vector<double> lam;
    cok_systems(P, L, coef, tau, st, lam, nullptr, nt);
    for (int64_t g = 0; g < P->N; ++g) P->status[g] = st[g];
#pragma omp parallel num_threads(nt)
    {
        std::vector<int32_t> cat(P->N + P->D);
        std::vector<double> p(L);
#pragma omp for schedule(dynamic, 1)
        for (int32_t r = 0; r < R; ++r) {
            std::fill(cat.begin(), cat.end(), -1);
            for (int64_t i = 0; i < P->D; ++i) cat[P->N + i] = data_cat[i];  // ExplicitInit
            for (int64_t t = 0; t < P->N; ++t) {
                const int64_t g = P->path[t];
                for (int l = 0; l < L; ++l) p[l] = pr[l];
                if (st[g] == SGS_NODE_KRIGED) {
                    const int32_t* nb = &P->nbr[(size_t)g * k];
                    const double* lg = &lam[(size_t)g * k * L * L];
                    for (int i = 0; i < P->cnt[g]; ++i)
                        for (int a = 0; a < L; ++a) {
                            const double ind = (cat[nb[i]] == a ? 1.0 : 0.0) - pr[a];
                            for (int l = 0; l < L; ++l) p[l] += lg[(size_t)(i * L + a) * L + l] * ind;
                        }
                }
                double tot = 0.0;
                for (int l = 0; l < L; ++l) {
                    p[l] = std::min(std::max(p[l], 0.0), 1.0);
                    tot += p[l];
                }
                if (!(tot > 0.0)) {
                    for (int l = 0; l < L; ++l) p[l] = pr[l];
                    tot = 1.0;
                }
                const double uu = u ? u[(size_t)r * P->N + g] : uniform_of(seed, g, r);
                int cc = L - 1;
                double cum = 0.0;
                for (int l = 0; l < L - 1; ++l) {
                    cum += p[l] / tot;
                    if (uu < cum) {
                        cc = l;
                        break;
                    }
                }
                cat[g] = cc;
            }
            for (int64_t g = 0; g < P->N; ++g) out[(size_t)r * P->N + g] = cat[g];
        }
    }
    return SGS_OK;
}

// ---------------------------------------------------------------------------
// Multivariate Gaussian simulation: a GaussianProcess(func, mean) whose func
// is a linear model of coregionalization over the plan's structures
// (src/processes/field/gaussian.jl:22-35; seqsim.jl:277-290 Kriging(func,
// mean) and the prior MvNormal(mean, sill(func)); :302-304 predictprob's
// MvNormal conditional; :335-340 one draw sets all variables of a node).
// Per node, the simple cokriging system of its n neighbours' L values (the
// same LHS, right-hand sides and singular rule as the indicator form above):
//   mu^_t = mean_t + sum_i sum_a Lambda[(i, a), t] (v_a(x_i) - mean_a),
//   v = mu^ + F z,  F the lower Cholesky factor of C(0) - c' Lambda
// (of C(0) for a prior node; a pivot not above the singular threshold gives a
// zero column).  z[(r L + a) N + g], or the normals of pseudo-node a N + g;
// out[(r L + a) N + g].
extern "C" int oracle_simulate_multivariate(oracle_plan* P, int32_t nvars, const double* mean, const double* coef,
                                            const double* data_val, int32_t R, const double* z, uint64_t seed,
                                            double* out, int nthreads) {
    if (!P || !out || R < 0 || nvars < 1 || nvars > 8 || !mean || !coef || (P->D > 0 && !data_val))
        return fail(SGS_ERR_ARG, "invalid argument");
    const int L = nvars, k = P->nmax, S = (int)P->vs.size();
    if (k * L > 64) return fail(SGS_ERR_ARG, "maxneighbors x variables above 64");
    double vmax = 0.0;  // largest variance of a variable
    for (int a = 0; a < L; ++a) {
        double v = 0.0;
        for (int s = 0; s < S; ++s) v += coef[((size_t)s * L + a) * L + a] * P->vs[s].sill;
        vmax = std::max(vmax, v);
    }
    if (!(vmax > 0.0)) return fail(SGS_ERR_ARG, "the model's variances must be positive");
    const double tau = kSingularTau * vmax;
    const int nt = nthreads_or_all(nthreads);
    std::vector<int8_t> st;
    std::vector<double> lam, fac;
    cok_systems(P, L, coef, tau, st, lam, &fac, nt);
    for (int64_t g = 0; g < P->N; ++g) P->status[g] = st[g];
    const int64_t N = P->N;
#pragma omp parallel num_threads(nt)
    {
        std::vector<double> vals((size_t)(N + P->D) * L), mu(L), zz(L);
#pragma omp for schedule(dynamic, 1)
        for (int32_t r = 0; r < R; ++r) {
            std::fill(vals.begin(), vals.end(), std::nan(""));
            for (int64_t i = 0; i < P->D * L; ++i) vals[(size_t)N * L + i] = data_val[i];  // ExplicitInit
            for (int64_t t = 0; t < N; ++t) {
                const int64_t g = P->path[t];
                for (int l = 0; l < L; ++l) mu[l] = mean[l];
                if (st[g] == SGS_NODE_KRIGED) {
                    const int32_t* nb = &P->nbr[(size_t)g * k];
                    const double* lg = &lam[(size_t)g * k * L * L];
                    for (int i = 0; i < P->cnt[g]; ++i)
                        for (int a = 0; a < L; ++a) {
                            const double d = vals[(size_t)nb[i] * L + a] - mean[a];
                            for (int l = 0; l < L; ++l) mu[l] += lg[(size_t)(i * L + a) * L + l] * d;
                        }
                }
                for (int a = 0; a < L; ++a)
                    zz[a] = z ? z[((size_t)r * L + a) * N + g] : normal_of(seed, (int64_t)a * N + g, r);
                const double* F = &fac[(size_t)g * L * L];
                for (int l = 0; l < L; ++l) {
                    double v = mu[l];
                    for (int u = 0; u <= l; ++u) v += F[l * L + u] * zz[u];
                    vals[(size_t)g * L + l] = v;
                }
            }
            for (int a = 0; a < L; ++a)
                for (int64_t g = 0; g < N; ++g) out[((size_t)r * L + a) * N + g] = vals[(size_t)g * L + a];
        }
    }
    return SGS_OK;
}

extern "C" int oracle_neighbors(const oracle_plan* P, int32_t* idx, int32_t* count) {
    if (!P) return fail(SGS_ERR_ARG, "null plan");
    if (idx) std::memcpy(idx, P->nbr.data(), P->nbr.size() * sizeof(int32_t));
    if (count) std::memcpy(count, P->cnt.data(), P->cnt.size() * sizeof(int32_t));
    return SGS_OK;
}

extern "C" int oracle_weights(const oracle_plan* P, double* w, double* sigma, int32_t* status) {
    if (!P) return fail(SGS_ERR_ARG, "null plan");
    if (w) std::memcpy(w, P->w.data(), P->w.size() * sizeof(double));
    if (sigma) std::memcpy(sigma, P->sigma.data(), P->sigma.size() * sizeof(double));
    if (status) std::memcpy(status, P->status.data(), P->status.size() * sizeof(int32_t));
    return SGS_OK;
}

extern "C" int oracle_levels(const oracle_plan* P, int32_t* level, int32_t* nlevels) {
    if (!P) return fail(SGS_ERR_ARG, "null plan");
    std::vector<int32_t> lv(P->N, 0);
    int32_t mx = -1;
    for (int64_t t = 0; t < P->N; ++t) {
        const int64_t g = P->path[t];
        int32_t l = 0;
        for (int a = 0; a < P->cnt[g]; ++a) {
            int32_t c = P->nbr[(size_t)g * P->nmax + a];
            if (c < P->N) l = std::max(l, lv[c] + 1);
        }
        lv[g] = l;
        mx = std::max(mx, l);
    }
    if (level) std::memcpy(level, lv.data(), lv.size() * sizeof(int32_t));
    if (nlevels) *nlevels = mx + 1;
    return SGS_OK;
}

extern "C" double oracle_covariance(const sgs_variogram* v, int32_t dim, const double* lag) {
    oracle_plan P;
    P.dim = dim;
    P.vario = *v;
    P.vs.assign(1, *v);
    P.vms.emplace_back();
    set_metric(P.vms.back(), dim, 1, v->ranges, v->rotation);
    P.sill = v->sill;
    set_metric(P.vmetric, dim, 1, v->ranges, v->rotation);
    double h[3] = {lag[0], lag[1], dim == 3 ? lag[2] : 0.0};
    return P.cov(h);
}

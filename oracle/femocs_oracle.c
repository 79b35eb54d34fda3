/* CPU oracle for the femocs_gb300 field-solve path -- TEST INFRASTRUCTURE ONLY.
 * See femocs_oracle.h for scope and pinning status. Compiled with -ffp-contract=off so the
 * floating-point operation sequence is the one written here on every host. */
#define _POSIX_C_SOURCE 199309L
#include "femocs_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

void orc_free(void* p) { free(p); }

/* ------------------------------------------------------------------ small vector algebra */
typedef struct { double x, y, z; } V3;

static double det2v(V3 a, V3 b) { /* a.x*(b.y-b.z) - a.y*(b.x-b.z) + a.z*(b.x-b.y) */
    return a.x * (b.y - b.z) - a.y * (b.x - b.z) + a.z * (b.x - b.y);
}
static double det3v(V3 a, V3 b, V3 c) {
    return a.x * (b.y * c.z - c.y * b.z) - b.x * (a.y * c.z - c.y * a.z) + c.x * (a.y * b.z - b.y * a.z);
}
static V3 ld3(const double* xyz, int i) { V3 v = {xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2]}; return v; }

/* ------------------------------------------------------------------ tet tables */
/* LinearTetrahedra::precompute, src/InterpolatorCells.cpp:560-628 */
void orc_tet_tables(int n_tets, const int32_t* tets, const double* xyz, double* det, double* centroid) {
    for (int t = 0; t < n_tets; ++t) {
        const int32_t* e = tets + 4 * (size_t)t;
        V3 v1 = ld3(xyz, e[0]), v2 = ld3(xyz, e[1]), v3 = ld3(xyz, e[2]), v4 = ld3(xyz, e[3]);
        double* d = det + 17 * (size_t)t;
        double a1 = det3v(v2, v3, v4), a2 = det3v(v1, v3, v4), a3 = det3v(v1, v2, v4), a4 = det3v(v1, v2, v3);
        d[0] = 1.0 / (a4 - a3 + a2 - a1);
        V3 P[4][3] = {{v2, v3, v4}, {v1, v3, v4}, {v1, v2, v4}, {v1, v2, v3}};
        for (int k = 0; k < 4; ++k) {
            V3 p = P[k][0], q = P[k][1], r = P[k][2];
            V3 ys = {p.y, q.y, r.y}, zs = {p.z, q.z, r.z}, xs = {p.x, q.x, r.x};
            /* the fourth minor is taken on the points, the others on the transposed vectors
             * (src/InterpolatorCells.cpp:586-626) */
            double m1 = det2v(ys, zs), m2 = det2v(xs, zs), m3 = det2v(xs, ys);
            double m4 = k == 3 ? det3v(p, q, r) : det3v(xs, ys, zs);
            double* o = d + 1 + 4 * k;
            if (k % 2 == 0) { o[0] = m1; o[1] = -m2; o[2] = m3; o[3] = -m4; }
            else { o[0] = -m1; o[1] = m2; o[2] = -m3; o[3] = m4; }
        }
        double cx = 0.0, cy = 0.0, cz = 0.0;
        for (int k = 0; k < 4; ++k) { V3 v = ld3(xyz, e[k]); cx += v.x; cy += v.y; cz += v.z; }
        centroid[3 * (size_t)t] = cx * (1.0 / 4);
        centroid[3 * (size_t)t + 1] = cy * (1.0 / 4);
        centroid[3 * (size_t)t + 2] = cz * (1.0 / 4);
    }
}

/* ------------------------------------------------------------------ FEM system */
/* femocs hex order: reference coordinates of the 8 nodes (src/InterpolatorCells.cpp:1319-1331) */
static const double HX[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const double HY[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const double HZ[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
/* the six faces of a hex in femocs order, vertices in cyclic order */
static const int HFACE[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}, {0, 1, 5, 4}, {3, 2, 6, 7}};

/* Q1 element stiffness with QGauss<3>(2) on the trilinear map (src/PoissonSolver.cpp:239-263) */
static void q1_element(const double X[8][3], double K[8][8]) {
    const double g = 1.0 / sqrt(3.0);
    memset(K, 0, sizeof(double) * 64);
    for (int q = 0; q < 8; ++q) {
        const double xi = (q & 1) ? g : -g, eta = (q & 2) ? g : -g, zeta = (q & 4) ? g : -g;
        double dN[8][3];
        for (int k = 0; k < 8; ++k) {
            dN[k][0] = HX[k] * (1 + eta * HY[k]) * (1 + zeta * HZ[k]) * 0.125;
            dN[k][1] = (1 + xi * HX[k]) * HY[k] * (1 + zeta * HZ[k]) * 0.125;
            dN[k][2] = (1 + xi * HX[k]) * (1 + eta * HY[k]) * HZ[k] * 0.125;
        }
        double J[3][3] = {{0}};  /* J[a][b] = d x_a / d xi_b */
        for (int k = 0; k < 8; ++k)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) J[a][b] += X[k][a] * dN[k][b];
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        double inv[3][3];
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        double G[8][3];  /* grad_x N_k = J^{-T} grad_xi N_k */
        for (int k = 0; k < 8; ++k)
            for (int a = 0; a < 3; ++a)
                G[k][a] = inv[0][a] * dN[k][0] + inv[1][a] * dN[k][1] + inv[2][a] * dN[k][2];
        const double jxw = fabs(det);
        for (int i = 0; i < 8; ++i)
            for (int j = 0; j < 8; ++j)
                K[i][j] += jxw * (G[i][0] * G[j][0] + G[i][1] * G[j][1] + G[i][2] * G[j][2]);
    }
}

typedef struct { int32_t v[4]; int32_t s[4]; int32_t cell; int8_t face; } FaceKey;
static int cmp_face(const void* a, const void* b) {
    const FaceKey* x = (const FaceKey*)a;
    const FaceKey* y = (const FaceKey*)b;
    for (int k = 0; k < 4; ++k) {
        if (x->s[k] != y->s[k]) return x->s[k] < y->s[k] ? -1 : 1;
    }
    if (x->cell != y->cell) return x->cell < y->cell ? -1 : 1;
    return x->face - y->face;
}
static void sort4(int32_t* a) {
    for (int i = 1; i < 4; ++i) {
        int32_t v = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
        a[j + 1] = v;
    }
}
static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

static int64_t find_col(const OrcSystem* s, int r, int c) {
    int64_t lo = s->rowptr[r], hi = s->rowptr[r + 1] - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) / 2;
        if (s->col[mid] == c) return mid;
        if (s->col[mid] < c) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

int orc_build_system(int n_vert, const double* xyz, int n_cells, const int32_t* cells,
                     double applied_field, int anode_dirichlet, double applied_potential, OrcSystem* sys) {
    memset(sys, 0, sizeof(*sys));
    sys->n = n_vert;
    /* ---- sparsity: all vertex pairs sharing a cell (DoFTools::make_sparsity_pattern) */
    int64_t npairs = 64 * (int64_t)n_cells;
    int64_t* keys = (int64_t*)malloc(sizeof(int64_t) * (size_t)npairs);
    if (!keys) return 1;
    for (int c = 0; c < n_cells; ++c)
        for (int i = 0; i < 8; ++i)
            for (int j = 0; j < 8; ++j)
                keys[64 * (int64_t)c + 8 * i + j] = ((int64_t)cells[8 * (size_t)c + i] << 32) | (uint32_t)cells[8 * (size_t)c + j];
    qsort(keys, (size_t)npairs, sizeof(int64_t), cmp_i64);
    int64_t nnz = 0;
    for (int64_t k = 0; k < npairs; ++k)
        if (k == 0 || keys[k] != keys[k - 1]) keys[nnz++] = keys[k];
    sys->nnz = nnz;
    sys->rowptr = (int64_t*)calloc((size_t)n_vert + 1, sizeof(int64_t));
    sys->col = (int32_t*)malloc(sizeof(int32_t) * (size_t)nnz);
    sys->val = (double*)calloc((size_t)nnz, sizeof(double));
    sys->rhs = (double*)calloc((size_t)n_vert, sizeof(double));
    sys->x = (double*)calloc((size_t)n_vert, sizeof(double));
    sys->constrained = (int8_t*)calloc((size_t)n_vert, 1);
    for (int64_t k = 0; k < nnz; ++k) {
        sys->rowptr[(keys[k] >> 32) + 1]++;
        sys->col[k] = (int32_t)(keys[k] & 0xffffffff);
    }
    for (int i = 0; i < n_vert; ++i) sys->rowptr[i + 1] += sys->rowptr[i];
    free(keys);

    /* ---- stiffness */
    for (int c = 0; c < n_cells; ++c) {
        double X[8][3], K[8][8];
        const int32_t* cv = cells + 8 * (size_t)c;
        for (int k = 0; k < 8; ++k)
            for (int a = 0; a < 3; ++a) X[k][a] = xyz[3 * (size_t)cv[k] + a];
        q1_element(X, K);
        for (int i = 0; i < 8; ++i)
            for (int j = 0; j < 8; ++j) sys->val[find_col(sys, cv[i], cv[j])] += K[i][j];
    }

    /* ---- boundary faces: faces of exactly one cell */
    int64_t nf = 6 * (int64_t)n_cells;
    FaceKey* fk = (FaceKey*)malloc(sizeof(FaceKey) * (size_t)nf);
    for (int c = 0; c < n_cells; ++c)
        for (int f = 0; f < 6; ++f) {
            FaceKey* k = &fk[6 * (int64_t)c + f];
            for (int q = 0; q < 4; ++q) k->v[q] = k->s[q] = cells[8 * (size_t)c + HFACE[f][q]];
            sort4(k->s);
            k->cell = c;
            k->face = (int8_t)f;
        }
    qsort(fk, (size_t)nf, sizeof(FaceKey), cmp_face);
    int64_t nb = 0;
    for (int64_t i = 0; i < nf;) {
        int64_t j = i + 1;
        while (j < nf && memcmp(fk[j].s, fk[i].s, sizeof(fk[i].s)) == 0) ++j;
        if (j - i == 1) fk[nb++] = fk[i];
        i = j;
    }
    double* ctr = (double*)malloc(sizeof(double) * 3 * (size_t)(nb ? nb : 1));
    double mn[3] = {1e16, 1e16, 1e16}, mx[3] = {-1e16, -1e16, -1e16};
    for (int64_t i = 0; i < nb; ++i)
        for (int a = 0; a < 3; ++a) {
            double s = 0.0;
            for (int q = 0; q < 4; ++q) s += xyz[3 * (size_t)fk[i].v[q] + a];
            ctr[3 * i + a] = s / 4.0;
            if (ctr[3 * i + a] > mx[a]) mx[a] = ctr[3 * i + a];
            if (ctr[3 * i + a] < mn[a]) mn[a] = ctr[3 * i + a];
        }
    const double eps = 1e-6;
    const double gp = 1.0 / sqrt(3.0);
    int n_top = 0;
    for (int64_t i = 0; i < nb; ++i) {
        const double x = ctr[3 * i], y = ctr[3 * i + 1], z = ctr[3 * i + 2];
        int side = fabs(x - mn[0]) <= eps || fabs(x - mx[0]) <= eps || fabs(y - mn[1]) <= eps || fabs(y - mx[1]) <= eps;
        int top = !side && fabs(z - mx[2]) <= eps;
        if (side) continue;
        if (top) {
            ++n_top;
            if (anode_dirichlet) {
                for (int q = 0; q < 4; ++q) { sys->constrained[fk[i].v[q]] = 2; }
                continue;
            }
            /* Neumann: b_i += sum_q N_i * bc * JxW over a 2x2 Gauss rule on the face */
            double P[4][3];
            for (int q = 0; q < 4; ++q)
                for (int a = 0; a < 3; ++a) P[q][a] = xyz[3 * (size_t)fk[i].v[q] + a];
            for (int qp = 0; qp < 4; ++qp) {
                const double s = (qp & 1) ? gp : -gp, t = (qp & 2) ? gp : -gp;
                const double N[4] = {0.25 * (1 - s) * (1 - t), 0.25 * (1 + s) * (1 - t),
                                     0.25 * (1 + s) * (1 + t), 0.25 * (1 - s) * (1 + t)};
                double ds[3], dt[3];
                for (int a = 0; a < 3; ++a) {
                    ds[a] = 0.25 * (-(1 - t) * P[0][a] + (1 - t) * P[1][a] + (1 + t) * P[2][a] - (1 + t) * P[3][a]);
                    dt[a] = 0.25 * (-(1 - s) * P[0][a] - (1 + s) * P[1][a] + (1 + s) * P[2][a] + (1 - s) * P[3][a]);
                }
                const double cx = ds[1] * dt[2] - ds[2] * dt[1], cy = ds[2] * dt[0] - ds[0] * dt[2],
                             cz = ds[0] * dt[1] - ds[1] * dt[0];
                const double jxw = sqrt(cx * cx + cy * cy + cz * cz);
                for (int q = 0; q < 4; ++q) sys->rhs[fk[i].v[q]] += N[q] * applied_field * jxw;
            }
        } else {
            /* bottom and the vacuum-metal interface: copper, phi = 0 */
            for (int q = 0; q < 4; ++q) sys->constrained[fk[i].v[q]] = 1;
        }
    }
    sys->n_top_faces = n_top;
    free(ctr);
    free(fk);

    /* ---- Dirichlet elimination (deal.II apply_boundary_values, eliminate_columns=true) */
    double* g = (double*)calloc((size_t)n_vert, sizeof(double));
    for (int i = 0; i < n_vert; ++i)
        if (sys->constrained[i] == 2) g[i] = applied_potential;
    for (int r = 0; r < n_vert; ++r) {
        if (sys->constrained[r]) {
            double diag = 0;
            for (int64_t k = sys->rowptr[r]; k < sys->rowptr[r + 1]; ++k) {
                if (sys->col[k] == r) diag = sys->val[k];
                else sys->val[k] = 0.0;
            }
            sys->rhs[r] = g[r] * diag;
            sys->x[r] = g[r];
        } else {
            for (int64_t k = sys->rowptr[r]; k < sys->rowptr[r + 1]; ++k) {
                int c = sys->col[k];
                if (sys->constrained[c]) {
                    sys->rhs[r] -= sys->val[k] * g[c];
                    sys->val[k] = 0.0;
                }
            }
        }
    }
    for (int i = 0; i < n_vert; ++i) sys->constrained[i] = sys->constrained[i] ? 1 : 0;
    free(g);
    return 0;
}

int orc_system_from_csr(int n, const int64_t* rowptr, const int32_t* col, const double* val, const double* rhs,
                        const double* x0, OrcSystem* sys) {
    memset(sys, 0, sizeof(*sys));
    sys->n = n;
    sys->nnz = rowptr[n];
    sys->rowptr = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
    sys->col = (int32_t*)malloc(sizeof(int32_t) * (size_t)sys->nnz);
    sys->val = (double*)malloc(sizeof(double) * (size_t)sys->nnz);
    sys->rhs = (double*)malloc(sizeof(double) * (size_t)n);
    sys->x = (double*)malloc(sizeof(double) * (size_t)n);
    sys->constrained = (int8_t*)calloc((size_t)n, 1);
    if (!sys->rowptr || !sys->col || !sys->val || !sys->rhs || !sys->x || !sys->constrained) return 1;
    memcpy(sys->rowptr, rowptr, sizeof(int64_t) * ((size_t)n + 1));
    memcpy(sys->col, col, sizeof(int32_t) * (size_t)sys->nnz);
    memcpy(sys->val, val, sizeof(double) * (size_t)sys->nnz);
    memcpy(sys->rhs, rhs, sizeof(double) * (size_t)n);
    if (x0) memcpy(sys->x, x0, sizeof(double) * (size_t)n);
    else memset(sys->x, 0, sizeof(double) * (size_t)n);
    return 0;
}

void orc_free_system(OrcSystem* s) {
    free(s->rowptr); free(s->col); free(s->val); free(s->rhs); free(s->x); free(s->constrained);
    memset(s, 0, sizeof(*s));
}

/* threads of the SpMV and vector operations of the CG (the SSOR sweeps stay sequential, as
 * deal.II's PreconditionSSOR); 1 (default) keeps every sum in a fixed order */
static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n > 0 ? n : 1; }

void orc_spmv(const OrcSystem* s, const double* x, double* y) {
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int r = 0; r < s->n; ++r) {
        double acc = 0.0;
        for (int64_t k = s->rowptr[r]; k < s->rowptr[r + 1]; ++k) acc += s->val[k] * x[s->col[k]];
        y[r] = acc;
    }
}

/* ||b - A x||_2 with every row's dot product compensated (Dot2 of Ogita, Rump and Oishi,
 * SIAM J. Sci. Comput. 26, 2005: FMA-split products, TwoSum additions), and the FP64
 * rounding floor of a plain evaluation, 2^-53 ||(|b| + |A||x|)||_2 */
void orc_residual_comp(const OrcSystem* s, const double* x, double* out2) {
    double rr = 0.0, ff = 0.0;
    for (int r = 0; r < s->n; ++r) {
        double p = s->rhs[r], err = 0.0, mag = fabs(s->rhs[r]);
        for (int64_t k = s->rowptr[r]; k < s->rowptr[r + 1]; ++k) {
            const double a = -s->val[k], xv = x[s->col[k]];
            const double h = a * xv, e = fma(a, xv, -h);
            const double t = p + h, z = t - p, q = (p - (t - z)) + (h - z);
            p = t;
            err += q + e;
            mag += fabs(h);
        }
        const double ri = p + err;
        rr += ri * ri;
        ff += mag * mag;
    }
    out2[0] = sqrt(rr);
    out2[1] = ldexp(sqrt(ff), -53);
}

static double dot(int n, const double* a, const double* b) {
    double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(g_threads) if (g_threads > 1)
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* SparseMatrix::precondition_SSOR semantics (forward sweep, scaling by om*(2-om)*a_ii,
 * backward sweep), as used by deal.II PreconditionSSOR */
static void ssor_apply(const OrcSystem* s, const double* src, double* dst, double om, const double* diag) {
    const int n = s->n;
    for (int r = 0; r < n; ++r) {
        double v = src[r];
        for (int64_t k = s->rowptr[r]; k < s->rowptr[r + 1]; ++k) {
            int c = s->col[k];
            if (c >= r) break;
            v -= om * s->val[k] * dst[c];
        }
        dst[r] = v / diag[r];
    }
    for (int r = 0; r < n; ++r) dst[r] *= om * (2. - om) * diag[r];
    for (int r = n - 1; r >= 0; --r) {
        double v = dst[r];
        for (int64_t k = s->rowptr[r + 1] - 1; k >= s->rowptr[r]; --k) {
            int c = s->col[k];
            if (c <= r) break;
            v -= om * s->val[k] * dst[c];
        }
        dst[r] = v / diag[r];
    }
}

/* SolverCG::solve (deal.II 9.2) with SolverControl(max_it, tol): success when the residual
 * norm <= tol, failure when the step count reaches max_it. */
static int cg_core(const OrcSystem* s, double* x, int precond /*0 id,1 ssor,2 jacobi*/, double om,
                   double tol, int max_it, int fixed_it) {
    const int n = s->n;
    double* g = (double*)malloc(sizeof(double) * (size_t)n);
    double* h = (double*)malloc(sizeof(double) * (size_t)n);
    double* d = (double*)malloc(sizeof(double) * (size_t)n);
    double* Ad = (double*)malloc(sizeof(double) * (size_t)n);
    double* diag = (double*)malloc(sizeof(double) * (size_t)n);
    for (int r = 0; r < n; ++r) {
        diag[r] = 1.0;
        for (int64_t k = s->rowptr[r]; k < s->rowptr[r + 1]; ++k)
            if (s->col[k] == r) diag[r] = s->val[k];
    }
#define PREC(src, dst)                                                     \
    do {                                                                   \
        if (precond == 1) ssor_apply(s, src, dst, om, diag);               \
        else if (precond == 2) for (int i_ = 0; i_ < n; ++i_) dst[i_] = src[i_] / diag[i_]; \
        else memcpy(dst, src, sizeof(double) * (size_t)n);                 \
    } while (0)
    orc_spmv(s, x, g);
    for (int i = 0; i < n; ++i) g[i] -= s->rhs[i];
    double res = sqrt(dot(n, g, g));
    int it = 0, status = 0; /* 0 iterate, 1 success, -1 failure */
    if (!fixed_it) status = res <= tol ? 1 : (0 >= max_it ? -1 : 0);
    if (status == 0) {
        PREC(g, h);
        for (int i = 0; i < n; ++i) d[i] = -h[i];
        double gh = dot(n, g, h);
        while (1) {
            ++it;
            orc_spmv(s, d, Ad);
            double alpha = dot(n, d, Ad);
            alpha = gh / alpha;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
            for (int i = 0; i < n; ++i) x[i] += alpha * d[i];
            double gg = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : gg) num_threads(g_threads) if (g_threads > 1)
            for (int i = 0; i < n; ++i) { g[i] += alpha * Ad[i]; gg += g[i] * g[i]; }
            res = sqrt(fabs(gg));
            if (fixed_it) { if (it >= fixed_it) break; }
            else {
                if (res <= tol) { status = 1; break; }
                if (it >= max_it || res != res) { status = -1; break; }
            }
            PREC(g, h);
            double beta = gh;
            gh = dot(n, g, h);
            beta = gh / beta;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
            for (int i = 0; i < n; ++i) d[i] = beta * d[i] - h[i];
        }
    }
#undef PREC
    free(g); free(h); free(d); free(Ad); free(diag);
    return status < 0 ? -it : it;
}

int orc_ssor_cg(const OrcSystem* s, double* x, double omega, double tol, int max_it) {
    return cg_core(s, x, omega > 0 ? 1 : 0, omega, tol, max_it, 0);
}
int orc_jacobi_cg(const OrcSystem* s, double* x, double tol, int max_it) {
    return cg_core(s, x, 2, 0.0, tol, max_it, 0);
}
double orc_ssor_cg_fixed(const OrcSystem* s, double* x, double omega, int n_it) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    cg_core(s, x, omega > 0 ? 1 : 0, omega, 0.0, n_it, n_it);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------------------------ nodal field */
/* LinearHexahedra::shape_fun_grads(hex, node), src/InterpolatorCells.cpp:1462-1505, and
 * InterpolatorCells::interp_gradient(cell, node), :425-439 */
static const int NAT_N[8][3] = {{1, 3, 4}, {0, 2, 5}, {3, 1, 6}, {2, 0, 7}, {5, 7, 0}, {4, 6, 1}, {7, 5, 2}, {6, 4, 3}};
static void hex_node_gradient(const double* xyz, const int32_t* hx, int node, const double* phi, double* out) {
    const double uvw[3] = {HX[node], HY[node], HZ[node]};
    const int* nn = NAT_N[node];
    double J[3][3];
    V3 v0 = ld3(xyz, hx[node]);
    for (int i = 0; i < 3; ++i) {
        V3 vi = ld3(xyz, hx[nn[i]]);
        const double f = uvw[i] * 0.5;
        J[i][0] = (v0.x - vi.x) * f;
        J[i][1] = (v0.y - vi.y) * f;
        J[i][2] = (v0.z - vi.z) * f;
    }
    V3 r0 = {J[0][0], J[0][1], J[0][2]}, r1 = {J[1][0], J[1][1], J[1][2]}, r2 = {J[2][0], J[2][1], J[2][2]};
    double Jdet = 1.0 / det3v(r0, r1, r2);
    double Ji[3][3] = {
        {J[1][1] * J[2][2] - J[2][1] * J[1][2], J[2][1] * J[0][2] - J[0][1] * J[2][2], J[0][1] * J[1][2] - J[1][1] * J[0][2]},
        {J[2][0] * J[1][2] - J[1][0] * J[2][2], J[0][0] * J[2][2] - J[2][0] * J[0][2], J[1][0] * J[0][2] - J[0][0] * J[1][2]},
        {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1], J[0][0] * J[1][1] - J[1][0] * J[0][1]}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Ji[i][j] *= Jdet;
    double sfg[8][3];
    memset(sfg, 0, sizeof(sfg));
    for (int i = 0; i < 3; ++i) {
        sfg[node][i] = 0.5 * (Ji[i][0] * uvw[0] + Ji[i][1] * uvw[1] + Ji[i][2] * uvw[2]);
        for (int j = 0; j < 3; ++j) sfg[nn[j]][i] = -0.5 * Ji[i][j] * uvw[j];
    }
    double e[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 8; ++k) {
        const double p = phi[hx[k]];
        e[0] -= sfg[k][0] * p;
        e[1] -= sfg[k][1] * p;
        e[2] -= sfg[k][2] * p;
    }
    out[0] = e[0]; out[1] = e[1]; out[2] = e[2];
}

void orc_nodal_field(int n_nodes, const double* xyz, int n_hexs, const int32_t* hexs,
                     const int32_t* hex_marker, const int8_t* is_vac, const double* phi, double* E) {
    double* acc = (double*)calloc(3 * (size_t)n_nodes, sizeof(double));
    int* cnt = (int*)calloc((size_t)n_nodes, sizeof(int));
    /* Interpolator::store_elfield sums over node2cells in ascending hex order */
    for (int h = 0; h < n_hexs; ++h) {
        if (hex_marker[h] <= 0) continue;
        const int32_t* hx = hexs + 8 * (size_t)h;
        for (int k = 0; k < 8; ++k) {
            double g[3];
            hex_node_gradient(xyz, hx, k, phi, g);
            const int nd = hx[k];
            acc[3 * (size_t)nd] += g[0];
            acc[3 * (size_t)nd + 1] += g[1];
            acc[3 * (size_t)nd + 2] += g[2];
            cnt[nd]++;
        }
    }
    for (int i = 0; i < n_nodes; ++i) {
        if (!is_vac[i]) continue;
        double f = cnt[i] > 0 ? 1.0 / cnt[i] : 0.0;
        if (cnt[i] > 0) {
            E[3 * (size_t)i] = acc[3 * (size_t)i] * f;
            E[3 * (size_t)i + 1] = acc[3 * (size_t)i + 1] * f;
            E[3 * (size_t)i + 2] = acc[3 * (size_t)i + 2] * f;
        } else {
            E[3 * (size_t)i] = E[3 * (size_t)i + 1] = E[3 * (size_t)i + 2] = 0.0;
        }
    }
    free(acc);
    free(cnt);
}

void orc_smooth_field(int n_tetnodes, const double* xyz, const int32_t* vptr, const int32_t* vidx,
                      double decay_factor, double* E) {
    for (int i = 0; i < n_tetnodes; ++i) {
        if (vptr[i + 1] == vptr[i]) continue;
        V3 p = ld3(xyz, i);
        double vx = 0, vy = 0, vz = 0, ws = 0;
        for (int k = vptr[i]; k < vptr[i + 1]; ++k) {
            const int nb = vidx[k];
            V3 q = ld3(xyz, nb);
            const double dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
            const double w = exp(decay_factor * sqrt(dx * dx + dy * dy + dz * dz));
            ws += w;
            vx += E[3 * (size_t)nb] * w;
            vy += E[3 * (size_t)nb + 1] * w;
            vz += E[3 * (size_t)nb + 2] * w;
        }
        if (ws > 0) {
            const double f = 1.0 / ws;
            E[3 * (size_t)i] = vx * f;
            E[3 * (size_t)i + 1] = vy * f;
            E[3 * (size_t)i + 2] = vz * f;
        }
    }
}

/* ------------------------------------------------------------------ location */
static const double ZERO = 1e-15;

/* LinearTetrahedra::point_in_cell, src/InterpolatorCells.cpp:631-649 */
static int pic(const OrcInterp* m, const double* p, int t) {
    const double* d = m->det + 17 * (size_t)t;
    for (int k = 0; k < 4; ++k) {
        const double* v = d + 1 + 4 * k;
        const double s = p[0] * v[0] + p[1] * v[1] + p[2] * v[2] + 1.0 * v[3];
        if (d[0] * s < -ZERO) return 0;
    }
    return 1;
}
/* LinearTetrahedra::shape_functions, :651-661 */
static void bcc(const OrcInterp* m, const double* p, int t, double* b) {
    const double* d = m->det + 17 * (size_t)t;
    for (int k = 0; k < 4; ++k) {
        const double* v = d + 1 + 4 * k;
        b[k] = ZERO + d[0] * (p[0] * v[0] + p[1] * v[1] + p[2] * v[2] + 1.0 * v[3]);
    }
}
/* InterpolatorCells<4>::locate_cell, :269-307 */
static int tet_locate(const OrcInterp* m, const double* p, int guess) {
    if (guess >= 0) {
        if (pic(m, p, guess)) return guess;
        for (int k = m->nbr_ptr[guess]; k < m->nbr_ptr[guess + 1]; ++k)
            if (pic(m, p, m->nbr_idx[k])) return m->nbr_idx[k];
    }
    double best = 1e100;
    int best_i = 0;
    for (int t = 0; t < m->n_tets; ++t) {
        if (m->search[t] && pic(m, p, t)) return t;
        const double* c = m->centroid + 3 * (size_t)t;
        const double dx = p[0] - c[0], dy = p[1] - c[1], dz = p[2] - c[2];
        const double d2 = dx * dx + dy * dy + dz * dz;
        if (d2 < best) { best = d2; best_i = t; }
    }
    return -best_i;
}
/* LinearHexahedra::locate_cell, :1536-1562 */
static int hex_locate(const OrcInterp* m, const double* p, int guess) {
    int t = tet_locate(m, p, guess / 4);
    int sign = t < 0 ? -1 : 1;
    t = abs(t);
    double b[4];
    bcc(m, p, t, b);
    for (int k = 0; k < 4; ++k) {
        int ok = 1;
        for (int j = 0; j < 4; ++j)
            if (j != k && !(b[k] >= b[j])) ok = 0;
        if (ok) return sign * (4 * t + k);
    }
    return -1;
}
/* LinearHexahedra::project_to_nat_coords + shape_functions, :1272-1353 */
static void hex_weights(const OrcInterp* m, const double* p, int hex, double* w) {
    const double* F = m->hexf + 24 * (size_t)hex;
    V3 f0 = {p[0] - F[0], p[1] - F[1], p[2] - F[2]};
    V3 f1 = {F[3], F[4], F[5]}, f2 = {F[6], F[7], F[8]}, f3 = {F[9], F[10], F[11]}, f4 = {F[12], F[13], F[14]};
    V3 f5 = {F[15], F[16], F[17]}, f6 = {F[18], F[19], F[20]}, f7 = {F[21], F[22], F[23]};
    double u = 0, v = 0, ww = 0;
    for (int i = 0; i < 20; ++i) {
        const double uv = u * v, uw = u * ww, vw = v * ww, uvw = uv * ww;
        V3 f = {f0.x - f1.x * u - f2.x * v - f3.x * ww - f4.x * uv - f5.x * uw - f6.x * vw - f7.x * uvw,
                f0.y - f1.y * u - f2.y * v - f3.y * ww - f4.y * uv - f5.y * uw - f6.y * vw - f7.y * uvw,
                f0.z - f1.z * u - f2.z * v - f3.z * ww - f4.z * uv - f5.z * uw - f6.z * vw - f7.z * uvw};
        V3 fu = {f1.x + f4.x * v + f5.x * ww + f7.x * vw, f1.y + f4.y * v + f5.y * ww + f7.y * vw, f1.z + f4.z * v + f5.z * ww + f7.z * vw};
        V3 fv = {f2.x + f4.x * u + f6.x * ww + f7.x * uw, f2.y + f4.y * u + f6.y * ww + f7.y * uw, f2.z + f4.z * u + f6.z * ww + f7.z * uw};
        V3 fw = {f3.x + f5.x * u + f6.x * v + f7.x * uv, f3.y + f5.y * u + f6.y * v + f7.y * uv, f3.z + f5.z * u + f6.z * v + f7.z * uv};
        double D = 1.0 / det3v(fu, fv, fw);
        const double du = det3v(f, fv, fw) * D, dv = det3v(fu, f, fw) * D, dw = det3v(fu, fv, f) * D;
        u += du; v += dv; ww += dw;
        if (du * du + dv * dv + dw * dw < ZERO) break;
    }
    w[0] = (1 - u) * (1 - v) * (1 - ww) / 8.0;
    w[1] = (1 + u) * (1 - v) * (1 - ww) / 8.0;
    w[2] = (1 + u) * (1 + v) * (1 - ww) / 8.0;
    w[3] = (1 - u) * (1 + v) * (1 - ww) / 8.0;
    w[4] = (1 - u) * (1 - v) * (1 + ww) / 8.0;
    w[5] = (1 + u) * (1 - v) * (1 + ww) / 8.0;
    w[6] = (1 + u) * (1 + v) * (1 + ww) / 8.0;
    w[7] = (1 - u) * (1 + v) * (1 + ww) / 8.0;
}

/* InterpolatorCells::interp_solution, :359-380 */
static void weighted(const OrcInterp* m, const int32_t* nodes, const double* w, int k, double* out) {
    double a[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < k; ++i) {
        const double* s = m->sol + 5 * (size_t)nodes[i];
        for (int c = 0; c < 5; ++c) a[c] += s[c] * w[i];
    }
    for (int c = 0; c < 5; ++c) out[c] = a[c];
}

void orc_locate_interpolate(const OrcInterp* m, int rank, int n_pts, const double* pts, int32_t* cells, double* out) {
    int cell = -1;
    for (int i = 0; i < n_pts; ++i) {
        const double* p = pts + 3 * (size_t)i;
        if (rank == 3) cell = hex_locate(m, p, abs(cell));
        else cell = tet_locate(m, p, abs(cell));
        cells[i] = cell;
        const int c = abs(cell);
        double w[10];
        if (rank == 1) {
            bcc(m, p, c, w);
            weighted(m, m->tets + 4 * (size_t)c, w, 4, out + 5 * (size_t)i);
        } else if (rank == 2) {
            double b[4];
            bcc(m, p, c, b);
            w[0] = b[0] * (2 * b[0] - 1); w[1] = b[1] * (2 * b[1] - 1);
            w[2] = b[2] * (2 * b[2] - 1); w[3] = b[3] * (2 * b[3] - 1);
            w[4] = 4 * b[0] * b[1]; w[5] = 4 * b[1] * b[2]; w[6] = 4 * b[2] * b[0];
            w[7] = 4 * b[0] * b[3]; w[8] = 4 * b[1] * b[3]; w[9] = 4 * b[2] * b[3];
            weighted(m, m->quad_nodes + 10 * (size_t)c, w, 10, out + 5 * (size_t)i);
        } else {
            hex_weights(m, p, c, w);
            weighted(m, m->hexs + 8 * (size_t)c, w, 8, out + 5 * (size_t)i);
        }
    }
}

/* ------------------------------------------------------------------ surface */
typedef struct {
    V3 v0, e1d, e2, pvd, n, c;
    double maxd;
} TriRow;

static V3 vsub(V3 a, V3 b) { V3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static V3 vmul(V3 a, double s) { V3 r = {a.x * s, a.y * s, a.z * s}; return r; }
/* Vec3::crossProduct / dotProduct, include/Primitives.h:307-313 */
static V3 vcross(V3 a, V3 v) {
    V3 r = {a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x};
    return r;
}
static double vdot(V3 a, V3 v) { return a.x * v.x + a.y * v.y + a.z * v.z; }

/* TetgenFaces::calc_appendices (src/TetgenCells.cpp:387-412) + LinearTriangles::precompute
 * (src/InterpolatorCells.cpp:1585-1637) */
static void tri_rows(const OrcSurface* s, TriRow* r) {
    for (int f = 0; f < s->n_tris; ++f) {
        const V3 v0 = ld3(s->xyz, s->tris[3 * (size_t)f]);
        const V3 v1 = ld3(s->xyz, s->tris[3 * (size_t)f + 1]);
        const V3 v2 = ld3(s->xyz, s->tris[3 * (size_t)f + 2]);
        const V3 e1 = vsub(v1, v0), e2 = vsub(v2, v0);
        V3 n = vcross(e1, e2);
        const double nn = sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
        if (nn > 0) n = vmul(n, 1 / nn);
        V3 c = {v0.x + v1.x, v0.y + v1.y, v0.z + v1.z};
        c.x = (c.x + v2.x) / 3.0; c.y = (c.y + v2.y) / 3.0; c.z = (c.z + v2.z) / 3.0;
        const V3 pv = vcross(n, e2);
        const double i_det = 1.0 / vdot(e1, pv);
        r[f].v0 = v0; r[f].e1d = vmul(e1, i_det); r[f].e2 = e2; r[f].pvd = vmul(pv, i_det);
        r[f].n = n; r[f].c = c; r[f].maxd = sqrt(e2.x * e2.x + e2.y * e2.y + e2.z * e2.z);
    }
}
/* LinearTriangles::point_in_cell, src/InterpolatorCells.cpp:1639-1650 */
static int tri_pic(const TriRow* r, const double* p) {
    const V3 pt = {p[0], p[1], p[2]};
    const V3 tv = vsub(pt, r->v0);
    const double u = vdot(tv, r->pvd);
    if (u < -ZERO || u > 1 + ZERO) return 0;
    const V3 q = vcross(tv, r->e1d);
    const double v = vdot(q, r->n);
    if (v < -ZERO || u + v > 1 + ZERO) return 0;
    return fabs(vdot(q, r->e2)) < r->maxd;
}
/* LinearTriangles::fast_distance, :1743-1747 */
static double tri_fast_distance(const TriRow* r, const double* p) {
    const V3 pt = {p[0], p[1], p[2]};
    const V3 q = vcross(vsub(pt, r->v0), r->e1d);
    return vdot(r->e2, q);
}

/* LinearTriangles::shape_functions, :1652-1660 */
static void tri_shape(const TriRow* r, const double* p, double* b) {
    const V3 pt = {p[0], p[1], p[2]};
    const V3 tv = vsub(pt, r->v0);
    const V3 q = vcross(tv, r->e1d);
    const double v = vdot(tv, r->pvd);
    const double w = vdot(q, r->n);
    const double u = 1.0 - v - w;
    b[0] = ZERO + u; b[1] = ZERO + v; b[2] = ZERO + w;
}
/* LinearHexahedra::point_in_cell, :1507-1528 */
static int hex_pic(const OrcInterp* m, const double* p, int hex) {
    double b[4];
    bcc(m, p, hex / 4, b);
    if (!(b[0] >= 0 && b[1] >= 0 && b[2] >= 0 && b[3] >= 0)) return 0;
    const int k = hex % 4;
    for (int j = 0; j < 4; ++j)
        if (j != k && !(b[k] >= b[j])) return 0;
    return 1;
}

void orc_surface_interpolate(const OrcInterp* m, const OrcSurface* s, int rank, int n_pts, const double* pts,
                             int32_t* cells, double* out) {
    const int nf = s->n_tris;
    TriRow* rows = (TriRow*)malloc(sizeof(TriRow) * (size_t)(nf ? nf : 1));
    tri_rows(s, rows);
    /* neighbours: for each node of the triangle, the other triangles of that node (ascending) */
    int* cnt = (int*)calloc((size_t)s->n_nodes + 1, sizeof(int));
    for (int f = 0; f < 3 * nf; ++f) cnt[s->tris[f] + 1]++;
    for (int i = 0; i < s->n_nodes; ++i) cnt[i + 1] += cnt[i];
    int* n2f = (int*)malloc(sizeof(int) * (size_t)(cnt[s->n_nodes] ? cnt[s->n_nodes] : 1));
    int* pos = (int*)malloc(sizeof(int) * (size_t)(s->n_nodes ? s->n_nodes : 1));
    memcpy(pos, cnt, sizeof(int) * (size_t)s->n_nodes);
    for (int f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) n2f[pos[s->tris[3 * (size_t)f + k]]++] = f;

    int cell = -1;
    for (int i = 0; i < n_pts; ++i) {
        const double* p = pts + 3 * (size_t)i;
        /* InterpolatorCells<3>::locate_cell (src/InterpolatorCells.cpp:269-307), guess abs(cell);
         * rank 3 keeps quadrangle cells and guesses their triangle (LinearQuadrangles::locate_cell,
         * :1969-1993, quads->to_tri = quad / 3) */
        const int guess = rank == 3 ? abs(cell) / 3 : abs(cell);
        int found = INT_MIN;
        if (guess < nf) {
            if (tri_pic(rows + guess, p)) found = guess;
            for (int k = 0; k < 3 && found == INT_MIN; ++k) {
                const int v = s->tris[3 * (size_t)guess + k];
                for (int q = cnt[v]; q < cnt[v + 1]; ++q) {
                    const int g = n2f[q];
                    if (g != guess && tri_pic(rows + g, p)) { found = g; break; }
                }
            }
        }
        if (found == INT_MIN) {
            double best = 1e100;
            int best_i = 0;
            for (int f = 0; f < nf; ++f) {
                if (tri_pic(rows + f, p)) { found = f; break; }
                const double dx = p[0] - rows[f].c.x, dy = p[1] - rows[f].c.y, dz = p[2] - rows[f].c.z;
                const double d2 = dx * dx + dy * dy + dz * dz;
                if (d2 < best) { best = d2; best_i = f; }
            }
            if (found == INT_MIN) found = -best_i;
        }
        if (rank == 3) {
            const int sign = found < 0 ? -1 : 1;
            const int tf = abs(found);
            double b[3];
            tri_shape(rows + tf, p, b);
            int k = -1;
            if (b[0] >= b[1] && b[0] >= b[2]) k = 0;
            else if (b[1] >= b[0] && b[1] >= b[2]) k = 1;
            else if (b[2] >= b[0] && b[2] >= b[1]) k = 2;
            cell = k < 0 ? -1 : sign * (3 * tf + k);
            cells[i] = cell;
            /* LinearQuadrangles::interp_solution (:1922-1940): the quadrangle's hexes are the
             * hexes of the triangle's two tets around the quadrangle's triangle vertex
             * (TetgenMesh::calc_quad2hex2quad_mapping, src/TetgenMesh.cpp:614-645) */
            const int q = abs(cell), tq = q / 3;
            const int v = s->tris[3 * (size_t)tq + q % 3];
            int hx[2];
            for (int r = 0; r < 2; ++r) {
                const int t = s->tri2tet[2 * (size_t)tq + r];
                int loc = 0;
                while (loc < 4 && m->tets[4 * (size_t)t + loc] != v) ++loc;
                hx[r] = 4 * t + (loc < 4 ? loc : 0);
            }
            int hex;
            if (fabs(tri_fast_distance(rows + tq, p)) <= 100.0 * ZERO) hex = hx[0];
            else if (hex_pic(m, p, hx[0])) hex = hx[0];
            else hex = hex_locate(m, p, hx[1]);
            double w8[8];
            hex_weights(m, p, abs(hex), w8);
            weighted(m, m->hexs + 8 * (size_t)abs(hex), w8, 8, out + 5 * (size_t)i);
            continue;
        }
        cell = found;
        cells[i] = cell;
        /* LinearTriangles::interp_solution (:1662-1686) / QuadraticTriangles (:1834-1856) */
        const int tri = abs(cell);
        const int t0 = s->tri2tet[2 * (size_t)tri], t1 = s->tri2tet[2 * (size_t)tri + 1];
        int tet;
        if (fabs(tri_fast_distance(rows + tri, p)) <= 100.0 * ZERO) tet = t0;
        else if (pic(m, p, t0)) tet = t0;
        else tet = tet_locate(m, p, t1);
        const int c = abs(tet);
        double w[10], b[4];
        bcc(m, p, c, b);
        if (rank == 1) {
            weighted(m, m->tets + 4 * (size_t)c, b, 4, out + 5 * (size_t)i);
        } else {
            w[0] = b[0] * (2 * b[0] - 1); w[1] = b[1] * (2 * b[1] - 1);
            w[2] = b[2] * (2 * b[2] - 1); w[3] = b[3] * (2 * b[3] - 1);
            w[4] = 4 * b[0] * b[1]; w[5] = 4 * b[1] * b[2]; w[6] = 4 * b[2] * b[0];
            w[7] = 4 * b[0] * b[3]; w[8] = 4 * b[1] * b[3]; w[9] = 4 * b[2] * b[3];
            weighted(m, m->quad_nodes + 10 * (size_t)c, w, 10, out + 5 * (size_t)i);
        }
    }
    free(rows); free(cnt); free(n2f); free(pos);
}

int orc_tet_neighbour_lists(int n_nodes, int n_tets, const int32_t* tets, const int32_t* face_nbr,
                            int32_t* ptr, int32_t* idx, int capacity) {
    int* cnt = (int*)calloc((size_t)n_nodes + 1, sizeof(int));
    for (int t = 0; t < n_tets; ++t)
        for (int k = 0; k < 4; ++k) cnt[tets[4 * (size_t)t + k] + 1]++;
    for (int i = 0; i < n_nodes; ++i) cnt[i + 1] += cnt[i];
    int* n2t = (int*)malloc(sizeof(int) * (size_t)(cnt[n_nodes] ? cnt[n_nodes] : 1));
    int* pos = (int*)malloc(sizeof(int) * (size_t)(n_nodes ? n_nodes : 1));
    memcpy(pos, cnt, sizeof(int) * (size_t)n_nodes);
    for (int t = 0; t < n_tets; ++t)
        for (int k = 0; k < 4; ++k) n2t[pos[tets[4 * (size_t)t + k]]++] = t;
    int n = 0;
    ptr[0] = 0;
    for (int t = 0; t < n_tets; ++t) {
        const int32_t* fn = face_nbr + 4 * (size_t)t;
        for (int j = 0; j < 4; ++j)
            if (fn[j] >= 0) { if (n < capacity) idx[n] = fn[j]; ++n; }
        for (int k = 0; k < 4; ++k) {
            const int v = tets[4 * (size_t)t + k];
            for (int q = cnt[v]; q < cnt[v + 1]; ++q) {
                const int u = n2t[q];
                if (u != t && u != fn[0] && u != fn[1] && u != fn[2] && u != fn[3]) { if (n < capacity) idx[n] = u; ++n; }
            }
        }
        ptr[t + 1] = n;
    }
    free(cnt); free(n2t); free(pos);
    return n;
}

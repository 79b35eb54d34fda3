/* Q2 (27-node) vacuum Poisson system in plain C -- TEST INFRASTRUCTURE ONLY.
 *
 * The same system as oracle/q2_oracle.py (the numpy restatement the GPU assembly is tested
 * against), built fast enough for the full 1.7e7-DoF benchmark mesh so that the CPU reference
 * arm can time the reference's solver on it without the product's library:
 *
 *   - DoFs: one per vacuum vertex, hex edge, hex face and hex interior, numbered in the order
 *     they are first met walking the cells and their 27 lattice nodes (x fastest); entities
 *     are identified by their sorted corner node ids;
 *   - element = tensor quadratic Lagrange hexahedron on the trilinear map of the cell,
 *     K_e[i][j] = sum_q w_q |det J_q| grad N_i . grad N_j over 3x3x3 Gauss points, the Q2
 *     analogue of PoissonSolver::assemble_local_cell (src/PoissonSolver.cpp:239-263); cell
 *     matrices are computed in parallel and every matrix entry sums its cell contributions in
 *     cell order, as the reference's WorkStream copier does serially (src/PoissonSolver.cpp:
 *     213-237, src/DealSolver.cpp:65-72): threads own interleaved rows, so the sums do not
 *     depend on the thread count;
 *   - boundary marking as DealSolver::mark_boundary (src/DealSolver.cpp:461-518): faces of one
 *     cell; x/y extremes of the face centroids are the natural sides, z max the top (Neumann
 *     value bc on 3x3 Gauss points, src/DealSolver.cpp:390-430), every other boundary face
 *     copper (phi = 0); with anode_dirichlet the top DoFs not on copper get v0;
 *   - symmetric Dirichlet elimination (MatrixTools::apply_boundary_values, called from
 *     src/DealSolver.cpp:433-440).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "femocs_oracle.h"

static const int QHX[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const int QHY[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const int QHZ[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

/* femocs local vertex at lattice corner (a, b, c), a, b, c in {0, 2} */
static int corner_of(int a, int b, int c) {
    for (int k = 0; k < 8; ++k)
        if (QHX[k] + 1 == a && QHY[k] + 1 == b && QHZ[k] + 1 == c) return k;
    return -1;
}

/* corners of lattice node L (x fastest): 1, 2, 4 or 8 femocs local vertices */
static int entity_corners(int L, int* out) {
    const int a = L % 3, b = (L / 3) % 3, c = L / 9;
    int ra[2], rb[2], rc[2], na = 0, nb = 0, nc = 0;
    if (a == 1) { ra[0] = 0; ra[1] = 2; na = 2; } else { ra[0] = a; na = 1; }
    if (b == 1) { rb[0] = 0; rb[1] = 2; nb = 2; } else { rb[0] = b; nb = 1; }
    if (c == 1) { rc[0] = 0; rc[1] = 2; nc = 2; } else { rc[0] = c; nc = 1; }
    int n = 0;
    for (int k = 0; k < nc; ++k)
        for (int j = 0; j < nb; ++j)
            for (int i = 0; i < na; ++i) out[n++] = corner_of(ra[i], rb[j], rc[k]);
    return n;
}

/* ------------------------------------------------------------------ entity hash map */
typedef struct {
    int32_t k[4];
    int32_t id; /* -1: empty */
} Slot;
typedef struct {
    Slot* s;
    uint64_t cap, n;
} Map;

static uint64_t mix(const int32_t* k) {
    uint64_t h = 0x9E3779B97F4A7C15ull;
    for (int i = 0; i < 4; ++i) {
        h ^= (uint64_t)(uint32_t)k[i] + 0x632BE59BD9B4E019ull + (h << 6) + (h >> 2);
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 31;
    }
    return h;
}
static int map_init(Map* m, uint64_t cap) {
    m->cap = cap;
    m->n = 0;
    m->s = (Slot*)malloc(sizeof(Slot) * cap);
    if (!m->s) return 1;
    for (uint64_t i = 0; i < cap; ++i) m->s[i].id = -1;
    return 0;
}
static Slot* map_find(Map* m, const int32_t* k) {
    uint64_t i = mix(k) & (m->cap - 1);
    for (;;) {
        Slot* s = &m->s[i];
        if (s->id < 0 || memcmp(s->k, k, sizeof(s->k)) == 0) return s;
        i = (i + 1) & (m->cap - 1);
    }
}
static int map_grow(Map* m) {
    Map g;
    if (map_init(&g, 2 * m->cap)) return 1;
    for (uint64_t i = 0; i < m->cap; ++i)
        if (m->s[i].id >= 0) {
            Slot* d = map_find(&g, m->s[i].k);
            *d = m->s[i];
        }
    g.n = m->n;
    free(m->s);
    *m = g;
    return 0;
}

static void sort_i32(int32_t* a, int n) {
    for (int i = 1; i < n; ++i) {
        int32_t v = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
        a[j + 1] = v;
    }
}

/* ------------------------------------------------------------------ element tables */
static double G3[3], W3[3];
static double DN[27][27][3]; /* grad_xi of the 27 shape functions at the 27 Gauss points */
static double D1[27][8][3];  /* grad_xi of the 8 trilinear map functions */
static double WQ[27];

static double lag(int a, double t) { return a == 0 ? 0.5 * t * (t - 1.0) : (a == 1 ? 1.0 - t * t : 0.5 * t * (t + 1.0)); }
static double dlag(int a, double t) { return a == 0 ? t - 0.5 : (a == 1 ? -2.0 * t : t + 0.5); }

static void init_tables(void) {
    G3[0] = -sqrt(0.6); G3[1] = 0.0; G3[2] = sqrt(0.6);
    W3[0] = 5.0 / 9.0; W3[1] = 8.0 / 9.0; W3[2] = 5.0 / 9.0;
    for (int q = 0; q < 27; ++q) {
        const int qa = q % 3, qb = (q / 3) % 3, qc = q / 9;
        const double x = G3[qa], y = G3[qb], z = G3[qc];
        WQ[q] = W3[qa] * W3[qb] * W3[qc];
        for (int L = 0; L < 27; ++L) {
            const int a = L % 3, b = (L / 3) % 3, c = L / 9;
            DN[q][L][0] = dlag(a, x) * lag(b, y) * lag(c, z);
            DN[q][L][1] = lag(a, x) * dlag(b, y) * lag(c, z);
            DN[q][L][2] = lag(a, x) * lag(b, y) * dlag(c, z);
        }
        for (int k = 0; k < 8; ++k) {
            D1[q][k][0] = 0.125 * QHX[k] * (1 + y * QHY[k]) * (1 + z * QHZ[k]);
            D1[q][k][1] = 0.125 * (1 + x * QHX[k]) * QHY[k] * (1 + z * QHZ[k]);
            D1[q][k][2] = 0.125 * (1 + x * QHX[k]) * (1 + y * QHY[k]) * QHZ[k];
        }
    }
}

/* K (27 x 27, row major) of one cell with corner coordinates P (femocs order) */
static void q2_element(const double P[8][3], double* K) {
    double G[27][3];
    memset(K, 0, sizeof(double) * 729);
    for (int q = 0; q < 27; ++q) {
        double J[3][3] = {{0}};
        for (int k = 0; k < 8; ++k)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) J[a][b] += P[k][a] * D1[q][k][b];
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
        /* grad_x N = J^-T grad_xi N */
        for (int L = 0; L < 27; ++L)
            for (int a = 0; a < 3; ++a)
                G[L][a] = inv[0][a] * DN[q][L][0] + inv[1][a] * DN[q][L][1] + inv[2][a] * DN[q][L][2];
        const double w = WQ[q] * fabs(det);
        for (int i = 0; i < 27; ++i)
            for (int j = i; j < 27; ++j) K[27 * i + j] += w * (G[i][0] * G[j][0] + G[i][1] * G[j][1] + G[i][2] * G[j][2]);
    }
    for (int i = 0; i < 27; ++i)
        for (int j = 0; j < i; ++j) K[27 * i + j] = K[27 * j + i];
}

static int64_t find_col(const OrcSystem* s, int r, int c) {
    int64_t lo = s->rowptr[r], hi = s->rowptr[r + 1] - 1;
    while (lo <= hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (s->col[mid] < c) lo = mid + 1;
        else if (s->col[mid] > c) hi = mid - 1;
        else return mid;
    }
    return -1;
}

/* lattice index of face node (u, v) of the face at lattice node L0 (two coordinates = 1) */
static int face_lattice(int L0, int u, int v) {
    const int a0 = L0 % 3, b0 = (L0 / 3) % 3, c0 = L0 / 9;
    int a, b, c;
    if (a0 != 1) { a = a0; b = u; c = v; }
    else if (b0 != 1) { a = u; b = b0; c = v; }
    else { a = u; b = v; c = c0; }
    return a + 3 * b + 9 * c;
}

int orc_q2_build_system(int n_nodes, const double* xyz, int n_cells, const int32_t* cells, double bc,
                        int anode_dirichlet, double v0, int n_threads, int32_t* cell_dofs, OrcSystem* sys,
                        double* timing_ms) {
    (void)n_nodes;
    memset(sys, 0, sizeof(*sys));
    if (n_cells <= 0) return 1;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    init_tables();
    /* ---- DoF numbering by first encounter */
    Map map;
    uint64_t cap = 64;
    while (cap < 16ull * (uint64_t)n_cells) cap <<= 1;
    if (map_init(&map, cap)) return 1;
    int corners[27][8], ncorner[27];
    for (int L = 0; L < 27; ++L) ncorner[L] = entity_corners(L, corners[L]);
    int32_t next = 0;
    for (int c = 0; c < n_cells; ++c) {
        const int32_t* cv = cells + 8 * (size_t)c;
        for (int L = 0; L < 27; ++L) {
            int32_t k[4] = {-1, -1, -1, -1};
            if (L == 13) {
                k[0] = -2 - c;
            } else {
                for (int i = 0; i < ncorner[L]; ++i) k[i] = cv[corners[L][i]];
                sort_i32(k, ncorner[L]);
            }
            Slot* s = map_find(&map, k);
            if (s->id < 0) {
                memcpy(s->k, k, sizeof(k));
                s->id = next++;
                if (++map.n * 10 > map.cap * 7 && map_grow(&map)) return 1;
            }
            cell_dofs[27 * (size_t)c + L] = s->id;
        }
    }
    free(map.s);
    const int n = next;
    sys->n = n;
    /* ---- dof -> (cell) incidence */
    int64_t* iptr = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    int32_t* icell = (int32_t*)malloc(sizeof(int32_t) * 27 * (size_t)n_cells);
    if (!iptr || !icell) return 1;
    for (size_t k = 0; k < 27 * (size_t)n_cells; ++k) iptr[cell_dofs[k] + 1]++;
    for (int i = 0; i < n; ++i) iptr[i + 1] += iptr[i];
    {
        int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
        memcpy(pos, iptr, sizeof(int64_t) * (size_t)n);
        for (int c = 0; c < n_cells; ++c)
            for (int L = 0; L < 27; ++L) icell[pos[cell_dofs[27 * (size_t)c + L]]++] = c;
        free(pos);
    }
    /* ---- sparsity: union of the cells' DoFs per row, sorted */
    sys->rowptr = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    int32_t* stamps = (int32_t*)malloc(sizeof(int32_t) * (size_t)n * nt);
    if (!stamps || !sys->rowptr) return 1;
    for (size_t i = 0; i < (size_t)n * nt; ++i) stamps[i] = -1;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int r = 0; r < n; ++r) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        int32_t* st = stamps + (size_t)n * tid;
        int64_t cnt = 0;
        for (int64_t p = iptr[r]; p < iptr[r + 1]; ++p)
            for (int L = 0; L < 27; ++L) {
                const int32_t d = cell_dofs[27 * (size_t)icell[p] + L];
                if (st[d] != r) { st[d] = r; ++cnt; }
            }
        sys->rowptr[r + 1] = cnt;
    }
    for (int i = 0; i < n; ++i) sys->rowptr[i + 1] += sys->rowptr[i];
    sys->nnz = sys->rowptr[n];
    sys->col = (int32_t*)malloc(sizeof(int32_t) * (size_t)sys->nnz);
    sys->val = (double*)calloc((size_t)sys->nnz, sizeof(double));
    sys->rhs = (double*)calloc((size_t)n, sizeof(double));
    sys->x = (double*)calloc((size_t)n, sizeof(double));
    sys->constrained = (int8_t*)calloc((size_t)n, 1);
    if (!sys->col || !sys->val || !sys->rhs || !sys->x || !sys->constrained) return 1;
    for (size_t i = 0; i < (size_t)n * nt; ++i) stamps[i] = -1;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int r = 0; r < n; ++r) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        int32_t* st = stamps + (size_t)n * tid;
        int32_t* out = sys->col + sys->rowptr[r];
        int64_t cnt = 0;
        for (int64_t p = iptr[r]; p < iptr[r + 1]; ++p)
            for (int L = 0; L < 27; ++L) {
                const int32_t d = cell_dofs[27 * (size_t)icell[p] + L];
                if (st[d] != r) { st[d] = r; out[cnt++] = d; }
            }
        sort_i32(out, (int)cnt);
    }
    free(stamps);
    free(iptr);
    free(icell);
    /* ---- stiffness: cell matrices in parallel chunks, serial scatter in cell order */
    const int chunk = 16384;
    double* Kbuf = (double*)malloc(sizeof(double) * 729 * (size_t)chunk);
    if (!Kbuf) return 1;
    double t_local = 0.0, t_scatter = 0.0;
    for (int c0 = 0; c0 < n_cells; c0 += chunk) {
        const int m = n_cells - c0 < chunk ? n_cells - c0 : chunk;
        double t0 = 0.0;
#ifdef _OPENMP
        t0 = omp_get_wtime();
#endif
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; ++i) {
            double P[8][3];
            const int32_t* cv = cells + 8 * (size_t)(c0 + i);
            for (int k = 0; k < 8; ++k)
                for (int a = 0; a < 3; ++a) P[k][a] = xyz[3 * (size_t)cv[k] + a];
            q2_element(P, Kbuf + 729 * (size_t)i);
        }
#ifdef _OPENMP
        const double t1 = omp_get_wtime();
        t_local += t1 - t0;
#endif
        /* each thread owns the rows r with r % T == its id and walks the cells in order, so
         * every entry still sums its cell contributions in cell order */
#pragma omp parallel
        {
            int tid = 0, T = 1;
#ifdef _OPENMP
            tid = omp_get_thread_num();
            T = omp_get_num_threads();
#endif
            for (int i = 0; i < m; ++i) {
                const int32_t* cd = cell_dofs + 27 * (size_t)(c0 + i);
                const double* K = Kbuf + 729 * (size_t)i;
                for (int a = 0; a < 27; ++a) {
                    const int r = cd[a];
                    if (r % T != tid) continue;
                    for (int b = 0; b < 27; ++b) sys->val[find_col(sys, r, cd[b])] += K[27 * a + b];
                }
            }
        }
#ifdef _OPENMP
        t_scatter += omp_get_wtime() - t1;
#endif
    }
    free(Kbuf);
    if (timing_ms) {
        timing_ms[0] = 1e3 * t_local;
        timing_ms[1] = 1e3 * t_scatter;
    }
    /* ---- boundary faces: face DoFs of exactly one (cell, lattice node) */
    static const int FACE_L[6] = {4, 10, 12, 14, 16, 22};
    int32_t* fcount = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    for (int c = 0; c < n_cells; ++c)
        for (int f = 0; f < 6; ++f) fcount[cell_dofs[27 * (size_t)c + FACE_L[f]]]++;
    /* boundary faces in the order of their DoF (= first encounter) */
    int64_t nb = 0;
    for (int i = 0; i < n; ++i) nb += fcount[i] == 1;
    int64_t* bface = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nb ? nb : 1)); /* cell * 27 + L */
    {
        int64_t* at = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
        for (int i = 0; i < n; ++i) at[i] = -1;
        for (int c = 0; c < n_cells; ++c)
            for (int f = 0; f < 6; ++f) {
                const int32_t d = cell_dofs[27 * (size_t)c + FACE_L[f]];
                if (fcount[d] == 1) at[d] = 27 * (int64_t)c + FACE_L[f];
            }
        int64_t k = 0;
        for (int i = 0; i < n; ++i)
            if (at[i] >= 0) bface[k++] = at[i];
        free(at);
    }
    free(fcount);
    double* ctr = (double*)malloc(sizeof(double) * 3 * (size_t)(nb ? nb : 1));
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < nb; ++i) {
        const int c = (int)(bface[i] / 27), L = (int)(bface[i] % 27);
        int cc[8];
        entity_corners(L, cc);
        for (int a = 0; a < 3; ++a) {
            double s = 0.0;
            for (int q = 0; q < 4; ++q) s += xyz[3 * (size_t)cells[8 * (size_t)c + cc[q]] + a];
            ctr[3 * i + a] = s / 4.0;
            if (ctr[3 * i + a] > mx[a]) mx[a] = ctr[3 * i + a];
            if (ctr[3 * i + a] < mn[a]) mn[a] = ctr[3 * i + a];
        }
    }
    const double eps = 1e-6;
    int8_t* kind = sys->constrained;  /* 0 free, 1 copper, 2 top */
    int64_t* top = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nb ? nb : 1));
    int64_t ntop = 0;
    for (int64_t i = 0; i < nb; ++i) {
        const double x = ctr[3 * i], y = ctr[3 * i + 1], z = ctr[3 * i + 2];
        if (fabs(x - mn[0]) <= eps || fabs(x - mx[0]) <= eps || fabs(y - mn[1]) <= eps || fabs(y - mx[1]) <= eps)
            continue;
        const int c = (int)(bface[i] / 27), L0 = (int)(bface[i] % 27);
        if (fabs(z - mx[2]) <= eps) {
            top[ntop++] = bface[i];
        } else {
            for (int v = 0; v < 3; ++v)
                for (int u = 0; u < 3; ++u) kind[cell_dofs[27 * (size_t)c + face_lattice(L0, u, v)]] = 1;
        }
    }
    sys->n_top_faces = (int)ntop;
    /* Neumann on the top faces: 3x3 Gauss on the bilinear face through its corner DoFs */
    for (int64_t i = 0; i < ntop; ++i) {
        const int c = (int)(top[i] / 27), L0 = (int)(top[i] % 27);
        int32_t fd[9];
        for (int v = 0; v < 3; ++v)
            for (int u = 0; u < 3; ++u) fd[u + 3 * v] = cell_dofs[27 * (size_t)c + face_lattice(L0, u, v)];
        for (int q = 0; q < 9; ++q)
            if (kind[fd[q]] == 0) kind[fd[q]] = 2;
        /* corner positions: the corner lattice nodes (0,0), (2,0), (2,2), (0,2) of the face */
        static const int CU[4] = {0, 2, 2, 0}, CV[4] = {0, 0, 2, 2};
        double P[4][3];
        for (int k = 0; k < 4; ++k) {
            int cc[8];
            entity_corners(face_lattice(L0, CU[k], CV[k]), cc);
            for (int a = 0; a < 3; ++a) P[k][a] = xyz[3 * (size_t)cells[8 * (size_t)c + cc[0]] + a];
        }
        for (int iv = 0; iv < 3; ++iv)
            for (int iu = 0; iu < 3; ++iu) {
                const double s = G3[iu], t = G3[iv];
                double ds[3], dt[3];
                for (int a = 0; a < 3; ++a) {
                    ds[a] = 0.25 * (-(1 - t) * P[0][a] + (1 - t) * P[1][a] + (1 + t) * P[2][a] - (1 + t) * P[3][a]);
                    dt[a] = 0.25 * (-(1 - s) * P[0][a] - (1 + s) * P[1][a] + (1 + s) * P[2][a] + (1 - s) * P[3][a]);
                }
                const double cx = ds[1] * dt[2] - ds[2] * dt[1], cy = ds[2] * dt[0] - ds[0] * dt[2],
                             cz = ds[0] * dt[1] - ds[1] * dt[0];
                const double jac = sqrt(cx * cx + cy * cy + cz * cz);
                for (int q = 0; q < 9; ++q)
                    sys->rhs[fd[q]] += W3[iu] * W3[iv] * lag(q % 3, s) * lag(q / 3, t) * bc * jac;
            }
    }
    free(top);
    free(ctr);
    free(bface);
    /* ---- Dirichlet elimination: rhs -= A g, fixed rows and columns zeroed but the diagonal,
     * rhs = diag * g on fixed rows (g = v0 on the top with a Dirichlet anode, else 0) */
    double* g = (double*)calloc((size_t)n, sizeof(double));
    for (int i = 0; i < n; ++i) {
        if (anode_dirichlet && kind[i] == 2) g[i] = v0;
        kind[i] = (int8_t)(kind[i] == 1 || (anode_dirichlet && kind[i] == 2));
    }
    for (int r = 0; r < n; ++r) {
        if (kind[r]) {
            double diag = 0.0;
            for (int64_t k = sys->rowptr[r]; k < sys->rowptr[r + 1]; ++k) {
                if (sys->col[k] == r) diag = sys->val[k];
                else sys->val[k] = 0.0;
            }
            sys->rhs[r] = g[r] * diag;
            sys->x[r] = g[r];
        } else {
            for (int64_t k = sys->rowptr[r]; k < sys->rowptr[r + 1]; ++k)
                if (kind[sys->col[k]]) {
                    sys->rhs[r] -= sys->val[k] * g[sys->col[k]];
                    sys->val[k] = 0.0;
                }
        }
    }
    free(g);
    return 0;
}

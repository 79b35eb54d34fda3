/* CPU oracle for the femocs_gb300 field-solve path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker (and the timed CPU baseline in bench.py),
 * never part of the product. It restates, in plain C, the reference FEMOCS algorithms for
 * the path; every function cites the reference file:line it follows. The FEM solve
 * (assembly, boundary conditions, SSOR-CG) cannot be pinned bit for bit against the
 * reference, because that part of the reference runs inside deal.II 9.2, which is not
 * available; it is pinned to the reference's analytic hemisphere-on-plane answer
 * (src/SolutionReader.cpp:501-524) by a convergence test. The cell-location, interpolation,
 * nodal-field and smoothing parts are pinned against golden vectors produced by the
 * reference's own compiled sources (oracle/ref_driver.cpp).
 */
#ifndef FEMOCS_ORACLE_H
#define FEMOCS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------- tet tables (src/InterpolatorCells.cpp:523-629) ---------- */
void orc_tet_tables(int n_tets, const int32_t* tets, const double* xyz,
                    double* det /* 17*n_tets */, double* centroid /* 3*n_tets */);

/* ---------- FEM system on the vacuum hexes ----------
 * cells: 8 vertex ids per cell (femocs hex order), vertex coordinates xyz (3*n_vert).
 * Builds the CSR pattern (sorted columns), the Q1 stiffness (src/PoissonSolver.cpp:239-263),
 * boundary marking (src/DealSolver.cpp:461-518), Neumann rhs on the top (src/DealSolver.cpp:390-430)
 * and the Dirichlet elimination (deal.II MatrixTools::apply_boundary_values, called from
 * src/DealSolver.cpp:438). The caller frees the CSR arrays with orc_free. */
typedef struct {
    int n;
    int64_t nnz;
    int64_t* rowptr;
    int32_t* col;
    double* val;
    double* rhs;
    double* x;              /* initial guess / solution, Dirichlet values preset */
    int8_t* constrained;    /* 1 if Dirichlet */
    int n_top_faces;
} OrcSystem;

int orc_build_system(int n_vert, const double* xyz, int n_cells, const int32_t* cells,
                     double applied_field, int anode_dirichlet, double applied_potential,
                     OrcSystem* sys);
void orc_free_system(OrcSystem* sys);
/* wrap a CSR system assembled elsewhere (arrays copied); diagonal must be present */
int orc_system_from_csr(int n, const int64_t* rowptr, const int32_t* col, const double* val, const double* rhs,
                        const double* x0, OrcSystem* sys);

/* Q2 (27-node) vacuum system (oracle/q2_oracle.c): cells = 8 femocs-ordered node ids per
 * vacuum hex, xyz of all nodes, bc = Neumann value on the top (-E0), n_threads for the cell
 * matrices and the sparsity (0: OpenMP default; results do not depend on it). cell_dofs
 * (27 * n_cells) receives the DoF of each lattice node; timing_ms (2, may be NULL) the
 * milliseconds of the cell matrices and of their scatter into the CSR matrix. */
int orc_q2_build_system(int n_nodes, const double* xyz, int n_cells, const int32_t* cells, double bc,
                        int anode_dirichlet, double v0, int n_threads, int32_t* cell_dofs, OrcSystem* sys,
                        double* timing_ms);

/* deal.II SolverCG + PreconditionSSOR(omega) (src/DealSolver.cpp:443-459); omega <= 0 gives
 * the identity preconditioner. Stop when ||b-Ax||_2 <= tol. Returns #iterations or
 * -#iterations when max_it is reached. */
int orc_ssor_cg(const OrcSystem* sys, double* x, double omega, double tol, int max_it);
/* Jacobi-preconditioned CG with the same stop test (plain GPU-CG counterpart). */
int orc_jacobi_cg(const OrcSystem* sys, double* x, double tol, int max_it);
/* threads of the CG's SpMV and vector operations (default 1: every sum in a fixed order);
 * the SSOR sweeps are always sequential, as deal.II's PreconditionSSOR */
void orc_set_threads(int n);
/* timing helper: run exactly n_it SSOR-CG iterations regardless of convergence */
double orc_ssor_cg_fixed(const OrcSystem* sys, double* x, double omega, int n_it);
void orc_spmv(const OrcSystem* sys, const double* x, double* y);
/* out2[0] = ||b - A x||_2 with compensated (Dot2) row products; out2[1] = the rounding floor
 * of a plain FP64 evaluation, 2^-53 ||(|b| + |A||x|)||_2 */
void orc_residual_comp(const OrcSystem* sys, const double* x, double* out2);

/* ---------- nodal field (src/Interpolator.cpp:125-140 + src/InterpolatorCells.cpp:1462-1505) ----
 * phi: per node of the hex mesh; out E: 3 per node, only nodes with is_vac[node] are set.  */
void orc_nodal_field(int n_nodes, const double* xyz, int n_hexs, const int32_t* hexs,
                     const int32_t* hex_marker, const int8_t* is_vac, const double* phi, double* E);
/* smoothing (src/Interpolator.cpp:142-170) with the pseudo-Voronoi stencils */
void orc_smooth_field(int n_tetnodes, const double* xyz, const int32_t* vptr, const int32_t* vidx,
                      double decay_factor, double* E);

/* ---------- location + interpolation (src/InterpolatorCells.cpp:269-307, 631-661,
 * 795-816, 1272-1353, 1536-1562; src/SolutionReader.cpp:136-165) ----------
 * rank 1/2 return tet indices, rank 3 hex indices, negative = outside. The chain starts
 * from a fresh reader (cell = -1). sol: 5 doubles per node (E, scalar1, phi).
 * out: 5 doubles per point. */
typedef struct {
    int n_tets;
    const int32_t* tets;
    const int8_t* search;       /* 1 for tets in the searched region (vacuum) */
    const double* det;          /* 17 per tet */
    const double* centroid;     /* 3 per tet */
    const int32_t* nbr_ptr;     /* candidate lists after a failed guess */
    const int32_t* nbr_idx;
    const int32_t* hexs;        /* 8 per hex */
    const double* hexf;         /* 24 per hex */
    const int32_t* quad_nodes;  /* 10 per tet */
    const double* sol;          /* 5 per node */
} OrcInterp;

void orc_locate_interpolate(const OrcInterp* m, int rank, int n_pts, const double* pts,
                            int32_t* cells, double* out);

/* ---------- surface (2-D) location + interpolation ----------
 * LinearTriangles / QuadraticTriangles (src/InterpolatorCells.cpp:1585-1686, 1791-1862):
 * triangle tables from the node coordinates (TetgenFaces::calc_appendices,
 * src/TetgenCells.cpp:387-412, and LinearTriangles::precompute), the chained triangle
 * location of a fresh reader (src/SolutionReader.cpp:43-55, 136-165) and the tet chosen
 * through the triangle's two tets. rank 1 interpolates linearly, rank 2 quadratically in
 * that tet; rank 3 (LinearQuadrangles, :1922-1993) works on the three quadrangles of each
 * triangle and interpolates trilinearly in the hex of the quadrangle. cells: triangle (ranks
 * 1, 2) or quadrangle 3*triangle+vertex (rank 3) per point (negative = nearest-centroid fallback). */
typedef struct {
    int n_tris;
    const int32_t* tris;     /* 3 node ids per triangle */
    const int32_t* tri2tet;  /* 2 tets per triangle, the first tried first */
    int n_nodes;
    const double* xyz;       /* 3 per node */
} OrcSurface;

void orc_surface_interpolate(const OrcInterp* m, const OrcSurface* s, int rank, int n_pts, const double* pts,
                             int32_t* cells, double* out);

/* neighbour lists exactly as the reference stores them (face neighbours, then
 * vertex-sharing tets with repeats), src/InterpolatorCells.cpp:537-558 */
int orc_tet_neighbour_lists(int n_nodes, int n_tets, const int32_t* tets, const int32_t* face_nbr,
                            int32_t* ptr /* n_tets+1 */, int32_t* idx /* capacity */, int capacity);

void orc_free(void* p);

#ifdef __cplusplus
}
#endif
#endif

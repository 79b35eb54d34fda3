/*
 * femocs_gb300 -- C ABI of the GB300 field-solve library.
 *
 * Part 1 reproduces the reference's C wrapper (include/Femocs_wrap.h:12-50 of FEMOCS) symbol
 * for symbol, so an MD code (or the Fortran module src/Femocs_wrap.f90) can link this
 * library in place of the deal.II CPU build. Conventions are the reference's: an opaque
 * handle, caller-owned SoA arrays of length n, status through int* retval
 * (0 = current solution used / success, 1 = previous solution / failure), n <= 0 disables
 * the call, no exceptions cross the boundary.
 *
 * Part 2 exposes the inner operator interface (the reference's PoissonSolver<3> verbs
 * setup / assemble / solve / export_solution, include/PoissonSolver.h:25-105, and the
 * Interpolator's extract_solution / locate / interpolate) on device-resident state, plus
 * mesh import and the seeded synthetic workloads used by the tests and the benchmark.
 *
 * All entry points are host functions; pointers are host pointers unless the name ends
 * in _device.
 */
#ifndef FEMOCS_GB300_H
#define FEMOCS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* =============================== Part 1: reference C wrapper =============================== */
typedef struct FEMOCS FEMOCS;

/* replaces create_femocs, include/Femocs_wrap.h:14 -- reads the configuration script */
FEMOCS* create_femocs(const char* conf_file);
/* replaces delete_femocs, include/Femocs_wrap.h:17 */
void delete_femocs(FEMOCS* femocs);
/* replaces femocs_run, include/Femocs_wrap.h:19 -- field solve (Femocs::run, src/Femocs.cpp:72) */
void femocs_run(FEMOCS* femocs, int* retval, int timestep, double time);
/* replaces femocs_import_file, include/Femocs_wrap.h:21 -- xyz/ckx atom files */
void femocs_import_file(FEMOCS* femocs, int* retval, const char* file_name);
/* replaces femocs_import_parcas, include/Femocs_wrap.h:23 -- not supported (sets retval=1) */
void femocs_import_parcas(FEMOCS* femocs, int* retval, int n_atoms, const double* x0, const double* x1,
                          const double* box, const int* nborlist);
/* replaces femocs_import_atoms, include/Femocs_wrap.h:26 */
void femocs_import_atoms(FEMOCS* femocs, int* retval, int n_atoms, const double* x, const double* y,
                         const double* z, const int* types);
/* replaces femocs_interpolate_elfield, include/Femocs_wrap.h:29 */
void femocs_interpolate_elfield(FEMOCS* femocs, int* retval, int n_points, const double* x, const double* y,
                                const double* z, double* Ex, double* Ey, double* Ez, double* Enorm, int* flag);
/* replaces femocs_interpolate_surface_elfield, include/Femocs_wrap.h:33 */
void femocs_interpolate_surface_elfield(FEMOCS* femocs, int* retval, int n_points, const double* x,
                                        const double* y, const double* z, double* Ex, double* Ey, double* Ez,
                                        double* Enorm, int* flag);
/* replaces femocs_interpolate_phi, include/Femocs_wrap.h:37 */
void femocs_interpolate_phi(FEMOCS* femocs, int* retval, int n_points, const double* x, const double* y,
                            const double* z, double* phi, int* flag);
/* replaces femocs_export_data, include/Femocs_wrap.h:41 */
void femocs_export_data(FEMOCS* femocs, int* retval, double* data, int n_points, const char* data_type);
/* replaces femocs_export_int, include/Femocs_wrap.h:43 */
void femocs_export_int(FEMOCS* femocs, int* retval, int* data, int n_points, const char* data_type);
/* replaces femocs_interpolate, include/Femocs_wrap.h:45 */
void femocs_interpolate(FEMOCS* femocs, int* retval, double* data, int* flag, int n_points, const char* data_type,
                        int near_surface, const double* x, const double* y, const double* z);
/* replace femocs_parse_int/double/string, include/Femocs_wrap.h:48-52 */
void femocs_parse_int(FEMOCS* femocs, int* retval, const char* command, int* arg);
void femocs_parse_double(FEMOCS* femocs, int* retval, const char* command, double* arg);
void femocs_parse_string(FEMOCS* femocs, int* retval, const char* command, char* arg);

/* Library extensions of the facade (no counterpart in Femocs_wrap.h). */
/* Tetrahedral mesh from arrays: nodes xyz (3*n_nodes), tets (4*n_tets, 0-based), region
 * markers (3 = vacuum, anything else = material); replaces the TetGen step of Femocs::run. */
void femocs_import_mesh(FEMOCS* femocs, int* retval, int n_nodes, const double* xyz, int n_tets, const int* tets,
                        const int* markers);
/* Statistics of the last femocs_run: iterations, refinement sweeps, status, relative
 * residual, solve milliseconds, #dofs, |b|, multigrid levels (as doubles). */
void femocs_last_solve(FEMOCS* femocs, int* retval, double* out8);
/* the 14 statistics of fgb_field_last_stats for the last femocs_run */
int fgb_femocs_last_stats(FEMOCS* femocs, double* out14);
/* M/A field-enhancement ratio of the last femocs_run (FieldReader::check_limits,
 * src/SolutionReader.cpp:538-556; limits from `field_tolerance`); 0 when the check did not run
 * (no `radius`, equal limits or a zero applied field) */
int fgb_femocs_enhancement(FEMOCS* femocs, double* ratio);
const char* femocs_last_error(void);
/* number of CUDA kernels the library has launched so far (all handles) */
long long fgb_kernel_launches(void);

/* =============================== Part 2: inner operator API =============================== */
typedef struct FGB_MESH FGB_MESH;    /* host-prepared mesh */
typedef struct FGB_FIELD FGB_FIELD;  /* device-resident Poisson system + interpolator */

typedef struct {
    double radius, height, box_half, slab, top, h, growth, margin; /* Angstrom */
} FgbNanotip;

/* mesh construction (host); returns NULL on error (see femocs_last_error) */
FGB_MESH* fgb_mesh_from_arrays(int n_nodes, const double* xyz, int n_tets, const int* tets, const int* markers);
FGB_MESH* fgb_mesh_read_gmsh(const char* path);
FGB_MESH* fgb_mesh_synthetic(const FgbNanotip* spec);
/* the same meshes prepared by kernels on the current CUDA device (tet -> hex split, grouping,
 * interpolation tables: src/Tethex.cpp:1037-1102, src/TetgenMesh.cpp:353-385,
 * src/InterpolatorCells.cpp:523-629, 1205-1267); tables equal bit for bit to the host
 * builder's; up to 2^21 tet vertices */
FGB_MESH* fgb_mesh_from_arrays_device(int n_nodes, const double* xyz, int n_tets, const int* tets, const int* markers);
FGB_MESH* fgb_mesh_synthetic_device(const FgbNanotip* spec);
/* Surface triangles for surface (2-D) location and interpolation. A prepared mesh starts with
 * its vacuum/metal interface faces (per vacuum tet ascending, faces opposite vertex 0..3 whose
 * neighbour is not vacuum; normal into the vacuum; tri2tet = {vacuum tet, metal tet}).
 * fgb_mesh_set_surface replaces them, e.g. by TetGen's surface triangles and their tet
 * pairs (TetgenMesh tris / tris.to_tets, src/TetgenMesh.cpp:592-612): 3 tet-mesh node ids and
 * 2 tets per triangle, the first tet tried first. Fields created afterwards use the new set. */
int fgb_mesh_set_surface(FGB_MESH* m, int n_tris, const int* tris, const int* tri2tet);
int64_t fgb_mesh_surface_tris(const FGB_MESH* m);
/* preparation time of a mesh: [device kernel ms (0 for the host builder), total ms] */
int fgb_mesh_prep_timing(const FGB_MESH* m, double* out2);
void fgb_mesh_free(FGB_MESH* m);
/* sizes: [n_tetnodes, n_tets, n_nodes, n_hexs, n_vac_vertices, n_vac_cells, n_nbr_idx, n_voro_idx,
 *         n_dofs, nnz, n_top_faces, n_sell] (n_dofs.. are 0 until a field is created) */
int fgb_mesh_sizes(const FGB_MESH* m, int64_t* out12);
/* copy a named host table into `out` (caller sized from fgb_mesh_sizes):
 * tet_nodes tet_marker tet_nbor node_xyz node_marker hex_nodes hex_marker tet_det
 * tet_centroid hex_coeffs nbr_ptr nbr_idx quad_nodes voro_ptr voro_idx vac_node2vertex
 * vac_cells node_parents (4 per node, -1 = unused) edgemax(double);
 * surface: surf_tris (3 per triangle) surf_tri2tet (2) surf_geo (19 doubles: vertex 0, edge1/D,
 * edge2, pvec/D, unit normal, |edge2|, centroid) surf_nbr_ptr surf_nbr_idx */
int fgb_mesh_export(const FGB_MESH* m, const char* name, void* out);

/* synthetic atoms/probes for a nanotip spec; two-call pattern: pass out=NULL to get the count */
int64_t fgb_synth_atoms(const FgbNanotip* spec, double latconst, double sigma, double cutoff, uint64_t seed,
                        double* xyz_out, int* type_out);
int64_t fgb_synth_probes(const FgbNanotip* spec, int n, uint64_t seed, double* xyz_out);

/* device field */
FGB_FIELD* fgb_field_create(const FGB_MESH* m);
/* element order 1 (Q1, the reference's element) or 2 (Q2: 27-node hexahedra on the same mesh;
 * phi at the mesh vertices feeds the same interpolator) */
FGB_FIELD* fgb_field_create_order(const FGB_MESH* m, int order);
/* Q2 fields: for every DoF one vacuum cell holding it and its lattice index L = a + 3b + 9c */
int fgb_field_q2_dofs(FGB_FIELD* f, int* dof_cell, int* dof_local);
/* Q1 / Q2 structure of a mesh built on the host only: DoFs, nonzeros, top faces, longest row */
int fgb_mesh_q1_sizes(const FGB_MESH* m, int64_t* out4);
/* 64-bit FNV-1a digest of every array of the host-built FEM structure (order 1 or 2; region 0
 * vacuum, 1 bulk), for regression checks of the builders */
uint64_t fgb_mesh_structure_digest(const FGB_MESH* m, int order, int region);
int fgb_mesh_q2_sizes(const FGB_MESH* m, int64_t* out4);
/* cell blocks of the mesh's Q2 structure (the element-by-element level 0 and outer SpMV of
 * Q2 fields), built on the host and checked against every invariant the kernels rely on;
 * out8 = blocks, largest block's cells, largest block's DoFs, block-local DoF entries, slots,
 * DoFs split over blocks, DoFs complete in one block, 64-bit digest of all arrays */
int fgb_mesh_cell_blocks(const FGB_MESH* m, int cells_per_block, int max_dofs, int64_t* out8);
void fgb_field_free(FGB_FIELD* f);
int fgb_field_sizes(const FGB_FIELD* f, int64_t* out4); /* n_dofs, nnz, n_top_faces, sell_entries */
/* PoissonSolver::setup(field, potential): applied_field is the Neumann value on the top
 * boundary (the reference passes -E0), applied_potential the anode value; zeroes phi */
int fgb_field_setup(FGB_FIELD* f, double applied_field, double applied_potential);
/* PoissonSolver::assemble(full_run); anode_dirichlet selects anode_bc = dirichlet */
int fgb_field_assemble(FGB_FIELD* f, int full_run, int anode_dirichlet);
/* CG solve; precision 0 = plain FP64 Jacobi-PCG, 1 = FP32 inner + FP64 refinement,
 * 2 = FP64 CG preconditioned by an FP32 multigrid V-cycle (hierarchy built on first use),
 * 3 = FP32 CG with that V-cycle and its FP32 level-0 operator (for Q2 the matrix-free
 * cell-block operator) inside FP64 iterative refinement on the assembled FP64 system.
 * inner_tol: residual reduction between FP64 refinements (<= 0: default 0.1 for precision
 * 1, 1e-3 for precision 3).
 * stats (may be NULL): iterations, refinements, status, rel_residual, bnorm, ms; a 7th slot
 * preset to -1 receives the device time of the solver kernel alone.
 * status: 1 converged; 2 converged to the FP64 floor (rel_tol below 1e-10 evaluates the true
 * residual compensated, and a solution whose residual is within twice 2^-53 |(|b| + |A||x|)|
 * is as accurate as an FP64 vector can be on that system); -1 iteration cap; -2 breakdown or
 * NaN; -3 FP64 refinements stopped reducing the residual (precision 1 and 3).
 * Returns #iterations (>0) when the status is 1 or 2, else -#iterations. */
int fgb_field_solve(FGB_FIELD* f, int precision, double rel_tol, double abs_tol, int max_iter, double inner_tol,
                    double* stats6);
/* phi per vacuum dof order is internal; these export per hex-mesh node (n_nodes values) */
/* statistics of the last solve (14 doubles): iterations, refinements, status, rel_residual,
 * bnorm, ms, solver-kernel ms (persistent mixed path), multigrid setup ms in that call,
 * levels, and with profiling on (multigrid path): level-0 smoother ms, smoother launches,
 * outer FP64 SpMV ms, SpMV launches; algorithmic bytes of one level-0 smoothing step */
int fgb_field_last_stats(const FGB_FIELD* f, double* out14);
/* Q2 fields: apply the finest multigrid level element by element by cell blocks (1, default:
 * half the bytes of the SELL matrix) or through the assembled SELL matrix (0); the hierarchy is
 * rebuilt at the next solve */
int fgb_field_set_level0_ebe(FGB_FIELD* f, int on);
/* outer SpMV of the multigrid PCG: 1 (Q1 default) reads the SELL matrix and the search
 * direction as FP32 hi/lo pairs with error-free products and compensated row sums (FP64-accurate
 * to ~2^-48 per term, off the FP64 pipe); 2 (Q2 default, Q2 only) does the same arithmetic
 * element by element over cell blocks (half the bytes); 0 uses the FP64 SELL matrix */
int fgb_field_set_outer_spmv(FGB_FIELD* f, int mode);
/* Q2 fields: limits of the cell blocks (hexes per block 1..256, DoFs per block 27..4096;
 * default 256 and 4096); the blocks and the hierarchy are rebuilt at the next solve */
int fgb_field_set_cell_blocks(FGB_FIELD* f, int cells_per_block, int max_dofs);
/* algorithmic bytes of one outer SpMV launch in the current mode (cell-block counts once the
 * blocks exist, i.e. after the first solve in mode 2) */
double fgb_field_outer_spmv_bytes(const FGB_FIELD* f);
/* Chebyshev smoothing of the finest multigrid level: steps before and after the coarse
 * correction (0: default, Q1 4, Q2 2) and the interval's lower end as a fraction of
 * lambda_max (0: default, Q1 0.04, Q2 0.06); the hierarchy is rebuilt at the next solve */
int fgb_field_set_smoothing(FGB_FIELD* f, int degree, double lo);
/* Chebyshev smoothing of a coarser multigrid level `level` >= 1 (Q2 fields: level 1 is the
 * Q1 system of the same mesh, default degree 4 on [0.04, 1.1], and the aggregation levels
 * below it degree 1; Q1 fields: the aggregation levels, default 3 on [0.06, 1.1]); degree 0 /
 * lo 0 = the default. Applied from the next
 * solve without rebuilding the hierarchy; the dense coarsest level is left alone */
int fgb_field_set_level_smoothing(FGB_FIELD* f, int level, int degree, double lo);
/* Q2 fields: form the assembled SELL matrices (FP64 and FP32 values of the eliminated system)
 * at every assembly (0) or only when something reads them (1, the default): the system
 * export, the Jacobi-preconditioned solvers, precision 3, a compensated true residual
 * (rel_tol below 1e-10), a nonzero Dirichlet value. The default multigrid PCG over the cell
 * blocks takes D^-1 and its FP64 true residual from the element matrices */
int fgb_field_set_lazy_matrix(FGB_FIELD* f, int on);
/* Q2 fields: element matrices of the full assembly on the tensor cores (1, default: per-point
 * factors in double-float arithmetic (~48 bits), error-free BF16 slices, tcgen05 products
 * accumulated exactly in FP32, levels combined as FP32 pairs into FP64) or on the FP32 pipe as
 * FP32 hi/lo pairs (0) */
int fgb_field_set_ke_tensor(FGB_FIELD* f, int on);
/* element matrices of the last full assembly (Q1: 64 per cell; Q2: 378 packed upper-triangle
 * entries per cell, row by row); returns the number of values (out may be NULL), -1 on error */
long long fgb_field_export_element_matrices(FGB_FIELD* f, double* out);
/* Q2 fields, level 0 by cell blocks: the element matrices reach the applying warps through a
 * shared-memory ring filled by bulk copies from a producer warp (1) or by their own loads (0,
 * default: 0.86 against 1.19 ms per smoothing step on the 1.7e7-DoF benchmark mesh) */
int fgb_field_set_level0_stream(FGB_FIELD* f, int on);
/* Q2 level 0 by cell blocks: the operator from the element matrices (kind 0) or, matrix-free,
 * from the geometric factors w_q |det J_q| J_q^-1 J_q^-T of the 27 Gauss points (kind 1: FP32,
 * 648 bytes per hex; kind 2: FP16, 324 bytes; the default) applied by sum factorisation.
 * Returns the kind in use (FP16 falls back to FP32 when a factor is beyond its range),
 * negative on error */
int fgb_field_set_level0_operator(FGB_FIELD* f, int kind);
/* Q2 level 0 by cell blocks: each applying warp asks L2 for the operator data (element matrix
 * or geometric factors) of the cells `cells` steps ahead of the ones it loads
 * (cp.async.bulk.prefetch; 0 = off, 1 = the default, at most 64) */
int fgb_field_set_level0_prefetch(FGB_FIELD* f, int cells);
/* multigrid PCG: the coarse-grid correction of level `level` (0 = finest) runs `cycles` (1..8)
 * cycles of the next level, each on the residual left by the ones before (1 = V-cycle); the
 * preconditioner stays symmetric */
int fgb_field_set_coarse_cycles(FGB_FIELD* f, int level, int cycles);
/* record CUDA event pairs around the multigrid path's hot launches (off by default) */
int fgb_field_set_profiling(FGB_FIELD* f, int on);
/* multigrid levels as "rows:nnz" separated by spaces, the coarsest "rows:rows^2:dense";
 * NUL-terminated, truncated to cap bytes; empty before the first multigrid solve */
int fgb_field_amg_levels(FGB_FIELD* f, char* buf, int cap);
int fgb_field_export_phi_nodes(FGB_FIELD* f, double* phi_nodes);
/* PIC space charge (PoissonSolver::assemble_space_charge_fast, src/PoissonSolver.cpp:300-319):
 * n particles at device positions d_xyz in vacuum hexes d_hex (NULL: located here, rank 3)
 * add N_k(p) * charge_factor (= q/eps0 * W_sp) to the rhs of their hex's DoFs at the next
 * fgb_field_assemble (before the Dirichlet values; full_run = 0 reuses the matrix, as
 * ProjectRunaway::make_pic_step). accumulate = 0 starts a new charge distribution.
 * n_skipped (may be NULL): particles outside the vacuum hexes. */
int fgb_field_space_charge(FGB_FIELD* f, int n, const double* d_xyz, const int* d_hex, double charge_factor,
                           int accumulate, int* n_skipped);
int fgb_field_clear_space_charge(FGB_FIELD* f);
/* wait for all work of this process on the current device */
int fgb_device_sync(void);
/* tensor-core self check on the current device: one 128 x 48 x 32 BF16 product of small
 * integers through the library's tcgen05 path against the host's; *max_err = largest absolute
 * difference (0 expected) */
int fgb_tc_selftest(double* max_err);
/* free and total device memory of the current device (cudaMemGetInfo) and, when uuid is not
 * NULL (room for 48 chars), its UUID in the form nvidia-smi prints ("GPU-xxxxxxxx-...") */
int fgb_device_info(size_t* free_bytes, size_t* total_bytes, char* uuid);
/* the solution in the field's own DoF order (n_dofs values) */
int fgb_field_export_solution(FGB_FIELD* f, double* x);
int fgb_field_import_phi_nodes(FGB_FIELD* f, const double* phi_nodes);
/* Interpolator::extract_solution: nodal E from phi, optional smoothing */
int fgb_field_extract(FGB_FIELD* f, int smoothen);
/* nodal solution, 5 doubles per node: Ex Ey Ez charge_density phi */
int fgb_field_get_nodal(FGB_FIELD* f, double* sol5);
int fgb_field_set_nodal(FGB_FIELD* f, const double* sol5);
/* locate + interpolate n points (xyz interleaved, host), rank 1/2/3; cells (n) and out (5n) */
int fgb_field_interpolate(FGB_FIELD* f, int n, const double* xyz, int rank, int* cells, double* out5,
                          int64_t* stats5);
/* same with device pointers (no copies) */
int fgb_field_interpolate_device(FGB_FIELD* f, int n, const double* d_xyz, int rank, int* d_cells, double* d_out5);
/* surface (2-D) location + interpolation on the mesh's surface triangles (LinearTriangles rank 1,
 * QuadraticTriangles rank 2, LinearQuadrangles rank 3: src/InterpolatorCells.cpp:1639-1686,
 * 1834-1856, 1922-1993, driven as SolutionReader::calc_full_interpolation with dim = 2,
 * src/SolutionReader.cpp:43-55); cells = triangle (ranks 1, 2) or quadrangle 3*tri+vertex
 * (rank 3) per point (negative: no triangle holds the point, nearest centroid) */
int fgb_field_interpolate_surface(FGB_FIELD* f, int n, const double* xyz, int rank, int* cells, double* out5);
int fgb_field_interpolate_surface_device(FGB_FIELD* f, int n, const double* d_xyz, int rank, int* d_cells,
                                         double* d_out5);
/* Allocation-free variant of fgb_field_interpolate_device (no counterpart in the reference).
 * Some callers cannot let a library allocate device memory during their timestep loop: MD
 * engines that hand the whole device memory to their own pool allocator, or run with a
 * device-memory footprint fixed at start-up, and pipelines that cannot afford the device
 * synchronisation a cudaMalloc implies. This entry point calls no cudaMalloc, cudaFree or
 * other allocating routine: its per-point scratch is a fixed file-scope device array that
 * every GPU on which a field is built keeps (about 5.2 MB) until the process exits.
 *   - at most 262144 points per call; larger n returns 1 with a message, nothing launched;
 *   - the caller passes device pointers for the points (3n doubles), the cells (n ints, or
 *     NULL) and the results (5n doubles); results are identical to fgb_field_interpolate_device;
 *   - asynchronous on the field's stream (fgb_field_stream); results are ready when that
 *     stream has completed the call;
 *   - all calls share the scratch array, so calls that overlap on the GPU (from different
 *     streams, threads or fields) race: serialise them;
 *   - the array's device address is looked up (cudaGetSymbolAddress, with the device current)
 *     when the first field is built on each device, so the array is held from then on and
 *     the calls themselves do no set-up;
 *   - a device reset (cudaDeviceReset) while the library is loaded is unsupported: the cached
 *     address of the array would be stale.
 * Returns 0 on success, 1 on error (femocs_last_error). */
int fgb_field_interpolate_device_noalloc(FGB_FIELD* f, int n, const double* d_xyz, int rank, int* d_cells,
                                         double* d_out5);
/* matrix after Dirichlet elimination in CSR (sorted columns) with the rhs, by dof;
 * dof2node maps dofs to mesh nodes */
int fgb_field_export_system(FGB_FIELD* f, int64_t* rowptr, int* col, double* val, double* rhs, int* dof2node);
/* average device time [ms] of one SpMV with FP64 (precision 0) or FP32 (1) values, or of
 * one level-0 multigrid Chebyshev smoothing step (2; builds the hierarchy if needed) */
double fgb_field_time_spmv(FGB_FIELD* f, int precision, int reps);
/* device stream the field works on (cudaStream_t) */
void* fgb_field_stream(FGB_FIELD* f);
/* borrowed handle to the device field a FEMOCS instance solved on (valid after femocs_run,
 * until the FEMOCS handle is deleted); free it with fgb_field_free (the field survives) */
FGB_FIELD* femocs_field(FEMOCS* femocs);
/* CUDA events on the field's stream (slots 0..7) for device-side timing */
int fgb_field_mark(FGB_FIELD* f, int slot);
double fgb_field_elapsed(FGB_FIELD* f, int slot_a, int slot_b);
/* plain device memory for callers without a CUDA runtime binding */
void* fgb_device_alloc(size_t bytes);
void fgb_device_free(void* p);
int fgb_memcpy_htod(void* dst, const void* src, size_t bytes);
int fgb_memcpy_dtoh(void* dst, const void* src, size_t bytes);

/* vacuum hexahedra of the synthetic nanotip mesh of `spec`; the core spacing h that gives
 * about target_hexes of them (spec's own h ignored); -1 on error */
long long fgb_nanotip_vacuum_hexes(const FgbNanotip* spec);
double fgb_nanotip_fit_spacing(const FgbNanotip* spec, double target_hexes);

/* ============================================================ Part 3: batched solves
 * Many meshes resident on one device in block-diagonal arrays, each solved by
 * multigrid-preconditioned FP64 CG with its own scalars; one CUDA graph launch advances
 * every admitted mesh. Meshes are added (admission by free device memory), solves are
 * admitted with an applied field (Neumann value -E0 on the top, phi = 0 on the metal, warm
 * start from the mesh's previous solution), stepped and collected. */
typedef struct FGB_BATCH FGB_BATCH;
/* use_graph: 1 = capture the iteration in a CUDA graph with a WHILE node, 2 = run each step as
 * one persistent cooperative kernel (grid-wide barriers between the phases, same results bit
 * for bit), 0 = host loop; autotune: time threads-per-row variants per level; grid_ctas:
 * 0 = 8 per SM (the work-list kernels of modes 0 and 1) */
FGB_BATCH* fgb_batch_create(int use_graph, int autotune, int grid_ctas);
void fgb_batch_free(FGB_BATCH* b);
/* slot >= 0; -1 when the free device memory minus hbm_reserve bytes does not admit the
 * mesh; INT32_MIN on error */
int fgb_batch_add_mesh(FGB_BATCH* b, const FGB_MESH* m, double hbm_reserve);
/* build n synthetic nanotip meshes on n_threads host threads (0: all cores) and add them;
 * slots[i] as fgb_batch_add_mesh */
int fgb_batch_add_synthetic(FGB_BATCH* b, int n, const FgbNanotip* specs, int n_threads, double hbm_reserve, int* slots);
int fgb_batch_remove_mesh(FGB_BATCH* b, int slot);
int fgb_batch_admit(FGB_BATCH* b, int slot, double E0, double rel_tol, int max_iter);
/* at most max_iters iterations of every admitted mesh; returns how many are still running */
int fgb_batch_step(FGB_BATCH* b, int max_iters);
/* finished solves since the last call: slots[k], res4 = iterations, status (1 converged,
 * -1 iteration cap, -2 breakdown), relative residual, |b|; returns the count */
int fgb_batch_collect(FGB_BATCH* b, int cap, int* slots, double* res4);
/* nodal phi/E recovery (+ smoothing) and device-pointer interpolation on the slot's stream */
int fgb_batch_extract(FGB_BATCH* b, int slot, int smoothen);
int fgb_batch_interpolate(FGB_BATCH* b, int slot, int n, const double* d_xyz, int rank, int* d_cells, double* d_out5);
int fgb_batch_sync_slot(FGB_BATCH* b, int slot);
int fgb_batch_export_phi_nodes(FGB_BATCH* b, int slot, double* phi_nodes);
int fgb_batch_export_nodal(FGB_BATCH* b, int slot, double* sol5_nodes);
int fgb_batch_reset_solution(FGB_BATCH* b, int slot);
/* ||b - A x|| / ||b|| in FP64 for the slot's current solution */
int fgb_batch_true_residual(FGB_BATCH* b, int slot, double* out);
int fgb_batch_info(FGB_BATCH* b, int slot, int64_t* out4); /* n_dofs, n_nodes, levels, 0 */
/* total dofs, device bytes, iterations of the last step, kernels per iteration, graph
 * launches, slots */
int fgb_batch_stats(FGB_BATCH* b, double* out6);
int fgb_batch_tuning(FGB_BATCH* b, char* buf, int cap);
/* CUDA event k (0..7) on the batch's solver stream; device ms between two events (-1 on error) */
int fgb_batch_mark(FGB_BATCH* b, int k);
double fgb_batch_elapsed(FGB_BATCH* b, int k0, int k1);

/* ============================================================ Part 4: serving
 * Field solves requested by concurrent MD runs, each with a resident mesh (a batch slot),
 * resident atoms and a result buffer. A request displaces the run's atoms by a Gaussian
 * step on the device, re-solves warm-started from the run's previous phi with the given
 * applied field, recovers the nodal field and interpolates E and phi at the atoms. One
 * scheduler thread batches continuously: requests arriving while others are on the device
 * join the next bounded solver launch; runs are admitted by free device memory. */
typedef struct FGB_SERVER FGB_SERVER;
FGB_SERVER* fgb_server_create(FGB_BATCH* b, double rel_tol, int max_iter, int iters_per_launch, int rank, int smoothen,
                              double hbm_reserve);
void fgb_server_free(FGB_SERVER* s);
/* launch policy, before fgb_server_start: solver iterations per graph launch while no request
 * waits for admission (idle_iters; 0 = iters_per_launch), and whether a launch ends after the
 * iteration in which one of its solves finished (stop_at_first) */
int fgb_server_set_launch_policy(FGB_SERVER* s, int idle_iters, int stop_at_first);
/* register a run (mesh placed by fgb_server_place_pending or later by the scheduler) */
int fgb_server_add_run(FGB_SERVER* s, const FGB_MESH* m, const double* xyz, int n_atoms, unsigned long long seed);
/* n synthetic runs: nanotip meshes of specs[i], n_atoms points each (surface atoms, topped
 * up with vacuum probes), built on host threads and placed */
int fgb_server_add_synthetic_runs(FGB_SERVER* s, int n, const FgbNanotip* specs, int n_atoms, unsigned long long seed,
                                  int n_threads);
int fgb_server_place_pending(FGB_SERVER* s, int n_threads); /* runs placed so far */
long long fgb_server_submit(FGB_SERVER* s, int run, double E0, double sigma); /* request id, -1 on error */
int fgb_server_start(FGB_SERVER* s);
int fgb_server_stop(FGB_SERVER* s);
int fgb_server_drain(FGB_SERVER* s, double timeout_s); /* 0 drained, 2 timed out */
/* Poisson arrivals: n requests at `rate` per second on uniformly chosen runs, applied field
 * base_fields[run] x (1 + 0.01 N(0,1)); returns when all have completed */
int fgb_server_run_poisson(FGB_SERVER* s, double rate, int n, double sigma, unsigned long long seed,
                           const double* base_fields);
/* completed requests: id, run, E0, iterations, status, rel_residual, t_submit, t_admit,
 * t_solved, t_done (seconds since the server was created); returns the count */
int fgb_server_records(FGB_SERVER* s, int cap, double* out10);
int fgb_server_clear_records(FGB_SERVER* s);
int fgb_server_last_result(FGB_SERVER* s, int run, double* out5, int* cells);
int fgb_server_reset_run(FGB_SERVER* s, int run); /* server stopped: zero warm start, initial atoms */
int fgb_server_info(FGB_SERVER* s, double* out4);  /* runs, solver launches, max requests in flight, 0 */
int fgb_server_run_info(FGB_SERVER* s, int run, int64_t* out2); /* slot (-1 pending), n_atoms */

/* ============================ Part 5: current and heat (bulk) ============================
 * The GPU counterpart of the reference's CurrentHeatSolver (src/CurrentHeatSolver.cpp) on the
 * bulk (metal) hexahedra of a mesh: Q1, 2x2x2 Gauss, boundary marking of
 * CurrentHeatSolver::mark_mesh (:535-539: x/y extremes natural, z min = copper bottom, the rest
 * = copper surface). Surface values are given per copper-surface face, in the order
 * fgb_heat_surface_faces lists them (the reference's order: bulk cells ascending, deal.II faces
 * x-, x+, y-, y+, z-, z+). The emission model that produces them is outside this library. */
typedef struct FGB_HEAT FGB_HEAT;
FGB_HEAT* fgb_heat_create(const FGB_MESH* m);
void fgb_heat_free(FGB_HEAT* h);
int fgb_heat_sizes(FGB_HEAT* h, int64_t* out3); /* n_dofs, nnz, n_surface_faces */
/* per surface face: centroid (3 doubles) and (hex id, femocs local face 0..5); either may be NULL */
int fgb_heat_surface_faces(FGB_HEAT* h, double* centroid3, int* hex_face2);
/* PhysicalQuantities resistivity table (src/PhysicalQuantities.cpp:31-64, 173-184): T ascending;
 * rho(T) = 10 * linear interpolation, T clamped to the table; sigma = 1/rho,
 * kappa = lorentz * T * sigma */
int fgb_heat_set_resistivity(FGB_HEAT* h, int n, const double* T, const double* rho);
/* CurrentHeatSolver::setup: T = t_ambient (also the bottom value), phi = 0; lorentz number and
 * volumetric heat capacity rho_cp [J/(K A^3)] (the reference uses 2.44e-8 and 3.4496e-24) */
int fgb_heat_setup(FGB_HEAT* h, double t_ambient, double lorentz, double rho_cp);
/* CurrentSolver::assemble + solve (:421-489): Laplace with sigma = 1, Neumann j per surface face,
 * phi = 0 at the bottom. Returns #iterations (< 0: not converged; INT32_MIN: error); precision
 * as fgb_field_solve; stats14 as fgb_field_last_stats (may be NULL) */
int fgb_heat_solve_current(FGB_HEAT* h, const double* face_j, int precision, double rel_tol, int max_iter,
                           double* stats14);
/* HeatSolver::assemble(dt) + solve (:116-153, :347-398): implicit Euler with
 * gamma = rho_cp / dt [s], kappa(T_prev), Joule source sigma(T_prev) |grad phi|^2, heat flux q per
 * surface face, T = t_ambient at the bottom */
int fgb_heat_solve_heat(FGB_HEAT* h, double delta_time_s, const double* face_q, int precision, double rel_tol,
                        int max_iter, double* stats14);
/* per hex-mesh node (NaN outside the bulk): temperature and current potential; either may be NULL */
int fgb_heat_export(FGB_HEAT* h, double* T_node, double* phi_node);
int fgb_heat_temperature_range(FGB_HEAT* h, double* out2); /* HeatSolver::check_limits extremes */

#ifdef __cplusplus
}
#endif
#endif

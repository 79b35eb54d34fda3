// Many independent Poisson systems resident on one GPU, solved together.
//
// Every mesh's system and multigrid hierarchy is placed into shared block-diagonal arrays:
// at each multigrid level a mesh owns a 256-row aligned range of rows (one CTA work unit
// = one 256-row block, so no block mixes meshes), the level-0 matrix is SELL-32 with
// 4-wide row chunks in FP64 and FP32, coarser levels and the transfer operators are FP32
// CSR addressed by (row begin, row length). Each mesh has its own CG scalars on the device,
// and dot products reduce per mesh in a fixed order (block partials, then the mesh's last
// block sums them), so a mesh's result does not depend on which other meshes share the
// launch.
//
// Kernels walk work lists of active 256-row blocks with a fixed grid, so the captured CUDA
// graph of one PCG iteration (FP64 SpMV, update, FP32 V-cycle, dot, direction) stays valid
// while meshes join and leave; only the lists (device arrays) change between launches. A
// mesh joins between iterations in phase NEW: its first pass through the iteration body
// computes r = b - A x from its warm start instead of the CG update. The body runs inside
// a conditional WHILE node that the device ends when every admitted mesh has converged or
// an iteration cap is reached.
#pragma once

#include <map>
#include <memory>
#include <mutex>

#include "amg.h"
#include "interp.h"
#include "prepared.h"

namespace fgb {

constexpr int kBatchRows = 256;   // rows per work unit (one CTA)

// First-fit allocator of element ranges inside one growable device array.
class RangePool {
public:
    explicit RangePool(size_t align = 1) : align_(align) {}
    // returns the offset, growing the capacity (by at least doubling) when needed
    size_t alloc(size_t n);
    void free(size_t off, size_t n);
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }
    bool grew() const { return grew_; }
    void clear_grew() { grew_ = false; }

private:
    size_t align_, cap_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    bool grew_ = false;
};

// Per-mesh scalars of the batched PCG (device array, one entry per slot).
struct BatchMeshState {
    double rz, alpha, beta, rr, tol2, bnorm;
    int iter, max_iter, done, status, phase;  // phase 0 NEW, 1 RUNNING
    unsigned int ticket;
    int blk0, nblk0;      // level-0 blocks [blk0, blk0 + nblk0)
    int depth;            // index of the mesh's dense (coarsest) level
    int dense_n;          // rows of the dense level
    long long dense_off;  // offset of the dense inverse in the dense pool
    int dense_row0;       // first row of the dense level in that level's row space
    int pad;
};

struct BatchSolveResult {
    int iterations = 0, status = 0;
    double rel_residual = 0;  // recursive residual at exit
    double bnorm = 0;
};

struct BatchOptions {
    int grid_ctas = 0;          // CTAs of the work-list kernels (0: 8 per SM)
    bool use_graph = true;      // capture the iteration as a CUDA graph with a WHILE node
    bool persistent = false;    // one persistent cooperative kernel per step instead (grid barriers between phases)
    bool autotune = true;       // pick threads-per-row of each coarse level by timing
};

struct BatchLevelDev;  // device arrays of one multigrid level (batch.cu)

class BatchSolver {
public:
    explicit BatchSolver(const BatchOptions& opt = BatchOptions());
    ~BatchSolver();
    BatchSolver(const BatchSolver&) = delete;
    BatchSolver& operator=(const BatchSolver&) = delete;

    // Build a mesh's system (Neumann top, phi = 0 on the metal, unit applied field),
    // its multigrid hierarchy and its interpolator, and place them into the shared arrays.
    // `hbm_reserve` bytes must stay free on the device after the placement, else the mesh
    // is not admitted and -1 is returned. Returns the slot.
    int add_mesh(std::shared_ptr<const PreparedMesh> pm, size_t hbm_reserve = 0);
    void remove_mesh(int slot);
    // bytes the placement of a mesh with n_dofs unknowns is expected to take (admission)
    static size_t estimate_bytes(long long n_dofs, long long n_hexs);

    // Queue a solve of `slot` with the given applied field (V/A, the Neumann value is -E0
    // on the top as in PoissonSolver::setup); warm start from the slot's last solution.
    void admit(int slot, double E0, double rel_tol, int max_iter);
    // Run at most `max_iters` iterations of every admitted, unfinished mesh (one graph
    // launch); with stop_at_first the launch also ends after the iteration in which a mesh
    // finished, so that its result can be taken at once. Returns the number of admitted
    // meshes still running afterwards.
    int step(int max_iters, bool stop_at_first = false);
    // Slots whose solve finished since the last call (converged or failed), with results.
    std::vector<std::pair<int, BatchSolveResult>> collect_finished();
    bool idle() const { return running_.empty(); }

    // Post-processing on the slot's own stream: nodal field (+ smoothing) and
    // location/interpolation of device points; phi / nodal export to the host.
    void extract(int slot, bool smoothen);
    DeviceMesh& interp(int slot);
    cudaStream_t slot_stream(int slot);
    void export_phi_nodes(int slot, double* phi_nodes);  // n_nodes values, 0 off the vacuum
    void reset_solution(int slot);                       // zero warm start
    double true_residual(int slot);                      // ||b - A x|| / ||b|| in FP64

    int n_slots() const { return (int)meshes_.size(); }
    int n_dofs(int slot) const;
    int n_nodes(int slot) const;
    int levels(int slot) const;
    long long total_rows() const;
    size_t device_bytes() const;
    std::string tuning() const;   // chosen threads-per-row per level
    cudaStream_t stream() const { return stream_; }
    long long launches() const { return launches_; }       // graph launches (or host loops)
    int last_iterations() const { return last_iters_; }    // iterations run by the last step
    int body_kernels() const { return body_kernels_; }     // kernels per iteration
    // CUDA events on the solver stream (k < 8) and the device time between two of them
    void mark(int k);
    float elapsed_ms(int a, int b);

private:
    struct Mesh;
    void place(Mesh& m, const FemStructure& fs, class FemDevice& fem, const AmgHost& h);
    void ensure_capacity();
    void rebuild_lists();
    void capture();
    void launch_iteration();      // one iteration body on stream_ (capture or fallback)
    void launch_persistent();     // the whole step as one cooperative kernel (kb_persistent)
    int persistent_grid_ = 0;
    void vcycle(int l);
    void tune();

    BatchOptions opt_;
    cudaStream_t stream_ = nullptr;
    int grid_ = 0;
    std::mutex mu_;
    std::vector<std::unique_ptr<Mesh>> meshes_;   // by slot (nullptr when removed)
    std::vector<int> running_;                    // admitted, not yet finished
    std::vector<int> admitted_pending_;
    int max_levels_ = 0;
    std::vector<std::unique_ptr<BatchLevelDev>> lv_;
    RangePool rows0_entries_{128};
    std::vector<std::unique_ptr<RangePool>> row_pools_, a_pools_, p_pools_, r_pools_;
    RangePool dense_pool_{64};
    // device arrays sized by the pools (batch.cu)
    struct Dev;
    std::unique_ptr<Dev> d_;
    bool dirty_ = true;           // layout changed: lists, graph and tuning are stale
    bool lists_dirty_ = true;
    cudaGraphExec_t exec_ = nullptr;
    cudaGraph_t graph_ = nullptr;
    long long launches_ = 0;
    std::vector<int> tpr_, p_tpr_, r_tpr_;
    std::map<long long, int> tune_cache_;  // size bucket -> threads per row
    std::vector<BatchMeshState> h_state_;
    int h_nrun_ = 0, body_kernels_ = 0, last_iters_ = 0;
    cudaEvent_t marks_[8] = {};
};

}  // namespace fgb

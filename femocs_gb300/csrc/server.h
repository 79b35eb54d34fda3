// Serving loop over a BatchSolver: field solves requested by concurrent MD runs.
//
// Each MD run owns a resident mesh (a batch slot), its atoms on the device and a result
// buffer. A request (run, applied field) displaces the run's atoms by a Gaussian step (on
// the device), re-solves the run's system warm-started from its previous phi, recovers the
// nodal field and interpolates E and phi at the atoms, then copies the result to the host.
// One scheduler thread does continuous batching: between bounded graph launches of the
// batch it admits every waiting request whose run is idle, so requests that arrive while
// others are on the device join the next launch; finished solves go straight to their
// run's stream for post-processing, which overlaps the next solver launches. Runs are
// admitted by free device memory: a run whose mesh does not fit waits until memory frees.
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>

#include "batch.h"

namespace fgb {

struct ServerOptions {
    double rel_tol = 1e-9;
    int max_iter = 500;
    int iters_per_launch = 4;     // solver iterations per graph launch between admissions
    int idle_iters = 0;           // per launch while no request waits (0: iters_per_launch)
    bool stop_at_first = false;   // end a launch after the iteration in which a solve finished
    int rank = 1;                 // interpolation rank (1 linear tet, 2 quadratic tet, 3 hex)
    bool smoothen = true;
    double hbm_reserve = 2e9;     // bytes left free when admitting a run's mesh
};

struct ServeRecord {
    long long id = 0;
    int run = 0;
    double E0 = 0;
    int iterations = 0, status = 0;
    double rel_residual = 0;
    double t_submit = 0, t_admit = 0, t_solved = 0, t_done = 0;  // seconds since server start
};

class FieldServer {
public:
    FieldServer(BatchSolver& batch, const ServerOptions& opt);
    ~FieldServer();

    // Register an MD run: mesh, atom positions (host, xyz interleaved). The mesh is placed
    // when free memory admits it (possibly later, by the scheduler). Returns the run id.
    int add_run(std::shared_ptr<const PreparedMesh> pm, const double* xyz, int n_atoms, uint64_t seed);
    // place the meshes of registered runs on n_threads host threads (0: all cores); runs
    // that free memory does not admit stay pending and are retried by the scheduler.
    // Returns how many runs are placed.
    int place_pending(int n_threads);
    // Submit one request (thread-safe); sigma: Gaussian displacement of every coordinate.
    long long submit(int run, double E0, double sigma);
    void start();
    void stop();
    // launch policy (before start): iterations per launch while no request waits, and whether
    // a launch ends as soon as one of its solves finished
    void set_launch_policy(int idle_iters, bool stop_at_first);
    // block until every submitted request has completed (or the timeout in seconds passes)
    bool drain(double timeout_s);
    // Poisson arrivals at `rate` per second, n requests, runs chosen uniformly, applied
    // field of each run's request = base field x (1 + 0.01 N(0,1)); blocks until drained.
    void run_poisson(double rate, int n, double sigma, uint64_t seed, const std::vector<double>& base_field);

    std::vector<ServeRecord> records();
    void clear_records();
    int n_runs() const { return (int)runs_.size(); }
    int run_slot(int run) const;
    int n_atoms(int run) const;
    // last result of a run: n_atoms x (Ex, Ey, Ez, |E|, phi) and the located cells
    void last_result(int run, double* out5, int32_t* cells);
    // zero the run's warm start and restore its initial atoms and step counter
    void reset_run(int run);
    double now() const;
    long long admitted_launches() const { return launches_; }
    int max_in_flight() const { return max_in_flight_; }

private:
    struct Run;
    void loop();
    void try_place_runs();
    void finalize_ready();

    BatchSolver& b_;
    ServerOptions opt_;
    std::vector<std::unique_ptr<Run>> runs_;
    std::mutex qmu_;
    std::condition_variable qcv_;
    std::deque<std::pair<int, ServeRecord>> inbox_;  // (run, record with sigma in E0 slot)
    std::deque<double> inbox_sigma_;
    std::vector<ServeRecord> done_;
    std::atomic<bool> stop_{false};
    std::thread th_;
    std::chrono::steady_clock::time_point t0_;
    long long next_id_ = 0, submitted_ = 0, completed_ = 0;
    long long launches_ = 0;
    int max_in_flight_ = 0;
    double last_place_try_ = -1e30;
    std::mutex dmu_;
    std::condition_variable dcv_;
};

}  // namespace fgb

// Serving loop (see server.h) and the device-side MD step stand-in.
#include <algorithm>
#include <cmath>
#include <random>

#include "server.h"

#include <omp.h>

namespace fgb {

namespace {

// SplitMix64 finaliser (Steele, Lea, Flood 2014): a counter-based 64-bit hash
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// xyz += sigma * N(0,1) per coordinate; normal deviates by Box-Muller from two hashed
// uniforms of (seed, step, coordinate)
__global__ void k_jitter(double* __restrict__ xyz, long long n3, double sigma, unsigned long long seed, long long step) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const unsigned long long key = splitmix64(seed ^ splitmix64((unsigned long long)step * 0x100000001B3ull)) + 2ull * i;
    const double u1 = ((double)(splitmix64(key) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = ((double)(splitmix64(key + 1) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    xyz[i] += sigma * sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

}  // namespace

struct FieldServer::Run {
    int id = 0, slot = -1;
    std::shared_ptr<const PreparedMesh> pm;  // until the mesh is placed
    int n = 0;
    uint64_t seed = 0;
    long long step = 0;
    std::vector<double> h_xyz0;
    DBuf<double> xyz, out;
    DBuf<int32_t> cells;
    double* h_out = nullptr;
    int32_t* h_cells = nullptr;
    std::deque<std::pair<ServeRecord, double>> queue;  // record, sigma
    int stage = 0;                                     // 0 idle, 1 solving, 2 post-processing
    ServeRecord cur;
    cudaEvent_t ev = nullptr;
};

FieldServer::FieldServer(BatchSolver& batch, const ServerOptions& opt) : b_(batch), opt_(opt) {
    t0_ = std::chrono::steady_clock::now();
}

FieldServer::~FieldServer() {
    stop();
    for (auto& r : runs_) {
        if (r->ev) cudaEventDestroy(r->ev);
        if (r->h_out) cudaFreeHost(r->h_out);
        if (r->h_cells) cudaFreeHost(r->h_cells);
    }
}

double FieldServer::now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

int FieldServer::add_run(std::shared_ptr<const PreparedMesh> pm, const double* xyz, int n_atoms, uint64_t seed) {
    FGB_REQUIRE(!th_.joinable(), "runs are registered before the server starts");
    FGB_REQUIRE(n_atoms > 0, "a run needs atoms");
    auto r = std::make_unique<Run>();
    r->id = (int)runs_.size();
    r->pm = std::move(pm);
    r->n = n_atoms;
    r->seed = seed;
    r->h_xyz0.assign(xyz, xyz + 3 * (size_t)n_atoms);
    r->xyz.upload(r->h_xyz0);
    r->out.resize(5 * (size_t)n_atoms);
    r->cells.resize(n_atoms);
    FGB_CUDA(cudaMallocHost(&r->h_out, 5 * sizeof(double) * n_atoms));
    FGB_CUDA(cudaMallocHost(&r->h_cells, sizeof(int32_t) * n_atoms));
    FGB_CUDA(cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming));
    FGB_CUDA(cudaDeviceSynchronize());
    runs_.push_back(std::move(r));
    return runs_.back()->id;
}

int FieldServer::place_pending(int n_threads) {
    FGB_REQUIRE(!th_.joinable(), "meshes are placed before the server starts");
    std::vector<Run*> todo;
    for (auto& r : runs_)
        if (r->slot < 0 && r->pm) todo.push_back(r.get());
    const int nt = std::max(1, std::min<int>(n_threads > 0 ? n_threads : (int)std::thread::hardware_concurrency(),
                                             (int)todo.size()));
    std::atomic<size_t> next{0};
    std::vector<std::string> err(nt);
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&, t] {
                omp_set_num_threads(1);  // the meshes are the parallelism: no nested teams
            try {
                for (size_t i = next++; i < todo.size(); i = next++) {
                    const int slot = b_.add_mesh(todo[i]->pm, (size_t)opt_.hbm_reserve);
                    if (slot >= 0) {
                        todo[i]->slot = slot;
                        todo[i]->pm.reset();
                    }
                }
            } catch (const std::exception& e) {
                err[t] = e.what();
            }
        });
    for (auto& th : pool) th.join();
    for (auto& e : err)
        if (!e.empty()) throw Error(e);
    int placed = 0;
    for (auto& r : runs_) placed += r->slot >= 0;
    return placed;
}

void FieldServer::try_place_runs() {
    for (auto& r : runs_) {
        if (r->slot >= 0 || !r->pm) continue;
        const int slot = b_.add_mesh(r->pm, (size_t)opt_.hbm_reserve);
        if (slot < 0) continue;  // not admitted: free memory too low, retried later
        r->slot = slot;
        r->pm.reset();
    }
}

int FieldServer::run_slot(int run) const { return runs_.at(run)->slot; }
int FieldServer::n_atoms(int run) const { return runs_.at(run)->n; }

long long FieldServer::submit(int run, double E0, double sigma) {
    FGB_REQUIRE(run >= 0 && run < (int)runs_.size(), "no such run");
    ServeRecord rec;
    rec.run = run;
    rec.E0 = E0;
    rec.t_submit = now();
    {
        std::lock_guard<std::mutex> lk(qmu_);
        rec.id = next_id_++;
        inbox_.push_back({run, rec});
        inbox_sigma_.push_back(sigma);
        ++submitted_;
    }
    qcv_.notify_one();
    return rec.id;
}

void FieldServer::start() {
    if (th_.joinable()) return;
    stop_ = false;
    th_ = std::thread([this] { loop(); });
}

void FieldServer::set_launch_policy(int idle_iters, bool stop_at_first) {
    FGB_REQUIRE(!th_.joinable(), "the launch policy is set before the server starts");
    FGB_REQUIRE(idle_iters >= 0, "idle iterations per launch must be >= 0");
    opt_.idle_iters = idle_iters;
    opt_.stop_at_first = stop_at_first;
}

void FieldServer::stop() {
    stop_ = true;
    qcv_.notify_all();
    if (th_.joinable()) th_.join();
}

bool FieldServer::drain(double timeout_s) {
    std::unique_lock<std::mutex> lk(dmu_);
    return dcv_.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        std::lock_guard<std::mutex> q(qmu_);
        return completed_ >= submitted_;
    });
}

void FieldServer::finalize_ready() {
    for (auto& r : runs_) {
        if (r->stage != 2) continue;
        const cudaError_t e = cudaEventQuery(r->ev);
        if (e == cudaErrorNotReady) continue;
        FGB_CUDA(e);
        r->cur.t_done = now();
        r->stage = 0;
        {
            std::lock_guard<std::mutex> lk(dmu_);
            done_.push_back(r->cur);
            std::lock_guard<std::mutex> q(qmu_);
            ++completed_;
        }
        dcv_.notify_all();
    }
}

void FieldServer::loop() {
    std::vector<int> slot2run;
    try {
        while (!stop_) {
            {
                std::lock_guard<std::mutex> lk(qmu_);
                while (!inbox_.empty()) {
                    auto item = inbox_.front();
                    inbox_.pop_front();
                    const double sigma = inbox_sigma_.front();
                    inbox_sigma_.pop_front();
                    runs_[item.first]->queue.push_back({item.second, sigma});
                }
            }
            if (now() - last_place_try_ > 0.5) {  // pending runs: retry admission twice a second
                last_place_try_ = now();
                try_place_runs();
            }
            slot2run.assign(std::max(1, b_.n_slots()), -1);
            for (auto& r : runs_)
                if (r->slot >= 0) slot2run[r->slot] = r->id;
            // admit every waiting request whose run is idle (continuous batching)
            for (auto& r : runs_) {
                if (r->slot < 0 || r->stage != 0 || r->queue.empty()) continue;
                auto [rec, sigma] = r->queue.front();
                r->queue.pop_front();
                r->step += 1;
                const long long n3 = 3LL * r->n;
                cudaStream_t s = b_.slot_stream(r->slot);
                if (sigma > 0)
                    FGB_LAUNCH(k_jitter<<<grid_for(n3, 256), 256, 0, s>>>(r->xyz.get(), n3, sigma, r->seed, r->step));
                b_.admit(r->slot, rec.E0, opt_.rel_tol, opt_.max_iter);
                rec.t_admit = now();
                r->cur = rec;
                r->stage = 1;
            }
            int in_flight = 0;
            for (auto& r : runs_) in_flight += r->stage != 0;
            max_in_flight_ = std::max(max_in_flight_, in_flight);
            if (!b_.idle()) {
                // short launches while requests wait for admission (new arrivals or runs
                // that are busy), long ones otherwise
                bool waiting = false;
                {
                    std::lock_guard<std::mutex> lk(qmu_);
                    waiting = !inbox_.empty();
                }
                for (auto& r : runs_) waiting = waiting || !r->queue.empty();
                const int cap = !waiting && opt_.idle_iters > 0 ? opt_.idle_iters : opt_.iters_per_launch;
                b_.step(cap, opt_.stop_at_first);
                ++launches_;
                for (auto& [slot, res] : b_.collect_finished()) {
                    Run& r = *runs_[slot2run[slot]];
                    r.cur.iterations = res.iterations;
                    r.cur.status = res.status;
                    r.cur.rel_residual = res.rel_residual;
                    r.cur.t_solved = now();
                    cudaStream_t s = b_.slot_stream(slot);
                    b_.extract(slot, opt_.smoothen);
                    b_.interp(slot).locate_interpolate(r.n, r.xyz.get(), opt_.rank, r.cells.get(), r.out.get(), nullptr);
                    FGB_CUDA(cudaMemcpyAsync(r.h_out, r.out.get(), 5 * sizeof(double) * r.n, cudaMemcpyDeviceToHost, s));
                    FGB_CUDA(cudaMemcpyAsync(r.h_cells, r.cells.get(), sizeof(int32_t) * r.n, cudaMemcpyDeviceToHost, s));
                    FGB_CUDA(cudaEventRecord(r.ev, s));
                    r.stage = 2;
                }
            }
            finalize_ready();
            bool post = false, queued = false;
            for (auto& r : runs_) {
                post = post || r->stage == 2;
                queued = queued || (!r->queue.empty() && r->stage == 0 && r->slot >= 0);
            }
            if (b_.idle() && !queued) {
                if (post) {
                    std::this_thread::sleep_for(std::chrono::microseconds(20));
                } else {
                    std::unique_lock<std::mutex> lk(qmu_);
                    qcv_.wait_for(lk, std::chrono::milliseconds(2), [&] { return !inbox_.empty() || stop_; });
                }
            }
        }
    } catch (const std::exception& e) {
        set_last_error(std::string("server loop stopped: ") + e.what());
        std::lock_guard<std::mutex> q(qmu_);
        completed_ = submitted_;  // release drain() waiters; records show what finished
        dcv_.notify_all();
    }
}

void FieldServer::run_poisson(double rate, int n, double sigma, uint64_t seed, const std::vector<double>& base_field) {
    FGB_REQUIRE(rate > 0 && n >= 0, "rate must be positive");
    FGB_REQUIRE((int)base_field.size() == (int)runs_.size(), "one base field per run");
    std::mt19937_64 g(seed);
    std::exponential_distribution<double> gap(rate);
    std::uniform_int_distribution<int> pick(0, (int)runs_.size() - 1);
    std::normal_distribution<double> var(0.0, 1.0);
    const auto start = std::chrono::steady_clock::now();
    double t = 0;
    for (int i = 0; i < n; ++i) {
        t += gap(g);
        const int run = pick(g);
        const double E0 = base_field[run] * (1.0 + 0.01 * var(g));
        std::this_thread::sleep_until(start + std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                                                  std::chrono::duration<double>(t)));
        submit(run, E0, sigma);
    }
    drain(600.0);
}

std::vector<ServeRecord> FieldServer::records() {
    std::lock_guard<std::mutex> lk(dmu_);
    return done_;
}

void FieldServer::clear_records() {
    std::lock_guard<std::mutex> lk(dmu_);
    done_.clear();
}

void FieldServer::last_result(int run, double* out5, int32_t* cells) {
    Run& r = *runs_.at(run);
    FGB_REQUIRE(r.stage == 0, "the run has a request in flight");
    if (out5) std::copy(r.h_out, r.h_out + 5 * (size_t)r.n, out5);
    if (cells) std::copy(r.h_cells, r.h_cells + r.n, cells);
}

void FieldServer::reset_run(int run) {
    FGB_REQUIRE(!th_.joinable(), "runs are reset while the server is stopped");
    Run& r = *runs_.at(run);
    FGB_REQUIRE(r.stage == 0 && r.queue.empty(), "the run has requests in flight");
    FGB_REQUIRE(r.slot >= 0, "the run's mesh is not placed");
    b_.reset_solution(r.slot);
    cudaStream_t s = b_.slot_stream(r.slot);
    FGB_CUDA(cudaMemcpyAsync(r.xyz.get(), r.h_xyz0.data(), sizeof(double) * r.h_xyz0.size(), cudaMemcpyHostToDevice, s));
    FGB_CUDA(cudaStreamSynchronize(s));
    r.step = 0;
}

}  // namespace fgb

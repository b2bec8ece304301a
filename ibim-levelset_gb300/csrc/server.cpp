// Request loop on one GPU (no counterpart in the reference: main.cpp solves one molecule per
// process).  Solve requests queue in arrival order and are admitted by device memory in two
// phases: a request starts (its level set) when its grids fit in the HBM budget beside what the
// requests in flight hold, and once its tree and lists are built its FMM phase (operator images,
// expansions, Krylov basis) is admitted by the bytes its exact operator, node and point counts
// need; a phase is always admitted when no other request holds memory of that phase, so the loop
// cannot stall.
//
// Two ways to run the admitted requests:
//   pool      (ibim_server_create) `slots` worker threads, each with its own context, run whole
//             solves concurrently on the device
//   lock-step (ibim_server_create_lockstep) worker threads prepare requests (level set, tube,
//             right-hand side, plan, operator images; batch.cu) while two solver threads take the
//             prepared requests in waves: a wave merges their plans so that every FMM stage is one
//             launch for all of them, and their GMRES iterations advance together.  Requests that
//             arrive while a wave runs are prepared meanwhile and join the next wave (continuous
//             batching at wave granularity); a wave holds requests of one shape (h, order, eps).
// Each request keeps its level set, tree, operators and Krylov basis resident until it finishes.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "solve.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long id = 0;
    std::vector<double> centers, charges, radii;
    ibim_config cfg{};
    double held = 0;    // device bytes this request holds in the budget
    bool fmm = false;   // past its level set
    Clock::time_point t_submit, t_start, t_end;
    int status = IBIM_OK;
    std::string error;
    ibim_result res{};
    bool done = false;
    ibim::BatchMol bm;  // lock-step: the prepared molecule
};

}  // namespace

struct ibim_server_s {
    int device = 0, slots = 1, max_wave = 1;
    bool lockstep = false;
    double budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;     // submitted, not started
    std::deque<Request *> prepared;  // lock-step: prepared, waiting for a wave
    std::map<long, std::unique_ptr<Request>> all;
    double in_flight_bytes = 0, peak_bytes = 0;
    int in_flight = 0, in_fmm = 0, preparing = 0;
    long next_id = 1, submitted = 0, completed = 0, waves = 0;
    bool stop = false;
    std::vector<std::thread> workers;
    std::vector<std::thread> solvers;  // lock-step: wave solvers (two waves at once)
    std::vector<ibim_ctx> wctx;  // the workers' contexts (prepared requests keep buffers on their streams)
};

namespace ibim {

// Level set: the grid, phi0 and the two stage buffers (four live during the reinitialisation)
// in the grid's precision, the flood-fill labels, and a margin for the tube arrays.
double estimate_levelset_bytes(const ibim_config &cfg) {
    const double cells = (double)cfg.n[0] * cfg.n[1] * cfg.n[2];
    const bool mixed = cfg.precision == IBIM_PRECISION_MIXED;
    return cells * (4.0 * (mixed ? 4.0 : 8.0) + 8.0) + 64e6;
}

// FMM phase for npoints tube points: tree nodes ~4.8 N / leaf size (15,193 nodes for 408,726
// points and 624,673 for 16.5 M at leaf 128), operators ~600 per tree level (2,239 for the
// 2,000-atom protein at 5 levels, 4,290 for 20,000 atoms at 7), each at the peak of its images
// (mixed: FP16 hi / lo tiles, BF16 digit tiles and the float-float operators they are cut from;
// FP64: the FP64 operator), per node the expansions and multipole images, per point ~1.1 KB plus
// the Krylov basis.
static double fmm_bytes(const ibim_config &cfg, double N, double nodes, double ops) {
    const double n4 = 4.0 * cfg.np * cfg.np * cfg.np;
    const double kpad = std::ceil(n4 / 16.0) * 16.0, mpad = std::ceil(n4 / 128.0) * 128.0;
    const double digits = kpad <= 800 ? 6.0 : 7.0;
    double per_op, per_node;
    if (cfg.precision == IBIM_PRECISION_FP64) {
        per_op = n4 * n4 * 8.0;
        per_node = n4 * 16.0;
    } else {
        per_op = 2.0 * mpad * kpad * 2.0 + digits * mpad * kpad * 2.0 + n4 * n4 * 8.0;
        per_node = n4 * 24.0 + kpad * 4.0 + digits * kpad * 2.0;
    }
    const double per_point = 1100.0 + 16.0 * (std::min(cfg.restart, 250) + 1);
    return ops * per_op + nodes * per_node + N * per_point;
}

double estimate_fmm_bytes(const ibim_config &cfg, long npoints) {
    const double N = (double)std::max(1L, npoints);
    const double mp = std::max(1, cfg.maxpoint);
    const double levels = std::ceil(std::log(std::max(1.0, N / mp)) / std::log(8.0)) + 1.0;
    return fmm_bytes(cfg, N, 4.8 * N / mp + 1.0, 600.0 * std::max(1.0, levels));
}

double plan_fmm_bytes(const Plan &P, const ibim_config &cfg) {
    return fmm_bytes(cfg, (double)P.ns, (double)P.tree.nnodes, (double)P.nops);
}

// Before the level set runs the tube size is unknown: guessed as a fifth of the grid's cells in
// a shell (the benchmark proteins' tubes hold 1/5.4 (2,000 atoms) to 1/9.2 (20,000 atoms) of the
// cells); the loops admit the FMM phase again with the real count.
double estimate_request_bytes(const ibim_config &cfg) {
    const double cells = (double)cfg.n[0] * cfg.n[1] * cfg.n[2];
    return std::max(estimate_levelset_bytes(cfg), estimate_fmm_bytes(cfg, (long)(cells / 5.0)));
}

void set_last_error(const std::string &msg);

}  // namespace ibim

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Admission of the head of the queue (its level set); called with the lock held.
bool can_start(ibim_server_s *S) {
    if (S->queue.empty()) return false;
    return S->in_flight == 0 || S->in_flight_bytes + ibim::estimate_levelset_bytes(S->queue.front()->cfg) <= S->budget;
}

Request *take_head(ibim_server_s *S) {
    Request *r = S->queue.front();
    S->queue.pop_front();
    S->in_flight++;
    r->held = ibim::estimate_levelset_bytes(r->cfg);
    S->in_flight_bytes += r->held;
    S->peak_bytes = std::max(S->peak_bytes, S->in_flight_bytes);
    r->t_start = Clock::now();
    return r;
}

// The FMM-phase admission of request r needing `bytes` (its grids are released first).
std::function<void(long)> fmm_admission(ibim_server_s *S, Request *r) {
    return [S, r](long bytes) {
        const double need = (double)bytes;
        std::unique_lock<std::mutex> lk(S->mu);
        S->in_flight_bytes -= r->held;
        r->held = 0;
        S->cv_work.notify_all();
        S->cv_work.wait(lk, [&] { return S->in_fmm == 0 || S->in_flight_bytes + need <= S->budget; });
        r->held = need;
        r->fmm = true;
        S->in_fmm++;
        S->in_flight_bytes += need;
        S->peak_bytes = std::max(S->peak_bytes, S->in_flight_bytes);
    };
}

// Request r finished (status set); called with the lock held.
void finish(ibim_server_s *S, Request *r) {
    r->t_end = Clock::now();
    S->in_flight--;
    S->in_flight_bytes = S->in_flight == 0 ? 0.0 : S->in_flight_bytes - r->held;
    r->held = 0;
    if (r->fmm) S->in_fmm--;
    S->completed++;
    r->done = true;
}

void pool_worker(ibim_server_s *S) {
    ibim_ctx ctx = nullptr;
    const int crc = ibim_ctx_create(S->device, &ctx);
    const std::string cerr = crc == IBIM_OK ? "" : ibim_last_error();
    for (;;) {
        Request *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return (S->stop && S->queue.empty()) || can_start(S); });
            if (S->queue.empty()) break;  // stop requested and nothing left
            r = take_head(S);
        }
        if (crc != IBIM_OK) {
            r->status = crc;
            r->error = cerr;
        } else {
            const std::function<void(long)> admit = fmm_admission(S, r);
            try {
                ibim::solve_host(&ctx->c, r->centers.data(), r->charges.data(), r->radii.data(),
                                 (int)r->charges.size(), r->cfg, r->res, &admit);
                r->status = IBIM_OK;
            } catch (const ibim::Error &e) {
                r->status = e.status;
                r->error = e.what();
            } catch (const std::exception &e) {
                r->status = IBIM_ERR_INVALID_ARGUMENT;
                r->error = e.what();
            }
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            finish(S, r);
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
    if (ctx) ibim_ctx_destroy(ctx);
}

void lockstep_worker(ibim_server_s *S, int t) {
    ibim_ctx ctx = S->wctx[t];
    for (;;) {
        Request *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return (S->stop && S->queue.empty()) || can_start(S); });
            if (S->queue.empty()) break;
            r = take_head(S);
            S->preparing++;
        }
        const std::function<void(long)> admit = fmm_admission(S, r);
        int st = IBIM_OK;
        std::string err;
        if (!ctx) {
            st = IBIM_ERR_CUDA;
            err = "server: no context for a preparation thread";
        } else {
            try {
                ibim::check_config(r->cfg);
                IBIM_REQUIRE(r->cfg.precision == IBIM_PRECISION_MIXED,
                             "server (lock-step): requests run the mixed-precision path");
                IBIM_CUDA(cudaSetDevice(S->device));
                ibim::set_current_ctx(&ctx->c);
                ibim::batch_prepare(&ctx->c, r->centers.data(), r->charges.data(), r->radii.data(),
                                    (int)r->charges.size(), r->cfg, r->res, r->bm, &admit);
                r->bm.index = 0;
            } catch (const ibim::Error &e) {
                st = e.status;
                err = e.what();
            } catch (const std::exception &e) {
                st = IBIM_ERR_INVALID_ARGUMENT;
                err = e.what();
            }
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->preparing--;
            if (st == IBIM_OK) {
                S->in_flight_bytes += r->bm.bytes - r->held;  // the prepared plan's own bytes
                r->held = r->bm.bytes;
                S->peak_bytes = std::max(S->peak_bytes, S->in_flight_bytes);
                S->prepared.push_back(r);
            } else {
                delete r->bm.prep;
                r->bm.prep = nullptr;
                delete r->bm.b_tree;
                r->bm.b_tree = nullptr;
                r->status = st;
                r->error = err;
                finish(S, r);
            }
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
}

void lockstep_solver(ibim_server_s *S) {
    ibim_ctx ctx = nullptr;
    const int crc = ibim_ctx_create(S->device, &ctx);
    const std::string cerr = crc == IBIM_OK ? "" : ibim_last_error();
    for (;;) {
        std::vector<Request *> wave;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] {
                return !S->prepared.empty() || (S->stop && S->queue.empty() && S->preparing == 0);
            });
            if (S->prepared.empty()) break;
            // the oldest prepared request and the prepared requests of its shape, in order
            const ibim_config key = S->prepared.front()->cfg;
            for (auto it = S->prepared.begin(); it != S->prepared.end() && (int)wave.size() < S->max_wave;) {
                if (ibim::batch_compatible((*it)->cfg, key)) {
                    wave.push_back(*it);
                    it = S->prepared.erase(it);
                } else {
                    ++it;
                }
            }
        }
        int st = crc;
        std::string err = cerr;
        std::vector<ibim::BatchMol> bm(wave.size());
        for (size_t k = 0; k < wave.size(); ++k) {
            bm[k] = wave[k]->bm;
            bm[k].index = (int)k;
            wave[k]->bm.prep = nullptr;
            wave[k]->bm.b_tree = nullptr;
        }
        if (crc == IBIM_OK) {
            try {
                IBIM_CUDA(cudaSetDevice(S->device));
                ibim::set_current_ctx(&ctx->c);
                ibim::WaveStats ws;
                ibim::batch_wave(&ctx->c, bm, ws);
            } catch (const ibim::Error &e) {
                st = e.status;
                err = e.what();
            } catch (const std::exception &e) {
                st = IBIM_ERR_INVALID_ARGUMENT;
                err = e.what();
            }
        }
        for (auto &b : bm) {
            delete b.prep;
            delete b.b_tree;
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->waves++;
            for (Request *r : wave) {
                r->status = st;
                r->error = err;
                finish(S, r);
            }
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
    if (ctx) ibim_ctx_destroy(ctx);
}

void stop_threads(ibim_server_s *S) {
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto &t : S->workers)
        if (t.joinable()) t.join();
    for (auto &t : S->solvers)
        if (t.joinable()) t.join();
    for (ibim_ctx c : S->wctx)
        if (c) ibim_ctx_destroy(c);
    S->wctx.clear();
}

// waves solved at once by the lock-step loop, each on its own context and stream
constexpr int kWaveSlots = 3;

int create(int device, int slots, int max_wave, double budget, bool lockstep, ibim_server *out) {
    if (!out || slots < 1 || slots > 64 || !(budget > 0) || max_wave < 1) {
        ibim::set_last_error("server: need an output handle, 1..64 threads, a positive wave size and HBM budget");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        ibim::set_last_error("server: no such CUDA device");
        return IBIM_ERR_CUDA;
    }
    auto *S = new ibim_server_s();
    S->device = device;
    S->slots = slots;
    S->max_wave = max_wave;
    S->lockstep = lockstep;
    S->budget = budget;
    try {
        if (lockstep) {
            S->wctx.assign(slots, nullptr);
            for (int i = 0; i < slots; ++i)
                if (ibim_ctx_create(device, &S->wctx[i]) != IBIM_OK) S->wctx[i] = nullptr;
            for (int i = 0; i < slots; ++i) S->workers.emplace_back(lockstep_worker, S, i);
            for (int i = 0; i < kWaveSlots; ++i) S->solvers.emplace_back(lockstep_solver, S);
        } else {
            for (int i = 0; i < slots; ++i) S->workers.emplace_back(pool_worker, S);
        }
    } catch (...) {
        stop_threads(S);
        delete S;
        ibim::set_last_error("server: could not start the worker threads");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    *out = S;
    return IBIM_OK;
}

}  // namespace

extern "C" {

int ibim_server_create(int device, int slots, double hbm_budget_bytes, ibim_server *out) {
    return create(device, slots, 1, hbm_budget_bytes, false, out);
}

int ibim_server_create_lockstep(int device, int workers, int max_wave, double hbm_budget_bytes, ibim_server *out) {
    return create(device, workers, max_wave, hbm_budget_bytes, true, out);
}

int ibim_server_destroy(ibim_server s) {
    if (!s) return IBIM_OK;
    stop_threads(s);
    delete s;
    return IBIM_OK;
}

int ibim_server_submit(ibim_server s, const double *centers, const double *charges, const double *radii, int natoms,
                       const ibim_config *cfg, long *id) {
    if (!s || !centers || !charges || !radii || !cfg || !id || natoms <= 0) {
        ibim::set_last_error("server submit: null argument or no atoms");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    auto r = std::make_unique<Request>();
    r->centers.assign(centers, centers + 3 * (size_t)natoms);
    r->charges.assign(charges, charges + natoms);
    r->radii.assign(radii, radii + natoms);
    r->cfg = *cfg;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            ibim::set_last_error("server submit: the server is shutting down");
            return IBIM_ERR_INVALID_ARGUMENT;
        }
        r->id = s->next_id++;
        *id = r->id;
        s->queue.push_back(r.get());
        s->all.emplace(r->id, std::move(r));
        s->submitted++;
    }
    s->cv_work.notify_all();
    return IBIM_OK;
}

static int report(ibim_server s, long id, bool block, int *done, int *status, ibim_result *res, double *latency_ms,
                  double *run_ms) {
    if (!s) {
        ibim::set_last_error("server: null handle");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) {
        ibim::set_last_error("server: unknown or already collected request id");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    Request *r = it->second.get();
    if (block) s->cv_done.wait(lk, [&] { return r->done; });
    if (done) *done = r->done ? 1 : 0;
    if (!r->done) return IBIM_OK;
    if (status) *status = r->status;
    if (res) *res = r->res;
    if (latency_ms) *latency_ms = ms_between(r->t_submit, r->t_end);
    if (run_ms) *run_ms = ms_between(r->t_start, r->t_end);
    if (r->status != IBIM_OK) ibim::set_last_error(r->error);
    s->all.erase(it);  // collected
    return IBIM_OK;
}

int ibim_server_poll(ibim_server s, long id, int *done, int *status, ibim_result *res, double *latency_ms,
                     double *run_ms) {
    return report(s, id, false, done, status, res, latency_ms, run_ms);
}

int ibim_server_wait(ibim_server s, long id, int *status, ibim_result *res, double *latency_ms, double *run_ms) {
    int done = 0;
    return report(s, id, true, &done, status, res, latency_ms, run_ms);
}

int ibim_server_stats(ibim_server s, double stats[8]) {
    if (!s || !stats) {
        ibim::set_last_error("server stats: null argument");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    stats[0] = (double)s->submitted;
    stats[1] = (double)s->completed;
    stats[2] = (double)s->in_flight;
    stats[3] = (double)s->queue.size();
    stats[4] = s->in_flight_bytes;
    stats[5] = s->peak_bytes;
    stats[6] = s->budget;
    stats[7] = (double)s->waves;
    return IBIM_OK;
}

double ibim_request_bytes_estimate(const ibim_config *cfg) { return cfg ? ibim::estimate_request_bytes(*cfg) : 0.0; }

double ibim_fmm_bytes_estimate(const ibim_config *cfg, long npoints) {
    return cfg ? ibim::estimate_fmm_bytes(*cfg, npoints) : 0.0;
}

}  // extern "C"

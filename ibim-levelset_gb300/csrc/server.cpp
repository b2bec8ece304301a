// Request loop on one GPU: solve requests queue in arrival order; `slots` worker threads, each
// with its own context (stream, second stream, workspace), take the head of the queue whenever
// the estimated device footprints of the requests in flight plus the head's stay within the HBM
// budget (a request is always admitted when nothing is in flight).  Requests therefore run
// concurrently on the device, each keeping its level set, tree, operators and Krylov basis
// resident until it finishes; a finished request frees its slot and its share of the budget for
// the next one in the queue.
//
// No counterpart in the reference (main.cpp solves one molecule per process).

#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long id = 0;
    std::vector<double> centers, charges, radii;
    ibim_config cfg{};
    double bytes = 0;
    Clock::time_point t_submit, t_start, t_end;
    int status = IBIM_OK;
    std::string error;
    ibim_result res{};
    bool done = false;
};

}  // namespace

struct ibim_server_s {
    int device = 0, slots = 1;
    double budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::map<long, std::unique_ptr<Request>> all;
    double in_flight_bytes = 0, peak_bytes = 0;
    int in_flight = 0;
    long next_id = 1, submitted = 0, completed = 0;
    bool stop = false;
    std::vector<std::thread> workers;
};

namespace ibim {

// Device footprint of one solve, estimated from its configuration before it runs: level-set
// grids (five live at once), tube points (at most a twentieth of the cells, ~2 KB each with
// their tree, near lists and Krylov basis) and the M2L operators (about 320 per tree level; 8
// bytes per entry on the FP64 path; on the mixed path the peak of 26 while the images are cut:
// BF16 digit tiles 14 + FP32 operators 4 + 3xTF32 tiles 8).
double estimate_request_bytes(const ibim_config &cfg) {
    const double cells = (double)cfg.n[0] * cfg.n[1] * cfg.n[2];
    const bool mixed = cfg.precision == IBIM_PRECISION_MIXED;
    const double grids = cells * 5.0 * (mixed ? 4.0 : 8.0);
    const double points = cells / 20.0;
    const double levels = std::max(3.0, std::ceil(std::log(std::max(1.0, points / cfg.maxpoint)) / std::log(8.0)) + 2.0);
    const double n4 = 4.0 * cfg.np * cfg.np * cfg.np;
    const double ops = 320.0 * levels * n4 * n4 * (mixed ? 26.0 : 8.0);
    return grids + points * 2048.0 + ops;
}

}  // namespace ibim

namespace {

void worker(ibim_server_s *S) {
    ibim_ctx ctx = nullptr;
    const int crc = ibim_ctx_create(S->device, &ctx);
    const std::string cerr = crc == IBIM_OK ? "" : ibim_last_error();
    for (;;) {
        Request *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] {
                return S->stop || (!S->queue.empty() &&
                                   (S->in_flight == 0 || S->in_flight_bytes + S->queue.front()->bytes <= S->budget));
            });
            if (S->queue.empty()) break;  // stop requested and nothing left
            r = S->queue.front();
            S->queue.pop_front();
            S->in_flight++;
            S->in_flight_bytes += r->bytes;
            S->peak_bytes = std::max(S->peak_bytes, S->in_flight_bytes);
        }
        r->t_start = Clock::now();
        if (crc != IBIM_OK) {
            r->status = crc;
            r->error = cerr;
        } else {
            r->status = ibim_solve(ctx, r->centers.data(), r->charges.data(), r->radii.data(), (int)r->charges.size(),
                                   &r->cfg, &r->res);
            if (r->status != IBIM_OK) r->error = ibim_last_error();
        }
        r->t_end = Clock::now();
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->in_flight--;
            S->in_flight_bytes = S->in_flight == 0 ? 0.0 : S->in_flight_bytes - r->bytes;
            S->completed++;
            r->done = true;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
    if (ctx) ibim_ctx_destroy(ctx);
}

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

extern "C" {

int ibim_server_create(int device, int slots, double hbm_budget_bytes, ibim_server *out) {
    if (!out || slots < 1 || slots > 64 || !(hbm_budget_bytes > 0)) {
        ibim::set_last_error("server: need an output handle, 1..64 slots and a positive HBM budget");
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
    S->budget = hbm_budget_bytes;
    try {
        for (int i = 0; i < slots; ++i) S->workers.emplace_back(worker, S);
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
        }
        S->cv_work.notify_all();
        for (auto &t : S->workers) t.join();
        delete S;
        ibim::set_last_error("server: could not start the worker threads");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    *out = S;
    return IBIM_OK;
}

int ibim_server_destroy(ibim_server s) {
    if (!s) return IBIM_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
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
    r->bytes = ibim::estimate_request_bytes(*cfg);
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

int ibim_server_stats(ibim_server s, double stats[7]) {
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
    return IBIM_OK;
}

double ibim_request_bytes_estimate(const ibim_config *cfg) { return cfg ? ibim::estimate_request_bytes(*cfg) : 0.0; }

}  // extern "C"

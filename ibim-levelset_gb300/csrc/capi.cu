// The C ABI (include/ibim.h): status codes, handles, and the whole-path entry points.
// Every entry point catches library errors and returns a status; ibim_last_error() gives text.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "fmm_common.cuh"
#include "solve.cuh"

namespace ibim {

void *device_alloc(size_t bytes, cudaStream_t s) {
    void *p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, bytes, s);
    if (e == cudaSuccess) return p;
    if (e != cudaErrorMemoryAllocation) IBIM_CUDA(e);
    (void)cudaGetLastError();
    int dev = 0;
    IBIM_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    IBIM_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    IBIM_CUDA(cudaDeviceSynchronize());  // every stream's pending frees have happened
    IBIM_CUDA(cudaMemPoolTrimTo(pool, 0));
    e = cudaMallocAsync(&p, bytes, s);
    if (e == cudaSuccess) return p;
    (void)cudaGetLastError();
    size_t fr = 0, tot = 0;
    uint64_t reserved = 0, used = 0;
    cudaMemGetInfo(&fr, &tot);
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "device allocation of %.3f GB: out of memory (device free %.2f of %.2f GB; pool reserved %.2f GB, "
                  "in use %.2f GB)",
                  bytes / 1e9, fr / 1e9, tot / 1e9, reserved / 1e9, used / 1e9);
    throw Error(IBIM_ERR_OUT_OF_MEMORY, msg);
}

static thread_local std::string g_last_error;
static thread_local Ctx *g_current = nullptr;
static std::atomic<long> g_launches{0};

void set_last_error(const std::string &msg) { g_last_error = msg; }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long launch_count() { return g_launches.load(); }
Ctx *current_ctx() { return g_current; }

void trace_mark(const char *phase) {
    static const bool on = std::getenv("IBIM_TRACE") != nullptr;
    if (!on) return;
    thread_local auto last = std::chrono::steady_clock::now();
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[ibim] %-30s %9.3f ms\n", phase, std::chrono::duration<double, std::milli>(now - last).count());
    last = now;
}
void set_current_ctx(Ctx *c) { g_current = c; }

void *Ctx::pinned_buffer(size_t bytes) {
    if (bytes > pinned_bytes) {
        if (pinned) cudaFreeHost(pinned);
        pinned = nullptr;
        pinned_bytes = 0;
        const size_t grow = std::max(bytes, (size_t)1 << 20);
        IBIM_CUDA(cudaMallocHost(&pinned, grow));
        pinned_bytes = grow;
    }
    return pinned;
}

Ctx::~Ctx() {
    if (pinned) cudaFreeHost(pinned);
}

cudaEvent_t Ctx::take_event() {
    if (ev_pool.empty()) {
        cudaEvent_t e;
        IBIM_CUDA(cudaEventCreate(&e));
        return e;
    }
    cudaEvent_t e = ev_pool.back();
    ev_pool.pop_back();
    return e;
}

// FMA chains (8 independent per thread) to measure the FP64 / FP32 issue rate of the device.
template <typename T>
__global__ void k_fma_chain(T *out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = (T)(threadIdx.x + q) * (T)1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < 8; ++q) x[q] = x[q] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += x[q];
    if (s == (T)1234.5) out[blockIdx.x] = s;
}

template <class F>
static int guard(F &&f) {
    try {
        f();
        return IBIM_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return IBIM_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return IBIM_ERR_INVALID_ARGUMENT;
    }
}

static void bind(Ctx *c) {
    IBIM_CUDA(cudaSetDevice(c->device));
    set_current_ctx(c);
}

// Single-kernel FMMs through the fused block: (input density slot, output field, sign) per
// reference kernel (electric.cpp:67-291); H is symmetric, so K3ab reads slot b, field G_a.
struct KernelMap {
    int slot, field;
    double sign;
};
static const KernelMap kKernelMap[16] = {
    {0, 0, 1.},  {1, 0, 1.},  {2, 0, 1.},                          // K1x K1y K1z -> F
    {3, 0, -1.},                                                    // K2: F = -K2 psi
    {0, 1, 1.},  {1, 2, 1.},  {2, 3, 1.},                          // K3xx K3yy K3zz
    {0, 2, 1.},  {1, 3, 1.},  {2, 1, 1.},                          // K3xy K3yz K3zx
    {0, 2, 1.},  {1, 3, 1.},  {2, 1, 1.},                          // K3yx K3zy K3xz (same pairs)
    {3, 1, -1.}, {3, 2, -1.}, {3, 3, -1.},                         // K4x K4y K4z: G = -K4 psi
};

void atoms_to_device(Ctx *c, const double *centers, const double *charges, int natoms, DevBuf<double> &a4) {
    std::vector<double> h(4 * (size_t)std::max(1, natoms));
    for (int a = 0; a < natoms; ++a) {
        h[4 * a] = centers[3 * a];
        h[4 * a + 1] = centers[3 * a + 1];
        h[4 * a + 2] = centers[3 * a + 2];
        h[4 * a + 3] = charges[a];
    }
    a4.alloc(h.size(), c->stream);
    a4.upload(h.data(), h.size());
    IBIM_CUDA(cudaStreamSynchronize(c->stream));
}

void check_config(const ibim_config &cfg) {
    IBIM_REQUIRE(cfg.h > 0, "h must be positive");
    IBIM_REQUIRE(cfg.n[0] > 0 && cfg.n[1] > 0 && cfg.n[2] > 0, "grid size must be positive");
    IBIM_REQUIRE(cfg.thickness > 0, "lvlset_thickness must be positive");
    IBIM_REQUIRE(cfg.np >= 2 && cfg.np <= 8, "fmm_np must be in [2, 8]");
    IBIM_REQUIRE(cfg.maxpoint > 0, "fmm_maxpoint must be positive");
    IBIM_REQUIRE(cfg.restart > 0 && cfg.maxiter > 0, "gmres_restart and gmres_maxiter must be positive");
    IBIM_REQUIRE(cfg.kp.dE > 0 && cfg.kp.dI > 0, "solvent_dE and solvent_dI must be positive");
    IBIM_REQUIRE(cfg.kp.kappa >= 0 && cfg.kp.tau >= 0, "solvent_kappa and tau must be non-negative");
    IBIM_REQUIRE(cfg.precision == IBIM_PRECISION_FP64 || cfg.precision == IBIM_PRECISION_MIXED ||
                     cfg.precision == IBIM_PRECISION_FP64_TC,
                 "unknown precision");
    IBIM_REQUIRE(cfg.jacobian == 0 || cfg.jacobian == 1, "jacobian must be 0 or 1");
    IBIM_REQUIRE(cfg.kp.k3_scaled == 0 || cfg.kp.k3_scaled == 1, "k3_scaled must be 0 or 1");
}

void fill_plan_stats(const Plan &P, ibim_result &res) {
    const TargetSet &S = *P.targets[0];
    res.fmm_nodes = P.tree.nnodes;
    res.fmm_v_pairs = S.nv_list;
    res.fmm_x_pairs = S.nx_list;
    res.fmm_near_pairs = S.near_pairs;
    res.fmm_operators = P.nops;
}

// main.cpp:45-60 with s = 1
static Grid *levelset_pipeline(Ctx *c, const double *centers_dev, const double *radii_dev, int natoms,
                               const ibim_config &cfg, int steps[2]) {
    // FP32 grids on the mixed path only
    const int gprec = cfg.precision == IBIM_PRECISION_MIXED ? IBIM_PRECISION_MIXED : IBIM_PRECISION_FP64;
    Grid *g = grid_create(c, cfg.n[0], cfg.n[1], cfg.n[2], cfg.lo[0], cfg.lo[1], cfg.lo[2], cfg.h, cfg.init, gprec);
    Grid *phi0 = nullptr;
    try {
        levelset_expand(*g, centers_dev, radii_dev, natoms, cfg.probe, cfg.band);
        levelset_evolve(*g, cfg.probe, 1.0, 0.2);
        grid_scale(*g, -1.0);
        phi0 = grid_create(c, cfg.n[0], cfg.n[1], cfg.n[2], cfg.lo[0], cfg.lo[1], cfg.lo[2], cfg.h, 0., gprec);
        grid_copy(*phi0, *g);
        steps[0] = levelset_reinitialize(*g, *phi0, cfg.reinit_t, 1.0, 0.5, cfg.thickness, cfg.thres);
        grid_copy(*phi0, *g);
        steps[1] = levelset_reinitialize(*g, *phi0, cfg.reinit_t, 1.0, 0.5, cfg.thickness, cfg.thres);
    } catch (...) {
        delete phi0;
        delete g;
        throw;
    }
    delete phi0;
    return g;
}

// main.cpp:45-64 and electric.cpp:9-60 up to the solve: level set, surface, right-hand side (in
// tube order), plan, operators and their images, and the area.
void solve_prepare(Ctx *c, const double *centers_dev, const double *radii_dev, const double *centers_host,
                   const double *charges_host, int natoms, const ibim_config &cfg, ibim_result &res,
                   const double *atoms4_dev, SolvePrep &out, const std::function<void(long)> *after_surface) {
    check_config(cfg);
    IBIM_REQUIRE(natoms > 0, "need at least one atom");
    std::memset(&res, 0, sizeof(res));
    cudaStream_t s = c->stream;
    trace_mark("solve: start");
    Timer t0(s);
    Grid *g = levelset_pipeline(c, centers_dev, radii_dev, natoms, cfg, res.reinit_steps);
    res.t_levelset_ms = t0.ms();
    res.grid_cells = (long)cfg.n[0] * cfg.n[1] * cfg.n[2];
    res.levelset_stages = 3 * ((int)(cfg.probe / (0.2 * cfg.h)) + 1 + res.reinit_steps[0] + res.reinit_steps[1]);
    Timer t1(s);
    try {
        out.tube = surface_extract(*g, cfg.thickness, &res.inclusion, cfg.jacobian != 0);
    } catch (...) {
        delete g;
        throw;
    }
    delete g;
    Tube *tube = out.tube;
    res.n_points = tube->n;
    res.t_surface_ms = t1.ms();
    trace_mark("solve: level set + surface");
    IBIM_REQUIRE(tube->n > 0, "the level set has no tube points");
    try {
        out.atoms4 = atoms4_dev;
        if (!out.atoms4) {
            atoms_to_device(c, centers_host, charges_host, natoms, out.a4);
            out.atoms4 = out.a4.ptr;
        }
        // the right-hand side needs only the tube and the atoms: it runs on the second stream
        // while the host builds the octree and its lists
        out.b_tube.alloc(2 * (size_t)tube->n, s);
        IBIM_CUDA(cudaEventRecord(c->ev_fork, s));
        IBIM_CUDA(cudaStreamWaitEvent(c->aux, c->ev_fork, 0));
        bie_rhs_tube(*tube, cfg.kp, out.atoms4, natoms, out.b_tube.ptr, c->aux, cfg.precision);
        IBIM_CUDA(cudaEventRecord(c->ev_join, c->aux));
        trace_mark("solve: atoms, rhs enqueued");
        auto w0 = std::chrono::steady_clock::now();
        out.P = make_plan(tube, true, centers_host, natoms, cfg.np, cfg.maxpoint, cfg.maxlevel, cfg.precision);
        Plan *P = out.P;
        IBIM_CUDA(cudaStreamSynchronize(s));
        // the caller may hold the operators back until their device memory (the plan's exact
        // operator and node counts) is free
        if (after_surface) (*after_surface)((long)std::llround(plan_fmm_bytes(*P, cfg)));
        const auto w1 = std::chrono::steady_clock::now();
        res.t_tree_ms = std::chrono::duration<double, std::milli>(w1 - w0).count();
        trace_mark("solve: plan synced");
        if (cfg.precision == IBIM_PRECISION_FP64 || !m2l_tc_supported()) {
            fmm_prepare_operators(*P, cfg.kp, IBIM_PRECISION_FP64);
            if (cfg.precision == IBIM_PRECISION_MIXED) fmm_prepare_operators(*P, cfg.kp, IBIM_PRECISION_MIXED);
        } else {
            // Mixed path in the scaled FP16 form: the FP16 images of the mixed operator and the
            // digit images of the FP64-class one (the refinement residual's) from one pass over
            // float-float operators.  Otherwise the digit images, then the TF32 images from FP32
            // operators rounded from the FP64 ones.  Afterwards only the images are used, so the
            // FP64 / float-float operators are released (the order keeps the peak at 26 bytes per
            // operator entry: FP64 8 + digits 14 + FP32 4, then digits + FP32 + TF32 images 8 once
            // the FP64 operators are gone)
            if (cfg.precision == IBIM_PRECISION_MIXED && mixed_uses_tc() && fmm_ensure_images_ff(*P, cfg.kp)) {
                // both images from one pass over the float-float operators
                fmm_release_fp64_operators(*P);
            } else {
                fmm_ensure_oz_images(*P, cfg.kp);
                if (cfg.precision == IBIM_PRECISION_MIXED) fmm_prepare_operators(*P, cfg.kp, IBIM_PRECISION_MIXED);
                fmm_release_fp64_operators(*P);
                if (cfg.precision == IBIM_PRECISION_MIXED && mixed_uses_tc()) fmm_ensure_tc_images(*P, cfg.kp);
            }
        }
        trace_mark("solve: operators enqueued");
        // the FP32 / float-float near lists of the target sets are built on the host while the
        // device computes the operators
        if (cfg.precision == IBIM_PRECISION_MIXED ||
            (cfg.precision == IBIM_PRECISION_FP64_TC && m2l_tc_supported() && near_ff_enabled()))
            for (TargetSet *ts : P->targets) mixed_lists_host(*P, *ts);
        // and the mixed plan's data (FP32 tables, leaf-relative coordinates, near lists on the
        // device), queued behind the operators instead of after them
        if (cfg.precision == IBIM_PRECISION_MIXED)
            for (TargetSet *ts : P->targets) prepare_mixed(*P, *ts);
        IBIM_CUDA(cudaStreamSynchronize(s));
        const auto w2 = std::chrono::steady_clock::now();
        res.t_operators_ms = std::chrono::duration<double, std::milli>(w2 - w1).count();
        res.t_plan_ms = std::chrono::duration<double, std::milli>(w2 - w0).count();
        trace_mark("solve: operators synced");
        IBIM_CUDA(cudaStreamWaitEvent(s, c->ev_join, 0));
        // area = sum of quadrature weights (electric.cpp:60)
        std::vector<double> w(tube->n);
        P->sw.download(w.data(), tube->n);
        IBIM_CUDA(cudaStreamSynchronize(s));
        double area = 0.;
        for (long i = 0; i < tube->n; ++i) area += w[i];
        res.area = area;
        fill_plan_stats(*P, res);
    } catch (...) {
        cudaStreamSynchronize(c->aux);  // the right-hand side may still read the tube and atoms
        throw;
    }
}

static void solve_impl(Ctx *c, const double *centers_dev, const double *radii_dev, const double *centers_host,
                       const double *charges_host, int natoms, const ibim_config &cfg, ibim_result &res,
                       const double *atoms4_dev, const std::function<void(long)> *after_surface = nullptr) {
    SolvePrep prep;
    solve_prepare(c, centers_dev, radii_dev, centers_host, charges_host, natoms, cfg, res, atoms4_dev, prep,
                  after_surface);
    electric_solve(*prep.P, cfg.kp, prep.atoms4, charges_host, natoms, cfg.restart, cfg.maxiter, cfg.tol,
                   cfg.precision, nullptr, nullptr, res, prep.b_tube.ptr);
    fill_plan_stats(*prep.P, res);
    trace_mark("solve: electric done");
}

void solve_host(Ctx *c, const double *centers, const double *charges, const double *radii, int natoms,
                const ibim_config &cfg, ibim_result &res, const std::function<void(long)> *after_surface) {
    IBIM_REQUIRE(centers && charges && radii && natoms > 0, "need at least one atom");
    IBIM_CUDA(cudaSetDevice(c->device));
    set_current_ctx(c);
    DevBuf<double> dc, dr;
    dc.alloc(3 * (size_t)natoms, c->stream);
    dr.alloc(natoms, c->stream);
    dc.upload(centers, 3 * (size_t)natoms);
    dr.upload(radii, natoms);
    solve_impl(c, dc.ptr, dr.ptr, centers, charges, natoms, cfg, res, nullptr, after_surface);
}

// Serialise a tree in the reference's node numbering (see ibim_plan_lists).
static void encode_lists(const TreeHost &T, int *buf, long cap, long *needed) {
    const int nn = T.nnodes;
    std::vector<int> lev_of_ref(nn);
    for (int i = 0; i < nn; ++i) lev_of_ref[T.ref_id[i]] = i;
    std::vector<int> out;
    out.push_back(nn);
    for (int r = 0; r < nn; ++r) {
        const int i = lev_of_ref[r];
        int level = 0;
        while (T.level_begin[level + 1] <= i) ++level;
        out.push_back(level);
        out.push_back(T.parent[i] < 0 ? -1 : T.ref_id[T.parent[i]]);
        out.push_back(T.leaf[i]);
        out.push_back(T.empty[i]);
        out.push_back(T.src_end[i] - T.src_begin[i]);
        const IdxSpan L[4] = {T.U[i], T.V[i], T.W[i], T.X[i]};
        for (const IdxSpan &l : L) {
            std::vector<int> v;
            for (int x : l) v.push_back(T.ref_id[x]);
            std::sort(v.begin(), v.end());
            out.push_back((int)v.size());
            out.insert(out.end(), v.begin(), v.end());
        }
    }
    if (needed) *needed = (long)out.size();
    if (buf && cap >= (long)out.size()) std::copy(out.begin(), out.end(), buf);
    else if (buf) throw Error(IBIM_ERR_INVALID_ARGUMENT, "list buffer too small");
}

}  // namespace ibim

using namespace ibim;

extern "C" {

const char *ibim_last_error(void) { return g_last_error.c_str(); }

const char *ibim_status_string(int st) {
    switch (st) {
        case IBIM_OK: return "ok";
        case IBIM_ERR_INVALID_ARGUMENT: return "invalid argument";
        case IBIM_ERR_CUDA: return "CUDA error";
        case IBIM_ERR_OUT_OF_MEMORY: return "out of memory";
        case IBIM_ERR_UNSUPPORTED_KERNEL: return "unsupported kernel";
        case IBIM_ERR_LIMIT: return "iteration limit reached";
        case IBIM_ERR_IO: return "I/O error";
        case IBIM_ERR_CALLBACK: return "operator callback failed";
        default: return "unknown status";
    }
}

void ibim_config_default(ibim_config *cfg) {
    // data/input.cfg and main.cpp constants; geometry left to the caller
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->band = 8;
    cfg->probe = 1.4;
    cfg->reinit_t = 60;
    cfg->thickness = 2;
    cfg->thres = 1e-4;
    cfg->np = 4;
    cfg->maxpoint = 160;
    cfg->maxlevel = 10;
    cfg->kp.kappa = 0.1257;
    cfg->kp.dE = 80.0;
    cfg->kp.dI = 1.0;
    cfg->kp.tau = 1.0;
    cfg->restart = 40;
    cfg->maxiter = 100;
    cfg->tol = 1e-5;
    cfg->precision = IBIM_PRECISION_FP64;
}

int ibim_ctx_create(int device, ibim_ctx *out) {
    return guard([&] {
        IBIM_REQUIRE(out != nullptr, "null output handle");
        int ndev = 0;
        IBIM_CUDA(cudaGetDeviceCount(&ndev));
        IBIM_REQUIRE(device >= 0 && device < ndev, "no such CUDA device");
        auto *h = new ibim_ctx_s();
        h->c.device = device;
        try {
            IBIM_CUDA(cudaSetDevice(device));
            IBIM_CUDA(cudaDeviceGetAttribute(&h->c.num_sms, cudaDevAttrMultiProcessorCount, device));
            // the far-field chain on the main stream is the critical path of a matvec; the near
            // field on the auxiliary stream fills the resources it leaves free
            int least = 0, greatest = 0;
            IBIM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            IBIM_CUDA(cudaStreamCreateWithPriority(&h->c.stream, cudaStreamNonBlocking, greatest));
            IBIM_CUDA(cudaStreamCreateWithPriority(&h->c.aux, cudaStreamNonBlocking, least));
            // device memory freed by a solve stays in the stream-ordered pool for the next one
            // instead of going back to the driver at every synchronisation (a solve allocates
            // several GB of operator images); ibim_ctx_trim hands it back
            cudaMemPool_t pool;
            IBIM_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
            uint64_t keep = UINT64_MAX;
            IBIM_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
            IBIM_CUDA(cudaEventCreateWithFlags(&h->c.ev_fork, cudaEventDisableTiming));
            IBIM_CUDA(cudaEventCreateWithFlags(&h->c.ev_join, cudaEventDisableTiming));
            IBIM_CUDA(cudaEventCreateWithFlags(&h->c.ev_near_fork, cudaEventDisableTiming));
            IBIM_CUDA(cudaEventCreateWithFlags(&h->c.ev_near_join, cudaEventDisableTiming));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int ibim_ctx_destroy(ibim_ctx ctx) {
    return guard([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->c.device);
        cudaStreamSynchronize(ctx->c.stream);
        if (ctx->c.aux) {
            cudaStreamSynchronize(ctx->c.aux);
            cudaStreamDestroy(ctx->c.aux);
        }
        if (ctx->c.ev_fork) cudaEventDestroy(ctx->c.ev_fork);
        if (ctx->c.ev_join) cudaEventDestroy(ctx->c.ev_join);
        if (ctx->c.ev_near_fork) cudaEventDestroy(ctx->c.ev_near_fork);
        if (ctx->c.ev_near_join) cudaEventDestroy(ctx->c.ev_near_join);
        cudaStreamDestroy(ctx->c.stream);
        delete ctx;
    });
}

void *ibim_ctx_stream(ibim_ctx ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

int ibim_ctx_trim(ibim_ctx ctx) {
    return guard([&] {
        IBIM_REQUIRE(ctx, "null context");
        bind(&ctx->c);
        IBIM_CUDA(cudaStreamSynchronize(ctx->c.stream));
        IBIM_CUDA(cudaStreamSynchronize(ctx->c.aux));
        cudaMemPool_t pool;
        IBIM_CUDA(cudaDeviceGetDefaultMemPool(&pool, ctx->c.device));
        IBIM_CUDA(cudaMemPoolTrimTo(pool, 0));
    });
}

long ibim_launch_count(void) { return launch_count(); }

int ibim_profile_enable(ibim_ctx ctx, unsigned mask) {
    return guard([&] {
        IBIM_REQUIRE(ctx, "null handle");
        ctx->c.prof_mask = mask;
    });
}

int ibim_profile_work(ibim_ctx ctx, double *flops, double *bytes, int ncat) {
    return guard([&] {
        IBIM_REQUIRE(ctx && flops && bytes, "null argument");
        for (int k = 0; k < ncat && k < PROF_NCAT; ++k) {
            flops[k] = ctx->c.prof_flops[k];
            bytes[k] = ctx->c.prof_bytes[k];
        }
    });
}

int ibim_profile_read(ibim_ctx ctx, double *ms, long *launches, int ncat) {
    return guard([&] {
        IBIM_REQUIRE(ctx && ms && launches, "null argument");
        Ctx &c = ctx->c;
        bind(&c);
        IBIM_CUDA(cudaStreamSynchronize(c.stream));
        for (int k = 0; k < PROF_NCAT; ++k) {
            double t = 0.;
            for (auto &pr : c.prof_ev[k]) {
                float m = 0.f;
                IBIM_CUDA(cudaEventElapsedTime(&m, pr.first, pr.second));
                t += m;
                c.ev_pool.push_back(pr.first);
                c.ev_pool.push_back(pr.second);
            }
            if (k < ncat) {
                ms[k] = t;
                launches[k] = (long)c.prof_ev[k].size();
            }
            c.prof_ev[k].clear();
            c.prof_flops[k] = c.prof_bytes[k] = 0.;
        }
    });
}

int ibim_measure_peak(ibim_ctx ctx, int kind, double *tflops) {
    return guard([&] {
        IBIM_REQUIRE(ctx && tflops && (kind == 0 || kind == 1), "invalid argument");
        Ctx &c = ctx->c;
        bind(&c);
        const int blocks = c.num_sms * 8, threads = 256, iters = kind == 0 ? 2048 : 16384;
        DevBuf<double> out;
        out.alloc(blocks, c.stream);
        auto launch = [&] {
            if (kind == 0)
                (count_launch(), k_fma_chain<double><<<blocks, threads, 0, c.stream>>>(out.ptr, iters, 0.999999, 1e-7));
            else
                (count_launch(), k_fma_chain<float><<<blocks, threads, 0, c.stream>>>((float *)out.ptr, iters, 0.999999f, 1e-7f));
            IBIM_CHECK_LAUNCH();
        };
        launch();
        double best = 1e30;
        for (int r = 0; r < 5; ++r) {
            Timer t(c.stream);
            launch();
            best = std::min(best, t.ms());
        }
        *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    });
}

int ibim_grid_create(ibim_ctx ctx, int nx, int ny, int nz, double sx, double sy, double sz, double dx, double value,
                     ibim_grid *out) {
    return guard([&] {
        IBIM_REQUIRE(ctx && out, "null handle");
        bind(&ctx->c);
        Grid *g = grid_create(&ctx->c, nx, ny, nz, sx, sy, sz, dx, value);
        *out = new ibim_grid_s{g};
    });
}

int ibim_grid_destroy(ibim_grid g) {
    return guard([&] {
        if (!g) return;
        bind(g->g->ctx);
        delete g->g;
        delete g;
    });
}

int ibim_grid_upload(ibim_grid g, const double *host) {
    return guard([&] {
        IBIM_REQUIRE(g && host, "null argument");
        Grid &G = *g->g;
        bind(G.ctx);
        if (G.prec == IBIM_PRECISION_FP64) {
            G.data.upload(host, G.cells());
        } else {
            std::vector<float> f(host, host + G.cells());
            G.data32.upload(f.data(), G.cells());
        }
        IBIM_CUDA(cudaStreamSynchronize(G.ctx->stream));
    });
}

int ibim_grid_download(ibim_grid g, double *host) {
    return guard([&] {
        IBIM_REQUIRE(g && host, "null argument");
        Grid &G = *g->g;
        bind(G.ctx);
        if (G.prec == IBIM_PRECISION_FP64) {
            G.data.download(host, G.cells());
            IBIM_CUDA(cudaStreamSynchronize(G.ctx->stream));
        } else {
            std::vector<float> f(G.cells());
            G.data32.download(f.data(), G.cells());
            IBIM_CUDA(cudaStreamSynchronize(G.ctx->stream));
            std::copy(f.begin(), f.end(), host);
        }
    });
}

int ibim_grid_set_geometry(ibim_grid g, double sx, double sy, double sz, double dx) {
    return guard([&] {
        IBIM_REQUIRE(g, "null handle");
        IBIM_REQUIRE(dx > 0, "dx must be positive");
        Grid &G = *g->g;
        G.sx = sx;
        G.sy = sy;
        G.sz = sz;
        G.dx = dx;
    });
}

int ibim_grid_scale(ibim_grid g, double s) {
    return guard([&] {
        IBIM_REQUIRE(g, "null handle");
        bind(g->g->ctx);
        grid_scale(*g->g, s);
    });
}

int ibim_grid_copy(ibim_grid dst, ibim_grid src) {
    return guard([&] {
        IBIM_REQUIRE(dst && src, "null handle");
        bind(dst->g->ctx);
        grid_copy(*dst->g, *src->g);
    });
}

int ibim_levelset_expand(ibim_grid g, const double *centers, const double *radii, int natoms, double probe, int band) {
    return guard([&] {
        IBIM_REQUIRE(g && (natoms == 0 || (centers && radii)), "null argument");
        IBIM_REQUIRE(natoms >= 0, "natoms must be non-negative");
        Ctx *c = g->g->ctx;
        bind(c);
        DevBuf<double> dc, dr;
        dc.alloc(3 * (size_t)natoms, c->stream);
        dr.alloc(natoms, c->stream);
        dc.upload(centers, 3 * (size_t)natoms);
        dr.upload(radii, natoms);
        levelset_expand(*g->g, dc.ptr, dr.ptr, natoms, probe, band);
        IBIM_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int ibim_levelset_evolve(ibim_grid g, double final_t, double vel, double cfl) {
    return guard([&] {
        IBIM_REQUIRE(g, "null handle");
        bind(g->g->ctx);
        levelset_evolve(*g->g, final_t, vel, cfl);
        IBIM_CUDA(cudaStreamSynchronize(g->g->ctx->stream));
    });
}

int ibim_levelset_reinitialize(ibim_grid g, ibim_grid phi0, double final_t, double vel, double cfl, int thickness,
                               double thres, int *steps) {
    return guard([&] {
        IBIM_REQUIRE(g && phi0, "null handle");
        bind(g->g->ctx);
        const int st = levelset_reinitialize(*g->g, *phi0->g, final_t, vel, cfl, thickness, thres);
        if (steps) *steps = st;
    });
}

int ibim_levelset_count_gradient(ibim_grid g, double thickness, double thres, long *bad, long *total,
                                 double *accum_error) {
    return guard([&] {
        IBIM_REQUIRE(g, "null handle");
        bind(g->g->ctx);
        levelset_count_gradient(*g->g, thickness, thres, bad, total, accum_error);
    });
}

int ibim_levelset_build(ibim_ctx ctx, const double *centers, const double *radii, int natoms, const ibim_config *cfg,
                        ibim_grid *out, int steps[2]) {
    return guard([&] {
        IBIM_REQUIRE(ctx && centers && radii && cfg && out, "null argument");
        IBIM_REQUIRE(natoms > 0, "need at least one atom");
        Ctx *c = &ctx->c;
        bind(c);
        DevBuf<double> dc, dr;
        dc.alloc(3 * (size_t)natoms, c->stream);
        dr.alloc(natoms, c->stream);
        dc.upload(centers, 3 * (size_t)natoms);
        dr.upload(radii, natoms);
        int st[2] = {0, 0};
        Grid *g = levelset_pipeline(c, dc.ptr, dr.ptr, natoms, *cfg, st);
        IBIM_CUDA(cudaStreamSynchronize(c->stream));
        if (steps) { steps[0] = st[0]; steps[1] = st[1]; }
        *out = new ibim_grid_s{g};
    });
}

int ibim_surface_extract(ibim_grid g, int thickness, ibim_tube *out, long *n_points, long *inclusion) {
    return ibim_surface_extract_jacobian(g, thickness, 0, out, n_points, inclusion);
}

int ibim_surface_extract_jacobian(ibim_grid g, int thickness, int jacobian, ibim_tube *out, long *n_points,
                                  long *inclusion) {
    return guard([&] {
        IBIM_REQUIRE(g && out, "null argument");
        IBIM_REQUIRE(jacobian == 0 || jacobian == 1, "jacobian must be 0 or 1");
        bind(g->g->ctx);
        long inc = 0;
        Tube *t = surface_extract(*g->g, thickness, &inc, jacobian != 0);
        IBIM_CUDA(cudaStreamSynchronize(g->g->ctx->stream));
        if (n_points) *n_points = t->n;
        if (inclusion) *inclusion = inc;
        *out = new ibim_tube_s{t};
    });
}

int ibim_tube_create(ibim_ctx ctx, const double *points, const double *normals, const double *weights, long n, double h,
                     ibim_tube *out) {
    return guard([&] {
        IBIM_REQUIRE(ctx && points && normals && weights && out, "null argument");
        IBIM_REQUIRE(n > 0 && h > 0, "tube needs n > 0 and h > 0");
        Ctx *c = &ctx->c;
        bind(c);
        Tube *t = new Tube();
        t->ctx = c;
        t->n = n;
        t->h = h;
        try {
            std::vector<double> tmp(n);
            DevBuf<double> *xyz[3] = {&t->x, &t->y, &t->z};
            DevBuf<double> *nrm[3] = {&t->nx, &t->ny, &t->nz};
            for (int a = 0; a < 3; ++a) {
                for (long i = 0; i < n; ++i) tmp[i] = points[3 * i + a];
                xyz[a]->alloc(n, c->stream);
                xyz[a]->upload(tmp.data(), n);
                IBIM_CUDA(cudaStreamSynchronize(c->stream));
                for (long i = 0; i < n; ++i) tmp[i] = normals[3 * i + a];
                nrm[a]->alloc(n, c->stream);
                nrm[a]->upload(tmp.data(), n);
                IBIM_CUDA(cudaStreamSynchronize(c->stream));
            }
            t->w.alloc(n, c->stream);
            t->w.upload(weights, n);
            IBIM_CUDA(cudaStreamSynchronize(c->stream));
        } catch (...) {
            delete t;
            throw;
        }
        *out = new ibim_tube_s{t};
    });
}

int ibim_tube_destroy(ibim_tube t) {
    return guard([&] {
        if (!t) return;
        bind(t->t->ctx);
        delete t->t;
        delete t;
    });
}

long ibim_tube_size(ibim_tube t) { return t ? t->t->n : -1; }

int ibim_tube_download(ibim_tube t, double *points, double *normals, double *weights) {
    return guard([&] {
        IBIM_REQUIRE(t, "null handle");
        Tube *T = t->t;
        bind(T->ctx);
        const long n = T->n;
        std::vector<double> a(n), b(n), c(n);
        auto three = [&](DevBuf<double> &X, DevBuf<double> &Y, DevBuf<double> &Z, double *dst) {
            X.download(a.data(), n);
            Y.download(b.data(), n);
            Z.download(c.data(), n);
            IBIM_CUDA(cudaStreamSynchronize(T->ctx->stream));
            for (long i = 0; i < n; ++i) {
                dst[3 * i] = a[i];
                dst[3 * i + 1] = b[i];
                dst[3 * i + 2] = c[i];
            }
        };
        if (points) three(T->x, T->y, T->z, points);
        if (normals) three(T->nx, T->ny, T->nz, normals);
        if (weights) {
            T->w.download(weights, n);
            IBIM_CUDA(cudaStreamSynchronize(T->ctx->stream));
        }
    });
}

int ibim_fmm_plan(ibim_tube src, const double *targets, long nt, int order, int maxpoint, int maxlevel, int precision,
                  ibim_plan *out) {
    return guard([&] {
        IBIM_REQUIRE(src && out, "null argument");
        IBIM_REQUIRE(targets == nullptr || nt > 0, "targets given with nt <= 0");
        bind(src->t->ctx);
        Plan *P = make_plan(src->t, targets == nullptr, targets, targets ? nt : 0, order, maxpoint, maxlevel, precision);
        *out = new ibim_plan_s{P};
    });
}

int ibim_plan_destroy(ibim_plan p) {
    return guard([&] {
        if (!p) return;
        bind(p->p->ctx);
        delete p->p;
        delete p;
    });
}

int ibim_plan_stats(ibim_plan p, long stats[8]) {
    return guard([&] {
        IBIM_REQUIRE(p && stats, "null argument");
        const Plan &P = *p->p;
        const TargetSet &S = *P.targets[0];
        long leaves = 0;
        for (int i = 0; i < P.tree.nnodes; ++i) leaves += P.tree.leaf[i];
        stats[0] = P.tree.nnodes;
        stats[1] = P.tree.nlevels;
        stats[2] = leaves;
        stats[3] = S.nv_list;
        stats[4] = S.nx_list;
        stats[5] = S.near_pairs;
        stats[6] = P.nops;
        stats[7] = S.ntleaves;
    });
}

int ibim_plan_lists(ibim_plan p, int which, int *buf, long cap, long *needed) {
    return guard([&] {
        IBIM_REQUIRE(p && which == 0, "invalid argument");
        encode_lists(p->p->tree, buf, cap, needed);
    });
}

int ibim_tree_lists_host(const double *points, long n, int maxpoint, int maxlevel, int *buf, long cap, long *needed) {
    return guard([&] {
        IBIM_REQUIRE(points && n > 0, "null or empty points");
        TreeHost T = build_tree(points, n, points, n, maxpoint, maxlevel);
        encode_lists(T, buf, cap, needed);
    });
}

int ibim_fmm_apply(ibim_plan p, int kernel, const ibim_kernel_params *kp, const double *in, double *out) {
    return guard([&] {
        IBIM_REQUIRE(p && kp && in && out, "null argument");
        if (kernel < 0 || kernel > IBIM_KERNEL_BIE_FUSED)
            throw Error(IBIM_ERR_UNSUPPORTED_KERNEL, "kernel id outside the reference's kernel set");
        Plan &P = *p->p;
        Ctx *c = P.ctx;
        bind(c);
        cudaStream_t s = c->stream;
        const long ns = P.ns;
        TargetSet &S = *P.targets[0];
        const long nt = S.nt;
        const int rows = kernel == IBIM_KERNEL_BIE_FUSED ? 4 : 1;
        DevBuf<double> hin;
        hin.alloc((size_t)rows * ns, s);
        hin.upload(in, (size_t)rows * ns);
        P.dens4.zero();
        if (rows == 4) {
            for (int d = 0; d < 4; ++d) permute(c, ns, P.src_perm.ptr, hin.ptr + d * ns, P.dens4.ptr + d * ns, false);
        } else {
            permute(c, ns, P.src_perm.ptr, hin.ptr, P.dens4.ptr + kKernelMap[kernel].slot * ns, false);
        }
        fmm_run(P, 0, *kp, P.dens4.ptr, S.out4.ptr, P.precision);
        DevBuf<double> hout;
        hout.alloc((size_t)rows * nt, s);
        if (rows == 4) {
            for (int d = 0; d < 4; ++d) permute(c, nt, S.perm_d.ptr, S.out4.ptr + d * nt, hout.ptr + d * nt, true);
        } else {
            permute(c, nt, S.perm_d.ptr, S.out4.ptr + kKernelMap[kernel].field * nt, hout.ptr, true);
        }
        hout.download(out, (size_t)rows * nt);
        IBIM_CUDA(cudaStreamSynchronize(s));
        if (rows == 1 && kKernelMap[kernel].sign < 0)
            for (long i = 0; i < nt; ++i) out[i] = -out[i];
    });
}

int ibim_bie_matvec(ibim_plan p, const ibim_kernel_params *kp, const double *x, double *y) {
    return guard([&] {
        IBIM_REQUIRE(p && kp && x && y, "null argument");
        Plan &P = *p->p;
        Ctx *c = P.ctx;
        bind(c);
        cudaStream_t s = c->stream;
        const long n = P.ns;
        DevBuf<double> hx, tx, ty, hy;
        hx.alloc(2 * n, s);
        tx.alloc(2 * n, s);
        ty.alloc(2 * n, s);
        hy.alloc(2 * n, s);
        hx.upload(x, 2 * n);
        permute(c, n, P.src_perm.ptr, hx.ptr, tx.ptr, false);
        permute(c, n, P.src_perm.ptr, hx.ptr + n, tx.ptr + n, false);
        bie_matvec(P, *kp, tx.ptr, ty.ptr, P.precision);
        permute(c, n, P.src_perm.ptr, ty.ptr, hy.ptr, true);
        permute(c, n, P.src_perm.ptr, ty.ptr + n, hy.ptr + n, true);
        hy.download(y, 2 * n);
        IBIM_CUDA(cudaStreamSynchronize(s));
    });
}

int ibim_bie_rhs(ibim_plan p, const ibim_kernel_params *kp, const double *centers, const double *charges, int natoms,
                 double *b) {
    return guard([&] {
        IBIM_REQUIRE(p && kp && centers && charges && b, "null argument");
        Plan &P = *p->p;
        Ctx *c = P.ctx;
        bind(c);
        cudaStream_t s = c->stream;
        const long n = P.ns;
        DevBuf<double> a4, tb, hb;
        atoms_to_device(c, centers, charges, natoms, a4);
        tb.alloc(2 * n, s);
        hb.alloc(2 * n, s);
        bie_rhs(P, *kp, a4.ptr, natoms, tb.ptr);
        permute(c, n, P.src_perm.ptr, tb.ptr, hb.ptr, true);
        permute(c, n, P.src_perm.ptr, tb.ptr + n, hb.ptr + n, true);
        hb.download(b, 2 * n);
        IBIM_CUDA(cudaStreamSynchronize(s));
    });
}

int ibim_gmres_solve(ibim_plan p, const ibim_kernel_params *kp, const double *b, double *x, int restart, int maxiter,
                     double tol, int precision, int *iters, int *gmres_status, double *residual) {
    return guard([&] {
        IBIM_REQUIRE(p && kp && b && x, "null argument");
        IBIM_REQUIRE(restart > 0 && maxiter > 0, "restart and maxiter must be positive");
        Plan &P = *p->p;
        Ctx *c = P.ctx;
        bind(c);
        cudaStream_t s = c->stream;
        const long n = P.ns;
        DevBuf<double> hb, hx, tb, tx;
        hb.alloc(2 * n, s);
        hx.alloc(2 * n, s);
        tb.alloc(2 * n, s);
        tx.alloc(2 * n, s);
        hb.upload(b, 2 * n);
        hx.upload(x, 2 * n);
        permute(c, n, P.src_perm.ptr, hb.ptr, tb.ptr, false);
        permute(c, n, P.src_perm.ptr, hb.ptr + n, tb.ptr + n, false);
        permute(c, n, P.src_perm.ptr, hx.ptr, tx.ptr, false);
        permute(c, n, P.src_perm.ptr, hx.ptr + n, tx.ptr + n, false);
        Krylov K(c, 2 * n, std::min(restart, 250));
        GmresStats st;
        auto A = [&](const double *in, double *o) { bie_matvec(P, *kp, in, o, precision); };
        const int rc = K.solve(A, tx.ptr, tb.ptr, maxiter, tol, false, st);
        permute(c, n, P.src_perm.ptr, tx.ptr, hx.ptr, true);
        permute(c, n, P.src_perm.ptr, tx.ptr + n, hx.ptr + n, true);
        hx.download(x, 2 * n);
        IBIM_CUDA(cudaStreamSynchronize(s));
        if (iters) *iters = st.iters;
        if (gmres_status) *gmres_status = rc;
        if (residual) *residual = st.residual;
    });
}

int ibim_gmres_host(ibim_ctx ctx, long n, ibim_apply_fn apply, void *user, const double *b, double *x, int restart,
                    int maxiter, double tol, int *iters, int *matvecs, int *gmres_status, double *residual) {
    return guard([&] {
        IBIM_REQUIRE(ctx && apply && b && x, "null argument");
        IBIM_REQUIRE(n > 0, "vector length must be positive");
        IBIM_REQUIRE(restart > 0 && maxiter > 0, "restart and maxiter must be positive");
        Ctx *c = &ctx->c;
        bind(c);
        cudaStream_t s = c->stream;
        DevBuf<double> db, dx;
        db.alloc(n, s);
        dx.alloc(n, s);
        db.upload(b, n);
        dx.upload(x, n);
        // the operator's input and output pass through pinned host buffers
        double *hin = nullptr, *hout = nullptr;
        IBIM_CUDA(cudaMallocHost((void **)&hin, sizeof(double) * n));
        struct Pinned {
            double *&a, *&b;
            ~Pinned() { if (a) cudaFreeHost(a); if (b) cudaFreeHost(b); }
        } pinned{hin, hout};
        IBIM_CUDA(cudaMallocHost((void **)&hout, sizeof(double) * n));
        auto A = [&](const double *in, double *o) {
            IBIM_CUDA(cudaMemcpyAsync(hin, in, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
            IBIM_CUDA(cudaStreamSynchronize(s));
            if (apply(user, hin, hout, n) != 0)
                throw Error(IBIM_ERR_CALLBACK, "the operator callback stopped the GMRES solve");
            IBIM_CUDA(cudaMemcpyAsync(o, hout, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            IBIM_CUDA(cudaStreamSynchronize(s));
        };
        Krylov K(c, n, std::min(restart, 250));
        GmresStats st;
        // x is arbitrary here: the first product A x is applied, as gmres.cpp:72 does
        const int rc = K.solve(A, dx.ptr, db.ptr, maxiter, tol, false, st);
        dx.download(x, n);
        IBIM_CUDA(cudaStreamSynchronize(s));
        if (iters) *iters = st.iters;
        if (matvecs) *matvecs = st.matvecs;
        if (gmres_status) *gmres_status = rc;
        if (residual) *residual = st.residual;
    });
}

int ibim_electric(ibim_tube tube, const double *centers, const double *charges, int natoms, const ibim_config *cfg,
                  double *x, double *atom_potential, ibim_result *res) {
    return guard([&] {
        IBIM_REQUIRE(tube && centers && charges && cfg && res, "null argument");
        IBIM_REQUIRE(natoms > 0, "need at least one atom");
        check_config(*cfg);
        Tube *T = tube->t;
        Ctx *c = T->ctx;
        bind(c);
        cudaStream_t s = c->stream;
        std::memset(res, 0, sizeof(*res));
        res->n_points = T->n;
        Plan *P = make_plan(T, true, centers, natoms, cfg->np, cfg->maxpoint, cfg->maxlevel, cfg->precision);
        try {
            std::vector<double> w(T->n);
            P->sw.download(w.data(), T->n);
            IBIM_CUDA(cudaStreamSynchronize(s));
            double area = 0.;
            for (long i = 0; i < T->n; ++i) area += w[i];
            res->area = area;
            DevBuf<double> a4, xt, xh;
            atoms_to_device(c, centers, charges, natoms, a4);
            xt.alloc(2 * T->n, s);
            std::vector<double> pot;
            electric_solve(*P, cfg->kp, a4.ptr, charges, natoms, cfg->restart, cfg->maxiter, cfg->tol, cfg->precision,
                           xt.ptr, &pot, *res);
            if (x) {
                xh.alloc(2 * T->n, s);
                permute(c, T->n, P->src_perm.ptr, xt.ptr, xh.ptr, true);
                permute(c, T->n, P->src_perm.ptr, xt.ptr + T->n, xh.ptr + T->n, true);
                xh.download(x, 2 * T->n);
                IBIM_CUDA(cudaStreamSynchronize(s));
            }
            if (atom_potential) std::copy(pot.begin(), pot.end(), atom_potential);
        } catch (...) {
            delete P;
            throw;
        }
        delete P;
    });
}

int ibim_solve(ibim_ctx ctx, const double *centers, const double *charges, const double *radii, int natoms,
               const ibim_config *cfg, ibim_result *res) {
    return guard([&] {
        IBIM_REQUIRE(ctx && centers && charges && radii && cfg && res, "null argument");
        IBIM_REQUIRE(natoms > 0, "need at least one atom");
        Ctx *c = &ctx->c;
        bind(c);
        DevBuf<double> dc, dr;
        dc.alloc(3 * (size_t)natoms, c->stream);
        dr.alloc(natoms, c->stream);
        dc.upload(centers, 3 * (size_t)natoms);
        dr.upload(radii, natoms);
        solve_impl(c, dc.ptr, dr.ptr, centers, charges, natoms, *cfg, *res, nullptr);
    });
}

int ibim_solve_dev(ibim_ctx ctx, const double *centers_dev, const double *charges_dev, const double *radii_dev,
                   int natoms, const ibim_config *cfg, ibim_result *res) {
    return guard([&] {
        IBIM_REQUIRE(ctx && centers_dev && charges_dev && radii_dev && cfg && res, "null argument");
        IBIM_REQUIRE(natoms > 0, "need at least one atom");
        Ctx *c = &ctx->c;
        bind(c);
        // the tree build and the energy sum run on the host: bring the atoms over once
        std::vector<double> hc(3 * (size_t)natoms), hq(natoms);
        IBIM_CUDA(cudaMemcpyAsync(hc.data(), centers_dev, sizeof(double) * 3 * natoms, cudaMemcpyDeviceToHost, c->stream));
        IBIM_CUDA(cudaMemcpyAsync(hq.data(), charges_dev, sizeof(double) * natoms, cudaMemcpyDeviceToHost, c->stream));
        IBIM_CUDA(cudaStreamSynchronize(c->stream));
        solve_impl(c, centers_dev, radii_dev, hc.data(), hq.data(), natoms, *cfg, *res, nullptr);
    });
}

int ibim_batch_solve(ibim_ctx ctx, int nmol, const int *natoms, const double *centers, const double *charges,
                     const double *radii, const ibim_config *cfgs, int max_wave, int wave_slots,
                     double hbm_budget_bytes, int workers, ibim_result *results, int *statuses, double *done_ms,
                     double *info) {
    return guard([&] {
        IBIM_REQUIRE(ctx, "null context");
        Ctx *c = &ctx->c;
        bind(c);
        batch_solve(c, nmol, natoms, centers, charges, radii, cfgs, max_wave, wave_slots, hbm_budget_bytes, workers,
                    results, statuses, done_ms, info);
        for (int i = 0; i < nmol; ++i)
            if (statuses[i] != IBIM_OK) throw Error(statuses[i], ibim_last_error());
    });
}

int ibim_autotune(ibim_ctx ctx, const double *centers, const double *charges, const double *radii, int natoms,
                  const ibim_config *cfg, int reps, long install_min_points, double *report) {
    return guard([&] {
        IBIM_REQUIRE(ctx && centers && charges && radii && cfg && report && natoms > 0, "null argument");
        IBIM_REQUIRE(cfg->precision == IBIM_PRECISION_MIXED, "autotune: tunes the mixed path's launches");
        check_config(*cfg);
        Ctx *c = &ctx->c;
        bind(c);
        cudaStream_t s = c->stream;
        reps = std::max(1, std::min(reps, 50));
        DevBuf<double> dc, dr;
        dc.alloc(3 * (size_t)natoms, s);
        dr.alloc(natoms, s);
        dc.upload(centers, 3 * (size_t)natoms);
        dr.upload(radii, natoms);
        long npts = 0;
        int timed = 0;
        // a candidate's cost: one solve's mix of products (25 mixed, one FP64-class residual), timed
        // with CUDA events on a plan prepared under the candidate's parameters
        auto cost = [&](const Tuning &t) -> double {
            tuning_override(&t);
            SolvePrep prep;
            ibim_result res;
            try {
                solve_prepare(c, dc.ptr, dr.ptr, centers, charges, natoms, *cfg, res, nullptr, prep);
            } catch (...) {
                tuning_override(nullptr);
                throw;
            }
            tuning_override(nullptr);
            Plan &P = *prep.P;
            for (TargetSet *ts : P.targets) prepare_mixed(P, *ts);
            npts = P.ns;
            DevBuf<double> x, y;
            x.alloc(2 * (size_t)P.ns, s);
            y.alloc(2 * (size_t)P.ns, s);
            permute(c, P.ns, P.src_perm.ptr, prep.b_tube.ptr, x.ptr, false);
            permute(c, P.ns, P.src_perm.ptr, prep.b_tube.ptr + P.ns, x.ptr + P.ns, false);
            // warm-up: the first mixed product sets the plan up, the second captures its graph
            bie_matvec(P, cfg->kp, x.ptr, y.ptr, IBIM_PRECISION_MIXED);
            bie_matvec(P, cfg->kp, x.ptr, y.ptr, IBIM_PRECISION_MIXED);
            bie_matvec(P, cfg->kp, x.ptr, y.ptr, IBIM_PRECISION_FP64_TC);
            // at least reps mixed products and about 30 ms of them, and as many FP64-class ones as
            // fit in the same time: short products are otherwise timed within launch jitter
            Timer t0(s);
            bie_matvec(P, cfg->kp, x.ptr, y.ptr, IBIM_PRECISION_MIXED);
            const double one32 = std::max(1e-3, t0.ms());
            const int n32 = std::max(reps, std::min(1000, (int)std::ceil(30.0 / one32)));
            Timer t1(s);
            for (int r = 0; r < n32; ++r) bie_matvec(P, cfg->kp, x.ptr, y.ptr, IBIM_PRECISION_MIXED);
            const double ms32 = t1.ms() / n32;
            const int n64 = std::max(1, std::min(50, (int)(30.0 / std::max(1e-3, 6.0 * ms32))));
            Timer t2(s);
            for (int r = 0; r < n64; ++r) bie_matvec(P, cfg->kp, x.ptr, y.ptr, IBIM_PRECISION_FP64_TC);
            const double ms64 = t2.ms() / n64;
            IBIM_REQUIRE(!m2l_tc_error(P), "autotune: a tensor-core M2L wait exceeded its bound");
            ++timed;
            return 25.0 * ms32 + ms64;
        };
        Tuning best;
        cost(best);  // untimed: the first candidate would otherwise also grow the memory pool
        timed = 0;
        const double base = cost(best);
        double best_cost = base;
        auto consider = [&](Tuning t) {
            const double v = cost(t);
            if (v < best_cost) {
                best_cost = v;
                best = t;
            }
        };
        // launch form of the tensor-core M2L (the CTA-pair forms in the scaled FP16 form only), then
        // the segment sizes, one coordinate at a time
        for (int f : {4, 6, 7}) {
            if (f != 4 && !m2l_tc_fp16_form()) continue;
            Tuning t = best;
            t.tc_form = f;
            consider(t);
        }
        for (long v : {1L << 15, 1L << 16, 1L << 18}) {
            Tuning t = best;
            t.near_seg_pairs = v;
            consider(t);
        }
        for (long v : {1L << 13, 1L << 15, 1L << 16}) {
            Tuning t = best;
            t.nearff_seg_pairs = v;
            consider(t);
        }
        // the minimum over the candidates is biased low: the best replaces the defaults only when a
        // second measurement of both confirms it by 2 %
        double best_ms = best_cost, default_ms = base;
        if (best.near_seg_pairs != Tuning().near_seg_pairs || best.nearff_seg_pairs != Tuning().nearff_seg_pairs ||
            best.tc_form != Tuning().tc_form) {
            const double b2 = cost(best), d2 = cost(Tuning());
            if (b2 < 0.98 * d2) {
                best_ms = b2;
                default_ms = d2;
            } else {
                best = Tuning();
                best_ms = default_ms = d2;
            }
        }
        report[0] = (double)npts;
        report[1] = (double)best.near_seg_pairs;
        report[2] = (double)best.nearff_seg_pairs;
        report[3] = (double)best.tc_form;
        report[4] = best_ms;
        report[5] = default_ms;
        report[6] = timed;
        if (install_min_points >= 0) {
            const int st = ibim_tuning_set(cfg->np, install_min_points, best.near_seg_pairs, best.nearff_seg_pairs,
                                           best.tc_form);
            if (st != IBIM_OK) throw Error(st, ibim_last_error());
        }
    });
}

int ibim_solve_pqr(ibim_ctx ctx, const char *pqr_path, const ibim_config *cfg, ibim_result *res) {
    return guard([&] {
        IBIM_REQUIRE(ctx && pqr_path && cfg && res, "null argument");
        std::ifstream f(pqr_path);
        if (!f.is_open()) throw Error(IBIM_ERR_IO, std::string("cannot open ") + pqr_path);
        std::vector<double> c, q, r;
        std::string line;
        // molecule.h:21-50: lines starting with ATOM; tokens 5..9 = x y z charge radius
        while (std::getline(f, line)) {
            if (line.rfind("ATOM", 0) != 0) continue;
            std::istringstream ss(line);
            std::vector<std::string> tok;
            std::string t;
            while (ss >> t) tok.push_back(t);
            if (tok.size() < 10) throw Error(IBIM_ERR_IO, "malformed ATOM line: " + line);
            try {
                c.push_back(std::stod(tok[5]));
                c.push_back(std::stod(tok[6]));
                c.push_back(std::stod(tok[7]));
                q.push_back(std::stod(tok[8]));
                r.push_back(std::stod(tok[9]));
            } catch (const std::exception &) {
                throw Error(IBIM_ERR_IO, "malformed ATOM line: " + line);
            }
        }
        if (q.empty()) throw Error(IBIM_ERR_IO, std::string("no ATOM lines in ") + pqr_path);
        const int rc = ibim_solve(ctx, c.data(), q.data(), r.data(), (int)q.size(), cfg, res);
        if (rc != IBIM_OK) throw Error(rc, g_last_error);
    });
}

}  // extern "C"

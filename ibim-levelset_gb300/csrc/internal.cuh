// Internal types shared by the translation units of libibim_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ibim.h"

namespace ibim {

// Thrown inside the library, converted to a status at the C ABI.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

void set_last_error(const std::string &msg);

#define IBIM_CUDA(call)                                                                                       \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess)                                                                                \
            throw ::ibim::Error(e_ == cudaErrorMemoryAllocation ? IBIM_ERR_OUT_OF_MEMORY : IBIM_ERR_CUDA,     \
                                std::string(#call) + ": " + cudaGetErrorString(e_) + " at " + __FILE__ + ":" + \
                                    std::to_string(__LINE__));                                                \
    } while (0)

#define IBIM_CHECK_LAUNCH() IBIM_CUDA(cudaGetLastError())

#define IBIM_REQUIRE(cond, msg)                                                   \
    do {                                                                          \
        if (!(cond)) throw ::ibim::Error(IBIM_ERR_INVALID_ARGUMENT, (msg));       \
    } while (0)

// cudaMallocAsync of `bytes` on `s`.  When the device is out of memory the stream-ordered pool
// may still hold freed blocks that no allocation of this size fits into (the pool keeps what
// solves free): wait for the device, hand the pool's unused memory back and try once more.  A
// second failure throws IBIM_ERR_OUT_OF_MEMORY with the device's and the pool's figures.
void *device_alloc(size_t bytes, cudaStream_t s);

// One molecule's M2L operator images in a merged plan: tensor-core words (hi, lo; FP16 row
// scales) and FP64-class digit tiles with their row scales.
struct MolImg {
    const void *tc_hi, *tc_lo;
    const float *tc_rsc;
    const uint16_t *oz_a;
    const double *oz_sig;
};

// Stream-ordered device buffer owned by a context.
template <typename T>
struct DevBuf {
    T *ptr = nullptr;
    size_t n = 0;
    cudaStream_t stream = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : ptr(o.ptr), n(o.n), stream(o.stream) { o.ptr = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { release(); ptr = o.ptr; n = o.n; stream = o.stream; o.ptr = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count, cudaStream_t s) {
        release();
        stream = s;
        n = count;
        if (count) ptr = static_cast<T *>(device_alloc(sizeof(T) * count, s));
    }
    void release() {
        if (ptr) cudaFreeAsync(ptr, stream);
        ptr = nullptr;
        n = 0;
    }
    void zero() { if (n) IBIM_CUDA(cudaMemsetAsync(ptr, 0, sizeof(T) * n, stream)); }
    void upload(const T *h, size_t count) {
        if (count > n) alloc(count, stream);
        if (count) IBIM_CUDA(cudaMemcpyAsync(ptr, h, sizeof(T) * count, cudaMemcpyHostToDevice, stream));
    }
    void upload(const std::vector<T> &v) { if (v.size() > n || !ptr) alloc(v.size(), stream); upload(v.data(), v.size()); }
    void download(T *h, size_t count) const {
        if (count) IBIM_CUDA(cudaMemcpyAsync(h, ptr, sizeof(T) * count, cudaMemcpyDeviceToHost, stream));
    }
};

// Host scratch array without value-initialisation, for large arrays that are written in full
// (by several threads) before they are read: a std::vector's zero fill is one serial pass.
template <class T> struct HostArr {
    std::unique_ptr<T[]> p;
    size_t n = 0;
    explicit HostArr(size_t k = 0) : p(k ? new T[k] : nullptr), n(k) {}
    T &operator[](size_t i) { return p[i]; }
    const T &operator[](size_t i) const { return p[i]; }
    T *data() { return p.get(); }
    const T *data() const { return p.get(); }
    size_t size() const { return n; }
};

// Kernel categories timed with CUDA events when profiling is enabled on a context.
enum ProfCat {
    PROF_EXPAND = 0, PROF_WENO, PROF_COUNT, PROF_FLOOD, PROF_TUBE, PROF_OPS, PROF_P2M, PROF_M2M, PROF_M2L_V,
    PROF_M2L_X, PROF_L2L, PROF_NEAR, PROF_RHS, PROF_GMRES, PROF_M2L_V64, PROF_M2L_X64, PROF_NEAR64, PROF_M2L_VOZ,
    PROF_L2P, PROF_L2P64, PROF_NEARFF,
    PROF_NCAT
};

// Number of kernels this library launched (all contexts).
void count_launch();
void count_launches(long n);  // n kernels at once (a graph replay), or -n for captured ones
long launch_count();

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // second stream for device work that overlaps host-side planning (the right-hand side),
    // forked from and joined back to `stream` by the two events
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the near field of a matvec runs on `aux` while the far field runs on `stream`
    cudaEvent_t ev_near_fork = nullptr, ev_near_join = nullptr;
    int num_sms = 0;
    unsigned prof_mask = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_ev[PROF_NCAT];
    double prof_flops[PROF_NCAT] = {0}, prof_bytes[PROF_NCAT] = {0};  // algorithmic work of profiled launches
    std::vector<cudaEvent_t> ev_pool;
    cudaEvent_t take_event();
    // pinned host staging for device-to-host copies on the solve's critical path (a pageable
    // destination goes through the driver's bounce buffer); grown on demand, kept with the context
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    void *pinned_buffer(size_t bytes);
    ~Ctx();
};

// Host phase trace for tuning: with IBIM_TRACE set, each mark prints to stderr the wall time
// since the previous mark on this thread.
void trace_mark(const char *phase);

// The context bound by the current C-ABI call on this thread.
Ctx *current_ctx();
void set_current_ctx(Ctx *c);

// Records CUDA events around the launches of one category when the context profiles it.
struct ProfScope {
    Ctx *c;
    int cat;
    cudaEvent_t a = nullptr;
    cudaStream_t s = nullptr;
    explicit ProfScope(int category, double flops = 0., double bytes = 0., cudaStream_t st = nullptr)
        : c(current_ctx()), cat(category) {
        if (c && (c->prof_mask & (1u << cat))) {
            s = st ? st : c->stream;
            a = c->take_event();
            cudaEventRecord(a, s);
            c->prof_flops[cat] += flops;
            c->prof_bytes[cat] += bytes;
        }
    }
    ~ProfScope() {
        if (a) {
            cudaEvent_t b = c->take_event();
            cudaEventRecord(b, s);
            c->prof_ev[cat].push_back({a, b});
        }
    }
};

struct Grid {
    Ctx *ctx;
    int nx, ny, nz;
    double sx, sy, sz, dx;
    int prec = IBIM_PRECISION_FP64;  // storage and stencil arithmetic: FP64, or FP32 (mixed path)
    DevBuf<double> data;
    DevBuf<float> data32;
    long cells() const { return (long)nx * ny * nz; }
};

// Tube points, SoA, in the reference's (i, j, k) extraction order.
struct Tube {
    Ctx *ctx;
    long n = 0;
    double h = 0;
    DevBuf<double> x, y, z, nx, ny, nz, w;  // w = raw cosine weight (levelset.cpp:576)
};

// Octree + interaction lists, host side (tree.cpp).  Node ids are level-ordered.
// Per-node index lists in one array (compressed rows): lists[i] is node i's list.
struct IdxSpan {
    const int *b, *e;
    const int *begin() const { return b; }
    const int *end() const { return e; }
    size_t size() const { return (size_t)(e - b); }
    int operator[](size_t k) const { return b[k]; }
};
struct NodeLists {
    std::vector<long> off;  // size nnodes + 1
    std::vector<int> idx;
    IdxSpan operator[](size_t i) const { return {idx.data() + off[i], idx.data() + off[i + 1]}; }
    size_t size() const { return off.empty() ? 0 : off.size() - 1; }
};

struct TreeHost {
    int p = 0, R = 0;
    int nnodes = 0, nlevels = 0;
    std::vector<int> level_begin;        // size nlevels + 1
    std::vector<double> center, radius;  // 3 per node
    std::vector<int> parent, index8, leaf, empty, coord;  // coord: 3 ints per node
    std::vector<int> src_begin, src_end, tgt_begin, tgt_end;
    std::vector<int> src_perm, tgt_perm;  // tree position -> caller index
    std::vector<int> ref_id;              // node id in the reference's numbering (bbfmm.cpp:88-91)
    // interaction lists per node
    NodeLists U, V, W, X;
};

TreeHost build_tree(const double *src, long ns, const double *tgt, long nt, int maxpoint, int maxlevel);


struct ChebTables;

// Targets binned into a plan's tree, with the work lists that depend on them.
struct TargetSet {
    long nt = 0;
    bool self = false;                 // the plan's sources
    std::vector<int> begin, end;       // per node, range in tree-ordered targets
    std::vector<int> perm;             // tree position -> caller index
    DevBuf<double> tx, ty, tz;         // tree order (self: unused, the source arrays are used)
    DevBuf<int> perm_d, tbeg, tend;
    std::vector<int> l2l_level_begin;
    DevBuf<int> l2l_nodes;
    DevBuf<int> v_src, v_tgt, v_chunk; // contraction pairs sorted by operator; chunks (op, begin, count)
    int nchunks = 0;
    DevBuf<int> v_chunk32;             // chunks of the FP32 contraction (larger)
    int nchunks32 = 0;
    DevBuf<int> v_chunk_tc;            // chunks of the tensor-core contraction (<= 128 pairs)
    int nchunks_tc = 0;
    DevBuf<int> v_chunk_tc2;           // chunks of the CTA-pair tensor-core contraction (<= 256 pairs)
    int nchunks_tc2 = 0;
    DevBuf<int> v_chunk_oz;            // chunks of the sliced FP64-class contraction (<= 64 pairs)
    int nchunks_oz = 0;
    DevBuf<int> chunk_mol_tc, chunk_mol_oz;  // merged plans: the molecule of each chunk
    long nvpairs = 0;                  // pairs of the operator contraction (V, plus X when x_as_ops)
    DevBuf<int> x_src, x_tgt;          // X pairs evaluated on the fly (when not x_as_ops)
    long nxpairs = 0;
    long nv_list = 0, nx_list = 0;     // V and X list sizes (bbfmm.cpp lists, pairs with sources)
    DevBuf<int> tleaf, near_ptr, near_range;
    std::vector<int> tl_h;             // target leaves (nodes with targets), node order
    int ntleaves = 0;
    long near_pairs = 0;
    bool near64_ready = false;         // near_ptr / near_range / near_seg built (FP64 kernel)
    // near-field work segments (one CTA each): {target leaf node, first range, end range, mode},
    // mode bit 0 = this segment adds the L2P term, bit 1 = the leaf has several segments (atomic
    // accumulation into a zeroed output); heaviest first
    DevBuf<int> near_seg;
    int nnear_seg = 0;
    bool near_atomic = false;
    DevBuf<double> out4;               // 4 x nt workspace
    // mixed precision
    bool mixed_ready = false;
    DevBuf<float> txf, tyf, tzf;       // target coordinates relative to their leaf centre
    DevBuf<int> near32_ptr, near32_range;  // per target leaf: source leaves (begin, end)
    DevBuf<float> near32_off;          // per source leaf entry: source leaf centre - target leaf centre
    DevBuf<float> near32_offl;         // its FP32 rounding error (float-float low word)
    DevBuf<float> txl, tyl, tzl;       // low words of the leaf-relative target coordinates
    int near32_entries = 0;
    DevBuf<int> near32_seg;            // work segments over the near32 ranges (as near_seg)
    int nnear32_seg = 0;
    bool near32_atomic = false;
    DevBuf<int> nearff_seg;            // finer segments over the same ranges for the float-float kernel
    int nnearff_seg = 0;
    bool nearff_atomic = false;
    // host copies of the near32 lists between mixed_lists_host and their upload
    bool mixed_host_ready = false;
    std::vector<int> h_ptr32, h_rng32, h_seg32, h_segff;
    std::vector<float> h_off32, h_offl32;
    DevBuf<float> x_off32;             // per X pair: source centre - target centre
};

// Launch parameters a plan takes from the tuning table (tuning.cpp) for its order and size.
struct Tuning {
    long near_seg_pairs = 1L << 17;    // FP32 near field: source-target pairs per work segment (CTA)
    long nearff_seg_pairs = 1L << 14;  // float-float near field
    int tc_form = 2;  // tensor-core M2L: 2 = two CTAs of two row tiles per SM, 4 = one CTA of four,
                      // 0 = persistent; 6, 7 = CTA pairs (2-SM MMAs of M = 256) with one or two
                      // row-tile pairs per CTA (0, 6 and 7 in the scaled FP16 form only)
};
// The table's parameters for Chebyshev order `order` and npoints sources (the entry of that order
// with the largest min_points <= npoints; defaults without one).  IBIM_TC_RT overrides tc_form.
Tuning tuning_for(int order, long npoints);
// Plans made on this thread while t is set use it instead of the table; nullptr restores the table.
void tuning_override(const Tuning *t);

// Tree over the sources + operators + target sets.
struct Plan {
    Ctx *ctx;
    Tube *tube;                 // sources
    long ns;
    int p, R, maxpoint, maxlevel, precision;
    Tuning tune;  // launch parameters for this plan's order and size
    TreeHost tree;
    // sources in tree order
    DevBuf<double> sx, sy, sz, snx, sny, snz, sw;  // sw = w * h^3
    DevBuf<int> src_perm;       // tree pos -> tube index
    // nodes
    DevBuf<double> ncenter, nradius;  // 3 per node
    DevBuf<int> nsrc_begin, nsrc_end, nparent, nindex8, nempty, nchild_first;
    int np2m = 0;
    DevBuf<int> p2m_nodes;
    std::vector<int> m2m_level_begin;
    DevBuf<int> m2m_nodes;
    DevBuf<int> near_next;      // work counter shared by the near-field launches of one matvec
    // M2L operators keyed by (target level, source level, centre offset), union over target sets:
    // the V list's, and (x_as_ops) the X list's, whose pairs then join the V contraction
    bool x_as_ops = true;
    int nops = 0;
    std::vector<int> op_key_h;
    DevBuf<int> op_key;
    DevBuf<double> ops64;          // nops * (4R)^2, column-major per operator
    DevBuf<float> ops32;
    std::vector<TargetSet *> targets;
    // tables and workspaces
    DevBuf<ChebTables> tables;
    DevBuf<double> root_r;
    DevBuf<double> mult, local, dens4;
    DevBuf<float> mult32, local32, dens32;
    DevBuf<float4> src8;           // near-field source records (mixed): {x, y, z, m_x}, {m_y, m_z, psi, 0}
    DevBuf<float> sxf, syf, szf;   // source coordinates relative to their leaf centre (mixed)
    DevBuf<float> sxl, syl, szl;   // their FP32 rounding errors (float-float low words)
    DevBuf<float4> src16;          // float-float near-field source records (FP64-class matvec)
    DevBuf<float2> opsff;          // M2L operators in float-float (hi, lo) for the FP64-class images
    bool opsff_ready = false;
    double kpff[5] = {0, 0, 0, 0, 0};
    DevBuf<float> nrad32;          // per node radius (mixed)
    DevBuf<unsigned char> tables32;  // ChebTables32
    bool mixed_ready = false;
    // tensor-core V-list M2L (m2l_tc.cu): 3xTF32 operand images, padded, for kernel parameters tc_key
    bool tc_ready = false;
    double tc_key[5] = {-1, -1, -1, -1, -1};
    int tc_kpad = 0, tc_mpad = 0;
    bool tc_h16 = false;               // images in the scaled FP16 form (else TF32)
    DevBuf<float> tc_a_hi, tc_a_lo, tc_b_hi, tc_b_lo;  // raw image words
    DevBuf<float> tc_rsc, tc_csc;      // FP16 form: operator row scales, multipole column scales
    DevBuf<int> tc_err;
    // FP64-class V-list M2L of the refinement residual (m2l_tc.cu): operators and multipoles as
    // exact BF16 integer slices under power-of-two row / column scales
    bool oz_ready = false;           // digit images valid for kernel parameters oz_key
    double oz_key[5] = {-1, -1, -1, -1, -1};
    int oz_kpad = 0, oz_mtiles = 0, oz_s = 7;  // digit images: K padded, row tiles, digits
    DevBuf<uint16_t> oz_a, oz_b;
    DevBuf<double> oz_sig, oz_tau;
    double kp64[5] = {-1, -1, -1, -1, -1}, kp32[5] = {-1, -1, -1, -1, -1};  // kernel parameters of the cached operators
    bool ops64_ready = false, ops32_ready = false;
    // a plan merged over several molecules (batch.cu): the molecule of every node and each
    // molecule's kappa-dependent near-field constants (FP32: kappa, -kappa log2 e, k2in / q4pi;
    // float-float: kappa hi, lo, k2in hi, lo)
    bool batched = false;
    DevBuf<int> node_mol;
    DevBuf<float4> kmol32, kmolff;
    DevBuf<int> mol_active;  // 1 while a molecule iterates: the heavy kernels skip the others' work
    // each molecule's operator images stay where its own plan built them: the M2L kernels take
    // the images of a chunk's molecule from mol_img (chunks carry the molecule's own operator
    // ids), and the merged plan owns the buffers
    DevBuf<MolImg> mol_img;
    std::vector<DevBuf<float>> own_f;
    std::vector<DevBuf<uint16_t>> own_u16;
    std::vector<DevBuf<double>> own_d;
    // the mixed-precision matvec as a CUDA graph (solve.cu bie_matvec): captured on its second call
    // with the same kernel parameters and replayed with its input and output staged through gx / gy
    struct MatvecGraph {
        cudaGraphExec_t exec = nullptr;
        double key[5] = {-1, -1, -1, -1, -1};
        long kernels = 0;  // kernel nodes of the graph
        int calls = 0;
        bool failed = false;
    } mvg;
    DevBuf<double> gx, gy;
    ~Plan() {
        if (mvg.exec) cudaGraphExecDestroy(mvg.exec); for (auto *t : targets) delete t; }
};

// FMM engine.  dens: 4 x ns (tree order), out: 4 x nt of target set `ts` (tree order).
void fmm_prepare_operators(Plan &P, const ibim_kernel_params &kp, int precision);
// m2l_sliced: the V-list M2L on the tensor cores by exact BF16 slicing (FP64-class accuracy),
// as used for the mixed path's refinement residual; false = FP64 pipe, the reference-exact path.
void fmm_run_fp64(Plan &P, int ts, const ibim_kernel_params &kp, const double *dens, double *out,
                  bool m2l_sliced = false);
void fmm_run_mixed(Plan &P, int ts, const ibim_kernel_params &kp, const double *dens, double *out);
void fmm_run(Plan &P, int ts, const ibim_kernel_params &kp, const double *dens, double *out, int precision);

// Tensor-core V-list M2L (m2l_tc.cu)
bool m2l_tc_supported();
// Tensor-core images from P.ops32, or in the FP16 form from float-float operators when ff is given.
void m2l_tc_pack(Plan &P, const float2 *ff = nullptr);
// Whether the mixed path's tensor-core M2L uses the scaled FP16 operand form.
bool m2l_tc_fp16_form();
void m2l_tc_run(Plan &P, TargetSet &S);
int m2l_tc_error(Plan &P);
// BF16 digit images and row scales from P.ops64, or from float-float operators when ff is given.
void m2l_oz_pack(Plan &P, const float2 *ff = nullptr);
// Both images (digit tiles and scaled FP16 tiles) of the float-float operators in one pass.
void m2l_pack_images_ff(Plan &P, const float2 *ff);
// Test check: the one-pass images equal the separate passes' word for word (throws otherwise).
void m2l_check_images_ff(Plan &P, const float2 *ff);
void m2l_oz_run(Plan &P, const TargetSet &S);
// Operator images for kernel parameters kp, built when missing or stale: the TF32 images (from
// FP32 operators, which are then released) and the digit images (from the FP64 operators).
void fmm_ensure_tc_images(Plan &P, const ibim_kernel_params &kp);
void fmm_ensure_oz_images(Plan &P, const ibim_kernel_params &kp);
// The mixed path's FP16 images and the FP64-class digit images together, from one set of
// float-float operators (scaled FP16 form, float-float operators enabled); false otherwise.
bool fmm_ensure_images_ff(Plan &P, const ibim_kernel_params &kp);
// Release the FP64 operators (rebuilt on demand) once only their digit images are needed.
void fmm_release_fp64_operators(Plan &P);
// Whether the mixed path's V-list M2L runs on the tensor cores on this device.
bool mixed_uses_tc();
// Whether the FP64-class matvec evaluates its near field in float-float (default; IBIM_NEAR_FF=0
// keeps native FP64).
bool near_ff_enabled();
// Whether the FP64-class operator images (digit slices, and the mixed path's FP16 images made
// beside them) come from float-float operators instead of FP64 ones (default; IBIM_OPS_FF=0).
bool ops_ff_enabled();
// The M2L operators in float-float into P.opsff (once per kernel-parameter set).
void fmm_prepare_operators_ff(Plan &P, const ibim_kernel_params &kp);
// Host half of prepare_mixed for one target set (no CUDA calls): the FP32 / float-float near
// lists and their work segments, kept in the target set until prepare_mixed uploads them, so a
// solve can build them while the device computes the M2L operators.
void mixed_lists_host(const Plan &P, TargetSet &S);
// Whether a matvec's near field runs on the auxiliary stream beside its far field (default on;
// IBIM_NEAR_OVERLAP=0 runs it after the far field with the L2P fused in).
bool near_overlap();
// CTAs per SM of the near-field launch that runs beside the far field (IBIM_NEAR_SIDE; 0, the
// default, is full occupancy); a drain launch after the far field takes the segments it leaves.
int near_side_ctas();

// Near-field work segments.  Target leaf k (node tl[k], nt[k] targets) owns source ranges
// ptr[k] .. ptr[k+1] of `rng` (begin, end pairs); consecutive ranges are grouped into segments of
// at most max(min_sources, max_pairs / nt[k]) sources, so no CTA carries much more than max_pairs
// source-target pairs; ranges longer than that are split first (split_long).  Output: 4 ints per
// segment (see TargetSet::near_seg), sorted by descending work; returns whether any leaf has
// several segments.
constexpr long NEAR_SEG_PAIRS = 1L << 17;   // FP64 and FP32 near fields
constexpr long NEAR_FF_SEG_PAIRS = 1L << 14;  // float-float near field (about 8 times the work a pair)
bool near_segments(const std::vector<int> &tl, const std::vector<int> &nt, std::vector<int> &ptr,
                   std::vector<int> &rng, bool split_long, std::vector<int> &seg, long max_pairs = NEAR_SEG_PAIRS,
                   long min_sources = 256);

// Plan creation (fmm.cu): target set 0 = the tube points when with_self, then `extra` (host
// (n, 3)) when n_extra > 0.
Plan *make_plan(Tube *t, bool with_self, const double *extra, long n_extra, int order, int maxpoint, int maxlevel,
                int precision);

// Level set (levelset.cu)
Grid *grid_create(Ctx *c, int nx, int ny, int nz, double sx, double sy, double sz, double dx, double value,
                  int prec = IBIM_PRECISION_FP64);
void levelset_expand(Grid &g, const double *centers_dev, const double *radii_dev, int natoms, double probe, int band);
void levelset_evolve(Grid &g, double final_t, double vel, double cfl);
int levelset_reinitialize(Grid &g, const Grid &phi0, double final_t, double vel, double cfl, int thickness,
                          double thres);
void levelset_count_gradient(const Grid &g, double thickness, double thres, long *bad, long *total, double *acc);
void grid_scale(Grid &g, double s);
void grid_copy(Grid &dst, const Grid &src);
// jacobian: multiply the weights by the surface Jacobian (opt-in; the reference has none)
Tube *surface_extract(Grid &g, int thickness, long *inclusion, bool jacobian = false);

// Timing helper
struct Timer {
    cudaEvent_t a, b;
    cudaStream_t s;
    explicit Timer(cudaStream_t st) : s(st) { cudaEventCreate(&a); cudaEventCreate(&b); cudaEventRecord(a, s); }
    ~Timer() { cudaEventDestroy(a); cudaEventDestroy(b); }
    double ms() { cudaEventRecord(b, s); cudaEventSynchronize(b); float m = 0; cudaEventElapsedTime(&m, a, b); return m; }
};

inline int div_up(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace ibim

struct ibim_ctx_s { ibim::Ctx c; };
struct ibim_grid_s { ibim::Grid *g; };
struct ibim_tube_s { ibim::Tube *t; };
struct ibim_plan_s { ibim::Plan *p; };

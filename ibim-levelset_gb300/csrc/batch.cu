// Many molecules solved together on one GPU (no counterpart in the reference: main.cpp solves one
// molecule per run).  The operator batched here is dmapping (electric.cpp:294-388) inside the mixed
// path's iterative refinement; GMRES follows gmres.cpp:50-164 for every molecule.
//
//   prepare     worker threads, each on its own context and streams, run the part of a solve before
//               GMRES (level set, tube, right-hand side, plan, operator images) for the molecules
//               in order, while the device bytes of the prepared molecules stay within the budget
//   merge       a wave of prepared molecules becomes one plan: sources, nodes, V/X pairs, near
//               lists and both target sets concatenated with offsets (node lists kept level by
//               level), so every FMM stage of a matvec (P2M, M2M per level, tensor-core M2L, L2L per
//               level, near field, L2P) is one launch over all molecules of the wave -- a flattened
//               multi-tree work list, replayed as one CUDA graph per matvec; the operator images
//               stay in each molecule's buffers (the M2L kernels find a chunk's by its molecule),
//               the near-field kernels take each target leaf's molecule for its kappa, and
//               near-field segments of all molecules are sorted by work
//   lock-step   GMRES advances every molecule of the wave together: one merged matvec per Arnoldi
//               step, modified Gram-Schmidt per molecule by segmented reductions of fixed shape,
//               one host synchronisation per step for all molecules' Givens rotations; molecules
//               leave the vector work as they converge
//   refinement  the mixed path's FP64 iterative refinement in lock-step: inner GMRES on the merged
//               mixed operator, then one merged FP64-class residual per pass for the wave
//   energy      polarizeMap (electric.cpp:442-505) on the merged atom targets: one FMM for the wave

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>

#include "fmm_common.cuh"
#include "solve.cuh"

namespace ibim {

namespace {

constexpr int BT = 256;     // threads of the segmented vector kernels
constexpr int BMAXB = 256;  // most blocks of one molecule's reduction

__device__ __forceinline__ double bsum(double v) {
    __shared__ double sh[BT / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.;
    if (threadIdx.x == 0)
        for (int w = 0; w < BT / 32; ++w) s += sh[w];
    __syncthreads();
    return s;  // valid in thread 0
}

// Molecule m's partial sums added in a fixed order; every thread gets the value.
__device__ __forceinline__ double bred(const double *__restrict__ part, int m, int nb) {
    __shared__ double v;
    double s = 0.;
    for (int q = threadIdx.x; q < nb; q += BT) s += part[(long)m * BMAXB + q];
    s = bsum(s);
    if (threadIdx.x == 0) v = s;
    __syncthreads();
    return v;
}

// The molecules a segmented launch works on (blockIdx.y indexes act), and where each one's part of
// a merged vector [phi (n); psi (n)] lies: its sources [off, off + len) in both halves.
struct Segs {
    const long *off, *len;
    const int *nblk, *act;
    long n;
};

__device__ __forceinline__ long bidx(long off, long len, long n, long i) {
    return i < len ? off + i : n + off + (i - len);
}

__global__ void __launch_bounds__(BT) k_bdot(Segs S, const double *__restrict__ a, const double *__restrict__ b,
                                             double *part) {
    const int m = S.act[blockIdx.y], nb = S.nblk[m];
    if ((int)blockIdx.x >= nb) return;
    const long o = S.off[m], L = S.len[m];
    double s = 0.;
    for (long i = blockIdx.x * (long)BT + threadIdx.x; i < 2 * L; i += (long)nb * BT) {
        const long q = bidx(o, L, S.n, i);
        s += a[q] * b[q];
    }
    s = bsum(s);
    if (threadIdx.x == 0) part[(long)m * BMAXB + blockIdx.x] = s;
}

// MGS step per molecule: h = <w, v_prev> from the partials, w -= h v_prev, then the partials of
// <w, v_next> (or <w, w> when v_next is null); h goes to hcol[m][slot].
__global__ void __launch_bounds__(BT) k_bmgs(Segs S, const double *__restrict__ part_in, double *w,
                                             const double *__restrict__ vprev, const double *__restrict__ vnext,
                                             double *part_out, double *hcol, int ldh, int slot) {
    const int m = S.act[blockIdx.y], nb = S.nblk[m];
    if ((int)blockIdx.x >= nb) return;
    const double h = bred(part_in, m, nb);
    if (blockIdx.x == 0 && threadIdx.x == 0) hcol[(long)m * ldh + slot] = h;
    const long o = S.off[m], L = S.len[m];
    double s = 0.;
    for (long i = blockIdx.x * (long)BT + threadIdx.x; i < 2 * L; i += (long)nb * BT) {
        const long q = bidx(o, L, S.n, i);
        const double wi = w[q] - h * vprev[q];
        w[q] = wi;
        s += wi * (vnext ? vnext[q] : wi);
    }
    s = bsum(s);
    if (threadIdx.x == 0) part_out[(long)m * BMAXB + blockIdx.x] = s;
}

// v = w / ||w|| per molecule, ||w|| from the partials of <w, w>, stored in hcol[m][slot].
__global__ void __launch_bounds__(BT) k_bnormalize(Segs S, const double *__restrict__ part_in,
                                                   const double *__restrict__ w, double *v, double *hcol, int ldh,
                                                   int slot) {
    const int m = S.act[blockIdx.y], nb = S.nblk[m];
    if ((int)blockIdx.x >= nb) return;
    const double nr = sqrt(bred(part_in, m, nb));
    if (blockIdx.x == 0 && threadIdx.x == 0) hcol[(long)m * ldh + slot] = nr;
    const double sc = 1.0 / nr;
    const long o = S.off[m], L = S.len[m];
    for (long i = blockIdx.x * (long)BT + threadIdx.x; i < 2 * L; i += (long)nb * BT) {
        const long q = bidx(o, L, S.n, i);
        v[q] = w[q] * sc;
    }
}

// ||.|| per molecule from the partials of <v, v> (one block per molecule).
__global__ void __launch_bounds__(BT) k_bnorm(Segs S, const double *__restrict__ part_in, double *hcol, int ldh,
                                              int slot) {
    const int m = S.act[blockIdx.y];
    const double nr = sqrt(bred(part_in, m, S.nblk[m]));
    if (threadIdx.x == 0) hcol[(long)m * ldh + slot] = nr;
}

// x += sum_{j < k} y_m[j] v_j per molecule (gmres.cpp:19-20, one daxpy per j in order).
__global__ void __launch_bounds__(BT) k_bupdate(Segs S, int k, const double *__restrict__ y, int ldy,
                                                const double *__restrict__ V, long n2, double *x) {
    const int m = S.act[blockIdx.y], nb = S.nblk[m];
    if ((int)blockIdx.x >= nb) return;
    const long o = S.off[m], L = S.len[m];
    const double *ym = y + (long)m * ldy;
    for (long i = blockIdx.x * (long)BT + threadIdx.x; i < 2 * L; i += (long)nb * BT) {
        const long q = bidx(o, L, S.n, i);
        double s = x[q];
        for (int j = 0; j < k; ++j) s += ym[j] * V[(long)j * n2 + q];
        x[q] = s;
    }
}

// c = a - b, x += d, c = a on the molecules' parts
__global__ void __launch_bounds__(BT) k_bsub(Segs S, const double *__restrict__ a, const double *__restrict__ b,
                                             double *c) {
    const int m = S.act[blockIdx.y], nb = S.nblk[m];
    if ((int)blockIdx.x >= nb) return;
    const long o = S.off[m], L = S.len[m];
    for (long i = blockIdx.x * (long)BT + threadIdx.x; i < 2 * L; i += (long)nb * BT) {
        const long q = bidx(o, L, S.n, i);
        c[q] = a[q] - b[q];
    }
}

__global__ void __launch_bounds__(BT) k_badd(Segs S, const double *__restrict__ d, double *x) {
    const int m = S.act[blockIdx.y], nb = S.nblk[m];
    if ((int)blockIdx.x >= nb) return;
    const long o = S.off[m], L = S.len[m];
    for (long i = blockIdx.x * (long)BT + threadIdx.x; i < 2 * L; i += (long)nb * BT) {
        const long q = bidx(o, L, S.n, i);
        x[q] += d[q];
    }
}

__global__ void __launch_bounds__(BT) k_bcopy(Segs S, const double *__restrict__ a, double *c) {
    const int m = S.act[blockIdx.y], nb = S.nblk[m];
    if ((int)blockIdx.x >= nb) return;
    const long o = S.off[m], L = S.len[m];
    for (long i = blockIdx.x * (long)BT + threadIdx.x; i < 2 * L; i += (long)nb * BT) {
        const long q = bidx(o, L, S.n, i);
        c[q] = a[q];
    }
}

// Records of w ints: dst = src + add[field]; negative values of the fields flagged in keep_neg
// (absent parent / child: -1) stay as they are.
__global__ void k_shift_ints(long nrec, int w, const int *__restrict__ src, int *dst, int4 add, int keep_neg) {
    const long n = nrec * w;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int f = (int)(i % w);
        const int a = f == 0 ? add.x : (f == 1 ? add.y : (f == 2 ? add.z : add.w));
        const int v = src[i];
        dst[i] = (v < 0 && ((keep_neg >> f) & 1)) ? v : v + a;
    }
}

// ---------------------------------------------------------------------------------------------
// merge
// ---------------------------------------------------------------------------------------------

template <class T>
size_t bytes_of(const DevBuf<T> &b) {
    return b.ptr ? b.n * sizeof(T) : 0;
}

// Device bytes a plan holds (its main buffers; the tube is counted by the caller).
size_t plan_bytes(const Plan &P) {
    size_t b = bytes_of(P.sx) * 7 + bytes_of(P.ncenter) * 2 + bytes_of(P.mult) + bytes_of(P.local) +
               bytes_of(P.dens4) + bytes_of(P.mult32) + bytes_of(P.local32) + bytes_of(P.dens32) + bytes_of(P.src8) +
               bytes_of(P.sxf) * 6 + bytes_of(P.src16) + bytes_of(P.tc_a_hi) + bytes_of(P.tc_a_lo) +
               bytes_of(P.tc_b_hi) + bytes_of(P.tc_b_lo) + bytes_of(P.tc_rsc) + bytes_of(P.tc_csc) + bytes_of(P.oz_a) +
               bytes_of(P.oz_b) + bytes_of(P.oz_sig) + bytes_of(P.oz_tau) + bytes_of(P.ops64) + bytes_of(P.ops32) +
               bytes_of(P.opsff) + bytes_of(P.nsrc_begin) * 6;
    for (const TargetSet *S : P.targets)
        b += bytes_of(S->v_src) * 2 + bytes_of(S->v_chunk_tc) + bytes_of(S->v_chunk_oz) + bytes_of(S->near32_range) +
             bytes_of(S->near32_off) * 2 + bytes_of(S->out4) + bytes_of(S->tx) * 3 + bytes_of(S->txf) * 6 +
             bytes_of(S->tbeg) * 2 + bytes_of(S->near_range) + bytes_of(S->near32_seg) + bytes_of(S->nearff_seg);
    return b;
}

template <class T>
void dcopy(T *dst, const T *src, size_t n, cudaStream_t s) {
    if (n) IBIM_CUDA(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
}

// dst = the molecules' arrays one after the other (count(m) elements of get(m)).
template <class T, class Get, class Count>
void cat_buf(DevBuf<T> &dst, int M, Get get, Count count, cudaStream_t s) {
    size_t tot = 0;
    for (int m = 0; m < M; ++m) tot += count(m);
    dst.alloc(std::max<size_t>(1, tot), s);
    size_t o = 0;
    for (int m = 0; m < M; ++m) {
        dcopy(dst.ptr + o, get(m), count(m), s);
        o += count(m);
    }
}

void shift_into(int *dst, const int *src, long nrec, int w, int4 add, int keep_neg, int sms, cudaStream_t s) {
    if (nrec <= 0) return;
    const int grid = (int)std::max<long>(1, std::min<long>(4L * sms, div_up(nrec * w, 256)));
    (count_launch(), k_shift_ints<<<grid, 256, 0, s>>>(nrec, w, src, dst, add, keep_neg));
    IBIM_CHECK_LAUNCH();
}

// dst = the molecules' int records (nrec(m) records of w ints at get(m)) with add(m) per field.
template <class Get, class Count, class Add>
void cat_shift(DevBuf<int> &dst, int M, int w, int keep_neg, Get get, Count nrec, Add add, int sms, cudaStream_t s) {
    long tot = 0;
    for (int m = 0; m < M; ++m) tot += nrec(m);
    dst.alloc((size_t)std::max<long>(1, tot * w), s);
    long o = 0;
    for (int m = 0; m < M; ++m) {
        shift_into(dst.ptr + o * w, get(m), nrec(m), w, add(m), keep_neg, sms, s);
        o += nrec(m);
    }
}

// Per-level node lists (level_begin of each molecule) merged level by level.
template <class GetNodes, class GetBegin, class Levels>
std::vector<int> cat_levels(DevBuf<int> &dst, int M, int nlev, GetNodes nodes, GetBegin lb, Levels nl,
                            const std::vector<long> &node_off, int sms, cudaStream_t s) {
    long tot = 0;
    for (int m = 0; m < M; ++m) tot += lb(m)[nl(m)];
    dst.alloc((size_t)std::max<long>(1, tot), s);
    std::vector<int> out(nlev + 1, 0);
    long o = 0;
    for (int l = 0; l < nlev; ++l) {
        out[l] = (int)o;
        for (int m = 0; m < M; ++m) {
            if (l >= nl(m)) continue;
            const int b = lb(m)[l], e = lb(m)[l + 1];
            shift_into(dst.ptr + o, nodes(m) + b, e - b, 1, make_int4((int)node_off[m], 0, 0, 0), 0, sms, s);
            o += e - b;
        }
    }
    out[nlev] = (int)o;
    return out;
}

struct WaveMol {
    long src_off = 0, node_off = 0;
    long tgt_off[2] = {0, 0};
    std::vector<int> perm_atoms;  // atom target set: tree position -> atom index
};

// Near-field segments of all molecules (one of the two segment lists), shifted to the merged
// plan's leaves and ranges, sorted by work (source-target pairs), heaviest first.
template <class SegBuf, class Nseg>
void merge_segments(DevBuf<int> &dst, const std::vector<Plan *> &mols, int ts, const std::vector<WaveMol> &W,
                    const std::vector<long> &ent_off, SegBuf segbuf, Nseg nseg, cudaStream_t s) {
    struct Rec {
        long work;
        int4 v;
    };
    std::vector<Rec> all;
    for (size_t m = 0; m < mols.size(); ++m) {
        const TargetSet &S = *mols[m]->targets[ts];
        const int ns_ = nseg(S);
        if (ns_ == 0) continue;
        std::vector<int> seg(4 * (size_t)ns_), rng(2 * (size_t)S.near32_entries);
        // the molecule's buffers belong to its worker's (idle) stream: plain synchronous copies
        IBIM_CUDA(cudaMemcpy(seg.data(), segbuf(S).ptr, sizeof(int) * seg.size(), cudaMemcpyDeviceToHost));
        if (!rng.empty())
            IBIM_CUDA(cudaMemcpy(rng.data(), S.near32_range.ptr, sizeof(int) * rng.size(), cudaMemcpyDeviceToHost));
        for (int k = 0; k < ns_; ++k) {
            const int leaf = seg[4 * k], r0 = seg[4 * k + 1], r1 = seg[4 * k + 2], mode = seg[4 * k + 3];
            long src = 0;
            for (int r = r0; r < r1; ++r) src += rng[2 * r + 1] - rng[2 * r];
            const long nt = (long)S.end[leaf] - S.begin[leaf];
            all.push_back({src * nt, make_int4(leaf + (int)W[m].node_off, r0 + (int)ent_off[m], r1 + (int)ent_off[m],
                                               mode)});
        }
    }
    std::stable_sort(all.begin(), all.end(), [](const Rec &a, const Rec &b) { return a.work > b.work; });
    std::vector<int> flat(4 * all.size());
    for (size_t k = 0; k < all.size(); ++k) {
        flat[4 * k] = all[k].v.x;
        flat[4 * k + 1] = all[k].v.y;
        flat[4 * k + 2] = all[k].v.z;
        flat[4 * k + 3] = all[k].v.w;
    }
    dst.alloc(std::max<size_t>(4, flat.size()), s);
    if (!flat.empty()) dst.upload(flat.data(), flat.size());
}

// The merged plan of a wave.  mols: prepared plans (mixed precision, with both target sets: tube
// points and atoms, FP16 tensor-core images and FP64-class digit images); kps: each molecule's
// kernel parameters; kp_rep: the parameters whose keys the merged images carry.
Plan *merge_wave(Ctx *c, Tube *mtube, const std::vector<Plan *> &mols, const std::vector<ibim_kernel_params> &kps,
                 const ibim_kernel_params &kp_rep, double h, std::vector<WaveMol> &W) {
    cudaStream_t s = c->stream;
    const int M = (int)mols.size(), sms = c->num_sms;
    const Plan &P0 = *mols[0];
    std::unique_ptr<Plan> B(new Plan());
    B->ctx = c;
    B->tube = mtube;
    B->p = P0.p;
    B->R = P0.R;
    B->maxpoint = P0.maxpoint;
    B->maxlevel = P0.maxlevel;
    B->precision = IBIM_PRECISION_MIXED;
    B->x_as_ops = true;
    B->batched = true;
    const int R = B->R, n4 = 4 * R;
    W.assign(M, WaveMol());
    long ns = 0, nn = 0, nops = 0;
    int nlev = 0;
    std::vector<long> node_off(M);
    for (int m = 0; m < M; ++m) {
        const Plan &P = *mols[m];
        IBIM_REQUIRE(P.p == P0.p && P.x_as_ops && P.targets.size() == 2 && P.tc_ready && P.oz_ready &&
                         P.tc_h16 == P0.tc_h16 && P.tc_kpad == P0.tc_kpad && P.tc_mpad == P0.tc_mpad &&
                         P.oz_kpad == P0.oz_kpad && P.oz_s == P0.oz_s && P.oz_mtiles == P0.oz_mtiles,
                     "batch: molecules with different plan shapes");
        W[m].src_off = ns;
        W[m].node_off = node_off[m] = nn;
        ns += P.ns;
        nn += P.tree.nnodes;
        nops += P.nops;
        nlev = std::max(nlev, P.tree.nlevels);
        W[m].perm_atoms = P.targets[1]->perm;
    }
    IBIM_REQUIRE(ns < INT_MAX / 2 && nn < INT_MAX && nops < INT_MAX, "batch: wave too large for 32-bit indices");
    B->ns = ns;
    B->nops = (int)nops;
    B->tree.nnodes = (int)nn;
    B->tree.nlevels = nlev;
    B->tree.p = B->p;
    B->tree.R = R;
    auto P_ = [&](int m) -> const Plan & { return *mols[m]; };
    // sources (tree order), nodes
    DevBuf<double> Plan::*src7[7] = {&Plan::sx, &Plan::sy, &Plan::sz, &Plan::snx, &Plan::sny, &Plan::snz, &Plan::sw};
    for (auto f : src7)
        cat_buf((*B).*f, M, [&](int m) { return (P_(m).*f).ptr; }, [&](int m) { return (size_t)P_(m).ns; }, s);
    DevBuf<float> Plan::*srcf[6] = {&Plan::sxf, &Plan::syf, &Plan::szf, &Plan::sxl, &Plan::syl, &Plan::szl};
    for (auto f : srcf)
        cat_buf((*B).*f, M, [&](int m) { return (P_(m).*f).ptr; }, [&](int m) { return (size_t)P_(m).ns; }, s);
    cat_buf(B->ncenter, M, [&](int m) { return P_(m).ncenter.ptr; }, [&](int m) { return 3 * (size_t)P_(m).tree.nnodes; }, s);
    cat_buf(B->nradius, M, [&](int m) { return P_(m).nradius.ptr; }, [&](int m) { return 3 * (size_t)P_(m).tree.nnodes; }, s);
    cat_buf(B->nrad32, M, [&](int m) { return P_(m).nrad32.ptr; }, [&](int m) { return 3 * (size_t)P_(m).tree.nnodes; }, s);
    auto nodes = [&](int m) { return (long)P_(m).tree.nnodes; };
    auto add_src = [&](int m) { return make_int4((int)W[m].src_off, 0, 0, 0); };
    auto add_node = [&](int m) { return make_int4((int)W[m].node_off, 0, 0, 0); };
    auto zero4 = [](int) { return make_int4(0, 0, 0, 0); };
    cat_shift(B->nsrc_begin, M, 1, 0, [&](int m) { return P_(m).nsrc_begin.ptr; }, nodes, add_src, sms, s);
    cat_shift(B->nsrc_end, M, 1, 0, [&](int m) { return P_(m).nsrc_end.ptr; }, nodes, add_src, sms, s);
    cat_shift(B->nparent, M, 1, 1, [&](int m) { return P_(m).nparent.ptr; }, nodes, add_node, sms, s);
    cat_shift(B->nchild_first, M, 1, 1, [&](int m) { return P_(m).nchild_first.ptr; }, nodes, add_node, sms, s);
    cat_shift(B->nindex8, M, 1, 0, [&](int m) { return P_(m).nindex8.ptr; }, nodes, zero4, sms, s);
    cat_shift(B->nempty, M, 1, 0, [&](int m) { return P_(m).nempty.ptr; }, nodes, zero4, sms, s);
    cat_shift(B->p2m_nodes, M, 1, 0, [&](int m) { return P_(m).p2m_nodes.ptr; },
              [&](int m) { return (long)P_(m).np2m; }, add_node, sms, s);
    B->np2m = 0;
    for (int m = 0; m < M; ++m) B->np2m += P_(m).np2m;
    B->m2m_level_begin = cat_levels(
        B->m2m_nodes, M, nlev, [&](int m) { return P_(m).m2m_nodes.ptr; },
        [&](int m) { return P_(m).m2m_level_begin.data(); }, [&](int m) { return P_(m).tree.nlevels; }, node_off, sms, s);
    // image shapes per operator and per node, from a molecule with operators
    int ref = -1;
    for (int m = 0; m < M && ref < 0; ++m)
        if (P_(m).nops > 0) ref = m;
    size_t oz_node = 0;
    if (ref >= 0) oz_node = P_(ref).oz_b.n / P_(ref).tree.nnodes;
    // the molecules' matvec workspaces are not used again: freed before the merged ones exist
    for (int m = 0; m < M; ++m) {
        Plan &P = *mols[m];
        auto drop = [&](auto &buf) {
            buf.stream = s;
            buf.release();
        };
        drop(P.mult), drop(P.local), drop(P.dens4), drop(P.mult32), drop(P.local32), drop(P.dens32);
        drop(P.src8), drop(P.tc_b_hi), drop(P.tc_b_lo), drop(P.tc_csc), drop(P.oz_b), drop(P.oz_tau);
    }
    // tables (the same for every molecule of one order), workspaces
    B->tables.alloc(1, s);
    dcopy(B->tables.ptr, P0.tables.ptr, 1, s);
    B->tables32.alloc(P0.tables32.n, s);
    dcopy(B->tables32.ptr, P0.tables32.ptr, P0.tables32.n, s);
    B->mult.alloc((size_t)nn * n4, s);
    B->local.alloc((size_t)nn * n4, s);
    B->dens4.alloc((size_t)4 * ns, s);
    B->mult32.alloc((size_t)nn * n4, s);
    B->local32.alloc((size_t)nn * n4, s);
    B->dens32.alloc((size_t)4 * ns, s);
    B->src8.alloc((size_t)2 * ns, s);
    B->near_next.alloc(1, s);
    B->mixed_ready = true;
    // operator images
    B->tc_h16 = P0.tc_h16;
    B->tc_kpad = P0.tc_kpad;
    B->tc_mpad = P0.tc_mpad;
    B->oz_kpad = P0.oz_kpad;
    B->oz_mtiles = P0.oz_mtiles;
    B->oz_s = P0.oz_s;
    const size_t tc_node = (size_t)B->tc_kpad / (B->tc_h16 ? 2 : 1);
    // the images are the bulk of a plan (GB per molecule): they stay where each molecule's plan
    // built them, owned by the merged plan from here on, and the kernels find them by molecule
    std::vector<MolImg> imgs(M);
    for (int m = 0; m < M; ++m) {
        Plan &P = *mols[m];
        imgs[m] = MolImg{P.tc_a_hi.ptr, P.tc_a_lo.ptr, P.tc_rsc.ptr, P.oz_a.ptr, P.oz_sig.ptr};
        auto adopt = [&](auto &own, auto &buf) {
            if (!buf.ptr) return;
            buf.stream = s;
            own.push_back(std::move(buf));
        };
        adopt(B->own_f, P.tc_a_hi);
        adopt(B->own_f, P.tc_a_lo);
        adopt(B->own_f, P.tc_rsc);
        adopt(B->own_u16, P.oz_a);
        adopt(B->own_d, P.oz_sig);
    }
    B->mol_img.alloc(M, s);
    B->mol_img.upload(imgs.data(), M);
    if (B->tc_h16) B->tc_csc.alloc((size_t)nn, s);
    B->tc_b_hi.alloc((size_t)nn * tc_node, s);
    B->tc_b_lo.alloc((size_t)nn * tc_node, s);
    B->tc_err.alloc(1, s);
    B->tc_err.zero();
    if (ref >= 0) {
        B->oz_b.alloc((size_t)nn * oz_node, s);
        B->oz_tau.alloc((size_t)nn, s);
    }
    double key[5] = {kp_rep.kappa, kp_rep.dE, kp_rep.dI, kp_rep.tau, (double)kp_rep.k3_scaled};
    for (int i = 0; i < 5; ++i) B->tc_key[i] = B->oz_key[i] = key[i];
    B->tc_ready = true;
    B->oz_ready = true;
    // molecule of each node, per-molecule near-field constants
    std::vector<int> nm((size_t)nn);
    std::vector<float4> k32(M), kff(M);
    for (int m = 0; m < M; ++m) {
        std::fill(nm.begin() + W[m].node_off, nm.begin() + W[m].node_off + P_(m).tree.nnodes, m);
        const KParams k = make_kparams(kps[m], h);
        k32[m] = make_float4((float)k.kappa, (float)(-k.kappa * 1.4426950408889634), (float)(k.k2in / k.q4pi), 0.f);
        const float kh = (float)k.kappa, ih = (float)k.k2in;
        kff[m] = make_float4(kh, (float)(k.kappa - (double)kh), ih, (float)(k.k2in - (double)ih));
    }
    B->node_mol.alloc(nm.size(), s);
    B->node_mol.upload(nm.data(), nm.size());
    B->kmol32.alloc(M, s);
    B->kmol32.upload(k32.data(), M);
    B->kmolff.alloc(M, s);
    B->kmolff.upload(kff.data(), M);
    // target sets: 0 = the tube points, 1 = the atoms
    for (int ts = 0; ts < 2; ++ts) {
        TargetSet *T = new TargetSet();
        B->targets.push_back(T);
        auto S_ = [&](int m) -> const TargetSet & { return *mols[m]->targets[ts]; };
        T->self = ts == 0;
        std::vector<long> tgt_off(M), pair_off(M), ent_off(M);
        long nt = 0, np = 0, ne = 0;
        for (int m = 0; m < M; ++m) {
            const TargetSet &S = S_(m);
            IBIM_REQUIRE(S.self == T->self && S.mixed_ready && S.nxpairs == 0, "batch: target sets not prepared");
            W[m].tgt_off[ts] = tgt_off[m] = nt;
            pair_off[m] = np;
            ent_off[m] = ne;
            nt += S.nt;
            np += S.nvpairs;
            ne += S.near32_entries;
            T->nv_list += S.nv_list;
            T->nx_list += S.nx_list;
            T->near_pairs += S.near_pairs;
            T->nchunks_tc += S.nchunks_tc;
            T->nchunks_oz += S.nchunks_oz;
            T->ntleaves += S.ntleaves;
            T->near32_atomic = T->near32_atomic || S.near32_atomic;
            T->nearff_atomic = T->nearff_atomic || S.nearff_atomic;
        }
        IBIM_REQUIRE(np < INT_MAX && ne < INT_MAX && nt < INT_MAX, "batch: wave too large for 32-bit indices");
        T->nt = nt;
        T->nvpairs = np;
        T->near32_entries = (int)ne;
        if (!T->self) {
            DevBuf<double> TargetSet::*t3[3] = {&TargetSet::tx, &TargetSet::ty, &TargetSet::tz};
            for (auto f : t3)
                cat_buf((*T).*f, M, [&](int m) { return (S_(m).*f).ptr; }, [&](int m) { return (size_t)S_(m).nt; }, s);
            DevBuf<float> TargetSet::*t6[6] = {&TargetSet::txf, &TargetSet::tyf, &TargetSet::tzf,
                                                &TargetSet::txl, &TargetSet::tyl, &TargetSet::tzl};
            for (auto f : t6)
                cat_buf((*T).*f, M, [&](int m) { return (S_(m).*f).ptr; }, [&](int m) { return (size_t)S_(m).nt; }, s);
        }
        auto add_tgt = [&](int m) { return make_int4((int)tgt_off[m], 0, 0, 0); };
        cat_shift(T->tbeg, M, 1, 0, [&](int m) { return S_(m).tbeg.ptr; }, nodes, add_tgt, sms, s);
        cat_shift(T->tend, M, 1, 0, [&](int m) { return S_(m).tend.ptr; }, nodes, add_tgt, sms, s);
        T->l2l_level_begin = cat_levels(
            T->l2l_nodes, M, nlev, [&](int m) { return S_(m).l2l_nodes.ptr; },
            [&](int m) { return S_(m).l2l_level_begin.data(); }, [&](int m) { return P_(m).tree.nlevels; }, node_off,
            sms, s);
        auto npair = [&](int m) { return (long)S_(m).nvpairs; };
        cat_shift(T->v_src, M, 1, 0, [&](int m) { return S_(m).v_src.ptr; }, npair, add_node, sms, s);
        cat_shift(T->v_tgt, M, 1, 0, [&](int m) { return S_(m).v_tgt.ptr; }, npair, add_node, sms, s);
        auto add_chunk = [&](int m) { return make_int4(0, (int)pair_off[m], 0, 0); };  // own operator ids
        cat_shift(T->v_chunk_tc, M, 3, 0, [&](int m) { return S_(m).v_chunk_tc.ptr; },
                  [&](int m) { return (long)S_(m).nchunks_tc; }, add_chunk, sms, s);
        cat_shift(T->v_chunk_oz, M, 3, 0, [&](int m) { return S_(m).v_chunk_oz.ptr; },
                  [&](int m) { return (long)S_(m).nchunks_oz; }, add_chunk, sms, s);
        cat_shift(T->tleaf, M, 1, 0, [&](int m) { return S_(m).tleaf.ptr; },
                  [&](int m) { return (long)S_(m).ntleaves; }, add_node, sms, s);
        auto add_rng = [&](int m) { return make_int4((int)W[m].src_off, (int)W[m].src_off, 0, 0); };
        cat_shift(T->near32_range, M, 2, 0, [&](int m) { return S_(m).near32_range.ptr; },
                  [&](int m) { return (long)S_(m).near32_entries; }, add_rng, sms, s);
        cat_buf(T->near32_off, M, [&](int m) { return S_(m).near32_off.ptr; },
                [&](int m) { return 3 * (size_t)S_(m).near32_entries; }, s);
        cat_buf(T->near32_offl, M, [&](int m) { return S_(m).near32_offl.ptr; },
                [&](int m) { return 3 * (size_t)S_(m).near32_entries; }, s);
        merge_segments(T->near32_seg, mols, ts, W, ent_off, [](const TargetSet &S) -> const DevBuf<int> & { return S.near32_seg; },
                       [](const TargetSet &S) { return S.nnear32_seg; }, s);
        merge_segments(T->nearff_seg, mols, ts, W, ent_off, [](const TargetSet &S) -> const DevBuf<int> & { return S.nearff_seg; },
                       [](const TargetSet &S) { return S.nnearff_seg; }, s);
        T->nnear32_seg = 0;
        T->nnearff_seg = 0;
        for (int m = 0; m < M; ++m) {
            T->nnear32_seg += S_(m).nnear32_seg;
            T->nnearff_seg += S_(m).nnearff_seg;
        }
        T->out4.alloc((size_t)4 * std::max<long>(1, nt), s);
        T->mixed_ready = true;
        // the molecule of each chunk (the heavy kernels skip molecules that stopped iterating)
        std::vector<int> cm_tc, cm_oz;
        for (int m = 0; m < M; ++m) {
            cm_tc.insert(cm_tc.end(), S_(m).nchunks_tc, m);
            cm_oz.insert(cm_oz.end(), S_(m).nchunks_oz, m);
        }
        if (cm_tc.empty()) cm_tc.push_back(0);
        if (cm_oz.empty()) cm_oz.push_back(0);
        T->chunk_mol_tc.alloc(cm_tc.size(), s);
        T->chunk_mol_tc.upload(cm_tc.data(), cm_tc.size());
        T->chunk_mol_oz.alloc(cm_oz.size(), s);
        T->chunk_mol_oz.upload(cm_oz.data(), cm_oz.size());
    }
    std::vector<int> ones(M, 1);
    B->mol_active.alloc(M, s);
    B->mol_active.upload(ones.data(), M);
    B->tune = tuning_for(B->p, ns);
    IBIM_CUDA(cudaStreamSynchronize(s));
    return B.release();
}

// ---------------------------------------------------------------------------------------------
// lock-step GMRES
// ---------------------------------------------------------------------------------------------

// gmres.cpp:23-43
void gen_rot(double dx, double dy, double &cs, double &sn) {
    if (dy == 0.0) {
        cs = 1.0;
        sn = 0.0;
    } else if (std::fabs(dy) > std::fabs(dx)) {
        const double t = dx / dy;
        sn = 1.0 / std::sqrt(1.0 + t * t);
        cs = t * sn;
    } else {
        const double t = dy / dx;
        cs = 1.0 / std::sqrt(1.0 + t * t);
        sn = t * cs;
    }
}
void apply_rot(double &dx, double &dy, double cs, double sn) {
    const double t = cs * dx + sn * dy;
    dy = -sn * dx + cs * dy;
    dx = t;
}

using Op = std::function<void(const double *, double *)>;

// Restarted GMRES(m) of every molecule of a merged plan at once.  Vectors are [phi (n); psi (n)]
// over the merged sources; molecule k owns sources [off[k], off[k] + len[k]).
struct Lockstep {
    Ctx *c;
    long n, n2;
    int mr, M, ldh, ldy;
    std::vector<long> off, len;
    std::vector<int> nblk;
    DevBuf<long> doff, dlen;
    DevBuf<int> dnblk, dact;  // three lists of molecules (regions of M)
    DevBuf<double> V, w, r, part, hcol, ydev;
    double *hpin = nullptr;   // hcol (M x ldh), then y (M x ldy)
    int *apin = nullptr;      // the three lists
    int act_n[3] = {0, 0, 0}, act_maxb[3] = {0, 0, 0};
    long merged_matvecs = 0;
    double active_sum = 0;    // molecules active over all merged matvecs (waste = 1 - sum / (M * matvecs))

    Lockstep(Ctx *c_, long n_, int mr_, const std::vector<long> &off_, const std::vector<long> &len_)
        : c(c_), n(n_), n2(2 * n_), mr(mr_), M((int)off_.size()), off(off_), len(len_) {
        cudaStream_t s = c->stream;
        ldh = mr + 2;
        ldy = mr + 1;
        nblk.resize(M);
        // reduction blocks per molecule, from its size only (the sums' order does not depend on the batch)
        for (int k = 0; k < M; ++k)
            nblk[k] = (int)std::min<long>(BMAXB, std::max<long>(1, (2 * len[k] + 64L * BT - 1) / (64L * BT)));
        doff.alloc(M, s);
        doff.upload(off.data(), M);
        dlen.alloc(M, s);
        dlen.upload(len.data(), M);
        dnblk.alloc(M, s);
        dnblk.upload(nblk.data(), M);
        dact.alloc(3 * (size_t)M, s);
        V.alloc((size_t)(mr + 1) * n2, s);
        V.zero();
        w.alloc(n2, s);
        r.alloc(n2, s);
        part.alloc(2 * (size_t)M * BMAXB, s);
        hcol.alloc((size_t)M * ldh, s);
        ydev.alloc((size_t)M * ldy, s);
        IBIM_CUDA(cudaMallocHost((void **)&hpin, sizeof(double) * M * (ldh + ldy)));
        IBIM_CUDA(cudaMallocHost((void **)&apin, sizeof(int) * 3 * M));
        IBIM_CUDA(cudaMallocHost((void **)&mpin, sizeof(int) * M));
        mask_of.resize(M);
        for (int k = 0; k < M; ++k) mask_of[k] = k;  // the merged plan starts with every molecule on
        IBIM_CUDA(cudaStreamSynchronize(s));
    }
    ~Lockstep() {
        if (hpin) cudaFreeHost(hpin);
        if (apin) cudaFreeHost(apin);
        if (mpin) cudaFreeHost(mpin);
    }
    Segs segs(int region) const { return {doff.ptr, dlen.ptr, dnblk.ptr, dact.ptr + (size_t)region * M, n}; }
    // a list of molecules into a region (after the stream's earlier copies from the pinned lists)
    void set_act(int region, const std::vector<int> &a) {
        sync();
        int mb = 1;
        for (size_t k = 0; k < a.size(); ++k) {
            apin[region * M + k] = a[k];
            mb = std::max(mb, nblk[a[k]]);
        }
        act_n[region] = (int)a.size();
        act_maxb[region] = mb;
        if (!a.empty())
            IBIM_CUDA(cudaMemcpyAsync(dact.ptr + (size_t)region * M, apin + region * M, sizeof(int) * a.size(),
                                      cudaMemcpyHostToDevice, c->stream));
    }
    dim3 grid(int region) const { return dim3(act_maxb[region], act_n[region]); }
    void sync() { IBIM_CUDA(cudaStreamSynchronize(c->stream)); }

    // ||v|| of the molecules of region 0; the partials of <v, v> stay in part[0..) for the next
    // k_bnormalize
    void norms(const double *v, std::vector<double> &out) {
        if (act_n[0] == 0) return;
        (count_launch(), k_bdot<<<grid(0), BT, 0, c->stream>>>(segs(0), v, v, part.ptr));
        (count_launch(), k_bnorm<<<dim3(1, act_n[0]), BT, 0, c->stream>>>(segs(0), part.ptr, hcol.ptr, ldh, 0));
        IBIM_CHECK_LAUNCH();
        IBIM_CUDA(cudaMemcpyAsync(hpin, hcol.ptr, sizeof(double) * M * ldh, cudaMemcpyDeviceToHost, c->stream));
        sync();
        for (int k = 0; k < act_n[0]; ++k) {
            const int m = apin[k];
            out[m] = hpin[(size_t)m * ldh];
        }
    }
    // the merged plan's molecule mask follows the molecules whose products are used
    Plan *plan = nullptr;
    std::vector<int> mask_of;  // the list the device mask was last set from
    int *mpin = nullptr;       // pinned mask (M)
    void set_mask(const std::vector<int> &act) {
        if (!plan || act == mask_of) return;
        sync();  // the previous mask copy has been read
        for (int k = 0; k < M; ++k) mpin[k] = 0;
        for (int m : act) mpin[m] = 1;
        IBIM_CUDA(cudaMemcpyAsync(plan->mol_active.ptr, mpin, sizeof(int) * M, cudaMemcpyHostToDevice, c->stream));
        mask_of = act;
    }
    void matvec(const Op &A, const double *in, double *o, const std::vector<int> &act) {
        set_mask(act);
        A(in, o);
        merged_matvecs++;
        active_sum += (double)act.size();
    }

    // x (zero on entry for the listed molecules) += the GMRES solution of A d = b per molecule.
    void solve(const Op &A, double *x, const double *b, std::vector<int> act, const std::vector<double> &tol,
               const std::vector<int> &maxit, std::vector<int> &iters, std::vector<int> &mvs, std::vector<int> &status,
               std::vector<double> &resid) {
        cudaStream_t s = c->stream;
        std::vector<double> normb(M, 1.0), beta(M, 0.0);
        set_act(0, act);
        if (act.empty()) return;
        (count_launch(), k_bcopy<<<grid(0), BT, 0, s>>>(segs(0), b, r.ptr));
        IBIM_CHECK_LAUNCH();
        norms(r.ptr, beta);  // x = 0: r = b
        std::vector<std::vector<double>> H(M), sv(M), cs(M), sn(M);
        auto leave = [&](std::vector<int> &from, const std::vector<int> &gone) {
            std::vector<int> keep;
            for (int m : from)
                if (std::find(gone.begin(), gone.end(), m) == gone.end()) keep.push_back(m);
            from.swap(keep);
        };
        {
            std::vector<int> done;
            for (int m : act) {
                normb[m] = beta[m] == 0.0 ? 1.0 : beta[m];
                resid[m] = beta[m] / normb[m];
                if (resid[m] <= tol[m]) {
                    status[m] = 0;
                    done.push_back(m);
                }
                H[m].assign((size_t)(mr + 1) * (mr + 1), 0.);
                sv[m].assign(mr + 1, 0.);
                cs[m].assign(mr + 1, 0.);
                sn[m].assign(mr + 1, 0.);
            }
            leave(act, done);
        }
        // x += V y for a group of molecules, y from back substitution over their first k columns
        // (gmres.cpp:9-21)
        auto update = [&](const std::vector<int> &grp, int k) {
            if (grp.empty() || k <= 0) return;
            for (int m : grp) {
                double *y = hpin + (size_t)M * ldh + (size_t)m * ldy;
                auto Hm = [&](int i, int j) { return H[m][(size_t)i * (mr + 1) + j]; };
                for (int q = 0; q < k; ++q) y[q] = sv[m][q];
                for (int q = k - 1; q >= 0; --q) {
                    y[q] /= Hm(q, q);
                    for (int l = q - 1; l >= 0; --l) y[l] -= Hm(l, q) * y[q];
                }
            }
            IBIM_CUDA(cudaMemcpyAsync(ydev.ptr, hpin + (size_t)M * ldh, sizeof(double) * M * ldy,
                                      cudaMemcpyHostToDevice, s));
            set_act(1, grp);
            (count_launch(), k_bupdate<<<grid(1), BT, 0, s>>>(segs(1), k, ydev.ptr, ldy, V.ptr, n2, x));
            IBIM_CHECK_LAUNCH();
            sync();  // the pinned y rows and list are reused
        };
        int j = 1;
        while (!act.empty()) {
            {
                std::vector<int> ex;
                for (int m : act)
                    if (j > maxit[m]) ex.push_back(m);
                leave(act, ex);  // out of iterations: not converged (status stays 1)
            }
            if (act.empty()) break;
            set_act(0, act);
            // v0 = r / beta from the partials of <r, r>
            (count_launch(), k_bnormalize<<<grid(0), BT, 0, s>>>(segs(0), part.ptr, r.ptr, V.ptr, hcol.ptr, ldh, 0));
            IBIM_CHECK_LAUNCH();
            for (int m : act) {
                std::fill(sv[m].begin(), sv[m].end(), 0.);
                sv[m][0] = beta[m];
            }
            int i = 0;
            for (i = 0; i < mr && !act.empty(); i++, j++) {
                {
                    std::vector<int> ex;
                    for (int m : act)
                        if (j > maxit[m]) ex.push_back(m);
                    if (!ex.empty()) {
                        update(ex, i);
                        leave(act, ex);
                        set_act(0, act);
                        if (act.empty()) break;
                    }
                }
                double *vi = V.ptr + (size_t)i * n2;
                matvec(A, vi, w.ptr, act);
                for (int m : act) {
                    iters[m]++;
                    mvs[m]++;
                }
                double *pa = part.ptr, *pb = part.ptr + (size_t)M * BMAXB;
                (count_launch(), k_bdot<<<grid(0), BT, 0, s>>>(segs(0), w.ptr, V.ptr, pa));
                for (int k = 1; k <= i + 1; ++k) {
                    const double *vnext = k <= i ? V.ptr + (size_t)k * n2 : nullptr;
                    (count_launch(), k_bmgs<<<grid(0), BT, 0, s>>>(segs(0), pa, w.ptr, V.ptr + (size_t)(k - 1) * n2,
                                                                   vnext, pb, hcol.ptr, ldh, k - 1));
                    std::swap(pa, pb);
                }
                (count_launch(), k_bnormalize<<<grid(0), BT, 0, s>>>(segs(0), pa, w.ptr, V.ptr + (size_t)(i + 1) * n2,
                                                                     hcol.ptr, ldh, i + 1));
                IBIM_CHECK_LAUNCH();
                IBIM_CUDA(cudaMemcpyAsync(hpin, hcol.ptr, sizeof(double) * M * ldh, cudaMemcpyDeviceToHost, s));
                sync();
                std::vector<int> conv;
                for (int m : act) {
                    auto Hm = [&](int a, int b_) -> double & { return H[m][(size_t)a * (mr + 1) + b_]; };
                    for (int k = 0; k <= i + 1; ++k) Hm(k, i) = hpin[(size_t)m * ldh + k];
                    for (int k = 0; k < i; ++k) apply_rot(Hm(k, i), Hm(k + 1, i), cs[m][k], sn[m][k]);
                    gen_rot(Hm(i, i), Hm(i + 1, i), cs[m][i], sn[m][i]);
                    apply_rot(Hm(i, i), Hm(i + 1, i), cs[m][i], sn[m][i]);
                    apply_rot(sv[m][i], sv[m][i + 1], cs[m][i], sn[m][i]);
                    resid[m] = std::fabs(sv[m][i + 1]) / normb[m];
                    if (resid[m] < tol[m]) conv.push_back(m);
                }
                if (!conv.empty()) {
                    update(conv, i + 1);
                    for (int m : conv) status[m] = 0;
                    leave(act, conv);
                    set_act(0, act);
                }
            }
            if (act.empty()) break;
            // restart: x += V y, then the true residual
            update(act, i);
            set_act(0, act);
            matvec(A, x, w.ptr, act);
            for (int m : act) mvs[m]++;
            (count_launch(), k_bsub<<<grid(0), BT, 0, s>>>(segs(0), b, w.ptr, r.ptr));
            IBIM_CHECK_LAUNCH();
            norms(r.ptr, beta);
            std::vector<int> conv;
            for (int m : act) {
                resid[m] = beta[m] / normb[m];
                if (resid[m] < tol[m]) {
                    status[m] = 0;
                    conv.push_back(m);
                }
            }
            leave(act, conv);
        }
    }
};

}  // namespace

// ---------------------------------------------------------------------------------------------
// one wave: merge, lock-step refinement, energy
// ---------------------------------------------------------------------------------------------

bool batch_compatible(const ibim_config &a, const ibim_config &b) {
    return a.precision == IBIM_PRECISION_MIXED && b.precision == IBIM_PRECISION_MIXED && a.h == b.h &&
           a.np == b.np && a.kp.dE == b.kp.dE && a.kp.dI == b.kp.dI && a.kp.tau == b.kp.tau &&
           a.kp.k3_scaled == b.kp.k3_scaled && a.restart == b.restart && a.jacobian == b.jacobian;
}

void batch_prepare(Ctx *c, const double *centers_host, const double *charges_host, const double *radii_host,
                   int natoms, const ibim_config &cfg, ibim_result &res, BatchMol &out,
                   const std::function<void(long)> *after_surface) {
    cudaStream_t s = c->stream;
    DevBuf<double> dc, dr;
    dc.alloc(3 * (size_t)natoms, s);
    dr.alloc(natoms, s);
    dc.upload(centers_host, 3 * (size_t)natoms);
    dr.upload(radii_host, natoms);
    std::unique_ptr<SolvePrep> prep(new SolvePrep());
    solve_prepare(c, dc.ptr, dr.ptr, centers_host, charges_host, natoms, cfg, res, nullptr, *prep, after_surface);
    Plan &P = *prep->P;
    for (TargetSet *ts : P.targets) prepare_mixed(P, *ts);
    std::unique_ptr<DevBuf<double>> b(new DevBuf<double>());
    b->alloc(2 * (size_t)P.ns, s);
    permute(c, P.ns, P.src_perm.ptr, prep->b_tube.ptr, b->ptr, false);
    permute(c, P.ns, P.src_perm.ptr, prep->b_tube.ptr + P.ns, b->ptr + P.ns, false);
    IBIM_CUDA(cudaStreamSynchronize(s));
    prep->b_tube.release();
    prep->a4.release();
    IBIM_CUDA(cudaStreamSynchronize(s));
    out.natoms = natoms;
    out.charges = charges_host;
    out.cfg = cfg;
    out.res = &res;
    out.bytes = (double)plan_bytes(P) + 2.0 * sizeof(double) * P.ns + 7.0 * sizeof(double) * prep->tube->n;
    out.prep = prep.release();
    out.b_tree = b.release();
}

void batch_wave(Ctx *c, std::vector<BatchMol> &mols, WaveStats &ws) {
    cudaStream_t s = c->stream;
    const int M = (int)mols.size();
    auto t0 = std::chrono::steady_clock::now();
    std::vector<Plan *> plans(M);
    std::vector<ibim_kernel_params> kps(M);
    for (int m = 0; m < M; ++m) {
        plans[m] = mols[m].prep->P;
        kps[m] = mols[m].cfg.kp;
    }
    const ibim_config &C0 = mols[0].cfg;
    Tube mtube;
    mtube.ctx = c;
    mtube.h = C0.h;
    std::vector<WaveMol> W;
    std::unique_ptr<Plan> B(merge_wave(c, &mtube, plans, kps, C0.kp, C0.h, W));
    mtube.n = B->ns;
    const long n = B->ns, n2 = 2 * n;
    // right-hand sides into the merged vector
    DevBuf<double> b, x, d, r, w;
    b.alloc(n2, s);
    x.alloc(n2, s);
    d.alloc(n2, s);
    r.alloc(n2, s);
    w.alloc(n2, s);
    x.zero();
    std::vector<long> off(M), len(M);
    for (int m = 0; m < M; ++m) {
        const long N = plans[m]->ns;
        off[m] = W[m].src_off;
        len[m] = N;
        dcopy(b.ptr + off[m], mols[m].b_tree->ptr, N, s);
        dcopy(b.ptr + n + off[m], mols[m].b_tree->ptr + N, N, s);
    }
    IBIM_CUDA(cudaStreamSynchronize(s));
    // the per-molecule plans are no longer needed: the merged plan owns their operator images
    for (int m = 0; m < M; ++m) {
        delete mols[m].prep;
        mols[m].prep = nullptr;
        delete mols[m].b_tree;
        mols[m].b_tree = nullptr;
    }
    auto t1 = std::chrono::steady_clock::now();
    ws.t_merge_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    Timer tm(s);
    const ibim_kernel_params kp = C0.kp;
    Op A32 = [&](const double *in, double *o) { bie_matvec(*B, kp, in, o, IBIM_PRECISION_MIXED); };
    Op A64 = [&](const double *in, double *o) { bie_matvec(*B, kp, in, o, IBIM_PRECISION_FP64_TC); };
    Lockstep L(c, n, std::max(1, std::min(C0.restart, 250)), off, len);
    L.plan = B.get();
    // FP64 iterative refinement of every molecule (electric_solve's mixed branch, in lock-step)
    std::vector<int> all(M);
    for (int m = 0; m < M; ++m) all[m] = m;
    std::vector<double> normb(M, 1.0), rel(M, 1.0), rn(M, 0.0);
    L.set_act(0, all);
    L.norms(b.ptr, normb);
    for (int m = 0; m < M; ++m)
        if (normb[m] == 0.0) normb[m] = 1.0;
    (count_launch(), k_bcopy<<<L.grid(0), BT, 0, s>>>(L.segs(0), b.ptr, r.ptr));
    IBIM_CHECK_LAUNCH();
    std::vector<int> iters(M, 0), mvs(M, 0), fp64(M, 0), outer_n(M, 0), left(M), gstatus(M, 1);
    for (int m = 0; m < M; ++m) left[m] = mols[m].cfg.maxiter;
    static const double factor = [] {
        const char *v = std::getenv("IBIM_IR_FACTOR");
        const double f = v ? std::atof(v) : 0.7;
        return f > 0.0 && f < 1.0 ? f : 0.7;
    }();
    std::vector<int> act = all;
    for (int outer = 0; outer < 8 && !act.empty(); ++outer) {
        IBIM_CUDA(cudaMemsetAsync(d.ptr, 0, sizeof(double) * n2, s));
        std::vector<double> tin(M, 0.5), res_in(M, 0.0);
        std::vector<int> it_in(M, 0), mv_in(M, 0), st_in(M, 1);
        for (int m : act) tin[m] = std::min(0.5, std::max(factor * mols[m].cfg.tol / rel[m], 3e-7));
        L.solve(A32, d.ptr, r.ptr, act, tin, left, it_in, mv_in, st_in, res_in);
        for (int m : act) {
            iters[m] += it_in[m];
            mvs[m] += mv_in[m];
            left[m] -= it_in[m];
            outer_n[m] = outer + 1;
        }
        L.set_act(0, act);
        (count_launch(), k_badd<<<L.grid(0), BT, 0, s>>>(L.segs(0), d.ptr, x.ptr));
        IBIM_CHECK_LAUNCH();
        L.matvec(A64, x.ptr, w.ptr, act);
        ws.merged_fp64++;
        for (int m : act) fp64[m]++;
        (count_launch(), k_bsub<<<L.grid(0), BT, 0, s>>>(L.segs(0), b.ptr, w.ptr, r.ptr));
        IBIM_CHECK_LAUNCH();
        L.norms(r.ptr, rn);
        std::vector<int> next;
        for (int m : act) {
            rel[m] = rn[m] / normb[m];
            if (rel[m] < mols[m].cfg.tol) gstatus[m] = 0;
            else if (left[m] > 0) next.push_back(m);
        }
        act.swap(next);
    }
    ws.merged_mixed = L.merged_matvecs - ws.merged_fp64;
    ws.active_frac = L.merged_matvecs ? L.active_sum / ((double)M * L.merged_matvecs) : 1.0;
    const double t_solve = tm.ms();
    if (m2l_tc_error(*B)) throw Error(IBIM_ERR_LIMIT, "tensor-core M2L: an MMA completion wait exceeded its bound");
    // polarizeMap + energy (electric.cpp:442-505) on the merged atom targets, every molecule on
    L.set_mask(all);
    Timer te(s);
    TargetSet &TA = *B->targets[1];
    bie_densities(*B, x.ptr, B->dens4.ptr);
    fmm_run(*B, 1, kp, B->dens4.ptr, TA.out4.ptr, IBIM_PRECISION_MIXED);
    std::vector<double> F(TA.nt);
    TA.out4.download(F.data(), TA.nt);
    IBIM_CUDA(cudaStreamSynchronize(s));
    const double t_energy = te.ms();
    ws.t_solve_ms = t_solve;
    ws.t_energy_ms = t_energy;
    L.sync();
    for (int m = 0; m < M; ++m) {
        ibim_result &R = *mols[m].res;
        const long o = W[m].tgt_off[1];
        std::vector<double> pot(mols[m].natoms, 0.);
        for (size_t q = 0; q < W[m].perm_atoms.size(); ++q) pot[W[m].perm_atoms[q]] = -F[o + q];
        double E = 0.;
        for (int a = 0; a < mols[m].natoms; ++a) E += pot[a] * mols[m].charges[a];
        R.energy = 0.5 * E;
        R.gmres_iters = iters[m];
        R.matvecs_fp64 = fp64[m];
        R.matvecs = mvs[m] + fp64[m];
        R.refinements = outer_n[m];
        R.residual = rel[m];
        R.gmres_status = gstatus[m];
        R.t_solve_ms = t_solve;
        R.t_energy_ms = t_energy;
    }
}

// ---------------------------------------------------------------------------------------------
// the whole batch: worker threads prepare molecules in order; waves merge and solve
// ---------------------------------------------------------------------------------------------

void batch_solve(Ctx *c, int nmol, const int *natoms, const double *centers, const double *charges,
                 const double *radii, const ibim_config *cfgs, int max_wave, int wave_slots, double budget,
                 int workers, ibim_result *results, int *statuses, double *done_ms, double *info) {
    const auto t_call = std::chrono::steady_clock::now();
    auto since_call = [&] {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_call).count();
    };
    IBIM_REQUIRE(nmol > 0 && natoms && centers && charges && radii && cfgs && results && statuses, "null argument");
    for (int i = 0; i < nmol; ++i) {
        check_config(cfgs[i]);
        IBIM_REQUIRE(natoms[i] > 0, "batch: every molecule needs at least one atom");
        IBIM_REQUIRE(cfgs[i].precision == IBIM_PRECISION_MIXED, "batch: the lock-step path is the mixed-precision path");
        IBIM_REQUIRE(batch_compatible(cfgs[i], cfgs[0]),
                     "batch: molecules must share h, fmm_np, eps, tau, k3_scaled, restart and jacobian "
                     "(kappa, geometry and tolerances may differ)");
    }
    IBIM_REQUIRE(m2l_tc_supported() && mixed_uses_tc() && m2l_tc_fp16_form() && near_ff_enabled() && ops_ff_enabled(),
                 "batch: needs the tensor-core mixed path (sm_103a, default switches)");
    max_wave = std::max(1, max_wave);
    wave_slots = std::max(1, std::min(wave_slots, 4));
    workers = std::max(1, std::min(workers, 16));
    if (budget <= 0) budget = 150e9;
    std::vector<long> aoff(nmol + 1, 0);
    for (int i = 0; i < nmol; ++i) aoff[i + 1] = aoff[i] + natoms[i];
    for (int i = 0; i < nmol; ++i) {
        statuses[i] = IBIM_OK;
        std::memset(&results[i], 0, sizeof(ibim_result));
        if (done_ms) done_ms[i] = 0.;
    }
    struct Job {
        BatchMol bm;
        double held = 0;   // bytes this molecule holds in the budget
        double est_fmm = 0;  // its FMM phase's admitted estimate
        bool fmm = false;  // past its level set (holds FMM-phase memory)
        bool ready = false, waiting = false;
        std::string err;
    };
    std::vector<Job> jobs(nmol);
    std::mutex mu;
    std::condition_variable cv;
    // admission: a molecule's level set is admitted by its grids' bytes, its FMM phase (once its
    // tube size is known) by an estimate from the point count, replaced by the prepared plan's
    // bytes; a phase is always admitted when nothing else holds memory of that phase
    int next = 0, held = 0, held_fmm = 0, nwaiting = 0;
    double held_bytes = 0, peak_bytes = 0;
    bool stop = false;
    const int device = c->device;
    auto can_take = [&] {
        return next < nmol && (held == 0 || held_bytes + estimate_levelset_bytes(cfgs[next]) <= budget);
    };
    // worker contexts: prepared plans keep buffers on their streams, so the contexts outlive them
    std::vector<ibim_ctx> wctx(workers, nullptr);
    std::vector<int> wrc(workers, IBIM_OK);
    std::vector<std::string> werr0(workers);
    for (int t = 0; t < workers; ++t) {
        wrc[t] = ibim_ctx_create(device, &wctx[t]);
        if (wrc[t] != IBIM_OK) werr0[t] = ibim_last_error();
    }
    auto destroy_workers = [&] {
        for (ibim_ctx w : wctx)
            if (w) ibim_ctx_destroy(w);
        set_current_ctx(c);
        IBIM_CUDA(cudaSetDevice(device));
    };
    auto worker = [&](int t) {
        ibim_ctx wc = wctx[t];
        for (;;) {
            int i;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || can_take() || next >= nmol; });
                if (stop || next >= nmol) break;
                i = next++;
                held++;
                jobs[i].held = estimate_levelset_bytes(cfgs[i]);
                held_bytes += jobs[i].held;
                peak_bytes = std::max(peak_bytes, held_bytes);
            }
            Job &J = jobs[i];
            int st = wrc[t];
            std::string err = werr0[t];
            const std::function<void(long)> admit = [&](long bytes) {
                const double need = (double)bytes;
                std::unique_lock<std::mutex> lk(mu);
                held_bytes -= J.held;  // the grids are gone
                J.held = 0;
                J.waiting = true;
                nwaiting++;
                cv.notify_all();
                cv.wait(lk, [&] { return stop || held_fmm == 0 || held_bytes + need <= budget; });
                nwaiting--;
                J.waiting = false;
                if (stop) throw Error(IBIM_ERR_INVALID_ARGUMENT, "batch: stopped");
                J.held = need;
                J.est_fmm = need;
                J.fmm = true;
                held_fmm++;
                held_bytes += need;
                peak_bytes = std::max(peak_bytes, held_bytes);
            };
            if (st == IBIM_OK) {
                Ctx *wctx_ = &wc->c;
                try {
                    IBIM_CUDA(cudaSetDevice(device));
                    set_current_ctx(wctx_);
                    batch_prepare(wctx_, centers + 3 * aoff[i], charges + aoff[i], radii + aoff[i], natoms[i],
                                  cfgs[i], results[i], J.bm, &admit);
                    J.bm.index = i;
                } catch (const Error &e) {
                    st = e.status;
                    err = e.what();
                } catch (const std::exception &e) {
                    st = IBIM_ERR_INVALID_ARGUMENT;
                    err = e.what();
                }
                if (st != IBIM_OK) {
                    delete J.bm.prep;
                    J.bm.prep = nullptr;
                    delete J.bm.b_tree;
                    J.bm.b_tree = nullptr;
                }
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                statuses[i] = st;
                J.err = err;
                if (st == IBIM_OK) {
                    held_bytes += J.bm.bytes - J.held;
                    J.held = J.bm.bytes;
                } else {
                    held_bytes -= J.held;
                    J.held = 0;
                    held--;
                    if (J.fmm) held_fmm--;
                    if (done_ms) done_ms[i] = since_call();
                }
                peak_bytes = std::max(peak_bytes, held_bytes);
                J.ready = true;
            }
            cv.notify_all();
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < workers; ++t) pool.emplace_back(worker, t);
    auto release_all = [&] {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        for (auto &t : pool) t.join();
        for (Job &J : jobs) {
            delete J.bm.prep;
            J.bm.prep = nullptr;
            delete J.bm.b_tree;
            J.bm.b_tree = nullptr;
        }
        destroy_workers();
    };
    int waves = 0, largest = 0;
    long merged_mixed = 0, merged_fp64 = 0;
    double active_w = 0, wave_ms = 0, bytes_actual = 0, bytes_est = 0;
    int done = 0;  // the next molecule not yet given to a wave
    // wave solvers: the caller's context and wave_slots - 1 more, each taking the next wave when
    // it is free, so that one wave's host synchronisations and launch gaps overlap another's work
    std::vector<ibim_ctx> sctx(std::max(0, wave_slots - 1), nullptr);
    for (auto &x : sctx)
        if (ibim_ctx_create(device, &x) != IBIM_OK) x = nullptr;
    std::exception_ptr solver_error;
    auto solver = [&](Ctx *sc) {
        try {
            for (;;) {
                std::vector<int> wave;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    // a wave: the next prepared molecules in order, up to max_wave; it starts when
                    // full, when nothing is left to prepare, or when a worker waits for memory
                    cv.wait(lk, [&] {
                        if (done >= nmol || solver_error) return true;
                        int e = done;
                        while (e < nmol && jobs[e].ready && e - done < max_wave) ++e;
                        if (e == done) return false;
                        if (e - done >= max_wave || e == nmol) return true;
                        return nwaiting > 0 || (next < nmol && !can_take());
                    });
                    if (done >= nmol || solver_error) break;
                    int e = done;
                    while (e < nmol && jobs[e].ready && (int)wave.size() < max_wave) {
                        if (statuses[e] == IBIM_OK) wave.push_back(e);
                        ++e;
                    }
                    done = e;
                }
                cv.notify_all();
                if (wave.empty()) continue;
                set_current_ctx(sc);
                IBIM_CUDA(cudaSetDevice(device));
                std::vector<BatchMol> bm(wave.size());
                double wave_bytes = 0, wb_act = 0, wb_est = 0;
                for (size_t k = 0; k < wave.size(); ++k) {
                    Job &J = jobs[wave[k]];
                    bm[k] = J.bm;
                    J.bm.prep = nullptr;
                    J.bm.b_tree = nullptr;
                    wave_bytes += J.held;
                    wb_act += J.bm.bytes;
                    wb_est += J.est_fmm;
                }
                WaveStats ws;
                int wst = IBIM_OK;
                std::string werr;
                try {
                    batch_wave(sc, bm, ws);
                } catch (const Error &e) {
                    wst = e.status;
                    werr = e.what();
                } catch (const std::exception &e) {
                    wst = IBIM_ERR_INVALID_ARGUMENT;
                    werr = e.what();
                }
                const double t_wave_done = since_call();
                for (auto &b : bm) {
                    delete b.prep;
                    delete b.b_tree;
                }
                {
                    std::lock_guard<std::mutex> lk(mu);
                    for (auto &b : bm) {
                        if (wst != IBIM_OK) {
                            statuses[b.index] = wst;
                            jobs[b.index].err = werr;
                        }
                        if (done_ms) done_ms[b.index] = t_wave_done;
                    }
                    waves++;
                    wave_ms += ws.t_merge_ms + ws.t_solve_ms + ws.t_energy_ms;
                    largest = std::max(largest, (int)wave.size());
                    merged_mixed += ws.merged_mixed;
                    merged_fp64 += ws.merged_fp64;
                    active_w += ws.active_frac * wave.size();
                    bytes_actual += wb_act;
                    bytes_est += wb_est;
                    held -= (int)wave.size();
                    held_fmm -= (int)wave.size();
                    held_bytes -= wave_bytes;
                    if (held == 0) held_bytes = 0;
                    for (int i : wave) jobs[i].held = 0;
                }
                cv.notify_all();
            }
        } catch (...) {
            std::lock_guard<std::mutex> lk(mu);
            if (!solver_error) solver_error = std::current_exception();
            cv.notify_all();
        }
    };
    std::vector<std::thread> solvers;
    for (ibim_ctx x : sctx)
        if (x) solvers.emplace_back(solver, &x->c);
    solver(c);
    for (auto &t : solvers) t.join();
    for (ibim_ctx x : sctx)
        if (x) ibim_ctx_destroy(x);
    set_current_ctx(c);
    if (solver_error) {
        release_all();
        std::rethrow_exception(solver_error);
    }
    release_all();
    std::string first_error;
    int first_status = IBIM_OK;
    for (int i = 0; i < nmol; ++i)
        if (statuses[i] != IBIM_OK && first_status == IBIM_OK) {
            first_status = statuses[i];
            first_error = "molecule " + std::to_string(i) + ": " + jobs[i].err;
        }
    if (first_status != IBIM_OK) set_last_error(first_error);
    if (info) {
        info[0] = waves;
        info[1] = largest;
        info[2] = peak_bytes;
        info[3] = (double)merged_mixed;
        info[4] = (double)merged_fp64;
        int ok = 0;
        for (int i = 0; i < nmol; ++i) ok += statuses[i] == IBIM_OK;
        info[5] = ok ? active_w / ok : 0.0;
        info[6] = wave_ms;
        info[7] = bytes_actual;
        info[8] = bytes_est;
    }
}

}  // namespace ibim

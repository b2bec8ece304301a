// Near field of the FP64-class matvec in float-float arithmetic on the FP32 pipes.
//
// GB300 runs FP32 at about 61 times its FP64 rate, so the 16 BIE kernels of the near field
// (electric.cpp:67-291, fused as in near_pair64) are evaluated with unevaluated sums of two
// floats (hi + lo, 48-bit significand; Dekker 1971, Knuth's two-sum, Shewchuk 1997 for the
// renormalisation): about 550 FP32 operations a pair instead of about 80 FP64 ones.  The
// exponential e^{-kappa r} is reduced by 1/64 steps against a table of e^{-j/64} and e^{-j}
// (split from the host's double exp) and finished by the degree-5 Taylor polynomial, whose
// truncation error at |f| <= 1/128 is below 4e-16; 1/sqrt(d2) is the FP32 estimate refined by
// one third-order (Halley-type) step evaluated in float-float.  Relative accuracy per pair is
// about 2^-44, the class of the sliced FP64 M2L it runs beside.
#include "internal.cuh"
#include "fmm_common.cuh"

namespace ibim {
namespace {

struct f2 {
    float h, l;
};

// exact a + b = s + e (Knuth)
__device__ __forceinline__ f2 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// exact a + b = s + e when |a| >= |b| (Dekker)
__device__ __forceinline__ f2 quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ f2 add(f2 a, f2 b) {
    const f2 s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ f2 neg(f2 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ f2 sub(f2 a, f2 b) { return add(a, neg(b)); }
__device__ __forceinline__ f2 addf(f2 a, float b) {
    const f2 s = two_sum(a.h, b);
    return quick_two_sum(s.h, __fadd_rn(s.l, a.l));
}
__device__ __forceinline__ f2 mul(f2 a, f2 b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
    return quick_two_sum(p, e);
}
__device__ __forceinline__ f2 sqr(f2 a) {
    const float p = __fmul_rn(a.h, a.h);
    const float e = __fmaf_rn(__fmul_rn(2.f, a.h), a.l, __fmaf_rn(a.h, a.h, -p));
    return quick_two_sum(p, e);
}
__device__ __forceinline__ f2 ld(const float2 v) { return {v.x, v.y}; }

// e^{-t}, t >= 0: t = k/64 + f with |f| <= 1/128, e^{-t} = e^{-(k>>6)} e^{-(k&63)/64} e^{-f}
// (tables E1, E0), e^{-f} = 1 - f + f^2/2 - f^3 (1/6 - f/24 + f^2/120); zero for t >= 64
// (e^{-64} < 2e-28 of the other terms).
__device__ __forceinline__ f2 exp_neg(f2 t, const float2 *E0, const float2 *E1) {
    const float kf = rintf(__fmul_rn(t.h, 64.f));
    if (!(kf < 4096.f)) return {0.f, 0.f};
    const int k = max(0, (int)kf);
    // t.h - k/64 is exact (Sterbenz: k/64 lies within a factor 2 of t.h for k >= 1)
    const f2 f = two_sum(__fsub_rn(t.h, __fmul_rn(kf, 0.015625f)), t.l);
    const float fh = f.h;
    const float c = __fmaf_rn(fh, __fmaf_rn(fh, 1.f / 120.f, -1.f / 24.f), 1.f / 6.f);
    const float u = __fmul_rn(__fmul_rn(__fmul_rn(fh, fh), fh), c);
    f2 a = two_sum(1.f, -fh);
    a = quick_two_sum(a.h, __fsub_rn(a.l, f.l));
    f2 v = sqr(f);
    v.h = __fmul_rn(v.h, 0.5f);
    v.l = __fmul_rn(v.l, 0.5f);
    a = add(a, v);
    a = addf(a, -u);
    return mul(mul(ld(E1[k >> 6]), ld(E0[k & 63])), a);
}

// Radial factors of the 16 kernels at squared distance d2 (radial64 in float-float): c1 (K1),
// c4 (K4), k2 (K2), hd and ho (K3: hd delta_ab + ho d_a d_b); false inside the cutoff r < tau h.
// kap: kappa in float-float and whether it is non-zero (the plan's, or the molecule's in a batch)
struct KapFF {
    f2 kappa, k2in;
    bool yukawa;
};

__device__ __forceinline__ KapFF kap_of(const KParamsFF &k) { return {ld(k.kappa), ld(k.k2in), k.yukawa != 0}; }

__device__ __forceinline__ bool radial_ff(const KParamsFF &k, const KapFF &kap, const float2 *E0, const float2 *E1,
                                          f2 d2, f2 &c1, f2 &c4, f2 &k2, f2 &hd, f2 &ho) {
    if (d2.h < k.vr2.x || (d2.h == k.vr2.x && d2.l < k.vr2.y)) return false;
    // 1/sqrt(d2): FP32 estimate y, then y (1 + e/2 + 3e^2/8) with e = 1 - d2 y^2 from exact products
    const float y = rsqrtf(d2.h);
    const float p = __fmul_rn(y, y), pe = __fmaf_rn(y, y, -p);
    const float zh = __fmul_rn(d2.h, p);
    const float ze = __fmaf_rn(d2.h, pe, __fmaf_rn(d2.l, p, __fmaf_rn(d2.h, p, -zh)));
    const float e = __fsub_rn(__fsub_rn(1.f, zh), ze);
    const f2 ir = quick_two_sum(y, __fmul_rn(y, __fmaf_rn(__fmul_rn(0.375f, e), e, __fmul_rn(0.5f, e))));
    const f2 r = mul(d2, ir), ir2 = sqr(ir), ir3 = mul(ir2, ir);
    f2 E = {1.f, 0.f}, t = {0.f, 0.f};
    if (kap.yukawa) {
        t = mul(kap.kappa, r);
        E = exp_neg(t, E0, E1);
    }
    const f2 et1 = mul(E, addf(t, 1.f));
    const f2 q3 = mul(ir3, ld(k.q4pi)), h3 = mul(ir3, ld(k.k3f));
    c1 = mul(addf(mul(ld(k.eps), et1), -1.f), q3);
    c4 = mul(addf(neg(mul(ld(k.ieps), et1)), 1.f), q3);
    k2 = mul(mul(addf(neg(E), 1.f), ir), ld(k.q4pi));
    hd = mul(addf(neg(et1), 1.f), h3);
    ho = mul(mul(addf(mul(E, addf(mul(addf(t, 3.f), t), 3.f)), -3.f), h3), ir2);
    return true;
}

// One source -> target update of the fused 4x4 block, the formulas of near_pair64
// (electric.cpp:67-291) in float-float; d = source - target.
__device__ __forceinline__ void pair_ff(const KParamsFF &k, const KapFF &kap, const float2 *E0, const float2 *E1, f2 dx,
                                        f2 dy, f2 dz, f2 m0, f2 m1, f2 m2, f2 psi, f2 acc[4]) {
    const f2 d2 = add(add(sqr(dx), sqr(dy)), sqr(dz));
    f2 c1, c4, k2, hd, ho;
    if (!radial_ff(k, kap, E0, E1, d2, c1, c4, k2, hd, ho)) {
        acc[0] = sub(acc[0], mul(kap.k2in, psi));
        return;
    }
    const f2 dm = add(add(mul(dx, m0), mul(dy, m1)), mul(dz, m2));
    acc[0] = add(acc[0], sub(mul(c1, dm), mul(k2, psi)));
    const f2 cm = sub(mul(ho, dm), mul(c4, psi));
    acc[1] = add(acc[1], add(mul(hd, m0), mul(dx, cm)));
    acc[2] = add(acc[2], add(mul(hd, m1), mul(dy, cm)));
    acc[3] = add(acc[3], add(mul(hd, m2), mul(dz, cm)));
}

__device__ __forceinline__ f2 split_d(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}

// Source records for one matvec, tree order, 4 float4 each: (x, y, z, m_x) high words,
// (x, y, z, m_x) low words, (m_y, m_z, psi, 0) high, (m_y, m_z, psi, 0) low; coordinates are
// relative to the source's leaf centre.
__global__ void k_pack_src_ff(long ns, const double *__restrict__ dens, const float *__restrict__ xh,
                              const float *__restrict__ yh, const float *__restrict__ zh, const float *__restrict__ xl,
                              const float *__restrict__ yl, const float *__restrict__ zl, float4 *rec) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ns; i += (long)gridDim.x * blockDim.x) {
        const f2 m0 = split_d(dens[i]), m1 = split_d(dens[ns + i]), m2 = split_d(dens[2 * ns + i]),
                 ps = split_d(dens[3 * ns + i]);
        rec[4 * i] = make_float4(xh[i], yh[i], zh[i], m0.h);
        rec[4 * i + 1] = make_float4(xl[i], yl[i], zl[i], m0.l);
        rec[4 * i + 2] = make_float4(m1.h, m2.h, ps.h, 0.f);
        rec[4 * i + 3] = make_float4(m1.l, m2.l, ps.l, 0.f);
    }
}

// Near field (U and W lists, source leaves in the target leaf's frame) of the FP64-class
// matvec, without the L2P.  Work segments (at most about 2^14 pairs) over the per-source-leaf
// ranges of the FP32 near lists; with a work counter the CTA takes segments until none is left, else it does segment
// blockIdx.x.  Threads = targets x source phases as in the FP32 kernel.
constexpr int NTF = 128, TILEF = 128;
// BATCH: a plan merged over several molecules (batch.cu); kappa and the inner K2 constant come from
// the target leaf's molecule (kmol: kappa hi, lo, k2in hi, lo per molecule).
template <bool BATCH>
__global__ void __launch_bounds__(NTF) k_near_ff(KParamsFF kp, const int4 *__restrict__ segs, int nseg, int *next,
                                                 const int *__restrict__ nrange, const float *__restrict__ noff,
                                                 const float *__restrict__ noffl, const int *__restrict__ tb_,
                                                 const int *__restrict__ te_, const float4 *__restrict__ rec,
                                                 const float *__restrict__ txh, const float *__restrict__ tyh,
                                                 const float *__restrict__ tzh, const float *__restrict__ txl,
                                                 const float *__restrict__ tyl, const float *__restrict__ tzl, long nt,
                                                 double *out, const float4 *__restrict__ kmol,
                                                 const int *__restrict__ node_mol, const int *__restrict__ mol_active) {
    __shared__ float S[14][TILEF];
    __shared__ double red[NTF][4];
    __shared__ float2 E0[64], E1[64];
    __shared__ int cur;
    if (threadIdx.x < 64) {
        E0[threadIdx.x] = kp.e0[threadIdx.x];
        E1[threadIdx.x] = kp.e1[threadIdx.x];
    }
    for (int it = 0;; ++it) {
        int si;
        if (next) {
            __syncthreads();  // every thread has read the previous segment number
            if (threadIdx.x == 0) cur = atomicAdd(next, 1);
            __syncthreads();
            si = cur;
            if (si >= nseg) break;
        } else {
            if (it > 0) break;
            si = blockIdx.x;
        }
        const int4 sg = segs[si];
        const int leaf = sg.x, r0 = sg.y, r1 = sg.z, mode = sg.w;
        const int tb = tb_[leaf], te = te_[leaf];
        KapFF kap = kap_of(kp);
        if (BATCH) {
            if (!mol_active[node_mol[leaf]]) continue;  // the molecule has stopped iterating
            const float4 km = kmol[node_mol[leaf]];
            kap = {{km.x, km.y}, {km.z, km.w}, km.x != 0.f};
        }
        __syncthreads();
        for (int t0 = tb; t0 < te; t0 += NTF) {
            const int nT = min(NTF, te - t0);
            const int nph = NTF / nT;
            const int my_t = threadIdx.x % nT, ph = threadIdx.x / nT;
            const bool active = ph < nph;
            f2 X = {0.f, 0.f}, Y = {0.f, 0.f}, Z = {0.f, 0.f};
            if (active) {
                X = {txh[t0 + my_t], txl[t0 + my_t]};
                Y = {tyh[t0 + my_t], tyl[t0 + my_t]};
                Z = {tzh[t0 + my_t], tzl[t0 + my_t]};
            }
            f2 acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            int rr = r0, pos = r1 > r0 ? nrange[2 * r0] : 0;
            while (rr < r1) {
                __syncthreads();
                int filled = 0;
                int lrr = rr, lpos = pos;
                while (lrr < r1 && filled < TILEF) {
                    const int e = nrange[2 * lrr + 1];
                    const int take = min(TILEF - filled, e - lpos);
                    const f2 ox = {noff[3 * lrr], noffl[3 * lrr]}, oy = {noff[3 * lrr + 1], noffl[3 * lrr + 1]},
                             oz = {noff[3 * lrr + 2], noffl[3 * lrr + 2]};
                    for (int q = threadIdx.x; q < take; q += blockDim.x) {
                        const long s = lpos + q;
                        const float4 A = __ldg(rec + 4 * s), B = __ldg(rec + 4 * s + 1), C = __ldg(rec + 4 * s + 2),
                                     D = __ldg(rec + 4 * s + 3);
                        const f2 x = add({A.x, B.x}, ox), y = add({A.y, B.y}, oy), z = add({A.z, B.z}, oz);
                        const int f = filled + q;
                        S[0][f] = x.h;
                        S[1][f] = x.l;
                        S[2][f] = y.h;
                        S[3][f] = y.l;
                        S[4][f] = z.h;
                        S[5][f] = z.l;
                        S[6][f] = A.w;
                        S[7][f] = B.w;
                        S[8][f] = C.x;
                        S[9][f] = D.x;
                        S[10][f] = C.y;
                        S[11][f] = D.y;
                        S[12][f] = C.z;
                        S[13][f] = D.z;
                    }
                    filled += take;
                    lpos += take;
                    if (lpos >= e) {
                        ++lrr;
                        if (lrr < r1) lpos = nrange[2 * lrr];
                    }
                }
                rr = lrr;
                pos = lpos;
                __syncthreads();
                if (active)
                    for (int q = ph; q < filled; q += nph)
                        pair_ff(kp, kap, E0, E1, sub({S[0][q], S[1][q]}, X), sub({S[2][q], S[3][q]}, Y),
                                sub({S[4][q], S[5][q]}, Z), {S[6][q], S[7][q]}, {S[8][q], S[9][q]},
                                {S[10][q], S[11][q]}, {S[12][q], S[13][q]}, acc);
            }
            __syncthreads();
            for (int o = 0; o < 4; ++o) red[threadIdx.x][o] = (double)acc[o].h + (double)acc[o].l;
            __syncthreads();
            if (threadIdx.x < nT) {
                for (int o = 0; o < 4; ++o) {
                    double f = 0.;
                    for (int q = 0; q < nph; ++q) f += red[threadIdx.x + q * nT][o];
                    double *dst = out + o * nt + t0 + threadIdx.x;
                    if (mode & 2) atomicAdd(dst, f);
                    else *dst = f;
                }
            }
            __syncthreads();
        }
    }
}

// M2L operators of the FP64-class paths in float-float (k_make_ops64's layout: column-major
// n4 x n4 per op, entry (row o R + ct, column in R + cs) = block entry (o, in) between target node
// ct and source node cs), written as (hi, lo) word pairs.  The per-op geometry (half-widths
// root / 2^level, lattice offset, Chebyshev nodes) is split once per block from FP64.
__global__ void __launch_bounds__(256) k_make_ops_ff(KParamsFF kp, const ChebTables *__restrict__ tab,
                                                     const int *__restrict__ keys, const double *__restrict__ root_r,
                                                     float2 *ops) {
    __shared__ float2 E0[64], E1[64];
    __shared__ f2 rt_s[3], rs_s[3], ch_s[MAXP];
    __shared__ float D_s[3];
    const int op = blockIdx.y;
    if (threadIdx.x < 64) {
        E0[threadIdx.x] = kp.e0[threadIdx.x];
        E1[threadIdx.x] = kp.e1[threadIdx.x];
    }
    if (threadIdx.x == 0) {
        const int lt = keys[5 * op], ls = keys[5 * op + 1];
        for (int a = 0; a < 3; ++a) {
            rt_s[a] = split_d(ldexp(root_r[a], -lt));
            rs_s[a] = split_d(ldexp(root_r[a], -ls));
            D_s[a] = (float)keys[5 * op + 2 + a];
        }
        for (int m = 0; m < tab->p; ++m) ch_s[m] = split_d(tab->cheb[m]);
    }
    __syncthreads();
    const int p = tab->p, R = tab->R, n4 = 4 * R;
    const long pair = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (pair >= (long)R * R) return;
    const int cs = (int)(pair / R), ct = (int)(pair % R);  // consecutive threads: consecutive rows
    const int ti[3] = {ct % p, (ct / p) % p, ct / (p * p)};
    const int si[3] = {cs % p, (cs / p) % p, cs / (p * p)};
    f2 d[3];
    for (int a = 0; a < 3; ++a)  // (D rt + rs cheb_s) - rt cheb_t, as op_geometry / k_make_ops64
        d[a] = sub(add(mul(rt_s[a], {D_s[a], 0.f}), mul(rs_s[a], ch_s[si[a]])), mul(rt_s[a], ch_s[ti[a]]));
    f2 b[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) b[q] = {0.f, 0.f};
    const f2 d2 = add(add(sqr(d[0]), sqr(d[1])), sqr(d[2]));
    f2 c1, c4, k2, hd, ho;
    if (radial_ff(kp, kap_of(kp), E0, E1, d2, c1, c4, k2, hd, ho)) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            b[a] = mul(d[a], c1);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const f2 v = mul(mul(ho, d[a]), d[c]);
                b[4 * (a + 1) + c] = a == c ? add(v, hd) : v;
            }
            b[4 * (a + 1) + 3] = neg(mul(d[a], c4));
        }
        b[3] = neg(k2);
    } else {
        b[3] = neg(ld(kp.k2in));
    }
    float2 *K = ops + (long)op * n4 * n4;
#pragma unroll
    for (int o = 0; o < 4; ++o)
#pragma unroll
        for (int in = 0; in < 4; ++in)
            K[(long)(in * R + cs) * n4 + (o * R + ct)] = make_float2(b[o * 4 + in].h, b[o * 4 + in].l);
}

float2 split_h(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

}  // namespace

KParamsFF make_kparams_ff(const KParams &k) {
    IBIM_REQUIRE(k.kappa >= 0., "kappa must be non-negative");
    KParamsFF f;
    f.kappa = split_h(k.kappa);
    f.eps = split_h(k.eps);
    f.ieps = split_h(k.ieps);
    f.k2in = split_h(k.k2in);
    f.q4pi = split_h(k.q4pi);
    f.vr2 = split_h(k.vr2);
    f.k3f = split_h(k.k3f);
    f.yukawa = k.kappa != 0.;
    for (int j = 0; j < 64; ++j) {
        f.e0[j] = split_h(std::exp(-j / 64.0));
        f.e1[j] = split_h(std::exp(-(double)j));
    }
    return f;
}

bool near_ff_enabled() {
    static const bool on = [] {
        const char *v = std::getenv("IBIM_NEAR_FF");
        return !(v && v[0] == '0');
    }();
    return on;
}

int near_ff_occupancy() {
    static const int occ = [] {
        int b = 0;
        IBIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_near_ff<false>, NTF, 0));
        return std::max(1, b);
    }();
    return occ;
}

void fmm_prepare_operators_ff(Plan &P, const ibim_kernel_params &kpp) {
    double key[5] = {kpp.kappa, kpp.dE, kpp.dI, kpp.tau, (double)kpp.k3_scaled};
    bool same = P.opsff_ready;
    for (int i = 0; i < 5; ++i) same = same && P.kpff[i] == key[i];
    if (same || P.nops == 0) return;
    cudaStream_t s = P.ctx->stream;
    const int R = P.R, n4 = 4 * R;
    P.opsff.alloc((size_t)P.nops * n4 * n4, s);
    const KParamsFF kff = make_kparams_ff(make_kparams(kpp, P.tube->h));
    dim3 g((unsigned)div_up((long)R * R, 256), P.nops);
    {
        ProfScope ps_(PROF_OPS);
        (count_launch(), k_make_ops_ff<<<g, 256, 0, s>>>(kff, P.tables.ptr, P.op_key.ptr, P.root_r.ptr, P.opsff.ptr));
    }
    IBIM_CHECK_LAUNCH();
    for (int i = 0; i < 5; ++i) P.kpff[i] = key[i];
    P.opsff_ready = true;
}

bool ops_ff_enabled() {
    static const bool on = [] {
        const char *v = std::getenv("IBIM_OPS_FF");
        return !(v && v[0] == '0');
    }();
    return on;
}

void near_ff_pack(Plan &P, const double *dens, cudaStream_t st) {
    if (P.src16.n < (size_t)4 * P.ns) P.src16.alloc((size_t)4 * std::max<long>(1, P.ns), st);
    const int grid = (int)std::max<long>(1, std::min<long>(8L * P.ctx->num_sms, div_up(P.ns, 256)));
    (count_launch(), k_pack_src_ff<<<grid, 256, 0, st>>>(P.ns, dens, P.sxf.ptr, P.syf.ptr, P.szf.ptr, P.sxl.ptr,
                                                         P.syl.ptr, P.szl.ptr, P.src16.ptr));
    IBIM_CHECK_LAUNCH();
}

void near_ff_run(Plan &P, const TargetSet &S, const KParamsFF &kp, double *out, cudaStream_t st, int grid, int *next) {
    if (S.nnearff_seg == 0) return;
    const float *xh = S.self ? P.sxf.ptr : S.txf.ptr, *yh = S.self ? P.syf.ptr : S.tyf.ptr,
                *zh = S.self ? P.szf.ptr : S.tzf.ptr;
    const float *xl = S.self ? P.sxl.ptr : S.txl.ptr, *yl = S.self ? P.syl.ptr : S.tyl.ptr,
                *zl = S.self ? P.szl.ptr : S.tzl.ptr;
    auto kern = P.batched ? k_near_ff<true> : k_near_ff<false>;
    (count_launch(), kern<<<grid, NTF, 0, st>>>(kp, reinterpret_cast<const int4 *>(S.nearff_seg.ptr), S.nnearff_seg,
                                                next, S.near32_range.ptr, S.near32_off.ptr, S.near32_offl.ptr,
                                                S.tbeg.ptr, S.tend.ptr, P.src16.ptr, xh, yh, zh, xl, yl, zl, S.nt, out,
                                                P.kmolff.ptr, P.node_mol.ptr, P.mol_active.ptr));
    IBIM_CHECK_LAUNCH();
}

}  // namespace ibim

// Mixed-precision FMM (sm_103a): the same tree, lists and Chebyshev approximation as the FP64
// path (fmm.cu), evaluated in FP32 for use inside FP64 iterative refinement.
//
//   coordinates  FP32, relative to the centre of the point's leaf (|x| <= leaf size), plus an
//                FP32 centre offset per (target leaf, source leaf) from an FP64 difference, so
//                that close pairs keep ~1e-7 relative accuracy
//   near field   FP32 pair kernel (rsqrt, exp on the SFU), per-tile sums added with Kahan
//                compensation
//   far field    P2M / M2M / L2L / L2P in FP32; V-list M2L as a batched FP32 contraction with
//                FP32 operators; X-list M2L on the fly in FP32
// Outputs are written as FP64 so the BIE combine and GMRES stay FP64.

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "fmm_common.cuh"

namespace ibim {

struct ChebTables32 {
    float cheb[MAXP];
    float tnode[MAXP][MAXP];
    float S[2][MAXP][MAXP];
    int p, R;
};

struct KParams32 {
    float kappa, eps, ieps, vr2, k2in, q4pi, k3f;
    float k2in_q, k3q;  // k2in / q4pi and k3f / q4pi: the near field's densities carry the 1 / (4 pi)
    float kappa_l2;     // -kappa log2(e): e^(-kappa r) = 2^(kappa_l2 r)
    float vr2_band;     // |d2 - vr2| below this: the cutoff is decided in FP64
    double vr2_64;      // the FP64 kernels' (tau h)^2
    float vr2_guard;    // vr2 + 2 vr2_band: every pair inside the cutoff or its band lies below
};

static KParams32 to32(const KParams &k) {
    return KParams32{(float)k.kappa,        (float)k.eps,  (float)k.ieps,
                     (float)(k.vr * k.vr),  (float)k.k2in, (float)k.q4pi,
                     (float)k.k3f,          (float)(k.k2in / k.q4pi), (float)(k.k3f / k.q4pi),
                     (float)(-k.kappa * 1.4426950408889634),
                     (float)(1e-4 * k.vr2), k.vr2, (float)(k.vr2 * (1.0 + 2e-4))};
}

namespace {


__device__ __forceinline__ void interp1f(const ChebTables32 &T, float x, float *out) {
    float Tk[MAXP];
    Tk[0] = 1.f;
    Tk[1] = x;
    for (int k = 2; k < T.p; ++k) Tk[k] = 2.f * x * Tk[k - 1] - Tk[k - 2];
    const float ip = 1.f / T.p;
    for (int m = 0; m < T.p; ++m) {
        float s = 0.f;
        for (int k = 0; k < T.p; ++k) s = fmaf(Tk[k], T.tnode[m][k], s);
        out[m] = (-1.f + 2.f * s) * ip;
    }
}

template <class TT>
__device__ __forceinline__ void load_tables(TT &T, const TT *__restrict__ g) {
    const int n = sizeof(TT) / 4;
    for (int t = threadIdx.x; t < n; t += blockDim.x) reinterpret_cast<int *>(&T)[t] = reinterpret_cast<const int *>(g)[t];
}

// Coordinates relative to the leaf centre, rounded to FP32 (xf) with the rounding error as a
// second FP32 word (xl: the float-float low word).
__global__ void k_rel_coords(int nleaf, const int *__restrict__ leaves, const int *__restrict__ b_,
                             const int *__restrict__ e_, const double *__restrict__ ctr, const double *__restrict__ x,
                             const double *__restrict__ y, const double *__restrict__ z, float *xf, float *yf,
                             float *zf, float *xl, float *yl, float *zl) {
    const int L = blockIdx.x < nleaf ? leaves[blockIdx.x] : -1;
    if (L < 0) return;
    const double cx = ctr[3 * L], cy = ctr[3 * L + 1], cz = ctr[3 * L + 2];
    for (int i = b_[L] + threadIdx.x; i < e_[L]; i += blockDim.x) {
        const double dx = x[i] - cx, dy = y[i] - cy, dz = z[i] - cz;
        xf[i] = (float)dx;
        yf[i] = (float)dy;
        zf[i] = (float)dz;
        xl[i] = (float)(dx - (double)xf[i]);
        yl[i] = (float)(dy - (double)yf[i]);
        zl[i] = (float)(dz - (double)zf[i]);
    }
}

__global__ void k_to_f32(long n, const double *__restrict__ a, float *b) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

// Densities to FP32: [4][ns] for P2M, and per source the near-field record
// {x, y, z, m_x | m_y, m_z, psi, 0} (leaf-relative coordinates) as two float4.
// Densities to FP32 (for P2M) and the near field's source records, whose densities carry the
// kernels' common factor q = 1 / (4 pi): {x, y, z, q m_x}, {q m_y, q m_z, q psi, 0}.
__global__ void k_pack_src32(long ns, const double *__restrict__ dens, const float *__restrict__ sx,
                             const float *__restrict__ sy, const float *__restrict__ sz, float *d32, float4 *src8,
                             double q) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ns; i += (long)gridDim.x * blockDim.x) {
        const double m0 = dens[i], m1 = dens[ns + i], m2 = dens[2 * ns + i], psi = dens[3 * ns + i];
        d32[i] = (float)m0;
        d32[ns + i] = (float)m1;
        d32[2 * ns + i] = (float)m2;
        d32[3 * ns + i] = (float)psi;
        src8[2 * i] = make_float4(sx[i], sy[i], sz[i], (float)(q * m0));
        src8[2 * i + 1] = make_float4((float)(q * m1), (float)(q * m2), (float)(q * psi), 0.f);
    }
}

// P2M in FP32 (bbfmm.h:507-519); coordinates relative to the leaf centre.
__global__ void __launch_bounds__(128) k_p2m32(const ChebTables32 *__restrict__ tab, const int *__restrict__ nodes,
                                               const int *__restrict__ sb, const int *__restrict__ se,
                                               const float *__restrict__ rad, const float *__restrict__ x,
                                               const float *__restrict__ y, const float *__restrict__ z,
                                               const float *__restrict__ dens, long ns, float *mult) {
    __shared__ ChebTables32 T;
    __shared__ float Sp[32][3][MAXP];
    __shared__ float D[4][32];
    load_tables(T, tab);
    const int node = nodes[blockIdx.x];
    const int b = sb[node], e = se[node];
    const float ir[3] = {1.f / rad[3 * node], 1.f / rad[3 * node + 1], 1.f / rad[3 * node + 2]};
    __syncthreads();
    const int p = T.p, R = T.R;
    float acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.f;
    for (int base = b; base < e; base += 32) {
        const int cnt = min(32, e - base);
        if (threadIdx.x < 96) {
            const int pt = threadIdx.x / 3, ax = threadIdx.x % 3;
            if (pt < cnt) {
                const float *X = ax == 0 ? x : (ax == 1 ? y : z);
                interp1f(T, X[base + pt] * ir[ax], Sp[pt][ax]);
            }
        } else {
            const int pt = threadIdx.x - 96;
            if (pt < cnt)
                for (int d = 0; d < 4; ++d) D[d][pt] = dens[d * ns + base + pt];
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int o = threadIdx.x + 128 * q;
            if (o < 4 * R) {
                const int d = o / R, cc = o % R;
                const int i = cc % p, j = (cc / p) % p, l = cc / (p * p);
                float s = acc[q];
                for (int pt = 0; pt < cnt; ++pt) s = fmaf(Sp[pt][0][i] * Sp[pt][1][j] * Sp[pt][2][l], D[d][pt], s);
                acc[q] = s;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int o = threadIdx.x + 128 * q;
        if (o < 4 * R) mult[(long)node * 4 * R + o] = acc[q];
    }
}

__device__ void kron_apply32(const ChebTables32 &T, int id, bool up, float *buf, float *tmp) {
    const int p = T.p, R = T.R;
    const int b[3] = {id & 1, (id >> 1) & 1, (id >> 2) & 1};
    for (int ax = 0; ax < 3; ++ax) {
        const int stride = ax == 0 ? 1 : (ax == 1 ? p : p * p);
        float *src = (ax & 1) ? tmp : buf;
        float *dst = (ax & 1) ? buf : tmp;
        for (int o = threadIdx.x; o < 4 * R; o += blockDim.x) {
            const int d = o / R, cc = o % R;
            const int idx = (cc / stride) % p;
            const int base = d * R + cc - idx * stride;
            float s = 0.f;
            for (int k = 0; k < p; ++k) s = fmaf(up ? T.S[b[ax]][k][idx] : T.S[b[ax]][idx][k], src[base + k * stride], s);
            dst[o] = s;
        }
        __syncthreads();
    }
}

// One warp's separable transfer (the 3 passes of kron_apply32) on its own buffers.
__device__ void kron_apply32_warp(const ChebTables32 &T, int id, bool up, float *buf, float *tmp) {
    const int p = T.p, R = T.R, lane = threadIdx.x & 31;
    const int b[3] = {id & 1, (id >> 1) & 1, (id >> 2) & 1};
    for (int ax = 0; ax < 3; ++ax) {
        const int stride = ax == 0 ? 1 : (ax == 1 ? p : p * p);
        float *src = (ax & 1) ? tmp : buf;
        float *dst = (ax & 1) ? buf : tmp;
        for (int o = lane; o < 4 * R; o += 32) {
            const int d = o / R, cc = o % R;
            const int idx = (cc / stride) % p;
            const int base = d * R + cc - idx * stride;
            float s = 0.f;
            for (int k = 0; k < p; ++k) s = fmaf(up ? T.S[b[ax]][k][idx] : T.S[b[ax]][idx][k], src[base + k * stride], s);
            dst[o] = s;
        }
        __syncwarp();
    }
}

// M2M in FP32 (bbfmm.h:521-533): one parent per block, warp c transfers child c (its three
// separable passes need no block barrier), then the block sums the eight results.
constexpr int M2M32_THREADS = 256;
__global__ void __launch_bounds__(M2M32_THREADS) k_m2m32(const ChebTables32 *__restrict__ tab,
                                                         const int *__restrict__ nodes,
                                                         const int *__restrict__ child_first,
                                                         const int *__restrict__ empty, float *mult) {
    extern __shared__ float smf[];  // [8 children][2][4R]
    __shared__ ChebTables32 T;
    load_tables(T, tab);
    __syncthreads();
    const int n4 = 4 * T.R;
    const int node = nodes[blockIdx.x];
    const int c8 = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ch = child_first[node] + c8;
    float *buf = smf + (size_t)c8 * 2 * n4, *tmp = buf + n4;
    // after three passes the result is in tmp (odd pass count)
    if (empty[ch]) {
        for (int o = lane; o < n4; o += 32) tmp[o] = 0.f;
    } else {
        for (int o = lane; o < n4; o += 32) buf[o] = mult[(long)ch * n4 + o];
        __syncwarp();
        kron_apply32_warp(T, c8, true, buf, tmp);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < n4; o += blockDim.x) {
        float a = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c) a += smf[(size_t)c * 2 * n4 + n4 + o];
        mult[(long)node * n4 + o] = a;
    }
}

__global__ void __launch_bounds__(128) k_l2l32(const ChebTables32 *__restrict__ tab, const int *__restrict__ nodes,
                                               const int *__restrict__ parent, const int *__restrict__ index8,
                                               float *local) {
    extern __shared__ float smf[];
    __shared__ ChebTables32 T;
    load_tables(T, tab);
    __syncthreads();
    const int n4 = 4 * T.R;
    float *buf = smf, *tmp = smf + n4;
    const int node = nodes[blockIdx.x];
    const int par = parent[node];
    for (int o = threadIdx.x; o < n4; o += blockDim.x) buf[o] = local[(long)par * n4 + o];
    __syncthreads();
    kron_apply32(T, index8[node], false, buf, tmp);
    for (int o = threadIdx.x; o < n4; o += blockDim.x) local[(long)node * n4 + o] += tmp[o];
}

// FP32 M2L operators (V and X keys), evaluated in FP64 and rounded (same layout as the FP64
// operators).
__global__ void k_make_ops32(const ChebTables *__restrict__ tab, const int *__restrict__ keys,
                             const double *__restrict__ root_r, KParams kp, float *ops) {
    const ChebTables &T = *tab;
    const int op = blockIdx.y;
    const int p = T.p, R = T.R, n4 = 4 * R;
    const int lt = keys[5 * op], ls = keys[5 * op + 1];
    double rt[3], rs[3];
    for (int a = 0; a < 3; ++a) {
        double vt = root_r[a], vs = root_r[a];
        for (int l = 0; l < lt; ++l) vt *= 0.5;
        for (int l = 0; l < ls; ++l) vs *= 0.5;
        rt[a] = vt;
        rs[a] = vs;
    }
    // consecutive threads take consecutive target nodes ct: contiguous stores along a row
    const long pair = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (pair >= (long)R * R) return;
    const int cs = (int)(pair / R), ct = (int)(pair % R);
    const int ti[3] = {ct % p, (ct / p) % p, ct / (p * p)};
    const int si[3] = {cs % p, (cs / p) % p, cs / (p * p)};
    double d[3];
    for (int a = 0; a < 3; ++a)
        d[a] = (keys[5 * op + 2 + a] * rt[a] + rs[a] * T.cheb[si[a]]) - rt[a] * T.cheb[ti[a]];
    double b[16];
    kblock64(kp, d[0], d[1], d[2], b);
    float *K = ops + (long)op * n4 * n4;
    for (int o = 0; o < 4; ++o)
        for (int in = 0; in < 4; ++in) K[(long)(in * R + cs) * n4 + (o * R + ct)] = (float)b[o * 4 + in];
}

// V-list M2L in FP32 as a register-tiled SIMT contraction.  Block = (row tile of 128 of the 4R
// output rows, chunk of <= 32 pairs sharing one operator).  Per 32-column step the operator tile
// (32 x 128, contiguous rows) and the pairs' multipole tile (32 x 32) are staged in shared
// memory; each thread owns a 4 x 4 (rows x pairs) block of outputs; the next operator tile is
// prefetched into registers while the current one is consumed.
constexpr int GM_BM = 128, GM_BN = 32, GM_BK = 32;
__global__ void __launch_bounds__(256) k_m2l_v32(int n4, const int *__restrict__ chunks, const int *__restrict__ vsrc,
                                                 const int *__restrict__ vtgt, const float *__restrict__ ops,
                                                 const float *__restrict__ mult, float *local) {
    __shared__ __align__(16) float As[GM_BK][GM_BM];
    __shared__ __align__(16) float Bs[GM_BK][GM_BN];
    __shared__ int src_s[GM_BN], tgt_s[GM_BN];
    const int op = chunks[3 * blockIdx.x], b = chunks[3 * blockIdx.x + 1], cnt = chunks[3 * blockIdx.x + 2];
    const int row0 = blockIdx.y * GM_BM;
    const int tid = threadIdx.x;
    if (tid < GM_BN) {
        src_s[tid] = tid < cnt ? vsrc[b + tid] : -1;
        tgt_s[tid] = tid < cnt ? vtgt[b + tid] : -1;
    }
    const float *K = ops + (long)op * n4 * n4;
    const int tr = tid / 8, tc = tid % 8;  // rows tr*4.., pairs tc*4..
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    // operator tile loader: 32 columns x 128 rows = 1024 float4, 4 per thread
    float4 pre[4];
    auto load_a = [&](int k0) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int idx = tid + 256 * v;      // 0..1023
            const int col = idx / 32, r4 = (idx % 32) * 4;
            const int gr = row0 + r4, gc = k0 + col;
            float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gc < n4) {
                const float *src = K + (long)gc * n4 + gr;
                if (gr + 3 < n4) {
                    val = *reinterpret_cast<const float4 *>(src);
                } else {
                    if (gr < n4) val.x = src[0];
                    if (gr + 1 < n4) val.y = src[1];
                    if (gr + 2 < n4) val.z = src[2];
                }
            }
            pre[v] = val;
        }
    };
    __syncthreads();
    load_a(0);
    for (int k0 = 0; k0 < n4; k0 += GM_BK) {
        __syncthreads();
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int idx = tid + 256 * v;
            *reinterpret_cast<float4 *>(&As[idx / 32][(idx % 32) * 4]) = pre[v];
        }
        // multipole tile: Bs[col][pair] = mult[src_pair][k0 + col]
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int idx = tid + 256 * v;  // 0..1023
            const int j = idx / 32, col = idx % 32;
            const int sn = src_s[j];
            Bs[col][j] = (sn >= 0 && k0 + col < n4) ? mult[(long)sn * n4 + k0 + col] : 0.f;
        }
        __syncthreads();
        if (k0 + GM_BK < n4) load_a(k0 + GM_BK);
#pragma unroll 8
        for (int kk = 0; kk < GM_BK; ++kk) {
            const float4 a = *reinterpret_cast<const float4 *>(&As[kk][tr * 4]);
            const float4 bb = *reinterpret_cast<const float4 *>(&Bs[kk][tc * 4]);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {bb.x, bb.y, bb.z, bb.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int t = tgt_s[tc * 4 + j];
        if (t < 0) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int row = row0 + tr * 4 + i;
            if (row < n4) atomicAdd(local + (long)t * n4 + row, acc[i][j]);
        }
    }
}

// Fused 4x4 block in FP32 (same formulas as kblock64).
__device__ __forceinline__ void kblock32(const KParams32 &k, float dx, float dy, float dz, float b[16]) {
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < k.vr2) {
#pragma unroll
        for (int i = 0; i < 16; ++i) b[i] = 0.f;
        b[3] = -k.k2in;
        return;
    }
    const float ir = rsqrtf(d2), r = d2 * ir, ir2 = ir * ir, ir3 = ir2 * ir;
    const float t = k.kappa * r, e = __expf(-t), et1 = e * (t + 1.f);
    const float q3 = ir3 * k.q4pi, h3 = ir3 * k.k3f;
    const float c1 = (k.eps * et1 - 1.f) * q3;
    const float c4 = (1.f - k.ieps * et1) * q3;
    const float k2 = (1.f - e) * ir * k.q4pi;
    const float hd = (1.f - et1) * h3;
    const float ho = (e * ((t + 3.f) * t + 3.f) - 3.f) * h3 * ir2;
    const float dd[3] = {dx, dy, dz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        b[a] = dd[a] * c1;
#pragma unroll
        for (int c = 0; c < 3; ++c) b[4 * (a + 1) + c] = ho * dd[a] * dd[c] + (a == c ? hd : 0.f);
        b[4 * (a + 1) + 3] = -dd[a] * c4;
    }
    b[3] = -k2;
}

// X-list M2L in FP32, kernel on the fly; off = source centre - target centre.
__global__ void __launch_bounds__(128) k_m2l_x32(const ChebTables32 *__restrict__ tab, KParams32 kp,
                                                 const int *__restrict__ xsrc, const int *__restrict__ xtgt,
                                                 const float *__restrict__ off, const float *__restrict__ rad,
                                                 const float *__restrict__ mult, float *local) {
    __shared__ ChebTables32 T;
    __shared__ float M[4 * MAXR];
    __shared__ float sp[3][MAXP], tp[3][MAXP];
    load_tables(T, tab);
    __syncthreads();
    const int s = xsrc[blockIdx.x], t = xtgt[blockIdx.x];
    const int p = T.p, R = T.R;
    for (int o = threadIdx.x; o < 4 * R; o += blockDim.x) M[o] = mult[(long)s * 4 * R + o];
    if (threadIdx.x < 3 * p) {
        const int a = threadIdx.x / p, m = threadIdx.x % p;
        sp[a][m] = off[3 * blockIdx.x + a] + rad[3 * s + a] * T.cheb[m];
        tp[a][m] = rad[3 * t + a] * T.cheb[m];
    }
    __syncthreads();
    for (int ct = threadIdx.x; ct < R; ct += blockDim.x) {
        const float tx = tp[0][ct % p], ty = tp[1][(ct / p) % p], tz = tp[2][ct / (p * p)];
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int cs = 0; cs < R; ++cs) {
            float b[16];
            kblock32(kp, sp[0][cs % p] - tx, sp[1][(cs / p) % p] - ty, sp[2][cs / (p * p)] - tz, b);
#pragma unroll
            for (int o = 0; o < 4; ++o)
#pragma unroll
                for (int in = 0; in < 4; ++in) acc[o] = fmaf(b[o * 4 + in], M[in * R + cs], acc[o]);
        }
        for (int o = 0; o < 4; ++o) atomicAdd(local + (long)t * 4 * R + o * R + ct, acc[o]);
    }
}

// Hardware approximations with subnormal inputs and results flushed to zero (PTX rsqrt.approx.ftz,
// ex2.approx.ftz): one instruction each, where the non-flushing forms also handle subnormals.
// The near field's distances and exponentials never come near the subnormal range.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float exp2_ftz(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Near field + L2P in FP32 for one target leaf per block: source leaves staged in shared memory
// in the target leaf's frame (two 16-byte loads per source record); per-tile partial sums are
// added with Kahan compensation.
constexpr int NT32 = 128, TILE32 = 256;
// BATCH: a plan merged over several molecules (batch.cu); the kappa-dependent constants come from
// the target leaf's molecule (kmol: kappa, -kappa log2 e, k2in / q4pi per molecule).
template <bool BATCH>
__global__ void __launch_bounds__(NT32) k_near32(const ChebTables32 *__restrict__ tab, KParams32 kp,
                                                 const int4 *__restrict__ segs,
                                                 const int *__restrict__ nrange, const float *__restrict__ noff,
                                                 const int *__restrict__ tb_, const int *__restrict__ te_,
                                                 const float *__restrict__ rad, const float4 *__restrict__ src8,
                                                 const float *__restrict__ tx, const float *__restrict__ ty,
                                                 const float *__restrict__ tz, long nt,
                                                 const float *__restrict__ local, double *out, int l2p_mask,
                                                 int nseg, int *next, const double *__restrict__ sx64,
                                                 const double *__restrict__ sy64, const double *__restrict__ sz64,
                                                 const double *__restrict__ tx64, const double *__restrict__ ty64,
                                                 const double *__restrict__ tz64, const float4 *__restrict__ kmol,
                                                 const int *__restrict__ node_mol, const int *__restrict__ mol_active) {
    __shared__ ChebTables32 T;
    // {x, y, z, q m_x}, {q m_y, q m_z, q psi, source index} in the target leaf's frame
    __shared__ float4 S4[TILE32][2];
    __shared__ float red[NT32][4];
    __shared__ int cur;
    load_tables(T, tab);
    // with a work counter the CTA takes segments until none is left (several launches may drain
    // the same counter); without one it does segment blockIdx.x
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
        float kap = kp.kappa, kl2 = kp.kappa_l2, k2q = kp.k2in_q;
        if (BATCH) {
            if (!mol_active[node_mol[leaf]]) continue;  // the molecule has stopped iterating
            const float4 km = kmol[node_mol[leaf]];
            kap = km.x;
            kl2 = km.y;
            k2q = km.z;
        }
        __syncthreads();
        for (int t0 = tb; t0 < te; t0 += NT32) {
            const int nT = min(NT32, te - t0);
            const int nph = NT32 / nT;
            const int my_t = threadIdx.x % nT, ph = threadIdx.x / nT;
            const bool active = ph < nph;
            float X = 0.f, Y = 0.f, Z = 0.f;
            if (active) { X = tx[t0 + my_t]; Y = ty[t0 + my_t]; Z = tz[t0 + my_t]; }
            const long tg64 = active ? t0 + my_t : t0;  // the target's FP64 coordinates, for the cutoff
            float sum[4] = {0.f, 0.f, 0.f, 0.f}, cmp[4] = {0.f, 0.f, 0.f, 0.f};
            // fill tiles across consecutive source leaves
            int rr = r0, pos = r1 > r0 ? nrange[2 * r0] : 0;
            while (rr < r1) {
                __syncthreads();
                int filled = 0;
                // sequentially pack up to TILE32 sources; each thread copies its slots
                int lrr = rr, lpos = pos;
                while (lrr < r1 && filled < TILE32) {
                    const int e = nrange[2 * lrr + 1];
                    const int take = min(TILE32 - filled, e - lpos);
                    const float ox = noff[3 * lrr], oy = noff[3 * lrr + 1], oz = noff[3 * lrr + 2];
                    for (int q = threadIdx.x; q < take; q += blockDim.x) {
                        const int si = lpos + q;
                        const float4 A = __ldg(src8 + 2 * si), B = __ldg(src8 + 2 * si + 1);
                        S4[filled + q][0] = make_float4(A.x + ox, A.y + oy, A.z + oz, A.w);
                        S4[filled + q][1] = make_float4(B.x, B.y, B.z, __int_as_float(si));
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
                if (active) {
                    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
                    // the densities carry 1 / (4 pi): the K1, K2, K4 factors lose it and the K3 ones
                    // take k3f / q4pi (near_pair64 has the unscaled form)
                    for (int q = ph; q < filled; q += nph) {
                        const float4 P0 = S4[q][0], P1 = S4[q][1];
                        const float dx = P0.x - X, dy = P0.y - Y, dz = P0.z - Z;
                        // the cutoff test is a discontinuity: d2 in the FP64 kernel's evaluation order
                        // (near_pair64), so points at exactly tau h decide alike in both precisions
                        const float d2 = dx * dx + dy * dy + dz * dz;
                        if (d2 < kp.vr2_guard) {  // rare: inside the cutoff or within rounding of it
                            bool inside = d2 < kp.vr2;
                            if (fabsf(d2 - kp.vr2) < kp.vr2_band) {
                                // within FP32 rounding of the cutoff: decide on the FP64 coordinates,
                                // as the FP64 and float-float kernels do
                                const int sj = __float_as_int(P1.w);
                                const double ex = sx64[sj] - tx64[tg64], ey = sy64[sj] - ty64[tg64],
                                             ez = sz64[sj] - tz64[tg64];
                                inside = ex * ex + ey * ey + ez * ez < kp.vr2_64;
                            }
                            if (inside) {
                                a0 = fmaf(-k2q, P1.z, a0);
                                continue;
                            }
                        }
                        const float ir = rsqrt_ftz(d2), r = d2 * ir, ir2 = ir * ir, ir3 = ir2 * ir;
                        const float t = kap * r, e = exp2_ftz(kl2 * r), et1 = fmaf(e, t, e);
                        const float h3 = ir3 * kp.k3q;
                        const float c1 = fmaf(kp.eps, et1, -1.f) * ir3;
                        const float c4 = fmaf(-kp.ieps, et1, 1.f) * ir3;
                        const float k2 = (1.f - e) * ir;
                        const float hd = (1.f - et1) * h3;
                        const float ho = fmaf(e, fmaf(t + 3.f, t, 3.f), -3.f) * h3 * ir2;
                        const float dm = fmaf(dx, P0.w, fmaf(dy, P1.x, dz * P1.y));
                        a0 = fmaf(c1, dm, fmaf(-k2, P1.z, a0));
                        const float cm = fmaf(ho, dm, -c4 * P1.z);
                        a1 = fmaf(hd, P0.w, fmaf(dx, cm, a1));
                        a2 = fmaf(hd, P1.x, fmaf(dy, cm, a2));
                        a3 = fmaf(hd, P1.y, fmaf(dz, cm, a3));
                    }
                    const float part[4] = {a0, a1, a2, a3};
    #pragma unroll
                    for (int o = 0; o < 4; ++o) {  // Kahan: sum += part
                        const float yk = part[o] - cmp[o];
                        const float tk = sum[o] + yk;
                        cmp[o] = (tk - sum[o]) - yk;
                        sum[o] = tk;
                    }
                }
            }
            __syncthreads();
            for (int o = 0; o < 4; ++o) red[threadIdx.x][o] = sum[o] - cmp[o];
            __syncthreads();
            if (threadIdx.x < nT) {
                double f[4] = {0., 0., 0., 0.};
                for (int q = 0; q < nph; ++q)
                    for (int o = 0; o < 4; ++o) f[o] += (double)red[threadIdx.x + q * nT][o];
                float l2p[4] = {0.f, 0.f, 0.f, 0.f};
                if (mode & l2p_mask & 1) {  // L2P by the leaf's first segment
                    float Sp[3][MAXP];
                    const float xyz[3] = {X, Y, Z};
                    for (int a = 0; a < 3; ++a) interp1f(T, xyz[a] / rad[3 * leaf + a], Sp[a]);
                    const int p = T.p, R = T.R;
                    const float *L = local + (long)leaf * 4 * R;
                    for (int c = 0; c < R; ++c) {
                        const float w = Sp[0][c % p] * Sp[1][(c / p) % p] * Sp[2][c / (p * p)];
                        for (int o = 0; o < 4; ++o) l2p[o] = fmaf(w, L[o * R + c], l2p[o]);
                    }
                }
                for (int o = 0; o < 4; ++o) {
                    double *dst = out + o * nt + t0 + threadIdx.x;
                    if (mode & 2) atomicAdd(dst, f[o] + (double)l2p[o]);
                    else *dst = f[o] + (double)l2p[o];
                }
            }
            __syncthreads();
        }
    }
}

// L2P alone (downPass leaf, bbfmm.h:600), one target leaf per block, added to the near-field
// sums already in `out`: the form used when the near field runs beside the far field.
__global__ void __launch_bounds__(NT32) k_l2p32(const ChebTables32 *__restrict__ tab, const int *__restrict__ tleaf,
                                                const int *__restrict__ tb_, const int *__restrict__ te_,
                                                const float *__restrict__ rad, const float *__restrict__ tx,
                                                const float *__restrict__ ty, const float *__restrict__ tz, long nt,
                                                const float *__restrict__ local, double *out) {
    __shared__ ChebTables32 T;
    __shared__ float Ls[4 * MAXR];                 // the leaf's local expansion
    __shared__ float W[3][NT32][MAXP + 1];         // per-thread interpolation weights (odd stride)
    load_tables(T, tab);
    const int leaf = tleaf[blockIdx.x];
    const int tb = tb_[leaf], te = te_[leaf];
    __syncthreads();  // the tables are loaded
    const int p = T.p, R = p * p * p;
    for (int i = threadIdx.x; i < 4 * R; i += blockDim.x) Ls[i] = local[(long)leaf * 4 * R + i];
    __syncthreads();
    float *w0 = W[0][threadIdx.x], *w1 = W[1][threadIdx.x], *w2 = W[2][threadIdx.x];
    for (int t = tb + threadIdx.x; t < te; t += blockDim.x) {
        interp1f(T, tx[t] / rad[3 * leaf], w0);
        interp1f(T, ty[t] / rad[3 * leaf + 1], w1);
        interp1f(T, tz[t] / rad[3 * leaf + 2], w2);
        float l2p[4] = {0.f, 0.f, 0.f, 0.f};
        int c = 0;
        for (int c2 = 0; c2 < p; ++c2) {
            const float s2 = w2[c2];
            for (int c1 = 0; c1 < p; ++c1) {
                const float s1 = w1[c1];
                for (int c0 = 0; c0 < p; ++c0, ++c) {
                    const float w = w0[c0] * s1 * s2;
#pragma unroll
                    for (int o = 0; o < 4; ++o) l2p[o] = fmaf(w, Ls[o * R + c], l2p[o]);
                }
            }
        }
        for (int o = 0; o < 4; ++o) out[o * nt + t] += (double)l2p[o];
    }
}

inline int ew(Ctx *c, long n) { return (int)std::max<long>(1, std::min<long>(8L * c->num_sms, div_up(n, 256))); }

void up_i(DevBuf<int> &b, const std::vector<int> &v, cudaStream_t s) {
    b.alloc(std::max<size_t>(1, v.size()), s);
    b.upload(v.data(), v.size());
}
void up_f(DevBuf<float> &b, const std::vector<float> &v, cudaStream_t s) {
    b.alloc(std::max<size_t>(1, v.size()), s);
    b.upload(v.data(), v.size());
}

}  // namespace

// Host half of the FP32 near lists (no CUDA calls; safe while device work is queued).
void mixed_lists_host(const Plan &P, TargetSet &S) {
    if (S.mixed_host_ready || S.mixed_ready) return;
    const TreeHost &T = P.tree;
    const int nn = T.nnodes;
    // near lists: U and W nodes expanded into their non-empty leaves (depth first, child 0
    // first), with centre offsets.  The non-empty leaves below a node form one contiguous run of
    // the tree's depth-first leaf order, so each target leaf's list is a concatenation of runs.
    std::vector<int> child_first(nn, -1);
    for (int i = nn - 1; i >= 0; --i)
        if (T.parent[i] >= 0) child_first[T.parent[i]] = i - T.index8[i];
    std::vector<int> cnt(nn, 0), first(nn, 0);
    for (int i = nn - 1; i >= 0; --i) {  // nodes are level-ordered: children after parents
        if (T.leaf[i])
            cnt[i] = T.src_end[i] > T.src_begin[i] ? 1 : 0;
        else if (child_first[i] >= 0)
            for (int c = 0; c < 8; ++c) cnt[i] += cnt[child_first[i] + c];
    }
    for (int i = 0; i < nn; ++i) {
        if (T.leaf[i] || child_first[i] < 0) continue;
        int f = first[i];
        for (int c = 0; c < 8; ++c) {
            first[child_first[i] + c] = f;
            f += cnt[child_first[i] + c];
        }
    }
    std::vector<int> dfs_leaf(std::max(1, nn > 0 ? cnt[0] : 0));
    for (int i = 0; i < nn; ++i)
        if (T.leaf[i] && cnt[i]) dfs_leaf[first[i]] = i;
    std::vector<int> tl32, nt32;
    for (int i = 0; i < nn; ++i)
        if (T.leaf[i] && S.end[i] > S.begin[i]) {
            tl32.push_back(i);
            nt32.push_back((int)(S.end[i] - S.begin[i]));
        }
    const long ntl = (long)tl32.size();
    std::vector<int> ptr(ntl + 1, 0);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < ntl; ++k) {
        const int i = tl32[k];
        int c = 0;
        for (int u : T.U[i]) c += cnt[u];
        for (int w : T.W[i]) c += cnt[w];
        ptr[k + 1] = c;
    }
    for (long k = 0; k < ntl; ++k) ptr[k + 1] += ptr[k];
    const long nent = ptr[ntl];
    std::vector<int> rng(2 * nent);
    std::vector<float> off(3 * nent), offl(3 * nent);
#pragma omp parallel for schedule(dynamic, 64)
    for (long k = 0; k < ntl; ++k) {
        const int i = tl32[k];
        long q = ptr[k];
        auto add_run = [&](int root) {
            for (int r = first[root]; r < first[root] + cnt[root]; ++r, ++q) {
                const int n = dfs_leaf[r];
                rng[2 * q] = T.src_begin[n];
                rng[2 * q + 1] = T.src_end[n];
                for (int a = 0; a < 3; ++a) {
                    const double d = T.center[3 * n + a] - T.center[3 * i + a];
                    off[3 * q + a] = (float)d;
                    offl[3 * q + a] = (float)(d - (double)(float)d);
                }
            }
        };
        for (int u : T.U[i]) add_run(u);
        for (int w : T.W[i]) add_run(w);
    }
    S.near32_atomic = near_segments(tl32, nt32, ptr, rng, false, S.h_seg32, P.tune.near_seg_pairs);
    S.nnear32_seg = tl32.empty() ? 0 : (int)S.h_seg32.size() / 4;
    S.nearff_atomic = near_segments(tl32, nt32, ptr, rng, false, S.h_segff, P.tune.nearff_seg_pairs, 128);
    S.nnearff_seg = tl32.empty() ? 0 : (int)S.h_segff.size() / 4;
    S.h_ptr32.swap(ptr);
    S.h_rng32.swap(rng);
    S.h_off32.swap(off);
    S.h_offl32.swap(offl);
    S.mixed_host_ready = true;
    trace_mark("mixed: near lists");
}

// Leaf-relative FP32 coordinates (high and low words), FP32 tables, and the FP32 near and X
// lists of a target set.
void prepare_mixed(Plan &P, TargetSet &S) {
    cudaStream_t s = P.ctx->stream;
    const TreeHost &T = P.tree;
    const int nn = T.nnodes;
    if (!P.mixed_ready) {
        ChebTables h64;
        cheb_tables_host(P.p, h64);
        ChebTables32 h;
        std::memset(&h, 0, sizeof(h));
        h.p = h64.p;
        h.R = h64.R;
        for (int i = 0; i < MAXP; ++i) {
            h.cheb[i] = (float)h64.cheb[i];
            for (int j = 0; j < MAXP; ++j) {
                h.tnode[i][j] = (float)h64.tnode[i][j];
                h.S[0][i][j] = (float)h64.S[0][i][j];
                h.S[1][i][j] = (float)h64.S[1][i][j];
            }
        }
        P.tables32.alloc(sizeof(ChebTables32), s);
        P.tables32.upload(reinterpret_cast<unsigned char *>(&h), sizeof(h));
        std::vector<float> r32(3 * nn);
        for (int i = 0; i < 3 * nn; ++i) r32[i] = (float)T.radius[i];
        up_f(P.nrad32, r32, s);
        P.sxf.alloc(P.ns, s);
        P.syf.alloc(P.ns, s);
        P.szf.alloc(P.ns, s);
        P.sxl.alloc(P.ns, s);
        P.syl.alloc(P.ns, s);
        P.szl.alloc(P.ns, s);
        std::vector<int> leaves;
        for (int i = 0; i < nn; ++i)
            if (T.leaf[i] && T.src_end[i] > T.src_begin[i]) leaves.push_back(i);
        DevBuf<int> dl;
        up_i(dl, leaves, s);
        if (!leaves.empty())
            (count_launch(), k_rel_coords<<<(int)leaves.size(), 128, 0, s>>>((int)leaves.size(), dl.ptr, P.nsrc_begin.ptr,
                                                                       P.nsrc_end.ptr, P.ncenter.ptr, P.sx.ptr, P.sy.ptr,
                                                                       P.sz.ptr, P.sxf.ptr, P.syf.ptr, P.szf.ptr,
                                                                       P.sxl.ptr, P.syl.ptr, P.szl.ptr));
        IBIM_CHECK_LAUNCH();
        const int n4 = 4 * P.R;
        P.mult32.alloc((size_t)nn * n4, s);
        P.local32.alloc((size_t)nn * n4, s);
        P.dens32.alloc((size_t)4 * P.ns, s);
        P.src8.alloc((size_t)2 * P.ns, s);
        const size_t smk = sizeof(float) * 3 * n4, smk_m2m = sizeof(float) * 16 * n4;
        if (smk_m2m > 48 * 1024)
            IBIM_CUDA(cudaFuncSetAttribute(k_m2m32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smk_m2m));
        if (smk > 48 * 1024)
            IBIM_CUDA(cudaFuncSetAttribute(k_l2l32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smk));
        IBIM_CUDA(cudaStreamSynchronize(s));
        P.mixed_ready = true;
    }
    if (S.mixed_ready) return;
    trace_mark("mixed: plan data");
    // target coordinates relative to their leaf
    if (S.self) {
        // the source arrays are used
    } else {
        std::vector<int> leaves;
        for (int i = 0; i < nn; ++i)
            if (T.leaf[i] && S.end[i] > S.begin[i]) leaves.push_back(i);
        S.txf.alloc(std::max<long>(1, S.nt), s);
        S.tyf.alloc(std::max<long>(1, S.nt), s);
        S.tzf.alloc(std::max<long>(1, S.nt), s);
        S.txl.alloc(std::max<long>(1, S.nt), s);
        S.tyl.alloc(std::max<long>(1, S.nt), s);
        S.tzl.alloc(std::max<long>(1, S.nt), s);
        DevBuf<int> dl;
        up_i(dl, leaves, s);
        if (!leaves.empty())
            (count_launch(), k_rel_coords<<<(int)leaves.size(), 128, 0, s>>>((int)leaves.size(), dl.ptr, S.tbeg.ptr,
                                                                       S.tend.ptr, P.ncenter.ptr, S.tx.ptr, S.ty.ptr,
                                                                       S.tz.ptr, S.txf.ptr, S.tyf.ptr, S.tzf.ptr,
                                                                       S.txl.ptr, S.tyl.ptr, S.tzl.ptr));
        IBIM_CHECK_LAUNCH();
        IBIM_CUDA(cudaStreamSynchronize(s));
    }
    if (!S.mixed_host_ready) mixed_lists_host(P, S);
    up_i(S.near32_seg, S.h_seg32, s);
    up_i(S.nearff_seg, S.h_segff, s);
    up_i(S.near32_ptr, S.h_ptr32, s);
    up_i(S.near32_range, S.h_rng32, s);
    up_f(S.near32_off, S.h_off32, s);
    up_f(S.near32_offl, S.h_offl32, s);
    S.near32_entries = (int)S.h_rng32.size() / 2;
    // X pair centre offsets (FP64 difference, rounded)
    std::vector<int> xs(std::max<long>(1, S.nxpairs)), xt(std::max<long>(1, S.nxpairs));
    if (S.nxpairs > 0) {
        S.x_src.download(xs.data(), S.nxpairs);
        S.x_tgt.download(xt.data(), S.nxpairs);
        IBIM_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<float> xo(3 * std::max<long>(1, S.nxpairs));
    for (long q = 0; q < S.nxpairs; ++q)
        for (int a = 0; a < 3; ++a) xo[3 * q + a] = (float)(T.center[3 * xs[q] + a] - T.center[3 * xt[q] + a]);
    up_f(S.x_off32, xo, s);
    IBIM_CUDA(cudaStreamSynchronize(s));
    S.mixed_ready = true;
    // the host copies are no longer needed
    std::vector<int>().swap(S.h_ptr32);
    std::vector<int>().swap(S.h_rng32);
    std::vector<int>().swap(S.h_seg32);
    std::vector<int>().swap(S.h_segff);
    std::vector<float>().swap(S.h_off32);
    std::vector<float>().swap(S.h_offl32);
    trace_mark("mixed: segments, uploads");
}


void fmm_prepare_operators_mixed(Plan &P, const KParams &k, const double *ops64) {
    cudaStream_t s = P.ctx->stream;
    const int R = P.R, n4 = 4 * R;
    const long n = (long)P.nops * n4 * n4;
    P.ops32.alloc((size_t)n, s);
    ProfScope ps_(PROF_OPS);
    if (ops64) {  // the same kernel values rounded to FP32, as k_make_ops32 would compute them
        (count_launch(), k_to_f32<<<ew(P.ctx, n), 256, 0, s>>>(n, ops64, P.ops32.ptr));
    } else {
        dim3 g(div_up((long)R * R, 256), P.nops);
        (count_launch(), k_make_ops32<<<g, 256, 0, s>>>(P.tables.ptr, P.op_key.ptr, P.root_r.ptr, k, P.ops32.ptr));
    }
    IBIM_CHECK_LAUNCH();
}

bool mixed_uses_tc() {
    static const bool simt_m2l = std::getenv("IBIM_M2L_SIMT") != nullptr;  // SIMT FP32 M2L for comparison
    return !simt_m2l && m2l_tc_supported();
}

bool near_overlap() {
    static const bool on = [] {
        const char *v = std::getenv("IBIM_NEAR_OVERLAP");
        return !(v && v[0] == '0');
    }();
    return on;
}

int near_side_ctas() {
    static const int n = [] {
        const char *v = std::getenv("IBIM_NEAR_SIDE");
        return v ? std::max(0, std::atoi(v)) : 0;
    }();
    return n;
}

void fmm_run_mixed(Plan &P, int ts, const ibim_kernel_params &kpp, const double *dens, double *out) {
    IBIM_REQUIRE(ts >= 0 && ts < (int)P.targets.size(), "no such target set");
    TargetSet &S = *P.targets[ts];
    prepare_mixed(P, S);
    const bool tc = mixed_uses_tc();
    if (tc)
        fmm_ensure_tc_images(P, kpp);
    else
        fmm_prepare_operators(P, kpp, IBIM_PRECISION_MIXED);
    Ctx *c = P.ctx;
    cudaStream_t s = c->stream;
    const TreeHost &T = P.tree;
    const int R = P.R, n4 = 4 * R;
    const KParams kp = make_kparams(kpp, P.tube->h);
    const KParams32 k32 = to32(kp);
    const ChebTables32 *tab = reinterpret_cast<const ChebTables32 *>(P.tables32.ptr);
    (count_launch(), k_pack_src32<<<ew(c, P.ns), 256, 0, s>>>(P.ns, dens, P.sxf.ptr, P.syf.ptr, P.szf.ptr,
                                                               P.dens32.ptr, P.src8.ptr, kp.q4pi));
    const float *tx = S.self ? P.sxf.ptr : S.txf.ptr;
    const float *ty = S.self ? P.syf.ptr : S.tyf.ptr;
    const float *tz = S.self ? P.szf.ptr : S.tzf.ptr;
    const double *tx64 = S.self ? P.sx.ptr : S.tx.ptr;
    const double *ty64 = S.self ? P.sy.ptr : S.ty.ptr;
    const double *tz64 = S.self ? P.sz.ptr : S.tz.ptr;
    // near field (U and W lists): needs only the packed sources.  With the overlap on it starts on
    // the auxiliary stream at full occupancy, CTAs taking work segments from a counter, and fills
    // the SMs the latency-bound far-field launches (P2M, M2M levels) leave idle; the L2P follows
    // the join.  A smaller side launch (IBIM_NEAR_SIDE CTAs per SM) leaves the rest to a drain
    // launch after the far field
    auto near = [&](cudaStream_t st, int l2p_mask, int grid, int *next, double flops) {
        ProfScope ps_(PROF_NEAR, flops, flops > 0 ? 28.0 * P.ns + 40.0 * S.nt : 0., st);
        auto kern = P.batched ? k_near32<true> : k_near32<false>;
        (count_launch(), kern<<<grid, NT32, 0, st>>>(tab, k32, reinterpret_cast<const int4 *>(S.near32_seg.ptr),
                                                  S.near32_range.ptr, S.near32_off.ptr, S.tbeg.ptr, S.tend.ptr,
                                                  P.nrad32.ptr, P.src8.ptr, tx, ty, tz, S.nt, P.local32.ptr, out,
                                                  l2p_mask, S.nnear32_seg, next, P.sx.ptr, P.sy.ptr, P.sz.ptr,
                                                  tx64, ty64, tz64, P.kmol32.ptr, P.node_mol.ptr, P.mol_active.ptr));
    };
    const bool overlap = near_overlap() && S.ntleaves > 0;
    static const int occ = [] {
        int b = 0;
        IBIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_near32<false>, NT32, 0));
        return std::max(1, b);
    }();
    const int full = occ * c->num_sms, side = near_side_ctas() > 0 ? near_side_ctas() * c->num_sms : full;
    if (overlap) {
        if (!P.near_next.ptr) P.near_next.alloc(1, s);
        IBIM_CUDA(cudaMemsetAsync(P.near_next.ptr, 0, sizeof(int), s));
        if (S.near32_atomic) IBIM_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 4 * S.nt, s));
        IBIM_CUDA(cudaEventRecord(c->ev_near_fork, s));
        IBIM_CUDA(cudaStreamWaitEvent(c->aux, c->ev_near_fork, 0));
        near(c->aux, 0, std::min(S.nnear32_seg, side), P.near_next.ptr,
             70.0 * S.near_pairs);
        IBIM_CUDA(cudaEventRecord(c->ev_near_join, c->aux));
    }
    try {
        if (P.np2m > 0) {
            ProfScope ps_(PROF_P2M, (8.0 * R + 6.0 * P.p * P.p) * P.ns, 28.0 * P.ns);
            (count_launch(), k_p2m32<<<P.np2m, 128, 0, s>>>(tab, P.p2m_nodes.ptr, P.nsrc_begin.ptr, P.nsrc_end.ptr,
                                                            P.nrad32.ptr, P.sxf.ptr, P.syf.ptr, P.szf.ptr, P.dens32.ptr,
                                                            P.ns, P.mult32.ptr));
        }
        const size_t smk = sizeof(float) * 3 * n4, smk_m2m = sizeof(float) * 16 * n4;
        for (int l = T.nlevels - 1; l >= 0; --l) {
            const int b = P.m2m_level_begin[l], e = P.m2m_level_begin[l + 1];
            if (e > b) {
                ProfScope ps_(PROF_M2M);
                (count_launch(), k_m2m32<<<e - b, M2M32_THREADS, smk_m2m, s>>>(tab, P.m2m_nodes.ptr + b, P.nchild_first.ptr,
                                                                                P.nempty.ptr, P.mult32.ptr));
            }
        }
        P.local32.zero();
        if (tc) {
            m2l_tc_run(P, S);
        } else if (S.nchunks32 > 0) {
            ProfScope ps_(PROF_M2L_V, 2.0 * n4 * (double)n4 * S.nvpairs, 4.0 * n4 * (2.0 * S.nvpairs + (double)n4 * P.nops));
            const dim3 grid(S.nchunks32, div_up(n4, GM_BM));
            (count_launch(), k_m2l_v32<<<grid, 256, 0, s>>>(n4, S.v_chunk32.ptr, S.v_src.ptr, S.v_tgt.ptr, P.ops32.ptr,
                                                            P.mult32.ptr, P.local32.ptr));
        }
        if (S.nxpairs > 0) {
            ProfScope ps_(PROF_M2L_X, 102.0 * R * (double)R * S.nxpairs, 8.0 * n4 * S.nxpairs);
            (count_launch(), k_m2l_x32<<<(int)S.nxpairs, 128, 0, s>>>(tab, k32, S.x_src.ptr, S.x_tgt.ptr, S.x_off32.ptr,
                                                                      P.nrad32.ptr, P.mult32.ptr, P.local32.ptr));
        }
        for (int l = 3; l < T.nlevels; ++l) {
            const int b = S.l2l_level_begin[l], e = S.l2l_level_begin[l + 1];
            if (e > b) {
                ProfScope ps_(PROF_L2L);
                (count_launch(), k_l2l32<<<e - b, 128, smk, s>>>(tab, S.l2l_nodes.ptr + b, P.nparent.ptr, P.nindex8.ptr,
                                                                 P.local32.ptr));
            }
        }
    } catch (...) {
        if (overlap) cudaStreamSynchronize(c->aux);  // the near field still reads dens and writes out
        throw;
    }
    if (overlap) {
        if (side < std::min(S.nnear32_seg, full)) near(s, 0, std::min(S.nnear32_seg, full), P.near_next.ptr, 0.);
        IBIM_CUDA(cudaStreamWaitEvent(s, c->ev_near_join, 0));
        ProfScope ps_(PROF_L2P, (10.0 * R + 6.0 * P.p * P.p) * S.nt, 16.0 * n4 * S.ntleaves + 44.0 * S.nt);
        (count_launch(), k_l2p32<<<S.ntleaves, NT32, 0, s>>>(tab, S.tleaf.ptr, S.tbeg.ptr, S.tend.ptr, P.nrad32.ptr,
                                                             tx, ty, tz, S.nt, P.local32.ptr, out));
    } else if (S.ntleaves > 0) {
        if (S.near32_atomic) IBIM_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 4 * S.nt, s));
        near(s, 1, S.nnear32_seg, nullptr, 70.0 * S.near_pairs);
    }
    IBIM_CHECK_LAUNCH();
}

}  // namespace ibim

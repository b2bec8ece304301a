// Black-box Chebyshev FMM on the GPU (sm_103a), FP64 path.
//
// Replaces bbfmm::kernel (bbfmm.h:200-624) for the reference's BIE kernel set.  One pass
// computes the fused 4-density -> 4-field operator (the 16 scalar FMMs of one matvec,
// electric.cpp:333-367, share one tree and one set of Chebyshev operators, so their sum is
// one FMM with a 4x4 kernel block):
//   inputs  m_x, m_y, m_z = phi n w,  psi = dphi w        (electric.cpp:324-329)
//   outputs F   = K1 . m - K2 psi                           (-> out1, electric.cpp:382)
//           G_a = sum_b H_ab m_b - K4_a psi, H = K3 block   (-> n . G = tmp1 - tmp2, :372-383)
// Same approximation as the reference: Chebyshev order p, leaf P2M/L2P through the tensor
// interpolant S_p (bbfmm.h:392-433), M2M/L2L through the 8 Kronecker operators (:305-367),
// M2L for V and X lists with the kernel at Chebyshev node pairs (:547-561), direct U and W
// lists (:577-595).
//
// Data layout in HBM: points SoA in tree order (each node owns a contiguous range);
// multipole / local coefficients per node as [4][p^3] with index z*p^2 + y*p + x.
// V-list M2L: the kernel at Chebyshev node pairs depends only on (level, source - target
// lattice offset), so those (4p^3)^2 operators are built once per plan and applied as a
// batched dense contraction (pairs grouped by operator).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>
#include <tuple>

#include <omp.h>

#include "fmm_common.cuh"

namespace ibim {

// ----------------------------------------------------------------------------------------
// Tables
// ----------------------------------------------------------------------------------------

void cheb_tables_host(int p, ChebTables &T) {
    std::memset(&T, 0, sizeof(T));
    T.p = p;
    T.R = p * p * p;
    for (int i = 0; i < p; ++i) T.cheb[i] = -std::cos((i + 0.5) * M_PI / p);
    auto poly = [&](double x, double *out) {
        out[0] = 1.0;
        if (p > 1) out[1] = x;
        for (int k = 2; k < p; ++k) out[k] = 2.0 * x * out[k - 1] - out[k - 2];
    };
    for (int m = 0; m < p; ++m) poly(T.cheb[m], T.tnode[m]);
    // parent -> child transfer S[bit][child node][parent node] (bbfmm.h:305-326)
    for (int a = 0; a < 2 * p; ++a) {
        const double x = a < p ? 0.5 * T.cheb[a] - 0.5 : 0.5 * T.cheb[a - p] + 0.5;
        double tx[MAXP];
        poly(x, tx);
        for (int m = 0; m < p; ++m) {
            double s = 0.;
            for (int k = 0; k < p; ++k) s += tx[k] * T.tnode[m][k];
            T.S[a / p][a % p][m] = (-1.0 + 2.0 * s) * (1.0 / p);
        }
    }
}

// ----------------------------------------------------------------------------------------
// FP64 kernels
// ----------------------------------------------------------------------------------------

namespace {

// P2M (upPass leaf, bbfmm.h:507-519): mult[leaf][d][c] = sum_pts S(pt, c) dens[d][pt].
__global__ void __launch_bounds__(128) k_p2m64(const ChebTables *__restrict__ tab, const int *__restrict__ nodes,
                                               const int *__restrict__ sb, const int *__restrict__ se,
                                               const double *__restrict__ ctr, const double *__restrict__ rad,
                                               const double *__restrict__ x, const double *__restrict__ y,
                                               const double *__restrict__ z, const double *__restrict__ dens, long ns,
                                               double *mult) {
    __shared__ ChebTables T;
    __shared__ double Sp[32][3][MAXP];
    __shared__ double D[4][32];
    if (threadIdx.x < sizeof(ChebTables) / 8) reinterpret_cast<double *>(&T)[threadIdx.x] = reinterpret_cast<const double *>(tab)[threadIdx.x];
    for (int t = threadIdx.x + 128; t < (int)(sizeof(ChebTables) / 8); t += 128)
        reinterpret_cast<double *>(&T)[t] = reinterpret_cast<const double *>(tab)[t];
    const int node = nodes[blockIdx.x];
    const int b = sb[node], e = se[node];
    const double c[3] = {ctr[3 * node], ctr[3 * node + 1], ctr[3 * node + 2]};
    const double r[3] = {rad[3 * node], rad[3 * node + 1], rad[3 * node + 2]};
    __syncthreads();
    const int p = T.p, R = T.R;
    double acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.;
    for (int base = b; base < e; base += 32) {
        const int cnt = min(32, e - base);
        if (threadIdx.x < 96) {
            const int pt = threadIdx.x / 3, ax = threadIdx.x % 3;
            if (pt < cnt) {
                const double *X = ax == 0 ? x : (ax == 1 ? y : z);
                interp1(T, (X[base + pt] - c[ax]) / r[ax], Sp[pt][ax]);
            }
        } else if (threadIdx.x < 128) {
            const int pt = threadIdx.x - 96;
            if (pt < cnt)
                for (int d = 0; d < 4; ++d) D[d][pt] = dens[d * ns + base + pt];
        }
        __syncthreads();
        for (int q = 0; q < 16; ++q) {
            const int o = threadIdx.x + 128 * q;
            if (o >= 4 * R) break;
            const int d = o / R, cc = o % R;
            const int i = cc % p, j = (cc / p) % p, l = cc / (p * p);
            double s = acc[q];
            for (int pt = 0; pt < cnt; ++pt) s += Sp[pt][0][i] * Sp[pt][1][j] * Sp[pt][2][l] * D[d][pt];
            acc[q] = s;
        }
        __syncthreads();
    }
    for (int q = 0; q < 16; ++q) {
        const int o = threadIdx.x + 128 * q;
        if (o >= 4 * R) break;
        mult[(long)node * 4 * R + o] = acc[q];
    }
}

// One separable Kronecker transfer (R[id] = S[b2] (x) S[b1] (x) S[b0], bbfmm.h:345-366) on a
// [4][p^3] block in shared memory.  up = true: child -> parent (R^T), else parent -> child (R).
__device__ void kron_apply(const ChebTables &T, int id, bool up, double *buf, double *tmp, int nthreads) {
    const int p = T.p, R = T.R;
    const int b[3] = {id & 1, (id >> 1) & 1, (id >> 2) & 1};
    // axis 0 (x, stride 1), axis 1 (y, stride p), axis 2 (z, stride p^2)
    for (int ax = 0; ax < 3; ++ax) {
        const int stride = ax == 0 ? 1 : (ax == 1 ? p : p * p);
        double *src = (ax & 1) ? tmp : buf;
        double *dst = (ax & 1) ? buf : tmp;
        for (int o = threadIdx.x; o < 4 * R; o += nthreads) {
            const int d = o / R, cc = o % R;
            const int idx = (cc / stride) % p;
            const int base = d * R + cc - idx * stride;
            double s = 0.;
            for (int k = 0; k < p; ++k) {
                // up:   out[n] = sum_k S[b][k][n] in[k];   down: out[k] = sum_n S[b][k][n] in[n]
                const double w = up ? T.S[b[ax]][k][idx] : T.S[b[ax]][idx][k];
                s += w * src[base + k * stride];
            }
            dst[o] = s;
        }
        __syncthreads();
    }
    // after 3 passes the result is in tmp (passes wrote tmp, buf, tmp)
}

// M2M (upPass, bbfmm.h:530-534): parent = sum over non-empty children R[i]^T child.
__global__ void __launch_bounds__(128) k_m2m64(const ChebTables *__restrict__ tab, const int *__restrict__ nodes,
                                               const int *__restrict__ child_first, const int *__restrict__ empty,
                                               double *mult) {
    extern __shared__ double sm[];
    __shared__ ChebTables T;
    for (int t = threadIdx.x; t < (int)(sizeof(ChebTables) / 8); t += blockDim.x)
        reinterpret_cast<double *>(&T)[t] = reinterpret_cast<const double *>(tab)[t];
    __syncthreads();
    const int R = T.R, n4 = 4 * R;
    double *buf = sm, *tmp = sm + n4, *acc = sm + 2 * n4;
    const int node = nodes[blockIdx.x];
    for (int o = threadIdx.x; o < n4; o += blockDim.x) acc[o] = 0.;
    const int c0 = child_first[node];
    for (int c8 = 0; c8 < 8; ++c8) {
        const int ch = c0 + c8;
        if (empty[ch]) continue;
        __syncthreads();
        for (int o = threadIdx.x; o < n4; o += blockDim.x) buf[o] = mult[(long)ch * n4 + o];
        __syncthreads();
        kron_apply(T, c8, true, buf, tmp, blockDim.x);
        for (int o = threadIdx.x; o < n4; o += blockDim.x) acc[o] += tmp[o];
    }
    __syncthreads();
    for (int o = threadIdx.x; o < n4; o += blockDim.x) mult[(long)node * n4 + o] = acc[o];
}

// L2L (downPass, bbfmm.h:566-567): child += R[index8] parent.
__global__ void __launch_bounds__(128) k_l2l64(const ChebTables *__restrict__ tab, const int *__restrict__ nodes,
                                               const int *__restrict__ parent, const int *__restrict__ index8,
                                               double *local) {
    extern __shared__ double sm[];
    __shared__ ChebTables T;
    for (int t = threadIdx.x; t < (int)(sizeof(ChebTables) / 8); t += blockDim.x)
        reinterpret_cast<double *>(&T)[t] = reinterpret_cast<const double *>(tab)[t];
    __syncthreads();
    const int R = T.R, n4 = 4 * R;
    double *buf = sm, *tmp = sm + n4;
    const int node = nodes[blockIdx.x];
    const int par = parent[node];
    for (int o = threadIdx.x; o < n4; o += blockDim.x) buf[o] = local[(long)par * n4 + o];
    __syncthreads();
    kron_apply(T, index8[node], false, buf, tmp, blockDim.x);
    for (int o = threadIdx.x; o < n4; o += blockDim.x) local[(long)node * n4 + o] += tmp[o];
}

// Build the M2L operators: op (target level, source level, centre offset D in target half-widths)
// -> K[col * 4R + row], row = out * R + ct, col = in * R + cs,
// entry = block(src_cheb(cs) - tgt_cheb(ct))[out][in], node positions D r_t + r_s cheb - r_t cheb.
// V operators (same level, D = 2 o) and X operators (coarser source leaf) share the layout.
__device__ __forceinline__ void op_geometry(const int *keys, int op, const double *root_r, double rt[3], double rs[3],
                                            int D[3]) {
    const int lt = keys[5 * op], ls = keys[5 * op + 1];
    for (int a = 0; a < 3; ++a) {
        double vt = root_r[a], vs = root_r[a];
        for (int l = 0; l < lt; ++l) vt *= 0.5;
        for (int l = 0; l < ls; ++l) vs *= 0.5;
        rt[a] = vt;
        rs[a] = vs;
        D[a] = keys[5 * op + 2 + a];
    }
}

__global__ void k_make_ops64(const ChebTables *__restrict__ tab, const int *__restrict__ keys,
                             const double *__restrict__ root_r, KParams kp, double *ops) {
    const ChebTables &T = *tab;
    const int op = blockIdx.y;
    const int p = T.p, R = T.R, n4 = 4 * R;
    double rt[3], rs[3];
    int D[3];
    op_geometry(keys, op, root_r, rt, rs, D);
    // consecutive threads take consecutive target nodes ct, so each output row is written by
    // contiguous 8-byte stores
    const long pair = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (pair >= (long)R * R) return;
    const int cs = (int)(pair / R), ct = (int)(pair % R);
    const int ti[3] = {ct % p, (ct / p) % p, ct / (p * p)};
    const int si[3] = {cs % p, (cs / p) % p, cs / (p * p)};
    double d[3];
    for (int a = 0; a < 3; ++a) d[a] = (D[a] * rt[a] + rs[a] * T.cheb[si[a]]) - rt[a] * T.cheb[ti[a]];
    double b[16];
    kblock64(kp, d[0], d[1], d[2], b);
    double *K = ops + (long)op * n4 * n4;
    for (int o = 0; o < 4; ++o)
        for (int in = 0; in < 4; ++in) K[(long)(in * R + cs) * n4 + (o * R + ct)] = b[o * 4 + in];
}

// V-list M2L as a batched contraction: chunk = (op, first pair, count <= M2L_CH); every
// thread owns rows r = tid + 256 q of the 4R outputs for all pairs of the chunk.
constexpr int M2L_CH = 8;
__global__ void __launch_bounds__(256) k_m2l_v64(int n4, const int *__restrict__ chunks, const int *__restrict__ vsrc,
                                                 const int *__restrict__ vtgt, const double *__restrict__ ops,
                                                 const double *__restrict__ mult, double *local) {
    extern __shared__ double Ms[];  // [M2L_CH][n4]
    const int op = chunks[3 * blockIdx.x], b = chunks[3 * blockIdx.x + 1], cnt = chunks[3 * blockIdx.x + 2];
    for (int j = 0; j < cnt; ++j) {
        const double *src = mult + (long)vsrc[b + j] * n4;
        for (int o = threadIdx.x; o < n4; o += blockDim.x) Ms[j * n4 + o] = src[o];
    }
    __syncthreads();
    const double *K = ops + (long)op * n4 * n4;
    constexpr int MAXQ = 8;  // n4 <= 2048
    double acc[MAXQ][M2L_CH];
#pragma unroll
    for (int q = 0; q < MAXQ; ++q)
#pragma unroll
        for (int j = 0; j < M2L_CH; ++j) acc[q][j] = 0.;
    const int nq = (n4 + 255) / 256;
    for (int col = 0; col < n4; ++col) {
        const double *Kc = K + (long)col * n4;
#pragma unroll
        for (int q = 0; q < MAXQ; ++q) {
            if (q >= nq) break;
            const int row = threadIdx.x + 256 * q;
            const double a = row < n4 ? __ldg(Kc + row) : 0.;
#pragma unroll
            for (int j = 0; j < M2L_CH; ++j) acc[q][j] += a * Ms[j * n4 + col];
        }
    }
#pragma unroll
    for (int q = 0; q < MAXQ; ++q) {
        if (q >= nq) break;
        const int row = threadIdx.x + 256 * q;
        if (row >= n4) continue;
#pragma unroll
        for (int j = 0; j < M2L_CH; ++j)
            if (j < cnt) atomicAdd(local + (long)vtgt[b + j] * n4 + row, acc[q][j]);
    }
}

// X-list M2L (bbfmm.h:556-560): coarser leaf -> node, kernel evaluated on the fly.
__global__ void __launch_bounds__(128) k_m2l_x64(const ChebTables *__restrict__ tab, KParams kp,
                                                 const int *__restrict__ xsrc, const int *__restrict__ xtgt,
                                                 const double *__restrict__ ctr, const double *__restrict__ rad,
                                                 const double *__restrict__ mult, double *local) {
    __shared__ ChebTables T;
    __shared__ double M[4 * MAXR];
    __shared__ double sp[3][MAXP], tp[3][MAXP];
    for (int t = threadIdx.x; t < (int)(sizeof(ChebTables) / 8); t += blockDim.x)
        reinterpret_cast<double *>(&T)[t] = reinterpret_cast<const double *>(tab)[t];
    __syncthreads();
    const int s = xsrc[blockIdx.x], t = xtgt[blockIdx.x];
    const int p = T.p, R = T.R;
    for (int o = threadIdx.x; o < 4 * R; o += blockDim.x) M[o] = mult[(long)s * 4 * R + o];
    if (threadIdx.x < 3 * p) {
        const int a = threadIdx.x / p, m = threadIdx.x % p;
        sp[a][m] = ctr[3 * s + a] + rad[3 * s + a] * T.cheb[m];
        tp[a][m] = ctr[3 * t + a] + rad[3 * t + a] * T.cheb[m];
    }
    __syncthreads();
    for (int ct = threadIdx.x; ct < R; ct += blockDim.x) {
        const double tx = tp[0][ct % p], ty = tp[1][(ct / p) % p], tz = tp[2][ct / (p * p)];
        double acc[4] = {0., 0., 0., 0.};
        for (int cs = 0; cs < R; ++cs) {
            double b[16];
            kblock64(kp, sp[0][cs % p] - tx, sp[1][(cs / p) % p] - ty, sp[2][cs / (p * p)] - tz, b);
#pragma unroll
            for (int o = 0; o < 4; ++o)
#pragma unroll
                for (int in = 0; in < 4; ++in) acc[o] += b[o * 4 + in] * M[in * R + cs];
        }
        for (int o = 0; o < 4; ++o) atomicAdd(local + (long)t * 4 * R + o * R + ct, acc[o]);
    }
}

// Near field + L2P for one target leaf per block (downPass leaf, bbfmm.h:571-609): U and W
// lists direct (source ranges in tree order), then the local expansion at the targets.
// Threads = targets x source phases; sources staged in shared memory tiles.
constexpr int NEAR_T = 128, NEAR_TILE = 128;
__global__ void __launch_bounds__(NEAR_T) k_near64(const ChebTables *__restrict__ tab, KParams kp,
                                                   const int4 *__restrict__ segs,
                                                   const int *__restrict__ near_range, const int *__restrict__ tb_,
                                                   const int *__restrict__ te_, const double *__restrict__ ctr,
                                                   const double *__restrict__ rad, const double *__restrict__ sx,
                                                   const double *__restrict__ sy, const double *__restrict__ sz,
                                                   const double *__restrict__ dens, long ns,
                                                   const double *__restrict__ tx, const double *__restrict__ ty,
                                                   const double *__restrict__ tz, long nt,
                                                   const double *__restrict__ local, double *out, int l2p_mask,
                                                   int nseg, int *next) {
    __shared__ ChebTables T;
    __shared__ double S[7][NEAR_TILE];
    __shared__ double red[NEAR_T][4];
    __shared__ int cur;
    for (int t = threadIdx.x; t < (int)(sizeof(ChebTables) / 8); t += blockDim.x)
        reinterpret_cast<double *>(&T)[t] = reinterpret_cast<const double *>(tab)[t];
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
        __syncthreads();
        for (int t0 = tb; t0 < te; t0 += NEAR_T) {
            const int nT = min(NEAR_T, te - t0);
            const int nph = NEAR_T / nT;
            const int my_t = threadIdx.x % nT, ph = threadIdx.x / nT;
            const bool active = ph < nph;
            double X = 0, Y = 0, Z = 0;
            if (active) { X = tx[t0 + my_t]; Y = ty[t0 + my_t]; Z = tz[t0 + my_t]; }
            double acc[4] = {0., 0., 0., 0.};
            for (int rr = r0; rr < r1; ++rr) {
                const int b = near_range[2 * rr], e = near_range[2 * rr + 1];
                for (int s0 = b; s0 < e; s0 += NEAR_TILE) {
                    const int cnt = min(NEAR_TILE, e - s0);
                    __syncthreads();
                    for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
                        S[0][q] = sx[s0 + q];
                        S[1][q] = sy[s0 + q];
                        S[2][q] = sz[s0 + q];
                        S[3][q] = dens[s0 + q];
                        S[4][q] = dens[ns + s0 + q];
                        S[5][q] = dens[2 * ns + s0 + q];
                        S[6][q] = dens[3 * ns + s0 + q];
                    }
                    __syncthreads();
                    if (active)
                        for (int q = ph; q < cnt; q += nph)
                            near_pair64(kp, S[0][q] - X, S[1][q] - Y, S[2][q] - Z, S[3][q], S[4][q], S[5][q], S[6][q],
                                        acc);
                }
            }
            for (int o = 0; o < 4; ++o) red[threadIdx.x][o] = acc[o];
            __syncthreads();
            if (threadIdx.x < nT) {
                double f[4] = {0., 0., 0., 0.};
                for (int q = 0; q < nph; ++q)
                    for (int o = 0; o < 4; ++o) f[o] += red[threadIdx.x + q * nT][o];
                // L2P (bbfmm.h:600): local expansion at the target, by the leaf's first segment
                double l2p[4] = {0., 0., 0., 0.};
                if (mode & l2p_mask & 1) {
                    double Sp[3][MAXP];
                    const double xyz[3] = {X, Y, Z};
                    for (int a = 0; a < 3; ++a) interp1(T, (xyz[a] - ctr[3 * leaf + a]) / rad[3 * leaf + a], Sp[a]);
                    const int p = T.p, R = T.R;
                    const double *L = local + (long)leaf * 4 * R;
                    for (int c = 0; c < R; ++c) {
                        const double w = Sp[0][c % p] * Sp[1][(c / p) % p] * Sp[2][c / (p * p)];
                        for (int o = 0; o < 4; ++o) l2p[o] += w * L[o * R + c];
                    }
                }
                for (int o = 0; o < 4; ++o) {
                    double *dst = out + o * nt + t0 + threadIdx.x;
                    if (mode & 2) atomicAdd(dst, f[o] + l2p[o]);
                    else *dst = f[o] + l2p[o];
                }
            }
            __syncthreads();
        }
    }
}

// L2P alone (bbfmm.h:600), one target leaf per block, added to the near-field sums already in
// `out`: the form used when the near field runs beside the far field.
__global__ void __launch_bounds__(NEAR_T) k_l2p64(const ChebTables *__restrict__ tab, const int *__restrict__ tleaf,
                                                  const int *__restrict__ tb_, const int *__restrict__ te_,
                                                  const double *__restrict__ ctr, const double *__restrict__ rad,
                                                  const double *__restrict__ tx, const double *__restrict__ ty,
                                                  const double *__restrict__ tz, long nt,
                                                  const double *__restrict__ local, double *out) {
    __shared__ ChebTables T;
    __shared__ double Ls[4 * MAXR];                // the leaf's local expansion
    __shared__ double W[3][NEAR_T][MAXP + 1];      // per-thread interpolation weights (odd stride)
    for (int t = threadIdx.x; t < (int)(sizeof(ChebTables) / 8); t += blockDim.x)
        reinterpret_cast<double *>(&T)[t] = reinterpret_cast<const double *>(tab)[t];
    const int leaf = tleaf[blockIdx.x];
    const int tb = tb_[leaf], te = te_[leaf];
    __syncthreads();
    const int p = T.p, R = p * p * p;
    for (int i = threadIdx.x; i < 4 * R; i += blockDim.x) Ls[i] = local[(long)leaf * 4 * R + i];
    __syncthreads();
    double *w0 = W[0][threadIdx.x], *w1 = W[1][threadIdx.x], *w2 = W[2][threadIdx.x];
    for (int t = tb + threadIdx.x; t < te; t += blockDim.x) {
        interp1(T, (tx[t] - ctr[3 * leaf]) / rad[3 * leaf], w0);
        interp1(T, (ty[t] - ctr[3 * leaf + 1]) / rad[3 * leaf + 1], w1);
        interp1(T, (tz[t] - ctr[3 * leaf + 2]) / rad[3 * leaf + 2], w2);
        double l2p[4] = {0., 0., 0., 0.};
        int c = 0;
        for (int c2 = 0; c2 < p; ++c2) {
            const double s2 = w2[c2];
            for (int c1 = 0; c1 < p; ++c1) {
                const double s1 = w1[c1];
                for (int c0 = 0; c0 < p; ++c0, ++c) {
                    const double w = w0[c0] * s1 * s2;
#pragma unroll
                    for (int o = 0; o < 4; ++o) l2p[o] += w * Ls[o * R + c];
                }
            }
        }
        for (int o = 0; o < 4; ++o) out[o * nt + t] += l2p[o];
    }
}

}  // namespace

// ----------------------------------------------------------------------------------------
// Plan
// ----------------------------------------------------------------------------------------

namespace {
__global__ void k_gather(long n, const int *__restrict__ perm, const double *__restrict__ a, double *b, double scale) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        b[i] = a[perm[i]] * scale;
}

void up_int(DevBuf<int> &b, const std::vector<int> &v, cudaStream_t s) {
    b.alloc(std::max<size_t>(1, v.size()), s);
    b.upload(v.data(), v.size());
}
}  // namespace

void plan_gather(Ctx *c, long n, const int *perm, const double *a, double *b, double scale) {
    if (n <= 0) return;
    (count_launch(), k_gather<<<(int)std::min<long>(4L * c->num_sms, div_up(n, 256)), 256, 0, c->stream>>>(n, perm, a, b, scale));
    IBIM_CHECK_LAUNCH();
}


bool near_segments(const std::vector<int> &tl, const std::vector<int> &nt, std::vector<int> &ptr,
                   std::vector<int> &rng, bool split_long, std::vector<int> &seg, long max_pairs, long min_sources) {
    const int nl = (int)tl.size();
    auto cap_of = [&](int k) { return std::max<long>(min_sources, max_pairs / std::max(1, nt[k])); };
    if (split_long && nl > 0) {  // leaves in parallel: piece counts, offsets, fill
        std::vector<int> p2(nl + 1, 0);
#pragma omp parallel for schedule(static) if (nl >= 4096)
        for (int k = 0; k < nl; ++k) {
            const long cap = cap_of(k);
            long c = 0;
            for (int r = ptr[k]; r < ptr[k + 1]; ++r) c += (rng[2 * r + 1] - rng[2 * r] + cap - 1) / cap;
            p2[k + 1] = (int)c;
        }
        for (int k = 0; k < nl; ++k) p2[k + 1] += p2[k];
        std::vector<int> r2(2 * (size_t)p2[nl]);
#pragma omp parallel for schedule(static) if (nl >= 4096)
        for (int k = 0; k < nl; ++k) {
            const long cap = cap_of(k);
            long q = p2[k];
            for (int r = ptr[k]; r < ptr[k + 1]; ++r)
                for (long b = rng[2 * r]; b < rng[2 * r + 1]; b += cap, ++q) {
                    r2[2 * q] = (int)b;
                    r2[2 * q + 1] = (int)std::min<long>(b + cap, rng[2 * r + 1]);
                }
        }
        ptr.swap(p2);
        rng.swap(r2);
    }
    if (nl == 0) {
        seg.assign(4, 0);
        return false;
    }
    // leaves in parallel: segment counts, offsets, then each leaf fills its own slots
    std::vector<long> soff(nl + 1, 0);
#pragma omp parallel for schedule(static) if (nl >= 4096)
    for (int k = 0; k < nl; ++k) {
        const long cap = cap_of(k);
        long acc = 0, c = 1;
        for (int r = ptr[k]; r < ptr[k + 1]; ++r) {
            const long len = rng[2 * r + 1] - rng[2 * r];
            if (acc > 0 && acc + len > cap) {
                ++c;
                acc = 0;
            }
            acc += len;
        }
        soff[k + 1] = c;
    }
    bool atomic = false;
    for (int k = 0; k < nl; ++k) {
        atomic = atomic || soff[k + 1] > 1;
        soff[k + 1] += soff[k];
    }
    const long nseg = soff[nl];
    std::vector<long> work(nseg);
    std::vector<std::array<int, 4>> body(nseg);
#pragma omp parallel for schedule(static) if (nl >= 4096)
    for (int k = 0; k < nl; ++k) {
        const long cap = cap_of(k), first = soff[k];
        const int multi = soff[k + 1] - first > 1 ? 2 : 0;
        long q = first, acc = 0;
        int r0 = ptr[k];
        auto emit = [&](int r1) {
            work[q] = acc * nt[k];
            body[q] = {tl[k], r0, r1, (q == first ? 1 : 0) | multi};
            ++q;
        };
        for (int r = ptr[k]; r < ptr[k + 1]; ++r) {
            const long len = rng[2 * r + 1] - rng[2 * r];
            if (acc > 0 && acc + len > cap) {
                emit(r);
                r0 = r;
                acc = 0;
            }
            acc += len;
        }
        emit(ptr[k + 1]);
    }
    // descending work, ties in leaf order: a stable LSD radix sort of the segments by
    // (max work - work), 11 bits a pass
    long maxw = 0;
    for (long q = 0; q < nseg; ++q) maxw = std::max(maxw, work[q]);
    std::vector<long> order(nseg), tmp(nseg);
    for (long q = 0; q < nseg; ++q) order[q] = q;
    for (int sh = 0; sh < 63 && (maxw >> sh) > 0; sh += 11) {
        std::array<long, 2049> c{};
        for (long q = 0; q < nseg; ++q) c[1 + (((maxw - work[order[q]]) >> sh) & 2047)]++;
        for (int d = 0; d < 2048; ++d) c[d + 1] += c[d];
        for (long q = 0; q < nseg; ++q) tmp[c[((maxw - work[order[q]]) >> sh) & 2047]++] = order[q];
        order.swap(tmp);
    }
    seg.resize(4 * nseg);
    for (long q = 0; q < nseg; ++q) std::memcpy(&seg[4 * q], body[order[q]].data(), 4 * sizeof(int));
    return atomic;
}

// Work lists of one target set: which nodes need locals, V pairs by operator, X pairs, and
// per target leaf the merged source ranges of its U and W lists.
// Dense index of the V-list operators: (level, source - target lattice offset in [-3, 3]^3).
// M2L operator keys, 5 ints: target level, source level, and the source-minus-target centre offset
// in units of the target node's half-width (per axis).  V pairs (same level, lattice offset o in
// [-3, 3]^3) have offset 2 o and a dense index; X pairs (a coarser source leaf) are hashed.
struct OpIndex {
    std::vector<int> dense;  // level * 343 + offset -> operator id, -1 when absent
    std::vector<int> keys;   // 5 ints per operator
    struct KeyHash {
        size_t operator()(const std::array<int, 5> &k) const {
            uint64_t h = 1469598103934665603ULL;  // FNV-1a over the five ints
            for (int v : k) h = (h ^ (uint32_t)v) * 1099511628211ULL;
            return (size_t)h;
        }
    };
    std::unordered_map<std::array<int, 5>, int, KeyHash> xmap;
    explicit OpIndex(int nlevels) : dense((size_t)std::max(1, nlevels) * 343, -1) {}
    int add(const std::array<int, 5> &k) {
        const int id = (int)keys.size() / 5;
        keys.insert(keys.end(), k.begin(), k.end());
        return id;
    }
    int get(int l, int ox, int oy, int oz) {
        IBIM_REQUIRE(ox >= -3 && ox <= 3 && oy >= -3 && oy <= 3 && oz >= -3 && oz <= 3, "V-list offset out of range");
        int &id = dense[(size_t)l * 343 + (ox + 3) * 49 + (oy + 3) * 7 + (oz + 3)];
        if (id < 0) id = add({l, l, 2 * ox, 2 * oy, 2 * oz});
        return id;
    }
    int get_x(int lt, int ls, int dx, int dy, int dz) {
        const std::array<int, 5> k{lt, ls, dx, dy, dz};
        auto it = xmap.find(k);
        if (it != xmap.end()) return it->second;
        const int id = add(k);
        xmap.emplace(k, id);
        return id;
    }
};

static void build_target_lists(Plan &P, TargetSet &S, OpIndex &opid) {
    const TreeHost &T = P.tree;
    cudaStream_t s = P.ctx->stream;
    const int nn = T.nnodes;
    auto has_t = [&](int i) { return S.end[i] > S.begin[i]; };
    auto has_s = [&](int i) { return T.src_end[i] > T.src_begin[i]; };
    std::vector<int> l2l, lb(T.nlevels + 1, 0);
    for (int l = 0; l < T.nlevels; ++l) {
        lb[l] = (int)l2l.size();
        for (int i = T.level_begin[l]; i < T.level_begin[l + 1]; ++i)
            if (l >= 3 && has_t(i)) l2l.push_back(i);
    }
    lb[T.nlevels] = (int)l2l.size();
    S.l2l_level_begin = lb;
    up_int(S.l2l_nodes, l2l, s);
    // V and X pairs grouped by operator with counting sorts: pairs are generated per target node
    // in parallel, new operator keys get ids in key order (V: dense index, X: sorted keys), and
    // each thread scatters its own contiguous node range, so the grouping is deterministic
    std::vector<int> xs, xt;
    std::vector<long> poff(nn + 1, 0);
    std::vector<long> vcount(nn, 0), xcount(nn, 0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nn; ++i) {
        if (!has_t(i)) continue;
        long v = 0, x = 0;
        for (int sidx : T.V[i]) v += has_s(sidx);
        for (int sidx : T.X[i]) x += has_s(sidx);
        vcount[i] = v;
        xcount[i] = x;
    }
    for (int i = 0; i < nn; ++i) {
        S.nv_list += vcount[i];
        S.nx_list += xcount[i];
        poff[i + 1] = poff[i] + vcount[i] + (P.x_as_ops ? xcount[i] : 0);
    }
    const long npair = poff[nn];
    HostArr<int> pkey(npair), psrc(npair), ptgt(npair);  // pkey: V dense index, or -1 - X slot
    std::vector<std::array<int, 5>> xkey;
    std::vector<long> xslot_of_pair;
    std::vector<long> xoff(nn + 1, 0);
    if (P.x_as_ops) {
        for (int i = 0; i < nn; ++i) xoff[i + 1] = xoff[i] + xcount[i];
        xkey.resize(xoff[nn]);
    }
    std::vector<int> level_of(nn);
    for (int l = 0; l < T.nlevels; ++l)
        for (int i = T.level_begin[l]; i < T.level_begin[l + 1]; ++i) level_of[i] = l;
    // which dense V keys occur: per-thread flags set while the pairs are generated, OR-ed afterwards
    const size_t nd = opid.dense.size();
    std::vector<std::vector<char>> vused(omp_get_max_threads(), std::vector<char>(nd, 0));
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < nn; ++i) {
        if (!has_t(i)) continue;
        const int l = level_of[i];
        char *used_t = vused[omp_get_thread_num()].data();
        long q = poff[i];
        for (int sidx : T.V[i]) {
            if (!has_s(sidx)) continue;
            const int ox = T.coord[3 * sidx] - T.coord[3 * i], oy = T.coord[3 * sidx + 1] - T.coord[3 * i + 1],
                      oz = T.coord[3 * sidx + 2] - T.coord[3 * i + 2];
            pkey[q] = l * 343 + (ox + 3) * 49 + (oy + 3) * 7 + (oz + 3);
            used_t[pkey[q]] = 1;
            psrc[q] = sidx;
            ptgt[q] = i;
            ++q;
        }
        if (!P.x_as_ops) continue;
        long xq = xoff[i];
        for (int sidx : T.X[i]) {
            if (!has_s(sidx)) continue;
            // centre offset in target half-widths: (2 c_s + 1) 2^(lt - ls) - (2 c_t + 1)
            const int ls = level_of[sidx], sh = l - ls;
            std::array<int, 5> k{l, ls, 0, 0, 0};
            for (int a = 0; a < 3; ++a)
                k[2 + a] = (2 * T.coord[3 * sidx + a] + 1) * (1 << sh) - (2 * T.coord[3 * i + a] + 1);
            xkey[xq] = k;
            pkey[q] = -1 - (int)xq;
            psrc[q] = sidx;
            ptgt[q] = i;
            ++q;
            ++xq;
        }
    }
    if (!P.x_as_ops) {
        for (int i = 0; i < nn; ++i) {
            if (!has_t(i)) continue;
            for (int sidx : T.X[i])
                if (has_s(sidx)) {
                    xs.push_back(sidx);
                    xt.push_back(i);
                }
        }
    }
    trace_mark("lists: pairs generated");
    // operator ids: V keys in dense-index order, then X keys in sorted order
    {
        std::vector<char> used(nd, 0);
        for (const auto &part : vused)
            for (size_t d = 0; d < nd; ++d) used[d] |= part[d];
        for (size_t d = 0; d < used.size(); ++d)
            if (used[d]) {
                const int l = (int)(d / 343), c = (int)(d % 343);
                opid.get(l, c / 49 - 3, (c / 7) % 7 - 3, c % 7 - 3);
            }
    }
    std::vector<int> xid(xkey.size());
    const long nx = (long)xkey.size();
    // X keys as 64-bit codes in the same order (levels 5 bits each, offsets 18 bits each biased
    // by 2^17) while every key fits, else the keys themselves: per-thread sorted unique keys,
    // merged; operator ids in sorted key order
    auto fits = [](const std::array<int, 5> &k) {
        return k[0] < 32 && k[1] < 32 && std::abs(k[2]) < (1 << 17) && std::abs(k[3]) < (1 << 17) &&
               std::abs(k[4]) < (1 << 17);
    };
    int all_fit = 1;
#pragma omp parallel for schedule(static) reduction(min : all_fit)
    for (long k = 0; k < nx; ++k) all_fit = std::min(all_fit, fits(xkey[k]) ? 1 : 0);
    auto ids_by_sorted_keys = [&](auto key_of, auto make_op) {
        using K = decltype(key_of(xkey[0]));
        std::vector<K> xc(nx);
        const int nthr = std::max(1, std::min({32, omp_get_max_threads(), (int)(nx / 4096) + 1}));
        std::vector<std::vector<K>> part(nthr);
#pragma omp parallel for schedule(static) num_threads(nthr)
        for (int t = 0; t < nthr; ++t) {
            const long k0 = nx * t / nthr, k1 = nx * (t + 1) / nthr;
            for (long k = k0; k < k1; ++k) xc[k] = key_of(xkey[k]);
            std::vector<K> &u = part[t];
            u.assign(xc.begin() + k0, xc.begin() + k1);
            std::sort(u.begin(), u.end());
            u.erase(std::unique(u.begin(), u.end()), u.end());
        }
        std::vector<K> u;
        for (auto &v : part) u.insert(u.end(), v.begin(), v.end());
        std::sort(u.begin(), u.end());
        u.erase(std::unique(u.begin(), u.end()), u.end());
        std::vector<int> uid(u.size());
        for (size_t k = 0; k < u.size(); ++k) uid[k] = make_op(u[k]);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < nx; ++k) xid[k] = uid[std::lower_bound(u.begin(), u.end(), xc[k]) - u.begin()];
    };
    if (nx > 0 && all_fit) {
        const uint64_t b17 = 1u << 17, m18 = (1u << 18) - 1;
        ids_by_sorted_keys(
            [&](const std::array<int, 5> &k) {
                return ((uint64_t)k[0] << 59) | ((uint64_t)k[1] << 54) | ((uint64_t)(k[2] + b17) << 36) |
                       ((uint64_t)(k[3] + b17) << 18) | (uint64_t)(k[4] + b17);
            },
            [&](uint64_t c) {
                return opid.get_x((int)(c >> 59), (int)((c >> 54) & 31), (int)((c >> 36) & m18) - (int)b17,
                                  (int)((c >> 18) & m18) - (int)b17, (int)(c & m18) - (int)b17);
            });
    } else if (nx > 0) {
        ids_by_sorted_keys([](const std::array<int, 5> &k) { return k; },
                           [&](const std::array<int, 5> &k) { return opid.get_x(k[0], k[1], k[2], k[3], k[4]); });
    }
    trace_mark("lists: operator ids");
    const int nop = (int)opid.keys.size() / 5;
    HostArr<int> pop(npair);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < npair; ++q) pop[q] = pkey[q] >= 0 ? opid.dense[pkey[q]] : xid[-1 - pkey[q]];
    // counting sort by operator; thread t owns pairs [t0, t1) and scatters them in order
    std::vector<long> opbeg(nop + 1, 0);
    HostArr<int> gs(npair), gt(npair);
    {
        const int nthr = std::max(1, std::min({64, omp_get_max_threads(), (int)(npair / 65536) + 1}));
        std::vector<std::vector<long>> hist(nthr, std::vector<long>(nop, 0));
#pragma omp parallel for schedule(static) num_threads(nthr)
        for (int t = 0; t < nthr; ++t) {
            const long t0 = npair * t / nthr, t1 = npair * (t + 1) / nthr;
            for (long q = t0; q < t1; ++q) hist[t][pop[q]]++;
        }
        long run = 0;
        for (int op = 0; op < nop; ++op) {
            opbeg[op] = run;
            for (int t = 0; t < nthr; ++t) {
                const long c = hist[t][op];
                hist[t][op] = run;
                run += c;
            }
        }
        opbeg[nop] = run;
#pragma omp parallel for schedule(static) num_threads(nthr)
        for (int t = 0; t < nthr; ++t) {
            const long t0 = npair * t / nthr, t1 = npair * (t + 1) / nthr;
            for (long q = t0; q < t1; ++q) {
                const long d = hist[t][pop[q]]++;
                gs[d] = psrc[q];
                gt[d] = ptgt[q];
            }
        }
    }
    // chunks (operator, first pair, count) of each contraction's width, in operator order:
    // counts per operator, offsets, then the operators in parallel
    std::vector<int> chunks, chunks32, chunks_tc, chunks_tc2, chunks_oz;
    auto cut = [&](std::vector<int> &out, int width) {
        std::vector<long> coff(nop + 1, 0);
        for (int op = 0; op < nop; ++op) coff[op + 1] = coff[op] + (opbeg[op + 1] - opbeg[op] + width - 1) / width;
        out.resize(3 * coff[nop]);
#pragma omp parallel for schedule(static) if (nop >= 256)
        for (int op = 0; op < nop; ++op) {
            const long b = opbeg[op], n = opbeg[op + 1] - opbeg[op];
            long c = coff[op];
            for (long q = 0; q < n; q += width, ++c) {
                out[3 * c] = op;
                out[3 * c + 1] = (int)(b + q);
                out[3 * c + 2] = (int)std::min<long>(width, n - q);
            }
        }
    };
    cut(chunks, M2L_CH);
    cut(chunks32, M2L_CH32);
    cut(chunks_tc, M2L_CHTC);
    cut(chunks_tc2, 2 * M2L_CHTC);
    cut(chunks_oz, M2L_CHOZ);
    trace_mark("lists: pairs grouped");
    S.nvpairs = npair;
    S.nchunks = (int)chunks.size() / 3;
    S.nchunks32 = (int)chunks32.size() / 3;
    up_int(S.v_chunk32, chunks32, s);
    S.nchunks_tc = (int)chunks_tc.size() / 3;
    up_int(S.v_chunk_tc, chunks_tc, s);
    S.nchunks_tc2 = (int)chunks_tc2.size() / 3;
    up_int(S.v_chunk_tc2, chunks_tc2, s);
    S.nchunks_oz = (int)chunks_oz.size() / 3;
    up_int(S.v_chunk_oz, chunks_oz, s);
    S.v_src.alloc(std::max<long>(1, npair), s);
    S.v_src.upload(gs.data(), npair);
    S.v_tgt.alloc(std::max<long>(1, npair), s);
    S.v_tgt.upload(gt.data(), npair);
    up_int(S.v_chunk, chunks, s);
    S.nxpairs = (long)xs.size();
    up_int(S.x_src, xs, s);
    up_int(S.x_tgt, xt, s);
    trace_mark("lists: chunks, uploads");
    // target leaves and the near-field pair count (U and W lists); the FP64 kernel's merged
    // source ranges are built on first use (near64_lists)
    std::vector<int> tl;
    for (int i = 0; i < nn; ++i)
        if (T.leaf[i] && has_t(i)) tl.push_back(i);
    long npairs = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : npairs)
    for (long k = 0; k < (long)tl.size(); ++k) {
        const int i = tl[k];
        long nsrc = 0;
        for (int sidx : T.U[i]) nsrc += T.src_end[sidx] - T.src_begin[sidx];
        for (int sidx : T.W[i]) nsrc += T.src_end[sidx] - T.src_begin[sidx];
        npairs += nsrc * (S.end[i] - S.begin[i]);
    }
    S.ntleaves = (int)tl.size();
    S.near_pairs = npairs;
    S.tl_h = tl;
    up_int(S.tleaf, tl, s);
    up_int(S.tbeg, S.begin, s);
    up_int(S.tend, S.end, s);
    S.out4.alloc((size_t)4 * std::max<long>(1, S.nt), s);
}

// Extra targets (e.g. atom centres): descend the source tree with the split rule of
// assignChildren (bbfmm.cpp:121-131) and keep each node's targets contiguous in DFS order.
static void bin_targets(Plan &P, TargetSet &S, const double *pts, long nt, const std::vector<int> &child_first) {
    const TreeHost &T = P.tree;
    const int nn = T.nnodes;
    std::vector<int> dfs(nn, 0);
    {
        std::vector<int> stack{0};
        int k = 0;
        while (!stack.empty()) {
            const int n = stack.back();
            stack.pop_back();
            dfs[n] = k++;
            if (!T.leaf[n])
                for (int c = 7; c >= 0; --c) stack.push_back(child_first[n] + c);
        }
    }
    std::vector<int> leaf_of(nt);
    for (long i = 0; i < nt; ++i) {
        const double *x = pts + 3 * i;
        int n = 0;
        while (!T.leaf[n]) {
            const double *c = &T.center[3 * n];
            const int ch = 4 * (x[2] < c[2] ? 0 : 1) + 2 * (x[1] < c[1] ? 0 : 1) + (x[0] < c[0] ? 0 : 1);
            n = child_first[n] + ch;
        }
        leaf_of[i] = n;
    }
    S.perm.resize(nt);
    for (long i = 0; i < nt; ++i) S.perm[i] = (int)i;
    std::stable_sort(S.perm.begin(), S.perm.end(), [&](int a, int b) { return dfs[leaf_of[a]] < dfs[leaf_of[b]]; });
    S.begin.assign(nn, 0);
    S.end.assign(nn, 0);
    std::vector<int> cnt(nn, 0);
    for (long i = 0; i < nt; ++i) cnt[leaf_of[i]]++;
    // leaves in DFS order get consecutive ranges; internal nodes span their children
    std::vector<int> order(nn);
    for (int i = 0; i < nn; ++i) order[dfs[i]] = i;
    int off = 0;
    for (int q = 0; q < nn; ++q) {
        const int n = order[q];
        if (T.leaf[n]) {
            S.begin[n] = off;
            S.end[n] = off + cnt[n];
            off += cnt[n];
        }
    }
    for (int n = nn - 1; n >= 0; --n)
        if (!T.leaf[n]) {
            S.begin[n] = S.begin[child_first[n]];
            S.end[n] = S.end[child_first[n] + 7];
        }
}

Plan *make_plan(Tube *t, bool with_self, const double *extra, long n_extra, int order, int maxpoint, int maxlevel,
                int precision) {
    IBIM_REQUIRE(order >= 2 && order <= MAXP, "fmm_np must be in [2, 8]");
    IBIM_REQUIRE(precision == IBIM_PRECISION_FP64 || precision == IBIM_PRECISION_MIXED ||
                     precision == IBIM_PRECISION_FP64_TC,
                 "unknown precision");
    IBIM_REQUIRE(t && t->n > 0, "plan needs a non-empty tube");
    IBIM_REQUIRE(with_self || (extra && n_extra > 0), "plan needs targets");
    Ctx *c = t->ctx;
    cudaStream_t s = c->stream;
    const long ns = t->n;
    std::vector<double> pts(3 * ns);
    {
        // through the context's pinned staging buffer
        double *h = static_cast<double *>(c->pinned_buffer(sizeof(double) * 3 * (size_t)ns));
        t->x.download(h, ns);
        t->y.download(h + ns, ns);
        t->z.download(h + 2 * ns, ns);
        IBIM_CUDA(cudaStreamSynchronize(s));
#pragma omp parallel for schedule(static) if (ns >= (1 << 16))
        for (long i = 0; i < ns; ++i) {
            pts[3 * i] = h[i];
            pts[3 * i + 1] = h[ns + i];
            pts[3 * i + 2] = h[2 * ns + i];
        }
    }
    Plan *P = new Plan();
    P->ctx = c;
    P->tube = t;
    // X pairs join the operator contraction; IBIM_X_ONTHEFLY keeps the on-the-fly X kernels
    // (kernel evaluated per pair, no operator storage)
    P->x_as_ops = std::getenv("IBIM_X_ONTHEFLY") == nullptr;
    P->ns = ns;
    P->p = order;
    P->R = order * order * order;
    P->maxpoint = maxpoint;
    P->maxlevel = maxlevel;
    P->precision = precision;
    P->tune = tuning_for(order, ns);
    try {
        trace_mark("plan: coordinates downloaded");
        P->tree = build_tree(pts.data(), ns, pts.data(), ns, maxpoint, maxlevel);
        trace_mark("plan: tree and lists");
        TreeHost &T = P->tree;
        const int nn = T.nnodes, R = P->R, n4 = 4 * R;
        T.p = order;
        T.R = R;
        P->src_perm.alloc(ns, s);
        P->src_perm.upload(T.src_perm.data(), ns);
        DevBuf<double> *dst[7] = {&P->sx, &P->sy, &P->sz, &P->snx, &P->sny, &P->snz, &P->sw};
        const DevBuf<double> *srcs[7] = {&t->x, &t->y, &t->z, &t->nx, &t->ny, &t->nz, &t->w};
        const double h3 = t->h * t->h * t->h;
        for (int k = 0; k < 7; ++k) {
            dst[k]->alloc(ns, s);
            // quadrature weight = w * s * h^3 with s = 1 (electric.cpp:33)
            plan_gather(c, ns, P->src_perm.ptr, srcs[k]->ptr, dst[k]->ptr, k == 6 ? h3 : 1.0);
        }
        P->ncenter.alloc(3 * nn, s);
        P->ncenter.upload(T.center.data(), 3 * nn);
        P->nradius.alloc(3 * nn, s);
        P->nradius.upload(T.radius.data(), 3 * nn);
        up_int(P->nsrc_begin, T.src_begin, s);
        up_int(P->nsrc_end, T.src_end, s);
        up_int(P->nparent, T.parent, s);
        up_int(P->nindex8, T.index8, s);
        up_int(P->nempty, T.empty, s);
        std::vector<int> child_first(nn, -1);
        for (int i = nn - 1; i >= 0; --i)
            if (T.parent[i] >= 0) child_first[T.parent[i]] = i - T.index8[i];
        up_int(P->nchild_first, child_first, s);
        auto has_s = [&](int i) { return T.src_end[i] > T.src_begin[i]; };
        std::vector<int> p2m, m2m, m2m_lb(T.nlevels + 1, 0);
        for (int i = 0; i < nn; ++i)
            if (T.leaf[i] && has_s(i)) p2m.push_back(i);
        for (int l = 0; l < T.nlevels; ++l) {
            m2m_lb[l] = (int)m2m.size();
            for (int i = T.level_begin[l]; i < T.level_begin[l + 1]; ++i)
                if (!T.leaf[i] && has_s(i)) m2m.push_back(i);
        }
        m2m_lb[T.nlevels] = (int)m2m.size();
        up_int(P->p2m_nodes, p2m, s);
        up_int(P->m2m_nodes, m2m, s);
        P->m2m_level_begin = m2m_lb;
        P->np2m = (int)p2m.size();
        OpIndex opid(T.nlevels);
        trace_mark("plan: node arrays enqueued");
        if (with_self) {
            TargetSet *S = new TargetSet();
            P->targets.push_back(S);
            S->self = true;
            S->nt = ns;
            S->begin = T.src_begin;
            S->end = T.src_end;
            S->perm = T.src_perm;
            up_int(S->perm_d, S->perm, s);
            build_target_lists(*P, *S, opid);
            trace_mark("plan: self target lists");
        }
        if (extra && n_extra > 0) {
            TargetSet *S = new TargetSet();
            P->targets.push_back(S);
            S->nt = n_extra;
            bin_targets(*P, *S, extra, n_extra, child_first);
            std::vector<double> tq[3];
            for (int a = 0; a < 3; ++a) {
                tq[a].resize(n_extra);
                for (long i = 0; i < n_extra; ++i) tq[a][i] = extra[3 * (long)S->perm[i] + a];
            }
            S->tx.alloc(n_extra, s);
            S->ty.alloc(n_extra, s);
            S->tz.alloc(n_extra, s);
            S->tx.upload(tq[0].data(), n_extra);
            S->ty.upload(tq[1].data(), n_extra);
            S->tz.upload(tq[2].data(), n_extra);
            up_int(S->perm_d, S->perm, s);
            build_target_lists(*P, *S, opid);
            trace_mark("plan: extra target lists");
        }
        P->nops = (int)opid.keys.size() / 5;
        P->op_key_h = opid.keys;
        if (P->op_key_h.empty()) P->op_key_h.assign(5, 0);
        up_int(P->op_key, P->op_key_h, s);
        ChebTables ht;
        cheb_tables_host(order, ht);
        P->tables.alloc(1, s);
        P->tables.upload(&ht, 1);
        P->root_r.alloc(3, s);
        P->root_r.upload(T.radius.data(), 3);
        P->mult.alloc((size_t)nn * n4, s);
        P->local.alloc((size_t)nn * n4, s);
        P->dens4.alloc((size_t)4 * ns, s);
        const size_t smem_k = sizeof(double) * 3 * n4;
        if (smem_k > 48 * 1024) {
            IBIM_CUDA(cudaFuncSetAttribute(k_m2m64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_k));
            IBIM_CUDA(cudaFuncSetAttribute(k_l2l64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_k));
        }
        const size_t sm = sizeof(double) * M2L_CH * n4;
        if (sm > 48 * 1024)
            IBIM_CUDA(cudaFuncSetAttribute(k_m2l_v64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        IBIM_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        delete P;
        throw;
    }
    return P;
}

void fmm_prepare_operators(Plan &P, const ibim_kernel_params &kp, int precision) {
    const double key[5] = {kp.kappa, kp.dE, kp.dI, kp.tau, (double)kp.k3_scaled};
    const bool is64 = precision == IBIM_PRECISION_FP64;
    double *cache = is64 ? P.kp64 : P.kp32;
    bool same = is64 ? P.ops64_ready : P.ops32_ready;
    for (int i = 0; i < 5; ++i) same = same && cache[i] == key[i];
    if (same || P.nops == 0) return;
    cudaStream_t s = P.ctx->stream;
    const int R = P.R, n4 = 4 * R;
    const KParams k = make_kparams(kp, P.tube->h);
    if (precision == IBIM_PRECISION_FP64) {
        P.ops64.alloc((size_t)P.nops * n4 * n4, s);
        dim3 g(div_up((long)R * R, 256), P.nops);
        { ProfScope ps_(PROF_OPS); (count_launch(), k_make_ops64<<<g, 256, 0, s>>>(P.tables.ptr, P.op_key.ptr, P.root_r.ptr, k, P.ops64.ptr)); }
        IBIM_CHECK_LAUNCH();
    } else {
        bool have64 = P.ops64_ready;
        for (int i = 0; i < 5; ++i) have64 = have64 && P.kp64[i] == key[i];
        fmm_prepare_operators_mixed(P, k, have64 ? P.ops64.ptr : nullptr);
    }
    for (int i = 0; i < 5; ++i) cache[i] = key[i];
    (is64 ? P.ops64_ready : P.ops32_ready) = true;
}

static void kp_key(const ibim_kernel_params &kp, double key[5]) {
    key[0] = kp.kappa;
    key[1] = kp.dE;
    key[2] = kp.dI;
    key[3] = kp.tau;
    key[4] = (double)kp.k3_scaled;
}

static bool same_key(const double a[5], const double b[5]) {
    for (int i = 0; i < 5; ++i)
        if (a[i] != b[i]) return false;
    return true;
}

void fmm_ensure_tc_images(Plan &P, const ibim_kernel_params &kp) {
    double key[5];
    kp_key(kp, key);
    if (P.tc_ready && same_key(P.tc_key, key)) return;
    if (m2l_tc_fp16_form() && P.opsff_ready && same_key(P.kpff, key)) {
        m2l_tc_pack(P, P.opsff.ptr);  // FP16 images from the float-float operators of the digit images
    } else {
        fmm_prepare_operators(P, kp, IBIM_PRECISION_MIXED);
        m2l_tc_pack(P);
    }
    // the images replace the FP32 operators on this path
    P.ops32.release();
    P.ops32_ready = false;
    for (int i = 0; i < 5; ++i) P.tc_key[i] = key[i];
    P.tc_ready = true;
}

void fmm_ensure_oz_images(Plan &P, const ibim_kernel_params &kp) {
    double key[5];
    kp_key(kp, key);
    if (P.oz_ready && same_key(P.oz_key, key)) return;
    if (P.precision != IBIM_PRECISION_FP64 && ops_ff_enabled()) {
        // FP64-class plans: operators in float-float on the FP32 pipes (2^-44 a value, below the
        // digit cut's 2^-43)
        fmm_prepare_operators_ff(P, kp);
        m2l_oz_pack(P, P.opsff.ptr);
    } else {
        fmm_prepare_operators(P, kp, IBIM_PRECISION_FP64);
        m2l_oz_pack(P);
    }
    for (int i = 0; i < 5; ++i) P.oz_key[i] = key[i];
    P.oz_ready = true;
}

bool fmm_ensure_images_ff(Plan &P, const ibim_kernel_params &kp) {
    if (P.precision == IBIM_PRECISION_FP64 || !ops_ff_enabled() || !m2l_tc_fp16_form()) return false;
    double key[5];
    kp_key(kp, key);
    if (P.oz_ready && same_key(P.oz_key, key) && P.tc_ready && same_key(P.tc_key, key)) return true;
    fmm_prepare_operators_ff(P, kp);
    m2l_pack_images_ff(P, P.opsff.ptr);
    const char *chk = std::getenv("IBIM_CHECK_IMAGES");  // read per call: a test switch
    if (chk && chk[0] == '1') m2l_check_images_ff(P, P.opsff.ptr);
    // the images replace the FP32 operators on this path
    P.ops32.release();
    P.ops32_ready = false;
    for (int i = 0; i < 5; ++i) P.oz_key[i] = P.tc_key[i] = key[i];
    P.oz_ready = P.tc_ready = true;
    return true;
}

void fmm_release_fp64_operators(Plan &P) {
    P.ops64.release();
    P.ops64_ready = false;
    P.opsff.release();
    P.opsff_ready = false;
}

// Merged U and W source ranges per target leaf and their work segments, for the FP64 near-field
// kernel (leaves in parallel, concatenated in leaf order).
void near64_lists(Plan &P, TargetSet &S) {
    if (S.near64_ready) return;
    const TreeHost &T = P.tree;
    cudaStream_t s = P.ctx->stream;
    const std::vector<int> &tl = S.tl_h;
    std::vector<std::vector<int>> per(tl.size());
#pragma omp parallel for schedule(dynamic, 32)
    for (long k = 0; k < (long)tl.size(); ++k) {
        const int i = tl[k];
        std::vector<std::pair<int, int>> rg;
        for (int sidx : T.U[i])
            if (T.src_end[sidx] > T.src_begin[sidx]) rg.push_back({T.src_begin[sidx], T.src_end[sidx]});
        for (int sidx : T.W[i])
            if (T.src_end[sidx] > T.src_begin[sidx]) rg.push_back({T.src_begin[sidx], T.src_end[sidx]});
        std::sort(rg.begin(), rg.end());
        std::vector<int> &mg = per[k];
        for (auto &r : rg) {
            if (!mg.empty() && mg.back() == r.first)
                mg.back() = r.second;
            else {
                mg.push_back(r.first);
                mg.push_back(r.second);
            }
        }
    }
    std::vector<int> nptr{0}, nr;
    for (size_t k = 0; k < tl.size(); ++k) {
        nr.insert(nr.end(), per[k].begin(), per[k].end());
        nptr.push_back((int)nr.size() / 2);
    }
    std::vector<int> ntk(tl.size()), seg;
    for (size_t k = 0; k < tl.size(); ++k) ntk[k] = (int)(S.end[tl[k]] - S.begin[tl[k]]);
    S.near_atomic = near_segments(tl, ntk, nptr, nr, true, seg);
    S.nnear_seg = tl.empty() ? 0 : (int)seg.size() / 4;
    up_int(S.near_seg, seg, s);
    up_int(S.near_ptr, nptr, s);
    up_int(S.near_range, nr, s);
    S.near64_ready = true;
}

// One FP64 FMM: dens (4 x ns, tree order) -> out (4 x nt of target set ts, tree order).
void fmm_run_fp64(Plan &P, int ts, const ibim_kernel_params &kpp, const double *dens, double *out, bool m2l_sliced) {
    IBIM_REQUIRE(ts >= 0 && ts < (int)P.targets.size(), "no such target set");
    const bool use_oz = m2l_sliced && (4 * P.R + 15) / 16 * 16 <= M2L_OZ_MAXK;
    if (use_oz)
        fmm_ensure_oz_images(P, kpp);
    else
        fmm_prepare_operators(P, kpp, IBIM_PRECISION_FP64);
    const TargetSet &S = *P.targets[ts];
    Ctx *c = P.ctx;
    cudaStream_t s = c->stream;
    const TreeHost &T = P.tree;
    const int R = P.R, n4 = 4 * R;
    const KParams kp = make_kparams(kpp, P.tube->h);
    const size_t smem_k = sizeof(double) * 3 * n4;
    const double *tx = S.self ? P.sx.ptr : S.tx.ptr;
    const double *ty = S.self ? P.sy.ptr : S.ty.ptr;
    const double *tz = S.self ? P.sz.ptr : S.tz.ptr;
    // near field (U and W lists, bbfmm.h:571-609): depends only on the densities.  With the
    // overlap on it starts on the auxiliary stream at full occupancy, CTAs taking work segments
    // from a counter, beside the far field; the L2P follows the join (see fmm_run_mixed).  The
    // FP64-class path evaluates it in float-float on the FP32 pipes over the FP32 near lists.
    const bool ff = m2l_sliced && near_ff_enabled() && S.ntleaves > 0;
    KParamsFF kff{};
    if (ff) {
        prepare_mixed(P, *P.targets[ts]);
        kff = make_kparams_ff(kp);
        near_ff_pack(P, dens, s);
    }
    if (!ff && S.ntleaves > 0) near64_lists(P, *P.targets[ts]);
    const int nseg = ff ? S.nnearff_seg : S.nnear_seg;
    const bool atomic = ff ? S.nearff_atomic : S.near_atomic;
    auto near = [&](cudaStream_t st, int l2p_mask, int grid, int *next, bool count_work) {
        if (ff) {
            ProfScope ps_(PROF_NEARFF, count_work ? NEAR_FF_FLOPS * S.near_pairs : 0.,
                          count_work ? 64.0 * P.ns + 40.0 * S.nt : 0., st);
            near_ff_run(P, S, kff, out, st, grid, next);
            return;
        }
        ProfScope ps_(PROF_NEAR64, count_work ? 70.0 * S.near_pairs : 0., count_work ? 56.0 * P.ns + 40.0 * S.nt : 0.,
                      st);
        (count_launch(), k_near64<<<grid, NEAR_T, 0, st>>>(P.tables.ptr, kp, reinterpret_cast<const int4 *>(S.near_seg.ptr),
                                                         S.near_range.ptr, S.tbeg.ptr, S.tend.ptr, P.ncenter.ptr,
                                                         P.nradius.ptr, P.sx.ptr, P.sy.ptr, P.sz.ptr, dens, P.ns, tx,
                                                         ty, tz, S.nt, P.local.ptr, out, l2p_mask, S.nnear_seg, next));
    };
    const bool overlap = near_overlap() && S.ntleaves > 0;
    static const int occ64 = [] {
        int b = 0;
        IBIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_near64, NEAR_T, 0));
        return std::max(1, b);
    }();
    const int full = (ff ? near_ff_occupancy() : occ64) * c->num_sms;
    const int side = near_side_ctas() > 0 ? near_side_ctas() * c->num_sms : full;
    if (overlap) {
        if (!P.near_next.ptr) P.near_next.alloc(1, s);
        IBIM_CUDA(cudaMemsetAsync(P.near_next.ptr, 0, sizeof(int), s));
        if (atomic) IBIM_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 4 * S.nt, s));
        IBIM_CUDA(cudaEventRecord(c->ev_near_fork, s));
        IBIM_CUDA(cudaStreamWaitEvent(c->aux, c->ev_near_fork, 0));
        near(c->aux, 0, std::min(nseg, side), P.near_next.ptr, true);
        IBIM_CUDA(cudaEventRecord(c->ev_near_join, c->aux));
    }
    try {
        if (P.np2m > 0) {
            ProfScope ps_(PROF_P2M, (8.0 * R + 6.0 * P.p * P.p) * P.ns, 56.0 * P.ns);
            (count_launch(), k_p2m64<<<P.np2m, 128, 0, s>>>(P.tables.ptr, P.p2m_nodes.ptr, P.nsrc_begin.ptr,
                                                            P.nsrc_end.ptr, P.ncenter.ptr, P.nradius.ptr, P.sx.ptr,
                                                            P.sy.ptr, P.sz.ptr, dens, P.ns, P.mult.ptr));
        }
        for (int l = T.nlevels - 1; l >= 0; --l) {
            const int b = P.m2m_level_begin[l], e = P.m2m_level_begin[l + 1];
            if (e > b) {
                ProfScope ps_(PROF_M2M);
                (count_launch(), k_m2m64<<<e - b, 128, smem_k, s>>>(P.tables.ptr, P.m2m_nodes.ptr + b,
                                                                    P.nchild_first.ptr, P.nempty.ptr, P.mult.ptr));
            }
        }
        P.local.zero();
        if (use_oz) {
            m2l_oz_run(P, S);
        } else if (S.nchunks > 0) {
            ProfScope ps_(PROF_M2L_V64, 2.0 * n4 * (double)n4 * S.nvpairs,
                          8.0 * n4 * (2.0 * S.nvpairs + (double)n4 * P.nops));
            (count_launch(), k_m2l_v64<<<S.nchunks, 256, sizeof(double) * M2L_CH * n4, s>>>(
                 n4, S.v_chunk.ptr, S.v_src.ptr, S.v_tgt.ptr, P.ops64.ptr, P.mult.ptr, P.local.ptr));
        }
        if (S.nxpairs > 0) {
            ProfScope ps_(PROF_M2L_X64, 102.0 * R * (double)R * S.nxpairs, 16.0 * n4 * S.nxpairs);
            (count_launch(), k_m2l_x64<<<(int)S.nxpairs, 128, 0, s>>>(P.tables.ptr, kp, S.x_src.ptr, S.x_tgt.ptr,
                                                                      P.ncenter.ptr, P.nradius.ptr, P.mult.ptr,
                                                                      P.local.ptr));
        }
        for (int l = 3; l < T.nlevels; ++l) {
            const int b = S.l2l_level_begin[l], e = S.l2l_level_begin[l + 1];
            if (e > b) {
                ProfScope ps_(PROF_L2L);
                (count_launch(), k_l2l64<<<e - b, 128, smem_k, s>>>(P.tables.ptr, S.l2l_nodes.ptr + b, P.nparent.ptr,
                                                                    P.nindex8.ptr, P.local.ptr));
            }
        }
    } catch (...) {
        if (overlap) cudaStreamSynchronize(c->aux);  // the near field still reads dens and writes out
        throw;
    }
    if (S.ntleaves > 0) {
        if (overlap) {
            if (side < std::min(nseg, full)) near(s, 0, std::min(nseg, full), P.near_next.ptr, false);
            IBIM_CUDA(cudaStreamWaitEvent(s, c->ev_near_join, 0));
        } else {
            if (atomic) IBIM_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 4 * S.nt, s));
            near(s, 1, nseg, nullptr, true);
        }
        if (overlap || ff) {  // the L2P runs on its own after the near field
            ProfScope ps_(PROF_L2P64, (10.0 * R + 6.0 * P.p * P.p) * S.nt, 32.0 * n4 * S.ntleaves + 88.0 * S.nt);
            (count_launch(), k_l2p64<<<S.ntleaves, NEAR_T, 0, s>>>(P.tables.ptr, S.tleaf.ptr, S.tbeg.ptr, S.tend.ptr,
                                                                   P.ncenter.ptr, P.nradius.ptr, tx, ty, tz, S.nt,
                                                                   P.local.ptr, out));
        }
    }
    IBIM_CHECK_LAUNCH();
}

void fmm_run(Plan &P, int ts, const ibim_kernel_params &kp, const double *dens, double *out, int precision) {
    if (precision == IBIM_PRECISION_FP64)
        fmm_run_fp64(P, ts, kp, dens, out, false);
    else if (precision == IBIM_PRECISION_FP64_TC)
        fmm_run_fp64(P, ts, kp, dens, out, m2l_tc_supported());
    else
        fmm_run_mixed(P, ts, kp, dens, out);
}

}  // namespace ibim

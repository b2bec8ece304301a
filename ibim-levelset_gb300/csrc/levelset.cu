// Level set and tube quadrature on the GPU (sm_103a).
//
// Replaces the reference's Grid / levelset / Surface (levelset.h:12-72, levelset.cpp:9-586):
//   k_expand        levelset::expand       (levelset.cpp:91-109)   atom-parallel ordered atomicMax
//   k_weno_stage    levelset::evolve / reinitialize (levelset.cpp:111-287), one TVD-RK3 stage
//   k_count_grad    levelset::countGradient (levelset.cpp:398-432)
//   k_cc_*          Surface BFS from cell 0 (levelset.cpp:444-524) as connected-component labelling
//   k_flood_tile    the same BFS as tiled label propagation (grids beyond 32-bit labels)
//   k_tube_*        cavity removal + tube points (levelset.cpp:529-583) as an ordered compaction
//
// Grid layout (same as the reference): row-major, index i*Ny*Nz + j*Nz + k, k fastest.
// Stencil reads clamp indices to the grid (Grid::get, levelset.cpp:28-33).
// Every kernel is instantiated for an FP64 grid (the reference-exact path) and an FP32 grid
// (the mixed-precision path: storage and WENO arithmetic in FP32; tube points are emitted in
// FP64 from the FP32 values).

#include "internal.cuh"

#include <cmath>
#include <mutex>
#include <string>

namespace ibim {

namespace {

struct Dims {
    int nx, ny, nz;
    __device__ __forceinline__ long idx(int i, int j, int k) const { return ((long)i * ny + j) * nz + k; }
    __device__ __forceinline__ long cidx(int i, int j, int k) const {
        i = min(max(i, 0), nx - 1);
        j = min(max(j, 0), ny - 1);
        k = min(max(k, 0), nz - 1);
        return idx(i, j, k);
    }
};

// Order-preserving maps to unsigned integers (for atomicMax on either precision).
__device__ __forceinline__ unsigned long long ord(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ unsigned ord(float v) {
    unsigned u = __float_as_uint(v);
    return (u >> 31) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ double unord(unsigned long long u) {
    u = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)u);
}
__device__ __forceinline__ float unord(unsigned u) {
    u = (u >> 31) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(u);
}
template <class T> struct OrdT;
template <> struct OrdT<double> { using type = unsigned long long; };
template <> struct OrdT<float> { using type = unsigned; };

template <class T>
__global__ void k_fill(T *g, long n, T v) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) g[i] = v;
}

template <class T>
__global__ void k_scale(T *g, long n, T s) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) g[i] *= s;
}

template <class T>
__global__ void k_encode(T *g, long n, int dir) {
    using U = typename OrdT<T>::type;
    U *u = reinterpret_cast<U *>(g);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (dir > 0)
            u[i] = ord(g[i]);
        else
            g[i] = unord(u[i]);
    }
}

// levelset::expand: g = max(g, (R_a + probe) - |x - c_a|) over the cube of +-r cells around
// each atom, r = (int)((R_a + probe)/dx) + band.  blockIdx.y = atom.  Cells outside the grid
// are skipped (the reference's Grid::set does not clamp).  The FP64 grid evaluates the distance
// as written, in FP64; the FP32 grid in FP32 from the atom's sub-cell offset (computed in FP64)
// plus whole cells, since FP64 square roots on GB300's narrow FP64 pipe dominated the kernel.
template <class T>
__global__ void k_expand(typename OrdT<T>::type *g, Dims d, double sx, double sy, double sz, double dx,
                         const double *__restrict__ centers, const double *__restrict__ radii, double probe,
                         int band) {
    const int a = blockIdx.y;
    const double cx = centers[3 * a], cy = centers[3 * a + 1], cz = centers[3 * a + 2];
    const double R = radii[a] + probe;
    const int r = (int)(R / dx) + band;
    const int icx = (int)((cx - sx) / dx), icy = (int)((cy - sy) / dx), icz = (int)((cz - sz) / dx);
    const int side = 2 * r + 1;
    const long total = (long)side * side * side;
    // FP32 grid: the atom's offset from its own cell, then whole cells
    const float fx = (float)((sx + icx * dx) - cx), fy = (float)((sy + icy * dx) - cy),
                fz = (float)((sz + icz * dx) - cz), h = (float)dx;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int c = icz - r + (int)(t % side);
        const int b = icy - r + (int)((t / side) % side);
        const int ia = icx - r + (int)(t / ((long)side * side));
        if (ia < 0 || b < 0 || c < 0 || ia >= d.nx || b >= d.ny || c >= d.nz) continue;
        if constexpr (sizeof(T) == 4) {
            const float px = fmaf((float)(ia - icx), h, fx), py = fmaf((float)(b - icy), h, fy),
                        pz = fmaf((float)(c - icz), h, fz);
            const float dist = (float)R - sqrtf(fmaf(px, px, fmaf(py, py, pz * pz)));
            atomicMax(g + d.idx(ia, b, c), ord(dist));
        } else {
            const double px = (sx + ia * dx) - cx, py = (sy + b * dx) - cy, pz = (sz + c * dx) - cz;
            const double dist = R - sqrt(px * px + py * py + pz * pz);
            atomicMax(g + d.idx(ia, b, c), ord((T)dist));
        }
    }
}

// Divisions of the WENO5 and RK3 formulas.  FP64 (the reference path) keeps IEEE divisions as
// written in levelset.cpp; FP32 (mixed path) multiplies by reciprocal constants and uses the fast
// hardware reciprocal (about 1 ulp), which the FP32 tolerance absorbs.
struct Div64 {
    __device__ static double q(double x, double c) { return x / c; }
    __device__ static double rcp(double x) { return 1.0 / x; }
    __device__ static double over_sqrt(double x, double y) { return x / sqrt(y); }
};
struct Div32 {
    __device__ static float q(float x, float c) { return x * __fdividef(1.0f, c); }
    __device__ static float rcp(float x) { return __fdividef(1.0f, x); }
    __device__ static float over_sqrt(float x, float y) { return x * rsqrtf(y); }
};
template <class T> struct DivOf;
template <> struct DivOf<double> { using type = Div64; };
template <> struct DivOf<float> { using type = Div32; };

// WENO5 one-sided derivatives along one axis from the 7 values w[0..6] centred on w[3]
// (levelset::setGradient, levelset.cpp:330-388; Jiang-Peng smoothness indicators, eps 1e-6).
template <class T>
__device__ __forceinline__ void weno5(const T w[7], T h, T &up, T &un) {
    using D = typename DivOf<T>::type;
    const T EPS_LS = (T)1e-6;
    T a = w[1] - w[0], b = w[2] - w[1], c = w[3] - w[2], d = w[4] - w[3], e = w[5] - w[4], f = w[6] - w[5];
    const T df = D::q(-b + (T)7.0 * (c + d) - e, (T)12.0);
    a = b - a;
    b = c - b;
    c = d - c;
    d = e - d;
    e = f - e;
    T s0 = (T)13.0 * (e - d) * (e - d) + (T)3.0 * (e - (T)3.0 * d) * (e - (T)3.0 * d);
    T s1 = (T)13.0 * (d - c) * (d - c) + (T)3.0 * (d + c) * (d + c);
    T s2 = (T)13.0 * (c - b) * (c - b) + (T)3.0 * ((T)3.0 * c - b) * ((T)3.0 * c - b);
    T a0 = D::rcp((EPS_LS + s0) * (EPS_LS + s0)), a1 = D::q((T)6.0, (EPS_LS + s1) * (EPS_LS + s1)),
      a2 = D::q((T)3.0, (EPS_LS + s2) * (EPS_LS + s2));
    T w1 = D::rcp(a0 + a1 + a2), w0 = a0 * w1, w2 = a2 * w1;
    up = D::q(df + D::q(w0 * (e - 2 * d + c), (T)3.0) + D::q((w2 - (T)0.5) * (d - (T)2.0 * c + b), (T)6.0), h);
    s0 = (T)13.0 * (a - b) * (a - b) + (T)3.0 * (a - (T)3.0 * b) * (a - (T)3.0 * b);
    s1 = (T)13.0 * (b - c) * (b - c) + (T)3.0 * (b + c) * (b + c);
    s2 = (T)13.0 * (c - d) * (c - d) + (T)3.0 * ((T)3.0 * c - d) * ((T)3.0 * c - d);
    a0 = D::rcp((EPS_LS + s0) * (EPS_LS + s0));
    a1 = D::q((T)6.0, (EPS_LS + s1) * (EPS_LS + s1));
    a2 = D::q((T)3.0, (EPS_LS + s2) * (EPS_LS + s2));
    w1 = D::rcp(a0 + a1 + a2);
    w0 = a0 * w1;
    w2 = a2 * w1;
    un = D::q(df - D::q(w0 * (a - 2 * b + c), (T)3.0) - D::q((w2 - (T)0.5) * (b - 2 * c + d), (T)6.0), h);
}

template <class T>
__device__ __forceinline__ void gradients(const T *__restrict__ g, const Dims &dm, int i, int j, int k, T h, T up[3],
                                          T un[3]) {
    T w[7];
#pragma unroll
    for (int l = 0; l < 7; ++l) w[l] = __ldg(g + dm.cidx(i - 3 + l, j, k));
    weno5(w, h, up[0], un[0]);
#pragma unroll
    for (int l = 0; l < 7; ++l) w[l] = __ldg(g + dm.cidx(i, j - 3 + l, k));
    weno5(w, h, up[1], un[1]);
#pragma unroll
    for (int l = 0; l < 7; ++l) w[l] = __ldg(g + dm.cidx(i, j, k - 3 + l));
    weno5(w, h, up[2], un[2]);
}

// levelset::getNorm(Dun, Dup) (levelset.cpp:294-301).
template <class T>
__device__ __forceinline__ T godunov(const T n[3], const T p[3]) {
    T v = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T m = fmax(n[a] > (T)0 ? n[a] : (T)0, p[a] < (T)0 ? -p[a] : (T)0);
        v += m * m;
    }
    return sqrt(v);
}

// One TVD-RK3 stage over the whole grid.  MODE 0: evolve (phi_t + vel|grad phi| = 0);
// MODE 1: reinitialize (phi_t + S(phi0)(|grad phi| - 1) = 0, S = phi0/sqrt(phi0^2 + dx^2)).
// STAGE 0: u1 = g - L(g); 1: u2 = (3g + u1 - L(u1))/4; 2: g = (g + 2(u2 - L(u2)))/3.
// COUNT (stage 0 only): also countGradient of src = g (levelset.cpp:398-432) from the same WENO
// gradients: among cells with |g| < band, |godunov(D-, D+) - 1| > thres into counts[0], the
// cells into counts[1], the sum of the deviations into accum.
template <int MODE, int STAGE, class T, bool COUNT = false>
__global__ void __launch_bounds__(256) k_weno_stage(Dims dm, T h, T dtv, T eps, const T *__restrict__ src, T *g, T *u1,
                                                    T *u2, const T *__restrict__ phi0, T band = (T)0,
                                                    T thres = (T)0, unsigned long long *counts = nullptr,
                                                    double *accum = nullptr) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z * blockDim.z + threadIdx.z;
    const bool in = i < dm.nx && j < dm.ny && k < dm.nz;
    if (!COUNT && !in) return;
    unsigned bad = 0, tot = 0;
    double acc = 0.;
    if (in) {
        T up[3], un[3];
        gradients(src, dm, i, j, k, h, up, un);
        const long I = dm.idx(i, j, k);
        T L;
        if (MODE == 0) {
            L = dtv * godunov(un, up);
        } else {
            const T p0 = phi0[I];
            const T sign = DivOf<T>::type::over_sqrt(p0, p0 * p0 + eps);
            const T nd = sign > (T)0 ? godunov(un, up) : godunov(up, un);
            L = dtv * sign * (nd - (T)1.0);
        }
        using D = typename DivOf<T>::type;
        if (COUNT && fabs(src[I]) < band) {
            const T nr = godunov(un, up);
            tot = 1;
            bad = fabs(nr - (T)1.0) > thres ? 1u : 0u;
            acc = fabs((double)nr - 1.0);
        }
        if (STAGE == 0)
            u1[I] = g[I] - L;
        else if (STAGE == 1)
            u2[I] = (3 * g[I] + u1[I] - L) * (T)0.25;
        else
            g[I] = D::q(g[I] + 2 * (u2[I] - L), (T)3.0);
    }
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            bad += __shfl_down_sync(0xffffffffu, bad, o);
            tot += __shfl_down_sync(0xffffffffu, tot, o);
            acc += __shfl_down_sync(0xffffffffu, acc, o);
        }
        __shared__ unsigned sb[8], st[8];
        __shared__ double sa[8];
        const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
        if ((tid & 31) == 0) {
            sb[tid >> 5] = bad;
            st[tid >> 5] = tot;
            sa[tid >> 5] = acc;
        }
        __syncthreads();
        if (tid == 0) {
            unsigned B = 0, Tt = 0;
            double A = 0;
            const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
            for (int w = 0; w < nw; ++w) {
                B += sb[w];
                Tt += st[w];
                A += sa[w];
            }
            if (Tt) {
                atomicAdd(counts, (unsigned long long)B);
                atomicAdd(counts + 1, (unsigned long long)Tt);
                atomicAdd(accum, A);
            }
        }
    }
}

// levelset::countGradient: among cells with |g| < thickness*dx, count | |grad g| - 1 | > thres.
template <class T>
__global__ void __launch_bounds__(256) k_count_grad(Dims dm, T h, T band, T thres, const T *__restrict__ g,
                                                    unsigned long long *counts, double *accum) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z * blockDim.z + threadIdx.z;
    unsigned bad = 0, tot = 0;
    double acc = 0.;
    if (i < dm.nx && j < dm.ny && k < dm.nz && fabs(g[dm.idx(i, j, k)]) < band) {
        T up[3], un[3];
        gradients(g, dm, i, j, k, h, up, un);
        const T nr = godunov(un, up);
        tot = 1;
        bad = fabs(nr - (T)1.0) > thres ? 1u : 0u;
        acc = fabs((double)nr - 1.0);
    }
    for (int o = 16; o > 0; o >>= 1) {
        bad += __shfl_down_sync(0xffffffffu, bad, o);
        tot += __shfl_down_sync(0xffffffffu, tot, o);
        acc += __shfl_down_sync(0xffffffffu, acc, o);
    }
    __shared__ unsigned sb[8], st[8];
    __shared__ double sa[8];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    if ((tid & 31) == 0) { sb[tid >> 5] = bad; st[tid >> 5] = tot; sa[tid >> 5] = acc; }
    __syncthreads();
    if (tid == 0) {
        unsigned B = 0, Tt = 0;
        double A = 0;
        const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
        for (int w = 0; w < nw; ++w) { B += sb[w]; Tt += st[w]; A += sa[w]; }
        if (Tt) {
            atomicAdd(counts, (unsigned long long)B);
            atomicAdd(counts + 1, (unsigned long long)Tt);
            atomicAdd(accum, A);
        }
    }
}

// Flood fill from cell 0 (Surface, levelset.cpp:444-524): a cell is reached when a 6-neighbour
// is reached and that neighbour has g > -tw.  Each block owns a TI x TJ x TK tile, iterates the
// rule to a fixed point in shared memory (halo = neighbours' state at launch), writes back and
// raises `changed` if it reached new cells.  The host relaunches until nothing changes.
// Tiles of 1024 cells (FK along k, the contiguous axis, FJ along j, FI along i).  A block loads
// its tile and a one-cell halo of visited flags and passability into shared memory and runs the
// propagation to a fixpoint inside the tile; with rounds > 1 it then writes its new cells, reloads
// the halo's flags (neighbouring tiles of the same launch may have moved the front meanwhile)
// and continues, up to `rounds` times.  Only unvisited -> visited transitions happen, so any
// schedule reaches the same fixpoint; the host relaunches until a launch changes nothing.
template <class T, int FK, int FJ, int FI>
__global__ void __launch_bounds__(FK *FJ *FI) k_flood_tile(Dims dm, T neg_tw, const T *__restrict__ g,
                                                           unsigned char *vis, int *changed, int rounds) {
    __shared__ unsigned char sv[FI + 2][FJ + 2][FK + 2];
    __shared__ unsigned char sp[FI + 2][FJ + 2][FK + 2];
    const int k0 = blockIdx.x * FK, j0 = blockIdx.y * FJ, i0 = blockIdx.z * FI;
    const int tid = threadIdx.x + FK * (threadIdx.y + FJ * threadIdx.z);
    constexpr int HALO = (FI + 2) * (FJ + 2) * (FK + 2);
    for (int t = tid; t < HALO; t += FK * FJ * FI) {
        const int kk = t % (FK + 2), jj = (t / (FK + 2)) % (FJ + 2), ii = t / ((FK + 2) * (FJ + 2));
        const int i = i0 + ii - 1, j = j0 + jj - 1, k = k0 + kk - 1;
        unsigned char v = 0, p = 0;
        if (i >= 0 && j >= 0 && k >= 0 && i < dm.nx && j < dm.ny && k < dm.nz) {
            const long I = dm.idx(i, j, k);
            v = vis[I];
            p = g[I] > neg_tw ? 1 : 0;
        }
        sv[ii][jj][kk] = v;
        sp[ii][jj][kk] = p;
    }
    __syncthreads();
    const int ti = threadIdx.z + 1, tj = threadIdx.y + 1, tk = threadIdx.x + 1;
    const int i = i0 + threadIdx.z, j = j0 + threadIdx.y, k = k0 + threadIdx.x;
    const bool inside = i < dm.nx && j < dm.ny && k < dm.nz;
    bool any = false;
    for (int round = 0; round < rounds; ++round) {
        if (round > 0) {
            // the halo's flags again, past L1 (other blocks of this launch write them)
            bool got = false;
            for (int t = tid; t < HALO; t += FK * FJ * FI) {
                const int kk = t % (FK + 2), jj = (t / (FK + 2)) % (FJ + 2), ii = t / ((FK + 2) * (FJ + 2));
                if (kk > 0 && kk <= FK && jj > 0 && jj <= FJ && ii > 0 && ii <= FI) continue;  // own cells
                const int hi = i0 + ii - 1, hj = j0 + jj - 1, hk = k0 + kk - 1;
                if (hi < 0 || hj < 0 || hk < 0 || hi >= dm.nx || hj >= dm.ny || hk >= dm.nz || sv[ii][jj][kk]) continue;
                if (__ldcg(vis + dm.idx(hi, hj, hk))) {
                    sv[ii][jj][kk] = 1;
                    got = got || sp[ii][jj][kk];
                }
            }
            if (!__syncthreads_or(got)) break;
        }
        bool mine = false;
        for (int it = 0; it < FK * FJ * FI; ++it) {
            int upd = 0;
            if (inside && !sv[ti][tj][tk]) {
                if ((sv[ti - 1][tj][tk] && sp[ti - 1][tj][tk]) || (sv[ti + 1][tj][tk] && sp[ti + 1][tj][tk]) ||
                    (sv[ti][tj - 1][tk] && sp[ti][tj - 1][tk]) || (sv[ti][tj + 1][tk] && sp[ti][tj + 1][tk]) ||
                    (sv[ti][tj][tk - 1] && sp[ti][tj][tk - 1]) || (sv[ti][tj][tk + 1] && sp[ti][tj][tk + 1])) {
                    upd = 1;
                }
            }
            __syncthreads();
            if (upd) { sv[ti][tj][tk] = 1; mine = true; }
            if (!__syncthreads_or(upd)) break;
        }
        if (inside && mine) vis[dm.idx(i, j, k)] = 1;
        any = any || mine;
    }
    if (__syncthreads_or(any) && tid == 0) atomicExch(changed, 1);
}

// The same visited set by connected-component labelling.  With passable(x) = g[x] > -tw, the
// propagation above (a cell is visited when a passable neighbour is) reaches from cell 0 exactly:
// cell 0, the passable cells connected to it through passable cells (6-neighbours), and their
// neighbours.  The passable components come from union-find on cell indices: a label is a cell of
// the same component at a smaller or equal index, a union hangs the larger root under the smaller
// (atomicMin), so each component's root is its smallest cell and cell 0's component (when cell 0
// is passable) has root 0.  The labels start at the first cell of each passable run along k
// (a max-scan per grid row), so only the j and i neighbours need unions.
constexpr int CC_K = 128;

// One warp per grid row (i, j): L = global index of the run start, -1 where impassable.
template <class T>
__global__ void __launch_bounds__(CC_K) k_cc_runs(Dims dm, T neg_tw, const T *__restrict__ g, int *L) {
    const long row = (blockIdx.x * (long)CC_K + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= (long)dm.nx * dm.ny) return;
    const long base = row * dm.nz;
    int carry = -1;  // run start (k) of the segment before, -1 when that segment ended impassable
    for (int k0 = 0; k0 < dm.nz; k0 += 32) {
        const int k = k0 + lane;
        const bool pass = k < dm.nz && g[base + k] > neg_tw;
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        // a run starts at k when k is passable and k - 1 is not (or k is the segment's first
        // cell and the previous segment ended impassable)
        const bool prev = lane > 0 ? ((pm >> (lane - 1)) & 1u) : carry >= 0;
        int v = pass && !prev ? k : (lane == 0 && pass ? carry : -1);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v = max(v, u);
        }
        if (k < dm.nz) L[base + k] = pass ? (int)(base + v) : -1;
        const int last = __shfl_sync(0xffffffffu, v, 31);
        carry = (pm >> 31) & 1u ? last : -1;
    }
}

// Root of x's component, halving the path on the way (a label always points to a smaller cell of
// the same component, so the chain strictly decreases and ends; reads past L1, as other blocks
// relabel concurrently).
__device__ __forceinline__ int cc_find(int *L, int x) {
    int p = __ldcg(L + x);
    while (p != x) {
        const int gp = __ldcg(L + p);
        if (gp != p) L[x] = gp;
        x = p;
        p = gp;
    }
    return x;
}

// The same without the halving writes: while the compression runs, the only write to a label is
// its owner's final one (its root), so no other thread can leave a cell pointing below its root.
__device__ __forceinline__ int cc_root(const int *L, int x) {
    int p = __ldcg(L + x);
    while (p != x) {
        x = p;
        p = __ldcg(L + x);
    }
    return x;
}

// Join the components of a and b.  Each retry follows a root that another thread has just hung
// under a smaller label, so the loop ends; it is bounded all the same, with an error flag.
__device__ __forceinline__ void cc_unite(int *L, int a, int b, int *err) {
    for (int it = 0; it < (1 << 20); ++it) {
        a = cc_find(L, a);
        b = cc_find(L, b);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicMin(L + b, a);
        if (old == b) return;
        b = old;
    }
    atomicExch(err, 1);
}

// Unions with the j - 1 and i - 1 neighbours; blocks of CC_K threads along k, one grid row
// (i, j) per blockIdx (z, y).
__global__ void __launch_bounds__(CC_K) k_cc_merge(Dims dm, int *L, int *err) {
    const int i = blockIdx.z, j = blockIdx.y;
    const long sj = dm.nz, si = (long)dm.ny * dm.nz;
    for (int k = blockIdx.x * CC_K + threadIdx.x; k < dm.nz; k += gridDim.x * CC_K) {
        const long I = dm.idx(i, j, k);
        if (__ldcg(L + I) < 0) continue;  // impassable cells keep -1
        if (j > 0 && __ldcg(L + I - sj) >= 0) cc_unite(L, (int)I, (int)(I - sj), err);
        if (i > 0 && __ldcg(L + I - si) >= 0) cc_unite(L, (int)I, (int)(I - si), err);
    }
}

__global__ void __launch_bounds__(CC_K) k_cc_compress(Dims dm, int *L) {
    const int i = blockIdx.z, j = blockIdx.y;
    for (int k = blockIdx.x * CC_K + threadIdx.x; k < dm.nz; k += gridDim.x * CC_K) {
        const long I = dm.idx(i, j, k);
        if (__ldcg(L + I) >= 0) L[I] = cc_root(L, (int)I);
    }
}

// visited: cell 0, the cells of root 0 and their neighbours (no cell has root 0 when cell 0 is
// impassable)
__global__ void __launch_bounds__(CC_K) k_cc_visited(Dims dm, const int *__restrict__ L, unsigned char *vis) {
    const int i = blockIdx.z, j = blockIdx.y;
    const long sj = dm.nz, si = (long)dm.ny * dm.nz;
    for (int k = blockIdx.x * CC_K + threadIdx.x; k < dm.nz; k += gridDim.x * CC_K) {
        const long I = dm.idx(i, j, k);
        const bool v = I == 0 || L[I] == 0 || (k > 0 && L[I - 1] == 0) || (k + 1 < dm.nz && L[I + 1] == 0) ||
                       (j > 0 && L[I - sj] == 0) || (j + 1 < dm.ny && L[I + sj] == 0) ||
                       (i > 0 && L[I - si] == 0) || (i + 1 < dm.nx && L[I + si] == 0);
        vis[I] = v ? 1 : 0;
    }
}

constexpr int TUBE_BLOCK = 1024;

// Cavity removal (levelset.cpp:529-537) and per-block tube counts in linear cell order.
template <class T>
__global__ void __launch_bounds__(TUBE_BLOCK) k_tube_count(long n, T tw, T cavity, T *g,
                                                           const unsigned char *__restrict__ vis, int *block_counts,
                                                           unsigned long long *ninc) {
    const long I = blockIdx.x * (long)TUBE_BLOCK + threadIdx.x;
    int in = 0;
    unsigned inc = 0;
    if (I < n) {
        T v = g[I];
        if (!vis[I] && fabs(v) < tw) {
            v = cavity;
            g[I] = v;
            inc = 1;
        }
        in = fabs(v) < tw ? 1 : 0;
    }
    const int c = __syncthreads_count(in);
    const int ci = __syncthreads_count(inc);
    if (threadIdx.x == 0) {
        block_counts[blockIdx.x] = c;
        if (ci) atomicAdd(ninc, (unsigned long long)ci);
    }
}

// Exclusive scan of the block counts (single block, sequential chunks; nb is a few thousand).
__global__ void k_scan_counts(const int *counts, int nb, long *offsets) {
    __shared__ long carry;
    __shared__ long wsum[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += blockDim.x) {
        const int i = base + threadIdx.x;
        long v = i < nb ? counts[i] : 0;
        long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            long y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            long s = threadIdx.x < (blockDim.x >> 5) ? wsum[threadIdx.x] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                long y = __shfl_up_sync(0xffffffffu, s, o);
                if (threadIdx.x >= o) s += y;
            }
            wsum[threadIdx.x] = s;
        }
        __syncthreads();
        const long before = (threadIdx.x >> 5) ? wsum[(threadIdx.x >> 5) - 1] : 0;
        if (i < nb) offsets[i] = carry + before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[nb] = carry;
}

// Tube points in (i, j, k) order (levelset.cpp:540-583): normal = (D- + D+)/2 (not normalised),
// projection P = x - n*phi, weight = (1 + cos(pi phi / tw)) / (2 tw), times the surface Jacobian
// when asked (opt-in); emitted in FP64.
// Surface Jacobian at grid point (i, j, k): J = 1 - phi (k1 + k2) + phi^2 k1 k2 with k1 + k2 and
// k1 k2 the sum and product of the principal curvatures of the level set through the point,
// from second-order central differences of phi (clamped at the grid edge):
//   k1 + k2 = div(grad phi / |grad phi|),   k1 k2 = grad phi^T adj(Hess phi) grad phi / |grad phi|^4.
// For a signed distance it is the area ratio of the zero level set to the level set through the
// point (a sphere of radius R at distance phi: (R / (R + phi))^2), independent of the sign
// convention of phi.
template <class T>
__device__ double surface_jacobian(const T *__restrict__ g, Dims dm, int i, int j, int k, double dx, double phi) {
    auto at = [&](int a, int b, int c) -> double {
        a = min(max(a, 0), dm.nx - 1);
        b = min(max(b, 0), dm.ny - 1);
        c = min(max(c, 0), dm.nz - 1);
        return (double)g[((long)a * dm.ny + b) * dm.nz + c];
    };
    const double c0 = at(i, j, k), h2 = dx * dx;
    const double fx = (at(i + 1, j, k) - at(i - 1, j, k)) / (2 * dx);
    const double fy = (at(i, j + 1, k) - at(i, j - 1, k)) / (2 * dx);
    const double fz = (at(i, j, k + 1) - at(i, j, k - 1)) / (2 * dx);
    const double fxx = (at(i + 1, j, k) - 2 * c0 + at(i - 1, j, k)) / h2;
    const double fyy = (at(i, j + 1, k) - 2 * c0 + at(i, j - 1, k)) / h2;
    const double fzz = (at(i, j, k + 1) - 2 * c0 + at(i, j, k - 1)) / h2;
    const double fxy = (at(i + 1, j + 1, k) - at(i + 1, j - 1, k) - at(i - 1, j + 1, k) + at(i - 1, j - 1, k)) / (4 * h2);
    const double fxz = (at(i + 1, j, k + 1) - at(i + 1, j, k - 1) - at(i - 1, j, k + 1) + at(i - 1, j, k - 1)) / (4 * h2);
    const double fyz = (at(i, j + 1, k + 1) - at(i, j + 1, k - 1) - at(i, j - 1, k + 1) + at(i, j - 1, k - 1)) / (4 * h2);
    const double g2 = fx * fx + fy * fy + fz * fz;
    if (!(g2 > 0.0)) return 1.0;
    const double gn = sqrt(g2);
    const double ksum = (fxx * (fy * fy + fz * fz) + fyy * (fx * fx + fz * fz) + fzz * (fx * fx + fy * fy) -
                         2 * (fx * fy * fxy + fx * fz * fxz + fy * fz * fyz)) /
                        (g2 * gn);
    const double kprod = (fx * fx * (fyy * fzz - fyz * fyz) + fy * fy * (fxx * fzz - fxz * fxz) +
                          fz * fz * (fxx * fyy - fxy * fxy) + 2 * fx * fy * (fxz * fyz - fxy * fzz) +
                          2 * fy * fz * (fxy * fxz - fyz * fxx) + 2 * fx * fz * (fxy * fyz - fxz * fyy)) /
                         (g2 * g2);
    return 1.0 - phi * ksum + phi * phi * kprod;
}

template <class T>
__global__ void __launch_bounds__(TUBE_BLOCK) k_tube_emit(Dims dm, double sx, double sy, double sz, double dx, T tw,
                                                          const T *__restrict__ g, const long *__restrict__ offsets,
                                                          double *px, double *py, double *pz, double *qx, double *qy,
                                                          double *qz, double *w, int jacobian) {
    const long n = (long)dm.nx * dm.ny * dm.nz;
    const long I = blockIdx.x * (long)TUBE_BLOCK + threadIdx.x;
    const T v = I < n ? g[I] : (T)0;
    const bool in = I < n && fabs(v) < tw;
    __shared__ int wcount[TUBE_BLOCK / 32];
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wcount[warp] = __popc(bal);
    __syncthreads();
    if (threadIdx.x < 32) {
        int s = wcount[threadIdx.x];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (threadIdx.x >= o) s += y;
        }
        wcount[threadIdx.x] = s;
    }
    __syncthreads();
    if (!in) return;
    const long pos = offsets[blockIdx.x] + (warp ? wcount[warp - 1] : 0) + __popc(bal & ((1u << lane) - 1));
    const int k = (int)(I % dm.nz), j = (int)((I / dm.nz) % dm.ny), i = (int)(I / ((long)dm.ny * dm.nz));
    T up[3], un[3];
    gradients(g, dm, i, j, k, (T)dx, up, un);
    const double nxv = (double)((un[0] + up[0]) * (T)0.5), nyv = (double)((un[1] + up[1]) * (T)0.5),
                 nzv = (double)((un[2] + up[2]) * (T)0.5);
    const double vd = (double)v, twd = (double)tw;
    px[pos] = (sx + i * dx) - nxv * vd;
    py[pos] = (sy + j * dx) - nyv * vd;
    pz[pos] = (sz + k * dx) - nzv * vd;
    qx[pos] = nxv;
    qy[pos] = nyv;
    qz[pos] = nzv;
    double wv = 0.5 * (1.0 + cos(M_PI * vd / twd)) / twd;
    if (jacobian) wv *= surface_jacobian(g, dm, i, j, k, dx, vd);
    w[pos] = wv;
}

inline dim3 stencil_block() { return dim3(32, 4, 2); }
inline dim3 stencil_grid(const Grid &g) {
    dim3 b = stencil_block();
    return dim3(div_up(g.nz, b.x), div_up(g.ny, b.y), div_up(g.nx, b.z));
}
inline Dims dims_of(const Grid &g) { return Dims{g.nx, g.ny, g.nz}; }

template <class T> T *gdata(Grid &g);
template <> double *gdata<double>(Grid &g) { return g.data.ptr; }
template <> float *gdata<float>(Grid &g) { return g.data32.ptr; }
template <class T> const T *gdata(const Grid &g) { return gdata<T>(const_cast<Grid &>(g)); }

template <class T>
void expand_t(Grid &g, const double *centers_dev, const double *radii_dev, int natoms, double probe, int band) {
    cudaStream_t s = g.ctx->stream;
    const long n = g.cells();
    T *d = gdata<T>(g);
    { ProfScope ps_(PROF_EXPAND); (count_launch(), k_encode<T><<<4 * g.ctx->num_sms, 256, 0, s>>>(d, n, +1)); }
    for (int a0 = 0; a0 < natoms; a0 += 65535) {
        const int na = std::min(65535, natoms - a0);
        dim3 grid(8, na);
        ProfScope ps_(PROF_EXPAND);
        (count_launch(), k_expand<T><<<grid, 256, 0, s>>>(reinterpret_cast<typename OrdT<T>::type *>(d), dims_of(g),
                                                           g.sx, g.sy, g.sz, g.dx, centers_dev + 3 * (long)a0,
                                                           radii_dev + a0, probe, band));
    }
    { ProfScope ps_(PROF_EXPAND); (count_launch(), k_encode<T><<<4 * g.ctx->num_sms, 256, 0, s>>>(d, n, -1)); }
    IBIM_CHECK_LAUNCH();
}

template <class T>
void evolve_t(Grid &g, double final_t, double vel, double cfl) {
    double dt = cfl * g.dx / vel;
    const int steps = (int)(final_t / dt) + 1;
    dt = final_t / (double)steps;
    cudaStream_t s = g.ctx->stream;
    DevBuf<T> u1, u2;
    u1.alloc(g.cells(), s);
    u2.alloc(g.cells(), s);
    const Dims dm = dims_of(g);
    const dim3 gr = stencil_grid(g), bl = stencil_block();
    const T dtv = (T)(dt * vel), h = (T)g.dx;
    T *G = gdata<T>(g);
    const double fl = 350.0 * g.cells(), by = 3.0 * sizeof(T) * g.cells();
    for (int st = 0; st < steps; ++st) {
        { ProfScope ps_(PROF_WENO, fl, by); (count_launch(), k_weno_stage<0, 0, T><<<gr, bl, 0, s>>>(dm, h, dtv, (T)0, G, G, u1.ptr, u2.ptr, nullptr)); }
        { ProfScope ps_(PROF_WENO, fl, by); (count_launch(), k_weno_stage<0, 1, T><<<gr, bl, 0, s>>>(dm, h, dtv, (T)0, u1.ptr, G, u1.ptr, u2.ptr, nullptr)); }
        { ProfScope ps_(PROF_WENO, fl, by); (count_launch(), k_weno_stage<0, 2, T><<<gr, bl, 0, s>>>(dm, h, dtv, (T)0, u2.ptr, G, u1.ptr, u2.ptr, nullptr)); }
    }
    IBIM_CHECK_LAUNCH();
}

template <class T>
void count_t(const Grid &g, double thickness, double thres, unsigned long long *cnt, double *acc) {
    ProfScope ps_(PROF_COUNT, 0., (double)sizeof(T) * g.cells());
    (count_launch(), k_count_grad<T><<<stencil_grid(g), stencil_block(), 0, g.ctx->stream>>>(
                         dims_of(g), (T)g.dx, (T)(thickness * g.dx), (T)thres, gdata<T>(g), cnt, acc));
}

template <class T>
int reinit_t(Grid &g, const Grid &phi0, double final_t, double vel, double cfl, int thickness, double thres) {
    double dt = cfl * g.dx / vel;
    const double eps = g.dx * g.dx;
    const int steps = (int)(final_t / dt) + 1;
    dt = final_t / (double)steps;
    cudaStream_t s = g.ctx->stream;
    DevBuf<T> u1, u2;
    DevBuf<double> acc;
    DevBuf<unsigned long long> cnt;
    u1.alloc(g.cells(), s);
    u2.alloc(g.cells(), s);
    cnt.alloc(2, s);
    acc.alloc(1, s);
    unsigned long long *hcnt = nullptr;
    IBIM_CUDA(cudaMallocHost((void **)&hcnt, 2 * sizeof(unsigned long long)));
    const Dims dm = dims_of(g);
    const dim3 gr = stencil_grid(g), bl = stencil_block();
    const T dtv = (T)(dt * vel), h = (T)g.dx;
    T *G = gdata<T>(g);
    const T *P0 = gdata<T>(phi0);
    const double fl = 350.0 * g.cells(), by = 4.0 * sizeof(T) * g.cells();
    int step = 0;
    // The count of the current grid comes from the first stage of the step that would follow: the
    // stage evaluates the same gradients of g.  When no cell is left to fix, or the steps are
    // spent, the stage's u1 is discarded and g is the grid the reference stops at.
    const T band = (T)(thickness * g.dx), th = (T)thres;
    try {
        for (;;) {
            cnt.zero();
            acc.zero();
            {
                ProfScope ps_(PROF_WENO, fl, by);
                (count_launch(), k_weno_stage<1, 0, T, true><<<gr, bl, 0, s>>>(dm, h, dtv, (T)eps, G, G, u1.ptr, u2.ptr,
                                                                              P0, band, th, cnt.ptr, acc.ptr));
            }
            IBIM_CHECK_LAUNCH();
            IBIM_CUDA(cudaMemcpyAsync(hcnt, cnt.ptr, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
            IBIM_CUDA(cudaStreamSynchronize(s));
            if (hcnt[0] == 0 || step >= steps) break;
            step++;
            { ProfScope ps_(PROF_WENO, fl, by); (count_launch(), k_weno_stage<1, 1, T><<<gr, bl, 0, s>>>(dm, h, dtv, (T)eps, u1.ptr, G, u1.ptr, u2.ptr, P0)); }
            { ProfScope ps_(PROF_WENO, fl, by); (count_launch(), k_weno_stage<1, 2, T><<<gr, bl, 0, s>>>(dm, h, dtv, (T)eps, u2.ptr, G, u1.ptr, u2.ptr, P0)); }
        }
    } catch (...) {
        cudaFreeHost(hcnt);
        throw;
    }
    cudaFreeHost(hcnt);
    return step;
}

// The visited set by relaunched tiled propagation (grids beyond 32-bit labels).
template <class T>
void flood_tiles(const Grid &g, const Dims &dm, double tw, const T *G, DevBuf<unsigned char> &vis) {
    cudaStream_t s = g.ctx->stream;
    const long n = g.cells();
    DevBuf<int> changed;
    vis.zero();
    changed.alloc(1, s);
    const unsigned char one = 1;
    IBIM_CUDA(cudaMemcpyAsync(vis.ptr, &one, 1, cudaMemcpyHostToDevice, s));
    // Up to 2^24 cells: tiles of 16 x 8 x 8 cells, 4 rounds a launch (the surface of the 2,000-atom
    // protein's 144 x 145 x 150 grid in 2.2 ms and 32 launches, against 2.9 ms and 64 with one
    // round of 32 x 8 x 4).  Larger grids: one round of 32 x 8 x 4, as the halo reloads of the
    // many tiles away from the front cost more than the launches they save there (the 20,000-atom
    // protein's 530 x 535 x 537 grid: 134 ms against 201 ms).
    const bool small = n <= (1L << 24);
    const int FK = small ? 16 : 32, FJ = 8, FI = small ? 8 : 4, rounds = small ? 4 : 1;
    const dim3 fb(FK, FJ, FI), fg(div_up(g.nz, FK), div_up(g.ny, FJ), div_up(g.nx, FI));
    // Each relaunch moves the front across at least one tile boundary along every open path,
    // so the count is bounded by the number of tiles; exceeding it is reported, not waited on.
    const long cap = (long)fg.x * fg.y * fg.z + 8;
    int *hflag = nullptr;
    IBIM_CUDA(cudaMallocHost((void **)&hflag, sizeof(int)));
    long it = 0;
    try {
        for (;;) {
            changed.zero();
            for (int r = 0; r < 4; ++r) {
                ProfScope ps_(PROF_FLOOD);
                if (small)
                    (count_launch(), k_flood_tile<T, 16, 8, 8><<<fg, fb, 0, s>>>(dm, (T)(-tw), G, vis.ptr, changed.ptr,
                                                                             rounds));
                else
                    (count_launch(), k_flood_tile<T, 32, 8, 4><<<fg, fb, 0, s>>>(dm, (T)(-tw), G, vis.ptr, changed.ptr,
                                                                             rounds));
            }
            IBIM_CHECK_LAUNCH();
            IBIM_CUDA(cudaMemcpyAsync(hflag, changed.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
            IBIM_CUDA(cudaStreamSynchronize(s));
            it += 4;
            if (!*hflag) break;
            if (it > cap) throw Error(IBIM_ERR_LIMIT, "surface flood fill did not converge within its bound");
        }
    } catch (...) {
        cudaFreeHost(hflag);
        throw;
    }
    cudaFreeHost(hflag);
}

template <class T>
Tube *surface_t(Grid &g, int thickness, long *inclusion, bool jacobian) {
    Ctx *c = g.ctx;
    cudaStream_t s = c->stream;
    const double tw = thickness * g.dx;
    const long n = g.cells();
    const Dims dm = dims_of(g);
    T *G = gdata<T>(g);
    DevBuf<unsigned char> vis;
    vis.alloc(n, s);
    if (n < (1L << 31) && g.nx <= 65535 && g.ny <= 65535) {
        // four passes: the surface of the 2,000-atom protein's 144 x 145 x 150 grid in 0.46 ms
        // (2.2 ms by relaunched propagation), of the 20,000-atom one's 530 x 535 x 537 in 17 ms (133)
        DevBuf<int> L, err;
        L.alloc(n, s);
        err.alloc(1, s);
        err.zero();
        const dim3 cb(CC_K), cg(std::min(div_up(g.nz, CC_K), 64), g.ny, g.nx);
        const long rows = (long)g.nx * g.ny;
        {
            ProfScope ps_(PROF_FLOOD);
            (count_launch(), k_cc_runs<T><<<(unsigned)div_up(rows * 32, (long)CC_K), CC_K, 0, s>>>(dm, (T)(-tw), G, L.ptr));
            (count_launch(), k_cc_merge<<<cg, cb, 0, s>>>(dm, L.ptr, err.ptr));
            (count_launch(), k_cc_compress<<<cg, cb, 0, s>>>(dm, L.ptr));
            (count_launch(), k_cc_visited<<<cg, cb, 0, s>>>(dm, L.ptr, vis.ptr));
        }
        IBIM_CHECK_LAUNCH();
        int herr = 0;
        err.download(&herr, 1);
        IBIM_CUDA(cudaStreamSynchronize(s));
        if (herr) throw Error(IBIM_ERR_LIMIT, "surface labelling: a union exceeded its retry bound");
    } else {
        flood_tiles<T>(g, dm, tw, G, vis);
    }
    const int nb = div_up(n, TUBE_BLOCK);
    DevBuf<int> counts;
    DevBuf<long> offsets;
    DevBuf<unsigned long long> ninc;
    counts.alloc(nb, s);
    offsets.alloc(nb + 1, s);
    ninc.alloc(1, s);
    ninc.zero();
    // the cavity value -(tw + 1e-15) (levelset.cpp:529) rounds to -tw in FP32; one ulp below
    // keeps such cells outside the tube in either precision
    const T cavity = sizeof(T) == 8 ? (T)(-(tw + 1e-15)) : (T)std::nextafter(-(float)tw, -1e30f);
    { ProfScope ps_(PROF_TUBE); (count_launch(), k_tube_count<T><<<nb, TUBE_BLOCK, 0, s>>>(n, (T)tw, cavity, G, vis.ptr, counts.ptr, ninc.ptr)); }
    { ProfScope ps_(PROF_TUBE); (count_launch(), k_scan_counts<<<1, 1024, 0, s>>>(counts.ptr, nb, offsets.ptr)); }
    IBIM_CHECK_LAUNCH();
    long total = 0;
    unsigned long long hinc = 0;
    IBIM_CUDA(cudaMemcpyAsync(&total, offsets.ptr + nb, sizeof(long), cudaMemcpyDeviceToHost, s));
    ninc.download(&hinc, 1);
    IBIM_CUDA(cudaStreamSynchronize(s));
    Tube *t = new Tube();
    t->ctx = c;
    t->n = total;
    t->h = g.dx;
    try {
        DevBuf<double> *arrs[7] = {&t->x, &t->y, &t->z, &t->nx, &t->ny, &t->nz, &t->w};
        for (auto *a : arrs) a->alloc(total > 0 ? total : 1, s);
        ProfScope ps_(PROF_TUBE);
        (count_launch(), k_tube_emit<T><<<nb, TUBE_BLOCK, 0, s>>>(dm, g.sx, g.sy, g.sz, g.dx, (T)tw, G, offsets.ptr,
                                                                  t->x.ptr, t->y.ptr, t->z.ptr, t->nx.ptr, t->ny.ptr,
                                                                  t->nz.ptr, t->w.ptr, jacobian ? 1 : 0));
        IBIM_CHECK_LAUNCH();
    } catch (...) {
        delete t;
        throw;
    }
    if (inclusion) *inclusion = (long)hinc;
    return t;
}

}  // namespace

Grid *grid_create(Ctx *c, int nx, int ny, int nz, double sx, double sy, double sz, double dx, double value, int prec) {
    IBIM_REQUIRE(nx > 0 && ny > 0 && nz > 0, "grid sizes must be positive");
    IBIM_REQUIRE(dx > 0, "grid spacing must be positive");
    IBIM_REQUIRE((double)nx * ny * nz < 4.0e9, "grid too large");
    Grid *g = new Grid();
    g->ctx = c;
    g->nx = nx; g->ny = ny; g->nz = nz;
    g->sx = sx; g->sy = sy; g->sz = sz; g->dx = dx;
    g->prec = prec;
    try {
        if (prec == IBIM_PRECISION_FP64) {
            g->data.alloc(g->cells(), c->stream);
            (count_launch(), k_fill<double><<<4 * c->num_sms, 256, 0, c->stream>>>(g->data.ptr, g->cells(), value));
        } else {
            g->data32.alloc(g->cells(), c->stream);
            (count_launch(), k_fill<float><<<4 * c->num_sms, 256, 0, c->stream>>>(g->data32.ptr, g->cells(), (float)value));
        }
        IBIM_CHECK_LAUNCH();
    } catch (...) {
        delete g;
        throw;
    }
    return g;
}

void levelset_expand(Grid &g, const double *centers_dev, const double *radii_dev, int natoms, double probe, int band) {
    if (natoms <= 0) return;
    if (g.prec == IBIM_PRECISION_FP64)
        expand_t<double>(g, centers_dev, radii_dev, natoms, probe, band);
    else
        expand_t<float>(g, centers_dev, radii_dev, natoms, probe, band);
}

void levelset_evolve(Grid &g, double final_t, double vel, double cfl) {
    IBIM_REQUIRE(vel > 0 && cfl > 0 && final_t >= 0, "evolve: invalid time step parameters");
    if (g.prec == IBIM_PRECISION_FP64)
        evolve_t<double>(g, final_t, vel, cfl);
    else
        evolve_t<float>(g, final_t, vel, cfl);
}

void levelset_count_gradient(const Grid &g, double thickness, double thres, long *bad, long *total, double *acc) {
    cudaStream_t s = g.ctx->stream;
    DevBuf<unsigned long long> cnt;
    DevBuf<double> a;
    cnt.alloc(2, s);
    a.alloc(1, s);
    cnt.zero();
    a.zero();
    if (g.prec == IBIM_PRECISION_FP64)
        count_t<double>(g, thickness, thres, cnt.ptr, a.ptr);
    else
        count_t<float>(g, thickness, thres, cnt.ptr, a.ptr);
    IBIM_CHECK_LAUNCH();
    unsigned long long h[2];
    double ha;
    cnt.download(h, 2);
    a.download(&ha, 1);
    IBIM_CUDA(cudaStreamSynchronize(s));
    if (bad) *bad = (long)h[0];
    if (total) *total = (long)h[1];
    if (acc) *acc = ha;
}

int levelset_reinitialize(Grid &g, const Grid &phi0, double final_t, double vel, double cfl, int thickness,
                          double thres) {
    IBIM_REQUIRE(phi0.nx == g.nx && phi0.ny == g.ny && phi0.nz == g.nz && phi0.prec == g.prec,
                 "reinitialize: phi0 size or precision mismatch");
    IBIM_REQUIRE(vel > 0 && cfl > 0 && final_t >= 0, "reinitialize: invalid time step parameters");
    return g.prec == IBIM_PRECISION_FP64 ? reinit_t<double>(g, phi0, final_t, vel, cfl, thickness, thres)
                                         : reinit_t<float>(g, phi0, final_t, vel, cfl, thickness, thres);
}

// Grid::operator*= (levelset.cpp:54-59)
void grid_scale(Grid &g, double sc) {
    if (g.prec == IBIM_PRECISION_FP64)
        (count_launch(), k_scale<double><<<4 * g.ctx->num_sms, 256, 0, g.ctx->stream>>>(g.data.ptr, g.cells(), sc));
    else
        (count_launch(), k_scale<float><<<4 * g.ctx->num_sms, 256, 0, g.ctx->stream>>>(g.data32.ptr, g.cells(), (float)sc));
    IBIM_CHECK_LAUNCH();
}

// Grid::operator= (levelset.cpp:61-73)
void grid_copy(Grid &dst, const Grid &src) {
    IBIM_REQUIRE(dst.cells() == src.cells() && dst.prec == src.prec, "grid copy: size or precision mismatch");
    const size_t bytes = (src.prec == IBIM_PRECISION_FP64 ? sizeof(double) : sizeof(float)) * src.cells();
    IBIM_CUDA(cudaMemcpyAsync(src.prec == IBIM_PRECISION_FP64 ? (void *)dst.data.ptr : (void *)dst.data32.ptr,
                              src.prec == IBIM_PRECISION_FP64 ? (const void *)src.data.ptr : (const void *)src.data32.ptr,
                              bytes, cudaMemcpyDeviceToDevice, dst.ctx->stream));
}

Tube *surface_extract(Grid &g, int thickness, long *inclusion, bool jacobian) {
    IBIM_REQUIRE(thickness > 0, "thickness must be positive");
    return g.prec == IBIM_PRECISION_FP64 ? surface_t<double>(g, thickness, inclusion, jacobian)
                                         : surface_t<float>(g, thickness, inclusion, jacobian);
}

}  // namespace ibim

// ---------------------------------------------------------------------------------------------
// Allocation-free level-set evolution
//
// Some callers cannot let a library allocate device memory: applications that reserve their
// whole HBM budget in their own pool at start-up, or loops that must never enter the CUDA
// allocator (cudaMalloc / cudaFree can synchronise the device and can fail under memory
// pressure in the middle of a run).  ibim_levelset_evolve_static runs levelset::evolve on a
// caller-owned FP64 device grid and takes its two TVD-RK3 stage buffers from the fixed array
// below instead of allocating them.  The array holds 2 x 524,288 doubles (8 MiB) and stays
// resident on every GPU that loads this library until the process exits; grids larger than
// 524,288 cells are rejected.  All calls share the array, so calls that overlap on the GPU
// (on different streams, or from different threads) race; the stage buffers are fully written
// before they are read, so nothing in the array has to start at zero.
// ---------------------------------------------------------------------------------------------

namespace ibim {
namespace {
constexpr long kStaticMaxCells = 1L << 19;
__device__ __align__(256) double g_static_stage[2 * kStaticMaxCells];
std::mutex g_static_mu;
double *g_static_addr[256] = {nullptr};  // per device, from cudaGetSymbolAddress
}  // namespace

}  // namespace ibim

extern "C" int ibim_levelset_evolve_static(double *grid_dev, int nx, int ny, int nz, double dx, double final_t,
                                           double vel, double cfl, void *stream) {
    using namespace ibim;
    if (!grid_dev || nx <= 0 || ny <= 0 || nz <= 0 || !(dx > 0) || !(vel > 0) || !(cfl > 0) || !(final_t >= 0)) {
        set_last_error("ibim_levelset_evolve_static: invalid argument");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    const long cells = (long)nx * ny * nz;
    if (cells > kStaticMaxCells) {
        set_last_error("ibim_levelset_evolve_static: grid of " + std::to_string(cells) +
                       " cells exceeds the fixed scratch limit of " + std::to_string(kStaticMaxCells) + " cells");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 256) {
        set_last_error(std::string("ibim_levelset_evolve_static: cudaGetDevice: ") + cudaGetErrorString(e));
        return IBIM_ERR_CUDA;
    }
    double *scratch = nullptr;
    {
        // first call on a device: look up the array's device address with that device current
        std::lock_guard<std::mutex> lock(g_static_mu);
        if (!g_static_addr[dev]) {
            e = cudaGetSymbolAddress((void **)&g_static_addr[dev], g_static_stage);
            if (e != cudaSuccess) {
                g_static_addr[dev] = nullptr;
                set_last_error(std::string("ibim_levelset_evolve_static: cudaGetSymbolAddress: ") +
                               cudaGetErrorString(e));
                return IBIM_ERR_CUDA;
            }
        }
        scratch = g_static_addr[dev];
    }
    double *u1 = scratch, *u2 = scratch + kStaticMaxCells;
    cudaStream_t s = (cudaStream_t)stream;
    double dt = cfl * dx / vel;
    const int steps = (int)(final_t / dt) + 1;
    dt = final_t / (double)steps;
    const Dims dm{nx, ny, nz};
    const dim3 bl = stencil_block(), gr(div_up(nz, bl.x), div_up(ny, bl.y), div_up(nx, bl.z));
    const double dtv = dt * vel;
    for (int st = 0; st < steps; ++st) {
        (count_launch(), k_weno_stage<0, 0, double><<<gr, bl, 0, s>>>(dm, dx, dtv, 0., grid_dev, grid_dev, u1, u2, nullptr));
        (count_launch(), k_weno_stage<0, 1, double><<<gr, bl, 0, s>>>(dm, dx, dtv, 0., u1, grid_dev, u1, u2, nullptr));
        (count_launch(), k_weno_stage<0, 2, double><<<gr, bl, 0, s>>>(dm, dx, dtv, 0., u2, grid_dev, u1, u2, nullptr));
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("ibim_levelset_evolve_static: launch: ") + cudaGetErrorString(e));
        return IBIM_ERR_CUDA;
    }
    return IBIM_OK;
}

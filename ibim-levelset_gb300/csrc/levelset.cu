// Level set and tube quadrature on the GPU (sm_103a), FP64.
//
// Replaces the reference's Grid / levelset / Surface (levelset.h:12-72, levelset.cpp:9-586):
//   k_expand        levelset::expand       (levelset.cpp:91-109)   atom-parallel ordered atomicMax
//   k_weno_stage    levelset::evolve / reinitialize (levelset.cpp:111-287), one TVD-RK3 stage
//   k_count_grad    levelset::countGradient (levelset.cpp:398-432)
//   k_flood_tile    Surface BFS from cell 0 (levelset.cpp:444-524) as tiled label propagation
//   k_tube_*        cavity removal + tube points (levelset.cpp:529-583) as an ordered compaction
//
// Grid layout (same as the reference): FP64, row-major, index i*Ny*Nz + j*Nz + k, k fastest.
// Stencil reads clamp indices to the grid (Grid::get, levelset.cpp:28-33).

#include "internal.cuh"

#include <cmath>

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

// Order-preserving map between doubles and unsigned 64-bit integers (for atomicMax).
__device__ __forceinline__ unsigned long long d2o(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double o2d(unsigned long long u) {
    u = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)u);
}

__global__ void k_fill(double *g, long n, double v) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) g[i] = v;
}

__global__ void k_scale(double *g, long n, double s) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) g[i] *= s;
}

__global__ void k_encode(double *g, long n, int dir) {
    unsigned long long *u = reinterpret_cast<unsigned long long *>(g);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (dir > 0)
            u[i] = d2o(g[i]);
        else
            g[i] = o2d(u[i]);
    }
}

// levelset::expand: g = max(g, (R_a + probe) - |x - c_a|) over the cube of +-r cells around
// each atom, r = (int)((R_a + probe)/dx) + band.  blockIdx.y = atom.  Cells outside the grid
// are skipped (the reference's Grid::set does not clamp).
__global__ void k_expand(unsigned long long *g, Dims d, double sx, double sy, double sz, double dx,
                         const double *__restrict__ centers, const double *__restrict__ radii, double probe,
                         int band) {
    const int a = blockIdx.y;
    const double cx = centers[3 * a], cy = centers[3 * a + 1], cz = centers[3 * a + 2];
    const double R = radii[a] + probe;
    const int r = (int)(R / dx) + band;
    const int icx = (int)((cx - sx) / dx), icy = (int)((cy - sy) / dx), icz = (int)((cz - sz) / dx);
    const int side = 2 * r + 1;
    const long total = (long)side * side * side;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int c = icz - r + (int)(t % side);
        const int b = icy - r + (int)((t / side) % side);
        const int ia = icx - r + (int)(t / ((long)side * side));
        if (ia < 0 || b < 0 || c < 0 || ia >= d.nx || b >= d.ny || c >= d.nz) continue;
        const double px = (sx + ia * dx) - cx, py = (sy + b * dx) - cy, pz = (sz + c * dx) - cz;
        const double dist = R - sqrt(px * px + py * py + pz * pz);
        atomicMax(g + d.idx(ia, b, c), d2o(dist));
    }
}

// WENO5 one-sided derivatives along one axis from the 7 values w[0..6] centred on w[3]
// (levelset::setGradient, levelset.cpp:330-388; Jiang-Peng smoothness indicators, eps 1e-6).
__device__ __forceinline__ void weno5(const double w[7], double h, double &up, double &un) {
    const double EPS_LS = 1e-6;
    double a = w[1] - w[0], b = w[2] - w[1], c = w[3] - w[2], d = w[4] - w[3], e = w[5] - w[4], f = w[6] - w[5];
    const double df = (-b + 7.0 * (c + d) - e) / 12.0;
    a = b - a;
    b = c - b;
    c = d - c;
    d = e - d;
    e = f - e;
    double s0 = 13.0 * (e - d) * (e - d) + 3.0 * (e - 3.0 * d) * (e - 3.0 * d);
    double s1 = 13.0 * (d - c) * (d - c) + 3.0 * (d + c) * (d + c);
    double s2 = 13.0 * (c - b) * (c - b) + 3.0 * (3.0 * c - b) * (3.0 * c - b);
    double a0 = 1.0 / ((EPS_LS + s0) * (EPS_LS + s0)), a1 = 6.0 / ((EPS_LS + s1) * (EPS_LS + s1)),
           a2 = 3.0 / ((EPS_LS + s2) * (EPS_LS + s2));
    double w1 = 1.0 / (a0 + a1 + a2), w0 = a0 * w1, w2 = a2 * w1;
    up = (df + w0 * (e - 2 * d + c) / 3.0 + (w2 - 0.5) * (d - 2.0 * c + b) / 6.0) / h;
    s0 = 13.0 * (a - b) * (a - b) + 3.0 * (a - 3.0 * b) * (a - 3.0 * b);
    s1 = 13.0 * (b - c) * (b - c) + 3.0 * (b + c) * (b + c);
    s2 = 13.0 * (c - d) * (c - d) + 3.0 * (3.0 * c - d) * (3.0 * c - d);
    a0 = 1.0 / ((EPS_LS + s0) * (EPS_LS + s0));
    a1 = 6.0 / ((EPS_LS + s1) * (EPS_LS + s1));
    a2 = 3.0 / ((EPS_LS + s2) * (EPS_LS + s2));
    w1 = 1.0 / (a0 + a1 + a2);
    w0 = a0 * w1;
    w2 = a2 * w1;
    un = (df - w0 * (a - 2 * b + c) / 3.0 - (w2 - 0.5) * (b - 2 * c + d) / 6.0) / h;
}

__device__ __forceinline__ void gradients(const double *__restrict__ g, const Dims &dm, int i, int j, int k,
                                          double h, double up[3], double un[3]) {
    double w[7];
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
__device__ __forceinline__ double godunov(const double n[3], const double p[3]) {
    double v = 0.;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double m = fmax(n[a] > 0. ? n[a] : 0., p[a] < 0. ? -p[a] : 0.);
        v += m * m;
    }
    return sqrt(v);
}

// One TVD-RK3 stage over the whole grid.  MODE 0: evolve (phi_t + vel|grad phi| = 0);
// MODE 1: reinitialize (phi_t + S(phi0)(|grad phi| - 1) = 0, S = phi0/sqrt(phi0^2 + dx^2)).
// STAGE 0: u1 = g - L(g); 1: u2 = (3g + u1 - L(u1))/4; 2: g = (g + 2(u2 - L(u2)))/3.
template <int MODE, int STAGE>
__global__ void __launch_bounds__(256) k_weno_stage(Dims dm, double h, double dtv, double eps,
                                                    const double *__restrict__ src, double *g, double *u1,
                                                    double *u2, const double *__restrict__ phi0) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= dm.nx || j >= dm.ny || k >= dm.nz) return;
    double up[3], un[3];
    gradients(src, dm, i, j, k, h, up, un);
    const long I = dm.idx(i, j, k);
    double L;
    if (MODE == 0) {
        L = dtv * godunov(un, up);
    } else {
        const double p0 = phi0[I];
        const double sign = p0 / sqrt(p0 * p0 + eps);
        const double nd = sign > 0. ? godunov(un, up) : godunov(up, un);
        L = dtv * sign * (nd - 1.0);
    }
    if (STAGE == 0)
        u1[I] = g[I] - L;
    else if (STAGE == 1)
        u2[I] = (3 * g[I] + u1[I] - L) / 4.0;
    else
        g[I] = (g[I] + 2 * (u2[I] - L)) / 3.0;
}

// levelset::countGradient: among cells with |g| < thickness*dx, count | |grad g| - 1 | > thres.
__global__ void __launch_bounds__(256) k_count_grad(Dims dm, double h, double band, double thres,
                                                    const double *__restrict__ g, unsigned long long *counts,
                                                    double *accum) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z * blockDim.z + threadIdx.z;
    unsigned bad = 0, tot = 0;
    double acc = 0.;
    if (i < dm.nx && j < dm.ny && k < dm.nz && fabs(g[dm.idx(i, j, k)]) < band) {
        double up[3], un[3];
        gradients(g, dm, i, j, k, h, up, un);
        const double nr = godunov(un, up);
        tot = 1;
        bad = fabs(nr - 1.0) > thres ? 1u : 0u;
        acc = fabs(nr - 1.0);
    }
    // warp then block reduction, one atomic per block
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
        unsigned B = 0, T = 0;
        double A = 0;
        const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
        for (int w = 0; w < nw; ++w) { B += sb[w]; T += st[w]; A += sa[w]; }
        if (T) {
            atomicAdd(counts, (unsigned long long)B);
            atomicAdd(counts + 1, (unsigned long long)T);
            atomicAdd(accum, A);
        }
    }
}

// Flood fill from cell 0 (Surface, levelset.cpp:444-524): a cell is reached when a 6-neighbour
// is reached and that neighbour has g > -tw.  Each block owns a TI x TJ x TK tile, iterates the
// rule to a fixed point in shared memory (halo = neighbours' state at launch), writes back and
// raises `changed` if it reached new cells.  The host relaunches until nothing changes.
constexpr int FT_K = 32, FT_J = 8, FT_I = 4;
__global__ void __launch_bounds__(FT_K *FT_J *FT_I) k_flood_tile(Dims dm, double neg_tw, const double *__restrict__ g,
                                                                 unsigned char *vis, int *changed) {
    __shared__ unsigned char sv[FT_I + 2][FT_J + 2][FT_K + 2];
    __shared__ unsigned char sp[FT_I + 2][FT_J + 2][FT_K + 2];
    const int k0 = blockIdx.x * FT_K, j0 = blockIdx.y * FT_J, i0 = blockIdx.z * FT_I;
    const int tid = threadIdx.x + FT_K * (threadIdx.y + FT_J * threadIdx.z);
    constexpr int HALO = (FT_I + 2) * (FT_J + 2) * (FT_K + 2);
    for (int t = tid; t < HALO; t += FT_K * FT_J * FT_I) {
        const int kk = t % (FT_K + 2), jj = (t / (FT_K + 2)) % (FT_J + 2), ii = t / ((FT_K + 2) * (FT_J + 2));
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
    bool mine = false;
    for (int it = 0; it < FT_K * FT_J * FT_I; ++it) {
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
    if (__syncthreads_or(mine) && tid == 0) atomicExch(changed, 1);
}

constexpr int TUBE_BLOCK = 1024;

// Cavity removal (levelset.cpp:529-537) and per-block tube counts in linear cell order.
__global__ void __launch_bounds__(TUBE_BLOCK) k_tube_count(long n, double tw, double *g,
                                                           const unsigned char *__restrict__ vis,
                                                           int *block_counts, unsigned long long *ninc) {
    const long I = blockIdx.x * (long)TUBE_BLOCK + threadIdx.x;
    int in = 0;
    unsigned inc = 0;
    if (I < n) {
        double v = g[I];
        if (!vis[I] && fabs(v) < tw) {
            v = -(tw + 1e-15);
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
        // inclusive warp scan
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
// projection P = x - n*phi, weight = (1 + cos(pi phi / tw)) / (2 tw).
__global__ void __launch_bounds__(TUBE_BLOCK) k_tube_emit(Dims dm, double sx, double sy, double sz, double dx,
                                                          double tw, const double *__restrict__ g,
                                                          const long *__restrict__ offsets, double *px, double *py,
                                                          double *pz, double *qx, double *qy, double *qz, double *w) {
    const long n = (long)dm.nx * dm.ny * dm.nz;
    const long I = blockIdx.x * (long)TUBE_BLOCK + threadIdx.x;
    const double v = I < n ? g[I] : 0.;
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
        wcount[threadIdx.x] = s;  // inclusive
    }
    __syncthreads();
    if (!in) return;
    const long pos = offsets[blockIdx.x] + (warp ? wcount[warp - 1] : 0) + __popc(bal & ((1u << lane) - 1));
    const int k = (int)(I % dm.nz), j = (int)((I / dm.nz) % dm.ny), i = (int)(I / ((long)dm.ny * dm.nz));
    double up[3], un[3];
    gradients(g, dm, i, j, k, dx, up, un);
    const double nxv = (un[0] + up[0]) * 0.5, nyv = (un[1] + up[1]) * 0.5, nzv = (un[2] + up[2]) * 0.5;
    px[pos] = (sx + i * dx) - nxv * v;
    py[pos] = (sy + j * dx) - nyv * v;
    pz[pos] = (sz + k * dx) - nzv * v;
    qx[pos] = nxv;
    qy[pos] = nyv;
    qz[pos] = nzv;
    w[pos] = 0.5 * (1.0 + cos(M_PI * v / tw)) / tw;
}

inline dim3 stencil_block() { return dim3(32, 4, 2); }
inline dim3 stencil_grid(const Grid &g) {
    dim3 b = stencil_block();
    return dim3(div_up(g.nz, b.x), div_up(g.ny, b.y), div_up(g.nx, b.z));
}
inline Dims dims_of(const Grid &g) { return Dims{g.nx, g.ny, g.nz}; }

}  // namespace

Grid *grid_create(Ctx *c, int nx, int ny, int nz, double sx, double sy, double sz, double dx, double value) {
    IBIM_REQUIRE(nx > 0 && ny > 0 && nz > 0, "grid sizes must be positive");
    IBIM_REQUIRE(dx > 0, "grid spacing must be positive");
    IBIM_REQUIRE((double)nx * ny * nz < 4.0e9, "grid too large");
    Grid *g = new Grid();
    g->ctx = c;
    g->nx = nx; g->ny = ny; g->nz = nz;
    g->sx = sx; g->sy = sy; g->sz = sz; g->dx = dx;
    try {
        g->data.alloc(g->cells(), c->stream);
        (count_launch(), k_fill<<<4 * c->num_sms, 256, 0, c->stream>>>(g->data.ptr, g->cells(), value));
        IBIM_CHECK_LAUNCH();
    } catch (...) {
        delete g;
        throw;
    }
    return g;
}

void levelset_expand(Grid &g, const double *centers_dev, const double *radii_dev, int natoms, double probe, int band) {
    if (natoms <= 0) return;
    IBIM_REQUIRE(natoms <= 65535 * 64, "too many atoms");
    cudaStream_t s = g.ctx->stream;
    const long n = g.cells();
    { ProfScope ps_(PROF_EXPAND); (count_launch(), k_encode<<<4 * g.ctx->num_sms, 256, 0, s>>>(g.data.ptr, n, +1)); }
    // atoms beyond gridDim.y's limit are processed in slices
    for (int a0 = 0; a0 < natoms; a0 += 65535) {
        const int na = std::min(65535, natoms - a0);
        dim3 grid(8, na);
        { ProfScope ps_(PROF_EXPAND); (count_launch(), k_expand<<<grid, 256, 0, s>>>(reinterpret_cast<unsigned long long *>(g.data.ptr), dims_of(g), g.sx, g.sy,
                                      g.sz, g.dx, centers_dev + 3 * (long)a0, radii_dev + a0, probe, band)); }
    }
    { ProfScope ps_(PROF_EXPAND); (count_launch(), k_encode<<<4 * g.ctx->num_sms, 256, 0, s>>>(g.data.ptr, n, -1)); }
    IBIM_CHECK_LAUNCH();
}

void levelset_evolve(Grid &g, double final_t, double vel, double cfl) {
    IBIM_REQUIRE(vel > 0 && cfl > 0 && final_t >= 0, "evolve: invalid time step parameters");
    double dt = cfl * g.dx / vel;
    const int steps = (int)(final_t / dt) + 1;
    dt = final_t / (double)steps;
    cudaStream_t s = g.ctx->stream;
    DevBuf<double> u1, u2;
    u1.alloc(g.cells(), s);
    u2.alloc(g.cells(), s);
    const Dims dm = dims_of(g);
    const dim3 gr = stencil_grid(g), bl = stencil_block();
    const double dtv = dt * vel, ih = g.dx;
    for (int st = 0; st < steps; ++st) {
        { ProfScope ps_(PROF_WENO, 350.0 * g.cells(), 24.0 * g.cells()); (count_launch(), k_weno_stage<0, 0><<<gr, bl, 0, s>>>(dm, ih, dtv, 0., g.data.ptr, g.data.ptr, u1.ptr, u2.ptr, nullptr)); }
        { ProfScope ps_(PROF_WENO, 350.0 * g.cells(), 24.0 * g.cells()); (count_launch(), k_weno_stage<0, 1><<<gr, bl, 0, s>>>(dm, ih, dtv, 0., u1.ptr, g.data.ptr, u1.ptr, u2.ptr, nullptr)); }
        { ProfScope ps_(PROF_WENO, 350.0 * g.cells(), 24.0 * g.cells()); (count_launch(), k_weno_stage<0, 2><<<gr, bl, 0, s>>>(dm, ih, dtv, 0., u2.ptr, g.data.ptr, u1.ptr, u2.ptr, nullptr)); }
    }
    IBIM_CHECK_LAUNCH();
}

void levelset_count_gradient(const Grid &g, double thickness, double thres, long *bad, long *total, double *acc) {
    cudaStream_t s = g.ctx->stream;
    DevBuf<unsigned long long> cnt;
    DevBuf<double> a;
    cnt.alloc(2, s);
    a.alloc(1, s);
    cnt.zero();
    a.zero();
    { ProfScope ps_(PROF_COUNT, 0., 8.0 * g.cells()); (count_launch(), k_count_grad<<<stencil_grid(g), stencil_block(), 0, s>>>(dims_of(g), g.dx, thickness * g.dx, thres,
                                                             g.data.ptr, cnt.ptr, a.ptr)); }
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
    IBIM_REQUIRE(phi0.nx == g.nx && phi0.ny == g.ny && phi0.nz == g.nz, "reinitialize: phi0 size mismatch");
    IBIM_REQUIRE(vel > 0 && cfl > 0 && final_t >= 0, "reinitialize: invalid time step parameters");
    double dt = cfl * g.dx / vel;
    const double eps = g.dx * g.dx;
    const int steps = (int)(final_t / dt) + 1;
    dt = final_t / (double)steps;
    cudaStream_t s = g.ctx->stream;
    DevBuf<double> u1, u2, acc;
    DevBuf<unsigned long long> cnt;
    u1.alloc(g.cells(), s);
    u2.alloc(g.cells(), s);
    cnt.alloc(2, s);
    acc.alloc(1, s);
    unsigned long long *hcnt = nullptr;
    IBIM_CUDA(cudaMallocHost((void **)&hcnt, 2 * sizeof(unsigned long long)));
    const Dims dm = dims_of(g);
    const dim3 gr = stencil_grid(g), bl = stencil_block();
    const double dtv = dt * vel, ih = g.dx, band = thickness * g.dx;
    auto count = [&]() -> unsigned long long {
        cnt.zero();
        { ProfScope ps_(PROF_COUNT, 0., 8.0 * g.cells()); (count_launch(), k_count_grad<<<gr, bl, 0, s>>>(dm, ih, band, thres, g.data.ptr, cnt.ptr, acc.ptr)); }
        IBIM_CHECK_LAUNCH();
        IBIM_CUDA(cudaMemcpyAsync(hcnt, cnt.ptr, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        IBIM_CUDA(cudaStreamSynchronize(s));
        return hcnt[0];
    };
    int step = 0;
    try {
        unsigned long long bad = count();
        while (bad != 0 && step < steps) {
            step++;
            { ProfScope ps_(PROF_WENO, 350.0 * g.cells(), 24.0 * g.cells()); (count_launch(), k_weno_stage<1, 0><<<gr, bl, 0, s>>>(dm, ih, dtv, eps, g.data.ptr, g.data.ptr, u1.ptr, u2.ptr,
                                                 phi0.data.ptr)); }
            { ProfScope ps_(PROF_WENO, 350.0 * g.cells(), 24.0 * g.cells()); (count_launch(), k_weno_stage<1, 1><<<gr, bl, 0, s>>>(dm, ih, dtv, eps, u1.ptr, g.data.ptr, u1.ptr, u2.ptr,
                                                 phi0.data.ptr)); }
            { ProfScope ps_(PROF_WENO, 350.0 * g.cells(), 24.0 * g.cells()); (count_launch(), k_weno_stage<1, 2><<<gr, bl, 0, s>>>(dm, ih, dtv, eps, u2.ptr, g.data.ptr, u1.ptr, u2.ptr,
                                                 phi0.data.ptr)); }
            bad = count();
        }
    } catch (...) {
        cudaFreeHost(hcnt);
        throw;
    }
    cudaFreeHost(hcnt);
    return step;
}

// Grid::operator*= (levelset.cpp:54-59)
void grid_scale(Grid &g, double sc) {
    (count_launch(), k_scale<<<4 * g.ctx->num_sms, 256, 0, g.ctx->stream>>>(g.data.ptr, g.cells(), sc));
    IBIM_CHECK_LAUNCH();
}

void grid_copy(Grid &dst, const Grid &src) {
    IBIM_REQUIRE(dst.cells() == src.cells(), "grid copy: size mismatch");
    IBIM_CUDA(cudaMemcpyAsync(dst.data.ptr, src.data.ptr, sizeof(double) * src.cells(), cudaMemcpyDeviceToDevice,
                              dst.ctx->stream));
}

Tube *surface_extract(Grid &g, int thickness, long *inclusion) {
    IBIM_REQUIRE(thickness > 0, "thickness must be positive");
    Ctx *c = g.ctx;
    cudaStream_t s = c->stream;
    const double tw = thickness * g.dx;
    const long n = g.cells();
    const Dims dm = dims_of(g);
    DevBuf<unsigned char> vis;
    DevBuf<int> changed;
    vis.alloc(n, s);
    vis.zero();
    changed.alloc(1, s);
    const unsigned char one = 1;
    IBIM_CUDA(cudaMemcpyAsync(vis.ptr, &one, 1, cudaMemcpyHostToDevice, s));
    const dim3 fb(FT_K, FT_J, FT_I), fg(div_up(g.nz, FT_K), div_up(g.ny, FT_J), div_up(g.nx, FT_I));
    // Each relaunch moves the front across at least one tile boundary along every open path,
    // so the count is bounded by the number of tiles; exceeding it is reported, not waited on.
    const long cap = (long)fg.x * fg.y * fg.z + 8;
    int *hflag = nullptr;
    IBIM_CUDA(cudaMallocHost((void **)&hflag, sizeof(int)));
    long it = 0;
    try {
        for (;;) {
            changed.zero();
            for (int r = 0; r < 4; ++r) { ProfScope ps_(PROF_FLOOD); (count_launch(), k_flood_tile<<<fg, fb, 0, s>>>(dm, -tw, g.data.ptr, vis.ptr, changed.ptr)); }
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
    const int nb = div_up(n, TUBE_BLOCK);
    DevBuf<int> counts;
    DevBuf<long> offsets;
    DevBuf<unsigned long long> ninc;
    counts.alloc(nb, s);
    offsets.alloc(nb + 1, s);
    ninc.alloc(1, s);
    ninc.zero();
    { ProfScope ps_(PROF_TUBE); (count_launch(), k_tube_count<<<nb, TUBE_BLOCK, 0, s>>>(n, tw, g.data.ptr, vis.ptr, counts.ptr, ninc.ptr)); }
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
        { ProfScope ps_(PROF_TUBE); (count_launch(), k_tube_emit<<<nb, TUBE_BLOCK, 0, s>>>(dm, g.sx, g.sy, g.sz, g.dx, tw, g.data.ptr, offsets.ptr, t->x.ptr,
                                             t->y.ptr, t->z.ptr, t->nx.ptr, t->ny.ptr, t->nz.ptr, t->w.ptr)); }
        IBIM_CHECK_LAUNCH();
    } catch (...) {
        delete t;
        throw;
    }
    if (inclusion) *inclusion = (long)hinc;
    return t;
}

}  // namespace ibim

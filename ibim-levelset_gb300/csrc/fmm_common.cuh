// Device helpers shared by the FMM translation units: Chebyshev tables, the fused BIE kernel
// block and the near-field pair update.
#pragma once

#include <cstring>

#include "internal.cuh"

namespace ibim {

constexpr int MAXP = 8;
constexpr int MAXR = MAXP * MAXP * MAXP;
constexpr int M2L_CH32 = 32;  // V pairs per chunk of the FP32 contraction
constexpr int M2L_CHTC = 128; // V pairs per chunk of the tensor-core contraction (MMA N)
constexpr int M2L_CHOZ = 128; // V pairs per chunk of the sliced FP64-class contraction (MMA N)
// Largest padded contraction length whose digit-group sums stay below 2^24 (exact in FP32):
// K * (2 * 64 * 32 + 5 * 32 * 32) < 2^24, i.e. orders p <= 7.
constexpr int M2L_OZ_MAXK = 1792;

// Chebyshev nodes, polynomials and parent -> child transfers for order p (bbfmm.h:273-326).
struct ChebTables {
    double cheb[MAXP];           // -cos((i + 1/2) pi / p)
    double tnode[MAXP][MAXP];    // T_k(cheb_m): [m][k]
    double S[2][MAXP][MAXP];     // S_p(child node, parent node) for the lower (0) / upper (1) half
    int p, R;
};

// Kernel parameters, prepared once (electric.cpp:52-58, :96-97).
struct KParams {
    double kappa, eps, ieps, vr, k2in, q4pi, vr2;
    double k3f;  // factor on the K3 block: 1 (the reference) or 1 / (4 pi) (k3_scaled)
};

inline KParams make_kparams(const ibim_kernel_params &kp, double h) {
    KParams k;
    k.kappa = kp.kappa;
    k.eps = kp.dE / kp.dI;
    k.ieps = kp.dI / kp.dE;
    k.vr = kp.tau * h;
    k.k2in = kp.kappa == 0. ? 0. : (std::exp(-kp.kappa * k.vr) - 1.0 + kp.kappa * k.vr) / kp.kappa / 2.0 / M_PI / k.vr / k.vr;
    k.q4pi = 1.0 / (4.0 * M_PI);
    k.vr2 = k.vr * k.vr;
    k.k3f = kp.k3_scaled ? k.q4pi : 1.0;
    return k;
}

// S_p(x, cheb_m), m < p: (-1 + 2 sum_k T_k(x) T_k(cheb_m)) / p (bbfmm.h:409-419).
__device__ __forceinline__ void interp1(const ChebTables &T, double x, double *out) {
    double Tk[MAXP];
    Tk[0] = 1.0;
    Tk[1] = x;
    for (int k = 2; k < T.p; ++k) Tk[k] = 2.0 * x * Tk[k - 1] - Tk[k - 2];
    for (int m = 0; m < T.p; ++m) {
        double s = 0.;
        for (int k = 0; k < T.p; ++k) s += Tk[k] * T.tnode[m][k];
        out[m] = (-1.0 + 2.0 * s) * (1.0 / T.p);
    }
}

// 1 / sqrt(x) for x > 0 in FP64: the FP32 reciprocal square root as seed (relative error below
// 2^-22) and two Newton steps y <- y (3 - x y^2) / 2, each squaring the error (2^-44, then below
// FP64 rounding).  This replaces the FP64 square root and three divisions of the formulas below,
// whose multi-instruction sequences dominated the FP64 pipe.
__device__ __forceinline__ double rsqrt64(double x) {
    double y = (double)rsqrtf((float)x);
    y = y * (1.5 - 0.5 * x * y * y);
    y = y * (1.5 - 0.5 * x * y * y);
    return y;
}

// Shared radial factors of the 16 kernels (electric.cpp:67-291) at squared distance d2 >= vr^2:
// c1 (K1), c4 (K4), k2 (K2), hd and ho (K3: hd delta_ab + ho d_a d_b).  With kappa = 0 the
// Yukawa factor e^{-kappa r} is 1 and the exponential is skipped (uniform branch).
__device__ __forceinline__ void radial64(const KParams &k, double d2, double &c1, double &c4, double &k2, double &hd,
                                         double &ho) {
    const double ir = rsqrt64(d2);
    const double r = d2 * ir, ir2 = ir * ir, ir3 = ir2 * ir;
    const double t = k.kappa * r;
    const double e = k.kappa == 0.0 ? 1.0 : exp(-t);
    const double et1 = e * (t + 1);
    const double q3 = ir3 * k.q4pi, h3 = ir3 * k.k3f;  // shared factors of K1, K4 and of K3
    c1 = (k.eps * et1 - 1.) * q3;
    c4 = (1. - k.ieps * et1) * q3;
    k2 = (1.0 - e) * ir * k.q4pi;
    hd = (1 - et1) * h3;
    ho = (e * ((t + 3) * t + 3) - 3.0) * h3 * ir2;
}

// Fused 4x4 block of the 16 BIE kernels (electric.cpp:67-291) at d = source - target.
// Rows: F, Gx, Gy, Gz.  Columns: m_x, m_y, m_z, psi.  Inside the cutoff r < tau h only the
// regularised K2 value remains (electric.cpp:96-97).
__device__ __forceinline__ void kblock64(const KParams &k, double dx, double dy, double dz, double b[16]) {
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < k.vr2) {
#pragma unroll
        for (int i = 0; i < 16; ++i) b[i] = 0.;
        b[3] = -k.k2in;
        return;
    }
    double c1, c4, k2, hd, ho;
    radial64(k, d2, c1, c4, k2, hd, ho);
    const double dd[3] = {dx, dy, dz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        b[a] = dd[a] * c1;
#pragma unroll
        for (int c = 0; c < 3; ++c) b[4 * (a + 1) + c] = ho * dd[a] * dd[c] + (a == c ? hd : 0.);
        b[4 * (a + 1) + 3] = -dd[a] * c4;
    }
    b[3] = -k2;
}

// One near-field source -> target update of the fused block (same formulas as kblock64).
__device__ __forceinline__ void near_pair64(const KParams &k, double dx, double dy, double dz, double m0, double m1,
                                            double m2, double psi, double acc[4]) {
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < k.vr2) {
        acc[0] -= k.k2in * psi;
        return;
    }
    double c1, c4, k2, hd, ho;
    radial64(k, d2, c1, c4, k2, hd, ho);
    const double dm = dx * m0 + dy * m1 + dz * m2;
    acc[0] += c1 * dm - k2 * psi;
    const double cm = ho * dm - c4 * psi;
    acc[1] += hd * m0 + dx * cm;
    acc[2] += hd * m1 + dy * cm;
    acc[3] += hd * m2 + dz * cm;
}

// Kernel parameters of the float-float near field (hi, lo word pairs) with the tables of its
// exponential: e0[j] = e^{-j/64}, e1[j] = e^{-j}.
struct KParamsFF {
    float2 kappa, eps, ieps, k2in, q4pi, vr2, k3f;
    int yukawa;
    float2 e0[64], e1[64];
};
KParamsFF make_kparams_ff(const KParams &k);
// FP32 flops (an FMA counts 2) of one float-float pair update outside the cutoff
constexpr double NEAR_FF_FLOPS = 690.0;
int near_ff_occupancy();
// Leaf-relative coordinates, FP32 near lists and segments of a target set (shared by the mixed
// path and the float-float near field).
void prepare_mixed(Plan &P, TargetSet &S);
// Pack one matvec's densities (4 x ns, FP64) into the float-float source records.
void near_ff_pack(Plan &P, const double *dens, cudaStream_t st);
// Near field without the L2P into out (4 x nt), over the float-float segments: grid CTAs, taking
// segments from *next when next is not null (else one segment per CTA).
void near_ff_run(Plan &P, const TargetSet &S, const KParamsFF &kp, double *out, cudaStream_t st, int grid, int *next);

// Chebyshev nodes and interpolation tables of order p (bbfmm.h:409-419), computed on the host.
void cheb_tables_host(int p, ChebTables &T);

void plan_gather(Ctx *c, long n, const int *perm, const double *a, double *b, double scale);
// ops64: the FP64 operators for the same kernel parameters (rounded instead of re-evaluated), or null
void fmm_prepare_operators_mixed(Plan &P, const KParams &k, const double *ops64);

}  // namespace ibim

/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C (OpenMP) restatement of the reference's (GaZ3ll3/ibim-levelset) CPU algorithm
 * for the implicit-boundary-integral Poisson-Boltzmann path: level set (levelset.cpp),
 * tube quadrature (levelset.cpp Surface), black-box Chebyshev FMM (bbfmm.h, bbfmm.cpp),
 * restarted GMRES (gmres.cpp) and the BIE operator / energy (electric.cpp).
 *
 * It is the checker of the CUDA path and the CPU baseline of the benchmark; nothing in
 * the product links it.  It is pinned against the reference's own outputs (the golden
 * fixtures in tests/golden/, generated by running the reference compiled from its sources).
 *
 * Units: Angstrom, rescale s = 1 (electric.cpp:13-42 with rescale = 1).
 */
#ifndef IBIM_ORACLE_H
#define IBIM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- level set (levelset.cpp) ---- */
void orc_expand(double *g, int nx, int ny, int nz, double lox, double loy, double loz, double h,
                int band, const double *centers, const double *radii, int natoms, double probe);
void orc_evolve(double *g, int nx, int ny, int nz, double h, double final_t, double vel, double cfl);
/* returns the number of pseudo-time steps taken (the loop of levelset.cpp:214-281) */
int orc_reinitialize(double *g, const double *phi0, int nx, int ny, int nz, double h, double final_t,
                     double vel, double cfl, int thickness, double thres);
long orc_count_gradient(const double *g, int nx, int ny, int nz, double h, double thickness, double thres,
                        double *accum_error, long *total);
/* Full geometry pipeline of main.cpp:45-60 (s = 1): fills g (nx*ny*nz), returns reinit steps
 * of the two passes in steps[2]. */
void orc_levelset_build(double *g, int nx, int ny, int nz, double lox, double loy, double loz, double h,
                        int band, double init, const double *centers, const double *radii, int natoms,
                        double probe, double reinit_t, int thickness, double thres, int steps[2]);
/* Surface(Grid&, levelset&, s=1) (levelset.cpp:437-586).  Modifies g (cavity cells).
 * Writes up to cap points as rows (x, y, z, nx, ny, nz, w).  Returns the number of tube points
 * (which may exceed cap: then call again with a larger buffer on a fresh grid). */
long orc_surface(double *g, int nx, int ny, int nz, double lox, double loy, double loz, double h,
                 int thickness, double *out7, long cap, long *inclusion);

/* ---- FMM tree (bbfmm.cpp) ---- */
typedef struct orc_tree orc_tree;
orc_tree *orc_tree_build(const double *src, int ns, const double *tgt, int nt, int maxpoint, int maxlevel);
void orc_tree_free(orc_tree *t);
int orc_tree_nnodes(const orc_tree *t);
/* per node: level, parent, leaf, empty, nsrc, ntgt, center[3], radius[3] */
void orc_tree_node(const orc_tree *t, int id, int *ints6, double *cr6);
/* list: 0=U 1=V 2=W 3=X; returns the size, writes up to cap sorted ids */
int orc_tree_list(const orc_tree *t, int id, int which, int *out, int cap);

/* ---- BIE kernels and FMM (bbfmm.h, electric.cpp:67-291) ---- */
typedef struct {
    double kappa, dE, dI, vr; /* vr = tau * h (vacant radius, electric.cpp:58) */
} orc_kparams;

/* Kernel ids.  0..15 are the reference's scalar kernels
 *   K1x K1y K1z K2 K3xx K3yy K3zz K3xy K3yz K3zx K3yx K3zy K3xz K4x K4y K4z
 * (electric.cpp:67-291); 16 = the fused 4x4 BIE block (inputs phiX phiY phiZ dphi,
 * outputs F = K1.m - K2 dphi and G = H m - K4 dphi, H the K3 Hessian block). */
#define ORC_KERNEL_FUSED 16

/* One FMM: dens is nd x ns (nd = 4 for the fused kernel, else 1), out is no x nt (no = 4 / 1),
 * both in the caller's point order.  `t` must have been built on the same src/tgt. */
void orc_fmm(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out);
/* Timing sample of orc_fmm: full upward pass, downward pass only on nodes with id % stride == 0. */
void orc_fmm_sample(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out,
                    int stride);
/* orc_fmm at the targets sel[0..nsel) only (their leaves and those leaves' ancestors in the
 * downward pass); equal to orc_fmm there.  Returns the number of leaves evaluated. */
int orc_fmm_targets(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out,
                    const int *sel, int nsel);

typedef struct {
    int np, maxpoint, maxlevel, restart, maxiter;
    double kappa, dE, dI, tau, tol;
    /* 0: one fused 4x4 FMM per matvec over a tree built once;
     * 1: reference-structured — 16 scalar FMMs per matvec, each building its own tree
     *    (electric.cpp:299-367), as the reference does. */
    int mode;
} orc_bie_params;

/* Right-hand side `load` (electric.cpp:395-412): b is 2N. surf7 rows are Surface output
 * (x, y, z, nx, ny, nz, w) with w the raw cosine weight (quadrature weight = w * h^3). */
void orc_rhs(const double *surf7, long N, const double *centers, const double *charges, int M,
             const orc_bie_params *bp, double *b);
/* The matvec dmapping (electric.cpp:294-388): y = x + D^-1 K x, x and y are 2N. */
void orc_matvec(const double *surf7, long N, double h, const orc_bie_params *bp, const double *x, double *y);
/* Full solve: RHS, GMRES(x0 = 0) (gmres.cpp:50-164), polarizeMap and energy (electric.cpp:442-505).
 * Returns the GMRES status (0 converged, 1 not).  x is 2N, atom_pot is M. */
int orc_solve(const double *surf7, long N, double h, const double *centers, const double *charges, int M,
              const orc_bie_params *bp, double *x, double *atom_pot, double *energy, int *iters, int *matvecs);

/* Restarted GMRES of gmres.cpp on a caller-supplied operator. */
typedef void (*orc_op)(void *ctx, const double *x, double *y);
int orc_gmres(orc_op A, void *ctx, long n, double *x, const double *b, int m, int max_iter, double tol,
              int *iters, int *matvecs);

#ifdef __cplusplus
}
#endif
#endif

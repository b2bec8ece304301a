// BIE operator and GMRES (solve.cu).
#pragma once

#include <functional>
#include <vector>

#include "internal.cuh"

namespace ibim {

struct GmresStats {
    int iters = 0, matvecs = 0;
    double residual = 0.;
    std::vector<double> history;
};

// Device Krylov workspace for GMRES(m) on vectors of length n.
struct Krylov {
    Ctx *ctx;
    long n;
    int m;
    DevBuf<double> V, w, r, part, hcol, ydev;
    double *hpin = nullptr;
    Krylov(Ctx *c, long n, int m);
    ~Krylov();
    double norm(const double *a);
    int solve(const std::function<void(const double *, double *)> &A, double *x, const double *b, int max_iter,
              double tol, bool x_is_zero, GmresStats &st);
};

void permute(Ctx *c, long n, const int *perm, const double *in, double *out, bool scatter);
void bie_matvec(Plan &P, const ibim_kernel_params &kp, const double *x, double *y, int precision);
// load (electric.cpp:395-412) in tree order; FP32 with compensated sums on a mixed plan.
void bie_rhs(Plan &P, const ibim_kernel_params &kp, const double *atoms4_dev, int natoms, double *b);
// b_tube: the right-hand side already computed in tube order (bie_rhs_tube), or null to compute
// it here.
void electric_solve(Plan &P, const ibim_kernel_params &kp, const double *atoms4_dev, const double *charges_host,
                    int natoms, int restart, int maxiter, double tol, int precision, double *x_tree_out,
                    std::vector<double> *atom_pot, ibim_result &res, const double *b_tube = nullptr);
// load (electric.cpp:395-412) on the tube points in tube order, on stream st; FP32 with
// compensated sums when precision is IBIM_PRECISION_MIXED.
void bie_rhs_tube(const Tube &t, const ibim_kernel_params &kp, const double *atoms4_dev, int natoms, double *b,
                  cudaStream_t st, int precision);

}  // namespace ibim

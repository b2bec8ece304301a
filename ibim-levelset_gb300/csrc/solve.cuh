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
// The four densities of dmapping (electric.cpp:324-329) from x (2 ns, tree order) into dens4.
void bie_densities(Plan &P, const double *x, double *dens4);
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

// The part of a whole solve before GMRES (capi.cu): the tube, its plan with operators and
// images, and the right-hand side in tube order (b_tube) from the atoms (atoms4: x, y, z, q).
struct SolvePrep {
    Tube *tube = nullptr;
    Plan *P = nullptr;
    DevBuf<double> a4, b_tube;
    const double *atoms4 = nullptr;
    SolvePrep() = default;
    SolvePrep(const SolvePrep &) = delete;
    ~SolvePrep() {
        if (P) cudaStreamSynchronize(P->ctx->aux);  // a failed solve may leave near-field work there
        delete P;
        delete tube;
    }
};
// after_surface (optional) runs once the plan's tree and lists exist, before its operators and
// images are built, with the FMM phase's device bytes (plan_fmm_bytes): an admission point.
void solve_prepare(Ctx *c, const double *centers_dev, const double *radii_dev, const double *centers_host,
                   const double *charges_host, int natoms, const ibim_config &cfg, ibim_result &res,
                   const double *atoms4_dev, SolvePrep &out,
                   const std::function<void(long)> *after_surface = nullptr);
// A whole solve from host atom arrays (ibim_solve) with the FMM-phase admission hook.
void solve_host(Ctx *c, const double *centers, const double *charges, const double *radii, int natoms,
                const ibim_config &cfg, ibim_result &res, const std::function<void(long)> *after_surface);
// Device bytes of a solve's phases, estimated from its configuration: the level set (grids), and
// the FMM phase for npoints tube points (plan, operator images at their peak, Krylov basis).
double estimate_levelset_bytes(const ibim_config &cfg);
double estimate_fmm_bytes(const ibim_config &cfg, long npoints);
// The FMM phase's bytes for a built plan (its operator and node counts are exact).
double plan_fmm_bytes(const Plan &P, const ibim_config &cfg);
// A request's footprint before its level set runs (the FMM phase for a tube point count guessed
// from the grid).
double estimate_request_bytes(const ibim_config &cfg);
// For the lock-step paths (batch.cu): the preparation of one molecule -- solve_prepare, the
// mixed near lists uploaded for both target sets, the right-hand side in tree order; bytes = the
// device memory the prepared molecule holds.
struct BatchMol {
    int index = 0;
    const double *charges = nullptr;  // host, natoms
    int natoms = 0;
    ibim_config cfg{};
    ibim_result *res = nullptr;
    SolvePrep *prep = nullptr;         // released once merged
    DevBuf<double> *b_tree = nullptr;  // right-hand side in tree order (2N)
    double bytes = 0;
};
void batch_prepare(Ctx *c, const double *centers_host, const double *charges_host, const double *radii_host,
                   int natoms, const ibim_config &cfg, ibim_result &res, BatchMol &out,
                   const std::function<void(long)> *after_surface = nullptr);
struct WaveStats {
    long merged_mixed = 0, merged_fp64 = 0;
    double active_frac = 0;
    double t_merge_ms = 0, t_solve_ms = 0, t_energy_ms = 0;
};
// One wave of prepared molecules (same h, order, eps, tau, restart): merged plan, lock-step
// refinement and GMRES, energies into each molecule's result.  The molecules' preparations are
// released once merged.
void batch_wave(Ctx *c, std::vector<BatchMol> &mols, WaveStats &ws);
// Whether two configurations can share a wave.
bool batch_compatible(const ibim_config &a, const ibim_config &b);
void check_config(const ibim_config &cfg);
void fill_plan_stats(const Plan &P, ibim_result &res);
void atoms_to_device(Ctx *c, const double *centers, const double *charges, int natoms, DevBuf<double> &a4);
// Many molecules in lock-step waves (batch.cu; the C ABI's ibim_batch_solve).
void batch_solve(Ctx *c, int nmol, const int *natoms, const double *centers, const double *charges,
                 const double *radii, const ibim_config *cfgs, int max_wave, int wave_slots, double budget,
                 int workers, ibim_result *results, int *statuses, double *done_ms, double *info);

}  // namespace ibim

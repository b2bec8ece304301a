// C++ drop-in layer over the C ABI (include/ibim.h) with the reference's class interfaces.
//
// The reference (GaZ3ll3/ibim-levelset) drives its path through these classes; code written
// against them keeps its shape, with the work done on the GPU:
//   Config            Config.h:15-22        (`key = value` lines; accepts lines without trailing
//                                           whitespace, which the reference's parser rejects)
//   Molecule          molecule.h:10-126     (PQR loader, getCenter, centralize)
//   Grid              levelset.h:12-30      (device grid; get/set go through a host mirror)
//   levelset          levelset.h:33-60      (expand, evolve, reinitialize, countGradient)
//   Surface           levelset.h:62-72      (nodes, normals, weight; device tube kept)
//   bbfmm::kernel     bbfmm.h:200-270       (eval = one of the reference's kernel ids)
//   GMRES             gmres.h:20-21         (any std::function<Vector(Vector&)> operator; Krylov
//                                           basis on the GPU, products through the callback)
//   BIEOperator       electric.cpp:294-412  (dmapping and load on the GPU, for GMRES's closure)
//   electric          electric.h:13         (prints the polarized energy, writes potent/energy files)
// Errors: a failing library call throws ibim::dropin::Error (status + message), where the
// reference would assert, exit or throw from std::stod.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <exception>
#include <functional>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../ibim.h"

namespace ibim {
namespace dropin {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(int st) {
    if (st != IBIM_OK) throw Error(st, ibim_last_error());
}

// One context (device 0) shared by every object, created on first use.
inline ibim_ctx context() {
    static ibim_ctx ctx = [] {
        ibim_ctx c = nullptr;
        check(ibim_ctx_create(0, &c));
        return c;
    }();
    return ctx;
}

class Config {
  public:
    std::map<std::string, std::string> options;
    void parse(std::istream &in) {
        for (std::string line; std::getline(in, line);) {
            std::istringstream iss(line);
            std::string id, eq, val;
            if (!(iss >> id) || id[0] == '#') continue;
            if (!(iss >> eq >> val) || eq != "=") {
                std::cout << "Incomplete configuration! Did you forget the space?" << std::endl;
                continue;
            }
            options[id] = val;
        }
    }
    void print() const {
        for (const auto &kv : options) std::cout << std::setw(15) << kv.first << " = " << kv.second << std::endl;
    }
    double num(const std::string &k) const {
        auto it = options.find(k);
        return it == options.end() ? 0.0 : std::atof(it->second.c_str());
    }
};

class Molecule {
  public:
    std::vector<std::array<double, 3>> centers;
    std::vector<double> radii, charges;
    std::array<double, 3> center{{0, 0, 0}};
    double radius = 0;
    int N = 0;

    // molecule.h:21-50: lines starting with ATOM, tokens 5..9 = x y z charge radius
    void load(const std::string &fileName) {
        std::ifstream f(fileName);
        if (!f.is_open()) throw Error(IBIM_ERR_IO, "cannot open " + fileName);
        for (std::string line; std::getline(f, line);) {
            if (line.rfind("ATOM", 0) != 0) continue;
            std::istringstream ss(line);
            std::vector<std::string> t;
            for (std::string b; ss >> b;) t.push_back(b);
            if (t.size() < 10) throw Error(IBIM_ERR_IO, "malformed ATOM line: " + line);
            centers.push_back({{std::stod(t[5]), std::stod(t[6]), std::stod(t[7])}});
            charges.push_back(std::stod(t[8]));
            radii.push_back(std::stod(t[9]));
        }
        N = (int)centers.size();
        if (N) getCenter();
    }
    // molecule.h:69-109
    void getCenter() {
        std::array<double, 3> lo = centers[0], hi = centers[0];
        for (int a = 0; a < 3; ++a) { lo[a] -= radii[0]; hi[a] += radii[0]; }
        for (int i = 1; i < N; ++i)
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], centers[i][a] - radii[i]);
                hi[a] = std::max(hi[a], centers[i][a] + radii[i]);
            }
        for (int a = 0; a < 3; ++a) center[a] = 0.5 * (lo[a] + hi[a]);
        radius = std::max(0.5 * (hi[0] - lo[0]), std::max(0.5 * (hi[1] - lo[1]), 0.5 * (hi[2] - lo[2])));
    }
    // molecule.h:112-125
    double centralize(double range) {
        const double s = range / radius;
        for (int i = 0; i < N; ++i) {
            for (int a = 0; a < 3; ++a) centers[i][a] = s * (centers[i][a] - center[a]);
            radii[i] *= s;
        }
        return s;
    }
    std::vector<double> flat_centers(double scale = 1.0) const {
        std::vector<double> c(3 * (size_t)N);
        for (int i = 0; i < N; ++i)
            for (int a = 0; a < 3; ++a) c[3 * i + a] = centers[i][a] * scale;
        return c;
    }
};

class levelset;

// Device grid.  Its origin and spacing come from the levelset that works on it (the reference
// keeps them there, levelset.h:35-38); the optional geometry arguments preset them.
class Grid {
  public:
    int Nx, Ny, Nz;
    ibim_grid h = nullptr;
    // Grid(Nx, Ny, Nz) (levelset.h:18): the reference leaves the values unset; zero here
    Grid(int nx, int ny, int nz) : Grid(0.0, nx, ny, nz) {}
    // Grid(val, Nx, Ny, Nz) (levelset.h:19)
    Grid(double val, int nx, int ny, int nz, double sx = 0, double sy = 0, double sz = 0, double dx = 1)
        : Nx(nx), Ny(ny), Nz(nz) {
        check(ibim_grid_create(context(), nx, ny, nz, sx, sy, sz, dx, val, &h));
    }
    Grid(const Grid &) = delete;
    ~Grid() { ibim_grid_destroy(h); }
    Grid &operator*=(double m) { check(ibim_grid_scale(h, m)); return *this; }
    Grid &operator=(const Grid &o) { check(ibim_grid_copy(h, o.h)); return *this; }
    std::vector<double> data() const {
        std::vector<double> v((size_t)Nx * Ny * Nz);
        check(ibim_grid_download(h, v.data()));
        return v;
    }
    // Grid::get clamps (levelset.cpp:28-33); reads go through a host copy
    double get(int i, int j, int k) const {
        i = std::min(std::max(i, 0), Nx - 1);
        j = std::min(std::max(j, 0), Ny - 1);
        k = std::min(std::max(k, 0), Nz - 1);
        return data()[((size_t)i * Ny + j) * Nz + k];
    }
    // Grid::set (levelset.cpp:35-37); writes go through a host copy
    void set(double val, int i, int j, int k) {
        std::vector<double> v = data();
        v[((size_t)i * Ny + j) * Nz + k] = val;
        check(ibim_grid_upload(h, v.data()));
    }
    void output(const std::string &file) const {
        std::ofstream f(file);
        for (double v : data()) f << v << "\n";
    }
};

class levelset {
  public:
    double dx, sx, sy, sz;
    int Nx, Ny, Nz, bandwidth, thickness;
    double thres;
    int jacobian = 0;  // opt-in key `jacobian`: surface Jacobian in the tube weights
    levelset(int nx, int ny, int nz, int band, double sx_, double sy_, double sz_, double dx_, Config &cfg)
        : dx(dx_), sx(sx_), sy(sy_), sz(sz_), Nx(nx), Ny(ny), Nz(nz), bandwidth(band) {
        thickness = (int)cfg.num("lvlset_thickness");
        thres = cfg.num("lvlset_thres");
        if (cfg.options.count("jacobian")) jacobian = (int)cfg.num("jacobian");
    }
    Grid *make_grid(double val) const { return new Grid(val, Nx, Ny, Nz, sx, sy, sz, dx); }
    void expand(Molecule &mol, Grid &g, double probe) {
        place(g);
        const std::vector<double> c = mol.flat_centers();
        check(ibim_levelset_expand(g.h, c.data(), mol.radii.data(), mol.N, probe, bandwidth));
    }
    void evolve(Grid &g, double final_t, double vel, double cfl) {
        place(g);
        check(ibim_levelset_evolve(g.h, final_t, vel, cfl));
    }
    int reinitialize(Grid &g, Grid &phi0, double final_t, double vel, double cfl) {
        place(g);
        place(phi0);
        int steps = 0;
        check(ibim_levelset_reinitialize(g.h, phi0.h, final_t, vel, cfl, thickness, thres, &steps));
        return steps;
    }
    long countGradient(Grid &g, double thick, double thr) {
        place(g);
        long bad = 0, total = 0;
        double acc = 0;
        check(ibim_levelset_count_gradient(g.h, thick, thr, &bad, &total, &acc));
        return bad;
    }
    // the grid takes this levelset's origin and spacing
    void place(Grid &g) const { check(ibim_grid_set_geometry(g.h, sx, sy, sz, dx)); }
};

class Surface {
  public:
    std::vector<std::array<double, 3>> nodes, normals;
    std::vector<double> weight;
    ibim_tube tube = nullptr;
    long inclusion = 0;
    double dx;
    Surface(Grid &g, levelset &ls, double /*s*/) : dx(ls.dx) {
        ls.place(g);
        long n = 0;
        check(ibim_surface_extract_jacobian(g.h, ls.thickness, ls.jacobian, &tube, &n, &inclusion));
        std::vector<double> p(3 * (size_t)n), q(3 * (size_t)n);
        weight.resize(n);
        check(ibim_tube_download(tube, p.data(), q.data(), weight.data()));
        nodes.resize(n);
        normals.resize(n);
        for (long i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) {
                nodes[i][a] = p[3 * i + a];
                normals[i][a] = q[3 * i + a];
            }
        std::cout << std::setw(15) << "INCLUSION" << " " << std::setw(8) << inclusion << std::endl;
    }
    Surface(const Surface &) = delete;
    ~Surface() { ibim_tube_destroy(tube); }
    void output(const std::string &file) const {
        std::ofstream f(file);
        for (const auto &p : nodes) f << p[0] << " " << p[1] << " " << p[2] << "\n";
    }
};

namespace bbfmm {
struct point {
    double x, y, z;
};
typedef std::vector<double> Vector;

// bbfmm::kernel with `eval` restricted to the reference's kernels (K1x..K4z = IBIM_K1X..IBIM_K4Z).
class kernel {
  public:
    int eval = -1;
    ibim_kernel_params kp{0.0, 80.0, 1.0, 1.0, 0};
    double h = 1.0;
    kernel() = default;
    kernel(const kernel &) = delete;
    ~kernel() {
        ibim_plan_destroy(plan_);
        ibim_tube_destroy(tube_);
    }
    void initialize(int nChebyshev, std::vector<point> &source, std::vector<point> &target, Vector &charge,
                    int nSource, int nTarget, int maxPoint, int maxLevel) {
        std::vector<double> s(3 * (size_t)nSource), zeros(3 * (size_t)nSource, 0.0), w(nSource, 0.0),
            t(3 * (size_t)nTarget);
        for (int i = 0; i < nSource; ++i) { s[3 * i] = source[i].x; s[3 * i + 1] = source[i].y; s[3 * i + 2] = source[i].z; }
        for (int i = 0; i < nTarget; ++i) { t[3 * i] = target[i].x; t[3 * i + 1] = target[i].y; t[3 * i + 2] = target[i].z; }
        check(ibim_tube_create(context(), s.data(), zeros.data(), w.data(), nSource, h, &tube_));
        check(ibim_fmm_plan(tube_, t.data(), nTarget, nChebyshev, maxPoint, maxLevel, IBIM_PRECISION_FP64, &plan_));
        charge_ = charge;
        nt_ = nTarget;
    }
    void run(Vector &out) {
        out.assign(nt_, 0.0);
        check(ibim_fmm_apply(plan_, eval, &kp, charge_.data(), out.data()));
    }

  private:
    ibim_tube tube_ = nullptr;
    ibim_plan plan_ = nullptr;
    Vector charge_;
    long nt_ = 0;
};
}  // namespace bbfmm

inline ibim_config config_from(const Config &cfg, const levelset &ls) {
    ibim_config c;
    ibim_config_default(&c);
    c.lo[0] = ls.sx; c.lo[1] = ls.sy; c.lo[2] = ls.sz;
    c.h = ls.dx;
    c.n[0] = ls.Nx; c.n[1] = ls.Ny; c.n[2] = ls.Nz;
    c.band = ls.bandwidth;
    c.thickness = ls.thickness;
    c.thres = ls.thres;
    c.np = (int)cfg.num("fmm_np");
    c.maxpoint = (int)cfg.num("fmm_maxpoint");
    c.maxlevel = (int)cfg.num("fmm_maxlevel");
    c.kp.kappa = cfg.num("solvent_kappa");
    c.kp.dE = cfg.num("solvent_dE");
    c.kp.dI = cfg.num("solvent_dI");
    c.kp.tau = cfg.num("tau");
    // opt-in modes with no counterpart in the reference (absent keys keep its behaviour)
    if (cfg.options.count("k3_scaled")) c.kp.k3_scaled = (int)cfg.num("k3_scaled");
    c.jacobian = ls.jacobian;
    c.restart = (int)cfg.num("gmres_restart");
    c.maxiter = (int)cfg.num("gmres_maxiter");
    c.tol = cfg.num("gmres_tol");
    return c;
}

typedef std::vector<double> Vector;

// int GMRES(std::function<Vector(Vector&)> A, Vector& x, Vector& b, int m, int max_iter, scalar_t tol)
// (gmres.h:20-21, gmres.cpp:50-164): restarted GMRES(m) on any operator A.  The Krylov basis,
// modified Gram-Schmidt and the updates run on the GPU in FP64 (ibim_gmres_host); every product
// A v is one call of A on a host Vector, as in the reference, starting with A x.  x holds the
// initial guess and receives the solution.  Returns 0 when converged, 1 when not (gmres.cpp:186);
// an exception thrown by A propagates to the caller with x unchanged.
inline int GMRES(const std::function<Vector(Vector &)> A, Vector &x, Vector &b, int m, int max_iter, double tol) {
    if (x.size() != b.size()) throw Error(IBIM_ERR_INVALID_ARGUMENT, "GMRES: x and b differ in length");
    struct Call {
        const std::function<Vector(Vector &)> *A;
        Vector in;
        std::exception_ptr err;
    } call{&A, Vector(), nullptr};
    auto tramp = +[](void *user, const double *xin, double *yout, long n) -> int {
        Call &c = *static_cast<Call *>(user);
        try {
            c.in.assign(xin, xin + n);
            const Vector y = (*c.A)(c.in);
            if ((long)y.size() != n) throw Error(IBIM_ERR_INVALID_ARGUMENT, "GMRES: the operator changed the length");
            std::copy(y.begin(), y.end(), yout);
            return 0;
        } catch (...) {
            c.err = std::current_exception();
            return 1;
        }
    };
    int iters = 0, matvecs = 0, status = 1;
    double resid = 0;
    const int st = ibim_gmres_host(context(), (long)b.size(), tramp, &call, b.data(), x.data(), m, max_iter, tol,
                                   &iters, &matvecs, &status, &resid);
    if (call.err) std::rethrow_exception(call.err);
    check(st);
    std::cout << (status == 0 ? "=============== CONVERGED =============" : "============= NOT CONVERGED ===========")
              << std::endl;
    return status;
}

// The BIE operator of electric() over a Surface, evaluated on the GPU: dmapping
// (electric.cpp:294-388) as the closure GMRES takes, and the right-hand side load
// (electric.cpp:395-412).  Vectors are (phi, dphi) of length 2N in the Surface's point order.
class BIEOperator {
  public:
    long N = 0;
    BIEOperator(levelset &ls, Surface &surf, Config &cfg, double rescale = 1.0) {
        N = (long)surf.nodes.size();
        std::vector<double> p(3 * (size_t)N), q(3 * (size_t)N);
        for (long i = 0; i < N; ++i)
            for (int a = 0; a < 3; ++a) {
                p[3 * i + a] = surf.nodes[i][a] / rescale;
                q[3 * i + a] = surf.normals[i][a];
            }
        check(ibim_tube_create(context(), p.data(), q.data(), surf.weight.data(), N, ls.dx / rescale, &tube_));
        kp_.kappa = cfg.num("solvent_kappa");
        kp_.dE = cfg.num("solvent_dE");
        kp_.dI = cfg.num("solvent_dI");
        kp_.tau = cfg.num("tau");
        kp_.k3_scaled = cfg.options.count("k3_scaled") ? (int)cfg.num("k3_scaled") : 0;
        check(ibim_fmm_plan(tube_, nullptr, 0, (int)cfg.num("fmm_np"), (int)cfg.num("fmm_maxpoint"),
                            (int)cfg.num("fmm_maxlevel"), IBIM_PRECISION_FP64, &plan_));
        rescale_ = rescale;
    }
    BIEOperator(const BIEOperator &) = delete;
    ~BIEOperator() {
        ibim_plan_destroy(plan_);
        ibim_tube_destroy(tube_);
    }
    Vector operator()(Vector &phi) const {
        if ((long)phi.size() != 2 * N) throw Error(IBIM_ERR_INVALID_ARGUMENT, "dmapping: length is not 2N");
        Vector y(2 * (size_t)N);
        check(ibim_bie_matvec(plan_, &kp_, phi.data(), y.data()));
        return y;
    }
    Vector load(Molecule &mol) const {
        const std::vector<double> c = mol.flat_centers(1.0 / rescale_);
        Vector b(2 * (size_t)N);
        check(ibim_bie_rhs(plan_, &kp_, c.data(), mol.charges.data(), mol.N, b.data()));
        return b;
    }

  private:
    ibim_tube tube_ = nullptr;
    ibim_plan plan_ = nullptr;
    ibim_kernel_params kp_{0.0, 80.0, 1.0, 1.0, 0};
    double rescale_ = 1.0;
};

// electric(Grid&, levelset&, Surface&, Molecule&, rescale, Config&) (electric.cpp:9-507): the
// solve in Angstrom (lengths divided by rescale), energy printed as the reference prints it,
// potent_file / energy_file written when the config names them.  Returns the energy.
inline double electric(Grid &, levelset &ls, Surface &surf, Molecule &mol, double rescale, Config &cfg) {
    const long n = (long)surf.nodes.size();
    std::vector<double> p(3 * (size_t)n), q(3 * (size_t)n);
    for (long i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            p[3 * i + a] = surf.nodes[i][a] / rescale;
            q[3 * i + a] = surf.normals[i][a];
        }
    ibim_tube t = nullptr;
    check(ibim_tube_create(context(), p.data(), q.data(), surf.weight.data(), n, ls.dx / rescale, &t));
    ibim_config c = config_from(cfg, ls);
    const std::vector<double> centers = mol.flat_centers(1.0 / rescale);
    std::vector<double> x(2 * (size_t)n), pot(mol.N);
    ibim_result r;
    const int st = ibim_electric(t, centers.data(), mol.charges.data(), mol.N, &c, x.data(), pot.data(), &r);
    ibim_tube_destroy(t);
    check(st);
    std::cout << std::setw(15) << "POINTS NUM" << " " << std::setw(8) << n << std::endl;
    std::cout << std::setw(15) << "AREA APPROX" << " " << std::setw(8) << r.area << " A^2" << std::endl;
    auto it = cfg.options.find("potent_file");
    if (it != cfg.options.end()) {
        std::ofstream f(it->second);
        for (double v : x) f << v << "\n";
    }
    it = cfg.options.find("energy_file");
    if (it != cfg.options.end()) {
        std::ofstream f(it->second);
        for (double v : pot) f << v << "\n";
    }
    std::cout << "polarized energy: " << std::setw(20) << std::scientific << r.energy << std::fixed << std::endl;
    return r.energy;
}

}  // namespace dropin
}  // namespace ibim

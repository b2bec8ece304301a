// Driver that runs the reference's own CPU code (levelset.cpp, bbfmm.{h,cpp},
// gmres.cpp, electric.cpp, compiled unmodified from the reference tree) on an
// explicit geometry, and dumps full-precision intermediates for the golden
// fixtures under tests/golden/.
//
// Test infrastructure only.  The reference's main.cpp:33-40 hard-wires a
// [-300,300]^3 box scaled to 2.5 x the molecule; this driver instead takes the
// box origin, grid size and spacing in Angstrom (rescale s = 1), and otherwise
// follows main.cpp:45-77 step by step:
//   expand(probe=1.4) -> evolve(1.4, vel=1, cfl=0.2) -> g *= -1 ->
//   reinitialize x2 (vel=1, cfl=0.5) -> Surface -> electric.
// The 16 BIE kernels are restated from electric.cpp:67-291 so that single
// FMMs and the GMRES solution can be dumped at 17 digits (electric() writes its
// files at 6 digits); electric() itself is also called and prints the energy.
//
// Usage: ibim_ref key=value ...   (see parse_args below for the keys)

#include "electric.h"

#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>

namespace {

std::map<std::string, std::string> g_args;

std::string arg(const std::string &k, const std::string &dflt = "") {
    auto it = g_args.find(k);
    return it == g_args.end() ? dflt : it->second;
}
double argf(const std::string &k, double d) { auto s = arg(k); return s.empty() ? d : atof(s.c_str()); }
int argi(const std::string &k, int d) { auto s = arg(k); return s.empty() ? d : atoi(s.c_str()); }

void dump(const std::string &path, const double *p, size_t n) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    fwrite(p, sizeof(double), n, f);
    fclose(f);
}

// Parameters of the BIE kernels (electric.cpp:52-58).
struct KP { double kappa, dE, dI, vr; };

// Restatement of the 16 kernels of electric.cpp:67-291, indexed
//  0 K1x 1 K1y 2 K1z 3 K2 4 K3xx 5 K3yy 6 K3zz 7 K3xy 8 K3yz 9 K3zx
// 10 K3yx 11 K3zy 12 K3xz 13 K4x 14 K4y 15 K4z
// (a = source, b = target; bbfmm.h:439,448-451).
double kern(int id, const KP &p, const bbfmm::point &a, const bbfmm::point &b) {
    const double dd[3] = {a.x - b.x, a.y - b.y, a.z - b.z};
    const double d = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
    const double r = sqrt(d);
    if (id == 3) {
        if (r < p.vr) {
            if (p.kappa == 0.) return 0.;
            return (exp(-p.kappa * p.vr) - 1.0 + p.kappa * p.vr) / p.kappa / 2.0 / M_PI / p.vr / p.vr;
        }
        return (1.0 - exp(-p.kappa * r)) / 4.0 / M_PI / r;
    }
    if (r < p.vr) return 0.;
    if (id <= 2) {
        return dd[id] * (p.dE / p.dI * exp(-p.kappa * r) * (p.kappa * r + 1) - 1.) / 4.0 / M_PI / r / d;
    }
    if (id >= 13) {
        return -dd[id - 13] * (p.dI / p.dE * exp(-p.kappa * r) * (p.kappa * r + 1) - 1.) / 4.0 / M_PI / r / d;
    }
    // K3 family: (df1, df2) per electric.cpp:103-266.
    static const int f1[9] = {0, 1, 2, 0, 1, 2, 0, 1, 2};
    static const int f2[9] = {0, 1, 2, 1, 2, 0, 1, 2, 0};
    const int k = id - 4;
    const double t = p.kappa * r;
    const double df1 = dd[f1[k]], df2 = dd[f2[k]];
    if (k < 3) {
        return (1 - exp(-t) * (t + 1)) * 1.0 / d / r + (exp(-t) * ((t + 3) * t + 3) - 3.0) * df1 * df2 / d / d / r;
    }
    return (exp(-t) * ((t + 3) * t + 3) - 3.0) * df1 * df2 / d / d / r;
}

// Density fed to each kernel (electric.cpp:333-348): 0 phiX, 1 phiY, 2 phiZ, 3 dphi.
const int kDensity[16] = {0, 1, 2, 3, 0, 1, 2, 0, 1, 2, 1, 2, 0, 3, 3, 3};

struct Tube {
    std::vector<bbfmm::point> pts;
    std::vector<double> w, nx, ny, nz;
};

void densities(const Tube &T, Vector &phi, Vector dens[4]) {
    const int N = (int)T.pts.size();
    for (int c = 0; c < 4; ++c) dens[c] = Vector(N);
    for (int i = 0; i < N; ++i) {
        dens[3](i) = phi(i + N) * T.w[i];
        dens[0](i) = phi(i) * T.nx[i] * T.w[i];
        dens[1](i) = phi(i) * T.ny[i] * T.w[i];
        dens[2](i) = phi(i) * T.nz[i] * T.w[i];
    }
}

void run16(const Tube &T, std::vector<bbfmm::point> &tgt, Vector dens[4], const KP &kp, int np, int maxPoint,
           int maxLevel, Vector out[16], const std::string &tree_dump) {
    std::vector<bbfmm::point> src = T.pts;
    for (int id = 0; id < 16; ++id) {
        bbfmm::kernel K;
        K.eval = [&kp, id](bbfmm::point &a, bbfmm::point &b) { return kern(id, kp, a, b); };
        K.initialize(np, src, tgt, dens[kDensity[id]], (int)src.size(), (int)tgt.size(), maxPoint, maxLevel);
        K.run(out[id]);
        if (id == 0 && !tree_dump.empty()) {
            FILE *f = fopen(tree_dump.c_str(), "w");
            for (size_t n = 0; n < K.t.dict.size(); ++n) {
                auto &nd = K.t.dict[n];
                fprintf(f, "%zu %d %d %d %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g", n, nd.nLevel, nd.parent,
                        (int)nd.isLeaf, (int)nd.isEmpty, nd.nSource, nd.nTarget, nd.center.x, nd.center.y,
                        nd.center.z, nd.radius.x, nd.radius.y, nd.radius.z);
                const unordered_set<index_t> *L[4] = {&nd.uList, &nd.vList, &nd.wList, &nd.xList};
                const char *nm[4] = {" U", " V", " W", " X"};
                for (int l = 0; l < 4; ++l) {
                    std::vector<int> v(L[l]->begin(), L[l]->end());
                    std::sort(v.begin(), v.end());
                    fprintf(f, "%s %zu", nm[l], v.size());
                    for (int x : v) fprintf(f, " %d", x);
                }
                fprintf(f, "\n");
            }
            fclose(f);
        }
    }
}

}  // namespace

int main(int argc, char **argv) {
    for (int i = 1; i < argc; ++i) {
        std::string s(argv[i]);
        auto eq = s.find('=');
        if (eq != std::string::npos) g_args[s.substr(0, eq)] = s.substr(eq + 1);
    }
    const std::string out = arg("out", ".");
    const int nx = argi("nx", 64), ny = argi("ny", nx), nz = argi("nz", nx);
    const double h = argf("h", 0.1875);
    const double lox = argf("lox", -6.0), loy = argf("loy", lox), loz = argf("loz", lox);
    const int band = argi("band", 8);
    const double init = argf("init", -2.0 * std::max(nx, std::max(ny, nz)));
    const double probe = argf("probe", 1.4);
    const double reinitT = argf("reinit_t", 1.0);

    Config cfg;
    const char *keys[] = {"lvlset_thickness", "lvlset_thres", "fmm_np", "fmm_maxpoint", "fmm_maxlevel",
                          "solvent_kappa", "solvent_dE", "solvent_dI", "tau", "gmres_restart",
                          "gmres_maxiter", "gmres_tol"};
    const char *dflt[] = {"3", "1e-4", "4", "64", "10", "0", "80", "1", "1.0", "30", "100", "1e-6"};
    for (int i = 0; i < 12; ++i) cfg.options[keys[i]] = arg(keys[i], dflt[i]);
    cfg.options["potent_file"] = out + "/ref.potent";
    cfg.options["energy_file"] = out + "/ref.energy";

    Molecule mol;
    mol.load(arg("pqr"));
    if (mol.centers.empty()) { fprintf(stderr, "no atoms in %s\n", arg("pqr").c_str()); return 2; }

    levelset ls(nx, ny, nz, band, lox, loy, loz, h, cfg);
    Grid g(init, nx, ny, nz);
    Grid phi0(0., nx, ny, nz);
    const size_t ncell = (size_t)nx * ny * nz;
    const bool grids = argi("dump_grids", 0) != 0;

    ls.expand(mol, g, probe);
    if (grids) dump(out + "/grid_expand.bin", g.data, ncell);
    ls.evolve(g, probe, 1.0, 0.2);
    if (grids) dump(out + "/grid_evolve.bin", g.data, ncell);
    g *= -1.0;
    phi0 = g;
    ls.reinitialize(g, phi0, reinitT, 1, 0.5);
    if (grids) dump(out + "/grid_reinit1.bin", g.data, ncell);
    phi0 = g;
    ls.reinitialize(g, phi0, reinitT, 1, 0.5);
    if (grids) dump(out + "/grid_reinit2.bin", g.data, ncell);

    Surface surf(g, ls, 1.0);
    if (grids) dump(out + "/grid_surface.bin", g.data, ncell);
    const int N = (int)surf.nodes.size();
    {
        std::vector<double> s7((size_t)N * 7);
        for (int i = 0; i < N; ++i) {
            for (int c = 0; c < 3; ++c) s7[(size_t)i * 7 + c] = surf.nodes[i].data[c];
            for (int c = 0; c < 3; ++c) s7[(size_t)i * 7 + 3 + c] = surf.normals[i].data[c];
            s7[(size_t)i * 7 + 6] = surf.weight[i];
        }
        dump(out + "/surface.bin", s7.data(), s7.size());
    }
    printf("REF_N %d\n", N);

    // Tube in Angstrom (electric.cpp:17-42 with rescale = 1).
    Tube T;
    const double dxa = ls.dx;
    for (int i = 0; i < N; ++i) {
        T.pts.emplace_back(surf.nodes[i].data[0], surf.nodes[i].data[1], surf.nodes[i].data[2]);
        T.w.push_back(surf.weight[i] * dxa * dxa * dxa);
        T.nx.push_back(surf.normals[i].data[0]);
        T.ny.push_back(surf.normals[i].data[1]);
        T.nz.push_back(surf.normals[i].data[2]);
    }
    KP kp{atof(cfg.options["solvent_kappa"].c_str()), atof(cfg.options["solvent_dE"].c_str()),
          atof(cfg.options["solvent_dI"].c_str()), atof(cfg.options["tau"].c_str()) * dxa};
    const int np = atoi(cfg.options["fmm_np"].c_str());
    const int maxPoint = atoi(cfg.options["fmm_maxpoint"].c_str());
    const int maxLevel = atoi(cfg.options["fmm_maxlevel"].c_str());

    if (argi("fmm_test", 0)) {
        // Deterministic test vector (2N): phi_i = sin(0.37 i) + 0.25, dphi_i = cos(0.11 i) - 0.5.
        Vector phi(2 * N);
        for (int i = 0; i < N; ++i) { phi(i) = sin(0.37 * i) + 0.25; phi(i + N) = cos(0.11 * i) - 0.5; }
        Vector dens[4], res[16];
        densities(T, phi, dens);
        std::vector<bbfmm::point> tgt = T.pts;
        run16(T, tgt, dens, kp, np, maxPoint, maxLevel, res, out + "/tree.txt");
        std::vector<double> all((size_t)16 * N);
        for (int k = 0; k < 16; ++k)
            for (int i = 0; i < N; ++i) all[(size_t)k * N + i] = res[k](i);
        dump(out + "/fmm16.bin", all.data(), all.size());
    }

    if (argi("solve", 0)) {
        // electric.cpp:294-388 (matvec) and :395-415 (right-hand side, GMRES).
        const double e1 = 0.5 * (1 + kp.dE / kp.dI), e2 = 0.5 * (1 + kp.dI / kp.dE);
        int nmatvec = 0;
        auto FullMap = [&](Vector &phi) {
            ++nmatvec;
            Vector dens[4], r[16];
            densities(T, phi, dens);
            std::vector<bbfmm::point> tgt = T.pts;
            run16(T, tgt, dens, kp, np, maxPoint, maxLevel, r, "");
            Vector o(2 * N);
            for (int i = 0; i < N; ++i) {
                double t1 = T.nx[i] * (r[4](i) + r[10](i) + r[9](i)) + T.ny[i] * (r[5](i) + r[7](i) + r[11](i)) +
                            T.nz[i] * (r[6](i) + r[12](i) + r[8](i));
                double t2 = T.nx[i] * r[13](i) + T.ny[i] * r[14](i) + T.nz[i] * r[15](i);
                o(i) = phi(i) + (r[0](i) + r[1](i) + r[2](i) - r[3](i)) / e1;
                o(i + N) = phi(i + N) + (t1 - t2) / e2;
            }
            return o;
        };
        Vector x(2 * N), b(2 * N);
        for (int i = 0; i < N; ++i) {
            for (int a = 0; a < mol.N; ++a) {
                const double dx = T.pts[i].x - mol.centers[a].data[0], dy = T.pts[i].y - mol.centers[a].data[1],
                             dz = T.pts[i].z - mol.centers[a].data[2];
                const double d = dx * dx + dy * dy + dz * dz, r = sqrt(d);
                b(i) += mol.charges[a] / kp.dI / 4.0 / M_PI / r / e1;
                b(i + N) -= mol.charges[a] / kp.dI / 4.0 / M_PI / d / r *
                            (T.nx[i] * dx + T.ny[i] * dy + T.nz[i] * dz) / e2;
            }
        }
        dump(out + "/rhs.bin", b.data(), 2 * (size_t)N);
        int rc = GMRES(FullMap, x, b, atoi(cfg.options["gmres_restart"].c_str()),
                       atoi(cfg.options["gmres_maxiter"].c_str()), atof(cfg.options["gmres_tol"].c_str()));
        dump(out + "/solution.bin", x.data(), 2 * (size_t)N);
        // polarizeMap (electric.cpp:442-485): 4 FMMs with the atoms as targets.
        std::vector<bbfmm::point> atoms;
        for (int a = 0; a < mol.N; ++a)
            atoms.emplace_back(mol.centers[a].data[0], mol.centers[a].data[1], mol.centers[a].data[2]);
        Vector dens[4];
        densities(T, x, dens);
        std::vector<double> pot(mol.N, 0.0);
        const int ids[4] = {0, 1, 2, 3};
        std::vector<bbfmm::point> src = T.pts;
        for (int q = 0; q < 4; ++q) {
            const int id = ids[q];
            bbfmm::kernel K;
            K.eval = [&kp, id](bbfmm::point &a, bbfmm::point &bb) { return kern(id, kp, a, bb); };
            K.initialize(np, src, atoms, dens[kDensity[id]], N, mol.N, maxPoint, maxLevel);
            Vector r;
            K.run(r);
            for (int a = 0; a < mol.N; ++a) pot[a] += (id == 3 ? r(a) : -r(a));
        }
        dump(out + "/atom_potential.bin", pot.data(), pot.size());
        double E = 0;
        for (int a = 0; a < mol.N; ++a) E += pot[a] * mol.charges[a];
        E *= 0.5;
        printf("REF_GMRES_RC %d\nREF_MATVECS %d\nREF_ENERGY_RESTATED %.17e\n", rc, nmatvec, E);
    }

    if (argi("electric", 0)) {
        std::cout.precision(17);
        electric(g, ls, surf, mol, 1.0, cfg);
    }
    fflush(stdout);
    return 0;
}

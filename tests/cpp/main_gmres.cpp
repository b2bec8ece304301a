// electric.cpp:390-415 of the reference written against the drop-in classes: the level set and
// Surface of main.cpp:45-64 (grids sized and placed by the levelset, as there), then the BIE
// closure FullMap, the right-hand side `load`, and GMRES(FullMap, start, load, m, max_iter, tol)
// exactly as electric.cpp:415 calls it.  The closure counts its calls.
// Usage: main_gmres <input.cfg>   (keys as main_dropin.cpp, with the box as nx ny nz lox loy loz;
// out_file = where to write the solution)
#include <cstdio>

#include "ibim/dropin.hpp"

using namespace ibim::dropin;

int main(int argc, char *argv[]) {
    if (argc <= 1) {
        std::cout << "USE " << argv[0] << " PATH_OF_CONFIG_FILE" << std::endl;
        return 0;
    }
    try {
        Config cfg;
        std::ifstream cfgFile(argv[1]);
        cfg.parse(cfgFile);
        Molecule mol;
        mol.load(cfg.options["pqr_file"]);
        // box: nx ny nz / lox loy loz (the reference's oracle driver's explicit geometry)
        const double h = cfg.num("h");
        const int nx = (int)cfg.num("nx"), ny = (int)cfg.num("ny"), nz = (int)cfg.num("nz");
        const int size = std::max(nx, std::max(ny, nz));
        levelset ls(nx, ny, nz, 8, cfg.num("lox"), cfg.num("loy"), cfg.num("loz"), h, cfg);
        Grid g(-2.0 * size, ls.Nx, ls.Ny, ls.Nz);
        Grid phi0(ls.Nx, ls.Ny, ls.Nz);
        ls.expand(mol, g, 1.4);
        ls.evolve(g, 1.4, 1.0, 0.2);
        g *= -1.0;
        phi0 = g;
        ls.reinitialize(g, phi0, cfg.num("reinit_step"), 1, 0.5);
        phi0 = g;
        ls.reinitialize(g, phi0, cfg.num("reinit_step"), 1, 0.5);
        Surface surf(g, ls, 1.0);
        const long N = (long)surf.nodes.size();

        BIEOperator dmapping(ls, surf, cfg);
        long calls = 0;
        auto FullMap = [&](Vector &phi) {
            ++calls;
            return dmapping(phi);
        };
        Vector start(2 * N, 0.);
        Vector load = dmapping.load(mol);
        const int rc = GMRES(FullMap, start, load, atoi(cfg.options["gmres_restart"].c_str()),
                             atoi(cfg.options["gmres_maxiter"].c_str()), atof(cfg.options["gmres_tol"].c_str()));
        std::FILE *f = std::fopen(cfg.options["out_file"].c_str(), "wb");
        if (!f) throw Error(IBIM_ERR_IO, "cannot write " + cfg.options["out_file"]);
        std::fwrite(start.data(), sizeof(double), start.size(), f);
        std::fclose(f);
        std::printf("DROPIN_POINTS %ld\nDROPIN_GMRES_RC %d\nDROPIN_MATVECS %ld\n", N, rc, calls);
    } catch (const Error &e) {
        std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
        return 2;
    }
    return 0;
}

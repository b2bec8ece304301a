// main.cpp:14-79 of the reference written against the drop-in classes (include/ibim/dropin.hpp),
// with an explicit box instead of the hard-wired [-300, 300]^3 rescaling: the same sequence of
// calls (grids sized by the levelset and placed by it, main.cpp:47-48), executed on the GPU.  Usage: main_dropin <input.cfg>
// (keys: pqr_file, lo, h, n, reinit_step, plus the reference's lvlset_*, fmm_*, solvent_*, tau,
// gmres_*, potent_file, energy_file keys; optional grid_file / node_file).
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
        const double lo = cfg.num("lo"), h = cfg.num("h");
        const int size = (int)cfg.num("n");
        levelset ls(size, size, size, 8, lo, lo, lo, h, cfg);
        Grid g(-2.0 * size, ls.Nx, ls.Ny, ls.Nz);
        Grid phi0(0., ls.Nx, ls.Ny, ls.Nz);
        ls.expand(mol, g, 1.4);
        ls.evolve(g, 1.4, 1.0, 0.2);
        g *= -1.0;
        phi0 = g;
        ls.reinitialize(g, phi0, cfg.num("reinit_step"), 1, 0.5);
        phi0 = g;
        ls.reinitialize(g, phi0, cfg.num("reinit_step"), 1, 0.5);
        Surface surf(g, ls, 1.0);
        // main.cpp:70-73 writes these under -DGRID; here when the config names the files
        if (cfg.options.count("grid_file")) g.output(cfg.options["grid_file"]);
        if (cfg.options.count("node_file")) surf.output(cfg.options["node_file"]);
        const double E = electric(g, ls, surf, mol, 1.0, cfg);
        std::printf("DROPIN_POINTS %zu\nDROPIN_ENERGY %.17e\n", surf.nodes.size(), E);
    } catch (const Error &e) {
        std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
        return 2;
    }
    return 0;
}

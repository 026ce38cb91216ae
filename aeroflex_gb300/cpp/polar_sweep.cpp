// Alpha sweep through the C++ layer (include/afx_rans.hpp), in the call
// order of AeroFLEX's driver (src/aeroflex/src/app.cpp:168-188):
// Settings from an INI file, compute_alphas(), solve_airfoil(mesh, db).
//
//   polar_sweep <config.ini> <mesh.msh> [<finer mesh.msh> ...]
//
// With several meshes they are solved in sequence for every angle, coarse to
// fine, as the reference's two-level multigrid run (rans.h:84-85).
// Prints one line per angle: alpha cl cd cm.
#include <cstdio>
#include <string>
#include <vector>

#include "afx_rans.hpp"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s config.ini mesh.msh\n", argv[0]);
        return 2;
    }
    try {
        rans::Rans r;
        r.settings.import_config_file(argv[1]);
        r.compute_alphas();
        rans::airfoil_db db;
        std::vector<std::string> levels(argv + 2, argv + argc);
        r.solve_airfoil(levels, db);
        for (size_t i = 0; i < db.alpha.size(); ++i)
            std::printf("%.6f %.17g %.17g %.17g\n", db.alpha[i], db.cl[i], db.cd[i], db.cmy[i]);
        std::printf("iterations %d\n", (int)r.iters);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}

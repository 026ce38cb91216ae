// Config 5's beam and coupling through the C++ layer (include/afx_coupling.hpp).
//
//   beam_coupling beam
//       the 50-element beam (EI 1e4, 1 m) under a uniform load of 1 N/m
//       (consistent nodal loads, 40,000 midpoints) and under a 3 N tip force:
//       prints the nodal deflections and slopes of both (host only)
//   beam_coupling couple <config.ini> <mesh.msh> <iterations>
//       the coupling loop on an FP64 implicit solver of the config's settings:
//       prints one line per iteration (cl cd tip deflection step size)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "afx_coupling.hpp"

static void print(const std::vector<double>& u) {
    for (double v : u) std::printf("%.17g ", v);
    std::printf("\n");
}

int main(int argc, char** argv) {
    try {
        if (argc >= 2 && std::strcmp(argv[1], "beam") == 0) {
            coupling::Beam b(50, 1e4, 1.0);
            std::vector<double> F(b.n_dof(), 0.0), row;
            const int n = 40000;
            for (int i = 0; i < n; ++i) {
                b.shape_row((i + 0.5) / n, row);
                for (int j = 0; j < b.n_dof(); ++j) F[j] += row[j] * (1.0 / n);
            }
            b.set_Load_Vector_From_Vector(F);
            print(b.get_Lin_Solve());
            std::vector<double> P(b.n_dof(), 0.0);
            P[b.n_dof() - 2] = 3.0;
            print(b.get_Solve(P));
            return 0;
        }
        if (argc >= 5 && std::strcmp(argv[1], "couple") == 0) {
            rans::Settings st(argv[2]);
            rans::mesh m(argv[3]);
            rans::solver s(m, st);
            s.init();
            coupling::Beam b(50, 1e4);
            const std::vector<double> v = st.bc_vars("farfield");  // T, mach, angle, p
            coupling::Coupling c(s, m, b, coupling::sea_level_dynamic_pressure(v[1]));
            for (int k = 0; k < std::atoi(argv[4]); ++k) {
                const auto& e = c.step(v[2]);
                std::printf("%.17g %.17g %.17g %.17g\n", e.cl, e.cd, e.tip_deflection_m, e.step_norm_m);
            }
            return 0;
        }
        std::fprintf(stderr, "usage: %s beam | couple config.ini mesh.msh iterations\n", argv[0]);
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
}

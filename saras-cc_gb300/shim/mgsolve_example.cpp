// Example caller of the C++ drop-in: reads a SARAS parameters.yaml, fills a
// right-hand side cos(2 pi x) cos(2 pi y) cos(2 pi z) (compatible with
// Neumann walls on a uniform grid) and calls multigrid_d3::mgSolve exactly as
// lsRK3_d3::timeAdvance does in the reference.
//
//   mgsolve_example parameters.yaml [--parse-only]
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>

#include "saras_shim.h"

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s parameters.yaml [--parse-only]\n", argv[0]);
        return 2;
    }
    saras_shim::parser p;
    std::unique_ptr<saras_shim::grid> gp;
    try {
        p = saras_shim::parser(argv[1]);
        gp.reset(new saras_shim::grid(p));
    } catch (const std::exception &e) {
        // the reference prints the same ERROR line and ends the job
        std::printf("%s\n", e.what());
        return 3;
    }
    const saras_shim::grid &g = *gp;
    std::printf("grid %dx%dx%d mesh %s domain %s levels %d vcCount %d tol %.1e pre/post %d/%d\n", p.Nx, p.Ny, p.Nz,
                p.meshType.c_str(), p.domainType.c_str(), saras_reference_levels(&g.desc), p.vcCount, p.vcTolerance,
                p.preSmooth, p.postSmooth);
    if (argc > 2 && std::strcmp(argv[2], "--parse-only") == 0) return 0;
    saras_shim::plainsf rhs(g), lhs(g);
    const double pi = std::acos(-1.0);
    for (int i = 0; i < p.Nx; i++)
        for (int j = 0; j < p.Ny; j++)
            for (int k = 0; k < p.Nz; k++)
                rhs.F(i, j, k) = std::cos(2 * pi * (i + 0.5) / p.Nx) * std::cos(2 * pi * (j + 0.5) / p.Ny) *
                                 std::cos(2 * pi * (k + 0.5) / p.Nz);
    try {
        saras_shim::multigrid_d3 mg(g, p);
        mg.mgSolve(lhs, rhs);
        // analytic solution of the continuous problem: -f / (12 pi^2)
        double err = 0.0, mean = 0.0, emean = 0.0;
        const double n = (double)p.Nx * p.Ny * p.Nz;
        for (int i = 0; i < p.Nx; i++)
            for (int j = 0; j < p.Ny; j++)
                for (int k = 0; k < p.Nz; k++) {
                    mean += lhs.F(i, j, k) / n;
                    emean += -rhs.F(i, j, k) / (12 * pi * pi) / n;
                }
        for (int i = 0; i < p.Nx; i++)
            for (int j = 0; j < p.Ny; j++)
                for (int k = 0; k < p.Nz; k++)
                    err = std::fmax(err, std::fabs((lhs.F(i, j, k) - mean) - (-rhs.F(i, j, k) / (12 * pi * pi) - emean)));
        std::printf("mgSolve: %d V-cycles, max deviation from -f/(12 pi^2): %.3e\n", mg.lastCycles, err);
    } catch (const std::exception &e) {
        std::printf("error: %s\n", e.what());
        return 3;
    }
    return 0;
}

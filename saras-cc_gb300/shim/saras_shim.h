// saras_shim.h -- C++ drop-in for SARAS-CC's multigrid and time-step classes over
// the GB300 C ABI (include/saras_gb300.h).
//
// A caller of the reference keeps its code: it builds a `parser` from
// parameters.yaml (the reference's key names), a `grid`, `plainsf` fields
// indexed from -pad, and calls multigrid_d3::mgSolve(outLHS, inpRHS) or
// lsRK3_d3::timeAdvance(V, P, T).  The classes mirror, for the hot path only:
//   parser          lib/io/parser.h (keys read at parser.cc:69-284, checks of
//                   parser.cc:299-411 thrown as std::invalid_argument)
//   grid            lib/grid/grid.h (sizes, pads, periodicity)
//   plainsf         lib/field/plainsf.h (F(i,j,k) from -pad, row-major, k fastest)
//   multigrid_d3/_d2 lib/poisson/poisson.h:148-205
//   lsRK3_d3/_d2, eulerCN_d3/_d2  lib/timestep/timestep.h (timeAdvance)
// Blitz++, MPI, yaml-cpp and HDF5 are not needed: fields are std::vector
// storage with the Blitz layout, and the YAML reader handles the flat
// "key": value form of the reference's parameters files.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/saras_gb300.h"

namespace saras_shim {

// ------------------------------------------------------------------ parser
class parser {
  public:
    // Program
    int probType = 5, rbcType = 2, forceType = 3;
    double Re = 1000, Ra = 1e7, Pr = 1.0;
    double Lx = 1, Ly = 1, Lz = 1;
    double gAxis[3] = {0, 0, -1};
    std::string domainType = "PPN";
    // Mesh
    std::string meshType = "UUU";
    double betaX = 1, betaY = 1, betaZ = 1;
    int Nx = 32, Ny = 32, Nz = 32;
    // Solver
    int dScheme = 1, nlScheme = 1, iScheme = 2;
    double cnTolerance = 1e-6, tStp = 1e-3;
    double tMax = std::numeric_limits<double>::infinity();  // "Final Time"; unchecked when absent
    double peLimit = 2.0, upParam = 0.8;
    // Multigrid
    int vcCount = 20, preSmooth = 3, postSmooth = 6, resType = 0;
    bool solveFlag = true, printResidual = false;
    double vcTolerance = 1e-6, mgTolerance = 1e-2, sorParam = 1.0;
    bool xPer = true, yPer = true, zPer = false;
    bool planar = false;

    parser() = default;

    // Reads the flat "Section": / "Key": value layout of parameters.yaml.
    explicit parser(const std::string &path, bool planar_build = false) : planar(planar_build) {
        std::ifstream in(path);
        if (!in) throw std::runtime_error("cannot open " + path);
        std::string line, section;
        while (std::getline(in, line)) {
            const size_t hash = line.find('#');
            if (hash != std::string::npos) line = line.substr(0, hash);
            if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
            const bool indented = line[0] == ' ' || line[0] == '\t';
            const size_t q0 = line.find('"'), q1 = line.find('"', q0 + 1);
            if (q0 == std::string::npos || q1 == std::string::npos) continue;
            const std::string key = line.substr(q0 + 1, q1 - q0 - 1);
            std::string val = line.substr(line.find(':', q1) + 1);
            val.erase(0, val.find_first_not_of(" \t"));
            while (!val.empty() && (val.back() == '\r' || val.back() == ' ')) val.pop_back();
            if (!indented) {
                section = key;
                continue;
            }
            kv[section + "/" + key] = val;
        }
        read();
        checkData();
    }

    std::map<std::string, std::string> kv;

    // parser::checkData (parser.cc:299-411), the checks that concern this
    // path, with the reference's messages.  The reference prints an ERROR
    // and ends the MPI job; a library cannot end its caller's process, so
    // the message is thrown as std::invalid_argument instead.  A WARNING is
    // printed and the value adjusted, as in the reference.
    void checkData() {
        auto fail = [](const std::string &m) { throw std::invalid_argument("ERROR: " + m + ". Aborting"); };
        if (Nx < 2) fail("Insufficient number of points along X axis");
        if (planar) {
            if (Ny != 1) {
                std::cout << "WARNING: The number of points along Y is greater than 1 although solver has been "
                             "compiled with PLANAR flag. Resetting Y Size to 1"
                          << std::endl;
                Ny = 1;
            }
        } else if (Ny == 1) {
            fail("Insufficient number of points along Y axis");
        }
        if (Nz < 2) fail("Insufficient number of points along Z axis");
        if (domainType.length() != 3) fail("Domain type string is not correct");
        if (meshType.length() != 3) fail("Mesh type string is not correct");
        if (tStp > tMax) fail("Time step is larger than the maximum duration assigned for simulation");
        if (resType > 2) fail("The specified value for printing error at end of V-Cycles is not defined");
    }

  private:
    static std::string unq(std::string s) {
        if (s.size() >= 2 && s.front() == '"') s = s.substr(1, s.size() - 2);
        return s;
    }
    bool has(const std::string &k) const { return kv.count(k) > 0; }
    double num(const std::string &k, double d) const { return has(k) ? std::stod(kv.at(k)) : d; }
    bool flag(const std::string &k, bool d) const {
        if (!has(k)) return d;
        const std::string v = kv.at(k);
        return v == "true" || v == "True" || v == "1";
    }
    void read() {
        probType = (int)num("Program/Problem Type", probType);
        rbcType = (int)num("Program/RBC Type", rbcType);
        forceType = (int)num("Program/Force", forceType);
        Re = num("Program/Reynolds Number", Re);
        Ra = num("Program/Rayleigh Number", Ra);
        Pr = num("Program/Prandtl Number", Pr);
        Lx = num("Program/X Length", Lx);
        Ly = num("Program/Y Length", Ly);
        Lz = num("Program/Z Length", Lz);
        if (has("Program/Domain Type")) domainType = unq(kv["Program/Domain Type"]);
        if (has("Program/Gravity Direction")) {
            std::string v = kv["Program/Gravity Direction"];
            for (char &c : v)
                if (c == '[' || c == ']' || c == ',') c = ' ';
            std::istringstream is(v);
            is >> gAxis[0] >> gAxis[1] >> gAxis[2];
        }
        if (has("Mesh/Mesh Type")) meshType = unq(kv["Mesh/Mesh Type"]);
        betaX = num("Mesh/X Beta", betaX);
        betaY = num("Mesh/Y Beta", betaY);
        betaZ = num("Mesh/Z Beta", betaZ);
        Nx = (int)num("Mesh/X Size", Nx);
        Ny = (int)num("Mesh/Y Size", Ny);
        Nz = (int)num("Mesh/Z Size", Nz);
        dScheme = (int)num("Solver/Differentiation Scheme", dScheme);
        nlScheme = (int)num("Solver/Non-Linear Term", nlScheme);
        iScheme = (int)num("Solver/Integration Scheme", iScheme);
        peLimit = num("Solver/Peclet Limit", peLimit);
        upParam = num("Solver/Central Bias", upParam);
        cnTolerance = num("Solver/Solve Tolerance", cnTolerance);
        tStp = num("Solver/Time-Step", tStp);
        tMax = num("Solver/Final Time", tMax);
        vcCount = (int)num("Multigrid/V-Cycle Count", vcCount);
        vcTolerance = num("Multigrid/Residual Tolerance", vcTolerance);
        solveFlag = flag("Multigrid/Solve Coarsest", solveFlag);
        mgTolerance = num("Multigrid/Solve Tolerance", mgTolerance);
        sorParam = num("Multigrid/SOR Parameter", sorParam);
        preSmooth = (int)num("Multigrid/Pre-Smoothing Count", preSmooth);
        postSmooth = (int)num("Multigrid/Post-Smoothing Count", postSmooth);
        resType = (int)num("Multigrid/Residual Type", resType);
        printResidual = flag("Multigrid/Print Residual", printResidual);
        // parser::setPeriodicity (parser.cc:460-469)
        xPer = domainType.size() > 0 && domainType[0] != 'N';
        yPer = domainType.size() > 1 && domainType[1] != 'N';
        zPer = domainType.size() > 2 && domainType[2] != 'N';
    }
};

inline int mesh_code(char c) { return c == 'S' ? SARAS_MESH_SINGLE_TANH : (c == 'D' ? SARAS_MESH_DOUBLE_TANH : 0); }

// -------------------------------------------------------------------- grid
class grid {
  public:
    const parser &inputParams;
    int pad;
    int dims;
    saras_grid_desc desc{};

    explicit grid(const parser &p) : inputParams(p) {
        // the pad from the differentiation scheme (grid.cc:69-77)
        if (p.dScheme == 1) {
            pad = 1;
        } else if (p.dScheme == 2) {
            pad = 2;
        } else {
            throw std::invalid_argument("Undefined finite differencing scheme in YAML file. ABORTING");
        }
        dims = p.planar ? 2 : 3;
        desc.dims = dims;
        desc.n[0] = p.Nx;
        desc.n[1] = p.planar ? 1 : p.Ny;
        desc.n[2] = p.Nz;
        desc.len[0] = p.Lx;
        desc.len[1] = p.Ly;
        desc.len[2] = p.Lz;
        for (int d = 0; d < 3; d++) desc.mesh_type[d] = mesh_code(p.meshType.size() > (size_t)d ? p.meshType[d] : 'U');
        desc.beta[0] = p.betaX;
        desc.beta[1] = p.betaY;
        desc.beta[2] = p.betaZ;
        desc.periodic[0] = p.xPer;
        desc.periodic[1] = p.yPer;
        desc.periodic[2] = p.zPer;
        desc.pad = pad;
        // grid::checkAnisotropy runs when an axis is stretched (grid.cc:117-142)
        bool stretched = false;
        for (int d = 0; d < 3; d++) stretched = stretched || (desc.mesh_type[d] != 0 && (dims == 3 || d != 1));
        if (stretched) {
            const double ar = anisotropy();
            if (ar > 7.0)
                std::cout << "\nWARNING: Grid anisotropy exceeds limits. Finite-difference calculations will be "
                             "inaccurate"
                          << std::endl;
            else
                std::cout << "\nMaximum grid anisotropy is " << ar << std::endl;
        }
    }

    // grid::checkAnisotropy (grid.cc:756-804): the largest ratio of two
    // widths of a cell, over the core cells and the ghost layer (widths
    // between consecutive centres -1..N along each axis); 0 when the host
    // metrics cannot be formed (no V-cycle hierarchy for these sizes).
    double anisotropy() const {
        double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++) {
            if (dims == 2 && d == 1) continue;
            std::vector<double> x((size_t)desc.n[d] + 2);
            int32_t n = 0;
            if (saras_grid_metrics(&desc, 0, 0, d, x.data(), nullptr, nullptr, &n) != SARAS_OK) return 0.0;
            lo[d] = std::numeric_limits<double>::infinity();
            for (int i = 0; i <= n; i++) {
                const double w = std::fabs(x[(size_t)i + 1] - x[(size_t)i]);
                lo[d] = std::min(lo[d], w);
                hi[d] = std::max(hi[d], w);
            }
        }
        double ar = 0.0;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                if (a != b && hi[a] > 0.0 && lo[b] > 0.0) ar = std::max(ar, hi[a] / lo[b]);
        return ar;
    }
};

// ----------------------------------------------------------------- plainsf
class plainsf {
  public:
    int n[3], p[3];
    std::vector<double> data;

    explicit plainsf(const grid &g) {
        for (int d = 0; d < 3; d++) {
            n[d] = g.desc.n[d];
            p[d] = (g.dims == 2 && d == 1) ? 1 : g.pad;
        }
        data.assign((size_t)(n[0] + 2 * p[0]) * (n[1] + 2 * p[1]) * (n[2] + 2 * p[2]), 0.0);
    }
    int64_t s0() const { return (int64_t)(n[1] + 2 * p[1]) * (n[2] + 2 * p[2]); }
    int64_t s1() const { return n[2] + 2 * p[2]; }
    double &F(int i, int j, int k) { return data[(size_t)((i + p[0]) * s0() + (j + p[1]) * s1() + (k + p[2]))]; }
    double F(int i, int j, int k) const {
        return data[(size_t)((i + p[0]) * s0() + (j + p[1]) * s1() + (k + p[2]))];
    }
    double *origin() { return data.data() + (p[0] * s0() + p[1] * s1() + p[2]); }
    const double *origin() const { return data.data() + (p[0] * s0() + p[1] * s1() + p[2]); }
    void strides(int64_t st[3]) const {
        st[0] = s0();
        st[1] = s1();
        st[2] = 1;
    }
};

using sfield = plainsf;  // the RK3 shim carries scalar fields as plain arrays

struct vfield {
    plainsf Vx, Vy, Vz;
    explicit vfield(const grid &g) : Vx(g), Vy(g), Vz(g) {}
};

inline void check(saras_status s, const char *what) {
    if (s != SARAS_OK && s != SARAS_NOT_CONVERGED)
        throw std::runtime_error(std::string(what) + ": " + saras_status_string(s) + " " + saras_last_error());
}

inline saras_mg_params mg_params_from(const parser &p) {
    saras_mg_params m;
    saras_mg_default_params(&m);
    m.vc_count = p.vcCount;
    m.vc_tolerance = p.vcTolerance;
    m.solve_flag = p.solveFlag;
    m.mg_tolerance = p.mgTolerance;
    m.sor_param = p.sorParam;
    m.pre_smooth = p.preSmooth;
    m.post_smooth = p.postSmooth;
    m.res_type = p.resType;
    m.print_residual = p.printResidual;
    return m;
}

// ----------------------------------------------------------------- poisson
class poisson {
  public:
    poisson(const grid &mesh, const parser &solParam, int precision = SARAS_PREC_FP64_EXACT)
        : mesh(mesh), inputParams(solParam) {
        saras_mg_params m = mg_params_from(solParam);
        m.precision = precision;
        check(saras_mg_create(&mesh.desc, &m, nullptr, &h), "saras_mg_create");
    }
    virtual ~poisson() { saras_mg_destroy(h); }
    poisson(const poisson &) = delete;
    poisson &operator=(const poisson &) = delete;

    // poisson::mgSolve (lib/poisson/poisson.cc:109-189)
    void mgSolve(plainsf &outLHS, const plainsf &inpRHS) {
        int64_t st[3];
        outLHS.strides(st);
        int32_t cycles = 0;
        check(saras_mg_solve(h, outLHS.origin(), inpRHS.origin(), st, nullptr, 0, &cycles), "mgSolve");
        lastCycles = cycles;
    }
    int lastCycles = 0;

  protected:
    const grid &mesh;
    const parser &inputParams;
    saras_mg *h = nullptr;
};

class multigrid_d3 : public poisson {
  public:
    multigrid_d3(const grid &mesh, const parser &solParam, int precision = SARAS_PREC_FP64_EXACT)
        : poisson(mesh, solParam, precision) {}
};

class multigrid_d2 : public poisson {
  public:
    multigrid_d2(const grid &mesh, const parser &solParam, int precision = SARAS_PREC_FP64_EXACT)
        : poisson(mesh, solParam, precision) {}
};

// ------------------------------------------------------------------- RK3
// The time integrator with the RBC boundary conditions of scalar::initTBCs /
// hydro::initVBCs / initPBCs for probType 5 (no-slip, hot bottom, cold top).
// lsRK3_d3 runs the low-storage RK3 (lsRK3_d3.cc:190-305), eulerCN_d3 the
// Euler/Crank-Nicolson step (eulerCN_d3.cc:178-268); the differentiation and
// non-linear schemes, "Peclet Limit" and "Central Bias" come from the parser.
// stencil_form SARAS_STENCIL_FAST takes the time-step stencils with fused
// multiply-adds (equal to the reference's arithmetic to rounding).
class timeIntegrator {
  public:
    timeIntegrator(const grid &mesh, const double &dt, int integration, int mg_precision,
                   int stencil_form = SARAS_STENCIL_EXACT)
        : mesh(mesh) {
        const parser &p = mesh.inputParams;
        saras_rk3_params r{};
        double fb = 1.0;
        check(saras_rbc_coefficients(p.rbcType, p.Ra, p.Pr, &r.nu, &r.kappa, &fb), "rbc coefficients");
        const double gn = std::sqrt(p.gAxis[0] * p.gAxis[0] + p.gAxis[1] * p.gAxis[1] + p.gAxis[2] * p.gAxis[2]);
        for (int d = 0; d < 3; d++) r.g_terms[d] = fb * p.gAxis[d] / gn;
        r.dt = dt;
        r.cn_tolerance = p.cnTolerance;
        r.with_scalar = 1;
        r.nl_scheme = p.nlScheme;
        r.pe_limit = p.peLimit;
        r.up_param = p.upParam;
        r.integration = integration;
        r.stencil_form = stencil_form;
        for (int f = 0; f < 6; f++) {
            r.bc_vx.type[f] = r.bc_vy.type[f] = r.bc_vz.type[f] = SARAS_FBC_DIRICHLET;
            r.bc_p.type[f] = SARAS_FBC_NEUMANN;
            r.bc_t.type[f] = f < 4 ? SARAS_FBC_NEUMANN : SARAS_FBC_DIRICHLET;
        }
        r.bc_t.value[4] = 1.0;
        r.mg = mg_params_from(p);
        r.mg.precision = mg_precision;
        check(saras_rk3_create(&mesh.desc, &r, nullptr, &h), "saras_rk3_create");
    }
    virtual ~timeIntegrator() { saras_rk3_destroy(h); }
    timeIntegrator(const timeIntegrator &) = delete;
    timeIntegrator &operator=(const timeIntegrator &) = delete;

    // timeAdvance(V, P, T); the fields are copied to the device and back
    // around each call.
    void timeAdvance(vfield &V, sfield &P, sfield &T) {
        int64_t st[3];
        P.strides(st);
        check(saras_rk3_upload(h, V.Vx.origin(), V.Vy.origin(), V.Vz.origin(), P.origin(), T.origin(),
                               primed ? nullptr : Pp.origin(), st),
              "upload");
        primed = true;
        check(saras_rk3_step(h, 1, nullptr, nullptr), "timeAdvance");
        check(saras_rk3_download(h, V.Vx.origin(), V.Vy.origin(), V.Vz.origin(), P.origin(), T.origin(), nullptr,
                                 st),
              "download");
    }

  private:
    const grid &mesh;
    saras_rk3 *h = nullptr;
    plainsf Pp{mesh};
    bool primed = false;
};

class lsRK3_d3 : public timeIntegrator {
  public:
    lsRK3_d3(const grid &mesh, const double &dt, int mg_precision = SARAS_PREC_FP64_EXACT,
             int stencil_form = SARAS_STENCIL_EXACT)
        : timeIntegrator(mesh, dt, 2, mg_precision, stencil_form) {}
};

class eulerCN_d3 : public timeIntegrator {
  public:
    eulerCN_d3(const grid &mesh, const double &dt, int mg_precision = SARAS_PREC_FP64_EXACT,
               int stencil_form = SARAS_STENCIL_EXACT)
        : timeIntegrator(mesh, dt, 1, mg_precision, stencil_form) {}
};

// lsRK3_d2 / eulerCN_d2: the same classes over a planar grid
using lsRK3_d2 = lsRK3_d3;
using eulerCN_d2 = eulerCN_d3;

}  // namespace saras_shim

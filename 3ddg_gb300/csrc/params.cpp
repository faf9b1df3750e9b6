// Parameter file parsing in the reference's "KEY = values" format
// (cppsrc/driver.cpp:129-196) and the compiled-in defaults
// (cppsrc/driver.cpp:48-65, cppsrc/BCParam.cpp:24).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

#include "dg3d.h"
#include "solver_internal.h"

extern "C" int dg_params_default(dg_params* p)
{
    if (!p) return dg::fail(DG_ERR_INVALID, "dg_params_default: null argument");
    std::memset(p, 0, sizeof *p);
    // driver.cpp globals
    const unsigned ne[3] = {4, 3, 2}, nb[3] = {5, 4, 6};
    const double w[3] = {1.0, 2.0, 3.0}, c[3] = {0.25, 0.5, 0.75};
    for (int a = 0; a < 3; a++) {
        p->num_elements[a] = (int)ne[a];
        p->num_blocks[a] = (int)nb[a];
        p->elem_width[a] = w[a];
        p->corner[a] = c[a];
    }
    p->order = 4;
    p->c0 = 1500.0;
    p->rho0 = 1000.0;
    p->b_over_a = 0.0;
    p->diff_const = 0.0;
    p->eval_advect = p->eval_diff = p->eval_sponge = 0;
    // BCParamDefault
    for (int a = 0; a < 3; a++) p->periodic[a] = 0;
    for (int f = 0; f < 6; f++) p->sponge_width[f] = 10;
    p->sigma_max = -1.0;
    for (int a = 0; a < 3; a++) p->ic_gauss[a] = 0;
    p->ic_drho_amp = -1.0;
    for (int a = 0; a < 3; a++) p->ic_v_amp[a] = -1.0;
    p->ic_sigma = -1.0;
    for (int a = 0; a < 3; a++) p->ic_center[a] = -1.0;
    // extensions
    p->precision = DG_PRECISION_FP64;
    p->rk_exact = 0;
    p->lumped_mass = 0;
    p->src_face = -1;
    p->src_amp = 0.0;
    p->src_freq = 1.0;
    p->src_cycles = 5.0;
    p->src_phase = 0.0;
    p->src_radius = 0.0;
    return DG_OK;
}

namespace {

template <typename T>
void read_n(std::istringstream& iss, T* v, int n)
{
    for (int i = 0; i < n; i++) iss >> v[i];
}

void read_bool(std::istringstream& iss, int* v, int n)
{
    for (int i = 0; i < n; i++) {
        bool b = v[i] != 0;
        iss >> b;
        v[i] = b ? 1 : 0;
    }
}

}  // namespace

extern "C" int dg_params_parse(const char* path, dg_params* p, double* dt, int* num_substeps,
                               int* num_outsteps, int* freq_terminal, int* bool_file,
                               const char* log_path)
{
    if (!path || !p) return dg::fail(DG_ERR_INVALID, "dg_params_parse: null argument");
    std::ifstream f(path);
    if (!f.is_open()) return dg::fail(DG_ERR_IO, std::string("Unable to open parameter file ") + path);
    std::ofstream log;
    if (log_path) {
        log.open(log_path);
        if (!log.is_open()) return dg::fail(DG_ERR_IO, std::string("Unable to open log file ") + log_path);
        log << "Parameters used:\n{\n";
    }
    std::string line;
    while (std::getline(f, line)) {
        if (log_path) log << "  " << line << "\n";
        if (line.empty() || line[0] == '#' || line.size() < 2) continue;
        size_t pos = line.find(" = ");
        if (pos == std::string::npos) {
            std::cerr << "WARNING: IGNORING INVALID PARAMETER LINE: \"" << line << "\"\n";
            continue;
        }
        std::string key = line.substr(0, pos);
        std::istringstream iss(line.substr(pos + 3));
        unsigned u3[3];
        if (key == "NUM_TIME_SUBSTEPS") { int v = 0; iss >> v; if (num_substeps) *num_substeps = v; }
        else if (key == "NUM_OUTSTEPS") { int v = 0; iss >> v; if (num_outsteps) *num_outsteps = v; }
        else if (key == "FREQ_TERMINAL") { int v = 0; iss >> v; if (freq_terminal) *freq_terminal = v; }
        else if (key == "BOOL_FILE") { bool v = true; iss >> v; if (bool_file) *bool_file = v ? 1 : 0; }
        else if (key == "C0") iss >> p->c0;
        else if (key == "RHO0") iss >> p->rho0;
        else if (key == "B_OVER_A") iss >> p->b_over_a;
        else if (key == "DIFF_CONST") iss >> p->diff_const;
        else if (key == "NUM_ELEMENTS") { read_n(iss, u3, 3); for (int a = 0; a < 3; a++) p->num_elements[a] = (int)u3[a]; }
        else if (key == "NUM_BLOCKS") { read_n(iss, u3, 3); for (int a = 0; a < 3; a++) p->num_blocks[a] = (int)u3[a]; }
        else if (key == "ORDER") iss >> p->order;
        else if (key == "ELEMENT_WIDTH") read_n(iss, p->elem_width, 3);
        else if (key == "STARTING_CORNER") read_n(iss, p->corner, 3);
        else if (key == "DT") { double v = 0; iss >> v; if (dt) *dt = v; }
        else if (key == "EVALUATE_DIFFUSION") read_bool(iss, &p->eval_diff, 1);
        else if (key == "EVALUATE_ADVECTION") read_bool(iss, &p->eval_advect, 1);
        else if (key == "EVALUATE_SPONGE") read_bool(iss, &p->eval_sponge, 1);
        else if (key == "BC_IS_PERIODIC") read_bool(iss, p->periodic, 3);
        else if (key == "BC_SIGMA_MAX") iss >> p->sigma_max;
        else if (key == "BC_SPONGE_WIDTH") { unsigned s6[6]; read_n(iss, s6, 6); for (int i = 0; i < 6; i++) p->sponge_width[i] = (int)s6[i]; }
        else if (key == "IC_X_GAUSS") read_bool(iss, &p->ic_gauss[0], 1);
        else if (key == "IC_Y_GAUSS") read_bool(iss, &p->ic_gauss[1], 1);
        else if (key == "IC_Z_GAUSS") read_bool(iss, &p->ic_gauss[2], 1);
        else if (key == "IC_DRHO_AMPLITUDE") iss >> p->ic_drho_amp;
        else if (key == "IC_VX_AMPLITUDE") iss >> p->ic_v_amp[0];
        else if (key == "IC_VY_AMPLITUDE") iss >> p->ic_v_amp[1];
        else if (key == "IC_VZ_AMPLITUDE") iss >> p->ic_v_amp[2];
        else if (key == "IC_SIGMA") iss >> p->ic_sigma;
        else if (key == "IC_CENTER_X") iss >> p->ic_center[0];
        else if (key == "IC_CENTER_Y") iss >> p->ic_center[1];
        else if (key == "IC_CENTER_Z") iss >> p->ic_center[2];
        // extensions of this package (ignored by the reference's parser)
        else if (key == "PRECISION") iss >> p->precision;
        else if (key == "RK_EXACT") read_bool(iss, &p->rk_exact, 1);
        else if (key == "LUMPED_MASS") read_bool(iss, &p->lumped_mass, 1);
        else if (key == "SRC_FACE") iss >> p->src_face;
        else if (key == "SRC_AMPLITUDE") iss >> p->src_amp;
        else if (key == "SRC_FREQUENCY") iss >> p->src_freq;
        else if (key == "SRC_CYCLES") iss >> p->src_cycles;
        else if (key == "SRC_PHASE") iss >> p->src_phase;
        else if (key == "SRC_RADIUS") iss >> p->src_radius;
        else std::cerr << "WARNING: IGNORING INVALID PARAMETER LINE: \"" << line << "\"\n";
    }
    if (log_path) log << "}\n";
    return DG_OK;
}

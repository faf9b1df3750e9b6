// Boundary / initial-condition parameters with the reference's field names
// (cppsrc/BCParam.h:13-36) and defaults (cppsrc/BCParam.cpp:24).
#pragma once

struct BCParam {
    bool IS_PERIODIC[3];
    unsigned int spongeWidth[6];
    double sigmaMax;
    bool IC_X_GAUSS;
    bool IC_Y_GAUSS;
    bool IC_Z_GAUSS;
    double IC_drho_amplitude;
    double IC_vx_amplitude;
    double IC_vy_amplitude;
    double IC_vz_amplitude;
    double IC_sigma;
    double IC_center_x;
    double IC_center_y;
    double IC_center_z;
};

extern const BCParam BCParamDefault;

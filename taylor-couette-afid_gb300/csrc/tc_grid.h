// tc_grid.h -- host-side grid, metric and coefficient arrays.
//
// The arrays are those CreateGrid.F90 and InitPressureSolver.F90 build into
// the Fortran module `param` (param.F90:33-63), stored 0-based: entry m holds
// the reference's index m+1.
#pragma once

#include <string>
#include <vector>

#include "../../include/tc_capi.h"

namespace tcgb {

struct Grid {
    int nthm = 0, nzm = 0, nrm = 0, nr = 0;
    double pi = 0, dxt = 0, dxz = 0, dxr = 0, dxtq = 0, dxzq = 0, dxrq = 0;
    // radial metrics, length nr
    std::vector<double> rc, rm, g2rc, g2rm, usrc, usrm, udx1vis1, udx1vis2, udx1qm,
        udx2c, udx2m, rudx2c, udx2rm, pvol, udx2mm, udx2cc;
    // momentum operators (CreateGrid.F90:194-322), length nr
    std::vector<double> ap1j, am1j, ac1j, ap2j, am2j, ac2j, ap2je, am2je, ac2je,
        ap3j, am3j, ac3j;
    // free-slip variants of the wall rows, index 0 = inner, 1 = outer
    double ap1j_fs[2] = {0, 0}, ac1j_fs[2] = {0, 0}, am1j_fs[2] = {0, 0};
    double ap3j_fs[2] = {0, 0}, ac3j_fs[2] = {0, 0}, am3j_fs[2] = {0, 0};
    // pressure operator (InitPressureSolver.F90:22-32), length nr
    std::vector<double> apph, amph, acph;
    // modified wavenumbers, lengths nthm and nzm
    std::vector<double> ak1, ak3;
};

// Validate a configuration for this implementation.  Returns "" when usable,
// else a message.
std::string validate(const tc_bou& b);

// Build the grid; returns "" or an error message.
std::string build_grid(const tc_bou& b, Grid& g);

// Pointer to one array of Grid by tc_grid_array id (nullptr if unknown).
const std::vector<double>* grid_array(const Grid& g, int which);

// RK3 / AB2 constants (InitTimeMarchScheme.F90:16-49), 0-based substeps.
void time_march_scheme(int nsst, double gam[3], double rom[3], double alm[3]);

}  // namespace tcgb

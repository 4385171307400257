// Plain structs shared by host and device code of the GB300 LIFE library.
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/life_gb300.h"

namespace life {

// Per-time-step scalars computed on the host with the C library's cos()
// (so they equal the reference's values bit for bit): the inlet ramp
// coefficient used by step t's boundary conditions (GridClass::getRampCoefficient,
// reference src/Grid.cpp:548-556) and step t's uniform Womersley force
// (src/Grid.cpp:52-62). With gravity beside the Womersley term the force
// differs per site and the table holds its pressure-gradient terms
// dpdx * cos(...) and dpdy * cos(...) instead.
struct StepScalars {
    double ramp;
    double fx, fy;
    float fx_f, fy_f;  // (float)fx, (float)fy for the reduced-precision kernels
    double ax, ay;     // dpdx * cos(...), dpdy * cos(...) of step t
    float ax_f, ay_f;
};

// Everything a lattice kernel needs, passed by value.
struct LatDev {
    int Nx, Ny, pitch;
    int wall[4];          // left, right, bottom, top (LIFE_* lattice types)
    long long S;          // sites per population plane (pitch * Ny)
    int cm;               // central moments collision
    int prec;             // population storage form (LIFE_PREC_*)
    int womersley;        // force_xy(t) from steps[]; else the constant Fx0/Fy0
    int convective;       // right wall is a convective outlet
    int has_ibm;
    double omega, cs;
    double Fx0, Fy0;      // constant force_xy (reference src/Grid.cpp:1035-1045)
    // the same values rounded to float once, on the host (FP32 kernels read
    // these instead of converting per site)
    float omega_f, Fx0_f, Fy0_f;
    double u0x, u0y;      // initial uniform velocity (ux0_p*Dt/Dx, uy0_p*Dt/Dx)
    int init_mode;        // 0: zero velocity (ramp), 1: inlet profile, 2: uniform u0
    int steps_cap;        // steps[] is a ring: time step t lives at t % steps_cap
    const StepScalars* steps;
    const double* u_in;   // [Ny][2] inlet profile
    const double* rho_in; // [Ny]
    // Convective outlet side state (reference GridClass::convectiveSpeed,
    // src/Grid.cpp:477-495, reads u of the previous step at the last three
    // columns; convectiveBC reads f_n[2,6,8] at the outlet column).
    double* outlet_u;           // [3][Ny][2] final u of columns Nx-3, Nx-2, Nx-1
    const double* outlet_f_prev;// [Ny][3] post-BC f[2,6,8] at Nx-1 of the previous step
    double* outlet_f_next;      // [Ny][3] written by the current step
    const double* delU;         // [Ny][2] convective speed term of the current step
    const double* force_ibm;    // [2][S] dense IBM force of the current step, or null
    // Inside a replayed graph the step index comes from device memory: when
    // t_dev is set, kernels use *t_dev + t_off instead of their t argument.
    const int* t_dev;
    int t_off;
    // WOMERSLEY with gravity (src/Grid.cpp:52-62): force_xy of step t at a
    // site is ((rho_n * Drho) * g + dpdx cos(...)) * (Dx Dt)^2 / Dm, with
    // rho_n the site's density after step t-1. The step reads those densities
    // from rho_prev and writes its own into rho_next (two buffers alternating
    // by step parity, pitch layout).
    int site_force;
    double Drho, gx, gy, fsc, Dm;  // fsc = (Dx Dt)^2
    float Drho_f, gx_f, gy_f, fscdm_f;
    const double* rho_prev;
    double* rho_next;
    // Pressure corners keep the normal velocity of the previous step
    // (applyBCs sets only the tangential one there, src/Grid.cpp:354-369):
    // u after step t-1 (corner_prev) and after step t (corner_next) of the
    // four corners, slot (i == Nx-1) + 2 (j == Ny-1), two components each.
    const double* corner_prev;
    double* corner_next;
    // Two counters of the one-launch step kernel with staged tiles: step t
    // hands out its tiles from tile_ctr[t & 1] and clears tile_ctr[(t+1) & 1]
    // for the next step.
    int* tile_ctr;
};

}  // namespace life

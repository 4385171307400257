/*
 * life_params_pack.h -- fill LifeCaseParams from a LIFE params.h.
 *
 * The reference configures a case at compile time (reference inc/params.h:26-110:
 * const globals and #define switches). Compile one C++ translation unit with
 * the case's params.h included first (e.g. g++ -include path/params.h -I
 * include -I include/life_ref_defs) and call life_pack_params(): every
 * constant expression is evaluated by the compiler exactly as in the
 * reference build, and the result is handed to life_case_create().
 * life_print_params() writes the values as decimal integers and hexadecimal
 * floats (exact), one per line.
 */
#ifndef LIFE_PARAMS_PACK_H
#define LIFE_PARAMS_PACK_H
#include <cstdio>
#include <cstring>

#include "life_gb300.h"

#ifndef PARAMS_H
#error "include the case's params.h before life_params_pack.h"
#endif

inline void life_pack_params(LifeCaseParams* p) {
    std::memset(p, 0, sizeof *p);
    p->Nx = Nx;
    p->Ny = Ny;
    p->height_p = height_p;
    p->rho_p = rho_p;
    p->nu_p = nu_p;
    p->omega = omega;
    p->ux0_p = ux0_p;
    p->uy0_p = uy0_p;
    p->gravityX = gravityX;
    p->gravityY = gravityY;
    p->dpdx = dpdx;
    p->dpdy = dpdy;
    p->wall_left = WALL_LEFT;
    p->wall_right = WALL_RIGHT;
    p->wall_bottom = WALL_BOTTOM;
    p->wall_top = WALL_TOP;
#ifdef PROFILE
    p->profile = PROFILE;
#else
    p->profile = LIFE_PROFILE_UNIFORM;
#endif
    p->uxInlet_p = uxInlet_p;
    p->uyInlet_p = uyInlet_p;
    p->alpha = alpha;
    p->delta = delta;
    p->relaxMax = relaxMax;
    p->subTol = subTol;
#ifdef CENTRAL_MOMENTS
    p->central_moments = 1;
#endif
#ifdef INLET_RAMP
    p->has_inlet_ramp = 1;
    p->inlet_ramp = INLET_RAMP;
#endif
#ifdef WOMERSLEY
    p->has_womersley = 1;
    p->womersley = WOMERSLEY;
#endif
#ifdef UNI_EPSILON
    p->uni_epsilon = 1;
#endif
#ifdef ORDERED
    p->ordered = 1;
#endif
#ifdef INITIAL_DEFLECT
    p->has_initial_deflect = 1;
    p->initial_deflect = INITIAL_DEFLECT;
#endif
    p->nSteps = nSteps;
    p->tinfo = tinfo;
    p->tVTK = tVTK;
    p->tRestart = tRestart;
    p->ref_nu = ref_nu;
    p->ref_rho = ref_rho;
    p->ref_P = ref_P;
    p->ref_L = ref_L;
    p->ref_U = ref_U;
    p->precision = LIFE_PREC_F64;
}

inline void life_print_params(const LifeCaseParams* p, FILE* out) {
#define LIFE_PI_(x) std::fprintf(out, "%d\n", (int)(x))
#define LIFE_PD_(x) std::fprintf(out, "%a\n", (double)(x))
    LIFE_PI_(p->Nx); LIFE_PI_(p->Ny); LIFE_PD_(p->height_p); LIFE_PD_(p->rho_p); LIFE_PD_(p->nu_p);
    LIFE_PD_(p->omega); LIFE_PD_(p->ux0_p); LIFE_PD_(p->uy0_p); LIFE_PD_(p->gravityX); LIFE_PD_(p->gravityY);
    LIFE_PD_(p->dpdx); LIFE_PD_(p->dpdy); LIFE_PI_(p->wall_left); LIFE_PI_(p->wall_right);
    LIFE_PI_(p->wall_bottom); LIFE_PI_(p->wall_top); LIFE_PI_(p->profile); LIFE_PD_(p->uxInlet_p);
    LIFE_PD_(p->uyInlet_p); LIFE_PD_(p->alpha); LIFE_PD_(p->delta); LIFE_PD_(p->relaxMax); LIFE_PD_(p->subTol);
    LIFE_PI_(p->central_moments); LIFE_PI_(p->has_inlet_ramp); LIFE_PD_(p->inlet_ramp);
    LIFE_PI_(p->has_womersley); LIFE_PD_(p->womersley); LIFE_PI_(p->uni_epsilon); LIFE_PI_(p->ordered);
    LIFE_PI_(p->has_initial_deflect); LIFE_PD_(p->initial_deflect); LIFE_PI_(p->nSteps); LIFE_PI_(p->tinfo);
    LIFE_PI_(p->tVTK); LIFE_PI_(p->tRestart); LIFE_PD_(p->ref_nu); LIFE_PD_(p->ref_rho); LIFE_PD_(p->ref_P);
    LIFE_PD_(p->ref_L); LIFE_PD_(p->ref_U);
#undef LIFE_PI_
#undef LIFE_PD_
}
#endif

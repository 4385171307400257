#include "fem_kernels.h"

using namespace life;

int setup_fem(LifeCase* c) {
    (void)c;
    return set_error(LIFE_ERR_INVALID, "flexible bodies are not built into this library version");
}

int fem_fsi_loop(LifeCase* c, int t, const void* A, const LatDev& L) {
    (void)c; (void)t; (void)A; (void)L;
    return set_error(LIFE_ERR_INVALID, "flexible bodies are not built into this library version");
}

extern "C" int life_case_get_fem(LifeCase* c, int32_t k, double* U, double* Udot, double* Udotdot, double* U_n,
                                 double* U_nm1, double* R_k, double* el_L, double* el_angle, double* node_pos,
                                 double* node_angle) {
    (void)c; (void)k; (void)U; (void)Udot; (void)Udotdot; (void)U_n; (void)U_nm1; (void)R_k; (void)el_L;
    (void)el_angle; (void)node_pos; (void)node_angle;
    return set_error(LIFE_ERR_INVALID, "no flexible bodies");
}

extern "C" int life_case_get_relax(LifeCase* c, double* relax) {
    (void)c;
    if (relax) *relax = 0.0;
    return LIFE_OK;
}

/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle for the LIFE hot path.
 *
 * A plain-C restatement of the LIFE reference's FP64 algorithm (lattice
 * Boltzmann stream-collide, boundary conditions, immersed-boundary coupling,
 * epsilon solve, corotational FEM with Newmark, Aitken-relaxed subiterations),
 * used by tests/ and by bench.py's CPU-baseline leg to check and time the GPU
 * path. The product library never links or calls it.
 *
 * Parity pin: the .npz files in tests/golden hold restart dumps written by the reference
 * binary itself (tests/golden/make_golden.py); tests/test_oracle_golden.py
 * checks this oracle against them.
 *
 * Layout matches the reference (id = i*Ny + j, f[id*9+v], u[id*2+d]).
 */
#ifndef LIFE_ORACLE_H
#define LIFE_ORACLE_H

#include "../include/life_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleCase OracleCase;

const char* oracle_last_error(void);
int oracle_create(const LifeCaseParams* p, const LifeBodyDesc* bodies, int nbodies,
                  OracleCase** out);
void oracle_destroy(OracleCase* c);
int oracle_step(OracleCase* c, int nsteps);
int oracle_time(const OracleCase* c);
int oracle_counts(const OracleCase* c, int* n_markers, int* n_bodies, int* n_flex,
                  int* sim_dofs);
int oracle_get_fields(const OracleCase* c, double* rho, double* u, double* f, double* fibm);
int oracle_set_fields(OracleCase* c, int t, const double* rho, const double* u,
                      const double* f, const double* fibm);
int oracle_get_markers(const OracleCase* c, double* pos, double* vel, double* force,
                       double* eps, double* ds, int* body_index);
int oracle_get_bodies(const OracleCase* c, int* ids, int* flexible, int* n_markers,
                      int* n_fem_nodes);
int oracle_get_fem(const OracleCase* c, int k, double* U, double* Udot, double* Udotdot,
                   double* U_n, double* U_nm1, double* R_k, double* el_L, double* el_angle,
                   double* node_pos, double* node_angle);
int oracle_get_relax(const OracleCase* c, double* relax, int* subits, double* subres);
/* Newton-Raphson iterations and residual of flexible body k's last dynamicFEM. */
int oracle_get_nr(const OracleCase* c, int k, int* itNR, double* resNR);
/* Dense LU solve exactly as the oracle's FEM/epsilon paths use it (row-major A,
 * first bc rows/cols dropped); exposed for unit tests. */
int oracle_solve(int dim, const double* A, const double* b, int bc, double* x);

#ifdef __cplusplus
}
#endif
#endif

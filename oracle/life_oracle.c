/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle for the LIFE hot path (FP64).
 *
 * A restatement of the LIFE reference algorithm (joconnor22/LIFE v1.0.3) in
 * plain C, used only by tests/ (as the oracle the CUDA path is compared with)
 * and by bench.py's CPU-baseline leg.
 * Every floating-point expression keeps the reference's operation order
 * (and the build disables FMA contraction) so that lattice results agree with
 * the reference binary bit for bit; each function cites the reference code it
 * follows. The one deliberate difference: the dense solves use the textbook
 * unblocked LU with partial pivoting (LAPACK dgetf2/dgetrs semantics) where
 * the reference links a system LAPACK (reference src/Utils.cpp:288-311), so
 * IBM/FEM quantities agree with the reference to rounding, not bit for bit.
 *
 * Parity pin: tests/test_oracle_golden.py compares against restart dumps
 * written by the reference binary (tests/golden/make_golden.py).
 */
#include "life_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Trigonometry of the per-step element update (element angle and rotation).
 * The default build calls the C library, as the reference does. Built with
 * -DLIFE_ORACLE_CR_TRIG (liblife_oracle_cr.so) it calls the correctly rounded
 * routines the GPU uses instead (life_gb300/csrc/crtrig.h, checked against
 * 300-bit arithmetic by tests/test_crtrig.py), so the device's remaining
 * arithmetic can be compared with this restatement bit for bit. Start-up
 * (the static pre-deflection, body construction) always uses the C library,
 * as the GPU path's host start-up does. */
#ifdef LIFE_ORACLE_CR_TRIG
#include "crtrig.h"
static double step_atan2(double y, double x) { return life_cr_atan2(y, x); }
static double step_sin(double x) { return life_cr_sin(x); }
static double step_cos(double x) { return life_cr_cos(x); }
double oracle_cr_sin(double x) { return life_cr_sin(x); }
double oracle_cr_cos(double x) { return life_cr_cos(x); }
double oracle_cr_atan2(double y, double x) { return life_cr_atan2(y, x); }
#else
static double step_atan2(double y, double x) { return atan2(y, x); }
static double step_sin(double x) { return sin(x); }
static double step_cos(double x) { return cos(x); }
#endif

#define NV 9
#define SUPP 9

/* D2Q9 directions in the reference's order (reference src/Grid.cpp:1248-1250). */
static const int CX[NV] = {0, 1, -1, 0, 0, 1, -1, 1, -1};
static const int CY[NV] = {0, 0, 0, 1, -1, 1, -1, -1, 1};
static const int OPP[NV] = {0, 2, 1, 4, 3, 6, 5, 8, 7};

static __thread char g_err[512];

const char* oracle_last_error(void) { return g_err; }

static int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

/* ------------------------------------------------------------------ types */

typedef struct {
    int i, j;
    double delta;
} Supp;

typedef struct {
    int body;                 /* owning body index */
    int ID;                   /* global marker ID */
    double pos[2], vel[2], force[2];
    double ds, epsilon;
    double interpMom[2], interpRho;
    int suppCount;
    Supp supp[SUPP];
} Marker;

typedef struct {
    int nodeID;
    double zeta1, zeta2;
} ForceMap;

typedef struct {
    double L0, L, angle, A, I, E, rho;
    double T[6][6], M[6][6], K_L[6][6], K_NL[6][6], R[6], F[6];
    int DOFs[6];
    int node[2];
    int nmap;
    ForceMap* fmap;
} Element;

typedef struct {
    int nNodes, nEl, bodyDOFs, bcDOFs;
    double L0, angle0, tCrit;
    int itNR;
    double resNR;
    double *M, *K, *R, *F, *U, *delU, *Udot, *Udotdot, *U_n, *U_nm1, *U_nm2, *Udot_n,
        *Udotdot_n, *U_km1, *R_k, *R_km1;
    double (*pos0)[2], (*pos)[2];
    double *angle0n, *anglen;
    Element* el;
    int nmap;
    int* mapEl;
    double* mapZeta;
    double subRes, subNum, subDen;
} FemBody;

typedef struct {
    int ID;
    int flex;                 /* 1 flexible, 0 rigid */
    int kind;                 /* LIFE_BODY_* */
    int nNodes;
    int* nodes;               /* marker indices */
    FemBody* fem;
} Body;

struct OracleCase {
    LifeCaseParams p;
    int Nx, Ny, t, tOffset;
    double Dx, Dt, Dm, Drho, tau, nu, c_s, omega;
    double w[NV];
    double *f, *f_n, *u, *u_n, *rho, *rho_n, *force_xy, *force_ibm;
    signed char* type;
    int nbc;
    int* bc;
    int* bcn;                 /* per BC site: nx, ny, normalDirection */
    double *delU, *u_in, *rho_in;
    int hasIBM, hasFlex, nFlex, simDOFs;
    int nm, nb;
    Marker* m;
    Body* b;
    int subIt;
    double relax, subRes, subNum, subDen;
};

#define SQ(x) ((x) * (x))
#define TH(x) ((x) * (x) * (x))
#define QU(x) ((x) * (x) * (x) * (x))

/* ------------------------------------------------------- small helpers */

/* Utils::diracDelta (reference inc/Utils.h:220-232) */
static double dirac(double dist) {
    double a = fabs(dist);
    if (a > 1.5) return 0.0;
    if (a > 0.5) return (5.0 - 3.0 * a - sqrt(-3.0 * SQ(1.0 - a) + 1.0)) / 6.0;
    return (1.0 + sqrt(1.0 - 3.0 * SQ(a))) / 3.0;
}

/* Utils::shiftAngle (inc/Utils.h:235-246) */
static double shift_angle(double angle) {
    angle = fmod(angle + M_PI, 2.0 * M_PI);
    if (angle < 0.0) angle += 2.0 * M_PI;
    return angle - M_PI;
}

static int sgn(double v) { return (0.0 < v) - (v < 0.0); }

static double dot(const double* a, const double* b, int n) {
    double r = 0.0;
    for (int i = 0; i < n; i++) r += a[i] * b[i];
    return r;
}

/* Textbook LU with partial pivoting on M = A_sub^T (column-major view of the
 * row-major trailing block), then the transposed solve -- the semantics of
 * Utils::solveLAPACK (reference src/Utils.cpp:288-311: dgetrf + dgetrs 'T'). */
int oracle_solve(int dim, const double* A, const double* b, int bc, double* x) {
    int n = dim - bc;
    double* M = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * (n > 0 ? n : 1));
    int* piv = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    if (!M || !piv) { free(M); free(piv); return fail(LIFE_ERR_NOMEM, "oracle: out of memory"); }
    for (int jj = 0; jj < n; jj++)
        for (int ii = 0; ii < n; ii++) M[ii + jj * n] = A[(size_t)(bc + jj) * dim + (bc + ii)];
    for (int j = 0; j < n; j++) {
        int jp = j;
        double amax = fabs(M[j + j * n]);
        for (int i = j + 1; i < n; i++) {
            double a = fabs(M[i + j * n]);
            if (a > amax) { amax = a; jp = i; }
        }
        piv[j] = jp;
        if (M[jp + j * n] != 0.0) {
            if (jp != j)
                for (int k = 0; k < n; k++) {
                    double tmp = M[j + k * n];
                    M[j + k * n] = M[jp + k * n];
                    M[jp + k * n] = tmp;
                }
            double r = 1.0 / M[j + j * n];
            for (int i = j + 1; i < n; i++) M[i + j * n] *= r;
        }
        for (int k = j + 1; k < n; k++) {
            double tmp = -M[j + k * n];
            for (int i = j + 1; i < n; i++) M[i + k * n] += M[i + j * n] * tmp;
        }
    }
    for (int i = 0; i < bc; i++) x[i] = 0.0;
    double* y = x + bc;
    for (int i = 0; i < n; i++) y[i] = b[bc + i];
    /* U^T w = b */
    for (int i = 0; i < n; i++) {
        double tmp = y[i];
        for (int k = 0; k < i; k++) tmp -= M[k + i * n] * y[k];
        y[i] = tmp / M[i + i * n];
    }
    /* L^T v = w (unit diagonal) */
    for (int i = n - 1; i >= 0; i--) {
        double tmp = y[i];
        for (int k = i + 1; k < n; k++) tmp -= M[k + i * n] * y[k];
        y[i] = tmp;
    }
    /* x = P v */
    for (int i = n - 1; i >= 0; i--)
        if (piv[i] != i) {
            double tmp = y[i];
            y[i] = y[piv[i]];
            y[piv[i]] = tmp;
        }
    free(M);
    free(piv);
    return LIFE_OK;
}

/* ------------------------------------------------------------- lattice */

/* GridClass::equilibrium (reference src/Grid.cpp:249-264) */
static inline double equilibrium(const OracleCase* c, int id, int v) {
    int cx = CX[v], cy = CY[v];
    double ux = c->u_n[id * 2 + 0], uy = c->u_n[id * 2 + 1];
    if (c->p.central_moments)
        return 0.25 * c->rho_n[id] * c->w[v] *
               (9.0 * SQ(cx) * SQ(ux) + 6.0 * cx * ux - 3.0 * SQ(ux) + 2.0) *
               (9.0 * SQ(cy) * SQ(uy) + 6.0 * cy * uy - 3.0 * SQ(uy) + 2.0);
    return c->rho_n[id] * c->w[v] *
           (1.0 + 3.0 * (cx * ux + cy * uy) +
            4.5 * (SQ(ux) * (SQ(cx) - 1.0 / 3.0) + SQ(uy) * (SQ(cy) - 1.0 / 3.0)) +
            9.0 * cx * cy * ux * uy);
}

/* GridClass::latticeForce (src/Grid.cpp:267-279) */
static inline double lattice_force(const OracleCase* c, int id, int v) {
    int cx = CX[v], cy = CY[v];
    double ux = c->u_n[id * 2 + 0], uy = c->u_n[id * 2 + 1];
    double Fx = c->force_xy[id * 2 + 0] + c->force_ibm[id * 2 + 0];
    double Fy = c->force_xy[id * 2 + 1] + c->force_ibm[id * 2 + 1];
    return 3.0 * c->w[v] *
           (Fx * (cx - ux + cx * 3.0 * (cx * ux + cy * uy)) +
            (Fy * (cy - uy + cy * 3.0 * (cx * ux + cy * uy))));
}

/* GridClass::streamCollide (src/Grid.cpp:103-246): push scheme */
static void stream_collide(OracleCase* c, int i, int j, int id) {
    const int Nx = c->Nx, Ny = c->Ny;
    double fs[NV];
    if (c->p.central_moments) {
        double k4Pre = 0.0, k5Pre = 0.0;
        for (int v = 0; v < NV; v++) {
            double cx = CX[v] - c->u_n[id * 2 + 0];
            double cy = CY[v] - c->u_n[id * 2 + 1];
            k4Pre += c->f_n[id * NV + v] * (SQ(cx) - SQ(cy));
            k5Pre += c->f_n[id * NV + v] * cx * cy;
        }
        const double cs = c->c_s, om = c->omega;
        double k0 = c->rho_n[id];
        double k1 = 0.5 * (c->force_xy[id * 2 + 0] + c->force_ibm[id * 2 + 0]);
        double k2 = 0.5 * (c->force_xy[id * 2 + 1] + c->force_ibm[id * 2 + 1]);
        double k3 = 2.0 * c->rho_n[id] * SQ(cs);
        double k4 = (1.0 - om) * k4Pre;
        double k5 = (1.0 - om) * k5Pre;
        double k6 = 0.5 * (c->force_xy[id * 2 + 1] + c->force_ibm[id * 2 + 1]) * SQ(cs);
        double k7 = 0.5 * (c->force_xy[id * 2 + 0] + c->force_ibm[id * 2 + 0]) * SQ(cs);
        double k8 = c->rho_n[id] * QU(cs);
        double ux = c->u_n[id * 2 + 0];
        double uy = c->u_n[id * 2 + 1];
        /* Inverse central-moment transform, De Rosis (2019); term order as in
         * src/Grid.cpp:143-223 (bit-exact parity depends on it). */
        fs[0] = (SQ(ux) * SQ(uy) - SQ(ux) - SQ(uy) + 1.0) * k0
              + (2.0 * ux * SQ(uy) - 2.0 * ux) * k1
              + (2.0 * uy * SQ(ux) - 2.0 * uy) * k2
              + (0.5 * SQ(ux) + 0.5 * SQ(uy) - 1.0) * k3
              + (0.5 * SQ(uy) - 0.5 * SQ(ux)) * k4
              + 4.0 * ux * uy * k5
              + 2.0 * uy * k6
              + 2.0 * ux * k7
              + k8;
        fs[1] = (0.5 * SQ(ux) - 0.5 * (SQ(ux) * SQ(uy)) - 0.5 * (ux * SQ(uy)) + 0.5 * ux) * k0
              + (ux - ux * SQ(uy) - 0.5 * SQ(uy) + 0.5) * k1
              + (-uy * SQ(ux) - uy * ux) * k2
              + (-0.25 * SQ(ux) - 0.25 * ux - 0.25 * SQ(uy) + 0.25) * k3
              + (0.25 * SQ(ux) + 0.25 * ux - 0.25 * SQ(uy) + 0.25) * k4
              + (-uy - 2.0 * ux * uy) * k5
              + (-uy) * k6
              + (-ux - 0.5) * k7
              - 0.5 * k8;
        fs[2] = (-0.5 * (SQ(ux) * SQ(uy)) + 0.5 * SQ(ux) + 0.5 * (ux * SQ(uy)) - 0.5 * ux) * k0
              + (ux - ux * SQ(uy) + 0.5 * SQ(uy) - 0.5) * k1
              + (-uy * SQ(ux) + uy * ux) * k2
              + (-0.25 * SQ(ux) + 0.25 * ux - 0.25 * SQ(uy) + 0.25) * k3
              + (0.25 * SQ(ux) - 0.25 * ux - 0.25 * SQ(uy) + 0.25) * k4
              + (uy - 2.0 * ux * uy) * k5
              + (-uy) * k6
              + (0.5 - ux) * k7
              - 0.5 * k8;
        fs[3] = (0.5 * SQ(uy) - 0.5 * (SQ(ux) * uy) - 0.5 * (SQ(ux) * SQ(uy)) + 0.5 * uy) * k0
              + (-ux * SQ(uy) - ux * uy) * k1
              + (uy - SQ(ux) * uy - 0.5 * SQ(ux) + 0.5) * k2
              + (-0.25 * SQ(ux) - 0.25 * SQ(uy) - 0.25 * uy + 0.25) * k3
              + (0.25 * SQ(ux) - 0.25 * SQ(uy) - 0.25 * uy - 0.25) * k4
              + (-ux - 2.0 * ux * uy) * k5
              + (-uy - 0.5) * k6
              + (-ux) * k7
              - 0.5 * k8;
        fs[4] = (-0.5 * (SQ(ux) * SQ(uy)) + 0.5 * (SQ(ux) * uy) + 0.5 * SQ(uy) - 0.5 * uy) * k0
              + (-ux * SQ(uy) + ux * uy) * k1
              + (uy - SQ(ux) * uy + 0.5 * SQ(ux) - 0.5) * k2
              + (-0.25 * SQ(ux) - 0.25 * SQ(uy) + 0.25 * uy + 0.25) * k3
              + (0.25 * SQ(ux) - 0.25 * SQ(uy) + 0.25 * uy - 0.25) * k4
              + (ux - 2.0 * ux * uy) * k5
              + (0.5 - uy) * k6
              + (-ux) * k7
              - 0.5 * k8;
        fs[5] = (0.25 * (SQ(ux) * SQ(uy)) + 0.25 * (SQ(ux) * uy) + 0.25 * (ux * SQ(uy)) + 0.25 * (ux * uy)) * k0
              + (0.25 * uy + 0.5 * (ux * uy) + 0.5 * (ux * SQ(uy)) + 0.25 * SQ(uy)) * k1
              + (0.25 * ux + 0.5 * (ux * uy) + 0.5 * (SQ(ux) * uy) + 0.25 * SQ(ux)) * k2
              + (0.125 * SQ(ux) + 0.125 * ux + 0.125 * SQ(uy) + 0.125 * uy) * k3
              + (-0.125 * SQ(ux) - 0.125 * ux + 0.125 * SQ(uy) + 0.125 * uy) * k4
              + (0.5 * ux + 0.5 * uy + ux * uy + 0.25) * k5
              + (0.5 * uy + 0.25) * k6
              + (0.5 * ux + 0.25) * k7
              + 0.25 * k8;
        fs[6] = (0.25 * (SQ(ux) * SQ(uy)) - 0.25 * (SQ(ux) * uy) - 0.25 * (ux * SQ(uy)) + 0.25 * (ux * uy)) * k0
              + (0.25 * uy - 0.5 * (ux * uy) + 0.5 * (ux * SQ(uy)) - 0.25 * SQ(uy)) * k1
              + (0.25 * ux - 0.5 * (ux * uy) + 0.5 * (SQ(ux) * uy) - 0.25 * SQ(ux)) * k2
              + (0.125 * SQ(ux) - 0.125 * ux + 0.125 * SQ(uy) - 0.125 * uy) * k3
              + (-0.125 * SQ(ux) + 0.125 * ux + 0.125 * SQ(uy) - 0.125 * uy) * k4
              + (ux * uy - 0.5 * uy - 0.5 * ux + 0.25) * k5
              + (0.5 * uy - 0.25) * k6
              + (0.5 * ux - 0.25) * k7
              + 0.25 * k8;
        fs[7] = (0.25 * (SQ(ux) * SQ(uy)) - 0.25 * (SQ(ux) * uy) + 0.25 * (ux * SQ(uy)) - 0.25 * (ux * uy)) * k0
              + (0.5 * (ux * SQ(uy)) - 0.5 * (ux * uy) - 0.25 * uy + 0.25 * SQ(uy)) * k1
              + (0.5 * (ux * uy) - 0.25 * ux + 0.5 * (SQ(ux) * uy) - 0.25 * SQ(ux)) * k2
              + (0.125 * SQ(ux) + 0.125 * ux + 0.125 * SQ(uy) - 0.125 * uy) * k3
              + (-0.125 * SQ(ux) - 0.125 * ux + 0.125 * SQ(uy) - 0.125 * uy) * k4
              + (0.5 * uy - 0.5 * ux + ux * uy - 0.25) * k5
              + (0.5 * uy - 0.25) * k6
              + (0.5 * ux + 0.25) * k7
              + 0.25 * k8;
        fs[8] = (0.25 * (SQ(ux) * SQ(uy)) + 0.25 * (SQ(ux) * uy) - 0.25 * (ux * SQ(uy)) - 0.25 * (ux * uy)) * k0
              + (0.5 * (ux * uy) - 0.25 * uy + 0.5 * (ux * SQ(uy)) - 0.25 * SQ(uy)) * k1
              + (0.5 * (SQ(ux) * uy) - 0.5 * (ux * uy) - 0.25 * ux + 0.25 * SQ(ux)) * k2
              + (0.125 * SQ(ux) - 0.125 * ux + 0.125 * SQ(uy) + 0.125 * uy) * k3
              + (-0.125 * SQ(ux) + 0.125 * ux + 0.125 * SQ(uy) + 0.125 * uy) * k4
              + (0.5 * ux - 0.5 * uy + ux * uy - 0.25) * k5
              + (0.5 * uy + 0.25) * k6
              + (0.5 * ux - 0.25) * k7
              + 0.25 * k8;
    } else {
        for (int v = 0; v < NV; v++)
            fs[v] = c->f_n[id * NV + v] + c->omega * (equilibrium(c, id, v) - c->f_n[id * NV + v]) +
                    (1.0 - 0.5 * c->omega) * lattice_force(c, id, v);
    }
    for (int v = 0; v < NV; v++) {
        int recv = ((i + CX[v] + Nx) % Nx) * Ny + ((j + CY[v] + Ny) % Ny);
        c->f[recv * NV + v] = fs[v];
    }
}

/* GridClass::macroscopic (src/Grid.cpp:282-299) */
static inline void macroscopic(OracleCase* c, int id) {
    double r = 0.0, mx = 0.0, my = 0.0;
    for (int v = 0; v < NV; v++) {
        r += c->f[id * NV + v];
        mx += CX[v] * c->f[id * NV + v];
        my += CY[v] * c->f[id * NV + v];
    }
    c->rho[id] = r;
    c->u[id * 2 + 0] = (mx + 0.5 * c->force_xy[id * 2 + 0]) / r;
    c->u[id * 2 + 1] = (my + 0.5 * c->force_xy[id * 2 + 1]) / r;
}

/* GridClass::getRampCoefficient (src/Grid.cpp:548-556) */
static double ramp_coefficient(const OracleCase* c) {
    if (c->p.has_inlet_ramp && c->Dt * c->t <= c->p.inlet_ramp)
        return (1.0 - cos(M_PI * c->Dt * c->t / c->p.inlet_ramp)) / 2.0;
    return 1.0;
}

/* Utils::extrapolate order 1 (inc/Utils.h:151-161) */
static inline double extrapolate1(const OracleCase* c, const double* vec, int nx, int ny, int i, int j) {
    int i1 = i + nx, i2 = i + 2 * nx, j1 = j + ny, j2 = j + 2 * ny;
    return 2.0 * vec[i1 * c->Ny + j1] - vec[i2 * c->Ny + j2];
}

/* Utils::zeroGradient order 2 (inc/Utils.h:200-210) on a 2-component array */
static inline double zero_gradient2(const OracleCase* c, const double* vec, int nx, int ny, int i, int j, int d) {
    int i1 = i + nx, i2 = i + 2 * nx, j1 = j + ny, j2 = j + 2 * ny;
    return (4.0 / 3.0) * vec[(i1 * c->Ny + j1) * 2 + d] - (1.0 / 3.0) * vec[(i2 * c->Ny + j2) * 2 + d];
}

/* GridClass::regularisedBC (src/Grid.cpp:387-465) */
static void regularised_bc(OracleCase* c, int i, int j, int id, const int nv[2], int nd) {
    double* f = c->f + (size_t)id * NV;
    int t = c->type[id];
    int corner = (nv[0] != 0 && nv[1] != 0);
    if (corner) {
        if (t == LIFE_VELOCITY || t == LIFE_WALL || t == LIFE_FREESLIP)
            c->rho_n[id] = extrapolate1(c, c->rho, nv[0], nv[1], i, j);
    } else {
        double fplus = 0.0, fzero = 0.0;
        for (int v = 0; v < NV; v++) {
            int cn = nd == 0 ? CX[v] : CY[v];
            if (cn == -nv[nd]) fplus += f[v];
            else if (cn == 0) fzero += f[v];
        }
        if (t == LIFE_VELOCITY || t == LIFE_WALL || t == LIFE_FREESLIP)
            c->rho_n[id] = (2.0 * fplus + fzero) / (1.0 - nv[nd] * c->u_n[id * 2 + nd]);
        else if (t == LIFE_PRESSURE)
            c->u_n[id * 2 + nd] = nv[nd] * (1.0 - (2.0 * fplus + fzero) / c->rho_n[id]);
    }
    double Sxx = 0.0, Syy = 0.0, Sxy = 0.0;
    for (int v = 0; v < NV; v++) {
        double feq = equilibrium(c, id, v);
        if (corner) {
            if (CX[v] == nv[0] || CY[v] == nv[1]) {
                if (nv[0] * CX[v] + nv[1] * CY[v] == 0) f[v] = feq;
                else f[v] = feq + (f[OPP[v]] - equilibrium(c, id, OPP[v]));
            }
        } else {
            int cn = nd == 0 ? CX[v] : CY[v];
            if (cn == nv[nd]) f[v] = feq + (f[OPP[v]] - equilibrium(c, id, OPP[v]));
        }
        double fneq = f[v] - feq;
        Sxx += CX[v] * CX[v] * fneq;
        Syy += CY[v] * CY[v] * fneq;
        Sxy += CX[v] * CY[v] * fneq;
    }
    const double cs = c->c_s;
    for (int v = 0; v < NV; v++)
        f[v] = equilibrium(c, id, v) +
               (c->w[v] / (2.0 * QU(cs))) * (((SQ(CX[v]) - SQ(cs)) * Sxx) + ((SQ(CY[v]) - SQ(cs)) * Syy) +
                                              (2.0 * CX[v] * CY[v] * Sxy));
}

/* GridClass::applyBCs (src/Grid.cpp:302-384) + convectiveBC (:468-474) */
static void apply_bcs(OracleCase* c, int k) {
    int id = c->bc[k];
    int i = id / c->Ny, j = id - i * c->Ny;
    int nv[2] = {c->bcn[k * 3 + 0], c->bcn[k * 3 + 1]};
    int nd = c->bcn[k * 3 + 2];
    double ramp = ramp_coefficient(c);
    switch (c->type[id]) {
    case LIFE_WALL:
        c->u_n[id * 2 + 0] = 0.0;
        c->u_n[id * 2 + 1] = 0.0;
        regularised_bc(c, i, j, id, nv, nd);
        break;
    case LIFE_VELOCITY:
        c->u_n[id * 2 + 0] = c->u_in[j * 2 + 0] * ramp;
        c->u_n[id * 2 + 1] = c->u_in[j * 2 + 1] * ramp;
        regularised_bc(c, i, j, id, nv, nd);
        break;
    case LIFE_FREESLIP:
        c->u_n[id * 2 + nd] = 0.0;
        for (int d = 0; d < 2; d++)
            if (d != nd) c->u_n[id * 2 + d] = zero_gradient2(c, c->u, nv[0], nv[1], i, j, d);
        regularised_bc(c, i, j, id, nv, nd);
        break;
    case LIFE_PRESSURE:
        c->rho_n[id] = c->rho_in[j];
        for (int d = 0; d < 2; d++)
            if (d != nd) c->u_n[id * 2 + d] = zero_gradient2(c, c->u, nv[0], nv[1], i, j, d);
        regularised_bc(c, i, j, id, nv, nd);
        break;
    case LIFE_CONVECTIVE: {
        double* f = c->f + (size_t)id * NV;
        const double* fn = c->f_n + (size_t)id * NV;
        const double* dU = c->delU + j * 2;
        f[2] = fn[2] + 3.0 * c->w[2] * (dU[0] * CX[2] + dU[1] * CY[2]);
        f[6] = fn[6] + 3.0 * c->w[6] * (dU[0] * CX[6] + dU[1] * CY[6]);
        f[8] = fn[8] + 3.0 * c->w[8] * (dU[0] * CX[8] + dU[1] * CY[8]);
        break;
    }
    default:
        break;
    }
}

/* GridClass::convectiveSpeed (src/Grid.cpp:477-495) */
static void convective_speed(OracleCase* c) {
    const int Nx = c->Nx, Ny = c->Ny;
    double uOut = 0.0;
    for (int j = 0; j < Ny; j++) uOut += c->u[((Nx - 1) * Ny + j) * 2 + 0];
    uOut /= (double)Ny;
    for (int j = 0; j < Ny; j++)
        for (int d = 0; d < 2; d++)
            c->delU[j * 2 + d] = (-uOut / 2.0) * (3.0 * c->u[((Nx - 1) * Ny + j) * 2 + d] -
                                                  4.0 * c->u[((Nx - 2) * Ny + j) * 2 + d] +
                                                  c->u[((Nx - 3) * Ny + j) * 2 + d]);
}

#define SWAPP(a, b) do { double* _t = (a); (a) = (b); (b) = _t; } while (0)

/* BGK stream-collide for one site with loop invariants hoisted into locals
 * (same arithmetic as stream_collide's BGK branch). */
static inline void stream_collide_bgk(int i, int j, int Nx, int Ny, double omega, const double* w,
                                      const double* restrict fn, const double* restrict rn,
                                      const double* restrict un, const double* restrict fxy,
                                      const double* restrict fib, double* restrict f) {
    const int id = i * Ny + j;
    const double ux = un[id * 2 + 0], uy = un[id * 2 + 1], rho = rn[id];
    const double Fx = fxy[id * 2 + 0] + fib[id * 2 + 0];
    const double Fy = fxy[id * 2 + 1] + fib[id * 2 + 1];
    for (int v = 0; v < NV; v++) {
        const int cx = CX[v], cy = CY[v];
        const double feq = rho * w[v] *
                           (1.0 + 3.0 * (cx * ux + cy * uy) +
                            4.5 * (SQ(ux) * (SQ(cx) - 1.0 / 3.0) + SQ(uy) * (SQ(cy) - 1.0 / 3.0)) +
                            9.0 * cx * cy * ux * uy);
        const double F = 3.0 * w[v] *
                         (Fx * (cx - ux + cx * 3.0 * (cx * ux + cy * uy)) +
                          (Fy * (cy - uy + cy * 3.0 * (cx * ux + cy * uy))));
        const double fv = fn[id * NV + v];
        const int recv = ((i + cx + Nx) % Nx) * Ny + ((j + cy + Ny) % Ny);
        f[recv * NV + v] = fv + omega * (feq - fv) + (1.0 - 0.5 * omega) * F;
    }
}

/* GridClass::lbmKernel (src/Grid.cpp:36-100) */
static void lbm_kernel(OracleCase* c) {
    const int Nx = c->Nx, Ny = c->Ny;
    if (c->p.wall_right == LIFE_CONVECTIVE) convective_speed(c);
    SWAPP(c->f_n, c->f);
    SWAPP(c->u_n, c->u);
    SWAPP(c->rho_n, c->rho);
    if (c->p.has_womersley) {
        const LifeCaseParams* p = &c->p;
        double ph = cos(2.0 * M_PI * c->t * c->Dt /
                        ((SQ(p->height_p) * M_PI) / (2.0 * SQ(p->womersley) * p->nu_p)));
        double sc = SQ(c->Dx * c->Dt);
#pragma omp parallel for schedule(static)
        for (int id = 0; id < Nx * Ny; id++) {
            c->force_xy[id * 2 + 0] = (c->rho_n[id] * c->Drho * p->gravityX + p->dpdx * ph) * sc / c->Dm;
            c->force_xy[id * 2 + 1] = (c->rho_n[id] * c->Drho * p->gravityY + p->dpdy * ph) * sc / c->Dm;
        }
    }
    const int bgk = !c->p.central_moments;
    const double omega = c->omega;
    const double* w = c->w;
    const double* restrict fn = c->f_n;
    const double* restrict rn = c->rho_n;
    const double* restrict un = c->u_n;
    const double* restrict fxy = c->force_xy;
    const double* restrict fib = c->force_ibm;
    double* restrict fo = c->f;
#pragma omp parallel
    {
#pragma omp for schedule(guided) collapse(2)
        for (int i = 0; i < Nx; i++)
            for (int j = 0; j < Ny; j++) {
                if (bgk) stream_collide_bgk(i, j, Nx, Ny, omega, w, fn, rn, un, fxy, fib, fo);
                else stream_collide(c, i, j, i * Ny + j);
            }
#pragma omp for schedule(guided)
        for (int id = 0; id < Nx * Ny; id++)
            if (c->type[id] == LIFE_FLUID) macroscopic(c, id);
#pragma omp for schedule(guided)
        for (int k = 0; k < c->nbc; k++) {
            apply_bcs(c, k);
            macroscopic(c, c->bc[k]);
        }
    }
}

/* ------------------------------------------------------------------ IBM */

/* IBMNodeClass::findSupport (src/IBMNode.cpp:139-179) */
static int find_support(OracleCase* c, Marker* m) {
    const double Dx = c->Dx;
    int inear = (int)round(m->pos[0] / Dx);
    int jnear = (int)round(m->pos[1] / Dx);
    m->suppCount = 0;
    for (int s = 0; s < SUPP; s++) { m->supp[s].i = 0; m->supp[s].j = 0; m->supp[s].delta = 0.0; }
    for (int i = inear - 2; i <= inear + 2; i++) {
        double distX = fabs(m->pos[0] / Dx - i);
        for (int j = jnear - 2; j <= jnear + 2; j++) {
            double distY = fabs(m->pos[1] / Dx - j);
            if (distX < 1.5 && distY < 1.5 && i >= 0 && i <= c->Nx - 1 && j >= 0 && j <= c->Ny - 1) {
                if (m->suppCount == SUPP)
                    return fail(LIFE_ERR_SUPPORT,
                                "Support buffer size is not big enough for number of support points...exiting");
                m->supp[m->suppCount].i = i;
                m->supp[m->suppCount].j = j;
                m->supp[m->suppCount].delta = dirac(distX) * dirac(distY);
                m->suppCount++;
            }
        }
    }
    return LIFE_OK;
}

/* IBMNodeClass::computeDs (src/IBMNode.cpp:182-204) */
static void compute_ds(OracleCase* c, int k) {
    Marker* m = &c->m[k];
    const Body* b = &c->b[m->body];
    double cur = 10.0;
    for (int n = 0; n < b->nNodes; n++) {
        const Marker* o = &c->m[b->nodes[n]];
        if (m->ID != o->ID) {
            double d[2] = {m->pos[0] - o->pos[0], m->pos[1] - o->pos[1]};
            double mag = sqrt(dot(d, d, 2)) / c->Dx;
            if (mag < cur) cur = mag;
        }
    }
    m->ds = cur;
}

/* ObjectsClass::computeEpsilon for one marker set (src/Objects.cpp:264-311) */
static int epsilon_for(OracleCase* c, const int* nodes, int dim) {
    double* A = (double*)calloc((size_t)dim * dim, sizeof(double));
    double* bvec = (double*)calloc((size_t)dim, sizeof(double));
    double* eps = (double*)malloc(sizeof(double) * dim);
    if (!A || !bvec || !eps) { free(A); free(bvec); free(eps); return fail(LIFE_ERR_NOMEM, "oracle: oom"); }
    const double Dx = c->Dx;
    for (int i = 0; i < dim; i++) {
        const Marker* ni = &c->m[nodes[i]];
        for (int j = 0; j < dim; j++) {
            const Marker* nj = &c->m[nodes[j]];
            for (int s = 0; s < ni->suppCount; s++) {
                double dvi = ni->supp[s].delta;
                double distX = fabs(nj->pos[0] / Dx - ni->supp[s].i);
                double distY = fabs(nj->pos[1] / Dx - ni->supp[s].j);
                double dvj = dirac(distX) * dirac(distY);
                A[(size_t)i * dim + j] += dvi * dvj;
            }
            A[(size_t)i * dim + j] *= 1.0 * 1.0 * nj->ds;
        }
    }
    for (int i = 0; i < dim; i++) bvec[i] = 1.0;
    int rc = oracle_solve(dim, A, bvec, 0, eps);
    if (rc == LIFE_OK)
        for (int i = 0; i < dim; i++) c->m[nodes[i]].epsilon = eps[i];
    free(A);
    free(bvec);
    free(eps);
    return rc;
}

/* ObjectsClass::computeEpsilon (src/Objects.cpp:235-321) */
static int compute_epsilon(OracleCase* c) {
    if (c->p.uni_epsilon) {
        int* all = (int*)malloc(sizeof(int) * (c->nm > 0 ? c->nm : 1));
        for (int k = 0; k < c->nm; k++) all[k] = k;
        int rc = c->nm > 0 ? epsilon_for(c, all, c->nm) : LIFE_OK;
        free(all);
        return rc;
    }
    for (int ib = 0; ib < c->nb; ib++)
        if (c->t == 0 || c->b[ib].flex) {
            int rc = epsilon_for(c, c->b[ib].nodes, c->b[ib].nNodes);
            if (rc) return rc;
        }
    return LIFE_OK;
}

/* IBMNodeClass::interpolate + forceCalc (src/IBMNode.cpp:26-58) */
static void interpolate_force(OracleCase* c, Marker* m) {
    m->interpRho = 0.0;
    m->interpMom[0] = m->interpMom[1] = 0.0;
    for (int s = 0; s < m->suppCount; s++) {
        int id = m->supp[s].i * c->Ny + m->supp[s].j;
        m->interpRho += c->rho[id] * m->supp[s].delta * 1.0 * 1.0;
        for (int d = 0; d < 2; d++)
            m->interpMom[d] += c->rho[id] * c->u[id * 2 + d] * m->supp[s].delta * 1.0 * 1.0;
    }
    double velScale = c->Dt / c->Dx;
    double s = velScale * m->interpRho;
    for (int d = 0; d < 2; d++) m->force[d] = 2.0 * (s * m->vel[d] - m->interpMom[d]);
}

/* ObjectsClass::ibmKernelSpread (src/Objects.cpp:120-149) with the ORDERED
 * marker-order reduction (src/IBMNode.cpp:61-94) and updateMacroscopic
 * (src/IBMNode.cpp:97-136). */
static void ibm_spread(OracleCase* c) {
    memset(c->force_ibm, 0, sizeof(double) * 2 * (size_t)c->Nx * c->Ny);
    for (int k = 0; k < c->nm; k++) {
        const Marker* m = &c->m[k];
        for (int s = 0; s < m->suppCount; s++) {
            int id = m->supp[s].i * c->Ny + m->supp[s].j;
            double Fx = m->force[0] * m->epsilon * m->ds * 1.0 * m->supp[s].delta;
            double Fy = m->force[1] * m->epsilon * m->ds * 1.0 * m->supp[s].delta;
            c->force_ibm[id * 2 + 0] += Fx;
            c->force_ibm[id * 2 + 1] += Fy;
        }
    }
    for (int k = 0; k < c->nm; k++) {
        const Marker* m = &c->m[k];
        for (int s = 0; s < m->suppCount; s++) {
            int id = m->supp[s].i * c->Ny + m->supp[s].j;
            double r = 0.0, ux = 0.0, uy = 0.0;
            for (int v = 0; v < NV; v++) {
                r += c->f[id * NV + v];
                ux += CX[v] * c->f[id * NV + v];
                uy += CY[v] * c->f[id * NV + v];
            }
            ux = (ux + 0.5 * (c->force_xy[id * 2 + 0] + c->force_ibm[id * 2 + 0])) / r;
            uy = (uy + 0.5 * (c->force_xy[id * 2 + 1] + c->force_ibm[id * 2 + 1])) / r;
            c->rho[id] = r;
            c->u[id * 2 + 0] = ux;
            c->u[id * 2 + 1] = uy;
        }
    }
}

/* ------------------------------------------------------------------ FEM */

static void mat6_mul(double R[6][6], const double A[6][6], const double B[6][6]) {
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) {
            double s = 0.0;
            for (int k = 0; k < 6; k++) s += A[i][k] * B[k][j];
            R[i][j] = s;
        }
}
static void mat6_T(double R[6][6], const double A[6][6]) {
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) R[i][j] = A[j][i];
}
static void mat6_vec(double r[6], const double A[6][6], const double v[6]) {
    for (int i = 0; i < 6; i++) {
        double s = 0.0;
        for (int j = 0; j < 6; j++) s += A[i][j] * v[j];
        r[i] = s;
    }
}

/* FEMElementClass::setElementTransform (src/FEMElement.cpp:255-262) */
static void el_transform(Element* e, int in_step) {
    const double ca = in_step ? step_cos(e->angle) : cos(e->angle);
    const double sa = in_step ? step_sin(e->angle) : sin(e->angle);
    e->T[0][0] = e->T[1][1] = e->T[3][3] = e->T[4][4] = ca;
    e->T[0][1] = e->T[3][4] = sa;
    e->T[1][0] = e->T[4][3] = -sa;
    e->T[2][2] = e->T[5][5] = 1.0;
}

/* FEMElementClass::setLocalMatrices (src/FEMElement.cpp:203-252) */
static void el_local(Element* e) {
    memset(e->M, 0, sizeof e->M);
    memset(e->K_L, 0, sizeof e->K_L);
    memset(e->K_NL, 0, sizeof e->K_NL);
    memset(e->R, 0, sizeof e->R);
    memset(e->F, 0, sizeof e->F);
    double L0 = e->L0, E = e->E, A = e->A, I = e->I;
    double C1 = e->rho * A * L0 / 420.0;
    e->M[0][0] = C1 * 140.0;
    e->M[0][3] = C1 * 70.0;
    e->M[1][1] = C1 * 156.0;
    e->M[1][2] = C1 * 22.0 * L0;
    e->M[1][4] = C1 * 54;
    e->M[1][5] = C1 * (-13.0 * L0);
    e->M[2][2] = C1 * 4.0 * SQ(L0);
    e->M[2][4] = C1 * 13.0 * L0;
    e->M[2][5] = C1 * (-3.0 * SQ(L0));
    e->M[3][3] = C1 * 140.0;
    e->M[4][4] = C1 * 156.0;
    e->M[4][5] = C1 * (-22.0 * L0);
    e->M[5][5] = C1 * 4.0 * SQ(L0);
    e->K_L[0][0] = E * A / L0;
    e->K_L[0][3] = -E * A / L0;
    e->K_L[1][1] = 12.0 * E * I / TH(L0);
    e->K_L[1][2] = 6.0 * E * I / SQ(L0);
    e->K_L[1][4] = -12.0 * E * I / TH(L0);
    e->K_L[1][5] = 6.0 * E * I / SQ(L0);
    e->K_L[2][2] = 4.0 * E * I / L0;
    e->K_L[2][4] = -6.0 * E * I / SQ(L0);
    e->K_L[2][5] = 2.0 * E * I / L0;
    e->K_L[3][3] = E * A / L0;
    e->K_L[4][4] = 12.0 * E * I / TH(L0);
    e->K_L[4][5] = -6.0 * E * I / SQ(L0);
    e->K_L[5][5] = 4.0 * E * I / L0;
    for (int i = 1; i < 6; i++)
        for (int j = 0; j < i; j++) {
            e->M[i][j] = e->M[j][i];
            e->K_L[i][j] = e->K_L[j][i];
        }
}

static void assemble_vec(const Element* e, const double loc[6], double* glob) {
    for (int i = 0; i < 6; i++) glob[e->DOFs[i]] += loc[i];
}
static void assemble_mat(const Element* e, const double loc[6][6], double* glob, int dim) {
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) glob[(size_t)e->DOFs[i] * dim + e->DOFs[j]] += loc[i][j];
}

/* FEMBodyClass::updateFEMValues (src/FEMBody.cpp:198-223) */
static void fem_update_values(FemBody* fb, int in_step) {
    for (int n = 0; n < fb->nNodes; n++) {
        for (int d = 0; d < 2; d++) fb->pos[n][d] = fb->pos0[n][d] + fb->U[n * 3 + d];
        fb->anglen[n] = fb->angle0n[n] + fb->U[n * 3 + 2];
    }
    for (int k = 0; k < fb->nEl; k++) {
        Element* e = &fb->el[k];
        double ev[2] = {fb->pos[e->node[1]][0] - fb->pos[e->node[0]][0],
                        fb->pos[e->node[1]][1] - fb->pos[e->node[0]][1]};
        e->angle = in_step ? step_atan2(ev[1], ev[0]) : atan2(ev[1], ev[0]);
        e->L = sqrt(dot(ev, ev, 2));
        el_transform(e, in_step);
    }
}

/* FEMElementClass::loadVector (src/FEMElement.cpp:27-69) */
static void el_load(OracleCase* c, const Body* b, FemBody* fb, Element* e) {
    double weight[2] = {e->rho * e->A * c->p.gravityX, e->rho * e->A * c->p.gravityY};
    double forceScale = c->Dm / SQ(c->Dt);
    double Tt[6][6];
    mat6_T(Tt, e->T);
    for (int n = 0; n < e->nmap; n++) {
        const Marker* node = &c->m[b->nodes[e->fmap[n].nodeID]];
        double a = e->fmap[n].zeta1, bb = e->fmap[n].zeta2;
        double s = -node->epsilon * 1.0 * forceScale;
        double g[2] = {s * node->force[0] + weight[0], s * node->force[1] + weight[1]};
        double F[2];
        for (int i = 0; i < 2; i++) {
            double acc = 0.0;
            for (int j = 0; j < 2; j++) acc += e->T[i][j] * g[j];
            F[i] = acc;
        }
        double L = e->L;
        e->R[0] = F[0] * 0.5 * L * (0.5 * bb - 0.5 * a + 0.25 * SQ(a) - 0.25 * SQ(bb));
        e->R[1] = F[1] * 0.5 * L * (0.5 * bb - 0.5 * a - SQ(a) * SQ(a) / 16.0 + SQ(bb) * SQ(bb) / 16.0 + 3.0 * SQ(a) / 8.0 - 3.0 * SQ(bb) / 8.0);
        e->R[2] = F[1] * 0.5 * L * (L * (-SQ(a) * SQ(a) + SQ(bb) * SQ(bb)) / 32.0 - L * (-TH(a) + TH(bb)) / 24.0 - L * (-SQ(a) + SQ(bb)) / 16.0 + L * (bb - a) / 8.0);
        e->R[3] = F[0] * 0.5 * L * (-0.25 * SQ(a) + 0.25 * SQ(bb) + 0.5 * bb - 0.5 * a);
        e->R[4] = F[1] * 0.5 * L * (0.5 * bb - 0.5 * a + SQ(a) * SQ(a) / 16.0 - SQ(bb) * SQ(bb) / 16.0 - 3.0 * SQ(a) / 8.0 + 3.0 * SQ(bb) / 8.0);
        e->R[5] = F[1] * 0.5 * L * (L * (-SQ(a) * SQ(a) + SQ(bb) * SQ(bb)) / 32.0 + L * (-TH(a) + TH(bb)) / 24.0 - L * (-SQ(a) + SQ(bb)) / 16.0 - L * (bb - a) / 8.0);
        double RG[6];
        mat6_vec(RG, Tt, e->R);
        assemble_vec(e, RG, fb->R);
    }
}

/* FEMElementClass::forceVector / massMatrix / stiffMatrix
 * (src/FEMElement.cpp:72-138) */
static void el_build(FemBody* fb, Element* e) {
    double u = (SQ(e->L) - SQ(e->L0)) / (e->L + e->L0);
    double th1 = shift_angle(fb->anglen[e->node[0]] - e->angle);
    double th2 = shift_angle(fb->anglen[e->node[1]] - e->angle);
    double F0 = (e->E * e->A / e->L0) * u;
    double M1 = (2 * e->E * e->I / e->L0) * (2.0 * th1 + th2);
    double M2 = (2 * e->E * e->I / e->L0) * (th1 + 2.0 * th2);
    e->F[0] = -F0;
    e->F[1] = (1.0 / e->L0) * (M1 + M2);
    e->F[2] = M1;
    e->F[3] = F0;
    e->F[4] = -(1.0 / e->L0) * (M1 + M2);
    e->F[5] = M2;
    double Tt[6][6], tmp[6][6], G[6][6], G2[6][6], FG[6];
    mat6_T(Tt, e->T);
    mat6_vec(FG, Tt, e->F);
    assemble_vec(e, FG, fb->F);
    mat6_mul(tmp, Tt, e->M);
    mat6_mul(G, tmp, e->T);
    assemble_mat(e, G, fb->M, fb->bodyDOFs);
    mat6_mul(tmp, Tt, e->K_L);
    mat6_mul(G, tmp, e->T);
    double Fa = -e->F[0], V0 = e->F[4], L0 = e->L0;
    e->K_NL[0][1] = -V0 / L0;
    e->K_NL[0][4] = V0 / L0;
    e->K_NL[1][0] = -V0 / L0;
    e->K_NL[1][1] = Fa / L0;
    e->K_NL[1][3] = V0 / L0;
    e->K_NL[1][4] = -Fa / L0;
    e->K_NL[3][1] = V0 / L0;
    e->K_NL[3][4] = -V0 / L0;
    e->K_NL[4][0] = V0 / L0;
    e->K_NL[4][1] = -Fa / L0;
    e->K_NL[4][3] = -V0 / L0;
    e->K_NL[4][4] = Fa / L0;
    mat6_mul(tmp, Tt, e->K_NL);
    mat6_mul(G2, tmp, e->T);
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) G[i][j] = G[i][j] + G2[i][j];
    assemble_mat(e, G, fb->K, fb->bodyDOFs);
}

/* FEMBodyClass::buildGlobalMatrices (src/FEMBody.cpp:90-109) */
static void fem_build_global(FemBody* fb) {
    size_t nn = (size_t)fb->bodyDOFs * fb->bodyDOFs;
    memset(fb->M, 0, sizeof(double) * nn);
    memset(fb->K, 0, sizeof(double) * nn);
    memset(fb->F, 0, sizeof(double) * fb->bodyDOFs);
    for (int k = 0; k < fb->nEl; k++) el_build(fb, &fb->el[k]);
}

/* FEMElementClass::shapeFuns (src/FEMElement.cpp:141-160) */
static void shape_funs(double res[2], const double v[6], double zeta, double L) {
    double N0 = 1.0 - (zeta + 1.0) / 2.0;
    double N1 = 1.0 - 3.0 * SQ((zeta + 1.0) / 2.0) + 2.0 * TH((zeta + 1.0) / 2.0);
    double N2 = ((zeta + 1.0) / 2.0 - 2.0 * SQ((zeta + 1.0) / 2.0) + TH((zeta + 1.0) / 2.0)) * L;
    double N3 = (zeta + 1.0) / 2.0;
    double N4 = 3.0 * SQ((zeta + 1.0) / 2.0) - 2.0 * TH((zeta + 1.0) / 2.0);
    double N5 = (-SQ((zeta + 1.0) / 2.0) + TH((zeta + 1.0) / 2.0)) * L;
    res[0] = v[0] * N0 + v[3] * N3;
    res[1] = v[1] * N1 + v[2] * N2 + v[4] * N4 + v[5] * N5;
}

/* FEMBodyClass::updateIBMValues (src/FEMBody.cpp:147-195) */
static void fem_update_ibm(OracleCase* c, Body* b) {
    FemBody* fb = b->fem;
    for (int i = 0; i < fb->nmap; i++) {
        Element* e = &fb->el[fb->mapEl[i]];
        double zeta = fb->mapZeta[i];
        double dU[6], dUd[6], lU[6], lUd[6];
        for (int k = 0; k < 6; k++) {
            dU[k] = fb->U[e->DOFs[k]];
            dUd[k] = fb->Udot[e->DOFs[k]];
        }
        for (int n = 0; n < 2; n++) {
            dU[n * 3 + 0] += fb->pos0[e->node[n]][0] - fb->pos[e->node[0]][0];
            dU[n * 3 + 1] += fb->pos0[e->node[n]][1] - fb->pos[e->node[0]][1];
            dU[n * 3 + 2] += fb->angle0n[e->node[n]] - e->angle;
            dU[n * 3 + 2] = shift_angle(dU[n * 3 + 2]);
        }
        mat6_vec(lU, e->T, dU);
        mat6_vec(lUd, e->T, dUd);
        double sU[2], sUd[2];
        shape_funs(sU, lU, zeta, e->L);
        shape_funs(sUd, lUd, zeta, e->L);
        double gU[2], gUd[2];
        for (int r = 0; r < 2; r++) {
            double a1 = 0.0, a2 = 0.0;
            for (int k = 0; k < 2; k++) {
                a1 += e->T[k][r] * sU[k];
                a2 += e->T[k][r] * sUd[k];
            }
            gU[r] = a1;
            gUd[r] = a2;
        }
        Marker* m = &c->m[b->nodes[i]];
        m->pos[0] = fb->pos[e->node[0]][0] + gU[0];
        m->pos[1] = fb->pos[e->node[0]][1] + gU[1];
        m->vel[0] = gUd[0];
        m->vel[1] = gUd[1];
    }
}

static double fem_a(const OracleCase* c, int which) {
    double Dt = c->Dt, al = c->p.alpha, de = c->p.delta;
    switch (which) {
    case 0: return 1.0 / (al * SQ(Dt));
    case 2: return 1.0 / (al * Dt);
    case 3: return 1.0 / (2.0 * al) - 1.0;
    case 6: return 1.0 / (al * SQ(Dt));
    case 7: return -1.0 / (al * Dt);
    case 8: return -(1.0 / (2.0 * al) - 1.0);
    case 9: return Dt * (1.0 - de);
    default: return de * Dt;
    }
}

/* FEMBodyClass::finishNewmark (src/FEMBody.cpp:129-144) */
static void fem_finish_newmark(const OracleCase* c, FemBody* fb) {
    double a6 = fem_a(c, 6), a7 = fem_a(c, 7), a8 = fem_a(c, 8), a9 = fem_a(c, 9), a10 = fem_a(c, 10);
    for (int i = 0; i < fb->bodyDOFs; i++) {
        fb->Udotdot[i] = a6 * (fb->U[i] - fb->U_n[i]) + a7 * fb->Udot_n[i] + a8 * fb->Udotdot_n[i];
        fb->Udot[i] = fb->Udot_n[i] + a9 * fb->Udotdot_n[i] + a10 * fb->Udotdot[i];
    }
}

/* FEMBodyClass::newtonRaphsonDynamic + setNewmark (src/FEMBody.cpp:71-126) */
static int fem_nr_dynamic(OracleCase* c, FemBody* fb) {
    int n = fb->bodyDOFs;
    fem_build_global(fb);
    double a0 = fem_a(c, 0), a2 = fem_a(c, 2), a3 = fem_a(c, 3);
    double* v = (double*)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) v[i] = a0 * (fb->U_n[i] - fb->U[i]) + a2 * fb->Udot[i] + a3 * fb->Udotdot[i];
    for (int i = 0; i < n; i++) {
        double s = 0.0;
        for (int j = 0; j < n; j++) s += fb->M[(size_t)i * n + j] * v[j];
        fb->F[i] = fb->R[i] - fb->F[i] + s;
    }
    for (size_t k = 0; k < (size_t)n * n; k++) fb->K[k] = fb->K[k] + a0 * fb->M[k];
    free(v);
    int rc = oracle_solve(n, fb->K, fb->F, fb->bcDOFs, fb->delU);
    if (rc) return rc;
    for (int i = 0; i < n; i++) fb->U[i] = fb->U[i] + fb->delU[i];
    fem_update_values(fb, 1);
    return LIFE_OK;
}

static double nr_residual(const OracleCase* c, const FemBody* fb) {
    return sqrt(dot(fb->delU, fb->delU, fb->bodyDOFs)) / (c->p.ref_L * sqrt((double)fb->bodyDOFs));
}

/* FEMBodyClass::dynamicFEM (src/FEMBody.cpp:26-68) with subResidual (:244-256) */
static int fem_dynamic(OracleCase* c, Body* b) {
    FemBody* fb = b->fem;
    int n = fb->bodyDOFs;
    memcpy(fb->U, fb->U_n, sizeof(double) * n);
    memcpy(fb->Udot, fb->Udot_n, sizeof(double) * n);
    memcpy(fb->Udotdot, fb->Udotdot_n, sizeof(double) * n);
    fem_update_values(fb, 1);
    memset(fb->R, 0, sizeof(double) * n);
    for (int k = 0; k < fb->nEl; k++) el_load(c, b, fb, &fb->el[k]);
    fb->itNR = 0;
    do {
        int rc = fem_nr_dynamic(c, fb);
        if (rc) return rc;
        fb->resNR = nr_residual(c, fb);
        fb->itNR++;
    } while (fb->resNR > 1e-10 && fb->itNR < 20);
    fem_finish_newmark(c, fb);
    fem_update_ibm(c, b);
    memcpy(fb->R_km1, fb->R_k, sizeof(double) * n);
    for (int i = 0; i < n; i++) fb->R_k[i] = fb->U[i] - fb->U_km1[i];
    fb->subRes = dot(fb->R_k, fb->R_k, n);
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n; i++) {
        double d = fb->R_k[i] - fb->R_km1[i];
        num += fb->R_km1[i] * d;
    }
    for (int i = 0; i < n; i++) {
        double d = fb->R_k[i] - fb->R_km1[i];
        den += d * d;
    }
    fb->subNum = num;
    fb->subDen = den;
    return LIFE_OK;
}

/* FEMBodyClass::predictor (src/FEMBody.cpp:259-289) */
static void fem_predictor(OracleCase* c, Body* b) {
    FemBody* fb = b->fem;
    int n = fb->bodyDOFs;
    if (c->t > 2)
        for (int i = 0; i < n; i++) fb->U[i] = 2.5 * fb->U_n[i] - 2.0 * fb->U_nm1[i] + 0.5 * fb->U_nm2[i];
    else if (c->t == 2)
        for (int i = 0; i < n; i++) fb->U[i] = 2.0 * fb->U_n[i] - fb->U_nm1[i];
    else if (c->t == 1)
        memcpy(fb->U, fb->U_n, sizeof(double) * n);
    fem_update_values(fb, 1);
    fem_finish_newmark(c, fb);
    fem_update_ibm(c, b);
    SWAPP(fb->U_km1, fb->U);
}

/* FEMBodyClass::resetValues (src/FEMBody.cpp:341-349) */
static void fem_reset(FemBody* fb) {
    SWAPP(fb->U_nm2, fb->U_nm1);
    SWAPP(fb->U_nm1, fb->U_n);
    SWAPP(fb->U_n, fb->U);
    SWAPP(fb->Udot_n, fb->Udot);
    SWAPP(fb->Udotdot_n, fb->Udotdot);
}

/* FEMBodyClass::setInitialDeflection + staticFEM (src/FEMBody.cpp:352-484) */
static int fem_initial_deflection(OracleCase* c, Body* b) {
    FemBody* fb = b->fem;
    int n = fb->bodyDOFs;
    double deflect = -c->p.initial_deflect;
    double E = fb->el[0].E, I = fb->el[0].I;
    double linearForce = 3.0 * E * I * deflect / SQ(fb->L0);
    double dFmax = linearForce / (double)100;
    double T[2][2] = {{cos(fb->angle0), -sin(fb->angle0)}, {sin(fb->angle0), cos(fb->angle0)}};
    double lf[2] = {0.0, dFmax};
    double gf[2];
    for (int i = 0; i < 2; i++) gf[i] = 0.0 + T[i][0] * lf[0] + T[i][1] * lf[1];
    fb->R[n - 3] = gf[0];
    fb->R[n - 2] = gf[1];
    double gain = 1e-3, TOL = 1e-10, err;
    int it = 0;
    double* rhs = (double*)malloc(sizeof(double) * n);
    do {
        fb->itNR = 0;
        do {
            fem_build_global(fb);
            for (int i = 0; i < n; i++) rhs[i] = fb->R[i] - fb->F[i];
            int rc = oracle_solve(n, fb->K, rhs, fb->bcDOFs, fb->delU);
            if (rc) { free(rhs); return rc; }
            for (int i = 0; i < n; i++) fb->U[i] = fb->U[i] + fb->delU[i];
            fem_update_values(fb, 0);
            fb->resNR = nr_residual(c, fb);
            fb->itNR++;
        } while (fb->resNR > TOL && fb->itNR < 20);
        fem_update_ibm(c, b);
        double dv[2] = {fb->U[n - 3], fb->U[n - 2]};
        double loc1 = 0.0 + T[0][1] * dv[0] + T[1][1] * dv[1];
        err = deflect - loc1 / fb->L0;
        double fc = err * gain;
        if (fabs(fc) > fabs(dFmax)) fc = sgn(fc) * fabs(dFmax);
        lf[1] += fc;
        for (int i = 0; i < 2; i++) gf[i] = 0.0 + T[i][0] * lf[0] + T[i][1] * lf[1];
        fb->R[n - 3] = gf[0];
        fb->R[n - 2] = gf[1];
        it++;
        if (it >= 10000) {
            free(rhs);
            return fail(LIFE_ERR_DEFLECT, "max iterations hit! Try changing the gain...exiting");
        }
    } while (fabs(err) > TOL);
    free(rhs);
    fb->itNR = 0;
    fb->resNR = 0.0;
    memset(fb->R, 0, sizeof(double) * n);
    memset(fb->delU, 0, sizeof(double) * n);
    return LIFE_OK;
}

/* ObjectsClass::femKernel (src/Objects.cpp:63-99) */
static int fem_kernel(OracleCase* c) {
    double res = 0.0, num = 0.0, den = 0.0;
    for (int ib = 0; ib < c->nb; ib++)
        if (c->b[ib].flex) {
            int rc = fem_dynamic(c, &c->b[ib]);
            if (rc) return rc;
            res += c->b[ib].fem->subRes;
            num += c->b[ib].fem->subNum;
            den += c->b[ib].fem->subDen;
        }
    c->subRes = sqrt(res) / (c->p.ref_L * sqrt((double)c->simDOFs));
    c->subNum = num;
    c->subDen = den;
    return LIFE_OK;
}

/* ObjectsClass::recomputeObjectVals (src/Objects.cpp:152-232) */
static int recompute_object_vals(OracleCase* c) {
    if (c->subIt == 0) {
        for (int ib = 0; ib < c->nb; ib++)
            if (c->b[ib].flex) {
                fem_reset(c->b[ib].fem);
                fem_predictor(c, &c->b[ib]);
            }
    } else {
        if (c->subIt == 1) {
            double a = fabs(c->relax);
            c->relax = (double)(sgn(c->relax) * (a < c->p.relaxMax ? a : c->p.relaxMax));
        } else {
            c->relax = -c->relax * c->subNum / c->subDen;
        }
        for (int ib = 0; ib < c->nb; ib++)
            if (c->b[ib].flex) {
                FemBody* fb = c->b[ib].fem;
                for (int i = 0; i < fb->bodyDOFs; i++)
                    fb->U[i] = fb->U_km1[i] + c->relax * (fb->U[i] - fb->U_km1[i]);
                fem_update_values(fb, 1);
                fem_finish_newmark(c, fb);
                fem_update_ibm(c, &c->b[ib]);
                SWAPP(fb->U_km1, fb->U);
            }
    }
    for (int k = 0; k < c->nm; k++)
        if (c->b[c->m[k].body].flex) {
            int rc = find_support(c, &c->m[k]);
            if (rc) return rc;
            compute_ds(c, k);
        }
    return compute_epsilon(c);
}

/* ObjectsClass::objectKernel (src/Objects.cpp:26-60) */
static int object_kernel(OracleCase* c) {
    c->subIt = 0;
    do {
        if (c->hasFlex) {
            int rc = recompute_object_vals(c);
            if (rc) return rc;
        }
        memset(c->force_ibm, 0, sizeof(double) * 2 * (size_t)c->Nx * c->Ny);
        for (int k = 0; k < c->nm; k++) interpolate_force(c, &c->m[k]);
        if (!c->hasFlex) break;
        int rc = fem_kernel(c);
        if (rc) return rc;
        c->subIt++;
    } while (c->subIt < 20 && c->subRes > c->p.subTol);
    ibm_spread(c);
    if (c->subIt == 20) return fail(LIFE_ERR_SUBITER, "Subiteration scheme hit %d iterations...exiting", c->subIt);
    return LIFE_OK;
}

/* --------------------------------------------------------- construction */

static void free_fem(FemBody* fb) {
    if (!fb) return;
    double** arrs[] = {&fb->M, &fb->K, &fb->R, &fb->F, &fb->U, &fb->delU, &fb->Udot, &fb->Udotdot,
                       &fb->U_n, &fb->U_nm1, &fb->U_nm2, &fb->Udot_n, &fb->Udotdot_n, &fb->U_km1,
                       &fb->R_k, &fb->R_km1, &fb->angle0n, &fb->anglen, &fb->mapZeta};
    for (size_t k = 0; k < sizeof arrs / sizeof arrs[0]; k++) free(*arrs[k]);
    free(fb->pos0);
    free(fb->pos);
    free(fb->mapEl);
    for (int k = 0; k < fb->nEl; k++) free(fb->el[k].fmap);
    free(fb->el);
    free(fb);
}

void oracle_destroy(OracleCase* c) {
    if (!c) return;
    free(c->f); free(c->f_n); free(c->u); free(c->u_n); free(c->rho); free(c->rho_n);
    free(c->force_xy); free(c->force_ibm); free(c->type); free(c->bc); free(c->bcn);
    free(c->delU); free(c->u_in); free(c->rho_in);
    for (int ib = 0; ib < c->nb; ib++) {
        free(c->b[ib].nodes);
        free_fem(c->b[ib].fem);
    }
    free(c->b);
    free(c->m);
    free(c);
}

static int add_marker(OracleCase* c, int body, const double pos[2]) {
    Marker* m = &c->m[c->nm];
    memset(m, 0, sizeof *m);
    m->body = body;
    m->ID = c->nm;
    m->pos[0] = pos[0];
    m->pos[1] = pos[1];
    Body* b = &c->b[body];
    b->nodes[b->nNodes++] = c->nm;
    return c->nm++;
}

/* FEMBodyClass::computeNodeMapping (src/FEMBody.cpp:292-338) */
static void fem_node_mapping(FemBody* fb, int nI, int nF) {
    fb->nmap = nI;
    fb->mapEl = (int*)calloc(nI, sizeof(int));
    fb->mapZeta = (double*)calloc(nI, sizeof(double));
    fb->mapEl[0] = 0;
    fb->mapZeta[0] = -1.0;
    for (int i = 1; i < nI; i++) {
        double r = i * ((nF - 1.0) / (nI - 1.0));
        if (fmod(r, 1.0) == 0.0) {
            fb->mapEl[i] = (int)floor(r) - 1;
            fb->mapZeta[i] = 1.0;
        } else {
            fb->mapEl[i] = (int)floor(r);
            fb->mapZeta[i] = fmod(r, 1.0) * 2.0 - 1.0;
        }
    }
    for (int e = 0; e < fb->nEl; e++) {
        Element* el = &fb->el[e];
        el->fmap = (ForceMap*)calloc(nI, sizeof(ForceMap));
        el->nmap = 0;
        for (int node = 0; node < nI; node++) {
            double n1 = -1 + 2.0 * (((double)node - 0.5) * ((nF - 1.0) / (nI - 1.0)) - (double)e) / 1.0;
            double n2 = -1 + 2.0 * (((double)node + 0.5) * ((nF - 1.0) / (nI - 1.0)) - (double)e) / 1.0;
            if ((n1 > -1.0 && n1 < 1.0) || (n2 > -1.0 && n2 < 1.0)) {
                if (n1 < -1.0) n1 = -1.0;
                if (n2 > 1.0) n2 = 1.0;
                el->fmap[el->nmap].nodeID = node;
                el->fmap[el->nmap].zeta1 = n1;
                el->fmap[el->nmap].zeta2 = n2;
                el->nmap++;
            }
        }
    }
}

/* FEMBodyClass ctor (src/FEMBody.cpp:487-578) + FEMElementClass ctor
 * (src/FEMElement.cpp:265-303) */
static FemBody* build_fem(OracleCase* c, const double pos[2], const LifeBodyDesc* d,
                          double angle, int nIBM) {
    FemBody* fb = (FemBody*)calloc(1, sizeof(FemBody));
    fb->bcDOFs = d->clamped ? 3 : 2;
    fb->angle0 = angle;
    fb->L0 = d->length;
    int nEl = d->n_elements > 0 ? d->n_elements : (int)floor(fb->L0 / c->Dx);
    fb->nEl = nEl;
    fb->nNodes = nEl + 1;
    fb->bodyDOFs = fb->nNodes * 3;
    fb->tCrit = (fb->L0 / nEl) / sqrt(d->E / d->rho);
    double T[2][2] = {{cos(angle), -sin(angle)}, {sin(angle), cos(angle)}};
    fb->pos0 = calloc(fb->nNodes, sizeof *fb->pos0);
    fb->pos = calloc(fb->nNodes, sizeof *fb->pos);
    fb->angle0n = calloc(fb->nNodes, sizeof(double));
    fb->anglen = calloc(fb->nNodes, sizeof(double));
    for (int i = 0; i < fb->nNodes; i++) {
        double p[2] = {i * fb->L0 / nEl, 0.0};
        double r[2];
        for (int a = 0; a < 2; a++) r[a] = 0.0 + T[a][0] * p[0] + T[a][1] * p[1];
        fb->pos0[i][0] = fb->pos[i][0] = pos[0] + r[0];
        fb->pos0[i][1] = fb->pos[i][1] = pos[1] + r[1];
        fb->angle0n[i] = fb->anglen[i] = angle;
    }
    fb->el = (Element*)calloc(nEl, sizeof(Element));
    double len = fb->L0 / nEl;
    for (int i = 0; i < nEl; i++) {
        Element* e = &fb->el[i];
        e->L0 = len;
        e->L = len;
        e->angle = angle;
        e->A = c->Dx * d->height;
        e->I = c->Dx * TH(d->height) / 12.0;
        e->E = d->E;
        e->rho = d->rho;
        e->node[0] = i;
        e->node[1] = i + 1;
        for (int a = 0; a < 2; a++)
            for (int k = 0; k < 3; k++) e->DOFs[a * 3 + k] = (i + a) * 3 + k;
        el_transform(e, 0);
        el_local(e);
    }
    fem_node_mapping(fb, nIBM, fb->nNodes);
    int n = fb->bodyDOFs;
    fb->M = calloc((size_t)n * n, sizeof(double));
    fb->K = calloc((size_t)n * n, sizeof(double));
    double** vecs[] = {&fb->R, &fb->F, &fb->U, &fb->delU, &fb->Udot, &fb->Udotdot, &fb->U_n,
                       &fb->U_nm1, &fb->U_nm2, &fb->Udot_n, &fb->Udotdot_n, &fb->U_km1, &fb->R_k,
                       &fb->R_km1};
    for (size_t k = 0; k < sizeof vecs / sizeof vecs[0]; k++) *vecs[k] = calloc(n, sizeof(double));
    return fb;
}

/* ObjectsClass::removeOverlapMarkers (src/Objects.cpp:867-938) */
static int remove_overlap(OracleCase* c) {
    int* erase = (int*)malloc(sizeof(int) * ((size_t)c->nm * c->nm + 1));
    int ne = 0;
    for (int n1 = 0; n1 < c->nm; n1++)
        for (int n2 = n1 + 1; n2 < c->nm; n2++) {
            double d[2] = {c->m[n1].pos[0] - c->m[n2].pos[0], c->m[n1].pos[1] - c->m[n2].pos[1]};
            double mag = sqrt(dot(d, d, 2)) / c->Dx;
            if (mag < 0.5) {
                int f1 = c->b[c->m[n1].body].flex, f2 = c->b[c->m[n2].body].flex;
                if (f1 && f2) {
                    free(erase);
                    return fail(LIFE_ERR_GEOMETRY, "Cannot place two flexible bodies so close to each other...exiting");
                }
                if (f1 && !f2) erase[ne++] = c->m[n2].ID;
                if (!f1 && f2) erase[ne++] = c->m[n1].ID;
                if (!f1 && !f2) erase[ne++] = c->m[n1].ID;
            }
        }
    for (int e = 0; e < ne; e++) {
        int k = -1;
        for (int n = 0; n < c->nm; n++)
            if (c->m[n].ID == erase[e]) { k = n; break; }
        if (k < 0) continue;
        Body* b = &c->b[c->m[k].body];
        int pos = -1;
        for (int n = 0; n < b->nNodes; n++)
            if (b->nodes[n] == k) pos = n;
        for (int n = pos; n + 1 < b->nNodes; n++) b->nodes[n] = b->nodes[n + 1];
        b->nNodes--;
        for (int ib = 0; ib < c->nb; ib++)
            for (int n = 0; n < c->b[ib].nNodes; n++)
                if (c->b[ib].nodes[n] > k) c->b[ib].nodes[n]--;
        memmove(&c->m[k], &c->m[k + 1], sizeof(Marker) * (size_t)(c->nm - k - 1));
        c->nm--;
    }
    for (int n = 0; n < c->nm; n++) c->m[n].ID = n;
    free(erase);
    return LIFE_OK;
}

static int build_objects(OracleCase* c, const LifeBodyDesc* bodies, int nbd) {
    int nbody = 0, nnode = 0;
    for (int k = 0; k < nbd; k++) {
        const LifeBodyDesc* d = &bodies[k];
        nbody += d->number;
        if (d->kind == LIFE_BODY_CIRCLE)
            nnode += d->number * (int)floor(2.0 * M_PI * d->radius / c->Dx);
        else
            nnode += d->number * ((int)floor(d->length / c->Dx) + 1);
    }
    c->b = (Body*)calloc(nbody > 0 ? nbody : 1, sizeof(Body));
    c->m = (Marker*)calloc(nnode > 0 ? nnode : 1, sizeof(Marker));
    for (int k = 0; k < nbd; k++) {
        const LifeBodyDesc* d = &bodies[k];
        int ID = d->id;
        for (int q = 0; q < d->number; q++) {
            double pos[2] = {d->x + q * d->dx, d->y + q * d->dy};
            Body* b = &c->b[c->nb];
            b->ID = ID++;
            b->kind = d->kind;
            int ib = c->nb++;
            if (d->kind == LIFE_BODY_CIRCLE) {
                /* IBMBodyClass circle ctor (src/IBMBody.cpp:45-76) */
                b->flex = 0;
                int nn = (int)floor(2.0 * M_PI * d->radius / c->Dx);
                b->nodes = (int*)calloc(nn > 0 ? nn : 1, sizeof(int));
                for (int i = 0; i < nn; i++) {
                    double p[2] = {pos[0] + d->radius * cos(i * 2.0 * M_PI / nn),
                                   pos[1] + d->radius * sin(i * 2.0 * M_PI / nn)};
                    add_marker(c, ib, p);
                }
            } else {
                /* IBMBodyClass filament ctor (src/IBMBody.cpp:79-135) */
                b->flex = d->flexible ? 1 : 0;
                double length = d->length;
                double angle = d->angle_deg * M_PI / 180.0;
                double T[2][2] = {{cos(angle), -sin(angle)}, {sin(angle), cos(angle)}};
                int nn = (int)floor(length / c->Dx) + 1;
                b->nodes = (int*)calloc(nn, sizeof(int));
                for (int i = 0; i < nn; i++) {
                    double p[2] = {i * length / (nn - 1), 0.0};
                    double r[2];
                    for (int a = 0; a < 2; a++) r[a] = 0.0 + T[a][0] * p[0] + T[a][1] * p[1];
                    double q2[2] = {pos[0] + r[0], pos[1] + r[1]};
                    add_marker(c, ib, q2);
                }
                if (b->flex) b->fem = build_fem(c, pos, d, angle, nn);
            }
        }
    }
    for (int i = 0; i < c->nb; i++)
        for (int j = i + 1; j < c->nb; j++)
            if (c->b[i].ID == c->b[j].ID)
                return fail(LIFE_ERR_GEOMETRY, "Duplicate body IDs in geometry.config...exiting");
    int rc = remove_overlap(c);
    if (rc) return rc;
    c->hasIBM = c->nb > 0;
    for (int ib = 0; ib < c->nb; ib++)
        if (c->b[ib].flex) c->hasFlex = 1;
    if (c->hasIBM) {
        /* ObjectsClass::initialiseObjects (src/Objects.cpp:941-961) */
        if (c->p.has_initial_deflect && c->hasFlex)
            for (int ib = 0; ib < c->nb; ib++)
                if (c->b[ib].flex) {
                    rc = fem_initial_deflection(c, &c->b[ib]);
                    if (rc) return rc;
                }
        for (int k = 0; k < c->nm; k++) {
            rc = find_support(c, &c->m[k]);
            if (rc) return rc;
            compute_ds(c, k);
        }
        rc = compute_epsilon(c);
        if (rc) return rc;
    }
    c->nFlex = c->simDOFs = 0;
    for (int ib = 0; ib < c->nb; ib++)
        if (c->b[ib].flex) {
            c->nFlex++;
            c->simDOFs += c->b[ib].fem->bodyDOFs;
        }
    return LIFE_OK;
}

/* GridClass::GridClass + initialiseGrid (src/Grid.cpp:916-1062, 1232-1289) */
int oracle_create(const LifeCaseParams* p, const LifeBodyDesc* bodies, int nbodies, OracleCase** out) {
    *out = NULL;
    if (p->Nx < 4 || p->Ny < 4) return fail(LIFE_ERR_INVALID, "oracle: lattice must be at least 4x4");
    if (p->wall_left == LIFE_CONVECTIVE || p->wall_bottom == LIFE_CONVECTIVE || p->wall_top == LIFE_CONVECTIVE)
        return fail(LIFE_ERR_INVALID, "Currently convective BC only supported for right boundary...exiting");
    OracleCase* c = (OracleCase*)calloc(1, sizeof(OracleCase));
    c->p = *p;
    const int Nx = p->Nx, Ny = p->Ny;
    c->Nx = Nx;
    c->Ny = Ny;
    double rho0 = 1.0;
    c->c_s = 1.0 / sqrt(3.0);
    c->w[0] = 4.0 / 9.0;
    for (int v = 1; v < 5; v++) c->w[v] = 1.0 / 9.0;
    for (int v = 5; v < 9; v++) c->w[v] = 1.0 / 36.0;
    c->omega = p->omega;
    c->t = 0;
    c->tau = 1.0 / p->omega;
    c->nu = (c->tau - 0.5) * SQ(c->c_s);
    c->Dx = p->height_p / (Ny - 1);
    c->Dt = SQ(c->Dx) * c->nu / p->nu_p;
    c->Dm = (p->rho_p / rho0) * TH(c->Dx);
    c->Drho = (p->rho_p / rho0);
    size_t n = (size_t)Nx * Ny;
    c->u = calloc(n * 2, sizeof(double));
    c->u_n = calloc(n * 2, sizeof(double));
    c->rho = malloc(n * sizeof(double));
    c->rho_n = malloc(n * sizeof(double));
    for (size_t k = 0; k < n; k++) c->rho[k] = c->rho_n[k] = rho0;
    c->force_xy = calloc(n * 2, sizeof(double));
    c->force_ibm = calloc(n * 2, sizeof(double));
    c->type = calloc(n, 1);
    c->f = calloc(n * NV, sizeof(double));
    c->f_n = calloc(n * NV, sizeof(double));
    c->u_in = calloc((size_t)Ny * 2, sizeof(double));
    c->rho_in = malloc((size_t)Ny * sizeof(double));
    for (int j = 0; j < Ny; j++) c->rho_in[j] = rho0;
    c->delU = calloc((size_t)Ny * 2, sizeof(double));
    c->bc = malloc(n * sizeof(int));
    /* type matrix; y walls override x walls at corners (src/Grid.cpp:925-951) */
    for (int i = 0; i < Nx; i++)
        for (int j = 0; j < Ny; j++) {
            int id = i * Ny + j;
            if (i == 0) c->type[id] = (signed char)p->wall_left;
            else if (i == Nx - 1) c->type[id] = (signed char)p->wall_right;
            if (j == 0) c->type[id] = (signed char)p->wall_bottom;
            else if (j == Ny - 1) c->type[id] = (signed char)p->wall_top;
            if (c->type[id] != LIFE_FLUID) c->bc[c->nbc++] = id;
        }
    /* normals (GridClass::getNormalVector, src/Grid.cpp:498-545) */
    c->bcn = malloc(sizeof(int) * 3 * (c->nbc > 0 ? c->nbc : 1));
    for (int k = 0; k < c->nbc; k++) {
        int id = c->bc[k], i = id / Ny, j = id - i * Ny;
        int nv[2] = {0, 0}, nd = 0;
        if (i == 0) { nv[0] = 1; nd = 0; }
        else if (i == Nx - 1) { nv[0] = -1; nd = 0; }
        if (j == 0) { nv[1] = 1; nd = 1; }
        else if (j == Ny - 1) { nv[1] = -1; nd = 1; }
        if (nv[0] != 0 && nv[1] != 0) {
            int tx = c->type[(i + nv[0]) * Ny + j], ty = c->type[i * Ny + j + nv[1]];
            if (tx == LIFE_FLUID && ty == LIFE_FLUID) {
                oracle_destroy(c);
                return fail(LIFE_ERR_INVALID, "Corner node is surrounded by fluid lattice sites...exiting");
            } else if (tx == LIFE_FLUID) { nd = 0; nv[1] = 0; }
            else if (ty == LIFE_FLUID) { nd = 1; nv[0] = 0; }
        }
        c->bcn[k * 3 + 0] = nv[0];
        c->bcn[k * 3 + 1] = nv[1];
        c->bcn[k * 3 + 2] = nd;
    }
    /* inlet profile (src/Grid.cpp:954-996) */
    for (int j = 0; j < Ny; j++) {
        double Dt = c->Dt, Dx = c->Dx;
        if (p->profile < 0) {
            c->u_in[j * 2 + 0] = p->uxInlet_p * Dt / Dx;
            c->u_in[j * 2 + 1] = p->uyInlet_p * Dt / Dx;
        } else if (p->profile == LIFE_PROFILE_PARABOLIC) {
            double R = p->height_p / 2.0, Y = j * Dx - R;
            c->u_in[j * 2 + 0] = 1.5 * (p->uxInlet_p * Dt / Dx) * (1.0 - SQ(Y / R));
            c->u_in[j * 2 + 1] = 1.5 * (p->uyInlet_p * Dt / Dx) * (1.0 - SQ(Y / R));
        } else if (p->profile == LIFE_PROFILE_SHEAR) {
            double H = p->height_p, Y = j * Dx;
            c->u_in[j * 2 + 0] = (p->uxInlet_p * Dt / Dx) * (Y / H);
            c->u_in[j * 2 + 1] = (p->uyInlet_p * Dt / Dx) * (Y / H);
        } else if (p->profile == LIFE_PROFILE_BOUNDARY_LAYER) {
            double H = p->height_p, Y = j * Dx;
            c->u_in[j * 2 + 0] = ((1.5 * p->uxInlet_p * Dt / Dx) / SQ(H)) * Y * (2.0 * H - Y);
            c->u_in[j * 2 + 1] = ((1.5 * p->uyInlet_p * Dt / Dx) / SQ(H)) * Y * (2.0 * H - Y);
        }
    }
    /* initial velocity (src/Grid.cpp:999-1028) */
    for (int i = 0; i < Nx; i++)
        for (int j = 0; j < Ny; j++) {
            int id = i * Ny + j;
            if (p->has_inlet_ramp) {
                c->u[id * 2 + 0] = 0.0;
                c->u[id * 2 + 1] = 0.0;
            } else if (p->profile >= 0) {
                c->u[id * 2 + 0] = c->u_in[j * 2 + 0];
                c->u[id * 2 + 1] = c->u_in[j * 2 + 1];
            } else {
                c->u[id * 2 + 0] = p->ux0_p * c->Dt / c->Dx;
                c->u[id * 2 + 1] = p->uy0_p * c->Dt / c->Dx;
            }
            if (c->type[id] == LIFE_WALL) {
                c->u[id * 2 + 0] = 0.0;
                c->u[id * 2 + 1] = 0.0;
            }
        }
    memcpy(c->u_n, c->u, n * 2 * sizeof(double));
    memcpy(c->rho_n, c->rho, n * sizeof(double));
    for (size_t id = 0; id < n; id++) {
        c->force_xy[id * 2 + 0] = (c->rho[id] * c->Drho * p->gravityX + p->dpdx) * SQ(c->Dx * c->Dt) / c->Dm;
        c->force_xy[id * 2 + 1] = (c->rho[id] * c->Drho * p->gravityY + p->dpdy) * SQ(c->Dx * c->Dt) / c->Dm;
    }
    for (size_t id = 0; id < n; id++)
        for (int v = 0; v < NV; v++) c->f[id * NV + v] = equilibrium(c, (int)id, v);
    memcpy(c->f_n, c->f, n * NV * sizeof(double));
    /* ObjectsClass ctor (src/Objects.cpp:1589-1624) */
    c->relax = p->relaxMax;
    int rc = build_objects(c, bodies, nbodies);
    if (rc) {
        oracle_destroy(c);
        return rc;
    }
    *out = c;
    return LIFE_OK;
}

/* main loop body: grid.t++ then grid.solver() (src/main.cpp:70-73) */
int oracle_step(OracleCase* c, int nsteps) {
    for (int s = 0; s < nsteps; s++) {
        c->t++;
        lbm_kernel(c);
        if (c->hasIBM) {
            int rc = object_kernel(c);
            if (rc) return rc;
        }
    }
    return LIFE_OK;
}

int oracle_time(const OracleCase* c) { return c->t; }

int oracle_counts(const OracleCase* c, int* n_markers, int* n_bodies, int* n_flex, int* sim_dofs) {
    if (n_markers) *n_markers = c->nm;
    if (n_bodies) *n_bodies = c->nb;
    if (n_flex) *n_flex = c->nFlex;
    if (sim_dofs) *sim_dofs = c->simDOFs;
    return LIFE_OK;
}

int oracle_get_fields(const OracleCase* c, double* rho, double* u, double* f, double* fibm) {
    size_t n = (size_t)c->Nx * c->Ny;
    if (rho) memcpy(rho, c->rho, n * sizeof(double));
    if (u) memcpy(u, c->u, n * 2 * sizeof(double));
    if (f) memcpy(f, c->f, n * NV * sizeof(double));
    if (fibm) memcpy(fibm, c->force_ibm, n * 2 * sizeof(double));
    return LIFE_OK;
}

/* GridClass::readRestart (src/Grid.cpp:1072-1160) */
int oracle_set_fields(OracleCase* c, int t, const double* rho, const double* u, const double* f,
                      const double* fibm) {
    size_t n = (size_t)c->Nx * c->Ny;
    c->t = t;
    c->tOffset = t;
    if (rho) memcpy(c->rho, rho, n * sizeof(double));
    if (u) memcpy(c->u, u, n * 2 * sizeof(double));
    if (f) memcpy(c->f, f, n * NV * sizeof(double));
    if (fibm) memcpy(c->force_ibm, fibm, n * 2 * sizeof(double));
    return LIFE_OK;
}

int oracle_get_markers(const OracleCase* c, double* pos, double* vel, double* force, double* eps,
                       double* ds, int* body_index) {
    for (int k = 0; k < c->nm; k++) {
        const Marker* m = &c->m[k];
        for (int d = 0; d < 2; d++) {
            if (pos) pos[k * 2 + d] = m->pos[d];
            if (vel) vel[k * 2 + d] = m->vel[d];
            if (force) force[k * 2 + d] = m->force[d];
        }
        if (eps) eps[k] = m->epsilon;
        if (ds) ds[k] = m->ds;
        if (body_index) body_index[k] = m->body;
    }
    return LIFE_OK;
}

int oracle_get_bodies(const OracleCase* c, int* ids, int* flexible, int* n_markers, int* n_fem_nodes) {
    for (int ib = 0; ib < c->nb; ib++) {
        if (ids) ids[ib] = c->b[ib].ID;
        if (flexible) flexible[ib] = c->b[ib].flex;
        if (n_markers) n_markers[ib] = c->b[ib].nNodes;
        if (n_fem_nodes) n_fem_nodes[ib] = c->b[ib].fem ? c->b[ib].fem->nNodes : 0;
    }
    return LIFE_OK;
}

int oracle_get_fem(const OracleCase* c, int k, double* U, double* Udot, double* Udotdot, double* U_n,
                   double* U_nm1, double* R_k, double* el_L, double* el_angle, double* node_pos,
                   double* node_angle) {
    int q = -1;
    for (int ib = 0; ib < c->nb; ib++)
        if (c->b[ib].flex && ++q == k) {
            const FemBody* fb = c->b[ib].fem;
            size_t nd = (size_t)fb->bodyDOFs * sizeof(double);
            if (U) memcpy(U, fb->U, nd);
            if (Udot) memcpy(Udot, fb->Udot, nd);
            if (Udotdot) memcpy(Udotdot, fb->Udotdot, nd);
            if (U_n) memcpy(U_n, fb->U_n, nd);
            if (U_nm1) memcpy(U_nm1, fb->U_nm1, nd);
            if (R_k) memcpy(R_k, fb->R_k, nd);
            for (int e = 0; e < fb->nEl; e++) {
                if (el_L) el_L[e] = fb->el[e].L;
                if (el_angle) el_angle[e] = fb->el[e].angle;
            }
            for (int n = 0; n < fb->nNodes; n++) {
                if (node_pos) { node_pos[n * 2] = fb->pos[n][0]; node_pos[n * 2 + 1] = fb->pos[n][1]; }
                if (node_angle) node_angle[n] = fb->anglen[n];
            }
            return LIFE_OK;
        }
    return fail(LIFE_ERR_INVALID, "oracle: no flexible body %d", k);
}

int oracle_get_nr(const OracleCase* c, int k, int* itNR, double* resNR) {
    int q = -1;
    for (int ib = 0; ib < c->nb; ib++)
        if (c->b[ib].flex && ++q == k) {
            if (itNR) *itNR = c->b[ib].fem->itNR;
            if (resNR) *resNR = c->b[ib].fem->resNR;
            return LIFE_OK;
        }
    return fail(LIFE_ERR_INVALID, "oracle: no flexible body %d", k);
}

int oracle_get_relax(const OracleCase* c, double* relax, int* subits, double* subres) {
    if (relax) *relax = c->relax;
    if (subits) *subits = c->subIt;
    if (subres) *subres = c->subRes;
    return LIFE_OK;
}

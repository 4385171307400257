/*
 * Stand-in for the reference's inc/defs.h, for a LIFE params.h compiled
 * against life_params_pack.h and for the reference-interface classes of
 * include/life_ref_shim: a params.h starts with #include "defs.h" and uses
 * these constants, enumerations and macros (reference inc/defs.h:34-58), and
 * the reference's main() uses the standard streams, `using namespace std`
 * and omp_get_wtime (inc/defs.h:21-27). The enumerator values are those of
 * the reference, so WALL_* and PROFILE settings map one to one onto
 * LIFE_FLUID..LIFE_CONVECTIVE and LIFE_PROFILE_*.
 */
#ifndef DEFS_H
#define DEFS_H
#include <array>
#include <cmath>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#else
#include <chrono>
/* wall-clock seconds, for builds without OpenMP (the GPU path needs none) */
inline double omp_get_wtime() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
inline void omp_set_num_threads(int) {}
#endif
using namespace std;

const string version = "v1.0.3 (GB300)";

const int dims = 2;
const int nVels = 9;
const int suppSize = 9;
const int nodeDOFs = 3;
const int elementNodes = 2;
const int elementDOFs = elementNodes * nodeDOFs;

enum eDirectionType {eX, eY};
enum eFlexibleType {eFlexible, eRigid};
enum eBCType {eClamped, eSupported};
enum eBodyType {eCircle, eFilament};
enum eLatType {eFluid, eWall, eVelocity, eFreeSlip, ePressure, eConvective};
enum eProfileType {eParabolic, eShear, eBoundaryLayer};

#define SQ(x) ((x) * (x))
#define TH(x) ((x) * (x) * (x))
#define QU(x) ((x) * (x) * (x) * (x))
#endif

/*
 * Stand-in for the reference's inc/defs.h when a LIFE params.h is compiled
 * against life_params_pack.h: a params.h starts with #include "defs.h" and
 * uses these constants, enumerations and macros (reference inc/defs.h:34-58). The
 * enumerator values are those of the reference, so WALL_* and PROFILE
 * settings map one to one onto LIFE_FLUID..LIFE_CONVECTIVE and
 * LIFE_PROFILE_*.
 */
#ifndef DEFS_H
#define DEFS_H
#include <cmath>
#include <string>
using namespace std;

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

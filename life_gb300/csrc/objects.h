// Host-side immersed bodies: construction from geometry lines, marker
// de-overlap, FEM set-up, and the start-up quantities (static pre-deflection,
// support, ds, epsilon). These run once per case on the host in FP64 with the
// reference's operation order; the per-step work runs on the device.
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "../../include/life_gb300.h"

namespace life {

struct Grid0 {  // lattice scalars the bodies need
    int Nx, Ny;
    double Dx, Dt, Dm;
    double gravityX, gravityY;
    double ref_L, alpha, delta;
};

struct HMarker {
    int body = 0;
    int ID = 0;
    double pos[2] = {0, 0}, vel[2] = {0, 0}, force[2] = {0, 0};
    double ds = 0, eps = 0;
    int nsupp = 0;
    int si[9] = {0}, sj[9] = {0};
    double sd[9] = {0};
};

struct HForceMap {
    int node;
    double z1, z2;
};

struct HElement {
    double L0 = 0, L = 0, angle = 0, A = 0, I = 0, E = 0, rho = 0;
    double T[6][6] = {{0}}, M[6][6] = {{0}}, KL[6][6] = {{0}}, KNL[6][6] = {{0}}, R[6] = {0}, F[6] = {0};
    int dof[6] = {0};
    int node[2] = {0, 0};
    std::vector<HForceMap> fmap;
};

struct HFem {
    int nNodes = 0, nEl = 0, dofs = 0, bc = 0;
    double L0 = 0, angle0 = 0, tCrit = 0;
    int itNR = 0;
    double resNR = 0;
    std::vector<double> pos0, pos, angle0n, anglen;  // pos: [n][2]
    std::vector<HElement> el;
    std::vector<int> mapEl;
    std::vector<double> mapZeta;
    std::vector<double> M, K, R, F, U, delU, Udot, Udotdot, U_n, U_nm1, U_nm2, Udot_n, Udotdot_n, U_km1, R_k, R_km1;
};

struct HBody {
    int ID = 0, flex = 0, kind = 0;
    std::vector<int> nodes;  // marker indices
    HFem* fem = nullptr;
};

struct HObjects {
    std::vector<HMarker> m;
    std::vector<HBody> b;
    bool hasIBM = false, hasFlex = false;
    int nFlex = 0, simDOFs = 0;
    ~HObjects();
};

// The marker pairs (n1 < n2) closer than half a lattice spacing, in
// (n1, n2) order: the test of ObjectsClass::removeOverlapMarkers
// (src/Objects.cpp:873-884) over all pairs. pos is [nm][2]. Returns LIFE_OK
// or an error code with *err set.
typedef int (*OverlapScan)(const double* pos, int nm, double Dx, std::vector<std::pair<int, int>>* pairs,
                           std::string* err);

// Builds bodies (ObjectsClass::geometryReadIn + IBMBodyClass ctors), removes
// overlapping markers and runs initialiseObjects. Returns LIFE_OK or an
// error code with *err set. With `scan`, marker sets of at least `scan_min`
// markers find their close pairs through it (the device kernel); smaller
// sets, or no scan, test the pairs on the host. Both apply the same test to
// the same values.
constexpr int kOverlapScanMin = 2048;
int build_objects(const Grid0& g, const LifeCaseParams& p, const LifeBodyDesc* d, int nd, HObjects& out,
                  std::string* err, OverlapScan scan = nullptr, int scan_min = kOverlapScanMin);

// IBM start-up helpers (also used after restarts).
int host_find_support(const Grid0& g, HMarker& m, std::string* err);
void host_compute_ds(const Grid0& g, HObjects& o, int k);
int host_compute_epsilon(const Grid0& g, HObjects& o, bool uni, bool first_step, std::string* err);

// Element matrices / transforms shared with the device upload.
void fem_element_transform(HElement& e);

}  // namespace life

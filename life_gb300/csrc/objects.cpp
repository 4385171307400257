// Host-side construction of the immersed bodies (see objects.h). Arithmetic
// keeps the reference's operation order; the translation unit is compiled
// without FMA contraction so start-up values equal the reference's.
#include "objects.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <numeric>
#include <thread>

#include "band_lu.h"

namespace life {

static const double PI = 3.14159265358979323846;
#define HSQ(x) ((x) * (x))
#define HTH(x) ((x) * (x) * (x))

HObjects::~HObjects() {
    for (auto& b : this->b) delete b.fem;
}

// Utils::diracDelta (reference inc/Utils.h:220-232)
static double dirac(double dist) {
    double a = std::fabs(dist);
    if (a > 1.5) return 0.0;
    if (a > 0.5) return (5.0 - 3.0 * a - std::sqrt(-3.0 * HSQ(1.0 - a) + 1.0)) / 6.0;
    return (1.0 + std::sqrt(1.0 - 3.0 * HSQ(a))) / 3.0;
}

// Utils::shiftAngle (inc/Utils.h:235-246)
static double shift_angle(double angle) {
    angle = std::fmod(angle + PI, 2.0 * PI);
    if (angle < 0.0) angle += 2.0 * PI;
    return angle - PI;
}

static int sgn(double v) { return (0.0 < v) - (v < 0.0); }

// IBMNodeClass::findSupport (src/IBMNode.cpp:139-179)
int host_find_support(const Grid0& g, HMarker& m, std::string* err) {
    const double Dx = g.Dx;
    int inear = (int)std::round(m.pos[0] / Dx), jnear = (int)std::round(m.pos[1] / Dx);
    m.nsupp = 0;
    for (int s = 0; s < 9; s++) { m.si[s] = 0; m.sj[s] = 0; m.sd[s] = 0.0; }
    for (int i = inear - 2; i <= inear + 2; i++) {
        double dX = std::fabs(m.pos[0] / Dx - i);
        for (int j = jnear - 2; j <= jnear + 2; j++) {
            double dY = std::fabs(m.pos[1] / Dx - j);
            if (dX < 1.5 && dY < 1.5 && i >= 0 && i <= g.Nx - 1 && j >= 0 && j <= g.Ny - 1) {
                if (m.nsupp == 9) {
                    if (err) *err = "Support buffer size is not big enough for number of support points...exiting";
                    return LIFE_ERR_SUPPORT;
                }
                m.si[m.nsupp] = i;
                m.sj[m.nsupp] = j;
                m.sd[m.nsupp] = dirac(dX) * dirac(dY);
                m.nsupp++;
            }
        }
    }
    return LIFE_OK;
}

// IBMNodeClass::computeDs (src/IBMNode.cpp:182-204)
void host_compute_ds(const Grid0& g, HObjects& o, int k) {
    HMarker& m = o.m[k];
    const HBody& b = o.b[m.body];
    double cur = 10.0;
    for (int n : b.nodes) {
        const HMarker& q = o.m[n];
        if (m.ID != q.ID) {
            double d0 = m.pos[0] - q.pos[0], d1 = m.pos[1] - q.pos[1];
            double dd = 0.0;
            dd += d0 * d0;
            dd += d1 * d1;
            double mag = std::sqrt(dd) / g.Dx;
            if (mag < cur) cur = mag;
        }
    }
    m.ds = cur;
}

// Epsilon system of one marker set (ObjectsClass::computeEpsilon,
// src/Objects.cpp:264-311), solved with the band-limited LU.
static int epsilon_set(const Grid0& g, HObjects& o, const std::vector<int>& nodes) {
    const int dim = (int)nodes.size();
    if (dim == 0) return LIFE_OK;
    std::vector<double> A((size_t)dim * dim, 0.0), b(dim, 1.0), x(dim);
    std::vector<int> piv(dim);
    const double Dx = g.Dx;
    for (int i = 0; i < dim; i++) {
        const HMarker& ni = o.m[nodes[i]];
        for (int j = 0; j < dim; j++) {
            const HMarker& nj = o.m[nodes[j]];
            double acc = 0.0;
            bool any = false;
            for (int s = 0; s < ni.nsupp; s++) {
                double dvi = ni.sd[s];
                double dX = std::fabs(nj.pos[0] / Dx - ni.si[s]);
                double dY = std::fabs(nj.pos[1] / Dx - ni.sj[s]);
                double dvj = dirac(dX) * dirac(dY);
                acc += dvi * dvj;
                any = true;
            }
            (void)any;
            A[(size_t)i * dim + j] = acc * (1.0 * 1.0 * nj.ds);
        }
    }
    int kl, ku;
    lu_bandwidth(A.data(), dim, 0, &kl, &ku);
    lu_band_factor(A.data(), dim, 0, kl, ku, piv.data());
    lu_band_solve(A.data(), dim, 0, kl, ku, piv.data(), b.data(), x.data());
    for (int i = 0; i < dim; i++) o.m[nodes[i]].eps = x[i];
    return LIFE_OK;
}

// Groups of markers whose epsilon rows can couple (|dx|,|dy| < 3 lattice
// units, in index order). A dense LU of the all-marker system factors each
// group independently with identical arithmetic, so solving per group gives
// the same result as the reference's single UNI_EPSILON solve.
static std::vector<std::vector<int>> coupling_groups(const Grid0& g, const HObjects& o, const std::vector<int>& set) {
    const int n = (int)set.size();
    std::vector<int> parent(n);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int a) {
        while (parent[a] != a) a = parent[a] = parent[parent[a]];
        return a;
    };
    for (int a = 0; a < n; a++)
        for (int c = a + 1; c < n; c++) {
            const HMarker& p = o.m[set[a]];
            const HMarker& q = o.m[set[c]];
            if (std::fabs(p.pos[0] - q.pos[0]) / g.Dx < 3.0 && std::fabs(p.pos[1] - q.pos[1]) / g.Dx < 3.0) {
                int ra = find(a), rc = find(c);
                if (ra != rc) parent[ra > rc ? ra : rc] = ra < rc ? ra : rc;
            }
        }
    std::vector<std::vector<int>> groups;
    std::vector<int> gid(n, -1);
    for (int a = 0; a < n; a++) {
        int r = find(a);
        if (gid[r] < 0) { gid[r] = (int)groups.size(); groups.emplace_back(); }
        groups[gid[r]].push_back(set[a]);
    }
    return groups;
}

int host_compute_epsilon(const Grid0& g, HObjects& o, bool uni, bool first_step, std::string* err) {
    (void)err;
    if (uni) {
        std::vector<int> all(o.m.size());
        std::iota(all.begin(), all.end(), 0);
        for (auto& grp : coupling_groups(g, o, all)) {
            int rc = epsilon_set(g, o, grp);
            if (rc) return rc;
        }
        return LIFE_OK;
    }
    for (auto& b : o.b)
        if (first_step || b.flex) {
            int rc = epsilon_set(g, o, b.nodes);
            if (rc) return rc;
        }
    return LIFE_OK;
}

// ------------------------------------------------------------------- FEM

void fem_element_transform(HElement& e) {
    e.T[0][0] = e.T[1][1] = e.T[3][3] = e.T[4][4] = std::cos(e.angle);
    e.T[0][1] = e.T[3][4] = std::sin(e.angle);
    e.T[1][0] = e.T[4][3] = -std::sin(e.angle);
    e.T[2][2] = e.T[5][5] = 1.0;
}

// FEMElementClass::setLocalMatrices (src/FEMElement.cpp:203-252)
static void element_local(HElement& e) {
    std::memset(e.M, 0, sizeof e.M);
    std::memset(e.KL, 0, sizeof e.KL);
    std::memset(e.KNL, 0, sizeof e.KNL);
    const double L0 = e.L0, E = e.E, A = e.A, I = e.I;
    const double C1 = e.rho * A * L0 / 420.0;
    e.M[0][0] = C1 * 140.0;
    e.M[0][3] = C1 * 70.0;
    e.M[1][1] = C1 * 156.0;
    e.M[1][2] = C1 * 22.0 * L0;
    e.M[1][4] = C1 * 54;
    e.M[1][5] = C1 * (-13.0 * L0);
    e.M[2][2] = C1 * 4.0 * HSQ(L0);
    e.M[2][4] = C1 * 13.0 * L0;
    e.M[2][5] = C1 * (-3.0 * HSQ(L0));
    e.M[3][3] = C1 * 140.0;
    e.M[4][4] = C1 * 156.0;
    e.M[4][5] = C1 * (-22.0 * L0);
    e.M[5][5] = C1 * 4.0 * HSQ(L0);
    e.KL[0][0] = E * A / L0;
    e.KL[0][3] = -E * A / L0;
    e.KL[1][1] = 12.0 * E * I / HTH(L0);
    e.KL[1][2] = 6.0 * E * I / HSQ(L0);
    e.KL[1][4] = -12.0 * E * I / HTH(L0);
    e.KL[1][5] = 6.0 * E * I / HSQ(L0);
    e.KL[2][2] = 4.0 * E * I / L0;
    e.KL[2][4] = -6.0 * E * I / HSQ(L0);
    e.KL[2][5] = 2.0 * E * I / L0;
    e.KL[3][3] = E * A / L0;
    e.KL[4][4] = 12.0 * E * I / HTH(L0);
    e.KL[4][5] = -6.0 * E * I / HSQ(L0);
    e.KL[5][5] = 4.0 * E * I / L0;
    for (int i = 1; i < 6; i++)
        for (int j = 0; j < i; j++) {
            e.M[i][j] = e.M[j][i];
            e.KL[i][j] = e.KL[j][i];
        }
}

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

// FEMBodyClass::updateFEMValues (src/FEMBody.cpp:198-223)
static void fem_update_values(HFem& f) {
    for (int n = 0; n < f.nNodes; n++) {
        for (int d = 0; d < 2; d++) f.pos[n * 2 + d] = f.pos0[n * 2 + d] + f.U[n * 3 + d];
        f.anglen[n] = f.angle0n[n] + f.U[n * 3 + 2];
    }
    for (auto& e : f.el) {
        double ev0 = f.pos[e.node[1] * 2] - f.pos[e.node[0] * 2];
        double ev1 = f.pos[e.node[1] * 2 + 1] - f.pos[e.node[0] * 2 + 1];
        e.angle = std::atan2(ev1, ev0);
        double dd = 0.0;
        dd += ev0 * ev0;
        dd += ev1 * ev1;
        e.L = std::sqrt(dd);
        fem_element_transform(e);
    }
}

// Products with an element rotation T (fem_element_transform): T is block
// diagonal, [[c, s], [-s, c]] on DOFs 0-1 and 3-4 and 1 on DOFs 2 and 5, so
// row or column q of T is non-zero only at the DOFs of q's block (t_blk).
// These forms skip the structurally zero terms of mat6_mul / mat6_vec and add
// the others in the same order. A skipped term is an exact zero, and adding a
// zero leaves a sum that started at +0 unchanged (such a sum is never -0), so
// every result equals the dense product's bit for bit.
static inline int t_blk(int q, int k[2]) {
    if (q == 2 || q == 5) {
        k[0] = q;
        return 1;
    }
    k[0] = q < 3 ? 0 : 3;
    k[1] = k[0] + 1;
    return 2;
}
// R = T^T A
static void mat6_tt_mul(double R[6][6], const double T[6][6], const double A[6][6]) {
    for (int i = 0; i < 6; i++) {
        int k[2];
        const int nk = t_blk(i, k);
        for (int j = 0; j < 6; j++) {
            double s = 0.0;
            for (int q = 0; q < nk; q++) s += T[k[q]][i] * A[k[q]][j];
            R[i][j] = s;
        }
    }
}
// R = A T
static void mat6_mul_t(double R[6][6], const double A[6][6], const double T[6][6]) {
    for (int j = 0; j < 6; j++) {
        int k[2];
        const int nk = t_blk(j, k);
        for (int i = 0; i < 6; i++) {
            double s = 0.0;
            for (int q = 0; q < nk; q++) s += A[i][k[q]] * T[k[q]][j];
            R[i][j] = s;
        }
    }
}
// r = T^T v
static void mat6_tt_vec(double r[6], const double T[6][6], const double v[6]) {
    for (int i = 0; i < 6; i++) {
        int k[2];
        const int nk = t_blk(i, k);
        double s = 0.0;
        for (int q = 0; q < nk; q++) s += T[k[q]][i] * v[k[q]];
        r[i] = s;
    }
}

// Largest |dof_i - dof_j| within one element: assembly writes K only there.
static int fem_half_band(const HFem& f) {
    int hw = 0;
    for (const auto& e : f.el) {
        int lo = e.dof[0], hi = e.dof[0];
        for (int k = 1; k < 6; k++) {
            lo = e.dof[k] < lo ? e.dof[k] : lo;
            hi = e.dof[k] > hi ? e.dof[k] : hi;
        }
        hw = hi - lo > hw ? hi - lo : hw;
    }
    return hw;
}

// forceVector + stiffMatrix of all elements for the static solve
// (FEMBodyClass::buildGlobalMatrices, src/FEMBody.cpp:90-109;
// src/FEMElement.cpp:72-138; the mass matrix is not used by
// newtonRaphsonStatic and is not formed). Every entry of K is the same sum in
// the same element order as the dense assembly. K is stored densely, but only
// entries with |row - col| <= 2 hw can be non-zero: assembly writes |.| <= hw
// and the band LU's fill-in reaches kl + ku <= 2 hw. Only those are cleared,
// the rest stay zero from the allocation.
static void fem_build_static(HFem& f, int hw) {
    const int n = f.dofs, w = 2 * hw;
    for (int r = 0; r < n; r++) {
        const int c0 = r - w > 0 ? r - w : 0, c1 = r + w < n - 1 ? r + w : n - 1;
        std::fill(f.K.begin() + (size_t)r * n + c0, f.K.begin() + (size_t)r * n + c1 + 1, 0.0);
    }
    std::fill(f.F.begin(), f.F.end(), 0.0);
    for (auto& e : f.el) {
        double u = (HSQ(e.L) - HSQ(e.L0)) / (e.L + e.L0);
        double th1 = shift_angle(f.anglen[e.node[0]] - e.angle);
        double th2 = shift_angle(f.anglen[e.node[1]] - e.angle);
        double F0 = (e.E * e.A / e.L0) * u;
        double M1 = (2 * e.E * e.I / e.L0) * (2.0 * th1 + th2);
        double M2 = (2 * e.E * e.I / e.L0) * (th1 + 2.0 * th2);
        e.F[0] = -F0;
        e.F[1] = (1.0 / e.L0) * (M1 + M2);
        e.F[2] = M1;
        e.F[3] = F0;
        e.F[4] = -(1.0 / e.L0) * (M1 + M2);
        e.F[5] = M2;
        double tmp[6][6], G[6][6], G2[6][6], FG[6];
        mat6_tt_vec(FG, e.T, e.F);
        for (int i = 0; i < 6; i++) f.F[e.dof[i]] += FG[i];
        mat6_tt_mul(tmp, e.T, e.KL);
        mat6_mul_t(G, tmp, e.T);
        const double Fa = -e.F[0], V0 = e.F[4], L0 = e.L0;
        e.KNL[0][1] = -V0 / L0;
        e.KNL[0][4] = V0 / L0;
        e.KNL[1][0] = -V0 / L0;
        e.KNL[1][1] = Fa / L0;
        e.KNL[1][3] = V0 / L0;
        e.KNL[1][4] = -Fa / L0;
        e.KNL[3][1] = V0 / L0;
        e.KNL[3][4] = -V0 / L0;
        e.KNL[4][0] = V0 / L0;
        e.KNL[4][1] = -Fa / L0;
        e.KNL[4][3] = -V0 / L0;
        e.KNL[4][4] = Fa / L0;
        mat6_tt_mul(tmp, e.T, e.KNL);
        mat6_mul_t(G2, tmp, e.T);
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < 6; j++) f.K[(size_t)e.dof[i] * n + e.dof[j]] += G[i][j] + G2[i][j];
    }
}

// FEMElementClass::shapeFuns (src/FEMElement.cpp:141-160)
static void shape_funs(double res[2], const double v[6], double zeta, double L) {
    double N0 = 1.0 - (zeta + 1.0) / 2.0;
    double N1 = 1.0 - 3.0 * HSQ((zeta + 1.0) / 2.0) + 2.0 * HTH((zeta + 1.0) / 2.0);
    double N2 = ((zeta + 1.0) / 2.0 - 2.0 * HSQ((zeta + 1.0) / 2.0) + HTH((zeta + 1.0) / 2.0)) * L;
    double N3 = (zeta + 1.0) / 2.0;
    double N4 = 3.0 * HSQ((zeta + 1.0) / 2.0) - 2.0 * HTH((zeta + 1.0) / 2.0);
    double N5 = (-HSQ((zeta + 1.0) / 2.0) + HTH((zeta + 1.0) / 2.0)) * L;
    res[0] = v[0] * N0 + v[3] * N3;
    res[1] = v[1] * N1 + v[2] * N2 + v[4] * N4 + v[5] * N5;
}

// FEMBodyClass::updateIBMValues (src/FEMBody.cpp:147-195)
static void fem_update_ibm(HObjects& o, HBody& b) {
    HFem& f = *b.fem;
    for (size_t i = 0; i < f.mapEl.size(); i++) {
        const HElement& e = f.el[f.mapEl[i]];
        const double zeta = f.mapZeta[i];
        double dU[6], dUd[6], lU[6], lUd[6];
        for (int k = 0; k < 6; k++) {
            dU[k] = f.U[e.dof[k]];
            dUd[k] = f.Udot[e.dof[k]];
        }
        for (int n = 0; n < 2; n++) {
            dU[n * 3 + 0] += f.pos0[e.node[n] * 2] - f.pos[e.node[0] * 2];
            dU[n * 3 + 1] += f.pos0[e.node[n] * 2 + 1] - f.pos[e.node[0] * 2 + 1];
            dU[n * 3 + 2] += f.angle0n[e.node[n]] - e.angle;
            dU[n * 3 + 2] = shift_angle(dU[n * 3 + 2]);
        }
        mat6_vec(lU, e.T, dU);
        mat6_vec(lUd, e.T, dUd);
        double sU[2], sUd[2];
        shape_funs(sU, lU, zeta, e.L);
        shape_funs(sUd, lUd, zeta, e.L);
        double gU[2], gUd[2];
        for (int r = 0; r < 2; r++) {
            double a1 = 0.0, a2 = 0.0;
            for (int k = 0; k < 2; k++) {
                a1 += e.T[k][r] * sU[k];
                a2 += e.T[k][r] * sUd[k];
            }
            gU[r] = a1;
            gUd[r] = a2;
        }
        HMarker& m = o.m[b.nodes[i]];
        m.pos[0] = f.pos[e.node[0] * 2] + gU[0];
        m.pos[1] = f.pos[e.node[0] * 2 + 1] + gU[1];
        m.vel[0] = gUd[0];
        m.vel[1] = gUd[1];
    }
}

// lu_bandwidth of a matrix whose entries with |row - col| > w are zero,
// scanning only the others (the same kl, ku).
static void band_extent(const double* A, int dim, int bc, int w, int* kl, int* ku) {
    int lo = 0, hi = 0;
    const int n = dim - bc;
    for (int j = 0; j < n; j++) {
        const int i0 = j - w > 0 ? j - w : 0, i1 = j + w < n - 1 ? j + w : n - 1;
        for (int i = i0; i <= i1; i++)
            if (A[(long long)(bc + j) * dim + (bc + i)] != 0.0) {
                if (i - j > lo) lo = i - j;
                if (j - i > hi) hi = j - i;
            }
    }
    *kl = lo;
    *ku = hi;
}

// FEMBodyClass::setInitialDeflection + staticFEM + newtonRaphsonStatic
// (src/FEMBody.cpp:352-484)
static int fem_initial_deflection(const Grid0& g, const LifeCaseParams& p, HObjects& o, HBody& b, std::string* err) {
    HFem& f = *b.fem;
    const int n = f.dofs;
    const double deflect = -p.initial_deflect;
    const double E = f.el[0].E, I = f.el[0].I;
    const double linearForce = 3.0 * E * I * deflect / HSQ(f.L0);
    const double dFmax = linearForce / (double)100;
    const double T[2][2] = {{std::cos(f.angle0), -std::sin(f.angle0)}, {std::sin(f.angle0), std::cos(f.angle0)}};
    double lf[2] = {0.0, dFmax}, gf[2];
    for (int i = 0; i < 2; i++) gf[i] = 0.0 + T[i][0] * lf[0] + T[i][1] * lf[1];
    f.R[n - 3] = gf[0];
    f.R[n - 2] = gf[1];
    std::vector<double> rhs(n);
    std::vector<int> piv(n);
    const int hw = fem_half_band(f);
    double errv;
    int it = 0;
    do {
        f.itNR = 0;
        do {
            fem_build_static(f, hw);
            for (int i = 0; i < n; i++) rhs[i] = f.R[i] - f.F[i];
            int kl, ku;
            band_extent(f.K.data(), n, f.bc, 2 * hw, &kl, &ku);
            lu_band_factor(f.K.data(), n, f.bc, kl, ku, piv.data());
            lu_band_solve(f.K.data(), n, f.bc, kl, ku, piv.data(), rhs.data(), f.delU.data());
            for (int i = 0; i < n; i++) f.U[i] = f.U[i] + f.delU[i];
            fem_update_values(f);
            double dd = 0.0;
            for (int i = 0; i < n; i++) dd += f.delU[i] * f.delU[i];
            f.resNR = std::sqrt(dd) / (g.ref_L * std::sqrt((double)n));
            f.itNR++;
        } while (f.resNR > 1e-10 && f.itNR < 20);
        fem_update_ibm(o, b);
        const double loc1 = 0.0 + T[0][1] * f.U[n - 3] + T[1][1] * f.U[n - 2];
        errv = deflect - loc1 / f.L0;
        double fc = errv * 1e-3;
        if (std::fabs(fc) > std::fabs(dFmax)) fc = sgn(fc) * std::fabs(dFmax);
        lf[1] += fc;
        for (int i = 0; i < 2; i++) gf[i] = 0.0 + T[i][0] * lf[0] + T[i][1] * lf[1];
        f.R[n - 3] = gf[0];
        f.R[n - 2] = gf[1];
        it++;
        if (it >= 10000) {
            if (err) *err = "max iterations hit! Try changing the gain...exiting";
            return LIFE_ERR_DEFLECT;
        }
    } while (std::fabs(errv) > 1e-10);
    f.itNR = 0;
    f.resNR = 0.0;
    std::fill(f.R.begin(), f.R.end(), 0.0);
    std::fill(f.delU.begin(), f.delU.end(), 0.0);
    return LIFE_OK;
}

// FEMBodyClass ctor (src/FEMBody.cpp:487-578), FEMElementClass ctor
// (src/FEMElement.cpp:265-303) and computeNodeMapping (src/FEMBody.cpp:292-338)
static HFem* build_fem(const Grid0& g, const double pos[2], const LifeBodyDesc& d, double angle, int nIBM) {
    HFem* f = new HFem();
    f->bc = d.clamped ? 3 : 2;
    f->angle0 = angle;
    f->L0 = d.length;
    const int nEl = d.n_elements > 0 ? d.n_elements : (int)std::floor(f->L0 / g.Dx);
    f->nEl = nEl;
    f->nNodes = nEl + 1;
    f->dofs = f->nNodes * 3;
    f->tCrit = (f->L0 / nEl) / std::sqrt(d.E / d.rho);
    const double T[2][2] = {{std::cos(angle), -std::sin(angle)}, {std::sin(angle), std::cos(angle)}};
    f->pos0.resize(f->nNodes * 2);
    f->pos.resize(f->nNodes * 2);
    f->angle0n.assign(f->nNodes, angle);
    f->anglen.assign(f->nNodes, angle);
    for (int i = 0; i < f->nNodes; i++) {
        const double p0 = i * f->L0 / nEl, p1 = 0.0;
        for (int a = 0; a < 2; a++) {
            double r = 0.0 + T[a][0] * p0 + T[a][1] * p1;
            f->pos0[i * 2 + a] = f->pos[i * 2 + a] = pos[a] + r;
        }
    }
    f->el.resize(nEl);
    const double len = f->L0 / nEl;
    for (int i = 0; i < nEl; i++) {
        HElement& e = f->el[i];
        e.L0 = len;
        e.L = len;
        e.angle = angle;
        e.A = g.Dx * d.height;
        e.I = g.Dx * HTH(d.height) / 12.0;
        e.E = d.E;
        e.rho = d.rho;
        e.node[0] = i;
        e.node[1] = i + 1;
        for (int a = 0; a < 2; a++)
            for (int k = 0; k < 3; k++) e.dof[a * 3 + k] = (i + a) * 3 + k;
        fem_element_transform(e);
        element_local(e);
    }
    const int nI = nIBM, nF = f->nNodes;
    f->mapEl.assign(nI, 0);
    f->mapZeta.assign(nI, 0.0);
    f->mapEl[0] = 0;
    f->mapZeta[0] = -1.0;
    for (int i = 1; i < nI; i++) {
        double r = i * ((nF - 1.0) / (nI - 1.0));
        if (std::fmod(r, 1.0) == 0.0) {
            f->mapEl[i] = (int)std::floor(r) - 1;
            f->mapZeta[i] = 1.0;
        } else {
            f->mapEl[i] = (int)std::floor(r);
            f->mapZeta[i] = std::fmod(r, 1.0) * 2.0 - 1.0;
        }
    }
    for (int e = 0; e < nEl; e++)
        for (int node = 0; node < nI; node++) {
            double n1 = -1 + 2.0 * (((double)node - 0.5) * ((nF - 1.0) / (nI - 1.0)) - (double)e) / 1.0;
            double n2 = -1 + 2.0 * (((double)node + 0.5) * ((nF - 1.0) / (nI - 1.0)) - (double)e) / 1.0;
            if ((n1 > -1.0 && n1 < 1.0) || (n2 > -1.0 && n2 < 1.0)) {
                if (n1 < -1.0) n1 = -1.0;
                if (n2 > 1.0) n2 = 1.0;
                f->el[e].fmap.push_back({node, n1, n2});
            }
        }
    const int n = f->dofs;
    f->M.assign((size_t)n * n, 0.0);
    f->K.assign((size_t)n * n, 0.0);
    for (auto* v : {&f->R, &f->F, &f->U, &f->delU, &f->Udot, &f->Udotdot, &f->U_n, &f->U_nm1, &f->U_nm2, &f->Udot_n,
                    &f->Udotdot_n, &f->U_km1, &f->R_k, &f->R_km1})
        v->assign(n, 0.0);
    return f;
}

// ObjectsClass::removeOverlapMarkers (src/Objects.cpp:867-938)
static int remove_overlap(const Grid0& g, HObjects& o, std::string* err, OverlapScan scan, int scan_min) {
    std::vector<int> erase;
    const int nm = (int)o.m.size();
    auto close_pair = [&](int n1, int n2) -> int {
        int f1 = o.b[o.m[n1].body].flex, f2 = o.b[o.m[n2].body].flex;
        if (f1 && f2) {
            if (err) *err = "Cannot place two flexible bodies so close to each other...exiting";
            return LIFE_ERR_GEOMETRY;
        }
        if (f1 && !f2) erase.push_back(o.m[n2].ID);
        if (!f1 && f2) erase.push_back(o.m[n1].ID);
        if (!f1 && !f2) erase.push_back(o.m[n1].ID);
        return LIFE_OK;
    };
    if (scan && nm >= scan_min) {
        std::vector<double> pos((size_t)nm * 2);
        for (int n = 0; n < nm; n++) {
            pos[2 * n] = o.m[n].pos[0];
            pos[2 * n + 1] = o.m[n].pos[1];
        }
        std::vector<std::pair<int, int>> pairs;
        if (int rc = scan(pos.data(), nm, g.Dx, &pairs, err)) return rc;
        for (const auto& pr : pairs)
            if (int rc = close_pair(pr.first, pr.second)) return rc;
    } else {
        for (int n1 = 0; n1 < nm; n1++)
            for (int n2 = n1 + 1; n2 < nm; n2++) {
                double d0 = o.m[n1].pos[0] - o.m[n2].pos[0], d1 = o.m[n1].pos[1] - o.m[n2].pos[1];
                double dd = 0.0;
                dd += d0 * d0;
                dd += d1 * d1;
                if (std::sqrt(dd) / g.Dx < 0.5)
                    if (int rc = close_pair(n1, n2)) return rc;
            }
    }
    for (int id : erase) {
        int k = -1;
        for (int n = 0; n < (int)o.m.size(); n++)
            if (o.m[n].ID == id) { k = n; break; }
        if (k < 0) continue;
        auto& nodes = o.b[o.m[k].body].nodes;
        for (size_t q = 0; q < nodes.size(); q++)
            if (nodes[q] == k) { nodes.erase(nodes.begin() + q); break; }
        for (auto& b : o.b)
            for (auto& q : b.nodes)
                if (q > k) q--;
        o.m.erase(o.m.begin() + k);
    }
    for (size_t n = 0; n < o.m.size(); n++) o.m[n].ID = (int)n;
    return LIFE_OK;
}

int build_objects(const Grid0& g, const LifeCaseParams& p, const LifeBodyDesc* d, int nd, HObjects& o,
                  std::string* err, OverlapScan scan, int scan_min) {
    for (int k = 0; k < nd; k++) {
        const LifeBodyDesc& bd = d[k];
        if (bd.kind != LIFE_BODY_CIRCLE && bd.kind != LIFE_BODY_FILAMENT) {
            if (err) *err = "unknown body kind";
            return LIFE_ERR_GEOMETRY;
        }
        int ID = bd.id;
        for (int q = 0; q < bd.number; q++) {
            const double pos[2] = {bd.x + q * bd.dx, bd.y + q * bd.dy};
            HBody b;
            b.ID = ID++;
            b.kind = bd.kind;
            const int ib = (int)o.b.size();
            if (bd.kind == LIFE_BODY_CIRCLE) {
                // IBMBodyClass circle ctor (src/IBMBody.cpp:45-76)
                b.flex = 0;
                const int nn = (int)std::floor(2.0 * PI * bd.radius / g.Dx);
                for (int i = 0; i < nn; i++) {
                    HMarker m;
                    m.body = ib;
                    m.ID = (int)o.m.size();
                    m.pos[0] = pos[0] + bd.radius * std::cos(i * 2.0 * PI / nn);
                    m.pos[1] = pos[1] + bd.radius * std::sin(i * 2.0 * PI / nn);
                    b.nodes.push_back((int)o.m.size());
                    o.m.push_back(m);
                }
            } else {
                // IBMBodyClass filament ctor (src/IBMBody.cpp:79-135)
                b.flex = bd.flexible ? 1 : 0;
                const double length = bd.length;
                const double angle = bd.angle_deg * PI / 180.0;
                const double T[2][2] = {{std::cos(angle), -std::sin(angle)}, {std::sin(angle), std::cos(angle)}};
                const int nn = (int)std::floor(length / g.Dx) + 1;
                for (int i = 0; i < nn; i++) {
                    const double p0 = i * length / (nn - 1), p1 = 0.0;
                    HMarker m;
                    m.body = ib;
                    m.ID = (int)o.m.size();
                    for (int a = 0; a < 2; a++) m.pos[a] = pos[a] + (0.0 + T[a][0] * p0 + T[a][1] * p1);
                    b.nodes.push_back((int)o.m.size());
                    o.m.push_back(m);
                }
                if (b.flex) b.fem = build_fem(g, pos, bd, angle, nn);
            }
            o.b.push_back(std::move(b));
        }
    }
    for (size_t i = 0; i < o.b.size(); i++)
        for (size_t j = i + 1; j < o.b.size(); j++)
            if (o.b[i].ID == o.b[j].ID) {
                if (err) *err = "Duplicate body IDs in geometry.config...exiting";
                return LIFE_ERR_GEOMETRY;
            }
    int rc = remove_overlap(g, o, err, scan, scan_min);
    if (rc) return rc;
    o.hasIBM = !o.b.empty();
    for (auto& b : o.b)
        if (b.flex) o.hasFlex = true;
    if (o.hasIBM) {
        // ObjectsClass::initialiseObjects (src/Objects.cpp:941-961)
        if (p.has_initial_deflect && o.hasFlex) {
            // Bodies are independent (each writes its own FEM state and its own
            // markers), so host threads take whole bodies; the first failing
            // body in body order reports its error, as the sequential loop would.
            std::vector<int> flex;
            for (size_t k = 0; k < o.b.size(); k++)
                if (o.b[k].flex) flex.push_back((int)k);
            std::vector<int> rcs(flex.size(), LIFE_OK);
            std::vector<std::string> errs(flex.size());
            std::atomic<int> next{0};
            auto work = [&]() {
                for (int q; (q = next++) < (int)flex.size();)
                    rcs[q] = fem_initial_deflection(g, p, o, o.b[flex[q]], &errs[q]);
            };
            const unsigned ncpu = std::thread::hardware_concurrency();
            const int nt = (int)std::min<size_t>(flex.size(), ncpu ? ncpu : 1);
            if (nt <= 1) {
                work();
            } else {
                std::vector<std::thread> pool;
                for (int k = 0; k < nt; k++) pool.emplace_back(work);
                for (auto& th : pool) th.join();
            }
            for (size_t q = 0; q < flex.size(); q++)
                if (rcs[q]) {
                    if (err) *err = errs[q];
                    return rcs[q];
                }
        }
        for (size_t k = 0; k < o.m.size(); k++) {
            rc = host_find_support(g, o.m[k], err);
            if (rc) return rc;
            host_compute_ds(g, o, (int)k);
        }
        rc = host_compute_epsilon(g, o, p.uni_epsilon != 0, true, err);
        if (rc) return rc;
    }
    o.nFlex = o.simDOFs = 0;
    for (auto& b : o.b)
        if (b.flex) {
            o.nFlex++;
            o.simDOFs += b.fem->dofs;
        }
    return LIFE_OK;
}

}  // namespace life

// Drop-in driver for a LIFE case directory: the reference's main()
// (src/main.cpp:25-94) with the solver replaced by the GB300 library.
//
// Build it like the reference, once per case, with the case's params.h
// force-included:
//
//   g++ -O2 -std=c++17 -include path/to/params.h -I include -I include/life_ref_defs \
//       life_gb300/host/life_main.cpp -L life_gb300/_lib -llife_gb300 \
//       -Wl,-rpath,$PWD/life_gb300/_lib -o LIFE_gb300
//
// and run it in the case directory (input/geometry.config optional). It
// prints the reference's info lines (time step, MLUPS, max velocity) every
// tinfo steps, writes the restart set Results/Restart/{Fluid,IBM,FEM}.restart
// every tRestart steps in the reference's binary layouts
// (GridClass::writeRestart, src/Grid.cpp:1163-1229; ObjectsClass::writeRestart,
// src/Objects.cpp:1206-1371), resumes from that set when Fluid.restart exists
// at start-up (Utils::readRestart, src/Utils.cpp:82-101: steps tOffset+1 ..
// tOffset+nSteps), and exits with status 99 and the reference's message on a
// fatal error.
// Set LIFE_PRECISION=f32 or f16 to pick a reduced-precision storage form.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "life_params_pack.h"

static void fatal(const char* what) {
    std::printf("\n\n%s: %s\n\n", what, life_last_error());
    std::exit(99);
}

struct Bodies {
    std::vector<int32_t> ids, flexible, n_markers, n_fem_nodes;
};

static Bodies bodies_of(LifeCase* c, const LifeCaseInfo& info) {
    Bodies b;
    b.ids.resize(info.n_bodies);
    b.flexible.resize(info.n_bodies);
    b.n_markers.resize(info.n_bodies);
    b.n_fem_nodes.resize(info.n_bodies);
    if (info.n_bodies &&
        life_case_get_bodies(c, b.ids.data(), b.flexible.data(), b.n_markers.data(), b.n_fem_nodes.data()))
        fatal("bodies");
    return b;
}

template <class T>
static void put(std::ofstream& o, const T& v) {
    o.write((const char*)&v, sizeof(T));
}
template <class T>
static T get(std::ifstream& in) {
    T v{};
    in.read((char*)&v, sizeof(T));
    return v;
}

static void write_restart(LifeCase* c, const LifeCaseInfo& info) {
    const size_t n = (size_t)info.Nx * info.Ny;
    std::vector<double> rho(n), u(2 * n), f(9 * n), fi(2 * n);
    if (life_case_get_fields(c, rho.data(), u.data(), f.data(), fi.data())) fatal("get_fields");
    std::filesystem::create_directories("Results/Restart");
    {
        const char* tmp = "Results/Restart/Fluid.restart.temp";
        std::ofstream out(tmp, std::ios::binary);
        put(out, (int)info.t);
        put(out, (int)info.Nx);
        put(out, (int)info.Ny);
        put(out, (double)omega);
        put(out, info.Dx);
        put(out, info.Dt);
        put(out, info.Dm);
        for (int i = 0; i < info.Nx; i++)
            for (int j = 0; j < info.Ny; j++) {
                const size_t id = (size_t)i * info.Ny + j;
                put(out, i);
                put(out, j);
                out.write((const char*)&rho[id], 8);
                out.write((const char*)&u[id * 2], 16);
                out.write((const char*)&fi[id * 2], 16);
                out.write((const char*)&f[id * 9], 72);
            }
        out.close();
        std::filesystem::rename(tmp, "Results/Restart/Fluid.restart");
    }
    if (info.n_markers == 0) return;
    const Bodies b = bodies_of(c, info);
    const int nm = info.n_markers;
    std::vector<double> pos(2 * nm), vel(2 * nm), force(2 * nm);
    if (life_case_get_markers(c, pos.data(), vel.data(), force.data(), nullptr, nullptr, nullptr)) fatal("markers");
    {
        std::ofstream out("Results/Restart/IBM.restart", std::ios::binary);
        put(out, (size_t)info.n_bodies);
        size_t m0 = 0;
        for (int ib = 0; ib < info.n_bodies; ib++) {
            put(out, (int)b.ids[ib]);
            put(out, (size_t)b.n_markers[ib]);
            for (int q = 0; q < b.n_markers[ib]; q++) {
                const size_t k = m0 + q;
                out.write((const char*)&pos[2 * k], 16);
                out.write((const char*)&vel[2 * k], 16);
                out.write((const char*)&force[2 * k], 16);
            }
            m0 += b.n_markers[ib];
        }
    }
    if (info.n_flex == 0) return;
    double relax = 0.0;
    life_case_get_relax(c, &relax);
    std::ofstream out("Results/Restart/FEM.restart", std::ios::binary);
    put(out, (int)info.n_flex);
    put(out, relax);
    int k = 0;
    for (int ib = 0; ib < info.n_bodies; ib++) {
        if (!b.flexible[ib]) continue;
        const int nn = b.n_fem_nodes[ib], dofs = 3 * nn, ne = nn - 1;
        std::vector<double> v[6], elL(ne), elA(ne), pos0(2 * nn), posn(2 * nn), ang0(nn), ang(nn);
        for (auto& x : v) x.resize(dofs);
        if (life_case_get_fem(c, k, v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(), v[5].data(),
                              elL.data(), elA.data(), posn.data(), ang.data()) ||
            life_case_get_fem0(c, k, pos0.data(), ang0.data()))
            fatal("fem");
        put(out, (int)b.ids[ib]);
        put(out, (size_t)ne);
        put(out, (size_t)nn);
        for (auto& x : v) out.write((const char*)x.data(), 8 * dofs);
        for (int e = 0; e < ne; e++) {
            put(out, elL[e]);
            put(out, elA[e]);
        }
        for (int q = 0; q < nn; q++) {
            out.write((const char*)&pos0[2 * q], 16);
            out.write((const char*)&posn[2 * q], 16);
            put(out, ang0[q]);
            put(out, ang[q]);
        }
        k++;
    }
}

// Utils::readRestart: Fluid.restart, then the bodies (matched by ID; bodies
// not in this run are skipped, count mismatches are fatal). Returns tOffset.
static int read_restart(LifeCase* c, const LifeCaseInfo& info) {
    std::ifstream in("Results/Restart/Fluid.restart", std::ios::binary);
    if (!in) fatal("Error opening Fluid.restart file");
    const int t = get<int>(in), nx = get<int>(in), ny = get<int>(in);
    get<double>(in);
    get<double>(in);
    get<double>(in);
    get<double>(in);
    if (nx != info.Nx || ny != info.Ny) {
        std::printf("\n\nGrid size does not match Fluid.restart file...exiting\n\n");
        std::exit(99);
    }
    const size_t n = (size_t)nx * ny;
    std::vector<double> rho(n), u(2 * n), f(9 * n), fi(2 * n);
    for (size_t id = 0; id < n; id++) {
        get<int>(in);
        get<int>(in);
        in.read((char*)&rho[id], 8);
        in.read((char*)&u[id * 2], 16);
        in.read((char*)&fi[id * 2], 16);
        in.read((char*)&f[id * 9], 72);
    }
    if (!in) fatal("Fluid.restart is truncated");
    if (life_case_set_fields(c, t, rho.data(), u.data(), f.data(), fi.data())) fatal("set_fields");
    if (info.n_markers == 0) return t;
    const Bodies b = bodies_of(c, info);
    std::vector<size_t> start(info.n_bodies + 1, 0);
    for (int ib = 0; ib < info.n_bodies; ib++) start[ib + 1] = start[ib] + b.n_markers[ib];
    auto body_of = [&](int id) {
        for (int ib = 0; ib < info.n_bodies; ib++)
            if (b.ids[ib] == id) return ib;
        return -1;
    };
    std::ifstream im("Results/Restart/IBM.restart", std::ios::binary);
    if (im) {
        const int nm = info.n_markers;
        std::vector<double> pos(2 * nm), vel(2 * nm), force(2 * nm);
        if (life_case_get_markers(c, pos.data(), vel.data(), force.data(), nullptr, nullptr, nullptr))
            fatal("markers");
        const size_t nb = get<size_t>(im);
        for (size_t q = 0; q < nb; q++) {
            const int id = get<int>(im);
            const size_t nn = get<size_t>(im);
            const int ib = body_of(id);
            if (ib < 0) {
                im.seekg((std::streamoff)(48 * nn), std::ios::cur);
                continue;
            }
            if (nn != (size_t)b.n_markers[ib]) {
                std::printf("\n\nNumber of nodes in IBM.restart do not match existing number of nodes...exiting\n\n");
                std::exit(99);
            }
            for (size_t m = 0; m < nn; m++) {
                const size_t k = start[ib] + m;
                im.read((char*)&pos[2 * k], 16);
                im.read((char*)&vel[2 * k], 16);
                im.read((char*)&force[2 * k], 16);
            }
        }
        if (life_case_set_markers(c, pos.data(), vel.data(), force.data())) fatal("set_markers");
    }
    std::ifstream ifm("Results/Restart/FEM.restart", std::ios::binary);
    if (ifm && info.n_flex) {
        const int nflex = get<int>(ifm);
        if (life_case_set_relax(c, get<double>(ifm))) fatal("set_relax");
        for (int q = 0; q < nflex; q++) {
            const int id = get<int>(ifm);
            const size_t ne = get<size_t>(ifm), nn = get<size_t>(ifm);
            const int ib = body_of(id);
            if (ib < 0 || !b.flexible[ib]) {
                ifm.seekg((std::streamoff)(8 * (6 * 3 * nn + 2 * ne + 6 * nn)), std::ios::cur);
                continue;
            }
            if (nn != (size_t)b.n_fem_nodes[ib] || ne + 1 != nn) {
                std::printf("\n\nNumber of nodes/elements in FEM.restart do not match existing number of "
                            "nodes/elements...exiting\n\n");
                std::exit(99);
            }
            int k = 0;
            for (int j = 0; j < ib; j++) k += b.flexible[j] ? 1 : 0;
            const size_t dofs = 3 * nn;
            std::vector<double> v[6], elL(ne), elA(ne), pos0(2 * nn), posn(2 * nn), ang0(nn), ang(nn);
            for (auto& x : v) {
                x.resize(dofs);
                ifm.read((char*)x.data(), 8 * dofs);
            }
            for (size_t e = 0; e < ne; e++) {
                elL[e] = get<double>(ifm);
                elA[e] = get<double>(ifm);
            }
            for (size_t m = 0; m < nn; m++) {
                ifm.read((char*)&pos0[2 * m], 16);
                ifm.read((char*)&posn[2 * m], 16);
                ang0[m] = get<double>(ifm);
                ang[m] = get<double>(ifm);
            }
            if (life_case_set_fem(c, k, v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(),
                                  v[5].data(), elL.data(), elA.data(), pos0.data(), posn.data(), ang0.data(),
                                  ang.data()))
                fatal("set_fem");
        }
    }
    return t;
}

int main() {
    LifeCaseParams p;
    life_pack_params(&p);
    if (const char* prec = std::getenv("LIFE_PRECISION")) {
        if (!std::strcmp(prec, "f32")) p.precision = LIFE_PREC_F32;
        else if (!std::strcmp(prec, "f16")) p.precision = LIFE_PREC_F16;
    }
    // geometry.config (ObjectsClass::geometryReadIn, src/Objects.cpp:324-488)
    std::vector<LifeBodyDesc> bodies;
    std::ifstream g("input/geometry.config");
    if (g) {
        std::stringstream ss;
        ss << g.rdbuf();
        const std::string text = ss.str();
        int32_t nb = 0;
        if (life_parse_geometry(text.c_str(), nullptr, 0, &nb)) fatal("geometry.config");
        bodies.resize(nb);
        if (nb && life_parse_geometry(text.c_str(), bodies.data(), nb, &nb)) fatal("geometry.config");
    }
    LifeCase* c = nullptr;
    if (life_case_create(&p, bodies.data(), (int32_t)bodies.size(), &c)) fatal("initialisation");
    LifeCaseInfo info;
    life_case_info(c, &info);
    std::printf("*** LIFE on GB300 ***\nNx = %d, Ny = %d, bodies = %d, markers = %d\n", info.Nx, info.Ny,
                info.n_bodies, info.n_markers);
    int tOffset = 0;
    if (std::filesystem::exists("Results/Restart/Fluid.restart")) {
        tOffset = read_restart(c, info);
        std::printf("Restarting from time step %d\n", tOffset);
    }
    auto t0 = std::chrono::steady_clock::now();
    int done = 0;
    for (int t = tOffset + 1; t <= tOffset + nSteps; t++) {
        if (life_case_step(c, 1)) fatal("step");
        done++;
        const bool info_now = (t % tinfo == 0), restart_now = (tRestart > 0 && t % tRestart == 0);
        if (info_now || restart_now) {
            if (life_case_sync(c)) fatal("step");
            life_case_info(c, &info);
        }
        if (info_now) {
            double vmax = 0.0;
            int32_t nan = 0;
            if (life_case_max_velocity(c, &vmax, &nan)) fatal("info");
            if (nan) {
                std::printf("\n\nSimulation blew up (t = %d)...exiting\n\n", t);
                std::exit(99);
            }
            const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            std::printf("Time step %d of %d\nMLUPS = %.4g\nMax Velocity = %.5g\n", t, nSteps,
                        (double)info.Nx * info.Ny * done / (1e6 * secs), vmax);
        }
        if (restart_now) write_restart(c, info);
    }
    life_case_sync(c);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("\n*** FINISHED LIFE ***\nSimulation took %.2f seconds\n", secs);
    life_case_destroy(c);
    return 0;
}

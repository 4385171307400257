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
// tinfo steps, writes Results/Restart/Fluid.restart every tRestart steps in
// the reference's binary layout (GridClass::writeRestart, src/Grid.cpp:1163-1229)
// and exits with status 99 and the reference's message on a fatal error.
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

static void write_fluid_restart(LifeCase* c, const LifeCaseInfo& info) {
    const size_t n = (size_t)info.Nx * info.Ny;
    std::vector<double> rho(n), u(2 * n), f(9 * n), fi(2 * n);
    if (life_case_get_fields(c, rho.data(), u.data(), f.data(), fi.data())) fatal("get_fields");
    std::filesystem::create_directories("Results/Restart");
    const char* tmp = "Results/Restart/Fluid.restart.temp";
    std::ofstream out(tmp, std::ios::binary);
    const int t = info.t, nx = info.Nx, ny = info.Ny;
    const double om = omega, dx = info.Dx, dt = info.Dt, dm = info.Dm;
    out.write((const char*)&t, 4);
    out.write((const char*)&nx, 4);
    out.write((const char*)&ny, 4);
    out.write((const char*)&om, 8);
    out.write((const char*)&dx, 8);
    out.write((const char*)&dt, 8);
    out.write((const char*)&dm, 8);
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            const size_t id = (size_t)i * ny + j;
            out.write((const char*)&i, 4);
            out.write((const char*)&j, 4);
            out.write((const char*)&rho[id], 8);
            out.write((const char*)&u[id * 2], 16);
            out.write((const char*)&fi[id * 2], 16);
            out.write((const char*)&f[id * 9], 72);
        }
    out.close();
    std::filesystem::rename(tmp, "Results/Restart/Fluid.restart");
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
    auto t0 = std::chrono::steady_clock::now();
    int done = 0;
    for (int t = 1; t <= nSteps; t++) {
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
        if (restart_now) write_fluid_restart(c, info);
    }
    life_case_sync(c);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("\n*** FINISHED LIFE ***\nSimulation took %.2f seconds\n", secs);
    life_case_destroy(c);
    return 0;
}

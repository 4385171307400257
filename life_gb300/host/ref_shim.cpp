// GridClass, ObjectsClass and Utils with the reference's interface (reference
// inc/Grid.h, inc/Objects.h, inc/Utils.h), backed by the GB300 library, so a
// LIFE main() written against the reference's classes (src/main.cpp:25-94)
// runs its time loop on the GPU unchanged. Declarations:
// include/life_ref_shim/{Grid,Objects,Utils}.h.
//
// Compile once per case with the case's params.h, like the reference:
//
//   g++ -O2 -std=c++17 -I <dir with params.h> -I include/life_ref_shim -I include \
//       -I include/life_ref_defs main.cpp life_gb300/host/ref_shim.cpp \
//       -L life_gb300/_lib -llife_gb300 -Wl,-rpath,<abs>/life_gb300/_lib
//
// What runs where: the time loop (GridClass::solver) is one life_case_step
// per call; the writers read the device state through the C-ABI and write the
// reference's files byte for byte (TotalForces.out, TipPositions.out,
// TipVelocities.out, the VTK files and the restart set). Fatal errors print
// the reference's message and exit with status 99 (inc/Utils.h:72-77).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "Grid.h"
#include "Objects.h"
#include "Utils.h"
#include "life_params_pack.h"

namespace fs = std::filesystem;

namespace {

[[noreturn]] void fail(const std::string& msg) {
    std::cout << std::endl << std::endl << msg << std::endl << std::endl;
    std::exit(99);
}

void check(int rc, const char* what) {
    if (rc) fail(std::string(life_last_error()[0] ? life_last_error() : what));
}

template <class T>
void put(std::ofstream& o, const T& v) {
    o.write(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <class T>
T get(std::ifstream& in) {
    T v{};
    in.read(reinterpret_cast<char*>(&v), sizeof(T));
    return v;
}

struct BodyTable {
    std::vector<int32_t> ids, flexible, n_markers, n_fem_nodes, kind, index;
};

BodyTable body_table(LifeCase* c) {
    LifeCaseInfo info;
    check(life_case_info(c, &info), "info");
    BodyTable b;
    const size_t nb = info.n_bodies, nm = info.n_markers;
    b.ids.resize(nb);
    b.flexible.resize(nb);
    b.n_markers.resize(nb);
    b.n_fem_nodes.resize(nb);
    b.kind.resize(nb);
    b.index.resize(nm);
    if (nb) {
        check(life_case_get_bodies(c, b.ids.data(), b.flexible.data(), b.n_markers.data(), b.n_fem_nodes.data()),
              "bodies");
        check(life_case_get_body_nodes(c, b.kind.data(), b.index.data()), "bodies");
    }
    return b;
}

LifeCaseInfo info_of(LifeCase* c) {
    LifeCaseInfo info;
    check(life_case_info(c, &info), "info");
    return info;
}

const char* endian_name(bool big) { return big ? "BigEndian" : "LittleEndian"; }

// One VTK PolyData piece: points and whether the outline is closed.
struct Piece {
    std::vector<double> xy;  // [n][2]
    bool closed;
};

void write_polydata(const std::string& fname, bool big, const std::vector<Piece>& pieces) {
    std::ofstream output(fname, std::ios::binary);
    if (!output.is_open()) fail("Error opening body VTK file...exiting");
    output << "<?xml version=\"1.0\"?>\n";
    output << "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"" << endian_name(big)
           << "\" header_type=\"UInt64\">\n";
    output << "\t<PolyData>\n";
    unsigned long long offset = 0;
    for (const Piece& p : pieces) {
        const size_t nn = p.xy.size() / 2, nl = p.closed ? nn : nn - 1;
        output << "\t\t<Piece NumberOfPoints=\"" << nn << "\" NumberOfVerts=\"" << 0 << "\" NumberOfLines=\"" << nl
               << "\" NumberOfStrips=\"" << 0 << "\" NumberOfPolys=\"" << 0 << "\">\n";
        output << "\t\t\t<Points>\n";
        output << "\t\t\t\t<DataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\" format=\"appended\" "
                  "offset=\""
               << offset << "\"/>\n";
        offset += 3 * nn * sizeof(double) + sizeof(unsigned long long);
        output << "\t\t\t</Points>\n";
        output << "\t\t\t<Lines>\n";
        output << "\t\t\t\t<DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\"" << offset
               << "\"/>\n";
        offset += 2 * nl * sizeof(long long) + sizeof(unsigned long long);
        output << "\t\t\t\t<DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"" << offset
               << "\"/>\n";
        offset += nl * sizeof(long long) + sizeof(unsigned long long);
        output << "\t\t\t</Lines>\n";
        output << "\t\t</Piece>\n";
    }
    output << "\t</PolyData>\n";
    output << "\t<AppendedData encoding=\"raw\">\n";
    output << "\t\t_";
    for (const Piece& p : pieces) {
        const size_t nn = p.xy.size() / 2, nl = p.closed ? nn : nn - 1;
        put(output, (unsigned long long)(3 * nn * sizeof(double)));
        for (size_t n = 0; n < nn; n++) {
            put(output, p.xy[2 * n]);
            put(output, p.xy[2 * n + 1]);
            put(output, 0.0);
        }
        put(output, (unsigned long long)(2 * nl * sizeof(long long)));
        for (size_t n = 0; n < nl; n++) {
            put(output, (long long)n);
            put(output, (long long)((n + 1) % nn));
        }
        put(output, (unsigned long long)(nl * sizeof(long long)));
        for (size_t n = 0; n < nl; n++) put(output, (long long)(2 * (n + 1)));
    }
    output << "\n\t</AppendedData>\n";
    output << "</VTKFile>\n";
}

// Keeps the header and the lines of steps before t (the reference drops
// output written after the restart point, src/Objects.cpp:1525-1585).
void truncate_after(const std::string& fname, int t) {
    if (!fs::exists(fname)) return;
    std::ifstream in(fname);
    std::vector<std::string> keep;
    std::string line;
    if (std::getline(in, line)) keep.push_back(line);
    while (std::getline(in, line)) {
        if (std::stoi(line) >= t) break;
        keep.push_back(line);
    }
    in.close();
    std::ofstream out("Results/Output.temp");
    for (size_t k = 0; k < keep.size(); k++) out << (k ? "\n" : "") << keep[k];
    out.close();
    fs::rename("Results/Output.temp", fname);
}

}  // namespace

// --------------------------------------------------------------- Utils ----

void Utils::writeHeader() {
    std::cout << std::endl << "*** LIFE " << version << " ***" << std::endl << std::endl;
    std::cout << "Lattice Boltzmann - immersed boundary - finite element solver, GB300 path" << std::endl;
}

bool Utils::createDirectories() {
    if (fs::exists("Results/Restart/Fluid.restart")) return true;
    std::error_code ec;
    if (fs::exists("Results")) fs::remove_all("Results", ec);
    if (ec || !fs::create_directory("Results")) fail("Problem creating results directory...exiting");
#ifdef VTK
    if (!fs::create_directory("Results/VTK")) fail("Problem creating VTK directory...exiting");
#endif
    if (!fs::create_directory("Results/Restart")) fail("Problem creating restart directory...exiting");
    return false;
}

void Utils::readRestart(GridClass& grid) {
    std::cout << std::endl << std::endl << std::endl << "*** READ IN RESTART DATA ***";
    std::cout << std::endl << std::endl << "Reading in restart files...";
    grid.readRestart();
    grid.oPtr->readRestart();
    // drop VTK files written after the restart point (src/Utils.cpp:170-236)
    if (fs::exists("Results/VTK"))
        for (const auto& e : fs::directory_iterator("Results/VTK")) {
            const std::string stem = e.path().stem().string();
            const size_t dot = stem.rfind('.');
            if (dot == std::string::npos) continue;
            const std::string kind = stem.substr(0, dot);
            if (kind != "Fluid" && kind != "IBM" && kind != "FEM") continue;
            if (std::atoi(stem.c_str() + dot + 1) > grid.t) fs::remove(e.path());
        }
    std::cout << "finished";
}

void Utils::writeRestart(GridClass& grid) {
    std::cout << std::endl << "Writing restart data...";
    grid.writeRestart();
    grid.oPtr->writeRestart();
    std::cout << "finished";
}

void Utils::writeInfo(GridClass& grid) {
    grid.writeInfo();
    grid.oPtr->writeInfo();
#ifdef FORCES
    grid.oPtr->writeTotalForces();
#endif
#ifdef TIPS
    grid.oPtr->writeTips();
#endif
}

void Utils::writeLog(GridClass& grid) {
    grid.writeLog();
    grid.oPtr->writeLog();
}

void Utils::writeVTK(GridClass& grid) {
#ifdef VTK
    std::cout << std::endl << "Writing VTK data...";
    grid.writeVTK();
    grid.oPtr->writeVTK();
    std::cout << "finished";
#else
    (void)grid;
#endif
}

// ----------------------------------------------------------- GridClass ----

GridClass::GridClass() : t(0), tOffset(0), oPtr(nullptr), gpu(nullptr), stepsDone(0) {
    std::cout << std::endl << std::endl << "Initialising grid...";
    life_pack_params(&params);
    if (const char* prec = std::getenv("LIFE_PRECISION")) {
        if (!std::strcmp(prec, "f32")) params.precision = LIFE_PREC_F32;
        else if (!std::strcmp(prec, "f16")) params.precision = LIFE_PREC_F16;
    }
    restartFlag = Utils::createDirectories();
    // scalings (src/Grid.cpp:1247-1260)
    c_s = 1.0 / sqrt(3.0);
    tau = 1.0 / omega;
    nu = (tau - 0.5) * SQ(c_s);
    Dx = height_p / (Ny - 1);
    Dt = SQ(Dx) * nu / nu_p;
    Dm = (rho_p / 1.0) * TH(Dx);
    Drho = (rho_p / 1.0);
    const unsigned one = 1;
    bigEndian = *reinterpret_cast<const unsigned char*>(&one) == 0;
    startTime = omp_get_wtime();
    loopTime = 0.0;
    std::cout << "finished";
}

GridClass::~GridClass() {
    if (gpu) life_case_destroy(gpu);
}

void GridClass::startClock() {
    life_case_sync(gpu);
    startTime = omp_get_wtime();
    stepsDone = 0;
}

void GridClass::solver() {
    // the caller's loop sets t to the step being solved; the device case
    // holds the state of step t - 1
    const LifeCaseInfo info = info_of(gpu);
    if (info.t != t - 1) fail("Time step " + std::to_string(t) + " does not follow the case's state");
    check(life_case_step(gpu, 1), "solver");
    stepsDone++;
}

void GridClass::writeInfo() {
    check(life_case_sync(gpu), "step");
    double maxVel = 0.0;
    int32_t nan = 0;
    check(life_case_max_velocity(gpu, &maxVel, &nan), "info");
    if (nan) {
#ifdef VTK
        Utils::writeVTK(*this);
#endif
        fail("Simulation blew up (t = " + std::to_string(t) + ")...exiting");
    }
    const double maxRe = (maxVel * Dx / Dt) * ref_L / ref_nu;
    loopTime = (t == tOffset || stepsDone == 0) ? 0.0 : (omp_get_wtime() - startTime) / stepsDone;
    std::cout << std::endl << std::endl;
    std::cout << "Time step " << t << " of " << tOffset + nSteps << std::endl;
    std::cout << std::setprecision(4) << "MLUPS = " << (loopTime > 0 ? Nx * Ny / (1000000.0 * loopTime) : 0.0)
              << std::endl;
    std::cout << std::setprecision(5) << "Max Velocity = " << maxVel << std::endl;
    std::cout << std::setprecision(5) << "Max Reynolds number = " << maxRe;
}

void GridClass::writeLog() {
    std::ofstream log("Results/Log.out", std::ios::app);
    log << "LIFE " << version << " on GB300\n\nGRID:\nNx = " << Nx << "\nNy = " << Ny << "\nDx = " << Dx
        << "\nDt = " << Dt << "\ntau = " << tau << "\nnu = " << nu << "\nStorage form = "
        << (params.precision == LIFE_PREC_F64 ? "FP64" : params.precision == LIFE_PREC_F32 ? "FP32" : "FP16")
        << "\n";
}

void GridClass::writeVTK() {
    const size_t n = (size_t)Nx * Ny;
    std::vector<double> dens(n), pres(n), vel(3 * n);
    check(life_case_get_vtk_fields(gpu, dens.data(), pres.data(), vel.data()), "vtk");
    std::ofstream output("Results/VTK/Fluid." + std::to_string(t) + ".vti", std::ios::binary);
    if (!output.is_open()) fail("Error opening fluid VTK file...exiting");
    output << "<?xml version=\"1.0\"?>\n";
    output << "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"" << endian_name(bigEndian)
           << "\" header_type=\"UInt64\">\n";
    output << "\t<ImageData WholeExtent=\"" << 0.0 << " " << Nx - 1 << " " << 0.0 << " " << Ny - 1 << " " << 0.0
           << " " << 0.0 << "\" Origin=\"" << 0.0 << " " << 0.0 << " " << 0.0 << "\" Spacing=\"" << Dx << " " << Dx
           << " " << Dx << "\">\n";
    output << "\t\t<Piece Extent=\"" << 0.0 << " " << Nx - 1 << " " << 0.0 << " " << Ny - 1 << " " << 0.0 << " "
           << 0.0 << "\">\n";
    output << "\t\t\t<PointData>\n";
    const unsigned long long block = n * sizeof(double) + sizeof(unsigned long long);
    output << "\t\t\t\t<DataArray type=\"Float64\" Name=\"Density\" format=\"appended\" offset=\"" << 0 << "\"/>\n";
    output << "\t\t\t\t<DataArray type=\"Float64\" Name=\"Pressure\" format=\"appended\" offset=\"" << block
           << "\"/>\n";
    output << "\t\t\t\t<DataArray type=\"Float64\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"appended\" "
              "offset=\""
           << 2 * block << "\"/>\n";
    output << "\t\t\t</PointData>\n\t\t</Piece>\n\t</ImageData>\n";
    output << "\t<AppendedData encoding=\"raw\">\n\t\t_";
    put(output, (unsigned long long)(n * sizeof(double)));
    output.write(reinterpret_cast<const char*>(dens.data()), n * sizeof(double));
    put(output, (unsigned long long)(n * sizeof(double)));
    output.write(reinterpret_cast<const char*>(pres.data()), n * sizeof(double));
    put(output, (unsigned long long)(3 * n * sizeof(double)));
    output.write(reinterpret_cast<const char*>(vel.data()), 3 * n * sizeof(double));
    output << "\n\t</AppendedData>\n</VTKFile>\n";
}

void GridClass::writeRestart() {
    const LifeCaseInfo info = info_of(gpu);
    const size_t n = (size_t)info.Nx * info.Ny;
    std::vector<double> rho(n), u(2 * n), f(9 * n), fi(2 * n);
    check(life_case_get_fields(gpu, rho.data(), u.data(), f.data(), fi.data()), "get_fields");
    const char* tmp = "Results/Restart/Fluid.restart.temp";
    std::ofstream out(tmp, std::ios::binary);
    if (!out) fail("Error opening Fluid.restart file...exiting");
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
            out.write(reinterpret_cast<const char*>(&rho[id]), 8);
            out.write(reinterpret_cast<const char*>(&u[id * 2]), 16);
            out.write(reinterpret_cast<const char*>(&fi[id * 2]), 16);
            out.write(reinterpret_cast<const char*>(&f[id * 9]), 72);
        }
    out.close();
    fs::rename(tmp, "Results/Restart/Fluid.restart");
}

void GridClass::readRestart() {
    std::ifstream in("Results/Restart/Fluid.restart", std::ios::binary);
    if (!in) fail("Error opening Fluid.restart file...exiting");
    const int tr = get<int>(in), nx = get<int>(in), ny = get<int>(in);
    for (int k = 0; k < 4; k++) get<double>(in);
    if (nx != Nx || ny != Ny) fail("Grid size does not match Fluid.restart file...exiting");
    const size_t n = (size_t)nx * ny;
    std::vector<double> rho(n), u(2 * n), f(9 * n), fi(2 * n);
    for (size_t id = 0; id < n; id++) {
        get<int>(in);
        get<int>(in);
        in.read(reinterpret_cast<char*>(&rho[id]), 8);
        in.read(reinterpret_cast<char*>(&u[id * 2]), 16);
        in.read(reinterpret_cast<char*>(&fi[id * 2]), 16);
        in.read(reinterpret_cast<char*>(&f[id * 9]), 72);
    }
    if (!in) fail("Fluid.restart is truncated...exiting");
    check(life_case_set_fields(gpu, tr, rho.data(), u.data(), f.data(), fi.data()), "set_fields");
    t = tOffset = tr;
}

// -------------------------------------------------------- ObjectsClass ----

ObjectsClass::ObjectsClass(GridClass& g) : hasIBM(false), hasFlex(false), nFlex(0), simDOFs(0), gPtr(&g) {
    std::cout << std::endl << std::endl << "Initialising objects...";
    g.oPtr = this;
    std::vector<LifeBodyDesc> bodies;
    std::ifstream gin("input/geometry.config");
    if (gin) {
        std::stringstream ss;
        ss << gin.rdbuf();
        const std::string text = ss.str();
        int32_t nb = 0;
        check(life_parse_geometry(text.c_str(), nullptr, 0, &nb), "geometry.config");
        bodies.resize(nb);
        if (nb) check(life_parse_geometry(text.c_str(), bodies.data(), nb, &nb), "geometry.config");
    }
    check(life_case_create(&g.params, bodies.data(), (int32_t)bodies.size(), &g.gpu), "initialisation");
    const LifeCaseInfo info = info_of(g.gpu);
    hasIBM = info.n_markers > 0;
    hasFlex = info.n_flex > 0;
    nFlex = info.n_flex;
    simDOFs = info.sim_dofs;
    std::cout << (hasIBM ? "found " + std::to_string(info.n_bodies) + " object(s)" : std::string("no bodies found"));
}

void ObjectsClass::writeInfo() {
    if (!hasFlex) return;
    LifeStatus st;
    check(life_case_status(gPtr->gpu, &st), "status");
    std::cout << std::endl;
    std::cout << "Current relaxation factor = " << st.relax << std::endl;
    std::cout << "Subiterations taking " << st.last_subits << " iterations to reach a residual of "
              << st.last_subres << std::endl;
}

void ObjectsClass::writeLog() {
    if (!hasIBM) return;
    const LifeCaseInfo info = info_of(gPtr->gpu);
    std::ofstream log("Results/Log.out", std::ios::app);
    log << "\nBODIES:\nbodies = " << info.n_bodies << "\nmarkers = " << info.n_markers
        << "\nflexible bodies = " << info.n_flex << "\nFEM DOFs = " << info.sim_dofs << "\n";
}

void ObjectsClass::writeTotalForces() {
    if (!hasIBM) return;
    const std::string fname = "Results/TotalForces.out";
    const bool existing = fs::exists(fname);
    std::ofstream output(fname, std::ios::app);
    output.precision(PRECISION);
    if (!output.is_open()) fail("Error opening forces file...exiting");
    if (!existing) output << "Timestep\tTime (s)\tFx (N)\tFy (N)\tCx\tCy";
    double F[2] = {0.0, 0.0};
    check(life_case_total_force(gPtr->gpu, &F[0], &F[1]), "forces");
    const double ND = 0.5 * ref_rho * SQ(ref_U) * ref_L;
    output << std::endl
           << gPtr->t << "\t" << gPtr->Dt * gPtr->t << "\t" << F[0] << "\t" << F[1] << "\t" << F[0] / ND << "\t"
           << F[1] / ND;
}

void ObjectsClass::writeTips() {
    if (!hasFlex) return;
    const std::string fp = "Results/TipPositions.out", fv = "Results/TipVelocities.out";
    const bool ep = fs::exists(fp), ev = fs::exists(fv);
    std::ofstream op(fp, std::ios::app), ov(fv, std::ios::app);
    op.precision(PRECISION);
    ov.precision(PRECISION);
    if (!op.is_open() || !ov.is_open()) fail("Error opening tip positions/velocities files...exiting");
    if (!ep) op << "Timestep\tTime (s)\tTipX\tTipY";
    if (!ev) ov << "Timestep\tTime (s)\tTipX\tTipY";
    op << std::endl << gPtr->t << "\t" << gPtr->Dt * gPtr->t;
    ov << std::endl << gPtr->t << "\t" << gPtr->Dt * gPtr->t;
    const BodyTable b = body_table(gPtr->gpu);
    const size_t nm = b.index.size();
    std::vector<double> pos(2 * nm), vel(2 * nm);
    check(life_case_get_markers(gPtr->gpu, pos.data(), vel.data(), nullptr, nullptr, nullptr, nullptr), "markers");
    size_t q = 0;
    for (size_t ib = 0; ib < b.ids.size(); ib++) {
        const size_t m = b.n_markers[ib];
        if (b.flexible[ib] && m) {
            const int last = b.index[q + m - 1];
            op << "\t" << pos[2 * last] << "\t" << pos[2 * last + 1];
            ov << "\t" << vel[2 * last] << "\t" << vel[2 * last + 1];
        }
        q += m;
    }
}

void ObjectsClass::writeVTK(bool writeIBM) {
    if (!((writeIBM && hasIBM) || (!writeIBM && hasFlex))) return;
    const BodyTable b = body_table(gPtr->gpu);
    std::vector<Piece> pieces;
    if (writeIBM) {
        const size_t nm = b.index.size();
        std::vector<double> pos(2 * nm);
        check(life_case_get_markers(gPtr->gpu, pos.data(), nullptr, nullptr, nullptr, nullptr, nullptr), "markers");
        size_t q = 0;
        for (size_t ib = 0; ib < b.ids.size(); ib++) {
            Piece p{{}, b.kind[ib] == LIFE_BODY_CIRCLE};
            for (int k = 0; k < b.n_markers[ib]; k++) {
                const int m = b.index[q + k];
                p.xy.push_back(pos[2 * m]);
                p.xy.push_back(pos[2 * m + 1]);
            }
            q += b.n_markers[ib];
            pieces.push_back(p);
        }
    } else {
        int k = 0;
        for (size_t ib = 0; ib < b.ids.size(); ib++) {
            if (!b.flexible[ib]) continue;
            Piece p{std::vector<double>(2 * (size_t)b.n_fem_nodes[ib]), false};
            check(life_case_get_fem(gPtr->gpu, k++, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                    nullptr, p.xy.data(), nullptr),
                  "fem");
            pieces.push_back(p);
        }
    }
    write_polydata(std::string("Results/VTK/") + (writeIBM ? "IBM" : "FEM") + "." + std::to_string(gPtr->t) + ".vtp",
                   gPtr->bigEndian, pieces);
#ifdef VTK_FEM
    if (writeIBM) writeVTK(false);
#endif
}

void ObjectsClass::writeRestart() {
    if (!hasIBM) return;
    LifeCase* c = gPtr->gpu;
    const LifeCaseInfo info = info_of(c);
    const BodyTable b = body_table(c);
    const int nm = info.n_markers;
    std::vector<double> pos(2 * nm), vel(2 * nm), force(2 * nm);
    check(life_case_get_markers(c, pos.data(), vel.data(), force.data(), nullptr, nullptr, nullptr), "markers");
    {
        std::ofstream out("Results/Restart/IBM.restart", std::ios::binary);
        put(out, (size_t)info.n_bodies);
        size_t q = 0;
        for (int ib = 0; ib < info.n_bodies; ib++) {
            put(out, (int)b.ids[ib]);
            put(out, (size_t)b.n_markers[ib]);
            for (int k = 0; k < b.n_markers[ib]; k++) {
                const int m = b.index[q + k];
                out.write(reinterpret_cast<const char*>(&pos[2 * m]), 16);
                out.write(reinterpret_cast<const char*>(&vel[2 * m]), 16);
                out.write(reinterpret_cast<const char*>(&force[2 * m]), 16);
            }
            q += b.n_markers[ib];
        }
    }
    if (!hasFlex) return;
    double relax = 0.0;
    check(life_case_get_relax(c, &relax), "relax");
    std::ofstream out("Results/Restart/FEM.restart", std::ios::binary);
    put(out, (int)info.n_flex);
    put(out, relax);
    int k = 0;
    for (int ib = 0; ib < info.n_bodies; ib++) {
        if (!b.flexible[ib]) continue;
        const int nn = b.n_fem_nodes[ib], dofs = 3 * nn, ne = nn - 1;
        std::vector<double> v[6], elL(ne), elA(ne), pos0(2 * nn), posn(2 * nn), ang0(nn), ang(nn);
        for (auto& x : v) x.resize(dofs);
        check(life_case_get_fem(c, k, v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(), v[5].data(),
                                elL.data(), elA.data(), posn.data(), ang.data()),
              "fem");
        check(life_case_get_fem0(c, k, pos0.data(), ang0.data()), "fem");
        put(out, (int)b.ids[ib]);
        put(out, (size_t)ne);
        put(out, (size_t)nn);
        for (auto& x : v) out.write(reinterpret_cast<const char*>(x.data()), 8 * dofs);
        for (int e = 0; e < ne; e++) {
            put(out, elL[e]);
            put(out, elA[e]);
        }
        for (int q = 0; q < nn; q++) {
            out.write(reinterpret_cast<const char*>(&pos0[2 * q]), 16);
            out.write(reinterpret_cast<const char*>(&posn[2 * q]), 16);
            put(out, ang0[q]);
            put(out, ang[q]);
        }
        k++;
    }
}

void ObjectsClass::readRestart() {
    LifeCase* c = gPtr->gpu;
    const LifeCaseInfo info = info_of(c);
    // drop force and tip lines written after the restart point
    truncate_after("Results/TotalForces.out", gPtr->t);
    truncate_after("Results/TipPositions.out", gPtr->t);
    truncate_after("Results/TipVelocities.out", gPtr->t);
    if (info.n_markers == 0) return;
    const BodyTable b = body_table(c);
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
        check(life_case_get_markers(c, pos.data(), vel.data(), force.data(), nullptr, nullptr, nullptr), "markers");
        const size_t nb = get<size_t>(im);
        for (size_t q = 0; q < nb; q++) {
            const int id = get<int>(im);
            const size_t nn = get<size_t>(im);
            const int ib = body_of(id);
            if (ib < 0) {
                im.seekg((std::streamoff)(48 * nn), std::ios::cur);
                continue;
            }
            if (nn != (size_t)b.n_markers[ib])
                fail("Number of nodes in IBM.restart do not match existing number of nodes...exiting");
            for (size_t m = 0; m < nn; m++) {
                const size_t k = b.index[start[ib] + m];
                im.read(reinterpret_cast<char*>(&pos[2 * k]), 16);
                im.read(reinterpret_cast<char*>(&vel[2 * k]), 16);
                im.read(reinterpret_cast<char*>(&force[2 * k]), 16);
            }
        }
        check(life_case_set_markers(c, pos.data(), vel.data(), force.data()), "set_markers");
    }
    std::ifstream ifm("Results/Restart/FEM.restart", std::ios::binary);
    if (!ifm || !info.n_flex) return;
    const int nflex = get<int>(ifm);
    check(life_case_set_relax(c, get<double>(ifm)), "set_relax");
    for (int q = 0; q < nflex; q++) {
        const int id = get<int>(ifm);
        const size_t ne = get<size_t>(ifm), nn = get<size_t>(ifm);
        const int ib = body_of(id);
        if (ib < 0 || !b.flexible[ib]) {
            ifm.seekg((std::streamoff)(8 * (6 * 3 * nn + 2 * ne + 6 * nn)), std::ios::cur);
            continue;
        }
        if (nn != (size_t)b.n_fem_nodes[ib] || ne + 1 != nn)
            fail("Number of nodes/elements in FEM.restart do not match existing number of nodes/elements...exiting");
        int k = 0;
        for (int j = 0; j < ib; j++) k += b.flexible[j] ? 1 : 0;
        const size_t dofs = 3 * nn;
        std::vector<double> v[6], elL(ne), elA(ne), pos0(2 * nn), posn(2 * nn), ang0(nn), ang(nn);
        for (auto& x : v) {
            x.resize(dofs);
            ifm.read(reinterpret_cast<char*>(x.data()), 8 * dofs);
        }
        for (size_t e = 0; e < ne; e++) {
            elL[e] = get<double>(ifm);
            elA[e] = get<double>(ifm);
        }
        for (size_t m = 0; m < nn; m++) {
            ifm.read(reinterpret_cast<char*>(&pos0[2 * m]), 16);
            ifm.read(reinterpret_cast<char*>(&posn[2 * m]), 16);
            ang0[m] = get<double>(ifm);
            ang[m] = get<double>(ifm);
        }
        check(life_case_set_fem(c, k, v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(), v[5].data(),
                                elL.data(), elA.data(), pos0.data(), posn.data(), ang0.data(), ang.data()),
              "set_fem");
    }
}

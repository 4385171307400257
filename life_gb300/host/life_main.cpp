// Drop-in driver for a LIFE case directory: a main() over the reference's
// class interface (GridClass, ObjectsClass, Utils; include/life_ref_shim),
// whose implementation (life_gb300/host/ref_shim.cpp) runs the time loop on
// the GPU. It makes the calls the reference's main() makes, in the same order
// (src/main.cpp:25-94), so the reference's own main.cpp can replace this file
// unchanged.
//
// Build once per case, like the reference, with the case directory (its
// params.h) first on the include path:
//
//   g++ -O2 -std=c++17 -I <case> -I include/life_ref_shim -I include -I include/life_ref_defs \
//       life_gb300/host/life_main.cpp life_gb300/host/ref_shim.cpp \
//       -L life_gb300/_lib -llife_gb300 -Wl,-rpath,$PWD/life_gb300/_lib -o LIFE_gb300
//
// and run it in the case directory (input/geometry.config optional). Output:
// the info lines every tinfo steps, Results/TotalForces.out and the tip files
// (FORCES / TIPS), Results/VTK every tVTK steps (VTK, VTK_FEM), the restart
// set every tRestart steps; it resumes from Results/Restart when Fluid.restart
// exists, and exits with status 99 and the reference's message on a fatal
// error. LIFE_PRECISION=f32 or f16 selects a reduced-precision storage form.
#include "Grid.h"
#include "Objects.h"
#include "Utils.h"

int main() {
    Utils::writeHeader();
    cout << endl << endl << "*** INITIALISING LIFE ***";
    const double wall0 = omp_get_wtime();

    GridClass grid;
    ObjectsClass objects(grid);
    if (grid.restartFlag) {
        Utils::readRestart(grid);
        cout << endl << "Restarting from time step " << grid.tOffset;
    }
    Utils::writeLog(grid);

    cout << endl << endl << endl << "*** STARTING LIFE ***";
    Utils::writeInfo(grid);
    Utils::writeVTK(grid);
    grid.startClock();

    const int last = grid.tOffset + nSteps;
    for (grid.t = grid.tOffset + 1; grid.t <= last; grid.t++) {
        grid.solver();
        if (grid.t % tinfo == 0) Utils::writeInfo(grid);
        if (grid.t % tVTK == 0) Utils::writeVTK(grid);
        if (tRestart > 0 && grid.t % tRestart == 0) Utils::writeRestart(grid);
    }

    cout << endl << endl << endl << "*** FINISHED LIFE ***";
    cout << fixed << setprecision(2) << endl << endl << "Simulation took " << omp_get_wtime() - wall0 << " seconds"
         << endl << endl << endl;
    return 0;
}

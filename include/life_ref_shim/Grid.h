/*
 * GridClass with the reference's public interface (reference inc/Grid.h:29-131),
 * backed by the GB300 library: a LIFE main() written against the reference's
 * classes (reference src/main.cpp:25-94) compiles unchanged against this
 * header, Objects.h and Utils.h and runs its time loop on the GPU.
 *
 * The lattice lives on the device (LifeCase, include/life_gb300.h). The public
 * members main() touches keep their meaning: t is the step solver() computes
 * next, tOffset the step a restart resumed from, Dx/Dt/Dm/Drho the
 * reference's scalings (src/Grid.cpp:1254-1260), restartFlag whether
 * Results/Restart/Fluid.restart existed at start-up (Utils::createDirectories,
 * src/Utils.cpp:47-79), oPtr the ObjectsClass built on this grid.
 *
 * Build like the reference, with the case's params.h first on the include
 * path (or force-included), the directory of this header, include/ and
 * include/life_ref_defs, and link life_gb300/host/ref_shim.cpp and
 * liblife_gb300.so. Set LIFE_PRECISION=f32 or f16 in the environment to run
 * a reduced-precision storage form.
 */
#ifndef GRID_H
#define GRID_H

#include "defs.h"
#include "life_gb300.h"

class ObjectsClass;

class GridClass {
    friend class ObjectsClass;

public:
    GridClass();
    ~GridClass();

    int t;             // time step
    int tOffset;       // time step a restart resumed from
    ObjectsClass* oPtr;
    double Dx, Dt, Dm, Drho;
    bool restartFlag;
    bool bigEndian;

    void solver();        // one time step on the GPU (GridClass::solver, src/Grid.cpp:25-33)
    void writeInfo();     // max velocity, NaN check, MLUPS (src/Grid.cpp:559-620)
    void writeLog();      // Results/Log.out grid section (src/Grid.cpp:623-786)
    void writeVTK();      // Results/VTK/Fluid.<t>.vti (src/Grid.cpp:790-913)
    void writeRestart();  // Results/Restart/Fluid.restart (src/Grid.cpp:1163-1229)
    void readRestart();   // (src/Grid.cpp:1072-1160)
    void startClock();

    // The GPU case (created by ObjectsClass, which reads the bodies).
    LifeCase* gb300() const { return gpu; }

private:
    LifeCase* gpu;
    LifeCaseParams params;
    double c_s, tau, nu;
    double startTime, loopTime;
    int stepsDone;
};

#endif  // GRID_H

/*
 * ObjectsClass with the reference's public interface (reference
 * inc/Objects.h:32-113), backed by the GB300 library (see Grid.h). The
 * constructor reads input/geometry.config with the reference's rules
 * (ObjectsClass::geometryReadIn, src/Objects.cpp:324-488) and creates the
 * device case; the per-step object kernels run inside GridClass::solver on
 * the GPU. The writers produce the reference's files from the device state.
 */
#ifndef OBJECTS_H
#define OBJECTS_H

#include "params.h"
#include "defs.h"

class GridClass;

class ObjectsClass {
    friend class GridClass;

public:
    explicit ObjectsClass(GridClass& g);
    ~ObjectsClass() {}

    bool hasIBM;      // any immersed bodies
    bool hasFlex;     // any flexible bodies
    int nFlex;        // flexible bodies
    int simDOFs;      // FEM degrees of freedom of the whole case

    void writeInfo();                     // FEM info (src/Objects.cpp:597-707)
    void writeLog();                      // Results/Log.out bodies section
    void writeVTK(bool writeIBM = true);  // IBM / FEM .vtp (src/Objects.cpp:710-865)
    void writeTotalForces();              // Results/TotalForces.out (src/Objects.cpp:491-539)
    void writeTips();                     // Results/Tip{Positions,Velocities}.out (src/Objects.cpp:542-594)
    void writeRestart();                  // IBM.restart / FEM.restart (src/Objects.cpp:1206-1371)
    void readRestart();                   // (src/Objects.cpp:979-1203)

private:
    GridClass* gPtr;
};

#endif  // OBJECTS_H

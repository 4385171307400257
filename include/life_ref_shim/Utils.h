/*
 * The Utils functions the reference's main() calls (reference
 * inc/Utils.h:26-60, src/Utils.cpp:20-167), backed by the GB300 library (see
 * Grid.h). They dispatch to GridClass and ObjectsClass as the reference's do.
 */
#ifndef UTILS_H
#define UTILS_H

#include "params.h"

class GridClass;

namespace Utils {
void writeHeader();
bool createDirectories();
void readRestart(GridClass& grid);
void writeRestart(GridClass& grid);
void writeInfo(GridClass& grid);
void writeLog(GridClass& grid);
void writeVTK(GridClass& grid);
}  // namespace Utils

#endif  // UTILS_H

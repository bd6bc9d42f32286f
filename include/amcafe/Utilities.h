// Drop-in Utilities (reference: src/src-mpi/Utilities.h). The reference uses
// this class for the EASM temperature's material properties and quadrature
// (Utilities.C:89-140, 142-168, 228-249); the engine sets those up when the
// Grid is created and evaluates them on the device inside
// TempField::EASM, so InitializeUT has nothing left to do. See Grid.h.
#ifndef UTILITIES_H
#define UTILITIES_H

#include <vector>

#include "BasePlate.h"
#include "Grid.h"
#include "Partition.h"

class Utilities {
 public:
  Utilities(Grid &g, Partition &part, BasePlate &bp) : _xyz(&g), _part(&part), _bp(&bp) {}
  void InitializeUT() {}

 private:
  Grid *_xyz;
  Partition *_part;
  BasePlate *_bp;
};

#endif

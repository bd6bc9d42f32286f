// Drop-in BasePlate (reference: src/src-mpi/BasePlate.h:12-31). The engine
// draws the baseplate's Voronoi sites and orientations inside
// VoxelsCA::InitializeVoxels, as the reference's InitializeVoxels does through
// BasePlate::GenerateVoxel (VoxelsCA.C:125-161, BasePlate.C:41-97); this class
// carries the public fields main1.C reads (Nzh). See Grid.h.
#ifndef BASEPLATE_H
#define BASEPLATE_H

#include <random>
#include <vector>

#include "Grid.h"
#include "Partition.h"

class BasePlate {
 public:
  // BasePlate::BasePlate (BasePlate.C:18-30)
  BasePlate(const Grid &g, Partition &part) : _xyz(&g), _part(&part) {
    cafe_grid c;
    amcafe_dropin::check(cafe_sim_grid(g.Engine(), &c), "BasePlate::BasePlate");
    height = c.bpH;
    mu = c.mu;
    Nzh = c.Nzh;
  }

  double height = 0;
  double mu = 0;
  int Ngrain = 0, Nzh = 0;
  std::vector<double> cTheta, jVals;
  std::vector<int> X, gNucleus;

 private:
  const Grid *_xyz;
  Partition *_part;
};

#endif

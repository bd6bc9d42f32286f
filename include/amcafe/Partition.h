// Drop-in Partition (reference: src/src-mpi/Partition.h:7-22) for a world of
// one rank: PartitionGraph2 (Partition.C:260-412) at world size 1 gives every
// cell to the rank in index order, with no ghost cells, and PassInformation
// (Partition.C:413-449) has nothing to exchange. The engine holds the whole
// box on one GPU. See Grid.h for how the drop-in classes work.
#ifndef PARTITION_H
#define PARTITION_H

#include <numeric>
#include <vector>

#include "Grid.h"

class Partition {
 public:
  Partition(Grid &g, int &myidIn, int &nprocsIn) : myid(myidIn), nprocs(nprocsIn), _xyz(&g) {}

  void PartitionGraph2() {
    const long long n = (long long)_xyz->nX[0] * _xyz->nX[1] * _xyz->nX[2];
    icellidLoc.resize((size_t)n);
    std::iota(icellidLoc.begin(), icellidLoc.end(), 0);
    ncellLoc = (int)n;
    nGhost = 0;
    nneighProc = 0;
  }
  void PartitionGraph() { PartitionGraph2(); }
  void PassInformation(std::vector<int> &) {}
  void PassInformation(std::vector<double> &) {}

  std::vector<int> icellidLoc, ineighProcId, ineigh2LocVals, ineigh2Locptr, iloc2NeighVals, iloc2Neighptr,
      ipointidLoc, iconnectivityLoc;
  std::vector<std::vector<int>> icellidLocAll;
  int ncellLoc = 0, nGhost = 0, nneighProc = 0, myid = 0, nprocs = 1, npointLoc = 0;

 private:
  Grid *_xyz;
};

#endif

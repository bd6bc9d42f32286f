// Drop-in Grid for AMCAFE's time loop (reference: src/src-mpi/Grid.h:8-93).
//
// The classes in this folder (Grid, Partition, BasePlate, Utilities,
// TempField, VoxelsCA, SampleOrientation) have the constructors, the methods
// that src/src-mpi/main1.C calls and the public fields of the reference's
// classes of the same names, so that main1.C compiles unchanged against them
// (-I include/amcafe -I include, link -lcafe_gpu) and runs its loop on the
// GPU engine behind include/cafe_gpu.h. They are header-only forwarders:
//
// * Grid owns the engine handle (cafe_sim_create on the deck in its
//   constructor, cafe_sim_destroy in its destructor); the other classes use
//   it through the Grid they are given. A handle belongs to one host thread,
//   like the reference's single-threaded rank.
// * The scalar public fields (Grid's deck values, laser state and clock,
//   TempField::tInd and DelT, VoxelsCA::nGrain, BasePlate::Nzh) are refreshed
//   from the engine after every forwarded call.
// * The per-cell public vectors stay on the device during the loop and are
//   copied into the std::vector members where the reference's loop observes
//   them: VoxelsCA::SetBuild (Build), VoxelsCA::WriteToHDF1 (gID, vState,
//   extents, centroidOct, cTheta, Build, TempField::TempCurr and BuildjID),
//   VoxelsCA::CleanLayer (cTheta), and on request by the Sync() methods
//   (an extension). Writing to these vectors does not change the engine's
//   state.
// * Errors: the engine's return codes become std::runtime_error (the
//   reference has no error codes; its own parse errors are exceptions).
//
// The device is CUDA device 0, or the one named by the environment variable
// CAFE_DEVICE. The world is one rank: Partition is the identity map with no
// ghost cells, whatever MPI reports.
#ifndef GRID_H
#define GRID_H

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "../cafe_gpu.h"

namespace amcafe_dropin {

inline void check(int rc, const char *where) {
  if (rc != CAFE_OK) throw std::runtime_error(std::string(where) + ": " + cafe_last_error());
}

inline int device_from_env() {
  const char *d = std::getenv("CAFE_DEVICE");
  return d ? std::atoi(d) : 0;
}

}  // namespace amcafe_dropin

class Grid {
 public:
  // Grid::Grid (Grid.C:15-109): reads the deck and derives the laser grid;
  // here cafe_sim_create, which also allocates the device state.
  Grid(std::string &filIn, int &myidIn, int &nprocsIn) : filInput(filIn), myid(myidIn), nprocs(nprocsIn) {
    cafe_options o = cafe_options();
    o.device = amcafe_dropin::device_from_env();
    amcafe_dropin::check(cafe_sim_create(filIn.c_str(), &o, &sim_), "Grid::Grid");
    Refresh();
  }
  ~Grid() {
    if (sim_) cafe_sim_destroy(sim_);
  }
  Grid(const Grid &) = delete;
  Grid &operator=(const Grid &) = delete;

  // Grid::UpdateLaser (Grid.C:110-164)
  void UpdateLaser() {
    amcafe_dropin::check(cafe_sim_update_laser(sim_), "Grid::UpdateLaser");
    Refresh();
  }
  // Grid::UpdateTime2 (Grid.C:334-339): time += dtIn, tInd += 1. The engine
  // advances by its own TempField::DelT, so dtIn must be that value (main1.C
  // passes TempF.DelT).
  void UpdateTime2(const double &dtIn) {
    if (dtIn != DelT_)
      throw std::invalid_argument("Grid::UpdateTime2: the engine advances by TempField::DelT only");
    amcafe_dropin::check(cafe_sim_update_time(sim_), "Grid::UpdateTime2");
    Refresh();
  }

  // Extension: the engine handle, and the refresh of the public scalars.
  cafe_sim *Engine() const { return sim_; }
  void Refresh() {
    cafe_grid c;
    amcafe_dropin::check(cafe_sim_grid(sim_, &c), "Grid::Refresh");
    nDim = 3;
    nX.assign(c.nX, c.nX + 3);
    dX.assign(c.dX, c.dX + 3);
    LX.assign(c.LX, c.LX + 3);
    offset.assign(c.offset, c.offset + 3);
    meltparam.assign(c.meltparam, c.meltparam + 4);
    gsize.assign(c.gsize, c.gsize + 2);
    for (int a = 0; a < 4; ++a) gbox[a] = c.gbox[a];
    deltaXmin = std::min(dX[0], std::min(dX[1], dX[2]));
    bmV = c.bmV;
    bmP = c.bmP;
    bmDelT = c.bmDelT;
    bhatch = c.bhatch;
    tL = c.tL;
    tS = c.tS;
    T0 = c.T0;
    layerT = c.layerT;
    bpH = c.bpH;
    mu = c.mu;
    lrate = c.lrate;
    rNmax = c.rNmax;
    Avel = c.Avel;
    nvel = c.nvel;
    gth0 = c.gth0;
    gth = c.gth;
    time = c.time;
    dt = c.DelT;
    DelT_ = c.DelT;
    outint = c.outint;
    patternID = c.patternID;
    outNL = c.outNL;
    EASM_Flag = c.EASM_Flag;
    nZlayer = c.nZlayer;
    Nzhg = c.Nzhg;
    Nsd = c.Nsd;
    Ntd = c.Ntd;
    NpT = c.NpT;
    isp = c.isp;
    inewscanflg = c.inewscanflg;
    inewlayerflg = c.inewlayerflg;
    indlayer = c.indlayer;
    ilaserLoc = c.ilaserLoc;
    tInd = c.tInd;
  }

  // public fields of Grid.h:48-93 (the laser point tables lcoor/lcoor2 stay
  // in the engine and are left empty here)
  std::string filInput;
  double deltaXmin = 0, deltaTcheck = 0, dt = 0, time = 0, gth0 = 0, gth = 0;
  std::vector<double> dX, meltparam, beamSTD, LX, offset, lcoor, lcoor2, gsize;
  std::vector<int> nX;
  int nDim = 3, tInd = 0, nnodePerCell = 8, ictrl = 3, nZlayer = 0, patternID = 0, outint = 1, myid = 0,
      nprocs = 1, outNL = 0, nTsd = 2, Nsd = 0, Ntd = 0, NpT = 0, inewscanflg = 0, inewlayerflg = 0, isp = 0,
      indlayer = 0, ilaserLoc = 0, Nzhg = 0, EASM_Flag = 0;
  double bmV = 0, bmP = 0, bhatch = 0;
  double tL = 0, tS = 0, T0 = 0;
  double mL = 0, c0 = 0, Gamma = 0, kP = 0, dL = 0, muN = 0, rho = 0, kappa = 0, dTempM = 0, dTempS = 0;
  double rNmax = 0, cP = 0, dP = 0, layerT = 0, ethresh = 0, deltaThresh = 0, mu = 0, bpH = 0, lrate = 0;
  double beamEta = 0, T0targ = 0, bmDelT = 0, gbox[4] = {0, 0, 0, 0}, Avel = 0, nvel = 0;
  std::string ntype = "Moore", neighOrder = "first";

 private:
  cafe_sim *sim_ = nullptr;
  double DelT_ = 0;
};

#endif

// Drop-in VoxelsCA (reference: src/src-mpi/VoxelsCA.h:13-137): the methods
// main1.C calls, forwarded to the GPU engine, and the public state vectors.
// The voxel state lives on the device; the vectors below are copied from it
// where the reference's loop observes the state (SetBuild: Build;
// WriteToHDF1 and Sync(): everything; CleanLayer: the grain table). See
// Grid.h.
#ifndef VOXELSCA_H
#define VOXELSCA_H

#include <random>
#include <string>
#include <vector>

#include "BasePlate.h"
#include "Grid.h"
#include "Partition.h"
#include "TempField.h"

class VoxelsCA {
 public:
  // VoxelsCA::VoxelsCA (VoxelsCA.C:34-74); the neighbour table is an
  // implicit 26-point stencil on the device.
  VoxelsCA(Grid &g, TempField &tf, Partition &part) : _xyz(&g), _temp(&tf), _part(&part) { RefreshGrains(); }

  // VoxelsCA::InitializeVoxels (VoxelsCA.C:125-161 with BasePlate::
  // GenerateVoxel, BasePlate.C:41-97)
  void InitializeVoxels(BasePlate &bpIn) {
    bp = &bpIn;
    amcafe_dropin::check(cafe_sim_initialize_voxels(sim()), "VoxelsCA::InitializeVoxels");
    RefreshGrains();
    bpIn.Ngrain = nGrain;
  }
  // VoxelsCA::AddLayer1 (VoxelsCA.C:887-982)
  void AddLayer1() {
    amcafe_dropin::check(cafe_sim_add_layer(sim()), "VoxelsCA::AddLayer1");
    RefreshGrains();
  }
  // VoxelsCA::UpdateVoxels (VoxelsCA.C:232-655)
  void UpdateVoxels() {
    amcafe_dropin::check(cafe_sim_update_voxels(sim()), "VoxelsCA::UpdateVoxels");
    RefreshGrains();
  }
  // VoxelsCA::CleanLayer (VoxelsCA.C:800-839)
  void CleanLayer() {
    amcafe_dropin::check(cafe_sim_clean_layer(sim()), "VoxelsCA::CleanLayer");
    RefreshGrains();
    SyncGrainTable();
  }
  // VoxelsCA::SetBuild (VoxelsCA.C:76-115). The engine marks from its own
  // BuildjID, which is TempField::BuildjID of this loop (what main1.C
  // passes); jlist and Ntot are checked for size only.
  void SetBuild(std::vector<int> jlist, int Ntot) {
    if ((size_t)Ntot != ncell()) throw std::invalid_argument("VoxelsCA::SetBuild: Ntot must be the cell count");
    (void)jlist;
    amcafe_dropin::check(cafe_sim_set_build(sim()), "VoxelsCA::SetBuild");
    Build.resize(ncell());
    amcafe_dropin::check(cafe_sim_download_build(sim(), Build.data()), "VoxelsCA::SetBuild");
  }
  // VoxelsCA::WriteToHDF1 (VoxelsCA.C:1592-1856): the reference's datasets
  // as raw files <filname>.h5.<dataset>.bin plus <filname>.h5.xdmf
  // (cafe_sim_write_output), then the public vectors are refreshed.
  void WriteToHDF1(const std::string &filname) {
    amcafe_dropin::check(cafe_sim_write_output(sim(), (filname + ".h5").c_str()), "VoxelsCA::WriteToHDF1");
    Sync();
  }

  // Extension: every public vector (and TempField::TempCurr, BuildjID) from
  // the device.
  void Sync() {
    const size_t n = ncell();
    gID.resize(n);
    vState.resize(n);
    extents.resize(n);
    centroidOct.resize(3 * n);
    Build.resize(n);
    amcafe_dropin::check(
        cafe_sim_download_state(sim(), gID.data(), vState.data(), extents.data(), centroidOct.data(), nullptr),
        "VoxelsCA::Sync");
    amcafe_dropin::check(cafe_sim_download_build(sim(), Build.data()), "VoxelsCA::Sync");
    RefreshGrains();
    SyncGrainTable();
    _temp->Sync();
  }

  std::vector<int> gID, gNucleus, ineighID, ineighptr;
  std::vector<int> vState, Build;  // 0=uninitialized; 1=liquid; 2=mushy; 3=solid
  std::vector<double> cTheta, extents, centroidOct;
  double vmax = 0;
  int nGrain = 0, seed0 = 2132512, seed1 = 2912351, NzhBP = 0;
  std::default_random_engine genlayer;

 private:
  cafe_sim *sim() const { return _xyz->Engine(); }
  size_t ncell() const { return (size_t)_xyz->nX[0] * _xyz->nX[1] * _xyz->nX[2]; }
  void RefreshGrains() {
    cafe_info i;
    amcafe_dropin::check(cafe_sim_info(sim(), &i), "VoxelsCA");
    nGrain = i.nGrain;
    NzhBP = i.Nzh;
    genlayer.seed(i.genlayer_state);
    _xyz->Refresh();
    _temp->Refresh();
  }
  void SyncGrainTable() {
    cTheta.resize(4 * (size_t)nGrain);
    int ng = 0;
    amcafe_dropin::check(cafe_sim_download_ctheta(sim(), cTheta.data(), (long long)cTheta.size(), &ng),
                         "VoxelsCA::Sync");
    cTheta.resize(4 * (size_t)ng);
    nGrain = ng;
  }
  Grid *_xyz;
  BasePlate *bp = nullptr;
  TempField *_temp;
  Partition *_part;
};

#endif

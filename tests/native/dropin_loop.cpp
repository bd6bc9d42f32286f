// A C++ time loop written against the drop-in classes of include/amcafe/
// (Grid, Partition, BasePlate, Utilities, TempField, VoxelsCA), calling them
// as the reference's main1.C does (main1.C:29-97), with the reference's
// output points (main1.C:76-84). Each output point is written as
// <outdir>/out<tInd>.h5.* and the state after the closing CleanLayer as
// <outdir>/final.h5.*. It also checks that the public vectors the classes
// refresh at WriteToHDF1 agree with the engine's own downloads. Test-only.
// Usage: dropin_loop <deck.in> <outdir>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "BasePlate.h"
#include "Grid.h"
#include "Partition.h"
#include "SampleOrientation.h"
#include "TempField.h"
#include "Utilities.h"
#include "VoxelsCA.h"

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s deck.in outdir\n", argv[0]);
    return 2;
  }
  std::string deck = argv[1], outdir = argv[2];
  int myid = 0, nprocs = 1;
  Grid g(deck, myid, nprocs);
  Partition part(g, myid, nprocs);
  part.PartitionGraph2();
  BasePlate bp(g, part);
  Utilities ut(g, part, bp);
  TempField tf(g, part, bp, ut);
  const int ncell = part.ncellLoc + part.nGhost;
  tf.InitializeAnalytic();
  ut.InitializeUT();
  VoxelsCA vox(g, tf, part);
  vox.InitializeVoxels(bp);
  const int nlayers = int(std::ceil(double(g.nX[2] - bp.Nzh) / double(g.nZlayer)));
  vox.AddLayer1();
  g.UpdateLaser();
  bool last = false;
  long steps = 0;
  while (!last) {
    tf.tInd = int(std::round(g.time / tf.DelT));
    if (g.EASM_Flag == 1)
      tf.EASM(tf.TempCurr, part.icellidLoc, ncell);
    else
      tf.AnalyticTempCurr(g.time, tf.TempCurr, part.icellidLoc, ncell);
    vox.UpdateVoxels();
    g.UpdateLaser();
    last = g.indlayer > nlayers;
    if (g.inewlayerflg == 1) vox.CleanLayer();
    if (tf.tInd % g.outint == 0 || last || (g.inewlayerflg == 1 && g.outNL == 0)) {
      vox.SetBuild(tf.BuildjID, ncell);
      vox.WriteToHDF1(outdir + "/out" + std::to_string(tf.tInd));
    }
    g.UpdateTime2(tf.DelT);
    if (g.inewlayerflg == 1) vox.AddLayer1();
    ++steps;
  }
  vox.CleanLayer();
  vox.WriteToHDF1(outdir + "/final");
  // the refreshed public vectors against the engine's downloads
  std::vector<int32_t> gid((size_t)ncell);
  cafe_sim_download_state(g.Engine(), gid.data(), nullptr, nullptr, nullptr, nullptr);
  for (int i = 0; i < ncell; ++i)
    if (gid[i] != vox.gID[i]) {
      std::fprintf(stderr, "VoxelsCA::gID differs from the engine at cell %d\n", i);
      return 1;
    }
  if ((int)vox.cTheta.size() != 4 * vox.nGrain || (int)tf.TempCurr.size() != ncell || (int)vox.Build.size() != ncell) {
    std::fprintf(stderr, "public vectors have the wrong sizes\n");
    return 1;
  }
  SampleOrientation so;
  std::vector<double> aa;
  so.GenerateSamples(3, 12345u, aa);
  std::printf("steps %ld nGrain %d layers %d orientation0 %.17g\n", steps, vox.nGrain, nlayers, aa[0]);
  return 0;
}

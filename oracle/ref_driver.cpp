// State-dumping driver for the reference sources (test infrastructure).
//
// Links against AMCAFE's own classes (src/src-mpi/{Grid,Partition,BasePlate,
// Utilities,TempField,VoxelsCA,SampleOrientation}.C, compiled unmodified with
// the single-rank shims in ref_shims/) and runs the same time loop as
// src/src-mpi/main1.C:18-101, writing the full CA state after every step so the
// oracle restatement and the GPU path can be compared with the reference
// itself. SetBuild is called where main1.C calls it so that the Build field
// evolves as in the reference. When CAFE_REF_DUMP_DIR is set, WriteToHDF1 also
// runs at every CAFE_REF_OUT_EVERY-th output point (default 1) as
// "out<tInd>" and after the closing CleanLayer as "final"; the ADIOS2 shim
// then writes its datasets as raw files into that directory.
//
// Usage: cafe_ref_dump <deck.in> <out.bin> [max_steps]   (CAFE_REF_EASM=1: EASM temperature)
// Record layout (little-endian): see oracle/cafe_dump.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "BasePlate.h"
#include "Grid.h"
#include "Partition.h"
#include "TempField.h"
#include "Utilities.h"
#include "VoxelsCA.h"
#include "mpi.h"

static void put_i32(FILE *fp, int32_t v) { std::fwrite(&v, 4, 1, fp); }
static void put_f64(FILE *fp, double v) { std::fwrite(&v, 8, 1, fp); }

static void dump_state(FILE *fp, int32_t tag, Grid &g, TempField &tf, VoxelsCA &vox, int ncell) {
  // record: magic, tag, tInd, nGrain, ncell, isp, indlayer, inewlayerflg, inewscanflg, time
  put_i32(fp, 0x43414645);  // 'CAFE'
  put_i32(fp, tag);
  put_i32(fp, tf.tInd);
  put_i32(fp, vox.nGrain);
  put_i32(fp, ncell);
  put_i32(fp, g.isp);
  put_i32(fp, g.indlayer);
  put_i32(fp, g.inewlayerflg);
  put_i32(fp, g.inewscanflg);
  put_f64(fp, g.time);
  std::fwrite(vox.gID.data(), 4, ncell, fp);
  std::fwrite(vox.vState.data(), 4, ncell, fp);
  std::fwrite(vox.extents.data(), 8, ncell, fp);
  std::fwrite(vox.centroidOct.data(), 8, 3 * (size_t)ncell, fp);
  std::fwrite(tf.TempCurr.data(), 8, ncell, fp);
  std::fwrite(tf.BuildjID.data(), 4, ncell, fp);
  std::fwrite(vox.cTheta.data(), 8, 4 * (size_t)vox.nGrain, fp);
}

int main(int argc, char *argv[]) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s deck.in out.bin [max_steps]\n", argv[0]);
    return 2;
  }
  long max_steps = argc > 3 ? std::atol(argv[3]) : -1;
  MPI_Init(NULL, NULL);
  int nprocs = 1, myid = 0;
  std::string filParamIn = argv[1];
  Grid g(filParamIn, myid, nprocs);
  // Grid::readInputFile lowercases each keyword before comparing it with
  // "EASM" (Grid.C:197-198, 276), so no deck selects the EASM temperature;
  // CAFE_REF_EASM=1 sets the flag that keyword was meant to set.
  if (std::getenv("CAFE_REF_EASM") && std::atoi(std::getenv("CAFE_REF_EASM")) == 1) g.EASM_Flag = 1;
  Partition part(g, myid, nprocs);
  part.PartitionGraph2();
  BasePlate bp(g, part);
  Utilities ut(g, part, bp);
  TempField TempF(g, part, bp, ut);
  int Ntot = part.ncellLoc + part.nGhost;
  TempF.InitializeAnalytic();
  ut.InitializeUT();
  VoxelsCA vox(g, TempF, part);
  vox.InitializeVoxels(bp);
  const char *out_dir = std::getenv("CAFE_REF_DUMP_DIR");
  long out_every = std::getenv("CAFE_REF_OUT_EVERY") ? std::atol(std::getenv("CAFE_REF_OUT_EVERY")) : 1;
  if (out_every < 1) out_every = 1;
  FILE *fp = std::fopen(argv[2], "wb");
  if (!fp) return 3;
  int nlayerTot = int(ceil((double)(g.nX[2] - bp.Nzh) / (double)g.nZlayer));
  bool bcheck = 0;
  vox.AddLayer1();
  g.UpdateLaser();
  dump_state(fp, 0, g, TempF, vox, Ntot);  // initial state (tag 0)
  long nstep = 0;
  while (!bcheck) {
    TempF.tInd = int(round(g.time / TempF.DelT));
    if (g.EASM_Flag == 1) {
      TempF.EASM(TempF.TempCurr, part.icellidLoc, Ntot);
    } else {
      TempF.AnalyticTempCurr(g.time, TempF.TempCurr, part.icellidLoc, Ntot);
    }
    vox.UpdateVoxels();
    g.UpdateLaser();
    bcheck = g.indlayer > nlayerTot;
    if (g.inewlayerflg == 1) vox.CleanLayer();
    int indOut = TempF.tInd % g.outint;
    if (indOut == 0 || bcheck || (g.inewlayerflg == 1 && g.outNL == 0)) {
      vox.SetBuild(TempF.BuildjID, Ntot);
      if (out_dir && (nstep + 1) % out_every == 0) vox.WriteToHDF1("out" + std::to_string(TempF.tInd));
    }
    g.UpdateTime2(TempF.DelT);
    if (g.inewlayerflg == 1) vox.AddLayer1();
    ++nstep;
    dump_state(fp, 1, g, TempF, vox, Ntot);  // after a step (tag 1)
    if (max_steps > 0 && nstep >= max_steps) break;
  }
  if (bcheck) {
    vox.CleanLayer();
    if (out_dir) vox.WriteToHDF1("final");
    dump_state(fp, 2, g, TempF, vox, Ntot);  // final state after the closing CleanLayer (tag 2)
  }
  std::fclose(fp);
  MPI_Finalize();
  return 0;
}

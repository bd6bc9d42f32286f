/* A C program driving one deck through the engine's C ABI (include/
 * cafe_gpu.h), the way a C caller replaces the reference's time loop
 * (main1.C:29-97): create, initialise, the loop with the datasets of
 * WriteToHDF1 written by the engine at every output point as
 * <outdir>/out<tInd>.h5.* (cafe_sim_set_output), the closing CleanLayer and a
 * last write as <outdir>/final.h5.*. Test-only.
 * Usage: capi_loop <deck.in> <outdir> */
#include <stdio.h>
#include <stdlib.h>

#include "cafe_gpu.h"

static void check(int rc, const char *what) {
  if (rc != CAFE_OK) {
    fprintf(stderr, "%s: %s\n", what, cafe_last_error());
    exit(1);
  }
}

int main(int argc, char **argv) {
  cafe_options opt = {0, 0, 0, 0, 0};
  cafe_sim *sim = NULL;
  cafe_info info;
  char path[4096];
  int done = 0;
  if (argc < 3) {
    fprintf(stderr, "usage: %s deck.in outdir\n", argv[0]);
    return 2;
  }
  check(cafe_sim_create(argv[1], &opt, &sim), "create");
  snprintf(path, sizeof path, "%s/out", argv[2]);
  check(cafe_sim_set_output(sim, path), "set_output");
  check(cafe_sim_initialize_voxels(sim), "initialize_voxels");
  check(cafe_sim_begin(sim), "begin");
  while (!done) check(cafe_sim_step(sim, &done), "step");
  check(cafe_sim_clean_layer(sim), "clean_layer");
  snprintf(path, sizeof path, "%s/final.h5", argv[2]);
  check(cafe_sim_write_output(sim, path), "write_output");
  check(cafe_sim_info(sim, &info), "info");
  printf("steps %lld nGrain %d\n", info.steps, info.nGrain);
  cafe_sim_destroy(sim);
  return 0;
}

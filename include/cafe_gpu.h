/* C ABI of the GB300 CA engine (libcafe_gpu.so).
 *
 * One cafe_sim is one realisation of AMCAFE's model on one GPU: the state of
 * its Grid, Partition (world size 1), BasePlate, TempField and VoxelsCA
 * objects (AMCAFE src/src-mpi/main1.C:29-42) with the voxel fields resident in
 * device memory. The entry points below replace, one for one, the member
 * functions that the reference's time loop (main1.C:60-96) calls; each cites
 * the reference function it stands in for. All functions return 0 on success
 * and a nonzero CAFE_E_* code otherwise (never abort); cafe_last_error()
 * returns a message for the calling thread. Calls on one handle must be
 * serialised by the caller (one host thread per handle); different handles
 * are independent.
 */
#ifndef CAFE_GPU_H
#define CAFE_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cafe_sim cafe_sim;

enum {
  CAFE_OK = 0,
  CAFE_E_ARG = 1,      /* bad argument or deck value */
  CAFE_E_CUDA = 2,     /* CUDA runtime error (message has the CUDA error string) */
  CAFE_E_CAPACITY = 3, /* an active-list, frontier or grain table capacity was exceeded */
  CAFE_E_STATE = 4,    /* call out of order (e.g. step before initialize) */
  CAFE_E_IO = 5        /* deck file could not be read */
};

typedef struct {
  int device;                  /* CUDA device ordinal */
  long long active_capacity;   /* max active-list length per step; 0 = automatic */
  long long grain_capacity;    /* initial grain-table capacity; 0 = automatic */
  int event_scan;              /* 0: keyed event selection (default); 1: evaluate every
                                  frontier cell at every event (the reference's scan) */
  int event_fill_helper;       /* 1: the event loop hands each new frontier row's set-up to a
                                  second thread block on another SM (same results; measured
                                  slower on this GPU: the selection, not the set-up, bounds an
                                  event); 0 (default): one block does everything */
} cafe_options;

typedef struct {
  int nx, ny, nz;
  double dx;
  int tInd;        /* Grid::tInd */
  double time;     /* Grid::time */
  int isp, indlayer, inewlayerflg, inewscanflg, ilaserLoc;
  int nGrain;      /* VoxelsCA::nGrain */
  int nlayerTot;   /* main1.C:59 */
  int Nzh;         /* BasePlate::Nzh */
  int done;        /* main1.C loop condition reached (indlayer > nlayerTot) */
  long long steps; /* loop iterations executed */
  double gth;      /* Grid::gth, current rotation of the laser grid */
  unsigned int genlayer_state; /* VoxelsCA::genlayer engine state (minstd_rand0) */
  int tf_tInd;     /* TempField::tInd of the last step (main1.C:64) */
  int output_due;  /* 1 when the last cafe_sim_step reached an output point of
                      main1.C:77-78 (it called SetBuild there; the reference
                      writes WriteToHDF1("<base>" + tf_tInd) at this point;
                      cafe_sim_set_output has the step write it there) */
} cafe_info;

typedef struct {
  unsigned long long events;       /* captures + nucleations */
  unsigned long long nucleations;
  unsigned long long max_active;   /* largest active list */
  unsigned long long max_rows;     /* largest frontier (capturing cells) */
  unsigned long long steps;        /* UpdateVoxels calls */
  unsigned long long negative_dt;  /* events with a negative capture time */
  unsigned long long sum_active;   /* sum over steps of the active-list length */
  unsigned long long sum_rows;     /* sum over steps of the frontier size */
  unsigned long long launches;     /* kernels launched by this handle since the last phase reset */
  unsigned long long exact_scan_steps; /* steps run with the full per-event scan */
  unsigned long long row_evaluations;  /* keyed-selection rounds that evaluated rows exactly */
  unsigned long long cycles_select;    /* event-loop SM cycles taking this event's winner */
  unsigned long long cycles_apply;     /* ... applying the capture/nucleation */
  unsigned long long cycles_fill;      /* ... new frontier row and next selection, side by side */
  unsigned long long graph_captures;   /* step graphs captured (one per handle unless buffers move) */
  unsigned long long easm_integrals;   /* EASM: Utilities::Integral evaluations (25 nodes each) */
  unsigned long long cycles_merge;     /* ... taking the next event's winner (the new row's
                                          result included) */
} cafe_stats;

/* Grid::Grid (Grid.C:15-109, deck parse Grid.C:165-318) + Partition::
 * PartitionGraph2 at world size 1 (Partition.C:260-412) + BasePlate::BasePlate
 * (BasePlate.C:18-30) + TempField::TempField/InitializeAnalytic
 * (TempField.C:16-77) + VoxelsCA::VoxelsCA (VoxelsCA.C:34-74). Allocates the
 * device state. opt may be NULL. */
int cafe_sim_create(const char *deck_path, const cafe_options *opt, cafe_sim **out);
void cafe_sim_destroy(cafe_sim *sim);

/* VoxelsCA::InitializeVoxels(BasePlate&) (VoxelsCA.C:125-161, BasePlate::
 * GenerateVoxel BasePlate.C:41-97). */
int cafe_sim_initialize_voxels(cafe_sim *sim);
/* VoxelsCA::AddLayer1 (VoxelsCA.C:887-982). */
int cafe_sim_add_layer(cafe_sim *sim);
/* Grid::UpdateLaser (Grid.C:110-164). */
int cafe_sim_update_laser(cafe_sim *sim);
/* TempField::AnalyticTempCurr (TempField.C:139-217), including the
 * end-of-scan check that may set Grid::inewscanflg / inewlayerflg. Sets
 * TempField::tInd = round(time/DelT) first (main1.C:64). */
int cafe_sim_temperature(cafe_sim *sim);
/* VoxelsCA::UpdateVoxels (VoxelsCA.C:232-655). */
int cafe_sim_update_voxels(cafe_sim *sim);
/* VoxelsCA::CleanLayer (VoxelsCA.C:800-839). */
int cafe_sim_clean_layer(cafe_sim *sim);
/* Grid::UpdateTime2(TempField::DelT) (Grid.C:334-339). */
int cafe_sim_update_time(cafe_sim *sim);

/* main1.C:60-61: AddLayer1 then the first UpdateLaser (after
 * initialize_voxels). */
int cafe_sim_begin(cafe_sim *sim);
/* One iteration of the main1.C:62-93 loop body, SetBuild at the output
 * points included, WriteToHDF1 left to the caller (cafe_info.output_due and
 * cafe_sim_write_output); *done = 1 when the loop condition ends the run. */
int cafe_sim_step(cafe_sim *sim, int *done);
/* Runs loop iterations until done or max_steps (> 0) iterations; then, when
 * done, the closing CleanLayer (main1.C:95). */
int cafe_sim_run(cafe_sim *sim, long long max_steps, long long *steps_done);
/* Waits for all queued device work; reports device-side errors. */
int cafe_sim_synchronize(cafe_sim *sim);

int cafe_sim_info(cafe_sim *sim, cafe_info *info);

/* The public scalars of the handle's Grid (Grid.h:48-93: deck values and the
 * quantities Grid::Grid derives from them, Grid.C:15-109, plus the laser
 * state that UpdateLaser and the temperature's end-of-scan check change),
 * TempField::DelT and tInd, BasePlate::Nzh and main1.C's nlayerTot. The
 * drop-in classes of include/amcafe/ mirror their public fields from it. */
typedef struct {
  int nX[3];
  double dX[3], LX[3], offset[3];
  double meltparam[4], gbox[4], gsize[2];
  double bmV, bmP, bmDelT, bhatch, tL, tS, T0, layerT, bpH, mu, lrate, rNmax, Avel, nvel;
  double gth0, gth, time;
  double DelT;  /* TempField::DelT */
  int outint, patternID, outNL, EASM_Flag, nZlayer, Nzhg, Nsd, Ntd, NpT;
  int isp, inewscanflg, inewlayerflg, indlayer, ilaserLoc, tInd;
  int tf_tInd;  /* TempField::tInd */
  int Nzh;      /* BasePlate::Nzh */
  int nlayerTot;
  int seed;     /* extension keyword "seed" (1: the reference's seeds) */
  int tmodel;   /* temperature: 0 analytic, 1 EASM ("easm 1"), 2 Rosenthal ("rosenthal eta k alpha") */
  double ros_eta, ros_k, ros_alpha; /* Rosenthal: absorptivity, W/(m K), m^2/s */
  double laser[3]; /* source of the next temperature call in the laser frame (TempField.C:145-154) */
  double dirp;     /* its scan direction term (TempField.C:167-171): > 0 along +x of that frame */
} cafe_grid;
int cafe_sim_grid(cafe_sim *sim, cafe_grid *grid);
/* SampleOrientation::GenerateSamples(n, seed, axisAngle)
 * (SampleOrientation.C:124-161) on the host with the host's libm, as the
 * engine draws baseplate and layer orientations: n uniformly distributed
 * orientations as (angle, axis x, y, z), 4 doubles each, into axis_angle. */
int cafe_generate_samples(int n, unsigned int seed, double *axis_angle);

/* Device-time accounting, for profiling: phases of one step, each bracketed
 * by CUDA events on the handle's stream when timing is on. */
enum {
  CAFE_PH_MELT = 0,      /* TempField::AnalyticTempCurr + SetLiquid3 on the pool box */
  CAFE_PH_CLASSIFY = 1,  /* ConvertSolid1(1) + active-set compaction */
  CAFE_PH_GATHER = 2,    /* active copies, neighbour lists, frontier numerators */
  CAFE_PH_EVENTS = 3,    /* the capture/nucleation event loop */
  CAFE_PH_WRITEBACK = 4, /* write-back + ConvertSolid1(0) */
  CAFE_PH_LAYER = 5,     /* CleanLayer / AddLayer1 device work */
  CAFE_NPHASE = 8
};
int cafe_sim_set_timing(cafe_sim *sim, int on);
/* Accumulated milliseconds and kernel launches per phase (nphase entries). */
int cafe_sim_phase_times(cafe_sim *sim, double *ms, long long *launches, int nphase, int reset);
/* The CUDA stream (cudaStream_t) all work of this handle is queued on. */
int cafe_sim_stream(cafe_sim *sim, void **stream);
/* Records CUDA event `slot` (0..7) on the handle's stream; cafe_sim_elapsed
 * waits for slot b and returns the device time between slots a and b. */
int cafe_sim_mark(cafe_sim *sim, int slot);
int cafe_sim_elapsed(cafe_sim *sim, int a, int b, double *ms);
int cafe_sim_stats(cafe_sim *sim, cafe_stats *stats);

/* VoxelsCA public fields gID, vState, extents, centroidOct (x,y,z interleaved,
 * 3 per cell) and TempField::BuildjID, N = nx*ny*nz entries each; any pointer
 * may be NULL. */
int cafe_sim_download_state(cafe_sim *sim, int32_t *gID, int32_t *vState, double *extents,
                            double *centroid, int32_t *buildjID);
/* TempField::TempCurr of the last cafe_sim_temperature call. */
int cafe_sim_download_temperature(cafe_sim *sim, double *temp);
/* VoxelsCA::cTheta, 4 per grain; cap = capacity of out in doubles; *ngrain gets nGrain. */
int cafe_sim_download_ctheta(cafe_sim *sim, double *ctheta, long long cap, int *ngrain);
/* Replaces the voxel state and grain table (same layouts as the downloads). */
int cafe_sim_upload_state(cafe_sim *sim, const int32_t *gID, const int32_t *vState,
                          const double *extents, const double *centroid, const double *ctheta,
                          int ngrain);

/* VoxelsCA::SetBuild(TempField::BuildjID) (VoxelsCA.C:76-115): every cell
 * of a grain that has a melted cell or a Build cell gets Build = 1. */
int cafe_sim_set_build(cafe_sim *sim);
/* VoxelsCA::Build (0/1), N entries. */
int cafe_sim_download_build(cafe_sim *sim, int32_t *build);
/* The per-cell datasets that VoxelsCA::WriteToHDF1 (VoxelsCA.C:1592-1854)
 * derives for output: Temperature (TempCurr of the last cafe_sim_temperature
 * call, as float; N entries) and the inverse-pole-figure colour maps IPFz,
 * IPFx, IPFy (RGB of the sample's build, x and y directions in each cell's
 * crystal frame, 3 floats per cell; 0 for cells without a grain), with the
 * reference's colouring as written (the y map's hue starts from the x map's
 * hue; the hue fraction is H/6). Any pointer may be NULL. */
int cafe_sim_download_output(cafe_sim *sim, float *temperature, float *ipfz, float *ipfx, float *ipfy);
/* VoxelsCA::WriteToHDF1(name) (VoxelsCA.C:1592-1854) with one raw file per
 * dataset in place of the HDF5 file: <prefix>.<dataset>.bin for the datasets
 * dims (3 int32: nX), VoxelDX (3 float: dX), gID, vState, Build (int32 per
 * cell), Temperature (float per cell), IPFz, IPFx, IPFy (3 float per cell)
 * and angleAxis (cTheta as float, 4 per grain), native byte order, in the
 * reference's cell order, and <prefix>.xdmf, an XDMF description of the
 * per-cell files as cell data on the voxel grid. The reference's file
 * <base><tInd>.h5 corresponds to prefix "<base><tInd>.h5". */
int cafe_sim_write_output(cafe_sim *sim, const char *prefix);

/* The output of main1.C:77-84 and 95-97 written by the loop itself: with a
 * non-empty base, cafe_sim_step writes the WriteToHDF1 datasets as
 * cafe_sim_write_output(sim, "<base><tf_tInd>.h5") at each output point,
 * after SetBuild and before UpdateTime2 and AddLayer1 (the reference's order:
 * at an output point that is also a layer change the written state is the
 * one before the new layer), and cafe_sim_run writes "<base><tf_tInd>.h5"
 * again after the closing CleanLayer. NULL or "" turns it off (the default);
 * a caller writing after cafe_sim_step returns sees the state after
 * AddLayer1. */
int cafe_sim_set_output(cafe_sim *sim, const char *base);

/* Checkpoint of the whole loop state (no counterpart in the reference, which
 * restarts from a deck): the Grid scalars (time, tInd, laser index, scan and
 * layer flags, layer, laser plane, rotation), TempField::tInd,
 * VoxelsCA::genlayer and nGrain, the loop counters, the voxel fields (gID,
 * vState, extents, centroidOct, BuildjID, Build) and cTheta, in one binary
 * file. cafe_sim_restore loads it into a handle created from the same deck
 * (instead of initialize_voxels and begin); the loop then continues with
 * cafe_sim_step and reaches the same results as the run that wrote it. A
 * restore that fails leaves the handle unusable until a successful one. */
int cafe_sim_checkpoint(cafe_sim *sim, const char *path);
int cafe_sim_restore(cafe_sim *sim, const char *path);

/* Growth log for the adjoint extension (no counterpart in the reference): with
 * three caller-owned device arrays of `cap` entries, every step appends, for
 * each frontier cell of the step (a mushy cell with a liquid neighbour), its
 * cell index, the step's Grid::tInd and its growth time: the extent it gained
 * in the step (VoxelsCA.C:511-516) over its growth velocity, i.e. the sum of
 * the event times it grew through. NULL arrays turn the log off. Setting the
 * arrays resets the count; a full log stops recording and makes
 * cafe_sim_growth_log_count report CAFE_E_CAPACITY. */
int cafe_sim_set_growth_log(cafe_sim *sim, int32_t *cells, int32_t *steps, double *tau, long long cap);
int cafe_sim_growth_log_count(cafe_sim *sim, long long *n);

/* Differentiable part of the step with hand-written adjoints (no counterpart
 * in the reference): the Rosenthal moving point source
 * T = T0 + eta P / (2 pi k R) exp(-v (R + xi) / (2 alpha)) on the cell
 * centres, source at (x_start + v t, y_src, z_src) at t = step dt, parameters
 * theta = {P, eta, v, a, n}.
 * cafe_adjoint_pool: melt-pool length, width, depth at step_final from the
 *   m-weighted moments of the soft melt indicator m = sigmoid((T - Tl)/tau_T)
 *   over the cells below the source plane (sqrt(12 var_x), sqrt(12 var_y),
 *   sqrt(3 E[depth^2])); with cot (3 values) also grad = cot . d out / d theta.
 * cafe_adjoint_growth: over a growth log (device arrays, n entries), the
 *   summed growth sum a (Tl - T)^n tau of the frozen event set; with grad,
 *   also cot * dG/dtheta.
 * Both run on `stream` (a cudaStream_t, NULL = legacy default stream) of the
 * current device and return when done. */
typedef struct {
  double k, alpha, T0, Tl;      /* W/(m K), m^2/s, K, K */
  double tau_T;                 /* width of the soft melt indicator, K */
  double x_start, y_src, z_src; /* source position at t = 0, m */
  double dt;                    /* time per step, s */
  double dx;                    /* voxel size, m */
  int nx, ny, nz;
  int step_final;               /* step of the pool shape */
} cafe_adjoint_setup;
int cafe_adjoint_pool(const cafe_adjoint_setup *setup, const double theta[5], const double *cot, double out[3],
                      double grad[5], void *stream);
int cafe_adjoint_growth(const cafe_adjoint_setup *setup, const double theta[5], const int32_t *cells,
                        const int32_t *steps, const double *tau, long long n, double cot, double *out,
                        double grad[5], void *stream);

/* Batched ensemble (no counterpart in the reference, which runs one
 * realisation per MPI job): n independent realisations, one deck each, on
 * one device, each a cafe_sim handle. threads <= 0 (the default): batched
 * launches, every step kernel launched once for all realisations (the event
 * loop one thread block per realisation), the launches of a batch step one
 * CUDA graph replayed every batch step, launch shapes chosen by timing
 * candidates on the first batch steps (cafe_batch_report gives the choice);
 * a realisation whose step cannot take the graphed path (EASM or Rosenthal
 * field) takes its plain step that batch step. threads >= 1: the realisations
 * step round-robin on their own streams from that many host threads. Either
 * way every realisation runs exactly the calls of a plain run
 * (initialize_voxels, begin, step until done, the closing clean_layer), so
 * its results are bit-identical to its plain run. */
typedef struct cafe_batch cafe_batch;
int cafe_batch_create(const char *const *decks, int n, const cafe_options *opt, int threads, cafe_batch **out);
/* Initialises every realisation that is new and runs each loop to its end, or
 * to max_steps (> 0) iterations per realisation; *steps_done (may be NULL)
 * gets the loop iterations of all realisations. Returns the first error. */
int cafe_batch_run(cafe_batch *b, long long max_steps, long long *steps_done);
int cafe_batch_size(const cafe_batch *b);
/* The i-th realisation's handle (owned by the batch), NULL if out of range. */
cafe_sim *cafe_batch_sim(cafe_batch *b, int i);
/* 1 when realisation i has finished its loop (closing CleanLayer applied). */
int cafe_batch_finished(const cafe_batch *b, int i);
/* Batched launches: kernels launched and batch steps taken so far, and the
 * autotuner's candidates and choice as a JSON object (empty for the
 * round-robin engine or before the first run); tuning may be NULL. */
int cafe_batch_report(const cafe_batch *b, long long *launches, long long *batch_steps, char *tuning, int cap);
void cafe_batch_destroy(cafe_batch *b);

/* Allocation-free CleanLayer renumbering on caller-owned device arrays. No
 * counterpart in the reference: it serves callers that cannot go to the CUDA
 * allocator mid-run (device memory owned by their own pool, or no tolerance
 * for the device-wide synchronisation of cudaFree). Same result as
 * cafe_sim_clean_layer: grains with no cells are dropped, the rest renumbered
 * 1..k in their old order, gid[] remapped in place and ctheta[] (4 doubles per
 * grain) packed in place; *ngrain_out receives k. gid and ctheta are device
 * pointers; stream is a cudaStream_t (NULL = legacy default stream). It calls
 * no cudaMalloc/cudaFree: its scratch is one file-scope device array sized for
 * CAFE_NOALLOC_MAX_GRAINS grains (about 10.5 MB, held by every GPU that loads
 * the library until exit); larger ngrain is rejected with CAFE_E_CAPACITY. The
 * first call on a device looks up that array's device address. Every call
 * ends by synchronising `stream`, so no call may be made while that stream is
 * being captured into a graph. All calls share the scratch: calls whose GPU
 * work overlaps race and must be serialised by the caller. gid[] is checked:
 * a grain ID outside 0..ngrain makes the call return CAFE_E_ARG with gid and
 * ctheta unchanged. After a CAFE_E_CUDA return the contents of gid and ctheta
 * are undefined. */
#define CAFE_NOALLOC_MAX_GRAINS (1 << 18)
int cafe_clean_layer_noalloc(int32_t *gid, long long ncell, double *ctheta, int ngrain,
                             int *ngrain_out, void *stream);

const char *cafe_last_error(void);

#ifdef __cplusplus
}
#endif
#endif

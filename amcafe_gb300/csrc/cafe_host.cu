// Host side of libcafe_gpu.so: the reference's Grid / BasePlate / TempField /
// VoxelsCA objects for one realisation, with the voxel state on the device,
// behind the C ABI of include/cafe_gpu.h.
//
// What stays on the host (cheap scalar state machines and the reference's
// host-side random draws, which use libstdc++ <random> exactly as AMCAFE does):
//   * the .in deck parser and derived values (Grid.C:15-109, 165-318),
//   * the laser path and scan/layer state machine (Grid.C:110-164),
//   * TempField scan order and ellipsoid parameters (TempField.C:16-77),
//   * Poisson grain counts, Voronoi sites and orientations of the baseplate
//     and of each powder layer (BasePlate.C:31-97, VoxelsCA.C:887-982).
// Everything per voxel runs on the device (cafe_kernels.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cafe_gpu.h"
#include "cafe_kernels.cu"
#include "cafe_batch_kernels.cuh"
#include "cafe_quadrature.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define CUDA_TRY(call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(CAFE_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                      \
  } while (0)

const int kSeed0 = 2132512, kSeed1 = 2912351;  // VoxelsCA.C:47-48
const unsigned int kSeedStride = 10000019u;     // per-realisation seed offset (keyword "seed")

// ------------------------------------------------------------------ Grid
struct GridH {
  int nX[3] = {128, 128, 64};
  double dX[3] = {1e-6, 1e-6, 1e-6};
  int outint = 1, patternID = 1, outNL = 0;
  int EASM_Flag = 0;  // Grid::EASM_Flag (keyword "easm", see parse_deck)
  int seed = 1;       // extension keyword "seed" (1: the reference's seeds)
  int nuc_gauss = 0;  // extension keyword "nucgauss mean sd"
  double nuc_mean = 0, nuc_sd = 1;
  int rosenthal = 0;  // extension keyword "rosenthal eta k alpha"
  double ros_eta = 0.35, ros_k = 20.0, ros_alpha = 5e-6;
  double tL = 1620, tS = 1531.5, T0 = 300, layerT = 25e-6, bpH = 0.0, mu = .01, lrate = 0;
  double meltparam[4] = {75e-6, 162.75e-6, 75e-6, 75e-6};
  double bhatch = 0, bmDelT = 0, bmV = 500e-3, bmP = 0, rNmax = .002;
  double offset[3] = {0, 0, 0};
  double gth0 = 0, gth = 0, Avel = 0, nvel = 0, gsize[2] = {0, 0};
  bool set_bmdelt = false, set_lrate = false;
  double LX[3];
  int nZlayer = 0, Nzhg = 0, Ntd = 0, Nsd = 0, NpT = 0;
  std::vector<double> lcoor, lcoor2;
  double gbox[4];
  int isp = 0, inewscanflg = 1, inewlayerflg = 1, indlayer = 1, ilaserLoc = 0, tInd = 0;
  double time = 0.0;
};

// Grid::readInputFile (Grid.C:165-318): whitespace-separated keywords,
// case-insensitive, '#' to end of line is a comment, the last character of
// the file is read twice (so the file must end in whitespace).
int parse_deck(const char *path, GridH &g) {
  std::ifstream f(path);
  if (!f) return fail(CAFE_E_IO, "cannot open deck '%s'", path);
  std::string data;
  char c = 0;
  while (!f.eof()) {
    f.get(c);
    if (c == '#')
      while (f && c != '\n') f.get(c);
    data.push_back(c);
  }
  g.bhatch = 1.53 * g.meltparam[2];
  std::istringstream in(data);
  std::string kw;
  auto num = [&](double &v) -> bool {
    if (!(in >> kw)) return false;
    char *end = nullptr;
    v = std::strtod(kw.c_str(), &end);
    return end != kw.c_str();
  };
  auto inum = [&](int &v) -> bool {
    if (!(in >> kw)) return false;
    char *end = nullptr;
    long x = std::strtol(kw.c_str(), &end, 10);
    v = (int)x;
    return end != kw.c_str();
  };
  in >> kw;
  while (in) {
    std::string key = kw;
    std::transform(key.begin(), key.end(), key.begin(), [](unsigned char s) { return (char)std::tolower(s); });
    bool ok = true;
    if (key == "dx") {
      ok = num(g.dX[0]);
      g.dX[1] = g.dX[2] = g.dX[0];
    } else if (key == "bmv") ok = num(g.bmV);
    else if (key == "bmp") ok = num(g.bmP);
    else if (key == "bmdelt") { ok = num(g.bmDelT); g.set_bmdelt = true; }
    else if (key == "nx") ok = inum(g.nX[0]) && inum(g.nX[1]) && inum(g.nX[2]);
    else if (key == "r") ok = num(g.rNmax);
    else if (key == "lt") ok = num(g.layerT);
    else if (key == "tl") ok = num(g.tL);
    else if (key == "ts") ok = num(g.tS);
    else if (key == "bhatch") ok = num(g.bhatch);
    else if (key == "mu") ok = num(g.mu);
    else if (key == "bph") ok = num(g.bpH);
    else if (key == "lrate") { ok = num(g.lrate); g.set_lrate = true; }
    else if (key == "outnl") ok = inum(g.outNL);
    // ntsd only sets Utilities::nTTemp (Utilities.C:163), which nothing reads
    else if (key == "ntsd") { int dummy; ok = inum(dummy); }
    else if (key == "offset") ok = num(g.offset[0]) && num(g.offset[1]) && num(g.offset[2]);
    else if (key == "meltparam")
      ok = num(g.meltparam[0]) && num(g.meltparam[1]) && num(g.meltparam[2]) && num(g.meltparam[3]);
    else if (key == "patternid") ok = inum(g.patternID);
    else if (key == "outint") ok = inum(g.outint);
    else if (key == "gridsize") ok = num(g.gsize[0]) && num(g.gsize[1]);
    else if (key == "gridtheta") ok = num(g.gth0);
    else if (key == "dendritegrowth2") ok = num(g.Avel) && num(g.nvel);
    // Grid.C:276 compares the lowercased keyword with "EASM", which never
    // matches; "easm 1" sets the flag that keyword was meant to set.
    else if (key == "easm") ok = inum(g.EASM_Flag);
    // extension: realisation seed s >= 1; offsets VoxelsCA's seed0/seed1
    // (VoxelsCA.C:47-48) by (s - 1) * kSeedStride and seeds the BasePlate
    // engine (BasePlate.h:28, default seed 1) with s, so s = 1 is the reference
    else if (key == "seed") ok = inum(g.seed) && g.seed >= 1;
    // extension: nucleation probability rX exp(-.5 x1^2) per capture event,
    // x1 = ((tL - T) - mean)/sd/sqrt(2) (the form of VoxelsCA.C:2545-2548)
    else if (key == "nucgauss") {
      ok = num(g.nuc_mean) && num(g.nuc_sd) && g.nuc_sd > 0;
      g.nuc_gauss = 1;
    }
    // extension: the Rosenthal moving point source (absorptivity,
    // conductivity W/(m K), diffusivity m^2/s) with power bmP and speed bmV
    else if (key == "rosenthal") {
      ok = num(g.ros_eta) && num(g.ros_k) && num(g.ros_alpha) && g.ros_eta > 0 && g.ros_k > 0 && g.ros_alpha > 0;
      g.rosenthal = 1;
    }
    if (!ok) return fail(CAFE_E_ARG, "deck '%s': bad value after keyword '%s'", path, key.c_str());
    in >> kw;
  }
  // Grid.C:57-58 reads an uninitialised bmV for the bmDelT default and lrate
  // has no default: both must come from the deck.
  if (!g.set_bmdelt) return fail(CAFE_E_ARG, "deck '%s' must set bmDelT", path);
  if (!g.set_lrate) return fail(CAFE_E_ARG, "deck '%s' must set lrate", path);
  for (int k = 0; k < 3; ++k)
    if (g.nX[k] < 1) return fail(CAFE_E_ARG, "deck '%s': nX must be positive", path);
  if (!(g.dX[0] > 0) || !(g.bmDelT > 0) || !(g.bmV > 0) || !(g.bhatch > 0))
    return fail(CAFE_E_ARG, "deck '%s': dx, bmDelT, bmV and bhatch must be positive", path);
  if ((long long)g.nX[0] * g.nX[1] * g.nX[2] > 2000000000LL)
    return fail(CAFE_E_ARG, "deck '%s': more than 2e9 voxels", path);
  return CAFE_OK;
}

// The laser points rotated by the current gth (Grid.C:82-103).
void grid_rotate_points(GridH &g, bool init) {
  double gmid0 = g.LX[0] / 2., gmid1 = g.LX[1] / 2.;
  double xlmin = (g.LX[0] - g.gsize[0]) / 2., ylmin = (g.LX[1] - g.gsize[1]) / 2.;
  for (int j2 = 0; j2 < g.Ntd; ++j2)
    for (int j1 = 0; j1 < g.Nsd; ++j1) {
      int k = g.Nsd * j2 + j1;
      if (init) {
        g.lcoor[2 * k] = j1 * g.bmDelT * g.bmV + xlmin;
        g.lcoor[2 * k + 1] = j2 * g.bhatch + ylmin;
      }
      g.lcoor2[2 * k] = std::cos(g.gth) * (g.lcoor[2 * k] - gmid0) -
                        std::sin(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid0;
      g.lcoor2[2 * k + 1] = std::sin(g.gth) * (g.lcoor[2 * k] - gmid0) +
                            std::cos(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid1;
    }
}
void grid_laser_grid(GridH &g, bool init) {
  g.gth += g.gth0;
  grid_rotate_points(g, init);
}

// Grid constructor tail (Grid.C:69-108).
int grid_derive(GridH &g) {
  for (int k = 0; k < 3; ++k) g.LX[k] = g.nX[k] * g.dX[k];
  if (g.bpH < std::numeric_limits<double>::epsilon()) g.bpH = g.layerT;
  g.nZlayer = (int)std::round(g.layerT / g.dX[2]);
  if (g.nZlayer < 1) return fail(CAFE_E_ARG, "layer thickness below one voxel");
  g.Nzhg = std::min(g.nX[2], int(std::ceil(g.bpH * .9999 / g.dX[2])));
  g.indlayer = 1;
  g.ilaserLoc = g.Nzhg + g.indlayer * g.nZlayer;
  double ntd = std::ceil(g.gsize[1] / g.bhatch) + 1, nsd = std::ceil(g.gsize[0] / (g.bmV * g.bmDelT)) + 1;
  if (!(ntd * nsd < 2e9) || ntd < 1 || nsd < 1) return fail(CAFE_E_ARG, "laser grid too large");
  g.Ntd = (int)ntd;
  g.Nsd = (int)nsd;
  g.NpT = g.Nsd * g.Ntd;
  if (g.NpT < 2) return fail(CAFE_E_ARG, "laser grid has fewer than two points (set gridsize)");
  g.lcoor.assign(2 * (size_t)g.NpT, 0.);
  g.lcoor2.assign(2 * (size_t)g.NpT, 0.);
  grid_laser_grid(g, true);
  g.gbox[0] = -g.bhatch / 2.;
  g.gbox[1] = g.LX[0] + g.bhatch / 2.;
  g.gbox[2] = -g.bhatch / 2.;
  g.gbox[3] = g.LX[1] + g.bhatch / 2.;
  return CAFE_OK;
}

// Grid::UpdateLaser (Grid.C:110-164).
void grid_update_laser(GridH &g) {
  int itmp, iflg = 0, irep = 0;
  if (std::fmod(g.isp + 1, g.Nsd) == 0) g.inewscanflg = 1;
  if (g.isp == g.NpT - 1) {
    g.inewscanflg = 1;
    g.inewlayerflg = 1;
    g.isp = 0;
    g.indlayer += 1;
  }
  while (irep == 0 || g.isp == 0) {
    irep += 1;
    itmp = g.isp;
    if (g.inewscanflg == 0 && itmp < g.NpT - 1) {
      g.isp += 1;
    } else {
      while (itmp < g.NpT - 1 && iflg == 0) {
        itmp += 1;
        double x = g.lcoor2[2 * itmp], y = g.lcoor2[2 * itmp + 1];
        if (x > g.gbox[0] && x < g.gbox[1] && y > g.gbox[2] && y < g.gbox[3]) iflg = 1;
      }
      if (itmp < g.NpT - 1) {
        g.isp = itmp;
        g.inewscanflg = 0;
      } else {
        g.inewlayerflg = 1;
        g.inewscanflg = 1;
        g.indlayer += 1;
        g.ilaserLoc = g.Nzhg + g.indlayer * g.nZlayer;
        g.isp = 0;
        grid_laser_grid(g, false);
      }
    }
  }
  if (irep == 1) g.inewlayerflg = 0;
}

// ------------------------------------------------------------------ orientations (host)
struct OrientConsts {
  double R1, a, aprime, beta, s2, s2q, s6pi, spi, s24, coeffA[7];
};
OrientConsts orient_consts() {
  // SampleOrientation::SampleOrientation (SampleOrientation.C:10-23) and the
  // constant factors of ComputeMap2/3 (SampleOrientation.C:72-103).
  OrientConsts k;
  double r = 1;
  k.R1 = std::pow(3.0 * M_PI / 4.0, 1.0 / 3.0) * r;
  k.a = std::pow(2.0 * M_PI / 3.0, 1.0 / 2.0) * k.R1;
  k.aprime = std::pow(4.0 * M_PI / 3.0, 1.0 / 3.0) * k.R1;
  const double cA[7] = {-0.500009615, -0.024866061, -0.004549382, 0.000511867,
                        -0.001650083, 0.000759335,  -0.000204042};
  for (int j = 0; j < 7; ++j) k.coeffA[j] = cA[j];
  k.beta = std::pow(M_PI / 6.0, 1.0 / 2.0);
  k.s2 = std::pow(2.0, 1.0 / 2.0);
  k.s2q = std::pow(2.0, 1.0 / 4.0);
  k.s6pi = std::pow(6 / M_PI, 1.0 / 2.0);
  k.spi = std::pow(M_PI, 1.0 / 2.0);
  k.s24 = std::pow(24, 1.0 / 2.0);
  return k;
}

// SampleOrientation::GenerateSamples (SampleOrientation.C:124-161) with the
// host libm, for baseplate and powder-layer grains. As compiled, the
// reference evaluates ComputeMap3's pair pow(q, 1/2) as a square root.
void host_generate_samples(int n, unsigned int seedL, std::vector<double> &out) {
  static const OrientConsts K = orient_consts();
  std::uniform_real_distribution<double> xrand(0.0, 1.0);
  std::default_random_engine g1(seedL);
  out.assign(4 * (size_t)n, 0.0);
  for (int jn = 0; jn < n; ++jn) {
    double u0 = xrand(g1), u1 = xrand(g1), u2 = xrand(g1);
    double xyz0[3] = {u0 - .5, u1 - .5, u2 - .5};
    double xyz[3] = {K.aprime * xyz0[0], K.aprime * xyz0[1], K.aprime * xyz0[2]};
    int P[3] = {1, 2, 3};
    double x = xyz[0], y = xyz[1], z = xyz[2];
    if ((std::fabs(x) <= z) && (std::fabs(y) <= z)) { P[0] = 1; P[1] = 2; P[2] = 3; }
    if ((z <= -std::fabs(x)) && (z <= -std::fabs(y))) { P[0] = -1; P[1] = 2; P[2] = -3; }
    if ((std::fabs(x) <= y) && (std::fabs(z) <= y)) { P[0] = 1; P[1] = -3; P[2] = 2; }
    if ((y <= -std::fabs(x)) && (y <= -std::fabs(z))) { P[0] = 1; P[1] = 3; P[2] = -2; }
    if ((std::fabs(z) < x) && (std::fabs(y) <= x)) { P[0] = -3; P[1] = 2; P[2] = 1; }
    if ((x <= -std::fabs(z)) && (x <= -std::fabs(y))) { P[0] = 3; P[1] = 2; P[2] = -1; }
    double xyz2[3], m1[3], m2[3], m3[3], xyzb[3];
    for (int j = 0; j < 3; ++j) xyz2[j] = P[j] / std::abs(P[j]) * xyz[std::abs(P[j]) - 1];
    for (int j = 0; j < 3; ++j) m1[j] = K.a / K.aprime * xyz2[j];
    {
      double x1 = m1[0], y1 = m1[1], T1 = 0, T2 = 0;
      if (std::fabs(y1) <= std::fabs(x1)) {
        if (std::fabs(x1) >= 1e-10) {
          double cang = std::cos(y1 * M_PI / 12 / x1);
          T1 = K.s2 * cang - 1;
          T2 = K.s2 * std::sin(y1 * M_PI / 12 / x1);
          double f = K.s2q * x1 / (K.beta * std::pow(K.s2 - cang, 1.0 / 2.0));
          T1 *= f;
          T2 *= f;
        }
      }
      if (std::fabs(x1) <= std::fabs(y1)) {
        if (std::fabs(y1) < 1e-10) {
          T1 = 0.0;
          T2 = 0.0;
        } else {
          double cang = std::cos(x1 * M_PI / 12 / y1);
          T1 = K.s2 * std::sin(x1 * M_PI / 12 / y1);
          T2 = K.s2 * cang - 1;
          double f = K.s2q * y1 / (K.beta * std::pow(K.s2 - cang, 1.0 / 2.0));
          T1 *= f;
          T2 *= f;
        }
      }
      m2[0] = T1;
      m2[1] = T2;
      m2[2] = m1[2];
    }
    {
      double x2 = m2[0], y2 = m2[1], z2 = m2[2];
      if (std::fabs(z2) < 1e-10) {
        m3[0] = m3[1] = m3[2] = 0;
      } else {
        double q = 1 - (x2 * x2 + y2 * y2) * M_PI / (24 * (z2 * z2));
        double sq = std::sqrt(q);
        m3[0] = sq * x2;
        m3[1] = sq * y2;
        m3[2] = K.s6pi * z2 - (x2 * x2 + y2 * y2) * K.spi / (K.s24 * z2);
      }
    }
    for (int j = 0; j < 3; ++j) xyzb[std::abs(P[j]) - 1] = P[j] / std::abs(P[j]) * m3[j];
    double ax0 = std::fabs(xyz0[0]), ax1 = std::fabs(xyz0[1]), ax2 = std::fabs(xyz0[2]);
    double pmax = (ax0 < ax1) ? ax1 : ax0;
    pmax = (pmax < ax2) ? ax2 : pmax;
    double rhoP = K.R1 * pmax / .5;
    double t = 1;
    for (int j = 1; j < 8; ++j) t += K.coeffA[j - 1] * std::pow(rhoP, 2.0 * j);
    double omega = 2.0 * std::acos(t);
    double tnorm = std::pow(xyzb[0] * xyzb[0] + xyzb[1] * xyzb[1] + xyzb[2] * xyzb[2], .5);
    out[4 * (size_t)jn] = omega;
    out[4 * (size_t)jn + 1] = xyzb[0] / tnorm;
    out[4 * (size_t)jn + 2] = xyzb[1] / tnorm;
    out[4 * (size_t)jn + 3] = xyzb[2] / tnorm;
  }
}

// ------------------------------------------------------------------ device buffers
template <class T>
int dalloc(T **p, size_t n, std::vector<void *> &owned) {
  *p = nullptr;
  if (n == 0) n = 1;
  CUDA_TRY(cudaMalloc((void **)p, n * sizeof(T)));
  owned.push_back((void *)*p);
  return CAFE_OK;
}

}  // namespace

// Lets the other translation units of the library (cafe_noalloc.cu,
// cafe_batch.cu) report errors.
void cafe_internal_set_error(const char *msg) { g_last_error = msg ? msg : ""; }

// A realisation that shares the GPU with `share` - 1 others (cafe_batch.cu):
// its grid-stride launches are sized for its share of the SMs, and the
// active-set compaction takes four 8-cell chunks per thread. Neither changes
// results (every pass is order-preserving or element-wise). `graphs` = 0 keeps
// its steps out of CUDA graphs (when several host threads drive a batch, a
// capture in one thread must not meet another thread's device-wide calls).
void cafe_internal_set_share(cafe_sim *s, int share, int graphs);
// the batched step engine (end of this file), driven by cafe_batch.cu
struct CafeBatchEngine;
CafeBatchEngine *cafe_internal_batch_engine_create(cafe_sim *const *sims, int n, int tune, int *rc);
void cafe_internal_batch_engine_destroy(CafeBatchEngine *E);
int cafe_internal_batch_engine_step(CafeBatchEngine *E, int *phase, long long *steps, int *stepped);

struct cafe_sim {
  GridH g;
  int device = 0;
  cudaStream_t stream = nullptr;
  // TempField
  std::vector<int> ispvec;
  double DelT = 0;
  int tf_tInd = 0;
  // BasePlate / VoxelsCA host state
  int Nzh = 0, nlayerTot = 0, nGrain = 0;
  std::default_random_engine bp_generator;  // BasePlate.h:28 (default seed)
  std::default_random_engine genlayer;      // VoxelsCA.h:129
  bool initialized = false, begun = false, done = false;
  bool closed = false;  // the closing CleanLayer of main1.C:95 has been applied
  // cafe_sim_set_output: files of WriteToHDF1 written by the loop itself at
  // its output points, "<base><TempField::tInd>.h5" (main1.C:79-83, 97)
  std::string out_base;
  long long steps = 0;
  // device
  CafeConsts K;
  CafeDev D;
  CafeStepParams P;      // last temperature parameters
  CafeEasm E;            // EASM tables (K.easm)
  bool easm_cold = false;  // some cell below the liquidus after the last EASM field
  bool have_P = false;
  bool have_prev_box = false;
  int prev_lo[3] = {0, 0, 0}, prev_hi[3] = {0, 0, 0};
  bool full_k2 = false;   // next solid->mushy pass must scan the whole box
  int event_scan = 0;     // 1: evaluate every frontier row at every event
  bool event_helper = false;  // the event loop's new-row fills run in a second block
  std::vector<void *> owned;
  int *h_pinned = nullptr;  // pinned host mirror of ctr + err
  // staging for host transfers (allocated on first use)
  unsigned char *xfer = nullptr;
  int *d_bad = nullptr;
  // per-phase device timing (CUDA events on `stream`) and kernel-launch counts
  bool timing = false;
  cudaEvent_t marks[8] = {nullptr};
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pend;
  std::vector<cudaEvent_t> ev_pool;
  double phase_ms[CAFE_NPHASE] = {0};
  long long phase_launch[CAFE_NPHASE] = {0};
  long long launches = 0;
  long long nblk = 0;       // dense pass blocks
  long long nblk_act = 0;   // active-set compaction blocks
  int act_chunks = 1;       // 8-cell chunks per thread of the compaction
  long long nblk_pos = 0;   // position compaction blocks
  int nsm = 1;
  int gsm = 1;              // SMs that grid-stride launches are sized for (nsm, or a share in a batch)
  // output (SetBuild / WriteToHDF1)
  bool output_due = false;
  uint8_t *gflag = nullptr;   // per-grain flags of SetBuild
  long long gflag_cap = 0;
  unsigned char *h_out = nullptr;  // pinned bounce buffer of the file writer
  // the device work of a step as one CUDA graph (see step_graph_launch)
  bool use_graph = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<unsigned char> graph_key;
  long long graph_launch[CAFE_NPHASE] = {0};
  long long graph_captures = 0;
};

void cafe_internal_set_share(cafe_sim *s, int share, int graphs) {
  if (!s || share < 1) return;
  s->use_graph = graphs != 0;
  s->gsm = std::max(4, s->nsm / share);
  s->act_chunks = CAFE_ACT_MAX_CHUNKS;
  long long per_block = (long long)CAFE_CELLS_PER_BLOCK * s->act_chunks;
  s->nblk_act = (s->K.N + per_block - 1) / per_block;
}

namespace {

cudaEvent_t ev_get(cafe_sim *s) {
  if (!s->ev_pool.empty()) {
    cudaEvent_t e = s->ev_pool.back();
    s->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
void resolve_phases(cafe_sim *s) {
  for (auto &p : s->pend) {
    float ms = 0.f;
    cudaEventSynchronize(p.second.second);
    cudaEventElapsedTime(&ms, p.second.first, p.second.second);
    s->phase_ms[p.first] += ms;
    s->ev_pool.push_back(p.second.first);
    s->ev_pool.push_back(p.second.second);
  }
  s->pend.clear();
}
// Brackets a group of launches of phase `ph`.
struct PhaseScope {
  cafe_sim *s;
  int ph;
  cudaEvent_t a = nullptr;
  PhaseScope(cafe_sim *s_, int ph_) : s(s_), ph(ph_) {
    if (s->timing) {
      a = ev_get(s);
      cudaEventRecord(a, s->stream);
    }
  }
  ~PhaseScope() {
    if (s->timing) {
      cudaEvent_t b = ev_get(s);
      cudaEventRecord(b, s->stream);
      s->pend.push_back({ph, {a, b}});
      if (s->pend.size() > 4096) resolve_phases(s);
    }
  }
};
#define LAUNCHED(ph, n)          \
  do {                            \
    s->launches += (n);           \
    s->phase_launch[ph] += (n);   \
  } while (0)

int sim_sync(cafe_sim *s) {
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  CUDA_TRY(cudaMemcpy(s->h_pinned, s->D.err, sizeof(int), cudaMemcpyDeviceToHost));
  int err = s->h_pinned[0];
  if (err) {
    return fail(CAFE_E_CAPACITY,
                "device capacity exceeded (flags 0x%x: 1 active list, 2 frontier rows, 4 grain "
                "table, 8 mushy list, 16 event cap; 32: the event loop's two blocks timed out "
                "waiting for each other); recreate with larger capacities",
                err);
  }
  return CAFE_OK;
}

int read_ctr(cafe_sim *s, int which, int *out) {
  CUDA_TRY(cudaMemcpyAsync(s->h_pinned + 1, s->D.ctr + which, sizeof(int), cudaMemcpyDeviceToHost,
                           s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  *out = s->h_pinned[1];
  return CAFE_OK;
}

// The next step's active-set compaction scans every z plane (after a state
// that no step produced: initialisation, upload, restore).
int full_active_range(cafe_sim *s) {
  k_set_int<<<1, 1, 0, s->stream>>>(s->D.ctr + CTR_ZLO, 0);
  k_set_int<<<1, 1, 0, s->stream>>>(s->D.ctr + CTR_ZHI, s->K.nz - 1);
  CUDA_TRY(cudaGetLastError());
  return CAFE_OK;
}

int grow_grains(cafe_sim *s, long long need) {
  if (need <= s->D.grain_cap) return CAFE_OK;
  long long cap = std::max<long long>(need * 2, (long long)s->D.grain_cap * 2);
  double *cth = nullptr, *rot = nullptr;
  CUDA_TRY(cudaMalloc((void **)&cth, cap * 4 * sizeof(double)));
  CUDA_TRY(cudaMalloc((void **)&rot, cap * 9 * sizeof(double)));
  CUDA_TRY(cudaMemcpyAsync(cth, s->D.cth, (size_t)s->D.grain_cap * 4 * sizeof(double),
                           cudaMemcpyDeviceToDevice, s->stream));
  CUDA_TRY(cudaMemcpyAsync(rot, s->D.rot, (size_t)s->D.grain_cap * 9 * sizeof(double),
                           cudaMemcpyDeviceToDevice, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  for (auto &p : s->owned) {
    if (p == (void *)s->D.cth) { cudaFree(p); p = (void *)cth; }
    else if (p == (void *)s->D.rot) { cudaFree(p); p = (void *)rot; }
  }
  s->D.cth = cth;
  s->D.rot = rot;
  s->D.grain_cap = (int)std::min<long long>(cap, 2000000000LL);
  return CAFE_OK;
}

// Bucket grid over Voronoi sites (CSR, ascending site index in each bucket).
struct HostSiteGrid {
  std::vector<int32_t> start, idx;
  double lo[3], h;
  int nb[3];
};
void build_site_grid(HostSiteGrid &G, const std::vector<double> &xyz, const double lo[3],
                     const double hi[3]) {
  int n = (int)(xyz.size() / 3);
  double vol = 1.0;
  for (int a = 0; a < 3; ++a) vol *= std::max(hi[a] - lo[a], 1e-300);
  G.h = std::cbrt(vol / std::max(1, n)) * 1.5;
  for (int a = 0; a < 3; ++a) {
    G.lo[a] = lo[a];
    G.nb[a] = std::max(1, std::min(512, (int)std::ceil((hi[a] - lo[a]) / G.h)));
  }
  // enlarge h if the bucket count per axis was clipped
  for (int a = 0; a < 3; ++a) G.h = std::max(G.h, (hi[a] - lo[a]) / G.nb[a] * (1 + 1e-12));
  size_t nbt = (size_t)G.nb[0] * G.nb[1] * G.nb[2];
  std::vector<int32_t> cnt(nbt + 1, 0), cell(n);
  for (int i = 0; i < n; ++i) {
    int b[3];
    for (int a = 0; a < 3; ++a) {
      double f = std::floor((xyz[3 * (size_t)i + a] - G.lo[a]) / G.h);
      b[a] = f < 0 ? 0 : (f > G.nb[a] - 1 ? G.nb[a] - 1 : (int)f);
    }
    cell[i] = (b[2] * G.nb[1] + b[1]) * G.nb[0] + b[0];
    cnt[cell[i] + 1]++;
  }
  for (size_t b = 0; b < nbt; ++b) cnt[b + 1] += cnt[b];
  G.start = cnt;
  G.idx.assign(n, 0);
  std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n; ++i) G.idx[fill[cell[i]]++] = i;
}

// Uploads sites + grid; returns the device view. Buffers are freed by the caller.
int upload_site_grid(cafe_sim *s, const std::vector<double> &xyz, const HostSiteGrid &G,
                     CafeSiteGrid &dv, std::vector<void *> &tmp) {
  double *dxyz;
  int32_t *dstart, *didx;
  CUDA_TRY(cudaMalloc((void **)&dxyz, std::max<size_t>(1, xyz.size()) * sizeof(double)));
  tmp.push_back(dxyz);
  CUDA_TRY(cudaMalloc((void **)&dstart, G.start.size() * sizeof(int32_t)));
  tmp.push_back(dstart);
  CUDA_TRY(cudaMalloc((void **)&didx, std::max<size_t>(1, G.idx.size()) * sizeof(int32_t)));
  tmp.push_back(didx);
  CUDA_TRY(cudaMemcpyAsync(dxyz, xyz.data(), xyz.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaMemcpyAsync(dstart, G.start.data(), G.start.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaMemcpyAsync(didx, G.idx.data(), G.idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s->stream));
  dv.xyz = dxyz;
  dv.start = dstart;
  dv.idx = didx;
  for (int a = 0; a < 3; ++a) {
    dv.lo[a] = G.lo[a];
    dv.nb[a] = G.nb[a];
  }
  dv.h = G.h;
  return CAFE_OK;
}

void free_tmp(cafe_sim *s, std::vector<void *> &tmp) {
  cudaStreamSynchronize(s->stream);
  for (void *p : tmp) cudaFree(p);
  tmp.clear();
}

int grid_blocks(long long work, int threads, cafe_sim *s) {
  long long b = (work + threads - 1) / threads;
  long long cap = (long long)s->gsm * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// Per-step temperature parameters (TempField.C:145-171) and the cell box
// outside which no cell can reach the liquidus.
void make_step_params(cafe_sim *s, CafeStepParams &P) {
  GridH &g = s->g;
  const int *isv = s->ispvec.data();
  P.lx = g.lcoor[2 * isv[g.isp]] - g.offset[0];
  P.ly = g.lcoor[2 * isv[g.isp] + 1] - g.offset[1];
  P.lz = g.ilaserLoc * g.dX[2] - g.offset[2];
  P.cg = std::cos(g.gth);
  P.sg = std::sin(g.gth);
  if (std::fmod(g.isp, g.Nsd) == 0)
    P.dirp = (g.lcoor[2 * isv[g.isp + 1]] - g.lcoor[2 * isv[g.isp]]);
  else
    P.dirp = (g.lcoor[2 * isv[g.isp]] - g.lcoor[2 * isv[g.isp - 1]]);
  P.ilaserLoc = g.ilaserLoc;
  P.tInd = g.tInd;
  const CafeConsts &K = s->K;
  P.any_hot_full = !(K.tS < K.tL) || !(K.T0 < K.tL);
  // half extents of the hot region in the laser frame, with a relative margin
  double A = std::max(K.bmDX0, K.a1[3]) * (1 + 1e-9);
  double B = std::max(K.a1[1], K.a1[4]) * (1 + 1e-9);
  double C = std::max(K.a1[2], K.a1[5]) * (1 + 1e-9);
  double c = std::fabs(P.cg), sn = std::fabs(P.sg);
  double hx = c * A + sn * B, hy = sn * A + c * B;
  // pool centre in the voxel frame: inverse rotation of the laser position
  double u = P.lx - K.hLX0, w = P.ly - K.hLX1;
  double X = P.cg * u - P.sg * w + K.hLX0, Y = P.sg * u + P.cg * w + K.hLX1;
  double lo[3] = {X - hx, Y - hy, P.lz - C}, hi[3] = {X + hx, Y + hy, P.lz + C};
  int nmax[3] = {g.nX[0], g.nX[1], g.nX[2]};
  for (int a = 0; a < 3; ++a) {
    double l = std::floor(lo[a] / g.dX[a] - 0.5) - 2, h = std::ceil(hi[a] / g.dX[a] - 0.5) + 3;
    if (!(l == l) || !(h == h)) { l = 0; h = nmax[a]; }
    l = std::max(0.0, std::min((double)nmax[a], l));
    h = std::max(0.0, std::min((double)nmax[a], h));
    P.lo[a] = (int)l;
    P.hi[a] = std::max((int)h, (int)l);
  }
  if (P.any_hot_full) {
    for (int a = 0; a < 3; ++a) {
      P.lo[a] = 0;
      P.hi[a] = nmax[a];
    }
  }
  // first z index whose cell centre lies above the laser plane (TempField.C:162)
  int kab = 0;
  while (kab < g.nX[2] && !(((double)kab + .5) * g.dX[2] > P.lz)) ++kab;
  P.kabove = kab;
  for (int a = 0; a < 3; ++a) {
    P.plo[a] = s->have_prev_box ? s->prev_lo[a] : 0;
    P.phi[a] = s->have_prev_box ? s->prev_hi[a] : 0;
  }
}

// TempField::EASM over the cells below the laser plane; the step's box becomes
// the box of the cells at or above the liquidus.
int easm_field(cafe_sim *s) {
  CafeStepParams &P = s->P;
  const CafeConsts &K = s->K;
  P.any_hot_full = 0;
  long long ncell = std::min<long long>(K.N, (long long)P.kabove * K.nxy);
  {
    PhaseScope ps(s, CAFE_PH_MELT);
    k_easm_reset<<<1, 32, 0, s->stream>>>(s->D);
    if (K.tmodel == 2) {
      if (ncell > 0)
        k_rosenthal<<<grid_blocks(ncell, 256, s), 256, 0, s->stream>>>(s->D, K, P, ncell);
      LAUNCHED(CAFE_PH_MELT, 2);
    } else {
      if (ncell > 0) {  // persistent: a few blocks per SM pull cells from a cursor
        k_easm<<<(int)std::min<long long>((ncell + 255) / 256, (long long)s->nsm * 3), 256, 0, s->stream>>>(
            s->D, K, P, s->E, ncell);
        k_easm_long<<<s->nsm * 3, 256, 0, s->stream>>>(s->D, K, P, s->E);
      }
      LAUNCHED(CAFE_PH_MELT, 3);
    }
  }
  CUDA_TRY(cudaGetLastError());
  int *h = s->h_pinned + 8;  // 7 ints: box lo, box hi, cold
  CUDA_TRY(cudaMemcpyAsync(h, s->D.ctr + CTR_EASM_BOX, 7 * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->easm_cold = h[6] != 0;
  if (h[3] < 0) {
    for (int a = 0; a < 3; ++a) P.lo[a] = P.hi[a] = 0;
  } else {
    for (int a = 0; a < 3; ++a) {
      P.lo[a] = h[a];
      P.hi[a] = h[3 + a] + 1;
    }
  }
  return CAFE_OK;
}

// ---- the device work of one step
// TempField::tInd (main1.C:64), the step parameters on the host and in device
// memory, the EASM field when selected, and the class-map capacity.
int step_plan(cafe_sim *s);

int step_prepare(cafe_sim *s) {
  int rc = step_plan(s);
  if (rc) return rc;
  k_put_params<<<1, 1, 0, s->stream>>>(s->D.Pd, s->P);
  LAUNCHED(CAFE_PH_MELT, 1);
  CUDA_TRY(cudaGetLastError());
  return CAFE_OK;
}

// The host part of a step's preparation: TempField::tInd, the parameters into
// s->P, the EASM field when selected, and the class-map capacity for the pool
// box (regrown only for the EASM field; the analytic pool box fits the map
// sized at creation).
int step_plan(cafe_sim *s) {
  GridH &g = s->g;
  s->tf_tInd = int(std::round(g.time / s->DelT));
  if (g.isp < 0 || g.isp >= g.NpT || (std::fmod(g.isp, g.Nsd) == 0 && g.isp + 1 >= g.NpT) ||
      (std::fmod(g.isp, g.Nsd) != 0 && g.isp < 1))
    return fail(CAFE_E_STATE, "laser index %d outside the scan grid", g.isp);
  make_step_params(s, s->P);
  s->have_P = true;
  if (s->K.easm) {
    int rc = easm_field(s);
    if (rc) return rc;
  }
  const CafeStepParams &P = s->P;
  long long nbox = (long long)(P.hi[0] - P.lo[0]) * (P.hi[1] - P.lo[1]) * (P.hi[2] - P.lo[2]);
  if (nbox > s->D.tcls_cap) {
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (auto &p : s->owned)
      if (p == (void *)s->D.tcls) {
        cudaFree(p);
        p = nullptr;
      }
    long long cap = std::max<long long>(nbox, 2 * s->D.tcls_cap);
    cap = std::min<long long>(cap, s->K.N);
    CUDA_TRY(cudaMalloc((void **)&s->D.tcls, cap));
    s->owned.push_back(s->D.tcls);
    s->D.tcls_cap = cap;
  }
  return CAFE_OK;
}

// SetLiquid3 + BuildjID + the class map over the pool box (k_melt). In a
// graph the grid is fixed (the kernel strides over the box it reads).
int launch_melt(cafe_sim *s, bool graph, const CafeStepParams *Pp) {
  const CafeStepParams &P = s->P;
  CUDA_TRY(cudaMemsetAsync(s->D.ctr + CTR_HOT, 0, sizeof(int), s->stream));
  long long nbox = (long long)(P.hi[0] - P.lo[0]) * (P.hi[1] - P.lo[1]) * (P.hi[2] - P.lo[2]);
  if (graph || nbox > 0) {
    PhaseScope ps(s, CAFE_PH_MELT);
    if (s->K.easm)
      k_melt_easm<<<grid_blocks(nbox, 256, s), 256, 0, s->stream>>>(s->D, s->K, P);
    else
      k_melt<<<graph ? s->gsm * 16 : grid_blocks(nbox, 256, s), 256, 0, s->stream>>>(s->D, s->K, Pp);
    LAUNCHED(CAFE_PH_MELT, 1);
  }
  CUDA_TRY(cudaGetLastError());
  return CAFE_OK;
}

// End-of-scan check of TempField (TempField.C:199-216), only when the laser is
// outside the grid box: host flags from "some cell at the liquidus" (read from
// the device, or `hot_known` when the caller has read it already).
int end_of_scan(cafe_sim *s, const int *hot_known = nullptr) {
  GridH &g = s->g;
  const CafeStepParams &P = s->P;
  const int *isv = s->ispvec.data();
  double x = g.lcoor2[2 * isv[g.isp]] - g.offset[0];
  double y = g.lcoor2[2 * isv[g.isp] + 1] - g.offset[1];
  if (x < g.gbox[0] || x > g.gbox[1] || y < g.gbox[2] || y > g.gbox[3]) {
    int hot = 0;
    if (s->K.tmodel == 1) {
      // TempField::EASM asks all_of(T >= tL) (TempField.C:123-125); cells
      // above the laser plane hold T = 0
      hot = (P.kabove >= g.nX[2] && !s->easm_cold) ? 1 : 0;
    } else if (hot_known) {
      hot = *hot_known;
    } else {
      int rc = read_ctr(s, CTR_HOT, &hot);
      if (rc) return rc;
    }
    if (hot == 0 || std::fmod(g.isp + 1, g.Nsd) == 0) g.inewscanflg = 1;
    if (g.isp == g.NpT - 1) {
      g.inewscanflg = 1;
      g.inewlayerflg = 1;
      g.isp = 0;
      g.indlayer += 1;
    }
  }
  return CAFE_OK;
}

// The event loop: one block, or with the fill helper two blocks launched
// cooperatively (both resident at once, which the hand-off between them
// needs). The hand-off's sequence words start at zero.
int launch_event_loop(cafe_sim *s, const CafeStepParams *Pp) {
  cudaStream_t st = s->stream;
  const CafeDev &D = s->D;
  const long long max_ev = D.act_cap + 1;
  const int allow_fast = s->event_scan ? 0 : 1;
  if (!s->event_helper) {
    k_event_loop<<<1, CAFE_LOOP_THREADS, 0, st>>>(s->D, s->K, Pp, max_ev, allow_fast);
    CUDA_TRY(cudaGetLastError());
    return CAFE_OK;
  }
  CUDA_TRY(cudaMemsetAsync(D.fill_seq, 0, 2 * sizeof(int), st));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2);
  cfg.blockDim = dim3(CAFE_LOOP_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CUDA_TRY(cudaLaunchKernelEx(&cfg, k_event_loop, s->D, s->K, Pp, max_ev, allow_fast));
  return CAFE_OK;
}

// VoxelsCA::UpdateVoxels on the device (no host synchronisation). In a graph
// the box kernels get fixed grids and read their boxes from the parameters.
int launch_voxels(cafe_sim *s, bool graph, const CafeStepParams *Pp) {
  CafeDev &D = s->D;
  const CafeConsts &K = s->K;
  const CafeStepParams &P = s->P;
  cudaStream_t st = s->stream;
  int nb = (int)s->nblk;
  {
    PhaseScope ps(s, CAFE_PH_CLASSIFY);
    if (s->full_k2) {
      k_solid2mushy_dense<<<nb, CAFE_DENSE_THREADS, 0, st>>>(D, K);
      LAUNCHED(CAFE_PH_CLASSIFY, 1);
      s->full_k2 = false;
    } else {
      long long vb = (long long)(P.hi[0] - P.lo[0] + 2) * (P.hi[1] - P.lo[1] + 2) * (P.hi[2] - P.lo[2] + 2);
      k_solid2mushy_pbox<<<graph ? s->gsm * 16 : grid_blocks(vb, 256, s), 256, 0, st>>>(D, K, Pp, 0);
      LAUNCHED(CAFE_PH_CLASSIFY, 1);
      long long pb = (long long)(P.phi[0] - P.plo[0] + 2) * (P.phi[1] - P.plo[1] + 2) * (P.phi[2] - P.plo[2] + 2);
      if (graph || (P.phi[0] > P.plo[0] && P.phi[1] > P.plo[1] && P.phi[2] > P.plo[2])) {
        k_solid2mushy_pbox<<<graph ? s->gsm * 16 : grid_blocks(pb, 256, s), 256, 0, st>>>(D, K, Pp, 1);
        LAUNCHED(CAFE_PH_CLASSIFY, 1);
      }
      k_solid2mushy_list<<<s->gsm * 4, 256, 0, st>>>(D, K);
      LAUNCHED(CAFE_PH_CLASSIFY, 1);
    }
    CUDA_TRY(cudaMemsetAsync(D.ctr + CTR_NLIQ, 0, sizeof(int), st));
    const int ab = (int)std::min<long long>(s->nblk_act, (long long)s->gsm * 8);  // persistent grid
    k_active_count<<<ab, CAFE_DENSE_THREADS, 0, st>>>(D, K, Pp, s->act_chunks, s->nblk_act);
    k_scan_blocks<<<1, 1024, 0, st>>>(D.blk, s->nblk_act, D.ctr + CTR_NA);
    k_active_scatter<<<ab, CAFE_DENSE_THREADS, 0, st>>>(D, K, Pp, s->act_chunks, s->nblk_act);
    LAUNCHED(CAFE_PH_CLASSIFY, 3);
  }
  int gb = s->gsm * 8;
  {
    PhaseScope ps(s, CAFE_PH_GATHER);
    k_gather<<<gb, 256, 0, st>>>(D, K, Pp);
    int nbp = (int)s->nblk_pos;
    k_lists_count<<<nbp, CAFE_DENSE_THREADS, 0, st>>>(D);
    k_scan_pairs<<<1, 1024, 0, st>>>(D.blk, s->nblk_pos, D.ctr + CTR_NA, D.ctr + CTR_NVS2, D.ctr + CTR_NROWS);
    k_lists_scatter<<<nbp, CAFE_DENSE_THREADS, 0, st>>>(D);
    if (K.easm)  // rows grow with per-cell velocities: the exact per-event scan
      k_set_int<<<1, 1, 0, st>>>(D.ctr + CTR_SLOW, 1);
    else
      CUDA_TRY(cudaMemsetAsync(D.ctr + CTR_SLOW, 0, sizeof(int), st));
    CUDA_TRY(cudaMemsetAsync(D.ctr + CTR_NPAIRS, 0, sizeof(int), st));
    k_rows_prep<<<s->gsm * 4, 256, 0, st>>>(D, K);
    k_rows_geo<<<s->gsm * 8, 256, 0, st>>>(D, K);
    k_rows_order<<<s->gsm * 4, 256, 0, st>>>(D, K);
    LAUNCHED(CAFE_PH_GATHER, 7);
  }
  {
    PhaseScope ps(s, CAFE_PH_EVENTS);
    int rc = launch_event_loop(s, Pp);
    if (rc) return rc;
    if (D.glog_cell) {
      k_glog_begin<<<s->gsm * 4, 256, 0, st>>>(D, Pp);
      LAUNCHED(CAFE_PH_EVENTS, 1);
    }
    k_rows_finalize<<<s->gsm * 4, 256, 0, st>>>(D);
    LAUNCHED(CAFE_PH_EVENTS, 2);
    if (D.glog_cell) {
      k_glog_end<<<s->gsm * 4, 256, 0, st>>>(D, K);
      k_glog_advance<<<1, 1, 0, st>>>(D);
      LAUNCHED(CAFE_PH_EVENTS, 2);
    }
  }
  {
    PhaseScope ps(s, CAFE_PH_WRITEBACK);
    k_writeback<<<gb, 256, 0, st>>>(D, K);
    k_mushy2solid<<<gb, 256, 0, st>>>(D, K);
    LAUNCHED(CAFE_PH_WRITEBACK, 2);
  }
  CUDA_TRY(cudaGetLastError());
  return CAFE_OK;
}

void voxels_done(cafe_sim *s) {
  const CafeStepParams &P = s->P;
  for (int a = 0; a < 3; ++a) {
    s->prev_lo[a] = P.lo[a];
    s->prev_hi[a] = P.hi[a];
  }
  s->have_prev_box = true;
}

// Everything the captured launches depend on besides the step parameters
// (which they read from device memory): device pointers, constants, launch
// shapes. A change (a regrown buffer, a new grain table) forces a new capture.
std::vector<unsigned char> graph_key(const cafe_sim *s) {
  std::vector<unsigned char> k(sizeof(CafeDev) + sizeof(CafeConsts) + 8 * sizeof(long long));
  unsigned char *p = k.data();
  std::memcpy(p, &s->D, sizeof(CafeDev));
  p += sizeof(CafeDev);
  std::memcpy(p, &s->K, sizeof(CafeConsts));
  p += sizeof(CafeConsts);
  long long v[8] = {s->gsm, s->act_chunks, s->nblk, s->nblk_act, s->nblk_pos, s->event_scan, s->nsm, 0};
  std::memcpy(p, v, sizeof v);
  return k;
}

// The melt pass and UpdateVoxels of a step as one graph launch (the kernels
// read the step's parameters from D.Pd): captured once per handle (again
// whenever graph_key changes) and replayed, so that a step costs two host
// launches (k_put_params and the graph) instead of about twenty-five API
// calls. Used when no phase timing is asked for, the temperature is analytic
// and no dense solid->mushy pass is due. (Graphs of several consecutive steps
// were measured slower on the device than one graph per step.)
int step_graph_launch(cafe_sim *s) {
  std::vector<unsigned char> key = graph_key(s);
  if (!s->graph_exec || key != s->graph_key) {
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->graph_exec = nullptr;
    s->graph = nullptr;
    long long before[CAFE_NPHASE];
    for (int p = 0; p < CAFE_NPHASE; ++p) before[p] = s->phase_launch[p];
    long long tot0 = s->launches;
    CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = launch_melt(s, true, s->D.Pd);
    if (!rc) rc = launch_voxels(s, true, s->D.Pd);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
    // the capture only recorded the launches: take back their counts
    for (int p = 0; p < CAFE_NPHASE; ++p) {
      s->graph_launch[p] = s->phase_launch[p] - before[p];
      s->phase_launch[p] = before[p];
    }
    s->launches = tot0;
    if (rc || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (rc) return rc;
      return fail(CAFE_E_CUDA, "step graph capture: %s", cudaGetErrorString(ce));
    }
    s->graph = g;
    CUDA_TRY(cudaGraphInstantiate(&s->graph_exec, g, 0));
    s->graph_key = key;
    s->graph_captures++;
  }
  CUDA_TRY(cudaGraphLaunch(s->graph_exec, s->stream));
  for (int p = 0; p < CAFE_NPHASE; ++p) {
    s->phase_launch[p] += s->graph_launch[p];
    s->launches += s->graph_launch[p];
  }
  return CAFE_OK;
}

bool graph_eligible(const cafe_sim *s) { return s->use_graph && !s->timing && !s->K.easm && !s->full_k2; }

// The rest of a loop iteration after its device work (main1.C:72-93).
int finish_after_laser(cafe_sim *s, bool bcheck, int *done) {
  int rc;
  if (s->g.inewlayerflg == 1 && (rc = cafe_sim_clean_layer(s))) return rc;
  // output point (main1.C:77-84): SetBuild; WriteToHDF1 is the caller's
  const GridH &g = s->g;
  s->output_due = (g.outint > 0 && s->tf_tInd % g.outint == 0) || bcheck || (g.inewlayerflg == 1 && g.outNL == 0);
  if (s->output_due && (rc = cafe_sim_set_build(s))) return rc;
  if (s->output_due && !s->out_base.empty()) {
    // WriteToHDF1 before UpdateTime2 and AddLayer1, as main1.C:79-88 orders them
    std::string name = s->out_base + std::to_string(s->tf_tInd) + ".h5";
    if ((rc = cafe_sim_write_output(s, name.c_str()))) return rc;
  }
  cafe_sim_update_time(s);
  if (s->g.inewlayerflg == 1 && (rc = cafe_sim_add_layer(s))) return rc;
  s->steps++;
  if (bcheck) s->done = true;
  if (done) *done = s->done ? 1 : 0;
  return CAFE_OK;
}
int finish_step(cafe_sim *s, int *done) {
  grid_update_laser(s->g);
  return finish_after_laser(s, s->g.indlayer > s->nlayerTot, done);
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

const char *cafe_last_error(void) { return g_last_error.c_str(); }

int cafe_sim_create(const char *deck_path, const cafe_options *opt, cafe_sim **out) {
  if (!deck_path || !out) return fail(CAFE_E_ARG, "null argument");
  *out = nullptr;
  cafe_sim *s = new cafe_sim();
  int rc = parse_deck(deck_path, s->g);
  if (!rc) rc = grid_derive(s->g);
  if (rc) {
    delete s;
    return rc;
  }
  GridH &g = s->g;
  s->device = opt ? opt->device : 0;
  s->event_scan = opt ? opt->event_scan : 0;
  s->event_helper = opt && opt->event_fill_helper;
  cudaError_t ce = cudaSetDevice(s->device);
  if (ce != cudaSuccess) {
    delete s;
    return fail(CAFE_E_CUDA, "cudaSetDevice(%d): %s", opt ? opt->device : 0, cudaGetErrorString(ce));
  }
  cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, s->device);
  {
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, s->device);
    if (!coop || s->nsm < 2) s->event_helper = false;
  }
  s->gsm = s->nsm;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return fail(CAFE_E_CUDA, "cudaStreamCreate failed");
  }
  // TempField (TempField.C:26-50)
  s->DelT = g.bmDelT;
  s->ispvec.assign(g.NpT, 0);
  if (g.patternID == 1 || g.patternID == 3) std::iota(s->ispvec.begin(), s->ispvec.end(), 0);
  if (g.patternID == 2 || g.patternID == 4) {
    for (int j = 0; j < g.Ntd; ++j) {
      int k = g.Nsd * j;
      if (std::fmod(j, 2) == 0)
        std::iota(s->ispvec.begin() + k, s->ispvec.begin() + k + g.Nsd, k);
      else
        for (int j1 = 0; j1 < g.Nsd; ++j1) s->ispvec[k + j1] = k + g.Nsd - 1 - j1;
    }
  }
  // BasePlate (BasePlate.C:20-30), main1.C:59
  s->Nzh = std::min(g.nX[2], int(std::ceil(g.bpH * .9999 / g.dX[2])));
  s->nlayerTot = int(std::ceil((double)(g.nX[2] - s->Nzh) / (double)g.nZlayer));
  const unsigned int seed0 = (unsigned int)kSeed0 + (unsigned int)(g.seed - 1) * kSeedStride;
  const unsigned int seed1 = (unsigned int)kSeed1 + (unsigned int)(g.seed - 1) * kSeedStride;
  s->genlayer.seed(seed1);
  s->bp_generator.seed((unsigned int)g.seed);
  // constants
  CafeConsts &K = s->K;
  K.nx = g.nX[0];
  K.ny = g.nX[1];
  K.nz = g.nX[2];
  K.nxy = K.nx * K.ny;
  K.N = (long long)K.nxy * K.nz;
  for (int a = 0; a < 3; ++a) K.dx[a] = g.dX[a];
  K.hLX0 = g.LX[0] / 2.;
  K.hLX1 = g.LX[1] / 2.;
  K.a1[0] = g.meltparam[0];
  K.a1[1] = g.meltparam[2];
  K.a1[2] = g.meltparam[3];
  K.a1[3] = g.meltparam[1];
  K.a1[4] = K.a1[1];
  K.a1[5] = K.a1[2];
  K.bmDX0 = s->DelT * g.bmV;
  K.tL = g.tL;
  K.tS = g.tS;
  K.T0 = g.T0;
  K.xi = g.tL * (1 + std::numeric_limits<double>::epsilon());
  K.Tcls[0] = g.T0;
  K.Tcls[1] = g.tS;
  K.Tcls[2] = K.xi;
  for (int c = 0; c < 3; ++c) {
    double T = K.Tcls[c];
    K.hot_cls[c] = T >= g.tL;
    K.gt_cls[c] = T > g.tL;
    K.vhat_cls[c] = T >= g.tL ? 0.0 : g.Avel * std::pow(g.tL - T, g.nvel);
  }
  K.nuc_gauss = g.nuc_gauss;
  K.nuc_mean = g.nuc_mean;
  K.nuc_sd = g.nuc_sd;
  if (g.EASM_Flag == 1 && g.rosenthal) {
    cafe_sim_destroy(s);
    return fail(CAFE_E_ARG, "a deck selects either the EASM or the Rosenthal temperature, not both");
  }
  K.tmodel = g.EASM_Flag == 1 ? 1 : (g.rosenthal ? 2 : 0);
  K.easm = K.tmodel != 0;
  K.Avel = g.Avel;
  K.nvel_i = 0;
  {
    const double pi = 3.14159265358979323846;
    K.ros_q = g.ros_eta * g.bmP / (2.0 * pi * g.ros_k);
    K.ros_c = g.bmV / (2.0 * g.ros_alpha);
    K.ros_rmin = 0.5 * std::min(g.dX[0], std::min(g.dX[1], g.dX[2]));
  }
  if (K.easm) {
    // per-cell velocities Avel pow(tL - T, nvel) are evaluated on the device
    // as correctly rounded integer powers
    if (!(g.nvel >= 1 && g.nvel <= 64 && g.nvel == (double)(int)g.nvel)) {
      cafe_sim_destroy(s);
      return fail(CAFE_E_ARG, "EASM and Rosenthal temperatures need an integer growth exponent in 1..64 "
                              "(dendritegrowth2)");
    }
    K.nvel_i = (int)g.nvel;
  }
  if (K.tmodel == 1) {
    CafeEasm &E = s->E;
    const double t = 80.0e-5;
    cafe_gauss_legendre(CAFE_EASM_NODES, 0.0, t, E.qx, E.qw);
    for (int i = 0; i < CAFE_EASM_NODES; ++i) {
      E.tx[i] = t - E.qx[i];
      E.r[i] = crm_pow_mhalf(E.tx[i]);
    }
    E.bmV = g.bmV;  // Utilities::InitializeUT (Utilities.C:143-146)
    E.Q = g.bmP;
    E.layerT = g.layerT;
  }
  K.rX = g.rNmax * std::pow(g.dX[0] * 1e6, 3.);
  K.DelT = s->DelT;
  K.ruq_dx = g.dX[0];
  K.seed0 = seed0;
  K.seed1 = seed1;
  OrientConsts oc = orient_consts();
  K.so_R1 = oc.R1;
  K.so_a = oc.a;
  K.so_aprime = oc.aprime;
  K.so_beta = oc.beta;
  K.so_s2 = oc.s2;
  K.so_s2q = oc.s2q;
  K.so_s6pi = oc.s6pi;
  K.so_spi = oc.spi;
  K.so_s24 = oc.s24;
  for (int j = 0; j < 7; ++j) K.so_coeffA[j] = oc.coeffA[j];
  K.s3 = std::pow(3.0, .5);
  K.s23 = std::pow(2.0 / 3.0, .5);
  // device buffers
  CafeDev &D = s->D;
  std::memset(&D, 0, sizeof D);
  long long N = K.N;
  long long acap = opt && opt->active_capacity > 0 ? opt->active_capacity
                                                   : std::min<long long>(N, std::max<long long>(1 << 20, N / 4));
  acap = std::min<long long>(acap, N);
  D.act_cap = acap;
  D.vs2_cap = acap;
  // frontier rows (mushy cells with a liquid neighbour): a thin shell around
  // the pool, far smaller than the active list; an explicit active capacity
  // raises this limit with it
  D.row_cap = std::min<long long>(acap, opt && opt->active_capacity > 0 ? (1LL << 22) : (1LL << 20));
  D.ev_cap = acap + 2;  // an event captures or nucleates one active cell
  double est = g.mu * (g.dX[0] * 1e6) * (g.dX[1] * 1e6) * g.nX[0] * g.nX[1] * (s->Nzh * g.dX[2] * 1e6) +
               (s->nlayerTot + 1) * g.lrate * (g.dX[0] * 1e6) * (g.dX[1] * 1e6) * g.nX[0] * g.nX[1] * (g.layerT * 1e6);
  long long gcap = opt && opt->grain_capacity > 0 ? opt->grain_capacity : (long long)(2 * est) + (1 << 16);
  D.grain_cap = (int)std::min<long long>(gcap, 2000000000LL);
  s->nblk = (N + CAFE_CELLS_PER_BLOCK - 1) / CAFE_CELLS_PER_BLOCK;
  s->act_chunks = N >= (1LL << 26) ? CAFE_ACT_MAX_CHUNKS : 1;
  {
    long long per_block = (long long)CAFE_CELLS_PER_BLOCK * s->act_chunks;
    s->nblk_act = (N + per_block - 1) / per_block;
  }
  s->nblk_pos = (acap + CAFE_CELLS_PER_BLOCK - 1) / CAFE_CELLS_PER_BLOCK;
  // the class map covers the pool box of a step; with the analytic field its
  // size is bounded by the pool extents (make_step_params), so it is sized
  // once here rather than regrown (a regrowth would change the device
  // pointers that the step graphs captured)
  if (!K.easm) {
    double A = std::max(K.bmDX0, K.a1[3]), B = std::max(K.a1[1], K.a1[4]), C = std::max(K.a1[2], K.a1[5]);
    double ext[3] = {2 * (A + B), 2 * (A + B), 2 * C};
    long long box = 1;
    for (int a = 0; a < 3; ++a) {
      double cells = ext[a] / g.dX[a] + 8;
      box *= (long long)std::min<double>((double)g.nX[a], cells == cells ? cells : (double)g.nX[a]);
    }
    D.tcls_cap = std::min<long long>(std::max<long long>(box, 1), N);
  }
  D.blk_cap = std::max(s->nblk, 2 * s->nblk_pos);
  auto &o = s->owned;
  if ((rc = dalloc(&D.state, N, o)) || (rc = dalloc(&D.gid, N, o)) || (rc = dalloc(&D.ext, N, o)) ||
      (rc = dalloc(&D.cx, N, o)) || (rc = dalloc(&D.cy, N, o)) || (rc = dalloc(&D.cz, N, o)) ||
      (rc = dalloc(&D.buildj, N, o)) || (rc = dalloc(&D.build, N, o)) || (rc = dalloc(&D.pos_of, N, o)) || (rc = dalloc(&D.liq, acap, o)) ||
      (rc = dalloc(&D.cth, 4 * (size_t)D.grain_cap, o)) || (rc = dalloc(&D.rot, 9 * (size_t)D.grain_cap, o)) ||
      (rc = dalloc(&D.act, acap, o)) || (rc = dalloc(&D.a_state, acap, o)) || (rc = dalloc(&D.a_cls, acap, o)) ||
      (rc = dalloc(&D.a_nn, acap, o)) || (rc = dalloc(&D.a_cold, acap, o)) || (rc = dalloc(&D.a_gid, acap, o)) ||
      (rc = dalloc(&D.a_liq, acap, o)) || (rc = dalloc(&D.a_frow, acap, o)) ||
      (rc = dalloc(&D.a_nbr, (size_t)acap * CAFE_NSLOT, o)) || (rc = dalloc(&D.a_ext, acap, o)) ||
      (rc = dalloc(&D.a_cx, acap, o)) || (rc = dalloc(&D.a_cy, acap, o)) || (rc = dalloc(&D.a_cz, acap, o)) ||
      (rc = dalloc(&D.a_ruq, acap, o)) || (rc = dalloc(&D.vs2, acap, o)) || (rc = dalloc(&D.row_pos, D.row_cap, o)) ||
      (rc = dalloc(&D.row_j, D.row_cap, o)) || (rc = dalloc(&D.row_alive, D.row_cap, o)) ||
      (rc = dalloc(&D.row_ord, (size_t)D.row_cap * CAFE_NSLOT, o)) || (rc = dalloc(&D.row_live, D.row_cap, o)) ||
      (rc = dalloc(&D.row_g, (size_t)D.row_cap * CAFE_NSLOT, o)) ||
      (rc = dalloc(&D.row_geo, (size_t)D.row_cap * CAFE_NSLOT * 4, o)) ||
      (rc = dalloc(&D.row_pairs, (size_t)D.row_cap * CAFE_NSLOT, o)) || (rc = dalloc(&D.blk, D.blk_cap, o)) ||
      (rc = dalloc(&D.row_E, D.row_cap, o)) || (rc = dalloc(&D.row_death, D.row_cap, o)) ||
      (rc = dalloc(&D.row_m, D.row_cap, o)) || (rc = dalloc(&D.ev_vd, D.ev_cap, o)) ||
      (rc = dalloc(&D.ev_vs, D.ev_cap, o)) ||
      (rc = dalloc(&D.row_stamp, D.row_cap, o)) || (rc = dalloc(&D.row_bslot, D.row_cap, o)) ||
      (rc = dalloc(&D.row_bq, D.row_cap, o)) ||
      (rc = dalloc(&D.row_key, D.row_cap, o)) || (rc = dalloc(&D.row_key2, D.row_cap, o)) ||
      (rc = dalloc(&D.row_bt, D.row_cap, o)) ||
      (rc = dalloc(&D.row_bruq, D.row_cap, o)) ||
      (rc = dalloc(&D.ctr, CTR_COUNT, o)) || (rc = dalloc(&D.err, 1, o)) || (rc = dalloc(&D.stat, STAT_COUNT, o)) ||
      (rc = dalloc(&D.Pd, 1, o)) || (rc = dalloc(&D.fill, 1, o)) || (rc = dalloc(&D.fill_seq, 2, o)) ||
      (rc = dalloc(&D.act_flags, (size_t)((N + CAFE_CELLS_PER_BLOCK - 1) / CAFE_CELLS_PER_BLOCK) * CAFE_DENSE_THREADS, o)) || (rc = dalloc(&D.tcls, std::max<long long>(D.tcls_cap, 1), o)) ||
      (K.easm && ((rc = dalloc(&D.temp, N, o)) || (rc = dalloc(&D.a_vh, acap, o)) ||
                  (rc = dalloc(&D.easm_q, (size_t)(D.easm_qcap = std::min<long long>(N, 1LL << 21)), o))))) {
    cafe_sim_destroy(s);
    return rc;
  }
  if (cudaMallocHost((void **)&s->h_pinned, 16 * sizeof(int)) != cudaSuccess) {
    cafe_sim_destroy(s);
    return fail(CAFE_E_CUDA, "cudaMallocHost failed");
  }
  cudaMemsetAsync(D.state, 0, N, s->stream);
  cudaMemsetAsync(D.gid, 0, N * sizeof(int32_t), s->stream);
  cudaMemsetAsync(D.ext, 0, N * sizeof(double), s->stream);
  cudaMemsetAsync(D.cx, 0, N * sizeof(double), s->stream);
  cudaMemsetAsync(D.cy, 0, N * sizeof(double), s->stream);
  cudaMemsetAsync(D.cz, 0, N * sizeof(double), s->stream);
  cudaMemsetAsync(D.buildj, 0, N, s->stream);
  cudaMemsetAsync(D.build, 0, N, s->stream);
  if (K.tmodel == 1) cudaMemsetAsync(D.temp, 0, N * sizeof(double), s->stream);
  // the Rosenthal field leaves cells above the laser plane at T0
  if (K.tmodel == 2) k_fill_f64<<<grid_blocks(N, 256, s), 256, 0, s->stream>>>(D.temp, N, K.T0);
  cudaMemsetAsync(D.pos_of, 0xff, N * sizeof(int32_t), s->stream);
  cudaMemsetAsync(D.ctr, 0, CTR_COUNT * sizeof(int), s->stream);
  cudaMemsetAsync(D.err, 0, sizeof(int), s->stream);
  cudaMemsetAsync(D.stat, 0, STAT_COUNT * sizeof(unsigned long long), s->stream);
  ce = cudaStreamSynchronize(s->stream);
  if (ce != cudaSuccess) {
    cafe_sim_destroy(s);
    return fail(CAFE_E_CUDA, "device initialisation: %s", cudaGetErrorString(ce));
  }
  *out = s;
  return CAFE_OK;
}

void cafe_sim_destroy(cafe_sim *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  resolve_phases(s);
  for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : s->marks)
    if (e) cudaEventDestroy(e);
  for (void *p : s->owned) cudaFree(p);
  if (s->h_pinned) cudaFreeHost(s->h_pinned);
  if (s->h_out) cudaFreeHost(s->h_out);
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

int cafe_sim_initialize_voxels(cafe_sim *s) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  if (s->initialized) return fail(CAFE_E_STATE, "initialize_voxels called twice");
  CUDA_TRY(cudaSetDevice(s->device));
  GridH &g = s->g;
  const CafeConsts &K = s->K;
  // BasePlate::GenerateNgrain / GenerateVoxel (BasePlate.C:31-53)
  double height = s->Nzh * (g.dX[2]);
  double rate = g.mu * (g.dX[0] * 1e6) * (g.dX[1] * 1e6) * g.nX[0] * g.nX[1] * (height * 1e6);
  if (!(rate > 0)) return fail(CAFE_E_ARG, "baseplate grain rate must be positive (mu, bpH)");
  std::poisson_distribution<int> ng(rate);
  int Ngrain = 0;
  while (Ngrain == 0) Ngrain = ng(s->bp_generator);
  std::vector<double> xs(3 * (size_t)Ngrain);
  std::uniform_real_distribution<double> xrand(0.0, 1.0);
  double Lx = g.dX[0] * g.nX[0], Ly = g.dX[1] * g.nX[1];
  for (int j = 0; j < Ngrain; ++j) {
    xs[3 * (size_t)j] = xrand(s->bp_generator) * Lx;
    xs[3 * (size_t)j + 1] = xrand(s->bp_generator) * Ly;
    xs[3 * (size_t)j + 2] = xrand(s->bp_generator) * height;
  }
  int rc = grow_grains(s, (long long)Ngrain + 1);
  if (rc) return rc;
  HostSiteGrid G;
  double lo[3] = {0, 0, 0}, hi[3] = {Lx, Ly, std::max(height, g.dX[2])};
  build_site_grid(G, xs, lo, hi);
  std::vector<void *> tmp;
  CafeSiteGrid dv;
  if ((rc = upload_site_grid(s, xs, G, dv, tmp))) return rc;
  long long nbp = (long long)s->Nzh * K.nxy;
  if (nbp > 0) k_baseplate<<<grid_blocks(nbp, 256, s), 256, 0, s->stream>>>(s->D, K, dv, s->Nzh);
  CUDA_TRY(cudaGetLastError());
  // VoxelsCA::Build of the baseplate cells (VoxelsCA.C:156-159)
  k_build_init<<<grid_blocks(K.N, 256, s), 256, 0, s->stream>>>(s->D, K);
  CUDA_TRY(cudaGetLastError());
  if ((rc = full_active_range(s))) return rc;
  // orientations (BasePlate.C:83-96)
  std::default_random_engine g1(531231);
  unsigned int sdloc = unsigned(double(g1()) / double(g1.max()) * std::pow(2.0, 32.0));
  std::vector<double> aa;
  host_generate_samples(Ngrain, sdloc, aa);
  CUDA_TRY(cudaMemcpyAsync(s->D.cth, aa.data(), aa.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  k_rot_range<<<grid_blocks(Ngrain, 128, s), 128, 0, s->stream>>>(s->D, 0, Ngrain);
  CUDA_TRY(cudaGetLastError());
  s->nGrain = Ngrain;
  s->h_pinned[2] = Ngrain;
  CUDA_TRY(cudaMemcpyAsync(s->D.ctr + CTR_NGRAIN, s->h_pinned + 2, sizeof(int), cudaMemcpyHostToDevice, s->stream));
  free_tmp(s, tmp);
  s->initialized = true;
  return sim_sync(s);
}

int cafe_sim_add_layer(cafe_sim *s) {
  if (!s || !s->initialized) return fail(CAFE_E_STATE, "add_layer before initialize_voxels");
  CUDA_TRY(cudaSetDevice(s->device));
  GridH &g = s->g;
  const CafeConsts &K = s->K;
  int rc = read_ctr(s, CTR_NGRAIN, &s->nGrain);
  if (rc) return rc;
  // VoxelsCA.C:898-917
  unsigned int sdloc = unsigned(double(s->genlayer()) / double(s->genlayer.max()) * std::pow(2.0, 32.0));
  double rate = g.lrate * (g.dX[0] * 1e6) * (g.dX[1] * 1e6) * g.nX[0] * g.nX[1] * (g.layerT * 1e6);
  if (!(rate > 0)) return fail(CAFE_E_ARG, "layer grain rate must be positive (lrate, lT)");
  std::poisson_distribution<int> ng(rate);
  int ng2 = 0;
  while (ng2 == 0) ng2 = ng(s->genlayer);
  int iz1 = g.ilaserLoc - g.nZlayer;
  double zloc0 = iz1 * g.dX[2];
  std::vector<double> xs(3 * (size_t)ng2);
  std::uniform_real_distribution<double> xrand(0.0, 1.0);
  double Lx = g.nX[0] * g.dX[0], Ly = g.nX[1] * g.dX[1];
  for (int j = 0; j < ng2; ++j) {
    xs[3 * (size_t)j] = xrand(s->genlayer) * Lx;
    xs[3 * (size_t)j + 1] = xrand(s->genlayer) * Ly;
    xs[3 * (size_t)j + 2] = xrand(s->genlayer) * g.layerT + zloc0;
  }
  HostSiteGrid G;
  double lo[3] = {0, 0, zloc0}, hi[3] = {Lx, Ly, zloc0 + std::max(g.layerT, g.dX[2])};
  build_site_grid(G, xs, lo, hi);
  std::vector<void *> tmp;
  CafeSiteGrid dv;
  if ((rc = upload_site_grid(s, xs, G, dv, tmp))) return rc;
  long long nslab = (long long)K.nxy * g.nZlayer;
  int32_t *gtmp, *used, *map;
  CUDA_TRY(cudaMalloc((void **)&gtmp, std::max<long long>(1, nslab) * sizeof(int32_t)));
  tmp.push_back(gtmp);
  CUDA_TRY(cudaMalloc((void **)&used, ng2 * sizeof(int32_t)));
  tmp.push_back(used);
  CUDA_TRY(cudaMalloc((void **)&map, ng2 * sizeof(int32_t)));
  tmp.push_back(map);
  CUDA_TRY(cudaMemsetAsync(used, 0, ng2 * sizeof(int32_t), s->stream));
  if (nslab > 0)
    k_layer_voronoi<<<grid_blocks(nslab, 256, s), 256, 0, s->stream>>>(K, dv, iz1, g.ilaserLoc, gtmp, used);
  CUDA_TRY(cudaGetLastError());
  std::vector<int32_t> hu(ng2), hm(ng2, 0);
  CUDA_TRY(cudaMemcpyAsync(hu.data(), used, ng2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  // contiguous renumbering of the used sites (VoxelsCA.C:938-951)
  int i2 = 0;
  for (int j = 0; j < ng2; ++j)
    if (hu[j]) hm[j] = i2++;
  if (i2 == ng2)
    for (int j = 0; j < ng2; ++j) hm[j] = j;
  CUDA_TRY(cudaMemcpyAsync(map, hm.data(), ng2 * sizeof(int32_t), cudaMemcpyHostToDevice, s->stream));
  k_layer_apply<<<grid_blocks(K.N, 256, s), 256, 0, s->stream>>>(s->D, K, iz1, g.ilaserLoc, gtmp, map, s->nGrain);
  LAUNCHED(CAFE_PH_LAYER, 3);
  CUDA_TRY(cudaGetLastError());
  int n0 = s->nGrain;
  s->nGrain += i2 + 1;
  if ((rc = grow_grains(s, s->nGrain + 1))) return rc;
  std::vector<double> aa;
  host_generate_samples(i2 + 1, sdloc, aa);
  CUDA_TRY(cudaMemcpyAsync(s->D.cth + 4LL * n0, aa.data(), aa.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  k_rot_range<<<grid_blocks(i2 + 1, 128, s), 128, 0, s->stream>>>(s->D, n0, s->nGrain);
  CUDA_TRY(cudaGetLastError());
  s->h_pinned[2] = s->nGrain;
  CUDA_TRY(cudaMemcpyAsync(s->D.ctr + CTR_NGRAIN, s->h_pinned + 2, sizeof(int), cudaMemcpyHostToDevice, s->stream));
  free_tmp(s, tmp);
  return sim_sync(s);
}

int cafe_sim_update_laser(cafe_sim *s) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  grid_update_laser(s->g);
  return CAFE_OK;
}

int cafe_sim_temperature(cafe_sim *s) {
  if (!s || !s->initialized) return fail(CAFE_E_STATE, "temperature before initialize_voxels");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = step_prepare(s);
  if (!rc) rc = launch_melt(s, false, s->D.Pd);
  if (!rc) rc = end_of_scan(s);
  return rc;
}

int cafe_sim_update_voxels(cafe_sim *s) {
  if (!s || !s->have_P) return fail(CAFE_E_STATE, "update_voxels before temperature");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = launch_voxels(s, false, s->D.Pd);
  if (rc) return rc;
  voxels_done(s);
  return CAFE_OK;
}

int cafe_sim_clean_layer(cafe_sim *s) {
  if (!s || !s->initialized) return fail(CAFE_E_STATE, "clean_layer before initialize_voxels");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = read_ctr(s, CTR_NGRAIN, &s->nGrain);
  if (rc) return rc;
  int ng = s->nGrain;
  int32_t *cnt = nullptr, *newid = nullptr;
  double *cth2 = nullptr, *rot2 = nullptr;
  // every temporary is freed on every return; the new grain tables leave the
  // list only once the handle owns them
  struct Temps {
    cafe_sim *s;
    std::vector<void *> p;
    ~Temps() { free_tmp(s, p); }
  } tmp{s, {}};
  CUDA_TRY(cudaMalloc((void **)&cnt, std::max(1, ng) * sizeof(int32_t)));
  tmp.p.push_back(cnt);
  CUDA_TRY(cudaMalloc((void **)&newid, std::max(1, ng) * sizeof(int32_t)));
  tmp.p.push_back(newid);
  CUDA_TRY(cudaMalloc((void **)&cth2, (size_t)s->D.grain_cap * 4 * sizeof(double)));
  tmp.p.push_back(cth2);
  CUDA_TRY(cudaMalloc((void **)&rot2, (size_t)s->D.grain_cap * 9 * sizeof(double)));
  tmp.p.push_back(rot2);
  CUDA_TRY(cudaMemsetAsync(cnt, 0, std::max(1, ng) * sizeof(int32_t), s->stream));
  LAUNCHED(CAFE_PH_LAYER, 3);
  k_grain_count<<<grid_blocks(s->K.N, 256, s), 256, 0, s->stream>>>(s->D, s->K, cnt);
  k_grain_renumber<<<1, 1024, 0, s->stream>>>(s->D, cnt, newid, cth2, rot2);
  k_gid_remap<<<grid_blocks(s->K.N, 256, s), 256, 0, s->stream>>>(s->D, s->K, newid);
  CUDA_TRY(cudaGetLastError());
  int nnew = 0;
  if ((rc = read_ctr(s, CTR_NVS2_END, &nnew))) return rc;
  for (auto &p : s->owned) {
    if (p == (void *)s->D.cth) { cudaFree(p); p = (void *)cth2; }
    else if (p == (void *)s->D.rot) { cudaFree(p); p = (void *)rot2; }
  }
  tmp.p.resize(2);  // cth2 and rot2 now belong to the handle
  s->D.cth = cth2;
  s->D.rot = rot2;
  s->nGrain = nnew;
  s->h_pinned[2] = nnew;
  CUDA_TRY(cudaMemcpyAsync(s->D.ctr + CTR_NGRAIN, s->h_pinned + 2, sizeof(int), cudaMemcpyHostToDevice, s->stream));
  free_tmp(s, tmp.p);
  return sim_sync(s);
}

int cafe_sim_update_time(cafe_sim *s) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  s->g.time += s->DelT;
  s->g.tInd += 1;
  return CAFE_OK;
}

int cafe_sim_begin(cafe_sim *s) {
  if (!s || !s->initialized) return fail(CAFE_E_STATE, "begin before initialize_voxels");
  if (s->begun) return fail(CAFE_E_STATE, "begin called twice");
  int rc = cafe_sim_add_layer(s);
  if (rc) return rc;
  grid_update_laser(s->g);
  s->begun = true;
  return CAFE_OK;
}

int cafe_sim_step(cafe_sim *s, int *done) {
  if (!s || !s->begun) return fail(CAFE_E_STATE, "step before begin");
  if (s->done) {
    if (done) *done = 1;
    return CAFE_OK;
  }
  int rc;
  if (graph_eligible(s)) {
    CUDA_TRY(cudaSetDevice(s->device));
    if ((rc = step_plan(s))) return rc;
    k_put_params<<<1, 1, 0, s->stream>>>(s->D.Pd, s->P);
    LAUNCHED(CAFE_PH_MELT, 1);
    CUDA_TRY(cudaGetLastError());
    if ((rc = step_graph_launch(s)) || (rc = end_of_scan(s))) return rc;
    voxels_done(s);
  } else {
    if ((rc = cafe_sim_temperature(s))) return rc;
    if ((rc = cafe_sim_update_voxels(s))) return rc;
  }
  return finish_step(s, done);
}

int cafe_sim_run(cafe_sim *s, long long max_steps, long long *steps_done) {
  if (!s || !s->begun) return fail(CAFE_E_STATE, "run before begin");
  long long n = 0;
  int done = s->done ? 1 : 0, rc;
  while (!done && (max_steps <= 0 || n < max_steps)) {
    if ((rc = cafe_sim_step(s, &done))) return rc;
    ++n;
  }
  if (done && !s->closed) {  // main1.C:95-97 run once, after the loop
    if ((rc = cafe_sim_clean_layer(s))) return rc;
    s->closed = true;
    if (!s->out_base.empty()) {
      std::string name = s->out_base + std::to_string(s->tf_tInd) + ".h5";
      if ((rc = cafe_sim_write_output(s, name.c_str()))) return rc;
    }
  }
  if (steps_done) *steps_done = n;
  return sim_sync(s);
}

int cafe_sim_synchronize(cafe_sim *s) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  CUDA_TRY(cudaSetDevice(s->device));
  return sim_sync(s);
}

int cafe_sim_info(cafe_sim *s, cafe_info *info) {
  if (!s || !info) return fail(CAFE_E_ARG, "null argument");
  int rc = read_ctr(s, CTR_NGRAIN, &s->nGrain);
  if (rc) return rc;
  const GridH &g = s->g;
  info->nx = g.nX[0];
  info->ny = g.nX[1];
  info->nz = g.nX[2];
  info->dx = g.dX[0];
  info->tInd = g.tInd;
  info->time = g.time;
  info->isp = g.isp;
  info->indlayer = g.indlayer;
  info->inewlayerflg = g.inewlayerflg;
  info->inewscanflg = g.inewscanflg;
  info->ilaserLoc = g.ilaserLoc;
  info->nGrain = s->nGrain;
  info->nlayerTot = s->nlayerTot;
  info->Nzh = s->Nzh;
  info->done = s->done ? 1 : 0;
  info->steps = s->steps;
  info->gth = g.gth;
  {
    std::ostringstream os;
    os << s->genlayer;
    info->genlayer_state = (unsigned int)std::stoul(os.str());
  }
  info->tf_tInd = s->tf_tInd;
  info->output_due = s->output_due ? 1 : 0;
  return CAFE_OK;
}

int cafe_sim_set_output(cafe_sim *s, const char *base) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  s->out_base = base ? base : "";
  return CAFE_OK;
}

int cafe_generate_samples(int n, unsigned int seed, double *axis_angle) {
  if (n < 0 || (n > 0 && !axis_angle)) return fail(CAFE_E_ARG, "cafe_generate_samples: bad argument");
  std::vector<double> v;
  host_generate_samples(n, seed, v);
  std::copy(v.begin(), v.end(), axis_angle);
  return CAFE_OK;
}

int cafe_sim_grid(cafe_sim *s, cafe_grid *out) {
  if (!s || !out) return fail(CAFE_E_ARG, "null argument");
  const GridH &g = s->g;
  for (int a = 0; a < 3; ++a) {
    out->nX[a] = g.nX[a];
    out->dX[a] = g.dX[a];
    out->LX[a] = g.LX[a];
    out->offset[a] = g.offset[a];
  }
  for (int a = 0; a < 4; ++a) {
    out->meltparam[a] = g.meltparam[a];
    out->gbox[a] = g.gbox[a];
  }
  out->gsize[0] = g.gsize[0];
  out->gsize[1] = g.gsize[1];
  out->bmV = g.bmV;
  out->bmP = g.bmP;
  out->bmDelT = g.bmDelT;
  out->bhatch = g.bhatch;
  out->tL = g.tL;
  out->tS = g.tS;
  out->T0 = g.T0;
  out->layerT = g.layerT;
  out->bpH = g.bpH;
  out->mu = g.mu;
  out->lrate = g.lrate;
  out->rNmax = g.rNmax;
  out->Avel = g.Avel;
  out->nvel = g.nvel;
  out->gth0 = g.gth0;
  out->gth = g.gth;
  out->time = g.time;
  out->DelT = s->DelT;
  out->outint = g.outint;
  out->patternID = g.patternID;
  out->outNL = g.outNL;
  out->EASM_Flag = g.EASM_Flag;
  out->nZlayer = g.nZlayer;
  out->Nzhg = g.Nzhg;
  out->Nsd = g.Nsd;
  out->Ntd = g.Ntd;
  out->NpT = g.NpT;
  out->isp = g.isp;
  out->inewscanflg = g.inewscanflg;
  out->inewlayerflg = g.inewlayerflg;
  out->indlayer = g.indlayer;
  out->ilaserLoc = g.ilaserLoc;
  out->tInd = g.tInd;
  out->tf_tInd = s->tf_tInd;
  out->Nzh = s->Nzh;
  out->nlayerTot = s->nlayerTot;
  out->seed = g.seed;
  out->tmodel = s->K.tmodel;
  out->ros_eta = g.ros_eta;
  out->ros_k = g.ros_k;
  out->ros_alpha = g.ros_alpha;
  out->laser[0] = out->laser[1] = out->laser[2] = out->dirp = 0.0;
  if (g.isp >= 0 && g.isp < g.NpT && g.Nsd > 0 && !((std::fmod(g.isp, g.Nsd) == 0 && g.isp + 1 >= g.NpT) ||
                                                    (std::fmod(g.isp, g.Nsd) != 0 && g.isp < 1))) {
    CafeStepParams P;
    make_step_params(s, P);
    out->laser[0] = P.lx;
    out->laser[1] = P.ly;
    out->laser[2] = P.lz;
    out->dirp = P.dirp;
  }
  return CAFE_OK;
}

int cafe_sim_stats(cafe_sim *s, cafe_stats *st) {
  if (!s || !st) return fail(CAFE_E_ARG, "null argument");
  unsigned long long v[STAT_COUNT];
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  CUDA_TRY(cudaMemcpy(v, s->D.stat, sizeof v, cudaMemcpyDeviceToHost));
  st->events = v[STAT_EVENTS];
  st->nucleations = v[STAT_NUC];
  st->max_active = v[STAT_MAXNA];
  st->max_rows = v[STAT_MAXROWS];
  st->steps = v[STAT_STEPS];
  st->negative_dt = v[STAT_NEGDT];
  st->sum_active = v[STAT_SUMNA];
  st->sum_rows = v[STAT_SUMROWS];
  st->launches = (unsigned long long)s->launches;
  st->exact_scan_steps = v[STAT_SLOWSTEPS];
  st->row_evaluations = v[STAT_EVALS];
  st->cycles_select = v[STAT_CYC_SELECT];
  st->cycles_apply = v[STAT_CYC_APPLY];
  st->cycles_fill = v[STAT_CYC_FILL];
  st->cycles_merge = v[STAT_CYC_OTHER];
  st->graph_captures = (unsigned long long)s->graph_captures;
  st->easm_integrals = v[STAT_EASM_INTEGRALS];
#ifdef CAFE_DETAIL_CYCLES
  fprintf(stderr, "cafe detail cycles:");
  for (int c = 0; c < 32; ++c) fprintf(stderr, " %llu", v[STAT_DETAIL + c]);
  fprintf(stderr, "\n");
#endif
  return CAFE_OK;
}

int cafe_sim_set_timing(cafe_sim *s, int on) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  resolve_phases(s);
  s->timing = on != 0;
  return CAFE_OK;
}

int cafe_sim_phase_times(cafe_sim *s, double *ms, long long *launches, int nphase, int reset) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  CUDA_TRY(cudaSetDevice(s->device));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  resolve_phases(s);
  for (int p = 0; p < nphase && p < CAFE_NPHASE; ++p) {
    if (ms) ms[p] = s->phase_ms[p];
    if (launches) launches[p] = s->phase_launch[p];
  }
  if (reset) {
    for (int p = 0; p < CAFE_NPHASE; ++p) {
      s->phase_ms[p] = 0;
      s->phase_launch[p] = 0;
    }
    s->launches = 0;
  }
  return CAFE_OK;
}

int cafe_sim_mark(cafe_sim *s, int slot) {
  if (!s || slot < 0 || slot >= 8) return fail(CAFE_E_ARG, "bad mark slot");
  CUDA_TRY(cudaSetDevice(s->device));
  if (!s->marks[slot]) CUDA_TRY(cudaEventCreate(&s->marks[slot]));
  CUDA_TRY(cudaEventRecord(s->marks[slot], s->stream));
  return CAFE_OK;
}

int cafe_sim_elapsed(cafe_sim *s, int a, int b, double *ms) {
  if (!s || !ms || a < 0 || a >= 8 || b < 0 || b >= 8 || !s->marks[a] || !s->marks[b])
    return fail(CAFE_E_ARG, "bad mark slots");
  CUDA_TRY(cudaEventSynchronize(s->marks[b]));
  float f = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&f, s->marks[a], s->marks[b]));
  *ms = f;
  return CAFE_OK;
}

int cafe_sim_stream(cafe_sim *s, void **stream) {
  if (!s || !stream) return fail(CAFE_E_ARG, "null argument");
  *stream = (void *)s->stream;
  return CAFE_OK;
}

// Staging buffer for layout conversions of host transfers: CAFE_XFER_BYTES
// of device memory plus an error word, allocated once per handle.
#define CAFE_XFER_BYTES (64LL << 20)
static int ensure_xfer(cafe_sim *s) {
  if (s->xfer) return CAFE_OK;
  int rc = dalloc(&s->xfer, CAFE_XFER_BYTES, s->owned);
  if (!rc) rc = dalloc(&s->d_bad, 1, s->owned);
  return rc;
}

int cafe_sim_download_state(cafe_sim *s, int32_t *gID, int32_t *vState, double *extents,
                            double *centroid, int32_t *buildjID) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc) return rc;
  if ((rc = ensure_xfer(s))) return rc;
  const long long N = s->K.N;
  cudaStream_t st = s->stream;
  // same layout: straight copies; others converted on the device chunk by chunk
  if (gID) CUDA_TRY(cudaMemcpyAsync(gID, s->D.gid, N * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  if (extents) CUDA_TRY(cudaMemcpyAsync(extents, s->D.ext, N * sizeof(double), cudaMemcpyDeviceToHost, st));
  const uint8_t *u8src[2] = {s->D.state, s->D.buildj};
  int32_t *i32dst[2] = {vState, buildjID};
  const long long ci = CAFE_XFER_BYTES / (long long)sizeof(int32_t);
  for (int f = 0; f < 2; ++f) {
    if (!i32dst[f]) continue;
    for (long long off = 0; off < N; off += ci) {
      long long n = std::min(ci, N - off);
      k_u8_to_i32<<<grid_blocks(n, 256, s), 256, 0, st>>>(u8src[f] + off, (int32_t *)s->xfer, n);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaMemcpyAsync(i32dst[f] + off, s->xfer, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    }
  }
  if (centroid) {
    const long long cc = CAFE_XFER_BYTES / (3LL * (long long)sizeof(double));
    for (long long off = 0; off < N; off += cc) {
      long long n = std::min(cc, N - off);
      k_interleave3<<<grid_blocks(n, 256, s), 256, 0, st>>>(s->D.cx + off, s->D.cy + off, s->D.cz + off,
                                                              (double *)s->xfer, n);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaMemcpyAsync(centroid + 3 * off, s->xfer, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  return CAFE_OK;
}

int cafe_sim_download_temperature(cafe_sim *s, double *temp) {
  if (!s || !temp) return fail(CAFE_E_ARG, "null argument");
  CUDA_TRY(cudaSetDevice(s->device));
  long long N = s->K.N;
  if (!s->have_P) {
    for (long long i = 0; i < N; ++i) temp[i] = 0.0;
    return CAFE_OK;
  }
  if (s->K.easm) {
    CUDA_TRY(cudaMemcpyAsync(temp, s->D.temp, N * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return CAFE_OK;
  }
  double *d;
  CUDA_TRY(cudaMalloc((void **)&d, N * sizeof(double)));
  k_temperature<<<grid_blocks(N, 256, s), 256, 0, s->stream>>>(s->K, s->P, d);
  cudaError_t e1 = cudaGetLastError();
  cudaError_t e2 = cudaMemcpyAsync(temp, d, N * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  cudaError_t e3 = cudaStreamSynchronize(s->stream);
  cudaFree(d);
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
    return fail(CAFE_E_CUDA, "temperature download failed");
  return CAFE_OK;
}

int cafe_sim_download_ctheta(cafe_sim *s, double *ctheta, long long cap, int *ngrain) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = read_ctr(s, CTR_NGRAIN, &s->nGrain);
  if (rc) return rc;
  if (ngrain) *ngrain = s->nGrain;
  if (ctheta) {
    if (cap < 4LL * s->nGrain) return fail(CAFE_E_ARG, "ctheta buffer too small (%lld < %lld)", cap, 4LL * s->nGrain);
    CUDA_TRY(cudaMemcpy(ctheta, s->D.cth, 4LL * s->nGrain * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return CAFE_OK;
}

int cafe_sim_upload_state(cafe_sim *s, const int32_t *gID, const int32_t *vState, const double *extents,
                          const double *centroid, const double *ctheta, int ngrain) {
  if (!s || !gID || !vState || !extents || !centroid || !ctheta || ngrain < 0)
    return fail(CAFE_E_ARG, "null or negative argument");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc) return rc;
  if ((rc = ensure_xfer(s)) || (rc = grow_grains(s, (long long)ngrain + 1))) return rc;
  const long long N = s->K.N;
  cudaStream_t st = s->stream;
  // the state is replaced from here on: the handle is usable again only after
  // a successful upload
  s->initialized = false;
  CUDA_TRY(cudaMemsetAsync(s->d_bad, 0, sizeof(int), st));
  CUDA_TRY(cudaMemcpyAsync(s->D.gid, gID, N * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  k_check_range_i32<<<grid_blocks(N, 256, s), 256, 0, st>>>(s->D.gid, N, ngrain, s->d_bad, 2);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(s->D.ext, extents, N * sizeof(double), cudaMemcpyHostToDevice, st));
  const long long ci = CAFE_XFER_BYTES / (long long)sizeof(int32_t);
  for (long long off = 0; off < N; off += ci) {
    long long n = std::min(ci, N - off);
    CUDA_TRY(cudaMemcpyAsync(s->xfer, vState + off, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    k_i32_to_u8_check<<<grid_blocks(n, 256, s), 256, 0, st>>>((const int32_t *)s->xfer, s->D.state + off, n, 3,
                                                                s->d_bad, 1);
    CUDA_TRY(cudaGetLastError());
  }
  const long long cc = CAFE_XFER_BYTES / (3LL * (long long)sizeof(double));
  for (long long off = 0; off < N; off += cc) {
    long long n = std::min(cc, N - off);
    CUDA_TRY(cudaMemcpyAsync(s->xfer, centroid + 3 * off, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
    k_deinterleave3<<<grid_blocks(n, 256, s), 256, 0, st>>>((const double *)s->xfer, s->D.cx + off, s->D.cy + off,
                                                              s->D.cz + off, n);
    CUDA_TRY(cudaGetLastError());
  }
  if (ngrain > 0) {
    CUDA_TRY(cudaMemcpyAsync(s->D.cth, ctheta, 4LL * ngrain * sizeof(double), cudaMemcpyHostToDevice, st));
    k_rot_range<<<grid_blocks(ngrain, 128, s), 128, 0, st>>>(s->D, 0, ngrain);
    CUDA_TRY(cudaGetLastError());
  }
  CUDA_TRY(cudaMemcpyAsync(s->h_pinned + 3, s->d_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  int bad = s->h_pinned[3];
  if (bad & 1) return fail(CAFE_E_ARG, "vState value outside 0..3");
  if (bad & 2) return fail(CAFE_E_ARG, "gID value outside 0..nGrain (%d)", ngrain);
  s->nGrain = ngrain;
  s->h_pinned[2] = ngrain;
  CUDA_TRY(cudaMemcpyAsync(s->D.ctr + CTR_NGRAIN, s->h_pinned + 2, sizeof(int), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(s->D.ctr + CTR_NLIQ, 0, sizeof(int), st));
  s->full_k2 = true;
  s->have_prev_box = false;
  if ((rc = full_active_range(s))) return rc;
  s->initialized = true;
  return sim_sync(s);
}

// ------------------------------------------------------------------ output
int cafe_sim_set_build(cafe_sim *s) {
  if (!s || !s->initialized) return fail(CAFE_E_STATE, "set_build before initialize_voxels");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = read_ctr(s, CTR_NGRAIN, &s->nGrain);
  if (rc) return rc;
  long long need = (long long)s->nGrain + 2;
  if (need > s->gflag_cap) {
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (auto &p : s->owned)
      if (p == (void *)s->gflag) {
        cudaFree(p);
        p = nullptr;
      }
    long long cap = std::max<long long>(need, 2 * s->gflag_cap + 4096);
    s->gflag = nullptr;
    s->gflag_cap = 0;
    if ((rc = dalloc(&s->gflag, cap, s->owned))) return rc;
    s->gflag_cap = cap;
  }
  CUDA_TRY(cudaMemsetAsync(s->gflag, 0, need, s->stream));
  k_build_flag<<<grid_blocks(s->K.N, 256, s), 256, 0, s->stream>>>(s->D, s->K, s->gflag);
  k_build_mark<<<grid_blocks(s->K.N, 256, s), 256, 0, s->stream>>>(s->D, s->K, s->gflag);
  LAUNCHED(CAFE_PH_LAYER, 2);
  CUDA_TRY(cudaGetLastError());
  return CAFE_OK;
}

int cafe_sim_download_build(cafe_sim *s, int32_t *build) {
  if (!s || !build) return fail(CAFE_E_ARG, "null argument");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc) return rc;
  if ((rc = ensure_xfer(s))) return rc;
  const long long N = s->K.N, ci = CAFE_XFER_BYTES / (long long)sizeof(int32_t);
  for (long long off = 0; off < N; off += ci) {
    long long n = std::min(ci, N - off);
    k_u8_to_i32<<<grid_blocks(n, 256, s), 256, 0, s->stream>>>(s->D.build + off, (int32_t *)s->xfer, n);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(build + off, s->xfer, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return CAFE_OK;
}

namespace {

// Constants of the colour triangle of WriteToHDF1 (VoxelsCA.C:1597-1613),
// evaluated by the host's libm as the reference evaluates them.
CafeIpfConsts ipf_consts() {
  double tp[2][3] = {{0.0, 2. / std::pow(2, .5) / (1. + 1. / std::pow(2, .5)),
                      2. / std::pow(3, .5) / (1. + 1. / std::pow(3, .5))},
                     {0.0, 0.0, 2. / std::pow(3, .5) / (1. + 1. / std::pow(3, .5))}};
  double m = std::tan(1. / 2. * std::atan2(tp[1][2], tp[0][2]));
  double a = std::pow(std::pow(tp[1][2] - tp[1][1], 2.) + std::pow(tp[0][2] - tp[0][1], 2.), .5);
  double b = std::pow(std::pow(tp[0][1], 2.) + std::pow(tp[1][1], 2.), 0.5);
  double c = std::pow(std::pow(tp[0][2], 2.) + std::pow(tp[1][2], 2.), 0.5);
  CafeIpfConsts C;
  C.y0 = 1. / 2. * std::pow((b + c - a) * (c + a - b) * (a + b - c) / (a + b + c), .5);
  C.x0 = C.y0 / m;
  C.sMax = std::pow(std::pow(C.x0, 2.) + std::pow(C.y0, 2.), .5);
  C.hoff = std::atan((tp[1][2] - C.y0) / (tp[0][2] - C.x0)) * 180 / M_PI;
  return C;
}

// The per-cell output datasets, produced chunk by chunk into the staging
// buffer: 0 Temperature, 1 IPFz, 2 IPFx, 3 IPFy, 4 Build (int32).
struct OutputSource {
  cafe_sim *s;
  float *gcol = nullptr;  // IPF colours per grain (9 floats)
  int ngrain = 0;
  ~OutputSource() {
    if (gcol) cudaFree(gcol);
  }
  int prepare(bool need_ipf) {
    int rc = ensure_xfer(s);
    if (rc) return rc;
    if ((rc = read_ctr(s, CTR_NGRAIN, &s->nGrain))) return rc;
    ngrain = s->nGrain;
    if (need_ipf && ngrain > 0) {
      CUDA_TRY(cudaMalloc((void **)&gcol, 9LL * ngrain * sizeof(float)));
      k_ipf_grains<<<grid_blocks(ngrain, 128, s), 128, 0, s->stream>>>(s->D.cth, ngrain, ipf_consts(), gcol);
      CUDA_TRY(cudaGetLastError());
    }
    return CAFE_OK;
  }
  static int cell_bytes(int which) { return (which >= 1 && which <= 3) ? 12 : 4; }
  long long chunk(int which) const { return CAFE_XFER_BYTES / cell_bytes(which); }
  // queues the production of cells [off, off+n) of dataset `which` into xfer
  int produce(int which, long long off, long long n) {
    cudaStream_t st = s->stream;
    int nb = grid_blocks(n, 256, s);
    if (which == 0) {
      if (s->K.easm)
        k_temp_copy_f<<<nb, 256, 0, st>>>(s->D.temp, off, n, (float *)s->xfer);
      else if (s->have_P)
        k_temperature_f<<<nb, 256, 0, st>>>(s->K, s->P, off, n, (float *)s->xfer);
      else
        CUDA_TRY(cudaMemsetAsync(s->xfer, 0, n * sizeof(float), st));
    } else if (which <= 3) {
      if (gcol)
        k_ipf_cells<<<nb, 256, 0, st>>>(s->D, gcol, which - 1, off, n, (float *)s->xfer);
      else
        CUDA_TRY(cudaMemsetAsync(s->xfer, 0, 12 * n, st));
    } else {
      k_build_i32<<<nb, 256, 0, st>>>(s->D, off, n, (int32_t *)s->xfer);
    }
    CUDA_TRY(cudaGetLastError());
    return CAFE_OK;
  }
};

int write_file(const std::string &path, const void *p, size_t bytes) {
  FILE *fp = std::fopen(path.c_str(), "wb");
  if (!fp) return fail(CAFE_E_IO, "cannot open '%s' for writing", path.c_str());
  size_t w = bytes ? std::fwrite(p, 1, bytes, fp) : 0;
  int cl = std::fclose(fp);
  if (w != bytes || cl != 0) return fail(CAFE_E_IO, "write to '%s' failed", path.c_str());
  return CAFE_OK;
}

// Streams `bytes` of device memory into an open file through the pinned
// bounce buffer.
int stream_to_file(cafe_sim *s, FILE *fp, const std::string &path, long long bytes, const void *dsrc) {
  for (long long off = 0; off < bytes; off += CAFE_XFER_BYTES) {
    long long n = std::min<long long>(CAFE_XFER_BYTES, bytes - off);
    CUDA_TRY(cudaMemcpyAsync(s->h_out, (const unsigned char *)dsrc + off, n, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (std::fwrite(s->h_out, 1, n, fp) != (size_t)n) return fail(CAFE_E_IO, "write to '%s' failed", path.c_str());
  }
  return CAFE_OK;
}

// <prefix>.xdmf: an XDMF description of the raw files, so that viewers read
// them as cell data on the uniform voxel grid (cell j = i + nx*(j + ny*k)).
int write_xdmf(cafe_sim *s, const char *prefix) {
  const GridH &g = s->g;
  std::string pre(prefix), leaf = pre.substr(pre.find_last_of('/') + 1);
  std::ostringstream x;
  x.precision(17);
  const int nx = g.nX[0], ny = g.nX[1], nz = g.nX[2];
  x << "<?xml version=\"1.0\" ?>\n<Xdmf Version=\"3.0\">\n <Domain>\n  <Grid Name=\"CA\" GridType=\"Uniform\">\n";
  x << "   <Topology TopologyType=\"3DCoRectMesh\" Dimensions=\"" << nz + 1 << " " << ny + 1 << " " << nx + 1
    << "\"/>\n";
  x << "   <Geometry GeometryType=\"ORIGIN_DXDYDZ\">\n";
  x << "    <DataItem Dimensions=\"3\" Format=\"XML\">0 0 0</DataItem>\n";
  x << "    <DataItem Dimensions=\"3\" Format=\"XML\">" << g.dX[2] << " " << g.dX[1] << " " << g.dX[0]
    << "</DataItem>\n   </Geometry>\n";
  struct Item {
    const char *name, *type;
    int comps;
  } items[7] = {{"gID", "Int", 1},           {"vState", "Int", 1}, {"Build", "Int", 1}, {"Temperature", "Float", 1},
                {"IPFz", "Float", 3},        {"IPFx", "Float", 3}, {"IPFy", "Float", 3}};
  for (const Item &it : items) {
    x << "   <Attribute Name=\"" << it.name << "\" AttributeType=\"" << (it.comps == 3 ? "Vector" : "Scalar")
      << "\" Center=\"Cell\">\n    <DataItem Dimensions=\"" << nz << " " << ny << " " << nx;
    if (it.comps == 3) x << " 3";
    x << "\" NumberType=\"" << it.type << "\" Precision=\"4\" Format=\"Binary\" Endian=\"Native\">" << leaf << "."
      << it.name << ".bin</DataItem>\n   </Attribute>\n";
  }
  x << "  </Grid>\n </Domain>\n</Xdmf>\n";
  const std::string body = x.str();
  return write_file(pre + ".xdmf", body.data(), body.size());
}

}  // namespace

int cafe_sim_download_output(cafe_sim *s, float *temperature, float *ipfz, float *ipfx, float *ipfy) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc) return rc;
  OutputSource src{s};
  if ((rc = src.prepare(ipfz || ipfx || ipfy))) return rc;
  float *dst[4] = {temperature, ipfz, ipfx, ipfy};
  const long long N = s->K.N;
  for (int w = 0; w < 4; ++w) {
    if (!dst[w]) continue;
    const int per = OutputSource::cell_bytes(w) / 4;
    const long long c = src.chunk(w);
    for (long long off = 0; off < N; off += c) {
      long long n = std::min(c, N - off);
      if ((rc = src.produce(w, off, n))) return rc;
      CUDA_TRY(cudaMemcpyAsync(dst[w] + per * off, s->xfer, n * OutputSource::cell_bytes(w), cudaMemcpyDeviceToHost,
                               s->stream));
    }
  }
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return CAFE_OK;
}

int cafe_sim_write_output(cafe_sim *s, const char *prefix) {
  if (!s || !prefix) return fail(CAFE_E_ARG, "null argument");
  if (!s->initialized) return fail(CAFE_E_STATE, "write_output before initialize_voxels");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc) return rc;
  if (!s->h_out && cudaMallocHost((void **)&s->h_out, CAFE_XFER_BYTES) != cudaSuccess) {
    s->h_out = nullptr;
    return fail(CAFE_E_CUDA, "cudaMallocHost of the output buffer failed");
  }
  OutputSource src{s};
  if ((rc = src.prepare(true))) return rc;
  const std::string base = std::string(prefix) + ".";
  const long long N = s->K.N;
  const GridH &g = s->g;
  int32_t dims[3] = {g.nX[0], g.nX[1], g.nX[2]};
  float vdx[3] = {(float)g.dX[0], (float)g.dX[1], (float)g.dX[2]};
  if ((rc = write_file(base + "dims.bin", dims, sizeof dims)) || (rc = write_file(base + "VoxelDX.bin", vdx, sizeof vdx)))
    return rc;
  // datasets in the reference's order
  const char *names[8] = {"gID", "vState", "Build", "Temperature", "IPFz", "IPFx", "IPFy", "angleAxis"};
  for (int d = 0; d < 8; ++d) {
    const std::string path = base + names[d] + ".bin";
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) return fail(CAFE_E_IO, "cannot open '%s' for writing", path.c_str());
    rc = CAFE_OK;
    if (d == 0) {
      rc = stream_to_file(s, fp, path, N * (long long)sizeof(int32_t), s->D.gid);
    } else if (d == 1) {
      const long long ci = CAFE_XFER_BYTES / (long long)sizeof(int32_t);
      for (long long off = 0; off < N && !rc; off += ci) {
        long long n = std::min(ci, N - off);
        k_u8_to_i32<<<grid_blocks(n, 256, s), 256, 0, s->stream>>>(s->D.state + off, (int32_t *)s->xfer, n);
        if (cudaGetLastError() != cudaSuccess) rc = fail(CAFE_E_CUDA, "vState conversion failed");
        if (!rc) rc = stream_to_file(s, fp, path, n * (long long)sizeof(int32_t), s->xfer);
      }
    } else if (d == 7) {
      // cTheta as float (VoxelsCA.C:1811)
      std::vector<double> cth(4 * (size_t)src.ngrain);
      std::vector<float> f(cth.size());
      if (!cth.empty() &&
          cudaMemcpy(cth.data(), s->D.cth, cth.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = fail(CAFE_E_CUDA, "cTheta download failed");
      for (size_t j = 0; j < cth.size(); ++j) f[j] = (float)cth[j];
      if (!rc && !f.empty() && std::fwrite(f.data(), sizeof(float), f.size(), fp) != f.size())
        rc = fail(CAFE_E_IO, "write to '%s' failed", path.c_str());
    } else {
      int which = d == 2 ? 4 : d - 3;  // Build, Temperature, IPFz, IPFx, IPFy
      const long long c = src.chunk(which);
      for (long long off = 0; off < N && !rc; off += c) {
        long long n = std::min(c, N - off);
        rc = src.produce(which, off, n);
        if (!rc) rc = stream_to_file(s, fp, path, n * OutputSource::cell_bytes(which), s->xfer);
      }
    }
    if (std::fclose(fp) != 0 && !rc) rc = fail(CAFE_E_IO, "write to '%s' failed", path.c_str());
    if (rc) return rc;
  }
  return write_xdmf(s, prefix);
}

// ------------------------------------------------------------------ checkpoint
namespace {
const char kCkptMagic[8] = {'C', 'A', 'F', 'E', 'C', 'K', 'P', 'T'};
struct CkptHeader {
  char magic[8];
  int32_t version, nx, ny, nz;
  double time, gth;
  int32_t tInd, isp, inewscanflg, inewlayerflg, indlayer, ilaserLoc, tf_tInd, nGrain, done, output_due;
  int64_t steps;
  uint32_t genlayer_state, pad;
};
// Reads `bytes` from fp into device memory dst through the pinned buffer.
int stream_from_file(cafe_sim *s, FILE *fp, const std::string &path, long long bytes, void *dst) {
  for (long long off = 0; off < bytes; off += CAFE_XFER_BYTES) {
    long long n = std::min<long long>(CAFE_XFER_BYTES, bytes - off);
    CUDA_TRY(cudaStreamSynchronize(s->stream));  // the previous chunk has left the buffer
    if (std::fread(s->h_out, 1, n, fp) != (size_t)n) return fail(CAFE_E_IO, "'%s' is truncated", path.c_str());
    CUDA_TRY(cudaMemcpyAsync((unsigned char *)dst + off, s->h_out, n, cudaMemcpyHostToDevice, s->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return CAFE_OK;
}
int ensure_host_buffer(cafe_sim *s) {
  if (!s->h_out && cudaMallocHost((void **)&s->h_out, CAFE_XFER_BYTES) != cudaSuccess) {
    s->h_out = nullptr;
    return fail(CAFE_E_CUDA, "cudaMallocHost of the transfer buffer failed");
  }
  return CAFE_OK;
}
}  // namespace

int cafe_sim_checkpoint(cafe_sim *s, const char *path) {
  if (!s || !path) return fail(CAFE_E_ARG, "null argument");
  if (!s->begun) return fail(CAFE_E_STATE, "checkpoint before begin");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc || (rc = ensure_host_buffer(s)) || (rc = read_ctr(s, CTR_NGRAIN, &s->nGrain))) return rc;
  const GridH &g = s->g;
  CkptHeader h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.nx = g.nX[0];
  h.ny = g.nX[1];
  h.nz = g.nX[2];
  h.time = g.time;
  h.gth = g.gth;
  h.tInd = g.tInd;
  h.isp = g.isp;
  h.inewscanflg = g.inewscanflg;
  h.inewlayerflg = g.inewlayerflg;
  h.indlayer = g.indlayer;
  h.ilaserLoc = g.ilaserLoc;
  h.tf_tInd = s->tf_tInd;
  h.nGrain = s->nGrain;
  h.done = s->done ? 1 : 0;
  h.output_due = s->output_due ? 1 : 0;
  h.steps = s->steps;
  {
    std::ostringstream os;
    os << s->genlayer;
    h.genlayer_state = (uint32_t)std::stoul(os.str());
  }
  const std::string p(path);
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(CAFE_E_IO, "cannot open '%s' for writing", path);
  const long long N = s->K.N;
  const CafeDev &D = s->D;
  if (std::fwrite(&h, sizeof h, 1, fp) != 1) rc = fail(CAFE_E_IO, "write to '%s' failed", path);
  // voxel fields in the device layout, then cTheta
  struct Part {
    const void *p;
    long long bytes;
  } parts[] = {{D.gid, N * 4}, {D.state, N}, {D.ext, N * 8}, {D.cx, N * 8}, {D.cy, N * 8},
               {D.cz, N * 8}, {D.buildj, N}, {D.build, N}, {D.cth, 32LL * s->nGrain}};
  for (const Part &pt : parts)
    if (!rc) rc = stream_to_file(s, fp, p, pt.bytes, pt.p);
  if (std::fclose(fp) != 0 && !rc) rc = fail(CAFE_E_IO, "write to '%s' failed", path);
  return rc;
}

int cafe_sim_restore(cafe_sim *s, const char *path) {
  if (!s || !path) return fail(CAFE_E_ARG, "null argument");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc || (rc = ensure_host_buffer(s)) || (rc = ensure_xfer(s))) return rc;
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(CAFE_E_IO, "cannot open '%s'", path);
  CkptHeader h;
  GridH &g = s->g;
  const long long N = s->K.N;
  if (std::fread(&h, sizeof h, 1, fp) != 1 || std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1) {
    std::fclose(fp);
    return fail(CAFE_E_ARG, "'%s' is not a checkpoint of this engine", path);
  }
  if (h.nx != g.nX[0] || h.ny != g.nX[1] || h.nz != g.nX[2] || h.nGrain < 0 || h.isp < 0 || h.isp >= g.NpT) {
    std::fclose(fp);
    return fail(CAFE_E_ARG, "checkpoint '%s' does not belong to this deck (grid %dx%dx%d)", path, h.nx, h.ny, h.nz);
  }
  if ((rc = grow_grains(s, (long long)h.nGrain + 1))) {
    std::fclose(fp);
    return rc;
  }
  // the state is replaced from here on: usable again only after a complete restore
  s->initialized = false;
  s->begun = false;
  CafeDev &D = s->D;
  struct Part {
    void *p;
    long long bytes;
  } parts[] = {{D.gid, N * 4}, {D.state, N}, {D.ext, N * 8}, {D.cx, N * 8}, {D.cy, N * 8},
               {D.cz, N * 8}, {D.buildj, N}, {D.build, N}, {D.cth, 32LL * h.nGrain}};
  for (const Part &pt : parts)
    if (!rc) rc = stream_from_file(s, fp, path, pt.bytes, pt.p);
  if (!rc && std::fgetc(fp) != EOF) rc = fail(CAFE_E_ARG, "'%s' has trailing data", path);
  std::fclose(fp);
  if (rc) return rc;
  // value checks (as cafe_sim_upload_state)
  cudaStream_t st = s->stream;
  CUDA_TRY(cudaMemsetAsync(s->d_bad, 0, sizeof(int), st));
  k_check_range_i32<<<grid_blocks(N, 256, s), 256, 0, st>>>(D.gid, N, h.nGrain, s->d_bad, 2);
  k_check_range_u8<<<grid_blocks(N, 256, s), 256, 0, st>>>(D.state, N, 3, s->d_bad, 1);
  k_check_range_u8<<<grid_blocks(N, 256, s), 256, 0, st>>>(D.buildj, N, 1, s->d_bad, 4);
  k_check_range_u8<<<grid_blocks(N, 256, s), 256, 0, st>>>(D.build, N, 1, s->d_bad, 4);
  if (h.nGrain > 0) k_rot_range<<<grid_blocks(h.nGrain, 128, s), 128, 0, st>>>(D, 0, h.nGrain);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(s->h_pinned + 3, s->d_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  int bad = s->h_pinned[3];
  if (bad) return fail(CAFE_E_ARG, "checkpoint '%s' holds out-of-range values (flags %d)", path, bad);
  // host state
  g.time = h.time;
  g.gth = h.gth;
  grid_rotate_points(g, false);
  g.tInd = h.tInd;
  g.isp = h.isp;
  g.inewscanflg = h.inewscanflg;
  g.inewlayerflg = h.inewlayerflg;
  g.indlayer = h.indlayer;
  g.ilaserLoc = h.ilaserLoc;
  s->tf_tInd = h.tf_tInd;
  s->genlayer.seed(h.genlayer_state);
  s->nGrain = h.nGrain;
  s->h_pinned[2] = h.nGrain;
  CUDA_TRY(cudaMemcpyAsync(D.ctr + CTR_NGRAIN, s->h_pinned + 2, sizeof(int), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(D.ctr + CTR_NLIQ, 0, sizeof(int), st));
  s->steps = h.steps;
  s->done = h.done != 0;
  s->closed = false;
  s->output_due = h.output_due != 0;
  s->have_P = false;
  s->full_k2 = true;          // the liquid list is rebuilt by a dense pass
  s->have_prev_box = false;
  if ((rc = full_active_range(s))) return rc;
  s->initialized = true;
  s->begun = true;
  return sim_sync(s);
}

// ------------------------------------------------------------------ growth log
int cafe_sim_set_growth_log(cafe_sim *s, int32_t *cells, int32_t *steps, double *tau, long long cap) {
  if (!s) return fail(CAFE_E_ARG, "null handle");
  if ((cells || steps || tau) && (!cells || !steps || !tau || cap <= 0 || cap > 0x7fffffffLL))
    return fail(CAFE_E_ARG, "growth log needs three device arrays and 0 < cap < 2^31");
  CUDA_TRY(cudaSetDevice(s->device));
  int rc = sim_sync(s);
  if (rc) return rc;
  s->D.glog_cell = cells;
  s->D.glog_step = steps;
  s->D.glog_tau = tau;
  s->D.glog_cap = cells ? cap : 0;
  CUDA_TRY(cudaMemsetAsync(s->D.ctr + CTR_GLOG_N, 0, 2 * sizeof(int), s->stream));
  return sim_sync(s);
}

int cafe_sim_growth_log_count(cafe_sim *s, long long *n) {
  if (!s || !n) return fail(CAFE_E_ARG, "null argument");
  CUDA_TRY(cudaSetDevice(s->device));
  int v = 0, over = 0, rc;
  if ((rc = read_ctr(s, CTR_GLOG_N, &v)) || (rc = read_ctr(s, CTR_GLOG_OVER, &over))) return rc;
  if (over) return fail(CAFE_E_CAPACITY, "growth log full after %d entries", v);
  *n = v;
  return CAFE_OK;
}

}  // extern "C"

// ====================================================================== batched steps
// One launch per step kernel for all realisations of a batch (the kernels of
// cafe_batch_kernels.cuh), captured once as a CUDA graph and replayed every
// batch step. The host keeps each realisation's own loop logic (laser state
// machine, end-of-scan check, layer changes, output points): per batch step it
// plans every looping realisation's step, uploads all step parameters at once,
// launches the graph, and reads back every realisation's "some cell at the
// liquidus" flag and error word at once. Realisations whose step cannot take
// the graphed path (EASM or Rosenthal field, a dense pass after an upload)
// take a plain cafe_sim_step on their own stream that batch step. Launch
// shapes (grid share per realisation, 8-cell chunks of the compaction) are
// picked by timing candidates on the first batch steps; neither changes any
// result, so a batched realisation ends bit-identical to its plain run.
struct CafeBatchEngine {
  std::vector<cafe_sim *> sims;
  int n = 0, device = 0, nsm = 1;
  cudaStream_t stream = nullptr;
  CafeBatchReal *dR = nullptr;
  std::vector<CafeBatchReal> hR;
  std::vector<char> hR_valid;
  int *dStart = nullptr;
  int *dActive = nullptr, *hActive = nullptr;
  CafeStepParams *dP = nullptr, *hP = nullptr;
  int *dReport = nullptr, *hReport = nullptr;
  int total[BK_COUNT] = {0};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> ev_plain;
  int share = 4, chunks = 1;      // launch shape in use
  bool loop_pairs = false;        // two event-loop blocks per realisation (fill helper)
  bool tuned = false;
  int tune_steps = 6;             // batch steps timed per candidate
  std::vector<std::pair<std::pair<int, int>, double>> trials;  // ((share, chunks), ms per batch step)
  size_t trial = 0;
  int trial_steps = 0;
  double trial_ms = 0;
  long long launches = 0, batch_steps = 0;
  std::string log;
};

namespace {

const int kBatchThreads[BK_COUNT] = {32, 256, 256, 256, 256, 32, CAFE_DENSE_THREADS, 1024, CAFE_DENSE_THREADS, 256,
                                     CAFE_DENSE_THREADS, 1024, CAFE_DENSE_THREADS, 32, 256, 256, 256,
                                     CAFE_LOOP_THREADS, 256, 256, 256, 32};

// blocks of realisation s in a batched launch of `kind` (its plain graphed
// step's grid, cafe_sim launch_melt / launch_voxels)
long long batch_blocks(const cafe_sim *s, int kind, bool loop_pairs) {
  const long long g = s->gsm;
  switch (kind) {
    case BK_LOOP: return loop_pairs ? 2 : 1;
    case BK_MELT: case BK_PBOX0: case BK_PBOX1: return g * 16;
    case BK_LIST: case BK_PREP: case BK_ORDER: case BK_FINAL: return g * 4;
    case BK_ACOUNT: case BK_ASCATTER: return std::max<long long>(1, std::min<long long>(s->nblk_act, g * 8));
    case BK_GATHER: case BK_GEO: case BK_WB: case BK_M2S: return g * 8;
    case BK_LCOUNT: case BK_LSCATTER: return std::max<long long>(1, s->nblk_pos);
    default: return 1;  // resets, scans, the event loop, the report
  }
}

void batch_set_shape(CafeBatchEngine *E, int gsm, int chunks) {
  E->share = gsm;
  E->chunks = chunks;
  for (cafe_sim *s : E->sims) {
    s->gsm = gsm;
    s->act_chunks = chunks;
    long long per_block = (long long)CAFE_CELLS_PER_BLOCK * chunks;
    s->nblk_act = (s->K.N + per_block - 1) / per_block;
  }
  std::fill(E->hR_valid.begin(), E->hR_valid.end(), 0);
}

int batch_capture(CafeBatchEngine *E) {
  if (E->exec) cudaGraphExecDestroy(E->exec);
  if (E->graph) cudaGraphDestroy(E->graph);
  E->exec = nullptr;
  E->graph = nullptr;
  const int n = E->n;
  std::vector<int> start((size_t)BK_COUNT * (n + 1));
  for (int k = 0; k < BK_COUNT; ++k) {
    long long acc = 0;
    for (int r = 0; r < n; ++r) {
      start[(size_t)k * (n + 1) + r] = (int)acc;
      acc += batch_blocks(E->sims[r], k, E->loop_pairs);
    }
    if (acc > 0x7fffffffLL) return fail(CAFE_E_CAPACITY, "batch: too many blocks in one launch");
    start[(size_t)k * (n + 1) + n] = (int)acc;
    E->total[k] = (int)acc;
  }
  CUDA_TRY(cudaMemcpyAsync(E->dStart, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, E->stream));
  CafeBatchArgs A;
  A.R = E->dR;
  A.start = E->dStart;
  A.active = E->dActive;
  A.report = E->dReport;
  A.n = n;
  const int *T = kBatchThreads;
  cudaStream_t st = E->stream;
  CUDA_TRY(cudaStreamSynchronize(st));
  CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  kb_reset_a<<<E->total[BK_RESET_A], T[BK_RESET_A], 0, st>>>(A);
  kb_melt<<<E->total[BK_MELT], T[BK_MELT], 0, st>>>(A);
  kb_solid2mushy_pbox0<<<E->total[BK_PBOX0], T[BK_PBOX0], 0, st>>>(A);
  kb_solid2mushy_pbox1<<<E->total[BK_PBOX1], T[BK_PBOX1], 0, st>>>(A);
  kb_solid2mushy_list<<<E->total[BK_LIST], T[BK_LIST], 0, st>>>(A);
  kb_reset_b<<<E->total[BK_RESET_B], T[BK_RESET_B], 0, st>>>(A);
  kb_active_count<<<E->total[BK_ACOUNT], T[BK_ACOUNT], 0, st>>>(A);
  kb_scan_blocks<<<E->total[BK_SCAN], T[BK_SCAN], 0, st>>>(A);
  kb_active_scatter<<<E->total[BK_ASCATTER], T[BK_ASCATTER], 0, st>>>(A);
  kb_gather<<<E->total[BK_GATHER], T[BK_GATHER], 0, st>>>(A);
  kb_lists_count<<<E->total[BK_LCOUNT], T[BK_LCOUNT], 0, st>>>(A);
  kb_scan_pairs<<<E->total[BK_SCANP], T[BK_SCANP], 0, st>>>(A);
  kb_lists_scatter<<<E->total[BK_LSCATTER], T[BK_LSCATTER], 0, st>>>(A);
  kb_reset_c<<<E->total[BK_RESET_C], T[BK_RESET_C], 0, st>>>(A);
  kb_rows_prep<<<E->total[BK_PREP], T[BK_PREP], 0, st>>>(A);
  kb_rows_geo<<<E->total[BK_GEO], T[BK_GEO], 0, st>>>(A);
  kb_rows_order<<<E->total[BK_ORDER], T[BK_ORDER], 0, st>>>(A);
  if (E->loop_pairs) {
    // every pair must be resident at once: a cooperative launch
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(E->total[BK_LOOP]);
    cfg.blockDim = dim3(T[BK_LOOP]);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kb_event_loop, A);
  } else {
    kb_event_loop<<<E->total[BK_LOOP], T[BK_LOOP], 0, st>>>(A);
  }
  kb_rows_finalize<<<E->total[BK_FINAL], T[BK_FINAL], 0, st>>>(A);
  kb_writeback<<<E->total[BK_WB], T[BK_WB], 0, st>>>(A);
  kb_mushy2solid<<<E->total[BK_M2S], T[BK_M2S], 0, st>>>(A);
  kb_report<<<E->total[BK_REPORT], T[BK_REPORT], 0, st>>>(A);
  cudaMemcpyAsync(E->hReport, E->dReport, 2 * (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaGraph_t g = nullptr;
  cudaError_t le = cudaGetLastError();
  cudaError_t ce = cudaStreamEndCapture(st, &g);
  if (le != cudaSuccess || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(CAFE_E_CUDA, "batch graph capture: %s", cudaGetErrorString(le != cudaSuccess ? le : ce));
  }
  E->graph = g;
  CUDA_TRY(cudaGraphInstantiate(&E->exec, g, 0));
  return CAFE_OK;
}

// A realisation's step takes the batched path unless it needs the plain one.
bool batch_eligible(const cafe_sim *s) { return !s->K.easm && !s->full_k2 && !s->timing; }

// The autotuner: candidates (grid share per realisation, compaction chunks)
// in turn for tune_steps batch steps each, then the fastest.
int batch_tune_next(CafeBatchEngine *E, double ms) {
  if (E->tuned) return CAFE_OK;
  E->trial_ms += ms;
  if (++E->trial_steps < E->tune_steps) return CAFE_OK;
  E->trials[E->trial].second = E->trial_ms / E->trial_steps;
  E->trial_ms = 0;
  E->trial_steps = 0;
  ++E->trial;
  int rc;
  if (E->trial < E->trials.size()) {
    batch_set_shape(E, E->trials[E->trial].first.first, E->trials[E->trial].first.second);
    return batch_capture(E);
  }
  size_t best = 0;
  for (size_t i = 1; i < E->trials.size(); ++i)
    if (E->trials[i].second < E->trials[best].second) best = i;
  char buf[256];
  std::string s = "{\"candidates\": [";
  for (size_t i = 0; i < E->trials.size(); ++i) {
    snprintf(buf, sizeof buf, "%s{\"grid_share_sms\": %d, \"compaction_chunks\": %d, \"ms_per_batch_step\": %.4f}",
             i ? ", " : "", E->trials[i].first.first, E->trials[i].first.second, E->trials[i].second);
    s += buf;
  }
  snprintf(buf, sizeof buf,
           "], \"chosen\": {\"grid_share_sms\": %d, \"compaction_chunks\": %d}, \"steps_each\": %d, "
           "\"event_loop_blocks\": %d}",
           E->trials[best].first.first, E->trials[best].first.second, E->tune_steps, E->loop_pairs ? 2 : 1);
  s += buf;
  E->log = s;
  E->tuned = true;
  batch_set_shape(E, E->trials[best].first.first, E->trials[best].first.second);
  if ((rc = batch_capture(E))) return rc;
  return CAFE_OK;
}

}  // namespace

CafeBatchEngine *cafe_internal_batch_engine_create(cafe_sim *const *sims, int n, int tune, int *rc_out) {
  CafeBatchEngine *E = new CafeBatchEngine;
  auto bail = [&](int rc) {
    *rc_out = rc;
    return (CafeBatchEngine *)nullptr;
  };
  E->sims.assign(sims, sims + n);
  E->n = n;
  E->device = sims[0]->device;
  for (int r = 0; r < n; ++r)
    if (sims[r]->device != E->device) {
      delete E;
      return bail(fail(CAFE_E_ARG, "batch: realisations on different devices"));
    }
  int rc = CAFE_OK;
  auto cu = [&](cudaError_t e, const char *what) {
    if (e != cudaSuccess && rc == CAFE_OK) rc = fail(CAFE_E_CUDA, "batch: %s: %s", what, cudaGetErrorString(e));
  };
  cu(cudaSetDevice(E->device), "cudaSetDevice");
  E->nsm = sims[0]->nsm;
  cu(cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  cu(cudaMalloc((void **)&E->dR, (size_t)n * sizeof(CafeBatchReal)), "cudaMalloc");
  cu(cudaMalloc((void **)&E->dStart, (size_t)BK_COUNT * (n + 1) * sizeof(int)), "cudaMalloc");
  cu(cudaMalloc((void **)&E->dActive, (size_t)n * sizeof(int)), "cudaMalloc");
  cu(cudaMalloc((void **)&E->dP, (size_t)n * sizeof(CafeStepParams)), "cudaMalloc");
  cu(cudaMalloc((void **)&E->dReport, 2 * (size_t)n * sizeof(int)), "cudaMalloc");
  cu(cudaMallocHost((void **)&E->hActive, (size_t)n * sizeof(int)), "cudaMallocHost");
  cu(cudaMallocHost((void **)&E->hP, (size_t)n * sizeof(CafeStepParams)), "cudaMallocHost");
  cu(cudaMallocHost((void **)&E->hReport, 2 * (size_t)n * sizeof(int)), "cudaMallocHost");
  cu(cudaEventCreate(&E->ev0), "cudaEventCreate");
  cu(cudaEventCreate(&E->ev1), "cudaEventCreate");
  E->ev_plain.assign(n, nullptr);
  for (int r = 0; r < n && rc == CAFE_OK; ++r) cu(cudaEventCreateWithFlags(&E->ev_plain[r], cudaEventDisableTiming), "cudaEventCreate");
  if (rc) {
    cafe_internal_batch_engine_destroy(E);
    return bail(rc);
  }
  E->hR.resize(n);
  E->hR_valid.assign(n, 0);
  {
    // event-loop pairs when every realisation has its helper on and all the
    // pairs fit on the GPU at once
    int per_sm = 0, coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, E->device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kb_event_loop, CAFE_LOOP_THREADS, 0);
    bool all = true;
    for (int r = 0; r < n; ++r) all = all && sims[r]->event_helper;
    E->loop_pairs = all && coop && (long long)per_sm * E->nsm >= 2LL * n;
  }
  // every realisation reads its step parameters from its slot of dP
  for (int r = 0; r < n; ++r) {
    cafe_sim *s = sims[r];
    cudaStreamSynchronize(s->stream);
    s->D.Pd = E->dP + r;
  }
  const int base = std::max(2, E->nsm / std::max(1, n));
  if (tune) {
    for (int g : {base, 2 * base, 4 * base})
      for (int c : {1, CAFE_ACT_MAX_CHUNKS}) E->trials.push_back({{g, c}, 0.0});
    batch_set_shape(E, E->trials[0].first.first, E->trials[0].first.second);
  } else {
    E->tuned = true;
    batch_set_shape(E, 2 * base, CAFE_ACT_MAX_CHUNKS);
    char buf[128];
    snprintf(buf, sizeof buf, "{\"chosen\": {\"grid_share_sms\": %d, \"compaction_chunks\": %d}, \"tuned\": false}",
             2 * base, CAFE_ACT_MAX_CHUNKS);
    E->log = buf;
  }
  if ((rc = batch_capture(E))) {
    cafe_internal_batch_engine_destroy(E);
    return bail(rc);
  }
  *rc_out = CAFE_OK;
  return E;
}

void cafe_internal_batch_engine_destroy(CafeBatchEngine *E) {
  if (!E) return;
  cudaSetDevice(E->device);
  if (E->stream) cudaStreamSynchronize(E->stream);
  if (E->exec) cudaGraphExecDestroy(E->exec);
  if (E->graph) cudaGraphDestroy(E->graph);
  if (E->ev0) cudaEventDestroy(E->ev0);
  if (E->ev1) cudaEventDestroy(E->ev1);
  for (cudaEvent_t e : E->ev_plain)
    if (e) cudaEventDestroy(e);
  cudaFree(E->dR);
  cudaFree(E->dStart);
  cudaFree(E->dActive);
  cudaFree(E->dP);
  cudaFree(E->dReport);
  cudaFreeHost(E->hActive);
  cudaFreeHost(E->hP);
  cudaFreeHost(E->hReport);
  if (E->stream) cudaStreamDestroy(E->stream);
  delete E;
}

const char *cafe_internal_batch_engine_log(const CafeBatchEngine *E) { return E ? E->log.c_str() : ""; }
long long cafe_internal_batch_engine_launches(const CafeBatchEngine *E) { return E ? E->launches : 0; }
long long cafe_internal_batch_engine_steps(const CafeBatchEngine *E) { return E ? E->batch_steps : 0; }

// One batch step for every realisation with phase[r] == 1 (looping); a
// realisation whose loop ends gets its closing CleanLayer (main1.C:95) and
// phase 2. *stepped counts the realisations that took a step. Returns the
// first error (with the realisation in the message).
int cafe_internal_batch_engine_step(CafeBatchEngine *E, int *phase, long long *steps, int *stepped) {
  CUDA_TRY(cudaSetDevice(E->device));
  const int n = E->n;
  int rc;
  int nact = 0, nplain = 0;
  *stepped = 0;
  // plan: the batched realisations' step parameters; plain steps for the rest
  for (int r = 0; r < n; ++r) {
    cafe_sim *s = E->sims[r];
    E->hActive[r] = 0;
    if (phase[r] != 1) continue;
    if (!batch_eligible(s)) {
      int done = 0;
      if ((rc = cafe_sim_step(s, &done))) return fail(rc, "realisation %d: %s", r, g_last_error.c_str());
      ++steps[r];
      ++*stepped;
      ++nplain;
      if (done) {
        if ((rc = cafe_sim_clean_layer(s))) return fail(rc, "realisation %d: %s", r, g_last_error.c_str());
        s->closed = true;
        phase[r] = 2;
      }
      CUDA_TRY(cudaEventRecord(E->ev_plain[r], s->stream));
      CUDA_TRY(cudaStreamWaitEvent(E->stream, E->ev_plain[r], 0));
      continue;
    }
    if ((rc = step_plan(s))) return fail(rc, "realisation %d: %s", r, g_last_error.c_str());
    E->hP[r] = s->P;
    E->hActive[r] = 1;
    ++nact;
    // the realisation's descriptor, uploaded again when a device buffer,
    // constant or launch shape of it changed (a regrown grain table, say)
    CafeBatchReal x;
    std::memset(&x, 0, sizeof x);
    x.D = s->D;
    x.K = s->K;
    x.act_chunks = s->act_chunks;
    x.allow_fast = s->event_scan ? 0 : 1;
    x.nblk_act = s->nblk_act;
    x.nblk_pos = s->nblk_pos;
    if (!E->hR_valid[r] || std::memcmp(&x, &E->hR[r], sizeof x) != 0) {
      E->hR[r] = x;
      E->hR_valid[r] = 1;
      CUDA_TRY(cudaMemcpyAsync(E->dR + r, &E->hR[r], sizeof x, cudaMemcpyHostToDevice, E->stream));
    }
  }
  (void)nplain;
  if (nact == 0) return CAFE_OK;
  CUDA_TRY(cudaMemcpyAsync(E->dP, E->hP, (size_t)n * sizeof(CafeStepParams), cudaMemcpyHostToDevice, E->stream));
  CUDA_TRY(cudaMemcpyAsync(E->dActive, E->hActive, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, E->stream));
  CUDA_TRY(cudaEventRecord(E->ev0, E->stream));
  CUDA_TRY(cudaGraphLaunch(E->exec, E->stream));
  CUDA_TRY(cudaEventRecord(E->ev1, E->stream));
  CUDA_TRY(cudaStreamSynchronize(E->stream));
  E->launches += BK_COUNT;
  E->batch_steps++;
  float ms = 0;
  cudaEventElapsedTime(&ms, E->ev0, E->ev1);
  // each batched realisation's host side of the step, as cafe_sim_step does it
  for (int r = 0; r < n; ++r) {
    if (!E->hActive[r]) continue;
    cafe_sim *s = E->sims[r];
    if (E->hReport[2 * r + 1])
      return fail(CAFE_E_CAPACITY,
                  "realisation %d: device capacity exceeded (flags 0x%x: 1 active list, 2 frontier rows, 4 grain "
                  "table, 8 mushy list, 16 event cap)",
                  r, E->hReport[2 * r + 1]);
    int hot = E->hReport[2 * r];
    if ((rc = end_of_scan(s, &hot))) return fail(rc, "realisation %d: %s", r, g_last_error.c_str());
    voxels_done(s);
    const bool layer = s->g.inewlayerflg == 1;
    int done = 0;
    if ((rc = finish_step(s, &done))) return fail(rc, "realisation %d: %s", r, g_last_error.c_str());
    ++steps[r];
    ++*stepped;
    if (done) {
      if ((rc = cafe_sim_clean_layer(s))) return fail(rc, "realisation %d: %s", r, g_last_error.c_str());
      s->closed = true;
      phase[r] = 2;
    } else if (layer || s->output_due) {
      // layer changes and output points queue work on the handle's stream
      CUDA_TRY(cudaEventRecord(E->ev_plain[r], s->stream));
      CUDA_TRY(cudaStreamWaitEvent(E->stream, E->ev_plain[r], 0));
    }
  }
  return batch_tune_next(E, ms);
}

// CPU oracle: a restatement of AMCAFE's per-time-step CA path, for tests only.
//
// THIS FILE IS TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load it, and only as the checker or as the
// timed CPU baseline -- never as part of the GPU product path.
//
// It restates, in single-rank form, the reference's main loop (main1.C:18-101)
// and everything it calls on the hot path: the .in parser and laser state
// machine (Grid.C), the analytic double-ellipsoid temperature and the EASM
// moving-Gaussian-source temperature (TempField.C, Utilities.C),
// Voronoi baseplate and powder layers (BasePlate.C, VoxelsCA.C AddLayer1),
// orientation sampling (SampleOrientation.C) and the CA step
// (VoxelsCA.C UpdateVoxels/SetLiquid3/ConvertSolid1/CleanLayer). Each routine
// cites the reference lines it follows. Results are pinned bit-for-bit against
// the reference itself (oracle/_ref, built from the unmodified sources) by the
// tests in tests/test_oracle_pin.py.
//
// Differences from the reference are result-preserving only:
//  * at world size 1, index lookups through icellidLoc (an iota) are direct;
//  * std::find over the sorted active list vI is a binary search;
//  * the per-candidate capture-time numerator pow(cos th sin ph,.5)*|R^T dn|_1
//    is cached per (capturing cell, neighbour) within a step (a pure function
//    of data that does not change while the cell is mushy);
//  * Voronoi nearest-site searches use a bucket grid with the same distance
//    expression and the same first-minimum tie rule;
//  * mushy cells with no liquid neighbour are skipped in the per-event scan
//    (they have zero growth velocity), except when the event time is not
//    finite, where the reference's 0*DtMin = NaN update is applied to them.
//
// libm selection (the functions the GPU evaluates on the device):
//   mode 0: glibc, as the reference;
//   mode 1: the correctly rounded functions of amcafe_gb300/csrc/cafe_crmath.h
//           (the device arithmetic);
//   mode 2: glibc with each result moved by one ulp with probability p
//           (a sensitivity probe for event-order stability).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <vector>
#include <time.h>

#include "../amcafe_gb300/csrc/cafe_crmath.h"
#include "../amcafe_gb300/csrc/cafe_quadrature.h"

namespace orc {

// ---------------------------------------------------------------- libm hook
struct LibmSel {
  int mode = 0;
  double p = 0.0;
  uint64_t s = 0x9e3779b97f4a7c15ull;
};
static LibmSel g_libm;

static double perturb(double v) {
  if (g_libm.mode != 2 || !std::isfinite(v) || v == 0.0) return v;
  uint64_t &s = g_libm.s;
  s ^= s << 13;
  s ^= s >> 7;
  s ^= s << 17;
  double u = (double)(s >> 11) * (1.0 / 9007199254740992.0);
  if (u >= g_libm.p) return v;
  return (s & 1) ? std::nextafter(v, INFINITY) : std::nextafter(v, -INFINITY);
}
static double m_atan2(double y, double x) {
  if (g_libm.mode == 1) return crm_atan2(y, x);
  return perturb(std::atan2(y, x));
}
static double m_cos(double x) {
  if (g_libm.mode == 1) return crm_cos(x);
  return perturb(std::cos(x));
}
static double m_sin(double x) {
  if (g_libm.mode == 1) return crm_sin(x);
  return perturb(std::sin(x));
}
static double m_acos(double x) {
  if (g_libm.mode == 1) return crm_acos(x);
  return perturb(std::acos(x));
}
// pow(x, 0.5): glibc's pow (not sqrt); the correctly rounded value is sqrt.
static double m_powh(double x) {
  if (g_libm.mode == 1) return crm_pow_half(x);
  return perturb(std::pow(x, 0.5));
}
// pow(x, 2.0): glibc returns x*x exactly (checked over 2e8 samples).
static double m_pow2(double x) {
  if (g_libm.mode == 1) return x * x;
  return std::pow(x, 2.0);
}
// pow(x, 2j) for the orientation polynomial (SampleOrientation.C:148).
static double m_pow_even(double x, int e) {
  if (g_libm.mode == 1) return crm_pow_int(x, e);
  return perturb(std::pow(x, (double)e));
}

// std::min / std::max exactly as libstdc++ defines them (NaN behaviour included).
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double smax(double a, double b) { return (a < b) ? b : a; }

// ---------------------------------------------------------------- Grid
// Grid::Grid defaults (Grid.C:18-65) and readInputFile (Grid.C:165-318).
struct Grid {
  int nX[3] = {128, 128, 64};
  double dX[3] = {1e-6, 1e-6, 1e-6};
  int outint = 1, patternID = 1, outNL = 0, nTsd = 0, EASM_Flag = 0;
  int seed = 1;  // extension keyword "seed" (1: the reference's seeds)
  int nuc_gauss = 0;  // extension keyword "nucgauss mean sd"
  double nuc_mean = 0, nuc_sd = 1;
  // extension keyword "rosenthal eta k alpha": the Rosenthal moving point
  // source (absorptivity, conductivity W/(m K), diffusivity m^2/s) in place
  // of the analytic field
  int rosenthal = 0;
  double ros_eta = 0.35, ros_k = 20.0, ros_alpha = 5e-6;
  double tL = 1620, tS = 1531.5, T0 = 300, layerT = 25e-6, bpH = 0.0, mu = .01;
  double lrate = 0.0;
  bool have_lrate = false, have_bmdelt = false;
  double meltparam[4] = {75e-6, 162.75e-6, 75e-6, 75e-6};
  double bhatch = 0, bmDelT = 0, bmV = 500e-3, bmP = 0, rNmax = .002;
  double offset[3] = {0, 0, 0};
  double gth0 = 0, gth = 0, Avel = 0, nvel = 0, gsize[2] = {0, 0};
  // derived (Grid.C:69-108)
  double LX[3];
  int nZlayer, Nzhg, Ntd, Nsd, NpT;
  std::vector<double> lcoor, lcoor2;
  double gbox[4];
  // laser / clock state
  int isp = 0, inewscanflg = 1, inewlayerflg = 1, indlayer = 1, ilaserLoc = 0, tInd = 0;
  double time = 0.0;
};

static bool read_deck(const char *path, Grid &g, std::string &err) {
  // Grid.C:170-191: read char by char; '#' skips to end of line; the last
  // character is stored twice because get() fails at EOF without changing c.
  std::ifstream f(path);
  if (!f) {
    err = "cannot open deck";
    return false;
  }
  std::string data;
  char c = 0;
  while (!f.eof()) {
    f.get(c);
    if (c == '#') {
      while (f && c != '\n') f.get(c);
    }
    data.push_back(c);
  }
  g.bhatch = 1.53 * g.meltparam[2];  // Grid.C:56
  std::istringstream in(data);
  std::string kw;
  in >> kw;
  auto next_d = [&](double &v) {
    in >> kw;
    v = std::stod(kw);
  };
  auto next_i = [&](int &v) {
    in >> kw;
    v = std::stoi(kw);
  };
  try {
    while (in) {
      std::transform(kw.begin(), kw.end(), kw.begin(),
                     [](unsigned char s) { return (char)std::tolower(s); });
      if (kw == "dx") {
        next_d(g.dX[0]);
        g.dX[1] = g.dX[0];
        g.dX[2] = g.dX[0];
      }
      if (kw == "bmv") next_d(g.bmV);
      if (kw == "bmp") next_d(g.bmP);
      if (kw == "bmdelt") {
        next_d(g.bmDelT);
        g.have_bmdelt = true;
      }
      if (kw == "nx") {
        next_i(g.nX[0]);
        next_i(g.nX[1]);
        next_i(g.nX[2]);
      }
      if (kw == "r") next_d(g.rNmax);
      if (kw == "lt") next_d(g.layerT);
      if (kw == "tl") next_d(g.tL);
      if (kw == "ts") next_d(g.tS);
      if (kw == "bhatch") next_d(g.bhatch);
      if (kw == "mu") next_d(g.mu);
      if (kw == "bph") next_d(g.bpH);
      if (kw == "lrate") {
        next_d(g.lrate);
        g.have_lrate = true;
      }
      if (kw == "outnl") next_i(g.outNL);
      if (kw == "ntsd") next_i(g.nTsd);
      if (kw == "offset") {
        next_d(g.offset[0]);
        next_d(g.offset[1]);
        next_d(g.offset[2]);
      }
      // Grid.C:276 compares the lowercased keyword with "EASM": never true.
      // The keyword "easm" selects the EASM temperature here (the flag that
      // keyword was meant to set); the reference reads it as an unknown word.
      if (kw == "easm") next_i(g.EASM_Flag);
      if (kw == "meltparam") {
        next_d(g.meltparam[0]);
        next_d(g.meltparam[1]);
        next_d(g.meltparam[2]);
        next_d(g.meltparam[3]);
      }
      if (kw == "patternid") next_i(g.patternID);
      if (kw == "outint") next_i(g.outint);
      if (kw == "gridsize") {
        next_d(g.gsize[0]);
        next_d(g.gsize[1]);
      }
      if (kw == "gridtheta") next_d(g.gth0);
      if (kw == "seed") next_i(g.seed);
      if (kw == "nucgauss") {
        g.nuc_gauss = 1;
        next_d(g.nuc_mean);
        next_d(g.nuc_sd);
      }
      if (kw == "rosenthal") {
        g.rosenthal = 1;
        next_d(g.ros_eta);
        next_d(g.ros_k);
        next_d(g.ros_alpha);
      }
      if (kw == "dendritegrowth2") {
        next_d(g.Avel);
        next_d(g.nvel);
      }
      in >> kw;
    }
  } catch (...) {
    err = "bad numeric value after keyword";
    return false;
  }
  // The reference reads an uninitialised bmV for the bmDelT default
  // (Grid.C:57-58) and never initialises lrate: both must be given.
  if (!g.have_bmdelt) {
    err = "deck must set bmDelT";
    return false;
  }
  if (!g.have_lrate) {
    err = "deck must set lrate";
    return false;
  }
  return true;
}

static void grid_derive(Grid &g) {
  // Grid.C:69-108
  for (int k = 0; k < 3; ++k) g.LX[k] = g.nX[k] * g.dX[k];
  if (g.bpH < std::numeric_limits<double>::epsilon()) g.bpH = g.layerT;
  g.nZlayer = (int)std::round(g.layerT / g.dX[2]);
  g.isp = 0;
  g.inewscanflg = 1;
  g.inewlayerflg = 1;
  g.Nzhg = std::min(g.nX[2], int(std::ceil(g.bpH * .9999 / g.dX[2])));
  g.indlayer = 1;
  g.ilaserLoc = g.Nzhg + g.indlayer * g.nZlayer;
  g.Ntd = int(std::ceil(g.gsize[1] / g.bhatch)) + 1;
  g.Nsd = int(std::ceil(g.gsize[0] / (g.bmV * g.bmDelT))) + 1;
  g.NpT = g.Nsd * g.Ntd;
  g.lcoor.assign(2 * (size_t)g.NpT, 0.);
  g.lcoor2.assign(2 * (size_t)g.NpT, 0.);
  double xlmin = (g.LX[0] - g.gsize[0]) / 2., ylmin = (g.LX[1] - g.gsize[1]) / 2.;
  double gmid0 = g.LX[0] / 2., gmid1 = g.LX[1] / 2.;
  g.gth += g.gth0;
  for (int j2 = 0; j2 < g.Ntd; ++j2)
    for (int j1 = 0; j1 < g.Nsd; ++j1) {
      int k = g.Nsd * j2 + j1;
      g.lcoor[2 * k] = j1 * g.bmDelT * g.bmV + xlmin;
      g.lcoor[2 * k + 1] = j2 * g.bhatch + ylmin;
      g.lcoor2[2 * k] =
          std::cos(g.gth) * (g.lcoor[2 * k] - gmid0) - std::sin(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid0;
      g.lcoor2[2 * k + 1] =
          std::sin(g.gth) * (g.lcoor[2 * k] - gmid0) + std::cos(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid1;
    }
  g.gbox[0] = -g.bhatch / 2.;
  g.gbox[1] = g.LX[0] + g.bhatch / 2.;
  g.gbox[2] = -g.bhatch / 2.;
  g.gbox[3] = g.LX[1] + g.bhatch / 2.;
}

// Grid::UpdateLaser (Grid.C:110-164).
static void update_laser(Grid &g) {
  int itmp, iflg = 0, irep = 0;
  if (std::fmod(g.isp + 1, g.Nsd) == 0) g.inewscanflg = 1;
  if (g.isp == (g.NpT - 1)) {
    g.inewscanflg = 1;
    g.inewlayerflg = 1;
    g.isp = 0;
    g.indlayer += 1;
  }
  while (irep == 0 || g.isp == 0) {
    irep += 1;
    itmp = g.isp;
    if (g.inewscanflg == 0 && itmp < (g.NpT - 1)) {
      g.isp += 1;
    } else {
      while (itmp < (g.NpT - 1) && iflg == 0) {
        itmp += 1;
        double x = g.lcoor2[2 * itmp], y = g.lcoor2[2 * itmp + 1];
        if (x > g.gbox[0] && x < g.gbox[1] && y > g.gbox[2] && y < g.gbox[3]) iflg = 1;
      }
      if (itmp < (g.NpT - 1)) {
        g.isp = itmp;
        g.inewscanflg = 0;
      } else {
        g.inewlayerflg = 1;
        g.inewscanflg = 1;
        g.indlayer += 1;
        g.ilaserLoc = g.Nzhg + g.indlayer * g.nZlayer;
        g.isp = 0;
        double gmid0 = g.LX[0] / 2., gmid1 = g.LX[1] / 2.;
        g.gth += g.gth0;
        for (int j2 = 0; j2 < g.Ntd; ++j2)
          for (int j1 = 0; j1 < g.Nsd; ++j1) {
            int k = g.Nsd * j2 + j1;
            g.lcoor2[2 * k] = std::cos(g.gth) * (g.lcoor[2 * k] - gmid0) -
                              std::sin(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid0;
            g.lcoor2[2 * k + 1] = std::sin(g.gth) * (g.lcoor[2 * k] - gmid0) +
                                  std::cos(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid1;
          }
      }
    }
  }
  if (irep == 1) g.inewlayerflg = 0;
}

// ---------------------------------------------------------------- orientations
// SampleOrientation (SampleOrientation.C:10-161): uniform rotations via the
// cube -> ball area-preserving map; output (omega, axis) per sample.
struct SampleConsts {
  double R1, a, aprime, beta, s2, s2q, s6pi, spi, s24, coeffA[7];
};
static SampleConsts sample_consts() {
  SampleConsts k;
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

// One rotation from three uniforms; `device_math` routes the transcendental
// calls through the selectable libm (nucleation happens inside the event loop).
static void orientation_from_uniforms(const SampleConsts &K, const double u[3], double out[4],
                                      bool device_math) {
  auto COS = [&](double x) { return device_math ? m_cos(x) : std::cos(x); };
  auto SIN = [&](double x) { return device_math ? m_sin(x) : std::sin(x); };
  auto ACOS = [&](double x) { return device_math ? m_acos(x) : std::acos(x); };
  auto POWH = [&](double x) { return device_math ? m_powh(x) : std::pow(x, 1.0 / 2.0); };
  auto POW2 = [&](double x) { return device_math ? m_pow2(x) : std::pow(x, 2); };
  auto POWE = [&](double x, int e) { return device_math ? m_pow_even(x, e) : std::pow(x, 2.0 * (e / 2)); };
  double xyz0[3] = {u[0] - .5, u[1] - .5, u[2] - .5};
  double xyz[3] = {K.aprime * xyz0[0], K.aprime * xyz0[1], K.aprime * xyz0[2]};
  int P[3] = {1, 2, 3};
  {  // GetPermutation (SampleOrientation.C:25-51): later tests override earlier ones
    double x = xyz[0], y = xyz[1], z = xyz[2];
    if ((std::fabs(x) <= z) && (std::fabs(y) <= z)) { P[0] = 1; P[1] = 2; P[2] = 3; }
    if ((z <= -std::fabs(x)) && (z <= -std::fabs(y))) { P[0] = -1; P[1] = 2; P[2] = -3; }
    if ((std::fabs(x) <= y) && (std::fabs(z) <= y)) { P[0] = 1; P[1] = -3; P[2] = 2; }
    if ((y <= -std::fabs(x)) && (y <= -std::fabs(z))) { P[0] = 1; P[1] = 3; P[2] = -2; }
    if ((std::fabs(z) < x) && (std::fabs(y) <= x)) { P[0] = -3; P[1] = 2; P[2] = 1; }
    if ((x <= -std::fabs(z)) && (x <= -std::fabs(y))) { P[0] = 3; P[1] = 2; P[2] = -1; }
  }
  double xyz2[3];
  for (int j = 0; j < 3; ++j) xyz2[j] = P[j] / std::abs(P[j]) * xyz[std::abs(P[j]) - 1];
  double m1[3];  // ComputeMap1 (:53-59)
  for (int j = 0; j < 3; ++j) m1[j] = K.a / K.aprime * xyz2[j];
  double m2[3];  // ComputeMap2 (:61-90)
  {
    double x = m1[0], y = m1[1], z = m1[2], T1 = 0, T2 = 0;
    if (std::fabs(y) <= std::fabs(x)) {
      if (std::fabs(x) < 1e-10) {
        T1 = 0.0;
        T2 = 0.0;
      } else {
        T1 = K.s2 * COS(y * M_PI / 12 / x) - 1;
        T2 = K.s2 * SIN(y * M_PI / 12 / x);
        T1 *= K.s2q * x / (K.beta * POWH(K.s2 - COS(y * M_PI / 12 / x)));
        T2 *= K.s2q * x / (K.beta * POWH(K.s2 - COS(y * M_PI / 12 / x)));
      }
    }
    if (std::fabs(x) <= std::fabs(y)) {
      if (std::fabs(y) < 1e-10) {
        T1 = 0.0;
        T2 = 0.0;
      } else {
        T1 = K.s2 * SIN(x * M_PI / 12 / y);
        T2 = K.s2 * COS(x * M_PI / 12 / y) - 1;
        T1 *= K.s2q * y / (K.beta * POWH(K.s2 - COS(x * M_PI / 12 / y)));
        T2 *= K.s2q * y / (K.beta * POWH(K.s2 - COS(x * M_PI / 12 / y)));
      }
    }
    m2[0] = T1;
    m2[1] = T2;
    m2[2] = z;
  }
  double m3[3];  // ComputeMap3 (:92-106)
  {
    double x = m2[0], y = m2[1], z = m2[2];
    if (std::fabs(z) < 1e-10) {
      m3[0] = m3[1] = m3[2] = 0;
    } else {
      // The compiled reference evaluates this pair of pow(q, 1.0/2.0) calls as
      // one vector square root (GCC's SLP vectorizer, -O2); the other
      // pow(., 1/2) calls of GenerateSamples stay glibc pow calls.
      double q = 1 - (POW2(x) + POW2(y)) * M_PI / (24 * POW2(z));
      double sq = std::sqrt(q);
      m3[0] = sq * x;
      m3[1] = sq * y;
      m3[2] = K.s6pi * z - (POW2(x) + POW2(y)) * K.spi / (K.s24 * z);
    }
  }
  double xyzb[3];
  for (int j = 0; j < 3; ++j) xyzb[std::abs(P[j]) - 1] = P[j] / std::abs(P[j]) * m3[j];
  double pmax = smax(smax(std::fabs(xyz0[0]), std::fabs(xyz0[1])), std::fabs(xyz0[2]));
  double rhoP = K.R1 * pmax / .5;
  double t = 1;
  for (int j = 1; j < 8; ++j) t += K.coeffA[j - 1] * POWE(rhoP, 2 * j);
  double omega = 2.0 * ACOS(t);
  double tnorm = POWH(POW2(xyzb[0]) + POW2(xyzb[1]) + POW2(xyzb[2]));
  out[0] = omega;
  out[1] = xyzb[0] / tnorm;
  out[2] = xyzb[1] / tnorm;
  out[3] = xyzb[2] / tnorm;
}


// GenerateSamples (SampleOrientation.C:124-161): engine seeded with seedL,
// three uniform variates per sample.
static void generate_samples(int n, unsigned int seedL, std::vector<double> &out, bool device_math) {
  static const SampleConsts K = sample_consts();
  std::uniform_real_distribution<double> xrand(0.0, 1.0);
  std::default_random_engine g1(seedL);
  out.assign(4 * (size_t)n, 0.0);
  for (int jn = 0; jn < n; ++jn) {
    double u[3];
    u[0] = xrand(g1);
    u[1] = xrand(g1);
    u[2] = xrand(g1);
    orientation_from_uniforms(K, u, &out[4 * (size_t)jn], device_math);
  }
}

// ---------------------------------------------------------------- Voronoi
// Nearest site with the reference's distance expression and first-minimum rule.
// sites: xyz triples; query point q. `dist` computes the rounded distance the
// reference computes. A bucket grid narrows the search; every site whose exact
// squared distance could round to a value <= the best found is examined.
struct SiteGrid {
  double lo[3], h;
  int nb[3];
  std::vector<int> start, idx;
  const std::vector<double> *sites;
};
static void site_grid_build(SiteGrid &G, const std::vector<double> &sites, const double lo[3],
                            const double hi[3]) {
  int n = (int)(sites.size() / 3);
  G.sites = &sites;
  double vol = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
  G.h = std::cbrt(vol / std::max(1, n)) * 1.5;
  for (int k = 0; k < 3; ++k) {
    G.lo[k] = lo[k];
    G.nb[k] = std::max(1, std::min(1024, (int)std::ceil((hi[k] - lo[k]) / G.h)));
  }
  size_t nbt = (size_t)G.nb[0] * G.nb[1] * G.nb[2];
  std::vector<int> cnt(nbt + 1, 0), cell(n);
  for (int i = 0; i < n; ++i) {
    int b[3];
    for (int k = 0; k < 3; ++k) {
      b[k] = (int)std::floor((sites[3 * i + k] - G.lo[k]) / G.h);
      b[k] = std::max(0, std::min(G.nb[k] - 1, b[k]));
    }
    cell[i] = (b[2] * G.nb[1] + b[1]) * G.nb[0] + b[0];
    cnt[cell[i] + 1]++;
  }
  for (size_t b = 0; b < nbt; ++b) cnt[b + 1] += cnt[b];
  G.start = cnt;
  G.idx.assign(n, 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n; ++i) G.idx[fill[cell[i]]++] = i;  // ascending site index per bucket
}
template <class Dist>
static int site_grid_nearest(const SiteGrid &G, const double q[3], Dist dist) {
  int qb[3];
  for (int k = 0; k < 3; ++k) {
    qb[k] = (int)std::floor((q[k] - G.lo[k]) / G.h);
    qb[k] = std::max(0, std::min(G.nb[k] - 1, qb[k]));
  }
  double best = INFINITY;
  int besti = -1;
  int rmax = std::max(G.nb[0], std::max(G.nb[1], G.nb[2]));
  for (int r = 0; r <= rmax; ++r) {
    if (besti >= 0) {
      // exact lower bound on the distance to any bucket of ring r
      double gap = (r - 1) * G.h;
      if (gap > 0 && gap * gap > best * (1.0 + 1e-9)) break;
    }
    for (int dz = -r; dz <= r; ++dz) {
      int bz = qb[2] + dz;
      if (bz < 0 || bz >= G.nb[2]) continue;
      for (int dy = -r; dy <= r; ++dy) {
        int by = qb[1] + dy;
        if (by < 0 || by >= G.nb[1]) continue;
        for (int dxx = -r; dxx <= r; ++dxx) {
          if (std::max(std::abs(dz), std::max(std::abs(dy), std::abs(dxx))) != r) continue;
          int bx = qb[0] + dxx;
          if (bx < 0 || bx >= G.nb[0]) continue;
          int b = (bz * G.nb[1] + by) * G.nb[0] + bx;
          for (int t = G.start[b]; t < G.start[b + 1]; ++t) {
            int i = G.idx[t];
            double d = dist(&(*G.sites)[3 * (size_t)i]);
            if (d < best || (d == best && i < besti)) {
              best = d;
              besti = i;
            }
          }
        }
      }
    }
  }
  return besti;
}

// ---------------------------------------------------------------- CA state
// Hard-coded seeds of the reference (VoxelsCA.C:47-49). The extension keyword
// "seed s" offsets both by (s - 1) * kSeedStride and seeds the baseplate
// engine with s (its default seed is 1), so s = 1 is the reference.
static const int kSeed0 = 2132512, kSeed1 = 2912351;
static const unsigned int kSeedStride = 10000019u;
static unsigned int seed0_of(const Grid &g) { return (unsigned int)kSeed0 + (unsigned int)(g.seed - 1) * kSeedStride; }
static unsigned int seed1_of(const Grid &g) { return (unsigned int)kSeed1 + (unsigned int)(g.seed - 1) * kSeedStride; }
struct State {
  Grid g;
  int N = 0, nx = 0, ny = 0, nz = 0, nxy = 0;
  std::vector<int> gID, vState, buildj, build;
  std::vector<double> extents, cen, temp, cTheta;
  int nGrain = 0, Nzh = 0;
  std::default_random_engine genlayer;
  // TempField (TempField.C:16-77)
  std::vector<int> ispvec;
  double DelT = 0, bmDX0 = 0, a1[6];
  // statistics
  long long n_events = 0, n_nuc = 0, max_na = 0, max_front = 0, n_steps = 0;
  long long n_negdt = 0, n_clamp = 0;  // events with DtMin < 0; extents clamped at 0 by them
  int tf_tInd = 0;  // TempField::tInd, set at the start of each step (main1.C:64)
};

static inline void cell_xyz(const State &S, int idx, int j[3]) {
  j[2] = idx / S.nxy;
  j[1] = (idx - S.nxy * j[2]) / S.nx;
  j[0] = idx - S.nxy * j[2] - S.nx * j[1];
}

// Moore neighbours of idx in ascending linear-index order (Grid.C:399-414, sorted at :375).
static inline int moore(const State &S, int idx, int out[26]) {
  int j[3];
  cell_xyz(S, idx, j);
  int n = 0;
  for (int dz = -1; dz <= 1; ++dz) {
    int z = j[2] + dz;
    if (z < 0 || z >= S.nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = j[1] + dy;
      if (y < 0 || y >= S.ny) continue;
      for (int dx = -1; dx <= 1; ++dx) {
        int x = j[0] + dx;
        if (x < 0 || x >= S.nx) continue;
        int k = S.nxy * z + S.nx * y + x;
        if (k != idx) out[n++] = k;
      }
    }
  }
  return n;
}

// BasePlate::GenerateVoxel (BasePlate.C:41-97) + VoxelsCA::InitializeVoxels (VoxelsCA.C:125-161).
static void init_baseplate(State &S) {
  Grid &g = S.g;
  S.Nzh = std::min(g.nX[2], int(std::ceil(g.bpH * .9999 / g.dX[2])));
  double height = S.Nzh * (g.dX[2]);
  std::default_random_engine generator((unsigned int)g.seed);  // BasePlate.h:28 (default seed 1)
  double rate = g.mu * (g.dX[0] * 1e6) * (g.dX[1] * 1e6) * g.nX[0] * g.nX[1] * (height * 1e6);
  std::poisson_distribution<int> ng(rate);
  int Ngrain = 0;
  while (Ngrain == 0) Ngrain = ng(generator);
  std::vector<double> Xsite(3 * (size_t)Ngrain);
  std::uniform_real_distribution<double> xrand(0.0, 1.0);
  double Lx = g.dX[0] * g.nX[0], Ly = g.dX[1] * g.nX[1];
  for (int j = 0; j < Ngrain; ++j) {
    Xsite[3 * j] = xrand(generator) * Lx;
    Xsite[3 * j + 1] = xrand(generator) * Ly;
    Xsite[3 * j + 2] = xrand(generator) * height;
  }
  SiteGrid G;
  double lo[3] = {0, 0, 0}, hi[3] = {Lx, Ly, std::max(height, g.dX[2])};
  site_grid_build(G, Xsite, lo, hi);
  int nbp = S.Nzh * S.nxy;
  for (int j = 0; j < nbp; ++j) {
    int c[3];
    cell_xyz(S, j, c);
    double q[3] = {(c[0] + .5) * g.dX[0], (c[1] + .5) * g.dX[1], (c[2] + .5) * g.dX[2]};
    int best = site_grid_nearest(G, q, [&](const double *X) {
      double a = q[0] - X[0], b = q[1] - X[1], d = q[2] - X[2];
      return a * a + b * b + d * d;
    });
    S.gID[j] = best + 1;
    S.vState[j] = (j < (S.Nzh - 1) * S.nxy) ? 3 : 2;
  }
  std::default_random_engine g1(531231);
  unsigned int sdloc = unsigned(double(g1()) / double(g1.max()) * std::pow(2.0, 32.0));
  generate_samples(Ngrain, sdloc, S.cTheta, false);
  S.nGrain = Ngrain;
  for (int j = 0; j < S.N; ++j) {
    if (S.gID[j] == 0) continue;
    int c[3];
    cell_xyz(S, j, c);
    S.cen[3 * (size_t)j] = (double(c[0]) + .5) * g.dX[0];
    S.cen[3 * (size_t)j + 1] = (double(c[1]) + .5) * g.dX[1];
    S.cen[3 * (size_t)j + 2] = (double(c[2]) + .5) * g.dX[2];
  }
}

// VoxelsCA::AddLayer1 (VoxelsCA.C:887-982).
static void add_layer(State &S) {
  Grid &g = S.g;
  unsigned int sdloc = unsigned(double(S.genlayer()) / double(S.genlayer.max()) * std::pow(2.0, 32.0));
  double rate = g.lrate * (g.dX[0] * 1e6) * (g.dX[1] * 1e6) * g.nX[0] * g.nX[1] * (g.layerT * 1e6);
  std::poisson_distribution<int> ng(rate);
  int ng2 = 0;
  while (ng2 == 0) ng2 = ng(S.genlayer);
  int iz1 = g.ilaserLoc - g.nZlayer;
  double zloc0 = iz1 * g.dX[2];
  std::vector<double> Xsite(3 * (size_t)ng2);
  std::uniform_real_distribution<double> xrand(0.0, 1.0);
  double Lx = g.nX[0] * g.dX[0], Ly = g.nX[1] * g.dX[1];
  for (int j = 0; j < ng2; ++j) {
    Xsite[3 * j] = xrand(S.genlayer) * Lx;
    Xsite[3 * j + 1] = xrand(S.genlayer) * Ly;
    Xsite[3 * j + 2] = xrand(S.genlayer) * g.layerT + zloc0;
  }
  int i3 = g.nX[0] * g.nX[1];
  std::vector<int> itmp(ng2, 0), gtmp((size_t)i3 * g.nZlayer, 0);
  SiteGrid G;
  double lo[3] = {0, 0, zloc0}, hi[3] = {Lx, Ly, zloc0 + std::max(g.layerT, g.dX[2])};
  site_grid_build(G, Xsite, lo, hi);
  for (int j3a = iz1; j3a < g.ilaserLoc; ++j3a)
    for (int j2a = 0; j2a < g.nX[1]; ++j2a)
      for (int j1a = 0; j1a < g.nX[0]; ++j1a) {
        double q[3] = {j1a * g.dX[0], j2a * g.dX[1], j3a * g.dX[2]};
        int i2 = site_grid_nearest(G, q, [&](const double *X) {
          double a = q[0] - X[0], b = q[1] - X[1], d = q[2] - X[2];
          return a * a + b * b + d * d;
        });
        int jind = i3 * (j3a - iz1) + g.nX[0] * j2a + j1a;
        gtmp[jind] = i2 + 1;
        itmp[i2] = 1;
      }
  int i2 = 0;
  for (int j = 0; j < ng2; ++j)
    if (itmp[j] == 1) {
      itmp[j] = i2;
      i2 += 1;
    }
  if (i2 != ng2)
    for (size_t j = 0; j < gtmp.size(); ++j) gtmp[j] = itmp[gtmp[j] - 1] + 1;
  for (int j = 0; j < S.N; ++j) {
    int j3 = j / i3;
    if (j3 >= iz1 && j3 < g.ilaserLoc) {
      int j2 = (j - i3 * j3) / g.nX[0];
      int j1 = j - i3 * j3 - g.nX[0] * j2;
      int jind = i3 * (j3 - iz1) + g.nX[0] * j2 + j1;
      S.gID[j] = S.nGrain + gtmp[jind];
      S.vState[j] = 3;
      S.cen[3 * (size_t)j] = (double(j1) + .5) * g.dX[0];
      S.cen[3 * (size_t)j + 1] = (double(j2) + .5) * g.dX[1];
      S.cen[3 * (size_t)j + 2] = (double(j3) + .5) * g.dX[2];
    }
  }
  S.nGrain += i2 + 1;
  std::vector<double> aa;
  generate_samples(i2 + 1, sdloc, aa, false);
  S.cTheta.insert(S.cTheta.end(), aa.begin(), aa.end());
  long iz = (long)g.nX[0] * g.nX[1] * g.ilaserLoc;
  for (int j = 0; j < S.N; ++j)
    if (j >= iz) {
      S.vState[j] = 0;
      S.gID[j] = 0;
    }
}

// VoxelsCA::CleanLayer (VoxelsCA.C:800-839).
static void clean_layer(State &S) {
  std::vector<long long> vol(S.nGrain, 0);
  for (int j = 0; j < S.N; ++j)
    if (S.gID[j] > 0) vol[S.gID[j] - 1]++;
  std::vector<int> newid(S.nGrain, 0);
  std::vector<double> ctmp;
  int k = 0;
  for (int j = 0; j < S.nGrain; ++j)
    if (vol[j] > 0) {
      for (int c = 0; c < 4; ++c) ctmp.push_back(S.cTheta[4 * (size_t)j + c]);
      newid[j] = ++k;
    }
  S.cTheta = ctmp;
  S.nGrain = k;
  for (int j = 0; j < S.N; ++j)
    if (S.gID[j] != 0) S.gID[j] = newid[S.gID[j] - 1];
}

// TempField ctor + InitializeAnalytic (TempField.C:16-77).
static void init_tempfield(State &S) {
  Grid &g = S.g;
  S.DelT = g.bmDelT;
  S.bmDX0 = S.DelT * g.bmV;
  S.ispvec.assign(g.NpT, 0);
  if (g.patternID == 1 || g.patternID == 3) std::iota(S.ispvec.begin(), S.ispvec.end(), 0);
  if (g.patternID == 2 || g.patternID == 4) {
    for (int j = 0; j < g.Ntd; ++j) {
      int k = g.Nsd * j;
      if (std::fmod(j, 2) == 0) {
        std::iota(S.ispvec.begin() + k, S.ispvec.begin() + k + g.Nsd, k);
      } else {
        for (int j1 = 0; j1 < g.Nsd; ++j1) S.ispvec[k + j1] = k + g.Nsd - 1 - j1;
      }
    }
  }
  S.a1[0] = g.meltparam[0];
  S.a1[1] = g.meltparam[2];
  S.a1[2] = g.meltparam[3];
  S.a1[3] = g.meltparam[1];
  S.a1[4] = S.a1[1];
  S.a1[5] = S.a1[2];
}

// TempField::AnalyticTempCurr (TempField.C:139-217).
static void analytic_temp(State &S) {
  Grid &g = S.g;
  std::fill(S.temp.begin(), S.temp.end(), g.T0);
  double xi = g.tL * (1 + std::numeric_limits<double>::epsilon());
  const int *isv = S.ispvec.data();
  double x = g.lcoor[2 * isv[g.isp]] - g.offset[0];
  double y = g.lcoor[2 * isv[g.isp] + 1] - g.offset[1];
  double z = g.ilaserLoc * g.dX[2] - g.offset[2];
  double cg = std::cos(g.gth), sg = std::sin(g.gth);
  double dirp;
  if (std::fmod(g.isp, g.Nsd) == 0)
    dirp = (g.lcoor[2 * isv[g.isp + 1]] - g.lcoor[2 * isv[g.isp]]);
  else
    dirp = (g.lcoor[2 * isv[g.isp]] - g.lcoor[2 * isv[g.isp - 1]]);
  for (int j = 0; j < S.N; ++j) {
    int c[3];
    cell_xyz(S, j, c);
    double x0 = (double(c[0]) + .5) * (g.dX[0]);
    double y0 = (double(c[1]) + .5) * (g.dX[1]);
    double zp = (double(c[2]) + .5) * (g.dX[2]);
    if (zp > z) continue;
    double xp = cg * (x0 - g.LX[0] / 2.) + sg * (y0 - g.LX[1] / 2.) + g.LX[0] / 2.;
    double yp = -sg * (x0 - g.LX[0] / 2.) + cg * (y0 - g.LX[1] / 2.) + g.LX[1] / 2.;
    double r0 = xp - x, r1 = yp - y, r2 = zp - z, dsq, T;
    if (dirp * r0 > 0) {
      double q1 = r1 / S.a1[1], q2 = r2 / S.a1[2];
      dsq = q1 * q1 + q2 * q2;
      T = (dsq < 1.0 && (std::fabs(r0) < S.bmDX0)) ? xi : g.tS;
    } else {
      double q0 = r0 / S.a1[3], q1 = r1 / S.a1[4], q2 = r2 / S.a1[5];
      dsq = q0 * q0 + q1 * q1 + q2 * q2;
      T = (dsq < 1.0) ? xi : g.tS;
    }
    S.temp[j] = T;
    if (T > g.tL)
      S.buildj[j] = 1;
    else if (T < g.T0)
      S.buildj[j] = 0;
  }
  double lx = g.lcoor2[2 * isv[g.isp]] - g.offset[0];
  double ly = g.lcoor2[2 * isv[g.isp] + 1] - g.offset[1];
  if (lx < g.gbox[0] || lx > g.gbox[1] || ly < g.gbox[2] || ly > g.gbox[3]) {
    int icheck = 0;
    for (int j = 0; j < S.N; ++j)
      if (S.temp[j] >= g.tL) {
        icheck = 1;
        break;
      }
    if (icheck == 0 || std::fmod(g.isp + 1, g.Nsd) == 0) g.inewscanflg = 1;
    if (g.isp == (g.NpT - 1)) {
      g.inewscanflg = 1;
      g.inewlayerflg = 1;
      g.isp = 0;
      g.indlayer += 1;
    }
  }
}

// ---------------------------------------------------------------- EASM
// TempField::EASM (TempField.C:79-137) with Utilities::EASM_Temp_LG, Integral,
// Temp_Fun_G and the 316L properties (Utilities.C:39-76, 105-140, 228-249).
// The 25-node Gauss-Legendre rule of the GSL call comes from
// cafe_quadrature.h, as in the reference built here (oracle/ref_shims).
static double m_exp(double x) {
  if (g_libm.mode == 1) return crm_exp(x);
  return perturb(std::exp(x));
}
// pow(x, -0.5)
static double m_pow_mhalf(double x) {
  if (g_libm.mode == 1) return crm_pow_mhalf(x);
  return perturb(std::pow(x, -0.5));
}
// pow(10, -e) of the property polynomials (correctly rounded: the decimal literal)
static double m_p10(int e) {
  if (g_libm.mode == 1) return e == 2 ? 1e-2 : e == 3 ? 1e-3 : e == 4 ? 1e-4 : 1e-5;
  return std::pow(10, -e);
}
// Utilities::Materials_316L: {cP, k, rho, alpha}
static void easm_materials(double T, double M[4]) {
  double rho, cP, k;
  if (T < 1660)
    rho = 8084.2 - 0.42086 * T - 3.8942 * m_p10(5) * T * T;
  else if (T >= 1660 && T < 3090)
    rho = 7432.7 + 3.9338 * m_p10(2) * T - 1.8007 * m_p10(4) * T * T;
  else
    rho = 6124.72;
  if (T < 1660)
    cP = 458.984 + 0.1328 * T;
  else
    cP = 769.855;
  if (T < 1660)
    k = 9.248 + 1.571 * m_p10(2) * T;
  else if (T >= 1660 && T < 3090)
    k = 12.41 + 3.279 * m_p10(3) * T;
  else
    k = 21.6465;
  M[0] = cP;
  M[1] = k;
  M[2] = rho;
  M[3] = k / (rho * cP);
}
struct EasmCtx {
  double L[3], R[3];
  double bmV, Q;
  double qx[25], qw[25];
};
// Utilities::Temp_Fun_G at time x of the integral (t = 8e-4 s)
static double easm_kernel(const EasmCtx &E, const double M[4], double x) {
  const double sigma = 50.0e-6, eta = 0.56, t = 80.0e-5;
  double C = eta * E.Q / (M_PI * M[2] * M[0] * std::sqrt(4 * M_PI * M[3]));
  double x0 = E.L[0] - E.bmV * t;
  double Lx = x0 + E.bmV * x;
  double Ly = E.L[1], Lz = E.L[2];
  double tx = t - x;
  double sig2 = m_pow2(sigma);
  double dx = E.R[0] - Lx, dy = E.R[1] - Ly, dz = std::fabs(E.R[2] - Lz);
  return C * m_pow_mhalf(tx) / (2 * M[3] * tx + sig2) *
         m_exp(-1 * (m_pow2(dx) + m_pow2(dy)) / (4 * M[3] * tx + 2 * sig2) - m_pow2(dz) / (4 * M[3] * tx));
}
// Utilities::Integral: 300 + sum_i w_i f(x_i)
static double easm_integral(const EasmCtx &E, double T) {
  double M[4];
  easm_materials(T, M);
  double s = 0.0;
  for (int i = 0; i < 25; ++i) s += E.qw[i] * easm_kernel(E, M, E.qx[i]);
  return 300 + s;
}
// Utilities::EASM_Temp_LG: damped fixed point on the property temperature
static double easm_temp_lg(const EasmCtx &E, double T) {
  double Told = T;
  int n = 0, nlim = 100;
  double tol = 10;
  double Tnew = easm_integral(E, T);
  while (std::fabs(Told - Tnew) > tol && n < nlim) {
    Told = Tnew;
    double T_temp = easm_integral(E, Told);
    Tnew = 0.5 * (Told + T_temp);
    n++;
  }
  return Tnew;
}
static void easm_temp(State &S) {
  Grid &g = S.g;
  std::fill(S.temp.begin(), S.temp.end(), 0.0);  // TempOut.assign(Ntot, 0)
  EasmCtx E;
  cafe_gauss_legendre(25, 0.0, 80.0e-5, E.qx, E.qw);
  E.bmV = g.bmV;
  E.Q = g.bmP;
  const int *isv = S.ispvec.data();
  double x = g.lcoor[2 * isv[g.isp]] - g.offset[0];
  double y = g.lcoor[2 * isv[g.isp] + 1] - g.offset[1];
  double z = g.ilaserLoc * g.dX[2] - g.offset[2];
  double cg = std::cos(g.gth), sg = std::sin(g.gth);
  E.L[0] = x;
  E.L[1] = y;
  E.L[2] = z;
  for (int j = 0; j < S.N; ++j) {
    int c[3];
    cell_xyz(S, j, c);
    double x0 = (double(c[0]) + .5) * (g.dX[0]);
    double y0 = (double(c[1]) + .5) * (g.dX[1]);
    double zp = (double(c[2]) + .5) * (g.dX[2]);
    if (zp > z) continue;
    double xp = cg * (x0 - g.LX[0] / 2.) + sg * (y0 - g.LX[1] / 2.) + g.LX[0] / 2.;
    double yp = -sg * (x0 - g.LX[0] / 2.) + cg * (y0 - g.LX[1] / 2.) + g.LX[1] / 2.;
    double T;
    if ((x0 > x) && (zp > (z - g.layerT))) {
      T = .99 * g.T0;
    } else {
      E.R[0] = xp;
      E.R[1] = yp;
      E.R[2] = zp;
      T = easm_temp_lg(E, S.temp[j]);
    }
    S.temp[j] = T;
    if (T > g.tL)
      S.buildj[j] = 1;
    else if (T < g.T0)
      S.buildj[j] = 0;
  }
  double lx = g.lcoor2[2 * isv[g.isp]] - g.offset[0];
  double ly = g.lcoor2[2 * isv[g.isp] + 1] - g.offset[1];
  if (lx < g.gbox[0] || lx > g.gbox[1] || ly < g.gbox[2] || ly > g.gbox[3]) {
    // all_of(T >= tL) here, where AnalyticTempCurr asks any_of
    int all = 1;
    for (int j = 0; j < S.N; ++j)
      if (!(S.temp[j] >= g.tL)) {
        all = 0;
        break;
      }
    if (all == 0 || std::fmod(g.isp + 1, g.Nsd) == 0) g.inewscanflg = 1;
    if (g.isp == (g.NpT - 1)) {
      g.inewscanflg = 1;
      g.inewlayerflg = 1;
      g.isp = 0;
      g.indlayer += 1;
    }
  }
}
// Extension "rosenthal eta k alpha" (no reference code): the Rosenthal
// solution for a point source of power eta P moving at v over a half space,
//   T = T0 + q / R exp(-c (R + xi)),  q = eta P / (2 pi k),  c = v / (2 alpha),
// in the laser frame of the analytic field (cell centres rotated by gth about
// the box centre, TempField.C:155-166), source at the laser point on the laser
// plane, xi the distance ahead of the source along the scan direction (the
// sign of the analytic field's dirp, TempField.C:167-171), R clamped below at
// half a voxel. Cells above the plane stay at T0. BuildjID and the
// end-of-scan check follow AnalyticTempCurr (TempField.C:180-216).
static void rosenthal_temp(State &S) {
  Grid &g = S.g;
  std::fill(S.temp.begin(), S.temp.end(), g.T0);
  const double pi = 3.14159265358979323846;
  const double q = g.ros_eta * g.bmP / (2.0 * pi * g.ros_k);
  const double c = g.bmV / (2.0 * g.ros_alpha);
  const double rmin = 0.5 * std::min(g.dX[0], std::min(g.dX[1], g.dX[2]));
  const int *isv = S.ispvec.data();
  double x = g.lcoor[2 * isv[g.isp]] - g.offset[0];
  double y = g.lcoor[2 * isv[g.isp] + 1] - g.offset[1];
  double z = g.ilaserLoc * g.dX[2] - g.offset[2];
  double cg = std::cos(g.gth), sg = std::sin(g.gth);
  double dirp;
  if (std::fmod(g.isp, g.Nsd) == 0)
    dirp = (g.lcoor[2 * isv[g.isp + 1]] - g.lcoor[2 * isv[g.isp]]);
  else
    dirp = (g.lcoor[2 * isv[g.isp]] - g.lcoor[2 * isv[g.isp - 1]]);
  const double sd = dirp > 0 ? 1.0 : (dirp < 0 ? -1.0 : 0.0);
  for (int j = 0; j < S.N; ++j) {
    int cc[3];
    cell_xyz(S, j, cc);
    double x0 = (double(cc[0]) + .5) * (g.dX[0]);
    double y0 = (double(cc[1]) + .5) * (g.dX[1]);
    double zp = (double(cc[2]) + .5) * (g.dX[2]);
    if (zp > z) continue;
    double xp = cg * (x0 - g.LX[0] / 2.) + sg * (y0 - g.LX[1] / 2.) + g.LX[0] / 2.;
    double yp = -sg * (x0 - g.LX[0] / 2.) + cg * (y0 - g.LX[1] / 2.) + g.LX[1] / 2.;
    double r0 = xp - x, r1 = yp - y, r2 = zp - z;
    double R = std::sqrt(r0 * r0 + r1 * r1 + r2 * r2);
    if (R < rmin) R = rmin;
    double xi = sd * r0;
    double T = g.T0 + q / R * m_exp(-(c * (R + xi)));
    S.temp[j] = T;
    if (T > g.tL)
      S.buildj[j] = 1;
    else if (T < g.T0)
      S.buildj[j] = 0;
  }
  double lx = g.lcoor2[2 * isv[g.isp]] - g.offset[0];
  double ly = g.lcoor2[2 * isv[g.isp] + 1] - g.offset[1];
  if (lx < g.gbox[0] || lx > g.gbox[1] || ly < g.gbox[2] || ly > g.gbox[3]) {
    int icheck = 0;
    for (int j = 0; j < S.N; ++j)
      if (S.temp[j] >= g.tL) {
        icheck = 1;
        break;
      }
    if (icheck == 0 || std::fmod(g.isp + 1, g.Nsd) == 0) g.inewscanflg = 1;
    if (g.isp == (g.NpT - 1)) {
      g.inewscanflg = 1;
      g.inewlayerflg = 1;
      g.isp = 0;
      g.indlayer += 1;
    }
  }
}

// main1.C:65-70: EASM when Grid::EASM_Flag is 1, else the analytic field (or
// the Rosenthal extension)
static void temperature(State &S) {
  if (S.g.EASM_Flag == 1)
    easm_temp(S);
  else if (S.g.rosenthal)
    rosenthal_temp(S);
  else
    analytic_temp(S);
}

// VoxelsCA::ConvertSolid1 (VoxelsCA.C:712-799), two-phase.
static void convert_solid(State &S, int iswitch) {
  std::vector<int> hit;
  int nb[26];
  for (int j = 0; j < S.N; ++j) {
    if (iswitch == 0 ? S.vState[j] != 2 : S.vState[j] != 3) continue;
    int n = moore(S, j, nb);
    bool ok = (iswitch == 0);
    for (int k = 0; k < n; ++k) {
      int v = S.vState[nb[k]];
      if (iswitch == 0 && v < 2) { ok = false; break; }
      if (iswitch == 1 && v == 1) { ok = true; break; }
    }
    if (ok) hit.push_back(j);
  }
  for (int j : hit) {
    if (iswitch == 0) {
      S.vState[j] = 3;
      S.extents[j] = 0.0;
    } else {
      S.vState[j] = 2;
    }
  }
}

// loadRotMat (VoxelsCA.h:94-107) for grain gid (1-based).
static void rot_matrix(const State &S, int gid, double R[3][3]) {
  const double *c = &S.cTheta[4 * (size_t)(gid - 1)];
  double omega = c[0], ax[3] = {c[1], c[2], c[3]};
  double co = m_cos(omega), so = m_sin(omega);
  R[0][0] = co + m_pow2(ax[0]) * (1 - co);
  R[0][1] = ax[0] * ax[1] * (1 - co) - ax[2] * so;
  R[0][2] = ax[0] * ax[2] * (1 - co) + ax[1] * so;
  R[1][0] = ax[0] * ax[1] * (1 - co) + ax[2] * so;
  R[1][1] = co + m_pow2(ax[1]) * (1 - co);
  R[1][2] = ax[1] * ax[2] * (1 - co) - ax[0] * so;
  R[2][0] = ax[2] * ax[0] * (1 - co) - ax[1] * so;
  R[2][1] = ax[2] * ax[1] * (1 - co) + ax[0] * so;
  R[2][2] = co + m_pow2(ax[2]) * (1 - co);
}

// Capture-time numerator for capturing octahedron (centre cen, rotation R) and
// neighbour cell nidx (VoxelsCA.C:409-424 without the "- ExtA").
static double candidate_g(const State &S, const double cen[3], const double R[3][3], int nidx) {
  int jx[3];
  cell_xyz(S, nidx, jx);
  double dnx[3];
  for (int k = 0; k < 3; ++k) dnx[k] = (double(jx[k]) + .5) * S.g.dX[k] - cen[k];
  double th = m_atan2(std::fabs(dnx[1]), std::fabs(dnx[0]));
  th = th > M_PI / 4.0 ? M_PI / 2.0 - th : th;
  double ph = m_atan2(m_powh(m_pow2(dnx[0]) + m_pow2(dnx[1])), std::fabs(dnx[2]));
  ph = ph < M_PI / 4.0 ? M_PI / 2.0 - ph : ph;
  double d0 = std::fabs(R[0][0] * dnx[0] + R[1][0] * dnx[1] + R[2][0] * dnx[2]);
  double d1 = std::fabs(R[0][1] * dnx[0] + R[1][1] * dnx[1] + R[2][1] * dnx[2]);
  double d2 = std::fabs(R[0][2] * dnx[0] + R[1][2] * dnx[1] + R[2][2] * dnx[2]);
  return m_powh(m_cos(th) * m_sin(ph)) * (d0 + d1 + d2);
}

// projectPointLine (VoxelsCA.h:78-93).
static void project_point_line(const double *A, const double *x0, const double *x1, double *xp) {
  double n[3];
  double snorm = m_powh(m_pow2(x1[0] - x0[0]) + m_pow2(x1[1] - x0[1]) + m_pow2(x1[2] - x0[2]));
  n[0] = (x1[0] - x0[0]) / snorm;
  n[1] = (x1[1] - x0[1]) / snorm;
  n[2] = (x1[2] - x0[2]) / snorm;
  double d = -(n[0] * A[0] + n[1] * A[1] + n[2] * A[2]);
  double t = (-d - n[0] * x0[0] - n[1] * x0[1] - n[2] * x0[2]) /
             (n[0] * (x1[0] - x0[0]) + n[1] * (x1[1] - x0[1]) + n[2] * (x1[2] - x0[2]));
  xp[0] = x0[0] + (x1[0] - x0[0]) * t;
  xp[1] = x0[1] + (x1[1] - x0[1]) * t;
  xp[2] = x0[2] + (x1[2] - x0[2]) * t;
}

// Decentered-octahedron capture (VoxelsCA.C:528-605): new half-diagonal and
// centre of captured cell icap from capturing cell (index jsidx, centre cjs, R).
static void capture_geometry(const State &S, int icap, int jsidx, const double cjs[3],
                             const double R[3][3], double *ext_out, double cen_out[3]) {
  static const double S0[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
  static const int SI[8][3] = {{0, 1, 2}, {1, 2, 3}, {0, 2, 4}, {2, 3, 4},
                               {0, 1, 5}, {1, 3, 5}, {0, 4, 5}, {3, 4, 5}};
  const double *dX = S.g.dX;
  int jx[3], jy[3];
  cell_xyz(S, icap, jx);
  cell_xyz(S, jsidx, jy);
  double l = m_powh(m_pow2((jx[0] - jy[0]) * dX[0]) + m_pow2((jx[1] - jy[1]) * dX[1]) +
                    m_pow2((jx[2] - jy[2]) * dX[2]));
  double dnx[3], locX[3];
  for (int k = 0; k < 3; ++k) dnx[k] = (double(jx[k]) + .5) * dX[k] - cjs[k];
  locX[0] = R[0][0] * dnx[0] + R[1][0] * dnx[1] + R[2][0] * dnx[2];
  locX[1] = R[0][1] * dnx[0] + R[1][1] * dnx[1] + R[2][1] * dnx[2];
  locX[2] = R[0][2] * dnx[0] + R[1][2] * dnx[1] + R[2][2] * dnx[2];
  double th = m_atan2(std::fabs(dnx[1]), std::fabs(dnx[0]));
  th = th > M_PI / 4.0 ? M_PI / 2.0 - th : th;
  double ph = m_atan2(m_powh(m_pow2(dnx[0]) + m_pow2(dnx[1])), std::fabs(dnx[2]));
  ph = ph < M_PI / 4.0 ? M_PI / 2.0 - ph : ph;
  double dr = std::fabs(locX[0]) + std::fabs(locX[1]) + std::fabs(locX[2]);
  double sd[6][3];
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 3; ++b) sd[a][b] = S0[a][b] * dr;
  int jInd = 4 * std::signbit(locX[2]) + 2 * std::signbit(locX[1]) + std::signbit(locX[0]);
  double dnorm[3];
  for (int a = 0; a < 3; ++a) {
    const double *c = sd[SI[jInd][a]];
    dnorm[a] = m_pow2(locX[0] - c[0]) + m_pow2(locX[1] - c[1]) + m_pow2(locX[2] - c[2]);
  }
  int imin = 0, imax = 0;  // std::min_element / std::max_element: first extreme
  for (int a = 1; a < 3; ++a) {
    if (dnorm[a] < dnorm[imin]) imin = a;
    if (dnorm[imax] < dnorm[a]) imax = a;
  }
  int k0, k1, k2;
  if (imin == imax) {
    k0 = 0;
    k1 = 1;
    k2 = 2;
  } else {
    k0 = imin;
    k2 = imax;
    k1 = 3 - imin - imax;
  }
  const double *p0 = sd[SI[jInd][k0]], *p1 = sd[SI[jInd][k1]], *p2 = sd[SI[jInd][k2]];
  double xI[3], xJ[3];
  project_point_line(locX, p0, p1, xI);
  project_point_line(locX, p0, p2, xJ);
  double d1I = m_powh(m_pow2(p0[0] - xI[0]) + m_pow2(p0[1] - xI[1]) + m_pow2(p0[2] - xI[2]));
  double dI2 = m_powh(m_pow2(p1[0] - xI[0]) + m_pow2(p1[1] - xI[1]) + m_pow2(p1[2] - xI[2]));
  double d1J = m_powh(m_pow2(p0[0] - xJ[0]) + m_pow2(p0[1] - xJ[1]) + m_pow2(p0[2] - xJ[2]));
  double dJ3 = m_powh(m_pow2(p2[0] - xJ[0]) + m_pow2(p2[1] - xJ[1]) + m_pow2(p2[2] - xJ[2]));
  static const double s3 = std::pow(3.0, .5), s23 = std::pow(2.0 / 3.0, .5);
  double L12 = .5 * (smin(d1I, s3 * l) + smin(dI2, s3 * l));
  double L13 = .5 * (smin(d1J, s3 * l) + smin(dJ3, s3 * l));
  double Lmud = s3 * (s23 * smax(L12, L13));
  double xiL = 1.0;
  *ext_out = m_powh(m_cos(th) * m_sin(ph)) * Lmud * xiL;
  const double *s0 = S0[SI[jInd][k0]];
  double dn2[3];
  for (int k = 0; k < 3; ++k) dn2[k] = p0[k] - Lmud * s0[k];
  double loc2[3];
  loc2[0] = R[0][0] * dn2[0] + R[0][1] * dn2[1] + R[0][2] * dn2[2];
  loc2[1] = R[1][0] * dn2[0] + R[1][1] * dn2[1] + R[1][2] * dn2[2];
  loc2[2] = R[2][0] * dn2[0] + R[2][1] * dn2[1] + R[2][2] * dn2[2];
  for (int k = 0; k < 3; ++k) cen_out[k] = cjs[k] + loc2[k];
}

// VoxelsCA::UpdateVoxels (VoxelsCA.C:232-655) at world size 1.
static void update_voxels(State &S) {
  Grid &g = S.g;
  const double tL = g.tL;
  // SetLiquid3 (VoxelsCA.C:1098-1116)
  {
    long iz1 = (long)g.ilaserLoc * S.nxy;
    for (int j = 0; j < S.N; ++j) {
      if (S.temp[j] >= tL) {
        if (j < S.nxy) {
          S.vState[j] = 2;
        } else if (j < iz1) {
          S.vState[j] = 1;
          S.gID[j] = 0;
        }
        S.extents[j] = 0.0;
      }
    }
  }
  convert_solid(S, 1);
  // active set (VoxelsCA.C:262-275)
  std::vector<int> vI;
  {
    int nb[26];
    for (int j = 0; j < S.N; ++j) {
      if (S.vState[j] == 2 || (S.vState[j] == 1 && S.temp[j] < tL)) {
        vI.push_back(j);
        int n = moore(S, j, nb);
        for (int k = 0; k < n; ++k)
          if (S.temp[nb[k]] >= tL) vI.push_back(nb[k]);
      }
    }
    std::sort(vI.begin(), vI.end());
    vI.erase(std::unique(vI.begin(), vI.end()), vI.end());
  }
  const int Na = (int)vI.size();
  S.max_na = std::max<long long>(S.max_na, Na);
  std::vector<int> vS(Na), G(Na);
  std::vector<double> T(Na), ExtA(Na), CenA(3 * (size_t)Na);
  for (int p = 0; p < Na; ++p) {
    int i = vI[p];
    vS[p] = S.vState[i];
    G[p] = S.gID[i];
    T[p] = S.temp[i];
    ExtA[p] = S.extents[i];
    for (int k = 0; k < 3; ++k) CenA[3 * (size_t)p + k] = S.cen[3 * (size_t)i + k];
  }
  // neighbour CSR into the active list (VoxelsCA.C:304-335)
  std::vector<int> nptr(Na + 1, 0), nid;
  nid.reserve(26 * (size_t)Na);
  {
    int nb[26];
    for (int p = 0; p < Na; ++p) {
      nptr[p] = (int)nid.size();
      int n = moore(S, vI[p], nb);
      for (int k = 0; k < n; ++k) {
        auto it = std::lower_bound(vI.begin(), vI.end(), nb[k]);
        if (it != vI.end() && *it == nb[k]) nid.push_back((int)(it - vI.begin()));
      }
    }
    nptr[Na] = (int)nid.size();
  }
  unsigned int sdloc = seed0_of(g) + 32 * g.tInd + 64 * S.nGrain;
  std::default_random_engine g1(30 * g.tInd + seed1_of(g));
  std::uniform_real_distribution<double> xrand1(0.0, 1.0);
  double rX = g.rNmax * std::pow(g.dX[0] * 1e6, 3.);
  std::vector<int> vs2ind;
  vs2ind.reserve(Na);
  for (int p = 0; p < Na; ++p)
    if (vS[p] == 2) vs2ind.push_back(p);
  int vSind2 = (int)vs2ind.size();
  std::vector<double> ruq(Na);
  for (int j = 0; j < Na; ++j) ruq[j] = (xrand1(g1) - .5) * g.dX[0] / 100.;
  // per-position bookkeeping: liquid-neighbour count and the all-cold test
  std::vector<int> liq(Na, 0);
  std::vector<char> cold(Na, 1);
  for (int p = 0; p < Na; ++p)
    for (int t = nptr[p]; t < nptr[p + 1]; ++t) {
      if (vS[nid[t]] == 1) liq[p]++;
      if (!(T[nid[t]] < tL)) cold[p] = 0;
    }
  // per-position growth velocity (VoxelsCA.C:405)
  // (the device evaluates the per-cell velocities of the EASM and Rosenthal
  // fields as correctly rounded integer powers)
  const bool cr_pow = g_libm.mode == 1 && (g.EASM_Flag == 1 || g.rosenthal) && g.nvel >= 1 && g.nvel <= 64 &&
                      g.nvel == (int)g.nvel;
  auto vhat_of = [&](int p) {
    if (T[p] >= tL) return 0.0;
    return g.Avel * (cr_pow ? crm_pow_int(tL - T[p], (int)g.nvel) : std::pow(tL - T[p], g.nvel));
  };
  // frontier: indices j into vs2ind with a liquid neighbour and all-cold neighbours
  std::vector<int> fr;
  for (int j = 0; j < vSind2; ++j)
    if (liq[vs2ind[j]] > 0 && cold[vs2ind[j]]) fr.push_back(j);
  // candidate numerator cache, per (position, slot)
  std::vector<double> gcache(nid.size(), NAN);
  std::vector<char> gvalid(nid.size(), 0);
  std::vector<double> vh(Na, 0.0);
  int countS = Na;
  double tinc = 0.0;
  long long nev = 0;
  while (vSind2 != countS && tinc < S.DelT) {
    countS = vSind2;
    double DtMin = 1e6, ruqflag = 1000;
    int js = -1, j1s = -1;
    size_t nfr = fr.size();
    S.max_front = std::max<long long>(S.max_front, (long long)nfr);
    for (size_t f = 0; f < nfr; ++f) {
      int i1 = vs2ind[fr[f]];
      double v = vhat_of(i1);
      vh[i1] = v;
      double Rm[3][3];
      bool have_R = false;
      int i5 = nptr[i1], i6 = nptr[i1 + 1] - i5;
      for (int j1 = 0; j1 < i6; ++j1) {
        int i4 = nid[i5 + j1];
        if (vS[i4] != 1) continue;
        if (!gvalid[i5 + j1]) {
          if (!have_R) {
            rot_matrix(S, G[i1], Rm);
            have_R = true;
          }
          gcache[i5 + j1] = candidate_g(S, &CenA[3 * (size_t)i1], Rm, vI[i4]);
          gvalid[i5 + j1] = 1;
        }
        double dr = gcache[i5 + j1] - ExtA[i1];
        double timeUntil = dr / v;
        double ruqs = .5 * (ruq[i1] + ruq[i4]);
        if (timeUntil <= DtMin) {
          if (timeUntil < DtMin) {
            DtMin = timeUntil;
            js = i1;
            j1s = j1;
            ruqflag = ruqs;
          } else if (ruqs < ruqflag) {
            DtMin = timeUntil;
            js = i1;
            j1s = j1;
            ruqflag = ruqs;
          }
        }
      }
    }
    if (DtMin >= 1e6 || js < 0) break;
    ++nev;
    int icap = nid[nptr[js] + j1s];
    // extension "nucgauss": rX exp(-.5 x1^2) with the captured cell's
    // undercooling, the form of VoxelsCA.C:2545-2548
    double rXe = rX;
    if (g.nuc_gauss) {
      double x1 = ((tL - T[icap]) - g.nuc_mean) / g.nuc_sd / 1.4142135623730951;
      rXe = rX * m_exp(-.5 * (x1 * x1));
    }
    if (xrand1(g1) < rXe) {
      // nucleation (VoxelsCA.C:483-505)
      std::vector<double> q;
      generate_samples(1, sdloc, q, true);
      vS[icap] = 2;
      vs2ind.push_back(icap);
      vSind2 += 1;
      S.nGrain += 1;
      G[icap] = S.nGrain;
      S.cTheta.insert(S.cTheta.end(), q.begin(), q.end());
      int jx[3];
      cell_xyz(S, vI[icap], jx);
      for (int k = 0; k < 3; ++k) CenA[3 * (size_t)icap + k] = (double(jx[k]) + .5) * g.dX[k];
      sdloc += 10;
      DtMin = 0.0;
      ExtA[icap] = 0.0;
      S.n_nuc++;
    } else {
      // growth of every mushy cell in the list (VoxelsCA.C:511-516)
      if (DtMin < 0.0) S.n_negdt++;
      if (std::isfinite(DtMin)) {
        for (size_t f = 0; f < nfr; ++f) {
          int i1 = vs2ind[fr[f]];
          ExtA[i1] += vh[i1] * DtMin;
          if (ExtA[i1] < 0.0) S.n_clamp++;
          ExtA[i1] = smax(ExtA[i1], 0.0);
        }
      } else {
        std::vector<char> infr(vs2ind.size(), 0);
        for (size_t f = 0; f < nfr; ++f) infr[fr[f]] = 1;
        for (int j = 0; j < countS; ++j) {
          int i1 = vs2ind[j];
          double v = infr[j] ? vh[i1] : 0.0;
          ExtA[i1] += v * DtMin;
          ExtA[i1] = smax(ExtA[i1], 0.0);
        }
      }
      vS[icap] = 2;
      vs2ind.push_back(icap);
      vSind2 += 1;
      G[icap] = G[js];
      double Rm[3][3], ext, cn[3];
      rot_matrix(S, G[js], Rm);
      capture_geometry(S, vI[icap], vI[js], &CenA[3 * (size_t)js], Rm, &ext, cn);
      ExtA[icap] = ext;
      for (int k = 0; k < 3; ++k) CenA[3 * (size_t)icap + k] = cn[k];
    }
    // bookkeeping for the next iteration: icap is no longer liquid
    for (int t = nptr[icap]; t < nptr[icap + 1]; ++t) liq[nid[t]]--;
    {
      std::vector<int> fr2;
      fr2.reserve(fr.size() + 1);
      for (int j : fr)
        if (liq[vs2ind[j]] > 0) fr2.push_back(j);
      if (liq[icap] > 0 && cold[icap]) fr2.push_back(vSind2 - 1);
      fr.swap(fr2);
    }
    tinc += DtMin;
  }
  S.n_events += nev;
  // write back (VoxelsCA.C:633-643)
  for (int p = 0; p < Na; ++p) {
    int i = vI[p];
    S.vState[i] = vS[p];
    S.gID[i] = G[p];
    S.extents[i] = ExtA[p];
    for (int k = 0; k < 3; ++k) S.cen[3 * (size_t)i + k] = CenA[3 * (size_t)p + k];
  }
  convert_solid(S, 0);
}


static void put_i32(FILE *fp, int32_t v) { std::fwrite(&v, 4, 1, fp); }
static void put_f64(FILE *fp, double v) { std::fwrite(&v, 8, 1, fp); }

// Same record layout as oracle/ref_driver.cpp (read by oracle/cafe_dump.py).
static void dump_state(FILE *fp, int tag, const State &S) {
  if (!fp) return;
  const Grid &g = S.g;
  put_i32(fp, 0x43414645);
  put_i32(fp, tag);
  put_i32(fp, S.tf_tInd);
  put_i32(fp, S.nGrain);
  put_i32(fp, S.N);
  put_i32(fp, g.isp);
  put_i32(fp, g.indlayer);
  put_i32(fp, g.inewlayerflg);
  put_i32(fp, g.inewscanflg);
  put_f64(fp, g.time);
  std::fwrite(S.gID.data(), 4, S.N, fp);
  std::fwrite(S.vState.data(), 4, S.N, fp);
  std::fwrite(S.extents.data(), 8, S.N, fp);
  std::fwrite(S.cen.data(), 8, 3 * (size_t)S.N, fp);
  std::fwrite(S.temp.data(), 8, S.N, fp);
  std::fwrite(S.buildj.data(), 4, S.N, fp);
  std::fwrite(S.cTheta.data(), 8, 4 * (size_t)S.nGrain, fp);
}

// VoxelsCA::SetBuild(TempField::BuildjID) (VoxelsCA.C:76-115): every voxel
// of a grain that has a melted voxel (BuildjID = 1) or a Build voxel becomes
// Build = 1; Build is never reset. (The reference's lists of grain IDs, with
// consecutive repeats removed, hold every grain that occurs, so membership is
// a per-grain flag.)
static void set_build(State &S) {
  std::vector<char> g1(S.nGrain + 2, 0), g2(S.nGrain + 2, 0);
  for (int j = 0; j < S.N; ++j)
    if (S.buildj[j] == 1 && S.gID[j] > 0) g1[S.gID[j]] = 1;
  for (int j = 0; j < S.N; ++j)
    if (S.gID[j] > 0 && g1[S.gID[j]]) S.build[j] = 1;
  for (int j = 0; j < S.N; ++j)
    if (S.build[j] == 1 && S.gID[j] > 0) g2[S.gID[j]] = 1;
  for (int j = 0; j < S.N; ++j)
    if (S.gID[j] > 0 && g2[S.gID[j]]) S.build[j] = 1;
}

// ---------------------------------------------------------------- output
// Inverse-pole-figure colouring of VoxelsCA::WriteToHDF1 (VoxelsCA.C:1592-
// 1810) for one grain: RGB (as floats) of the sample z (build), x and y
// directions in the crystal frame. The constants of the colour triangle come
// from the same expressions as the reference's; `hx` carries the hue of the x
// direction into the y direction, where the reference adds to it instead of
// starting from the y direction's own hue, and the hue fraction is H/6 as the
// reference writes it.
struct IpfConsts {
  double x0, y0, sMax, hoff;  // hoff = atan((triPts[1][2]-y0)/(triPts[0][2]-x0))*180/M_PI
};
static IpfConsts ipf_consts() {
  double tp[2][3] = {{0.0, 2. / std::pow(2, .5) / (1. + 1. / std::pow(2, .5)),
                      2. / std::pow(3, .5) / (1. + 1. / std::pow(3, .5))},
                     {0.0, 0.0, 2. / std::pow(3, .5) / (1. + 1. / std::pow(3, .5))}};
  double m = std::tan(1. / 2. * std::atan2(tp[1][2], tp[0][2]));
  double a = std::pow(std::pow(tp[1][2] - tp[1][1], 2.) + std::pow(tp[0][2] - tp[0][1], 2.), .5);
  double b = std::pow(std::pow(tp[0][1], 2.) + std::pow(tp[1][1], 2.), 0.5);
  double c = std::pow(std::pow(tp[0][2], 2.) + std::pow(tp[1][2], 2.), 0.5);
  IpfConsts K;
  K.y0 = 1. / 2. * std::pow((b + c - a) * (c + a - b) * (a + b - c) / (a + b + c), .5);
  K.x0 = K.y0 / m;
  K.sMax = std::pow(std::pow(K.x0, 2.) + std::pow(K.y0, 2.), .5);
  K.hoff = std::atan((tp[1][2] - K.y0) / (tp[0][2] - K.x0)) * 180 / M_PI;
  return K;
}
static double m_atan(double x) {
  if (g_libm.mode == 1) return crm_atan2(x, 1.0);
  return perturb(std::atan(x));
}
// one direction: H enters as the hue to start from when !own_hue
static void ipf_dir(const IpfConsts &K, const double R[3][3], const double v[3], bool own_hue, double &H,
                    float rgb[3]) {
  double vCD[3];
  vCD[0] = std::fabs(R[0][0] * v[0] + R[1][0] * v[1] + R[2][0] * v[2]);
  vCD[1] = std::fabs(R[0][1] * v[0] + R[1][1] * v[1] + R[2][1] * v[2]);
  vCD[2] = std::fabs(R[0][2] * v[0] + R[1][2] * v[1] + R[2][2] * v[2]);
  std::sort(vCD, vCD + 3);
  std::swap(vCD[0], vCD[1]);
  vCD[2] = smin(vCD[2], 1.0);
  double xp = 2. * vCD[0] / (1. + vCD[2]);
  double yp = 2. * vCD[1] / (1. + vCD[2]);
  if (own_hue) {
    H = m_atan((yp - K.y0) / (xp - K.x0)) * 180. / M_PI;
    if (xp < K.x0) H += 180;
  }
  H = H + 240 - K.hoff;
  double V = 1.;
  double S = m_powh(m_pow2(xp - K.x0) + m_pow2(yp - K.y0));
  S = S / K.sMax * 0.8 + 0.2;
  if (H >= 360.0) H = 0.0;
  int icase = (int)std::floor(H / 60.0);
  double ff = H / 6.0 - icase;
  double p = V * (1. - S), q = V * (1. - S * ff), t = V * (1. - (S * (1. - ff)));
  rgb[0] = rgb[1] = rgb[2] = 0.0f;
  if (S <= 0.0) return;
  double r = 0, gg = 0, bb = 0;
  bool set = true;
  switch (icase) {
    case 0: r = V; gg = t; bb = p; break;
    case 1: r = q; gg = V; bb = p; break;
    case 2: r = p; gg = V; bb = t; break;
    case 3: r = p; gg = q; bb = V; break;
    case 4: r = t; gg = p; bb = V; break;
    case 5: r = V; gg = p; bb = q; break;
    default: set = false;
  }
  if (set) {
    rgb[0] = (float)r;
    rgb[1] = (float)gg;
    rgb[2] = (float)bb;
  }
}
// rotation of WriteToHDF1 (VoxelsCA.C:1635-1644), with pow(a, 2.0)
static void ipf_rot(const double *c, double R[3][3]) {
  double omega = c[0], ax[3] = {c[1], c[2], c[3]};
  R[0][0] = m_cos(omega) + m_pow2(ax[0]) * (1 - m_cos(omega));
  R[0][1] = ax[0] * ax[1] * (1 - m_cos(omega)) - ax[2] * m_sin(omega);
  R[0][2] = ax[0] * ax[2] * (1 - m_cos(omega)) + ax[1] * m_sin(omega);
  R[1][0] = ax[0] * ax[1] * (1 - m_cos(omega)) + ax[2] * m_sin(omega);
  R[1][1] = m_cos(omega) + m_pow2(ax[1]) * (1 - m_cos(omega));
  R[1][2] = ax[1] * ax[2] * (1 - m_cos(omega)) - ax[0] * m_sin(omega);
  R[2][0] = ax[2] * ax[0] * (1 - m_cos(omega)) - ax[1] * m_sin(omega);
  R[2][1] = ax[2] * ax[1] * (1 - m_cos(omega)) + ax[0] * m_sin(omega);
  R[2][2] = m_cos(omega) + m_pow2(ax[2]) * (1 - m_cos(omega));
}
// IPF colours of grains 1..ngrain (9 floats per grain: z, x, y directions).
static void ipf_grains(const std::vector<double> &cTheta, int ngrain, std::vector<float> &out) {
  IpfConsts K = ipf_consts();
  out.assign(9 * (size_t)ngrain, 0.0f);
  const double vz[3] = {0.0, 0.0, 1.0}, vx[3] = {1.0, 0.0, 0.0}, vy[3] = {0.0, 1.0, 0.0};
  for (int g = 0; g < ngrain; ++g) {
    double R[3][3], H = 0.0;
    ipf_rot(&cTheta[4 * (size_t)g], R);
    ipf_dir(K, R, vz, true, H, &out[9 * (size_t)g]);
    ipf_dir(K, R, vx, true, H, &out[9 * (size_t)g + 3]);
    ipf_dir(K, R, vy, false, H, &out[9 * (size_t)g + 6]);
  }
}

static std::string g_out_dir;  // output directory (empty: no output)
static long g_out_every = 1;

static void write_bin(const std::string &path, const void *p, size_t bytes) {
  FILE *fp = std::fopen(path.c_str(), "wb");
  if (!fp) return;
  std::fwrite(p, 1, bytes, fp);
  std::fclose(fp);
}
// The datasets of WriteToHDF1 (VoxelsCA.C:1822-1854) as raw files
// <dir>/<name>.h5.<dataset>.bin.
static void write_output(const State &S, const std::string &name) {
  const std::string b = g_out_dir + "/" + name + ".h5.";
  std::vector<float> ipf;
  ipf_grains(S.cTheta, S.nGrain, ipf);
  std::vector<float> z(3 * (size_t)S.N, 0.0f), x(3 * (size_t)S.N, 0.0f), y(3 * (size_t)S.N, 0.0f), T(S.N);
  for (int j = 0; j < S.N; ++j) {
    T[j] = (float)S.temp[j];
    int g = S.gID[j];
    if (g < 1) continue;
    for (int a = 0; a < 3; ++a) {
      z[3 * (size_t)j + a] = ipf[9 * (size_t)(g - 1) + a];
      x[3 * (size_t)j + a] = ipf[9 * (size_t)(g - 1) + 3 + a];
      y[3 * (size_t)j + a] = ipf[9 * (size_t)(g - 1) + 6 + a];
    }
  }
  std::vector<float> cth(S.cTheta.begin(), S.cTheta.begin() + 4 * (size_t)S.nGrain);
  write_bin(b + "gID.bin", S.gID.data(), 4 * (size_t)S.N);
  write_bin(b + "vState.bin", S.vState.data(), 4 * (size_t)S.N);
  write_bin(b + "Build.bin", S.build.data(), 4 * (size_t)S.N);
  write_bin(b + "Temperature.bin", T.data(), 4 * (size_t)S.N);
  write_bin(b + "IPFz.bin", z.data(), 12 * (size_t)S.N);
  write_bin(b + "IPFx.bin", x.data(), 12 * (size_t)S.N);
  write_bin(b + "IPFy.bin", y.data(), 12 * (size_t)S.N);
  write_bin(b + "angleAxis.bin", cth.data(), 4 * cth.size());
}

static int setup(State &S, const char *deck) {
  std::string err;
  if (!read_deck(deck, S.g, err)) {
    std::fprintf(stderr, "oracle: %s: %s\n", deck, err.c_str());
    return 1;
  }
  grid_derive(S.g);
  S.nx = S.g.nX[0];
  S.ny = S.g.nX[1];
  S.nz = S.g.nX[2];
  S.nxy = S.nx * S.ny;
  S.N = S.nxy * S.nz;
  S.gID.assign(S.N, 0);
  S.vState.assign(S.N, 0);
  S.buildj.assign(S.N, 0);
  S.build.assign(S.N, 0);  // VoxelsCA::Build (VoxelsCA.C:43)
  S.extents.assign(S.N, 0.0);
  S.cen.assign(3 * (size_t)S.N, 0.0);
  S.temp.assign(S.N, 0.0);
  S.genlayer.seed(seed1_of(S.g));
  init_tempfield(S);
  init_baseplate(S);
  // every baseplate cell with a grain starts as Build (VoxelsCA.C:156-159)
  for (int k = 0; k < S.N; ++k)
    if (S.gID[k] != 0) S.build[k] = 1;
  return 0;
}

}  // namespace orc

using namespace orc;

// Wall-clock budget for the loops below (0 = none); set by cafe_oracle_set_budget.
static double g_max_seconds = 0.0;

extern "C" {

void cafe_oracle_set_budget(double seconds) { g_max_seconds = seconds; }
// 0: cafe_oracle_run_window leaves its input arrays untouched (they may be
// read-only mappings shared by several processes); 1 (default): the state
// reached is copied back into them.
static int g_window_writeback = 1;
void cafe_oracle_set_window_writeback(int on) { g_window_writeback = on != 0; }

// Output of the following cafe_oracle_run calls: the datasets of
// VoxelsCA::WriteToHDF1 as raw files <dir>/out<tInd>.h5.<name>.bin at every
// `every`-th output point and <dir>/final.h5.<name>.bin after the closing
// CleanLayer; dir NULL or empty turns output off.
void cafe_oracle_set_output(const char *dir, long every) {
  g_out_dir = dir ? dir : "";
  g_out_every = every > 0 ? every : 1;
}

// Runs the whole main1.C time loop on deck `deck`. dump_stride: 0 = write only
// the initial and final records, k > 0 = also every k-th step. max_steps > 0
// stops early. stats (may be NULL, else 10 entries) receives
// {steps, events, nucleations, max active-list size, max frontier, nGrain, N,
// loop nanoseconds, events with DtMin < 0, extents those clamped at 0}.
int cafe_oracle_run(const char *deck, const char *dump_path, long max_steps, int dump_stride,
                    int libm_mode, double perturb_p, unsigned long long perturb_seed,
                    long long *stats) {
  g_libm.mode = libm_mode;
  g_libm.p = perturb_p;
  g_libm.s = perturb_seed ? perturb_seed : 0x9e3779b97f4a7c15ull;
  State S;
  if (setup(S, deck)) return 1;
  FILE *fp = dump_path && dump_path[0] ? std::fopen(dump_path, "wb") : nullptr;
  Grid &g = S.g;
  int nlayerTot = int(std::ceil((double)(g.nX[2] - S.Nzh) / (double)g.nZlayer));
  bool bcheck = false;
  add_layer(S);
  update_laser(g);
  dump_state(fp, 0, S);
  long nstep = 0;
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  while (!bcheck) {
    S.tf_tInd = int(std::round(g.time / S.DelT));
    temperature(S);
    update_voxels(S);
    update_laser(g);
    bcheck = g.indlayer > nlayerTot;
    if (g.inewlayerflg == 1) clean_layer(S);
    // output point of main1.C:76-84: SetBuild, then WriteToHDF1
    if (S.tf_tInd % g.outint == 0 || bcheck || (g.inewlayerflg == 1 && g.outNL == 0)) {
      set_build(S);
      if (!g_out_dir.empty() && (nstep + 1) % g_out_every == 0) write_output(S, "out" + std::to_string(S.tf_tInd));
    }
    // UpdateTime2 (Grid.C:334-339)
    g.time += S.DelT;
    g.tInd += 1;
    if (g.inewlayerflg == 1) add_layer(S);
    ++nstep;
    S.n_steps = nstep;
    if (dump_stride > 0 && nstep % dump_stride == 0) dump_state(fp, 1, S);
    if (max_steps > 0 && nstep >= max_steps) break;
    if (g_max_seconds > 0) {
      clock_gettime(CLOCK_MONOTONIC, &t1);
      if ((t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec) > g_max_seconds) break;
    }
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (bcheck) {
    clean_layer(S);
    if (!g_out_dir.empty()) write_output(S, "final");  // main1.C:95-97
    dump_state(fp, 2, S);
  } else if (dump_stride <= 0 || nstep % dump_stride != 0) {
    dump_state(fp, 1, S);
  }
  if (fp) std::fclose(fp);
  if (stats) {
    stats[0] = S.n_steps;
    stats[1] = S.n_events;
    stats[2] = S.n_nuc;
    stats[3] = S.max_na;
    stats[4] = S.max_front;
    stats[5] = S.nGrain;
    stats[6] = S.N;
    stats[7] = (long long)((t1.tv_sec - t0.tv_sec) * 1000000000LL + (t1.tv_nsec - t0.tv_nsec));
    stats[8] = S.n_negdt;
    stats[9] = S.n_clamp;
  }
  return 0;
}

// Grid/TempField/VoxelsCA scalars of a running simulation (for resuming).
struct cafe_oracle_window {
  int isp, inewscanflg, inewlayerflg, indlayer, ilaserLoc, tInd;
  double time, gth;
  unsigned int genlayer_state;
  int ngrain;
};

// Runs `nsteps` loop iterations of `deck` starting from the given state (the
// arrays have N = nx*ny*nz entries; centroid holds x,y,z per cell), without
// the initial baseplate/layer construction. Wall seconds of the loop go to
// *seconds. The final state is written back into the arrays (if non-NULL);
// stats (may be NULL, else 10 entries) as for cafe_oracle_run, without the
// loop nanoseconds (entry 7).
int cafe_oracle_run_window(const char *deck, const cafe_oracle_window *w, int32_t *gID, int32_t *vState,
                           double *ext, double *cen, int32_t *buildj, double *cth, long nsteps,
                           int libm_mode, double *seconds, long long *stats, int *ngrain_out) {
  g_libm.mode = libm_mode;
  State S;
  std::string err;
  if (!read_deck(deck, S.g, err)) {
    std::fprintf(stderr, "oracle: %s: %s\n", deck, err.c_str());
    return 1;
  }
  grid_derive(S.g);
  S.nx = S.g.nX[0];
  S.ny = S.g.nX[1];
  S.nz = S.g.nX[2];
  S.nxy = S.nx * S.ny;
  S.N = S.nxy * S.nz;
  S.Nzh = std::min(S.g.nX[2], int(std::ceil(S.g.bpH * .9999 / S.g.dX[2])));
  init_tempfield(S);
  Grid &g = S.g;
  g.isp = w->isp;
  g.inewscanflg = w->inewscanflg;
  g.inewlayerflg = w->inewlayerflg;
  g.indlayer = w->indlayer;
  g.ilaserLoc = w->ilaserLoc;
  g.tInd = w->tInd;
  g.time = w->time;
  g.gth = w->gth;
  {
    double gmid0 = g.LX[0] / 2., gmid1 = g.LX[1] / 2.;
    for (int k = 0; k < g.NpT; ++k) {
      g.lcoor2[2 * k] = std::cos(g.gth) * (g.lcoor[2 * k] - gmid0) - std::sin(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid0;
      g.lcoor2[2 * k + 1] = std::sin(g.gth) * (g.lcoor[2 * k] - gmid0) + std::cos(g.gth) * (g.lcoor[2 * k + 1] - gmid1) + gmid1;
    }
  }
  S.genlayer.seed(w->genlayer_state);
  S.nGrain = w->ngrain;
  S.gID.assign(gID, gID + S.N);
  S.vState.assign(vState, vState + S.N);
  S.buildj.assign(buildj, buildj + S.N);
  S.extents.assign(ext, ext + S.N);
  S.cen.assign(cen, cen + 3 * (size_t)S.N);
  S.temp.assign(S.N, 0.0);
  S.cTheta.assign(cth, cth + 4 * (size_t)w->ngrain);
  int nlayerTot = int(std::ceil((double)(g.nX[2] - S.Nzh) / (double)g.nZlayer));
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  long n = 0;
  bool bcheck = false;
  while (!bcheck && n < nsteps) {
    if (g_max_seconds > 0) {
      clock_gettime(CLOCK_MONOTONIC, &t1);
      if ((t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec) > g_max_seconds) break;
    }
    S.tf_tInd = int(std::round(g.time / S.DelT));
    temperature(S);
    update_voxels(S);
    update_laser(g);
    bcheck = g.indlayer > nlayerTot;
    if (g.inewlayerflg == 1) clean_layer(S);
    g.time += S.DelT;
    g.tInd += 1;
    if (g.inewlayerflg == 1) add_layer(S);
    ++n;
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (seconds) *seconds = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
  if (stats) {
    stats[0] = n;
    stats[1] = S.n_events;
    stats[2] = S.n_nuc;
    stats[3] = S.max_na;
    stats[4] = S.max_front;
    stats[5] = S.nGrain;
    stats[6] = S.N;
    stats[8] = S.n_negdt;
    stats[9] = S.n_clamp;
  }
  if (ngrain_out) *ngrain_out = S.nGrain;
  if (!g_window_writeback) return 0;
  std::memcpy(gID, S.gID.data(), S.N * sizeof(int32_t));
  std::memcpy(vState, S.vState.data(), S.N * sizeof(int32_t));
  std::memcpy(buildj, S.buildj.data(), S.N * sizeof(int32_t));
  std::memcpy(ext, S.extents.data(), S.N * sizeof(double));
  std::memcpy(cen, S.cen.data(), 3 * (size_t)S.N * sizeof(double));
  return 0;
}

// n uniform variates of std::uniform_real_distribution<double>(0,1) on
// std::default_random_engine(seed), after skipping `skip` variates.
void cafe_oracle_std_uniforms(unsigned int seed, long skip, long n, double *out) {
  std::default_random_engine e(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  for (long i = 0; i < skip; ++i) u(e);
  for (long i = 0; i < n; ++i) out[i] = u(e);
}

// GenerateSamples(n, seed) restated; libm_mode selects the transcendental functions.
void cafe_oracle_orientations(unsigned int seed, int n, int libm_mode, double *out) {
  g_libm.mode = libm_mode;
  std::vector<double> v;
  generate_samples(n, seed, v, true);
  std::memcpy(out, v.data(), v.size() * sizeof(double));
  g_libm.mode = 0;
}

// Rotation matrix of one axis-angle orientation (loadRotMat), row-major.
void cafe_oracle_rotmat(const double *cth4, int libm_mode, double *R9) {
  g_libm.mode = libm_mode;
  State S;
  S.cTheta.assign(cth4, cth4 + 4);
  double R[3][3];
  rot_matrix(S, 1, R);
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) R9[3 * a + b] = R[a][b];
  g_libm.mode = 0;
}

}  // extern "C"

// Device-side data structures and per-cell physics of the CA step.
//
// Layout in HBM (one realisation, N = nx*ny*nz cells, x fastest):
//   state  u8[N]   vState (0 powder/empty, 1 liquid, 2 mushy, 3 solid)
//   gid    i32[N]  grain ID (0 = none)
//   ext    f64[N]  octahedron half-diagonal ("extents")
//   cx,cy,cz f64[N] octahedron centre ("centroidOct"), structure of arrays
//   buildj u8[N]   TempField::BuildjID (sticky "was above liquidus")
//   pos_of i32[N]  position of a cell in this step's active list, -1 otherwise
// Grain table: cth f64[4*G] (axis-angle, cTheta) and rot f64[9*G] (loadRotMat).
// Active list (sorted cell indices, the reference's vI) and per-position
// copies (vS, G, T class, ExtA, CentroidA, ruq, neighbour positions) are sized
// by the active capacity.
#ifndef CAFE_DEVICE_CUH
#define CAFE_DEVICE_CUH
#include <stdint.h>

#include "cafe_crmath.h"
#include "cafe_rng.h"

#define CAFE_NSLOT 26

// Error bits written to CafeDev::err by device code.
enum {
  CAFE_ERR_ACTIVE_CAP = 1,
  CAFE_ERR_ROW_CAP = 2,
  CAFE_ERR_GRAIN_CAP = 4,
  CAFE_ERR_MUSHY_CAP = 8,
  CAFE_ERR_ITER_CAP = 16,
  CAFE_ERR_SYNC = 32,  // a bounded wait between the event loop's two blocks ran out
};

// The new-row fill that the event loop's main block hands to its helper
// block (k_event_loop with two blocks): the row, the captured cell's active
// position, the event, the cell's grain, centre and extent, the time, and
// the helper's result (the order key of the row's largest |g|).
struct CafeFillReq {
  int r, p, e, gid;
  double c[3], ext, T;
  unsigned long long gk;
};

// Scalars that change every step (computed on the host from Grid/TempField).
struct CafeStepParams {
  double lx, ly, lz;  // laser x, y (scan frame) and the laser plane height
  double cg, sg;      // cos(gth), sin(gth) (host libm, as TempField.C:163-166)
  double dirp;        // scan direction sign source (TempField.C:167-171)
  int lo[3], hi[3];   // cell box ("pool box") outside which T cannot reach the liquidus
  int plo[3], phi[3]; // pool box of the previous step (liquid cells may remain there)
  int kabove;         // first z index with cell centre above the laser plane (T = T0)
  int ilaserLoc;
  int tInd;           // Grid::tInd (seeds of VoxelsCA.C:338-340)
  int any_hot_full;   // 1: evaluate T exactly everywhere below the plane
};

// Constants of the inverse-pole-figure colour triangle of
// VoxelsCA::WriteToHDF1 (VoxelsCA.C:1597-1613), computed on the host.
struct CafeIpfConsts {
  double x0, y0, sMax;
  double hoff;  // atan((triPts[1][2]-y0)/(triPts[0][2]-x0))*180/M_PI
};

// Scalars fixed for a run.
struct CafeConsts {
  int nx, ny, nz, nxy;
  long long N;
  double dx[3];
  double hLX0, hLX1;  // LX/2
  double a1[6];       // TempField::a1 (TempField.C:69-76)
  double bmDX0;       // DelT * bmV
  double tL, tS, T0, xi;
  double Tcls[3];     // temperature per class: 0 = T0 (above laser plane), 1 = tS, 2 = xi
  double vhat_cls[3]; // growth velocity per class (VoxelsCA.C:405), host libm pow
  int hot_cls[3];     // T >= tL
  int gt_cls[3];      // T > tL (BuildjID)
  double rX;          // rNmax * pow(dx*1e6, 3)
  double DelT;
  double ruq_dx;      // dX[0]
  unsigned int seed0, seed1;
  // SampleOrientation constants (SampleOrientation.C:15-22)
  double so_R1, so_a, so_aprime, so_beta, so_s2, so_s2q, so_s6pi, so_spi, so_s24, so_coeffA[7];
  double s3, s23;     // pow(3,.5), pow(2/3,.5) (VoxelsCA.C:583-585)
  // a per-cell temperature field (EASM, TempField::EASM, or the Rosenthal
  // extension): temperatures in CafeDev::temp, per-cell growth velocities in
  // CafeDev::a_vh; tmodel 1 = EASM, 2 = Rosenthal (0 = the analytic field)
  int easm;
  int tmodel;
  // Rosenthal extension: T = T0 + ros_q / R exp(-ros_c (R + xi)), R >= ros_rmin
  double ros_q, ros_c, ros_rmin;
  double Avel;        // Grid::Avel
  int nvel_i;         // Grid::nvel (an integer when easm)
  // Gaussian-undercooling nucleation (extension keyword "nucgauss mean sd")
  int nuc_gauss;
  double nuc_mean, nuc_sd;
};

// Tables of the EASM temperature (TempField.C:79-137, Utilities.C:105-140,
// 228-249), computed on the host: the 25-node Gauss-Legendre rule on
// [0, 8e-4 s], t - x_i and (t - x_i)^(-1/2) per node.
#define CAFE_EASM_NODES 25
// A cell whose fixed point has not converged after CAFE_EASM_LANE_INTEGRALS
// integrals in the lane-per-cell pass continues in the warp-per-cell pass.
#define CAFE_EASM_LANE_INTEGRALS 4
struct CafeEasmItem {
  long long idx;
  double Told, Tnew;
  int n, pad;
};
struct CafeEasm {
  double qw[CAFE_EASM_NODES], qx[CAFE_EASM_NODES], tx[CAFE_EASM_NODES], r[CAFE_EASM_NODES];
  double bmV, Q, layerT;
};

struct CafeDev {
  // dense fields
  uint8_t *state;
  int32_t *gid;
  double *ext, *cx, *cy, *cz;
  uint8_t *buildj;
  int32_t *pos_of;
  // temperature class of every cell of the pool box, written by k_melt
  uint8_t *tcls;
  long long tcls_cap;
  // VoxelsCA::Build (0/1 per cell)
  uint8_t *build;
  // EASM mode: TempField::TempCurr per cell, growth velocity per active position
  double *temp, *a_vh;
  // EASM cells handed from the lane-per-cell pass to the warp-per-cell pass
  struct CafeEasmItem *easm_q;
  long long easm_qcap;
  // growth log (cafe_sim_set_growth_log): per frontier row of each step its
  // cell, the step's Grid::tInd and its growth time (extent gained / velocity);
  // caller-owned device arrays, glog_cap entries, NULL when off
  int32_t *glog_cell, *glog_step;
  double *glog_tau;
  long long glog_cap;
  // this step's parameters (the kernels of a step read them from here)
  CafeStepParams *Pd;
  // activity flags of the compaction, one word per thread of the counting
  // pass (bit c: its c-th cell), reused by the scattering pass
  uint32_t *act_flags;
  // liquid cells left by the previous step (cell indices)
  int32_t *liq;
  // grains
  double *cth, *rot;
  int grain_cap;
  // active list and per-position copies
  int32_t *act;
  long long act_cap;
  uint8_t *a_state, *a_cls, *a_nn, *a_cold;
  int32_t *a_gid, *a_liq, *a_frow, *a_nbr;
  double *a_ext, *a_cx, *a_cy, *a_cz, *a_ruq;
  // mushy list (vs2ind) and frontier rows
  int32_t *vs2;
  long long vs2_cap;
  int32_t *row_pos, *row_j;
  uint8_t *row_alive, *row_ord;
  uint32_t *row_live;
  double *row_g;
  // per (row, slot): extent and centre (x, y, z) given to the neighbour when
  // this slot captures it, 4 doubles
  double *row_geo;
  long long row_cap;
  // (row, slot) pairs whose capture geometry the row set-up evaluates, as
  // row * 32 + slot, row_cap * CAFE_NSLOT entries
  int32_t *row_pairs;
  // rows during the event loop: row_E is the row cell's extent (ExtA)
  // including the growth of events 1..row_m, copied back to a_ext afterwards;
  // a row grows at the events (birth, row_death]; row_key orders the rows by
  // estimated absolute capture time; row_b* hold the exact best candidate of
  // the iteration row_stamp (row_bq: the position that slot captures);
  // row_key2 is the key of the row's smallest candidate time apart from slot
  // row_bslot at that evaluation, the row's key once that slot is captured
  // by another row
  double *row_E;
  int32_t *row_m, *row_death, *row_stamp, *row_bslot, *row_bq;
  unsigned long long *row_key, *row_key2;
  double *row_bt, *row_bruq;
  // per-event growth: ev_vd[e] = fl(v * DtMin_e) (+0 for a nucleation),
  // ev_vs[e] = running sum of ev_vd
  double *ev_vd, *ev_vs;
  long long ev_cap;
  // scan scratch
  int32_t *blk;       // per-block counts / offsets
  long long blk_cap;
  // the event loop's fill hand-off: the request, and two sequence numbers
  // (posted by the main block, done by the helper; zeroed before each launch)
  CafeFillReq *fill;
  int *fill_seq;
  // device scalars
  int *ctr;           // see CTR_* below
  int *err;
  unsigned long long *stat;  // event statistics
};

enum {
  CTR_NA = 0,      // active-list length
  CTR_NVS2,        // mushy-list length at step start
  CTR_NROWS,       // frontier rows at step start
  CTR_NGRAIN,      // grains in the table
  CTR_HOT,         // any T >= tL this step
  CTR_NEV,         // events this step
  CTR_NNUC,        // nucleations this step
  CTR_NVS2_END,    // mushy-list length after the event loop
  CTR_NLIQ,        // liquid cells listed by the last write-back
  CTR_SLOW,        // 1: this step's rows do not share one growth velocity
  CTR_NROWS_END,   // frontier rows after the event loop
  CTR_NPAIRS,      // (row, slot) pairs listed for the row set-up
  CTR_EASM_BOX,    // 6 slots: box of the cells at or above the liquidus (EASM)
  CTR_EASM_COLD = CTR_EASM_BOX + 6,  // 1: some cell below the liquidus (EASM)
  CTR_EASM_CURSOR = CTR_EASM_COLD + 2,  // 2 slots, 8-byte aligned: next cell of the EASM field
  CTR_EASM_QN = CTR_EASM_CURSOR + 2,    // cells queued for the warp-per-cell pass
  CTR_EASM_QHEAD,                       // next queued cell to take
  CTR_GLOG_N,                           // growth-log entries written
  CTR_GLOG_OVER,                        // 1: the growth log ran out of room
  CTR_ZLO, CTR_ZHI,                     // z range of the mushy and liquid cells after the last step
  CTR_COUNT
};
static_assert(CTR_EASM_CURSOR % 2 == 0, "64-bit cursor needs an 8-byte aligned slot");
enum { STAT_EVENTS = 0, STAT_NUC, STAT_MAXNA, STAT_MAXROWS, STAT_STEPS, STAT_NEGDT, STAT_SUMNA, STAT_SUMROWS,
       STAT_SLOWSTEPS, STAT_EVALS, STAT_CYC_SELECT, STAT_CYC_APPLY, STAT_CYC_FILL, STAT_CYC_OTHER,
       STAT_EASM_INTEGRALS, STAT_DETAIL, STAT_COUNT = STAT_DETAIL + 32 };

// --------------------------------------------------------------- temperature
// TempField::AnalyticTempCurr (TempField.C:155-190) for one cell; returns the
// class 0 (T0, above the laser plane), 1 (tS) or 2 (xi = tL(1+eps)).
__device__ __forceinline__ int cafe_temp_class_exact(const CafeConsts &K, const CafeStepParams &P, int i,
                                               int j, int k) {
  double zp = ((double)k + .5) * K.dx[2];
  if (zp > P.lz) return 0;
  if (!P.any_hot_full &&
      (i < P.lo[0] || i >= P.hi[0] || j < P.lo[1] || j >= P.hi[1] || k < P.lo[2] || k >= P.hi[2]))
    return 1;
  double x0 = ((double)i + .5) * K.dx[0];
  double y0 = ((double)j + .5) * K.dx[1];
  double xp = P.cg * (x0 - K.hLX0) + P.sg * (y0 - K.hLX1) + K.hLX0;
  double yp = -P.sg * (x0 - K.hLX0) + P.cg * (y0 - K.hLX1) + K.hLX1;
  double r0 = xp - P.lx, r1 = yp - P.ly, r2 = zp - P.lz;
  bool in;
  if (P.dirp * r0 > 0) {
    double q1 = r1 / K.a1[1], q2 = r2 / K.a1[2];
    double dsq = q1 * q1 + q2 * q2;
    in = (dsq < 1.0) && (fabs(r0) < K.bmDX0);
  } else {
    double q0 = r0 / K.a1[3], q1 = r1 / K.a1[4], q2 = r2 / K.a1[5];
    double dsq = q0 * q0 + q1 * q1 + q2 * q2;
    in = dsq < 1.0;
  }
  return in ? 2 : 1;
}

// Extension "rosenthal eta k alpha": the Rosenthal moving point source at the
// laser point (laser frame of the analytic field, TempField.C:155-166), xi the
// distance ahead of it along the scan direction (the sign of dirp), R clamped
// below at half a voxel; cells above the laser plane keep T0. The operation
// order is the oracle's (no contraction).
__device__ __forceinline__ double cafe_rosenthal_T(const CafeConsts &K, const CafeStepParams &P, int i, int j,
                                                   int k) {
  double zp = ((double)k + .5) * K.dx[2];
  if (zp > P.lz) return K.T0;
  double x0 = ((double)i + .5) * K.dx[0];
  double y0 = ((double)j + .5) * K.dx[1];
  double xp = P.cg * (x0 - K.hLX0) + P.sg * (y0 - K.hLX1) + K.hLX0;
  double yp = -P.sg * (x0 - K.hLX0) + P.cg * (y0 - K.hLX1) + K.hLX1;
  double r0 = xp - P.lx, r1 = yp - P.ly, r2 = zp - P.lz;
  double R = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
  if (R < K.ros_rmin) R = K.ros_rmin;
  double sd = P.dirp > 0 ? 1.0 : (P.dirp < 0 ? -1.0 : 0.0);
  double xi = sd * r0;
  return K.T0 + K.ros_q / R * crm_exp(-(K.ros_c * (R + xi)));
}

__device__ __forceinline__ void cafe_cell_xyz(const CafeConsts &K, long long idx, int &i, int &j,
                                              int &k) {
  // N < 2^31 (checked on the host), so 32-bit unsigned division suffices
  unsigned int u = (unsigned int)idx, nxy = (unsigned int)K.nxy, nx = (unsigned int)K.nx;
  unsigned int kk = u / nxy, r = u - kk * nxy, jj = r / nx;
  k = (int)kk;
  j = (int)jj;
  i = (int)(r - jj * nx);
}

// Temperature class of a cell from the per-step class map (integer work only):
// above the laser plane T0, outside the pool box tS, inside it the class that
// k_melt computed with cafe_temp_class_exact.
__device__ __forceinline__ int cafe_cls(const CafeDev &D, const CafeStepParams &P, int i, int j, int k) {
  if (k >= P.kabove) return 0;
  if (i < P.lo[0] || i >= P.hi[0] || j < P.lo[1] || j >= P.hi[1] || k < P.lo[2] || k >= P.hi[2]) return 1;
  long long bx = P.hi[0] - P.lo[0], by = P.hi[1] - P.lo[1];
  return D.tcls[((long long)(k - P.lo[2]) * by + (j - P.lo[1])) * bx + (i - P.lo[0])];
}

// --------------------------------------------------------------- geometry
// loadRotMat (VoxelsCA.h:94-107), row-major R[3*a+b].
__device__ __forceinline__ void cafe_rot_from_cth(const double *c, double *R) {
  double omega = c[0], a0 = c[1], a1 = c[2], a2 = c[3];
  double co = crm_cos(omega), so = crm_sin(omega);
  R[0] = co + (a0 * a0) * (1 - co);
  R[1] = a0 * a1 * (1 - co) - a2 * so;
  R[2] = a0 * a2 * (1 - co) + a1 * so;
  R[3] = a0 * a1 * (1 - co) + a2 * so;
  R[4] = co + (a1 * a1) * (1 - co);
  R[5] = a1 * a2 * (1 - co) - a0 * so;
  R[6] = a2 * a0 * (1 - co) - a1 * so;
  R[7] = a2 * a1 * (1 - co) + a0 * so;
  R[8] = co + (a2 * a2) * (1 - co);
}

// One neighbour slot of a capturing cell: the capturing cell (si,sj,sk) with
// octahedron centre cs and rotation R, the liquid neighbour (ci,cj,ck).
// g: the capture-time numerator pow(cos th sin ph,.5)*|R^T dn|_1
// (VoxelsCA.C:409-424, without "- ExtA"); ext and cen: the extent and centre
// the neighbour receives if this slot captures it (the decentered octahedron
// construction, VoxelsCA.C:528-605). Both parts share dn, th, ph and R^T dn,
// which the reference evaluates with identical expressions at the two places.
//
// The computation is split into parts with no data dependence between them
// (the th and ph chains, the two point-line projections) so that the event
// loop can run them in different warps; cafe_capture_geometry runs them all in
// one thread. Every part is the same expression sequence wherever it runs.
__device__ __forceinline__ void cafe_geo_dn(const CafeConsts &K, int ci, int cj, int ck, const double *cs,
                                            double *dn) {
  dn[0] = ((double)ci + .5) * K.dx[0] - cs[0];
  dn[1] = ((double)cj + .5) * K.dx[1] - cs[1];
  dn[2] = ((double)ck + .5) * K.dx[2] - cs[2];
}
// cos(th), th = atan2(|dy|,|dx|) folded at pi/4
__device__ __forceinline__ double cafe_geo_costh(const double *dn) {
  const double pi4 = 3.14159265358979323846 / 4.0, pi2 = 3.14159265358979323846 / 2.0;
  double th = crm_atan2(fabs(dn[1]), fabs(dn[0]));
  th = th > pi4 ? pi2 - th : th;
  return crm_cos(th);
}
// sin(ph), ph = atan2(sqrt(dx^2+dy^2),|dz|) folded at pi/4
__device__ __forceinline__ double cafe_geo_sinph(const double *dn) {
  const double pi4 = 3.14159265358979323846 / 4.0, pi2 = 3.14159265358979323846 / 2.0;
  double ph = crm_atan2(crm_pow_half(dn[0] * dn[0] + dn[1] * dn[1]), fabs(dn[2]));
  ph = ph < pi4 ? pi2 - ph : ph;
  return crm_sin(ph);
}
// distance between the capturing and the captured cell centres
__device__ __forceinline__ double cafe_geo_l(const CafeConsts &K, int ci, int cj, int ck, int si, int sj,
                                             int sk) {
  double q0 = (ci - si) * K.dx[0], q1 = (cj - sj) * K.dx[1], q2 = (ck - sk) * K.dx[2];
  return crm_pow_half(q0 * q0 + q1 * q1 + q2 * q2);
}
// dn in the crystal frame, R^T dn, and its 1-norm
__device__ __forceinline__ double cafe_geo_loc(const double *R, const double *dn, double *loc) {
  loc[0] = R[0] * dn[0] + R[3] * dn[1] + R[6] * dn[2];
  loc[1] = R[1] * dn[0] + R[4] * dn[1] + R[7] * dn[2];
  loc[2] = R[2] * dn[0] + R[5] * dn[1] + R[8] * dn[2];
  return fabs(loc[0]) + fabs(loc[1]) + fabs(loc[2]);
}
// Corner triple of the octant of loc on the octahedron of half-diagonal dr
// (loadS, VoxelsCA.h:56-77), ordered nearest, middle, farthest from loc;
// returns the index into S0 of the nearest corner's direction. A corner S0*dr
// has one nonzero coordinate (+-dr; the others are +0 for finite dr), so
// loc - corner is loc itself on two axes and the squared distances
// e0*e0 + e1*e1 + e2*e2 share those squares; operands are selected per corner
// so the sums keep the reference's order. Distances are compared as bit
// patterns (non-negative doubles).
__device__ __forceinline__ int cafe_geo_corners(const double *loc, double dr, double (*pk)[3]) {
  const signed char S0[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
  const unsigned char SI[8][3] = {{0, 1, 2}, {1, 2, 3}, {0, 2, 4}, {2, 3, 4},
                                  {0, 1, 5}, {1, 3, 5}, {0, 4, 5}, {3, 4, 5}};
  int jInd = 4 * (signbit(loc[2]) ? 1 : 0) + 2 * (signbit(loc[1]) ? 1 : 0) + (signbit(loc[0]) ? 1 : 0);
  int kk[3];
  if ((crm_bits(dr) & CRM_BITS_INF) != CRM_BITS_INF) {
    double L0 = loc[0] * loc[0], L1 = loc[1] * loc[1], L2 = loc[2] * loc[2];
    long long db[3];
    for (int a = 0; a < 3; ++a) {
      int idx = SI[jInd][a];
      int ax = idx < 3 ? idx : idx - 3;
      double cv = idx < 3 ? dr : -dr;
      double la = ax == 0 ? loc[0] : (ax == 1 ? loc[1] : loc[2]);
      double e = la - cv;
      double D = e * e;
      double A = ax == 0 ? D : L0, B = ax == 1 ? D : L1, C = ax == 2 ? D : L2;
      db[a] = crm_bits((A + B) + C);
    }
    int imin = 0, imax = 0;
    for (int a = 1; a < 3; ++a) {
      if (db[a] < db[imin]) imin = a;
      if (db[imax] < db[a]) imax = a;
    }
    if (imin == imax) {
      kk[0] = 0;
      kk[1] = 1;
      kk[2] = 2;
    } else {
      kk[0] = imin;
      kk[2] = imax;
      kk[1] = 3 - imin - imax;
    }
    for (int a = 0; a < 3; ++a) {
      int idx = SI[jInd][kk[a]];
      int ax = idx < 3 ? idx : idx - 3;
      double cv = idx < 3 ? dr : -dr;
      for (int b = 0; b < 3; ++b) pk[a][b] = b == ax ? cv : 0.0;
    }
    return SI[jInd][kk[0]];
  }
  // non-finite dr: the reference's arithmetic as written
  double corner[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) corner[a][b] = (double)S0[SI[jInd][a]][b] * dr;
  double dnorm[3];
  for (int a = 0; a < 3; ++a) {
    double e0 = loc[0] - corner[a][0], e1 = loc[1] - corner[a][1], e2 = loc[2] - corner[a][2];
    dnorm[a] = e0 * e0 + e1 * e1 + e2 * e2;
  }
  int imin = 0, imax = 0;
  for (int a = 1; a < 3; ++a) {
    if (dnorm[a] < dnorm[imin]) imin = a;
    if (dnorm[imax] < dnorm[a]) imax = a;
  }
  if (imin == imax) {
    kk[0] = 0;
    kk[1] = 1;
    kk[2] = 2;
  } else {
    kk[0] = imin;
    kk[2] = imax;
    kk[1] = 3 - imin - imax;
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) pk[a][b] = corner[kk[a]][b];
  return SI[jInd][kk[0]];
}
// projectPointLine (VoxelsCA.h:78-93)
__device__ __forceinline__ void cafe_project(const double *A, const double *x0, const double *x1,
                                             double *xp) {
  double e0 = x1[0] - x0[0], e1 = x1[1] - x0[1], e2 = x1[2] - x0[2];
  double snorm = crm_pow_half(e0 * e0 + e1 * e1 + e2 * e2);
  double n0 = e0 / snorm, n1 = e1 / snorm, n2 = e2 / snorm;
  double d = -(n0 * A[0] + n1 * A[1] + n2 * A[2]);
  double t = (-d - n0 * x0[0] - n1 * x0[1] - n2 * x0[2]) / (n0 * e0 + n1 * e1 + n2 * e2);
  xp[0] = x0[0] + e0 * t;
  xp[1] = x0[1] + e1 * t;
  xp[2] = x0[2] + e2 * t;
}
// Projection of loc onto the edge p0-p1 and the distances of the foot point
// to p0 and to p1 (VoxelsCA.C:566-577 for one of the two edges).
__device__ __forceinline__ void cafe_geo_edge(const double *loc, const double *p0, const double *p1,
                                              double *d0, double *d1) {
  double x[3];
  cafe_project(loc, p0, p1, x);
  double e0, e1, e2;
  e0 = p0[0] - x[0]; e1 = p0[1] - x[1]; e2 = p0[2] - x[2];
  *d0 = crm_pow_half(e0 * e0 + e1 * e1 + e2 * e2);
  e0 = p1[0] - x[0]; e1 = p1[1] - x[1]; e2 = p1[2] - x[2];
  *d1 = crm_pow_half(e0 * e0 + e1 * e1 + e2 * e2);
}
// Half-diagonal Lmud of the new octahedron (VoxelsCA.C:578-582).
__device__ __forceinline__ double cafe_geo_lmud(const CafeConsts &K, double l, double d1I, double dI2,
                                                double d1J, double dJ3) {
  double s3l = K.s3 * l;
  // std::min(a,b) = (b < a) ? b : a ; std::max(a,b) = (a < b) ? b : a
  double L12 = .5 * (((s3l < d1I) ? s3l : d1I) + ((s3l < dI2) ? s3l : dI2));
  double L13 = .5 * (((s3l < d1J) ? s3l : d1J) + ((s3l < dJ3) ? s3l : dJ3));
  return K.s3 * (K.s23 * ((L12 < L13) ? L13 : L12));
}
// Centre of the new octahedron (VoxelsCA.C:583-604): nearest corner p0 moved
// back by Lmud along its direction, rotated to the lab frame, plus cs.
__device__ __forceinline__ void cafe_geo_centre(const double *R, const double *cs, const double *p0, int s0i,
                                                double Lmud, double *cen) {
  const signed char S0[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
  const signed char *s0 = S0[s0i];
  double m0 = p0[0] - Lmud * (double)s0[0];
  double m1 = p0[1] - Lmud * (double)s0[1];
  double m2 = p0[2] - Lmud * (double)s0[2];
  double g0 = R[0] * m0 + R[1] * m1 + R[2] * m2;
  double g1 = R[3] * m0 + R[4] * m1 + R[5] * m2;
  double g2 = R[6] * m0 + R[7] * m1 + R[8] * m2;
  cen[0] = cs[0] + g0;
  cen[1] = cs[1] + g1;
  cen[2] = cs[2] + g2;
}
__device__ __noinline__ void cafe_capture_geometry(const CafeConsts &K, int ci, int cj, int ck,
                                                   int si, int sj, int sk, const double *cs,
                                                   const double *R, double *g_out,
                                                   double *ext_out, double *cen_out) {
  double l = cafe_geo_l(K, ci, cj, ck, si, sj, sk);
  double dn[3], loc[3];
  cafe_geo_dn(K, ci, cj, ck, cs, dn);
  double dr = cafe_geo_loc(R, dn, loc);
  double f = crm_pow_half(cafe_geo_costh(dn) * cafe_geo_sinph(dn));
  *g_out = f * dr;
  double pk[3][3];
  int s0i = cafe_geo_corners(loc, dr, pk);
  double d1I, dI2, d1J, dJ3;
  cafe_geo_edge(loc, pk[0], pk[1], &d1I, &dI2);
  cafe_geo_edge(loc, pk[0], pk[2], &d1J, &dJ3);
  double Lmud = cafe_geo_lmud(K, l, d1I, dI2, d1J, dJ3);
  *ext_out = f * Lmud * 1.0;
  cafe_geo_centre(R, cs, pk[0], s0i, Lmud, cen_out);
}

// One orientation of SampleOrientation::GenerateSamples (SampleOrientation.C:
// 124-161) for a single sample with engine seed `seed`.
__device__ __noinline__ void cafe_sample_orientation(const CafeConsts &K, unsigned int seed,
                                                     double *out) {
  cafe_uniform_stream st;
  st.x = cafe_minstd_seed(seed);
  double u0 = cafe_uniform_next(&st), u1 = cafe_uniform_next(&st), u2 = cafe_uniform_next(&st);
  double xyz0[3] = {u0 - .5, u1 - .5, u2 - .5};
  double xyz[3] = {K.so_aprime * xyz0[0], K.so_aprime * xyz0[1], K.so_aprime * xyz0[2]};
  int P[3] = {1, 2, 3};
  {
    double x = xyz[0], y = xyz[1], z = xyz[2];
    if ((fabs(x) <= z) && (fabs(y) <= z)) { P[0] = 1; P[1] = 2; P[2] = 3; }
    if ((z <= -fabs(x)) && (z <= -fabs(y))) { P[0] = -1; P[1] = 2; P[2] = -3; }
    if ((fabs(x) <= y) && (fabs(z) <= y)) { P[0] = 1; P[1] = -3; P[2] = 2; }
    if ((y <= -fabs(x)) && (y <= -fabs(z))) { P[0] = 1; P[1] = 3; P[2] = -2; }
    if ((fabs(z) < x) && (fabs(y) <= x)) { P[0] = -3; P[1] = 2; P[2] = 1; }
    if ((x <= -fabs(z)) && (x <= -fabs(y))) { P[0] = 3; P[1] = 2; P[2] = -1; }
  }
  double xyz2[3];
  for (int j = 0; j < 3; ++j) {
    int a = P[j] < 0 ? -P[j] : P[j];
    xyz2[j] = (double)(P[j] / a) * xyz[a - 1];
  }
  double m1[3];
  for (int j = 0; j < 3; ++j) m1[j] = K.so_a / K.so_aprime * xyz2[j];
  const double PI = 3.14159265358979323846;
  double m2[3];
  {
    double x = m1[0], y = m1[1], z = m1[2], T1 = 0, T2 = 0;
    if (fabs(y) <= fabs(x)) {
      if (fabs(x) < 1e-10) {
        T1 = 0.0;
        T2 = 0.0;
      } else {
        double ang = y * PI / 12 / x;
        double cang = crm_cos(ang);
        T1 = K.so_s2 * cang - 1;
        T2 = K.so_s2 * crm_sin(ang);
        double f = K.so_s2q * x / (K.so_beta * crm_pow_half(K.so_s2 - cang));
        T1 *= f;
        T2 *= f;
      }
    }
    if (fabs(x) <= fabs(y)) {
      if (fabs(y) < 1e-10) {
        T1 = 0.0;
        T2 = 0.0;
      } else {
        double ang = x * PI / 12 / y;
        double cang = crm_cos(ang);
        T1 = K.so_s2 * crm_sin(ang);
        T2 = K.so_s2 * cang - 1;
        double f = K.so_s2q * y / (K.so_beta * crm_pow_half(K.so_s2 - cang));
        T1 *= f;
        T2 *= f;
      }
    }
    m2[0] = T1;
    m2[1] = T2;
    m2[2] = z;
  }
  double m3[3];
  {
    double x = m2[0], y = m2[1], z = m2[2];
    if (fabs(z) < 1e-10) {
      m3[0] = m3[1] = m3[2] = 0;
    } else {
      double q = 1 - (x * x + y * y) * PI / (24 * (z * z));
      double sq = crm_pow_half(q);
      m3[0] = sq * x;
      m3[1] = sq * y;
      m3[2] = K.so_s6pi * z - (x * x + y * y) * K.so_spi / (K.so_s24 * z);
    }
  }
  double xyzb[3];
  for (int j = 0; j < 3; ++j) {
    int a = P[j] < 0 ? -P[j] : P[j];
    xyzb[a - 1] = (double)(P[j] / a) * m3[j];
  }
  double ax0 = fabs(xyz0[0]), ax1 = fabs(xyz0[1]), ax2 = fabs(xyz0[2]);
  double pmax = (ax0 < ax1) ? ax1 : ax0;
  pmax = (pmax < ax2) ? ax2 : pmax;
  double rhoP = K.so_R1 * pmax / .5;
  double t = 1;
  for (int j = 1; j < 8; ++j) t += K.so_coeffA[j - 1] * crm_pow_int(rhoP, 2 * j);
  double omega = 2.0 * crm_acos(t);
  double tnorm = crm_pow_half(xyzb[0] * xyzb[0] + xyzb[1] * xyzb[1] + xyzb[2] * xyzb[2]);
  out[0] = omega;
  out[1] = xyzb[0] / tnorm;
  out[2] = xyzb[1] / tnorm;
  out[3] = xyzb[2] / tnorm;
}

#endif

// Test-only link-time routing of the reference's libm calls (linked with
// -Wl,--wrap for each symbol below, see oracle/Makefile target
// _ref/cafe_ref_dump_cr).
//
// The engine evaluates some of the reference's transcendental calls with the
// correctly rounded functions of amcafe_gb300/csrc/cafe_crmath.h and the rest
// with the host's glibc. This shim makes the reference's own, unmodified code
// do the same, so that the reference itself can be compared with the engine
// bit for bit on decks where glibc's rounding and the correctly rounded value
// lead to different capture decisions:
//   * inside VoxelsCA::UpdateVoxels (VoxelsCA.C:232-655: capture geometry,
//     loadRotMat, nucleation's GenerateSamples): atan2, cos, sin, sincos, acos
//     and pow(x, 0.5), pow(x, 2), pow(x, 2j) are correctly rounded;
//   * inside TempField::EASM (TempField.C:79-137 and the Utilities integrand
//     it calls): exp, pow(x, -0.5), pow(x, 2) and pow(10, -e) are correctly
//     rounded; the laser-grid rotation's sincos stays glibc;
//   * everywhere else (laser grid, analytic temperature, baseplate and layer
//     orientations, Poisson draws, output) every call goes to glibc.
#include <cmath>
#include <cstdint>

#include "../../amcafe_gb300/csrc/cafe_crmath.h"

enum { CTX_GLIBC = 0, CTX_VOXELS = 1, CTX_EASM = 2 };
static int g_ctx = CTX_GLIBC;

class VoxelsCA;
class TempField;

extern "C" {
double __real_atan2(double, double);
double __real_cos(double);
double __real_sin(double);
void __real_sincos(double, double *, double *);
double __real_acos(double);
double __real_pow(double, double);
double __real_exp(double);

// VoxelsCA::UpdateVoxels() and TempField::EASM(std::vector<double>&,
// std::vector<int>&, int), by their mangled names
void __real__ZN8VoxelsCA12UpdateVoxelsEv(VoxelsCA *self);
void __real__ZN9TempField4EASMERSt6vectorIdSaIdEERS0_IiSaIiEEi(TempField *self, void *T, void *ids, int n);

void __wrap__ZN8VoxelsCA12UpdateVoxelsEv(VoxelsCA *self) {
  int saved = g_ctx;
  g_ctx = CTX_VOXELS;
  __real__ZN8VoxelsCA12UpdateVoxelsEv(self);
  g_ctx = saved;
}

void __wrap__ZN9TempField4EASMERSt6vectorIdSaIdEERS0_IiSaIiEEi(TempField *self, void *T, void *ids, int n) {
  int saved = g_ctx;
  g_ctx = CTX_EASM;
  __real__ZN9TempField4EASMERSt6vectorIdSaIdEERS0_IiSaIiEEi(self, T, ids, n);
  g_ctx = saved;
}

double __wrap_atan2(double y, double x) { return g_ctx == CTX_VOXELS ? crm_atan2(y, x) : __real_atan2(y, x); }
double __wrap_cos(double x) { return g_ctx == CTX_VOXELS ? crm_cos(x) : __real_cos(x); }
double __wrap_sin(double x) { return g_ctx == CTX_VOXELS ? crm_sin(x) : __real_sin(x); }
void __wrap_sincos(double x, double *s, double *c) {
  if (g_ctx == CTX_VOXELS) {
    *s = crm_sin(x);
    *c = crm_cos(x);
  } else {
    __real_sincos(x, s, c);
  }
}
double __wrap_acos(double x) { return g_ctx == CTX_VOXELS ? crm_acos(x) : __real_acos(x); }
double __wrap_exp(double x) { return g_ctx == CTX_EASM ? crm_exp(x) : __real_exp(x); }

double __wrap_pow(double x, double y) {
  if (g_ctx == CTX_VOXELS) {
    if (y == 0.5) return crm_pow_half(x);
    if (y == 2.0) return x * x;
    if (y == std::floor(y) && y >= 2.0 && y <= 64.0 && std::fmod(y, 2.0) == 0.0) return crm_pow_int(x, (int)y);
  } else if (g_ctx == CTX_EASM) {
    if (y == -0.5) return crm_pow_mhalf(x);
    if (y == 2.0) return x * x;
    if (x == 10.0 && (y == -2.0 || y == -3.0 || y == -4.0 || y == -5.0))
      return y == -2.0 ? 1e-2 : y == -3.0 ? 1e-3 : y == -4.0 ? 1e-4 : 1e-5;
  }
  return __real_pow(x, y);
}
}  // extern "C"

// Test-only wrapper exposing the host side of amcafe_gb300/csrc/cafe_rng.h and
// cafe_crmath.h through a C ABI, so the tests can compare them with libstdc++
// and with correctly rounded reference values. Built by tests/test_headers.py.
#include <stdint.h>

#include "../../amcafe_gb300/csrc/cafe_crmath.h"
#include "../../amcafe_gb300/csrc/cafe_rng.h"

extern "C" {
void hc_uniforms_at(uint32_t seed, uint64_t skip, long n, double *out) {
  uint32_t s = cafe_minstd_seed(seed);
  for (long i = 0; i < n; ++i) out[i] = cafe_uniform_at(s, skip + (uint64_t)i);
}
void hc_uniforms_stream(uint32_t seed, long n, double *out) {
  cafe_uniform_stream st;
  st.x = cafe_minstd_seed(seed);
  for (long i = 0; i < n; ++i) out[i] = cafe_uniform_next(&st);
}
void hc_eval(int fn, long n, const double *x, const double *y, double *out) {
  for (long i = 0; i < n; ++i) {
    switch (fn) {
      case 0: out[i] = crm_atan2(x[i], y[i]); break;
      case 1: out[i] = crm_cos(x[i]); break;
      case 2: out[i] = crm_sin(x[i]); break;
      case 3: out[i] = crm_acos(x[i]); break;
      case 4: out[i] = crm_pow_half(x[i]); break;
      case 6: out[i] = crm_exp(x[i]); break;
      case 7: out[i] = crm_pow_mhalf(x[i]); break;
      default: out[i] = crm_pow_int(x[i], (int)y[i]); break;
    }
  }
}
}

// Batched ensemble: many independent realisations stepped concurrently on one
// GPU.
//
// A realisation is one cafe_sim handle. Two engines step them:
// * batched launches (threads <= 0, the default): every step kernel is
//   launched once for all realisations, each realisation's blocks running its
//   own state, the event loop one block per realisation; the launches of a
//   batch step form one CUDA graph, replayed every batch step, and the launch
//   shapes are picked by a built-in autotuner (cafe_host.cu, batched steps);
// * host round-robin (threads >= 1): each realisation steps on its own CUDA
//   stream, `threads` host threads issuing one step (one graph launch) per
//   realisation and turn.
// Either way each realisation runs the same loop as a plain run
// (cafe_sim_initialize_voxels, cafe_sim_begin, the loop iterations until done,
// the closing cafe_sim_clean_layer), so its results are those of its plain run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cafe_gpu.h"

void cafe_internal_set_error(const char *msg);
void cafe_internal_set_share(cafe_sim *s, int share, int graphs);
struct CafeBatchEngine;
CafeBatchEngine *cafe_internal_batch_engine_create(cafe_sim *const *sims, int n, int tune, int *rc);
void cafe_internal_batch_engine_destroy(CafeBatchEngine *E);
int cafe_internal_batch_engine_step(CafeBatchEngine *E, int *phase, long long *steps, int *stepped);
const char *cafe_internal_batch_engine_log(const CafeBatchEngine *E);
long long cafe_internal_batch_engine_launches(const CafeBatchEngine *E);
long long cafe_internal_batch_engine_steps(const CafeBatchEngine *E);

struct cafe_batch {
  std::vector<cafe_sim *> sims;
  std::vector<long long> steps;
  std::vector<int> phase;  // 0 created, 1 looping, 2 finished (closing CleanLayer applied)
  int threads = 1;         // host threads of the round-robin engine; 0: batched launches
  CafeBatchEngine *engine = nullptr;
};

extern "C" {

int cafe_batch_create(const char *const *decks, int n, const cafe_options *opt, int threads, cafe_batch **out) {
  if (!decks || n <= 0 || !out) {
    cafe_internal_set_error("cafe_batch_create: null or empty argument");
    return CAFE_E_ARG;
  }
  *out = nullptr;
  cafe_batch *b = new cafe_batch;
  for (int i = 0; i < n; ++i) {
    cafe_sim *s = nullptr;
    int rc = decks[i] ? cafe_sim_create(decks[i], opt, &s) : CAFE_E_ARG;
    if (rc) {
      if (!decks[i]) cafe_internal_set_error("cafe_batch_create: null deck path");
      for (cafe_sim *t : b->sims) cafe_sim_destroy(t);
      delete b;
      return rc;
    }
    b->sims.push_back(s);
  }
  b->steps.assign(n, 0);
  b->phase.assign(n, 0);
  if (threads <= 0) {
    b->threads = 0;  // batched launches (the engine is made at the first run)
  } else {
    // host round-robin: with one thread a step is two launches (parameters
    // and the step's CUDA graph); several threads contend for the driver
    b->threads = std::min(threads, n);
    for (cafe_sim *s : b->sims) cafe_internal_set_share(s, n, b->threads == 1);
  }
  *out = b;
  return CAFE_OK;
}

int cafe_batch_size(const cafe_batch *b) { return b ? (int)b->sims.size() : 0; }

cafe_sim *cafe_batch_sim(cafe_batch *b, int i) {
  if (!b || i < 0 || i >= (int)b->sims.size()) return nullptr;
  return b->sims[i];
}

int cafe_batch_run(cafe_batch *b, long long max_steps, long long *steps_done) {
  if (!b) {
    cafe_internal_set_error("cafe_batch_run: null handle");
    return CAFE_E_ARG;
  }
  const int n = (int)b->sims.size(), T = b->threads;
  if (T == 0) {
    for (int i = 0; i < n; ++i) {
      if (b->phase[i] != 0) continue;
      int rc = cafe_sim_initialize_voxels(b->sims[i]);
      if (!rc) rc = cafe_sim_begin(b->sims[i]);
      if (rc) {
        std::string m = "realisation " + std::to_string(i) + ": " + cafe_last_error();
        cafe_internal_set_error(m.c_str());
        return rc;
      }
      b->phase[i] = 1;
    }
    if (!b->engine) {
      int rc = CAFE_OK;
      b->engine = cafe_internal_batch_engine_create(b->sims.data(), n, 1, &rc);
      if (!b->engine) return rc;
    }
    std::vector<int> ph(n);
    while (true) {
      bool any = false;
      for (int i = 0; i < n; ++i) {
        ph[i] = (b->phase[i] == 1 && (max_steps <= 0 || b->steps[i] < max_steps)) ? 1 : 0;
        any = any || ph[i];
      }
      if (!any) break;
      int stepped = 0;
      int rc = cafe_internal_batch_engine_step(b->engine, ph.data(), b->steps.data(), &stepped);
      for (int i = 0; i < n; ++i)
        if (ph[i] == 2) b->phase[i] = 2;
      if (rc) return rc;
    }
    for (int i = 0; i < n; ++i) {
      int rc = cafe_sim_synchronize(b->sims[i]);
      if (rc) {
        std::string m = "realisation " + std::to_string(i) + ": " + cafe_last_error();
        cafe_internal_set_error(m.c_str());
        return rc;
      }
    }
    if (steps_done) {
      long long tot = 0;
      for (long long v : b->steps) tot += v;
      *steps_done = tot;
    }
    return CAFE_OK;
  }
  std::vector<int> rcs(n, 0);
  std::vector<std::string> msgs(n);
  auto fail = [&](int i, int rc) {
    rcs[i] = rc;
    const char *m = cafe_last_error();
    msgs[i] = m ? m : "";
  };
  auto worker = [&](int t) {
    std::vector<int> mine;
    for (int i = t; i < n; i += T) mine.push_back(i);
    for (int i : mine) {
      if (b->phase[i] != 0) continue;
      int rc = cafe_sim_initialize_voxels(b->sims[i]);
      if (!rc) rc = cafe_sim_begin(b->sims[i]);
      if (rc) {
        fail(i, rc);
        b->phase[i] = 2;
      } else {
        b->phase[i] = 1;
      }
    }
    // one step of each unfinished realisation in turn: their kernels queue on
    // their own streams and run side by side
    bool more = true;
    while (more) {
      more = false;
      for (int i : mine) {
        if (b->phase[i] != 1 || rcs[i]) continue;
        if (max_steps > 0 && b->steps[i] >= max_steps) continue;
        int done = 0;
        int rc = cafe_sim_step(b->sims[i], &done);
        if (rc) {
          fail(i, rc);
          continue;
        }
        b->steps[i] += 1;
        if (done) {
          rc = cafe_sim_clean_layer(b->sims[i]);  // main1.C:95
          if (rc) fail(i, rc);
          b->phase[i] = 2;
        } else {
          more = true;
        }
      }
    }
    for (int i : mine)
      if (!rcs[i]) {
        int rc = cafe_sim_synchronize(b->sims[i]);
        if (rc) fail(i, rc);
      }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < T; ++t) pool.emplace_back(worker, t);
  worker(0);
  for (auto &th : pool) th.join();
  if (steps_done) {
    long long tot = 0;
    for (long long s : b->steps) tot += s;
    *steps_done = tot;
  }
  for (int i = 0; i < n; ++i)
    if (rcs[i]) {
      std::string m = "realisation " + std::to_string(i) + ": " + msgs[i];
      cafe_internal_set_error(m.c_str());
      return rcs[i];
    }
  return CAFE_OK;
}

int cafe_batch_finished(const cafe_batch *b, int i) {
  if (!b || i < 0 || i >= (int)b->sims.size()) return -1;
  return b->phase[i] == 2 ? 1 : 0;
}

int cafe_batch_report(const cafe_batch *b, long long *launches, long long *batch_steps, char *tuning, int cap) {
  if (!b) {
    cafe_internal_set_error("cafe_batch_report: null handle");
    return CAFE_E_ARG;
  }
  if (launches) *launches = cafe_internal_batch_engine_launches(b->engine);
  if (batch_steps) *batch_steps = cafe_internal_batch_engine_steps(b->engine);
  if (tuning && cap > 0) {
    const char *log = b->engine ? cafe_internal_batch_engine_log(b->engine) : "";
    std::strncpy(tuning, log, (size_t)cap - 1);
    tuning[cap - 1] = 0;
  }
  return CAFE_OK;
}

void cafe_batch_destroy(cafe_batch *b) {
  if (!b) return;
  cafe_internal_batch_engine_destroy(b->engine);
  for (cafe_sim *s : b->sims) cafe_sim_destroy(s);
  delete b;
}

}  // extern "C"

// Batched ensemble: many independent realisations stepped concurrently on one
// GPU (host code only).
//
// A realisation is one cafe_sim handle with its own CUDA stream, so the work of
// different realisations overlaps on the device: the capture/nucleation loop
// of each step is one thread block, and a batch keeps one such block per
// realisation in flight at once instead of one for the whole GPU. Host threads
// (one by default; each owning every T-th realisation) issue the steps
// round-robin, one step (one CUDA graph launch) per realisation and turn; each
// realisation runs the same loop as a plain run (cafe_sim_initialize_voxels,
// cafe_sim_begin, the loop iterations until done, the closing
// cafe_sim_clean_layer), so its results are those of its plain run.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cafe_gpu.h"

void cafe_internal_set_error(const char *msg);
void cafe_internal_set_share(cafe_sim *s, int share, int graphs);

struct cafe_batch {
  std::vector<cafe_sim *> sims;
  std::vector<long long> steps;
  std::vector<int> phase;  // 0 created, 1 looping, 2 finished (closing CleanLayer applied)
  int threads = 1;
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
  // one host thread by default: a step is two launches (parameters and the
  // step's CUDA graph), and one thread issues them for many realisations
  // faster than several threads contending for the driver
  b->threads = std::max(1, std::min(threads > 0 ? threads : 1, n));
  for (cafe_sim *s : b->sims) cafe_internal_set_share(s, n, b->threads == 1);
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

void cafe_batch_destroy(cafe_batch *b) {
  if (!b) return;
  for (cafe_sim *s : b->sims) cafe_sim_destroy(s);
  delete b;
}

}  // extern "C"

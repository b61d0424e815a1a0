// Serving: a request loop that runs many simulations of different sizes and
// durations on one GPU at once.
//
// There is no counterpart in the reference, which runs one network per
// process (src/openmp/infoli.c:124-735); every request here is that program's
// network update on its own inputs, through an infoli_sim handle.
//
// Life of a request:
//   queued   -> admitted when its device-memory estimate fits the HBM budget
//               (first in, first out; a later request may pass one that does
//               not fit yet, unless that one has waited longer than the
//               backfill limit);
//   prepared -> one of the preparation threads builds its plan and uploads
//               its state and topology (infoli_sim_create with a share of the
//               SMs sized to its work);
//   running  -> launched on its own stream as soon as its CTAs fit beside the
//               running simulations (the grids of all running simulations
//               never exceed the SM count, so every persistent grid is
//               co-resident and none waits on another); its work overlaps
//               the others' on the device.  Among prepared requests, those
//               submitted longer ago than the age limit go first (oldest
//               first), then the shortest estimated work (edges x steps);
//               a negative age limit keeps arrival order;
//   done     -> final state copied to the host, device memory released; the
//               record waits for infoli_server_wait.
// A request's result does not depend on what runs beside it: its plan and
// launches depend only on the request itself.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/infoli_gpu.h"
#include "infoli_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int n = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col;
  std::vector<float> g;
  float g_uniform = 0.04f;
  std::vector<float> init;  // 19 x n
  int n_steps = 0;
  int pulse_start = 20000, pulse_end = 20499;
  float pulse_amp = 6.0f;
  int flags = 0;
  // scheduling
  int grid = 0;
  double work = 0;  // estimated edge evaluations (plus a per-cell share) over the whole run
  int64_t est_bytes = 0, dev_bytes = 0, admit_bytes = 0;
  double submit_s = 0, admit_s = 0, prep_start_s = 0, prepared_s = 0, start_s = 0, done_s = 0;
  int phase = 0;  // 0 queued, 1 admitted (preparing), 2 prepared, 3 running, 4 done
  int status = INFOLI_OK;
  char err[256] = {0};
  infoli_sim* sim = nullptr;
  std::vector<float> result;
};

}  // namespace

struct infoli_server {
  std::vector<float> params;
  int device = 0, nsm = 0, max_active = 64, flags = 0;
  int64_t budget = 0, work_per_cta = 0;
  double backfill_s = 1.0;
  double age_s = 10.0;  // < 0: launch in arrival order
  Clock::time_point t0;
  std::mutex m;
  std::condition_variable cv_sched, cv_prep, cv_done;
  std::deque<Request*> queue;    // waiting for admission
  std::deque<Request*> to_prep;  // admitted, waiting for a preparation thread
  std::vector<Request*> ready;   // prepared, waiting for SMs
  std::vector<Request*> running;
  std::map<int64_t, Request*> all;
  int64_t next_id = 1, completed = 0, mem_in_use = 0;
  int grid_in_use = 0, preparing = 0;
  bool stop = false;
  std::thread sched;
  std::vector<std::thread> prep;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Device bytes a request's handle will hold: the planner's 16-bit edge
// entries with up to one padded lane-chunk per receiver, per-edge
// conductances when given, descriptors (16 bytes per <= 32 edges), per-cell
// state (17 floats + V_dend double buffer + FP64 Ca2+ + two stamped words).
int64_t estimate_bytes(int64_t n, int64_t edges, bool edge_g) {
  const int64_t entries = edges + 32 * n;
  return 2 * entries + (edge_g ? 4 * entries : 0) + entries / 2 + 112 * n + (4 << 20);
}

// CTAs for a request: enough for one thread per cell, and about one CTA per
// work_per_cta edge evaluations per step, up to the whole GPU.
int grid_for(const infoli_server* sv, int64_t n, int64_t edges) {
  const int64_t by_cells = (n + 1023) / 1024;
  const int64_t by_work = (edges + 64 * n + sv->work_per_cta - 1) / sv->work_per_cta;
  return (int)std::min<int64_t>(sv->nsm, std::max<int64_t>(1, std::max(by_cells, by_work)));
}

void finish(infoli_server* sv, Request* r, int status, const char* msg) {
  // caller holds the lock
  r->status = status;
  if (msg) snprintf(r->err, sizeof r->err, "%s", msg);
  r->phase = 4;
  r->done_s = sv->now();
  ++sv->completed;
  sv->cv_done.notify_all();
}

// Preparation threads: plan + upload, outside the lock.
void prep_loop(infoli_server* sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->m);
  for (;;) {
    sv->cv_prep.wait(lk, [&] { return sv->stop || !sv->to_prep.empty(); });
    if (sv->stop) return;
    Request* r = sv->to_prep.front();
    sv->to_prep.pop_front();
    ++sv->preparing;
    r->prep_start_s = sv->now();
    lk.unlock();
    InfoliRange nvtx_range("infoli_server_prepare");
    infoli_sim_desc d;
    std::memset(&d, 0, sizeof d);
    d.n_cells = r->n;
    d.params = sv->params.data();
    d.init_state = r->init.data();
    d.row_ptr = r->row_ptr.data();
    d.col = r->col.empty() ? nullptr : r->col.data();
    d.g = r->g.empty() ? nullptr : r->g.data();
    d.g_uniform = r->g_uniform;
    d.flags = r->flags;
    d.device = sv->device;
    d.grid = r->grid;
    infoli_sim* sim = nullptr;
    int rc = infoli_sim_create(&d, &sim);
    char msg[256] = {0};
    if (rc == INFOLI_OK) rc = infoli_sim_set_stimulus_pulse(sim, r->pulse_start, r->pulse_end, r->pulse_amp);
    if (rc != INFOLI_OK) snprintf(msg, sizeof msg, "%s", infoli_last_error());
    int64_t bytes = 0;
    if (sim) infoli_sim_memory(sim, &bytes);
    // the inputs are on the device now
    std::vector<int64_t>().swap(r->row_ptr);
    std::vector<int32_t>().swap(r->col);
    std::vector<float>().swap(r->g);
    std::vector<float>().swap(r->init);
    lk.lock();
    --sv->preparing;
    if (rc != INFOLI_OK) {
      if (sim) infoli_sim_destroy(sim);
      sv->mem_in_use -= r->est_bytes;
      finish(sv, r, rc, msg);
    } else {
      r->sim = sim;
      r->dev_bytes = bytes;
      // account the measured size from here on
      sv->mem_in_use += bytes - r->est_bytes;
      r->est_bytes = bytes;
      r->phase = 2;
      r->prepared_s = sv->now();
      sv->ready.push_back(r);
    }
    sv->cv_sched.notify_all();
  }
}

// Scheduler: admission, launches, retirement.
void sched_loop(infoli_server* sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->m);
  while (!sv->stop) {
    bool progress = false;
    // retire finished simulations
    for (size_t i = 0; i < sv->running.size();) {
      Request* r = sv->running[i];
      lk.unlock();
      int q = infoli_sim_query(r->sim);
      int rc = INFOLI_OK;
      char msg[256] = {0};
      if (q != 0) {
        if (q < 0) {
          rc = q;
          snprintf(msg, sizeof msg, "%s", infoli_last_error());
        } else {
          r->result.resize((size_t)INFOLI_NSTATE * r->n);
          rc = infoli_sim_get_state(r->sim, r->result.data());
          if (rc != INFOLI_OK) snprintf(msg, sizeof msg, "%s", infoli_last_error());
        }
        infoli_sim_destroy(r->sim);
      }
      lk.lock();
      if (q != 0) {
        r->sim = nullptr;
        sv->running.erase(sv->running.begin() + i);
        sv->grid_in_use -= r->grid;
        sv->mem_in_use -= r->est_bytes;
        finish(sv, r, rc, rc == INFOLI_OK ? nullptr : msg);
        progress = true;
      } else {
        ++i;
      }
    }
    // admit by HBM budget, first in first out with bounded backfill
    const double t = sv->now();
    for (auto it = sv->queue.begin(); it != sv->queue.end();) {
      Request* r = *it;
      const int admitted_or_running = (int)(sv->running.size() + sv->ready.size() + sv->to_prep.size()) + sv->preparing;
      if (admitted_or_running >= sv->max_active) break;
      if (sv->mem_in_use + r->est_bytes <= sv->budget) {
        sv->mem_in_use += r->est_bytes;
        r->phase = 1;
        r->admit_s = t;
        sv->to_prep.push_back(r);
        it = sv->queue.erase(it);
        sv->cv_prep.notify_one();
        progress = true;
        continue;
      }
      if (it == sv->queue.begin() && t - r->submit_s > sv->backfill_s) break;  // the head waits no longer
      ++it;
    }
    // launch prepared simulations whose grids fit beside the running ones:
    // requests submitted more than age_s ago first (oldest first), then the
    // shortest estimated work first
    if (sv->age_s >= 0) {
      std::stable_sort(sv->ready.begin(), sv->ready.end(), [&](const Request* a, const Request* b) {
        const bool oa = t - a->submit_s > sv->age_s, ob = t - b->submit_s > sv->age_s;
        if (oa != ob) return oa;
        return oa ? a->submit_s < b->submit_s : a->work < b->work;
      });
    }
    for (size_t i = 0; i < sv->ready.size();) {
      Request* r = sv->ready[i];
      if (sv->grid_in_use + r->grid > sv->nsm) {
        ++i;
        continue;
      }
      sv->grid_in_use += r->grid;
      sv->ready.erase(sv->ready.begin() + i);
      r->phase = 3;
      r->start_s = sv->now();
      lk.unlock();
      int rc = infoli_sim_launch(r->sim, r->n_steps);
      char msg[256] = {0};
      if (rc != INFOLI_OK) snprintf(msg, sizeof msg, "%s", infoli_last_error());
      lk.lock();
      if (rc != INFOLI_OK) {
        infoli_sim_destroy(r->sim);
        r->sim = nullptr;
        sv->grid_in_use -= r->grid;
        sv->mem_in_use -= r->est_bytes;
        finish(sv, r, rc, msg);
      } else {
        sv->running.push_back(r);
      }
      progress = true;
    }
    if (!progress) {
      // poll running simulations every 100 us; wake at once on submissions
      sv->cv_sched.wait_for(lk, std::chrono::microseconds(100));
    }
  }
}

}  // namespace

extern "C" int infoli_server_create(const infoli_server_desc* d, infoli_server** out) {
  infoli__clear_error();
  if (!d || !out || !d->params) return infoli__fail(INFOLI_ERR_ARG, "server_create: bad argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || d->device < 0 || d->device >= ndev)
    return infoli__fail(INFOLI_ERR_CUDA, "server_create: no CUDA device %d", d->device);
  infoli_server* sv = new infoli_server();
  sv->params.assign(d->params, d->params + INFOLI_NPARAM);
  sv->device = d->device;
  sv->flags = d->flags;
  sv->max_active = d->max_active > 0 ? d->max_active : 64;
  sv->age_s = d->age_ms > 0 ? d->age_ms * 1e-3 : d->age_ms < 0 ? -1.0 : 10.0;
  sv->work_per_cta = d->work_per_cta > 0 ? d->work_per_cta : (int64_t)1 << 15;
  sv->backfill_s = d->backfill_ms > 0 ? d->backfill_ms * 1e-3 : 1.0;
  cudaSetDevice(sv->device);
  cudaDeviceGetAttribute(&sv->nsm, cudaDevAttrMultiProcessorCount, sv->device);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  sv->budget = d->hbm_budget > 0 ? d->hbm_budget : (int64_t)(0.8 * (double)free_b);
  sv->t0 = Clock::now();
  const int np = d->prep_threads > 0 ? d->prep_threads : 4;
  sv->sched = std::thread(sched_loop, sv);
  for (int i = 0; i < np; ++i) sv->prep.emplace_back(prep_loop, sv);
  *out = sv;
  return INFOLI_OK;
}

extern "C" int infoli_server_submit(infoli_server* sv, const infoli_request_desc* q, int64_t* id) {
  infoli__clear_error();
  if (!sv || !q || !id || q->n_cells <= 0 || q->n_steps < 0 || !q->row_ptr ||
      (!q->init_state && !q->init_values))
    return infoli__fail(INFOLI_ERR_ARG, "server_submit: bad argument");
  const int n = q->n_cells;
  const int64_t edges = q->row_ptr[n];
  if (edges < 0 || (edges > 0 && !q->col)) return infoli__fail(INFOLI_ERR_ARG, "server_submit: bad topology");
  Request* r = new Request();
  r->n = n;
  r->row_ptr.assign(q->row_ptr, q->row_ptr + n + 1);
  if (edges > 0) r->col.assign(q->col, q->col + edges);
  if (q->g && edges > 0) r->g.assign(q->g, q->g + edges);
  r->g_uniform = q->g_uniform;
  r->init.resize((size_t)INFOLI_NSTATE * n);
  if (q->init_state) {
    std::memcpy(r->init.data(), q->init_state, r->init.size() * sizeof(float));
  } else {
    for (int k = 0; k < INFOLI_NSTATE; ++k)
      std::fill(r->init.begin() + (size_t)k * n, r->init.begin() + (size_t)(k + 1) * n, q->init_values[k]);
  }
  r->n_steps = q->n_steps;
  r->pulse_start = q->pulse_start;
  r->pulse_end = q->pulse_end;
  r->pulse_amp = q->pulse_amp;
  r->flags = sv->flags;
  r->est_bytes = estimate_bytes(n, edges, q->g != nullptr);
  r->admit_bytes = r->est_bytes;
  r->grid = grid_for(sv, n, edges);
  // the cell update costs about as much as 100 edge evaluations per cell-step
  r->work = ((double)edges + 100.0 * (double)n) * (double)q->n_steps;
  std::lock_guard<std::mutex> lk(sv->m);
  if (r->est_bytes > sv->budget) {
    const long long need = (long long)r->est_bytes, have = (long long)sv->budget;
    delete r;
    return infoli__fail(INFOLI_ERR_CAPACITY, "server_submit: request needs ~%lld bytes, budget is %lld", need, have);
  }
  r->id = sv->next_id++;
  r->submit_s = sv->now();
  sv->all[r->id] = r;
  sv->queue.push_back(r);
  *id = r->id;
  sv->cv_sched.notify_all();
  return INFOLI_OK;
}

extern "C" int infoli_server_poll(infoli_server* sv, int64_t id) {
  infoli__clear_error();
  if (!sv) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  std::lock_guard<std::mutex> lk(sv->m);
  auto it = sv->all.find(id);
  if (it == sv->all.end()) return infoli__fail(INFOLI_ERR_ARG, "server_poll: unknown request %lld", (long long)id);
  const int ph = it->second->phase;
  return ph == 0 ? 0 : ph == 4 ? 2 : 1;
}

extern "C" int infoli_server_wait(infoli_server* sv, int64_t id, float* out_state, infoli_request_info* info) {
  infoli__clear_error();
  if (!sv) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  std::unique_lock<std::mutex> lk(sv->m);
  auto it = sv->all.find(id);
  if (it == sv->all.end()) return infoli__fail(INFOLI_ERR_ARG, "server_wait: unknown request %lld", (long long)id);
  Request* r = it->second;
  sv->cv_done.wait(lk, [&] { return r->phase == 4; });
  sv->all.erase(it);
  lk.unlock();
  if (info) {
    info->id = r->id;
    info->n_cells = r->n;
    info->n_steps = r->n_steps;
    info->grid = r->grid;
    info->device_bytes = r->dev_bytes;
    info->admitted_bytes = r->admit_bytes;
    info->submit_s = r->submit_s;
    info->admit_s = r->admit_s;
    info->prepared_s = r->prepared_s;
    info->prep_start_s = r->prep_start_s;
    info->start_s = r->start_s;
    info->done_s = r->done_s;
    info->status = r->status;
  }
  int rc = r->status;
  if (rc == INFOLI_OK && out_state) std::memcpy(out_state, r->result.data(), r->result.size() * sizeof(float));
  if (rc != INFOLI_OK) infoli__fail(rc, "request %lld: %s", (long long)r->id, r->err);
  delete r;
  return rc;
}

extern "C" int infoli_server_status(infoli_server* sv, int* queued, int* active, int64_t* completed,
                                    int64_t* hbm_in_use) {
  infoli__clear_error();
  if (!sv) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  std::lock_guard<std::mutex> lk(sv->m);
  if (queued) *queued = (int)sv->queue.size();
  if (active) *active = (int)(sv->running.size() + sv->ready.size() + sv->to_prep.size()) + sv->preparing;
  if (completed) *completed = sv->completed;
  if (hbm_in_use) *hbm_in_use = sv->mem_in_use;
  return INFOLI_OK;
}

extern "C" int infoli_server_destroy(infoli_server* sv) {
  infoli__clear_error();
  if (!sv) return INFOLI_OK;
  {
    std::lock_guard<std::mutex> lk(sv->m);
    sv->stop = true;
  }
  sv->cv_sched.notify_all();
  sv->cv_prep.notify_all();
  if (sv->sched.joinable()) sv->sched.join();
  for (std::thread& t : sv->prep)
    if (t.joinable()) t.join();
  for (auto& kv : sv->all) {
    Request* r = kv.second;
    if (r->sim) {
      infoli_sim_sync(r->sim);
      infoli_sim_destroy(r->sim);
    }
    delete r;
  }
  delete sv;
  return INFOLI_OK;
}

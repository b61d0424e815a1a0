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
//               and of the lane's launch in flight never exceed the SM
//               count, so every persistent grid is co-resident and none
//               waits on another); its work overlaps the others' on the
//               device.  Among prepared requests, those submitted longer ago
//               than the age limit go first (oldest first), then the
//               shortest estimated work (edges x steps); a negative age
//               limit keeps arrival order;
//   done     -> final state copied to the host, device memory released; the
//               record waits for infoli_server_wait.
// Small, light requests (at most kLaneMaxCells cells, one conductance, few
// edges per CTA of their cluster) take the lane instead: preparation packs their bitmask rows and uploads them with
// the state to buffers of their own; the scheduler relaunches the batched
// cluster kernel over all of them every lane_chunk steps, on the SMs the
// persistent grids leave (at least lane_sms when it is set: persistent grids
// are capped at the SM count minus lane_sms), so a request that arrives while others run
// joins at the next launch, and one whose steps are done leaves.
// A request's result does not depend on what runs beside it: its path, plan
// and arithmetic depend only on the request itself.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/infoli_gpu.h"
#include "infoli_internal.h"
#include "infoli_lane.h"

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
  // the lane
  bool lane = false;
  uint32_t* d_bits = nullptr;
  float* d_st = nullptr;
  double* d_ca = nullptr;
  int steps_done = 0, chunk = 0, lane_launches = 0;
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
  // the lane: prepared small requests, in arrival order; those of the launch
  // in flight are in lane_run (with lane_nets, which the launch reads)
  infoli_lane* lane = nullptr;
  int lane_sms = 0, lane_chunk = 2000, lane_inflight = 0;
  int64_t lane_edges = 24576;  // < 0: any
  bool lane_busy = false;
  std::vector<Request*> lane_reqs;
  std::vector<Request*> lane_run;
  std::vector<infoli::LaneNet> lane_nets;
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

// Device bytes of a lane request: bitmask rows (two pad words each), the
// state, FP64 Ca2+.
int64_t lane_bytes(int64_t n) { return 4 * n * ((n + 31) / 32 + 2) + 4 * INFOLI_NSTATE * n + 8 * n + (1 << 20); }

// CTAs for a request: enough for one thread per cell, and about one CTA per
// work_per_cta edge evaluations per step, up to the whole GPU less the SMs
// left to the lane.
int grid_for(const infoli_server* sv, int64_t n, int64_t edges) {
  const int64_t by_cells = (n + 1023) / 1024;
  const int64_t by_work = (edges + 64 * n + sv->work_per_cta - 1) / sv->work_per_cta;
  const int64_t cap = sv->lane ? sv->nsm - sv->lane_sms : sv->nsm;
  return (int)std::min<int64_t>(cap, std::max<int64_t>(1, std::max(by_cells, by_work)));
}

void lane_free(infoli_server* sv, Request* r) {
  cudaStream_t s = static_cast<cudaStream_t>(infoli__lane_stream(sv->lane));
  for (void* p : {(void*)r->d_bits, (void*)r->d_st, (void*)r->d_ca})
    if (p) cudaFreeAsync(p, s);
  r->d_bits = nullptr;
  r->d_st = nullptr;
  r->d_ca = nullptr;
}

// Plan-free preparation of a lane request (caller does not hold the lock):
// bitmask rows and state to device buffers of its own.  Returns 0, -2 when
// the request cannot take the lane (a repeated sender), or an error status.
int lane_prepare(infoli_server* sv, Request* r, cudaStream_t s, char* msg, size_t msg_len) {
  const int n = r->n;
  std::vector<uint32_t> bits((size_t)n * ((n + 31) / 32 + 2));
  const int pk = infoli__lane_pack_bits(n, r->row_ptr.data(), r->col.empty() ? nullptr : r->col.data(),
                                        bits.data());
  if (pk == -2) return -2;
  if (pk != 0) {
    snprintf(msg, msg_len, "request topology: a sender id is outside [0, n_cells)");
    return INFOLI_ERR_ARG;
  }
  std::vector<double> ca((size_t)n);
  for (int c = 0; c < n; ++c) ca[c] = (double)r->init[(size_t)4 * n + c];
  // from the library's pool: the default pool would hand freed memory back at
  // synchronisation points, and unmapping waits for every kernel on the device
  cudaMemPool_t pool = infoli__device_pool(sv->device);
  cudaError_t e = pool ? cudaSuccess : cudaErrorMemoryAllocation;
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync((void**)&r->d_bits, bits.size() * sizeof(uint32_t), pool, s);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync((void**)&r->d_st, r->init.size() * sizeof(float), pool, s);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync((void**)&r->d_ca, ca.size() * sizeof(double), pool, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r->d_bits, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r->d_st, r->init.data(), r->init.size() * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(r->d_ca, ca.data(), ca.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    snprintf(msg, msg_len, "lane upload: %s", cudaGetErrorString(e));
    for (void* p : {(void*)r->d_bits, (void*)r->d_st, (void*)r->d_ca})
      if (p) cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
    r->d_bits = nullptr;
    r->d_st = nullptr;
    r->d_ca = nullptr;
    return INFOLI_ERR_NOMEM;
  }
  return INFOLI_OK;
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
  cudaStream_t up = nullptr;
  cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking);
  std::unique_lock<std::mutex> lk(sv->m);
  for (;;) {
    sv->cv_prep.wait(lk, [&] { return sv->stop || !sv->to_prep.empty(); });
    if (sv->stop) break;
    Request* r = sv->to_prep.front();
    sv->to_prep.pop_front();
    ++sv->preparing;
    r->prep_start_s = sv->now();
    lk.unlock();
    InfoliRange nvtx_range("infoli_server_prepare");
    if (r->lane) {
      char lmsg[256] = {0};
      const int lrc = lane_prepare(sv, r, up, lmsg, sizeof lmsg);
      if (lrc != -2) {
        std::vector<int64_t>().swap(r->row_ptr);
        std::vector<int32_t>().swap(r->col);
        std::vector<float>().swap(r->init);
        lk.lock();
        --sv->preparing;
        if (lrc != INFOLI_OK) {
          sv->mem_in_use -= r->est_bytes;
          finish(sv, r, lrc, lmsg);
        } else {
          r->dev_bytes = r->est_bytes;
          r->phase = 2;
          r->prepared_s = sv->now();
          sv->lane_reqs.push_back(r);
        }
        sv->cv_sched.notify_all();
        continue;
      }
      r->lane = false;  // a repeated sender: the persistent path sums it as given
      r->grid = grid_for(sv, r->n, (int64_t)r->col.size());
    }
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
  lk.unlock();
  if (up) cudaStreamDestroy(up);
}

// The lane's launch in flight has finished (or failed): advance its
// requests, retire those that are done.  Caller holds the lock.
void lane_complete(infoli_server* sv, std::unique_lock<std::mutex>& lk, int q) {
  std::vector<Request*> done;
  for (Request* r : sv->lane_run) {
    if (q > 0) r->steps_done += r->chunk;
    ++r->lane_launches;
    if (q < 0 || r->steps_done >= r->n_steps) done.push_back(r);
  }
  sv->lane_run.clear();
  sv->lane_nets.clear();
  sv->lane_busy = false;
  sv->lane_inflight = 0;
  if (done.empty()) return;
  char qmsg[256] = {0};
  if (q < 0) snprintf(qmsg, sizeof qmsg, "%s", infoli_last_error());
  for (Request* r : done) sv->lane_reqs.erase(std::find(sv->lane_reqs.begin(), sv->lane_reqs.end(), r));
  lk.unlock();
  cudaStream_t s = static_cast<cudaStream_t>(infoli__lane_stream(sv->lane));
  std::vector<int> rcs(done.size(), q < 0 ? q : INFOLI_OK);
  for (size_t k = 0; k < done.size() && q >= 0; ++k) {
    Request* r = done[k];
    const int n = r->n;
    r->result.resize((size_t)INFOLI_NSTATE * n);
    std::vector<double> ca((size_t)n);
    cudaError_t e = cudaMemcpyAsync(r->result.data(), r->d_st, r->result.size() * sizeof(float),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ca.data(), r->d_ca, ca.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      rcs[k] = INFOLI_ERR_CUDA;
      snprintf(qmsg, sizeof qmsg, "lane read-back: %s", cudaGetErrorString(e));
    } else {
      for (int c = 0; c < n; ++c) r->result[(size_t)4 * n + c] = (float)ca[c];
    }
  }
  for (Request* r : done) lane_free(sv, r);
  lk.lock();
  for (size_t k = 0; k < done.size(); ++k) {
    sv->mem_in_use -= done[k]->est_bytes;
    finish(sv, done[k], rcs[k], rcs[k] == INFOLI_OK ? nullptr : qmsg);
  }
}

// Launch the lane over the prepared small requests that fit on the SMs the
// persistent grids leave (earliest prepared first; the others wait for the
// next launch with their state on the device).  Caller holds the lock.
bool lane_start(infoli_server* sv, std::unique_lock<std::mutex>& lk) {
  if (sv->lane_busy || sv->lane_reqs.empty()) return false;
  const int cap = sv->nsm - sv->grid_in_use;
  int used = 0;
  for (Request* r : sv->lane_reqs) {
    const int c = infoli__lane_ctas(r->n);
    if (used + c > cap) continue;
    used += c;
    r->chunk = std::min(sv->lane_chunk, r->n_steps - r->steps_done);
    if (r->phase != 3) {
      r->phase = 3;
      r->start_s = sv->now();
    }
    sv->lane_run.push_back(r);
    infoli::LaneNet q{};
    q.st = r->d_st;
    q.ca = r->d_ca;
    q.bits = r->d_bits;
    q.n = r->n;
    q.g = r->g_uniform;
    q.step0 = r->steps_done;
    q.n_steps = r->chunk;
    q.pulse_start = r->pulse_start;
    q.pulse_end = r->pulse_end;
    q.pulse_amp = r->pulse_amp;
    sv->lane_nets.push_back(q);
  }
  if (sv->lane_run.empty()) return false;
  sv->lane_busy = true;
  sv->lane_inflight = used;
  lk.unlock();
  const int rc = infoli__lane_launch(sv->lane, sv->lane_nets.data(), (int)sv->lane_nets.size());
  lk.lock();
  if (rc != INFOLI_OK) lane_complete(sv, lk, rc);
  return true;
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
    // the lane's launch in flight
    if (sv->lane_busy) {
      lk.unlock();
      const int q = infoli__lane_query(sv->lane);
      lk.lock();
      if (q != 0) {
        lane_complete(sv, lk, q);
        progress = true;
      }
    }
    // admit by HBM budget, first in first out with bounded backfill
    const double t = sv->now();
    for (auto it = sv->queue.begin(); it != sv->queue.end();) {
      Request* r = *it;
      const int admitted_or_running =
          (int)(sv->running.size() + sv->ready.size() + sv->to_prep.size() + sv->lane_reqs.size()) + sv->preparing;
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
    // SMs the lane holds: its launch in flight, and at least lane_sms while it
    // has requests (so persistent grids never take the whole device from it)
    const int lane_hold = std::max(sv->lane_inflight, sv->lane_reqs.empty() ? 0 : sv->lane_sms);
    for (size_t i = 0; i < sv->ready.size();) {
      Request* r = sv->ready[i];
      if (sv->grid_in_use + lane_hold + r->grid > sv->nsm) {
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
    // the lane, on the SMs the persistent grids leave
    if (sv->lane && lane_start(sv, lk)) progress = true;
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
  if (d->lane_sms >= 0) {
    sv->lane_sms = std::min(d->lane_sms, sv->nsm - 1);
    sv->lane_chunk = d->lane_chunk_steps > 0 ? d->lane_chunk_steps : 2000;
    sv->lane_edges = d->lane_edges_per_cta > 0 ? d->lane_edges_per_cta : d->lane_edges_per_cta < 0 ? -1 : 24576;
    if (infoli__lane_create(sv->device, d->params, (d->flags & INFOLI_F_KAHAN) ? 1 : 0, &sv->lane) != INFOLI_OK) {
      const std::string msg = infoli_last_error();
      delete sv;
      return infoli__fail(INFOLI_ERR_CUDA, "server_create: %s", msg.c_str());
    }
  }
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
  // the lane: small, light networks with one conductance (path chosen from the
  // request alone).  A lane request runs on its own cluster of one CTA per
  // 1,024 cells; a persistent grid would spread it over more SMs, so only
  // requests whose lane step stays short take the lane: at most lane_edges
  // edges per CTA of the cluster (dense small networks measured several
  // times slower in the lane than on their persistent share).
  r->lane = sv->lane != nullptr && n <= kLaneMaxCells && q->g == nullptr &&
            (sv->lane_edges < 0 || edges <= sv->lane_edges * (int64_t)infoli__lane_ctas(n));
  r->est_bytes = r->lane ? lane_bytes(n) : estimate_bytes(n, edges, q->g != nullptr);
  r->admit_bytes = r->est_bytes;
  r->grid = r->lane ? infoli__lane_ctas(n) : grid_for(sv, n, edges);
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
    info->lane = r->lane ? 1 : 0;
    info->lane_launches = r->lane_launches;
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
  if (active)
    *active = (int)(sv->running.size() + sv->ready.size() + sv->to_prep.size() + sv->lane_reqs.size()) + sv->preparing;
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
  if (sv->lane) cudaStreamSynchronize(static_cast<cudaStream_t>(infoli__lane_stream(sv->lane)));
  for (auto& kv : sv->all) {
    Request* r = kv.second;
    if (r->sim) {
      infoli_sim_sync(r->sim);
      infoli_sim_destroy(r->sim);
    }
    if (sv->lane) lane_free(sv, r);
    delete r;
  }
  infoli__lane_destroy(sv->lane);
  delete sv;
  return INFOLI_OK;
}

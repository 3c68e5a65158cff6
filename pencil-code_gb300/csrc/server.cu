// server.cu -- request server with continuous batching over the box/batch API.
//
// A background thread runs rounds.  Each round it admits waiting requests in
// arrival order while their device memory (pcgb_params_bytes) fits the budget
// and the active count is below max_active, creates and seeds their boxes on
// the device, and picks the requests to advance: the oldest request and the
// younger requests of its class (precision, field count, kernel variant and tile) that
// fit into the kernel waves the oldest one occupies on its own (tiles rounded
// up to whole waves of the GPU), so batching never lengthens the oldest
// request's substeps; when that leaves less than one wave of work on the
// device, younger requests of the other classes fill it.  The picked requests
// advance by `steps` RK3 steps (the smaller of round_steps and the fewest steps
// any of them still needs) with one persistent batched launch per substep per
// class, each class on its own stream so that the classes run side by side.
// Finished boxes are retired (diagnostics, optional copy of the final f), which
// frees their memory for the next admissions.  Requests arriving while a round
// runs join at the next round.  max_active = 1 gives FIFO one-at-a-time service.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "boundcond.h"
#include "../../include/pcgb300.h"
#include "params_check.h"
#include "pcgb_box.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  long long id = 0;
  pcgb_params p;
  int nsteps = 0;
  unsigned long long seed = 0;
  double noise = 0.0, abc = 0.0;
  double* f_out = nullptr;
  double t_submit = 0, t_start = -1, t_finish = -1;
  pcgb_box* box = nullptr;
  int done_steps = 0;
  size_t bytes = 0;
  int status = 0;   // 0 queued, 1 active, 2 done, -1 failed
  double diag[PCGB_NSLOT + 3];
};

struct ClassBatch {
  std::vector<pcgb_box*> members;
  pcgb_batch* batch = nullptr;
};

}  // namespace

struct pcgb_server {
  size_t budget = 0;
  int max_active = 1;
  int round_steps = 10;
  std::mutex mu;
  std::condition_variable cv, done_cv;
  std::deque<Req*> queue;
  std::vector<Req*> active;
  std::map<long long, Req*> all;
  std::map<int, ClassBatch> batches;   // key: ((upwinding*2 + dfloat)*16 + precision)*16 + nf
  std::thread th;
  bool stop = false;
  size_t used = 0, peak_bytes = 0;
  int peak_active = 0;
  long long rounds = 0, completed = 0, next_id = 0;
  Clock::time_point t0;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  void run();
  bool start_box(Req* r);
  void finish_box(Req* r, bool ok);
};

bool pcgb_server::start_box(Req* r) {
  r->box = pcgb_box_create(&r->p);
  if (!r->box) return false;
  const int nf = r->p.lentropy ? 8 : 7, iax = nf - 3;
  for (int k = 0; k < nf; ++k)
    if (pcgb_box_init_field(r->box, k, 0, 0, 0, 0, 0, 0, 0)) return false;
  if (r->abc != 0.0)
    for (int k = 0; k < 3; ++k)
      if (pcgb_box_init_field(r->box, k, 2, r->abc, 1.0, 1.0, 1.0, 1.0, 0)) return false;
  for (int k = 0; k < 3; ++k)
    if (pcgb_box_init_field(r->box, iax + k, 1, r->noise, 0, 0, 0, 0, r->seed * 8 + k)) return false;
  return true;
}

void pcgb_server::finish_box(Req* r, bool ok) {
  if (ok && r->box) {
    if (pcgb_box_diag(r->box, r->diag, PCGB_NSLOT + 3)) ok = false;
    if (ok && r->f_out && pcgb_box_store(r->box, r->f_out)) ok = false;
  }
  if (r->box) pcgb_box_destroy(r->box);
  r->box = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  used -= r->bytes;
  r->t_finish = now();
  r->status = ok ? 2 : -1;
  ++completed;
  done_cv.notify_all();
}

static int class_key(const Req* r) {
  const int upw = (r->p.lupw_uu || r->p.lupw_lnrho) ? 1 : 0;   // the upwinding kernel variant is its own class
  // the compensated FP32 state runs kernels compiled per substep, the plain one does not:
  // separate classes keep every request's result bitwise the one it has alone
  const int comp = (r->p.precision == 4 && r->p.comp) ? 1 : 0;
  // a batched launch carries one tile variant
  return ((((upw * 2 + comp) * 2 + r->p.dfloat) * 16 + r->p.precision) * 16 + (r->p.lentropy ? 8 : 7)) * 8 +
         r->p.tile;
}

// Tiling of a request that names none: FP32 pairs on (16,8) tiles with two CTAs per SM
// for boxes under a wave of (32,8) column tiles, on the 12-warp (32,12) tile above;
// double-float pairs on the 6-warp (16,12) tile; FP64 field-major (16,8).  z-depth n/4
// within [16, 64]: short sweeps give small boxes enough tiles, long ones keep the
// six-plane ring prologue of each tile a small share of a large box's planes.
static void request_tiling(pcgb_params& p) {
  if (p.tile < 0) {
    if (p.precision == 4) {
      const bool upw = p.lupw_uu || p.lupw_lnrho;
      const long long px = 16 + (p.nx + 8 + 15) / 16 * 16, ps = px * (p.ny + 6), fs = ps * (p.nz + 6);
      const bool offsets32 = 2 * fs + 8 * ps < (1LL << 32);   // the 12-warp tile's element offsets
      p.tile = ((long long)((p.nx + 31) / 32) * ((p.ny + 7) / 8) >= 152 && !upw && offsets32) ? 7 : 6;
    } else {
      p.tile = p.dfloat ? 5 : 1;
    }
  }
  if (p.zdepth <= 0) p.zdepth = std::min(64, std::max(16, p.nz / 4));
}

static long long box_tiles(pcgb_box* b) {
  int v[8] = {0};
  pcgb_box_info(b, v, 8);
  return v[7];
}

void pcgb_server::run() {
  // the server thread drives the engine: its own stream between rounds, one per class in them
  cudaStream_t own = nullptr;
  cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking);
  void* prev_stream = pcgb::engine_swap_stream(own);
  std::map<int, cudaStream_t> streams;
  while (true) {
    std::vector<Req*> admitted;
    {
      std::unique_lock<std::mutex> lk(mu);
      while (!stop && queue.empty() && active.empty()) cv.wait_for(lk, std::chrono::milliseconds(50));
      if (stop) break;
      while (!queue.empty() && (int)active.size() < max_active && used + queue.front()->bytes <= budget) {
        Req* r = queue.front();
        queue.pop_front();
        used += r->bytes;
        r->status = 1;
        active.push_back(r);
        admitted.push_back(r);
      }
      if (used > peak_bytes) peak_bytes = used;
      if ((int)active.size() > peak_active) peak_active = (int)active.size();
      if (active.empty()) {   // the head of the queue does not fit an empty device: fail it
        if (!queue.empty()) {
          Req* r = queue.front();
          queue.pop_front();
          r->status = -1;
          r->t_finish = now();
          ++completed;
          done_cv.notify_all();
        }
        continue;
      }
    }
    for (Req* r : admitted) {
      r->t_start = now();
      if (!start_box(r)) {
        finish_box(r, false);
        std::lock_guard<std::mutex> lk(mu);
        active.erase(std::find(active.begin(), active.end(), r));
      }
    }
    std::vector<Req*> act;
    {
      std::lock_guard<std::mutex> lk(mu);
      act = active;   // arrival order
    }
    if (act.empty()) continue;
    // requests advanced this round: the oldest one, its class within the oldest one's waves,
    // then (if less than one wave is busy) the other classes up to one wave
    std::vector<Req*> sel;
    {
      Req* head = act[0];
      const int hk = class_key(head);
      const long long wave = pcgb::box_wave(head->box);
      const long long cap = (box_tiles(head->box) + wave - 1) / wave * wave;
      long long busy = 0;
      std::vector<char> picked(act.size(), 0);
      for (size_t i = 0; i < act.size(); ++i) {
        const long long t = box_tiles(act[i]->box);
        if (class_key(act[i]) == hk && (i == 0 || busy + t <= cap)) { sel.push_back(act[i]); busy += t; picked[i] = 1; }
      }
      if (busy < wave)
        for (size_t i = 0; i < act.size(); ++i) {
          const long long t = box_tiles(act[i]->box);
          if (!picked[i] && busy + t <= wave) { sel.push_back(act[i]); busy += t; }
        }
    }
    int steps = round_steps;
    for (Req* r : sel) steps = std::min(steps, r->nsteps - r->done_steps);
    if (steps < 1) steps = 1;
    // one batch per class; rebuilt when its membership changed
    std::map<int, std::vector<pcgb_box*>> cls;
    for (Req* r : sel) cls[class_key(r)].push_back(r->box);
    // a class whose launches could not be issued fails its members; otherwise every
    // request's own device state decides (one box turning non-finite fails that box only)
    std::map<int, bool> class_ok;
    std::vector<cudaStream_t> used_streams;
    for (auto& kv : cls) {
      cudaStream_t& cs = streams[kv.first];
      if (!cs) cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
      pcgb::engine_swap_stream(cs);
      used_streams.push_back(cs);
      class_ok[kv.first] = true;
      ClassBatch& cb = batches[kv.first];
      if (cb.members != kv.second || !cb.batch) {
        if (cb.batch) pcgb_batch_destroy(cb.batch);
        cb.members = kv.second;
        cb.batch = pcgb_batch_create(cb.members.data(), (int)cb.members.size(), 1);
        if (!cb.batch) { class_ok[kv.first] = false; continue; }
      }
      if (pcgb_batch_steps(cb.batch, steps, 0, 0)) class_ok[kv.first] = false;
    }
    bool streams_ok = true;
    for (cudaStream_t cs : used_streams)
      if (cudaStreamSynchronize(cs) != cudaSuccess) streams_ok = false;
    pcgb::engine_swap_stream(own);
    for (auto it = batches.begin(); it != batches.end();) {
      if (!cls.count(it->first)) {
        if (it->second.batch) pcgb_batch_destroy(it->second.batch);
        it = batches.erase(it);
      } else {
        ++it;
      }
    }
    ++rounds;
    for (Req* r : sel) {
      const bool ok = streams_ok && class_ok[class_key(r)] && pcgb_box_sync(r->box) == 0;
      if (!ok) pcgb_clear_error();
      r->done_steps += steps;
      if (r->done_steps >= r->nsteps || !ok) {
        // the batch that holds this box is rebuilt next round (membership changes)
        for (auto& kv : batches) {
          auto& m = kv.second.members;
          if (std::find(m.begin(), m.end(), r->box) != m.end()) {
            if (kv.second.batch) pcgb_batch_destroy(kv.second.batch);
            kv.second.batch = nullptr;
            m.clear();
          }
        }
        finish_box(r, ok);
        std::lock_guard<std::mutex> lk(mu);
        active.erase(std::find(active.begin(), active.end(), r));
      }
    }
  }
  for (auto& kv : batches)
    if (kv.second.batch) pcgb_batch_destroy(kv.second.batch);
  batches.clear();
  cudaStreamSynchronize(own);
  pcgb::engine_swap_stream(prev_stream);
  for (auto& kv : streams)
    if (kv.second) cudaStreamDestroy(kv.second);
  cudaStreamDestroy(own);
}

extern "C" pcgb_server* pcgb_server_create(size_t mem_budget_bytes, int max_active, int round_steps) {
  if (mem_budget_bytes == 0 || max_active < 1 || round_steps < 1) return nullptr;
  pcgb_server* s = new pcgb_server();
  s->budget = mem_budget_bytes;
  s->max_active = max_active;
  s->round_steps = round_steps;
  s->t0 = Clock::now();
  s->th = std::thread([s] { s->run(); });
  return s;
}

extern "C" long long pcgb_server_submit(pcgb_server* s, const pcgb_params* p, int nsteps, unsigned long long seed,
                                        double noise_ampl, double abc_ampl, double* f_out) {
  if (!s || !p || nsteps < 1) return -1;
  if (p->lforcing_hel) return -1;   // the step-end helical forcing runs through the box API only
  for (int d = 0; d < 3; ++d)
    if (!pcgb::axis_periodic(*p, d)) return -1;   // so do the ghost passes of non-periodic boundaries
  Req* r = new Req();
  r->p = *p;
  request_tiling(r->p);
  r->nsteps = nsteps;
  r->seed = seed;
  r->noise = noise_ampl;
  r->abc = abc_ampl;
  r->f_out = f_out;
  r->bytes = pcgb_params_bytes(&r->p);
  if (r->bytes == 0) { delete r; return -1; }
  std::memset(r->diag, 0, sizeof(r->diag));
  std::lock_guard<std::mutex> lk(s->mu);
  r->id = s->next_id++;
  r->t_submit = s->now();
  s->all[r->id] = r;
  s->queue.push_back(r);
  s->cv.notify_all();
  return r->id;
}

extern "C" int pcgb_server_poll(pcgb_server* s, long long id, double* times, double* diag) {
  if (!s) return -2;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return -2;
  Req* r = it->second;
  if (r->status == 2 || r->status == -1) {
    if (times) { times[0] = r->t_submit; times[1] = r->t_start; times[2] = r->t_finish; }
    if (diag) std::memcpy(diag, r->diag, sizeof(r->diag));
    return r->status == 2 ? 1 : -1;
  }
  return 0;
}

extern "C" int pcgb_server_drain(pcgb_server* s, double timeout_s) {
  if (!s) return -1;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s);
  while (s->completed < s->next_id) {
    if (s->done_cv.wait_until(lk, deadline) == std::cv_status::timeout && s->completed < s->next_id) return 1;
  }
  return 0;
}

extern "C" int pcgb_server_stats(pcgb_server* s, double* st, int n) {
  if (!s || !st) return -1;
  std::lock_guard<std::mutex> lk(s->mu);
  const double v[6] = {(double)s->next_id, (double)s->completed, (double)s->active.size(), (double)s->peak_active,
                       (double)s->peak_bytes, (double)s->rounds};
  for (int i = 0; i < n && i < 6; ++i) st[i] = v[i];
  return 0;
}

extern "C" void pcgb_server_destroy(pcgb_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  for (Req* r : s->active)
    if (r->box) pcgb_box_destroy(r->box);
  for (auto& kv : s->all) delete kv.second;
  delete s;
}

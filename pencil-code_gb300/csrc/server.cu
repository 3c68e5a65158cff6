// server.cu -- request server with continuous batching over the box/batch API.
//
// A background thread runs rounds: it admits waiting requests in arrival
// order while their device memory (pcgb_params_bytes) fits the budget and the
// active count is below max_active, creates and seeds their boxes on the
// device, advances every active box by `steps` RK3 steps (steps = the smaller
// of round_steps and the fewest steps any active box still needs) with one
// persistent batched launch per substep per class (precision, field count),
// then retires finished boxes (diagnostics, optional copy of the final f),
// which frees their memory for the next admissions.  Requests arriving while
// a round runs join at the next round boundary.  max_active = 1 turns the
// same loop into FIFO one-at-a-time service.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "boundcond.h"
#include "../../include/pcgb300.h"
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

void pcgb_server::run() {
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
      act = active;
    }
    if (act.empty()) continue;
    int steps = round_steps;
    for (Req* r : act) steps = std::min(steps, r->nsteps - r->done_steps);
    if (steps < 1) steps = 1;
    // one batch per class; rebuilt when its membership changed
    std::map<int, std::vector<pcgb_box*>> cls;
    for (Req* r : act) {
      const int upw = (r->p.lupw_uu || r->p.lupw_lnrho) ? 1 : 0;   // the upwinding kernel variant is its own class
      cls[((upw * 2 + r->p.dfloat) * 16 + r->p.precision) * 16 + (r->p.lentropy ? 8 : 7)].push_back(r->box);
    }
    bool ok = true;
    for (auto& kv : cls) {
      ClassBatch& cb = batches[kv.first];
      if (cb.members != kv.second || !cb.batch) {
        if (cb.batch) pcgb_batch_destroy(cb.batch);
        cb.members = kv.second;
        cb.batch = pcgb_batch_create(cb.members.data(), (int)cb.members.size(), 1);
        if (!cb.batch) { ok = false; continue; }
      }
      if (pcgb_batch_steps(cb.batch, steps, 0, 0)) ok = false;
    }
    for (auto it = batches.begin(); it != batches.end();) {
      if (!cls.count(it->first)) {
        if (it->second.batch) pcgb_batch_destroy(it->second.batch);
        it = batches.erase(it);
      } else {
        ++it;
      }
    }
    if (!act.empty()) pcgb_box_sync(act[0]->box);
    ++rounds;
    for (Req* r : act) {
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
  // (16,8) tiles suit small boxes: packed pairs for FP32 and double-float, field-major for FP64
  if (r->p.tile < 0) r->p.tile = (r->p.precision == 4 || r->p.dfloat) ? 6 : 1;
  if (r->p.zdepth <= 0) r->p.zdepth = 16;
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

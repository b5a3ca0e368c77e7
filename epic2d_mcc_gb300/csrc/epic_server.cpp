// Continuous-batching serving loop (include/epic2d_serve.h): one scheduler
// thread admits arriving runs against a device-memory budget and a slot
// limit, keeps every admitted run resident on its own stream, and advances
// all of them in graph-replayed chunks that overlap on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/epic2d.h"
#include "../../include/epic2d_serve.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Run {
  epic_request req;
  epic_result res;
  int64_t bytes = 0;
  bool exclusive = false;
  epic_sim* sim = nullptr;
  int steps_enq = 0, steps_done = 0;
  std::deque<std::pair<cudaEvent_t, int>> chunks;  // recorded after each enqueued chunk
  bool done = false;
};

// Runs admitted alone: those whose FP64 solve is a cooperative launch with one
// CTA per SM (the PCG, red-black SOR), which would wait for the whole GPU
// beside other runs.  The mixed form's spectral solve is a cooperative launch
// too, sized to its lattice's tiles (at most two CTAs per SM); served runs
// share the GPU with it.  Every grid-wide wait is bounded (a run whose wait
// gives up fails with EPIC_ERR_TIMEOUT instead of hanging).
bool needs_exclusive(const epic_config& c) {
  const bool spectral = c.precision == EPIC_PRECISION_MIXED && c.nx >= 3 && c.ny >= 3 &&
                        (c.solver == EPIC_SOLVER_PCG || (c.solver == EPIC_SOLVER_GS && c.dx == c.dy));
  if (spectral) return false;
  if (c.solver == EPIC_SOLVER_PCG) return true;
  return c.solver == EPIC_SOLVER_GS && c.sor_mode == EPIC_SOR_REDBLACK;
}

}  // namespace

struct epic_server {
  int64_t budget = 0;
  int max_inflight = 1;
  int chunk = 16;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::vector<Run*> runs;        // by id
  std::deque<Run*> pending;      // by arrival
  std::vector<Run*> inflight;
  std::thread th;
  bool started = false, stop = false;
  Clock::time_point t0;
  std::vector<double> ela, exc, ion;
  double e_min = 0, e_max = 0;
  int64_t used = 0, peak_bytes = 0;
  int peak_inflight = 0;
  int64_t finished = 0;
  std::vector<cudaEvent_t> events;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  cudaEvent_t take_event() {
    if (!events.empty()) {
      cudaEvent_t e = events.back();
      events.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
  }

  void finish(Run* r, int status) {
    r->res.status = status;
    r->res.finish_s = now();
    if (r->sim) {
      epic_destroy(r->sim);
      r->sim = nullptr;
    }
    for (auto& c : r->chunks) events.push_back(c.first);
    r->chunks.clear();
    r->done = true;
    finished++;
  }

  // Creates, loads and starts a run (all on the run's stream, asynchronously).
  int admit(Run* r) {
    const epic_request& q = r->req;
    int st = epic_create(&q.cfg, &r->sim);
    if (st) return st;
    for (int k = 0; k < q.num_species && !st; k++) st = epic_add_species(r->sim, &q.species[k], nullptr);
    for (int k = 0; k < q.num_conductors && !st; k++) st = epic_add_conductor(r->sim, &q.conductors[k]);
    for (int k = 0; k < q.num_emitters && !st; k++) st = epic_add_emitter(r->sim, &q.emitters[k]);
    if (!st && q.collisions && !ela.empty())
      st = epic_set_log_cross_sections(r->sim, ela.data(), exc.data(), ion.data(), (int64_t)ela.size(), e_min, e_max);
    // the host loader keeps particles out of conductors (it blocks the
    // scheduler for the load); the device loader places the rest
    if (!st) st = q.num_conductors ? epic_load_particles(r->sim, (uint32_t)q.load_seed)
                                   : epic_load_particles_device(r->sim, q.load_seed);
    if (!st) st = epic_initial_field_async(r->sim);
    return st;
  }

  // Results of a finished run: status of its work, digest, energies.
  int conclude(Run* r) {
    int st = epic_sync(r->sim);
    if (st) return st;
    st = epic_digest(r->sim, r->res.digest);
    if (st) return st;
    double ke = 0;
    for (int k = 0; k < r->req.num_species; k++) {
      double e3[3];
      if ((st = epic_compute_ke(r->sim, k, 0, e3))) return st;
      ke += e3[0] + e3[1] + e3[2];
    }
    r->res.kinetic_energy = ke;
    return epic_compute_pe(r->sim, 0, &r->res.potential_energy);
  }

  bool tick() {
    bool progressed = false;
    const double t = now();
    // Advance resident runs.
    for (size_t i = 0; i < inflight.size();) {
      Run* r = inflight[i];
      int st = EPIC_OK;
      while (!r->chunks.empty()) {
        const cudaError_t q = cudaEventQuery(r->chunks.front().first);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) {
          st = EPIC_ERR_CUDA;
          break;
        }
        r->steps_done += r->chunks.front().second;
        events.push_back(r->chunks.front().first);
        r->chunks.pop_front();
        progressed = true;
      }
      while (!st && r->steps_enq < r->req.steps && r->chunks.size() < 2) {
        const int k = std::min(chunk, r->req.steps - r->steps_enq);
        st = epic_run_async(r->sim, k, r->req.collisions);
        if (st) break;
        cudaEvent_t e = take_event();
        cudaEventRecord(e, (cudaStream_t)epic_stream(r->sim));
        r->chunks.push_back({e, k});
        r->steps_enq += k;
        progressed = true;
      }
      if (st || (r->steps_done == r->req.steps && r->chunks.empty())) {
        if (!st) st = conclude(r);
        used -= r->bytes;
        finish(r, st);
        inflight.erase(inflight.begin() + i);
        progressed = true;
        cv.notify_all();
        continue;
      }
      i++;
    }
    // Admit arrivals.
    while (!pending.empty()) {
      Run* r = pending.front();
      if (r->req.arrival_s > t) break;
      if ((int)inflight.size() >= max_inflight) break;
      bool excl_running = false;
      for (Run* x : inflight) excl_running |= x->exclusive;
      if (excl_running || (r->exclusive && !inflight.empty())) break;
      if (used + r->bytes > budget) {
        if (!inflight.empty()) break;
        pending.pop_front();  // can never fit
        finish(r, EPIC_ERR_BUDGET);
        progressed = true;
        cv.notify_all();
        continue;
      }
      pending.pop_front();
      r->res.admit_s = now();
      int st = admit(r);
      if (st) {
        finish(r, st);
        cv.notify_all();
      } else {
        inflight.push_back(r);
        used += r->bytes;
        peak_bytes = std::max(peak_bytes, used);
        peak_inflight = std::max(peak_inflight, (int)inflight.size());
      }
      progressed = true;
    }
    return progressed;
  }

  void loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      const bool busy = tick();
      if (busy) continue;
      // Idle: sleep until the next arrival or a short poll interval.
      double wait = 2e-4;
      if (inflight.empty() && !pending.empty()) wait = std::max(0.0, pending.front()->req.arrival_s - now());
      if (inflight.empty() && pending.empty()) wait = 0.05;
      cv.wait_for(lk, std::chrono::duration<double>(std::min(wait, 0.05)));
    }
  }
};

extern "C" {

int64_t epic_estimate_bytes(const epic_config* c, const epic_species_desc* sp, int nsp, int collisions) {
  if (!c || (!sp && nsp > 0)) return -1;
  const int64_t N = (int64_t)c->nx * c->ny;
  const bool mixed = c->precision == EPIC_PRECISION_MIXED;
  int64_t b = N * 8 * (4 + 2 + 8) + N * 16 * nsp;  // phi rho efx efy, ef, 8 solver vectors, den + acc
  if (mixed) {
    b += N * 8;                                                            // ef32
    b += 3 * N * 4 + ((int64_t)c->nx * c->nx + (int64_t)c->ny * c->ny) * 4;  // spectral D, scratch, transforms
  }
  int64_t cmax = 0, nmax = 0;
  for (int k = 0; k < nsp; k++) {
    const int64_t n = sp[k].numparticle;
    const int64_t cap = sp[k].capacity > 0 ? sp[k].capacity : n + n / 2 + 4096;
    b += cap * (mixed ? 24 : 40) + (cap / 1024 + 2) * 8;
    cmax = std::max(cmax, cap);
    nmax = std::max(nmax, n);
  }
  b += nmax * 40;                                           // loader / upload staging
  if (c->sort_every > 0) b += cmax * (16 + (mixed ? 24 : 40)) + 512 * 4 * (cmax / 4096 + 1);
  if (collisions && nsp > 0) {
    const int64_t ecap = sp[0].capacity > 0 ? sp[0].capacity : (int64_t)sp[0].numparticle * 3 / 2 + 4096;
    b += ecap * 8 + std::max<int64_t>(ecap / 8, 65536) * 80 + 4 * 1000 * 8 * 8;
  }
  return b + b / 64 + (8 << 20);
}

epic_status epic_server_create(int64_t budget, int max_inflight, int chunk_steps, epic_server** out) {
  if (!out || budget <= 0 || max_inflight < 1 || chunk_steps < 1) return EPIC_ERR_INVALID;
  epic_server* s = new epic_server();
  s->budget = budget;
  s->max_inflight = max_inflight;
  s->chunk = chunk_steps;
  cudaGetDevice(&s->device);
  s->t0 = Clock::now();
  *out = s;
  return EPIC_OK;
}

void epic_server_destroy(epic_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->th.joinable()) s->th.join();
  for (Run* r : s->inflight) {
    if (r->sim) epic_destroy(r->sim);
    for (auto& c : r->chunks) s->events.push_back(c.first);
  }
  for (Run* r : s->runs) delete r;
  for (cudaEvent_t e : s->events) cudaEventDestroy(e);
  delete s;
}

epic_status epic_server_set_log_cross_sections(epic_server* s, const double* ela, const double* exc,
                                               const double* ion, int64_t n, double e_min, double e_max) {
  if (!s || !ela || !exc || !ion || n < 2) return EPIC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->ela.assign(ela, ela + n);
  s->exc.assign(exc, exc + n);
  s->ion.assign(ion, ion + n);
  s->e_min = e_min;
  s->e_max = e_max;
  return EPIC_OK;
}

epic_status epic_server_submit(epic_server* s, const epic_request* q, int64_t* id) {
  if (!s || !q || q->num_species < 1 || q->num_species > 8 || q->steps < 0) return EPIC_ERR_INVALID;
  if (q->num_conductors < 0 || q->num_conductors > EPIC_REQUEST_MAX_CONDUCTORS || q->num_emitters < 0 ||
      q->num_emitters > EPIC_REQUEST_MAX_EMITTERS)
    return EPIC_ERR_INVALID;
  Run* r = new Run();
  r->req = *q;
  // Room for the injections: a species that emitters feed gets the default
  // capacity plus every particle they add over the run.
  for (int e = 0; e < q->num_emitters; e++) {
    const epic_emitter& m = q->emitters[e];
    if (m.species_idx1 < 0 || m.species_idx1 >= q->num_species || m.species_idx2 < 0 ||
        m.species_idx2 >= q->num_species || m.numparticle < 0) {
      delete r;
      return EPIC_ERR_INVALID;
    }
  }
  for (int k = 0; k < q->num_species; k++) {
    int64_t inj = 0;
    for (int e = 0; e < q->num_emitters; e++) {
      const epic_emitter& m = q->emitters[e];
      if (m.species_idx1 == k || m.species_idx2 == k) inj += (int64_t)m.numparticle * q->steps;
    }
    epic_species_desc& d = r->req.species[k];
    if (inj > 0) {
      const int64_t base = d.capacity > 0 ? d.capacity : d.numparticle + d.numparticle / 2 + 4096;
      d.capacity = base + inj;
    }
  }
  q = &r->req;
  std::memset(&r->res, 0, sizeof(r->res));
  r->res.arrival_s = q->arrival_s;
  r->bytes = epic_estimate_bytes(&q->cfg, q->species, q->num_species, q->collisions);
  r->res.bytes = r->bytes;
  r->exclusive = needs_exclusive(q->cfg);
  int64_t np = 0;
  for (int k = 0; k < q->num_species; k++) np += q->species[k].numparticle;
  r->res.particle_steps = np * (int64_t)q->steps;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->res.id = (int64_t)s->runs.size();
    s->runs.push_back(r);
    auto it = std::upper_bound(s->pending.begin(), s->pending.end(), r,
                               [](const Run* a, const Run* b) { return a->req.arrival_s < b->req.arrival_s; });
    s->pending.insert(it, r);
  }
  s->cv.notify_all();
  if (id) *id = r->res.id;
  return EPIC_OK;
}

epic_status epic_server_start(epic_server* s) {
  if (!s) return EPIC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->started) return EPIC_ERR_INVALID;
  s->started = true;
  s->t0 = Clock::now();
  s->th = std::thread([s] { s->loop(); });
  return EPIC_OK;
}

epic_status epic_server_wait(epic_server* s, double timeout_s) {
  if (!s) return EPIC_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                 [s] { return s->finished == (int64_t)s->runs.size(); });
  return ok ? EPIC_OK : EPIC_ERR_TIMEOUT;
}

epic_status epic_server_result(epic_server* s, int64_t id, epic_result* out) {
  if (!s || !out) return EPIC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (id < 0 || id >= (int64_t)s->runs.size()) return EPIC_ERR_INVALID;
  *out = s->runs[id]->res;
  return s->runs[id]->done ? EPIC_OK : EPIC_ERR_INVALID;
}

epic_status epic_server_get_stats(epic_server* s, epic_server_stats* o) {
  if (!s || !o) return EPIC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(o, 0, sizeof(*o));
  std::vector<double> lat;
  double first = 1e300, last = 0, pst = 0;
  for (Run* r : s->runs) {
    o->submitted++;
    if (!r->done) continue;
    if (r->res.status != EPIC_OK) {
      o->failed++;
      continue;
    }
    o->completed++;
    lat.push_back(r->res.finish_s - r->res.arrival_s);
    first = std::min(first, r->res.arrival_s);
    last = std::max(last, r->res.finish_s);
    pst += (double)r->res.particle_steps;
  }
  if (!lat.empty()) {
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) {  // nearest rank
      size_t k = (size_t)std::ceil(p * lat.size());
      return lat[std::min(lat.size(), std::max<size_t>(k, 1)) - 1];
    };
    o->p50_latency_s = pct(0.50);
    o->p99_latency_s = pct(0.99);
    double sum = 0;
    for (double v : lat) sum += v;
    o->mean_latency_s = sum / lat.size();
    o->max_latency_s = lat.back();
    o->makespan_s = last - first;
    o->particle_steps_per_s = o->makespan_s > 0 ? pst / o->makespan_s : 0;
  }
  o->peak_bytes = s->peak_bytes;
  o->peak_inflight = s->peak_inflight;
  return EPIC_OK;
}

}  // extern "C"

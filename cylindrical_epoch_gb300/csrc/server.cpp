// server.cpp -- request loop for parameter scans (cyl_server_* in cylpic.h).
//
// A queue of jobs and a pool of worker threads on one GPU.  The head of the
// queue is admitted when its estimated device memory fits the HBM budget
// (strict arrival order, so a large job cannot be starved by small ones); a
// worker then loads the job's species on the host with the reference's
// loader and KISS stream, creates a handle (its own non-blocking CUDA
// stream), picks the push tile shape of a mixed-form run (timed once per
// deck shape, see g_tile_choice), runs the steps as CUDA graphs of 16 steps,
// reads the diagnostics and destroys the handle, which returns the job's
// memory to the budget.
// Workers run their jobs at the same time, so the kernels of several runs
// overlap on the device; a new job is admitted as soon as a worker and
// memory are free.
// In batched mode (cyl_server_create_batched) a worker only loads a small
// mixed-form job (at most one push tile per SM) and creates its handle; one
// stepper thread advances all such open jobs, those with the same number of
// modes together as one cyl_batch (one push launch per step over all their
// tiles), and jobs join and leave the batch at 16-step boundaries
// (continuous batching).  Larger and FP64-form jobs fill the device alone
// and run on their worker's stream as above.
//
// The server is host code on top of the public C ABI; it has no counterpart
// in the reference, which runs one deck per MPI job.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cylpic.h"

namespace {

constexpr int CHUNK_STEPS = 16;

struct Job {
  int64_t id = 0;
  cyl_job_desc desc{};
  std::vector<std::vector<double>> profile, phase;  // owned copies of the laser vectors
  cyl_job_result res{};
};

// Mixed-form tile shape chosen for each deck shape (device, nx, ny, modes,
// particles per cell of the first species), shared by every server of the
// process: the first run of a deck shape times the shapes (cyl_tune_tiles),
// later runs reuse the choice, so a deck runs the same kernels alone and in
// a mix, whatever else is on the device.
std::mutex g_tile_mu;
std::map<std::vector<int64_t>, int> g_tile_choice;

double now_since(const std::chrono::steady_clock::time_point& t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct cyl_server_s {
  int device = 0;
  int64_t budget = 0, in_use = 0;
  int running = 0;
  bool stop = false;
  int64_t next_id = 1;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::map<int64_t, std::unique_ptr<Job>> jobs;
  std::vector<std::thread> workers;
  // batched mode: the workers only open jobs; one stepper thread advances
  // every open job, the mixed-form ones in batches (cyl_batch_step)
  bool batched = false;
  int max_batch = 16;
  int64_t batch_tiles = 0;  // a mixed-form run joins the batches when its tiles (16 x 8 cells) are at most this
  int loading = 0;  // jobs being opened by workers
  struct Active {
    Job* job;
    cyl_handle h;
    int64_t done, n0;
  };
  std::vector<Active> active;
  std::condition_variable cv_active;
  std::thread stepper;
};

namespace {

// Load the job's species on the host (the reference's loader and KISS
// stream), create its handle and initialise it; a mixed-form run then gets
// its push tile shape (timed once per deck shape, see g_tile_choice) when
// `tune`, i.e. unless it is to be batched.  Returns CYL_OK or the failing
// call's status.
int open_job(cyl_server_s* srv, Job* job, bool tune, cyl_handle* out, int64_t* n0_out) {
  if (cudaSetDevice(srv->device) != cudaSuccess) return CYL_ERR_CUDA;
  const cyl_job_desc& d = job->desc;
  cyl_rng_state rng;
  cyl_rng_init(&rng, d.seed);
  const bool counter = d.rng_mode == CYL_RNG_COUNTER;
  // host load of every mobile species (auto_load order, ids continue across species)
  struct Host {
    std::vector<double> x, y, z, px, py, pz, w;
    std::vector<int64_t> id;
  };
  std::vector<Host> hp((size_t)d.nspecies);
  int64_t id_base = 0, n0 = 0;
  for (int i = 0; i < d.nspecies && !counter; ++i) {
    if (d.species[i].immobile) continue;
    int64_t n = 0;
    int r = cyl_host_load_species(&d.grid, &d.species[i], &rng, id_base, nullptr, nullptr, nullptr, nullptr,
                                  nullptr, nullptr, nullptr, nullptr, &n);
    if (r != CYL_OK) return r;
    Host& h = hp[(size_t)i];
    h.x.resize((size_t)n); h.y.resize((size_t)n); h.z.resize((size_t)n);
    h.px.resize((size_t)n); h.py.resize((size_t)n); h.pz.resize((size_t)n);
    h.w.resize((size_t)n); h.id.resize((size_t)n);
    r = cyl_host_load_species(&d.grid, &d.species[i], &rng, id_base, h.x.data(), h.y.data(), h.z.data(),
                              h.px.data(), h.py.data(), h.pz.data(), h.w.data(), h.id.data(), &n);
    if (r != CYL_OK) return r;
    id_base += n;
    n0 += n;
  }
  cyl_laser_desc las[8];
  for (int k = 0; k < d.nlasers; ++k) {
    las[k] = d.lasers[k];
    las[k].profile = job->profile[(size_t)k].data();
    las[k].phase = job->phase[(size_t)k].data();
  }
  cyl_handle h = nullptr;
  int r = cyl_create(&d.grid, d.species, d.nspecies, las, d.nlasers, &rng, &h);
  if (r != CYL_OK) return r;
  for (int i = 0; i < d.nspecies && r == CYL_OK && !counter; ++i) {
    Host& p = hp[(size_t)i];
    const int64_t n = (int64_t)p.x.size();
    if (n == 0) continue;
    r = cyl_upload_particles(h, i, p.x.data(), p.y.data(), p.z.data(), p.px.data(), p.py.data(), p.pz.data(),
                             p.w.data(), p.id.data(), n);
  }
  hp.clear();
  // counter mode: every mobile species loaded on the device (ids continue
  // across species as in the host load), window injection on the device
  for (int i = 0; i < d.nspecies && r == CYL_OK && counter; ++i) {
    if (d.species[i].immobile) continue;
    int64_t n = 0;
    r = cyl_load_species_device(h, i, (uint64_t)(uint32_t)d.seed, id_base, &n);
    id_base += n;
    n0 += n;
  }
  if (r == CYL_OK && counter) r = cyl_set_injection_stream(h, CYL_RNG_COUNTER, (uint64_t)(uint32_t)d.seed);
  if (r == CYL_OK) r = cyl_initialise(h);
  if (r == CYL_OK && d.grid.precision == CYL_PREC_MIXED && tune) {
    const std::vector<int64_t> key = {srv->device, d.grid.nx, d.grid.ny, d.grid.n_mode,
                                      d.nspecies > 0 ? (int64_t)(d.species[0].npart_per_cell * 1000.0) : 0};
    int shape = -1;
    {
      std::lock_guard<std::mutex> lock(g_tile_mu);
      auto it = g_tile_choice.find(key);
      if (it != g_tile_choice.end()) shape = it->second;
    }
    if (shape >= 0) {
      r = cyl_tune_tiles(h, CYL_TUNE_SET, &shape);
    } else {
      r = cyl_tune_tiles(h, CYL_TUNE_TIME, &shape);
      if (r == CYL_OK) {
        std::lock_guard<std::mutex> lock(g_tile_mu);
        g_tile_choice.emplace(key, shape);
      }
    }
  }
  if (r != CYL_OK) {
    cyl_destroy(h);
    return r;
  }
  *out = h;
  *n0_out = n0;
  return CYL_OK;
}

// Read the results of a finished (or failed) run and destroy its handle.
int close_job(Job* job, cyl_handle h, int64_t done, int64_t n0, int r) {
  const cyl_job_desc& d = job->desc;
  if (r == CYL_OK) r = cyl_diagnostics(h, &job->res.diag);
  // steps enqueued without a sync (batches, a batched job's last steps)
  // report a raised device error word here
  if (r == CYL_OK && job->res.diag.device_error != 0) r = CYL_ERR_DEVICE_FLAG;
  if (r == CYL_OK) r = cyl_get_run_state(h, &job->res.state);
  if (r == CYL_OK) {
    int64_t n1 = 0;
    for (int i = 0; i < d.nspecies; ++i)
      if (!d.species[i].immobile) n1 += job->res.state.n_live[i];
    job->res.particle_steps = 0.5 * (double)(n0 + n1) * (double)done;
  }
  cyl_destroy(h);
  return r;
}

// Open, step (graphs of 16 steps on the run's own stream), close.
int run_job(cyl_server_s* srv, Job* job) {
  cyl_handle h = nullptr;
  int64_t n0 = 0;
  int r = open_job(srv, job, true, &h, &n0);
  if (r != CYL_OK) return r;
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    job->res.t_start = now_since(srv->t0);
  }
  int64_t done = 0;
  while (r == CYL_OK && done < job->desc.nsteps) {
    const int k = (int)std::min<int64_t>(CHUNK_STEPS, job->desc.nsteps - done);
    r = cyl_step_graph(h, k);
    if (r == CYL_OK) done += k;
    std::lock_guard<std::mutex> lock(srv->mu);
    job->res.steps_done = done;
  }
  return close_job(job, h, done, n0, r);
}

// Record a finished job and return its memory to the budget.
void retire(cyl_server_s* srv, Job* job, int r) {
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->in_use -= job->res.device_bytes;
    srv->running -= 1;
    job->res.error = r;
    job->res.t_end = now_since(srv->t0);
    job->res.status = (r == CYL_OK) ? CYL_JOB_DONE : CYL_JOB_FAILED;
  }
  srv->cv_work.notify_all();
  srv->cv_done.notify_all();
}

// Is the job one for the batches?  A mixed-form run whose push has at most
// one 16 x 8-cell tile per SM cannot fill the device alone, and many such
// runs stepped as separate streams lose to one launch over all their tiles;
// a larger run fills the device by itself, and a batch's per-step join of
// all members would only cost it the overlap of one run's field stages with
// another's push, so it runs alone on its own stream like an FP64-form run.
bool batchable(const cyl_server_s* srv, const cyl_job_desc& d) {
  if (d.grid.precision != CYL_PREC_MIXED) return false;
  int32_t tx = 0, ty = 0;
  if (cyl_tile_shape(0, &tx, &ty) != CYL_OK || tx < 1 || ty < 1) return false;
  const int64_t tiles = (((int64_t)d.grid.nx + tx - 1) / tx) * (((int64_t)d.grid.ny + ty - 1) / ty);
  return tiles <= srv->batch_tiles;
}

// Batched mode (at most max_batch jobs open at once, counting those being
// loaded and those run alone): advance every batched job by up to
// CHUNK_STEPS steps per pass, those with the same number of modes together
// (cyl_batch_step, at most max_batch per call, whole 16-step chunks; a job
// with fewer steps left finishes alone on its own stream); retire the
// finished ones.  New jobs join at the next pass.
void stepper_main(cyl_server_s* srv) {
  cudaSetDevice(srv->device);
  std::map<int, cyl_batch> batches;
  for (;;) {
    std::vector<cyl_server_s::Active> act;
    {
      std::unique_lock<std::mutex> lock(srv->mu);
      srv->cv_active.wait(lock, [&] {
        return !srv->active.empty() || (srv->stop && srv->queue.empty() && srv->loading == 0);
      });
      if (srv->active.empty()) break;
      act = srv->active;
    }
    std::map<int, std::vector<size_t>> groups;  // runs by modes
    for (size_t a = 0; a < act.size(); ++a) groups[act[a].job->desc.grid.n_mode].push_back(a);
    std::vector<int> err(act.size(), CYL_OK);
    std::vector<int64_t> stepped(act.size(), 0);
    for (auto& g : groups) {
      const int M = g.first;
      if (!batches.count(M)) {
        cyl_batch b = nullptr;
        const int rc = cyl_batch_create(srv->max_batch, &b);
        if (rc != CYL_OK) {
          for (size_t a : g.second) err[a] = rc;
          continue;
        }
        batches[M] = b;
      }
      // a job with fewer than CHUNK_STEPS steps left takes its last steps
      // alone (asynchronously, on its own stream), so that the batch keeps
      // stepping whole graph-captured chunks
      std::vector<size_t> full;
      for (size_t a : g.second) {
        const int64_t left = act[a].job->desc.nsteps - act[a].done;
        if (left >= CHUNK_STEPS) {
          full.push_back(a);
        } else {
          err[a] = cyl_step_async(act[a].h, (int32_t)left);
          stepped[a] = err[a] == CYL_OK ? left : 0;
        }
      }
      for (size_t s0 = 0; s0 < full.size(); s0 += (size_t)srv->max_batch) {
        const size_t s1 = std::min(full.size(), s0 + (size_t)srv->max_batch);
        std::vector<cyl_handle> hs;
        for (size_t q = s0; q < s1; ++q) hs.push_back(act[full[q]].h);
        const int rc = cyl_batch_step(batches[M], hs.data(), (int32_t)hs.size(), CHUNK_STEPS);
        for (size_t q = s0; q < s1; ++q) {
          err[full[q]] = rc;
          stepped[full[q]] = rc == CYL_OK ? CHUNK_STEPS : 0;
        }
      }
    }
    // bookkeeping; finished or failed jobs leave the active set
    std::vector<cyl_server_s::Active> leaving;
    std::vector<int> leaving_err;
    {
      std::lock_guard<std::mutex> lock(srv->mu);
      for (size_t a = 0; a < act.size(); ++a) {
        for (auto& x : srv->active)
          if (x.job == act[a].job) {
            x.done += stepped[a];
            x.job->res.steps_done = x.done;
            if (err[a] != CYL_OK || x.done >= x.job->desc.nsteps) {
              leaving.push_back(x);
              leaving_err.push_back(err[a]);
            }
          }
      }
      for (auto& l : leaving)
        srv->active.erase(std::remove_if(srv->active.begin(), srv->active.end(),
                                         [&](const cyl_server_s::Active& x) { return x.job == l.job; }),
                          srv->active.end());
    }
    for (size_t q = 0; q < leaving.size(); ++q) {
      const int r = close_job(leaving[q].job, leaving[q].h, leaving[q].done, leaving[q].n0, leaving_err[q]);
      retire(srv, leaving[q].job, r);
    }
  }
  for (auto& b : batches) cyl_batch_destroy(b.second);
}

void worker_main(cyl_server_s* srv) {
  for (;;) {
    Job* job = nullptr;
    bool to_stepper = false;
    {
      std::unique_lock<std::mutex> lock(srv->mu);
      // admit the head of the queue when it fits (or when nothing else holds
      // memory); in batched mode also while fewer than max_batch jobs are open,
      // so that queued jobs wait for a place instead of slowing every open one
      srv->cv_work.wait(lock, [&] {
        if (srv->queue.empty()) return srv->stop;
        if (srv->batched && srv->running >= srv->max_batch) return false;
        const int64_t need = srv->queue.front()->res.device_bytes;
        return srv->in_use + need <= srv->budget || srv->in_use == 0;
      });
      if (srv->queue.empty()) return;
      job = srv->queue.front();
      srv->queue.pop_front();
      srv->in_use += job->res.device_bytes;
      srv->running += 1;
      job->res.status = CYL_JOB_RUNNING;
      to_stepper = srv->batched && batchable(srv, job->desc);
      if (to_stepper) srv->loading += 1;  // with the pop, so the stepper never misses it
    }
    if (!to_stepper) {
      retire(srv, job, run_job(srv, job));
      continue;
    }
    cyl_handle h = nullptr;
    int64_t n0 = 0;
    const int r = open_job(srv, job, false, &h, &n0);
    {
      std::lock_guard<std::mutex> lock(srv->mu);
      srv->loading -= 1;
      if (r == CYL_OK) {
        job->res.t_start = now_since(srv->t0);
        srv->active.push_back({job, h, 0, n0});
      }
    }
    if (r != CYL_OK) retire(srv, job, r);
    srv->cv_active.notify_all();
  }
}

}  // namespace

extern "C" {

static int server_create(int64_t hbm_budget_bytes, int32_t workers, bool batched, int32_t max_batch,
                         cyl_server* out) {
  if (!out || workers < 1 || workers > 64 || hbm_budget_bytes < 0) return CYL_ERR_BAD_ARG;
  if (batched && (max_batch < 1 || max_batch > 1024)) return CYL_ERR_BAD_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CYL_ERR_NO_DEVICE;
  auto* srv = new cyl_server_s();
  if (cudaGetDevice(&srv->device) != cudaSuccess) {
    delete srv;
    return CYL_ERR_CUDA;
  }
  if (hbm_budget_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      delete srv;
      return CYL_ERR_CUDA;
    }
    const int64_t reserve = (int64_t)2 << 30;
    hbm_budget_bytes = std::max<int64_t>((int64_t)free_b - reserve, (int64_t)free_b / 2);
  }
  srv->budget = hbm_budget_bytes;
  srv->batched = batched;
  srv->max_batch = max_batch;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, srv->device) != cudaSuccess) {
    delete srv;
    return CYL_ERR_CUDA;
  }
  srv->batch_tiles = sms;
  srv->t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < workers; ++i) srv->workers.emplace_back(worker_main, srv);
  if (batched) srv->stepper = std::thread(stepper_main, srv);
  *out = srv;
  return CYL_OK;
}

int cyl_server_create(int64_t hbm_budget_bytes, int32_t workers, cyl_server* out) {
  return server_create(hbm_budget_bytes, workers, false, 0, out);
}

int cyl_server_create_batched(int64_t hbm_budget_bytes, int32_t loaders, int32_t max_batch, cyl_server* out) {
  return server_create(hbm_budget_bytes, loaders, true, max_batch, out);
}

int cyl_server_submit(cyl_server s, const cyl_job_desc* job, int64_t* job_id) {
  if (!s || !job || !job_id) return CYL_ERR_BAD_ARG;
  if (job->nspecies < 0 || job->nspecies > 8 || job->nlasers < 0 || job->nlasers > 8 || job->nsteps < 0)
    return CYL_ERR_BAD_ARG;
  if (job->rng_mode != CYL_RNG_KISS && job->rng_mode != CYL_RNG_COUNTER) return CYL_ERR_BAD_ARG;
  int64_t bytes = 0;
  int r = cyl_estimate_device_bytes(&job->grid, job->species, job->nspecies, &bytes);
  if (r != CYL_OK) return r;
  auto j = std::make_unique<Job>();
  j->desc = *job;
  const size_t nprof = (size_t)job->grid.ny + 1;
  for (int k = 0; k < job->nlasers; ++k) {
    if (!job->lasers[k].profile || !job->lasers[k].phase) return CYL_ERR_BAD_ARG;
    j->profile.emplace_back(job->lasers[k].profile, job->lasers[k].profile + nprof);
    j->phase.emplace_back(job->lasers[k].phase, job->lasers[k].phase + nprof);
    j->desc.lasers[k].profile = nullptr;
    j->desc.lasers[k].phase = nullptr;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->stop) return CYL_ERR_BAD_ARG;
  if (bytes > s->budget) return CYL_ERR_OUT_OF_MEMORY;
  j->id = s->next_id++;
  j->res.status = CYL_JOB_QUEUED;
  j->res.error = CYL_OK;
  j->res.device_bytes = bytes;
  j->res.t_submit = now_since(s->t0);
  *job_id = j->id;
  s->queue.push_back(j.get());
  s->jobs.emplace(j->id, std::move(j));
  s->cv_work.notify_all();
  return CYL_OK;
}

int cyl_server_poll(cyl_server s, int64_t job_id, cyl_job_result* out) {
  if (!s || !out) return CYL_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end()) return CYL_ERR_BAD_ARG;
  *out = it->second->res;
  return CYL_OK;
}

int cyl_server_wait(cyl_server s, int64_t job_id, double timeout_s, cyl_job_result* out) {
  if (!s || !out || !(timeout_s >= 0.0)) return CYL_ERR_BAD_ARG;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end()) return CYL_ERR_BAD_ARG;
  Job* j = it->second.get();
  const bool ok = s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), [&] {
    return j->res.status == CYL_JOB_DONE || j->res.status == CYL_JOB_FAILED;
  });
  *out = j->res;
  return ok ? CYL_OK : CYL_ERR_TIMEOUT;
}

int cyl_server_stats(cyl_server s, int32_t* queued, int32_t* running, int64_t* bytes_in_use) {
  if (!s) return CYL_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  if (queued) *queued = (int32_t)s->queue.size();
  if (running) *running = s->running;
  if (bytes_in_use) *bytes_in_use = s->in_use;
  return CYL_OK;
}

int cyl_server_destroy(cyl_server s) {
  if (!s) return CYL_ERR_BAD_ARG;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  s->cv_active.notify_all();
  if (s->stepper.joinable()) s->stepper.join();
  delete s;
  return CYL_OK;
}

}  // extern "C"

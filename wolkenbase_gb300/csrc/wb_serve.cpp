/* Request loop around the classify path: wb_server (serving) and
 * wb_classify_batch (batching).
 *
 * Jobs move QUEUED -> PREP -> READY -> CLASSIFY -> DONE.  prep_slots worker
 * threads each take the queue head when the HBM budget admits it, bind it to
 * a context (its own stream and resident buffers) and run the octree build,
 * the tile scan and the classify set-up there.  One classifier thread takes
 * every READY job (or, in WB_FLUSH_FULL mode, waits until nothing more can be
 * admitted) and classifies them together with one launch of a captured graph
 * (wb_batch_launch); scans of newly admitted jobs overlap with it on their
 * own streams.  A finished job's context goes back to the idle pool with its
 * buffers, so the next job of similar size allocates nothing.
 *
 * Memory: a busy context is charged max(bytes it holds, the job's estimate),
 * an idle one what it holds; a job is admitted only if the sum stays within
 * the budget, after freeing idle contexts' buffers if that is needed.  A job
 * that outgrows its estimate (WB_ENOMEM from its context) is re-queued at the
 * head with twice the estimate, up to the whole budget.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include "wb_internal.h"

namespace
{
struct JobRec
{
  int64_t id = 0;
  wb_job spec{};
  wb_job_status st{};
  wb_ctx *ctx = nullptr;
  uint64_t est = 0;
  bool paged = false;   /* above the whole budget: runs alone with paging */
  cudaEvent_t ev = nullptr;
};

/* Device bytes a job of n records is expected to hold: the pipeline's buffers
 * come to about 310 bytes per point (sort keys and values twice, the leaf
 * store and its decoded coordinates, the column grid, the tile lists and the
 * classify set-up, each grown with 1/8 slack), plus the uploaded records. */
uint64_t estimateBytes(const wb_job &j)
{
  uint64_t n = j.cloud.n;
  uint64_t per = 340 + (j.cloud.device_resident ? 0 : j.cloud.stride);
  return n * per + (64ull << 20);
}
}  // namespace

struct wb_server
{
  wb_server_config cfg{};
  uint64_t budget = 0;
  std::mutex m;
  std::condition_variable cv;
  std::deque<JobRec *> queue;
  std::vector<JobRec *> ready;
  std::unordered_map<int64_t, JobRec *> jobs;
  std::vector<wb_ctx *> all, idle;
  std::unordered_map<const wb_ctx *, JobRec *> busy;
  int64_t nextId = 0;
  int prepBusy = 0, classifying = 0;
  bool headBlocked = false, stop = false;
  std::vector<std::thread> preps;
  std::thread classifier;
  cudaStream_t clsStream = nullptr;
  WbBatch *batch = nullptr;
  std::chrono::steady_clock::time_point t0;
  wb_server_stats stats{};
  uint64_t graphLaunches = 0;
  std::string err;

  double now() const
  {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace
{
/* Bytes charged now: idle contexts hold what they hold; busy ones at least
 * their job's estimate. */
uint64_t heldBytes(const wb_server *s)
{
  uint64_t h = 0;
  for (const wb_ctx *c : s->all)
  {
    uint64_t u = c->used;
    auto it = s->busy.find(c);
    h += it == s->busy.end() ? u : std::max<uint64_t>(u, it->second->est);
  }
  return h;
}

/* Picks a context for the queue head if the budget admits it (lock held). */
bool admit(wb_server *s, JobRec *&job, wb_ctx *&ctx)
{
  job = nullptr;
  ctx = nullptr;
  if (s->queue.empty())
  {
    s->headBlocked = false;
    return false;
  }
  JobRec *j = s->queue.front();
  // an idle context already big enough, else the biggest idle one, else a new one
  wb_ctx *best = nullptr;
  for (wb_ctx *c : s->idle)
    if (c->used >= j->est && (!best || c->used < best->used))
      best = c;
  if (!best)
    for (wb_ctx *c : s->idle)
      if (!best || c->used > best->used)
        best = c;
  uint64_t held = heldBytes(s), bu = best ? (uint64_t)best->used : 0;
  uint64_t need = held - bu + std::max<uint64_t>(bu, j->est);
  if (need > s->budget)
  {
    // free the buffers of the other idle contexts
    for (wb_ctx *c : s->idle)
      if (c != best && c->used)
      {
        need -= c->used;
        wb_release_buffers(c);
        if (need <= s->budget)
          break;
      }
  }
  if (need > s->budget)
  {
    // the classifier may be waiting for exactly this (WB_FLUSH_FULL)
    if (!s->headBlocked)
      s->cv.notify_all();
    s->headBlocked = true;
    return false;
  }
  s->headBlocked = false;
  if (!best)
  {
    best = wb_open(s->cfg.device, 0);
    if (!best)
    {
      if (!s->headBlocked)
        s->cv.notify_all();
      s->headBlocked = true;
      return false;
    }
    s->all.push_back(best);
  }
  else
    s->idle.erase(std::find(s->idle.begin(), s->idle.end(), best));
  job = j;
  ctx = best;
  return true;
}

void finish(wb_server *s, JobRec *j, int rc, const std::string &msg)
{
  j->st.rc = rc;
  j->st.state = rc ? WB_JOB_FAILED : WB_JOB_DONE;
  j->st.t_done = s->now();
  if (rc)
  {
    s->stats.failed++;
    s->err = "job " + std::to_string(j->id) + ": " + msg;
  }
  else
  {
    s->stats.completed++;
    s->stats.points += j->st.n_points;
  }
  if (j->ctx)
  {
    s->busy.erase(j->ctx);
    s->idle.push_back(j->ctx);
    j->ctx = nullptr;
  }
  if (j->ev)
  {
    cudaEventDestroy(j->ev);
    j->ev = nullptr;
  }
}

int runPrep(JobRec *j, wb_ctx *c, double gridPoints, uint64_t hostBudget)
{
  c->budget = std::max<uint64_t>(c->used, j->est);
  c->grid_points = gridPoints;
  int rc = wb_set_paging(c, j->paged ? hostBudget : 0);
  if (rc == 0)
    rc = wb_build_impl(c, &j->spec.cloud);
  if (rc == 0)
    rc = wb_scan_impl(c, &j->spec.params);
  if (rc == 0)
    rc = wb_classify_stage(c, &j->spec.params, j->spec.cls, 0);
  if (rc == 0 && !j->ev && cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming) != cudaSuccess)
    rc = wb_fail(c, WB_ECUDA, "cudaEventCreate failed");
  if (rc == 0 && cudaEventRecord(j->ev, c->stream) != cudaSuccess)
    rc = wb_fail(c, WB_ECUDA, "cudaEventRecord failed");
  return rc;
}

void prepLoop(wb_server *s)
{
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->m);
  for (;;)
  {
    JobRec *j = nullptr;
    wb_ctx *c = nullptr;
    s->cv.wait(lk, [&] { return s->stop || admit(s, j, c); });
    if (!j)
      return;
    s->queue.pop_front();
    j->ctx = c;
    s->busy[c] = j;
    j->st.state = WB_JOB_PREP;
    j->st.t_admit = s->now();
    j->st.reserved_bytes = j->est;
    s->prepBusy++;
    s->stats.peak_bytes = std::max<uint64_t>(s->stats.peak_bytes, heldBytes(s));
    double gp = s->cfg.grid_points;
    lk.unlock();
    int rc = runPrep(j, c, gp, s->cfg.host_budget);
    std::string msg = rc ? c->err : std::string();
    if (rc && j->paged)
      wb_release_buffers(c);   // no host-memory buffers left behind for the next job
    lk.lock();
    s->prepBusy--;
    s->stats.peak_bytes = std::max<uint64_t>(s->stats.peak_bytes, heldBytes(s));
    if (rc == 0)
    {
      j->st.state = WB_JOB_READY;
      j->st.t_ready = s->now();
      s->ready.push_back(j);
    }
    else if (rc == WB_ENOMEM && j->est < s->budget)
    {
      // outgrew its estimate: back to the head of the queue with a larger one
      j->est = std::min<uint64_t>(j->est * 2, s->budget);
      s->busy.erase(c);
      s->idle.push_back(c);
      j->ctx = nullptr;
      j->st.state = WB_JOB_QUEUED;
      s->queue.push_front(j);
    }
    else
      finish(s, j, rc, msg);
    s->cv.notify_all();
  }
}

bool flushNow(const wb_server *s)
{
  if (s->ready.empty())
    return false;
  if (s->cfg.flush == WB_FLUSH_EAGER || s->stop || (int)s->ready.size() >= s->cfg.max_batch)
    return true;
  // full batches: wait while more jobs can still become ready
  return s->prepBusy == 0 && (s->queue.empty() || s->headBlocked);
}

/* The autotuner (first batch, classifier thread, lock not held): times the
 * settings on the batch's jobs, largest first, up to about 8M points
 * (wb_autotune_jobs). */
double autotune(wb_server *s, std::vector<JobRec *> &batch, int &shape, int &chunk, double &gridPoints,
                std::string &err)
{
  auto t0 = std::chrono::steady_clock::now();
  std::vector<JobRec *> order(batch);
  std::sort(order.begin(), order.end(), [](JobRec *x, JobRec *y) { return x->ctx->nd > y->ctx->nd; });
  std::vector<WbTuneJob> jobs;
  uint64_t pts = 0;
  for (JobRec *j : order)
  {
    if (!jobs.empty() && pts + j->ctx->nd > 8000000)
      continue;
    jobs.push_back(WbTuneJob{j->ctx, &j->spec.params, j->spec.cls, 0});
    pts += j->ctx->nd;
  }
  if (wb_autotune_jobs(s->batch, jobs.data(), (int)jobs.size(), s->clsStream, &shape, &chunk, &gridPoints, err) == 0)
    err.clear();
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void classifyLoop(wb_server *s)
{
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->m);
  for (;;)
  {
    s->cv.wait(lk, [&] { return flushNow(s) || (s->stop && s->prepBusy == 0 && s->ready.empty()); });
    if (s->ready.empty())
      return;
    int k = std::min<int>((int)s->ready.size(), s->cfg.max_batch);
    std::vector<JobRec *> batch(s->ready.begin(), s->ready.begin() + k);
    s->ready.erase(s->ready.begin(), s->ready.begin() + k);
    std::vector<wb_ctx *> ctxs;
    for (JobRec *j : batch)
    {
      j->st.state = WB_JOB_CLASSIFY;
      ctxs.push_back(j->ctx);
    }
    s->classifying++;
    lk.unlock();
    std::string err;
    int rc = 0;
    for (JobRec *j : batch)
      if (cudaStreamWaitEvent(s->clsStream, j->ev, 0) != cudaSuccess)
        rc = WB_ECUDA;
    // tune on a batch whose largest job gives a sample big enough to time
    size_t biggest = 0;
    for (JobRec *j : batch)
      biggest = std::max<size_t>(biggest, j->ctx->nd);
    if (rc == 0 && s->cfg.autotune && !s->stats.tuned && biggest >= 1000000)
    {
      int shape = s->cfg.shape, chunk = s->cfg.chunk;
      double gp = s->cfg.grid_points;
      std::string terr;
      double ms = autotune(s, batch, shape, chunk, gp, terr);
      std::lock_guard<std::mutex> g(s->m);
      s->cfg.shape = shape;
      s->cfg.chunk = chunk;
      s->cfg.grid_points = gp;
      s->stats.tuned = 1;
      s->stats.tune_ms = ms;
      if (!terr.empty())
        s->err = "autotune: " + terr;
    }
    uint64_t launches = 0;
    if (rc == 0)
      rc = wb_batch_launch(s->batch, ctxs.data(), k, s->clsStream, s->cfg.shape, s->cfg.chunk, &launches, err);
    // wait even after a failed launch: the jobs' contexts go back to the pool
    // and must not be reused while work that reads them may still run
    cudaError_t e = cudaStreamSynchronize(s->clsStream);
    if (rc == 0 && e != cudaSuccess)
    {
      rc = WB_ECUDA;
      err = std::string("fused classify: ") + cudaGetErrorString(e);
    }
    if (rc == 0)
      wb_batch_collect(s->batch, ctxs.data(), k);
    // a paged job's context gives its host memory back before it serves
    // another job (whose buffers must not stay in host memory)
    for (JobRec *j : batch)
      if (j->paged)
        wb_release_buffers(j->ctx);
    lk.lock();
    s->classifying--;
    s->graphLaunches += launches;
    if (rc == 0)
    {
      s->stats.fused_launches++;
      s->stats.fused_jobs += k;
    }
    for (JobRec *j : batch)
    {
      if (rc == 0)
      {
        j->st.n_ground = j->ctx->n_ground;
        j->st.n_ambiguous = j->ctx->n_ambiguous;
        j->st.batch_jobs = k;
      }
      finish(s, j, rc, err);
    }
    s->cv.notify_all();
  }
}
}  // namespace

extern "C" {

wb_server *wb_server_open(const wb_server_config *cfg)
{
  if (!cfg)
  {
    wb_fail(nullptr, WB_EINVAL, "wb_server_open: cfg is NULL");
    return nullptr;
  }
  WbDeviceGuard deviceGuard(cfg->device);
  wb_ctx *probe = wb_open(cfg->device, 0);   // validates the device
  if (!probe)
    return nullptr;
  wb_server *s = new (std::nothrow) wb_server;
  if (!s)
  {
    wb_close(probe);
    return nullptr;
  }
  s->cfg = *cfg;
  if (s->cfg.prep_slots <= 0)
    s->cfg.prep_slots = 4;
  if (s->cfg.max_batch <= 0 || s->cfg.max_batch > WB_BATCH_MAX)
    s->cfg.max_batch = WB_BATCH_MAX;
  if (s->cfg.shape < 0 || s->cfg.shape >= WB_N_SHAPES)
    s->cfg.shape = 0;
  if (!(s->cfg.grid_points > 0))
    s->cfg.grid_points = 64;
  if (s->cfg.chunk <= 0)
    s->cfg.chunk = 1;
  size_t freeB = 0, totalB = 0;
  cudaMemGetInfo(&freeB, &totalB);
  s->budget = cfg->hbm_budget ? cfg->hbm_budget : (uint64_t)(freeB * 0.8);
  s->stats.budget = s->budget;
  // keep freed stream-ordered blocks in the pool for the next job
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, cfg->device) == cudaSuccess)
  {
    uint64_t thr = s->budget;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  s->all.push_back(probe);
  s->idle.push_back(probe);
  std::string err;
  if (cudaStreamCreateWithFlags(&s->clsStream, cudaStreamNonBlocking) != cudaSuccess ||
      wb_batch_create(cfg->device, &s->batch, err) != 0)
  {
    wb_fail(nullptr, WB_ECUDA, "wb_server_open: " + (err.empty() ? std::string("stream creation failed") : err));
    if (s->clsStream)
      cudaStreamDestroy(s->clsStream);
    wb_close(probe);
    delete s;
    return nullptr;
  }
  s->t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < s->cfg.prep_slots; i++)
    s->preps.emplace_back(prepLoop, s);
  s->classifier = std::thread(classifyLoop, s);
  return s;
}

void wb_server_close(wb_server *s)
{
  if (!s)
    return;
  {
    std::lock_guard<std::mutex> lk(s->m);
    for (JobRec *j : s->queue)
    {
      j->st.state = WB_JOB_CANCELLED;
      j->st.rc = WB_ECANCELED;
      s->stats.cancelled++;
    }
    s->queue.clear();
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto &t : s->preps)
    t.join();
  s->classifier.join();
  WbDeviceGuard deviceGuard(s->cfg.device);
  for (wb_ctx *c : s->all)
    wb_close(c);
  wb_batch_destroy(s->batch);
  cudaStreamDestroy(s->clsStream);
  for (auto &kv : s->jobs)
  {
    if (kv.second->ev)
      cudaEventDestroy(kv.second->ev);
    delete kv.second;
  }
  delete s;
}

const char *wb_server_error(const wb_server *s)
{
  return s ? s->err.c_str() : wb_last_error(nullptr);
}

int64_t wb_submit(wb_server *s, const wb_job *job)
{
  if (!s || !job || (job->cloud.n && (!job->cloud.records || !job->cls)))
    return WB_EINVAL;
  if (job->cloud.stride < 12 || !(job->params.max_slope > 0))
    return WB_EINVAL;
  JobRec *j = new (std::nothrow) JobRec;
  if (!j)
    return WB_ENOMEM;
  j->spec = *job;
  j->est = std::min<uint64_t>(estimateBytes(*job), 0xffffffffffffull);
  std::lock_guard<std::mutex> lk(s->m);
  if (s->stop)
  {
    delete j;
    return WB_ESTATE;
  }
  j->id = s->nextId++;
  j->st.state = WB_JOB_QUEUED;
  j->st.tag = job->tag;
  j->st.n_points = job->cloud.n;
  j->st.t_submit = s->now();
  if (j->est > s->budget && s->cfg.host_budget)
  {
    // runs alone, holding the whole HBM budget, with the rest in host memory
    j->paged = true;
    j->est = s->budget;
    s->queue.push_back(j);
  }
  else if (j->est > s->budget)
  {
    // cannot be admitted even alone
    j->st.state = WB_JOB_FAILED;
    j->st.rc = WB_ENOMEM;
    j->st.t_done = j->st.t_submit;
    s->stats.failed++;
    s->err = "job " + std::to_string(j->id) + ": needs about " + std::to_string(j->est) + " bytes, budget " +
             std::to_string(s->budget);
  }
  else
    s->queue.push_back(j);
  s->jobs[j->id] = j;
  s->stats.submitted++;
  s->cv.notify_all();
  return j->id;
}

int wb_poll(wb_server *s, int64_t id, wb_job_status *st)
{
  if (!s || !st)
    return WB_EINVAL;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end())
    return WB_ENOTFOUND;
  *st = it->second->st;
  return 0;
}

static bool ended(int state)
{
  return state == WB_JOB_DONE || state == WB_JOB_FAILED || state == WB_JOB_CANCELLED;
}

int wb_wait(wb_server *s, int64_t id, double timeout_s, wb_job_status *st)
{
  if (!s)
    return WB_EINVAL;
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end())
    return WB_ENOTFOUND;
  JobRec *j = it->second;
  auto done = [&] { return ended(j->st.state); };
  if (timeout_s < 0)
    s->cv.wait(lk, done);
  else if (!s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
  {
    if (st)
      *st = j->st;
    return WB_ETIMEDOUT;
  }
  if (st)
    *st = j->st;
  return 0;
}

int wb_cancel(wb_server *s, int64_t id)
{
  if (!s)
    return WB_EINVAL;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end())
    return WB_ENOTFOUND;
  JobRec *j = it->second;
  if (j->st.state != WB_JOB_QUEUED)
    return WB_EBUSY;
  s->queue.erase(std::find(s->queue.begin(), s->queue.end(), j));
  j->st.state = WB_JOB_CANCELLED;
  j->st.rc = WB_ECANCELED;
  j->st.t_done = s->now();
  s->stats.cancelled++;
  s->cv.notify_all();
  return 0;
}

int wb_release(wb_server *s, int64_t id)
{
  if (!s)
    return WB_EINVAL;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end())
    return WB_ENOTFOUND;
  if (!ended(it->second->st.state))
    return WB_EBUSY;
  delete it->second;
  s->jobs.erase(it);
  return 0;
}

int wb_server_stats_get(wb_server *s, wb_server_stats *out)
{
  if (!s || !out)
    return WB_EINVAL;
  std::lock_guard<std::mutex> lk(s->m);
  *out = s->stats;
  out->held_bytes = heldBytes(s);
  out->contexts = (int)s->all.size();
  out->queued = (int)s->queue.size();
  out->running = s->prepBusy + (int)s->ready.size() + s->classifying;
  uint64_t l = s->graphLaunches;
  for (wb_ctx *c : s->all)
    l += c->launches;
  out->kernel_launches = l;
  out->now = s->now();
  out->shape = s->cfg.shape;
  out->chunk = s->cfg.chunk;
  out->grid_points = s->cfg.grid_points;
  return 0;
}

int wb_classify_batch(wb_server *s, const wb_job *jobs, int k, int *rcs)
{
  if (!s || (k > 0 && !jobs) || k < 0)
    return WB_EINVAL;
  std::vector<int64_t> ids(k);
  int worst = 0;
  for (int i = 0; i < k; i++)
  {
    ids[i] = wb_submit(s, &jobs[i]);
    if (ids[i] < 0 && rcs)
      rcs[i] = (int)ids[i];
    if (ids[i] < 0)
      worst = (int)ids[i];
  }
  for (int i = 0; i < k; i++)
  {
    if (ids[i] < 0)
      continue;
    wb_job_status st;
    wb_wait(s, ids[i], -1, &st);
    if (rcs)
      rcs[i] = st.rc;
    if (st.rc)
      worst = st.rc;
    wb_release(s, ids[i]);
  }
  return worst;
}

}  // extern "C"
